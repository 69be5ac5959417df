// Probability of a bit pattern over a caller-owned device state vector,
// computed without allocating any memory.
//
// Who needs this: callers that cannot call cudaMalloc (or any allocating
// routine) at the point where they ask for a probability — for example code
// running under a foreign memory manager that owns every device allocation,
// or a host thread that must not take the allocator's locks while another
// library holds the device.  The regular path (gsim_get_probability) needs an
// engine and its grown-on-demand scratch buffers; this entry point takes a
// raw device pointer and uses only the fixed scratch array below.
//
// Scratch: g_noalloc_scratch, a file-scope __device__ array of
// kScratchDoubles doubles (about 32 KB) that every GPU which loads this
// library holds until the process exits.  Slots [0, kMaxBlocks) take the
// per-block partial sums, slot kMaxBlocks the completion counter (must start
// at zero; cleared by every call), slot kMaxBlocks + 1 the result.  All
// calls share the array and it keeps the last call's contents, so calls
// that overlap on the GPU (different streams, or different host threads)
// race on it and must be serialised by the caller.
//
// Set-up: host code cannot use the array's name as a device address (on the
// host it names a stand-in object; a kernel given that address faults or, on
// systems where the GPU reaches host memory, silently reads the wrong
// memory).  The first call on each device therefore resolves the array's
// device address with cudaGetSymbolAddress while that device is current and
// caches it, keyed by the device's current CUDA context: a call under another
// context (after cudaDeviceReset, or a caller's own driver-API context)
// resolves it again.  That first call is also when the CUDA runtime loads
// this file's module and places the array (lazy module loading); from then
// on nothing is allocated.  A caller that must not see even that placement
// makes one warm-up call (or sets CUDA_MODULE_LOADING=EAGER) first.  Make
// the first call on a device before any stream capture on that device.
//
// The call is synchronous: it waits for its stream and returns the result
// on the host.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gb300sim.h"
#include "common.cuh"

namespace gsim {
extern thread_local std::string g_last_error;
}

namespace {

constexpr int kMaxBlocks = 4096;                          // partial-sum slots
constexpr uint64_t kMinPerBlock = uint64_t(1) << 14;       // amplitudes per block before the grid grows
constexpr uint64_t kMaxUnits = uint64_t(1) << 32;          // largest summed subspace
constexpr int kScratchDoubles = kMaxBlocks + 8;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_addr[kMaxDevices] = {};
CUcontext g_ctx[kMaxDevices] = {};

// cuCtxGetCurrent through the runtime's driver entry point (no link to libcuda)
using CtxGetCurrent = CUresult (*)(CUcontext *);
CtxGetCurrent ctx_get_current() {
  static CtxGetCurrent fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrent>(p);
  }();
  return fn;
}

struct Spec {
  uint8_t pos[64];
  int n;
};

template <typename T>
__global__ void __launch_bounds__(256) masked_norm_noalloc(const gsim::cplx_t<T> *__restrict__ psi,
                                                           uint64_t units, uint64_t val, Spec ms,
                                                           double *scratch, unsigned nblk) {
  // Sum |psi_i|^2 over this block's share of the subspace (grid-stride,
  // FP64 carried); the grid is at most kMaxBlocks blocks, one slot each.
  double acc = 0.;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < units; u += stride)
    acc += gsim::norm2_fp64(psi[gsim::insert_zeros(u, ms.pos, ms.n) | val]);
  acc = gsim::block_sum(acc);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = acc;
    __threadfence();
    unsigned *count = reinterpret_cast<unsigned *>(&scratch[kMaxBlocks]);
    last = atomicAdd(count, 1u) == nblk - 1;
  }
  __syncthreads();
  if (!last) return;
  // The last block to finish adds the partials in a fixed order.
  __threadfence();
  double s = 0.;
  for (unsigned b = threadIdx.x; b < nblk; b += blockDim.x)
    s += const_cast<volatile double *>(scratch)[b];
  s = gsim::block_sum(s);
  if (threadIdx.x == 0) {
    scratch[kMaxBlocks + 1] = s;
    *reinterpret_cast<unsigned *>(&scratch[kMaxBlocks]) = 0u;
  }
}

int fail_with(int code, const std::string &msg) {
  gsim::g_last_error = msg;
  return code;
}

}  // namespace

extern "C" GSIM_API int gsim_probability_noalloc(const void *d_state, int precision,
                                                 uint32_t nqubits, uint64_t mask, uint64_t value,
                                                 double *out, void *stream) {
  if (!d_state || !out) return fail_with(GSIM_ERR_VALUE, "probability_noalloc(): null pointer");
  if (precision != GSIM_C64 && precision != GSIM_C128)
    return fail_with(GSIM_ERR_VALUE, "probability_noalloc(): unknown precision");
  if (nqubits > 48) return fail_with(GSIM_ERR_VALUE, "probability_noalloc(): too many qubits");
  if (nqubits < 64 && (mask >> nqubits) != 0)
    return fail_with(GSIM_ERR_VALUE, "probability_noalloc(): mask names bits beyond the state");
  if ((value & ~mask) != 0) return fail_with(GSIM_ERR_VALUE, "probability_noalloc(): value outside mask");
  Spec ms;
  std::memset(&ms, 0, sizeof(ms));
  for (unsigned b = 0; b < 64; ++b)
    if ((mask >> b) & 1) ms.pos[ms.n++] = uint8_t(b);
  const uint64_t units = uint64_t(1) << (nqubits - unsigned(ms.n));
  if (units > kMaxUnits)
    return fail_with(GSIM_ERR_LENGTH,
                     "probability_noalloc(): the summed subspace has " + std::to_string(units) +
                         " amplitudes; the fixed scratch supports at most 2^32");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail_with(GSIM_ERR_CUDA, std::string("probability_noalloc(): no usable device: ") +
                                        cudaGetErrorString(e));
  CUcontext ctx = nullptr;
  if (CtxGetCurrent f = ctx_get_current()) f(&ctx);
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev] || g_ctx[dev] != ctx) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return fail_with(GSIM_ERR_CUDA, std::string("probability_noalloc(): cudaGetSymbolAddress: ") +
                                            cudaGetErrorString(e));
      g_addr[dev] = static_cast<double *>(p);
      g_ctx[dev] = ctx;
    }
    scratch = g_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // enough blocks to fill the GPU for mid-size subspaces, one scratch slot each
  const unsigned nblk = unsigned(std::min<uint64_t>(kMaxBlocks, (units + kMinPerBlock - 1) / kMinPerBlock));
  e = cudaMemsetAsync(&scratch[kMaxBlocks], 0, sizeof(double), s);  // the counter starts at zero
  if (e == cudaSuccess) {
    if (precision == GSIM_C64)
      masked_norm_noalloc<float><<<nblk, 256, 0, s>>>(static_cast<const float2 *>(d_state), units, value, ms,
                                                      scratch, nblk);
    else
      masked_norm_noalloc<double><<<nblk, 256, 0, s>>>(static_cast<const double2 *>(d_state), units, value,
                                                       ms, scratch, nblk);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, &scratch[kMaxBlocks + 1], sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return fail_with(GSIM_ERR_CUDA, std::string("probability_noalloc(): ") + cudaGetErrorString(e));
  return GSIM_OK;
}
