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
// caches it; make that first call before any stream capture on the device.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gb300sim.h"
#include "common.cuh"

namespace gsim {
extern thread_local std::string g_last_error;
}

namespace {

constexpr int kMaxBlocks = 4096;
constexpr uint64_t kPerBlock = uint64_t(1) << 20;  // amplitudes summed by one block
constexpr uint64_t kMaxUnits = uint64_t(kMaxBlocks) * kPerBlock;  // 2^32 amplitudes
constexpr int kScratchDoubles = kMaxBlocks + 8;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_addr[kMaxDevices] = {};

struct Spec {
  uint8_t pos[64];
  int n;
};

template <typename T>
__global__ void __launch_bounds__(256) masked_norm_noalloc(const gsim::cplx_t<T> *__restrict__ psi,
                                                           uint64_t units, uint64_t val, Spec ms,
                                                           double *scratch, unsigned nblk) {
  // Sum |psi_i|^2 over this block's share of the subspace (FP64 carried).
  const uint64_t u0 = uint64_t(blockIdx.x) * kPerBlock;
  const uint64_t u1 = min(units, u0 + kPerBlock);
  double acc = 0.;
  for (uint64_t u = u0 + threadIdx.x; u < u1; u += blockDim.x)
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
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return fail_with(GSIM_ERR_CUDA, std::string("probability_noalloc(): cudaGetSymbolAddress: ") +
                                            cudaGetErrorString(e));
      g_addr[dev] = static_cast<double *>(p);
    }
    scratch = g_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned nblk = unsigned((units + kPerBlock - 1) / kPerBlock);
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
