// Fused dense k-qubit gates (k = 5, 6) on complex64 states with the 5th
// generation tensor cores (tcgen05, TMEM accumulators), split-precision
// 3xTF32 with FP32 accumulation.
//
// Per tile of 128 amplitude groups (one group = the 2^k amplitudes that differ
// only in the target bits):
//   D[g][c] = sum_kk A[g][kk] * B[c][kk]
//   A[g][2j + s]  = component s (re, im) of input amplitude j of group g
//   B[2a][2j]   = Re U[a][j]   B[2a][2j+1]   = -Im U[a][j]
//   B[2a+1][2j] = Im U[a][j]   B[2a+1][2j+1] =  Re U[a][j]
// so D[g][2a], D[g][2a+1] are the real and imaginary parts of output a.
// M = 128 groups (TMEM lanes), N = K = 2^(k+1).  Each operand is split in
// shared memory into hi = tf32(x) and lo = tf32(x - hi); three MMAs per
// K-step accumulate hi*hi + hi*lo + lo*hi.  B (the unitary) stays resident
// in shared memory for the whole kernel; A is gathered from HBM in chunks
// of 64 real components (32 amplitudes) per group.
//
// Roles: all 128 threads gather/split A and run the epilogue (thread t owns
// group t = TMEM lane t); thread 0 issues the MMAs; completion is signalled
// by tcgen05.commit on an mbarrier whose wait is bounded (on timeout the
// kernel records an error code and frees TMEM before returning).
// Shared-memory operands use the canonical K-major, no-swizzle layout:
// 8-row x 16-byte core matrices; LBO = core stride along K, SBO = stride
// between 8-row groups.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "kernels.hpp"

namespace gsim {
namespace {

constexpr int kKC = 64;  // real K components per A chunk

struct TcArgs {
  uint64_t groups;      // number of amplitude groups
  uint64_t ctrl_set;
  int nins, k;
  uint8_t ins[64];
  uint64_t off[64];     // offset of amplitude j of a group (j < 2^k, k <= 6)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Byte offset of element (row, kk) in a K-major no-swizzle operand whose rows
// hold kcols fp32 elements.
__device__ __forceinline__ uint32_t kmajor_off(uint32_t row, uint32_t kk, uint32_t kcols) {
  return ((row >> 3) * (kcols >> 2) + (kk >> 2)) * 128u + (row & 7u) * 16u + (kk & 3u) * 4u;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((addr >> 4) & 0x3FFFu);
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, no swizzle
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

// Bounded wait for the mbarrier phase `parity`; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (uint32_t it = 0; it < (1u << 24); ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (it > 1024) __nanosleep(64);
  }
  return false;
}

template <int NCOL>
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// K = N = 2^(k+1); B (N x K, hi and lo) resident; A chunks of 128 x kKC.
template <int KQ>
__global__ void __launch_bounds__(128, 1) tc_gate_kernel(float2 *__restrict__ psi, const float *__restrict__ b_hi,
                                                         const float *__restrict__ b_lo,
                                                         const __grid_constant__ TcArgs A, int *err) {
  constexpr int D = 1 << KQ;       // complex dimension
  constexpr int K = 2 * D;         // real K (= N)
  constexpr int N = K;
  constexpr int NCH = K / kKC;     // A chunks per tile
  constexpr uint32_t A_BYTES = 128u * kKC * 4u;
  constexpr uint32_t B_BYTES = uint32_t(N) * K * 4u;
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char *a_hi = sm, *a_lo = sm + A_BYTES, *bh = sm + 2 * A_BYTES, *bl = bh + B_BYTES;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(bl + B_BYTES);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 1);
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5;
  // B: copy the pre-split unitary into the K-major core layout.
  for (int e = tid; e < N * K; e += 128) {
    const int c = e / K, kk = e % K;
    const uint32_t o = kmajor_off(uint32_t(c), uint32_t(kk), uint32_t(K));
    *reinterpret_cast<float *>(bh + o) = b_hi[e];
    *reinterpret_cast<float *>(bl + o) = b_lo[e];
  }
  if (tid == 0) {
    abort_flag = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(uint32_t(N < 32 ? 32 : N))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t mb = smem_u32(mbar);
  // idesc: D = F32, A = B = TF32, both K-major, N >> 3, M >> 4 (M = 128).
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(128 >> 4) << 24);
  const uint32_t ahi_a = smem_u32(a_hi), alo_a = smem_u32(a_lo), bh_a = smem_u32(bh), bl_a = smem_u32(bl);
  uint32_t phase = 0;
  const uint64_t ntiles = (A.groups + 127) / 128;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t g = tile * 128 + uint64_t(tid);
    const bool active = g < A.groups;
    const uint64_t base = active ? (insert_zeros(g, A.ins, A.nins) | A.ctrl_set) : 0;
    for (int ch = 0; ch < NCH; ++ch) {
      // gather + split this chunk of 32 amplitudes (64 real components)
#pragma unroll 8
      for (int jj = 0; jj < kKC / 2; ++jj) {
        const int j = ch * (kKC / 2) + jj;
        float2 x = make_float2(0.f, 0.f);
        if (active) x = __ldcs(psi + base + A.off[j]);
        const float hr = tf32_round(x.x), hi_ = tf32_round(x.y);
        const float lr = tf32_round(x.x - hr), li = tf32_round(x.y - hi_);
        const uint32_t o0 = kmajor_off(uint32_t(tid), uint32_t(2 * jj), kKC);
        const uint32_t o1 = kmajor_off(uint32_t(tid), uint32_t(2 * jj + 1), kKC);
        *reinterpret_cast<float *>(a_hi + o0) = hr;
        *reinterpret_cast<float *>(a_hi + o1) = hi_;
        *reinterpret_cast<float *>(a_lo + o0) = lr;
        *reinterpret_cast<float *>(a_lo + o1) = li;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (abort_flag) break;
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
        for (int s = 0; s < kKC / 8; ++s) {
          // K-step s of this chunk: A cores 2s, 2s+1; B cores at the global K offset
          const uint32_t ak = uint32_t(2 * s) * 128u;
          const uint32_t bk = uint32_t(ch * (kKC / 4) + 2 * s) * 128u;
          const uint64_t dah = smem_desc(ahi_a + ak, 128u, (kKC / 4) * 128u);
          const uint64_t dal = smem_desc(alo_a + ak, 128u, (kKC / 4) * 128u);
          const uint64_t dbh = smem_desc(bh_a + bk, 128u, (K / 4) * 128u);
          const uint64_t dbl = smem_desc(bl_a + bk, 128u, (K / 4) * 128u);
          const uint32_t acc0 = (ch > 0 || s > 0) ? 1u : 0u;
          mma_tf32(tmem, dal, dbh, idesc, acc0);
          mma_tf32(tmem, dah, dbl, idesc, 1u);
          mma_tf32(tmem, dah, dbh, idesc, 1u);
        }
        mma_commit(mb);
      }
      if (!mbar_wait(mb, phase)) {
        if (tid == 0) atomicExch(err, 1);
        abort_flag = 1;
      }
      phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      __syncthreads();
      if (abort_flag) break;
    }
    if (abort_flag) break;
    // epilogue: TMEM lane (32 warp + lane) = group; N fp32 columns = D complex outputs
    const uint32_t lane_base = uint32_t(warp * 32) << 16;
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tmem_ld16<16>(tmem + lane_base + uint32_t(c0), v);
      if (active) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int a = c0 / 2 + q;
          __stcs(psi + base + A.off[a], make_float2(v[2 * q], v[2 * q + 1]));
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(uint32_t(N < 32 ? 32 : N))
                 : "memory");
}

template <int KQ>
cudaError_t launch_tc_k(void *psi, unsigned nq, const DenseOp &op, const float *d_bhi, const float *d_blo,
                        int *d_err, cudaStream_t s) {
  constexpr int D = 1 << KQ, K = 2 * D, N = K;
  TcArgs A;
  std::memset(&A, 0, sizeof(A));
  std::vector<unsigned> ins(op.pos.begin(), op.pos.end());
  for (unsigned b = 0; b < 64; ++b)
    if ((op.ctrl_mask >> b) & 1) ins.push_back(b);
  std::sort(ins.begin(), ins.end());
  if (ins.size() > nq) throw std::invalid_argument("gate wider than the state");
  A.nins = int(ins.size());
  for (size_t i = 0; i < ins.size(); ++i) A.ins[i] = uint8_t(ins[i]);
  A.k = KQ;
  A.ctrl_set = op.ctrl_mask;
  for (int j = 0; j < D; ++j)
    for (int l = 0; l < KQ; ++l)
      if ((j >> l) & 1) A.off[j] |= uint64_t(1) << op.pos[l];
  A.groups = uint64_t(1) << (nq - ins.size());
  const size_t smem = 2 * size_t(128) * kKC * 4 + 2 * size_t(N) * K * 4 + 16;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(tc_gate_kernel<KQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    attr = true;
  }
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t ntiles = (A.groups + 127) / 128;
  const unsigned grid = unsigned(std::max<uint64_t>(1, std::min<uint64_t>(ntiles, uint64_t(sms))));
  tc_gate_kernel<KQ><<<grid, 128, smem, s>>>(static_cast<float2 *>(psi), d_bhi, d_blo, A, d_err);
  return cudaGetLastError();
}

}  // namespace

// B operand (N x K row-major real embedding of U, split hi/lo in TF32) on the host.
void tc_split_unitary(const std::vector<cplx> &U, int k, std::vector<float> &hi, std::vector<float> &lo) {
  const int D = 1 << k, K = 2 * D;
  hi.assign(size_t(K) * K, 0.f);
  lo.assign(size_t(K) * K, 0.f);
  auto tf32 = [](float x) {  // round to nearest (ties away), 10 explicit mantissa bits
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
  };
  for (int a = 0; a < D; ++a)
    for (int j = 0; j < D; ++j) {
      const double re = U[size_t(a) * D + j].real(), im = U[size_t(a) * D + j].imag();
      const double vals[4] = {re, -im, im, re};  // (2a,2j) (2a,2j+1) (2a+1,2j) (2a+1,2j+1)
      const int rows[4] = {2 * a, 2 * a, 2 * a + 1, 2 * a + 1}, cols[4] = {2 * j, 2 * j + 1, 2 * j, 2 * j + 1};
      for (int t = 0; t < 4; ++t) {
        const float h = tf32(float(vals[t]));
        const float l = tf32(float(vals[t] - double(h)));
        hi[size_t(rows[t]) * K + cols[t]] = h;
        lo[size_t(rows[t]) * K + cols[t]] = l;
      }
    }
}

cudaError_t launch_tc_gate(void *psi, unsigned nq, const DenseOp &op, const float *d_bhi, const float *d_blo,
                           int *d_err, cudaStream_t s) {
  switch (op.pos.size()) {
    case 5: return launch_tc_k<5>(psi, nq, op, d_bhi, d_blo, d_err, s);
    case 6: return launch_tc_k<6>(psi, nq, op, d_bhi, d_blo, d_err, s);
    default: throw std::invalid_argument("tensor-core gate kernel supports 5 or 6 targets");
  }
}

}  // namespace gsim
