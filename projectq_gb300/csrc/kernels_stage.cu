// Stage kernel: many gates per pass over the state through shared-memory tiles.
//
// One CTA owns one tile at a time: the 2^L amplitudes that share the values
// of all non-local bits (see stage.hpp).  The tile is 2^(L-m) runs of 2^m
// contiguous amplitudes in HBM, loaded and stored with 16-byte accesses into
// shared memory laid out in tile order; between load and store every
// operation of the stage is applied in shared memory:
//   dense 1- or 2-qubit operations on local targets, with local controls
//   checked per amplitude group and non-local controls once per tile;
//   diagonal operations over up to 6 qubits anywhere in the index (non-local
//   bits come from the tile's base index).
// Grid: persistent CTAs, a multiple of the SM count, striding over tiles.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "kernels.hpp"
#include "stage.hpp"

namespace gsim {
namespace {

struct StageArgs {
  uint64_t ntiles;
  uint32_t L, m, h, nops;
  uint8_t lpos[64];  // ascending global positions of the tile bits
};

template <typename T>
__device__ __forceinline__ cplx_t<T> cmul(cplx_t<T> a, cplx_t<T> b) {
  return mkc<T>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
template <typename T>
__device__ __forceinline__ void cfma(cplx_t<T> m, cplx_t<T> v, T &re, T &im) {
  re = fma(m.x, v.x, re);
  re = fma(-m.y, v.y, re);
  im = fma(m.x, v.y, im);
  im = fma(m.y, v.x, im);
}

template <typename T>
__device__ __forceinline__ void load_tile(cplx_t<T> *__restrict__ tile, const cplx_t<T> *__restrict__ psi,
                                          uint64_t base, const uint64_t *__restrict__ segoff, uint32_t TS,
                                          uint32_t m) {
  if constexpr (sizeof(T) == 4) {
    if (m >= 1) {
      const uint32_t nvec = TS >> 1, mask = (1u << m) - 1;
      for (uint32_t v = threadIdx.x; v < nvec; v += blockDim.x) {
        const uint32_t p = v << 1;
        const uint64_t g = base + segoff[p >> m] + (p & mask);
        *reinterpret_cast<float4 *>(tile + p) = __ldcs(reinterpret_cast<const float4 *>(psi + g));
      }
      return;
    }
  }
  const uint32_t mask = (1u << m) - 1;
  for (uint32_t p = threadIdx.x; p < TS; p += blockDim.x) tile[p] = psi[base + segoff[p >> m] + (p & mask)];
}

template <typename T>
__device__ __forceinline__ void store_tile(const cplx_t<T> *__restrict__ tile, cplx_t<T> *__restrict__ psi,
                                           uint64_t base, const uint64_t *__restrict__ segoff, uint32_t TS,
                                           uint32_t m) {
  if constexpr (sizeof(T) == 4) {
    if (m >= 1) {
      const uint32_t nvec = TS >> 1, mask = (1u << m) - 1;
      for (uint32_t v = threadIdx.x; v < nvec; v += blockDim.x) {
        const uint32_t p = v << 1;
        const uint64_t g = base + segoff[p >> m] + (p & mask);
        __stcs(reinterpret_cast<float4 *>(psi + g), *reinterpret_cast<const float4 *>(tile + p));
      }
      return;
    }
  }
  const uint32_t mask = (1u << m) - 1;
  for (uint32_t p = threadIdx.x; p < TS; p += blockDim.x) psi[base + segoff[p >> m] + (p & mask)] = tile[p];
}

template <typename T>
__global__ void __launch_bounds__(256) stage_kernel(cplx_t<T> *__restrict__ psi, const __grid_constant__ StageArgs A,
                                                    const StageOpDev *__restrict__ ops,
                                                    const cplx_t<T> *__restrict__ pool) {
  using C = cplx_t<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t TS = 1u << A.L;
  C *tile = reinterpret_cast<C *>(smem);
  uint64_t *segoff = reinterpret_cast<uint64_t *>(smem + size_t(TS) * sizeof(C));
  const uint32_t nseg = 1u << A.h;
  for (uint32_t s = threadIdx.x; s < nseg; s += blockDim.x) {
    uint64_t o = 0;
    for (uint32_t b = 0; b < A.h; ++b)
      if ((s >> b) & 1) o |= uint64_t(1) << A.lpos[A.m + b];
    segoff[s] = o;
  }
  __syncthreads();
  for (uint64_t t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
    const uint64_t base = insert_zeros(t, A.lpos, int(A.L));
    load_tile<T>(tile, psi, base, segoff, TS, A.m);
    __syncthreads();
    for (uint32_t o = 0; o < A.nops; ++o) {
      const StageOpDev op = ops[o];
      if ((base & op.gctrl) != op.gctrl) continue;  // non-local controls: same for the whole tile
      const C *M = pool + op.mat;
      if (op.kind == 1) {
        // diagonal: psi_p *= D[bits of the op's qubits]
        uint32_t cidx = 0;
#pragma unroll
        for (int j = 0; j < 6; ++j)
          if (j < int(op.k) && op.tbit[j] == 0xFF) cidx |= uint32_t((base >> op.gbit[j]) & 1) << j;
        for (uint32_t p = threadIdx.x; p < TS; p += blockDim.x) {
          uint32_t idx = cidx;
#pragma unroll
          for (int j = 0; j < 6; ++j)
            if (j < int(op.k) && op.tbit[j] != 0xFF) idx |= ((p >> op.tbit[j]) & 1u) << j;
          tile[p] = cmul<T>(tile[p], M[idx]);
        }
      } else if (op.k == 1) {
        const uint32_t tb = op.tbit[0], d = 1u << tb, lc = op.lctrl;
        const C m00 = M[0], m01 = M[1], m10 = M[2], m11 = M[3];
        for (uint32_t g = threadIdx.x; g < (TS >> 1); g += blockDim.x) {
          const uint32_t p0 = ((g >> tb) << (tb + 1)) | (g & (d - 1));
          if ((p0 & lc) != lc) continue;
          const C a = tile[p0], b = tile[p0 + d];
          T r0 = T(0), i0 = T(0), r1 = T(0), i1 = T(0);
          cfma<T>(m00, a, r0, i0);
          cfma<T>(m01, b, r0, i0);
          cfma<T>(m10, a, r1, i1);
          cfma<T>(m11, b, r1, i1);
          tile[p0] = mkc<T>(r0, i0);
          tile[p0 + d] = mkc<T>(r1, i1);
        }
      } else {
        const uint32_t t0 = op.tbit[0], t1 = op.tbit[1], lc = op.lctrl;
        const uint32_t lo = min(t0, t1), hi = max(t0, t1);
        const uint32_t d0 = 1u << t0, d1 = 1u << t1;
        C mm[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) mm[j] = M[j];
        for (uint32_t g = threadIdx.x; g < (TS >> 2); g += blockDim.x) {
          uint32_t p = ((g >> lo) << (lo + 1)) | (g & ((1u << lo) - 1));
          p = ((p >> hi) << (hi + 1)) | (p & ((1u << hi) - 1));
          if ((p & lc) != lc) continue;
          C v[4] = {tile[p], tile[p + d0], tile[p + d1], tile[p + d0 + d1]};
          C out[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            T re = T(0), im = T(0);
#pragma unroll
            for (int j = 0; j < 4; ++j) cfma<T>(mm[r * 4 + j], v[j], re, im);
            out[r] = mkc<T>(re, im);
          }
          tile[p] = out[0];
          tile[p + d0] = out[1];
          tile[p + d1] = out[2];
          tile[p + d0 + d1] = out[3];
        }
      }
      __syncthreads();
    }
    store_tile<T>(tile, psi, base, segoff, TS, A.m);
    __syncthreads();
  }
}

int stage_sms() {
  static int n = 0;
  if (!n) {
    int d = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
    if (n <= 0) n = 1;
  }
  return n;
}

template <typename T>
cudaError_t launch_stage_t(void *psi, unsigned nq, const StagePlan &plan, const void *d_ops,
                           const void *d_pool, cudaStream_t s) {
  StageArgs A;
  std::memset(&A, 0, sizeof(A));
  A.L = plan.L;
  unsigned m = 0;
  while (m < plan.lpos.size() && plan.lpos[m] == m) ++m;
  A.m = std::min<unsigned>(m, plan.L);
  A.h = A.L - A.m;
  A.nops = uint32_t(plan.ops.size());
  A.ntiles = uint64_t(1) << (nq - plan.L);
  for (size_t i = 0; i < plan.lpos.size(); ++i) A.lpos[i] = uint8_t(plan.lpos[i]);
  const size_t smem = (size_t(1) << A.L) * sizeof(cplx_t<T>) + (size_t(1) << A.h) * 8;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(stage_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    attr_set = true;
  }
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stage_kernel<T>, 256, smem);
  per_sm = std::max(1, per_sm);
  const uint64_t grid = std::min<uint64_t>(A.ntiles, uint64_t(stage_sms()) * per_sm);
  stage_kernel<T><<<unsigned(grid), 256, smem, s>>>(static_cast<cplx_t<T> *>(psi), A,
                                                    static_cast<const StageOpDev *>(d_ops),
                                                    static_cast<const cplx_t<T> *>(d_pool));
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_stage(int prec, void *psi, unsigned nq, const StagePlan &plan, const void *d_ops,
                         const void *d_pool, cudaStream_t s) {
  if (plan.ops.empty()) return cudaSuccess;
  return prec == 1 ? launch_stage_t<float>(psi, nq, plan, d_ops, d_pool, s)
                   : launch_stage_t<double>(psi, nq, plan, d_ops, d_pool, s);
}

}  // namespace gsim
