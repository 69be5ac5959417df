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

struct alignas(16) StageTable {
  unsigned char bytes[kStageTableBytes];  // [SubstageDev...][SubOpDev...] of one stage
};

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

// ---- register substages (stage.hpp: build_substages) ----------------------
// s(p) = p ^ fold(p >> rho) is linear over XOR: s(a ^ b) = s(a) ^ s(b), so a
// thread's offsets are its own s(.) XOR compile-time constants.
__host__ __device__ constexpr uint32_t swz(uint32_t p, uint32_t rho) {
  uint32_t x = p >> rho, f = 0;
  const uint32_t mask = (1u << rho) - 1;
  while (x) {
    f ^= x & mask;
    x >>= rho;
  }
  return p ^ f;
}

template <typename T>
__device__ __forceinline__ void cmac_k(int kd, cplx_t<T> m, cplx_t<T> v, T &re, T &im) {
  if (kd & 1) {
    re = fma(m.x, v.x, re);
    im = fma(m.x, v.y, im);
  }
  if (kd & 2) {
    re = fma(-m.y, v.y, re);
    im = fma(m.y, v.x, im);
  }
}

// One 1-qubit operation on register bit B, matrix class CLS (stage.hpp):
// 0 general complex, 1 real, 2 real diagonal / imaginary off-diagonal,
// 4 anti-diagonal.  `amask` selects the group bases j the operation touches.
// (A second, mask-free copy of these paths for operations without register
// controls measured 24% slower on the 30-qubit circuit: the larger hot code
// costs more than the per-group tests it saves.)
template <typename T, int R, int B, int CLS>
__device__ __forceinline__ void reg_dense1(cplx_t<T> (&v)[1 << R], uint32_t amask, const cplx_t<T> *M) {
  const cplx_t<T> m00 = M[0], m01 = M[1], m10 = M[2], m11 = M[3];
#pragma unroll
  for (int j = 0; j < (1 << R); ++j) {
    if ((j >> B) & 1) continue;
    if (!((amask >> j) & 1)) continue;
    const cplx_t<T> a = v[j], b = v[j | (1 << B)];
    T r0, i0, r1, i1;
    if constexpr (CLS == 1) {
      r0 = fma(m00.x, a.x, m01.x * b.x);
      i0 = fma(m00.x, a.y, m01.x * b.y);
      r1 = fma(m10.x, a.x, m11.x * b.x);
      i1 = fma(m10.x, a.y, m11.x * b.y);
    } else if constexpr (CLS == 2) {
      r0 = fma(m00.x, a.x, -m01.y * b.y);
      i0 = fma(m00.x, a.y, m01.y * b.x);
      r1 = fma(-m10.y, a.y, m11.x * b.x);
      i1 = fma(m10.y, a.x, m11.x * b.y);
    } else if constexpr (CLS == 4) {
      r0 = fma(m01.x, b.x, -m01.y * b.y);
      i0 = fma(m01.x, b.y, m01.y * b.x);
      r1 = fma(m10.x, a.x, -m10.y * a.y);
      i1 = fma(m10.x, a.y, m10.y * a.x);
    } else {
      r0 = fma(m00.x, a.x, fma(-m00.y, a.y, fma(m01.x, b.x, -m01.y * b.y)));
      i0 = fma(m00.x, a.y, fma(m00.y, a.x, fma(m01.x, b.y, m01.y * b.x)));
      r1 = fma(m10.x, a.x, fma(-m10.y, a.y, fma(m11.x, b.x, -m11.y * b.y)));
      i1 = fma(m10.x, a.y, fma(m10.y, a.x, fma(m11.x, b.y, m11.y * b.x)));
    }
    v[j] = mkc<T>(r0, i0);
    v[j | (1 << B)] = mkc<T>(r1, i1);
  }
}

template <typename T, int R, int B>
__device__ __forceinline__ void reg_dense1_cls(cplx_t<T> (&v)[1 << R], const SubOpDev &op, const cplx_t<T> *M) {
  switch (op.cls) {
    case 1: reg_dense1<T, R, B, 1>(v, op.amask, M); break;
    case 2: reg_dense1<T, R, B, 2>(v, op.amask, M); break;
    case 4: reg_dense1<T, R, B, 4>(v, op.amask, M); break;
    default: reg_dense1<T, R, B, 0>(v, op.amask, M); break;
  }
}

template <typename T, int R, int B>
__device__ __forceinline__ void reg_swap(cplx_t<T> (&v)[1 << R], const SubOpDev &op) {
#pragma unroll
  for (int j = 0; j < (1 << R); ++j) {
    if ((j >> B) & 1) continue;
    if (!((op.amask >> j) & 1)) continue;
    const cplx_t<T> a = v[j];
    v[j] = v[j | (1 << B)];
    v[j | (1 << B)] = a;
  }
}

template <typename T, int R, int B0, int B1>
__device__ __forceinline__ void reg_dense2(cplx_t<T> (&v)[1 << R], const SubOpDev &op, const cplx_t<T> *M) {
  // matrix rows are re-read from shared memory (broadcast) per group rather
  // than held in 32 registers: this path sets the kernel's register budget
#pragma unroll
  for (int j = 0; j < (1 << R); ++j) {
    if (((j >> B0) & 1) || ((j >> B1) & 1)) continue;
    if (!((op.amask >> j) & 1)) continue;
    const int j1 = j | (1 << B0), j2 = j | (1 << B1), j3 = j1 | (1 << B1);
    const cplx_t<T> x[4] = {v[j], v[j1], v[j2], v[j3]};
    cplx_t<T> y[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      T re = T(0), im = T(0);
#pragma unroll
      for (int b = 0; b < 4; ++b) cfma<T>(M[a * 4 + b], x[b], re, im);
      y[a] = mkc<T>(re, im);
    }
    v[j] = y[0];
    v[j1] = y[1];
    v[j2] = y[2];
    v[j3] = y[3];
  }
}

// Diagonal with one register qubit (register bit B): two factors.
template <typename T, int R, int B>
__device__ __forceinline__ void reg_diag1(cplx_t<T> (&v)[1 << R], cplx_t<T> f0, cplx_t<T> f1) {
#pragma unroll
  for (int j = 0; j < (1 << R); ++j) v[j] = cmul<T>(v[j], ((j >> B) & 1) ? f1 : f0);
}

template <typename T, int R>
__device__ __forceinline__ void reg_apply(cplx_t<T> (&v)[1 << R], const SubOpDev &op, const cplx_t<T> *M,
                                          uint32_t row, uint64_t base) {
  if (op.kind == 2) {
    // index bits from row and non-local qubits (once), register qubits (table)
    uint32_t cidx = 0;
    for (int q = 0; q < int(op.dk); ++q) {
      if (op.dloc[q] == 1) cidx |= ((row >> op.didx[q]) & 1u) << q;
      else if (op.dloc[q] == 2) cidx |= uint32_t((base >> op.didx[q]) & 1) << q;
    }
    if (op.dreg == 0) {  // one factor for all of this thread's amplitudes
      const cplx_t<T> f = M[cidx];
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) v[j] = cmul<T>(v[j], f);
      return;
    }
    if (op.dreg == 1) {
      const cplx_t<T> f0 = M[cidx], f1 = M[cidx | (1u << op.dq)];
      switch (op.dB) {
        case 0: reg_diag1<T, R, 0>(v, f0, f1); break;
        case 1: if constexpr (R > 1) reg_diag1<T, R, 1>(v, f0, f1); break;
        case 2: if constexpr (R > 2) reg_diag1<T, R, 2>(v, f0, f1); break;
        case 3: if constexpr (R > 3) reg_diag1<T, R, 3>(v, f0, f1); break;
        case 4: if constexpr (R > 4) reg_diag1<T, R, 4>(v, f0, f1); break;
      }
      return;
    }
    const uint4 jt = *reinterpret_cast<const uint4 *>(op.jidx);
    uint4 jt2 = make_uint4(0, 0, 0, 0);
    if constexpr (R > 4) jt2 = *reinterpret_cast<const uint4 *>(op.jidx + 16);
    const uint32_t jw[8] = {jt.x, jt.y, jt.z, jt.w, jt2.x, jt2.y, jt2.z, jt2.w};
#pragma unroll
    for (int j = 0; j < (1 << R); ++j) {
      const uint32_t idx = cidx | ((jw[j >> 2] >> (8 * (j & 3))) & 0xFFu);
      v[j] = cmul<T>(v[j], M[idx]);
    }
    return;
  }
  if (op.kind == 0 && op.swap) {
    // exactly X on a register bit (CNOT, Toffoli...): exchange registers
    switch (op.rb[0]) {
      case 0: reg_swap<T, R, 0>(v, op); break;
      case 1: if constexpr (R > 1) reg_swap<T, R, 1>(v, op); break;
      case 2: if constexpr (R > 2) reg_swap<T, R, 2>(v, op); break;
      case 3: if constexpr (R > 3) reg_swap<T, R, 3>(v, op); break;
      case 4: if constexpr (R > 4) reg_swap<T, R, 4>(v, op); break;
    }
    return;
  }
  if (op.kind == 0) {
    switch (op.rb[0]) {
      case 0: reg_dense1_cls<T, R, 0>(v, op, M); break;
      case 1: if constexpr (R > 1) reg_dense1_cls<T, R, 1>(v, op, M); break;
      case 2: if constexpr (R > 2) reg_dense1_cls<T, R, 2>(v, op, M); break;
      case 3: if constexpr (R > 3) reg_dense1_cls<T, R, 3>(v, op, M); break;
      case 4: if constexpr (R > 4) reg_dense1_cls<T, R, 4>(v, op, M); break;
    }
    return;
  }
  const int key = op.rb[0] * 8 + op.rb[1];
#define GSIM_D2(a, b) \
  case a * 8 + b:     \
    if constexpr (R > a && R > b) reg_dense2<T, R, a, b>(v, op, M); \
    break;
  switch (key) {
    GSIM_D2(0, 1) GSIM_D2(1, 0) GSIM_D2(0, 2) GSIM_D2(2, 0) GSIM_D2(0, 3) GSIM_D2(3, 0)
    GSIM_D2(1, 2) GSIM_D2(2, 1) GSIM_D2(1, 3) GSIM_D2(3, 1) GSIM_D2(2, 3) GSIM_D2(3, 2)
    GSIM_D2(0, 4) GSIM_D2(4, 0) GSIM_D2(1, 4) GSIM_D2(4, 1) GSIM_D2(2, 4) GSIM_D2(4, 2)
    GSIM_D2(3, 4) GSIM_D2(4, 3)
  }
#undef GSIM_D2
}

template <typename T, int R>
__global__ void __launch_bounds__(256, R > 4 ? 2 : 3) stage_reg_kernel(cplx_t<T> *__restrict__ psi, const __grid_constant__ StageArgs A,
                                                        const __grid_constant__ StageTable Tb,
                                                        const unsigned char *__restrict__ pool_src, uint32_t nsubs,
                                                        uint32_t sops_off, uint32_t pool_bytes, uint32_t rho) {
  // The substage and operation descriptors are read from the kernel parameter
  // (constant bank): every thread of a warp reads the same descriptor, so the
  // per-operation control flow runs on warp-uniform values.  Shared memory:
  // the tile (2^L amplitudes, swizzled), the segment offsets, then a copy of
  // the matrices and diagonal tables (indexed per thread).
  using C = cplx_t<T>;
  constexpr uint32_t TS = 1u << (R + 8);
  constexpr int PER = sizeof(T) == 4 ? TS / 512 : TS / 256;  // 16-byte loads per thread per tile
  extern __shared__ __align__(16) unsigned char smem[];
  C *tile = reinterpret_cast<C *>(smem);
  uint64_t *segoff = reinterpret_cast<uint64_t *>(smem + size_t(TS) * sizeof(C));
  // the table starts 16-byte aligned (the segment table can be a single entry)
  unsigned char *tab = smem + size_t(TS) * sizeof(C) + (((size_t(1) << A.h) * 8 + 15) & ~size_t(15));
  const uint32_t nseg = 1u << A.h;
  for (uint32_t s = threadIdx.x; s < nseg; s += blockDim.x) {
    uint64_t o = 0;
    for (uint32_t b = 0; b < A.h; ++b)
      if ((s >> b) & 1) o |= uint64_t(1) << A.lpos[A.m + b];
    segoff[s] = o;
  }
  for (uint32_t i = threadIdx.x; i < pool_bytes / 16; i += blockDim.x)
    reinterpret_cast<uint4 *>(tab)[i] = reinterpret_cast<const uint4 *>(pool_src)[i];
  __syncthreads();
  const SubstageDev *subs = reinterpret_cast<const SubstageDev *>(Tb.bytes);
  const SubOpDev *ops = reinterpret_cast<const SubOpDev *>(Tb.bytes + sops_off);
  const C *pool = reinterpret_cast<const C *>(tab);
  const uint32_t row = threadIdx.x;
  const uint32_t mask = (1u << A.m) - 1;
  constexpr uint32_t RHO = sizeof(T) == 4 ? 4u : 3u;  // the planner's bank-class bits (checked at launch)
  // this thread's tile positions are (t + 256 i) << 1 (complex64) or t + 256 i
  const uint32_t sw_t = sizeof(T) == 4 ? swz(threadIdx.x << 1, RHO) : swz(threadIdx.x, RHO);
  for (uint64_t t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
    const uint64_t base = insert_zeros(t, A.lpos, int(A.L));
    // Issue every load of the tile before the first shared-memory store.
    if constexpr (sizeof(T) == 4) {
      float4 x[PER];
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const uint32_t p = (threadIdx.x + i * 256u) << 1;
        x[i] = __ldcs(reinterpret_cast<const float4 *>(psi + base + segoff[p >> A.m] + (p & mask)));
      }
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const uint32_t sp = sw_t ^ swz(512u * i, RHO);  // s(p), p = (t + 256 i) << 1; s(p + 1) = s(p) ^ 1
        tile[sp] = make_float2(x[i].x, x[i].y);
        tile[sp ^ 1u] = make_float2(x[i].z, x[i].w);
      }
    } else {
      C x[PER];
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const uint32_t p = threadIdx.x + i * 256u;
        x[i] = __ldcs(psi + base + segoff[p >> A.m] + (p & mask));
      }
#pragma unroll
      for (int i = 0; i < PER; ++i) tile[sw_t ^ swz(256u * i, RHO)] = x[i];
    }
    __syncthreads();
    for (uint32_t si = 0; si < nsubs; ++si) {
      const SubstageDev &S = subs[si];
      uint32_t srow = 0;
#pragma unroll
      for (int b = 0; b < 8; ++b)
        if ((row >> b) & 1) srow ^= S.rowsw[b];
      const uint32_t o1 = S.op_end;
      uint32_t o = S.op_begin;
      uint32_t lx = 0;  // swaps folded into the load addresses (kind 4, first in the list)
      for (; o < o1 && ops[o].kind == 4; ++o) {
        const SubOpDev &op = ops[o];
        if ((base & op.gctrl) == op.gctrl && (row & op.tctrl) == op.tctrl) lx ^= op.sdelta;
      }
      C v[1 << R];
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) v[j] = tile[srow ^ lx ^ S.soff[j]];
      uint32_t sx = 0;  // swaps folded into the store addresses (kind 3)
      for (; o < o1; ++o) {
        const SubOpDev &op = ops[o];
        if ((base & op.gctrl) != op.gctrl) continue;
        if ((row & op.tctrl) != op.tctrl) continue;
        if (op.kind == 3) {
          sx ^= op.sdelta;
          continue;
        }
        reg_apply<T, R>(v, op, pool + op.mat, row, base);
      }
      srow ^= sx;
#pragma unroll
      for (int j = 0; j < (1 << R); ++j) tile[srow ^ S.soff[j]] = v[j];
      __syncthreads();
    }
    if constexpr (sizeof(T) == 4) {
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const uint32_t p = (threadIdx.x + i * 256u) << 1;
        const uint32_t sp = sw_t ^ swz(512u * i, RHO);
        const float2 a = tile[sp], b = tile[sp ^ 1u];
        __stcs(reinterpret_cast<float4 *>(psi + base + segoff[p >> A.m] + (p & mask)), make_float4(a.x, a.y, b.x, b.y));
      }
    } else {
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const uint32_t p = threadIdx.x + i * 256u;
        __stcs(psi + base + segoff[p >> A.m] + (p & mask), tile[sw_t ^ swz(256u * i, RHO)]);
      }
    }
    __syncthreads();
  }
}

// ---- packed-pair kernel (complex64; stage.hpp: build_substages_pk) --------
// Each thread holds 16 pairs of amplitudes as RE[jj] = (Re a, Re a'),
// IM[jj] = (Im a, Im a'), the two amplitudes of a pair differing only in the
// stage's pack bit, which no operation touches.  Every operation therefore
// treats both halves alike and runs on packed f32x2 FMAs (one instruction per
// two amplitudes).  Shared memory holds the tile as two arrays of pairs,
// one 16-byte element per pair, tp[s(q)] = (RE, IM); descriptors, offset tables, matrices (entries as broadcast
// pairs (x, x), (y, y), (-y, -y)) and diagonal tables live in shared memory
// too and are read with warp-broadcast 16-byte loads.
namespace pk {

// A pair of floats lives in one 64-bit register pair (low half = the
// amplitude with pack bit 0), and the packed FMAs take it as one .b64
// operand: with float2 (two separate 32-bit values) the compiler re-paired
// the halves around every packed instruction (two integer-pipe moves per
// 64-bit value per operation, measured).
using f2 = unsigned long long;
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 neg2(f2 a) { return a ^ 0x8000000080000000ull; }  // both halves' signs
__device__ __forceinline__ f2 pack2(float lo, float hi) {
  f2 d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
__device__ __forceinline__ float lo2(f2 a) { return __uint_as_float(uint32_t(a)); }
__device__ __forceinline__ float hi2(f2 a) { return __uint_as_float(uint32_t(a >> 32)); }

__device__ __forceinline__ uint32_t swz(uint32_t q) { return q ^ (((q >> 3) ^ (q >> 6) ^ (q >> 9)) & 7u); }

// Dense 1-qubit operation on register pair-bit B; M = X00 X01 X10 X11,
// Y00 Y01 Y10 Y11, N00 N01 N10 N11 (N = -Y), each a broadcast pair.
template <int B, int CLS, bool MASKED>
__device__ __forceinline__ void dense1(f2 (&RE)[16], f2 (&IM)[16], const f2 *__restrict__ M, uint32_t amask) {
  f2 X00, X01, X10, X11, Y00, Y01, Y10, Y11, N00, N01, N10, N11;
  X00 = M[0]; X01 = M[1]; X10 = M[2]; X11 = M[3];
  if constexpr (CLS != 1) {
    Y00 = M[4]; Y01 = M[5]; Y10 = M[6]; Y11 = M[7];
    // -Y as negated operands (free in the packed FMA): fewer live registers
    N00 = neg2(Y00); N01 = neg2(Y01); N10 = neg2(Y10); N11 = neg2(Y11);
  }
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    if ((j >> B) & 1) continue;
    constexpr int D = 1 << B;
    const int k = j + D;
    const f2 ar = RE[j], ai = IM[j], br = RE[k], bi = IM[k];
    f2 a_r, a_i, b_r, b_i;
    if constexpr (CLS == 1) {  // real
      a_r = fma2(X00, ar, mul2(X01, br));
      a_i = fma2(X00, ai, mul2(X01, bi));
      b_r = fma2(X10, ar, mul2(X11, br));
      b_i = fma2(X10, ai, mul2(X11, bi));
    } else if constexpr (CLS == 2) {  // real diagonal, imaginary off-diagonal (Rx)
      a_r = fma2(X00, ar, mul2(N01, bi));
      a_i = fma2(X00, ai, mul2(Y01, br));
      b_r = fma2(X11, br, mul2(N10, ai));
      b_i = fma2(X11, bi, mul2(Y10, ar));
    } else if constexpr (CLS == 4) {  // anti-diagonal
      a_r = fma2(X01, br, mul2(N01, bi));
      a_i = fma2(X01, bi, mul2(Y01, br));
      b_r = fma2(X10, ar, mul2(N10, ai));
      b_i = fma2(X10, ai, mul2(Y10, ar));
    } else {  // general complex
      a_r = fma2(X00, ar, fma2(N00, ai, fma2(X01, br, mul2(N01, bi))));
      a_i = fma2(X00, ai, fma2(Y00, ar, fma2(X01, bi, mul2(Y01, br))));
      b_r = fma2(X10, ar, fma2(N10, ai, fma2(X11, br, mul2(N11, bi))));
      b_i = fma2(X10, ai, fma2(Y10, ar, fma2(X11, bi, mul2(Y11, br))));
    }
    if constexpr (MASKED) {  // pairs outside the register controls keep their values (selects, no branches)
      const bool c = (amask >> j) & 1u;
      RE[j] = c ? a_r : ar;
      IM[j] = c ? a_i : ai;
      RE[k] = c ? b_r : br;
      IM[k] = c ? b_i : bi;
    } else {
      RE[j] = a_r;
      IM[j] = a_i;
      RE[k] = b_r;
      IM[k] = b_i;
    }
  }
}

// a <-> b in place: three XORs through PTX, so both keep their registers
__device__ __forceinline__ void xswap(f2 &a, f2 &b) {
  asm("xor.b64 %0, %0, %1;\n\txor.b64 %1, %1, %0;\n\txor.b64 %0, %0, %1;" : "+l"(a), "+l"(b));
}

// X on register pair-bit B for the pairs whose register controls C (a
// compile-time mask over the register index) are all set: a fixed exchange
// of those pairs only (selects over every pair, with the mask at run time,
// cost about 1.5x as many instructions).
template <int B, int C>
__device__ __forceinline__ void swapc(f2 (&RE)[16], f2 (&IM)[16]) {
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    if (((j >> B) & 1) || (j & C) != C) continue;
    const int k = j + (1 << B);
    // in place (XOR exchange through PTX): each register keeps its
    // allocation, where a renaming swap leaves the dispatch merge to move
    // them back (ptxas: 1 KB of spills)
    xswap(RE[j], RE[k]);
    xswap(IM[j], IM[k]);
  }
}

// Register-controlled X on bit B by its control mask: the eight subsets of
// the other three register bits.
template <int B>
__device__ __forceinline__ void swap_ctl(f2 (&RE)[16], f2 (&IM)[16], uint32_t cmask) {
  constexpr int O0 = B == 0 ? 2 : 1, O1 = B <= 1 ? 4 : 2, O2 = B <= 2 ? 8 : 4;  // the other bits
  switch (cmask) {
    case 0: swapc<B, 0>(RE, IM); break;
    case O0: swapc<B, O0>(RE, IM); break;
    case O1: swapc<B, O1>(RE, IM); break;
    case O2: swapc<B, O2>(RE, IM); break;
    case O0 | O1: swapc<B, O0 | O1>(RE, IM); break;
    case O0 | O2: swapc<B, O0 | O2>(RE, IM); break;
    case O1 | O2: swapc<B, O1 | O2>(RE, IM); break;
    default: swapc<B, O0 | O1 | O2>(RE, IM); break;
  }
}

// (RE, IM) *= F with F = Fx + i Fy per half: RE' = Fx RE - Fy IM, IM' = Fx IM + Fy RE
__device__ __forceinline__ void cmul(f2 &re, f2 &im, f2 fx, f2 fy, f2 fn) {
  // both products first: each output's last instruction is then the last use
  // of its own input, and the result stays in that input's registers (with
  // the other order ptxas moved about 20 registers per diagonal operation at
  // the dispatch merge, and the kernel spilled)
  const f2 t1 = mul2(fn, im), t2 = mul2(fy, re);
  re = fma2(fx, re, t1);
  im = fma2(fx, im, t2);
}

template <int B>
__device__ __forceinline__ void diag1(f2 (&RE)[16], f2 (&IM)[16], const ulonglong2 *e0, const ulonglong2 *e1) {
  const ulonglong2 a0 = e0[0], b0 = e0[1], a1 = e1[0], b1 = e1[1];
  const f2 x0 = a0.x, y0 = a0.y, n0 = b0.x;
  const f2 x1 = a1.x, y1 = a1.y, n1 = b1.x;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    if ((j >> B) & 1) cmul(RE[j], IM[j], x1, y1, n1);
    else cmul(RE[j], IM[j], x0, y0, n0);
  }
}

// Diagonal whose register qubits are the register pair-bits in MASK: for
// each value e of those bits, the table entry cidx | jidx[e] (jidx depends on
// the masked bits only) multiplies every pair whose masked bits equal e.
template <int MASK>
__device__ __forceinline__ void diagm(f2 (&RE)[16], f2 (&IM)[16], const ulonglong2 *T, const uint8_t *jidx,
                                      uint32_t cidx) {
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    if (e & ~MASK) continue;  // e runs over the values of the masked bits
    const uint32_t idx = cidx | jidx[e];
    const ulonglong2 a = T[2 * idx], b = T[2 * idx + 1];
#pragma unroll
    for (int j = 0; j < 16; ++j)
      if ((j & MASK) == e) cmul(RE[j], IM[j], a.x, a.y, b.x);
  }
}

template <int B, int CLS>
__device__ __forceinline__ void dense1_m(f2 (&RE)[16], f2 (&IM)[16], const f2 *M, uint32_t amask, bool masked) {
  if (masked) dense1<B, CLS, true>(RE, IM, M, amask);
  else dense1<B, CLS, false>(RE, IM, M, amask);
}

template <int B>
__device__ __forceinline__ void dense1_cls(f2 (&RE)[16], f2 (&IM)[16], const f2 *M, uint32_t amask, uint32_t cls,
                                           bool masked) {
  switch (cls) {
    case 1: dense1_m<B, 1>(RE, IM, M, amask, masked); break;
    case 2: dense1_m<B, 2>(RE, IM, M, amask, masked); break;
    case 4: dense1_m<B, 4>(RE, IM, M, amask, masked); break;
    default: dense1_m<B, 0>(RE, IM, M, amask, masked); break;
  }
}

__device__ __forceinline__ void apply_op(f2 (&RE)[16], f2 (&IM)[16], const unsigned char *__restrict__ blob,
                                         const PkOpDev &op, uint32_t code, uint32_t row, uint64_t base,
                                         uint32_t &sx) {
  const uint32_t kind = code & 15u, B = (code >> 4) & 15u;
  if (kind <= kPkSwap) {  // dense or swap on register pair-bit B: one indexed branch
    const f2 *M = reinterpret_cast<const f2 *>(blob + op.data);
    const uint32_t cls = (code >> 8) & 15u;
    const bool masked = (code >> 12) & 1u;
    switch (kind * 4 + B) {
      case 0: dense1_cls<0>(RE, IM, M, op.amask, cls, masked); break;
      case 1: dense1_cls<1>(RE, IM, M, op.amask, cls, masked); break;
      case 2: dense1_cls<2>(RE, IM, M, op.amask, cls, masked); break;
      case 3: dense1_cls<3>(RE, IM, M, op.amask, cls, masked); break;
      case 4: swap_ctl<0>(RE, IM, cls); break;  // cls: the swap's register controls
      case 5: swap_ctl<1>(RE, IM, cls); break;
      case 6: swap_ctl<2>(RE, IM, cls); break;
      default: swap_ctl<3>(RE, IM, cls); break;
    }
    return;
  }
  if (kind == kPkStoreXor) {
    sx ^= op.amask;
    return;
  }
  // diagonal: table index bits of the row and non-local qubits
  uint32_t cidx = 0;
  const uint32_t nsrc = op.nsrc;  // at most 6: a merged diagonal spans at most 6 qubits
#pragma unroll
  for (uint32_t i = 0; i < 6; ++i) {
    if (i >= nsrc) break;
    const uint32_t sidx = op.src[i];
    const uint32_t bit = (sidx & 0x80u) ? uint32_t((base >> (sidx & 0x7Fu)) & 1u) : (row >> sidx) & 1u;
    cidx |= bit << op.sbit[i];
  }
  const ulonglong2 *T = reinterpret_cast<const ulonglong2 *>(blob + op.data);  // 32-byte entries
  if (kind == kPkDiag0) {
    const ulonglong2 a = T[2 * cidx], b = T[2 * cidx + 1];
    const f2 x = a.x, y = a.y, n = b.x;
#pragma unroll
    for (int j = 0; j < 16; ++j) cmul(RE[j], IM[j], x, y, n);
    return;
  }
  if (kind == kPkDiag1) {
    const ulonglong2 *e0 = T + 2 * cidx, *e1 = T + 2 * (cidx | (1u << op.dq));
    switch (B) {
      case 0: diag1<0>(RE, IM, e0, e1); break;
      case 1: diag1<1>(RE, IM, e0, e1); break;
      case 2: diag1<2>(RE, IM, e0, e1); break;
      default: diag1<3>(RE, IM, e0, e1); break;
    }
    return;
  }
  // several register qubits, register-bit mask B (2 to 4 bits): one table
  // entry per value of those bits, loaded once for all pairs sharing it
  switch (B) {
    case 3: diagm<3>(RE, IM, T, op.jidx, cidx); break;
    case 5: diagm<5>(RE, IM, T, op.jidx, cidx); break;
    case 6: diagm<6>(RE, IM, T, op.jidx, cidx); break;
    case 9: diagm<9>(RE, IM, T, op.jidx, cidx); break;
    case 10: diagm<10>(RE, IM, T, op.jidx, cidx); break;
    case 12: diagm<12>(RE, IM, T, op.jidx, cidx); break;
    case 7: diagm<7>(RE, IM, T, op.jidx, cidx); break;
    case 11: diagm<11>(RE, IM, T, op.jidx, cidx); break;
    case 13: diagm<13>(RE, IM, T, op.jidx, cidx); break;
    case 14: diagm<14>(RE, IM, T, op.jidx, cidx); break;
    default: diagm<15>(RE, IM, T, op.jidx, cidx); break;
  }
}

}  // namespace pk

__global__ void __launch_bounds__(256, 2) stage_pk_kernel(float2 *__restrict__ psi, const __grid_constant__ StageArgs A,
                                                          const unsigned char *__restrict__ blob_src,
                                                          uint32_t blob_bytes, uint32_t nsubs, uint32_t P) {
  using pk::f2;
  extern __shared__ __align__(16) unsigned char smem[];
  ulonglong2 *tp = reinterpret_cast<ulonglong2 *>(smem);  // tp[s(q)] = (RE, IM) of pair q
  uint64_t *segoff = reinterpret_cast<uint64_t *>(smem + 65536);
  const uint32_t nseg = 1u << A.h;
  unsigned char *blob = smem + 65536 + ((nseg * 8 + 15) & ~15u);
  for (uint32_t s = threadIdx.x; s < nseg; s += blockDim.x) {
    uint64_t o = 0;
    for (uint32_t b = 0; b < A.h; ++b)
      if ((s >> b) & 1) o |= uint64_t(1) << A.lpos[A.m + b];
    segoff[s] = o;
  }
  for (uint32_t i = threadIdx.x; i < blob_bytes / 16; i += blockDim.x)
    reinterpret_cast<uint4 *>(blob)[i] = reinterpret_cast<const uint4 *>(blob_src)[i];
  __syncthreads();
  const PkSubDev *subs = reinterpret_cast<const PkSubDev *>(blob);
  const PkOpDev *ops = reinterpret_cast<const PkOpDev *>(blob + ((nsubs * sizeof(PkSubDev) + 15) & ~15u));
  const uint32_t row = threadIdx.x;
  const uint32_t rmask = (1u << A.m) - 1;
  // The first tile is loaded here; each later tile's loads are issued in the
  // same loop that writes the previous tile back (every shared-memory slot
  // is read, written to HBM and refilled by one thread), so their latency
  // overlaps the stores and one barrier per tile goes.
  uint64_t t = blockIdx.x;
  uint64_t base = t < A.ntiles ? insert_zeros(t, A.lpos, int(A.L)) : 0;
  if (t < A.ntiles) {
    // HBM -> shared memory: pairs along P (tile position p = q with bit P inserted)
    if (P == 0) {
      float4 x[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const uint32_t p = (threadIdx.x + 256u * i) << 1;
        x[i] = __ldcs(reinterpret_cast<const float4 *>(psi + base + segoff[p >> A.m] + (p & rmask)));
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const uint32_t sq = pk::swz(threadIdx.x + 256u * i);
        tp[sq] = make_ulonglong2(pk::pack2(x[i].x, x[i].z), pk::pack2(x[i].y, x[i].w));
      }
    } else {
      float4 x[8], y[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const uint32_t q = (threadIdx.x + 256u * i) << 1;
        const uint32_t p0 = ((q >> P) << (P + 1)) | (q & ((1u << P) - 1)), p1 = p0 | (1u << P);
        x[i] = __ldcs(reinterpret_cast<const float4 *>(psi + base + segoff[p0 >> A.m] + (p0 & rmask)));
        y[i] = __ldcs(reinterpret_cast<const float4 *>(psi + base + segoff[p1 >> A.m] + (p1 & rmask)));
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const uint32_t q = (threadIdx.x + 256u * i) << 1;
        const uint32_t s0 = pk::swz(q), s1 = pk::swz(q + 1);
        tp[s0] = make_ulonglong2(pk::pack2(x[i].x, y[i].x), pk::pack2(x[i].y, y[i].y));
        tp[s1] = make_ulonglong2(pk::pack2(x[i].z, y[i].z), pk::pack2(x[i].w, y[i].w));
      }
    }
  }
  __syncthreads();
  while (t < A.ntiles) {
    for (uint32_t si = 0; si < nsubs; ++si) {
      const PkSubDev S = subs[si];
      const uint32_t *tab = reinterpret_cast<const uint32_t *>(blob + S.tab);
      const uint32_t srow = tab[row];
      uint32_t o = S.op_begin;
      uint32_t lx = 0;
      for (; o < S.op_end; ++o) {
        const PkOpDev &op = ops[o];
        if (op.code != kPkLoadXor) break;
        if ((base & op.gctrl) == op.gctrl && (row & op.tctrl) == op.tctrl) lx ^= op.amask;
      }
      f2 RE[16], IM[16];
      {
        const uint4 *lt = reinterpret_cast<const uint4 *>(tab + 256);
        const uint32_t a0 = srow ^ lx;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          const uint4 l = lt[g];
          const uint32_t off[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const uint32_t a = a0 ^ off[e];
            const ulonglong2 v = tp[a];
            RE[4 * g + e] = v.x;
            IM[4 * g + e] = v.y;
          }
        }
      }
      uint32_t sx = 0;
      for (; o < S.op_end; ++o) {
        const PkOpDev &op = ops[o];
        const uint32_t code = op.code;
        // controls are tested only for operations that have them
        if ((code & kPkCtl) && !((base & op.gctrl) == op.gctrl && (row & op.tctrl) == op.tctrl)) continue;
        pk::apply_op(RE, IM, blob, op, code, row, base, sx);
      }
      {
        const uint4 *st = reinterpret_cast<const uint4 *>(tab + 272);
        const uint32_t a0 = srow ^ sx;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          const uint4 l = st[g];
          const uint32_t off[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const uint32_t a = a0 ^ off[e];
            tp[a] = make_ulonglong2(RE[4 * g + e], IM[4 * g + e]);
          }
        }
      }
      __syncthreads();
    }
    // shared memory -> HBM, and the next tile's loads into the same slots
    const uint64_t tn = t + gridDim.x;
    const bool more = tn < A.ntiles;
    // past the last tile the loads re-read the current tile (valid addresses,
    // the data is never used): no conditional around them
    const uint64_t bn = more ? insert_zeros(tn, A.lpos, int(A.L)) : base;
    if (P == 0) {
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {  // two halves: 8 loads in flight per thread, fewer live registers
        asm volatile("" ::: "memory");  // keep the second half's loads after the first half's stores
        float4 x[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const uint32_t p = (threadIdx.x + 256u * (i + 8 * h)) << 1;
          x[i] = __ldcs(reinterpret_cast<const float4 *>(psi + bn + segoff[p >> A.m] + (p & rmask)));
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const uint32_t q = threadIdx.x + 256u * (i + 8 * h), p = q << 1;
          const uint32_t sq = pk::swz(q);
          const ulonglong2 v = tp[sq];
          const f2 r = v.x, m = v.y;
          __stcs(reinterpret_cast<float4 *>(psi + base + segoff[p >> A.m] + (p & rmask)),
                 make_float4(pk::lo2(r), pk::lo2(m), pk::hi2(r), pk::hi2(m)));
          tp[sq] = make_ulonglong2(pk::pack2(x[i].x, x[i].z), pk::pack2(x[i].y, x[i].w));
        }
      }
    } else {
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        asm volatile("" ::: "memory");
        float4 x[4], y[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const uint32_t q = (threadIdx.x + 256u * (i + 4 * h)) << 1;
          const uint32_t p0 = ((q >> P) << (P + 1)) | (q & ((1u << P) - 1)), p1 = p0 | (1u << P);
          x[i] = __ldcs(reinterpret_cast<const float4 *>(psi + bn + segoff[p0 >> A.m] + (p0 & rmask)));
          y[i] = __ldcs(reinterpret_cast<const float4 *>(psi + bn + segoff[p1 >> A.m] + (p1 & rmask)));
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const uint32_t q = (threadIdx.x + 256u * (i + 4 * h)) << 1;
          const uint32_t p0 = ((q >> P) << (P + 1)) | (q & ((1u << P) - 1)), p1 = p0 | (1u << P);
          const uint32_t s0 = pk::swz(q), s1 = pk::swz(q + 1);
          const ulonglong2 v0 = tp[s0], v1 = tp[s1];
          const f2 r0 = v0.x, m0 = v0.y, r1 = v1.x, m1 = v1.y;
          __stcs(reinterpret_cast<float4 *>(psi + base + segoff[p0 >> A.m] + (p0 & rmask)),
                 make_float4(pk::lo2(r0), pk::lo2(m0), pk::lo2(r1), pk::lo2(m1)));
          __stcs(reinterpret_cast<float4 *>(psi + base + segoff[p1 >> A.m] + (p1 & rmask)),
                 make_float4(pk::hi2(r0), pk::hi2(m0), pk::hi2(r1), pk::hi2(m1)));
          tp[s0] = make_ulonglong2(pk::pack2(x[i].x, y[i].x), pk::pack2(x[i].y, y[i].y));
          tp[s1] = make_ulonglong2(pk::pack2(x[i].z, y[i].z), pk::pack2(x[i].w, y[i].w));
        }
      }
    }
    __syncthreads();
    t = tn;
    base = bn;
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
  // set on every launch: attributes belong to the current device, and the
  // call is cheap next to a pass over the state
  cudaError_t ae = cudaFuncSetAttribute(stage_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
  if (ae != cudaSuccess) return ae;
  if constexpr (sizeof(T) == 4) {
    if (!plan.pk.empty()) {
      // Packed-pair substages: d_ops holds the blob (stage.hpp, build_substages_pk).
      // runs of at least 2^5 amplitudes: 16-byte aligned loads, at most 2^8 segments
      if (plan.L != kPkTileBits || plan.pack < 0 || A.m < 5 || plan.pk.size() % 16 || plan.pk.size() > kPkBlobMax)
        return cudaErrorInvalidValue;
      const size_t smem_pk = 65536 + (((size_t(1) << A.h) * 8 + 15) & ~size_t(15)) + plan.pk.size();
      ae = cudaFuncSetAttribute(stage_pk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 65536 + 2048 + int(kPkBlobMax));
      if (ae != cudaSuccess) return ae;
      int per_sm = 1;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stage_pk_kernel, 256, smem_pk);
      per_sm = std::max(1, per_sm);
      const uint64_t grid = std::min<uint64_t>(A.ntiles, uint64_t(stage_sms()) * per_sm);
      stage_pk_kernel<<<unsigned(grid), 256, smem_pk, s>>>(static_cast<float2 *>(psi), A,
                                                           static_cast<const unsigned char *>(d_ops),
                                                           uint32_t(plan.pk.size()), plan.pk_nsubs,
                                                           uint32_t(plan.pack));
      return cudaGetLastError();
    }
  }
  if (!plan.subs.empty()) {
    // Register substages: d_ops holds the table [SubstageDev...][SubOpDev...][pool].
    constexpr int R = sizeof(T) == 4 ? int(kRegBitsC64) : int(kRegBitsC128);
    if (plan.r != unsigned(R) || plan.L != unsigned(R) + 8 || plan.rho != (sizeof(T) == 4 ? 4u : 3u))
      return cudaErrorInvalidValue;
    const uint32_t sops_off = uint32_t(stage_subs_bytes(plan));
    const uint32_t pool_off = sops_off + uint32_t((plan.sops.size() * sizeof(SubOpDev) + 15) / 16 * 16);
    const uint32_t pool_bytes = uint32_t((plan.pool.size() * sizeof(cplx_t<T>) + 15) / 16 * 16);
    if (sops_off + plan.sops.size() * sizeof(SubOpDev) > kStageTableBytes) return cudaErrorInvalidValue;
    thread_local StageTable tb;  // host staging of the kernel parameter (copied at launch)
    std::memcpy(tb.bytes, plan.subs.data(), plan.subs.size() * sizeof(SubstageDev));
    std::memcpy(tb.bytes + sops_off, plan.sops.data(), plan.sops.size() * sizeof(SubOpDev));
    const size_t smem_reg = (size_t(1) << A.L) * sizeof(cplx_t<T>) + (((size_t(1) << A.h) * 8 + 15) & ~size_t(15)) +
                            pool_bytes;
    if (smem_reg > 200 * 1024) return cudaErrorInvalidValue;
    ae = cudaFuncSetAttribute(stage_reg_kernel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (ae != cudaSuccess) return ae;
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stage_reg_kernel<T, R>, 256, smem_reg);
    per_sm = std::max(1, per_sm);
    const uint64_t grid = std::min<uint64_t>(A.ntiles, uint64_t(stage_sms()) * per_sm);
    stage_reg_kernel<T, R><<<unsigned(grid), 256, smem_reg, s>>>(
        static_cast<cplx_t<T> *>(psi), A, tb, static_cast<const unsigned char *>(d_ops) + pool_off,
        uint32_t(plan.subs.size()), sops_off, pool_bytes, plan.rho);
    return cudaGetLastError();
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
