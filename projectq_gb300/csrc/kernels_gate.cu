// Controlled dense k-qubit gate kernels (k = 1..5) for the GB300 simulator.
//
// Semantics follow the reference kernels (projectq/backends/_sim/_cppkernels/
// nointrin/kernel{1..5}.hpp): for every base index I whose target bits are 0
// and whose control bits are 1, v = psi[I + subsets of targets] and
// psi[...] <- M v.  The design is GB300-first, not a translation:
//  - each thread owns whole amplitude groups, found by inserting the target
//    (0) and control (1) bits into a compact unit index, so controls cost no
//    bandwidth: only the 2^(N-c) controlled amplitudes are touched;
//  - the matrix travels in the kernel's parameter space (constant bank,
//    broadcast to every lane), together with per-entry kinds (zero / real /
//    imaginary / complex) and identity-row masks, so diagonal and monomial
//    gates (Z, S, T, Rz, X, CNOT, Toffoli, CZ...) load and store only the
//    amplitudes they change and spend no FLOPs on zero entries — this matters
//    for the complex128 path, which is FP64-bound on GB300;
//  - complex64 groups whose lowest bit is free are processed two adjacent
//    groups per thread with 16-byte (float4) loads and stores.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <stdexcept>

#include "common.cuh"
#include "kernels.hpp"

namespace gsim {

template <typename T, int K>
struct DenseParams {
  static constexpr int D = 1 << K;
  cplx_t<T> m[D * D];
  uint64_t off[D];
  uint64_t units;
  uint64_t ctrl_set;
  uint32_t rowmask;
  uint32_t loadmask;
  int nins;
  uint8_t kind[D * D];  // 0 zero, 1 real, 2 imaginary, 3 complex
  uint8_t ins[64];      // ascending insert positions (targets and controls)
};

template <typename T>
__device__ __forceinline__ void cmac(int kd, cplx_t<T> m, T vr, T vi, T &re, T &im) {
  if (kd == 1) {
    re = fma(m.x, vr, re);
    im = fma(m.x, vi, im);
  } else if (kd == 2) {
    re = fma(-m.y, vi, re);
    im = fma(m.y, vr, im);
  } else if (kd == 3) {
    re = fma(m.x, vr, re);
    re = fma(-m.y, vi, re);
    im = fma(m.x, vi, im);
    im = fma(m.y, vr, im);
  }
}

template <typename T, int K>
__global__ void __launch_bounds__(256) dense_kernel(cplx_t<T> *__restrict__ psi,
                                                    const __grid_constant__ DenseParams<T, K> P) {
  constexpr int D = 1 << K;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < P.units; u += stride) {
    const uint64_t base = insert_zeros(u, P.ins, P.nins) | P.ctrl_set;
    cplx_t<T> v[D];
#pragma unroll
    for (int j = 0; j < D; ++j)
      v[j] = ((P.loadmask >> j) & 1) ? psi[base + P.off[j]] : mkc<T>(T(0), T(0));
#pragma unroll
    for (int r = 0; r < D; ++r) {
      if (!((P.rowmask >> r) & 1)) continue;
      T re = T(0), im = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) cmac<T>(P.kind[r * D + j], P.m[r * D + j], v[j].x, v[j].y, re, im);
      psi[base + P.off[r]] = mkc<T>(re, im);
    }
  }
}

// complex64, lowest bit free: each unit is two adjacent groups (16-byte I/O).
template <int K>
__global__ void __launch_bounds__(256) dense_kernel_vec2(float2 *__restrict__ psi,
                                                         const __grid_constant__ DenseParams<float, K> P) {
  constexpr int D = 1 << K;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < P.units; u += stride) {
    const uint64_t base = insert_zeros(u << 1, P.ins, P.nins) | P.ctrl_set;
    float4 v[D];
#pragma unroll
    for (int j = 0; j < D; ++j)
      v[j] = ((P.loadmask >> j) & 1) ? *reinterpret_cast<const float4 *>(psi + base + P.off[j])
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int r = 0; r < D; ++r) {
      if (!((P.rowmask >> r) & 1)) continue;
      float r0 = 0.f, i0 = 0.f, r1 = 0.f, i1 = 0.f;
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const int kd = P.kind[r * D + j];
        cmac<float>(kd, P.m[r * D + j], v[j].x, v[j].y, r0, i0);
        cmac<float>(kd, P.m[r * D + j], v[j].z, v[j].w, r1, i1);
      }
      *reinterpret_cast<float4 *>(psi + base + P.off[r]) = make_float4(r0, i0, r1, i1);
    }
  }
}

// Wide gates (k = 6, 7 targets, or any k): a CTA gathers whole amplitude
// groups into shared memory, then each thread computes one output row of one
// group, reading the matrix row from global memory (L1/L2 resident; 2^k x 2^k
// complex).  Used for gates wider than the register kernels handle.
struct WideArgs {
  uint64_t units;      // number of groups
  uint64_t ctrl_set;
  int nins, k;         // insert count, targets
  uint8_t ins[64];
  uint64_t off[128];   // offset of matrix index j
};

// Gates of k >= 5 targets on CUDA cores.  A block has D = 2^k threads, one per
// output row r, and takes kWideGroups amplitude groups at a time: the groups
// are gathered into shared memory, then every thread walks the columns j
// reading U^T[j][r] (consecutive r: coalesced, and reused for all the
// groups) and the group inputs x[g][j] (shared-memory broadcasts).
constexpr int kWideGroups = 8;

template <typename T>
__global__ void __launch_bounds__(128) wide_kernel(cplx_t<T> *__restrict__ psi, const cplx_t<T> *__restrict__ Ut,
                                                   const __grid_constant__ WideArgs A) {
  extern __shared__ __align__(16) unsigned char smem_w[];
  cplx_t<T> *buf = reinterpret_cast<cplx_t<T> *>(smem_w);
  const int D = 1 << A.k;
  const int r = threadIdx.x;  // blockDim.x == D
  for (uint64_t g0 = uint64_t(blockIdx.x) * kWideGroups; g0 < A.units;
       g0 += uint64_t(gridDim.x) * kWideGroups) {
    uint64_t base[kWideGroups];
#pragma unroll
    for (int g = 0; g < kWideGroups; ++g) {
      const uint64_t gg = g0 + uint64_t(g);
      base[g] = gg < A.units ? (insert_zeros(gg, A.ins, A.nins) | A.ctrl_set) : 0;
      buf[g * D + r] = gg < A.units ? psi[base[g] + A.off[r]] : mkc<T>(T(0), T(0));
    }
    __syncthreads();
    T re[kWideGroups], im[kWideGroups];
#pragma unroll
    for (int g = 0; g < kWideGroups; ++g) re[g] = im[g] = T(0);
    for (int j = 0; j < D; ++j) {
      const cplx_t<T> m = __ldg(Ut + size_t(j) * D + r);
#pragma unroll
      for (int g = 0; g < kWideGroups; ++g) {
        const cplx_t<T> x = buf[g * D + j];
        re[g] = fma(m.x, x.x, fma(-m.y, x.y, re[g]));
        im[g] = fma(m.x, x.y, fma(m.y, x.x, im[g]));
      }
    }
#pragma unroll
    for (int g = 0; g < kWideGroups; ++g)
      if (g0 + uint64_t(g) < A.units) psi[base[g] + A.off[r]] = mkc<T>(re[g], im[g]);
    __syncthreads();
  }
}

namespace {

int g_num_sms = 0;
int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

unsigned grid_for(uint64_t units, int threads, int per_sm) {
  uint64_t want = (units + threads - 1) / threads;
  uint64_t cap = uint64_t(num_sms()) * per_sm;
  return unsigned(std::max<uint64_t>(1, std::min(want, cap)));
}

template <typename T, int K>
cudaError_t launch_dense_k(T *, void *psi, unsigned nq, const DenseOp &op, cudaStream_t s) {
  constexpr int D = 1 << K;
  DenseParams<T, K> P;
  std::memset(&P, 0, sizeof(P));
  // Sorted insert positions (targets then controls merged).
  std::vector<unsigned> ins(op.pos.begin(), op.pos.end());
  for (unsigned b = 0; b < 64; ++b)
    if ((op.ctrl_mask >> b) & 1) ins.push_back(b);
  std::sort(ins.begin(), ins.end());
  if (ins.size() > nq) throw std::invalid_argument("gate wider than the state");
  P.nins = int(ins.size());
  for (size_t i = 0; i < ins.size(); ++i) P.ins[i] = uint8_t(ins[i]);
  P.ctrl_set = op.ctrl_mask;
  for (int j = 0; j < D; ++j) {
    uint64_t o = 0;
    for (int l = 0; l < K; ++l)
      if ((j >> l) & 1) o |= uint64_t(1) << op.pos[l];
    P.off[j] = o;
  }
  uint32_t rowmask = 0, loadmask = 0;
  for (int r = 0; r < D; ++r) {
    bool ident = true;
    for (int j = 0; j < D; ++j) {
      const cplx z = op.m[size_t(r) * D + j];
      const cplx e = (r == j) ? cplx(1., 0.) : cplx(0., 0.);
      if (z != e) ident = false;
    }
    if (!ident) rowmask |= 1u << r;
  }
  for (int r = 0; r < D; ++r) {
    for (int j = 0; j < D; ++j) {
      const cplx z = op.m[size_t(r) * D + j];
      const T re = T(z.real()), im = T(z.imag());
      P.m[r * D + j] = mkc<T>(re, im);
      uint8_t kd = (re != T(0) ? 1 : 0) | (im != T(0) ? 2 : 0);
      P.kind[r * D + j] = kd;
      if (((rowmask >> r) & 1) && kd) loadmask |= 1u << j;
    }
  }
  P.rowmask = rowmask;
  P.loadmask = loadmask;
  if (rowmask == 0) return cudaSuccess;  // identity on the controlled subspace
  const unsigned free_bits = nq - unsigned(ins.size());
  const bool vec2 = sizeof(T) == 4 && K <= 4 && free_bits >= 1 && ins[0] != 0;
  if (vec2) {
    P.units = uint64_t(1) << (free_bits - 1);
    if constexpr (sizeof(T) == 4 && K <= 4) {
      dense_kernel_vec2<K><<<grid_for(P.units, 256, 8), 256, 0, s>>>(
          reinterpret_cast<float2 *>(psi), P);
    }
  } else {
    P.units = uint64_t(1) << free_bits;
    dense_kernel<T, K><<<grid_for(P.units, 256, 8), 256, 0, s>>>(
        reinterpret_cast<cplx_t<T> *>(psi), P);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_wide_t(void *psi, unsigned nq, const DenseOp &op, const void *d_matrix, cudaStream_t s) {
  WideArgs A;
  std::memset(&A, 0, sizeof(A));
  const int k = int(op.pos.size()), D = 1 << k;
  std::vector<unsigned> ins(op.pos.begin(), op.pos.end());
  for (unsigned b = 0; b < 64; ++b)
    if ((op.ctrl_mask >> b) & 1) ins.push_back(b);
  std::sort(ins.begin(), ins.end());
  if (ins.size() > nq) throw std::invalid_argument("gate wider than the state");
  A.nins = int(ins.size());
  for (size_t i = 0; i < ins.size(); ++i) A.ins[i] = uint8_t(ins[i]);
  A.k = k;
  A.ctrl_set = op.ctrl_mask;
  for (int j = 0; j < D; ++j)
    for (int l = 0; l < k; ++l)
      if ((j >> l) & 1) A.off[j] |= uint64_t(1) << op.pos[l];
  A.units = uint64_t(1) << (nq - ins.size());
  if (k < 5 || k > 7) throw std::invalid_argument("the wide-gate kernel takes 5 to 7 targets");
  const size_t smem = size_t(kWideGroups) * D * sizeof(cplx_t<T>);
  const uint64_t blocks =
      std::min<uint64_t>((A.units + kWideGroups - 1) / kWideGroups, uint64_t(num_sms()) * (2048 / D));
  wide_kernel<T><<<unsigned(std::max<uint64_t>(1, blocks)), unsigned(D), smem, s>>>(
      static_cast<cplx_t<T> *>(psi), static_cast<const cplx_t<T> *>(d_matrix), A);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_dense_t(void *psi, unsigned nq, const DenseOp &op, cudaStream_t s) {
  T *tag = nullptr;
  switch (op.pos.size()) {
    case 1: return launch_dense_k<T, 1>(tag, psi, nq, op, s);
    case 2: return launch_dense_k<T, 2>(tag, psi, nq, op, s);
    case 3: return launch_dense_k<T, 3>(tag, psi, nq, op, s);
    case 4: return launch_dense_k<T, 4>(tag, psi, nq, op, s);
    case 5: return launch_dense_k<T, 5>(tag, psi, nq, op, s);
    default: throw std::invalid_argument("dense gate kernel supports 1..5 target qubits");
  }
}

}  // namespace

cudaError_t launch_dense(int prec, void *psi, unsigned nq, const DenseOp &op, cudaStream_t s) {
  return prec == 1 ? launch_dense_t<float>(psi, nq, op, s) : launch_dense_t<double>(psi, nq, op, s);
}

cudaError_t launch_wide(int prec, void *psi, unsigned nq, const DenseOp &op, const void *d_matrix,
                        cudaStream_t s) {
  if (op.pos.size() < 1 || op.pos.size() > 7) throw std::invalid_argument("wide gate kernel supports 1..7 targets");
  return prec == 1 ? launch_wide_t<float>(psi, nq, op, d_matrix, s) : launch_wide_t<double>(psi, nq, op, d_matrix, s);
}

}  // namespace gsim
