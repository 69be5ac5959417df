// Adjoint-method gradient support: one fused pass per gate of the reverse
// sweep over the two state vectors psi (the circuit state) and lam (H psi
// carried backwards).
//
// For gate l with target t and control mask c, over every amplitude pair
// (i0, i1 = i0 | 2^t) with the controls satisfied:
//   - if the gate is parametrised, a per-block partial of
//       Im <lam| Pi_c G |psi>     (G = X, Y, Z for Rx, Ry, Rz;
//                                  G = I for the phase Ph, |1><1| for R)
//     computed from the amplitudes before the update (FP32 products carried
//     in FP64 for complex64, FP64 for complex128);
//   - psi <- U^dagger psi and lam <- U^dagger lam (U the gate's 2x2 matrix).
// Bytes per step: both vectors read and written once (4 x 2^(N-c) x B).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "kernels.hpp"

namespace gsim {
namespace {

struct AdjStep {
  double u[8];       // U^dagger, row-major 2x2, interleaved (re, im)
  uint64_t ctrl;     // control mask
  uint8_t ins[64];   // ascending insert positions: target and controls
  int nins;
  int target;
  int gen;           // -1 none, 0 X, 1 Y, 2 Z, 3 identity (Ph), 4 |1><1| (R)
  int col;           // output column of the partial sums
};

// (a, b) <- U^dagger (a, b) by matrix class (chosen on the host from exact
// zeros and ones of U^dagger; each class drops only terms that are exactly
// zero, so all classes give the general formula's values):
// 0 general, 1 real (Ry), 2 real diagonal / imaginary off-diagonal (Rx),
// 3 diagonal (Rz, Ph, R), 4 exact swap (X, CNOT).
template <typename T, int CLS>
__device__ __forceinline__ void mv(const AdjStep &S, cplx_t<T> &a, cplx_t<T> &b) {
  const T u00r = T(S.u[0]), u00i = T(S.u[1]), u01r = T(S.u[2]), u01i = T(S.u[3]);
  const T u10r = T(S.u[4]), u10i = T(S.u[5]), u11r = T(S.u[6]), u11i = T(S.u[7]);
  const T ar = a.x, ai = a.y, br = b.x, bi = b.y;
  if constexpr (CLS == 4) {
    a.x = br;
    a.y = bi;
    b.x = ar;
    b.y = ai;
  } else if constexpr (CLS == 3) {
    a.x = fma(u00r, ar, -u00i * ai);
    a.y = fma(u00r, ai, u00i * ar);
    b.x = fma(u11r, br, -u11i * bi);
    b.y = fma(u11r, bi, u11i * br);
  } else if constexpr (CLS == 2) {
    a.x = fma(u00r, ar, -u01i * bi);
    a.y = fma(u00r, ai, u01i * br);
    b.x = fma(u11r, br, -u10i * ai);
    b.y = fma(u11r, bi, u10i * ar);
  } else if constexpr (CLS == 1) {
    a.x = fma(u00r, ar, u01r * br);
    a.y = fma(u00r, ai, u01r * bi);
    b.x = fma(u10r, ar, u11r * br);
    b.y = fma(u10r, ai, u11r * bi);
  } else {
    a.x = fma(u00r, ar, fma(-u00i, ai, fma(u01r, br, -u01i * bi)));
    a.y = fma(u00r, ai, fma(u00i, ar, fma(u01r, bi, u01i * br)));
    b.x = fma(u10r, ar, fma(-u10i, ai, fma(u11r, br, -u11i * bi)));
    b.y = fma(u10r, ai, fma(u10i, ar, fma(u11r, bi, u11i * br)));
  }
}

// Im(conj(x) y)
template <typename T> __device__ __forceinline__ T im_cdot(cplx_t<T> x, cplx_t<T> y) {
  return fma(x.x, y.y, -x.y * y.x);
}
// Re(conj(x) y)
template <typename T> __device__ __forceinline__ T re_cdot(cplx_t<T> x, cplx_t<T> y) {
  return fma(x.x, y.x, x.y * y.y);
}

template <typename T, int CLS>
__global__ void __launch_bounds__(256) adjoint_step_kernel(cplx_t<T> *__restrict__ psi,
                                                           cplx_t<T> *__restrict__ lam, uint64_t units,
                                                           const __grid_constant__ AdjStep S,
                                                           double *part, int nblk) {
  const uint64_t d = uint64_t(1) << S.target;
  double acc = 0.;
  T mini = T(0);
  int cnt = 0;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < units; u += stride) {
    const uint64_t i0 = insert_zeros(u, S.ins, S.nins) | S.ctrl, i1 = i0 + d;
    cplx_t<T> b0 = psi[i0], b1 = psi[i1], a0 = lam[i0], a1 = lam[i1];
    if (S.gen >= 0) {
      T v;
      switch (S.gen) {
        case 0: v = im_cdot<T>(a0, b1) + im_cdot<T>(a1, b0); break;                  // X
        case 1: v = -re_cdot<T>(a0, b1) + re_cdot<T>(a1, b0); break;                 // Y: Im(-i c01 + i c10)
        case 2: v = im_cdot<T>(a0, b0) - im_cdot<T>(a1, b1); break;                  // Z
        case 3: v = im_cdot<T>(a0, b0) + im_cdot<T>(a1, b1); break;                  // identity
        default: v = im_cdot<T>(a1, b1); break;                                       // |1><1|
      }
      mini += v;
      if (++cnt == 8) {
        acc += double(mini);
        mini = T(0);
        cnt = 0;
      }
    }
    mv<T, CLS>(S, b0, b1);
    mv<T, CLS>(S, a0, a1);
    psi[i0] = b0;
    psi[i1] = b1;
    lam[i0] = a0;
    lam[i1] = a1;
  }
  if (S.gen >= 0) {
    const double s = block_sum(acc + double(mini));
    if (threadIdx.x == 0) part[size_t(S.col) * nblk + blockIdx.x] = s;
  }
}

template <typename T>
void launch_adjoint_cls(int cls, cplx_t<T> *psi, cplx_t<T> *lam, uint64_t units, const AdjStep &S, double *d_part,
                        int nblk, cudaStream_t s) {
  switch (cls) {
    case 1: adjoint_step_kernel<T, 1><<<nblk, 256, 0, s>>>(psi, lam, units, S, d_part, nblk); break;
    case 2: adjoint_step_kernel<T, 2><<<nblk, 256, 0, s>>>(psi, lam, units, S, d_part, nblk); break;
    case 3: adjoint_step_kernel<T, 3><<<nblk, 256, 0, s>>>(psi, lam, units, S, d_part, nblk); break;
    case 4: adjoint_step_kernel<T, 4><<<nblk, 256, 0, s>>>(psi, lam, units, S, d_part, nblk); break;
    default: adjoint_step_kernel<T, 0><<<nblk, 256, 0, s>>>(psi, lam, units, S, d_part, nblk); break;
  }
}

}  // namespace

int adjoint_blocks(unsigned nq) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t units = uint64_t(1) << (nq > 0 ? nq - 1 : 0);
  return int(std::max<uint64_t>(1, std::min<uint64_t>((units + 255) / 256, uint64_t(sms) * 4)));
}

cudaError_t launch_adjoint_step(int prec, void *psi, void *lam, unsigned nq, const AdjointGate &g,
                                int col, double *d_part, int nblk, cudaStream_t s) {
  AdjStep S;
  std::memset(&S, 0, sizeof(S));
  // U^dagger = conj(U)^T
  S.u[0] = g.u[0].real();
  S.u[1] = -g.u[0].imag();
  S.u[2] = g.u[2].real();
  S.u[3] = -g.u[2].imag();
  S.u[4] = g.u[1].real();
  S.u[5] = -g.u[1].imag();
  S.u[6] = g.u[3].real();
  S.u[7] = -g.u[3].imag();
  S.ctrl = g.ctrl_mask;
  S.target = int(g.target);
  S.gen = g.gen;
  S.col = col;
  int n = 0;
  for (unsigned b = 0; b < 64; ++b)
    if (b == g.target || ((g.ctrl_mask >> b) & 1)) S.ins[n++] = uint8_t(b);
  S.nins = n;
  const uint64_t units = uint64_t(1) << (nq - unsigned(n));
  const double *u = S.u;  // U^dagger (re, im) x 4
  int cls = 0;
  if (u[0] == 0 && u[1] == 0 && u[6] == 0 && u[7] == 0 && u[2] == 1 && u[3] == 0 && u[4] == 1 && u[5] == 0)
    cls = 4;
  else if (u[2] == 0 && u[3] == 0 && u[4] == 0 && u[5] == 0)
    cls = 3;
  else if (u[1] == 0 && u[3] == 0 && u[5] == 0 && u[7] == 0)
    cls = 1;
  else if (u[1] == 0 && u[7] == 0 && u[2] == 0 && u[4] == 0)
    cls = 2;
  if (prec == 1)
    launch_adjoint_cls<float>(cls, static_cast<float2 *>(psi), static_cast<float2 *>(lam), units, S, d_part, nblk, s);
  else
    launch_adjoint_cls<double>(cls, static_cast<double2 *>(psi), static_cast<double2 *>(lam), units, S, d_part, nblk,
                               s);
  return cudaGetLastError();
}

}  // namespace gsim
