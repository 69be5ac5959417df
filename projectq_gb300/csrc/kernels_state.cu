// State-vector kernels other than gates: reductions (FP64), measurement
// support, projection, shrink, precision conversion, Pauli strings, Taylor
// steps of time evolution and arithmetic permutations (emulate_math).
//
// FP64 on GB300 runs at a small fraction of the FP32 rate, so complex64
// reductions square and add in FP32 over short runs of 8 amplitudes and
// carry the running sums in FP64; complex128 reductions are FP64 throughout.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <stdexcept>

#include "common.cuh"
#include "kernels.hpp"

namespace gsim {
namespace {

int g_sms = 0;
int sms() {
  if (!g_sms) {
    int d = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, d);
    if (g_sms <= 0) g_sms = 1;
  }
  return g_sms;
}
unsigned grid(uint64_t work, int threads, int per_sm = 8) {
  uint64_t want = (work + threads - 1) / threads;
  uint64_t cap = uint64_t(sms()) * per_sm;
  return unsigned(std::max<uint64_t>(1, std::min(want, cap)));
}

// FP64-carried sum of |z|^2.
template <typename T> struct NormAcc;
template <> struct NormAcc<double> {
  double s = 0.;
  __device__ void add(double2 z) { s = fma(z.x, z.x, fma(z.y, z.y, s)); }
  __device__ double get() const { return s; }
};
template <> struct NormAcc<float> {
  double s = 0.;
  float f = 0.f;
  int c = 0;
  __device__ void add(float2 z) {
    f = fmaf(z.x, z.x, fmaf(z.y, z.y, f));
    if (++c == 8) {
      s += double(f);
      f = 0.f;
      c = 0;
    }
  }
  __device__ double get() const { return s + double(f); }
};

// x with its sign bit flipped when neg & 1 (integer work, no floating-point
// multiply).
__device__ __forceinline__ double flip(double r, uint32_t neg) {
  return __longlong_as_double(__double_as_longlong(r) ^ (static_cast<long long>(neg & 1u) << 63));
}
__device__ __forceinline__ float flip(float r, uint32_t neg) {
  return __int_as_float(__float_as_int(r) ^ static_cast<int>((neg & 1u) << 31));
}

struct MaskSpec {
  uint8_t pos[64];
  int n;
};
MaskSpec mask_spec(uint64_t mask) {
  MaskSpec m;
  std::memset(&m, 0, sizeof(m));
  for (unsigned b = 0; b < 64; ++b)
    if ((mask >> b) & 1) m.pos[m.n++] = uint8_t(b);
  return m;
}

constexpr int kPartMax = 4096;

template <typename T>
__global__ void __launch_bounds__(256) masked_norm_kernel(const cplx_t<T> *__restrict__ psi,
                                                          uint64_t units, uint64_t val, MaskSpec ms,
                                                          double *part) {
  NormAcc<T> acc;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < units; u += stride)
    acc.add(psi[insert_zeros(u, ms.pos, ms.n) | val]);
  const double s = block_sum(acc.get());
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void column_sums_kernel(const double *__restrict__ part, int nblk, double *out) {
  double s = 0.;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += part[size_t(blockIdx.x) * nblk + b];
  s = block_sum(s);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

template <typename T>
__global__ void __launch_bounds__(256) project_scale_kernel(cplx_t<T> *__restrict__ psi, uint64_t n,
                                                            uint64_t mask, uint64_t val,
                                                            const double *d_norm) {
  const double inv = 1. / sqrt(*d_norm);
  const T f = T(inv);
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    if ((i & mask) != val) {
      psi[i] = mkc<T>(T(0), T(0));
    } else {
      cplx_t<T> z = psi[i];
      z.x *= f;
      z.y *= f;
      psi[i] = z;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) classical_flags_kernel(const cplx_t<T> *__restrict__ psi,
                                                              uint64_t units, unsigned pos,
                                                              double tol, int *flags) {
  int up = 0, down = 0;
  const uint8_t p = uint8_t(pos);
  const uint64_t d = uint64_t(1) << pos;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < units; u += stride) {
    const uint64_t i = insert_zeros(u, &p, 1);
    up |= norm2_fp64(psi[i]) > tol;
    down |= norm2_fp64(psi[i + d]) > tol;
  }
  up = __any_sync(0xffffffffu, up);
  down = __any_sync(0xffffffffu, down);
  if ((threadIdx.x & 31) == 0) {
    if (up) atomicOr(&flags[0], 1);
    if (down) atomicOr(&flags[1], 1);
  }
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

template <typename T>
__global__ void __launch_bounds__(256) classical_first_kernel(const cplx_t<T> *__restrict__ psi,
                                                              uint64_t units, unsigned pos,
                                                              double tol,
                                                              unsigned long long *first) {
  unsigned long long best = ~0ull;
  const uint8_t p = uint8_t(pos);
  const uint64_t d = uint64_t(1) << pos;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < units; u += stride) {
    const uint64_t i = insert_zeros(u, &p, 1);
    if (norm2_fp64(psi[i]) > tol || norm2_fp64(psi[i + d]) > tol) {
      best = u;
      break;  // later u of this thread are larger
    }
  }
  best = warp_min_u64(best);
  if ((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(first, best);
}

template <typename T>
__global__ void __launch_bounds__(256) shrink_kernel(const cplx_t<T> *__restrict__ src,
                                                     cplx_t<T> *__restrict__ dst, uint64_t n_out,
                                                     unsigned pos, uint64_t add) {
  const uint8_t p = uint8_t(pos);
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n_out; j += stride)
    dst[j] = src[insert_zeros(j, &p, 1) + add];
}

// Measurement: per block of 2^lb amplitudes, the sum of |psi_i|^2.  Its uses
// are the approximate running sum that picks each block's candidate binades
// and the exact test "every amplitude of the block is 0".  complex128: FP64.
// complex64: FP32 (GB300's FP64 pipe made this pass several times longer than
// reading the state), with a block of nonzero amplitudes whose FP32 sum
// underflows reported as the smallest positive double, so the zero test stays
// exact; a candidate that misses only sends the block to the element loop.
template <typename T>
__global__ void __launch_bounds__(256) block_norm_sums_kernel(const cplx_t<T> *__restrict__ psi,
                                                              uint64_t n, unsigned lb,
                                                              double *sums) {
  const uint64_t b0 = uint64_t(blockIdx.x) << lb;
  const uint64_t b1 = min(n, b0 + (uint64_t(1) << lb));
  if constexpr (sizeof(T) == 4) {
    __shared__ float ws[8];
    __shared__ unsigned wn[8];
    float s = 0.f;
    unsigned nz = 0;
    for (uint64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
      const float2 z = psi[i];
      s = fmaf(z.x, z.x, fmaf(z.y, z.y, s));
      nz |= (__float_as_uint(z.x) | __float_as_uint(z.y)) << 1;  // sign bits out: -0 is 0
    }
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_down_sync(0xffffffffu, s, o);
      nz |= __shfl_down_sync(0xffffffffu, nz, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
      ws[w] = s;
      wn[w] = nz;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      unsigned any = 0;
      for (int k = 0; k < int(blockDim.x >> 5); ++k) {
        t += ws[k];
        any |= wn[k];
      }
      sums[blockIdx.x] = t > 0.f || t != t ? double(t) : (any ? 4.9406564584124654e-324 : 0.);
    }
  } else {
    double s = 0.;
    for (uint64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) s += norm2_fp64(psi[i]);
    s = block_sum(s);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
  }
}

// x / 2^(e-52) rounded to nearest as an integer; flags bit 0 = exact tie,
// bit 1 = too large (>= 2^45 units) for the block sum to stay exact.
__device__ __forceinline__ unsigned long long grid_units(double x, int e, int &flag) {
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(x));
  if (bits == 0ull) return 0ull;
  const int ef = int(bits >> 52);
  unsigned long long m = bits & ((1ull << 52) - 1);
  int k;
  if (ef == 0) {
    k = -1074;
  } else {
    m |= 1ull << 52;
    k = ef - 1075;
  }
  const int sh = (e - 52) - k;
  unsigned long long q;
  if (sh <= 0) {
    if (-sh >= 11) {
      flag |= 2;
      return 0ull;
    }
    q = m << (-sh);
  } else if (sh >= 64) {
    q = 0ull;
  } else {
    q = m >> sh;
    const unsigned long long rem = m & ((1ull << sh) - 1);
    const unsigned long long half = 1ull << (sh - 1);
    if (rem > half) q += 1;
    else if (rem == half) flag |= 1;
  }
  if (q >= (1ull << 45)) flag |= 2;
  return q;
}

template <typename T>
__global__ void __launch_bounds__(256) block_grid_sums_kernel(const cplx_t<T> *__restrict__ psi,
                                                              uint64_t n, unsigned lb,
                                                              const int16_t *cand,
                                                              unsigned long long *units,
                                                              uint8_t *flags) {
  __shared__ unsigned long long ws[3][8];
  __shared__ int wf[3][8];
  const uint64_t b = blockIdx.x;
  const uint64_t b0 = b << lb;
  const uint64_t b1 = min(n, b0 + (uint64_t(1) << lb));
  int e[3];
  bool on[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    e[c] = cand[3 * b + c];
    on[c] = e[c] != -32768;
  }
  unsigned long long s[3] = {0ull, 0ull, 0ull};
  int f[3] = {0, 0, 0};
  for (uint64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
    const double x = norm2_fp64(psi[i]);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if (on[c]) s[c] += grid_units(x, e[c], f[c]);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
      f[c] |= __shfl_down_sync(0xffffffffu, f[c], o);
    }
    if (lane == 0) {
      ws[c][w] = s[c];
      wf[c][w] = f[c];
    }
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int c = threadIdx.x;
    unsigned long long t = 0ull;
    int fl = 0;
    for (int k = 0; k < int(blockDim.x >> 5); ++k) {
      t += ws[c][k];
      fl |= wf[c][k];
    }
    units[3 * b + c] = t;
    flags[3 * b + c] = uint8_t(on[c] ? fl : 4);
  }
}

template <typename D, typename S>
__global__ void convert_kernel(D *__restrict__ dst, const S *__restrict__ src, uint64_t n) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    D d;
    d.x = src[i].x;
    d.y = src[i].y;
    dst[i] = d;
  }
}

// Copy of `bytes` bytes by the SMs: 16-byte loads from `src` (here the device
// view of page-locked host memory) and 16-byte stores, then the 8-byte tail.
__global__ void pull_kernel(uint4 *__restrict__ dst, const uint4 *__restrict__ src, uint64_t n16) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = src[i];
}

// ---- Pauli expectation ---------------------------------------------------
constexpr int kTermsPerLaunch = 8;
struct ExpTerm {
  uint64_t sign_mask;
  float factor;  // +-2 / +-1 / 0
  int which;     // 0: real part of conj(psi_i) psi_j, 1: imaginary part
};
struct ExpBatch {
  ExpTerm t[kTermsPerLaunch];
  int nterms;
};

template <typename T>
__global__ void __launch_bounds__(256) pauli_expect_kernel(const cplx_t<T> *__restrict__ psi,
                                                           uint64_t units, uint64_t xmask,
                                                           int hbit, ExpBatch B, double *part,
                                                           int nblk, int col0) {
  double acc[kTermsPerLaunch];
  T mini[kTermsPerLaunch];
#pragma unroll
  for (int t = 0; t < kTermsPerLaunch; ++t) {
    acc[t] = 0.;
    mini[t] = T(0);
  }
  int cnt = 0;
  const uint8_t hb = uint8_t(hbit < 0 ? 0 : hbit);
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < units; u += stride) {
    uint64_t i;
    T ar, ai;
    if (hbit < 0) {
      i = u;
      const cplx_t<T> a = psi[i];
      ar = a.x * a.x + a.y * a.y;
      ai = T(0);
    } else {
      i = insert_zeros(u, &hb, 1);
      const cplx_t<T> a = psi[i], b = psi[i ^ xmask];
      ar = fma(a.x, b.x, a.y * b.y);   // Re(conj(a) b)
      ai = fma(a.x, b.y, -a.y * b.x);  // Im(conj(a) b)
    }
#pragma unroll
    for (int t = 0; t < kTermsPerLaunch; ++t) {
      if (t < B.nterms) {
        const T v = B.t[t].which ? ai : ar;
        const uint32_t neg = uint32_t(__popcll(i & B.t[t].sign_mask)) & 1u;
        mini[t] = fma(flip(T(B.t[t].factor), neg), v, mini[t]);
      }
    }
    if (++cnt == 8) {
#pragma unroll
      for (int t = 0; t < kTermsPerLaunch; ++t) {
        acc[t] += double(mini[t]);
        mini[t] = T(0);
      }
      cnt = 0;
    }
  }
  for (int t = 0; t < B.nterms; ++t) {
    const double s = block_sum(acc[t] + double(mini[t]));
    if (threadIdx.x == 0) part[size_t(col0 + t) * nblk + blockIdx.x] = s;
  }
}

// ---- sums of Pauli strings ------------------------------------------------
// Up to kSmemTerms terms are staged in shared memory per block (the rest of a
// longer list is read through L1).  Each thread issues the gathers of four
// terms before it uses them, so four loads per thread are in flight; terms
// sharing a flip mask gather the same address (an L1 hit).  The terms are
// summed in list order.
constexpr int kSmemTerms = 1024;

// Dynamic shared memory of a launch: term_smem_bytes<Term>(nterms).
template <typename Term>
__device__ __forceinline__ const Term *stage_terms(const Term *__restrict__ terms, int nterms) {
  if (nterms > kSmemTerms) return terms;
  extern __shared__ __align__(16) unsigned char term_smem[];
  auto *sm = reinterpret_cast<Term *>(term_smem);
  for (int t = threadIdx.x; t < nterms; t += blockDim.x) sm[t] = terms[t];
  __syncthreads();
  return sm;
}
template <typename Term> size_t term_smem_bytes(int nterms) {
  return nterms > kSmemTerms ? 0 : size_t(nterms) * sizeof(Term);
}

// sum_t r_t (P_t v)_j in FP64 for real-coefficient terms: with a = v.x, b =
// v.y (ny even) or a = v.y, b = v.x (ny odd), the term adds +-r a to the real
// part and +-r b to the imaginary part; the signs ((-1)^popcount(j & z) and
// those of (-i)^ny) are applied to r by flipping its sign bit.
__device__ __forceinline__ void real_term_add(const PauliRealTermDev &pt, double2 g, uint64_t j, double &re,
                                              double &im) {
  const uint32_t par = uint32_t(__popcll(j & pt.sign_mask)) & 1u;
  const uint32_t ny = uint32_t(pt.ny);
  const bool odd = ny & 1u;
  const double a = odd ? g.y : g.x, b = odd ? g.x : g.y;
  re = fma(flip(pt.r, par ^ (ny >> 1)), a, re);               // negative for ny = 2, 3
  im = fma(flip(pt.r, par ^ ((ny ^ (ny >> 1)) & 1u)), b, im);  // negative for ny = 1, 2
}
__device__ __forceinline__ void pauli_real_sum(const double2 *__restrict__ v, uint64_t j,
                                               const PauliRealTermDev *tp, int nterms, double &re, double &im) {
  int t = 0;
  for (; t + 4 <= nterms; t += 4) {
    double2 g[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) g[u] = v[j ^ tp[t + u].xmask];
#pragma unroll
    for (int u = 0; u < 4; ++u) real_term_add(tp[t + u], g[u], j, re, im);
  }
  for (; t < nterms; ++t) real_term_add(tp[t], v[j ^ tp[t].xmask], j, re, im);
}

// c_t (P_t v)_j with (P_t v)_j = (-1)^{popcount(j & sign)} v_{j ^ x} and
// c_t = cre + i cim (the term's phase folded in), accumulated in A: 4 FMAs.
template <typename A, typename V>
__device__ __forceinline__ void complex_term_add(const PauliApplyTermDev &pt, V g, uint64_t j, A &re, A &im) {
  const uint32_t par = uint32_t(__popcll(j & pt.sign_mask)) & 1u;
  const A cr = flip(A(pt.cre), par), ci = flip(A(pt.cim), par);
  re = fma(cr, A(g.x), fma(-ci, A(g.y), re));
  im = fma(cr, A(g.y), fma(ci, A(g.x), im));
}
template <typename A, typename V>
__device__ __forceinline__ void pauli_sum(const V *__restrict__ v, uint64_t j, const PauliApplyTermDev *tp,
                                          int nterms, A &re, A &im) {
  int t = 0;
  for (; t + 4 <= nterms; t += 4) {
    V g[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) g[u] = v[j ^ tp[t + u].xmask];
#pragma unroll
    for (int u = 0; u < 4; ++u) complex_term_add(tp[t + u], g[u], j, re, im);
  }
  for (; t < nterms; ++t) complex_term_add(tp[t], v[j ^ tp[t].xmask], j, re, im);
}

// ---- Pauli application (apply_qubit_operator) ----------------------------
template <typename T>
__global__ void __launch_bounds__(256) pauli_apply_kernel(const cplx_t<T> *__restrict__ in,
                                                          cplx_t<T> *__restrict__ out, uint64_t n,
                                                          const PauliApplyTermDev *__restrict__ terms,
                                                          int nterms) {
  const PauliApplyTermDev *tp = stage_terms<PauliApplyTermDev>(terms, nterms);
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    T re = T(0), im = T(0);
    pauli_sum<T>(in, i, tp, nterms, re, im);
    out[i] = mkc<T>(re, im);
  }
}

__global__ void __launch_bounds__(256) taylor_step_kernel(
    const double2 *__restrict__ vec, double2 *__restrict__ vnext, double2 *__restrict__ out,
    uint64_t n, const PauliRealTermDev *__restrict__ terms, int nterms, double cre, double cim,
    uint64_t ctrl, double *part) {
  const PauliRealTermDev *tp = stage_terms<PauliRealTermDev>(terms, nterms);
  double nrm = 0.;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += stride) {
    // (P_t vec)_j = phase * sign * vec[j ^ x], exact; times the real c_t
    double ur = 0., ui = 0.;
    pauli_real_sum(vec, j, tp, nterms, ur, ui);
    const double zr = ur * cre - ui * cim;
    const double zi = ur * cim + ui * cre;
    vnext[j] = make_double2(zr, zi);
    if ((j & ctrl) == ctrl) {
      double2 o = out[j];
      o.x += zr;
      o.y += zi;
      out[j] = o;
      nrm = fma(zr, zr, fma(zi, zi, nrm));
    }
  }
  const double s = block_sum(nrm);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// One Chebyshev order: w = scale * sum_t c_t (P_t cur)_j - prev_j (prev not
// read on the first order, has_prev = 0); w replaces prev in place (every
// thread reads prev only at its own j, and gathers only from cur); where
// (j & ctrl) == ctrl: out_j += a * w.
__global__ void __launch_bounds__(256) chebyshev_step_kernel(
    const double2 *__restrict__ cur, double2 *__restrict__ prev, double2 *__restrict__ out, uint64_t n,
    const PauliRealTermDev *__restrict__ terms, int nterms, double scale, int has_prev, double are,
    double aim, uint64_t ctrl) {
  const PauliRealTermDev *tp = stage_terms<PauliRealTermDev>(terms, nterms);
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += stride) {
    double ur = 0., ui = 0.;
    pauli_real_sum(cur, j, tp, nterms, ur, ui);
    double wr = scale * ur, wi = scale * ui;
    if (has_prev) {
      const double2 p = prev[j];
      wr -= p.x;
      wi -= p.y;
    }
    prev[j] = make_double2(wr, wi);
    if ((j & ctrl) == ctrl) {
      double2 o = out[j];
      o.x += are * wr - aim * wi;
      o.y += are * wi + aim * wr;
      out[j] = o;
    }
  }
}

// out_j = a * psi_j where (j & ctrl) == ctrl, else psi_j.
__global__ void scale_ctrl_kernel(const double2 *__restrict__ psi, double2 *__restrict__ out, uint64_t n,
                                  uint64_t ctrl, double are, double aim) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += stride) {
    const double2 p = psi[j];
    out[j] = (j & ctrl) == ctrl ? make_double2(are * p.x - aim * p.y, are * p.y + aim * p.x) : p;
  }
}

// psi <- a psi + b P psi over the controlled subspace.  With x != 0 a thread
// owns the pair (j, j ^ x), j with the pivot bit clear, and writes both; with
// x == 0 the map is diagonal, one amplitude per index.
template <typename T>
__global__ void __launch_bounds__(256) pauli_rotation_kernel(cplx_t<T> *__restrict__ psi, uint64_t units,
                                                             const __grid_constant__ PauliRotationDev r) {
  const T are = T(r.are), aim = T(r.aim), bre = T(r.bre), bim = T(r.bim);
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < units; u += stride) {
    const uint64_t j = insert_zeros(u, r.pos, r.npos) | r.ctrl;
    const cplx_t<T> p = psi[j];
    const T sj = (__popcll(j & r.zmask) & 1) ? T(-1) : T(1);
    if (r.xmask == 0) {
      const T fr = are + sj * bre, fi = aim + sj * bim;
      psi[j] = mkc<T>(fr * p.x - fi * p.y, fr * p.y + fi * p.x);
      continue;
    }
    const uint64_t k = j ^ r.xmask;
    const cplx_t<T> q = psi[k];
    const T sk = (__popcll(k & r.zmask) & 1) ? T(-1) : T(1);
    // new p = a p + sj b q ; new q = a q + sk b p
    const T cr = sj * bre, ci = sj * bim, dr = sk * bre, di = sk * bim;
    psi[j] = mkc<T>(are * p.x - aim * p.y + cr * q.x - ci * q.y, are * p.y + aim * p.x + cr * q.y + ci * q.x);
    psi[k] = mkc<T>(are * q.x - aim * q.y + dr * p.x - di * p.y, are * q.y + aim * q.x + dr * p.y + di * p.x);
  }
}

__global__ void phase_ctrl_kernel(double2 *__restrict__ out, double2 *__restrict__ vec, uint64_t n,
                                  uint64_t ctrl, double cre, double cim) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += stride) {
    double2 o = out[j];
    if ((j & ctrl) == ctrl) {
      const double r = o.x * cre - o.y * cim;
      const double i = o.x * cim + o.y * cre;
      o = make_double2(r, i);
      out[j] = o;
    }
    vec[j] = o;
  }
}

// ---- emulate_math --------------------------------------------------------
__device__ __forceinline__ uint32_t extract_reg(uint64_t i, const MathRegsDev &R) {
  uint32_t x = 0;
  for (int b = 0; b < R.width; ++b) x |= uint32_t((i >> R.pos[b]) & 1) << b;
  return x;
}
__device__ __forceinline__ uint64_t deposit_reg(uint64_t i, uint32_t y, const MathRegsDev &R) {
  for (int b = 0; b < R.width; ++b) {
    const uint64_t bit = uint64_t(1) << R.pos[b];
    i = ((y >> b) & 1) ? (i | bit) : (i & ~bit);
  }
  return i;
}
template <typename T> __device__ __forceinline__ cplx_t<T> add0(cplx_t<T> v);
template <> __device__ __forceinline__ double2 add0<double>(double2 v) {
  return make_double2(__dadd_rn(0., v.x), __dadd_rn(0., v.y));
}
template <> __device__ __forceinline__ float2 add0<float>(float2 v) {
  return make_float2(__fadd_rn(0.f, v.x), __fadd_rn(0.f, v.y));
}

template <typename T>
__global__ void __launch_bounds__(256) math_scatter_kernel(const cplx_t<T> *__restrict__ in,
                                                           cplx_t<T> *__restrict__ out, uint64_t n,
                                                           const MathRegsDev R,
                                                           const uint32_t *__restrict__ table) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t d = i;
    if ((i & R.ctrl) == R.ctrl) d = deposit_reg(i, table[extract_reg(i, R)], R);
    out[d] = add0<T>(in[i]);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) math_gather_kernel(const cplx_t<T> *__restrict__ in,
                                                          cplx_t<T> *__restrict__ out, uint64_t n,
                                                          const MathRegsDev R,
                                                          const uint64_t *__restrict__ inv_off,
                                                          const uint32_t *__restrict__ inv_src) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += stride) {
    if ((j & R.ctrl) != R.ctrl) {
      out[j] = add0<T>(in[j]);
      continue;
    }
    const uint32_t y = extract_reg(j, R);
    T re = T(0), im = T(0);
    for (uint64_t k = inv_off[y]; k < inv_off[y + 1]; ++k) {
      const cplx_t<T> v = in[deposit_reg(j, inv_src[k], R)];
      re += v.x;
      im += v.y;
    }
    out[j] = mkc<T>(re, im);
  }
}

template <typename A, typename B>
__global__ void __launch_bounds__(256) compare_kernel(const A *__restrict__ a, const B *__restrict__ b,
                                                      uint64_t n, double *part, int nblk,
                                                      unsigned long long *maxbits) {
  double re = 0., im = 0., mx = 0.;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double ar = a[i].x, ai = a[i].y, br = b[i].x, bi = b[i].y;
    re = fma(ar, br, fma(ai, bi, re));   // Re(conj(a) b)
    im = fma(ar, bi, fma(-ai, br, im));  // Im(conj(a) b)
    const double dr = ar - br, di = ai - bi;
    mx = fmax(mx, sqrt(fma(dr, dr, di * di)));
  }
  re = block_sum(re);
  if (threadIdx.x == 0) part[blockIdx.x] = re;
  im = block_sum(im);
  if (threadIdx.x == 0) part[nblk + blockIdx.x] = im;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits, static_cast<unsigned long long>(__double_as_longlong(mx)));
}

}  // namespace

cudaError_t launch_compare(int pa, const void *a, int pb, const void *b, uint64_t n, double *d_part,
                           double *d_out, cudaStream_t s) {
  const int nblk = int(std::min<unsigned>(grid(n, 256), 2048));
  cudaMemsetAsync(d_out + 2, 0, 8, s);
  auto *mx = reinterpret_cast<unsigned long long *>(d_out + 2);
  if (pa == 1 && pb == 1)
    compare_kernel<float2, float2><<<nblk, 256, 0, s>>>(static_cast<const float2 *>(a), static_cast<const float2 *>(b), n, d_part, nblk, mx);
  else if (pa == 1 && pb == 0)
    compare_kernel<float2, double2><<<nblk, 256, 0, s>>>(static_cast<const float2 *>(a), static_cast<const double2 *>(b), n, d_part, nblk, mx);
  else if (pa == 0 && pb == 1)
    compare_kernel<double2, float2><<<nblk, 256, 0, s>>>(static_cast<const double2 *>(a), static_cast<const float2 *>(b), n, d_part, nblk, mx);
  else
    compare_kernel<double2, double2><<<nblk, 256, 0, s>>>(static_cast<const double2 *>(a), static_cast<const double2 *>(b), n, d_part, nblk, mx);
  column_sums_kernel<<<2, 256, 0, s>>>(d_part, nblk, d_out);
  return cudaGetLastError();
}

// ---- launchers -------------------------------------------------------------

cudaError_t launch_masked_norm(int prec, const void *psi, unsigned nq, uint64_t mask,
                               uint64_t val, double *d_part, double *d_out, cudaStream_t s) {
  MaskSpec ms = mask_spec(mask);
  const uint64_t units = uint64_t(1) << (nq - ms.n);
  const unsigned g = std::min<unsigned>(grid(units, 256, 8), kPartMax);
  if (prec == 1)
    masked_norm_kernel<float><<<g, 256, 0, s>>>(static_cast<const float2 *>(psi), units, val, ms, d_part);
  else
    masked_norm_kernel<double><<<g, 256, 0, s>>>(static_cast<const double2 *>(psi), units, val, ms, d_part);
  column_sums_kernel<<<1, 1024, 0, s>>>(d_part, int(g), d_out);
  return cudaGetLastError();
}

cudaError_t launch_column_sums(const double *d_part, int nblk, int ncols, double *d_out,
                               cudaStream_t s) {
  if (ncols > 0) column_sums_kernel<<<ncols, 256, 0, s>>>(d_part, nblk, d_out);
  return cudaGetLastError();
}

cudaError_t launch_project_scale(int prec, void *psi, unsigned nq, uint64_t mask, uint64_t val,
                                 const double *d_norm, cudaStream_t s) {
  const uint64_t n = uint64_t(1) << nq;
  if (prec == 1)
    project_scale_kernel<float><<<grid(n, 256), 256, 0, s>>>(static_cast<float2 *>(psi), n, mask, val, d_norm);
  else
    project_scale_kernel<double><<<grid(n, 256), 256, 0, s>>>(static_cast<double2 *>(psi), n, mask, val, d_norm);
  return cudaGetLastError();
}

cudaError_t launch_classical_flags(int prec, const void *psi, unsigned nq, unsigned pos,
                                   double tol, int *d_flags, cudaStream_t s) {
  const uint64_t units = uint64_t(1) << (nq - 1);
  if (prec == 1)
    classical_flags_kernel<float><<<grid(units, 256), 256, 0, s>>>(static_cast<const float2 *>(psi), units, pos, tol, d_flags);
  else
    classical_flags_kernel<double><<<grid(units, 256), 256, 0, s>>>(static_cast<const double2 *>(psi), units, pos, tol, d_flags);
  return cudaGetLastError();
}

cudaError_t launch_classical_first(int prec, const void *psi, unsigned nq, unsigned pos,
                                   double tol, unsigned long long *d_first, cudaStream_t s) {
  const uint64_t units = uint64_t(1) << (nq - 1);
  // One unit per thread in index order keeps the early break meaningful.
  const unsigned g = unsigned(std::min<uint64_t>((units + 255) / 256, 1u << 30));
  if (prec == 1)
    classical_first_kernel<float><<<g, 256, 0, s>>>(static_cast<const float2 *>(psi), units, pos, tol, d_first);
  else
    classical_first_kernel<double><<<g, 256, 0, s>>>(static_cast<const double2 *>(psi), units, pos, tol, d_first);
  return cudaGetLastError();
}

cudaError_t launch_shrink(int prec, const void *src, void *dst, unsigned nq, unsigned pos,
                          int value, cudaStream_t s) {
  const uint64_t n_out = uint64_t(1) << (nq - 1);
  const uint64_t add = value ? (uint64_t(1) << pos) : 0;
  if (prec == 1)
    shrink_kernel<float><<<grid(n_out, 256), 256, 0, s>>>(static_cast<const float2 *>(src), static_cast<float2 *>(dst), n_out, pos, add);
  else
    shrink_kernel<double><<<grid(n_out, 256), 256, 0, s>>>(static_cast<const double2 *>(src), static_cast<double2 *>(dst), n_out, pos, add);
  return cudaGetLastError();
}

cudaError_t launch_block_norm_sums(int prec, const void *psi, uint64_t n, unsigned lb,
                                   double *d_sums, cudaStream_t s) {
  const uint64_t nb = (n + (uint64_t(1) << lb) - 1) >> lb;
  if (prec == 1)
    block_norm_sums_kernel<float><<<unsigned(nb), 256, 0, s>>>(static_cast<const float2 *>(psi), n, lb, d_sums);
  else
    block_norm_sums_kernel<double><<<unsigned(nb), 256, 0, s>>>(static_cast<const double2 *>(psi), n, lb, d_sums);
  return cudaGetLastError();
}

cudaError_t launch_block_grid_sums(int prec, const void *psi, uint64_t n, unsigned lb,
                                   const int16_t *d_cand, unsigned long long *d_units,
                                   uint8_t *d_flags, cudaStream_t s) {
  const uint64_t nb = (n + (uint64_t(1) << lb) - 1) >> lb;
  if (prec == 1)
    block_grid_sums_kernel<float><<<unsigned(nb), 256, 0, s>>>(static_cast<const float2 *>(psi), n, lb, d_cand, d_units, d_flags);
  else
    block_grid_sums_kernel<double><<<unsigned(nb), 256, 0, s>>>(static_cast<const double2 *>(psi), n, lb, d_cand, d_units, d_flags);
  return cudaGetLastError();
}

cudaError_t launch_pull(void *dst, const void *src, uint64_t bytes, cudaStream_t s) {
  if ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | bytes) & 15u) return cudaErrorInvalidValue;
  const uint64_t n16 = bytes / 16;
  if (!n16) return cudaSuccess;
  const unsigned blocks = unsigned(std::min<uint64_t>((n16 + 511) / 512, uint64_t(sms()) * 8));
  pull_kernel<<<blocks, 512, 0, s>>>(static_cast<uint4 *>(dst), static_cast<const uint4 *>(src), n16);
  return cudaGetLastError();
}

cudaError_t launch_convert(int dst_prec, void *dst, int src_prec, const void *src, uint64_t n,
                           cudaStream_t s) {
  const unsigned g = grid(n, 256);
  if (dst_prec == 1 && src_prec == 0)
    convert_kernel<float2, double2><<<g, 256, 0, s>>>(static_cast<float2 *>(dst), static_cast<const double2 *>(src), n);
  else if (dst_prec == 0 && src_prec == 1)
    convert_kernel<double2, float2><<<g, 256, 0, s>>>(static_cast<double2 *>(dst), static_cast<const float2 *>(src), n);
  else
    return cudaMemcpyAsync(dst, src, n * (dst_prec == 1 ? 8 : 16), cudaMemcpyDeviceToDevice, s);
  return cudaGetLastError();
}

int pauli_expect_blocks(unsigned nq) {
  const uint64_t units = uint64_t(1) << (nq > 0 ? nq - 1 : 0);
  return int(std::min<unsigned>(grid(units, 256, 4), 1024));
}

cudaError_t launch_pauli_expect(int prec, const void *psi, unsigned nq, uint64_t xmask,
                                const PauliTermDev *h_terms, int nterms, double *d_part,
                                int nblk, cudaStream_t s) {
  // h_terms is host memory here: the batch travels as a kernel parameter.
  int hbit = -1;
  for (int b = 63; b >= 0; --b)
    if ((xmask >> b) & 1) {
      hbit = b;
      break;
    }
  const uint64_t units = hbit < 0 ? (uint64_t(1) << nq) : (uint64_t(1) << (nq - 1));
  for (int t0 = 0; t0 < nterms; t0 += kTermsPerLaunch) {
    ExpBatch B;
    std::memset(&B, 0, sizeof(B));
    B.nterms = std::min(kTermsPerLaunch, nterms - t0);
    for (int t = 0; t < B.nterms; ++t) {
      const PauliTermDev &pt = h_terms[t0 + t];
      B.t[t].sign_mask = pt.sign_mask;
      if (hbit < 0) {
        // Diagonal term: Re[(-i)^q] |psi_i|^2 (q odd only for products of
        // factors on one qubit, e.g. Y X = -i Z, whose real part is 0).
        const int q = pt.phase & 3;
        B.t[t].factor = q == 0 ? 1.f : q == 2 ? -1.f : 0.f;
        B.t[t].which = 0;
      } else {
        // c = (-1)^popcount(x & sign_mask); q = #Y mod 4 (see header).
        const bool cpos = (__builtin_popcountll(xmask & pt.sign_mask) & 1) == 0;
        const int q = pt.phase & 3;
        if (cpos) {
          B.t[t].which = 0;
          B.t[t].factor = q == 0 ? 2.f : q == 2 ? -2.f : 0.f;
        } else {
          B.t[t].which = 1;
          B.t[t].factor = q == 1 ? 2.f : q == 3 ? -2.f : 0.f;
        }
      }
    }
    if (prec == 1)
      pauli_expect_kernel<float><<<nblk, 256, 0, s>>>(static_cast<const float2 *>(psi), units, xmask, hbit, B, d_part, nblk, t0);
    else
      pauli_expect_kernel<double><<<nblk, 256, 0, s>>>(static_cast<const double2 *>(psi), units, xmask, hbit, B, d_part, nblk, t0);
  }
  return cudaGetLastError();
}

cudaError_t launch_pauli_apply(int prec, const void *in, void *out, unsigned nq,
                               const PauliApplyTermDev *d_terms, int nterms, cudaStream_t s) {
  const uint64_t n = uint64_t(1) << nq;
  if (prec == 1)
    pauli_apply_kernel<float><<<grid(n, 256), 256, term_smem_bytes<PauliApplyTermDev>(nterms), s>>>(static_cast<const float2 *>(in), static_cast<float2 *>(out), n, d_terms, nterms);
  else
    pauli_apply_kernel<double><<<grid(n, 256), 256, term_smem_bytes<PauliApplyTermDev>(nterms), s>>>(static_cast<const double2 *>(in), static_cast<double2 *>(out), n, d_terms, nterms);
  return cudaGetLastError();
}

cudaError_t launch_taylor_step(const double2 *vec, double2 *vec_next, double2 *out, unsigned nq,
                               const PauliRealTermDev *d_terms, int nterms, double coeff_re,
                               double coeff_im, uint64_t ctrl, double *d_part, double *d_norm,
                               cudaStream_t s) {
  const uint64_t n = uint64_t(1) << nq;
  const unsigned g = std::min<unsigned>(grid(n, 256), kPartMax);
  taylor_step_kernel<<<g, 256, term_smem_bytes<PauliRealTermDev>(nterms), s>>>(vec, vec_next, out, n, d_terms, nterms, coeff_re, coeff_im, ctrl, d_part);
  column_sums_kernel<<<1, 1024, 0, s>>>(d_part, int(g), d_norm);
  return cudaGetLastError();
}

cudaError_t launch_phase_ctrl(double2 *out, double2 *vec, uint64_t n, uint64_t ctrl, double cre,
                              double cim, cudaStream_t s) {
  phase_ctrl_kernel<<<grid(n, 256), 256, 0, s>>>(out, vec, n, ctrl, cre, cim);
  return cudaGetLastError();
}

cudaError_t launch_chebyshev_step(const double2 *cur, double2 *prev, double2 *out, unsigned nq,
                                  const PauliRealTermDev *d_terms, int nterms, double scale, bool has_prev,
                                  double a_re, double a_im, uint64_t ctrl, cudaStream_t s) {
  const uint64_t n = uint64_t(1) << nq;
  chebyshev_step_kernel<<<grid(n, 256), 256, term_smem_bytes<PauliRealTermDev>(nterms), s>>>(cur, prev, out, n, d_terms, nterms, scale, has_prev ? 1 : 0,
                                                     a_re, a_im, ctrl);
  return cudaGetLastError();
}

cudaError_t launch_scale_ctrl(const double2 *psi, double2 *out, uint64_t n, uint64_t ctrl, double a_re,
                              double a_im, cudaStream_t s) {
  scale_ctrl_kernel<<<grid(n, 256), 256, 0, s>>>(psi, out, n, ctrl, a_re, a_im);
  return cudaGetLastError();
}

cudaError_t launch_pauli_rotation(int prec, void *psi, unsigned nq, const PauliRotationDev &r,
                                  cudaStream_t s) {
  if (r.npos < 0 || unsigned(r.npos) > nq) return cudaErrorInvalidValue;
  const uint64_t units = uint64_t(1) << (nq - unsigned(r.npos));
  if (prec == 1)
    pauli_rotation_kernel<float><<<grid(units, 256), 256, 0, s>>>(static_cast<float2 *>(psi), units, r);
  else
    pauli_rotation_kernel<double><<<grid(units, 256), 256, 0, s>>>(static_cast<double2 *>(psi), units, r);
  return cudaGetLastError();
}

cudaError_t launch_math_gather(int prec, const void *in, void *out, unsigned nq,
                               const MathRegsDev &regs, const uint64_t *d_inv_off,
                               const uint32_t *d_inv_src, cudaStream_t s) {
  const uint64_t n = uint64_t(1) << nq;
  if (prec == 1)
    math_gather_kernel<float><<<grid(n, 256), 256, 0, s>>>(static_cast<const float2 *>(in), static_cast<float2 *>(out), n, regs, d_inv_off, d_inv_src);
  else
    math_gather_kernel<double><<<grid(n, 256), 256, 0, s>>>(static_cast<const double2 *>(in), static_cast<double2 *>(out), n, regs, d_inv_off, d_inv_src);
  return cudaGetLastError();
}

cudaError_t launch_math_scatter(int prec, const void *in, void *out, unsigned nq,
                                const MathRegsDev &regs, const uint32_t *d_table,
                                cudaStream_t s) {
  const uint64_t n = uint64_t(1) << nq;
  if (prec == 1)
    math_scatter_kernel<float><<<grid(n, 256), 256, 0, s>>>(static_cast<const float2 *>(in), static_cast<float2 *>(out), n, regs, d_table);
  else
    math_scatter_kernel<double><<<grid(n, 256), 256, 0, s>>>(static_cast<const double2 *>(in), static_cast<double2 *>(out), n, regs, d_table);
  return cudaGetLastError();
}

}  // namespace gsim
