// Shared device-side helpers of the GB300 simulator core.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace gsim {

// Amplitude storage types: complex64 = float2, complex128 = double2.
template <typename T> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };
template <typename T> using cplx_t = typename cplx_of<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx_t<T> mkc(T re, T im) {
  cplx_t<T> c;
  c.x = re;
  c.y = im;
  return c;
}

// Insert a bit of value 0 at each of the n ascending positions pos[0..n).
// Maps a compact index over the remaining bits to a full state index.
__device__ __forceinline__ uint64_t insert_zeros(uint64_t u, const uint8_t *pos, int n) {
  for (int i = 0; i < n; ++i) {
    const uint32_t p = pos[i];
    const uint64_t lo = u & ((uint64_t(1) << p) - 1);
    u = ((u >> p) << (p + 1)) | lo;
  }
  return u;
}

// |z|^2 in FP64, rounded the way the reference's std::norm compiles with FMA
// contraction: fma(re, re, im*im).  For complex64 input the two products are
// exact in FP64, so this is the correctly rounded sum.
__device__ __forceinline__ double norm2_fp64(double2 z) {
  return __fma_rn(z.x, z.x, __dmul_rn(z.y, z.y));
}
__device__ __forceinline__ double norm2_fp64(float2 z) {
  const double x = z.x, y = z.y;
  return __fma_rn(x, x, __dmul_rn(y, y));
}

// Block-wide FP64 sum; the result is valid in thread 0.  blockDim.x must be a
// multiple of 32 and at most 1024.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double warp_part[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) warp_part[w] = v;
  __syncthreads();
  v = 0.;
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    v = lane < nw ? warp_part[lane] : 0.;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

}  // namespace gsim
