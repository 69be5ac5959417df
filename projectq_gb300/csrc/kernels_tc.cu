// Fused dense k-qubit gates (k = 4 to 7) on complex64 states with the 5th
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
// M = 128 groups (TMEM lanes), N = K = 2^(k+1).  Each operand is split into
// hi = tf32(x) and lo = tf32(x - hi); three MMAs per K-step accumulate
// lo*hi + hi*lo + hi*hi.
//
// The kernel is persistent (one CTA per SM) and warp-specialised:
//   warps 0-7   producers: gather 16 amplitudes of a group per K-chunk from
//               HBM (two threads per group, the loads of the next kPrefetch
//               chunks in flight; 16-byte pair loads when a target is bit 0),
//               split them into TF32 hi/lo and write both into a ring of
//               shared-memory stages;
//   warps 8-11  epilogue: read a finished accumulator from TMEM
//               (tcgen05.ld, warp w owns TMEM lanes 32*(w%4)..) and store the
//               outputs back in place;
//   warp 12     MMA issue (one thread): tcgen05.mma per K-step, tcgen05.commit
//               to release a stage and to publish an accumulator;
//   warp 13     (k = 7 only) streams the unitary's K-chunk for each stage
//               into shared memory with cp.async.bulk; for k <= 6 the whole
//               operand B stays resident.
// Two TMEM accumulators let the epilogue of one tile overlap the MMAs of the
// next.  Every mbarrier wait is bounded: on timeout the thread records an
// error code, raises a CTA-wide abort flag that the other waits poll, and
// all threads meet at the end where TMEM is freed.
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

constexpr int kRows = 128;         // groups per tile (MMA M, TMEM lanes)
constexpr int kKC = 32;            // real K components per chunk (16 amplitudes)
constexpr int kAmpsPerChunk = kKC / 2;
constexpr int kProducers = 256;    // warps 0-7
constexpr int kEpilogue = 128;     // warps 8-11
constexpr int kMmaWarp = 12;
constexpr int kLoaderWarp = 13;
constexpr int kPrefetch = 4;       // K-chunks of loads in flight per producer thread (5 measured slower,
                                   // k = 5 gates 15.7 -> 18.4 ms at 32 qubits; 6: spills at k = 5 and no gain
                                   // at k = 6, 7)
constexpr uint32_t kStageA = uint32_t(kRows) * kKC * 4u;  // one split (hi or lo) of an A chunk

template <int KQ>
struct TcCfg {
  static constexpr int D = 1 << KQ;
  static constexpr int K = 2 * D;
  static constexpr int N = K;
  static constexpr int NCH = K / kKC;
  static constexpr bool kStream = KQ >= 7;  // B streamed per chunk instead of resident
  static constexpr int S = KQ <= 5 ? 4 : (KQ == 6 ? 3 : 2);
  static constexpr uint32_t kStageB = kStream ? uint32_t(N) * kKC * 4u : 0u;  // one split of a B chunk
  static constexpr uint32_t kBResident = kStream ? 0u : uint32_t(N) * K * 4u;  // one split of all of B
  static constexpr uint32_t kStageBytes = 2 * kStageA + 2 * kStageB;
  static constexpr uint32_t kBarOff = 2 * kBResident + S * kStageBytes;
  // input norms handed from the producers to the epilogue: float [NB][kRows][2 halves]
  static constexpr int NB = KQ == 6 ? 2 : 4;
  static constexpr uint32_t kNormOff = kBarOff + 256;
  static constexpr uint32_t kSmem = kNormOff + uint32_t(NB) * kRows * 2 * 4;
  static constexpr int kThreads = kStream ? 448 : 416;
  static constexpr uint32_t kTmemCols = 2u * N < 32u ? 32u : 2u * N;
};

struct TcArgs {
  uint64_t groups;      // number of amplitude groups
  uint64_t ctrl_set;
  int nins, k;
  uint8_t ins[64];
  uint64_t off[128];    // offset of amplitude j of a group (j < 2^k, k <= 7)
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
__host__ __device__ __forceinline__ uint32_t kmajor_off(uint32_t row, uint32_t kk, uint32_t kcols) {
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

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.release.cta.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(mbar)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(mbar),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(mbar), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s: far above any legitimate wait

// Bounded wait for the mbarrier phase `parity`.  Gives up (false) when the
// CTA's abort flag is raised or after kWaitLimitNs of wall time (measured on
// the global timer, so the bound holds however long one try_wait suspends),
// in which case it records the error and raises the abort flag itself.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, volatile int *abort_flag, int *err) {
  if (mbar_try(mbar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try(mbar, parity)) return true;
    if (*abort_flag) return false;
    if (global_ns() - t0 > kWaitLimitNs) break;
  }
  *abort_flag = 1;
  atomicExch(err, 1);
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

// 64 consecutive accumulator columns of this warp's 32 TMEM lanes (one
// register per column), with the wait for the load inside the same asm so the
// values are only used after they have arrived.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64]) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 columns (k = 4: the whole accumulator of one tile), same contract.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

template <int NC>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float (&v)[NC]) {
  if constexpr (NC == 64) tmem_ld64(taddr, v);
  else tmem_ld32(taddr, v);
}

__device__ __forceinline__ uint64_t group_base(const TcArgs &A, uint64_t g) {
  return insert_zeros(g, A.ins, A.nins) | A.ctrl_set;
}

// Producer: one K-chunk (8 amplitudes of one group) into registers.  PAIR:
// the first target is bit 0, so amplitudes j and j + 1 (j even) are adjacent
// and 16-byte aligned in the state: one 16-byte load per pair.
template <bool PAIR>
__device__ __forceinline__ void gather8(const float2 *__restrict__ psi, const TcArgs &A, uint64_t base, bool active,
                                        int ch, int half, float2 (&x)[8]) {
  if constexpr (PAIR) {
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
      const int j = ch * kAmpsPerChunk + half * 8 + q;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (active) v = *reinterpret_cast<const float4 *>(psi + base + A.off[j]);
      x[q] = make_float2(v.x, v.y);
      x[q + 1] = make_float2(v.z, v.w);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int j = ch * kAmpsPerChunk + half * 8 + q;
      x[q] = active ? psi[base + A.off[j]] : make_float2(0.f, 0.f);
    }
  }
}

// Producer: split 8 amplitudes into TF32 hi/lo and store them as 4 pairs of
// 16-byte core-matrix rows (K components 4p..4p+3 of this chunk).
__device__ __forceinline__ void split_store(unsigned char *st, int row, int half, const float2 (&x)[8]) {
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const float2 a = x[2 * p], b = x[2 * p + 1];
    float4 h, l;
    h.x = tf32_round(a.x);
    h.y = tf32_round(a.y);
    h.z = tf32_round(b.x);
    h.w = tf32_round(b.y);
    l.x = tf32_round(a.x - h.x);
    l.y = tf32_round(a.y - h.y);
    l.z = tf32_round(b.x - h.z);
    l.w = tf32_round(b.y - h.w);
    const uint32_t o = kmajor_off(uint32_t(row), uint32_t(half * 16 + 4 * p), uint32_t(kKC));
    *reinterpret_cast<float4 *>(st + o) = h;
    *reinterpret_cast<float4 *>(st + kStageA + o) = l;
  }
}

// RENORM: U is unitary and each group's outputs are rescaled to the group's
// input norm (a compile-time choice, so the plain kernel carries none of it).
template <int KQ, bool PAIR, bool RENORM>
__global__ void __launch_bounds__(TcCfg<KQ>::kThreads, 1)
    tc_gate_kernel(float2 *__restrict__ psi, const float *__restrict__ bsrc, const __grid_constant__ TcArgs A,
                   int *err) {
  using Cfg = TcCfg<KQ>;
  constexpr int N = Cfg::N, K = Cfg::K, NCH = Cfg::NCH, S = Cfg::S;
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char *bres = sm;                             // resident B: hi then lo (k <= 6)
  unsigned char *stages = sm + 2 * Cfg::kBResident;    // S x [A hi | A lo | B hi | B lo]
  uint64_t *bars = reinterpret_cast<uint64_t *>(sm + Cfg::kBarOff);
  // bars: full[S], empty[S], accf[2], acce[2], drain, (abort flag), (TMEM slot), nfull[NB], nemp[NB]
  volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 2 * S + 5);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * S + 6);
  float *nin = reinterpret_cast<float *>(sm + Cfg::kNormOff);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + S), accf0 = smem_u32(bars + 2 * S),
                 acce0 = smem_u32(bars + 2 * S + 2), drain = smem_u32(bars + 2 * S + 4),
                 nfull0 = smem_u32(bars + 2 * S + 7), nemp0 = smem_u32(bars + 2 * S + 7 + Cfg::NB);

  if constexpr (!Cfg::kStream) {
    const uint4 *src = reinterpret_cast<const uint4 *>(bsrc);
    uint4 *dst = reinterpret_cast<uint4 *>(bres);
    for (uint32_t e = tid; e < 2 * Cfg::kBResident / 16; e += blockDim.x) dst[e] = __ldg(src + e);
  }
  if (tid == 0) {
    *abort_flag = 0;
    for (int s = 0; s < S; ++s) {
      mbar_init(full0 + 8 * s, kProducers + (Cfg::kStream ? 1 : 0));
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, kEpilogue);
    }
    mbar_init(drain, 1);
    for (int b = 0; b < Cfg::NB; ++b) {
      mbar_init(nfull0 + 8 * b, kProducers);
      mbar_init(nemp0 + 8 * b, kEpilogue);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(Cfg::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint64_t ntiles = (A.groups + kRows - 1) / kRows;

  if (warp < kProducers / 32) {
    // ---- producers -------------------------------------------------------
    // A load cursor runs kPrefetch chunks ahead of the publish cursor: the
    // registers of a chunk are refilled right after it was published, so
    // about kPrefetch x 8 loads per thread are in flight.
    const int row = tid & (kRows - 1), half = tid >> 7;
    const uint64_t mine = blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    const uint64_t total = mine * NCH;
    uint64_t lt = blockIdx.x, loaded = 0;
    int lc = 0;
    bool lact = false;
    uint64_t lbase = 0;
    if (total) {
      const uint64_t g = lt * kRows + uint64_t(row);
      lact = g < A.groups;
      lbase = lact ? group_base(A, g) : 0;
    }
    auto load_next = [&](float2 (&x)[8]) {
      if (loaded >= total) return;
      gather8<PAIR>(psi, A, lbase, lact, lc, half, x);
      ++loaded;
      if (++lc == NCH) {
        lc = 0;
        lt += gridDim.x;
        if (lt < ntiles) {
          const uint64_t g = lt * kRows + uint64_t(row);
          lact = g < A.groups;
          lbase = lact ? group_base(A, g) : 0;
        }
      }
    };
    uint64_t it = 0;
    float nacc = 0.f;  // this thread's share of its group's input norm (renorm)
    auto publish = [&](const float2 (&x)[8]) -> bool {
      const int s = int(it % S);
      const uint32_t u = uint32_t(it / S);
      if (u > 0 && !mbar_wait(empty0 + 8 * s, (u - 1) & 1u, abort_flag, err)) return false;
      split_store(stages + size_t(s) * Cfg::kStageBytes, row, half, x);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(full0 + 8 * s);
      if constexpr (RENORM) {
#pragma unroll
        for (int q = 0; q < 8; ++q) nacc = fmaf(x[q].x, x[q].x, fmaf(x[q].y, x[q].y, nacc));
        if (int(it % NCH) == NCH - 1) {  // the tile's last chunk: hand the norm to the epilogue
          const uint32_t ti = uint32_t(it / NCH), b = ti % Cfg::NB, ub = ti / Cfg::NB;
          if (ub > 0 && !mbar_wait(nemp0 + 8 * b, (ub - 1) & 1u, abort_flag, err)) return false;
          nin[(b * kRows + row) * 2 + half] = nacc;
          mbar_arrive(nfull0 + 8 * b);
          nacc = 0.f;
        }
      }
      ++it;
      return true;
    };
    float2 x[kPrefetch][8];
#pragma unroll
    for (int b = 0; b < kPrefetch; ++b) load_next(x[b]);
    bool ok = true;
    while (ok && it < total) {
#pragma unroll
      for (int b = 0; b < kPrefetch; ++b) {
        if (it >= total) break;
        if (!publish(x[b])) {
          ok = false;
          break;
        }
        load_next(x[b]);
      }
    }
  } else if (warp < (kProducers + kEpilogue) / 32) {
    // ---- epilogue --------------------------------------------------------
    const int row = 32 * (warp & 3) + lane;
    const uint32_t lane_base = uint32_t(32 * (warp & 3)) << 16;
    uint32_t i = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const uint32_t b = i & 1u, u = i >> 1;
      if (!mbar_wait(accf0 + 8 * b, u & 1u, abort_flag, err)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t g = tile * kRows + uint64_t(row);
      const bool active = g < A.groups;
      const uint64_t base = active ? group_base(A, g) : 0;
      // EC columns (EC / 2 outputs) per TMEM load: one wait per load
      constexpr int EC = N < 64 ? N : 64;
      // The tensor cores' FP32 accumulation shrinks sums slightly (measured
      // 1e-8 x K relative per gate, always downwards), which for a unitary U
      // is a loss of norm; each group's outputs are rescaled to the group's
      // input norm (exact for unitary U up to FP32 rounding).
      auto store_cols = [&](const float (&v)[EC], int c0) {
        if (!active) return;
        if constexpr (PAIR) {
#pragma unroll
          for (int q = 0; q < EC / 2; q += 2)
            __stcs(reinterpret_cast<float4 *>(psi + base + A.off[c0 / 2 + q]),
                   make_float4(v[2 * q], v[2 * q + 1], v[2 * q + 2], v[2 * q + 3]));
        } else {
#pragma unroll
          for (int q = 0; q < EC / 2; ++q) __stcs(psi + base + A.off[c0 / 2 + q], make_float2(v[2 * q], v[2 * q + 1]));
        }
      };
      if constexpr (RENORM) {
        const uint32_t nb = i % Cfg::NB, nu = i / Cfg::NB;
        if (!mbar_wait(nfull0 + 8 * nb, nu & 1u, abort_flag, err)) break;
        const float s_in = nin[(nb * kRows + row) * 2] + nin[(nb * kRows + row) * 2 + 1];
        mbar_arrive(nemp0 + 8 * nb);
        float s_out = 0.f;
        if constexpr (N == EC) {
          // k <= 5: one TMEM load holds the row; norm, scale and store from registers
          float v[EC];
          tmem_ld<EC>(tmem + lane_base + b * uint32_t(N), v);
#pragma unroll
          for (int q = 0; q < EC; ++q) s_out = fmaf(v[q], v[q], s_out);
          const float scale = (s_out > 0.f && s_in > 0.f) ? sqrtf(s_in / s_out) : 1.f;
#pragma unroll
          for (int q = 0; q < EC; ++q) v[q] *= scale;
          store_cols(v, 0);
        } else {
#pragma unroll 1
          for (int c0 = 0; c0 < N; c0 += EC) {
            float v[EC];
            tmem_ld<EC>(tmem + lane_base + b * uint32_t(N) + uint32_t(c0), v);
#pragma unroll
            for (int q = 0; q < EC; ++q) s_out = fmaf(v[q], v[q], s_out);
          }
          const float scale = (s_out > 0.f && s_in > 0.f) ? sqrtf(s_in / s_out) : 1.f;
#pragma unroll 1
          for (int c0 = 0; c0 < N; c0 += EC) {
            float v[EC];
            tmem_ld<EC>(tmem + lane_base + b * uint32_t(N) + uint32_t(c0), v);
#pragma unroll
            for (int q = 0; q < EC; ++q) v[q] *= scale;
            store_cols(v, c0);
          }
        }
      } else {
#pragma unroll 1
        for (int c0 = 0; c0 < N; c0 += EC) {
          float v[EC];
          tmem_ld<EC>(tmem + lane_base + b * uint32_t(N) + uint32_t(c0), v);
          store_cols(v, c0);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(acce0 + 8 * b);
    }
  } else if (warp == kMmaWarp) {
    // ---- MMA issue -------------------------------------------------------
    if (lane == 0) {
      // idesc: D = F32, A = B = TF32, both K-major, N >> 3, M >> 4 (M = 128).
      const uint32_t idesc =
          (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(kRows >> 4) << 24);
      const uint32_t st0 = smem_u32(stages), br = smem_u32(bres);
      uint64_t it = 0;
      uint32_t i = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++i) {
        const uint32_t b = i & 1u, u = i >> 1;
        if (u > 0 && !mbar_wait(acce0 + 8 * b, (u - 1) & 1u, abort_flag, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dcol = tmem + b * uint32_t(N);
        for (int ch = 0; ch < NCH; ++ch, ++it) {
          const int s = int(it % S);
          if (!mbar_wait(full0 + 8 * s, uint32_t(it / S) & 1u, abort_flag, err)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = st0 + uint32_t(s) * Cfg::kStageBytes;
#pragma unroll
          for (int ks = 0; ks < kKC / 8; ++ks) {
            const uint32_t ak = uint32_t(2 * ks) * 128u;
            const uint64_t dah = smem_desc(sa + ak, 128u, (kKC / 4) * 128u);
            const uint64_t dal = smem_desc(sa + kStageA + ak, 128u, (kKC / 4) * 128u);
            uint64_t dbh, dbl;
            if constexpr (Cfg::kStream) {
              const uint32_t sb = sa + 2 * kStageA;
              dbh = smem_desc(sb + ak, 128u, (kKC / 4) * 128u);
              dbl = smem_desc(sb + Cfg::kStageB + ak, 128u, (kKC / 4) * 128u);
            } else {
              const uint32_t bk = uint32_t(ch * (kKC / 4) + 2 * ks) * 128u;
              dbh = smem_desc(br + bk, 128u, (K / 4) * 128u);
              dbl = smem_desc(br + Cfg::kBResident + bk, 128u, (K / 4) * 128u);
            }
            const uint32_t acc0 = (ch > 0 || ks > 0) ? 1u : 0u;
            mma_tf32(dcol, dal, dbh, idesc, acc0);
            mma_tf32(dcol, dah, dbl, idesc, 1u);
            mma_tf32(dcol, dah, dbh, idesc, 1u);
          }
          mma_commit(empty0 + 8 * s);
        }
        if (!ok) break;
        mma_commit(accf0 + 8 * b);
      }
    }
  } else if (Cfg::kStream && warp == kLoaderWarp) {
    // ---- B chunk loader (k = 7) --------------------------------------------
    if (lane == 0) {
      const uint32_t st0 = smem_u32(stages);
      const char *src = reinterpret_cast<const char *>(bsrc);
      uint64_t it = 0;
      bool ok = true;
      for (uint64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        for (int ch = 0; ch < NCH; ++ch, ++it) {
          const int s = int(it % S);
          const uint32_t u = uint32_t(it / S);
          if (u > 0 && !mbar_wait(empty0 + 8 * s, (u - 1) & 1u, abort_flag, err)) {
            ok = false;
            break;
          }
          const uint32_t dst = st0 + uint32_t(s) * Cfg::kStageBytes + 2 * kStageA;
          mbar_arrive_tx(full0 + 8 * s, 2 * Cfg::kStageB);
          bulk_g2s(dst, src + size_t(ch) * 2 * Cfg::kStageB, 2 * Cfg::kStageB, full0 + 8 * s);
        }
      }
    }
  }
  // Before TMEM is freed every MMA must have completed: one more commit
  // tracks all MMAs this thread issued (also after an abort).
  if (warp == kMmaWarp && lane == 0) {
    mma_commit(drain);
    const uint64_t t0 = global_ns();
    while (!mbar_try(drain, 0u) && global_ns() - t0 < kWaitLimitNs) {
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::kTmemCols)
                 : "memory");
}

// U unitary (to 1e-10): the norms of two fixed pseudo-random vectors are kept.
bool tc_is_unitary(const std::vector<cplx> &U, int k) {
  const size_t D = size_t(1) << k;
  uint64_t st = 0x9E3779B97F4A7C15ull;
  for (int trial = 0; trial < 2; ++trial) {
    std::vector<cplx> v(D);
    double nv = 0;
    for (size_t j = 0; j < D; ++j) {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      const double re = double(int64_t(st >> 11) % 1000003) / 1000003.0 - 0.5;
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      const double im = double(int64_t(st >> 11) % 1000003) / 1000003.0 - 0.5;
      v[j] = cplx(re, im);
      nv += re * re + im * im;
    }
    double nw = 0;
    for (size_t a = 0; a < D; ++a) {
      cplx w = 0;
      for (size_t j = 0; j < D; ++j) w += U[a * D + j] * v[j];
      nw += std::norm(w);
    }
    if (!(std::abs(nw - nv) <= 1e-10 * nv)) return false;
  }
  return true;
}

template <int KQ, bool PAIR>
cudaError_t launch_tc_kp(void *psi, unsigned nq, const DenseOp &op, const float *d_b, int *d_err, bool renorm,
                         cudaStream_t s) {
  using Cfg = TcCfg<KQ>;
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
  for (int j = 0; j < Cfg::D; ++j)
    for (int l = 0; l < KQ; ++l)
      if ((j >> l) & 1) A.off[j] |= uint64_t(1) << op.pos[l];
  A.groups = uint64_t(1) << (nq - ins.size());
  const bool rn = renorm && tc_is_unitary(op.m, KQ);
  auto *kern = rn ? tc_gate_kernel<KQ, PAIR, true> : tc_gate_kernel<KQ, PAIR, false>;
  // set on every launch: attributes belong to the current device
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::kSmem));
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t ntiles = (A.groups + kRows - 1) / kRows;
  const unsigned grid = unsigned(std::max<uint64_t>(1, std::min<uint64_t>(ntiles, uint64_t(sms))));
  kern<<<grid, Cfg::kThreads, Cfg::kSmem, s>>>(static_cast<float2 *>(psi), d_b, A, d_err);
  return cudaGetLastError();
}

template <int KQ>
cudaError_t launch_tc_k(void *psi, unsigned nq, const DenseOp &op, const float *d_b, int *d_err, bool renorm,
                        cudaStream_t s) {
  if (op.pos[0] == 0) return launch_tc_kp<KQ, true>(psi, nq, op, d_b, d_err, renorm, s);
  return launch_tc_kp<KQ, false>(psi, nq, op, d_b, d_err, renorm, s);
}

}  // namespace

// The same gate with its targets in ascending bit order (rows and columns of
// the matrix permuted to match), so that a target at bit 0 is matrix bit 0.
DenseOp tc_sorted_targets(const DenseOp &op) {
  const size_t k = op.pos.size(), D = size_t(1) << k;
  std::vector<unsigned> perm(k);
  for (size_t l = 0; l < k; ++l) perm[l] = unsigned(l);
  std::sort(perm.begin(), perm.end(), [&](unsigned a, unsigned b) { return op.pos[a] < op.pos[b]; });
  DenseOp out;
  out.ctrl_mask = op.ctrl_mask;
  out.pos.resize(k);
  for (size_t l = 0; l < k; ++l) out.pos[l] = op.pos[perm[l]];
  std::vector<size_t> old(D, 0);  // new index -> old index
  for (size_t j = 0; j < D; ++j)
    for (size_t l = 0; l < k; ++l)
      if ((j >> l) & 1) old[j] |= size_t(1) << perm[l];
  out.m.resize(D * D);
  for (size_t a = 0; a < D; ++a)
    for (size_t j = 0; j < D; ++j) out.m[a * D + j] = op.m[old[a] * D + old[j]];
  return out;
}

size_t tc_operand_floats(int k) { return size_t(2) * size_t(2 << k) * size_t(2 << k); }

// Operand B (the real embedding of U, split hi/lo in TF32) laid out in the
// shared-memory core-matrix order the kernel consumes:
//   k <= 6: [hi: N x K][lo: N x K]                      (copied once per CTA)
//   k = 7:  for each K-chunk: [hi: N x kKC][lo: N x kKC] (one bulk copy per stage)
void tc_prepare_operand(const std::vector<cplx> &U, int k, float *out) {
  const int D = 1 << k, K = 2 * D, N = K;
  auto tf32 = [](float x) {  // round to nearest (ties away), 10 explicit mantissa bits
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
  };
  const bool stream = k >= 7;
  auto place = [&](int row, int col, float h, float l) {
    size_t o;
    size_t split;
    if (!stream) {
      o = kmajor_off(uint32_t(row), uint32_t(col), uint32_t(K)) / 4;
      split = size_t(N) * K;
    } else {
      const int ch = col / kKC, kk = col % kKC;
      o = size_t(ch) * 2 * N * kKC + kmajor_off(uint32_t(row), uint32_t(kk), uint32_t(kKC)) / 4;
      split = size_t(N) * kKC;
    }
    out[o] = h;
    out[o + split] = l;
  };
  for (int a = 0; a < D; ++a)
    for (int j = 0; j < D; ++j) {
      const double re = U[size_t(a) * D + j].real(), im = U[size_t(a) * D + j].imag();
      const double vals[4] = {re, -im, im, re};  // (2a,2j) (2a,2j+1) (2a+1,2j) (2a+1,2j+1)
      const int rows[4] = {2 * a, 2 * a, 2 * a + 1, 2 * a + 1}, cols[4] = {2 * j, 2 * j + 1, 2 * j, 2 * j + 1};
      for (int t = 0; t < 4; ++t) {
        const float h = tf32(float(vals[t]));
        const float l = tf32(float(vals[t] - double(h)));
        place(rows[t], cols[t], h, l);
      }
    }
}

cudaError_t launch_tc_gate(void *psi, unsigned nq, const DenseOp &op, const float *d_b, int *d_err, bool renorm,
                           cudaStream_t s) {
  switch (op.pos.size()) {
    case 4: return launch_tc_k<4>(psi, nq, op, d_b, d_err, renorm, s);
    case 5: return launch_tc_k<5>(psi, nq, op, d_b, d_err, renorm, s);
    case 6: return launch_tc_k<6>(psi, nq, op, d_b, d_err, renorm, s);
    case 7: return launch_tc_k<7>(psi, nq, op, d_b, d_err, renorm, s);
    default: throw std::invalid_argument("tensor-core gate kernel supports 4 to 7 targets");
  }
}

}  // namespace gsim
