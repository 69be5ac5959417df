// Stage planner for GSIM_FUSION_STAGED: many gates per pass over the state.
//
// A stage is one pass of the stage kernel (kernels_stage.cu) over the state.
// The state is cut into tiles of 2^L amplitudes that share the values of all
// "non-local" bits; a tile's local bits are the m lowest bit positions (so
// each tile is made of 2^(L-m) contiguous runs of 2^m amplitudes, read and
// written with coalesced 16-byte accesses) plus up to L-m higher positions
// chosen per stage.  A CTA loads a tile into shared memory, applies the
// stage's operations in order, and writes it back.
//
//  - A non-diagonal gate needs its targets local; its controls can be
//    anywhere (local: checked per amplitude, non-local: per tile).
//  - A diagonal gate (Z, S, T, Rz, Ph, CZ, controlled phases...) needs no
//    locality at all: it becomes a diagonal operation over its targets and
//    controls, evaluated from the amplitude's global index.
//  - Gates with more than 2 non-diagonal targets leave the stage and run as
//    their own dense kernel.
//
// Planning is greedy in circuit order with a look-ahead window: a gate that
// does not fit blocks its qubits, and later gates that touch no blocked
// qubit (so they commute with every skipped gate) still join the stage.
// Inside a stage, consecutive operations on the same targets and controls are
// multiplied together, and runs of diagonal operations are merged (FP64).
// The reference has no counterpart (its fusion is fusion.hpp's dense
// clusters); the results equal applying the same gates one by one, up to
// rounding.
#pragma once

#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstddef>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "ops.hpp"

namespace gsim {

struct StageGate {
  std::vector<cplx> m;        // 2^k x 2^k, matrix bit l <-> pos[l]
  std::vector<unsigned> pos;  // target bit positions
  uint64_t ctrl_mask = 0;     // control bit positions
};

// Device-side description of one operation of a stage (see kernels_stage.cu).
struct StageOpDev {
  uint32_t kind;     // 0: dense on local targets, 1: diagonal
  uint32_t k;        // number of targets (dense) or diagonal qubits
  uint32_t mat;      // offset of the matrix / diagonal in the stage's pool (complex elements)
  uint32_t lctrl;    // local controls (tile-bit mask)
  uint64_t gctrl;    // non-local controls (global bit mask)
  uint8_t tbit[8];   // tile-bit index of target / diagonal qubit j, 0xFF if non-local
  uint8_t gbit[8];   // global bit position of diagonal qubit j
};

// Register substages.  The register kernel gives each of its 256 threads
// 2^r amplitudes of the tile in registers: the thread's "row" (a value of
// the L - r row bits) times every value of the r register bits R.  A
// substage is a run of the stage's operations whose dense targets all lie in
// R; it costs one shared-memory round trip however many operations it holds.
// Diagonal operations join any substage.  Shared memory holds the tile in a
// swizzled order s(p) = p ^ fold(p >> rho), fold XOR-ing rho-bit chunks, so
// tile bit b lands in bank class b mod rho; the five lane bits are chosen to
// cover every class, which makes each register access conflict-free.
// Register bits per thread of the register-substage kernel (tile = 2^(r + 8)
// amplitudes, 256 threads): 32 complex64 / 8 complex128 amplitudes per thread.
constexpr unsigned kRegBitsC64 = 5, kRegBitsC128 = 3, kMaxRegBits = 5;
// Substage and operation descriptors of one register stage travel as a kernel
// parameter (constant bank: warp-uniform reads); stages whose descriptors
// exceed this run on the one-pass-per-operation kernel instead.
constexpr size_t kStageTableBytes = 24576;

struct alignas(16) SubOpDev {
  uint8_t jidx[32]; // diagonal: index bits contributed by the register qubits, per j (16-byte aligned)
  uint64_t gctrl;   // non-local controls (global mask)
  uint32_t kind;    // 0 dense 1-qubit, 1 dense 2-qubit, 2 diagonal, 3 / 4 swap folded into the stores / loads
  uint32_t mat;     // offset in the stage's pool
  uint32_t jctrl;   // controls among the register bits (mask over j)
  uint32_t tctrl;   // controls among the row bits (mask over the row index)
  uint8_t rb[2];    // dense: register-bit index of matrix bit 0 / 1
  uint8_t ek[4];    // dense 1-qubit: kinds of m00 m01 m10 m11 (0 zero, 1 real, 2 imag, 3 complex)
  uint8_t dk;       // diagonal: number of qubits
  uint8_t dloc[6];  // diagonal qubit q: 0 register bit, 1 row bit, 2 non-local
  uint8_t didx[6];  //   its register-bit index / row-bit index / global bit position
  uint8_t swap;     // dense 1-qubit: 1 if the matrix is exactly [[0, 1], [1, 0]]
  uint8_t cls;      // dense 1-qubit matrix class: 0 general, 1 real, 2 real diagonal with
                    // imaginary off-diagonal (Rx), 3 exact swap, 4 anti-diagonal
  uint8_t dreg;     // diagonal: number of its qubits that are register bits
  uint32_t amask;   // dense: register indices j that are group bases with the controls satisfied
  uint8_t dq, dB;   // diagonal with dreg == 1: that qubit's index bit and register bit
  uint8_t pad[2];
  uint32_t sdelta;  // kinds 3, 4 (a swap folded into the stores / loads): the address XOR, soff[1 << B]
  uint32_t pad2;
};
static_assert(sizeof(SubOpDev) % 16 == 0, "SubOpDev must keep 16-byte alignment in arrays");
static_assert(offsetof(SubOpDev, jidx) == 0, "jidx is read with 16-byte loads");
struct SubstageDev {
  uint32_t op_begin, op_end;
  uint32_t soff[32];   // swizzled offset of register index j (XOR with the row's offset)
  uint32_t rowsw[16];  // swizzled offset of row bit i; a row's offset is the XOR of its set bits
};

struct StagePlan {
  unsigned L = 0;                 // tile bits
  std::vector<unsigned> lpos;     // ascending global positions of the tile bits (lpos[i] = i for i < m)
  std::vector<StageOpDev> ops;
  std::vector<cplx> pool;         // matrices / diagonals, FP64 (converted at upload)
  uint32_t ngates = 0;            // logical gates applied
  unsigned r = 0, rho = 0;        // register bits and bank-class bits (0: no register substages)
  std::vector<SubstageDev> subs;
  std::vector<SubOpDev> sops;
  int pack = -1;                  // tile bit that no operation touches (packed-pair kernel), -1: none
  std::vector<unsigned char> pk;  // packed-pair blob (build_substages_pk), empty: not used
  uint32_t pk_nsubs = 0;
};

// Bytes of the SubstageDev array as uploaded (the SubOpDev array follows it).
inline size_t stage_subs_bytes(const StagePlan &sp) {
  return (sp.subs.size() * sizeof(SubstageDev) + 15) / 16 * 16;
}

// s(p) = p ^ fold(p >> rho): fold XORs the rho-bit chunks of its argument.
inline uint32_t tile_swizzle(uint32_t p, unsigned rho) {
  uint32_t x = p >> rho, f = 0;
  const uint32_t mask = (1u << rho) - 1;
  while (x) {
    f ^= x & mask;
    x >>= rho;
  }
  return p ^ f;
}

// Split sp.ops into register substages of r register bits (256 threads:
// sp.L == r + 8).  Entry kinds let 1-qubit operations skip zero entries.
inline void build_substages(StagePlan &sp, unsigned r, unsigned rho) {
  if (r == 0 || r > kMaxRegBits || sp.L < r || sp.L - r > 16)
    throw std::invalid_argument("build_substages: unsupported register / row split");
  sp.r = r;
  sp.rho = rho;
  sp.subs.clear();
  sp.sops.clear();
  const unsigned L = sp.L;
  const size_t nops = sp.ops.size();
  // Qubits (global positions) each operation touches, for the commutation test:
  // operations commute when they share no qubit, or when both are diagonal.
  std::vector<uint64_t> touch(nops, 0);
  std::vector<uint32_t> tmask(nops, 0);
  for (size_t o = 0; o < nops; ++o) {
    const StageOpDev &op = sp.ops[o];
    for (unsigned q = 0; q < op.k; ++q)
      touch[o] |= uint64_t(1) << (op.tbit[q] == 0xFF ? op.gbit[q] : sp.lpos[op.tbit[q]]);
    if (op.kind == 0) {
      for (unsigned q = 0; q < op.k; ++q) tmask[o] |= 1u << op.tbit[q];
      for (unsigned b = 0; b < L; ++b)
        if ((op.lctrl >> b) & 1) touch[o] |= uint64_t(1) << sp.lpos[b];
      touch[o] |= op.gctrl;
    }
  }
  std::vector<std::vector<size_t>> preds(nops);
  for (size_t b = 0; b < nops; ++b)
    for (size_t a = 0; a < b; ++a)
      if ((touch[a] & touch[b]) && !(sp.ops[a].kind == 1 && sp.ops[b].kind == 1)) preds[b].push_back(a);
  std::vector<char> done(nops, 0);
  size_t ndone = 0;
  while (ndone < nops) {
    // List scheduling: take every ready operation that fits the register set.
    uint32_t R = 0;  // tile-bit mask
    std::vector<size_t> chosen;
    bool progress = true;
    while (progress) {
      progress = false;
      for (size_t o = 0; o < nops; ++o) {
        if (done[o]) continue;
        bool ready = true;
        for (size_t p : preds[o])
          if (!done[p]) {
            ready = false;
            break;
          }
        if (!ready) continue;
        if (sp.ops[o].kind == 0) {
          if (unsigned(__builtin_popcount(R | tmask[o])) > r) continue;
          R |= tmask[o];
        }
        done[o] = 1;
        ++ndone;
        chosen.push_back(o);
        progress = true;
      }
    }
    // Pad R to r bits, taking bits from the bank classes with most spare bits.
    while (unsigned(__builtin_popcount(R)) < r) {
      int best = -1, best_count = -1;
      for (unsigned b = 0; b < L; ++b) {
        if ((R >> b) & 1) continue;
        int cnt = 0;
        for (unsigned c = 0; c < L; ++c)
          if (!((R >> c) & 1) && c % rho == b % rho) ++cnt;
        if (cnt > best_count) {
          best_count = cnt;
          best = int(b);
        }
      }
      R |= 1u << best;
    }
    // Register bits ascending; row bits: one per bank class first (lanes).
    std::vector<unsigned> rbits, rows, rest;
    for (unsigned b = 0; b < L; ++b)
      if ((R >> b) & 1) rbits.push_back(b);
    std::vector<char> cls(rho, 0);
    for (unsigned b = 0; b < L; ++b) {
      if ((R >> b) & 1) continue;
      if (!cls[b % rho] && rows.size() < 5) {
        cls[b % rho] = 1;
        rows.push_back(b);
      } else {
        rest.push_back(b);
      }
    }
    for (unsigned b : rest) rows.push_back(b);
    SubstageDev sd;
    std::memset(&sd, 0, sizeof(sd));
    sd.op_begin = uint32_t(sp.sops.size());
    for (uint32_t x = 0; x < (1u << r); ++x) {
      uint32_t pos = 0;
      for (unsigned q = 0; q < r; ++q)
        if ((x >> q) & 1) pos |= 1u << rbits[q];
      sd.soff[x] = tile_swizzle(pos, rho);
    }
    for (size_t q = 0; q < rows.size(); ++q) sd.rowsw[q] = tile_swizzle(1u << rows[q], rho);
    auto reg_index = [&](unsigned tb) {
      return int(std::find(rbits.begin(), rbits.end(), tb) - rbits.begin());
    };
    auto row_index = [&](unsigned tb) {
      return int(std::find(rows.begin(), rows.end(), tb) - rows.begin());
    };
    for (size_t o : chosen) {
      const StageOpDev &op = sp.ops[o];
      SubOpDev so;
      std::memset(&so, 0, sizeof(so));
      so.mat = op.mat;
      so.gctrl = op.gctrl;
      for (unsigned b = 0; b < L; ++b) {
        if (!((op.lctrl >> b) & 1)) continue;
        if ((R >> b) & 1)
          so.jctrl |= 1u << reg_index(b);
        else
          so.tctrl |= 1u << row_index(b);
      }
      if (op.kind == 1) {
        so.kind = 2;
        so.dk = uint8_t(op.k);
        for (uint32_t x = 0; x < (1u << r) && x < 32; ++x) {
          uint32_t idx = 0;
          for (unsigned q = 0; q < op.k; ++q)
            if (op.tbit[q] != 0xFF && ((R >> op.tbit[q]) & 1) && ((x >> reg_index(op.tbit[q])) & 1)) idx |= 1u << q;
          so.jidx[x] = uint8_t(idx);
        }
        for (unsigned q = 0; q < op.k; ++q) {
          if (op.tbit[q] == 0xFF) {
            so.dloc[q] = 2;
            so.didx[q] = op.gbit[q];
          } else if ((R >> op.tbit[q]) & 1) {
            so.dloc[q] = 0;
            so.didx[q] = uint8_t(reg_index(op.tbit[q]));
            so.dreg++;
            so.dq = uint8_t(q);
            so.dB = so.didx[q];
          } else {
            so.dloc[q] = 1;
            so.didx[q] = uint8_t(row_index(op.tbit[q]));
          }
        }
      } else {
        so.kind = op.k == 1 ? 0 : 1;
        for (unsigned q = 0; q < op.k; ++q) so.rb[q] = uint8_t(reg_index(op.tbit[q]));
        if (op.k == 1) {
          for (int e = 0; e < 4; ++e) {
            const cplx z = sp.pool[op.mat + e];
            so.ek[e] = uint8_t((z.real() != 0. ? 1 : 0) | (z.imag() != 0. ? 2 : 0));
          }
          const cplx *mm = &sp.pool[op.mat];
          so.swap = mm[0] == cplx(0., 0.) && mm[1] == cplx(1., 0.) && mm[2] == cplx(1., 0.) &&
                    mm[3] == cplx(0., 0.);
          const bool real = mm[0].imag() == 0. && mm[1].imag() == 0. && mm[2].imag() == 0. && mm[3].imag() == 0.;
          const bool rx = mm[0].imag() == 0. && mm[3].imag() == 0. && mm[1].real() == 0. && mm[2].real() == 0.;
          const bool anti = mm[0] == cplx(0., 0.) && mm[3] == cplx(0., 0.);
          so.cls = so.swap ? 3 : real ? 1 : rx ? 2 : anti ? 4 : 0;
        }
        uint32_t tm = 0;
        for (unsigned q = 0; q < op.k; ++q) tm |= 1u << so.rb[q];
        for (uint32_t x = 0; x < (1u << r); ++x)
          if (!(x & tm) && (x & so.jctrl) == so.jctrl) so.amask |= 1u << x;
      }
      sp.sops.push_back(so);
    }
    // An X on register bit B whose controls are all row or non-local bits is
    // not applied to the registers when no other operation of the substage
    // touches B before it (then it is folded into the loads, kind 4) or after
    // it (folded into the stores, kind 3): it only exchanges where j and
    // j ^ (1 << B) live, and since soff is linear that is an XOR of
    // soff[1 << B] on every load or store address of the threads whose
    // controls hold.  Folded loads go first in the list, folded stores last.
    {
      auto regs_of = [](const SubOpDev &so) {
        uint32_t regs = so.jctrl;
        if (so.kind == 2) {
          for (unsigned q = 0; q < so.dk; ++q)
            if (so.dloc[q] == 0) regs |= 1u << so.didx[q];
        } else {
          regs |= 1u << so.rb[0];
          if (so.kind == 1) regs |= 1u << so.rb[1];
        }
        return regs;
      };
      auto foldable = [](const SubOpDev &so) { return so.kind == 0 && so.swap && so.jctrl == 0; };
      const size_t b0 = sd.op_begin;
      std::vector<SubOpDev> front, mid, back;
      uint32_t earlier = 0;
      for (size_t i = b0; i < sp.sops.size(); ++i) {
        SubOpDev so = sp.sops[i];
        if (foldable(so) && !((earlier >> so.rb[0]) & 1)) {
          so.kind = 4;
          so.sdelta = sd.soff[1u << so.rb[0]];
          front.push_back(so);
        } else {
          earlier |= regs_of(so);
          mid.push_back(so);
        }
      }
      std::vector<SubOpDev> kept;
      uint32_t later = 0;
      for (size_t i = mid.size(); i-- > 0;) {
        SubOpDev so = mid[i];
        if (foldable(so) && !((later >> so.rb[0]) & 1)) {
          so.kind = 3;
          so.sdelta = sd.soff[1u << so.rb[0]];
          back.push_back(so);
        } else {
          later |= regs_of(so);
          kept.push_back(so);
        }
      }
      sp.sops.resize(b0);
      sp.sops.insert(sp.sops.end(), front.begin(), front.end());
      sp.sops.insert(sp.sops.end(), kept.rbegin(), kept.rend());
      sp.sops.insert(sp.sops.end(), back.begin(), back.end());
    }
    sd.op_end = uint32_t(sp.sops.size());
    sp.subs.push_back(sd);
  }
}

// ---- packed-pair register substages (complex64) ---------------------------
// The packed-pair stage kernel (kernels_stage.cu, stage_pk_kernel) needs a
// tile bit P that no operation of the stage touches.  Amplitudes are held as
// pairs along P: a "pair" q is a tile position with bit P removed (12 bits),
// and shared memory keeps one 16-byte element per pair, (Re psi(q, P=0),
// Re psi(q, P=1), Im psi(q, P=0), Im psi(q, P=1)).  Every operation acts on both halves of
// a pair identically (P is not among its qubits), so the arithmetic runs on
// packed f32x2 FMAs.  A thread holds 16 pairs (32 amplitudes): register index
// jj over 4 register pair-bits, and its row (0..255) over the other 8.
// Pair positions in shared memory are swizzled, s(q) = q ^ fold3(q >> 3), so
// pair-bit b lands in bank class b mod 3; a substage's first three lanes
// cover the three classes where its register choice leaves them free, which
// makes the 16-byte accesses of each quarter warp conflict-free.
constexpr unsigned kPkTileBits = 13;      // 2^13 amplitudes = 4096 pairs per tile
constexpr size_t kPkBlobMax = 40 * 1024;  // shared-memory budget for descriptors, tables and data

struct PkSubDev {  // one substage
  uint32_t op_begin, op_end;  // its operations (PkOpDev index range)
  uint32_t tab;               // blob offset of rowtab[256], ldoff[16], stoff[16] (uint32)
  uint32_t pad;
};
static_assert(sizeof(PkSubDev) == 16, "PkSubDev is read with one 16-byte load");

// Operation kinds of the packed-pair kernel.
enum : uint32_t {
  kPkDense = 0,     // 1-qubit dense on register pair-bit b, matrix class cls
  kPkSwap = 1,      // X on register pair-bit b (register controls in amask)
  kPkDiag0 = 2,     // diagonal without register qubits: one factor per thread
  kPkDiag1 = 3,     // diagonal with one register qubit (pair-bit b): two factors
  kPkDiagN = 4,     // diagonal with several register qubits (b: their pair-bit mask): a factor per value of them
  kPkLoadXor = 5,   // X folded into the load addresses (row / tile controls only)
  kPkStoreXor = 6,  // X folded into the store addresses
};

// Operations with row or tile controls carry this flag in their code: the
// kernel tests controls only for them.
constexpr uint32_t kPkCtl = 1u << 13;

struct alignas(16) PkOpDev {
  uint32_t code;     // kind | b << 4 | cls << 8 | masked << 12 | kPkCtl (kPkDiagN: b is a pair-bit mask;
                     // kPkSwap: register controls in place of cls; kPkLoadXor: the kind alone, its controls
                     // always tested)
  uint32_t data;     // blob offset of the operation's data (16-byte aligned)
  uint32_t amask;    // dense / swap with register controls: the register indices it pairs from (16 bits);
                     // folded X: the address XOR
  uint32_t tctrl;    // controls among the row bits (mask over the row index)
  uint64_t gctrl;    // non-local controls (global bit mask)
  uint32_t dq;       // diagonal with one register qubit: that qubit's table-index bit
  uint32_t nsrc;     // diagonal: number of its qubits that are row bits or non-local
  uint8_t src[8];    // those qubits: bit 7 set = non-local (bits 0-6: global position), else the row bit
  uint8_t sbit[8];   // their table-index bits
  uint8_t jidx[16];  // diagonal with several register qubits: table-index bits of register index jj
};
static_assert(sizeof(PkOpDev) == 64, "PkOpDev is read with 16-byte loads");

inline uint32_t pk_swizzle(uint32_t q) { return tile_swizzle(q, 3); }

// Build the packed-pair substages of a complex64 stage whose plan has a pack
// bit (sp.pack >= 0, untouched by every operation) and only 1-qubit dense
// operations; returns false (the stage keeps the other kernels) otherwise.
inline bool build_substages_pk(StagePlan &sp) {
  sp.pk.clear();
  sp.pk_nsubs = 0;
  if (sp.L != kPkTileBits || sp.pack < 0) return false;
  const unsigned L = sp.L, P = unsigned(sp.pack);
  const size_t nops = sp.ops.size();
  for (const StageOpDev &op : sp.ops)
    if (op.kind == 0 && op.k != 1) return false;
  auto qbit = [&](unsigned tb) { return tb < P ? tb : tb - 1; };  // tile bit -> pair bit
  // touched tile bits per operation (non-local qubits in gtouch), commutation as in build_substages
  std::vector<uint32_t> ttouch(nops, 0), tmask(nops, 0);
  std::vector<uint64_t> gtouch(nops, 0);
  for (size_t o = 0; o < nops; ++o) {
    const StageOpDev &op = sp.ops[o];
    for (unsigned q = 0; q < op.k; ++q) {
      if (op.tbit[q] == 0xFF) gtouch[o] |= uint64_t(1) << op.gbit[q];
      else ttouch[o] |= 1u << op.tbit[q];
    }
    if (op.kind == 0) {
      tmask[o] = 1u << op.tbit[0];
      ttouch[o] |= op.lctrl;
      gtouch[o] |= op.gctrl;
    }
    if ((ttouch[o] >> P) & 1) return false;  // the pack bit must be untouched
  }
  // predecessors of each operation as a bitset over the operations
  const size_t nwords = (nops + 63) / 64;
  std::vector<uint64_t> predbits(nops * nwords, 0);
  for (size_t b = 0; b < nops; ++b)
    for (size_t a = 0; a < b; ++a)
      if (((ttouch[a] & ttouch[b]) || (gtouch[a] & gtouch[b])) && !(sp.ops[a].kind == 1 && sp.ops[b].kind == 1))
        predbits[b * nwords + (a >> 6)] |= uint64_t(1) << (a & 63);
  struct Sub {
    std::vector<size_t> ops;
    uint32_t R;  // register tile bits (P included)
  };
  std::vector<Sub> subs;
  std::vector<uint64_t> donebits(nwords, 0), trial(nwords, 0);
  std::vector<size_t> memo(size_t(1) << L, 0);  // scheduled count per key, valid where memo_gen == gen
  std::vector<uint32_t> memo_gen(size_t(1) << L, 0);
  uint32_t gen = 0;
  std::vector<uint32_t> cands4;  // the sets of 4 tile bits besides P, in increasing order
  for (uint32_t cand = 0; cand < (1u << L); ++cand)
    if (!((cand >> P) & 1) && __builtin_popcount(cand) == 4) cands4.push_back(cand);
  size_t ndone = 0;
  while (ndone < nops) {
    // The substage's register bits: of every set of 4 tile bits besides P,
    // the one under which list scheduling takes the most operations now
    // (ties: the first such set in enumeration order).
    // List scheduling under register bits R: every operation that is not yet
    // done, fits R (dense ones: their target) and whose predecessors are all
    // done.  Predecessors have lower indices, so one pass in index order
    // reaches the fixed point.  Done sets are bitsets over the operations.
    auto schedule = [&](uint32_t R, std::vector<uint64_t> &dn, std::vector<size_t> *chosen) {
      size_t taken = 0;
      for (size_t o = 0; o < nops; ++o) {
        if ((dn[o >> 6] >> (o & 63)) & 1) continue;
        if (sp.ops[o].kind == 0 && (tmask[o] & ~R)) continue;
        bool ready = true;
        for (size_t w = 0; w < nwords && ready; ++w) ready = !(predbits[o * nwords + w] & ~dn[w]);
        if (!ready) continue;
        dn[o >> 6] |= uint64_t(1) << (o & 63);
        ++taken;
        if (chosen) chosen->push_back(o);
      }
      return taken;
    };
    uint32_t R = 0;
    size_t best_taken = 0;
    for (uint32_t b = 0, k = 0; b < L && k < 4; ++b)  // a valid set whatever happens below
      if (b != P) R |= 1u << b, ++k;
    R |= 1u << P;
    // the result depends on a set only through the target bits of the
    // operations not yet done: each such intersection is scheduled once
    uint32_t needed = 0;
    for (size_t o = 0; o < nops; ++o)
      if (sp.ops[o].kind == 0 && !((donebits[o >> 6] >> (o & 63)) & 1)) needed |= tmask[o];
    ++gen;
    for (uint32_t cand : cands4) {
      const uint32_t key = cand & needed;
      if (memo_gen[key] != gen) {
        trial = donebits;
        memo[key] = schedule(cand | (1u << P), trial, nullptr);
        memo_gen[key] = gen;
      }
      const size_t taken = memo[key];
      if (taken > best_taken) {
        best_taken = taken;
        R = cand | (1u << P);
      }
    }
    std::vector<size_t> chosen;
    ndone += schedule(R, donebits, &chosen);
    // pad to 5 register bits, from the bank classes (pair-bit mod 3) with most spare bits
    while (unsigned(__builtin_popcount(R)) < 5) {
      int best = -1, best_count = -1;
      for (unsigned b = 0; b < L; ++b) {
        if ((R >> b) & 1) continue;
        int cnt = 0;
        for (unsigned c = 0; c < L; ++c)
          if (!((R >> c) & 1) && c != P && qbit(c) % 3 == qbit(b) % 3) ++cnt;
        if (cnt > best_count) {
          best_count = cnt;
          best = int(b);
        }
      }
      R |= 1u << best;
    }
    subs.push_back(Sub{chosen, R});
  }
  // serialise: [PkSubDev...][PkOpDev...][tables, data]
  std::vector<PkSubDev> dsubs;
  std::vector<PkOpDev> dops;
  std::vector<unsigned char> data;
  auto put = [&](const void *p, size_t n) {
    const size_t off = data.size();
    data.resize(off + ((n + 15) & ~size_t(15)), 0);
    std::memcpy(data.data() + off, p, n);
    return off;
  };
  // operation data shared between substages: dense matrices and diagonal tables
  std::vector<size_t> opdata(nops, 0);
  for (size_t o = 0; o < nops; ++o) {
    const StageOpDev &op = sp.ops[o];
    const cplx *M = &sp.pool[op.mat];
    if (op.kind == 0) {
      float d[24];  // X00 X01 X10 X11, Y.., -Y.. as broadcast pairs
      for (int e = 0; e < 4; ++e) {
        const float x = float(M[e].real()), y = float(M[e].imag());
        d[2 * e] = d[2 * e + 1] = x;
        d[8 + 2 * e] = d[8 + 2 * e + 1] = y;
        d[16 + 2 * e] = d[16 + 2 * e + 1] = -y;
      }
      opdata[o] = put(d, sizeof(d));
    } else {
      std::vector<float> t(size_t(8) << op.k);  // entry: (fx,fx) (fy,fy) (-fy,-fy) (0,0)
      for (size_t x = 0; x < (size_t(1) << op.k); ++x) {
        const float fx = float(M[x].real()), fy = float(M[x].imag());
        float *e = &t[8 * x];
        e[0] = e[1] = fx;
        e[2] = e[3] = fy;
        e[4] = e[5] = -fy;
        e[6] = e[7] = 0.f;
      }
      opdata[o] = put(t.data(), t.size() * sizeof(float));
    }
  }
  for (const Sub &sb : subs) {
    const uint32_t R = sb.R;
    std::vector<unsigned> rq, rows, rest;  // register pair-bits (jj bit k), row pair-bits (row bit i)
    std::vector<unsigned> rtile;           // register tile bits (jj bit k)
    for (unsigned b = 0; b < L; ++b)
      if (((R >> b) & 1) && b != P) {
        rq.push_back(qbit(b));
        rtile.push_back(b);
      }
    std::vector<char> cls(3, 0);
    for (unsigned b = 0; b < L; ++b) {
      if (((R >> b) & 1)) continue;
      const unsigned qb = qbit(b);
      if (!cls[qb % 3] && rows.size() < 3) {
        cls[qb % 3] = 1;
        rows.push_back(qb);
      } else {
        rest.push_back(qb);
      }
    }
    for (unsigned qb : rest) rows.push_back(qb);
    auto reg_of_tile = [&](unsigned tb) {
      return int(std::find(rtile.begin(), rtile.end(), tb) - rtile.begin());
    };
    auto row_of_tile = [&](unsigned tb) {
      const unsigned qb = qbit(tb);
      return int(std::find(rows.begin(), rows.end(), qb) - rows.begin());
    };
    auto deposit_jj = [&](uint32_t jj) {
      uint32_t q = 0;
      for (unsigned k = 0; k < 4; ++k)
        if ((jj >> k) & 1) q |= 1u << rq[k];
      return q;
    };
    // each operation of the substage as a packed-pair descriptor
    struct Cand {
      PkOpDev d;
      uint32_t regs;    // register bits (over jj) it touches
      bool swap;        // an X (candidate for folding)
      bool xor_type;    // no register controls (foldable as an address XOR)
      uint32_t t, c;    // swap: target bit and register-control mask (over jj)
    };
    std::vector<Cand> cands;
    for (size_t o : sb.ops) {
      const StageOpDev &op = sp.ops[o];
      Cand cd;
      std::memset(&cd.d, 0, sizeof(cd.d));
      cd.d.data = uint32_t(opdata[o]);
      cd.d.gctrl = op.gctrl;
      cd.regs = 0;
      cd.swap = false;
      cd.xor_type = false;
      cd.t = cd.c = 0;
      if (op.kind == 0) {
        uint32_t jc = 0;
        for (unsigned b = 0; b < L; ++b) {
          if (!((op.lctrl >> b) & 1)) continue;
          if ((R >> b) & 1) jc |= 1u << reg_of_tile(b);
          else cd.d.tctrl |= 1u << row_of_tile(b);
        }
        const unsigned bb = unsigned(reg_of_tile(op.tbit[0]));
        const cplx *mm = &sp.pool[op.mat];
        const bool swap = mm[0] == cplx(0., 0.) && mm[1] == cplx(1., 0.) && mm[2] == cplx(1., 0.) &&
                          mm[3] == cplx(0., 0.);
        const bool real = mm[0].imag() == 0. && mm[1].imag() == 0. && mm[2].imag() == 0. && mm[3].imag() == 0.;
        const bool rx = mm[0].imag() == 0. && mm[3].imag() == 0. && mm[1].real() == 0. && mm[2].real() == 0.;
        const bool anti = mm[0] == cplx(0., 0.) && mm[3] == cplx(0., 0.);
        const uint32_t cls = real ? 1 : rx ? 2 : anti ? 4 : 0;
        for (uint32_t jj = 0; jj < 16; ++jj)
          if (!((jj >> bb) & 1) && (jj & jc) == jc) cd.d.amask |= 1u << jj;
        const uint32_t masked = jc ? 1u : 0u;
        // swap: bits 8-11 carry its register controls (over the register index) instead of a class
        cd.d.code = (swap ? kPkSwap : kPkDense) | (bb << 4) | ((swap ? jc : cls) << 8) | (masked << 12);
        cd.regs = (1u << bb) | jc;
        cd.swap = swap;
        cd.xor_type = swap && jc == 0;
        cd.t = bb;
        cd.c = jc;
      } else {
        unsigned dreg = 0, dbreg = 0, dqb = 0;
        for (unsigned q = 0; q < op.k; ++q) {
          if (op.tbit[q] == 0xFF) {
            cd.d.src[cd.d.nsrc] = uint8_t(0x80 | op.gbit[q]);
            cd.d.sbit[cd.d.nsrc++] = uint8_t(q);
          } else if ((R >> op.tbit[q]) & 1) {
            const unsigned k = unsigned(reg_of_tile(op.tbit[q]));
            for (uint32_t jj = 0; jj < 16; ++jj)
              if ((jj >> k) & 1) cd.d.jidx[jj] |= uint8_t(1u << q);
            cd.regs |= 1u << k;
            ++dreg;
            dbreg = k;
            dqb = q;
          } else {
            cd.d.src[cd.d.nsrc] = uint8_t(row_of_tile(op.tbit[q]));
            cd.d.sbit[cd.d.nsrc++] = uint8_t(q);
          }
        }
        cd.d.dq = dqb;
        // kPkDiag1: b = its register pair-bit; kPkDiagN: b = the mask of its register pair-bits
        cd.d.code = dreg == 0 ? kPkDiag0 : dreg == 1 ? (kPkDiag1 | (dbreg << 4)) : (kPkDiagN | (cd.regs << 4));
      }
      cands.push_back(cd);
    }
    // Fold X gates at the start / end of the substage into the load / store
    // addresses: those with only row / tile controls as an address XOR,
    // those with only register controls as a permutation of the offset table.
    // A folded XOR moves outside the folded permutations, so it may not
    // target a control bit of one of them.
    const size_t nc = cands.size();
    std::vector<char> fold(nc, 0);  // 1: front, 2: back
    std::vector<uint32_t> perm_front(16), perm_back(16);
    for (uint32_t jj = 0; jj < 16; ++jj) perm_front[jj] = perm_back[jj] = jj;
    {
      uint32_t blocked = 0, pctrl = 0;
      for (size_t i = 0; i < nc; ++i) {
        const Cand &cd = cands[i];
        const bool perm_ok = cd.swap && !cd.xor_type && cd.d.tctrl == 0 && cd.d.gctrl == 0;
        if (cd.swap && !(blocked & cd.regs) && (cd.xor_type ? !((pctrl >> cd.t) & 1) : perm_ok)) {
          fold[i] = 1;
          if (!cd.xor_type) {  // perm = perm o sigma
            std::vector<uint32_t> np(16);
            for (uint32_t jj = 0; jj < 16; ++jj) {
              const uint32_t sj = (jj & cd.c) == cd.c ? jj ^ (1u << cd.t) : jj;
              np[jj] = perm_front[sj];
            }
            perm_front = np;
            pctrl |= cd.c;
          }
          continue;
        }
        blocked |= cd.regs;
      }
      blocked = 0;
      pctrl = 0;
      for (size_t i = nc; i-- > 0;) {
        if (fold[i]) continue;
        const Cand &cd = cands[i];
        const bool perm_ok = cd.swap && !cd.xor_type && cd.d.tctrl == 0 && cd.d.gctrl == 0;
        if (cd.swap && !(blocked & cd.regs) && (cd.xor_type ? !((pctrl >> cd.t) & 1) : perm_ok)) {
          fold[i] = 2;
          if (!cd.xor_type) {  // store map B^-1: perm_back = perm_back o sigma, scanning backwards
            std::vector<uint32_t> np(16);
            for (uint32_t jj = 0; jj < 16; ++jj) {
              const uint32_t sj = (jj & cd.c) == cd.c ? jj ^ (1u << cd.t) : jj;
              np[jj] = perm_back[sj];
            }
            perm_back = np;
            pctrl |= cd.c;
          }
          continue;
        }
        blocked |= cd.regs;
      }
    }
    PkSubDev sd;
    std::memset(&sd, 0, sizeof(sd));
    sd.op_begin = uint32_t(dops.size());
    for (size_t i = 0; i < nc; ++i)
      if (fold[i] == 1 && cands[i].xor_type) {
        PkOpDev d = cands[i].d;
        d.code = kPkLoadXor;
        d.amask = pk_swizzle(1u << rq[cands[i].t]);
        dops.push_back(d);
      }
    for (size_t i = 0; i < nc; ++i)
      if (!fold[i]) dops.push_back(cands[i].d);
    for (size_t i = nc; i-- > 0;)  // any order: XORs commute
      if (fold[i] == 2 && cands[i].xor_type) {
        PkOpDev d = cands[i].d;
        d.code = kPkStoreXor;
        d.amask = pk_swizzle(1u << rq[cands[i].t]);
        dops.push_back(d);
      }
    sd.op_end = uint32_t(dops.size());
    uint32_t tab[256 + 32];
    for (uint32_t row = 0; row < 256; ++row) {
      uint32_t q = 0;
      for (unsigned i = 0; i < 8; ++i)
        if ((row >> i) & 1) q |= 1u << rows[i];
      tab[row] = pk_swizzle(q);
    }
    for (uint32_t jj = 0; jj < 16; ++jj) {
      tab[256 + jj] = pk_swizzle(deposit_jj(perm_front[jj]));
      tab[272 + jj] = pk_swizzle(deposit_jj(perm_back[jj]));
    }
    sd.tab = uint32_t(put(tab, sizeof(tab)));
    dsubs.push_back(sd);
  }
  // final layout; offsets in the descriptors are made absolute
  const size_t subs_bytes = (dsubs.size() * sizeof(PkSubDev) + 15) & ~size_t(15);
  const size_t ops_bytes = dops.size() * sizeof(PkOpDev);
  const size_t head = subs_bytes + ops_bytes;
  if (head + data.size() > kPkBlobMax) return false;
  for (PkSubDev &d : dsubs) d.tab += uint32_t(head);
  for (PkOpDev &d : dops) {
    d.data += uint32_t(head);
    if (d.code != kPkLoadXor && (d.gctrl || d.tctrl)) d.code |= kPkCtl;
  }
  sp.pk.assign(head + data.size(), 0);
  std::memcpy(sp.pk.data(), dsubs.data(), dsubs.size() * sizeof(PkSubDev));
  std::memcpy(sp.pk.data() + subs_bytes, dops.data(), ops_bytes);
  std::memcpy(sp.pk.data() + head, data.data(), data.size());
  sp.pk_nsubs = uint32_t(dsubs.size());
  return true;
}

// One step of the plan: either a stage or a single wide dense gate.
struct PlanStep {
  bool is_stage = true;
  StagePlan stage;
  DenseOp dense;
  uint32_t ngates = 1;
};

class StagePlanner {
 public:
  // L: tile bits; m: contiguous low bits; window: look-ahead in gates.
  // pack: give every stage a tile bit that none of its gates touches where
  // possible (StagePlan::pack), for the packed-pair kernel.
  StagePlanner(unsigned nq, unsigned L, unsigned m, size_t window = 512, bool pack = false)
      : nq_(nq), L_(std::min(L, nq)), m_(std::min(m, std::min(L, nq))), window_(window), pack_(pack) {}

  std::vector<PlanStep> plan(const std::vector<StageGate> &gates) const {
    // Classify every gate once.
    std::vector<Item> items(gates.size());
    for (size_t i = 0; i < gates.size(); ++i) items[i] = classify(gates[i]);
    std::vector<PlanStep> steps;
    std::vector<char> done(gates.size(), 0);
    size_t first = 0;
    while (true) {
      while (first < gates.size() && done[first]) ++first;
      if (first >= gates.size()) break;
      if (items[first].wide) {
        PlanStep st;
        st.is_stage = false;
        st.dense.m = gates[first].m;
        st.dense.pos = gates[first].pos;
        st.dense.ctrl_mask = gates[first].ctrl_mask;
        steps.push_back(std::move(st));
        done[first] = 1;
        continue;
      }
      // Place gates for a stage with `cap` local bits for dense targets.
      auto place = [&](unsigned cap, uint64_t &local) {
        local = low_mask();
        uint64_t blocked = 0;
        std::vector<size_t> placed;
        size_t scanned = 0;
        for (size_t i = first; i < gates.size() && scanned < window_; ++i) {
          if (done[i]) continue;
          ++scanned;
          const Item &it = items[i];
          if (it.touch & blocked) {
            blocked |= it.touch;
            continue;
          }
          if (it.wide) {
            blocked |= it.touch;
            continue;
          }
          if (!it.diag) {
            const uint64_t nl = local | it.tmask;
            if (unsigned(__builtin_popcountll(nl)) > cap) {
              blocked |= it.touch;
              continue;
            }
            local = nl;
          }
          placed.push_back(i);
        }
        return placed;
      };
      uint64_t local = 0;
      std::vector<size_t> placed = place(L_, local);
      uint64_t touched = 0;
      for (size_t i : placed) touched |= items[i].touch;
      if (pack_ && L_ > m_ + 1 && !(fill_local_pack(local, touched) & ~touched)) {
        // every local bit is a dense target of the stage and no qubit is free:
        // place again with one local bit fewer, which leaves room for a pack bit
        uint64_t local2 = 0;
        std::vector<size_t> placed2 = place(L_ - 1, local2);
        uint64_t touched2 = 0;
        for (size_t i : placed2) touched2 |= items[i].touch;
        if (!placed2.empty() && (fill_local_pack(local2, touched2) & ~touched2)) {
          placed.swap(placed2);
          local = local2;
          touched = touched2;
        }
      }
      for (size_t i : placed) done[i] = 1;
      steps.push_back(PlanStep{});
      PlanStep &st = steps.back();
      st.is_stage = true;
      st.ngates = uint32_t(placed.size());
      const uint64_t full = pack_ ? fill_local_pack(local, touched) : fill_local(local);
      build_stage(gates, items, placed, full, st.stage);
      if (pack_) st.stage.pack = choose_pack(st.stage, touched);
    }
    return steps;
  }

 private:
  struct Item {
    bool diag = false;   // diagonal over (targets ∪ controls), at most 6 qubits
    bool wide = false;   // non-diagonal with more than 2 targets
    uint64_t tmask = 0;  // target positions
    uint64_t touch = 0;  // targets ∪ controls
  };

  uint64_t low_mask() const { return m_ >= 64 ? ~0ull : ((uint64_t(1) << m_) - 1); }

  static bool is_diagonal(const StageGate &g) {
    const size_t d = size_t(1) << g.pos.size();
    for (size_t r = 0; r < d; ++r)
      for (size_t c = 0; c < d; ++c)
        if (r != c && g.m[r * d + c] != cplx(0., 0.)) return false;
    return true;
  }

  Item classify(const StageGate &g) const {
    Item it;
    for (unsigned p : g.pos) it.tmask |= uint64_t(1) << p;
    it.touch = it.tmask | g.ctrl_mask;
    it.diag = is_diagonal(g) && __builtin_popcountll(it.touch) <= 6;
    it.wide = !it.diag && g.pos.size() > 2;
    return it;
  }

  // Complete the local set to exactly L bits with the lowest unused positions.
  uint64_t fill_local(uint64_t local) const {
    for (unsigned b = 0; b < nq_ && unsigned(__builtin_popcountll(local)) < L_; ++b) local |= uint64_t(1) << b;
    return local;
  }

  // As fill_local, but when no local bit is free of the stage's gates, the
  // first added bit is a qubit that none of them touches (the pack bit).
  // As fill_local, but when every local bit is used by the stage's gates,
  // the first added bit is a qubit that none of them touches (the pack bit).
  uint64_t fill_local_pack(uint64_t local, uint64_t touched) const {
    if (!(local & ~touched) && unsigned(__builtin_popcountll(local)) < L_) {
      for (unsigned b = 0; b < nq_; ++b)
        if (!((local >> b) & 1) && !((touched >> b) & 1)) {
          local |= uint64_t(1) << b;
          break;
        }
    }
    return fill_local(local);
  }

  // The pack bit: a tile bit no gate of the stage touches.  Preference:
  // global bit 0 (one 16-byte load holds two whole pairs), a bit above the
  // contiguous runs, a run bit >= 2, then bit 1 (whose pairs split each
  // 32-byte sector between two loads).
  int choose_pack(const StagePlan &sp, uint64_t touched) const {
    int best = -1, best_rank = 99;
    for (unsigned t = 0; t < sp.lpos.size(); ++t) {
      if ((touched >> sp.lpos[t]) & 1) continue;
      const unsigned g = sp.lpos[t];
      const int rank = g == 0 ? 0 : g >= m_ ? 1 : g >= 2 ? 2 : 3;
      if (rank < best_rank) {
        best_rank = rank;
        best = int(t);
      }
    }
    return best;
  }

  struct Op {
    bool diag;
    std::vector<unsigned> q;   // dense: target positions (matrix bit order); diag: qubits (ascending)
    uint64_t ctrl = 0;         // dense only
    std::vector<cplx> m;       // dense: 2^k x 2^k; diag: 2^k entries
  };

  static Op to_op(const StageGate &g, const Item &it) {
    Op op;
    if (!it.diag) {
      op.diag = false;
      op.q = g.pos;
      op.ctrl = g.ctrl_mask;
      op.m = g.m;
      return op;
    }
    // Diagonal over the ascending set of targets and controls.
    op.diag = true;
    for (unsigned b = 0; b < 64; ++b)
      if ((it.touch >> b) & 1) op.q.push_back(b);
    const size_t K = op.q.size(), D = size_t(1) << K, d = size_t(1) << g.pos.size();
    op.m.assign(D, cplx(1., 0.));
    for (size_t x = 0; x < D; ++x) {
      bool ctrl_ok = true;
      size_t local = 0;
      for (size_t j = 0; j < K; ++j) {
        const bool bit = (x >> j) & 1;
        if ((g.ctrl_mask >> op.q[j]) & 1) {
          if (!bit) ctrl_ok = false;
        }
      }
      if (!ctrl_ok) continue;
      for (size_t l = 0; l < g.pos.size(); ++l) {
        const size_t j = size_t(std::lower_bound(op.q.begin(), op.q.end(), g.pos[l]) - op.q.begin());
        if ((x >> j) & 1) local |= size_t(1) << l;
      }
      op.m[x] = g.m[local * d + local];
    }
    return op;
  }

  // a <- b * a (b applied after a), both dense on the same targets/controls.
  static void mul_into(Op &a, const Op &b) {
    const size_t d = size_t(1) << a.q.size();
    std::vector<cplx> r(d * d, cplx(0., 0.));
    for (size_t i = 0; i < d; ++i)
      for (size_t k = 0; k < d; ++k) {
        const cplx bik = b.m[i * d + k];
        if (bik == cplx(0., 0.)) continue;
        for (size_t j = 0; j < d; ++j) r[i * d + j] += bik * a.m[k * d + j];
      }
    a.m.swap(r);
  }

  // Merge two diagonal ops into one over the union of their qubits.
  static Op merge_diag(const Op &a, const Op &b) {
    Op o;
    o.diag = true;
    uint64_t u = 0;
    for (unsigned q : a.q) u |= uint64_t(1) << q;
    for (unsigned q : b.q) u |= uint64_t(1) << q;
    for (unsigned x = 0; x < 64; ++x)
      if ((u >> x) & 1) o.q.push_back(x);
    const size_t D = size_t(1) << o.q.size();
    o.m.assign(D, cplx(1., 0.));
    auto sub = [&](const Op &s, size_t x) {
      size_t idx = 0;
      for (size_t j = 0; j < s.q.size(); ++j) {
        const size_t pj = size_t(std::lower_bound(o.q.begin(), o.q.end(), s.q[j]) - o.q.begin());
        if ((x >> pj) & 1) idx |= size_t(1) << j;
      }
      return s.m[idx];
    };
    for (size_t x = 0; x < D; ++x) o.m[x] = sub(b, x) * sub(a, x);
    return o;
  }

  static bool same_shape(const Op &a, const Op &b) {
    return !a.diag && !b.diag && a.q == b.q && a.ctrl == b.ctrl;
  }

  void build_stage(const std::vector<StageGate> &gates, const std::vector<Item> &items,
                   const std::vector<size_t> &placed, uint64_t local, StagePlan &sp) const {
    sp.L = unsigned(__builtin_popcountll(local));
    sp.lpos.clear();
    for (unsigned b = 0; b < 64; ++b)
      if ((local >> b) & 1) sp.lpos.push_back(b);
    sp.ngates = uint32_t(placed.size());
    // Operations in order, merged where that changes nothing but rounding: a
    // new operation looks back past the operations it commutes with (no shared
    // qubit, or both diagonal) for one of the same shape (dense: same targets
    // and controls, multiplied) or a diagonal one (union of at most 6 qubits,
    // merged), and joins it there.  The stage kernel's time follows its
    // operation count; this merges 21% of the operations of the 30-qubit
    // random circuit that in-order merging leaves.
    auto touch_of = [](const Op &o) {
      uint64_t t = o.diag ? 0 : o.ctrl;
      for (unsigned q : o.q) t |= uint64_t(1) << q;
      return t;
    };
    std::vector<Op> ops;
    for (size_t i : placed) {
      Op op = to_op(gates[i], items[i]);
      const uint64_t ot = touch_of(op);
      bool merged = false;
      for (size_t e = ops.size(); e-- > 0;) {
        Op &prev = ops[e];
        if (same_shape(prev, op)) {
          mul_into(prev, op);
          merged = true;
          break;
        }
        if (prev.diag && op.diag) {
          if (__builtin_popcountll(touch_of(prev) | ot) <= 6) {
            prev = merge_diag(prev, op);
            merged = true;
            break;
          }
          continue;  // diagonal operations commute
        }
        if (touch_of(prev) & ot) break;  // a shared qubit: op stays after prev
      }
      if (!merged) ops.push_back(std::move(op));
    }
    auto tile_bit = [&](unsigned p) -> int {
      auto it = std::lower_bound(sp.lpos.begin(), sp.lpos.end(), p);
      return (it != sp.lpos.end() && *it == p) ? int(it - sp.lpos.begin()) : -1;
    };
    sp.ops.clear();
    sp.pool.clear();
    for (const Op &op : ops) {
      StageOpDev d;
      std::memset(&d, 0, sizeof(d));
      d.kind = op.diag ? 1 : 0;
      d.k = uint32_t(op.q.size());
      d.mat = uint32_t(sp.pool.size());
      std::memset(d.tbit, 0xFF, sizeof(d.tbit));
      for (size_t j = 0; j < op.q.size(); ++j) {
        const int tb = tile_bit(op.q[j]);
        d.tbit[j] = tb < 0 ? 0xFF : uint8_t(tb);
        d.gbit[j] = uint8_t(op.q[j]);
      }
      if (!op.diag) {
        for (unsigned b = 0; b < 64; ++b) {
          if (!((op.ctrl >> b) & 1)) continue;
          const int tb = tile_bit(b);
          if (tb >= 0)
            d.lctrl |= 1u << tb;
          else
            d.gctrl |= uint64_t(1) << b;
        }
      }
      sp.pool.insert(sp.pool.end(), op.m.begin(), op.m.end());
      sp.ops.push_back(d);
    }
  }

  unsigned nq_, L_, m_;
  size_t window_;
  bool pack_;
};

}  // namespace gsim
