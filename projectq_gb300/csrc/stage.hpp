// Fusion planner used by GSIM_FUSION_STAGED: groups consecutive gates into
// clusters of at most kmax matrix qubits and composes each cluster in FP64.
//
// Difference from the reference's greedy rule (fusion.hpp + simulator.hpp:
// 204-222): clusters close only when the next gate would not fit (no eager
// run at 4 qubits), the width limit follows the storage precision (complex64
// gates stay HBM-bound up to 4 matrix qubits on GB300's FP32 pipes, while
// complex128 is FP64-bound, so clusters there stay at 2 qubits, where fusing
// costs no extra FP64 work per amplitude), and a control shared by all gates
// of a cluster stays a control.  The composed unitary is the ordered product
// of the same gates, so results agree with unfused application to rounding.
#pragma once

#include <algorithm>
#include <complex>
#include <cstdint>
#include <vector>

#include "kernels.hpp"

namespace gsim {

struct StageGate {
  std::vector<cplx> m;        // 2^k x 2^k, matrix bit l <-> pos[l]
  std::vector<unsigned> pos;  // target bit positions
  uint64_t ctrl_mask = 0;     // control bit positions
};

class StagePlanner {
 public:
  StagePlanner(unsigned nq, int prec, unsigned kmax)
      : nq_(nq), kmax_(std::max(1u, std::min(kmax, prec == 1 ? 4u : 2u))) {}

  std::vector<DenseOp> fuse(const std::vector<StageGate> &gates,
                            std::vector<uint32_t> *counts = nullptr) const {
    std::vector<DenseOp> out;
    size_t i = 0;
    while (i < gates.size()) {
      // Grow a cluster starting at gate i.
      uint64_t shared = gates[i].ctrl_mask;
      uint64_t qubits = mask_of(gates[i].pos);
      size_t j = i + 1;
      while (j < gates.size()) {
        const StageGate &g = gates[j];
        const uint64_t ns = shared & g.ctrl_mask;
        const uint64_t nq = qubits | mask_of(g.pos) | (shared & ~ns) | (g.ctrl_mask & ~ns);
        if (unsigned(__builtin_popcountll(nq)) > kmax_) break;
        shared = ns;
        qubits = nq;
        ++j;
      }
      out.push_back(compose(gates, i, j, qubits, shared));
      if (counts) counts->push_back(uint32_t(j - i));
      i = j;
    }
    return out;
  }

 private:
  static uint64_t mask_of(const std::vector<unsigned> &pos) {
    uint64_t m = 0;
    for (unsigned p : pos) m |= uint64_t(1) << p;
    return m;
  }

  // Product of gates [i, j) as one matrix over `qubits` (ascending bit
  // positions), controlled by `shared`.
  DenseOp compose(const std::vector<StageGate> &gates, size_t i, size_t j, uint64_t qubits,
                  uint64_t shared) const {
    DenseOp op;
    for (unsigned b = 0; b < 64; ++b)
      if ((qubits >> b) & 1) op.pos.push_back(b);
    op.ctrl_mask = shared;
    const size_t K = op.pos.size(), D = size_t(1) << K;
    auto local = [&](unsigned p) {
      return unsigned(std::lower_bound(op.pos.begin(), op.pos.end(), p) - op.pos.begin());
    };
    if (j - i == 1 && gates[i].ctrl_mask == shared) {
      // A single gate: keep its own bit order (no composition needed).
      op.pos = gates[i].pos;
      op.m = gates[i].m;
      return op;
    }
    std::vector<cplx> M(D * D, cplx(0., 0.)), T(D * D);
    for (size_t r = 0; r < D; ++r) M[r * D + r] = 1.;
    for (size_t g = i; g < j; ++g) {
      const StageGate &G = gates[g];
      const size_t k = G.pos.size(), d = size_t(1) << k;
      std::vector<size_t> off(d, 0);
      size_t tmask = 0;
      for (size_t l = 0; l < k; ++l) tmask |= size_t(1) << local(G.pos[l]);
      for (size_t a = 0; a < d; ++a)
        for (size_t l = 0; l < k; ++l)
          if ((a >> l) & 1) off[a] |= size_t(1) << local(G.pos[l]);
      size_t cmask = 0;  // controls folded into the matrix
      for (unsigned b = 0; b < 64; ++b)
        if (((G.ctrl_mask & ~shared) >> b) & 1) cmask |= size_t(1) << local(b);
      T = M;
      for (size_t r = 0; r < D; ++r) {
        if (r & tmask) continue;
        if ((r & cmask) != cmask) continue;  // control not satisfied: identity
        for (size_t a = 0; a < d; ++a) {
          cplx *dst = &T[(r + off[a]) * D];
          for (size_t c = 0; c < D; ++c) dst[c] = 0.;
          for (size_t b = 0; b < d; ++b) {
            const cplx w = G.m[a * d + b];
            if (w == cplx(0., 0.)) continue;
            const cplx *src = &M[(r + off[b]) * D];
            for (size_t c = 0; c < D; ++c) dst[c] += w * src[c];
          }
        }
      }
      M.swap(T);
    }
    op.m = std::move(M);
    return op;
  }

  unsigned nq_;
  unsigned kmax_;
};

}  // namespace gsim
