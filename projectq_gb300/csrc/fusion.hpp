// Gate fusion with the reference's greedy rule.
//
// Behaviour follows projectq/backends/_sim/_cppkernels/fusion.hpp:39-165 and
// the admission rule of simulator.hpp:204-222: gates are queued while the
// union of their qubits stays below 4; the batch runs as soon as it spans 4
// or 5 qubits, or before a gate that would widen it past 5 or that would turn
// a shared control into a matrix qubit.  Controls shared by every queued
// gate stay controls (a mask in the kernel); the rest are folded into the
// matrices.  The composed matrix is built in FP64 on the host (at most
// 32 x 32 here, or 2^kmax for the wider planners).
#pragma once

#include <algorithm>
#include <complex>
#include <set>
#include <vector>

namespace gsim {

struct FusedItem {
  std::vector<std::complex<double>> m;  // dim x dim, row-major
  std::vector<unsigned> ids;            // matrix bit l <-> ids[l]
};

class RefFusion {
 public:
  using cplx = std::complex<double>;

  unsigned num_qubits() const { return unsigned(qubits_.size()); }
  size_t size() const { return items_.size(); }
  const std::set<unsigned> &controls() const { return ctrls_; }

  void insert(std::vector<cplx> m, std::vector<unsigned> ids, const std::vector<unsigned> &ctrl) {
    for (unsigned q : ids) qubits_.insert(q);
    // Controls not shared by every gate become matrix qubits (fusion.hpp:130-160).
    std::set<unsigned> dropped = ctrls_;
    for (unsigned c : ctrl) {
      if (ctrls_.count(c)) {
        dropped.erase(c);
      } else if (!items_.empty()) {
        embed_controls(m, ids, {c});
        qubits_.insert(c);
      } else {
        ctrls_.insert(c);
      }
    }
    if (!dropped.empty()) {
      std::vector<unsigned> nc(dropped.begin(), dropped.end());
      for (unsigned c : nc) {
        ctrls_.erase(c);
        qubits_.insert(c);
      }
      for (auto &it : items_) embed_controls(it.m, it.ids, nc);
    }
    items_.push_back(FusedItem{std::move(m), std::move(ids)});
  }

  // Compose every queued gate, in order, into one matrix over the sorted qubit
  // set; returns that set (matrix bit l <-> ids[l]) and the shared controls.
  void compose(std::vector<cplx> &M, std::vector<unsigned> &ids, std::vector<unsigned> &ctrl) const {
    ids.assign(qubits_.begin(), qubits_.end());
    const size_t D = size_t(1) << ids.size();
    M.assign(D * D, cplx(0., 0.));
    for (size_t i = 0; i < D; ++i) M[i * D + i] = 1.;
    std::vector<cplx> tmp(D * D);
    for (auto const &it : items_) {
      std::vector<unsigned> bit(it.ids.size());
      for (size_t l = 0; l < it.ids.size(); ++l)
        bit[l] = unsigned(std::lower_bound(ids.begin(), ids.end(), it.ids[l]) - ids.begin());
      left_multiply(M, tmp, D, it, bit);
    }
    ctrl.assign(ctrls_.begin(), ctrls_.end());
  }

 private:
  // m <- [I 0; 0 m] with the new controls as the top matrix bits.
  static void embed_controls(std::vector<cplx> &m, std::vector<unsigned> &ids,
                             const std::vector<unsigned> &nc) {
    const size_t d = size_t(1) << ids.size();
    const size_t D = d << nc.size();
    std::vector<cplx> out(D * D, cplx(0., 0.));
    const size_t off = D - d;
    for (size_t i = 0; i < off; ++i) out[i * D + i] = 1.;
    for (size_t i = 0; i < d; ++i)
      for (size_t j = 0; j < d; ++j) out[(off + i) * D + off + j] = m[i * d + j];
    m.swap(out);
    ids.insert(ids.end(), nc.begin(), nc.end());
  }

  // M <- G M where G is item acting on the matrix bits `bit`.
  static void left_multiply(std::vector<cplx> &M, std::vector<cplx> &tmp, size_t D,
                            const FusedItem &it, const std::vector<unsigned> &bit) {
    const size_t k = bit.size(), d = size_t(1) << k;
    size_t gmask = 0;
    for (unsigned b : bit) gmask |= size_t(1) << b;
    std::vector<size_t> off(d, 0);
    for (size_t j = 0; j < d; ++j)
      for (size_t l = 0; l < k; ++l)
        if ((j >> l) & 1) off[j] |= size_t(1) << bit[l];
    for (size_t r = 0; r < D; ++r) {
      if (r & gmask) continue;  // r is a base row (gate bits 0)
      for (size_t a = 0; a < d; ++a) {
        cplx *dst = &tmp[(r + off[a]) * D];
        for (size_t c = 0; c < D; ++c) dst[c] = 0.;
        for (size_t b = 0; b < d; ++b) {
          const cplx g = it.m[a * d + b];
          if (g == cplx(0., 0.)) continue;
          const cplx *src = &M[(r + off[b]) * D];
          for (size_t c = 0; c < D; ++c) dst[c] += g * src[c];
        }
      }
    }
    M.swap(tmp);
  }

  std::set<unsigned> qubits_;
  std::vector<FusedItem> items_;
  std::set<unsigned> ctrls_;
};

}  // namespace gsim
