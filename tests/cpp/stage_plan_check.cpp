// Test harness (CPU): runs the stage planner of projectq_gb300/csrc/stage.hpp
// and executes every planned step with the stage kernel's semantics on the
// host, so the planner's tiling, operation merging and control handling can
// be checked against the oracle without a GPU.
#include <complex>
#include <cstdint>
#include <vector>

#include "../../projectq_gb300/csrc/stage.hpp"

using gsim::cplx;

namespace {

void apply_dense(std::vector<cplx> &psi, unsigned nq, const gsim::DenseOp &op) {
  const size_t k = op.pos.size(), d = size_t(1) << k;
  for (size_t i = 0; i < (size_t(1) << nq); ++i) {
    bool base = true;
    for (unsigned p : op.pos)
      if ((i >> p) & 1) base = false;
    if (!base || (i & op.ctrl_mask) != op.ctrl_mask) continue;
    std::vector<cplx> v(d), o(d, 0.);
    std::vector<size_t> off(d, 0);
    for (size_t j = 0; j < d; ++j)
      for (size_t l = 0; l < k; ++l)
        if ((j >> l) & 1) off[j] |= size_t(1) << op.pos[l];
    for (size_t j = 0; j < d; ++j) v[j] = psi[i + off[j]];
    for (size_t r = 0; r < d; ++r)
      for (size_t j = 0; j < d; ++j) o[r] += op.m[r * d + j] * v[j];
    for (size_t r = 0; r < d; ++r) psi[i + off[r]] = o[r];
  }
}

void apply_stage(std::vector<cplx> &psi, unsigned nq, const gsim::StagePlan &sp) {
  const unsigned L = sp.L;
  const size_t TS = size_t(1) << L, ntiles = size_t(1) << (nq - L);
  std::vector<cplx> tile(TS);
  for (size_t t = 0; t < ntiles; ++t) {
    size_t base = t;
    for (unsigned p : sp.lpos) base = ((base >> p) << (p + 1)) | (base & ((size_t(1) << p) - 1));
    auto gidx = [&](size_t p) {
      size_t g = base;
      for (unsigned b = 0; b < L; ++b)
        if ((p >> b) & 1) g |= size_t(1) << sp.lpos[b];
      return g;
    };
    for (size_t p = 0; p < TS; ++p) tile[p] = psi[gidx(p)];
    for (auto const &op : sp.ops) {
      if ((base & op.gctrl) != op.gctrl) continue;
      const cplx *M = sp.pool.data() + op.mat;
      if (op.kind == 1) {
        uint32_t cidx = 0;
        for (unsigned j = 0; j < op.k; ++j)
          if (op.tbit[j] == 0xFF) cidx |= uint32_t((base >> op.gbit[j]) & 1) << j;
        for (size_t p = 0; p < TS; ++p) {
          uint32_t idx = cidx;
          for (unsigned j = 0; j < op.k; ++j)
            if (op.tbit[j] != 0xFF) idx |= uint32_t((p >> op.tbit[j]) & 1) << j;
          tile[p] *= M[idx];
        }
        continue;
      }
      const size_t k = op.k, d = size_t(1) << k;
      for (size_t p = 0; p < TS; ++p) {
        bool base_p = true;
        for (unsigned j = 0; j < k; ++j)
          if ((p >> op.tbit[j]) & 1) base_p = false;
        if (!base_p || (p & op.lctrl) != op.lctrl) continue;
        std::vector<size_t> off(d, 0);
        for (size_t j = 0; j < d; ++j)
          for (size_t l = 0; l < k; ++l)
            if ((j >> l) & 1) off[j] |= size_t(1) << op.tbit[l];
        std::vector<cplx> v(d), o(d, 0.);
        for (size_t j = 0; j < d; ++j) v[j] = tile[p + off[j]];
        for (size_t r = 0; r < d; ++r)
          for (size_t j = 0; j < d; ++j) o[r] += M[r * d + j] * v[j];
        for (size_t r = 0; r < d; ++r) tile[p + off[r]] = o[r];
      }
    }
    for (size_t p = 0; p < TS; ++p) psi[gidx(p)] = tile[p];
  }
}

}  // namespace

extern "C" int stage_plan_apply(unsigned nq, unsigned L, unsigned m, size_t ngates, const uint32_t *ks,
                                const uint32_t *targets, const uint64_t *ctrl_masks, const double *mats,
                                double *state, uint32_t *nstages_out) {
  std::vector<gsim::StageGate> gates(ngates);
  size_t to = 0, mo = 0;
  for (size_t g = 0; g < ngates; ++g) {
    const size_t k = ks[g], d = size_t(1) << k;
    for (size_t l = 0; l < k; ++l) gates[g].pos.push_back(targets[to++]);
    gates[g].ctrl_mask = ctrl_masks[g];
    gates[g].m.resize(d * d);
    for (size_t i = 0; i < d * d; ++i, mo += 2) gates[g].m[i] = cplx(mats[mo], mats[mo + 1]);
  }
  gsim::StagePlanner planner(nq, L, m);
  auto steps = planner.plan(gates);
  std::vector<cplx> psi(size_t(1) << nq);
  for (size_t i = 0; i < psi.size(); ++i) psi[i] = cplx(state[2 * i], state[2 * i + 1]);
  uint32_t ns = 0;
  for (auto const &st : steps) {
    if (st.is_stage) {
      apply_stage(psi, nq, st.stage);
      ++ns;
    } else {
      apply_dense(psi, nq, st.dense);
    }
  }
  for (size_t i = 0; i < psi.size(); ++i) {
    state[2 * i] = psi[i].real();
    state[2 * i + 1] = psi[i].imag();
  }
  *nstages_out = ns;
  return 0;
}
