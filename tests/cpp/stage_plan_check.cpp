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

// set when a planned operation's metadata disagrees with itself; the entry
// point then returns 1
bool g_inconsistent = false;

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

// The register kernel's semantics: the tile in swizzled order, each substage
// loading 2^r amplitudes per row into "registers", applying its operations
// with register / row / non-local controls, and storing them back.
void apply_stage_substages(std::vector<cplx> &psi, unsigned nq, const gsim::StagePlan &sp) {
  const unsigned L = sp.L, r = sp.r;
  const size_t TS = size_t(1) << L, ntiles = size_t(1) << (nq - L), nrows = TS >> r;
  std::vector<cplx> smem(TS);
  for (size_t t = 0; t < ntiles; ++t) {
    size_t base = t;
    for (unsigned p : sp.lpos) base = ((base >> p) << (p + 1)) | (base & ((size_t(1) << p) - 1));
    auto gidx = [&](size_t p) {
      size_t g = base;
      for (unsigned b = 0; b < L; ++b)
        if ((p >> b) & 1) g |= size_t(1) << sp.lpos[b];
      return g;
    };
    for (size_t p = 0; p < TS; ++p) smem[gsim::tile_swizzle(uint32_t(p), sp.rho)] = psi[gidx(p)];
    for (auto const &S : sp.subs) {
      for (uint32_t row = 0; row < nrows; ++row) {
        uint32_t srow = 0;
        for (unsigned b = 0; b < L - r; ++b)
          if ((row >> b) & 1) srow ^= S.rowsw[b];
        std::vector<cplx> v(size_t(1) << r);
        uint32_t o = S.op_begin, lx = 0;
        for (; o < S.op_end && sp.sops[o].kind == 4; ++o) {  // swaps folded into the load addresses
          const gsim::SubOpDev &op = sp.sops[o];
          if (op.sdelta != S.soff[1u << op.rb[0]]) g_inconsistent = true;
          if ((base & op.gctrl) == op.gctrl && (row & op.tctrl) == op.tctrl) lx ^= op.sdelta;
        }
        for (uint32_t j = 0; j < v.size(); ++j) v[j] = smem[srow ^ lx ^ S.soff[j]];
        uint32_t sx = 0;
        for (; o < S.op_end; ++o) {
          const gsim::SubOpDev &op = sp.sops[o];
          if (op.kind == 4) g_inconsistent = true;  // load folds must lead the list
          if ((base & op.gctrl) != op.gctrl) continue;
          if ((row & op.tctrl) != op.tctrl) continue;
          if (op.kind == 3) {  // swap folded into the store addresses
            if (op.sdelta != S.soff[1u << op.rb[0]]) g_inconsistent = true;
            sx ^= op.sdelta;
            continue;
          }
          const cplx *M = sp.pool.data() + op.mat;
          if (op.kind == 2) {
            // the kernel's three paths: one factor (no register qubit), two
            // factors selected by register bit dB (one), a table (more)
            uint32_t cidx = 0;
            unsigned nreg = 0;
            for (unsigned q = 0; q < op.dk; ++q) {
              if (op.dloc[q] == 0) ++nreg;
              else if (op.dloc[q] == 1) cidx |= ((row >> op.didx[q]) & 1u) << q;
              else cidx |= uint32_t((base >> op.didx[q]) & 1) << q;
            }
            if (nreg != op.dreg) g_inconsistent = true;
            for (uint32_t j = 0; j < v.size(); ++j) {
              uint32_t idx = cidx;
              if (op.dreg == 1) {
                idx |= ((j >> op.dB) & 1u) << op.dq;
              } else if (op.dreg > 1) {
                for (unsigned q = 0; q < op.dk; ++q)
                  if (op.dloc[q] == 0) idx |= ((j >> op.didx[q]) & 1u) << q;
              }
              v[j] *= M[idx];
            }
          } else if (op.kind == 0) {
            // the kernel's 1-qubit paths: group bases from amask, one formula per class
            const unsigned B = op.rb[0];
            const cplx m00 = M[0], m01 = M[1], m10 = M[2], m11 = M[3];
            for (uint32_t j = 0; j < v.size(); ++j) {
              if ((j >> B) & 1) continue;
              if (!((op.amask >> j) & 1)) continue;
              const cplx a = v[j], b = v[j | (1u << B)];
              cplx o0, o1;
              if (op.cls == 3) {
                o0 = b;
                o1 = a;
              } else if (op.cls == 1) {
                o0 = cplx(m00.real() * a.real() + m01.real() * b.real(), m00.real() * a.imag() + m01.real() * b.imag());
                o1 = cplx(m10.real() * a.real() + m11.real() * b.real(), m10.real() * a.imag() + m11.real() * b.imag());
              } else if (op.cls == 2) {
                o0 = cplx(m00.real() * a.real() - m01.imag() * b.imag(), m00.real() * a.imag() + m01.imag() * b.real());
                o1 = cplx(-m10.imag() * a.imag() + m11.real() * b.real(), m10.imag() * a.real() + m11.real() * b.imag());
              } else if (op.cls == 4) {
                o0 = m01 * b;
                o1 = m10 * a;
              } else {
                o0 = m00 * a + m01 * b;
                o1 = m10 * a + m11 * b;
              }
              v[j] = o0;
              v[j | (1u << B)] = o1;
            }
          } else {
            const unsigned k = op.kind == 0 ? 1 : 2, d = 1u << k;
            uint32_t tm = 0;
            for (unsigned q = 0; q < k; ++q) tm |= 1u << op.rb[q];
            for (uint32_t j = 0; j < v.size(); ++j) {
              if ((j & tm) || !((op.amask >> j) & 1)) continue;
              std::vector<uint32_t> jj(d);
              for (uint32_t a = 0; a < d; ++a) {
                jj[a] = j;
                for (unsigned q = 0; q < k; ++q)
                  if ((a >> q) & 1) jj[a] |= 1u << op.rb[q];
              }
              std::vector<cplx> x(d), y(d, 0.);
              for (uint32_t a = 0; a < d; ++a) x[a] = v[jj[a]];
              for (uint32_t a = 0; a < d; ++a)
                for (uint32_t b = 0; b < d; ++b) y[a] += M[a * d + b] * x[b];
              for (uint32_t a = 0; a < d; ++a) v[jj[a]] = y[a];
            }
          }
        }
        for (uint32_t j = 0; j < v.size(); ++j) smem[srow ^ sx ^ S.soff[j]] = v[j];
      }
    }
    for (size_t p = 0; p < TS; ++p) psi[gidx(p)] = smem[gsim::tile_swizzle(uint32_t(p), sp.rho)];
  }
}

}  // namespace

extern "C" int stage_plan_apply(unsigned nq, unsigned L, unsigned m, unsigned r, unsigned rho, size_t ngates,
                                const uint32_t *ks,
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
  for (auto &st : steps) {
    if (st.is_stage) {
      if (r > 0 && st.stage.L > r) {
        gsim::build_substages(st.stage, r, rho);
        apply_stage_substages(psi, nq, st.stage);
      } else {
        apply_stage(psi, nq, st.stage);
      }
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
  const bool bad = g_inconsistent;
  g_inconsistent = false;
  return bad ? 1 : 0;
}

// Number of operations in the planned stages (after merging) and of stages.
extern "C" int stage_plan_count_ops(unsigned nq, unsigned L, unsigned m, size_t ngates, const uint32_t *ks,
                                    const uint32_t *targets, const uint64_t *ctrl_masks, const double *mats,
                                    uint32_t *nops_out, uint32_t *nstages_out) {
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
  uint32_t nops = 0, ns = 0;
  for (auto &st : planner.plan(gates))
    if (st.is_stage) {
      nops += uint32_t(st.stage.ops.size());
      ++ns;
    }
  *nops_out = nops;
  *nstages_out = ns;
  return 0;
}
