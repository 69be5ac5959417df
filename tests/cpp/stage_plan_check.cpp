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

// The packed-pair kernel's semantics (stage_pk_kernel), read from the blob
// build_substages_pk serialises: pairs along the pack bit in swizzled pair
// order, the per-substage row / load / store offset tables, folded X gates,
// and every operation kind with the data layout the kernel reads (FP32
// broadcast pairs, evaluated here in FP64).
void apply_stage_pk(std::vector<cplx> &psi, unsigned nq, const gsim::StagePlan &sp) {
  const unsigned L = sp.L, P = unsigned(sp.pack);
  const size_t ntiles = size_t(1) << (nq - L);
  const unsigned char *blob = sp.pk.data();
  const size_t subs_bytes = (sp.pk_nsubs * sizeof(gsim::PkSubDev) + 15) & ~size_t(15);
  const auto *subs = reinterpret_cast<const gsim::PkSubDev *>(blob);
  const auto *ops = reinterpret_cast<const gsim::PkOpDev *>(blob + subs_bytes);
  struct Pair {
    cplx h[2];
  };
  std::vector<Pair> sm(4096);
  auto fl = [&](uint32_t off) { return reinterpret_cast<const float *>(blob + off); };
  for (size_t t = 0; t < ntiles; ++t) {
    size_t base = t;
    for (unsigned p : sp.lpos) base = ((base >> p) << (p + 1)) | (base & ((size_t(1) << p) - 1));
    auto gidx = [&](size_t p) {
      size_t g = base;
      for (unsigned b = 0; b < L; ++b)
        if ((p >> b) & 1) g |= size_t(1) << sp.lpos[b];
      return g;
    };
    for (size_t p = 0; p < (size_t(1) << L); ++p) {
      const uint32_t q = uint32_t(((p >> (P + 1)) << P) | (p & ((size_t(1) << P) - 1)));
      sm[gsim::pk_swizzle(q)].h[(p >> P) & 1] = psi[gidx(p)];
    }
    for (uint32_t si = 0; si < sp.pk_nsubs; ++si) {
      const gsim::PkSubDev &S = subs[si];
      if (S.tab % 16) g_inconsistent = true;
      const uint32_t *tab = reinterpret_cast<const uint32_t *>(blob + S.tab);
      for (uint32_t row = 0; row < 256; ++row) {
        const uint32_t srow = tab[row];
        uint32_t o = S.op_begin, lx = 0;
        for (; o < S.op_end && ops[o].code == gsim::kPkLoadXor; ++o)
          if ((base & ops[o].gctrl) == ops[o].gctrl && (row & ops[o].tctrl) == ops[o].tctrl) lx ^= ops[o].amask;
        Pair v[16];
        for (uint32_t jj = 0; jj < 16; ++jj) v[jj] = sm[srow ^ lx ^ tab[256 + jj]];
        uint32_t sx = 0;
        for (; o < S.op_end; ++o) {
          const gsim::PkOpDev &op = ops[o];
          const uint32_t kind = op.code & 15u, B = (op.code >> 4) & 15u, cls = (op.code >> 8) & 15u;
          const bool masked = (op.code >> 12) & 1u;
          if (kind == gsim::kPkLoadXor || kind > gsim::kPkStoreXor || (B > 3 && kind != gsim::kPkDiagN) ||
              op.data % 16)
            g_inconsistent = true;
          // the kernel tests controls only under the flag, so the flag must mark every controlled operation
          if (((op.code & gsim::kPkCtl) != 0) != (op.gctrl != 0 || op.tctrl != 0)) g_inconsistent = true;
          const bool on = !(op.code & gsim::kPkCtl) || ((base & op.gctrl) == op.gctrl && (row & op.tctrl) == op.tctrl);
          if (kind == gsim::kPkStoreXor) {
            if (on) sx ^= op.amask;
            continue;
          }
          if (!on) continue;
          if (kind == gsim::kPkDense || kind == gsim::kPkSwap) {
            cplx m[4] = {0., 1., 1., 0.};
            if (kind == gsim::kPkDense) {
              const float *d = fl(op.data);
              for (int e = 0; e < 4; ++e) {
                m[e] = cplx(d[2 * e], d[8 + 2 * e]);
                if (d[2 * e + 1] != d[2 * e] || d[16 + 2 * e] != -d[8 + 2 * e]) g_inconsistent = true;
              }
              const bool real = m[0].imag() == 0 && m[1].imag() == 0 && m[2].imag() == 0 && m[3].imag() == 0;
              const bool rx = m[0].imag() == 0 && m[3].imag() == 0 && m[1].real() == 0 && m[2].real() == 0;
              const bool anti = m[0] == cplx(0.) && m[3] == cplx(0.);
              if ((cls == 1 && !real) || (cls == 2 && !rx) || (cls == 4 && !anti)) g_inconsistent = true;
            } else {
              if (!masked && (op.amask & 0xFFFFu) == 0) g_inconsistent = true;
              // the kernel swaps the pairs of its register controls (code bits 8-11), not amask's
              uint32_t want = 0;
              for (uint32_t j = 0; j < 16; ++j)
                if (!((j >> B) & 1) && (j & cls) == cls) want |= 1u << j;
              if ((cls >> B) & 1 || want != (op.amask & 0xFFFFu) || masked != (cls != 0)) g_inconsistent = true;
            }
            for (uint32_t j = 0; j < 16; ++j) {
              if ((j >> B) & 1) continue;
              const bool c = (op.amask >> j) & 1u;
              if (!masked && kind == gsim::kPkDense && !c) g_inconsistent = true;
              if (!c) continue;
              const uint32_t k = j | (1u << B);
              for (int h = 0; h < 2; ++h) {
                const cplx a = v[j].h[h], b = v[k].h[h];
                v[j].h[h] = m[0] * a + m[1] * b;
                v[k].h[h] = m[2] * a + m[3] * b;
              }
            }
            continue;
          }
          uint32_t cidx = 0;
          for (uint32_t i = 0; i < op.nsrc; ++i) {
            const uint32_t sidx = op.src[i];
            const uint32_t bit = (sidx & 0x80u) ? uint32_t((base >> (sidx & 0x7Fu)) & 1u) : (row >> sidx) & 1u;
            cidx |= bit << op.sbit[i];
          }
          const float *T = fl(op.data);
          auto factor = [&](uint32_t idx) {
            if (T[8 * idx + 4] != -T[8 * idx + 2] || T[8 * idx + 1] != T[8 * idx]) g_inconsistent = true;
            return cplx(T[8 * idx], T[8 * idx + 2]);
          };
          for (uint32_t j = 0; j < 16; ++j) {
            uint32_t idx = cidx;
            if (kind == gsim::kPkDiag1) {
              idx |= ((j >> B) & 1u) << op.dq;
              if (op.jidx[j] != (((j >> B) & 1u) << op.dq)) g_inconsistent = true;
            } else if (kind == gsim::kPkDiagN) {
              // the kernel reads the entry of the masked bits' value
              if (op.jidx[j] != op.jidx[j & B] || __builtin_popcount(B) < 2) g_inconsistent = true;
              idx |= op.jidx[j & B];
            } else if (op.jidx[j]) {
              g_inconsistent = true;
            }
            const cplx f = factor(idx);
            v[j].h[0] *= f;
            v[j].h[1] *= f;
          }
        }
        for (uint32_t jj = 0; jj < 16; ++jj) sm[srow ^ sx ^ tab[272 + jj]] = v[jj];
      }
    }
    for (size_t p = 0; p < (size_t(1) << L); ++p) {
      const uint32_t q = uint32_t(((p >> (P + 1)) << P) | (p & ((size_t(1) << P) - 1)));
      psi[gidx(p)] = sm[gsim::pk_swizzle(q)].h[(p >> P) & 1];
    }
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

// The complex64 planning path: stages with a pack bit through the
// packed-pair semantics, the others through the register-substage ones.
extern "C" int stage_plan_apply_pk(unsigned nq, size_t ngates, const uint32_t *ks, const uint32_t *targets,
                                   const uint64_t *ctrl_masks, const double *mats, double *state,
                                   uint32_t *nstages_out, uint32_t *npk_out, uint32_t *pack_kind) {
  std::vector<gsim::StageGate> gates(ngates);
  size_t to = 0, mo = 0;
  for (size_t g = 0; g < ngates; ++g) {
    const size_t k = ks[g], d = size_t(1) << k;
    for (size_t l = 0; l < k; ++l) gates[g].pos.push_back(targets[to++]);
    gates[g].ctrl_mask = ctrl_masks[g];
    gates[g].m.resize(d * d);
    for (size_t i = 0; i < d * d; ++i, mo += 2) gates[g].m[i] = cplx(mats[mo], mats[mo + 1]);
  }
  gsim::StagePlanner planner(nq, gsim::kPkTileBits, 5, 512, true);
  auto steps = planner.plan(gates);
  std::vector<cplx> psi(size_t(1) << nq);
  for (size_t i = 0; i < psi.size(); ++i) psi[i] = cplx(state[2 * i], state[2 * i + 1]);
  uint32_t ns = 0, npk = 0;
  for (auto &st : steps) {
    if (st.is_stage) {
      if (st.stage.L == gsim::kPkTileBits && gsim::build_substages_pk(st.stage)) {
        apply_stage_pk(psi, nq, st.stage);
        ++npk;
        // pack bit: 0 = global bit 0, 1 = inside the contiguous runs, 2 = above them
        const unsigned g = st.stage.lpos[unsigned(st.stage.pack)];
        ++pack_kind[g == 0 ? 0 : g < 5 ? 1 : 2];
      } else if (st.stage.L == gsim::kPkTileBits) {
        gsim::build_substages(st.stage, 5, 4);
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
  *npk_out = npk;
  const bool bad = g_inconsistent;
  g_inconsistent = false;
  return bad ? 1 : 0;
}
