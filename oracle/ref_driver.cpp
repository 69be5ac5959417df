// ORACLE (reference build) — test infrastructure only.
//
// A thin extern "C" driver around the reference engine itself: it includes
// ProjectQ's projectq/backends/_sim/_cppkernels/simulator.hpp from the
// reference tree (the include path is given by oracle/build_ref.sh; no
// reference source is copied into this repository) and exposes the same
// entry points as oracle/oracle_sim.cpp under the prefix `rsim_`.  The
// shared library lands in oracle/_ref/, which is not committed.  It is used
// on the CPU to pin the oracle restatement and to generate golden fixtures.

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "simulator.hpp"

namespace {
thread_local std::string g_err;
using cplx = std::complex<double>;
using MatrixType = std::vector<std::vector<cplx, aligned_allocator<cplx, 64>>>;
using QuRegs = std::vector<std::vector<unsigned>>;

template <class F>
int guard(F &&f) {
  try {
    f();
    return 0;
  } catch (const std::length_error &e) {
    g_err = e.what();
    return 3;
  } catch (const std::invalid_argument &e) {
    g_err = e.what();
    return 2;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}
std::vector<unsigned> vu(const uint32_t *p, size_t n) { return std::vector<unsigned>(p, p + n); }
QuRegs regs_of(const uint32_t *ids, const uint32_t *sizes, size_t nregs) {
  QuRegs regs(nregs);
  size_t o = 0;
  for (size_t r = 0; r < nregs; ++r)
    for (uint32_t b = 0; b < sizes[r]; ++b) regs[r].push_back(ids[o++]);
  return regs;
}
Simulator::Term term_at(const uint32_t *off, const uint32_t *q, const uint8_t *pa, size_t t) {
  Simulator::Term term;
  for (uint32_t f = off[t]; f < off[t + 1]; ++f) term.emplace_back(q[f], char(pa[f]));
  return term;
}
}  // namespace

#define S reinterpret_cast<Simulator *>(e)
extern "C" {
const char *rsim_last_error(void) { return g_err.c_str(); }
int rsim_create(uint32_t seed, int, void **out) {
  return guard([&] { *out = new Simulator(seed); });
}
int rsim_destroy(void *e) {
  delete S;
  return 0;
}
int rsim_allocate_qubit(void *e, uint32_t id) {
  return guard([&] { S->allocate_qubit(id); });
}
int rsim_deallocate_qubit(void *e, uint32_t id) {
  return guard([&] { S->deallocate_qubit(id); });
}
int rsim_get_classical_value(void *e, uint32_t id, double tol, int *out) {
  return guard([&] { *out = S->get_classical_value(id, tol); });
}
int rsim_is_classical(void *e, uint32_t id, double tol, int *out) {
  return guard([&] { *out = S->is_classical(id, tol); });
}
int rsim_measure_qubits(void *e, const uint32_t *ids, size_t n, uint8_t *out) {
  return guard([&] {
    auto r = S->measure_qubits_return(vu(ids, n));
    for (size_t i = 0; i < n; ++i) out[i] = r[i];
  });
}
int rsim_apply_controlled_gate(void *e, const double *m, uint32_t k, const uint32_t *ids,
                               const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    size_t d = size_t(1) << k;
    MatrixType M(d);
    for (size_t i = 0; i < d; ++i) {
      M[i].resize(d);
      for (size_t j = 0; j < d; ++j) M[i][j] = cplx(m[2 * (i * d + j)], m[2 * (i * d + j) + 1]);
    }
    S->apply_controlled_gate(M, vu(ids, k), vu(ctrl, nctrl));
  });
}
int rsim_run(void *e) {
  return guard([&] { S->run(); });
}
int rsim_emulate_math_add_constant(void *e, int32_t a, const uint32_t *ri, const uint32_t *rs,
                                   size_t nr, const uint32_t *c, size_t nc) {
  return guard([&] { S->emulate_math_addConstant(a, regs_of(ri, rs, nr), vu(c, nc)); });
}
int rsim_emulate_math_add_constant_modn(void *e, int32_t a, int32_t N, const uint32_t *ri,
                                        const uint32_t *rs, size_t nr, const uint32_t *c,
                                        size_t nc) {
  return guard([&] { S->emulate_math_addConstantModN(a, N, regs_of(ri, rs, nr), vu(c, nc)); });
}
int rsim_emulate_math_multiply_by_constant_modn(void *e, int32_t a, int32_t N,
                                                const uint32_t *ri, const uint32_t *rs,
                                                size_t nr, const uint32_t *c, size_t nc) {
  return guard(
      [&] { S->emulate_math_multiplyByConstantModN(a, N, regs_of(ri, rs, nr), vu(c, nc)); });
}
int rsim_emulate_math_table(void *e, const uint64_t *table, const uint32_t *ri,
                            const uint32_t *rs, size_t nr, const uint32_t *c, size_t nc) {
  return guard([&] {
    std::vector<unsigned> shift(nr, 0);
    for (size_t r = 1; r < nr; ++r) shift[r] = shift[r - 1] + rs[r - 1];
    auto f = [&](std::vector<int> &res) {
      uint64_t x = 0;
      for (size_t r = 0; r < res.size(); ++r) x |= uint64_t(uint32_t(res[r])) << shift[r];
      uint64_t y = table[x];
      for (size_t r = 0; r < res.size(); ++r)
        res[r] = int((y >> shift[r]) & ((uint64_t(1) << rs[r]) - 1));
    };
    S->emulate_math(f, regs_of(ri, rs, nr), vu(c, nc));
  });
}
int rsim_get_expectation_value(void *e, const uint32_t *off, const uint32_t *q,
                               const uint8_t *pa, const double *coeffs, size_t nterms,
                               const uint32_t *ids, size_t nids, double *out) {
  return guard([&] {
    Simulator::TermsDict td;
    for (size_t t = 0; t < nterms; ++t) td.emplace_back(term_at(off, q, pa, t), coeffs[t]);
    *out = S->get_expectation_value(td, vu(ids, nids));
  });
}
int rsim_apply_qubit_operator(void *e, const uint32_t *off, const uint32_t *q, const uint8_t *pa,
                              const double *coeffs, size_t nterms, const uint32_t *ids,
                              size_t nids) {
  return guard([&] {
    Simulator::ComplexTermsDict td;
    for (size_t t = 0; t < nterms; ++t)
      td.emplace_back(term_at(off, q, pa, t), cplx(coeffs[2 * t], coeffs[2 * t + 1]));
    S->apply_qubit_operator(td, vu(ids, nids));
  });
}
int rsim_emulate_time_evolution(void *e, const uint32_t *off, const uint32_t *q,
                                const uint8_t *pa, const double *coeffs, size_t nterms,
                                double time, const uint32_t *ids, size_t nids,
                                const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    Simulator::TermsDict td;
    for (size_t t = 0; t < nterms; ++t) td.emplace_back(term_at(off, q, pa, t), coeffs[t]);
    S->emulate_time_evolution(td, time, vu(ids, nids), vu(ctrl, nctrl));
  });
}
int rsim_get_probability(void *e, const uint8_t *bits, const uint32_t *ids, size_t n,
                         double *out) {
  return guard([&] {
    std::vector<bool> b(bits, bits + n);
    *out = S->get_probability(b, vu(ids, n));
  });
}
int rsim_get_amplitude(void *e, const uint8_t *bits, const uint32_t *ids, size_t n,
                       double *out) {
  return guard([&] {
    std::vector<bool> b(bits, bits + n);
    auto a = S->get_amplitude(b, vu(ids, n));
    out[0] = a.real();
    out[1] = a.imag();
  });
}
int rsim_set_wavefunction(void *e, const void *wf, int, size_t len, const uint32_t *ordering,
                          size_t n) {
  return guard([&] {
    Simulator::StateVector v(len);
    std::memcpy(v.data(), wf, len * sizeof(cplx));
    S->set_wavefunction(v, vu(ordering, n));
  });
}
int rsim_collapse_wavefunction(void *e, const uint32_t *ids, size_t n, const uint8_t *values,
                               size_t nvalues) {
  return guard([&] {
    std::vector<bool> v(values, values + nvalues);
    S->collapse_wavefunction(vu(ids, n), v);
  });
}
int rsim_num_qubits(void *e, uint32_t *out) {
  return guard([&] { *out = unsigned(std::get<0>(S->cheat()).size()); });
}
int rsim_get_mapping(void *e, uint32_t *ids, uint32_t *pos, size_t cap) {
  return guard([&] {
    auto m = std::get<0>(S->cheat());
    size_t i = 0;
    for (auto const &p : m) {
      if (i >= cap) break;
      ids[i] = p.first;
      pos[i] = p.second;
      ++i;
    }
  });
}
int rsim_get_state(void *e, void *host, int, size_t offset, size_t count) {
  return guard([&] {
    auto &v = std::get<1>(S->cheat());
    if (offset + count > v.size()) throw std::length_error("state range out of bounds");
    std::memcpy(host, v.data() + offset, count * sizeof(cplx));
  });
}
int rsim_synchronize(void *) { return 0; }
}
