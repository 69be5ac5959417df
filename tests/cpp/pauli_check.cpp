// C wrappers around projectq_gb300/csrc/pauli.hpp for the CPU tests.
#include <complex>
#include <cstring>

#include "../../projectq_gb300/csrc/pauli.hpp"

extern "C" {

// Factors (pos[i], pauli[i]) in order -> xmask, zmask, ny; returns 0 on a bad character.
int pauli_term(const unsigned *pos, const char *pauli, int n, unsigned long long *x, unsigned long long *z,
               int *ny) {
  std::vector<std::pair<unsigned, char>> f;
  for (int i = 0; i < n; ++i) f.emplace_back(pos[i], pauli[i]);
  gsim::PauliTerm t;
  if (!gsim::pauli_term_of(f, t)) return 0;
  *x = t.xmask;
  *z = t.sign_mask;
  *ny = t.ny;
  return 1;
}

int paulis_commute(unsigned long long xa, unsigned long long za, unsigned long long xb, unsigned long long zb) {
  gsim::PauliTerm a, b;
  a.xmask = xa;
  a.sign_mask = za;
  b.xmask = xb;
  b.sign_mask = zb;
  return gsim::paulis_commute(a, b) ? 1 : 0;
}

// out: 2 * 4^w doubles (re, im interleaved), row-major.
void pauli_exp(unsigned w, unsigned lx, unsigned lz, double are, double aim, double bre, double bim, double *out) {
  auto m = gsim::pauli_exp_matrix(w, lx, lz, {are, aim}, {bre, bim});
  std::memcpy(out, m.data(), m.size() * sizeof(m[0]));
}

// J_0..J_K(x); returns K + 1 (0 if cap is too small).
int bessel_orders(double x, double tol, double *out, int cap) {
  auto j = gsim::bessel_j_orders(x, tol);
  if (int(j.size()) > cap) return 0;
  std::memcpy(out, j.data(), j.size() * sizeof(double));
  return int(j.size());
}
}
