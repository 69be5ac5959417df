// Host-side Pauli-string arithmetic of the engine (no CUDA headers, so a
// host-only harness can check it): the term form the kernels use, the
// commutation test, a term's exponential as a small dense gate, and the
// Bessel coefficients of the Chebyshev expansion of exp(-i tau x).
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <utility>
#include <vector>

namespace gsim {

// P = (-i)^ny X^xmask Z^sign_mask acting as
//   (P psi)_i = (-i)^ny (-1)^{popcount(i & sign_mask)} psi_{i ^ xmask}.
struct PauliTerm {
  uint64_t xmask = 0, sign_mask = 0;
  int ny = 0;          // phase (-i)^ny
  bool empty = false;  // no factors: the identity term of simulator.hpp:394-395
};

// One term from its factors (bit position, 'X' | 'Y' | 'Z') in the order
// given.  The factors are applied in that order, as apply_term does through
// the gate path (simulator.hpp:538-550), so the product is F_last ... F_first.
// It is kept as i^k X^x Z^z (per qubit X^{x_q} Z^{z_q}): Y = i X Z, and moving
// a new factor's Z past an existing X on the same qubit costs a sign.  Then
// X^x Z^z psi has (-1)^{popcount(x & z)} (-1)^{popcount(i & z)} psi_{i ^ x} at
// i.  Returns false for a character other than X, Y, Z.
inline bool pauli_term_of(const std::vector<std::pair<unsigned, char>> &factors, PauliTerm &pt) {
  pt = PauliTerm{};
  pt.empty = factors.empty();
  int k = 0;
  for (auto const &f : factors) {
    const uint64_t bit = uint64_t(1) << f.first;
    const char c = f.second;
    if (c != 'X' && c != 'Y' && c != 'Z') return false;
    const bool fx = c == 'X' || c == 'Y', fz = c == 'Z' || c == 'Y';
    if (c == 'Y') k += 1;
    if (fz && (pt.xmask & bit)) k += 2;
    if (fx) pt.xmask ^= bit;
    if (fz) pt.sign_mask ^= bit;
  }
  const int ipow = (k + 2 * (__builtin_popcountll(pt.xmask & pt.sign_mask) & 1)) & 3;
  pt.ny = (4 - ipow) & 3;  // (-i)^ny == i^ipow
  return true;
}

// Two Pauli strings commute iff their symplectic product x_a.z_b + z_a.x_b is even.
inline bool paulis_commute(const PauliTerm &a, const PauliTerm &b) {
  return ((__builtin_popcountll(a.xmask & b.sign_mask) + __builtin_popcountll(a.sign_mask & b.xmask)) & 1) == 0;
}

// a I + b X^lx Z^lz on w qubits (local bit i = i-th qubit of the support),
// row-major 2^w x 2^w, with (X^lx Z^lz)[r][r ^ lx] = (-1)^{popcount(r & lz)}.
// For exp(-i theta P), P = (-i)^ny X^x Z^z Hermitian: a = cos(theta), b =
// -i sin(theta) (-i)^ny.
inline std::vector<std::complex<double>> pauli_exp_matrix(unsigned w, uint32_t lx, uint32_t lz,
                                                          std::complex<double> a, std::complex<double> b) {
  const size_t d = size_t(1) << w;
  std::vector<std::complex<double>> m(d * d, std::complex<double>(0., 0.));
  for (size_t r = 0; r < d; ++r) {
    m[r * d + r] += a;
    m[r * d + (r ^ lx)] += (__builtin_popcount(uint32_t(r) & lz) & 1) ? -b : b;
  }
  return m;
}

// J_0(x) .. J_K(x) for x >= 0 by Miller's backward recurrence
// J_{k-1} = (2k / x) J_k - J_{k+1}, started far above x (where J decays
// super-exponentially) and normalised with J_0 + 2 sum_{k>=1} J_{2k} = 1;
// K is the first order >= x whose remaining coefficients sum, doubled, to at
// most tol.  x = 0 gives {1}.
inline std::vector<double> bessel_j_orders(double x, double tol) {
  if (!(x > 0.)) return {1.0};
  const int top = int(x + 20.0 * std::cbrt(x) + 60.0);
  const int M = top + (top & 1);
  std::vector<double> j(size_t(M) + 2, 0.0);
  j[size_t(M)] = 1e-300;
  for (int k = M; k >= 1; --k) {
    j[size_t(k) - 1] = (2.0 * k / x) * j[size_t(k)] - j[size_t(k) + 1];
    if (std::abs(j[size_t(k) - 1]) > 1e250)
      for (int i = k - 1; i <= M + 1; ++i) j[size_t(i)] *= 1e-250;
  }
  double norm = j[0];
  for (int k = 2; k <= M; k += 2) norm += 2.0 * j[size_t(k)];
  for (auto &v : j) v /= norm;
  std::vector<double> suffix(size_t(M) + 3, 0.0);
  for (int k = M + 1; k >= 0; --k) suffix[size_t(k)] = suffix[size_t(k) + 1] + std::abs(j[size_t(k)]);
  int K = int(std::ceil(x));
  while (K < M && 2.0 * suffix[size_t(K) + 1] > tol) ++K;
  j.resize(size_t(K) + 1);
  return j;
}

}  // namespace gsim
