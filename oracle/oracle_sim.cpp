// ORACLE — test infrastructure only.
//
// A CPU restatement of ProjectQ's native simulator core
// (projectq/backends/_sim/_cppkernels/simulator.hpp, fusion.hpp and the
// kernels in nointrin/kernel{1..5}.hpp), written from the reference's
// algorithm, with OpenMP where the reference uses it.  It exposes the same
// C ABI as include/gb300sim.h with the prefix `osim_` instead of `gsim_`, so
// the tests can drive the CUDA engine and this oracle with the same calls.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
// this library, and only to check results or as the CPU baseline.  The product
// path (libgb300sim.so) never links or calls it.
//
// Parity pins: tests/test_oracle_cpu.py checks this oracle against the
// reference's known-answer tests (projectq/backends/_sim/_simulator_test.py)
// restated, and against fixtures produced by the reference engine itself
// (tests/golden/make_golden.py, which runs the reference's compiled _cppsim).
//
// Deliberate deviations from the reference, all on inputs the reference
// treats as undefined: an unknown qubit id raises a runtime error instead of
// being inserted into the map at bit position 0 (std::map::operator[] in
// simulator.hpp:78,95,112,150,497,554), and size mismatches that the
// reference only assert()s (simulator.hpp:196,443) raise a length error.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <random>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "../include/gb300sim.h"

namespace {

using cplx = std::complex<double>;
using StateVector = std::vector<cplx>;

thread_local std::string g_err;

// |z|^2 exactly as the reference's std::norm compiles with FMA contraction
// (libstdc++ computes x*x + y*y; g++ -O3 with FMA fuses it to fma(x, x, y*y)).
inline double norm2(const cplx &z) { return std::fma(z.real(), z.real(), z.imag() * z.imag()); }

// One queued gate: dense matrix (row-major dim x dim) on qubit ids idx
// (fusion.hpp:25-37).
struct Item {
  std::vector<cplx> m;
  std::vector<unsigned> idx;
  size_t dim() const { return size_t(1) << idx.size(); }
};

// Gate fusion, restating fusion.hpp:39-165.
struct Fusion {
  std::set<unsigned> set_;       // all qubits the fused matrix acts on
  std::vector<Item> items_;      // queued gates
  std::set<unsigned> ctrl_set_;  // controls common to every queued gate

  unsigned num_qubits() const { return unsigned(set_.size()); }
  size_t size() const { return items_.size(); }

  // fusion.hpp:112-128: embed `matrix` as the bottom-right block of a matrix
  // with the new controls as its top bits.
  static void add_controls(std::vector<cplx> &matrix, std::vector<unsigned> &idx,
                           const std::vector<unsigned> &new_ctrls) {
    size_t d = size_t(1) << idx.size();
    idx.insert(idx.end(), new_ctrls.begin(), new_ctrls.end());
    size_t F = size_t(1) << new_ctrls.size();
    size_t D = F * d;
    std::vector<cplx> nm(D * D, 0.);
    size_t off = D - d;
    for (size_t i = 0; i < off; ++i) nm[i * D + i] = 1.;
    for (size_t i = 0; i < d; ++i)
      for (size_t j = 0; j < d; ++j) nm[(off + i) * D + off + j] = matrix[i * d + j];
    matrix.swap(nm);
  }

  // fusion.hpp:130-160.
  void handle_controls(std::vector<cplx> &matrix, std::vector<unsigned> &idx,
                       const std::vector<unsigned> &ctrls) {
    std::set<unsigned> unhandled = ctrl_set_;
    for (unsigned c : ctrls) {
      if (ctrl_set_.count(c) == 0) {
        if (!items_.empty()) {
          add_controls(matrix, idx, {c});
          set_.insert(c);
        } else {
          ctrl_set_.insert(c);
        }
      } else {
        unhandled.erase(c);
      }
    }
    if (!unhandled.empty()) {
      std::vector<unsigned> nc(unhandled.begin(), unhandled.end());
      for (unsigned c : nc) {
        ctrl_set_.erase(c);
        set_.insert(c);
      }
      for (auto &it : items_) add_controls(it.m, it.idx, nc);
    }
  }

  // fusion.hpp:56-63.
  void insert(std::vector<cplx> matrix, std::vector<unsigned> idx,
              const std::vector<unsigned> &ctrls) {
    for (unsigned q : idx) set_.insert(q);
    handle_controls(matrix, idx, ctrls);
    items_.push_back(Item{std::move(matrix), std::move(idx)});
  }

  // fusion.hpp:65-109: compose all items, in order, into one dense matrix over
  // the sorted qubit set (FP64), each item left-multiplied.
  void perform_fusion(std::vector<cplx> &M, std::vector<unsigned> &ids,
                      std::vector<unsigned> &ctrls) const {
    ids.assign(set_.begin(), set_.end());
    size_t N = ids.size(), D = size_t(1) << N;
    M.assign(D * D, 0.);
    for (size_t i = 0; i < D; ++i) M[i * D + i] = 1.;
    std::vector<cplx> col(D);
    for (auto const &it : items_) {
      std::vector<size_t> pos(it.idx.size());
      for (size_t l = 0; l < it.idx.size(); ++l)
        pos[l] = size_t(std::lower_bound(ids.begin(), ids.end(), it.idx[l]) - ids.begin());
      size_t d = it.dim();
      for (size_t k = 0; k < D; ++k) {
        for (size_t i = 0; i < D; ++i) col[i] = M[i * D + k];
        for (size_t i = 0; i < D; ++i) {
          size_t li = 0;
          for (size_t l = 0; l < pos.size(); ++l) li |= ((i >> pos[l]) & 1) << l;
          cplx r = 0.;
          for (size_t j = 0; j < d; ++j) {
            size_t src = i;
            for (size_t l = 0; l < pos.size(); ++l)
              if (((j >> l) & 1) != ((i >> pos[l]) & 1)) src ^= size_t(1) << pos[l];
            r += col[src] * it.m[li * d + j];
          }
          M[i * D + k] = r;
        }
      }
    }
    ctrls.assign(ctrl_set_.begin(), ctrl_set_.end());
  }
};

struct Error {
  int code;
  std::string msg;
};
[[noreturn]] void fail(int code, const std::string &m) { throw Error{code, m}; }

struct OSim {
  unsigned N = 0;
  StateVector vec{cplx(1., 0.)};
  std::map<unsigned, unsigned> map;
  Fusion fused;
  unsigned fmin = 4, fmax = 5;  // simulator.hpp:48-49
  unsigned max_gate = 5;        // simulator.hpp:522
  int fusion_mode = GSIM_FUSION_REFERENCE;
  std::mt19937 eng;
  std::uniform_real_distribution<double> dist{0., 1.};

  explicit OSim(unsigned seed) : eng(seed) {}

  unsigned pos_of(unsigned id) const {
    auto it = map.find(id);
    if (it == map.end()) fail(GSIM_ERR_RUNTIME, "Unknown qubit id " + std::to_string(id) + ".");
    return it->second;
  }
  size_t ctrl_mask(const std::vector<unsigned> &ctrls) const {  // simulator.hpp:551-556
    size_t m = 0;
    for (unsigned c : ctrls) m |= size_t(1) << pos_of(c);
    return m;
  }
  bool check_ids(const std::vector<unsigned> &ids) const {  // simulator.hpp:558-563
    for (unsigned id : ids)
      if (!map.count(id)) return false;
    return true;
  }

  // simulator.hpp:55-74.
  void allocate_qubit(unsigned id) {
    if (map.count(id))
      fail(GSIM_ERR_RUNTIME, "AllocateQubit: ID already exists. Qubit IDs should be unique.");
    map[id] = N++;
    vec.resize(size_t(1) << N, cplx(0., 0.));
  }

  // simulator.hpp:76-91.
  bool get_classical_value(unsigned id, double tol) {
    run();
    size_t delta = size_t(1) << pos_of(id);
    for (size_t i = 0; i < vec.size(); i += 2 * delta)
      for (size_t j = 0; j < delta; ++j) {
        if (norm2(vec[i + j]) > tol) return false;
        if (norm2(vec[i + j + delta]) > tol) return true;
      }
    return false;
  }

  // simulator.hpp:93-108.
  bool is_classical(unsigned id, double tol) {
    run();
    size_t delta = size_t(1) << pos_of(id);
    int up = 0, down = 0;
    long long n = (long long)vec.size();
#pragma omp parallel for schedule(static) reduction(| : up, down)
    for (long long i = 0; i < n; i += 2 * (long long)delta)
      for (size_t j = 0; j < delta; ++j) {
        up |= norm2(vec[i + j]) > tol;
        down |= norm2(vec[i + j + delta]) > tol;
      }
    return 1 == (up ^ down);
  }

  // simulator.hpp:110-143.
  void collapse_vector(unsigned id, bool value, bool shrink) {
    run();
    unsigned pos = pos_of(id);
    size_t delta = size_t(1) << pos;
    if (!shrink) {
      for (size_t i = 0; i < vec.size(); i += 2 * delta)
        for (size_t j = 0; j < delta; ++j) vec[i + j + size_t(!value) * delta] = 0.;
      return;
    }
    StateVector nv(size_t(1) << (N - 1));
    for (size_t i = 0; i < vec.size(); i += 2 * delta)
      std::copy_n(&vec[i + size_t(value) * delta], delta, &nv[i / 2]);
    vec.swap(nv);
    for (auto &p : map)
      if (p.second > pos) p.second--;
    map.erase(id);
    N--;
  }

  // simulator.hpp:145-186; `rnd` replaces the draw of simulator.hpp:153.
  std::vector<uint8_t> measure_at(const std::vector<unsigned> &ids, double rnd) {
    run();
    std::vector<unsigned> positions(ids.size());
    for (size_t i = 0; i < ids.size(); ++i) positions[i] = pos_of(ids[i]);
    double P = 0.;
    size_t pick = 0;
    while (P < rnd && pick < vec.size()) P += norm2(vec[pick++]);
    pick--;  // wraps to SIZE_MAX when rnd == 0, as in the reference
    std::vector<uint8_t> res(ids.size());
    size_t mask = 0, val = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
      bool r = ((pick >> positions[i]) & 1) == 1;
      res[i] = r;
      mask |= size_t(1) << positions[i];
      val |= size_t(r) << positions[i];
    }
    double nrm = 0.;
    long long n = (long long)vec.size();
#pragma omp parallel for reduction(+ : nrm) schedule(static)
    for (long long i = 0; i < n; ++i) {
      if ((size_t(i) & mask) != val)
        vec[i] = 0.;
      else
        nrm += norm2(vec[i]);
    }
    nrm = 1. / std::sqrt(nrm);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) vec[i] *= nrm;
    return res;
  }
  std::vector<uint8_t> measure(const std::vector<unsigned> &ids) {
    run();
    double rnd = dist(eng);
    return measure_at(ids, rnd);
  }

  // simulator.hpp:194-202.
  void deallocate_qubit(unsigned id) {
    run();
    pos_of(id);
    if (!is_classical(id, 1e-12))
      fail(GSIM_ERR_RUNTIME,
           "Error: Qubit has not been measured / uncomputed! There is most likely a bug in "
           "your code.");
    bool value = get_classical_value(id, 1e-12);
    collapse_vector(id, value, true);
  }

  // simulator.hpp:204-222.
  void apply_controlled_gate(std::vector<cplx> m, const std::vector<unsigned> &ids,
                             const std::vector<unsigned> &ctrl) {
    for (unsigned q : ids) pos_of(q);
    for (unsigned q : ctrl) pos_of(q);
    if (fusion_mode == GSIM_FUSION_NONE) {
      fused.insert(m, ids, ctrl);
      run();
      return;
    }
    Fusion f = fused;
    f.insert(m, ids, ctrl);
    if (f.num_qubits() >= fmin && f.num_qubits() <= fmax) {
      fused = f;
      run();
    } else if (f.num_qubits() > fmax || (f.num_qubits() - ids.size()) > fused.num_qubits()) {
      run();
      fused.insert(m, ids, ctrl);
    } else {
      fused = f;
    }
  }

  // Dense controlled k-qubit gate, the semantics of nointrin/kernel{1..5}.hpp:
  // for every index I with all target bits 0 and (I & ctrlmask) == ctrlmask,
  // v = psi[I + subsets of targets]; psi[...] <- M v.  Matrix bit l <-> pos[l].
  // Loop structure as the reference's: an OpenMP loop over runs of indices
  // below the lowest target bit (contiguous in memory), unrolled in k.
  template <int K>
  void kernel_k(const std::vector<cplx> &M, const std::vector<unsigned> &pos, size_t ctrlmask) {
    constexpr size_t D = size_t(1) << K;
    std::vector<unsigned> sorted(pos.begin(), pos.end());
    std::sort(sorted.begin(), sorted.end());
    size_t off[D];
    for (size_t j = 0; j < D; ++j) {
      off[j] = 0;
      for (size_t l = 0; l < K; ++l)
        if ((j >> l) & 1) off[j] |= size_t(1) << pos[l];
    }
    double mr[D * D], mi[D * D];
    for (size_t i = 0; i < D * D; ++i) {
      mr[i] = M[i].real();
      mi[i] = M[i].imag();
    }
    const unsigned p0 = sorted[0];
    const size_t inner = size_t(1) << p0;
    const long long runs = (long long)(vec.size() >> (K + p0));
    double *psi = reinterpret_cast<double *>(vec.data());
#pragma omp parallel for schedule(static)
    for (long long r = 0; r < runs; ++r) {
      size_t base = size_t(r) << p0;
      for (unsigned p : sorted) base = ((base >> p) << (p + 1)) | (base & ((size_t(1) << p) - 1));
      for (size_t x = 0; x < inner; ++x) {
        const size_t I = base + x;
        if ((I & ctrlmask) != ctrlmask) continue;
        double vr[D], vi[D];
        for (size_t j = 0; j < D; ++j) {
          vr[j] = psi[2 * (I + off[j])];
          vi[j] = psi[2 * (I + off[j]) + 1];
        }
        for (size_t a = 0; a < D; ++a) {
          double sr = 0., si = 0.;
          for (size_t j = 0; j < D; ++j) {
            sr += mr[a * D + j] * vr[j] - mi[a * D + j] * vi[j];
            si += mr[a * D + j] * vi[j] + mi[a * D + j] * vr[j];
          }
          psi[2 * (I + off[a])] = sr;
          psi[2 * (I + off[a]) + 1] = si;
        }
      }
    }
  }
  void kernel(const std::vector<cplx> &M, const std::vector<unsigned> &pos, size_t ctrlmask) {
    switch (pos.size()) {
      case 1: return kernel_k<1>(M, pos, ctrlmask);
      case 2: return kernel_k<2>(M, pos, ctrlmask);
      case 3: return kernel_k<3>(M, pos, ctrlmask);
      case 4: return kernel_k<4>(M, pos, ctrlmask);
      case 5: return kernel_k<5>(M, pos, ctrlmask);
      default: fail(GSIM_ERR_VALUE, "Gates with more than 5 qubits are not supported!");
    }
  }

  // simulator.hpp:487-527.
  void run() {
    if (fused.size() < 1) return;
    std::vector<cplx> M;
    std::vector<unsigned> ids, ctrls;
    fused.perform_fusion(M, ids, ctrls);
    // The reference throws before it clears the queue (simulator.hpp:522-526).
    if (ids.size() > max_gate)
      fail(GSIM_ERR_VALUE, "Gates with more than 5 qubits are not supported!");
    std::vector<unsigned> pos(ids.size());
    for (size_t l = 0; l < ids.size(); ++l) pos[l] = pos_of(ids[l]);
    kernel(M, pos, ctrl_mask(ctrls));
    fused = Fusion();
  }

  // simulator.hpp:224-269, with f given as a table over the packed register
  // value (a lookup replaces the per-index callback of _cppsim.cpp:33-41).
  template <class F>
  void emulate_math(F const &f, std::vector<std::vector<unsigned>> quregs,
                    const std::vector<unsigned> &ctrl) {
    run();
    size_t cm = ctrl_mask(ctrl);
    for (auto &qr : quregs)
      for (auto &q : qr) q = pos_of(q);
    StateVector nv(vec.size(), cplx(0., 0.));
    std::vector<int> res(quregs.size());
    for (size_t i = 0; i < vec.size(); ++i) {
      if ((cm & i) == cm) {
        for (size_t r = 0; r < quregs.size(); ++r) {
          res[r] = 0;
          for (size_t b = 0; b < quregs[r].size(); ++b)
            res[r] |= int(((i >> quregs[r][b]) & 1) << b);
        }
        f(res);
        size_t ni = i;
        for (size_t r = 0; r < quregs.size(); ++r)
          for (size_t b = 0; b < quregs[r].size(); ++b)
            if (((ni >> quregs[r][b]) & 1) != size_t((res[r] >> b) & 1))
              ni ^= size_t(1) << quregs[r][b];
        nv[ni] += vec[i];
      } else {
        nv[i] += vec[i];
      }
    }
    vec.swap(nv);
  }

  // apply_term, simulator.hpp:538-550: Pauli factors through the gate path.
  void apply_term(const std::vector<std::pair<unsigned, char>> &term,
                  const std::vector<unsigned> &ids) {
    const cplx I(0., 1.);
    const std::vector<cplx> X = {0., 1., 1., 0.}, Y = {0., -I, I, 0.}, Z = {1., 0., 0., -1.};
    for (auto const &op : term) {
      if (op.first >= ids.size()) fail(GSIM_ERR_VALUE, "Pauli term index out of range.");
      const std::vector<cplx> &g = op.second == 'X' ? X : op.second == 'Y' ? Y : Z;
      apply_controlled_gate(g, {ids[op.first]}, {});
    }
    run();
  }

  // simulator.hpp:292-322.
  double get_expectation_value(
      const std::vector<std::pair<std::vector<std::pair<unsigned, char>>, double>> &td,
      const std::vector<unsigned> &ids) {
    run();
    double expectation = 0.;
    StateVector cur = vec;
    long long n = (long long)vec.size();
    for (auto const &term : td) {
      apply_term(term.first, ids);
      double delta = 0.;
#pragma omp parallel for reduction(+ : delta) schedule(static)
      for (long long i = 0; i < n; ++i) {
        delta += cur[i].real() * vec[i].real() + cur[i].imag() * vec[i].imag();
        vec[i] = cur[i];
      }
      expectation += term.second * delta;
    }
    return expectation;
  }

  // simulator.hpp:324-350.
  void apply_qubit_operator(
      const std::vector<std::pair<std::vector<std::pair<unsigned, char>>, cplx>> &td,
      const std::vector<unsigned> &ids) {
    run();
    StateVector nst(vec.size(), cplx(0., 0.)), cur = vec;
    long long n = (long long)vec.size();
    for (auto const &term : td) {
      apply_term(term.first, ids);
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < n; ++i) {
        nst[i] += term.second * vec[i];
        vec[i] = cur[i];
      }
    }
    vec.swap(nst);
  }

  // simulator.hpp:352-368.
  double get_probability(const std::vector<uint8_t> &bits, const std::vector<unsigned> &ids) {
    run();
    if (!check_ids(ids))
      fail(GSIM_ERR_RUNTIME,
           "get_probability(): Unknown qubit id. Please make sure you have called eng.flush().");
    size_t mask = 0, bs = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
      mask |= size_t(1) << map.at(ids[i]);
      bs |= size_t(bits[i] ? 1 : 0) << map.at(ids[i]);
    }
    double p = 0.;
    long long n = (long long)vec.size();
#pragma omp parallel for reduction(+ : p) schedule(static)
    for (long long i = 0; i < n; ++i)
      if ((size_t(i) & mask) == bs) p += norm2(vec[i]);
    return p;
  }

  // simulator.hpp:370-384.
  cplx get_amplitude(const std::vector<uint8_t> &bits, const std::vector<unsigned> &ids) {
    run();
    size_t chk = 0, index = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
      auto it = map.find(ids[i]);
      if (it == map.end()) break;
      chk |= size_t(1) << it->second;
      index |= size_t(bits[i] ? 1 : 0) << it->second;
    }
    if (chk + 1 != vec.size())
      fail(GSIM_ERR_RUNTIME,
           "The second argument to get_amplitude() must be a permutation of all allocated "
           "qubits. Please make sure you have called eng.flush().");
    return vec[index];
  }

  // simulator.hpp:386-438.
  void emulate_time_evolution(
      const std::vector<std::pair<std::vector<std::pair<unsigned, char>>, double>> &tdict,
      double time, const std::vector<unsigned> &ids, const std::vector<unsigned> &ctrl) {
    run();
    const cplx I(0., 1.);
    double tr = 0., op_nrm = 0.;
    std::vector<std::pair<std::vector<std::pair<unsigned, char>>, double>> td;
    for (auto const &t : tdict) {
      if (t.first.empty())
        tr += t.second;
      else {
        td.push_back(t);
        op_nrm += std::abs(t.second);
      }
    }
    unsigned s = unsigned(std::abs(time) * op_nrm + 1.);
    cplx correction = std::exp(-time * I * tr / double(s));
    StateVector out = vec;
    size_t cm = ctrl_mask(ctrl);
    long long n = (long long)vec.size();
    for (unsigned i = 0; i < s; ++i) {
      double nrm_change = 1.;
      for (unsigned k = 0; nrm_change > 1.e-12; ++k) {
        cplx coeff = (-time * I) / double(s * (k + 1));
        StateVector cur = vec;
        StateVector update(vec.size(), 0.);
        for (auto const &tup : td) {
          apply_term(tup.first, ids);
#pragma omp parallel for schedule(static)
          for (long long j = 0; j < n; ++j) {
            update[j] += vec[j] * tup.second;
            vec[j] = cur[j];
          }
        }
        nrm_change = 0.;
#pragma omp parallel for reduction(+ : nrm_change) schedule(static)
        for (long long j = 0; j < n; ++j) {
          update[j] *= coeff;
          vec[j] = update[j];
          if ((size_t(j) & cm) == cm) {
            out[j] += update[j];
            nrm_change += norm2(update[j]);
          }
        }
        nrm_change = std::sqrt(nrm_change);
      }
#pragma omp parallel for schedule(static)
      for (long long j = 0; j < n; ++j) {
        if ((size_t(j) & cm) == cm) out[j] *= correction;
        vec[j] = out[j];
      }
    }
  }

  // simulator.hpp:440-454.
  void set_wavefunction(const StateVector &wf, const std::vector<unsigned> &ordering) {
    run();
    if (map.size() != ordering.size() || !check_ids(ordering))
      fail(GSIM_ERR_RUNTIME,
           "set_wavefunction(): Invalid mapping provided. Please make sure all qubits have been "
           "allocated previously (call eng.flush()).");
    if (wf.size() != (size_t(1) << ordering.size()))
      fail(GSIM_ERR_LENGTH, "set_wavefunction(): wavefunction has the wrong length.");
    for (size_t i = 0; i < ordering.size(); ++i) map[ordering[i]] = unsigned(i);
    vec = wf;
  }

  // simulator.hpp:456-485.
  void collapse_wavefunction(const std::vector<unsigned> &ids, const std::vector<uint8_t> &vals) {
    run();
    if (ids.size() != vals.size())
      fail(GSIM_ERR_LENGTH, "collapse_wavefunction(): ids and values size mismatch");
    if (!check_ids(ids))
      fail(GSIM_ERR_RUNTIME,
           "collapse_wavefunction(): Unknown qubit id(s) provided. Try calling eng.flush() "
           "before invoking this function.");
    size_t mask = 0, val = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
      mask |= size_t(1) << map.at(ids[i]);
      val |= size_t(vals[i] ? 1 : 0) << map.at(ids[i]);
    }
    double nrm = 0.;
    long long n = (long long)vec.size();
#pragma omp parallel for reduction(+ : nrm) schedule(static)
    for (long long i = 0; i < n; ++i)
      if ((size_t(i) & mask) == val) nrm += norm2(vec[i]);
    if (nrm < 1.e-12)
      fail(GSIM_ERR_RUNTIME, "collapse_wavefunction(): Invalid collapse! Probability is ~0.");
    nrm = 1. / std::sqrt(nrm);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
      if ((size_t(i) & mask) != val)
        vec[i] = 0.;
      else
        vec[i] *= nrm;
    }
  }
};

template <class F>
int guard(F &&f) {
  try {
    f();
    return GSIM_OK;
  } catch (const Error &e) {
    g_err = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    g_err = "out of host memory";
    return GSIM_ERR_MEMORY;
  } catch (const std::exception &e) {
    g_err = e.what();
    return GSIM_ERR_RUNTIME;
  }
}

std::vector<unsigned> vec_u(const uint32_t *p, size_t n) {
  return std::vector<unsigned>(p, p + n);
}

using Term = std::vector<std::pair<unsigned, char>>;

Term term_at(const uint32_t *off, const uint32_t *q, const uint8_t *pa, size_t t) {
  Term term;
  for (uint32_t f = off[t]; f < off[t + 1]; ++f) {
    char c = char(pa[f]);
    if (c != 'X' && c != 'Y' && c != 'Z') fail(GSIM_ERR_VALUE, "Pauli must be X, Y or Z.");
    term.emplace_back(q[f], c);
  }
  return term;
}

std::vector<std::vector<unsigned>> regs_of(const uint32_t *ids, const uint32_t *sizes,
                                           size_t nregs) {
  std::vector<std::vector<unsigned>> regs(nregs);
  size_t o = 0;
  for (size_t r = 0; r < nregs; ++r)
    for (uint32_t b = 0; b < sizes[r]; ++b) regs[r].push_back(ids[o++]);
  return regs;
}

}  // namespace

extern "C" {

const char *osim_last_error(void) { return g_err.c_str(); }

int osim_create(uint32_t seed, int precision, gsim_engine **out) {
  (void)precision;
  return guard([&] { *out = reinterpret_cast<gsim_engine *>(new OSim(seed)); });
}
int osim_destroy(gsim_engine *e) {
  delete reinterpret_cast<OSim *>(e);
  return GSIM_OK;
}
#define S reinterpret_cast<OSim *>(e)
int osim_allocate_qubit(gsim_engine *e, uint32_t id) {
  return guard([&] { S->allocate_qubit(id); });
}
int osim_deallocate_qubit(gsim_engine *e, uint32_t id) {
  return guard([&] { S->deallocate_qubit(id); });
}
int osim_get_classical_value(gsim_engine *e, uint32_t id, double tol, int *out) {
  return guard([&] { *out = S->get_classical_value(id, tol); });
}
int osim_is_classical(gsim_engine *e, uint32_t id, double tol, int *out) {
  return guard([&] { *out = S->is_classical(id, tol); });
}
int osim_measure_qubits(gsim_engine *e, const uint32_t *ids, size_t n, uint8_t *out) {
  return guard([&] {
    auto r = S->measure(vec_u(ids, n));
    std::copy(r.begin(), r.end(), out);
  });
}
int osim_measure_qubits_at(gsim_engine *e, const uint32_t *ids, size_t n, double rnd,
                           uint8_t *out) {
  return guard([&] {
    auto r = S->measure_at(vec_u(ids, n), rnd);
    std::copy(r.begin(), r.end(), out);
  });
}
int osim_apply_controlled_gate(gsim_engine *e, const double *m, uint32_t k, const uint32_t *ids,
                               const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    size_t d = size_t(1) << k;
    std::vector<cplx> M(d * d);
    for (size_t i = 0; i < d * d; ++i) M[i] = cplx(m[2 * i], m[2 * i + 1]);
    S->apply_controlled_gate(M, vec_u(ids, k), vec_u(ctrl, nctrl));
  });
}
int osim_run(gsim_engine *e) {
  return guard([&] { S->run(); });
}
int osim_emulate_math_add_constant(gsim_engine *e, int32_t a, const uint32_t *reg_ids,
                                   const uint32_t *reg_sizes, size_t nregs, const uint32_t *ctrl,
                                   size_t nctrl) {
  return guard([&] {
    // simulator.hpp:275 (int arithmetic; wraps like two's complement).
    S->emulate_math(
        [a](std::vector<int> &res) {
          for (auto &x : res) x = int(uint32_t(x) + uint32_t(a));
        },
        regs_of(reg_ids, reg_sizes, nregs), vec_u(ctrl, nctrl));
  });
}
int osim_emulate_math_add_constant_modn(gsim_engine *e, int32_t a, int32_t N,
                                        const uint32_t *reg_ids, const uint32_t *reg_sizes,
                                        size_t nregs, const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    if (N == 0) fail(GSIM_ERR_VALUE, "modulus N must be nonzero");
    S->emulate_math(  // simulator.hpp:282
        [a, N](std::vector<int> &res) {
          for (auto &x : res) x = int(uint32_t(x) + uint32_t(a)) % N;
        },
        regs_of(reg_ids, reg_sizes, nregs), vec_u(ctrl, nctrl));
  });
}
int osim_emulate_math_multiply_by_constant_modn(gsim_engine *e, int32_t a, int32_t N,
                                                const uint32_t *reg_ids,
                                                const uint32_t *reg_sizes, size_t nregs,
                                                const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    if (N == 0) fail(GSIM_ERR_VALUE, "modulus N must be nonzero");
    S->emulate_math(  // simulator.hpp:289
        [a, N](std::vector<int> &res) {
          for (auto &x : res) x = int(uint32_t(x) * uint32_t(a)) % N;
        },
        regs_of(reg_ids, reg_sizes, nregs), vec_u(ctrl, nctrl));
  });
}
int osim_emulate_math_table(gsim_engine *e, const uint64_t *table, const uint32_t *reg_ids,
                            const uint32_t *reg_sizes, size_t nregs, const uint32_t *ctrl,
                            size_t nctrl) {
  return guard([&] {
    auto regs = regs_of(reg_ids, reg_sizes, nregs);
    std::vector<unsigned> shift(nregs, 0);
    for (size_t r = 1; r < nregs; ++r) shift[r] = shift[r - 1] + reg_sizes[r - 1];
    S->emulate_math(
        [&](std::vector<int> &res) {
          uint64_t x = 0;
          for (size_t r = 0; r < res.size(); ++r) x |= uint64_t(uint32_t(res[r])) << shift[r];
          uint64_t y = table[x];
          for (size_t r = 0; r < res.size(); ++r)
            res[r] = int((y >> shift[r]) & ((uint64_t(1) << reg_sizes[r]) - 1));
        },
        regs, vec_u(ctrl, nctrl));
  });
}
int osim_get_expectation_value(gsim_engine *e, const uint32_t *off, const uint32_t *q,
                               const uint8_t *pa, const double *coeffs, size_t nterms,
                               const uint32_t *ids, size_t nids, double *out) {
  return guard([&] {
    std::vector<std::pair<Term, double>> td;
    for (size_t t = 0; t < nterms; ++t) td.emplace_back(term_at(off, q, pa, t), coeffs[t]);
    *out = S->get_expectation_value(td, vec_u(ids, nids));
  });
}
int osim_apply_qubit_operator(gsim_engine *e, const uint32_t *off, const uint32_t *q,
                              const uint8_t *pa, const double *coeffs, size_t nterms,
                              const uint32_t *ids, size_t nids) {
  return guard([&] {
    std::vector<std::pair<Term, cplx>> td;
    for (size_t t = 0; t < nterms; ++t)
      td.emplace_back(term_at(off, q, pa, t), cplx(coeffs[2 * t], coeffs[2 * t + 1]));
    S->apply_qubit_operator(td, vec_u(ids, nids));
  });
}
int osim_emulate_time_evolution(gsim_engine *e, const uint32_t *off, const uint32_t *q,
                                const uint8_t *pa, const double *coeffs, size_t nterms,
                                double time, const uint32_t *ids, size_t nids,
                                const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    std::vector<std::pair<Term, double>> td;
    for (size_t t = 0; t < nterms; ++t) td.emplace_back(term_at(off, q, pa, t), coeffs[t]);
    S->emulate_time_evolution(td, time, vec_u(ids, nids), vec_u(ctrl, nctrl));
  });
}
int osim_get_probability(gsim_engine *e, const uint8_t *bits, const uint32_t *ids, size_t n,
                         double *out) {
  return guard([&] { *out = S->get_probability(std::vector<uint8_t>(bits, bits + n), vec_u(ids, n)); });
}
int osim_get_amplitude(gsim_engine *e, const uint8_t *bits, const uint32_t *ids, size_t n,
                       double *out) {
  return guard([&] {
    cplx a = S->get_amplitude(std::vector<uint8_t>(bits, bits + n), vec_u(ids, n));
    out[0] = a.real();
    out[1] = a.imag();
  });
}
int osim_set_wavefunction(gsim_engine *e, const void *wf, int dtype, size_t len,
                          const uint32_t *ordering, size_t n) {
  return guard([&] {
    StateVector v(len);
    if (dtype == GSIM_C64) {
      const float *f = static_cast<const float *>(wf);
      for (size_t i = 0; i < len; ++i) v[i] = cplx(f[2 * i], f[2 * i + 1]);
    } else {
      const double *d = static_cast<const double *>(wf);
      for (size_t i = 0; i < len; ++i) v[i] = cplx(d[2 * i], d[2 * i + 1]);
    }
    S->set_wavefunction(v, vec_u(ordering, n));
  });
}
int osim_collapse_wavefunction(gsim_engine *e, const uint32_t *ids, size_t n,
                               const uint8_t *values, size_t nvalues) {
  return guard([&] {
    S->collapse_wavefunction(vec_u(ids, n), std::vector<uint8_t>(values, values + nvalues));
  });
}
int osim_num_qubits(gsim_engine *e, uint32_t *out) {
  return guard([&] {
    S->run();
    *out = S->N;
  });
}
int osim_get_mapping(gsim_engine *e, uint32_t *ids, uint32_t *positions, size_t cap) {
  return guard([&] {
    size_t i = 0;
    for (auto const &p : S->map) {
      if (i >= cap) break;
      ids[i] = p.first;
      positions[i] = p.second;
      ++i;
    }
  });
}
int osim_get_state(gsim_engine *e, void *host, int dtype, size_t offset, size_t count) {
  return guard([&] {
    S->run();
    if (offset + count > S->vec.size()) fail(GSIM_ERR_LENGTH, "state range out of bounds");
    if (dtype == GSIM_C64) {
      float *f = static_cast<float *>(host);
      for (size_t i = 0; i < count; ++i) {
        f[2 * i] = float(S->vec[offset + i].real());
        f[2 * i + 1] = float(S->vec[offset + i].imag());
      }
    } else {
      std::memcpy(host, &S->vec[offset], count * sizeof(cplx));
    }
  });
}
int osim_set_fusion(gsim_engine *e, int mode, uint32_t kmax) {
  return guard([&] {
    S->run();
    S->fusion_mode = mode == GSIM_FUSION_NONE ? GSIM_FUSION_NONE : GSIM_FUSION_REFERENCE;
    (void)kmax;
  });
}
int osim_synchronize(gsim_engine *e) {
  (void)e;
  return GSIM_OK;
}
#undef S
}
