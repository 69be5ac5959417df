// GB300 state-vector engine: host logic and the C ABI of include/gb300sim.h.
//
// The engine owns one state vector in device memory (complex128 or
// complex64), the qubit-id -> bit-position map, the pending-gate queue and
// one CUDA stream.  Every method mirrors a method of the reference engine
// (projectq/backends/_sim/_cppkernels/simulator.hpp), cited at each one; the
// data paths are GB300 kernels (kernels_gate.cu, kernels_state.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <unordered_map>
#include <random>
#include <set>
#include <string>
#include <vector>

#include "../../include/gb300sim.h"
#include "fusion.hpp"
#include "kernels.hpp"
#include "pauli.hpp"
#include "stage.hpp"

namespace gsim {

struct Error {
  int code;
  std::string msg;
};
[[noreturn]] void fail(int code, const std::string &m) { throw Error{code, m}; }

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess)                                                           \
      fail(GSIM_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e_) +     \
                              " (" #x ")");                                          \
  } while (0)

thread_local std::string g_last_error;

// Device buffer that grows on demand (never shrinks until the engine dies).
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  void *get(size_t need) {
    if (need > bytes) {
      if (p) CK(cudaFree(p));
      p = nullptr;
      bytes = 0;
      if (cudaMalloc(&p, need) != cudaSuccess) {
        cudaGetLastError();
        fail(GSIM_ERR_MEMORY, "cudaMalloc of " + std::to_string(need) + " bytes failed");
      }
      bytes = need;
    }
    return p;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};
struct HostBuf {
  void *p = nullptr;
  size_t bytes = 0;
  void *get(size_t need) {
    if (need > bytes) {
      if (p) cudaFreeHost(p);
      p = nullptr;
      bytes = 0;
      if (cudaMallocHost(&p, need) != cudaSuccess) {
        cudaGetLastError();
        fail(GSIM_ERR_MEMORY, "cudaMallocHost failed");
      }
      bytes = need;
    }
    return p;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
};

class Engine {
 public:
  Engine(uint32_t seed, int prec) : prec_(prec), bpa_(prec == GSIM_C64 ? 8 : 16), rng_(seed) {
    if (prec != GSIM_C64 && prec != GSIM_C128) fail(GSIM_ERR_VALUE, "unknown precision");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      fail(GSIM_ERR_CUDA, "no CUDA device available");
    }
    CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    ensure_capacity(0);
    set_basis_zero();
  }
  ~Engine() {
    if (stream_) cudaStreamSynchronize(stream_);
    for (cudaEvent_t ev : timer_)
      if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : ev_pool_) cudaEventDestroy(ev);
    for (DevBuf *b : {&state_, &scratch_, &part_, &small_, &aux1_, &aux2_, &aux3_, &table_, &table2_, &upload_dev_})
      b->release();
    pinned_.release();
    for (int k = 0; k < kUploadSlots; ++k) {
      upload_host_[k].release();
      if (upload_ev_[k]) cudaEventDestroy(upload_ev_[k]);
    }
    for (UploadSlot &sl : mslots_) {
      sl.dev.release();
      sl.host.release();
      if (sl.ev) cudaEventDestroy(sl.ev);
    }
    if (stream_) cudaStreamDestroy(stream_);
  }

  // ---- simulator.hpp:55-74 ------------------------------------------------
  void allocate_qubit(unsigned id) {
    if (map_.count(id))
      fail(GSIM_ERR_RUNTIME, "AllocateQubit: ID already exists. Qubit IDs should be unique.");
    if (N_ >= 40) fail(GSIM_ERR_MEMORY, "too many qubits");
    ensure_capacity(N_ + 1);
    const size_t half = size_t(1) << N_;
    CK(cudaMemsetAsync(static_cast<char *>(state_.p) + half * bpa_, 0, half * bpa_, stream_));
    map_[id] = N_++;
  }

  // ---- simulator.hpp:194-202 ----------------------------------------------
  void deallocate_qubit(unsigned id) {
    run();
    const unsigned pos = pos_of(id);
    if (!is_classical(id, 1e-12))
      fail(GSIM_ERR_RUNTIME,
           "Error: Qubit has not been measured / uncomputed! There is most likely a bug in your "
           "code.");
    const bool value = get_classical_value(id, 1e-12);
    // collapse_vector(id, value, shrink=true), simulator.hpp:110-143.
    if (pos == N_ - 1) {
      if (value) {
        const size_t half = size_t(1) << (N_ - 1);
        CK(cudaMemcpyAsync(state_.p, static_cast<char *>(state_.p) + half * bpa_, half * bpa_,
                           cudaMemcpyDeviceToDevice, stream_));
      }
    } else {
      void *dst = scratch();
      CK(launch_shrink(prec_, state_.p, dst, N_, pos, value ? 1 : 0, stream_));
      std::swap(state_, scratch_);
    }
    for (auto &p : map_)
      if (p.second > pos) p.second--;
    map_.erase(id);
    N_--;
  }

  // ---- simulator.hpp:76-91 ------------------------------------------------
  bool get_classical_value(unsigned id, double tol) {
    run();
    const unsigned pos = pos_of(id);
    if (N_ == 0) return false;
    auto *d_first = static_cast<unsigned long long *>(small_.get(4096));
    CK(cudaMemsetAsync(d_first, 0xff, sizeof(unsigned long long), stream_));
    CK(launch_classical_first(prec_, state_.p, N_, pos, tol, d_first, stream_));
    unsigned long long first = 0;
    CK(cudaMemcpyAsync(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    if (first == ~0ull) return false;  // unreachable for a normalised state
    const uint64_t lo = ((first >> pos) << (pos + 1)) | (first & ((uint64_t(1) << pos) - 1));
    return !(norm2_at(lo) > tol);
  }

  // ---- simulator.hpp:93-108 -----------------------------------------------
  bool is_classical(unsigned id, double tol) {
    run();
    const unsigned pos = pos_of(id);
    if (N_ == 0) return false;
    int *d_flags = static_cast<int *>(small_.get(4096));
    CK(cudaMemsetAsync(d_flags, 0, 2 * sizeof(int), stream_));
    CK(launch_classical_flags(prec_, state_.p, N_, pos, tol, d_flags, stream_));
    int f[2];
    CK(cudaMemcpyAsync(f, d_flags, sizeof(f), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    return 1 == (f[0] ^ f[1]);
  }

  // ---- simulator.hpp:145-186 ----------------------------------------------
  std::vector<uint8_t> measure(const std::vector<unsigned> &ids, bool have_rnd, double rnd) {
    run();
    std::vector<unsigned> positions(ids.size());
    for (size_t i = 0; i < ids.size(); ++i) positions[i] = pos_of(ids[i]);
    if (!have_rnd) rnd = dist_(rng_);
    const uint64_t pick = sample(rnd);
    std::vector<uint8_t> res(ids.size());
    uint64_t mask = 0, val = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
      const bool r = ((pick >> positions[i]) & 1) == 1;
      res[i] = r;
      mask |= uint64_t(1) << positions[i];
      val |= uint64_t(r) << positions[i];
    }
    double *d_norm = static_cast<double *>(small_.get(4096));
    CK(launch_masked_norm(prec_, state_.p, N_, mask, val, part(), d_norm, stream_));
    CK(launch_project_scale(prec_, state_.p, N_, mask, val, d_norm, stream_));
    return res;
  }

  // ---- simulator.hpp:204-222 ----------------------------------------------
  void apply_controlled_gate(std::vector<cplx> m, const std::vector<unsigned> &ids,
                             const std::vector<unsigned> &ctrl) {
    if (ids.empty()) fail(GSIM_ERR_VALUE, "apply_controlled_gate(): a gate needs target qubits");
    std::set<unsigned> seen;
    for (unsigned q : ids) {
      pos_of(q);
      if (!seen.insert(q).second) fail(GSIM_ERR_VALUE, "apply_controlled_gate(): repeated target qubit");
    }
    for (unsigned q : ctrl) {
      pos_of(q);
      if (!seen.insert(q).second)
        fail(GSIM_ERR_VALUE, "apply_controlled_gate(): a control is also a target or repeated");
    }
    counters_[0] += 1;
    submit_gate(std::move(m), ids, ctrl);
  }
  // Queue (or fuse, or run) a validated gate under the current fusion mode.
  void submit_gate(std::vector<cplx> m, const std::vector<unsigned> &ids, const std::vector<unsigned> &ctrl) {
    if (mode_ == GSIM_FUSION_STAGED || mode_ == GSIM_FUSION_LEARNED) {
      queue_.push_back(QueuedGate{std::move(m), ids, ctrl});
      if (queue_.size() >= kMaxQueue) run();
      return;
    }
    if (mode_ == GSIM_FUSION_NONE) {
      fused_.insert(std::move(m), ids, ctrl);
      run();
      return;
    }
    RefFusion f = fused_;
    f.insert(m, ids, ctrl);
    const unsigned nf = f.num_qubits();
    if (nf >= fmin_ && nf <= fmax_) {
      fused_ = std::move(f);
      run();
    } else if (nf > fmax_ || (nf - unsigned(ids.size())) > fused_.num_qubits()) {
      run();
      fused_.insert(std::move(m), ids, ctrl);
    } else {
      fused_ = std::move(f);
    }
  }

  // ---- simulator.hpp:487-527 ----------------------------------------------
  void run() {
    run_planned();
    if (tc_used_) {
      // a tensor-core launch records a timeout in a device flag: check it here
      int h = 0;
      int *d_err = reinterpret_cast<int *>(static_cast<char *>(small_.get(4096)) + 2048);
      CK(cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream_));
      CK(cudaStreamSynchronize(stream_));
      tc_used_ = false;
      if (h) fail(GSIM_ERR_CUDA, "tensor-core gate kernel: the MMA completion wait timed out");
    }
  }

  void run_planned() {
    if (mode_ == GSIM_FUSION_STAGED) {
      run_staged();
      return;
    }
    if (mode_ == GSIM_FUSION_LEARNED) {
      run_learned();
      return;
    }
    if (fused_.size() < 1) return;
    std::vector<cplx> M;
    std::vector<unsigned> ids, ctrls;
    fused_.compose(M, ids, ctrls);
    const unsigned limit = mode_ == GSIM_FUSION_REFERENCE ? std::max(max_gate_, fmax_) : 7u;
    if (ids.size() > limit)
      fail(GSIM_ERR_VALUE, "Gates with more than " + std::to_string(limit) +
                               " qubits are not supported!");
    DenseOp op;
    op.m = std::move(M);
    for (unsigned q : ids) op.pos.push_back(pos_of(q));
    for (unsigned c : ctrls) op.ctrl_mask |= uint64_t(1) << pos_of(c);
    fused_ = RefFusion();
    exec_dense(op);
  }

  // ---- simulator.hpp:224-290 ----------------------------------------------
  // f maps the packed register value to the packed result (per-register
  // results already truncated to their widths).
  template <class F>
  void emulate_math(F const &f, const std::vector<unsigned> &reg_ids,
                    const std::vector<unsigned> &reg_sizes, const std::vector<unsigned> &ctrl) {
    run();
    uint64_t cm = 0;
    for (unsigned c : ctrl) cm |= uint64_t(1) << pos_of(c);
    MathRegsDev R;
    std::memset(&R, 0, sizeof(R));
    unsigned W = 0;
    for (unsigned s : reg_sizes) W += s;
    if (W != reg_ids.size()) fail(GSIM_ERR_VALUE, "emulate_math(): register sizes do not match ids");
    if (W > 26) fail(GSIM_ERR_VALUE, "emulate_math(): at most 26 register qubits are supported");
    uint64_t used = 0;
    for (unsigned b = 0; b < W; ++b) {
      const unsigned p = pos_of(reg_ids[b]);
      if ((used >> p) & 1) fail(GSIM_ERR_VALUE, "emulate_math(): repeated register qubit");
      if ((cm >> p) & 1) fail(GSIM_ERR_VALUE, "emulate_math(): a control qubit is in a register");
      used |= uint64_t(1) << p;
      R.pos[b] = uint8_t(p);
    }
    R.width = int(W);
    R.ctrl = cm;
    const size_t T = size_t(1) << W;
    std::vector<uint32_t> table(T);
    std::vector<uint32_t> count(T, 0);
    for (size_t x = 0; x < T; ++x) {
      table[x] = uint32_t(f(uint64_t(x)) & (T - 1));
      count[table[x]]++;
    }
    bool bijective = true;
    for (size_t y = 0; y < T && bijective; ++y) bijective = count[y] == 1;
    void *dst = scratch();
    if (bijective) {
      auto *d_table = static_cast<uint32_t *>(table_.get(T * 4));
      CK(cudaMemcpyAsync(d_table, table.data(), T * 4, cudaMemcpyHostToDevice, stream_));
      CK(launch_math_scatter(prec_, state_.p, dst, N_, R, d_table, stream_));
    } else {
      // Inverse lists, each sorted by the sources' bit pattern in the state
      // index: the reference accumulates colliding amplitudes in index order.
      std::vector<uint64_t> off(T + 1, 0);
      for (size_t y = 0; y < T; ++y) off[y + 1] = off[y] + count[y];
      std::vector<uint32_t> src(T);
      std::vector<uint64_t> fill(off.begin(), off.end() - 1);
      std::vector<uint32_t> order(T);
      for (size_t x = 0; x < T; ++x) order[x] = uint32_t(x);
      auto key = [&](uint32_t x) {
        uint64_t k = 0;
        for (unsigned b = 0; b < W; ++b) k |= uint64_t((x >> b) & 1) << R.pos[b];
        return k;
      };
      std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key(a) < key(b); });
      for (uint32_t x : order) src[fill[table[x]]++] = x;
      auto *d_off = static_cast<uint64_t *>(table_.get((T + 1) * 8));
      auto *d_src = static_cast<uint32_t *>(table2_.get(T * 4));
      CK(cudaMemcpyAsync(d_off, off.data(), (T + 1) * 8, cudaMemcpyHostToDevice, stream_));
      CK(cudaMemcpyAsync(d_src, src.data(), T * 4, cudaMemcpyHostToDevice, stream_));
      CK(launch_math_gather(prec_, state_.p, dst, N_, R, d_off, d_src, stream_));
    }
    std::swap(state_, scratch_);
    // The host tables must outlive the asynchronous copies.
    CK(cudaStreamSynchronize(stream_));
  }

  // ---- simulator.hpp:292-322 ----------------------------------------------
  double get_expectation_value(const std::vector<PauliTerm> &terms, const std::vector<double> &coeffs) {
    run();
    const int nt = int(terms.size());
    if (nt == 0) return 0.;
    const int nblk = pauli_expect_blocks(N_);
    double *d_part = static_cast<double *>(aux1_.get(size_t(nt) * nblk * 8));
    double *d_out = static_cast<double *>(aux2_.get(size_t(nt) * 8));
    // Group terms by flip mask: one read pass of the state per group.
    std::map<uint64_t, std::vector<int>> groups;
    for (int t = 0; t < nt; ++t) groups[terms[t].xmask].push_back(t);
    // Columns are laid out group by group; remember each term's column.
    std::vector<int> col(nt);
    int c0 = 0;
    for (auto const &g : groups) {
      std::vector<PauliTermDev> dev;
      for (int t : g.second) {
        col[t] = c0 + int(dev.size());
        dev.push_back(PauliTermDev{terms[t].sign_mask, terms[t].ny & 3, 0});
      }
      CK(launch_pauli_expect(prec_, state_.p, N_, g.first, dev.data(), int(dev.size()),
                             d_part + size_t(c0) * nblk, nblk, stream_));
      c0 += int(dev.size());
    }
    CK(launch_column_sums(d_part, nblk, nt, d_out, stream_));
    std::vector<double> delta(nt);
    CK(cudaMemcpyAsync(delta.data(), d_out, nt * 8, cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    double e = 0.;
    for (int t = 0; t < nt; ++t) e += coeffs[t] * delta[col[t]];
    return e;
  }

  // ---- simulator.hpp:324-350 ----------------------------------------------
  void apply_qubit_operator(const std::vector<PauliTerm> &terms, const std::vector<cplx> &coeffs) {
    run();
    std::vector<PauliApplyTermDev> dev(terms.size());
    for (size_t t = 0; t < terms.size(); ++t) dev[t] = apply_term_dev(terms[t], coeffs[t]);
    auto *d_terms = static_cast<PauliApplyTermDev *>(aux3_.get(std::max<size_t>(1, dev.size()) * sizeof(PauliApplyTermDev)));
    if (!dev.empty())
      CK(cudaMemcpyAsync(d_terms, dev.data(), dev.size() * sizeof(dev[0]), cudaMemcpyHostToDevice, stream_));
    void *dst = scratch();
    CK(launch_pauli_apply(prec_, state_.p, dst, N_, d_terms, int(dev.size()), stream_));
    std::swap(state_, scratch_);
    CK(cudaStreamSynchronize(stream_));
  }

  // exp(-i t H) for H = sum_k c_k P_k whose terms commute pairwise, as the
  // exact product of exp(-i t c_k P_k) = cos(t c_k) I - i sin(t c_k) P_k --
  // what ProjectQ's commuting-terms decomposition
  // (setups/decompositions/time_evolution.py:28-52) expresses in gates --
  // without the Taylor series.  A term on at most kTermGateQubits qubits
  // becomes one controlled gate on its support, queued for the planner, so
  // many terms share a pass over the state (ZZ and Z terms are diagonal gates);
  // a wider term is one pass of the rotation kernel.  The identity terms'
  // phase exp(-i t tr) goes into the first exponential.  Returns false (and
  // does nothing) unless every term commutes with every other and none acts
  // on a control qubit.
  static constexpr unsigned kTermGateQubits = 5;
  bool evolve_commuting(const std::vector<PauliTerm> &terms, const std::vector<double> &coeffs,
                        double time, const std::vector<unsigned> &ctrl, uint64_t cm) {
    std::vector<size_t> ks;
    double tr = 0.;
    for (size_t t = 0; t < terms.size(); ++t) {
      if (terms[t].empty) {
        tr += coeffs[t];
        continue;
      }
      if ((terms[t].xmask | terms[t].sign_mask) & cm) return false;
      ks.push_back(t);
    }
    if (ks.empty()) return false;
    for (size_t a = 0; a < ks.size(); ++a)
      for (size_t b = a + 1; b < ks.size(); ++b)
        if (!paulis_commute(terms[ks[a]], terms[ks[b]])) return false;
    std::vector<unsigned> id_at(N_, 0);
    for (auto const &kv : map_) id_at[kv.second] = kv.first;
    std::vector<unsigned> cids;  // the controls once each (the gates' own validation rejects repeats)
    for (unsigned c : ctrl)
      if (std::find(cids.begin(), cids.end(), c) == cids.end()) cids.push_back(c);
    static const cplx ph[4] = {cplx(1, 0), cplx(0, -1), cplx(-1, 0), cplx(0, 1)};  // (-i)^ny
    cplx g = std::exp(cplx(0., -time * tr));
    for (size_t k : ks) {
      const PauliTerm &p = terms[k];
      const double th = time * coeffs[k];
      const cplx a = g * std::cos(th), b = g * cplx(0., -std::sin(th)) * ph[p.ny & 3];
      g = 1.;
      const uint64_t supp = p.xmask | p.sign_mask;
      const unsigned w = unsigned(__builtin_popcountll(supp));
      if (w <= kTermGateQubits) {
        // the gate on the support, local bit i = i-th lowest support position
        std::vector<unsigned> ids, at;
        for (unsigned q = 0; q < N_; ++q)
          if ((supp >> q) & 1) {
            ids.push_back(id_at[q]);
            at.push_back(q);
          }
        uint32_t lx = 0, lz = 0;
        for (unsigned i = 0; i < w; ++i) {
          lx |= uint32_t((p.xmask >> at[i]) & 1) << i;
          lz |= uint32_t((p.sign_mask >> at[i]) & 1) << i;
        }
        submit_gate(pauli_exp_matrix(w, lx, lz, a, b), ids, cids);
      } else {
        run();
        PauliRotationDev rd{};
        rd.xmask = p.xmask;
        rd.zmask = p.sign_mask;
        rd.ctrl = cm;
        rd.are = a.real();
        rd.aim = a.imag();
        rd.bre = b.real();
        rd.bim = b.imag();
        const uint64_t piv = p.xmask & (~p.xmask + 1);
        const uint64_t ins = piv | cm;
        for (unsigned q = 0; q < N_; ++q)
          if ((ins >> q) & 1) rd.pos[rd.npos++] = uint8_t(q);
        CK(launch_pauli_rotation(prec_, state_.p, N_, rd, stream_));
        const uint64_t bytes = 2 * (uint64_t(1) << (N_ - unsigned(__builtin_popcountll(cm)))) * bpa_;
        counters_[1] += 1;
        counters_[2] += bytes;
        counters_[3] += 1;
      }
    }
    run();
    counters_[4] += 1;
    return true;
  }

  // ---- simulator.hpp:386-438 ----------------------------------------------
  void emulate_time_evolution(const std::vector<PauliTerm> &terms, const std::vector<double> &coeffs,
                              double time, const std::vector<unsigned> &ctrl) {
    run();
    uint64_t cm = 0;
    for (unsigned c : ctrl) cm |= uint64_t(1) << pos_of(c);
    if (te_mode_ >= 1 && evolve_commuting(terms, coeffs, time, ctrl, cm)) return;
    double tr = 0., op_nrm = 0.;
    std::vector<PauliRealTermDev> dev;
    for (size_t t = 0; t < terms.size(); ++t) {
      if (terms[t].empty) {
        tr += coeffs[t];
      } else {
        dev.push_back(PauliRealTermDev{terms[t].xmask, terms[t].sign_mask, coeffs[t], terms[t].ny & 3, 0});
        op_nrm += std::abs(coeffs[t]);
      }
    }
    // terms that share a flip mask next to each other (their gathers hit L1)
    std::stable_sort(dev.begin(), dev.end(),
                     [](const PauliRealTermDev &a, const PauliRealTermDev &b) { return a.xmask < b.xmask; });
    const unsigned s = unsigned(std::abs(time) * op_nrm + 1.);
    const cplx I(0., 1.);
    const cplx corr = std::exp(-time * I * tr / double(s));
    // Chebyshev where configured, or where the learned planner's cost model
    // predicts it faster than the series (both reach the series' accuracy)
    const bool cheb = te_mode_ == 2 || (te_mode_ == 1 && mode_ == GSIM_FUSION_LEARNED && !cm_.empty() &&
                                        chebyshev_predicted_faster(int(dev.size()), s, time, op_nrm, cm));
    counters_[cheb ? 6 : 5] += 1;
    const size_t n = size_t(1) << N_;
    auto *vec = static_cast<double2 *>(aux1_.get(n * 16));
    auto *nxt = static_cast<double2 *>(aux2_.get(n * 16));
    auto *out = static_cast<double2 *>(scratch_c128(n));
    CK(launch_convert(0, vec, prec_ == GSIM_C64 ? 1 : 0, state_.p, n, stream_));
    auto *d_terms = static_cast<PauliRealTermDev *>(aux3_.get(std::max<size_t>(1, dev.size()) * sizeof(PauliRealTermDev)));
    if (!dev.empty())
      CK(cudaMemcpyAsync(d_terms, dev.data(), dev.size() * sizeof(dev[0]), cudaMemcpyHostToDevice, stream_));
    if (cheb) {
      evolve_chebyshev(vec, nxt, out, d_terms, int(dev.size()), op_nrm, time, tr, cm);
    } else {
      CK(cudaMemcpyAsync(out, vec, n * 16, cudaMemcpyDeviceToDevice, stream_));
      taylor_steps(vec, nxt, out, d_terms, int(dev.size()), s, time, corr, cm);
    }
    CK(launch_convert(prec_ == GSIM_C64 ? 1 : 0, state_.p, 0, out, n, stream_));
    CK(cudaStreamSynchronize(stream_));
    // aux1_/aux2_ hold two full complex128 vectors: give the memory back.
    aux1_.release();
    aux2_.release();
  }

  // The reference's series: s steps, each summed until the controlled part of
  // an order's update has norm <= 1e-12, then the identity terms' phase.
  void taylor_steps(double2 *vec, double2 *nxt, double2 *out, const PauliRealTermDev *d_terms, int nterms,
                    unsigned s, double time, cplx corr, uint64_t cm) {
    const cplx I(0., 1.);
    const size_t n = size_t(1) << N_;
    double *d_norm = static_cast<double *>(small_.get(4096));
    for (unsigned i = 0; i < s; ++i) {
      double nrm_change = 1.;
      for (unsigned k = 0; nrm_change > 1.e-12; ++k) {
        const cplx coeff = (-time * I) / double(s * (k + 1));
        const int e0 = profiling_ ? record_event() : -1;
        CK(launch_taylor_step(vec, nxt, out, N_, d_terms, nterms, coeff.real(), coeff.imag(),
                              cm, part(), d_norm, stream_));
        if (profiling_) profile_evolution_step(4, nterms, cm, e0);
        std::swap(vec, nxt);
        double h = 0.;
        CK(cudaMemcpyAsync(&h, d_norm, 8, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        nrm_change = std::sqrt(h);
        if (k > 100000) fail(GSIM_ERR_RUNTIME, "emulate_time_evolution(): Taylor series did not converge");
      }
      CK(launch_phase_ctrl(out, vec, n, cm, corr.real(), corr.imag(), stream_));
    }
  }

  // exp(-i t H') psi by its Chebyshev expansion (Jacobi-Anger):
  //   exp(-i tau x) = J_0(tau) + 2 sum_{k>=1} (-i)^k J_k(tau) T_k(x),
  // with A = H' / beta (beta = sum |c_t| >= ||H'||, so ||A|| <= 1), tau =
  // t beta, T_k(A) psi by u_{k+1} = 2 A u_k - u_{k-1}, truncated where the
  // remaining coefficients sum below 1e-16 (each ||T_k(A) psi|| <= 1).  About
  // |tau| + 40 applications of H' where the series needs ~16 |tau|.  Then the
  // identity terms' phase exp(-i t tr) on the controlled part.
  void evolve_chebyshev(double2 *vec, double2 *nxt, double2 *out, const PauliRealTermDev *d_terms, int nterms,
                        double beta, double time, double tr, uint64_t cm) {
    const size_t n = size_t(1) << N_;
    const double tau = time * beta;
    std::vector<double> J = bessel_j_orders(std::abs(tau), 1e-16);
    if (tau < 0)
      for (size_t k = 1; k < J.size(); k += 2) J[k] = -J[k];
    static const cplx mi[4] = {cplx(1, 0), cplx(0, -1), cplx(-1, 0), cplx(0, 1)};  // (-i)^k
    CK(launch_scale_ctrl(vec, out, n, cm, J[0], 0., stream_));
    double2 *cur = vec, *other = nxt;
    for (size_t k = 1; k < J.size(); ++k) {
      const cplx a = 2. * J[k] * mi[k & 3];
      // k = 1: other <- A u_0; k >= 2: other (holding u_{k-2}) <- 2 A u_{k-1} - u_{k-2}
      const int e0 = profiling_ ? record_event() : -1;
      CK(launch_chebyshev_step(cur, other, out, N_, d_terms, nterms, (k == 1 ? 1. : 2.) / beta, k >= 2,
                               a.real(), a.imag(), cm, stream_));
      if (profiling_) profile_evolution_step(5, nterms, cm, e0);
      std::swap(cur, other);
    }
    const cplx corr = std::exp(cplx(0., -time * tr));
    CK(launch_phase_ctrl(out, vec, n, cm, corr.real(), corr.imag(), stream_));
  }

  // Profiler record of one Taylor-series (kind 4) or Chebyshev (kind 5) step
  // launch: k = terms; bytes = (terms + 1) complex128 vectors.
  void profile_evolution_step(uint32_t kind, int nterms, uint64_t cm, int e0) {
    const int e1 = record_event();
    Prof p;
    std::memset(&p.rec, 0, sizeof(p.rec));
    p.rec.kind = kind;
    p.rec.k = uint32_t(nterms);
    p.rec.nctrl = uint32_t(__builtin_popcountll(cm));
    p.rec.nqubits = N_;
    p.rec.bytes = uint64_t(nterms + 1) * (uint64_t(1) << N_) * 16;
    p.rec.precision = uint32_t(prec_);
    p.ev0 = e0;
    p.ev1 = e1;
    prof_.push_back(p);
  }

  // The learned planner's choice between the reference's Taylor series and
  // the Chebyshev expansion for one non-commuting evolution: predicted step
  // times times step counts.  The series takes s steps of K orders each, K
  // the first order whose term x^K / K! (x = |t| sum|c| / s) drops below the
  // 1e-12 stop (an upper bound of the update's norm), plus a host round trip
  // per order for that stop; the expansion takes as many steps as it has
  // Bessel coefficients.
  static constexpr double kOrderRoundTripMs = 0.03;  // the series' host read of each order's norm
  static constexpr double kStepGapMs = 0.002;         // host launch gap per expansion step
  bool chebyshev_predicted_faster(int nterms, unsigned s, double time, double op_nrm, uint64_t cm) {
    const double x = std::abs(time) * op_nrm / double(s);
    unsigned K = 1;
    for (double term = x; term > 1e-12 && K < 60; ++K) term *= x / double(K + 1);
    const size_t ncheb = bessel_j_orders(std::abs(time * op_nrm), 1e-16).size();
    gsim_launch_record r;
    std::memset(&r, 0, sizeof(r));
    r.k = uint32_t(nterms);
    r.nctrl = uint32_t(__builtin_popcountll(cm));
    r.nqubits = N_;
    r.bytes = uint64_t(nterms + 1) * (uint64_t(1) << N_) * 16;
    r.precision = uint32_t(prec_);
    r.kind = 4;
    const double t_taylor = double(s) * double(K) * (predict_ms(r) + kOrderRoundTripMs);
    r.kind = 5;
    const double t_cheb = double(ncheb) * (predict_ms(r) + kStepGapMs);
    last_te_pred_[0] = t_taylor;
    last_te_pred_[1] = t_cheb;
    return t_cheb < t_taylor;
  }

  // ---- simulator.hpp:352-368 ----------------------------------------------
  double get_probability(const std::vector<uint8_t> &bits, const std::vector<unsigned> &ids) {
    run();
    if (!check_ids(ids))
      fail(GSIM_ERR_RUNTIME,
           "get_probability(): Unknown qubit id. Please make sure you have called eng.flush().");
    if (bits.size() != ids.size()) fail(GSIM_ERR_LENGTH, "get_probability(): bits and ids size mismatch");
    uint64_t mask = 0, val = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
      mask |= uint64_t(1) << map_.at(ids[i]);
      val |= uint64_t(bits[i] ? 1 : 0) << map_.at(ids[i]);
    }
    return masked_norm_host(mask, val);
  }

  // ---- simulator.hpp:370-384 ----------------------------------------------
  cplx get_amplitude(const std::vector<uint8_t> &bits, const std::vector<unsigned> &ids) {
    run();
    uint64_t chk = 0, index = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
      auto it = map_.find(ids[i]);
      if (it == map_.end()) break;
      chk |= uint64_t(1) << it->second;
      index |= uint64_t(i < bits.size() && bits[i] ? 1 : 0) << it->second;
    }
    if (chk + 1 != (uint64_t(1) << N_))
      fail(GSIM_ERR_RUNTIME,
           "The second argument to get_amplitude() must be a permutation of all allocated qubits. "
           "Please make sure you have called eng.flush().");
    return amp_at(index);
  }

  // ---- simulator.hpp:440-454 ----------------------------------------------
  void set_wavefunction(const void *wf, int dtype, size_t len, const std::vector<unsigned> &ordering) {
    run();
    if (map_.size() != ordering.size() || !check_ids(ordering))
      fail(GSIM_ERR_RUNTIME,
           "set_wavefunction(): Invalid mapping provided. Please make sure all qubits have been "
           "allocated previously (call eng.flush()).");
    if (len != (size_t(1) << ordering.size()))
      fail(GSIM_ERR_LENGTH, "set_wavefunction(): the wavefunction must have 2^n amplitudes");
    if (dtype != GSIM_C64 && dtype != GSIM_C128) fail(GSIM_ERR_VALUE, "unknown dtype");
    for (size_t i = 0; i < ordering.size(); ++i) map_[ordering[i]] = unsigned(i);
    upload(wf, dtype, 0, len);
  }

  // ---- simulator.hpp:456-485 ----------------------------------------------
  void collapse_wavefunction(const std::vector<unsigned> &ids, const std::vector<uint8_t> &values) {
    run();
    if (ids.size() != values.size())
      fail(GSIM_ERR_LENGTH, "collapse_wavefunction(): ids and values size mismatch");
    if (!check_ids(ids))
      fail(GSIM_ERR_RUNTIME,
           "collapse_wavefunction(): Unknown qubit id(s) provided. Try calling eng.flush() before "
           "invoking this function.");
    uint64_t mask = 0, val = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
      mask |= uint64_t(1) << map_.at(ids[i]);
      val |= uint64_t(values[i] ? 1 : 0) << map_.at(ids[i]);
    }
    double *d_norm = static_cast<double *>(small_.get(4096));
    CK(launch_masked_norm(prec_, state_.p, N_, mask, val, part(), d_norm, stream_));
    double nrm = 0.;
    CK(cudaMemcpyAsync(&nrm, d_norm, 8, cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    if (nrm < 1.e-12)
      fail(GSIM_ERR_RUNTIME, "collapse_wavefunction(): Invalid collapse! Probability is ~0.");
    CK(launch_project_scale(prec_, state_.p, N_, mask, val, d_norm, stream_));
  }

  // ---- cheat, simulator.hpp:529-532 ---------------------------------------
  unsigned num_qubits() {
    run();
    return N_;
  }
  const std::map<unsigned, unsigned> &mapping() const { return map_; }
  void get_state(void *host, int dtype, size_t offset, size_t count) {
    run();
    if (offset + count > (size_t(1) << N_)) fail(GSIM_ERR_LENGTH, "state range out of bounds");
    if (dtype != GSIM_C64 && dtype != GSIM_C128) fail(GSIM_ERR_VALUE, "unknown dtype");
    download(host, dtype, offset, count);
  }
  void device_view(void **ptr, size_t *len, int *dtype) {
    run();
    CK(cudaStreamSynchronize(stream_));
    *ptr = state_.p;
    *len = size_t(1) << N_;
    *dtype = prec_;
  }
  void synchronize() { CK(cudaStreamSynchronize(stream_)); }

  // ---- adjoint-method gradient (no reference counterpart) -----------------
  // E = <psi|H|psi> with psi = U(theta) |current state>, and dE/dtheta by one
  // reverse sweep over psi and lam = H psi, un-applying the gates; psi is
  // reloaded from checkpoints stored every `ckpt` gates of the forward pass.
  // The engine's own state is left unchanged.
  void adjoint(const std::vector<AdjointGate> &gates, const std::vector<int> &param,
               const std::vector<double> &scale, size_t nparams, const std::vector<PauliTerm> &terms,
               const std::vector<double> &coeffs, unsigned ckpt, double *energy, double *grad) {
    run();
    const size_t n = size_t(1) << N_;
    void *psi = aux1_.get(n * bpa_);
    void *lam = aux2_.get(n * bpa_);
    CK(cudaMemcpyAsync(psi, state_.p, n * bpa_, cudaMemcpyDeviceToDevice, stream_));
    std::vector<DevBuf> ck;
    std::vector<int> ck_at(gates.size(), -1);  // checkpoint index holding the state after gate i
    // Forward pass with the stage planner, one plan per segment between
    // checkpoints (the planner's passes end exactly at a segment's last
    // gate).  The stage executor works on state_, so the forward copy takes
    // its place for the duration.
    struct SwapBack {  // restores state_ also when a launch fails
      DevBuf &a, &b;
      SwapBack(DevBuf &x, DevBuf &y) : a(x), b(y) { std::swap(a, b); }
      ~SwapBack() { std::swap(a, b); }
    };
    {
      SwapBack forward_on_copy(state_, aux1_);
      for (size_t s0 = 0; s0 < gates.size();) {
        const size_t s1 = ckpt ? std::min(gates.size(), s0 + ckpt) : gates.size();
        std::vector<StageGate> seg;
        seg.reserve(s1 - s0);
        for (size_t i = s0; i < s1; ++i) {
          StageGate g;
          g.m.assign(gates[i].u, gates[i].u + 4);
          g.pos = {gates[i].target};
          g.ctrl_mask = gates[i].ctrl_mask;
          seg.push_back(std::move(g));
        }
        std::vector<PlanStep> steps = plan_staged(seg);
        execute_staged(steps);
        if (ckpt && s1 < gates.size()) {
          ck.emplace_back();
          void *c = ck.back().get(n * bpa_);
          CK(cudaMemcpyAsync(c, state_.p, n * bpa_, cudaMemcpyDeviceToDevice, stream_));
          ck_at[s1 - 1] = int(ck.size()) - 1;
        }
        s0 = s1;
      }
    }
    std::vector<PauliApplyTermDev> dev(terms.size());
    for (size_t t = 0; t < terms.size(); ++t) dev[t] = apply_term_dev(terms[t], cplx(coeffs[t], 0.));
    auto *d_terms = static_cast<PauliApplyTermDev *>(aux3_.get(std::max<size_t>(1, dev.size()) * sizeof(PauliApplyTermDev)));
    if (!dev.empty())
      CK(cudaMemcpyAsync(d_terms, dev.data(), dev.size() * sizeof(dev[0]), cudaMemcpyHostToDevice, stream_));
    CK(launch_pauli_apply(prec_, psi, lam, N_, d_terms, int(dev.size()), stream_));
    double *d_out = static_cast<double *>(small_.get(4096));
    CK(launch_compare(prec_, psi, prec_, lam, n, part(), d_out, stream_));
    double e3[3];
    CK(cudaMemcpyAsync(e3, d_out, 24, cudaMemcpyDeviceToHost, stream_));
    const int nblk = adjoint_blocks(N_);
    size_t ncols = 0;
    for (int p : param) ncols += p >= 0;
    auto *d_part = static_cast<double *>(table_.get(std::max<size_t>(1, ncols) * nblk * 8));
    std::vector<int> col(gates.size(), -1);
    int c = 0;
    for (size_t i = gates.size(); i-- > 0;) {
      if (param[i] >= 0) col[i] = c++;
      CK(launch_adjoint_step(prec_, psi, lam, N_, gates[i], col[i], d_part, nblk, stream_));
      if (i > 0 && ck_at[i - 1] >= 0)
        CK(cudaMemcpyAsync(psi, ck[ck_at[i - 1]].p, n * bpa_, cudaMemcpyDeviceToDevice, stream_));
    }
    std::vector<double> g(ncols);
    if (ncols) {
      auto *d_g = static_cast<double *>(table2_.get(ncols * 8));
      CK(launch_column_sums(d_part, nblk, int(ncols), d_g, stream_));
      CK(cudaMemcpyAsync(g.data(), d_g, ncols * 8, cudaMemcpyDeviceToHost, stream_));
    }
    CK(cudaStreamSynchronize(stream_));
    for (auto &b : ck) b.release();
    *energy = e3[0];
    std::fill(grad, grad + nparams, 0.);
    for (size_t i = 0; i < gates.size(); ++i)
      if (param[i] >= 0) grad[param[i]] += scale[i] * g[col[i]];
  }

  // <this|other>, max |this_i - other_i| (no reference counterpart).
  void compare(Engine &other, double *out) {
    run();
    other.run();
    if (N_ != other.N_ || map_ != other.map_)
      fail(GSIM_ERR_VALUE, "compare_states(): the engines hold different qubits or orderings");
    CK(cudaStreamSynchronize(other.stream_));
    double *d_out = static_cast<double *>(small_.get(4096));
    CK(launch_compare(prec_, state_.p, other.prec_, other.state_.p, uint64_t(1) << N_, part(), d_out, stream_));
    CK(cudaMemcpyAsync(out, d_out, 24, cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
  }

  // ---- learned planner -----------------------------------------------------
  // The cost model maps the features of one kernel launch (launch_features)
  // to its predicted log(milliseconds); the learned planner sums predictions
  // over candidate plans of the queued gates.
  static constexpr int kFeatures = 20;
  void set_cost_model(int F, int H, const float *params) {
    if (F != kFeatures || H < 1 || H > 256) fail(GSIM_ERR_VALUE, "cost model: unexpected layer sizes");
    cm_H_ = H;
    cm_.assign(params, params + (size_t(H) * F + H + size_t(H) * H + H + H + 1));
    memo_.clear();
  }
  // allowed[n] != 0: learned plans may run on an n-qubit state; elsewhere the
  // greedy fixed-size fusion runs (regimes where measured wall time did not
  // beat it).
  void set_learned_regimes(const uint8_t *allowed, size_t n) {
    learned_ok_.assign(65, 1);
    for (size_t i = 0; i < std::min<size_t>(n, 65); ++i) learned_ok_[i] = allowed[i] ? 1 : 0;
  }
  int last_choice() const { return last_choice_; }
  void last_prediction(double *out) const { std::copy(last_pred_, last_pred_ + 3, out); }
  void predict_rows(const float *x, size_t n, float *out) const {
    if (cm_.empty()) fail(GSIM_ERR_VALUE, "no cost model installed");
    for (size_t i = 0; i < n; ++i) out[i] = predict(x + i * kFeatures);
  }

  void set_fusion(int mode, unsigned kmax) {
    run();
    if (mode != GSIM_FUSION_REFERENCE && mode != GSIM_FUSION_NONE && mode != GSIM_FUSION_STAGED &&
        mode != GSIM_FUSION_LEARNED)
      fail(GSIM_ERR_VALUE, "unknown fusion mode");
    mode_ = mode;
    if (mode == GSIM_FUSION_REFERENCE && kmax) {  // widest cluster of the greedy fixed-size rule
      if (kmax > 7) fail(GSIM_ERR_VALUE, "set_fusion(): clusters of at most 7 qubits");
      fmax_ = kmax;
      fmin_ = std::min(4u, kmax);
    }
    if (mode == GSIM_FUSION_STAGED && kmax >= 6) {  // kmax >= 6 selects the tile width in staged mode
      tile_bits_c64_ = std::min(kmax, 14u);
      tile_bits_c128_ = std::min(kmax - 1, 13u);
    }
  }
  void reserve(unsigned nq) { ensure_capacity(nq); }
  void set_stage_kernel(int mode) {
    if (mode < 0 || mode > 2) fail(GSIM_ERR_VALUE, "stage kernel mode must be 0, 1 or 2");
    stage_kernel_ = mode;
  }
  void set_upload_mode(int mode) {
    if (mode != 0 && mode != 1) fail(GSIM_ERR_VALUE, "upload mode must be 0 (copy engine) or 1 (SM reads)");
    upload_mode_ = mode;
  }
  // 0 off, 1 on with the per-group norm restoration of unitary gates
  // (default), 2 on without it
  void set_tensor_cores(int mode) {
    run();
    if (mode < 0 || mode > 2) fail(GSIM_ERR_VALUE, "tensor-core mode must be 0, 1 or 2");
    use_tc_ = mode != 0;
    tc_mode_ = mode == 0 ? 1 : mode;
  }

  void set_time_evolution(int mode) {
    if (mode < 0 || mode > 2)
      fail(GSIM_ERR_VALUE, "time-evolution mode must be 0 (Taylor series), 1 (exact for commuting terms, else "
                           "Taylor) or 2 (exact for commuting terms, else Chebyshev)");
    te_mode_ = mode;
  }

  // ---- timing -------------------------------------------------------------
  void timer_mark(int slot) {
    if (slot < 0 || slot >= 16) fail(GSIM_ERR_VALUE, "timer slot must be 0..15");
    if (!timer_[slot]) CK(cudaEventCreate(&timer_[slot]));
    CK(cudaEventRecord(timer_[slot], stream_));
  }
  float timer_elapsed(int a, int b) {
    if (a < 0 || a >= 16 || b < 0 || b >= 16 || !timer_[a] || !timer_[b])
      fail(GSIM_ERR_VALUE, "timer slots not recorded");
    CK(cudaEventSynchronize(timer_[b]));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, timer_[a], timer_[b]));
    return ms;
  }
  void profile_enable(bool on) {
    run();
    profiling_ = on;
  }
  size_t profile_fetch(gsim_launch_record *out, size_t cap) {
    run();
    CK(cudaStreamSynchronize(stream_));
    size_t n = std::min(cap, prof_.size());
    for (size_t i = 0; i < n; ++i) {
      gsim_launch_record r = prof_[i].rec;
      CK(cudaEventElapsedTime(&r.ms, ev_pool_[prof_[i].ev0], ev_pool_[prof_[i].ev1]));
      out[i] = r;
    }
    return prof_.size();
  }
  void profile_clear() {
    CK(cudaStreamSynchronize(stream_));
    prof_.clear();
    ev_next_ = 0;
  }
  uint64_t counter(size_t i) const { return i < 7 ? counters_[i] : 0; }
  void reset_counters() { std::fill(std::begin(counters_), std::end(counters_), 0); }

 private:
  struct QueuedGate {
    std::vector<cplx> m;
    std::vector<unsigned> ids, ctrl;
  };
  static constexpr size_t kMaxQueue = 4096;

  unsigned pos_of(unsigned id) const {
    auto it = map_.find(id);
    if (it == map_.end())
      fail(GSIM_ERR_RUNTIME, "Unknown qubit id " + std::to_string(id) +
                                 ". Please make sure you have called eng.flush().");
    return it->second;
  }
  bool check_ids(const std::vector<unsigned> &ids) const {
    for (unsigned id : ids)
      if (!map_.count(id)) return false;
    return true;
  }

  PauliApplyTermDev apply_term_dev(const PauliTerm &t, cplx c) const {
    // (P psi)_i = (-i)^{#Y} (-1)^{popcount(i & (Y|Z))} psi_{i ^ X}.
    static const cplx ph[4] = {cplx(1, 0), cplx(0, -1), cplx(-1, 0), cplx(0, 1)};
    const cplx w = c * ph[t.ny & 3];
    return PauliApplyTermDev{t.xmask, t.sign_mask, w.real(), w.imag()};
  }

  double *part() { return static_cast<double *>(part_.get(4096 * 8)); }
  void *scratch() { return scratch_.get(cap_ * bpa_); }
  void *scratch_c128(size_t n) {
    // emulate_time_evolution's third complex128 vector: reuse the scratch
    // buffer when it is large enough.
    return scratch_.get(std::max(cap_ * bpa_, n * 16));
  }

  void ensure_capacity(unsigned nq) {
    const size_t need = size_t(1) << std::max(nq, 10u);
    if (need <= cap_) return;
    void *np = nullptr;
    if (cudaMalloc(&np, need * bpa_) != cudaSuccess) {
      cudaGetLastError();
      fail(GSIM_ERR_MEMORY, "cudaMalloc of the state vector (" + std::to_string(need * bpa_) +
                                " bytes) failed");
    }
    if (state_.p) {
      CK(cudaMemcpyAsync(np, state_.p, (size_t(1) << N_) * bpa_, cudaMemcpyDeviceToDevice, stream_));
      CK(cudaStreamSynchronize(stream_));
      state_.release();
    }
    state_.p = np;
    state_.bytes = need * bpa_;
    cap_ = need;
    scratch_.release();  // regrown on demand at the new capacity
  }
  void set_basis_zero() {
    CK(cudaMemsetAsync(state_.p, 0, bpa_, stream_));
    if (prec_ == GSIM_C64) {
      const float one[2] = {1.f, 0.f};
      CK(cudaMemcpyAsync(state_.p, one, 8, cudaMemcpyHostToDevice, stream_));
    } else {
      const double one[2] = {1., 0.};
      CK(cudaMemcpyAsync(state_.p, one, 16, cudaMemcpyHostToDevice, stream_));
    }
    CK(cudaStreamSynchronize(stream_));
  }

  void exec_dense(const DenseOp &op, uint32_t ngates = 1) {
    const unsigned c = unsigned(__builtin_popcountll(op.ctrl_mask));
    const uint64_t bytes = 2 * (uint64_t(1) << (N_ - c)) * bpa_;
    int e0 = -1;
    if (profiling_) e0 = record_event();
    const size_t kq = op.pos.size();
    const int route = dense_kind(kq);
    if (route == 3) {
      // tensor cores: U embedded as a real 2^(k+1) square matrix, TF32 hi/lo
      const DenseOp sop = tc_sorted_targets(op);
      const size_t nb = tc_operand_floats(int(kq)) * 4;
      char *h = nullptr;
      UploadSlot &sl = next_slot(nb, h);
      tc_prepare_operand(sop.m, int(kq), reinterpret_cast<float *>(h));
      const void *d = finish_slot(sl, h, nb);
      int *d_err = reinterpret_cast<int *>(static_cast<char *>(small_.get(4096)) + 2048);
      if (!tc_used_) CK(cudaMemsetAsync(d_err, 0, sizeof(int), stream_));
      CK(launch_tc_gate(state_.p, N_, sop, static_cast<const float *>(d), d_err, tc_mode_ == 1, stream_));
      tc_used_ = true;
    } else if (route == 2) {
      const size_t D = size_t(1) << op.pos.size();
      std::vector<cplx> mt(D * D);  // the wide kernel reads U transposed
      for (size_t r = 0; r < D; ++r)
        for (size_t j = 0; j < D; ++j) mt[j * D + r] = op.m[r * D + j];
      void *dm = upload_matrix(mt, D * D);
      CK(launch_wide(prec_, state_.p, N_, op, dm, stream_));
    } else {
      CK(launch_dense(prec_, state_.p, N_, op, stream_));
    }
    if (profiling_) {
      const int e1 = record_event();
      Prof p;
      std::memset(&p.rec, 0, sizeof(p.rec));
      p.rec.kind = uint32_t(route);
      p.rec.k = uint32_t(op.pos.size());
      p.rec.nctrl = c;
      p.rec.nqubits = N_;
      for (unsigned q : op.pos) p.rec.targets |= uint64_t(1) << q;
      p.rec.bytes = bytes;
      p.rec.precision = uint32_t(prec_);
      p.rec.ngates = ngates;
      p.ev0 = e0;
      p.ev1 = e1;
      prof_.push_back(p);
    }
    counters_[1] += 1;
    counters_[2] += bytes;
    counters_[3] += 1;
  }
  // A ring of upload slots (pinned host staging + device buffer): a slot's
  // host buffer is rewritten only after its previous copy has run, so the
  // host can prepare the next few matrices while earlier kernels execute.
  struct UploadSlot {
    DevBuf dev;
    HostBuf host;
    cudaEvent_t ev = nullptr;
  };
  UploadSlot &next_slot(size_t bytes, char *&h) {
    UploadSlot &sl = mslots_[mslot_next_];
    mslot_next_ = (mslot_next_ + 1) % mslots_.size();
    if (sl.ev) CK(cudaEventSynchronize(sl.ev));
    h = static_cast<char *>(sl.host.get(bytes));
    sl.dev.get(bytes);
    return sl;
  }
  void *finish_slot(UploadSlot &sl, const char *h, size_t bytes) {
    CK(cudaMemcpyAsync(sl.dev.p, h, bytes, cudaMemcpyHostToDevice, stream_));
    if (!sl.ev) CK(cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
    CK(cudaEventRecord(sl.ev, stream_));
    return sl.dev.p;
  }
  // Copy a matrix in the state's precision to device memory.
  void *upload_matrix(const std::vector<cplx> &m, size_t count) {
    const size_t bytes = count * bpa_;
    char *h = nullptr;
    UploadSlot &sl = next_slot(bytes, h);
    for (size_t i = 0; i < count; ++i) {
      if (prec_ == GSIM_C64) {
        reinterpret_cast<float *>(h)[2 * i] = float(m[i].real());
        reinterpret_cast<float *>(h)[2 * i + 1] = float(m[i].imag());
      } else {
        reinterpret_cast<double *>(h)[2 * i] = m[i].real();
        reinterpret_cast<double *>(h)[2 * i + 1] = m[i].imag();
      }
    }
    return finish_slot(sl, h, bytes);
  }
  int record_event() {
    if (ev_next_ >= ev_pool_.size()) {
      cudaEvent_t ev;
      CK(cudaEventCreate(&ev));
      ev_pool_.push_back(ev);
    }
    const int i = int(ev_next_++);
    CK(cudaEventRecord(ev_pool_[i], stream_));
    return i;
  }

  void run_staged();
  std::vector<PlanStep> plan_stages(const std::vector<StageGate> &gates) const;
  void build_stage_data(StagePlan &sp) const;
  std::vector<PlanStep> plan_staged(const std::vector<StageGate> &gates) const;
  void execute_staged(std::vector<PlanStep> &steps, bool build = false);
  void exec_stage(const StagePlan &sp, const void *d_ops, const void *d_pool);
  void run_learned();
  std::vector<StageGate> queued_positions() const;
  std::vector<DenseOp> reference_plan(const std::vector<StageGate> &gates) const;
  // a cluster: gates [begin, end) fused into one dense launch on matrix
  // qubits q with shared controls c (bit masks of positions)
  struct Cluster {
    size_t begin = 0, end = 0;
    uint64_t q = 0, c = 0;
  };
  std::vector<Cluster> greedy_clusters(const std::vector<StageGate> &gates) const;
  std::vector<Cluster> learned_clusters(const std::vector<StageGate> &gates);
  gsim_launch_record dense_record(uint64_t q, uint64_t c) const;
  double predict_ms(const gsim_launch_record &r);
  double clusters_ms(const std::vector<Cluster> &cl);
  double staged_ms(const std::vector<PlanStep> &steps);
  void exec_clusters(std::vector<StageGate> &gates, const std::vector<Cluster> &cl);
  float predict(const float *f) const;
  int dense_kind(size_t kq) const {
    if (prec_ == GSIM_C64 && use_tc_ && kq >= 4 && kq <= 7 && N_ >= kq + 7) return 3;
    return kq > 5 ? 2 : 0;
  }

  double masked_norm_host(uint64_t mask, uint64_t val) {
    double *d_norm = static_cast<double *>(small_.get(4096));
    CK(launch_masked_norm(prec_, state_.p, N_, mask, val, part(), d_norm, stream_));
    double h = 0.;
    CK(cudaMemcpyAsync(&h, d_norm, 8, cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    return h;
  }
  cplx amp_at(uint64_t index) {
    if (prec_ == GSIM_C64) {
      float a[2];
      CK(cudaMemcpyAsync(a, static_cast<char *>(state_.p) + index * 8, 8, cudaMemcpyDeviceToHost, stream_));
      CK(cudaStreamSynchronize(stream_));
      return cplx(a[0], a[1]);
    }
    double a[2];
    CK(cudaMemcpyAsync(a, static_cast<char *>(state_.p) + index * 16, 16, cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    return cplx(a[0], a[1]);
  }
  static double norm2_host(double re, double im) { return std::fma(re, re, im * im); }
  double norm2_at(uint64_t index) {
    const cplx a = amp_at(index);
    return norm2_host(a.real(), a.imag());
  }

  // Host <-> device transfers with precision conversion through the scratch
  // buffer, in chunks.
  // Device view of page-locked host memory (cudaHostRegister / cudaMallocHost)
  // covering all of [host, host + bytes), or nullptr when either end is
  // pageable or the two ends are not one contiguous device view.
  static const void *locked_device_view(const void *host, size_t bytes) {
    auto view = [](const void *p) -> const char * {
      cudaPointerAttributes a;
      if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
      return a.type == cudaMemoryTypeHost ? static_cast<const char *>(a.devicePointer) : nullptr;
    };
    if (!bytes) return nullptr;
    const char *first = view(host), *last = view(static_cast<const char *>(host) + bytes - 1);
    if (!first || !last || last - first != std::ptrdiff_t(bytes - 1)) return nullptr;
    return first;
  }
  void upload(const void *host, int dtype, size_t offset, size_t count) {
    const size_t hb = dtype == GSIM_C64 ? 8 : 16;
    if (dtype == prec_ && upload_mode_ == 1) {
      // the SMs read page-locked host memory directly (16-byte aligned buffers)
      const void *view = locked_device_view(host, count * bpa_);
      char *dst = static_cast<char *>(state_.p) + offset * bpa_;
      if (view && !((reinterpret_cast<uintptr_t>(view) | reinterpret_cast<uintptr_t>(dst) | (count * bpa_)) & 15u)) {
        CK(launch_pull(dst, view, count * bpa_, stream_));
        CK(cudaStreamSynchronize(stream_));
        return;
      }
    }
    if (dtype == prec_) {
      CK(cudaMemcpyAsync(static_cast<char *>(state_.p) + offset * bpa_, host, count * bpa_,
                         cudaMemcpyHostToDevice, stream_));
      CK(cudaStreamSynchronize(stream_));
      return;
    }
    char *stage = static_cast<char *>(scratch());
    const size_t chunk = std::max<size_t>(1, (cap_ * bpa_) / hb);
    for (size_t o = 0; o < count; o += chunk) {
      const size_t c = std::min(chunk, count - o);
      CK(cudaMemcpyAsync(stage, static_cast<const char *>(host) + o * hb, c * hb, cudaMemcpyHostToDevice, stream_));
      CK(launch_convert(prec_ == GSIM_C64 ? 1 : 0, static_cast<char *>(state_.p) + (offset + o) * bpa_,
                        dtype == GSIM_C64 ? 1 : 0, stage, c, stream_));
      CK(cudaStreamSynchronize(stream_));
    }
  }
  void download(void *host, int dtype, size_t offset, size_t count) {
    const size_t hb = dtype == GSIM_C64 ? 8 : 16;
    if (dtype == prec_) {
      CK(cudaMemcpyAsync(host, static_cast<char *>(state_.p) + offset * bpa_, count * bpa_,
                         cudaMemcpyDeviceToHost, stream_));
      CK(cudaStreamSynchronize(stream_));
      return;
    }
    char *stage = static_cast<char *>(scratch());
    const size_t chunk = std::max<size_t>(1, (cap_ * bpa_) / hb);
    for (size_t o = 0; o < count; o += chunk) {
      const size_t c = std::min(chunk, count - o);
      CK(launch_convert(dtype == GSIM_C64 ? 1 : 0, stage, prec_ == GSIM_C64 ? 1 : 0,
                        static_cast<char *>(state_.p) + (offset + o) * bpa_, c, stream_));
      CK(cudaMemcpyAsync(static_cast<char *>(host) + o * hb, stage, c * hb, cudaMemcpyDeviceToHost, stream_));
      CK(cudaStreamSynchronize(stream_));
    }
  }

  // Index picked by the reference's sampling loop (simulator.hpp:152-160):
  //   P = 0; pick = 0; while (P < rnd && pick < n) P += |psi[pick++]|^2; pick--;
  // reproduced exactly, including FP64 rounding of the running sum.
  uint64_t sample(double rnd);
  double seq_block(uint64_t b0, uint64_t cnt, double P, double rnd, uint64_t &pick, bool &done);

  int prec_;
  size_t bpa_;
  unsigned N_ = 0;
  std::map<unsigned, unsigned> map_;
  DevBuf state_, scratch_, part_, small_, aux1_, aux2_, aux3_, table_, table2_;
  HostBuf pinned_;
  size_t cap_ = 0;
  cudaStream_t stream_ = nullptr;
  std::mt19937 rng_;
  std::uniform_real_distribution<double> dist_{0., 1.};
  RefFusion fused_;
  unsigned fmin_ = 4, fmax_ = 5, max_gate_ = 5;
  int mode_ = GSIM_FUSION_REFERENCE;
  std::vector<QueuedGate> queue_;
  unsigned tile_bits_c64_ = kRegBitsC64 + 8, tile_bits_c128_ = kRegBitsC128 + 8;
  int stage_kernel_ = 2;  // 0 one pass per operation, 1 register substages, 2 packed pairs (complex64)
  bool use_tc_ = true;
  int tc_mode_ = 1;
  int te_mode_ = 1;  // emulate_time_evolution: 0 Taylor only, 1 exact for commuting terms else Taylor, 2 ... else Chebyshev
  int upload_mode_ = 1;  // host -> device state copies: 0 copy engine, 1 SM reads of page-locked memory
  bool tc_used_ = false;
  std::array<UploadSlot, 4> mslots_;
  size_t mslot_next_ = 0;
  std::vector<float> cm_;  // cost-model weights (host copy)
  double last_te_pred_[2] = {0., 0.};  // predicted ms of the series and the expansion, last evolution
  int cm_H_ = 0;
  int last_choice_ = -1;
  std::vector<uint8_t> learned_ok_ = std::vector<uint8_t>(65, 1);
  std::unordered_map<uint64_t, double> memo_;  // launch key -> predicted ms
  double last_pred_[3] = {0, 0, 0};                // predicted ms: greedy, staged, learned clusters
  DevBuf upload_dev_;
  // Page-locked staging of stage uploads, a ring of slots: a flush's copies
  // run in stream order between its launches, so a slot is written again
  // only after the copies of the flush that used it kUploadSlots flushes ago.
  static constexpr int kUploadSlots = 4;
  HostBuf upload_host_[kUploadSlots];
  cudaEvent_t upload_ev_[kUploadSlots] = {};
  int upload_slot_ = 0;
  uint64_t counters_[7] = {0, 0, 0, 0, 0, 0, 0};
  // timing
  cudaEvent_t timer_[16] = {};
  struct Prof {
    gsim_launch_record rec;
    int ev0, ev1;
  };
  bool profiling_ = false;
  std::vector<Prof> prof_;
  std::vector<cudaEvent_t> ev_pool_;
  size_t ev_next_ = 0;
};

// Sequential reference loop over [b0, b0 + cnt) starting from running sum P.
double Engine::seq_block(uint64_t b0, uint64_t cnt, double P, double rnd, uint64_t &pick,
                         bool &done) {
  char *h = static_cast<char *>(pinned_.get(cnt * bpa_));
  CK(cudaMemcpyAsync(h, static_cast<char *>(state_.p) + b0 * bpa_, cnt * bpa_, cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  for (uint64_t i = 0; i < cnt; ++i) {
    if (!(P < rnd)) {
      done = true;
      return P;
    }
    double re, im;
    if (prec_ == GSIM_C64) {
      re = reinterpret_cast<float *>(h)[2 * i];
      im = reinterpret_cast<float *>(h)[2 * i + 1];
    } else {
      re = reinterpret_cast<double *>(h)[2 * i];
      im = reinterpret_cast<double *>(h)[2 * i + 1];
    }
    P += norm2_host(re, im);
    pick = b0 + i + 1;
  }
  return P;
}

uint64_t Engine::sample(double rnd) {
  const uint64_t n = uint64_t(1) << N_;
  uint64_t pick = 0;
  bool done = false;
  if (!(0. < rnd)) return ~uint64_t(0);  // loop never runs: pick-- wraps
  constexpr unsigned lb = 13;
  if (n <= (uint64_t(1) << 16)) {
    seq_block(0, n, 0., rnd, pick, done);
    return pick - 1;
  }
  // Blocked exact replay.  Within a block where the running sum P stays in
  // one binade [2^e, 2^(e+1)), every addition rounds to the grid 2^(e-52),
  // so fl(P + x) = P + round(x) unless x sits exactly half-way between grid
  // points.  Block sums of round(x) are exact 64-bit integers computed in
  // parallel for three candidate binades per block; the host replays the
  // blocks in order and falls back to the element loop for a block that
  // changes binade, holds a tie, or reaches rnd.
  const uint64_t B = n >> lb;
  auto *d_sums = static_cast<double *>(aux1_.get(B * 8));
  CK(launch_block_norm_sums(prec_, state_.p, n, lb, d_sums, stream_));
  std::vector<double> sums(B);
  CK(cudaMemcpyAsync(sums.data(), d_sums, B * 8, cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  std::vector<int16_t> cand(3 * B);
  double Q = 0.;
  for (uint64_t b = 0; b < B; ++b) {
    if (Q > 0. && std::isfinite(Q)) {
      const int e = std::ilogb(Q);
      for (int c = 0; c < 3; ++c) cand[3 * b + c] = int16_t(e - 1 + c);
    } else {
      for (int c = 0; c < 3; ++c) cand[3 * b + c] = int16_t(-32768);
    }
    Q += sums[b];
  }
  auto *d_cand = static_cast<int16_t *>(aux2_.get(3 * B * 2 + 3 * B * 8 + 3 * B + 64));
  auto *d_units = reinterpret_cast<unsigned long long *>(
      reinterpret_cast<char *>(d_cand) + ((3 * B * 2 + 15) / 16) * 16);
  auto *d_flags = reinterpret_cast<uint8_t *>(d_units + 3 * B);
  CK(cudaMemcpyAsync(d_cand, cand.data(), 3 * B * 2, cudaMemcpyHostToDevice, stream_));
  CK(launch_block_grid_sums(prec_, state_.p, n, lb, d_cand, d_units, d_flags, stream_));
  std::vector<unsigned long long> units(3 * B);
  std::vector<uint8_t> flags(3 * B);
  CK(cudaMemcpyAsync(units.data(), d_units, 3 * B * 8, cudaMemcpyDeviceToHost, stream_));
  CK(cudaMemcpyAsync(flags.data(), d_flags, 3 * B, cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  double P = 0.;
  const uint64_t bsz = uint64_t(1) << lb;
  for (uint64_t b = 0; b < B && !done; ++b) {
    const uint64_t b0 = b * bsz;
    if (P == 0.) {
      if (sums[b] == 0.) {
        pick = b0 + bsz;  // every x in the block is 0: P stays 0 < rnd
        continue;
      }
      P = seq_block(b0, bsz, P, rnd, pick, done);
      continue;
    }
    const int e = std::ilogb(P);
    int c = -1;
    for (int k = 0; k < 3; ++k)
      if (cand[3 * b + k] == e) c = k;
    bool fast = c >= 0 && flags[3 * b + c] == 0 && e > -1000;
    if (fast) {
      const double G = std::ldexp(1., e - 52);
      const unsigned long long p = (unsigned long long)(P / G);  // exact: P is a multiple of G
      const unsigned long long S = units[3 * b + c];
      if (p + S < (1ull << 53)) {
        const double Pn = double(p + S) * G;
        if (Pn < rnd) {
          P = Pn;
          pick = b0 + bsz;
          continue;
        }
      }
    }
    P = seq_block(b0, bsz, P, rnd, pick, done);
  }
  return pick - 1;
}

// The stages of `gates`: which gates run in which pass, their tile bits and
// merged operations (StagePlanner); the kernels' substage data comes after.
std::vector<PlanStep> Engine::plan_stages(const std::vector<StageGate> &gates) const {
  // Tiles of 2^(r + 8) amplitudes (64 KB complex64, 32 KB complex128), with
  // runs of 2^5 / 2^4 contiguous amplitudes (256 bytes) in HBM.
  const unsigned L = prec_ == GSIM_C64 ? tile_bits_c64_ : tile_bits_c128_;
  const unsigned m = prec_ == GSIM_C64 ? 5 : 4;
  // complex64 stages get a pack bit where possible (the packed-pair kernel)
  const bool pk = prec_ == GSIM_C64 && stage_kernel_ == 2;
  StagePlanner planner(N_, L, m, 512, pk);
  return planner.plan(gates);
}

// A stage's substages for its kernel: packed pairs (complex64, with a pack
// bit), else register substages where the tile is 2^(r + 8) amplitudes (256
// threads), else none (the pass kernel).
void Engine::build_stage_data(StagePlan &sp) const {
  const unsigned r = prec_ == GSIM_C64 ? kRegBitsC64 : kRegBitsC128, rho = prec_ == GSIM_C64 ? 4 : 3;
  if (!(stage_kernel_ >= 1 && sp.L == r + 8)) return;
  if (prec_ == GSIM_C64 && stage_kernel_ == 2 && build_substages_pk(sp)) return;
  build_substages(sp, r, rho);
  if (stage_subs_bytes(sp) + sp.sops.size() * sizeof(SubOpDev) > kStageTableBytes) {
    sp.subs.clear();  // descriptors too large for the kernel parameter
    sp.sops.clear();
  }
}

std::vector<PlanStep> Engine::plan_staged(const std::vector<StageGate> &gates) const {
  std::vector<PlanStep> steps = plan_stages(gates);
  for (auto &st : steps)
    if (st.is_stage) build_stage_data(st.stage);
  return steps;
}

// The queued gates as stages, each stage's substages built just before its
// launch: the host builds stage k + 1 while the GPU runs stage k.
void Engine::run_staged() {
  if (queue_.empty()) return;
  std::vector<StageGate> gates = queued_positions();
  queue_.clear();
  std::vector<PlanStep> steps = plan_stages(gates);
  execute_staged(steps, true);
}

// Launch the steps in order.  Every stage's descriptors, tables and matrices
// go to their own slice of one page-locked staging buffer and are copied by
// their own cudaMemcpyAsync right before the stage's launch; the buffer is
// sized up front by an upper bound per stage (the substage data is at most
// kPkBlobMax / kStageTableBytes / the operation array, plus the matrices).
// build: the stages' substages are built here, one stage at a time.
void Engine::execute_staged(std::vector<PlanStep> &steps, bool build) {
  const size_t esz = bpa_;
  auto round16 = [](size_t n) { return (n + 15) / 16 * 16; };
  size_t bound = 0;
  for (auto const &st : steps) {
    if (!st.is_stage) continue;
    const StagePlan &sp = st.stage;
    bound += std::max({kPkBlobMax, kStageTableBytes, round16(sp.ops.size() * sizeof(StageOpDev))}) +
             round16(sp.pool.size() * esz);
  }
  char *host = nullptr, *dev = nullptr;
  if (bound) {
    upload_slot_ = (upload_slot_ + 1) % kUploadSlots;
    if (upload_ev_[upload_slot_]) CK(cudaEventSynchronize(upload_ev_[upload_slot_]));  // the slot is free again
    host = static_cast<char *>(upload_host_[upload_slot_].get(bound));
    dev = static_cast<char *>(upload_dev_.get(bound));
  }
  size_t off = 0;
  for (auto &st : steps) {
    if (!st.is_stage) {
      exec_dense(st.dense);
      continue;
    }
    StagePlan &sp = st.stage;
    if (build) build_stage_data(sp);
    const size_t o = off;
    // this stage's bytes, checked against the staging buffer before any write
    const size_t ops_bytes = !sp.pk.empty() ? round16(sp.pk.size())
                             : !sp.subs.empty() ? stage_subs_bytes(sp) + round16(sp.sops.size() * sizeof(SubOpDev))
                                                : round16(sp.ops.size() * sizeof(StageOpDev));
    const size_t need = ops_bytes + (sp.pk.empty() ? round16(sp.pool.size() * esz) : 0);
    if (o + need > bound) fail(GSIM_ERR_RUNTIME, "stage upload larger than its bound");
    size_t pool = 0;
    if (!sp.pk.empty()) {  // the packed-pair blob carries its own data
      std::memcpy(host + o, sp.pk.data(), sp.pk.size());
      off += round16(sp.pk.size());
      pool = off;
    } else {
      if (!sp.subs.empty()) {
        std::memcpy(host + o, sp.subs.data(), sp.subs.size() * sizeof(SubstageDev));
        std::memcpy(host + o + stage_subs_bytes(sp), sp.sops.data(), sp.sops.size() * sizeof(SubOpDev));
        off += stage_subs_bytes(sp) + round16(sp.sops.size() * sizeof(SubOpDev));
      } else {
        std::memcpy(host + o, sp.ops.data(), sp.ops.size() * sizeof(StageOpDev));
        off += round16(sp.ops.size() * sizeof(StageOpDev));
      }
      pool = off;  // for register stages the pool directly follows the operations
      if (prec_ == GSIM_C64) {
        float *f = reinterpret_cast<float *>(host + pool);
        for (size_t j = 0; j < sp.pool.size(); ++j) {
          f[2 * j] = float(sp.pool[j].real());
          f[2 * j + 1] = float(sp.pool[j].imag());
        }
      } else {
        std::memcpy(host + pool, sp.pool.data(), sp.pool.size() * 16);
      }
      off += round16(sp.pool.size() * esz);
    }
    CK(cudaMemcpyAsync(dev + o, host + o, off - o, cudaMemcpyHostToDevice, stream_));
    exec_stage(sp, dev + o, dev + pool);
  }
  if (bound) {
    cudaEvent_t &ev = upload_ev_[upload_slot_];
    if (!ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, stream_));
  }
}

void Engine::exec_stage(const StagePlan &sp, const void *d_ops, const void *d_pool) {
  const uint64_t bytes = 2 * (uint64_t(1) << N_) * bpa_;
  int e0 = -1;
  if (profiling_) e0 = record_event();
  CK(launch_stage(prec_, state_.p, N_, sp, d_ops, d_pool, stream_));
  if (profiling_) {
    const int e1 = record_event();
    Prof p;
    std::memset(&p.rec, 0, sizeof(p.rec));
    p.rec.kind = 1;
    p.rec.k = uint32_t(sp.ops.size());
    p.rec.nqubits = N_;
    for (unsigned q : sp.lpos) p.rec.targets |= uint64_t(1) << q;
    p.rec.bytes = bytes;
    p.rec.precision = uint32_t(prec_);
    p.rec.ngates = sp.ngates;
    p.rec.aux = sp.pk.empty() ? uint32_t(sp.subs.size()) : (sp.pk_nsubs | (1u << 16));
    p.ev0 = e0;
    p.ev1 = e1;
    prof_.push_back(p);
  }
  counters_[1] += 1;
  counters_[2] += bytes;
  counters_[3] += 1;
}


std::vector<StageGate> Engine::queued_positions() const {
  std::vector<StageGate> gates;
  gates.reserve(queue_.size());
  for (auto const &g : queue_) {
    StageGate sg;
    sg.m = g.m;
    for (unsigned id : g.ids) sg.pos.push_back(pos_of(id));
    for (unsigned c : g.ctrl) sg.ctrl_mask |= uint64_t(1) << pos_of(c);
    gates.push_back(std::move(sg));
  }
  return gates;
}

// The reference's greedy fusion (simulator.hpp:204-222) replayed over a gate
// list: the dense operations it would launch.
std::vector<DenseOp> Engine::reference_plan(const std::vector<StageGate> &gates) const {
  std::vector<DenseOp> out;
  RefFusion cur;
  auto flush = [&](RefFusion &f) {
    if (f.size() < 1) return;
    std::vector<cplx> M;
    std::vector<unsigned> q, c;
    f.compose(M, q, c);
    DenseOp op;
    op.m = std::move(M);
    op.pos = q;  // positions were used as ids
    for (unsigned x : c) op.ctrl_mask |= uint64_t(1) << x;
    out.push_back(std::move(op));
    f = RefFusion();
  };
  for (auto const &g : gates) {
    std::vector<unsigned> ctrl;
    for (unsigned b = 0; b < 64; ++b)
      if ((g.ctrl_mask >> b) & 1) ctrl.push_back(b);
    RefFusion f = cur;
    f.insert(g.m, g.pos, ctrl);
    const unsigned nf = f.num_qubits();
    if (nf >= fmin_ && nf <= fmax_) {
      cur = std::move(f);
      flush(cur);
    } else if (nf > fmax_ || (nf - unsigned(g.pos.size())) > cur.num_qubits()) {
      flush(cur);
      cur.insert(g.m, g.pos, ctrl);
    } else {
      cur = std::move(f);
    }
  }
  flush(cur);
  return out;
}

namespace {
// The reference's cluster admission (fusion.hpp:130-160) on qubit sets only:
// add gate g to a cluster with matrix qubits q, shared controls c and n gates.
void cluster_insert(uint64_t &q, uint64_t &c, size_t &n, const StageGate &g) {
  uint64_t t = 0;
  for (unsigned p : g.pos) t |= uint64_t(1) << p;
  q |= t;
  const uint64_t dropped = c & ~g.ctrl_mask;  // shared controls this gate lacks
  const uint64_t fresh = g.ctrl_mask & ~c;
  if (n) {
    q |= fresh;  // new controls become matrix qubits
  } else {
    c |= fresh;
  }
  if (dropped) {
    c &= ~dropped;
    q |= dropped;
  }
  ++n;
}
constexpr double kLaunchGapMs = 0.002;  // host launch gap added per kernel launch
}  // namespace

// Features of one kernel launch: the cost model's input, shared by training
// (recorded launches) and planning (candidate launches).
void launch_features(const gsim_launch_record &r, float *f) {
  std::fill(f, f + Engine::kFeatures, 0.f);
  const double B = r.precision == GSIM_C64 ? 8.0 : 16.0;
  const double amps = std::ldexp(1.0, int(r.nqubits));
  auto lg = [](double x) { return float(std::log2(1.0 + x)); };
  f[0] = float(r.nqubits) / 32.f;
  f[1] = r.precision == GSIM_C64 ? 1.f : 0.f;
  double flops;
  if (r.kind == 4 || r.kind == 5) {  // a Taylor-series or Chebyshev step of emulate_time_evolution: k = terms
    f[r.kind == 4 ? 17 : 18] = 1.f;
    f[19] = float(r.k) / 64.f;
    f[7] = float(r.nctrl) / 8.f;
    flops = amps * double(r.k);
  } else if (r.kind == 1) {  // stage: k = operations, aux = substages | packed-pair flag << 16
    f[3] = 1.f;
    flops = amps * double(r.k);
    f[12] = float(r.k) / 64.f;
    f[13] = float(r.aux & 0xFFFFu) / 32.f;
    f[16] = (r.aux >> 16) & 1u ? 1.f : 0.f;
  } else {
    f[2 + std::min<uint32_t>(r.kind, 3u)] = 1.f;
    const double touched = std::ldexp(1.0, int(r.nqubits) - int(r.nctrl));
    flops = touched * std::ldexp(1.0, int(r.k));
    f[6] = float(r.k) / 8.f;
    f[7] = float(r.nctrl) / 8.f;
    f[8] = r.targets ? float(__builtin_ctzll(r.targets)) / 32.f : 0.f;
    f[9] = float(__builtin_popcountll(r.targets & 0xFull)) / 4.f;
  }
  f[10] = lg(double(r.bytes)) / 48.f;
  f[11] = lg(flops) / 48.f;
  f[14] = amps * B <= 96e6 ? 1.f : 0.f;  // the state fits in L2
  f[15] = 1.f;
}

// The greedy fixed-size fusion (simulator.hpp:204-222) as clusters.
std::vector<Engine::Cluster> Engine::greedy_clusters(const std::vector<StageGate> &gates) const {
  std::vector<Cluster> out;
  Cluster cur;
  size_t n = 0;
  auto flush = [&](size_t end) {
    if (n) {
      cur.end = end;
      out.push_back(cur);
    }
    cur = Cluster();
    cur.begin = end;
    n = 0;
  };
  for (size_t i = 0; i < gates.size(); ++i) {
    const StageGate &g = gates[i];
    uint64_t q2 = cur.q, c2 = cur.c;
    size_t n2 = n;
    cluster_insert(q2, c2, n2, g);
    const unsigned nf = unsigned(__builtin_popcountll(q2));
    const unsigned nt = unsigned(g.pos.size());
    if (nf >= fmin_ && nf <= fmax_) {
      cur.q = q2, cur.c = c2, n = n2;
      flush(i + 1);
    } else if (nf > fmax_ || (nf - nt) > unsigned(__builtin_popcountll(cur.q))) {
      flush(i);
      cluster_insert(cur.q, cur.c, n, g);
    } else {
      cur.q = q2, cur.c = c2, n = n2;
    }
  }
  flush(gates.size());
  return out;
}

gsim_launch_record Engine::dense_record(uint64_t q, uint64_t c) const {
  gsim_launch_record r;
  std::memset(&r, 0, sizeof(r));
  const unsigned k = unsigned(__builtin_popcountll(q)), nc = unsigned(__builtin_popcountll(c));
  r.kind = uint32_t(dense_kind(k));
  r.k = k;
  r.nctrl = nc;
  r.nqubits = N_;
  r.targets = q;
  r.bytes = 2 * (uint64_t(1) << (N_ - nc)) * bpa_;
  r.precision = uint32_t(prec_);
  return r;
}

double Engine::predict_ms(const gsim_launch_record &r) {
  // The features depend only on these fields (bytes follows from nqubits,
  // nctrl and precision), so they key the memo of predictions.
  const uint64_t lowt = r.targets ? uint64_t(__builtin_ctzll(r.targets)) : 0;
  const uint64_t key = uint64_t(r.kind & 7u) | (uint64_t(r.k & 255u) << 3) | (uint64_t(r.nctrl & 63u) << 11) |
                       (lowt << 17) | (uint64_t(__builtin_popcountll(r.targets & 0xFull)) << 23) |
                       (uint64_t(r.nqubits & 63u) << 26) | (uint64_t(r.precision & 1u) << 32) |
                       (uint64_t(r.aux & 0x1FFFFu) << 33);
  auto it = memo_.find(key);
  if (it != memo_.end()) return it->second;
  float f[kFeatures];
  launch_features(r, f);
  const double ms = std::exp(double(predict(f)));
  memo_.emplace(key, ms);
  return ms;
}

double Engine::clusters_ms(const std::vector<Cluster> &cl) {
  double t = 0;
  for (auto const &c : cl) t += predict_ms(dense_record(c.q, c.c)) + kLaunchGapMs;
  return t;
}

double Engine::staged_ms(const std::vector<PlanStep> &steps) {
  double t = 0;
  for (auto const &st : steps) {
    if (!st.is_stage) {
      uint64_t q = 0;
      for (unsigned p : st.dense.pos) q |= uint64_t(1) << p;
      t += predict_ms(dense_record(q, st.dense.ctrl_mask)) + kLaunchGapMs;
      continue;
    }
    gsim_launch_record r;
    std::memset(&r, 0, sizeof(r));
    r.kind = 1;
    r.k = uint32_t(st.stage.ops.size());
    r.aux = st.stage.pk.empty() ? uint32_t(st.stage.subs.size()) : (st.stage.pk_nsubs | (1u << 16));
    r.nqubits = N_;
    r.bytes = 2 * (uint64_t(1) << N_) * bpa_;
    r.precision = uint32_t(prec_);
    t += predict_ms(r) + kLaunchGapMs;
  }
  return t;
}

// Cluster boundaries chosen by the cost model: walking the gates in order,
// the next gate joins the open cluster when the predicted time of the merged
// launch is below that of the open cluster plus the gate on its own (one
// launch more); clusters hold at most 7 qubits in complex64 (tensor cores
// from 5 targets up) and 5 in complex128 (FP64 on CUDA cores).
std::vector<Engine::Cluster> Engine::learned_clusters(const std::vector<StageGate> &gates) {
  const int cap = prec_ == GSIM_C64 ? 7 : 5;
  std::vector<Cluster> out;
  Cluster cur;
  size_t n = 0;
  for (size_t i = 0; i < gates.size(); ++i) {
    const StageGate &g = gates[i];
    if (n == 0) {
      cur = Cluster();
      cur.begin = i;
      cur.end = i + 1;
      cluster_insert(cur.q, cur.c, n, g);
      continue;
    }
    Cluster m = cur;
    size_t n2 = n;
    cluster_insert(m.q, m.c, n2, g);
    m.end = i + 1;
    bool merge = false;
    if (__builtin_popcountll(m.q) <= cap) {
      Cluster one;
      size_t n1 = 0;
      cluster_insert(one.q, one.c, n1, g);
      const double t_merge = predict_ms(dense_record(m.q, m.c));
      const double t_split = predict_ms(dense_record(cur.q, cur.c)) + predict_ms(dense_record(one.q, one.c)) +
                             kLaunchGapMs;
      merge = t_merge <= t_split;
    }
    if (merge) {
      cur = m;
      n = n2;
    } else {
      out.push_back(cur);
      cur = Cluster();
      cur.begin = i;
      cur.end = i + 1;
      n = 0;
      cluster_insert(cur.q, cur.c, n, g);
    }
  }
  if (n) out.push_back(cur);
  return out;
}

// Compose each cluster's gates in order (the reference's fusion object,
// positions used as ids) and launch it as one dense gate.
void Engine::exec_clusters(std::vector<StageGate> &gates, const std::vector<Cluster> &cl) {
  for (auto const &c : cl) {
    RefFusion f;
    for (size_t i = c.begin; i < c.end; ++i) {
      std::vector<unsigned> ctrl;
      for (unsigned b = 0; b < 64; ++b)
        if ((gates[i].ctrl_mask >> b) & 1) ctrl.push_back(b);
      f.insert(std::move(gates[i].m), gates[i].pos, ctrl);
    }
    std::vector<cplx> M;
    std::vector<unsigned> q, cs;
    f.compose(M, q, cs);
    if (q.size() > 7) fail(GSIM_ERR_RUNTIME, "learned planner: cluster wider than 7 qubits");
    DenseOp op;
    op.m = std::move(M);
    op.pos = q;
    for (unsigned x : cs) op.ctrl_mask |= uint64_t(1) << x;
    exec_dense(op);
  }
}

float Engine::predict(const float *x) const {
  const int F = kFeatures, H = cm_H_;
  const float *W1 = cm_.data(), *b1 = W1 + size_t(H) * F, *W2 = b1 + H, *b2 = W2 + size_t(H) * H, *W3 = b2 + H,
              *b3 = W3 + H;
  std::vector<float> a1(H), a2(H);
  for (int o = 0; o < H; ++o) {
    float s = b1[o];
    for (int i = 0; i < F; ++i) s = std::fma(W1[o * F + i], x[i], s);
    a1[o] = std::max(s, 0.f);
  }
  for (int o = 0; o < H; ++o) {
    float s = b2[o];
    for (int i = 0; i < H; ++i) s = std::fma(W2[o * H + i], a1[i], s);
    a2[o] = std::max(s, 0.f);
  }
  float s = b3[0];
  for (int i = 0; i < H; ++i) s = std::fma(W3[i], a2[i], s);
  return s;
}

// GSIM_FUSION_LEARNED: the queued gates run as the plan with the lowest
// predicted time among the greedy fixed-size clusters, the cost-model
// clusters and the stage plan.  Without a cost model, or on a state size
// where learned plans did not beat the greedy fusion in measured wall time,
// the greedy fixed-size fusion runs.
void Engine::run_learned() {
  if (queue_.empty()) return;
  std::vector<StageGate> gates = queued_positions();
  queue_.clear();
  if (cm_.empty() || !learned_ok_[std::min<unsigned>(N_, 64)]) {
    for (auto const &op : reference_plan(gates)) exec_dense(op);
    last_choice_ = GSIM_FUSION_REFERENCE;
    return;
  }
  std::vector<PlanStep> staged = plan_staged(gates);
  const std::vector<Cluster> learned = learned_clusters(gates);
  const double t_greedy = clusters_ms(greedy_clusters(gates));
  const double t_staged = staged_ms(staged);
  const double t_learned = clusters_ms(learned);
  // The stage plan is kept unless another is predicted at least 10% faster:
  // the model's error on one launch is about 15%, and near-ties measured no
  // better than the stage plan.
  int best = GSIM_FUSION_STAGED;
  double best_t = t_staged;
  const double margin = 0.9;
  if (t_greedy < margin * best_t) best = GSIM_FUSION_REFERENCE, best_t = t_greedy;
  if (t_learned < margin * t_staged && t_learned < best_t) best = GSIM_FUSION_LEARNED, best_t = t_learned;
  last_choice_ = best;
  last_pred_[0] = t_greedy;
  last_pred_[1] = t_staged;
  last_pred_[2] = t_learned;
  if (best == GSIM_FUSION_STAGED) {
    execute_staged(staged);
  } else if (best == GSIM_FUSION_LEARNED) {
    exec_clusters(gates, learned);
  } else {
    for (auto const &op : reference_plan(gates)) exec_dense(op);
  }
}

}  // namespace gsim

// ===========================================================================
// C ABI
// ===========================================================================
using gsim::Engine;
using gsim::Error;
using gsim::fail;

namespace {
template <class F>
int guard(F &&f) {
  try {
    f();
    return GSIM_OK;
  } catch (const Error &e) {
    gsim::g_last_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    gsim::g_last_error = "out of host memory";
    return GSIM_ERR_MEMORY;
  } catch (const std::invalid_argument &e) {
    gsim::g_last_error = e.what();
    return GSIM_ERR_VALUE;
  } catch (const std::exception &e) {
    gsim::g_last_error = e.what();
    return GSIM_ERR_RUNTIME;
  }
}
Engine *E(gsim_engine *e) {
  if (!e) gsim::fail(GSIM_ERR_VALUE, "null engine handle");
  return reinterpret_cast<Engine *>(e);
}
std::vector<unsigned> vu(const uint32_t *p, size_t n) {
  return n ? std::vector<unsigned>(p, p + n) : std::vector<unsigned>();
}
std::vector<unsigned> reg_sizes(const uint32_t *s, size_t n) { return vu(s, n); }

// Pauli terms in CSR form -> engine terms (positions resolved through ids,
// factors combined by pauli_term_of in the order given).
std::vector<gsim::PauliTerm> terms_of(Engine *eng, const uint32_t *off, const uint32_t *q,
                                      const uint8_t *pa, size_t nterms, const uint32_t *ids,
                                      size_t nids) {
  const std::map<unsigned, unsigned> &m = eng->mapping();
  std::vector<gsim::PauliTerm> out(nterms);
  std::vector<std::pair<unsigned, char>> factors;
  for (size_t t = 0; t < nterms; ++t) {
    factors.clear();
    for (uint32_t f = off[t]; f < off[t + 1]; ++f) {
      if (q[f] >= nids) gsim::fail(GSIM_ERR_VALUE, "Pauli term acts on a qubit index outside the qureg");
      auto it = m.find(ids[q[f]]);
      if (it == m.end())
        gsim::fail(GSIM_ERR_RUNTIME, "Unknown qubit id. Please make sure you have called eng.flush().");
      factors.emplace_back(it->second, char(pa[f]));
    }
    if (!gsim::pauli_term_of(factors, out[t])) gsim::fail(GSIM_ERR_VALUE, "Pauli must be X, Y or Z");
  }
  return out;
}
std::vector<unsigned> reg_shift(const uint32_t *sizes, size_t nregs) {
  std::vector<unsigned> sh(nregs, 0);
  for (size_t r = 1; r < nregs; ++r) sh[r] = sh[r - 1] + sizes[r - 1];
  return sh;
}
// Per-register function on 32-bit ints, as the reference's lambdas
// (simulator.hpp:275,282,289); results are truncated to the register width.
template <class F>
int math_fast(gsim_engine *e, F f, const uint32_t *reg_ids, const uint32_t *sizes,
                     size_t nregs, const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    size_t W = 0;
    for (size_t r = 0; r < nregs; ++r) W += sizes[r];
    auto sh = reg_shift(sizes, nregs);
    auto g = [&](uint64_t x) {
      uint64_t y = 0;
      for (size_t r = 0; r < nregs; ++r) {
        const uint64_t mask = (uint64_t(1) << sizes[r]) - 1;
        const int v = int((x >> sh[r]) & mask);
        const int res = f(v);
        y |= (uint64_t(uint32_t(res)) & mask) << sh[r];
      }
      return y;
    };
    E(e)->emulate_math(g, vu(reg_ids, W), reg_sizes(sizes, nregs), vu(ctrl, nctrl));
  });
}

}  // namespace

extern "C" {

const char *gsim_last_error(void) { return gsim::g_last_error.c_str(); }

int gsim_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int gsim_create(uint32_t seed, int precision, gsim_engine **out) {
  return guard([&] {
    if (!out) gsim::fail(GSIM_ERR_VALUE, "null output pointer");
    *out = reinterpret_cast<gsim_engine *>(new Engine(seed, precision));
  });
}
int gsim_destroy(gsim_engine *e) {
  return guard([&] { delete reinterpret_cast<Engine *>(e); });
}
int gsim_allocate_qubit(gsim_engine *e, uint32_t id) {
  return guard([&] { E(e)->allocate_qubit(id); });
}
int gsim_deallocate_qubit(gsim_engine *e, uint32_t id) {
  return guard([&] { E(e)->deallocate_qubit(id); });
}
int gsim_get_classical_value(gsim_engine *e, uint32_t id, double tol, int *out) {
  return guard([&] { *out = E(e)->get_classical_value(id, tol) ? 1 : 0; });
}
int gsim_is_classical(gsim_engine *e, uint32_t id, double tol, int *out) {
  return guard([&] { *out = E(e)->is_classical(id, tol) ? 1 : 0; });
}
int gsim_measure_qubits(gsim_engine *e, const uint32_t *ids, size_t n, uint8_t *out) {
  return guard([&] {
    auto r = E(e)->measure(vu(ids, n), false, 0.);
    std::copy(r.begin(), r.end(), out);
  });
}
int gsim_measure_qubits_at(gsim_engine *e, const uint32_t *ids, size_t n, double rnd, uint8_t *out) {
  return guard([&] {
    auto r = E(e)->measure(vu(ids, n), true, rnd);
    std::copy(r.begin(), r.end(), out);
  });
}
int gsim_apply_controlled_gate(gsim_engine *e, const double *m, uint32_t k, const uint32_t *ids,
                               const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    if (k == 0 || k > 16) gsim::fail(GSIM_ERR_VALUE, "apply_controlled_gate(): bad gate width");
    const size_t d = size_t(1) << k;
    std::vector<gsim::cplx> M(d * d);
    for (size_t i = 0; i < d * d; ++i) M[i] = gsim::cplx(m[2 * i], m[2 * i + 1]);
    E(e)->apply_controlled_gate(std::move(M), vu(ids, k), vu(ctrl, nctrl));
  });
}
int gsim_apply_gates(gsim_engine *e, size_t n, const uint32_t *nt, const uint32_t *nc, const uint32_t *qubits,
                     const double *mats, size_t *failed_at) {
  size_t g = 0;
  const int rc = guard([&] {
    size_t qo = 0, mo = 0;
    for (; g < n; ++g) {
      const uint32_t k = nt[g];
      if (k == 0 || k > 16) gsim::fail(GSIM_ERR_VALUE, "apply_gates(): bad gate width");
      const size_t d = size_t(1) << k;
      std::vector<gsim::cplx> M(d * d);
      for (size_t i = 0; i < d * d; ++i) M[i] = gsim::cplx(mats[mo + 2 * i], mats[mo + 2 * i + 1]);
      E(e)->apply_controlled_gate(std::move(M), vu(qubits + qo, k), vu(qubits + qo + k, nc[g]));
      qo += k + nc[g];
      mo += 2 * d * d;
    }
  });
  if (failed_at) *failed_at = rc == GSIM_OK ? n : g;
  return rc;
}
int gsim_run(gsim_engine *e) {
  return guard([&] { E(e)->run(); });
}

int gsim_emulate_math_add_constant(gsim_engine *e, int32_t a, const uint32_t *reg_ids,
                                   const uint32_t *reg_sizes_, size_t nregs, const uint32_t *ctrl,
                                   size_t nctrl) {
  return math_fast(e, [a](int x) { return int(uint32_t(x) + uint32_t(a)); }, reg_ids, reg_sizes_,
                   nregs, ctrl, nctrl);
}
int gsim_emulate_math_add_constant_modn(gsim_engine *e, int32_t a, int32_t N, const uint32_t *reg_ids,
                                        const uint32_t *reg_sizes_, size_t nregs,
                                        const uint32_t *ctrl, size_t nctrl) {
  if (N == 0) {
    gsim::g_last_error = "modulus N must be nonzero";
    return GSIM_ERR_VALUE;
  }
  return math_fast(e, [a, N](int x) { return int(uint32_t(x) + uint32_t(a)) % N; }, reg_ids,
                   reg_sizes_, nregs, ctrl, nctrl);
}
int gsim_emulate_math_multiply_by_constant_modn(gsim_engine *e, int32_t a, int32_t N,
                                                const uint32_t *reg_ids, const uint32_t *reg_sizes_,
                                                size_t nregs, const uint32_t *ctrl, size_t nctrl) {
  if (N == 0) {
    gsim::g_last_error = "modulus N must be nonzero";
    return GSIM_ERR_VALUE;
  }
  return math_fast(e, [a, N](int x) { return int(uint32_t(x) * uint32_t(a)) % N; }, reg_ids,
                   reg_sizes_, nregs, ctrl, nctrl);
}
int gsim_emulate_math_table(gsim_engine *e, const uint64_t *table, const uint32_t *reg_ids,
                            const uint32_t *sizes, size_t nregs, const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    size_t W = 0;
    for (size_t r = 0; r < nregs; ++r) W += sizes[r];
    if (W > 26) gsim::fail(GSIM_ERR_VALUE, "emulate_math(): at most 26 register qubits are supported");
    auto sh = reg_shift(sizes, nregs);
    auto g = [&](uint64_t x) {
      const uint64_t y = table[x];
      uint64_t r = 0;
      for (size_t k = 0; k < nregs; ++k) {
        const uint64_t mask = (uint64_t(1) << sizes[k]) - 1;
        r |= ((y >> sh[k]) & mask) << sh[k];
      }
      return r;
    };
    E(e)->emulate_math(g, vu(reg_ids, W), reg_sizes(sizes, nregs), vu(ctrl, nctrl));
  });
}

int gsim_get_expectation_value(gsim_engine *e, const uint32_t *off, const uint32_t *q,
                               const uint8_t *pa, const double *coeffs, size_t nterms,
                               const uint32_t *ids, size_t nids, double *out) {
  return guard([&] {
    Engine *eng = E(e);
    eng->run();
    auto terms = terms_of(eng, off, q, pa, nterms, ids, nids);
    *out = eng->get_expectation_value(terms, std::vector<double>(coeffs, coeffs + nterms));
  });
}
int gsim_apply_qubit_operator(gsim_engine *e, const uint32_t *off, const uint32_t *q,
                              const uint8_t *pa, const double *coeffs, size_t nterms,
                              const uint32_t *ids, size_t nids) {
  return guard([&] {
    Engine *eng = E(e);
    eng->run();
    auto terms = terms_of(eng, off, q, pa, nterms, ids, nids);
    std::vector<gsim::cplx> c(nterms);
    for (size_t t = 0; t < nterms; ++t) c[t] = gsim::cplx(coeffs[2 * t], coeffs[2 * t + 1]);
    eng->apply_qubit_operator(terms, c);
  });
}
int gsim_emulate_time_evolution(gsim_engine *e, const uint32_t *off, const uint32_t *q,
                                const uint8_t *pa, const double *coeffs, size_t nterms, double time,
                                const uint32_t *ids, size_t nids, const uint32_t *ctrl, size_t nctrl) {
  return guard([&] {
    Engine *eng = E(e);
    eng->run();
    auto terms = terms_of(eng, off, q, pa, nterms, ids, nids);
    eng->emulate_time_evolution(terms, std::vector<double>(coeffs, coeffs + nterms), time, vu(ctrl, nctrl));
  });
}
int gsim_get_probability(gsim_engine *e, const uint8_t *bits, const uint32_t *ids, size_t n, double *out) {
  return guard([&] { *out = E(e)->get_probability(std::vector<uint8_t>(bits, bits + n), vu(ids, n)); });
}
int gsim_get_amplitude(gsim_engine *e, const uint8_t *bits, const uint32_t *ids, size_t n, double *out) {
  return guard([&] {
    auto a = E(e)->get_amplitude(std::vector<uint8_t>(bits, bits + n), vu(ids, n));
    out[0] = a.real();
    out[1] = a.imag();
  });
}
int gsim_set_wavefunction(gsim_engine *e, const void *wf, int dtype, size_t len, const uint32_t *ordering,
                          size_t n) {
  return guard([&] { E(e)->set_wavefunction(wf, dtype, len, vu(ordering, n)); });
}
int gsim_collapse_wavefunction(gsim_engine *e, const uint32_t *ids, size_t n, const uint8_t *values,
                               size_t nvalues) {
  return guard([&] {
    E(e)->collapse_wavefunction(vu(ids, n), std::vector<uint8_t>(values, values + nvalues));
  });
}
int gsim_num_qubits(gsim_engine *e, uint32_t *out) {
  return guard([&] { *out = E(e)->num_qubits(); });
}
int gsim_get_mapping(gsim_engine *e, uint32_t *ids, uint32_t *positions, size_t cap) {
  return guard([&] {
    size_t i = 0;
    for (auto const &p : E(e)->mapping()) {
      if (i >= cap) break;
      ids[i] = p.first;
      positions[i] = p.second;
      ++i;
    }
  });
}
int gsim_get_state(gsim_engine *e, void *host, int dtype, size_t offset, size_t count) {
  return guard([&] { E(e)->get_state(host, dtype, offset, count); });
}
int gsim_state_device_ptr(gsim_engine *e, void **ptr, size_t *len, int *dtype) {
  return guard([&] { E(e)->device_view(ptr, len, dtype); });
}
int gsim_synchronize(gsim_engine *e) {
  return guard([&] { E(e)->synchronize(); });
}
int gsim_set_fusion(gsim_engine *e, int mode, uint32_t kmax) {
  return guard([&] { E(e)->set_fusion(mode, kmax); });
}
int gsim_reserve(gsim_engine *e, uint32_t nqubits) {
  return guard([&] { E(e)->reserve(nqubits); });
}
int gsim_get_counters(gsim_engine *e, uint64_t *out, size_t n) {
  return guard([&] {
    for (size_t i = 0; i < n; ++i) out[i] = E(e)->counter(i);
  });
}
int gsim_reset_counters(gsim_engine *e) {
  return guard([&] { E(e)->reset_counters(); });
}
int gsim_adjoint_gradient(gsim_engine *e, size_t nops, const uint8_t *kind, const uint32_t *target,
                          const uint32_t *ctrl_off, const uint32_t *ctrl_ids, const int32_t *param,
                          const double *mats, const double *theta, size_t nparams,
                          const uint32_t *term_offsets, const uint32_t *op_qubit, const uint8_t *op_pauli,
                          const double *coeffs, size_t nterms, const uint32_t *ids, size_t nids,
                          uint32_t checkpoint_every, double *energy, double *grad) {
  return guard([&] {
    Engine *eng = E(e);
    eng->run();
    const auto &m = eng->mapping();
    auto pos = [&](uint32_t id) {
      auto it = m.find(id);
      if (it == m.end()) fail(GSIM_ERR_RUNTIME, "adjoint_gradient(): unknown qubit id " + std::to_string(id));
      return it->second;
    };
    std::vector<gsim::AdjointGate> gates(nops);
    std::vector<int> prm(nops, -1);
    std::vector<double> scale(nops, 0.);
    using gsim::cplx;
    const cplx I(0., 1.);
    for (size_t i = 0; i < nops; ++i) {
      gsim::AdjointGate &g = gates[i];
      g.target = pos(target[i]);
      for (uint32_t c = ctrl_off[i]; c < ctrl_off[i + 1]; ++c) {
        const unsigned p = pos(ctrl_ids[c]);
        if (p == g.target) fail(GSIM_ERR_VALUE, "adjoint_gradient(): a control is also the target");
        g.ctrl_mask |= uint64_t(1) << p;
      }
      if (kind[i] == 0) {
        for (int j = 0; j < 4; ++j) g.u[j] = cplx(mats[8 * i + 2 * j], mats[8 * i + 2 * j + 1]);
        continue;
      }
      if (param[i] < 0 || size_t(param[i]) >= nparams)
        fail(GSIM_ERR_VALUE, "adjoint_gradient(): parameter index out of range");
      prm[i] = param[i];
      const double t = theta[param[i]], c = std::cos(0.5 * t), s = std::sin(0.5 * t);
      switch (kind[i]) {
        case 1:  // Rx (projectq/ops/_gates.py:276-281)
          g.u[0] = c; g.u[1] = -I * s; g.u[2] = -I * s; g.u[3] = c; g.gen = 0; scale[i] = 1.;
          break;
        case 2:  // Ry (:290-295)
          g.u[0] = c; g.u[1] = -s; g.u[2] = s; g.u[3] = c; g.gen = 1; scale[i] = 1.;
          break;
        case 3:  // Rz (:304-309)
          g.u[0] = std::exp(-0.5 * I * t); g.u[1] = 0.; g.u[2] = 0.; g.u[3] = std::exp(0.5 * I * t);
          g.gen = 2; scale[i] = 1.;
          break;
        case 4:  // Ph (:267)
          g.u[0] = std::exp(I * t); g.u[1] = 0.; g.u[2] = 0.; g.u[3] = std::exp(I * t); g.gen = 3; scale[i] = -2.;
          break;
        case 5:  // R (diag(1, e^{i t}))
          g.u[0] = 1.; g.u[1] = 0.; g.u[2] = 0.; g.u[3] = std::exp(I * t); g.gen = 4; scale[i] = -2.;
          break;
        default:
          fail(GSIM_ERR_VALUE, "adjoint_gradient(): unknown gate kind");
      }
    }
    auto terms = terms_of(eng, term_offsets, op_qubit, op_pauli, nterms, ids, nids);
    eng->adjoint(gates, prm, scale, nparams, terms, std::vector<double>(coeffs, coeffs + nterms),
                 checkpoint_every, energy, grad);
  });
}
int gsim_compare_states(gsim_engine *a, gsim_engine *b, double *out) {
  return guard([&] { E(a)->compare(*E(b), out); });
}
int gsim_launch_features(const gsim_launch_record *recs, size_t n, float *out, size_t nfeat) {
  return guard([&] {
    if (nfeat < size_t(Engine::kFeatures)) fail(GSIM_ERR_LENGTH, "launch_features(): nfeat < 20");
    for (size_t i = 0; i < n; ++i) {
      float f[Engine::kFeatures];
      gsim::launch_features(recs[i], f);
      std::fill(out + i * nfeat, out + (i + 1) * nfeat, 0.f);
      std::copy(f, f + Engine::kFeatures, out + i * nfeat);
    }
  });
}
int gsim_set_cost_model(gsim_engine *e, int nfeatures, int hidden, const float *params) {
  return guard([&] { E(e)->set_cost_model(nfeatures, hidden, params); });
}
int gsim_set_learned_regimes(gsim_engine *e, const uint8_t *allowed, size_t count) {
  return guard([&] {
    if (count > 65) fail(GSIM_ERR_LENGTH, "set_learned_regimes(): at most 65 entries");
    E(e)->set_learned_regimes(allowed, count);
  });
}
int gsim_cost_model_predict(gsim_engine *e, const float *features, size_t n, float *out) {
  return guard([&] { E(e)->predict_rows(features, n, out); });
}
int gsim_last_plan_choice(gsim_engine *e, int *mode, double *pred_ms) {
  return guard([&] {
    *mode = E(e)->last_choice();
    if (pred_ms) E(e)->last_prediction(pred_ms);
  });
}
int gsim_set_upload_mode(gsim_engine *e, int mode) {
  return guard([&] { E(e)->set_upload_mode(mode); });
}
int gsim_set_stage_kernel(gsim_engine *e, int mode) {
  return guard([&] { E(e)->set_stage_kernel(mode); });
}
int gsim_set_tensor_cores(gsim_engine *e, int mode) {
  return guard([&] { E(e)->set_tensor_cores(mode); });
}
int gsim_set_time_evolution(gsim_engine *e, int mode) {
  return guard([&] { E(e)->set_time_evolution(mode); });
}
int gsim_set_device(int device) {
  return guard([&] { CK(cudaSetDevice(device)); });
}
int gsim_timer_mark(gsim_engine *e, int slot) {
  return guard([&] { E(e)->timer_mark(slot); });
}
int gsim_timer_elapsed(gsim_engine *e, int a, int b, float *ms) {
  return guard([&] { *ms = E(e)->timer_elapsed(a, b); });
}
int gsim_profile_enable(gsim_engine *e, int on) {
  return guard([&] { E(e)->profile_enable(on != 0); });
}
int gsim_profile_fetch(gsim_engine *e, gsim_launch_record *out, size_t cap, size_t *n) {
  return guard([&] { *n = E(e)->profile_fetch(out, cap); });
}
int gsim_profile_clear(gsim_engine *e) {
  return guard([&] { E(e)->profile_clear(); });
}
int gsim_host_register(void *ptr, size_t bytes) {
  return guard([&] { CK(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault)); });
}
int gsim_host_unregister(void *ptr) {
  return guard([&] { CK(cudaHostUnregister(ptr)); });
}

}  // extern "C"
