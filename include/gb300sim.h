/*
 * gb300sim.h — C ABI of the GB300 (sm_103a) state-vector simulator core.
 *
 * The library libgb300sim.so is a drop-in for the native engine behind
 * ProjectQ's Python backend `projectq.backends.Simulator`, i.e. the pybind11
 * class `projectq.backends._sim._cppsim.Simulator` bound in
 * projectq/backends/_sim/_cppsim.cpp:45-66 and implemented in
 * projectq/backends/_sim/_cppkernels/simulator.hpp:37-575.  Each entry point
 * below names the reference method it replaces (file:line).
 *
 * Conventions
 *  - Every function returns an int status: GSIM_OK (0) or one of the GSIM_ERR_*
 *    codes.  The message of the last failure on the calling thread is returned
 *    by gsim_last_error().  The codes mirror the C++ exception classes the
 *    reference throws and pybind11 translates:
 *      std::runtime_error    -> GSIM_ERR_RUNTIME -> Python RuntimeError
 *      std::invalid_argument -> GSIM_ERR_VALUE   -> Python ValueError
 *      std::length_error     -> GSIM_ERR_LENGTH  -> Python ValueError
 *  - Qubits are named by caller-chosen 32-bit ids.  The engine keeps the
 *    id -> bit-position map (simulator.hpp:42,567); the i-th allocated qubit
 *    takes bit position i (simulator.hpp:57).
 *  - Matrices are 2^k x 2^k complex128, row-major, interleaved (re, im):
 *    2 * 4^k doubles.  Matrix bit l corresponds to ids[l] (ids[0] = LSB),
 *    as in the reference kernels (fusion.hpp:79-100).
 *  - Pauli terms are passed in CSR form: term t owns the factors
 *    [term_offsets[t], term_offsets[t+1]) of op_qubit[] (an index into ids[])
 *    and op_pauli[] (the characters 'X', 'Y', 'Z').  This is the reference's
 *    Term = vector<pair<unsigned, char>> (simulator.hpp:44-46).
 *  - All state lives in device memory of the current CUDA device.  Calls are
 *    asynchronous on the engine's own stream except where a host result is
 *    returned.  An engine is not thread-safe (as in the reference).
 */
#ifndef GB300SIM_H_
#define GB300SIM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSIM_OK 0
#define GSIM_ERR_RUNTIME 1
#define GSIM_ERR_VALUE 2
#define GSIM_ERR_LENGTH 3
#define GSIM_ERR_CUDA 4
#define GSIM_ERR_MEMORY 5

/* Storage precision of the state vector. */
#define GSIM_C128 0 /* complex128: the plain method, same arithmetic as the reference */
#define GSIM_C64 1  /* complex64 storage, FP64 reductions */

/* Fusion planners (the reference has exactly one: GSIM_FUSION_REFERENCE). */
#define GSIM_FUSION_REFERENCE 0 /* simulator.hpp:204-222 + fusion.hpp, window 4..5 */
#define GSIM_FUSION_NONE 1      /* every gate is its own pass */
#define GSIM_FUSION_STAGED 2    /* shared-memory tiles: many gates per HBM pass */
#define GSIM_FUSION_LEARNED 3   /* per flush, the planner a learned cost model predicts fastest */

#if defined(__GNUC__)
#define GSIM_API __attribute__((visibility("default")))
#else
#define GSIM_API
#endif

typedef struct gsim_engine gsim_engine;

/* Message of the last failed call on this thread ("" if none). */
GSIM_API const char *gsim_last_error(void);

/* Number of CUDA devices visible (0 when no GPU); never fails. */
GSIM_API int gsim_device_count(void);

/* Simulator(seed) — simulator.hpp:48-53 (_cppsim.cpp:46).  precision is
 * GSIM_C128 or GSIM_C64.  The RNG is std::mt19937(seed) feeding
 * std::uniform_real_distribution<double>(0, 1), as in the reference. */
GSIM_API int gsim_create(uint32_t seed, int precision, gsim_engine **out);

/* ~Simulator — simulator.hpp:534-535.  Frees all device memory of the engine. */
GSIM_API int gsim_destroy(gsim_engine *e);

/* allocate_qubit — simulator.hpp:55-74.  The new qubit is the new top bit. */
GSIM_API int gsim_allocate_qubit(gsim_engine *e, uint32_t id);

/* deallocate_qubit — simulator.hpp:194-202.  RUNTIME error if not classical. */
GSIM_API int gsim_deallocate_qubit(gsim_engine *e, uint32_t id);

/* get_classical_value — simulator.hpp:76-91. */
GSIM_API int gsim_get_classical_value(gsim_engine *e, uint32_t id, double tol, int *out);

/* is_classical — simulator.hpp:93-108. */
GSIM_API int gsim_is_classical(gsim_engine *e, uint32_t id, double tol, int *out);

/* measure_qubits / measure_qubits_return — simulator.hpp:145-192.  One draw
 * of the engine RNG per call; out[i] in {0,1}. */
GSIM_API int gsim_measure_qubits(gsim_engine *e, const uint32_t *ids, size_t n, uint8_t *out);

/* measure_qubits with the uniform draw supplied by the caller instead of the
 * engine RNG (same sampling rule, simulator.hpp:152-160), for parity checks
 * "at a given draw". */
GSIM_API int gsim_measure_qubits_at(gsim_engine *e, const uint32_t *ids, size_t n, double rnd,
                           uint8_t *out);

/* A stream of n gates in one call, the same as n gsim_apply_controlled_gate
 * calls in order (no reference counterpart: the reference's Python layer calls
 * apply_controlled_gate per gate, _simulator.py:404-415).  Gate g has nt[g]
 * targets and nc[g] controls; `qubits` holds, gate after gate, its targets
 * then its controls; `mats` holds, gate after gate, its 2^nt x 2^nt matrix
 * (row-major, interleaved re/im).  On an error, the gates before the failing
 * one have been queued and *failed_at (if not NULL) is its index. */
GSIM_API int gsim_apply_gates(gsim_engine *e, size_t n, const uint32_t *nt, const uint32_t *nc,
                              const uint32_t *qubits, const double *mats, size_t *failed_at);

/* apply_controlled_gate — simulator.hpp:204-222 (fusion: fusion.hpp:56-63). */
GSIM_API int gsim_apply_controlled_gate(gsim_engine *e, const double *m, uint32_t k,
                               const uint32_t *ids, const uint32_t *ctrl, size_t nctrl);

/* run — simulator.hpp:487-527: apply every pending gate.  VALUE error for a
 * fused gate wider than the engine's maximum (5, as in simulator.hpp:522). */
GSIM_API int gsim_run(gsim_engine *e);

/* emulate_math_addConstant — simulator.hpp:272-276.  Registers are given as
 * reg_ids (all registers concatenated) and reg_sizes[nregs]. */
GSIM_API int gsim_emulate_math_add_constant(gsim_engine *e, int32_t a, const uint32_t *reg_ids,
                                   const uint32_t *reg_sizes, size_t nregs,
                                   const uint32_t *ctrl, size_t nctrl);

/* emulate_math_addConstantModN — simulator.hpp:279-283. */
GSIM_API int gsim_emulate_math_add_constant_modn(gsim_engine *e, int32_t a, int32_t N,
                                        const uint32_t *reg_ids, const uint32_t *reg_sizes,
                                        size_t nregs, const uint32_t *ctrl, size_t nctrl);

/* emulate_math_multiplyByConstantModN — simulator.hpp:286-290. */
GSIM_API int gsim_emulate_math_multiply_by_constant_modn(gsim_engine *e, int32_t a, int32_t N,
                                                const uint32_t *reg_ids,
                                                const uint32_t *reg_sizes, size_t nregs,
                                                const uint32_t *ctrl, size_t nctrl);

/* emulate_math with a caller function — simulator.hpp:224-269 and
 * _cppsim.cpp:33-41.  Instead of one callback per basis state, the caller
 * tabulates the function once: table[x] is the packed output for the packed
 * register input x (register 0 in the lowest reg_sizes[0] bits, and so on),
 * for all 2^W inputs, W = sum(reg_sizes) <= 26. */
GSIM_API int gsim_emulate_math_table(gsim_engine *e, const uint64_t *table, const uint32_t *reg_ids,
                            const uint32_t *reg_sizes, size_t nregs, const uint32_t *ctrl,
                            size_t nctrl);

/* get_expectation_value — simulator.hpp:292-322 (+ apply_term :538-550).
 * Real coefficients, as the reference's TermsDict (simulator.hpp:45). */
GSIM_API int gsim_get_expectation_value(gsim_engine *e, const uint32_t *term_offsets,
                               const uint32_t *op_qubit, const uint8_t *op_pauli,
                               const double *coeffs, size_t nterms, const uint32_t *ids,
                               size_t nids, double *out);

/* apply_qubit_operator — simulator.hpp:324-350.  Complex coefficients,
 * interleaved (re, im): 2 * nterms doubles. */
GSIM_API int gsim_apply_qubit_operator(gsim_engine *e, const uint32_t *term_offsets,
                              const uint32_t *op_qubit, const uint8_t *op_pauli,
                              const double *coeffs, size_t nterms, const uint32_t *ids,
                              size_t nids);

/* emulate_time_evolution — simulator.hpp:386-438.  Real coefficients.
 * By default, when every pair of non-identity terms commutes and no term acts
 * on a control, exp(-i t H) is applied exactly as the product of the terms'
 * exponentials (one gate per term, fused by the planner); otherwise by the
 * reference's Taylor series (see gsim_set_time_evolution). */
GSIM_API int gsim_emulate_time_evolution(gsim_engine *e, const uint32_t *term_offsets,
                                const uint32_t *op_qubit, const uint8_t *op_pauli,
                                const double *coeffs, size_t nterms, double time,
                                const uint32_t *ids, size_t nids, const uint32_t *ctrl,
                                size_t nctrl);

/* get_probability — simulator.hpp:352-368.  bits[i] in {0,1}. */
GSIM_API int gsim_get_probability(gsim_engine *e, const uint8_t *bits, const uint32_t *ids, size_t n,
                         double *out);

/* get_amplitude — simulator.hpp:370-384.  out = (re, im). */
GSIM_API int gsim_get_amplitude(gsim_engine *e, const uint8_t *bits, const uint32_t *ids, size_t n,
                       double *out);

/* set_wavefunction — simulator.hpp:440-454.  wf holds len complex values of
 * dtype GSIM_C128 (interleaved doubles) or GSIM_C64 (interleaved floats),
 * in host memory. */
GSIM_API int gsim_set_wavefunction(gsim_engine *e, const void *wf, int dtype, size_t len,
                          const uint32_t *ordering, size_t n);

/* collapse_wavefunction — simulator.hpp:456-485.  values[i] in {0,1}. */
GSIM_API int gsim_collapse_wavefunction(gsim_engine *e, const uint32_t *ids, size_t n,
                               const uint8_t *values, size_t nvalues);

/* cheat — simulator.hpp:529-532, split in three calls so that no Python list
 * of 2^N objects is built: the map (gsim_num_qubits + gsim_get_mapping) and a
 * copy of [offset, offset+count) of the state into host memory as dtype. */
GSIM_API int gsim_num_qubits(gsim_engine *e, uint32_t *out);
GSIM_API int gsim_get_mapping(gsim_engine *e, uint32_t *ids, uint32_t *positions, size_t cap);
GSIM_API int gsim_get_state(gsim_engine *e, void *host, int dtype, size_t offset, size_t count);

/* Zero-copy view of the flushed device state (no reference counterpart; the
 * reference returns a list copy, _cppsim.cpp:65).  Valid until the next call
 * that changes the qubit count. */
GSIM_API int gsim_state_device_ptr(gsim_engine *e, void **ptr, size_t *len, int *dtype);

/* Wait for all work queued on the engine's stream. */
GSIM_API int gsim_synchronize(gsim_engine *e);

/* Select the fusion planner (GSIM_FUSION_*).  kmax (0 = unchanged): for
 * GSIM_FUSION_REFERENCE the widest cluster of the greedy rule (1..7; the
 * reference's is 5); for GSIM_FUSION_STAGED values >= 6 set the tile width. */
GSIM_API int gsim_set_fusion(gsim_engine *e, int mode, uint32_t kmax);

/* The tcgen05 tensor-core kernel for fused complex64 gates of 4 to 7 targets
 * (3xTF32 split precision): mode 0 off (CUDA cores), 1 on (default) with the
 * norm of every amplitude group restored after a unitary gate (the tensor
 * cores' FP32 accumulation otherwise loses about 1e-8 x 2^(k+1) of the norm
 * per gate), 2 on without that restoration. */
GSIM_API int gsim_set_tensor_cores(gsim_engine *e, int mode);

/* The stage kernel of GSIM_FUSION_STAGED: mode 2 (default) packed pairs
 * for complex64 stages that have a tile bit none of their gates touches
 * (amplitude pairs along that bit on packed f32x2 arithmetic; other stages
 * and complex128 as mode 1), 1 register substages, 0 one shared-memory pass
 * per operation.  All modes give the same results up to FP rounding. */
GSIM_API int gsim_set_stage_kernel(gsim_engine *e, int mode);

/* How emulate_time_evolution evaluates exp(-i t H): mode 1 (default) exactly,
 * as the product of exp(-i t c_k P_k) over the terms, when they commute
 * pairwise and none acts on a control (the commuting case that ProjectQ's
 * setups/decompositions/time_evolution.py:28-52 decomposes), else as mode 0;
 * mode 0 always by the Taylor series of simulator.hpp:386-438 (the two agree to
 * the series' truncation, about 1e-12); mode 2 as mode 1, but non-commuting
 * terms by the Chebyshev expansion of exp(-i t H) (Bessel coefficients,
 * truncated at 1e-16): about |t| sum|c| + 40 applications of H where the
 * series takes about 16 |t| sum|c|. */
GSIM_API int gsim_set_time_evolution(gsim_engine *e, int mode);

/* How set_wavefunction moves a host state that is already in the engine's
 * precision: 1 (default) the SMs read it through the device view of
 * page-locked host memory (gsim_host_register / cudaMallocHost, 16-byte
 * aligned), falling back to the copy engine for pageable memory; 0 always one
 * cudaMemcpyAsync on the copy engine.  On GB300 the SM reads held 43 ms per
 * 8 GiB where the copy engine's first transfer after a long kernel sequence
 * took 0.4-0.8 s. */
GSIM_API int gsim_set_upload_mode(gsim_engine *e, int mode);

/* Preallocate device memory for nqubits qubits (avoids regrowth). */
GSIM_API int gsim_reserve(gsim_engine *e, uint32_t nqubits);

/* Counters since creation or the last reset:
 *  out[0] logical gates submitted, out[1] kernel launches for gates,
 *  out[2] algorithmic bytes moved by gate kernels (2 x touched amplitudes
 *  x bytes per amplitude), out[3] gate passes over the state, out[4] time
 *  evolutions applied as a product of term exponentials, out[5] time
 *  evolutions by the Taylor series, out[6] by the Chebyshev expansion. */
GSIM_API int gsim_get_counters(gsim_engine *e, uint64_t *out, size_t n);
GSIM_API int gsim_reset_counters(gsim_engine *e);

/* ---- Timing, device and host-memory helpers (no reference counterpart) ---- */

/* FP64 inner product <a|b> and max_i |a_i - b_i| of two engines' flushed
 * states (same device, same qubits and ordering; precisions may differ):
 * out[0] = Re, out[1] = Im, out[2] = max. */
GSIM_API int gsim_compare_states(gsim_engine *a, gsim_engine *b, double *out);

/* Make `device` current for the calling thread before gsim_create. */
GSIM_API int gsim_set_device(int device);

/* Record CUDA event `slot` (0..15) on the engine's stream; gsim_timer_elapsed
 * waits for event b and returns the milliseconds between events a and b. */
GSIM_API int gsim_timer_mark(gsim_engine *e, int slot);
GSIM_API int gsim_timer_elapsed(gsim_engine *e, int a, int b, float *ms);

/* Per-launch profile of gate kernels: when enabled, every gate-kernel launch
 * (and every step launch of a non-commuting time evolution) is bracketed by
 * CUDA events on the engine's stream.  fetch waits for the
 * stream and copies up to cap records. */
typedef struct gsim_launch_record {
  uint32_t kind;      /* 0 dense gate kernel (CUDA cores, k <= 5), 1 stage kernel,
                         2 wide gate kernel (k = 6, 7), 3 tensor-core gate kernel,
                         4 Taylor-series step and 5 Chebyshev step of
                         emulate_time_evolution (non-commuting terms) */
  uint32_t k;         /* matrix qubits (stage kernel: operations in the stage;
                         evolution steps: Pauli terms) */
  uint32_t nctrl;     /* control qubits */
  uint32_t nqubits;   /* state qubits */
  uint64_t targets;   /* bit mask of the matrix qubits' positions */
  uint64_t bytes;     /* algorithmic bytes: 2 x touched amplitudes x bytes/amplitude */
  uint32_t precision; /* GSIM_C128 or GSIM_C64 */
  uint32_t ngates;    /* logical gates applied by the launch */
  float ms;           /* device time of the launch */
  uint32_t aux;       /* stage kernel: register substages (0: one pass per operation),
                         | 1 << 16 for the packed-pair kernel */
} gsim_launch_record;
GSIM_API int gsim_profile_enable(gsim_engine *e, int on);
GSIM_API int gsim_profile_fetch(gsim_engine *e, gsim_launch_record *out, size_t cap, size_t *n);
GSIM_API int gsim_profile_clear(gsim_engine *e);

/* Page-lock (pin) a caller's host buffer so that set_wavefunction/get_state
 * copies run at full link speed; unregister before freeing it. */
GSIM_API int gsim_host_register(void *ptr, size_t bytes);
GSIM_API int gsim_host_unregister(void *ptr);

/* ---- Adjoint-method gradient (no reference counterpart) ---------------------
 * E(theta) = <psi|H|psi> with psi = U_nops ... U_1 |current state>, and
 * grad[j] = dE/dtheta_j, by one reverse sweep that un-applies the gates to
 * psi and to lam = H psi (kernels_adjoint.cu); the engine's state is left
 * unchanged.  Gate i acts on qubit target[i] with controls
 * ctrl_ids[ctrl_off[i] .. ctrl_off[i+1]); kind[i]: 0 fixed 2x2 matrix
 * mats[8i .. 8i+8) (row-major, interleaved re/im), 1 Rx, 2 Ry, 3 Rz, 4 Ph,
 * 5 R (ProjectQ's matrices) of angle theta[param[i]].  H: Pauli terms with
 * real coefficients (as gsim_get_expectation_value).  checkpoint_every > 0
 * stores psi every that many gates on the way forward and reloads it on the
 * way back (bounds the drift of un-applying gates in complex64). */
GSIM_API int gsim_adjoint_gradient(gsim_engine *e, size_t nops, const uint8_t *kind,
                                   const uint32_t *target, const uint32_t *ctrl_off,
                                   const uint32_t *ctrl_ids, const int32_t *param,
                                   const double *mats, const double *theta, size_t nparams,
                                   const uint32_t *term_offsets, const uint32_t *op_qubit,
                                   const uint8_t *op_pauli, const double *coeffs, size_t nterms,
                                   const uint32_t *ids, size_t nids, uint32_t checkpoint_every,
                                   double *energy, double *grad);

/* ---- Learned fusion planner (no reference counterpart) ----------------------
 * The cost model predicts log(milliseconds) of one kernel launch from 20
 * features of it; GSIM_FUSION_LEARNED sums the predictions over three
 * candidate plans of the queued gates (the greedy fixed-size clusters of
 * the reference's rule, clusters whose boundaries the model chooses, the
 * stage plan) and runs the cheapest.  It also chooses, for each
 * emulate_time_evolution of non-commuting terms, between the reference's
 * Taylor series and the Chebyshev expansion by the predicted step times
 * times the step counts (gsim_get_counters reports which ran).
 * gsim_launch_features: the features of n launch records (out: n x nfeat,
 * nfeat >= 20), the same function the planner applies to candidate launches;
 * needs no engine and no GPU.
 * gsim_set_cost_model: install trained weights (nfeatures = 20, `hidden`
 * units per layer, layout of gsim_mlp_get_params; params must hold all
 * H*F + H + H*H + H + H + 1 values, it is read without a length).
 * gsim_set_learned_regimes: allowed[n] != 0 lets learned plans run on
 * n-qubit states (n < count <= 65); elsewhere, and without a cost model, the
 * learned mode runs the greedy fixed-size fusion.
 * gsim_last_plan_choice: the plan the last learned flush ran
 * (GSIM_FUSION_REFERENCE greedy clusters, _STAGED, _LEARNED model clusters)
 * and, when pred_ms is not NULL, the three predicted times (greedy, stage,
 * model clusters) in milliseconds. */
GSIM_API int gsim_launch_features(const gsim_launch_record *recs, size_t n, float *out, size_t nfeat);
GSIM_API int gsim_set_cost_model(gsim_engine *e, int nfeatures, int hidden, const float *params);
GSIM_API int gsim_set_learned_regimes(gsim_engine *e, const uint8_t *allowed, size_t count);
GSIM_API int gsim_last_plan_choice(gsim_engine *e, int *mode, double *pred_ms);
/* The planner's own evaluation of the installed network (host FP32, the same
 * arithmetic as gsim_mlp_predict's kernel) on n feature rows of 20. */
GSIM_API int gsim_cost_model_predict(gsim_engine *e, const float *features, size_t n, float *out);

/* The cost model's network: F inputs -> H -> H -> 1 (ReLU), FP32, with
 * hand-written forward, backward and Adam kernels (mlp.cu).  Parameters are
 * one array: W1[H][F], b1[H], W2[H][H], b2[H], W3[H], b3. */
GSIM_API int gsim_mlp_create(int F, int H, uint32_t seed, void **out);
GSIM_API int gsim_mlp_destroy(void *mlp);
GSIM_API int gsim_mlp_num_params(void *mlp, size_t *out);
GSIM_API int gsim_mlp_get_params(void *mlp, float *out);
GSIM_API int gsim_mlp_set_params(void *mlp, const float *in);
GSIM_API int gsim_mlp_predict(void *mlp, const float *X, int B, float *out);
GSIM_API int gsim_mlp_gradient(void *mlp, const float *X, const float *y, int B, float *grad, double *loss);
GSIM_API int gsim_mlp_train(void *mlp, const float *X, const float *y, int B, int epochs, float lr,
                            double *loss);

/* ---- Allocation-free probability (no counterpart in the reference) ----------
 * Sum of |psi_i|^2 over the indices i with (i & mask) == value, for a state
 * vector the caller owns in device memory (2^nqubits amplitudes of
 * `precision`), written to the host double *out after waiting on `stream`
 * (a cudaStream_t; NULL = the legacy default stream).  For callers that
 * cannot allocate device memory at the point of the call — code whose device
 * memory belongs to another allocator (a framework's caching pool that must
 * see every allocation), or a thread that must not take the CUDA allocator's
 * locks while other work owns the device: it calls no cudaMalloc/cudaFree or
 * allocating library routine; its partial sums live in a fixed ~32 KB
 * __device__ array that every GPU loading the library keeps until exit.
 * Limit: the summed subspace (2^(nqubits - popcount(mask)) amplitudes) may
 * hold at most 2^32 amplitudes; larger requests fail with GSIM_ERR_LENGTH.
 * The first call on a device (and CUDA context) resolves the array's address
 * with cudaGetSymbolAddress; with lazy module loading that first call is
 * also when the runtime places the array, so "allocates nothing" holds from
 * the second call on (or from the first with CUDA_MODULE_LOADING=EAGER).
 * Make that first call before any stream capture.  The call is synchronous:
 * it waits for `stream` and returns the result on the host.  Calls that
 * overlap on the GPU share the array and race, so serialise them. */
GSIM_API int gsim_probability_noalloc(const void *d_state, int precision, uint32_t nqubits,
                                      uint64_t mask, uint64_t value, double *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GB300SIM_H_ */
