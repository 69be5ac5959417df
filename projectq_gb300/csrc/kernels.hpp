// Host-side declarations of the CUDA kernels' launchers.  Plain C++: the
// engine (engine.cu) plans the work, these functions enqueue it on a stream.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <vector>

#include "ops.hpp"

namespace gsim {

// prec: 0 = complex128 state, 1 = complex64 state.
cudaError_t launch_dense(int prec, void *psi, unsigned nq, const DenseOp &op, cudaStream_t s);
// Fused dense gates of 4 to 7 targets on a complex64 state with tcgen05
// tensor cores (3xTF32).  d_b: the real embedding of U split into TF32 hi and
// lo parts, laid out by tc_prepare_operand (tc_operand_floats(k) floats);
// *d_err is set when a wait inside the kernel times out.
size_t tc_operand_floats(int k);
// The gate with its targets sorted ascending (matrix permuted to match): the
// kernel loads and stores adjacent amplitude pairs when a target is bit 0.
DenseOp tc_sorted_targets(const DenseOp &op);
void tc_prepare_operand(const std::vector<cplx> &U, int k, float *out);
// renorm: when U is unitary, rescale each amplitude group's outputs to the
// group's input norm (undoes the tensor cores' downward accumulation bias).
cudaError_t launch_tc_gate(void *psi, unsigned nq, const DenseOp &op, const float *d_b, int *d_err, bool renorm,
                           cudaStream_t s);
// Gates of 5 to 7 targets on CUDA cores; d_matrix: the 2^k x 2^k matrix
// TRANSPOSED (column j contiguous: element [j][r] = U[r][j]) in the state's
// precision in device memory.
cudaError_t launch_wide(int prec, void *psi, unsigned nq, const DenseOp &op, const void *d_matrix,
                        cudaStream_t s);

// ---- stage kernel (many gates per pass through shared-memory tiles) -----
struct StagePlan;  // defined in stage.hpp
// d_ops: the plan's StageOpDev array, d_pool: its matrices in the state's
// precision, both already in device memory.
cudaError_t launch_stage(int prec, void *psi, unsigned nq, const StagePlan &plan, const void *d_ops,
                         const void *d_pool, cudaStream_t s);

// ---- reductions and state kernels (kernels_state.cu) ---------------------
// Sum over indices i with (i & mask) == val of |psi_i|^2 (FP64 accumulation).
// Writes the result to *d_out (device).  d_part: >= 4096 doubles of scratch.
cudaError_t launch_masked_norm(int prec, const void *psi, unsigned nq, uint64_t mask,
                               uint64_t val, double *d_part, double *d_out, cudaStream_t s);

// psi_i <- 0 where (i & mask) != val, psi_i <- psi_i / sqrt(*d_norm) otherwise.
cudaError_t launch_project_scale(int prec, void *psi, unsigned nq, uint64_t mask, uint64_t val,
                                 const double *d_norm, cudaStream_t s);

// d_flags[0] |= any |psi_i|^2 > tol with bit pos = 0; d_flags[1] likewise for bit = 1.
cudaError_t launch_classical_flags(int prec, const void *psi, unsigned nq, unsigned pos,
                                   double tol, int *d_flags, cudaStream_t s);
// d_first = min pair index p (bit pos removed) where either side exceeds tol.
cudaError_t launch_classical_first(int prec, const void *psi, unsigned nq, unsigned pos,
                                   double tol, unsigned long long *d_first, cudaStream_t s);

// dst <- src with bit `pos` removed, keeping the half where that bit == value.
cudaError_t launch_shrink(int prec, const void *src, void *dst, unsigned nq, unsigned pos,
                          int value, cudaStream_t s);

// Measurement sampling support (see measure.cu).
cudaError_t launch_block_norm_sums(int prec, const void *psi, uint64_t n, unsigned log_block,
                                   double *d_sums, cudaStream_t s);
cudaError_t launch_block_grid_sums(int prec, const void *psi, uint64_t n, unsigned log_block,
                                   const int16_t *d_cand, unsigned long long *d_units,
                                   uint8_t *d_flags, cudaStream_t s);

// Convert between storage precisions: dst_prec/src_prec 0 = c128, 1 = c64.
// SM-driven copy (16-byte aligned pointers and size), used to read page-locked
// host memory through its device view.
cudaError_t launch_pull(void *dst, const void *src, uint64_t bytes, cudaStream_t s);
cudaError_t launch_convert(int dst_prec, void *dst, int src_prec, const void *src, uint64_t n,
                           cudaStream_t s);

// Pauli strings.  For one group of terms that share the flip mask x:
// part[t * nblk + b] = per-block partial of Re<psi| P_t |psi> / coefficient.
struct PauliTermDev {
  uint64_t sign_mask;  // Y|Z positions: sign (-1)^popcount(i & sign_mask)
  int32_t phase;       // number of Y factors mod 4 (phase (-i)^phase)
  int32_t pad;
};
cudaError_t launch_pauli_expect(int prec, const void *psi, unsigned nq, uint64_t xmask,
                                const PauliTermDev *d_terms, int nterms, double *d_part,
                                int nblk, cudaStream_t s);
int pauli_expect_blocks(unsigned nq);
// Column sums: out[c] = sum_b part[c * nblk + b], fixed order.
cudaError_t launch_column_sums(const double *d_part, int nblk, int ncols, double *d_out,
                               cudaStream_t s);

// out_i = sum_t coeff_t (P_t in)_i for a list of terms (complex coefficients).
struct PauliApplyTermDev {
  uint64_t xmask;
  uint64_t sign_mask;
  double cre, cim;  // coefficient times (-i)^{#Y}
};
cudaError_t launch_pauli_apply(int prec, const void *in, void *out, unsigned nq,
                               const PauliApplyTermDev *d_terms, int nterms, cudaStream_t s);

// A term with a real coefficient r (a Hamiltonian's): r P with
// P = (-i)^ny X^x Z^sign_mask.  (-i)^ny only swaps and negates the real and
// imaginary parts, so the kernels spend 2 FP64 FMAs per term and amplitude.
struct PauliRealTermDev {
  uint64_t xmask;
  uint64_t sign_mask;
  double r;
  int32_t ny;
  int32_t pad;
};

// One Taylor order of emulate_time_evolution, all FP64 (complex128 vectors):
//   upd_j = coeff * sum_t c_t (P_t vec)_j ; vec_next_j = upd_j ;
//   where (j & ctrl) == ctrl: out_j += upd_j and part += |upd_j|^2.
cudaError_t launch_taylor_step(const double2 *vec, double2 *vec_next, double2 *out, unsigned nq,
                               const PauliRealTermDev *d_terms, int nterms, double coeff_re,
                               double coeff_im, uint64_t ctrl, double *d_part, double *d_norm,
                               cudaStream_t s);
// out_j *= corr where (j & ctrl) == ctrl; vec_j = out_j.
cudaError_t launch_phase_ctrl(double2 *out, double2 *vec, uint64_t n, uint64_t ctrl, double cre,
                              double cim, cudaStream_t s);

// One order of the Chebyshev expansion of exp(-i t H) (complex128 vectors):
//   w_j = scale * sum_t c_t (P_t cur)_j - prev_j   (no prev term if !has_prev),
//   prev_j <- w_j, and where (j & ctrl) == ctrl: out_j += a w_j.
cudaError_t launch_chebyshev_step(const double2 *cur, double2 *prev, double2 *out, unsigned nq,
                                  const PauliRealTermDev *d_terms, int nterms, double scale, bool has_prev,
                                  double a_re, double a_im, uint64_t ctrl, cudaStream_t s);
// out_j = a psi_j where (j & ctrl) == ctrl, psi_j elsewhere.
cudaError_t launch_scale_ctrl(const double2 *psi, double2 *out, uint64_t n, uint64_t ctrl, double a_re,
                              double a_im, cudaStream_t s);

// One Pauli exponential in place, on the amplitudes whose control bits are
// all set:  psi <- a psi + b P psi, with (P psi)_j = (-1)^{popcount(j & z)}
// psi_{j ^ x} (the term's own phase folded into b by the host).  For
// exp(-i theta c P') with P' = phase X^x Z^z: a = g cos(theta), b =
// -i g sin(theta) phase, g an optional global phase.  x and z must not meet
// ctrl.  One read and one write of every controlled amplitude.
struct PauliRotationDev {
  uint64_t xmask, zmask, ctrl;
  double are, aim, bre, bim;
  uint8_t pos[64];  // pivot (lowest bit of x, if any) and control positions, ascending
  int npos;
};
cudaError_t launch_pauli_rotation(int prec, void *psi, unsigned nq, const PauliRotationDev &r,
                                  cudaStream_t s);

// emulate_math: out_j = sum over sources s of in_s, gathered through an
// inverse table (CSR) over the packed register value, in the reference's
// accumulation order; uncontrolled indices are copied.
struct MathRegsDev {
  uint8_t pos[64];  // bit positions of the packed register value, LSB first
  int width;        // total number of register bits W
  uint64_t ctrl;    // control mask
};
cudaError_t launch_math_gather(int prec, const void *in, void *out, unsigned nq,
                               const MathRegsDev &regs, const uint64_t *d_inv_off,
                               const uint32_t *d_inv_src, cudaStream_t s);
// Bijective case: out[deposit(j, table[x])] = in[j] + 0.0 (a scatter).
cudaError_t launch_math_scatter(int prec, const void *in, void *out, unsigned nq,
                                const MathRegsDev &regs, const uint32_t *d_table,
                                cudaStream_t s);

// <a|b> and max_i |a_i - b_i| of two state vectors (FP64): d_out[0] = Re,
// d_out[1] = Im, d_out[2] = max.  d_part: >= 4096 doubles.
cudaError_t launch_compare(int prec_a, const void *a, int prec_b, const void *b, uint64_t n,
                           double *d_part, double *d_out, cudaStream_t s);

// Adjoint gradient: one reverse-sweep step over (psi, lam) for a 1-target gate
// u (2x2 row-major, FP64) with controls; gen selects the generator whose
// Im<lam|Pi_c G|psi> is reduced into column `col` of d_part (-1: none;
// 0 X, 1 Y, 2 Z, 3 identity, 4 |1><1|).
struct AdjointGate {
  cplx u[4];
  unsigned target = 0;
  uint64_t ctrl_mask = 0;
  int gen = -1;
};
int adjoint_blocks(unsigned nq);
cudaError_t launch_adjoint_step(int prec, void *psi, void *lam, unsigned nq, const AdjointGate &g,
                                int col, double *d_part, int nblk, cudaStream_t s);

}  // namespace gsim
