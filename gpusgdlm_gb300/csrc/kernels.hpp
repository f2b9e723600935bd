// Launch wrappers for the SGDLM device kernels.  Every wrapper enqueues work on
// the given stream and returns without synchronising; all device buffers are
// owned by the engine (engine.cpp).
//
// Device layouts (R column-major, as handed over by the reference's Rcpp layer,
// rSGDLM/src/SGDLM/RcppWrapper.cpp):
//   m_t   : P x m         (series j at j*P)
//   C_t   : P x P x m     (series j at j*P*P, column-major within)
//   n_t,s_t,beta : m
//   delta : P x P x m
//   p     : m (unsigned)
//   sp    : P x m (unsigned; < m*m marks a Gamma position row + m*col)
// Draw buffers are series-major (GB300 layout, coalesced over draws):
//   lambda: m x n         (series j, draw i at j*n + i)
//   theta : m x n x P     (series j, draw i, coefficient k at (j*n + i)*P + k)
//   y     : n x m         (draw i, series j at i*m + j) == reference (m, nsim)
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace sgdlm {

// Per-draw status bits written by the sampler and LU kernels.
enum : int {
  DRAW_FLAG_GAMMA_CAP = 1,      // gamma sampler hit its attempt cap
  DRAW_FLAG_PIVOT = 2,          // no-pivot LU multiplier above threshold -> pivoted redo
  DRAW_FLAG_SINGULAR = 4,       // zero / non-finite pivot: weight 0, forecast NaN
  DRAW_FLAG_REDONE = 8,         // draw was refactored by the pivoting fallback
  DRAW_FLAG_FULL_PIVOT = 16,    // ... over the full matrix (its sparse levels failed)
};

// Philox key and epoch of one sampling call.  When dev_epoch is set (fused,
// graph-replayable step) the epoch is *dev_epoch + epoch, read on the device.
struct RngKey {
  uint32_t k0, k1, epoch;
  const uint32_t *dev_epoch;
};

// Advances the device-side epoch counter by `delta` (fused step).
void launch_advance_epoch(cudaStream_t s, uint32_t *dev_epoch, uint32_t delta);

// (a1) conjugate update, warp per series.  rSGDLM/src/SGDLM/SGDLM.cu:10-113
void launch_posterior(cudaStream_t s, int m, int P, const unsigned *p, double *m_t,
                      double *C_t, double *n_t, double *s_t, const double *y,
                      const double *F);

// (a2) discount step.  rSGDLM/src/SGDLM/SGDLM.cu:115-149
void launch_prior(cudaStream_t s, int m, int P, const unsigned *p, double *C_t,
                  double *n_t, double *W_t, const double *beta, const double *delta);

// Upper Cholesky factor U (U'U = C) of the leading p x p block, zero elsewhere,
// in double and in the sampling precision.  rSGDLM/src/kernel_functions.cuh:845-902
// Evolution-matrix step of the prior: a = G m, R = G R G' with the reference's
// cut-offs (rSGDLM/src/SGDLM/SGDLM.cu:151-178).
void launch_evo_prior(cudaStream_t s, int m, int P, const unsigned *p, double *m_t,
                      double *C_t, const double *G);
void launch_to_float(cudaStream_t s, size_t n, const double *src, float *dst);
void launch_cholesky(cudaStream_t s, int m, int P, const unsigned *p, const double *C,
                     double *U64, float *U32);

// The draws' Gamma entries (the simultaneous-parent coefficients), draw-major in
// the CSR order of the rows of Gamma: row j holds series j's coefficients at the
// positions sp[j*P + k] < m*m, in increasing k, from rowptr[j] on (GammaRows).
// Draw i's entry q is v[i*nnz + q].  That order is also the order of increasing
// theta index j*P + k, i.e. the elimination plan's level-0 order.  The sampler
// writes this copy beside the series-major theta; the LU and iterative-solve
// kernels read a draw's nnz values as one run.
template <typename T> struct GammaDraws {
  T *v;                 // nsim * nnz, or nullptr: not written
  const int *rowptr;    // m + 1
  const unsigned *sp;   // P x m
  int nnz;
};

// (a3) lambda_ij ~ Gamma(n_j/2, rate n_j s_j/2); theta_ij = m_j + U_j' z/sqrt(s_j lambda_ij).
// rSGDLM/src/SGDLM/SGDLM.cu:623-677
template <typename T>
void launch_sample(cudaStream_t s, int m, int P, long n, const double *m_t,
                   const double *n_t, const double *s_t, const T *U, RngKey key,
                   T *lambda, T *theta, GammaDraws<T> gd, int *draw_flags,
                   // p_j (the Cholesky factors' cut), or nullptr: all P coefficients
                   const unsigned *p = nullptr);

// (a9) multi-step evolution of forecast draws.  rSGDLM/src/SGDLM/SGDLM.cu:679-762
template <typename T>
void launch_evolve(cudaStream_t s, int m, int P, long n, const unsigned *p,
                   const double *r_t, const double *c_t, const double *beta,
                   const T *UW, RngKey key, bool compat_unscaled_omega,
                   bool compat_beta_no_boost, T *lambda, T *theta, GammaDraws<T> gd,
                   int *draw_flags, const T *G = nullptr);

// (a4)/(a8) batched LU of (I - Gamma_i): log|det| per draw, and optionally the
// forecast solve y_i = (I - Gamma_i)^-1 nu_i with one refinement step.
struct LuPlan {
  int m, P;
  int mp;              // m rounded up to the 32-wide block size (pivoting redo)
  int dp;              // dense core rounded up to 32 (fast pass)
  int grid, block;     // persistent grid of the fast pass
  int fb_grid;         // grid of the pivoting redo
  size_t smem, smem_fallback;
  int vals_smem;       // the sparse levels' value slots live in shared memory
  int prog_smem;       // the solve phase stages the level programs in shared memory
  int tc;              // trailing updates on the tensor cores (tcgen05)
  size_t scratch_elems_per_cta;  // dense core + per-draw values of the sparse levels
  size_t fb_elems_per_cta;       // the redo's: the above, or a full m_p x m_p slab
  int fb_core_smem;              // the redo factors the dense core in shared memory
  size_t scratch_elems_total;    // covers both passes
};
// Tuning knobs of the fast pass: allow_tc = 0 keeps the FFMA instantiation where
// the tensor-core one would apply; max_grid > 0 caps the persistent grid (fewer
// CTAs, more draws each: room for other work on the GPU at the same time).
struct LuOptions {
  int allow_tc = 1;
  int max_grid = 0;
  int allow_warp = 1;  // m <= kWarpLuMaxM: one warp per draw (launch_lu_warp)
};
constexpr int kWarpLuMaxM = 32;
// Warp-per-draw LU with partial pivoting for m <= kWarpLuMaxM: log|det| of every
// draw and, when y != nullptr, the forecast solve y_i = (I - Gamma_i)^-1 nu_i
// (nu series-major, nu[r*n + i]; y draw-major, y[i*m + r]).
template <typename T>
void launch_lu_warp(cudaStream_t s, int m, int P, long n, int num_sms, const unsigned *sp,
                    const T *theta, double *logdet, int *draw_flags,
                    const double *nu, double *y);
// core_n / nv / n_solve / prog_len come from the elimination plan (core_n = m and
// the others 0 without one).
template <typename T>
LuPlan plan_lu(int m, int P, long n, int num_sms, int core_n, int nv, int n_solve = 0,
               int prog_len = 0, LuOptions opt = LuOptions{});
// Row-wise list of the Gamma entries of (I - Gamma): for row r, entries
// rowptr[r] .. rowptr[r+1]-1 are (e = j*P + k, column).  Built on the host from
// the parental sets; gives the forecast residual a fixed summation order.
struct GammaRows {
  const int *rowptr;   // m + 1
  const int2 *ent;     // nnz
  // external predictors: for series j, the k with sp[j*P + k] >= m*m are
  // ext_k[ext_ptr[j] .. ext_ptr[j+1]-1] (the terms of nu's mean)
  const int *ext_ptr;  // m + 1
  const int *ext_k;
};
struct EliminationPlan;
template <typename T>
// theta: the draws series-major; theta_g: their Gamma entries (GammaDraws layout,
// ep.nnz0 per draw), or nullptr (then gathered from theta).
void launch_lu(cudaStream_t s, const LuPlan &plan, long n, const EliminationPlan &ep,
               const unsigned *sp, const T *theta, const T *theta_g, T *scratch,
               double *logdet, int *draw_flags,
               // forecast solve (x == nullptr: log|det| only)
               const double *x, const T *lambda, RngKey key, bool refine, double *y,
               GammaRows rows,
               // the forecast right-hand sides of all draws (launch_forecast_nu), or
               // nullptr: the LU kernel generates them itself
               const double *nu_in = nullptr,
               // n + 1 ints, [0] zero on entry: the draws flagged for the pivoted redo
               // are appended ([0] their count, [1..] their indices), or nullptr
               int *pivot_list = nullptr,
               // the same form: only the listed draws are factored, or nullptr: all
               const int *draw_list = nullptr);
// Forecast solves of FP32 draws by fixed-point iteration on the sparse Gamma_i
// (forecast_kernels.cu).  ok = 0: the shared-memory working set of a draw does
// not fit, every draw keeps the factorising path.
struct JacobiPlan {
  int ok, grid, threads, nnz;  // threads: m rounded up to 32; nnz: ELL slots per row (8..32)
  size_t smem;
  // thread t takes row order[t] (the rows by decreasing length, so that a warp's
  // rows are of similar length and its sweeps stop at its own longest row), or
  // nullptr: thread t takes row t
  const int *order;
};
// m <= 1024 and at most 32 simultaneous parents per series, else ok = 0.
JacobiPlan plan_jacobi(int m, int max_row, int num_sms);
// y (draw-major) of every draw whose iteration converges (logdet[i] set to NaN:
// not factored); the others are appended to list (n + 1 ints, [0] zero on entry).
// theta_g: the draws' Gamma entries (GammaDraws layout, nnz per draw); nu:
// series-major right-hand sides.
void launch_forecast_jacobi(cudaStream_t s, const JacobiPlan &jp, int m, int P, long n,
                            GammaRows rows, const float *theta_g, int nnz, const double *nu,
                            double *y,
                            double *logdet, int *list);
// The forecast right-hand sides nu_ij = z_ij / sqrt(lambda_ij) + x_j' phi_ij of all
// draws (series-major, nu[j*n + i]); theta series-major; x32: an FP32 copy of x
// (used for FP32 draws).  SGDLM.cu:574-590 (batchedComputeNuPlusMu,
// kernel_functions.cuh:1156-1178).
template <typename T>
void launch_forecast_nu(cudaStream_t s, int m, int P, long n, GammaRows rows, const T *theta,
                        const double *x, const float *x32, const T *lambda, RngKey key,
                        double *nu);
template <typename T>
void launch_lu_fallback(cudaStream_t s, const LuPlan &plan, long n, const EliminationPlan &ep,
                        const unsigned *sp, const T *theta, const T *theta_g, T *scratch,
                        double *logdet, int *draw_flags, const double *x,
                        const T *lambda, RngKey key, double *y, GammaRows rows,
                        // the list launch_lu appended to (only those draws are
                        // visited), or nullptr: every draw's flag is read
                        const int *pivot_list = nullptr);

// (a5) importance weights from log|det| by FP64 log-sum-exp (three launches).
// out6 = {sum_det, ess, max_logdet, n_finite, sum_w2, 0}; part: scratch of
// 4 * kWeightBlocks doubles.  rSGDLM/src/SGDLM/SGDLM.cu:325-335
constexpr int kWeightBlocks = 1024;
void launch_weights(cudaStream_t s, long n, const double *logdet, double *w,
                    double *out6, double *part);

// (a6)/(a7) VB moments and refit.  rSGDLM/src/SGDLM/SGDLM.cu:341-500
struct VbScratch {
  double *part_a;   // chunks x m x (P + 2)
  double *part_b;   // chunks x m x P*P
  int chunks;
  long chunk_draws;  // draws per chunk (a multiple of the passes' 128-draw sub-chunk)
};
// The VB passes run one block per (chunk of draws, series); the chunks are sized
// for the SM count (about two full waves of blocks).
void vb_chunking(long n, int m, int num_sms, int *chunks, long *chunk_draws);
template <typename T>
void launch_vb(cudaStream_t s, int m, int P, long n, const unsigned *p,
               const double *n_t, const double *s_t, const double *w, const T *lambda,
               const T *theta, VbScratch scr, double *mean_m, double *mean_C,
               double *mean_n, double *mean_s, double *mean_lambda,
               double *mean_log_lambda, double *mean_Q, int *series_flags);

// Device-side ESS gate of the fused filter step: copy (mean_m, mean_C, mean_n,
// mean_s) into the state when stats[1] (ESS) > threshold.
void launch_gate(cudaStream_t s, int m, int P, const double *stats, double threshold,
                 const double *mean_m, const double *mean_C, const double *mean_n,
                 const double *mean_s, double *m_t, double *C_t, double *n_t,
                 double *s_t, double *accepted);

}  // namespace sgdlm
