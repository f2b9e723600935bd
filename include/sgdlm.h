/*
 * sgdlm.h - C ABI of the GB300 SGDLM filtering engine.
 *
 * One handle = one engine on one GPU with one CUDA stream, like one
 * SGDLM::HostWrapper<double> of the reference (rSGDLM/src/SGDLM/HostWrapper.hpp:13-99)
 * constructed by HostWrapperFactory<double>::create (HostWrapperFactory.cu:5-35).
 * Every entry point mirrors one method of that interface: same arguments, same
 * meaning, same column-major host layouts, same state-order rules.  Where the
 * reference logs an error and returns silently (rSGDLM/src/logger.hpp:160-165,
 * HostWrapperImpl.cu:1239-1286) these functions log the same condition and return
 * a non-zero sgdlm_status instead; the state is left unchanged.
 *
 * Host arrays are caller-owned, double precision, R column-major:
 *   m_t P x m, C_t P x P x m, n_t/s_t/beta m, delta P x P x m, p m (unsigned),
 *   sp P x m (unsigned; values < m*m address (I - Gamma) at row + m*col, any value
 *   >= m*m - e.g. R's NA_integer_ - marks an external predictor),
 *   y_t m, F_t P x m, forecast output m x nsim.
 * Calls are synchronous (like the reference) unless named *_device.
 */
#ifndef SGDLM_GB300_H_
#define SGDLM_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgdlm_engine *sgdlm_handle;

typedef enum {
  SGDLM_OK = 0,
  SGDLM_ERR_BAD_DIM = 1,        /* dimension mismatch (RcppWrapper.cpp:80-92, 170-174, 264-271) */
  SGDLM_ERR_NOT_INIT = 2,       /* device memory not initialised (HostWrapperImpl.cu:1240-1246) */
  SGDLM_ERR_WRONG_STATE = 3,    /* prior/posterior order (HostWrapperImpl.cu:1268-1286) */
  SGDLM_ERR_SIM_NOT_INIT = 4,   /* simulation memory not initialised (HostWrapperImpl.cu:1249-1255) */
  SGDLM_ERR_DEVICE = 5,         /* CUDA error (the reference only logs these, loggerGPU.cuh:26-60) */
  SGDLM_ERR_BAD_ARG = 6,        /* null pointer, nsim = 0, invalid parental set */
  SGDLM_ERR_NO_DEVICE = 7,      /* no CUDA device (HostWrapperImpl.cu:22-25) */
  SGDLM_ERR_OUT_OF_MEMORY = 8,
  SGDLM_ERR_UNSUPPORTED = 9,    /* size beyond this build's limits (max_p > 64, m > 800) */
  SGDLM_ERR_EVO_DISABLED = 10   /* evolution matrices not enabled (HostWrapperImpl.cu:1258-1265) */
} sgdlm_status;

typedef enum {
  SGDLM_PRECISION_FP64 = 0,  /* every kernel in FP64 (the reference's DOUBLETYPE=double) */
  SGDLM_PRECISION_MIXED = 1  /* draws, LU and solves in FP32 (+FP64 refinement);
                                posterior/prior, log-sum-exp, moments' sums, Newton in FP64 */
} sgdlm_precision;

/* Reference-behaviour switches (on by default: the drop-in reproduces the
 * reference's sampling distributions, including these two defects). */
enum {
  /* scale_omegas (kernel_functions.cuh:986-1001) is launched with its z index
   * fixed at 0 (SGDLM.cu:718-722), so only draw 0 of series 0 gets the
   * 1/sqrt(c lambda) scale; every other evolution innovation stays N(0, W). */
  SGDLM_COMPAT_UNSCALED_EVOLUTION = 1u,
  /* make_gamma_1/make_beta (kernel_functions.cuh:644-798) apply Marsaglia-Tsang
   * to shapes below one without the U^(1/a) boost. */
  SGDLM_COMPAT_BETA_NO_BOOST = 2u,
  SGDLM_COMPAT_REFERENCE = 3u,
  SGDLM_COMPAT_NONE = 0u
};

typedef struct {
  /* last computeVBPosterior / computeForecast */
  double ess;                /* (sum w)^2 / sum w^2 of the normalised IS weights */
  double sum_det_weights;    /* sum_i |det(I - Gamma_i)| (reference output) */
  double max_log_det;
  uint64_t draws_pivoted;    /* draws redone with partial pivoting */
  uint64_t draws_singular;   /* draws with a singular (I - Gamma): weight 0 / NaN forecast */
  uint64_t gamma_cap_hits;   /* gamma draws that hit the sampler's attempt cap */
  uint64_t newton_fallbacks; /* series whose VB Newton solve did not converge */
  /* CUDA-event timings of the last call's phases, milliseconds */
  double ms_sample, ms_lu, ms_weights, ms_vb, ms_total;
  double ms_lu_forecast;
  /* last computeForecast: draws whose solve needed the LU factorisation (the rest
   * converged in the iterative solve of FP32 draws; all draws in FP64) */
  uint64_t forecast_draws_factored;
  /* of draws_pivoted: draws whose sparse levels failed too (a zero, non-finite or
   * huge level pivot multiplier), pivoted over the full matrix; the others were
   * pivoted in the dense core only */
  uint64_t draws_pivoted_full;
} sgdlm_stats;

/* ---- lifetime (HostWrapperFactory.cu:5-35, HostWrapperImpl.cu:12-105) ---- */
int sgdlm_create(size_t no_gpus, sgdlm_handle *out);
int sgdlm_destroy(sgdlm_handle h);
int sgdlm_init_memory(sgdlm_handle h, size_t m, size_t max_p);       /* initMemory :130 */
int sgdlm_clear_memory(sgdlm_handle h);                               /* clearMemory :281 */
int sgdlm_get_no_series(sgdlm_handle h, size_t *m);                   /* getNoSeries :108 */
int sgdlm_get_max_p(sgdlm_handle h, size_t *max_p);                   /* getMaxP :115 */
int sgdlm_get_no_gpus(sgdlm_handle h, size_t *no_gpus);
int sgdlm_init_sim_memory(sgdlm_handle h, size_t nsim, size_t nsim_batch); /* initSimMemory :321 */
int sgdlm_clear_sim_memory(sgdlm_handle h);                           /* clearSimMemory :514 */
int sgdlm_get_nsim(sgdlm_handle h, size_t *nsim);                     /* getNSim :307 */
int sgdlm_get_nsim_batch(sgdlm_handle h, size_t *nsim_batch);         /* getNSimBatch :314 */
int sgdlm_is_prior(sgdlm_handle h, int *is_prior);                    /* isPrior :590 */
int sgdlm_set_is_prior(sgdlm_handle h, int is_prior);                 /* isPrior(bool) :597 */

/* ---- parameters (HostWrapperImpl.cu:604-797); a NULL pointer skips that array ---- */
int sgdlm_get_parameters(sgdlm_handle h, double *m_t, double *C_t, double *n_t, double *s_t);
int sgdlm_set_parameters(sgdlm_handle h, const double *m_t, const double *C_t,
                         const double *n_t, const double *s_t);
int sgdlm_get_discount_factors(sgdlm_handle h, double *beta, double *delta);
int sgdlm_set_discount_factors(sgdlm_handle h, const double *beta, const double *delta);
int sgdlm_get_parental_sets(sgdlm_handle h, unsigned *p, unsigned *sp);
int sgdlm_set_parental_sets(sgdlm_handle h, const unsigned *p, const unsigned *sp);

/* ---- filtering (HostWrapperImpl.cu:799-1228) ---- */
int sgdlm_compute_posterior(sgdlm_handle h, const double *y_t, const double *F_t); /* :1024 */
int sgdlm_compute_vb_posterior(sgdlm_handle h, double *mean_m_t, double *mean_C_t,
                               double *mean_n_t, double *mean_s_t, double *is_weights,
                               double *sum_det_weights);                           /* :1060 */
int sgdlm_compute_prior(sgdlm_handle h, int evolve_forecast_variables);            /* :800 */
int sgdlm_init_forecast_priors(sgdlm_handle h);                                    /* :540 */
int sgdlm_evolve_forecast_samples(sgdlm_handle h);                                 /* :880 */
/* Evolution-matrix variants (state evolution theta_t = G_t theta_{t-1} + omega_t):
 * computePrior(const DOUBLE *G, bool) (HostWrapperImpl.cu:837-877) -- the prior
 * step, then a = G m and R = G R G' with the reference's cut-offs; G_tp1 is
 * max_p x max_p x m, column-major per series (R's array(…, c(max_p, max_p, m))).
 * evolveForecastSamples(const DOUBLE *G) (HostWrapperImpl.cu:904-946) -- the
 * evolution of forecast draws with theta = G theta before adding chol(W)' omega. */
/* getEvolutionMatrixConfiguration (HostWrapper.hpp:19, HostWrapperImpl.cu:122-127):
 * whether evolution matrices are enabled. */
int sgdlm_get_evolution_matrix_configuration(sgdlm_handle h, int *use);
/* manageEvoMemory (HostWrapper.hpp:31, HostWrapperImpl.cu:231-279): enable (device
 * memory for G, zeroed) or disable (memory released) the evolution matrices; the
 * setting survives sgdlm_init_memory.  The four G functions below return
 * SGDLM_ERR_EVO_DISABLED unless enabled, as the reference logs and returns. */
int sgdlm_manage_evo_memory(sgdlm_handle h, int use);
/* getEvolutionMatrix / setEvolutionMatrix (HostWrapper.hpp:57-59,
 * HostWrapperImpl.cu:717-755): G_t is max_p x max_p x m; NULL copies nothing. */
int sgdlm_get_evolution_matrix(sgdlm_handle h, double *G_t);
int sgdlm_set_evolution_matrix(sgdlm_handle h, const double *G_t);
int sgdlm_compute_evo_prior(sgdlm_handle h, const double *G_tp1, int evolve_forecast_variables);
int sgdlm_evolve_forecast_samples_evo(sgdlm_handle h, const double *G_tp1);
/* y_tp1 (m x nsim, draw-major) in page-locked, device-mapped host memory (e.g.
 * cudaHostAlloc) is written by the LU kernels directly over the host link; any
 * other destination receives a copy after them.  The values are the same. */
int sgdlm_compute_forecast(sgdlm_handle h, double *y_tp1, const double *x_tp1,
                           double *lambdas, double *thetas,
                           int use_existing_lambdas_and_thetas);                   /* :949 */

/* Copies the current draw buffers to host in the reference's draw-major layouts,
 * lambdas (m x nsim) and thetas (max_p x m x nsim) as in computeForecastDebug
 * (RcppWrapper.cpp:557-569), and the last per-draw log|det(I - Gamma)| (nsim).
 * Any pointer may be NULL. */
int sgdlm_get_draws(sgdlm_handle h, double *lambdas, double *thetas, double *log_dets);

/* ---- engine options (no counterpart in the reference's interface) ---- */
int sgdlm_set_precision(sgdlm_handle h, int precision);
int sgdlm_get_precision(sgdlm_handle h, int *precision);
int sgdlm_set_compat(sgdlm_handle h, unsigned flags);
/* Levels of sparse pre-elimination of (I - Gamma) before the dense LU (default 4;
 * 0 = dense LU of the whole matrix).  Each level eliminates a greedy independent
 * set of the parent graph; results are equal up to rounding. */
int sgdlm_set_elimination_levels(sgdlm_handle h, int levels);
/* Levels actually planned and the size of the remaining dense core. */
int sgdlm_get_elimination_info(sgdlm_handle h, int *levels, int *core_n);
int sgdlm_get_compat(sgdlm_handle h, unsigned *flags);
/* Random stream: Philox4x32-10 keyed by seed; epoch counts sampling calls.  The
 * reference seeds cuRAND with 1234 + 100*gpu (HostWrapperImpl.cu:63-64) and
 * never exposes the state; (seed, epoch) here is a complete checkpoint. */
int sgdlm_set_rng_state(sgdlm_handle h, uint64_t seed, uint64_t epoch);
int sgdlm_get_rng_state(sgdlm_handle h, uint64_t *seed, uint64_t *epoch);
int sgdlm_get_stats(sgdlm_handle h, sgdlm_stats *out);
int sgdlm_set_log_level(sgdlm_handle h, int level);   /* RcppWrapper.cpp:834-839 */
int sgdlm_get_log_level(sgdlm_handle h, int *level);  /* RcppWrapper.cpp:827-832 */
/* Last error message of this handle (empty string if none). */
const char *sgdlm_last_error(sgdlm_handle h);

/* ---- learned importance proposal (no counterpart in the reference) ----
 * The reference samples the VB importance draws from the decoupled naive
 * posterior (SGDLM.cu:623-677).  With SGDLM_PROPOSAL_LEARNED a per-series network
 * (features of the naive posterior and of the series' simultaneous parents ->
 * 128 -> GELU -> 128 -> GELU -> location shift and log-scales of theta_j and
 * log-corrections of (n_j, s_j); BF16 weights, FP32 accumulation) is trained
 * online by Adam on (naive posterior -> VB-refitted posterior) pairs of the
 * first train_steps computeVBPosterior calls whose ESS exceeds nsim/2, then
 * deployed: later calls draw from the corrected normal-gamma proposal, with
 * importance weights that stay exact density ratios
 * (log w = log|det(I - Gamma)| + sum_j [log p_j - log q_j]), and fall back to the
 * plain proposal when the learned weights' ESS is below ess_fraction * nsim.
 * computeVBPosterior only (the fused device step keeps the plain proposal);
 * max_p <= 24. */
enum { SGDLM_PROPOSAL_PLAIN = 0, SGDLM_PROPOSAL_LEARNED = 1 };
typedef struct {
  int mode;             /* SGDLM_PROPOSAL_PLAIN or SGDLM_PROPOSAL_LEARNED */
  int train_steps;      /* training calls before deployment (500) */
  int iters_per_step;   /* Adam iterations after each training call (4) */
  int batch;            /* samples per Adam iteration (4096) */
  double lr;            /* Adam step size (1e-3) */
  double ess_fraction;  /* fall back to the plain proposal below this ESS / nsim (0.5) */
  uint64_t seed;        /* initial weights and training batches */
} sgdlm_proposal_config;
typedef struct {
  uint64_t training_calls;  /* calls whose pairs trained the network */
  uint64_t samples;         /* (series, call) pairs in the replay buffer */
  uint64_t adam_steps;
  uint64_t learned_calls;   /* calls that drew from the learned proposal */
  uint64_t fallbacks;       /* of those, calls redone with the plain proposal */
  double last_loss;         /* masked MSE of the last Adam iteration */
  double ess_learned;       /* last call: ESS of the learned proposal's weights (0: not run) */
  double ess_plain;         /* last call: ESS of the plain proposal's weights (0: not run) */
  int deployed;             /* training finished, the learned proposal is in use */
  int used_learned;         /* the last call's moments came from the learned proposal */
} sgdlm_proposal_info;
/* Configures the proposal (a NULL cfg restores the plain defaults); a new
 * configuration restarts training from freshly initialised weights. */
int sgdlm_set_proposal(sgdlm_handle h, const sgdlm_proposal_config *cfg);
int sgdlm_get_proposal(sgdlm_handle h, sgdlm_proposal_config *cfg);
int sgdlm_get_proposal_info(sgdlm_handle h, sgdlm_proposal_info *info);
/* The network's sizes: parameters (flat FP32 layout W1 (128 x F), b1, W2 (128 x
 * 128), b2, W3 (O x 128), b3), features F = 2 max_p + 5, outputs O = 2 max_p + 2. */
int sgdlm_proposal_sizes(sgdlm_handle h, size_t *n_params, int *n_features, int *n_outputs);
int sgdlm_proposal_get_params(sgdlm_handle h, float *params);
int sgdlm_proposal_set_params(sgdlm_handle h, const float *params);
/* One forward and backward pass on host data (batch rows of normalised features
 * X (F), targets Y (O) and mask (O)): the masked MSE and the gradient of every
 * parameter (flat layout); the parameters are left unchanged. */
int sgdlm_proposal_loss_and_gradient(sgdlm_handle h, size_t batch, const float *X, const float *Y,
                                     const float *mask, double *loss, float *grad);
/* The last learned call's proposal q (m_q P x m, C_q P x P x m, n_q, s_q m) and
 * the draws' log weights (nsim); any pointer may be NULL. */
int sgdlm_get_proposal_state(sgdlm_handle h, double *m_q, double *C_q, double *n_q, double *s_q,
                             double *log_weights);

/* ---- fused device-resident filter step (GB300 path; asynchronous) ----
 * One README time step (README.md:103-154) on the handle's stream with no host
 * synchronisation: computePosterior(y, F) -> computeVBPosterior(nsim) ->
 * setPosteriorParameters(VB) if ESS > ess_threshold -> computePrior() ->
 * computeForecast(nsim, x_tp1).  All pointers are device pointers:
 *   d_y (m), d_F (P x m), d_x (P x m, may be NULL: no forecast),
 *   d_forecast (m x nsim, may be NULL), d_is_weights (nsim, may be NULL),
 *   d_step_stats (8 doubles: ESS, sum_det, accepted, max_log_det, ...; may be NULL).
 * Requires the prior state and initialised simulation memory.  The host-side
 * prior/posterior flag ends in the prior state, as after the reference's step. */
int sgdlm_filter_step_device(sgdlm_handle h, const double *d_y, const double *d_F,
                             const double *d_x, double ess_threshold, double *d_forecast,
                             double *d_is_weights, double *d_step_stats);
/* log|det(I - Gamma_i)| of n draws for callers that cannot allocate device
 * memory (no counterpart in the reference).  Inputs and outputs are the
 * caller's device buffers: d_theta FP32 draws, series-major (m, n, max_p) as the
 * engine stores them; d_sp the parental sets (max_p x m, as in
 * sgdlm_set_parental_sets); d_log_det (n doubles) and d_flags (n ints, per-draw
 * status bits) receive the results.  The LU working matrices live in a 16 MiB
 * static device array instead of allocated scratch.  m is at most 736 (the LU
 * block's shared memory; larger m returns SGDLM_ERR_UNSUPPORTED) and max_p at
 * most 64.  The first call in each CUDA context looks that array up (make it
 * outside stream capture); calls that overlap on the GPU share the array and
 * race.  Runs on `stream` (a cudaStream_t) and returns without synchronising. */
int sgdlm_log_det_noalloc(size_t m, size_t max_p, size_t n, const float *d_theta,
                          const unsigned *d_sp, double *d_log_det, int *d_flags, void *stream);
/* ---- LU tuning and the batched multi-instance step (no counterpart in the
 * reference, which runs one engine per handle and per stream,
 * HostWrapperImpl.cu:47-61) ---- */
/* Fast-pass options of the batched LU: allow_tensor_cores = 0 keeps the FFMA
 * path where the tensor-core one applies (d_p <= 224, mixed precision);
 * max_ctas > 0 caps its persistent grid (more draws per CTA, fewer CTAs: room
 * for other instances on the GPU).  Results equal up to rounding. */
int sgdlm_set_lu_options(sgdlm_handle h, int allow_tensor_cores, int max_ctas);
/* Forecast solves of FP32 draws: 1 (default) the fixed-point iteration on the
 * sparse Gamma_i first (draws that do not converge are factored), 0 every draw
 * factored.  Results equal to the refinement tolerance. */
int sgdlm_set_forecast_solver(sgdlm_handle h, int iterative);
int sgdlm_get_lu_options(sgdlm_handle h, int *allow_tensor_cores, int *max_ctas);
/* Small systems (m <= 32): 1 (default) one warp per draw, each lane one row, LU
 * with partial pivoting (no redo pass, forecasts of FP32 draws refined three times);
 * 0 the block LU kernels as for larger m.  in_use: whether this engine's m takes
 * the warp path. */
int sgdlm_set_warp_lu(sgdlm_handle h, int enable);
int sgdlm_get_warp_lu(sgdlm_handle h, int *enabled, int *in_use);
typedef struct {
  int levels;           /* chosen sparse elimination levels */
  int tensor_cores;     /* chosen: 1 tensor-core fast pass, 0 FFMA */
  int core_n;           /* dense core of the chosen plan */
  double ms;            /* its LU time for nsim draws (median of 3) */
  double ms_candidates[8]; /* levels {0, 2, 4, 6} x tensor cores {1, 0} (-1: not run) */
} sgdlm_lu_tuning;
/* Times the batched LU of the current draws' distribution (draws sampled once
 * from the current parameters, the RNG epoch left unchanged) over the
 * candidates and keeps the fastest; overwrites the draw buffers.  Needs
 * initialised simulation memory. */
int sgdlm_tune_lu(sgdlm_handle h, sgdlm_lu_tuning *out);

typedef struct sgdlm_batch *sgdlm_batch_handle;
/* A batch over `count` engines (each in the prior state with simulation memory)
 * that advance together.  The engines stay owned by the caller and must outlive
 * the batch. */
int sgdlm_batch_create(const sgdlm_handle *handles, size_t count, sgdlm_batch_handle *out);
int sgdlm_batch_destroy(sgdlm_batch_handle b);
/* Records one fused time step of every engine (sgdlm_filter_step_device with
 * instance i's device pointers, arrays of `count`; d_x, d_forecast, d_is_weights,
 * d_step_stats may be NULL arrays or hold NULLs) into one CUDA graph whose
 * branches, one per engine, run concurrently.  Re-recording replaces it. */
int sgdlm_batch_record(sgdlm_batch_handle b, const double *const *d_y, const double *const *d_F,
                       const double *const *d_x, double ess_threshold,
                       double *const *d_forecast, double *const *d_is_weights,
                       double *const *d_step_stats);
/* One time step of every engine: one graph launch, ordered after the engines'
 * earlier work and before their later work; returns without synchronising.
 * The inputs are read from the recorded pointers (refresh them before). */
int sgdlm_batch_step(sgdlm_batch_handle b);
typedef struct {
  int buckets;                 /* m buckets (m rounded up to 32) tuned */
  int lu_plans_kept;           /* 1: the per-bucket LU plans made the step faster and are kept */
  int concurrency;             /* chosen c: each engine's LU grid capped at (2 x SMs) / c */
  double ms_untuned;           /* batch step time before tuning */
  double ms_per_step;          /* batch step time with the chosen plans and c */
  double ms_candidates[4];     /* c = 1, 2, 4, 8 */
} sgdlm_batch_tuning;
/* Autotuner: per m bucket, sgdlm_tune_lu on one engine and its choice applied
 * to the bucket, kept only if the whole batch step gets faster; then the
 * concurrency c.  Every candidate is timed over `replays` recorded steps (the
 * engines' parameters and RNG states are restored after each), so the tuned
 * step is never slower than the untuned one as measured.  Re-records with the
 * choice.  Needs a recording. */
int sgdlm_batch_autotune(sgdlm_batch_handle b, int replays, sgdlm_batch_tuning *out);

/* The handle's CUDA stream (cudaStream_t), for events and graph capture. */
int sgdlm_get_stream(sgdlm_handle h, void **stream);
/* Blocks until the handle's stream is idle. */
int sgdlm_synchronize(sgdlm_handle h);
/* Kernel launches issued by this handle so far (for launch accounting). */
int sgdlm_get_launch_count(sgdlm_handle h, uint64_t *count);

#ifdef __cplusplus
}
#endif

#endif /* SGDLM_GB300_H_ */
