/*
 * mocat_gb300 C ABI (libmocatgb.so) -- the drop-in boundary of the
 * particle-system step of mocat (propagate -> weight -> logsumexp/ESS ->
 * resample -> gather) on GB300 (sm_103a).
 *
 * Conventions
 *   - Every entry point returns an int status (MGB_OK = 0); nothing throws.
 *   - Pointers suffixed _dev are caller-owned device memory; _host are host
 *     memory read during the call only.  No entry point allocates: the
 *     caller queries *_workspace() and passes a device workspace of at least
 *     that many bytes (256-byte aligned).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream); all work is
 *     enqueued on it and the call returns without synchronising.
 *   - Keys are jax.random PRNG keys: two uint32 words (PRNGKey(seed) =
 *     {0, seed}).  Draws reproduce jax.random's threefry2x32 counter layout.
 *   - Particle states are float32, dimension-major ("SoA"): x[j * n + i] is
 *     component j of particle i.  The reference's arrays are particle-major
 *     (n, d); the Python layer transposes once at entry and exit.
 *   - Device-side failures that cannot be returned synchronously (a spin
 *     wait that ran out, degenerate weights) are OR-ed into an int32 error
 *     word the caller passes (err_dev, may be NULL): bit 1 = a bounded wait
 *     ran out, bit 2 = every weight was zero / non-finite.
 * Thread-safety: calls on different streams with different workspaces are
 * independent; the only global mutable state is the fixed scratch array of
 * mgb_resample_systematic_u_noalloc and the mutex-guarded autotune cache of
 * mgb_pf_sv_batch_autotune.
 */
#ifndef MOCAT_GB300_H
#define MOCAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  MGB_OK = 0,
  MGB_ERR_BAD_ARG = 1,
  MGB_ERR_UNSUPPORTED = 2,
  MGB_ERR_LAUNCH = 3,
  MGB_ERR_WORKSPACE = 4,
  MGB_ERR_DEVICE_TIMEOUT = 5,
  MGB_ERR_NONFINITE_WEIGHTS = 6,
  MGB_ERR_CUDA = 7
};

/* resampling schemes */
enum {
  MGB_RESAMPLE_SYSTEMATIC = 0,  /* new: u = uniform(key), thresholds (k + u)/n      */
  MGB_RESAMPLE_MULTINOMIAL = 1, /* new: inverse CDF at sorted uniforms from n+1 exponentials(key) */
  MGB_RESAMPLE_CATEGORICAL = 2  /* mocat's random.categorical(key, lw, (n,)) Gumbel-max, O(n^2) */
};

const char *mgb_status_string(int status);
int mgb_version(void);

/* ------------------------------------------------------------ jax.random
 * Replace the jax.random calls of the reference's hot path:
 *   random.split          mocat/src/ssm/filtering.py:181, 267, 278, 294; mocat/src/transport/smc.py:82
 *   random bits/uniform   (categorical's Gumbel draw) mocat/src/ssm/filtering.py:199
 *   random.normal         mocat/src/ssm/linear_gaussian/linear_gaussian.py:51, 94
 */
int mgb_random_bits(const uint32_t *key_dev, int64_t n, uint32_t *out_dev, void *stream);
int mgb_split(const uint32_t *key_dev, int64_t num, uint32_t *out_dev /* (num, 2) */, void *stream);
int mgb_uniform(const uint32_t *key_dev, int64_t n, float *out_dev, void *stream);
int mgb_normal(const uint32_t *key_dev, int64_t n, float *out_dev, void *stream);
int mgb_exponential(const uint32_t *key_dev, int64_t n, float *out_dev, void *stream);
int mgb_gumbel(const uint32_t *key_dev, int64_t n, float *out_dev, void *stream);
/* vmap(lambda k: random.normal(k, (d,)))(keys): out (nkeys, d) particle-major */
int mgb_normal_keys(const uint32_t *keys_dev, int64_t nkeys, int64_t d, float *out_dev, void *stream);
/* the library's own float maths on device (op 0 = log, 1 = exp, 2 = erfinv) */
int mgb_math_eval(int op, const float *x_dev, int64_t n, float *out_dev, void *stream);

/* --------------------------------------------------- logsumexp and ESS
 * Replaces log_ess_log_weight / ess_log_weight (mocat/src/metrics.py:69-78) and
 * jax.scipy.special.logsumexp as used at mocat/src/transport/smc.py:160, 214-215.
 * out4_dev = {max, logsumexp(lw), logsumexp(2 lw), ess} in float64.
 */
size_t mgb_lse_ess_workspace(int64_t n);
int mgb_lse_ess(const float *lw_dev, int64_t n, double *out4_dev, void *ws_dev, size_t ws_bytes, void *stream);

/* --------------------------------------------------------- resampling
 * Replaces _resample / resample_particles (mocat/src/ssm/filtering.py:196-217)
 * and SMCSampler.resample's index draw (mocat/src/transport/smc.py:61-67).
 * Ancestors are int32 in [0, n).  Weights are quantised to 62-bit fixed
 * point, so systematic / multinomial ancestors are independent of summation
 * order.  key_dev is the step key (mocat's int_rand_key).
 */
size_t mgb_resample_workspace(int64_t n, int scheme);
int mgb_resample(const float *lw_dev, int64_t n, int scheme, const uint32_t *key_dev, int32_t *ancestors_dev,
                 void *ws_dev, size_t ws_bytes, int32_t *err_dev, void *stream);
/* systematic with the uniform fed in as its 23-bit mantissa: u = m23 * 2^-23 */
int mgb_resample_systematic_u(const float *lw_dev, int64_t n, uint32_t m23, int32_t *ancestors_dev, void *ws_dev,
                              size_t ws_bytes, int32_t *err_dev, void *stream);

/* Systematic resampling that allocates nothing.  No counterpart in the
 * reference: it is for callers that cannot allocate device memory (an XLA
 * custom call or framework-built CUDA-graph node handed only its buffers, a
 * plugin inside a process whose allocator owns the device heap).  Same result
 * as mgb_resample_systematic_u; the scratch lives in a fixed device array
 * inside the library (256 KiB, resident on each device that loads it until
 * exit), so n must not exceed MGB_NOALLOC_MAX_N (else MGB_ERR_UNSUPPORTED).
 * The first call in each CUDA context looks up that array's address (cached
 * per context ID, so a context made after cudaDeviceReset looks it up again):
 * make it before any stream capture.  Calls share the array; calls that
 * overlap on the GPU race on it. */
#define MGB_NOALLOC_MAX_N (1 << 24)
int mgb_resample_systematic_u_noalloc(const float *lw_dev, int64_t n, uint32_t m23, int32_t *ancestors_dev,
                                      int32_t *err_dev, void *stream);

/* ------------------------------------------------ bounded device waits
 * Every spin wait in the library's kernels (the persistent filter's grid
 * barrier, the decoupled-lookback tile scan) gives up after a fixed number of
 * polls, raises bit 1 of the error word and lets the kernel finish, so a
 * wait that cannot end costs a bounded delay and an error status instead of a
 * hung GPU.  mgb_wait_selftest makes one such wait run out on purpose, with
 * the library's own wait code and a given poll limit (1 .. 2^22), on a wait
 * that nothing will satisfy: a grid barrier one block short
 * (MGB_WAIT_GRID_BARRIER) or a lookback whose predecessor tile never
 * publishes (MGB_WAIT_LOOKBACK).  It returns MGB_ERR_DEVICE_TIMEOUT when the
 * wait ran out and reported it (the expected result), synchronising `stream`.
 * No counterpart in the reference, whose JAX code has no device waits
 * (its only run-time guard is mocat/src/transport/smc.py:174-175).
 * ws_dev: mgb_wait_selftest_workspace() bytes. */
#define MGB_WAIT_GRID_BARRIER 0
#define MGB_WAIT_LOOKBACK 1
size_t mgb_wait_selftest_workspace(void);
int mgb_wait_selftest(int which, int32_t polls, void *ws_dev, size_t ws_bytes, void *stream);

/* ---------------------------------------------------------------- gather
 * Replaces the fancy-index gathers x[..., idx, :] (mocat/src/ssm/filtering.py:199)
 * and cdict.__getitem__ (mocat/src/core.py:46-56): out[k, :] = x[anc[k], :]
 * for a particle-major (n_in, width) float32 array (any width; vectorised
 * when rows are 16-byte aligned).
 */
int mgb_gather_rows(const float *x_dev, int64_t width, const int32_t *ancestors_dev, int64_t n_out, float *out_dev,
                    void *stream);

/* --------------------------------------- particle filter, linear Gaussian
 * TimeHomogenousLinearGaussian (mocat/src/ssm/linear_gaussian/linear_gaussian.py:142-261)
 * with BootstrapFilter (mocat/src/ssm/filtering.py:142-170):
 *   x_t = F x_{t-1} + Lq eps,  eps = normal(split(k_t, n)[i], (d,))
 *   potential(x, y) = 0.5 |(y - H x) @ P|^2 + c
 * Model matrices are host pointers, row-major float32:
 *   F, Lq, C0: d x d (transition_matrix, transition_covariance_sqrt,
 *   initial_covariance_sqrt); H: dy x d (likelihood_matrix); P: dy x dy
 *   (likelihood_precision_sqrt); m0: d; c = (dy log 2 pi - log det_prec) / 2.
 * Compiled (d, dy): (d, 1) for d in {1,2,3,4,5,8,10}; (d, d) for d in {2,3,4,5,8,10}.
 * mgb_pf_lg_init / mgb_pf_lg_propagate / mgb_pf_lg_run also take any other d, dy <= 32
 * (run-time-dimension kernels, the same values, one launch per phase and step); the
 * other entry points that take this model need a compiled pair.
 */
typedef struct {
  int32_t d, dy;
  const float *F, *Lq, *H, *P, *C0, *m0;
  float c;
} mgb_lg_model;

/* initiate_particles (mocat/src/ssm/filtering.py:173-193): x (d, n), lw (n) */
int mgb_pf_lg_init(const mgb_lg_model *model_host, int64_t n, const uint32_t *key_dev, const float *y0_dev,
                   float *x_dev, float *lw_dev, void *stream);
/* one propagate_and_intermediate_weight step (mocat/src/ssm/filtering.py:294-303):
 * x_new[:, i] = F x_prev[:, anc[i]] + Lq eps_i, lw_new = lw_prev - potential.
 * ancestors_dev == NULL means no resampling (identity); lw_prev_dev == NULL means 0. */
int mgb_pf_lg_propagate(const mgb_lg_model *model_host, int64_t n, const uint32_t *key_t_dev, const float *y_t_dev,
                        const float *x_prev_dev, const int32_t *ancestors_dev, const float *lw_prev_dev,
                        float *x_new_dev, float *lw_new_dev, void *stream);

/* outputs of a whole-filter run (device pointers, each may be NULL) */
typedef struct {
  double *log_z;      /* scalar: log-marginal-likelihood estimate from the log-weights */
  float *ess;         /* (T,) ESS after each step (filtering.py:310) */
  int32_t *resampled; /* (T,) 1 if step t began with a resample */
  float *x_hist;      /* (T, d, n) particle history, dimension-major per step */
  float *lw_hist;     /* (T, n) log-weight history */
  float *x_final;     /* (d, n) final particles */
  float *lw_final;    /* (n,) final log-weights */
  int32_t *err;       /* device error word */
  uint64_t *trace;    /* (T * 10 + 1024) diagnostics of the persistent kernel (NULL = off):
                         [t * 10 + k] device-clock ns at the phase boundaries of step t seen by
                         block 0 (start, propagate done, barrier, combine done, tile sums done,
                         barrier, tile-sum scan done, offspring runs written, barrier);
                         [T * 10 + b] (b < 1024) ns block b spent propagating step 1 */
} mgb_pf_outputs;

/* run_particle_filter_for_marginals (mocat/src/ssm/filtering.py:255-324) with
 * ESS-triggered resampling (resample at t when ess_{t-1} < ess_threshold * n).
 * Systematic resampling with even n <= 2^21 runs as one persistent cooperative
 * kernel for all T steps; OR-ing MGB_RUN_LAUNCH_PER_STEP into `scheme` forces
 * the launch-per-step path (same results). */
#define MGB_RUN_LAUNCH_PER_STEP 0x100
size_t mgb_pf_lg_workspace(int64_t n, int64_t T, int32_t d, int scheme);
int mgb_pf_lg_run(const mgb_lg_model *model_host, int64_t n, int64_t T, const uint32_t *key_dev, const float *y_dev,
                  float ess_threshold, int scheme, void *ws_dev, size_t ws_bytes, const mgb_pf_outputs *out,
                  void *stream);

/* ----------------------------------------------- adjoint: d log Z / d theta
 * Gradient of the bootstrap filter's log Z (run_particle_filter_for_marginals,
 * mocat/src/ssm/filtering.py:255-324, as mgb_pf_lg_run) with the ancestors and
 * resampling decisions held fixed, for a model with H = I and diagonal Lq, P:
 * theta = (A = F, log q, log r) with q_k = Lq_kk^2, r_k = P_kk^-2.  One call
 * runs the taped forward filter (ancestors of every step, (x, lw) every
 * ckpt_every steps), then the backward pass, recomputing each segment of
 * ckpt_every steps from its checkpoint.
 * grad_dev (d*d + 2d floats): dA row-major, then d/dlog q_k, then d/dlog r_k.
 * log_z_dev (1 double) and resampled_dev (T int32) may be NULL.  scheme:
 * systematic or multinomial.  Synchronises `stream` once, between the passes.
 * The forward pass is one persistent cooperative launch (the whole GPU) for
 * systematic resampling with even n <= 2^21; OR-ing MGB_RUN_LAUNCH_PER_STEP into
 * `scheme` runs it one launch per phase instead, which lets gradients on
 * several streams overlap (same results, log Z within 1e-6). */
size_t mgb_pf_lg_grad_workspace(int64_t n, int64_t T, int32_t d, int32_t ckpt_every);
int mgb_pf_lg_grad(const mgb_lg_model *model_host, int64_t n, int64_t T, const uint32_t *key_dev, const float *y_dev,
                   float ess_threshold, int scheme, int32_t ckpt_every, void *ws_dev, size_t ws_bytes,
                   double *log_z_dev, float *grad_dev, int32_t *resampled_dev, void *stream);

/* ------------------------------ score by Fisher's identity (smoothed, PaRIS)
 * Consistent estimate of d log p(y) / d theta for the model of mgb_pf_lg_grad
 * (H = I, diagonal Lq and P; theta = (A = F, log q, log r)), made along the
 * same bootstrap filter (run_particle_filter_for_marginals,
 * mocat/src/ssm/filtering.py:255-324, as mgb_pf_lg_run on `key`): by Fisher's
 * identity the score is the smoothed expectation of the complete-data score,
 * and each particle carries that additive functional forward, PaRIS-style,
 * averaged over `backward_draws` (K, 1..4) backward draws per step: the
 * particle's own ancestor, then draws of an independent-Metropolis chain with
 * `mcmc_steps` (L) uniform proposals each, (K - 1) L <= 4096.  K = 1 traces
 * the statistic along the genealogy only.  Unlike mgb_pf_lg_grad (the
 * gradient of the log Z estimate with the resampling held fixed, which does
 * not converge to the score), the error of this estimate falls as n grows.
 * smoothing_key_dev (2 words) seeds the backward draws; T <= 2^20.
 * grad_dev: d*d + 2d floats in mgb_pf_lg_grad's layout (summed in float64).
 * log_z_dev, resampled_dev (T) and draws_dev ((T, n, K) int32: the source
 * particle index of every backward draw, row t >= 1) may be NULL.
 * One launch per phase and step on `stream`; no host synchronisation. */
size_t mgb_pf_lg_score_workspace(int64_t n, int64_t T, int32_t d);
int mgb_pf_lg_score(const mgb_lg_model *model_host, int64_t n, int64_t T, const uint32_t *key_dev,
                    const uint32_t *smoothing_key_dev, const float *y_dev, float ess_threshold, int scheme,
                    int32_t backward_draws, int32_t mcmc_steps, void *ws_dev, size_t ws_bytes, double *log_z_dev,
                    float *grad_dev, int32_t *resampled_dev, int32_t *draws_dev, void *stream);

/* mgb_pf_lg_score for B filters at once (keys_dev and smoothing_keys_dev: (B, 2)),
 * one launch per phase and step for all B: every per-step kernel runs one
 * filter per grid row on that filter's workspace slab, so B latency-bound
 * filters share each launch.  Systematic resampling, even n.  Each filter's
 * log Z and score equal those of mgb_pf_lg_score with its keys, bit for bit.
 * log_z_dev: B doubles (may be NULL); grad_dev: (B, d*d + 2d) floats.
 * No counterpart in the reference beyond mgb_pf_lg_score's (one filter per call there). */
size_t mgb_pf_lg_score_batch_workspace(int64_t n, int64_t T, int32_t d, int64_t B);
int mgb_pf_lg_score_batch(const mgb_lg_model *model_host, int64_t n, int64_t T, int64_t B, const uint32_t *keys_dev,
                          const uint32_t *smoothing_keys_dev, const float *y_dev, float ess_threshold,
                          int32_t backward_draws, int32_t mcmc_steps, void *ws_dev, size_t ws_bytes, double *log_z_dev,
                          float *grad_dev, void *stream);

/* --------------------------------------------- backward simulation (FFBSi)
 * backward_simulation with maximum_rejections = 0, i.e. backward_simulation_full
 * (mocat/src/ssm/backward.py:217-245, full_resampling :20-40), for a linear-Gaussian
 * transition: t_keys = split(key, T); the M samples at T-1 are
 * categorical(t_keys[T-1], lw_{T-1}, (M,)); for t = T-2 .. 0 sample j takes
 * argmax_i gumbel(split(t_keys[t], M)[j], (N,))_i + lw_{t,i} - transition_potential(x_t^i -> xs_{t+1}^j),
 * transition_potential(x0 -> x1) = 0.5 |(x1 - F x0) @ Pq|^2 + cq.
 * x_hist (T, d, N) dimension-major (the filter's history), lw_hist (T, N);
 * out (T, d, M) sampled trajectories, idx (T, M) the chosen particle indices.
 * 1 <= d <= 32 (d in {1,2,3,4,5,8,10} compiled, any other d on the run-time-dimension
 * kernels; the same operations); M N < 2^32.  The same range holds for every entry point
 * that takes an mgb_lg_transition (stitching, potential pairs, the rejection variants). */
typedef struct {
  int32_t d;
  const float *F;  /* d x d transition_matrix (host) */
  const float *Pq; /* d x d transition_precision_sqrt (host) */
  float cq;        /* (d log 2 pi - log transition_precision_det) / 2 */
} mgb_lg_transition;
/* full_stitch (mocat/src/ssm/online_smoothing.py:21-41): keys = split(key, M0);
 * idx_j = argmax_i gumbel(keys[j], (M1,))_i + lw1_i - transition_potential(x0_j -> x1_i);
 * x0 (d, M0), x1 (d, M1) dimension-major. */
int mgb_stitch_lg(const mgb_lg_transition *transition_host, int64_t M0, int64_t M1, const float *x0_dev,
                  const float *x1_dev, const float *lw1_dev, const uint32_t *key_dev, int32_t *idx_dev, void *stream);
/* out_i = lw_i + transition_potential(x0_i -> x1_i) (lw_dev NULL: the potential alone) --
 * the non-interacting log-weight of fixed_lag_stitching (online_smoothing.py:191-193) */
int mgb_transition_potential_pairs(const mgb_lg_transition *transition_host, int64_t M, const float *x0_dev,
                                   const float *x1_dev, const float *lw_dev, float *out_dev, void *stream);
size_t mgb_ffbsi_workspace(int64_t N, int64_t T, int32_t d);
int mgb_ffbsi_lg(const mgb_lg_transition *transition_host, int64_t T, int64_t N, int64_t M, const float *x_hist_dev,
                 const float *lw_hist_dev, const uint32_t *key_dev, float *out_dev, int32_t *idx_dev, void *ws_dev,
                 size_t ws_bytes, void *stream);

/* ------------------------------------ particle filter, optimal proposal
 * OptimalNonLinearGaussianParticleFilter (mocat/src/ssm/nonlinear_gaussian.py:134-281)
 * for a linear transition f(x) = F x with linear-Gaussian observations:
 *   init:  x_0 = (m0 + K0 (y_0 - H m0)) + eps C0c, lw_0 = 0
 *   step:  mx = F x_prev[a_i], r = y_t - H mx,
 *          x_new = (mx + K r) + S eps_i, lw_new = lw_res - (0.5 |r W|^2 + cw)
 * with eps = normal(split(k, n)[0], (n, d)) -- one key for the whole (n, d)
 * draw (nonlinear_gaussian.py:275).  Matrices are host pointers, row-major
 * float32, computed as the reference's startup (:154-184) does:
 *   F (d x d) transition matrix; H (dy x d) likelihood_matrix;
 *   K (d x dy) proposal_kalman_gain; S (d x d) proposal_covariance_sqrt;
 *   W (dy x dy) weight_precision_sqrt; cw = (dy log 2 pi - log weight_precision_det) / 2;
 *   K0 (d x dy) initial_kalman_gain; C0c (d x d) initial_conditioned_covariance_sqrt;
 *   m0 (d) initial_mean.
 * Supported (d, dy): the compiled pairs of mgb_lg_model, and any other pair with d, dy <= 32
 * on the run-time-dimension instance (the same operations in the same order); n d < 2^32.
 */
typedef struct {
  int32_t d, dy;
  const float *F, *H, *K, *S, *W;
  float cw;
  const float *K0, *C0c, *m0;
} mgb_opt_model;

int mgb_pf_opt_init(const mgb_opt_model *model_host, int64_t n, const uint32_t *key_dev, const float *y0_dev,
                    float *x_dev, float *lw_dev, void *stream);
/* propose_and_intermediate_weight_vectorised (nonlinear_gaussian.py:264-281) for one step;
 * ancestors_dev == NULL: no resampling; lw_prev_dev == NULL: 0 */
int mgb_pf_opt_propagate(const mgb_opt_model *model_host, int64_t n, const uint32_t *key_t_dev, const float *y_t_dev,
                         const float *x_prev_dev, const int32_t *ancestors_dev, const float *lw_prev_dev,
                         float *x_new_dev, float *lw_new_dev, void *stream);
/* run_particle_filter_for_marginals with this filter (launch per step; outputs as mgb_pf_lg_run) */
size_t mgb_pf_opt_workspace(int64_t n, int64_t T, int32_t d, int scheme);
int mgb_pf_opt_run(const mgb_opt_model *model_host, int64_t n, int64_t T, const uint32_t *key_dev, const float *y_dev,
                   float ess_threshold, int scheme, void *ws_dev, size_t ws_bytes, const mgb_pf_outputs *out,
                   void *stream);

/* ------------------------------------- one-dimensional non-linear benchmark
 * BootstrapFilter on NonLinear1DBenchmark (mocat/src/ssm/scenarios/nonlinear1d.py:16-80):
 *   x_0 = normal(key_i, (1,)) initial_sd
 *   x_t = 0.5 x + 25 x / (1 + x^2) + 8 cos(1.2 t_prev) + normal(key_i, (1,)) transition_sd
 *   potential(x, y) = 0.5 ((y - x^2 / 20) / likelihood_sd)^2 + c,  c = log(2 pi) / 2 in float32
 * key_i = split(k, n)[i]; particles and log-weights are (n) float32.
 * 8 cos(1.2 t) is 8 * float(cos(double(1.2f * t))).
 */
typedef struct {
  float initial_sd, transition_sd, likelihood_sd;
  float c;
} mgb_nl1d_model;

/* initiate_particles (filtering.py:173-193); y0_dev == NULL: zero weights */
int mgb_pf_nl1d_init(const mgb_nl1d_model *model_host, int64_t n, const uint32_t *key_dev, const float *y0_dev,
                     float *x_dev, float *lw_dev, void *stream);
/* propose_and_intermediate_weight_vectorised (filtering.py:124-139) for one step from
 * t_previous; ancestors_dev == NULL: no resampling; lw_prev_dev == NULL: 0 */
int mgb_pf_nl1d_propagate(const mgb_nl1d_model *model_host, int64_t n, const uint32_t *key_t_dev, const float *y_t_dev,
                          float t_previous, const float *x_prev_dev, const int32_t *ancestors_dev,
                          const float *lw_prev_dev, float *x_new_dev, float *lw_new_dev, void *stream);
/* run_particle_filter_for_marginals (filtering.py:255-324); t_dev holds the T times
 * (step t uses t_dev[t-1] as t_previous); outputs as mgb_pf_lg_run with d = 1 */
size_t mgb_pf_nl1d_workspace(int64_t n, int64_t T, int scheme);
int mgb_pf_nl1d_run(const mgb_nl1d_model *model_host, int64_t n, int64_t T, const uint32_t *key_dev, const float *y_dev,
                    const float *t_dev, float ess_threshold, int scheme, void *ws_dev, size_t ws_bytes,
                    const mgb_pf_outputs *out, void *stream);
/* Backward simulation and stitching with this model's transition
 * (transition_potential, nonlinear1d.py:48-54):
 *   transition_potential(x0 at t_prev -> x1) = 0.5 ((x1 - mean(x0, t_prev)) / transition_sd)^2 + c
 * with the key flows of mgb_ffbsi_lg / mgb_stitch_lg / mgb_transition_potential_pairs.
 * mgb_ffbsi_nl1d: x_hist (T, N), lw_hist (T, N), t_dev the T times (step t's
 * transition leaves t_dev[t]); out (T, M), idx (T, M); workspace mgb_ffbsi_workspace(N, T, 1). */
int mgb_ffbsi_nl1d(const mgb_nl1d_model *model_host, int64_t T, int64_t N, int64_t M, const float *x_hist_dev,
                   const float *lw_hist_dev, const float *t_dev, const uint32_t *key_dev, float *out_dev,
                   int32_t *idx_dev, void *ws_dev, size_t ws_bytes, void *stream);
int mgb_stitch_nl1d(const mgb_nl1d_model *model_host, int64_t M0, int64_t M1, const float *x0_dev,
                    const float *x1_dev, const float *lw1_dev, float t_previous, const uint32_t *key_dev,
                    int32_t *idx_dev, void *stream);
int mgb_transition_potential_pairs_nl1d(const mgb_nl1d_model *model_host, int64_t M, const float *x0_dev,
                                        const float *x1_dev, float t_previous, const float *lw_dev, float *out_dev,
                                        void *stream);

/* Backward simulation and stitching with the stochastic-volatility transition (dim 1,
 * stochastic_volatility.py:78-85): transition_potential(x0 -> x1) = 0.5 ((x1 - phi x0) pq sqrt(dt))^2,
 * pq = transition_precision_sqrt (1 / sqrt(transition_covariance)), no normaliser (the reference's
 * 2-D precision square root carries no det), dt = t_new - t_prev.  Key flows as the
 * linear-Gaussian entries.  mgb_ffbsi_sv takes the T times on the HOST (t_host), step t using
 * t_host[t + 1] - t_host[t]; x_hist, lw_hist (T, N) device; workspace mgb_ffbsi_workspace(N, T, 1). */
int mgb_ffbsi_sv(float phi, float pq, int64_t T, int64_t N, int64_t M, const float *x_hist_dev,
                 const float *lw_hist_dev, const float *t_host, const uint32_t *key_dev, float *out_dev,
                 int32_t *idx_dev, void *ws_dev, size_t ws_bytes, void *stream);
int mgb_stitch_sv(float phi, float pq, int64_t M0, int64_t M1, const float *x0_dev, const float *x1_dev,
                  const float *lw1_dev, float dt, const uint32_t *key_dev, int32_t *idx_dev, void *stream);
int mgb_transition_potential_pairs_sv(float phi, float pq, int64_t M, const float *x0_dev, const float *x1_dev,
                                      float dt, const float *lw_dev, float *out_dev, void *stream);

/* ------------------------------ backward simulation and stitching by rejection
 * maximum_rejections > 0: backward_simulation_rejection (mocat/src/ssm/backward.py:172-214,
 * rejection_resampling :54-169) and rejection_stitching (mocat/src/ssm/online_smoothing.py:59-175,
 * called by fixed_lag_stitching :178-209).  n items with fixed states each draw an index into a pool
 * of Np particles with log-weights lw, accepting pair (i, j) with probability
 * exp(-transition_potential) / bound:
 *   (c0, u0, k0) = split(key, 3); idx = categorical(c0, lw, (n,)); dens_i = exp(-potential(i, idx_i));
 *   bound = max dens > init_bound_param ? max dens * bound_inflation : init_bound_param;
 *   unaccepted_i = uniform(u0, (n,))_i > dens_i / bound; key_i = split(k0, n)_i; evals = n;
 *   up to maximum_rejections - 1 rounds while any item is unaccepted: evals += #unaccepted; each
 *   unaccepted item: (key_i, c, u) = split(key_i, 3), idx_i = categorical(c, lw), dens_i, accept
 *   unless uniform(u) > dens_i / bound; if the round's max dens > bound: bound = max dens *
 *   bound_inflation and every item is unaccepted again;
 *   then each unaccepted item: idx_i = categorical(key_i, lw - potential(i, .)); evals += Np * #unaccepted.
 * Backward simulation: items = the M samples at t+1, pool = the N filter particles at t, keys and
 * the last step as mgb_ffbsi_lg; evals (T, int64, device): evals[0] = 0, evals[t+1] = step t's
 * count (the reference's append(0, ...) layout).  Stitching: items = x0 (M), pool = x1 (M),
 * evals (1, int64, device).  These entry points synchronise their stream (the host reads a
 * device flag between groups of rounds); not for stream capture. */
typedef struct {
  int32_t maximum_rejections; /* >= 1 */
  float init_bound_param;     /* transition_dens_bound_parameter */
  float bound_inflation;
} mgb_rejection_config;
size_t mgb_ffbsi_rejection_workspace(int64_t N, int64_t M, int64_t T, int32_t d);
size_t mgb_stitch_rejection_workspace(int64_t M, int32_t d);
int mgb_ffbsi_rejection_lg(const mgb_lg_transition *transition_host, const mgb_rejection_config *cfg_host, int64_t T,
                           int64_t N, int64_t M, const float *x_hist_dev, const float *lw_hist_dev,
                           const uint32_t *key_dev, float *out_dev, int32_t *idx_dev, int64_t *evals_dev,
                           void *ws_dev, size_t ws_bytes, void *stream);
int mgb_ffbsi_rejection_nl1d(const mgb_nl1d_model *model_host, const mgb_rejection_config *cfg_host, int64_t T,
                             int64_t N, int64_t M, const float *x_hist_dev, const float *lw_hist_dev,
                             const float *t_dev, const uint32_t *key_dev, float *out_dev, int32_t *idx_dev,
                             int64_t *evals_dev, void *ws_dev, size_t ws_bytes, void *stream);
int mgb_stitch_rejection_lg(const mgb_lg_transition *transition_host, const mgb_rejection_config *cfg_host, int64_t M,
                            const float *x0_dev, const float *x1_dev, const float *lw1_dev, const uint32_t *key_dev,
                            int32_t *idx_dev, int64_t *evals_dev, void *ws_dev, size_t ws_bytes, void *stream);
int mgb_stitch_rejection_nl1d(const mgb_nl1d_model *model_host, const mgb_rejection_config *cfg_host, int64_t M,
                              const float *x0_dev, const float *x1_dev, const float *lw1_dev, float t_previous,
                              const uint32_t *key_dev, int32_t *idx_dev, int64_t *evals_dev, void *ws_dev,
                              size_t ws_bytes, void *stream);
int mgb_ffbsi_rejection_sv(float phi, float pq, const mgb_rejection_config *cfg_host, int64_t T, int64_t N,
                           int64_t M, const float *x_hist_dev, const float *lw_hist_dev, const float *t_host,
                           const uint32_t *key_dev, float *out_dev, int32_t *idx_dev, int64_t *evals_dev,
                           void *ws_dev, size_t ws_bytes, void *stream);
int mgb_stitch_rejection_sv(float phi, float pq, const mgb_rejection_config *cfg_host, int64_t M,
                            const float *x0_dev, const float *x1_dev, const float *lw1_dev, float dt,
                            const uint32_t *key_dev, int32_t *idx_dev, int64_t *evals_dev, void *ws_dev,
                            size_t ws_bytes, void *stream);

/* ------------------------------- many stochastic-volatility filters at once
 * B independent run_particle_filter_for_marginals calls (mocat/src/ssm/filtering.py:255-324)
 * with BootstrapFilter on StochasticVolatility, d = 1
 * (mocat/src/ssm/scenarios/stochastic_volatility.py:71-108), each with its own
 * particle count n_b, length T_b, observations y[y_off_b : y_off_b + T_b] and key
 * keys[2b : 2b + 2]; the reference runs them one after another.  All filters
 * run in one persistent launch: each CTA takes bundles of filters of similar
 * size and length from a work queue and keeps every filter's particles in
 * shared memory for all of its steps.
 *   x_t = phi x_{t-1} + bsig eps,  x_0 = c0 eps + m0,  eps = normal(split(k_t, n)[i], (1,))
 *   potential(x, y) = (0.5 y^2 r2) exp(-x) + 0.5 x + cB
 * Resampling is ESS-triggered (ess_{t-1} < ess_threshold * n_b), multinomial or
 * systematic.  1 <= T_b, 2 <= n_b <= MGB_SV_BATCH_MAX_N.
 */
#define MGB_SV_BATCH_MAX_N 8192
typedef struct {
  float phi;  /* transition_matrix */
  float bsig; /* transition_covariance_sqrt * sqrt(t_new - t_prev) */
  float r2;   /* likelihood_precision_diag_sqrt ** 2 */
  float cB;   /* (log 2 pi - log r2) / 2 */
  float c0;   /* initial_covariance_sqrt */
  float m0;   /* initial_mean */
} mgb_sv_model;

/* One series with the particle history: run_particle_filter_for_marginals
 * (filtering.py:255-324) with BootstrapFilter on StochasticVolatility (dim 1),
 * outputs as mgb_pf_lg_run with d = 1.  Here model->bsig is
 * transition_covariance_sqrt (the dt = 1 value): step t scales it by
 * sqrt(t_dev[t] - t_dev[t-1]) (propagate: by sqrt(dt)).  Systematic resampling
 * with even n <= 2^21 runs as one persistent launch. */
int mgb_pf_sv_init(const mgb_sv_model *model_host, int64_t n, const uint32_t *key_dev, const float *y0_dev,
                   float *x_dev, float *lw_dev, void *stream);
int mgb_pf_sv_propagate(const mgb_sv_model *model_host, int64_t n, const uint32_t *key_dev, const float *y_dev,
                        float dt, const float *x_prev_dev, const int32_t *ancestors_dev, const float *lw_prev_dev,
                        float *x_new_dev, float *lw_new_dev, void *stream);
size_t mgb_pf_sv_workspace(int64_t n, int64_t T, int scheme);
int mgb_pf_sv_run(const mgb_sv_model *model_host, int64_t n, int64_t T, const uint32_t *key_dev, const float *y_dev,
                  const float *t_dev, float ess_threshold, int scheme, void *ws_dev, size_t ws_bytes,
                  const mgb_pf_outputs *out, void *stream);

/* The d-dimensional stochastic-volatility model (mocat/src/ssm/scenarios/
 * stochastic_volatility.py:15-108) with a diagonal likelihood covariance R, on
 * run-time-dimension kernels (1 <= d <= 32):
 *   x_0 = C0 normal(key, (d,)) + m0                   (initial_sample :71-76)
 *   x_t = A x_{t-1} + (Lq normal(key, (d,))) sqrt(dt)  (transition_sample :87-94)
 *   potential(x, y) = cB + sum_j (0.5 x_j + 0.5 y_j^2 r2_j exp(-x_j))   (:96-102)
 * with r2 = 1 / R and cB = (d log 2 pi - sum_j log r2_j) / 2.  Host pointers,
 * row-major float32. */
typedef struct {
  int32_t d;
  const float *A, *Lq, *C0, *m0; /* transition_matrix, transition_covariance_sqrt,
                                    initial_covariance_sqrt (d x d); initial_mean (d) */
  const float *r2;                /* (d) 1 / likelihood_covariance_diag */
  float cB;
} mgb_svd_model;
/* initiate_particles / one propagate step (dt = t_new - t_previous) / the whole filter
 * with the times t_dev (T,) (run_particle_filter_for_marginals, filtering.py:255-324),
 * arguments and outputs as mgb_pf_sv_*; x is (d, n) dimension-major; one launch per
 * phase and step */
int mgb_pf_svd_init(const mgb_svd_model *model_host, int64_t n, const uint32_t *key_dev, const float *y0_dev,
                    float *x_dev, float *lw_dev, void *stream);
int mgb_pf_svd_propagate(const mgb_svd_model *model_host, int64_t n, const uint32_t *key_dev, const float *y_dev,
                         float dt, const float *x_prev_dev, const int32_t *ancestors_dev, const float *lw_prev_dev,
                         float *x_new_dev, float *lw_new_dev, void *stream);
size_t mgb_pf_svd_workspace(int64_t n, int64_t T, int32_t d, int scheme);
int mgb_pf_svd_run(const mgb_svd_model *model_host, int64_t n, int64_t T, const uint32_t *key_dev,
                   const float *y_dev, const float *t_dev, float ess_threshold, int scheme, void *ws_dev,
                   size_t ws_bytes, const mgb_pf_outputs *out, void *stream);

/* launch shape of a batched run (from mgb_pf_sv_batch_plan / _autotune) */
typedef struct {
  int32_t threads;     /* CTA size: 256, 512 or 1024 */
  int32_t ppt;         /* particles per thread: a filter of slot size s runs on max(32, s / ppt) threads */
  int32_t ctas_per_sm; /* CTAs per SM (0 = as many as fit) */
  int32_t nbundles;    /* number of bundles (written by the planner) */
  int64_t smem_bytes;  /* dynamic shared memory per CTA (written by the planner) */
} mgb_sv_launch;

/* Host-side planner: validates n/T, groups the filters into bundles (filters
 * of one power-of-two slot size, similar T) and orders the bundles longest
 * first.  Writes order_host (B,) and bundles_host (4 * B int32: first, count,
 * slot, reserved) and fills launch->nbundles / smem_bytes.  threads / ppt /
 * ctas_per_sm are read from *launch. */
int mgb_pf_sv_batch_plan(int64_t B, const int32_t *n_host, const int32_t *T_host, mgb_sv_launch *launch,
                         int32_t *order_host, int32_t *bundles_host);
/* One launch over all filters.  order_dev / bundles_dev are the planner's
 * arrays copied to the device; counter_dev is one int32 of scratch (reset by
 * the call).  logz_dev (B,) receives log Z_b, nres_dev (B,) the number of
 * resampling steps (may be NULL).  Graph-capturable. */
int mgb_pf_sv_batch_run(const mgb_sv_model *model_host, int64_t B, const int32_t *n_dev, const int32_t *T_dev,
                        const int64_t *y_off_dev, const float *y_dev, const uint32_t *keys_dev,
                        const mgb_sv_launch *launch, const int32_t *order_dev, const int32_t *bundles_dev,
                        float ess_threshold, int scheme, int32_t *counter_dev, double *logz_dev, int32_t *nres_dev,
                        int32_t *err_dev, void *stream);
/* Autotuner: times every candidate launch shape on this batch, each filter cut
 * to probe_steps steps (<= 0: full length), and writes the fastest to *best.
 * Results are cached per (device, scheme, batch signature) behind a mutex.
 * Needs mgb_pf_sv_batch_autotune_workspace(B) bytes of device scratch;
 * synchronises `stream`; not capturable. */
size_t mgb_pf_sv_batch_autotune_workspace(int64_t B);
int mgb_pf_sv_batch_autotune(const mgb_sv_model *model_host, int64_t B, const int32_t *n_host, const int32_t *T_host,
                             const int32_t *n_dev, const int32_t *T_dev, const int64_t *y_off_dev, const float *y_dev,
                             const uint32_t *keys_dev, float ess_threshold, int scheme, int32_t probe_steps,
                             void *ws_dev, size_t ws_bytes, mgb_sv_launch *best, float *best_ms, void *stream);

/* ----------------------- tempered SMC on Bayesian logistic regression
 * MetropolisedSMCSampler (mocat/src/transport/smc.py:229-373) with MALA moves
 * (Underdamped(leapfrog_steps=1, friction=inf), mocat/src/mcmc/standard_mcmc.py:72-153,
 * Metropolis correction mocat/src/mcmc/metropolis.py:48-70), adaptive
 * temperatures by regula falsi on the ESS (smc.py:311-326, utils.py:205-237),
 * driven as mocat.run does (sample.py:110-148), for B independent posteriors
 * (one key each) advanced in lockstep.  Scenario: beta ~ N(0, s^2 I),
 * y_i ~ Bernoulli(sigmoid(x_i . beta)); prior potential |beta|^2 / (2 s^2),
 * likelihood potential sum_i softplus(x_i . beta) - y_i x_i . beta.
 * Resampling (ess <= ess_threshold_resample N) is systematic.
 * N <= MGB_SMC_MAX_N; d in {2, 3, 5, 10, 20, 50}.
 * The same sampler also takes (fields after `precision`; zero keeps the setting above):
 *   RandomWalk moves (standard_mcmc.py:20-64): x' = x + sqrt(stepsize) e, alpha = min(1, exp(U - U'));
 *   Underdamped with leapfrog_steps L and a finite friction f (standard_mcmc.py:72-153,
 *     utils.leapfrog :108-156): p = -p exp(-f eps) + sqrt(1 - exp(-2 f eps)) e, L leapfrog steps, the
 *     momenta kept per particle (resampled with it) between moves and iterations;
 *   a temperature_schedule (smc.py:100-125, leading 0 removed): tau_i = schedule[i];
 *   prior draws with their own scale (a scenario whose prior_sample and prior_potential differ);
 *   the Gaussian likelihood of toy_examples.Gaussian (scenarios/toy_examples.py:17-51):
 *     0.5 |(x - mean) @ prec_sqrt^T|^2, prec_sqrt = inv(chol(covariance)), X and y unused.
 */
enum { MGB_MOVE_UNDERDAMPED = 0, MGB_MOVE_RANDOM_WALK = 1 };
enum { MGB_LIK_LOGISTIC = 0, MGB_LIK_GAUSSIAN = 1 };
#define MGB_SMC_MAX_N 24576
enum { MGB_PREC_FP32 = 0, MGB_PREC_BF16 = 1 };

/* logistic potential and gradient for P parameter rows beta (P, d):
 * lik[p] = sum_i softplus(x_i . beta_p) - y_i x_i . beta_p, grad[p] = X^T (sigmoid(X beta_p) - y).
 * X (n_data, d) row-major float32; precision MGB_PREC_BF16 also needs Xbf16, the
 * (n_data, 64) bf16 zero-padded copy of X. */
size_t mgb_logreg_workspace(int64_t P, int64_t n_data, int32_t d, int precision);
int mgb_logreg_potential_grad(const float *X_dev, const float *y_dev, int64_t n_data, int32_t d, const float *beta_dev,
                              int64_t P, float *lik_dev, float *grad_dev, int precision, const void *Xbf16_dev,
                              void *ws_dev, size_t ws_bytes, void *stream);

typedef struct {
  int32_t B, N, d;              /* posteriors, particles per posterior, dimension */
  int32_t mcmc_steps;           /* MALA moves per temperature */
  float stepsize;               /* Underdamped stepsize */
  float prior_scale;            /* s */
  float ess_threshold_retain;   /* target ESS fraction of the temperature bisection */
  float ess_threshold_resample; /* resample when ess <= this * N */
  float bisection_tol;
  int32_t max_bisection_iter;
  float max_temperature;
  int32_t max_iter;             /* SMC iterations (also the history length - 1) */
  int32_t precision;            /* MGB_PREC_FP32 or MGB_PREC_BF16 (potential on the tensor cores) */
  int32_t move;                 /* MGB_MOVE_UNDERDAMPED or MGB_MOVE_RANDOM_WALK */
  int32_t leapfrog_steps;       /* Underdamped leapfrog steps (0: 1) */
  float friction;               /* Underdamped friction (<= 0 or infinite: fresh momenta, MALA / HMC) */
  float prior_sample_scale;     /* prior draws prior_sample_scale * normal (0: prior_scale) */
  int32_t n_schedule;           /* > 0: temperatures from schedule_dev; max_iter = n_schedule */
  const float *schedule_dev;    /* (n_schedule) device */
  int32_t likelihood;           /* MGB_LIK_LOGISTIC or MGB_LIK_GAUSSIAN */
  const float *gauss_mean_dev;  /* (d) device, MGB_LIK_GAUSSIAN */
  const float *gauss_prec_sqrt_dev; /* (d, d) row-major device, MGB_LIK_GAUSSIAN */
  int32_t resampling;           /* MGB_RESAMPLE_SYSTEMATIC (O(N), default) or MGB_RESAMPLE_CATEGORICAL
                                   (the reference's random.categorical, smc.py:61-71: O(N^2) Gumbel-max
                                   draws, N <= 46340) */
} mgb_smc_logreg_config;

/* device pointers into the sampler's workspace */
typedef struct {
  float *value;                 /* (B N, d) particles */
  float *log_weight;            /* (B N) */
  float *likelihood_potential;  /* (B N) */
  float *temperature;           /* (B) */
  float *ess;                   /* (B) */
  double *log_norm_constant;    /* (B) */
  int32_t *iter;                /* (B) iterations done */
  int32_t *active;              /* (B) 1 while the posterior has not terminated */
  float *hist_temperature;      /* (B, hist_len) entry 0 = after startup, i = after iteration i */
  double *hist_log_norm_constant;
  float *hist_ess;
  float *hist_alpha;            /* mean acceptance probability of the iteration's moves */
  int32_t *hist_resampled;
  int32_t hist_len;
} mgb_smc_views;

size_t mgb_smc_logreg_workspace(const mgb_smc_logreg_config *cfg, int64_t n_data);
int mgb_smc_logreg_views(const mgb_smc_logreg_config *cfg, void *ws_dev, mgb_smc_views *out);
/* startup (prior draws, potentials, first temperature); keys_dev (B, 2) */
int mgb_smc_logreg_init(const mgb_smc_logreg_config *cfg, const float *X_dev, const float *y_dev,
                        const void *Xbf16_dev, int64_t n_data, const uint32_t *keys_dev, void *ws_dev,
                        size_t ws_bytes, void *stream);
/* d log Z / d prior_scale of each posterior (out_dev (B) doubles) from the
 * current weighted particles by the Fisher identity,
 * E_post[|beta|^2 / s^3 - d / s]; meaningful once the posterior is reached
 * (temperature 1). */
int mgb_smc_logreg_prior_scale_grad(const mgb_smc_logreg_config *cfg, void *ws_dev, double *out_dev, void *stream);
/* one SMC iteration of every active posterior (the caller loops while any
 * views.active[b] is set) */
int mgb_smc_logreg_step(const mgb_smc_logreg_config *cfg, const float *X_dev, const float *y_dev,
                        const void *Xbf16_dev, int64_t n_data, void *ws_dev, size_t ws_bytes, void *stream);

/* ---------------------------------------------- Kalman filter and smoother
 * run_kalman_filter_for_marginals / run_kalman_smoother_for_marginals
 * (mocat/src/ssm/linear_gaussian/kalman.py:16-57, 60-104) for B observation sequences of the
 * same time-homogeneous model at once, float32 as the reference computes:
 *   t = 0: K = C0 H' (H C0 H' + R)^-1, mean = m0 + K (y_0 - H m0), cov = C0 - K H C0, where C0 is
 *          the initial covariance square root (the reference uses it as the covariance at t = 0);
 *   t > 0: predict F mean, F cov F' + Q, then the same update;
 *   smoother: A = F P_t F' + Q, G = P_t F' A^-1, mean_t += G (mean_{t+1}^s - F mean_t),
 *             cov_t += G (cov_{t+1}^s - A) G'.
 * Matrices are host pointers, row-major float32: F, Q (d x d), H (dy x d), R (dy x dy), m0 (d),
 * C0 (d x d).  y (B, T, dy); means (B, T, d); covs (B, T, d, d).  loglik (B doubles, may be NULL):
 * the prediction-error log-likelihood sum_t log N(y_t; H mean_{t|t-1}, S_t) (new).
 * lag_ones (B, T-1, d, d; may be NULL) replaces run_kalman_smoother_for_marginals_and_lag_ones
 * (kalman.py:60-94): <mean_t^f, mean_{t+1}^s> + G (cov_{t+1}^s + <mean_{t+1}^s - mean_{t+1}^f,
 * mean_{t+1}^s>), the reference's 1-D `@` products being dot products.
 * (d, dy): the compiled pairs of mgb_lg_model, or any other d, dy <= 32 (a run-time-dimension
 * instance of the same kernels). */
typedef struct {
  int32_t d, dy;
  const float *F, *Q, *H, *R, *m0, *C0;
} mgb_kalman_model;
int mgb_kalman_filter(const mgb_kalman_model *model_host, int64_t B, int64_t T, const float *y_dev,
                      float *means_dev, float *covs_dev, double *loglik_dev, void *stream);
int mgb_kalman_smoother(const mgb_kalman_model *model_host, int64_t B, int64_t T, const float *filter_means_dev,
                        const float *filter_covs_dev, float *means_dev, float *covs_dev, float *lag_ones_dev,
                        void *stream);

/* ------------------------------------------------ ABC-SMC (likelihood-free)
 * MetropolisedABCSMCSampler (mocat/src/abc/smc.py:101-245) with RandomWalkABC moves and the
 * Metropolis correction (mocat/src/abc/mcmc.py:59-103, mocat/src/mcmc/metropolis.py:48-70),
 * driven as mocat.run (mocat/src/sample.py:110-148), on the ABC LinearGaussian scenario
 * (mocat/src/abc/scenarios/linear_gaussian.py): prior N(m0, C0 C0^T), simulated data
 * H x + L eps, distance |sim - data|_2 (mocat/src/abc/abc.py:36-39).  B posteriors with keys
 * (B, 2), N particles each.
 *   weights 0 / -inf (distance <= threshold), ESS = exp(log #alive);
 *   thresholds: schedule[iter] (index clamped) or jnp.quantile(distances,
 *     ess_threshold_retain ess / N) with linear interpolation;
 *   resampling when ess < ess_threshold_resample N: systematic (the reference: random.categorical);
 *   moves: mcmc_steps random-walk proposals x + sqrt(stepsize) eps per alive particle, stepsize
 *     the per-dimension variance (ddof 1) of the particles / d * 2.38^2 after every iteration
 *     (adapt_stepsize = 1, the reference's default) or fixed;
 *   termination: mean acceptance of the moves <= termination_alpha, or iter >= max_iter.
 * Supported (d, dy): (1,1) (2,1) (2,2) (3,2) (3,3) (5,5) (10,10); 2 <= N <= MGB_ABC_MAX_N. */
#define MGB_ABC_MAX_N 65536
typedef struct {
  int32_t d, dy;
  const float *m0;   /* (d) prior_mean (host) */
  const float *C0;   /* d x d prior_covariance_sqrt */
  const float *P0;   /* d x d prior_precision_sqrt */
  float c0;          /* (d log 2 pi - log prior_precision_det) / 2 */
  const float *H;    /* dy x d likelihood_matrix */
  const float *L;    /* dy x dy likelihood_covariance_sqrt */
  const float *data; /* (dy) observed data */
} mgb_abc_lg_model;

typedef struct {
  int32_t B, N, mcmc_steps, max_iter;
  float ess_threshold_retain, ess_threshold_resample, termination_alpha;
  int32_t adapt_stepsize; /* 1: variance-scaled stepsize (default sampler); 0: `stepsize` fixed */
  float stepsize;
  int32_t n_schedule;     /* 0: adaptive thresholds */
  const float *schedule;  /* (n_schedule) thresholds (host); max_iter = n_schedule in the reference */
} mgb_abc_smc_config;

/* device pointers into the sampler's workspace */
typedef struct {
  float *value;           /* (B N, d) particle-major */
  float *distance;        /* (B N) */
  float *log_weight;      /* (B N) 0 or -inf */
  float *prior_potential; /* (B N) */
  float *alpha;           /* (B N) each particle's mean acceptance over its last moves */
  float *stepsize;        /* (B, d) */
  float *threshold;       /* (B) */
  float *ess;             /* (B) */
  float *alpha_mean;      /* (B) */
  int32_t *iter;          /* (B) */
  int32_t *active;        /* (B) 1 while the posterior has not terminated */
  float *hist_threshold;  /* (B, hist_len) entry 0 = after startup, i = after iteration i */
  float *hist_ess;
  float *hist_alpha;
  int32_t *hist_resampled;
  int32_t hist_len;
} mgb_abc_views;

size_t mgb_abc_smc_workspace(const mgb_abc_smc_config *cfg, int32_t d);
int mgb_abc_smc_views(const mgb_abc_smc_config *cfg, int32_t d, void *ws_dev, mgb_abc_views *out);
/* startup (ABCSMCSampler.startup, abc/smc.py:44-85 and :129-149): prior draws, potentials,
 * simulations, distances, first threshold; the schedule is copied into the workspace */
int mgb_abc_smc_init(const mgb_abc_smc_config *cfg, const mgb_abc_lg_model *model_host, const uint32_t *keys_dev,
                     void *ws_dev, size_t ws_bytes, void *stream);
/* one SMCSampler.update of every active posterior (the caller loops while any views.active[b]) */
int mgb_abc_smc_step(const mgb_abc_smc_config *cfg, const mgb_abc_lg_model *model_host, void *ws_dev,
                     size_t ws_bytes, void *stream);

/* g-and-k scenarios (mocat/src/abc/scenarios/gk.py:81-175: GKTransformedUniformPrior, d = 4, and
 * GKOnlyATransformedUniformPrior, d = 1) with the thinned-order-statistics summary of
 * tests/test_abc_gk.py (sorted draws at ranks floor(j n_unsummarised / n_summary)) under the
 * same sampler and config.  prior N(0, I); parameters constrained by prior_min + Phi(x)
 * (prior_max - prior_min); a simulation draws n_unsummarised uniforms in [buffer, 1 - buffer],
 * z = Phi^-1(u), v = A + B (1 + c (1 - e^{-g z}) / (1 + e^{-g z})) z (1 + z^2)^k (A-only: B = 1,
 * g = 2 and the exponent c, as the reference writes it).  Phi uses the Numerical Recipes erfc
 * fit and Phi^-1 the library's erfinv, so values are not XLA's bit for bit.
 * mgb_abc_gk_simulate: summaries (P, n_summary) and/or distances (P) of parameter rows x (P, d)
 * with keys (P, 2) (likelihood_sample then distance_function). */
typedef struct {
  int32_t d;               /* 4 or 1 */
  int32_t n_unsummarised;  /* draws per simulation, <= 2048 */
  int32_t n_summary;       /* thinned order statistics */
  float c;                 /* 0.8 */
  float prior_min, prior_max, buffer;  /* 0, 10, 1e-5 */
  const float *data_dev;   /* (n_summary) observed summary */
} mgb_abc_gk_model;
size_t mgb_abc_gk_workspace(const mgb_abc_smc_config *cfg, int32_t d);
int mgb_abc_gk_smc_init(const mgb_abc_smc_config *cfg, const mgb_abc_gk_model *model_host, const uint32_t *keys_dev,
                        void *ws_dev, size_t ws_bytes, void *stream);
int mgb_abc_gk_smc_step(const mgb_abc_smc_config *cfg, const mgb_abc_gk_model *model_host, void *ws_dev,
                        size_t ws_bytes, void *stream);
int mgb_abc_gk_simulate(const mgb_abc_gk_model *model_host, int64_t P, const float *x_dev, const uint32_t *keys_dev,
                        float *summary_dev, float *dist_dev, void *stream);

/* VanillaABC (mocat/src/abc/importance.py:16-118) run as mocat.run does: a chain of n prior draws
 * with sequential keys ((K, s) = split(K) for x_0, one split for its prior potential, one for its
 * simulation; then (K, k1, k2, k3) = split(K, 4) per draw), log_weight = 0 where distance <
 * threshold else -inf.  acceptance_rate >= 0 replaces the threshold by
 * jnp.quantile(distance, acceptance_rate) (clean_chain_ar); threshold_out (device, 1 float)
 * receives the threshold used.  x (n, d), pp, dist, lw (n) device outputs. */
/* RandomWalkABC run as an MCMC sampler (abc/mcmc.py:16-100 with the Metropolis correction,
 * mocat.run): B independent chains (keys_dev (B, 2)) of n states each with a fixed stepsize and
 * threshold: x' = x + sqrt(stepsize) normal, accepted with probability
 * min(1, exp(pp - pp') [dist' < threshold]).  x (B, n, d), dist, pp, alpha (B, n) device
 * outputs; one thread per chain (the chain is serial). */
int mgb_abc_mcmc_lg(const mgb_abc_lg_model *model_host, int64_t B, int64_t n, const uint32_t *keys_dev, float stepsize,
                    float threshold, float *x_dev, float *distance_dev, float *prior_potential_dev, float *alpha_dev,
                    void *stream);
/* RandomWalkABC() with the RMMetropolisDiagStepsize correction (mocat/src/abc/mcmc.py:105-140,
 * mocat/src/mcmc/metropolis.py:73-160) at the sampler's defaults: the chain starts at threshold
 * 50 and stepsize 1 per dimension, post_mean x_0, diag_post_cov = stepsize d / 2.38^2; after
 * every step, with rm = scale * iter^-neg_exp:
 *   threshold <- exp(log threshold - rm (alpha - target))
 *   r = min(rm, 1 - 1e-3); diag_post_cov <- (1 - r) diag_post_cov + r (x - post_mean)^2;
 *   post_mean <- (1 - r) post_mean + r x; stepsize <- diag_post_cov / d * 2.38^2.
 * B independent chains (keys_dev (B, 2)) of n states; x (B, n, d), alpha (B, n), threshold
 * (B, n) and stepsize (B, n, d) device outputs, each state's values after its adaptation.
 * target: the tuning target of alpha (0.1 in the reference); scale > 0: rm_stepsize_scale;
 * neg_exp >= 0: rm_stepsize_neg_exponent (2/3). */
int mgb_abc_mcmc_rm_lg(const mgb_abc_lg_model *model_host, int64_t B, int64_t n, const uint32_t *keys_dev,
                       float target, float scale, float neg_exp, float *x_dev, float *alpha_dev, float *threshold_dev,
                       float *stepsize_dev, void *stream);
/* RandomWalkABC(stepsize, threshold) chains on a g-and-k scenario (model_host->data_dev required),
 * one CTA per chain: x_0 = normal(split(key)[1], (d,)), prior potential 0.5 |x|^2, the key chain and
 * Metropolis step of mgb_abc_mcmc_lg; x (B, n, d), distance, prior_potential, alpha (B, n). */
int mgb_abc_mcmc_gk(const mgb_abc_gk_model *model_host, int64_t B, int64_t n, const uint32_t *keys_dev, float stepsize,
                    float threshold, float *x_dev, float *distance_dev, float *prior_potential_dev, float *alpha_dev,
                    void *stream);
/* the same adaptive chain on a g-and-k scenario (model_host->data_dev required), one CTA per
 * chain: x_0 = normal(split(key)[1], (d,)), prior potential 0.5 |x|^2, one g-and-k simulation
 * per step; outputs as mgb_abc_mcmc_rm_lg (the reference's TestMCMCGK / TestMCMCGKOnlyA). */
int mgb_abc_mcmc_rm_gk(const mgb_abc_gk_model *model_host, int64_t B, int64_t n, const uint32_t *keys_dev,
                       float target, float scale, float neg_exp, float *x_dev, float *alpha_dev, float *threshold_dev,
                       float *stepsize_dev, void *stream);
size_t mgb_abc_vanilla_workspace(int64_t n);
int mgb_abc_vanilla_lg(const mgb_abc_lg_model *model_host, int64_t n, const uint32_t *key_dev, float threshold,
                       float acceptance_rate, void *ws_dev, size_t ws_bytes, float *x_dev, float *prior_potential_dev,
                       float *distance_dev, float *log_weight_dev, float *threshold_out_dev, void *stream);
int mgb_abc_vanilla_gk(const mgb_abc_gk_model *model_host, int64_t n, const uint32_t *key_dev, float threshold,
                       float acceptance_rate, void *ws_dev, size_t ws_bytes, float *x_dev, float *prior_potential_dev,
                       float *distance_dev, float *log_weight_dev, float *threshold_out_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif
