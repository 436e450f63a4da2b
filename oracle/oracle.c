/*
 * ORACLE -- test infrastructure only (see oracle_rng.h).  CPU restatement of
 * mocat's particle-system step, used by tests/ as the checker and by bench.py
 * as the timed CPU baseline.  Never linked into the product library.
 *
 * What it restates (reference paths are relative to the mocat project):
 *   - run_particle_filter_for_marginals / initiate_particles:
 *       mocat/src/ssm/filtering.py:173-193, 255-324 (ESS trigger :286-292,
 *       key reuse of int_rand_key for resampling and split :291/:294,
 *       lw reset :292);
 *   - BootstrapFilter weights: filtering.py:142-170;
 *   - TimeHomogenousLinearGaussian sampling/potentials:
 *       mocat/src/ssm/linear_gaussian/linear_gaussian.py:46-51, 86-94, 118-128;
 *       gaussian_potential mocat/src/utils.py:49-105 (vectorised branch :90-104);
 *   - StochasticVolatility: mocat/src/ssm/scenarios/stochastic_volatility.py:71-102;
 *   - NonLinear1DBenchmark: mocat/src/ssm/scenarios/nonlinear1d.py:16-80;
 *   - OptimalNonLinearGaussianParticleFilter fused step:
 *       mocat/src/ssm/nonlinear_gaussian.py:198-209, 264-281;
 *   - ESS / logsumexp: mocat/src/metrics.py:69-78 (max-shifted logsumexp of
 *       jax.scipy.special.logsumexp, shift 0 when the max is not finite);
 *   - _resample via random.categorical (Gumbel-max): filtering.py:196-199.
 * New capabilities restated here with the same arithmetic as the device code:
 *   systematic and sorted-uniform multinomial resampling on 62-bit fixed-point
 *   weights (exact integer prefix sums, so ancestors do not depend on the
 *   summation order), and the log-marginal-likelihood accumulated from the
 *   filter's own log-weights.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle_rng.h"

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ RNG arrays */

void o_threefry_block(uint32_t k0, uint32_t k1, const uint32_t *c0, const uint32_t *c1,
                      int64_t n, uint32_t *r0, uint32_t *r1)
{
    for (int64_t i = 0; i < n; ++i) o_threefry2x32(k0, k1, c0[i], c1[i], &r0[i], &r1[i]);
}

void o_random_bits(const uint32_t *key, int64_t n, uint32_t *out)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) out[p] = o_bits_at(key[0], key[1], (uint64_t)n, (uint64_t)p);
}

void o_split(const uint32_t *key, int64_t num, uint32_t *out)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < num; ++i)
        o_split_at(key[0], key[1], (uint64_t)num, (uint64_t)i, &out[2 * i], &out[2 * i + 1]);
}

void o_uniform(const uint32_t *key, int64_t n, float *out)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) out[p] = o_bits_to_unit(o_bits_at(key[0], key[1], (uint64_t)n, (uint64_t)p));
}

void o_normal(const uint32_t *key, int64_t n, float *out)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) out[p] = o_bits_to_normal(o_bits_at(key[0], key[1], (uint64_t)n, (uint64_t)p));
}

void o_exponential(const uint32_t *key, int64_t n, float *out)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p)
        out[p] = o_bits_to_exponential(o_bits_at(key[0], key[1], (uint64_t)n, (uint64_t)p));
}

void o_gumbel(const uint32_t *key, int64_t n, float *out)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) out[p] = o_bits_to_gumbel(o_bits_at(key[0], key[1], (uint64_t)n, (uint64_t)p));
}

void o_math_logf(const float *x, int64_t n, float *out) { for (int64_t i = 0; i < n; ++i) out[i] = o_logf(x[i]); }
void o_math_expf(const float *x, int64_t n, float *out) { for (int64_t i = 0; i < n; ++i) out[i] = o_expf(x[i]); }
void o_math_erfinvf(const float *x, int64_t n, float *out) { for (int64_t i = 0; i < n; ++i) out[i] = o_erfinvf(x[i]); }

/* ------------------------------------------------------------- LSE and ESS */

/* out = {max, lse(lw), lse(2 lw), ess}; metrics.py:69-78 in float64. */
void o_lse_ess(const float *lw, int64_t n, double *out)
{
    double m = -INFINITY;
    int nan = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (lw[i] != lw[i]) nan = 1;
        else if ((double)lw[i] > m) m = lw[i];
    }
    if (nan) { out[0] = out[1] = out[2] = out[3] = NAN; return; }
    double sh = isfinite(m) ? m : 0.0;
    double s1 = 0.0, s2 = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s1, s2)
    for (int64_t i = 0; i < n; ++i) {
        double e = exp((double)lw[i] - sh);
        s1 += e;
        s2 += e * e;
    }
    double lse = log(s1) + sh, lse2 = log(s2) + 2.0 * sh;
    out[0] = m;
    out[1] = lse;
    out[2] = lse2;
    out[3] = exp(2.0 * lse - lse2);
}

/* ------------------------------------------------------ fixed-point weights */

int o_ceil_log2(uint64_t n)
{
    int b = 0;
    while (b < 63 && ((uint64_t)1 << b) < n) ++b;
    return b;
}

/* Shift used to quantise normalised weights exp(lw - max) in (0, 1] so that
 * the total of n of them stays below 2^62. */
int o_weight_shift(int64_t n) { return 61 - o_ceil_log2((uint64_t)n); }

/* q_i = trunc(expf(lw_i - max) * 2^S); returns 0 when the weights are
 * degenerate (a NaN or +inf log-weight, or every weight zero). */
int o_quantise(const float *lw, int64_t n, uint64_t *q)
{
    float m = -INFINITY;
    for (int64_t i = 0; i < n; ++i) {
        if (lw[i] != lw[i] || lw[i] == INFINITY) return 0;
        if (lw[i] > m) m = lw[i];
    }
    if (m == -INFINITY) return 0;
    float scale = ldexpf(1.0f, o_weight_shift(n));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float e = o_expf(lw[i] - m);
        q[i] = (uint64_t)(e * scale);
    }
    uint64_t tot = 0;
    for (int64_t i = 0; i < n; ++i) tot += q[i];
    return tot > 0;
}

/* a_k = #{ i : C_i * den <= num_k * Q }, C inclusive prefix of q, num_k
 * non-decreasing.  Two-pointer merge. */
static void o_merge_search(const uint64_t *C, int64_t n, uint64_t Q, const uint64_t *num, uint64_t den,
                           int64_t nout, int32_t *anc)
{
    int64_t i = 0;
    for (int64_t k = 0; k < nout; ++k) {
        u128 rhs = (u128)num[k] * Q;
        while (i < n && (u128)C[i] * den <= rhs) ++i;
        anc[k] = (int32_t)(i < n ? i : n - 1);
    }
}

/* Systematic resampling: u = m 2^-23 (m = bits >> 9 of the step key);
 * threshold numerators k 2^23 + m over denominator n 2^23. */
int o_resample_systematic(const float *lw, int64_t n, uint32_t m23, int32_t *anc)
{
    uint64_t *q = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    uint64_t *num = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    int ok = o_quantise(lw, n, q);
    if (ok) {
        for (int64_t i = 1; i < n; ++i) q[i] += q[i - 1];
        for (int64_t k = 0; k < n; ++k) num[k] = ((uint64_t)k << 23) + m23;
        o_merge_search(q, n, q[n - 1], num, (uint64_t)n << 23, n, anc);
    } else {
        for (int64_t k = 0; k < n; ++k) anc[k] = 0;
    }
    free(q);
    free(num);
    return ok;
}

/* Multinomial resampling by inverse CDF at sorted uniforms built from n+1
 * exponential spacings E = exponential(key, (n+1,)), quantised by 2^SE. */
int o_exp_shift(int64_t n) { return 56 - o_ceil_log2((uint64_t)n + 1); }

int o_resample_multinomial(const float *lw, int64_t n, const uint32_t *key, int32_t *anc)
{
    uint64_t *q = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    uint64_t *S = (uint64_t *)calloc((size_t)(n + 1), sizeof(uint64_t));
    int ok = o_quantise(lw, n, q);
    if (ok) {
        float sc = ldexpf(1.0f, o_exp_shift(n));
        uint64_t acc = 0;
        for (int64_t j = 0; j <= n; ++j) {
            float E = o_bits_to_exponential(o_bits_at(key[0], key[1], (uint64_t)n + 1, (uint64_t)j));
            acc += (uint64_t)(E * sc);
            S[j] = acc;
        }
        for (int64_t i = 1; i < n; ++i) q[i] += q[i - 1];
        if (S[n] == 0) ok = 0;
        else o_merge_search(q, n, q[n - 1], S, S[n], n, anc);
    }
    if (!ok) for (int64_t k = 0; k < n; ++k) anc[k] = 0;
    free(q);
    free(S);
    return ok;
}

/* random.categorical(key, lw, shape=(nout,)) = argmax_i(gumbel[k, i] + lw_i),
 * gumbel drawn with shape (nout, n) (first maximum wins, as jnp.argmax;
 * NaN entries are skipped and an all-NaN row gives index 0). */
void o_resample_gumbel(const float *lw, int64_t n, int64_t nout, const uint32_t *key, int32_t *anc)
{
    uint64_t tot = (uint64_t)n * (uint64_t)nout;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nout; ++k) {
        float best = -INFINITY;
        int32_t bi = 0;
        int have = 0;
        for (int64_t i = 0; i < n; ++i) {
            float g = o_bits_to_gumbel(o_bits_at(key[0], key[1], tot, (uint64_t)k * (uint64_t)n + (uint64_t)i));
            float v = g + lw[i];
            if (v == v && (!have || v > best)) { best = v; bi = (int32_t)i; have = 1; }
        }
        anc[k] = bi;
    }
}

/* --------------------------------------------------- linear-Gaussian model */

typedef struct {
    int d, dy;
    const float *F;   /* d x d transition_matrix */
    const float *Lq;  /* d x d transition_covariance_sqrt */
    const float *H;   /* dy x d likelihood_matrix */
    const float *P;   /* dy x dy likelihood_precision_sqrt */
    float c;          /* (dy log 2pi - log likelihood_precision_det) / 2 */
    const float *C0;  /* d x d initial_covariance_sqrt */
    const float *m0;  /* d initial_mean */
} o_lg_model;

/* likelihood_potential(x, y) = 0.5 |(y - H x) @ P|^2 + c  (linear_gaussian.py:118-128) */
static inline float o_lg_potential(const o_lg_model *md, const float *x, const float *y)
{
    float diff[64];
    for (int j = 0; j < md->dy; ++j) {
        const float *h = md->H + j * md->d;
        float hx = h[0] * x[0];
        for (int k = 1; k < md->d; ++k) hx = fmaf(h[k], x[k], hx);
        diff[j] = y[j] - hx;
    }
    float quad = 0.0f;
    for (int k = 0; k < md->dy; ++k) {
        float v = diff[0] * md->P[k];
        for (int j = 1; j < md->dy; ++j) v = fmaf(diff[j], md->P[j * md->dy + k], v);
        quad = k == 0 ? v * v : fmaf(v, v, quad);
    }
    return 0.5f * quad + md->c;
}

/* normal(key, (d,)) into e */
static inline void o_normal_vec(uint32_t k0, uint32_t k1, int d, float *e)
{
    for (int j = 0; j < d; ++j) e[j] = o_bits_to_normal(o_bits_at(k0, k1, (uint64_t)d, (uint64_t)j));
}

/* initiate_particles with TimeHomogenousLinearGaussian.initial_sample:
 * x_i = C0 @ normal(split(key, n)[i], (d,)) + m0; lw_i = -potential(x_i, y0).
 * x is particle-major (n, d). */
void o_lg_init(const o_lg_model *md, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw)
{
    const int d = md->d;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t a0, a1;
        float e[64];
        o_split_at(key[0], key[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
        o_normal_vec(a0, a1, d, e);
        float *xi = x + i * d;
        for (int r = 0; r < d; ++r) {
            const float *c = md->C0 + r * d;
            float v = c[0] * e[0];
            for (int k = 1; k < d; ++k) v = fmaf(c[k], e[k], v);
            xi[r] = v + md->m0[r];
        }
        lw[i] = y0 ? -o_lg_potential(md, xi, y0) : 0.0f;
    }
}

/* Bootstrap propagate + weight for one step (filtering.py:294-303):
 * key_i = split(k_t, n)[i]; x_new = F x_src + Lq normal(key_i, (d,));
 * lw_new = lw_res - potential(x_new, y_t).  anc may be NULL (no resampling),
 * lw_prev NULL means lw_res = 0. */
void o_lg_propagate(const o_lg_model *md, int64_t n, const uint32_t *kt, const float *y, const float *x_prev,
                    const int32_t *anc, const float *lw_prev, float *x_new, float *lw_new)
{
    const int d = md->d;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t a0, a1;
        float e[64];
        o_split_at(kt[0], kt[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
        o_normal_vec(a0, a1, d, e);
        const float *xs = x_prev + (int64_t)(anc ? anc[i] : i) * d;
        float *xn = x_new + i * d;
        for (int r = 0; r < d; ++r) {
            const float *f = md->F + r * d;
            const float *l = md->Lq + r * d;
            float fx = f[0] * xs[0];
            for (int k = 1; k < d; ++k) fx = fmaf(f[k], xs[k], fx);
            float le = l[0] * e[0];
            for (int k = 1; k < d; ++k) le = fmaf(l[k], e[k], le);
            xn[r] = fx + le;
        }
        float lres = lw_prev ? lw_prev[i] : 0.0f;
        lw_new[i] = lres - o_lg_potential(md, xn, y);
    }
}

/* Whole filter (filtering.py:255-324) with resampling scheme
 * 0 = systematic, 1 = multinomial (sorted uniforms), 2 = categorical (Gumbel-max).
 * Outputs: logZ (log-marginal-likelihood built from the log-weights),
 * ess[T], resampled[T] (resampled[t] = 1 when step t started with a resample),
 * optional histories x_hist (T, n, d) and lw_hist (T, n) (NULL to skip). */
typedef struct o_score_ctx o_score_ctx;
static double o_lg_run_impl(const o_lg_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                            float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out,
                            float *x_hist, float *lw_hist, int32_t *anc_hist, o_score_ctx *sc);

double o_lg_run(const o_lg_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out,
                float *x_hist, float *lw_hist)
{
    return o_lg_run_impl(md, n, T, key, y, ess_threshold, scheme, ess_out, resampled_out, x_hist, lw_hist, NULL, NULL);
}

/* o_lg_run that also records the ancestors: anc_hist (T, n), row t written
 * when step t resampled (the rows of the other steps are left as they are). */
double o_lg_run_tape(const o_lg_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                     float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out, int32_t *anc_hist)
{
    return o_lg_run_impl(md, n, T, key, y, ess_threshold, scheme, ess_out, resampled_out, NULL, NULL, anc_hist, NULL);
}

/* Key schedule of run_particle_filter_for_marginals (filtering.py:267-278):
 * out[0..1] = split(key)[1] (the initial draw), out[2t..2t+1] = split(split(key)[0], T-1)[t-1]. */
void o_lg_step_keys(const uint32_t *key, int64_t T, uint32_t *out)
{
    uint32_t keys2[4];
    o_split(key, 2, keys2);
    out[0] = keys2[2];
    out[1] = keys2[3];
    if (T > 1) o_split(keys2, T - 1, out + 2);
}

/* eps (n, d): eps[i] = normal(split(k, n)[i], (d,)), the bootstrap draws of one step */
void o_lg_normals(const uint32_t *kt, int64_t n, int d, float *e)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t a0, a1;
        o_split_at(kt[0], kt[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
        o_normal_vec(a0, a1, d, e + i * d);
    }
}

/* ------------------------------------- score by Fisher's identity (PaRIS)
 * d log p(y_{0:T-1}) / d theta for theta = (F, log q, log r) of a model with
 * H = I, Lq = diag(sqrt q), P = diag(1 / sqrt r), by Fisher's identity
 *   score = E[ sum_t h_t(x_{t-1}, x_t) + sum_t g_t(x_t) | y ],
 *   h_t: dF_kl = e_k x_{t-1,l} / q_k,  dlog q_k = e_k^2 / (2 q_k) - 1/2  (e = x_t - F x_{t-1}),
 *   g_t: dlog r_k = (y_k - x_k)^2 / (2 r_k) - 1/2,
 * estimated along the bootstrap filter of o_lg_run by PaRIS (Olsson and
 * Westerborn, Bernoulli 23(3), 2017): every particle carries the statistic
 *   tau_t^i = (1/K) sum_k [tau_{t-1}^{J_k} + h_t(x_{t-1}^{J_k}, x_t^i)] + g_t(x_t^i),
 * and the estimate is sum_i W_{T-1}^i tau_{T-1}^i.  The K backward draws J_k
 * follow Dau and Chopin ("On backward smoothing algorithms", Ann. Statist.
 * 51(5), 2023): J_1 is the particle's own ancestor, and each further draw
 * continues an independent-Metropolis chain over the step's source
 * population m = 0..n-1 (the resampled particles x_{t-1}^{a_m}, or all
 * x_{t-1}^m with their weights when step t did not resample), target
 * exp(lb_m) f(x_t^i | x_{t-1}^{src(m)}) with lb = 0 (resampled) or lw_{t-1},
 * proposal uniform over m, L proposals per draw.  The random numbers of
 * proposal s of particle i at step t: (w0, w1) = threefry2x32(skey, (i, (t << 12) | s)),
 * m' = (w0 * n) >> 32, E = exponential(w1); accept when (lf' - lf) + E > 0.
 * Every float operation is written out in the order the GPU kernel uses. */
struct o_score_ctx {
    int K, L;
    uint32_t skey[2];
    float iq[64], half_iq[64], half_ir[64];
    int P, TS;
    float *tau_a, *tau_b;   /* (n, TS) */
    float *mu;              /* (n, d + 1): F x_src, lb */
    int32_t *draws;         /* (T, n, K) or NULL */
    float *lw_last;         /* (n): the filter's final log-weights */
};

static inline float o_score_lf(const float *xi, const float *mu, const float *iq, int d)
{
    float s2 = 0.0f;
    for (int r = 0; r < d; ++r) {
        float dr = xi[r] - mu[r];
        s2 = fmaf(dr * dr, iq[r], s2);
    }
    return mu[d] - 0.5f * s2;
}

static void o_score_init(o_score_ctx *sc, const o_lg_model *md, int64_t n, const float *x, const float *y0)
{
    const int d = md->d;
    for (int64_t i = 0; i < n; ++i) {
        float *to = sc->tau_a + i * sc->TS;
        for (int q = 0; q < sc->TS; ++q) to[q] = 0.0f;
        for (int r = 0; r < d; ++r) {
            float dr = y0[r] - x[i * d + r];
            to[d * d + d + r] = dr * dr * sc->half_ir[r] - 0.5f;
        }
    }
}

static void o_score_step(o_score_ctx *sc, const o_lg_model *md, int64_t n, int64_t t, const float *xprev,
                         const float *xnew, const int32_t *anc, const float *lw_prev, const float *yt)
{
    const int d = md->d, K = sc->K, L = sc->L, TS = sc->TS, MS = d + 1;
    float *mu = sc->mu;
#pragma omp parallel for schedule(static)
    for (int64_t m = 0; m < n; ++m) {
        const float *xs = xprev + (int64_t)(anc ? anc[m] : m) * d;
        for (int r = 0; r < d; ++r) {
            const float *f = md->F + r * d;
            float fx = f[0] * xs[0];
            for (int k = 1; k < d; ++k) fx = fmaf(f[k], xs[k], fx);
            mu[m * MS + r] = fx;
        }
        mu[m * MS + d] = anc ? 0.0f : lw_prev[m];
    }
    const float invK = (float)(1.0 / K);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const float *xi = xnew + i * d;
        int64_t mk[4], jk[4];
        mk[0] = i;
        int64_t cur = i;
        float lcur = o_score_lf(xi, mu + i * MS, sc->iq, d);
        for (int k = 1; k < K; ++k) {
            for (int l = 0; l < L; ++l) {
                uint32_t w0, w1;
                o_threefry2x32(sc->skey[0], sc->skey[1], (uint32_t)i, ((uint32_t)t << 12) | (uint32_t)((k - 1) * L + l),
                               &w0, &w1);
                const int64_t prop = (int64_t)(((uint64_t)w0 * (uint64_t)n) >> 32);
                const float E = o_bits_to_exponential(w1);
                const float lp = o_score_lf(xi, mu + prop * MS, sc->iq, d);
                if ((lp - lcur) + E > 0.0f) { cur = prop; lcur = lp; }
            }
            mk[k] = cur;
        }
        float e[4][64], v[4][64];
        const float *xp[4], *tp[4];
        for (int k = 0; k < K; ++k) {
            jk[k] = anc ? anc[mk[k]] : mk[k];
            xp[k] = xprev + jk[k] * d;
            tp[k] = sc->tau_a + jk[k] * TS;
            for (int r = 0; r < d; ++r) {
                e[k][r] = xi[r] - mu[mk[k] * MS + r];
                v[k][r] = e[k][r] * sc->iq[r];
            }
            if (sc->draws) sc->draws[(t * n + i) * K + k] = (int32_t)jk[k];
        }
        float *to = sc->tau_b + i * TS;
        for (int q = 0; q < TS; ++q) {
            float acc = 0.0f, out;
            if (q < d * d) {
                const int r = q / d, c = q % d;
                for (int k = 0; k < K; ++k) { acc = acc + tp[k][q]; acc = acc + v[k][r] * xp[k][c]; }
                out = acc * invK;
            } else if (q < d * d + d) {
                const int r = q - d * d;
                for (int k = 0; k < K; ++k) { acc = acc + tp[k][q]; acc = acc + (e[k][r] * e[k][r] * sc->half_iq[r] - 0.5f); }
                out = acc * invK;
            } else if (q < sc->P) {
                const int r = q - d * d - d;
                for (int k = 0; k < K; ++k) acc = acc + tp[k][q];
                float dr = yt[r] - xi[r];
                out = acc * invK + (dr * dr * sc->half_ir[r] - 0.5f);
            } else {
                out = 0.0f;
            }
            to[q] = out;
        }
    }
    float *tmp = sc->tau_a; sc->tau_a = sc->tau_b; sc->tau_b = tmp;
}

/* The score estimate of the filter run o_lg_run(md, n, T, key, y, ...) would
 * make: grad (d*d + 2d doubles) = sum_i W^i tau^i (float64 sum in particle
 * order) with W = exp(lw_{T-1} - LSE), plus log Z, ess, resampled as o_lg_run;
 * draws (T, n, K) (row 0 untouched) may be NULL.  K in 1..4, (K-1) L < 4096. */
double o_lg_score(const o_lg_model *md, int64_t n, int64_t T, const uint32_t *key, const uint32_t *skey,
                  const float *y, float ess_threshold, int scheme, int K, int L, double *grad, float *ess_out,
                  int32_t *resampled_out, int32_t *draws)
{
    const int d = md->d;
    o_score_ctx sc;
    sc.K = K; sc.L = L;
    sc.skey[0] = skey[0]; sc.skey[1] = skey[1];
    for (int r = 0; r < d; ++r) {
        const double q = (double)md->Lq[r * d + r] * (double)md->Lq[r * d + r];
        const double pr = (double)md->P[r * d + r];
        sc.iq[r] = (float)(1.0 / q);
        sc.half_iq[r] = (float)(0.5 / q);
        sc.half_ir[r] = (float)(0.5 * pr * pr);
    }
    sc.P = d * d + 2 * d;
    sc.TS = (sc.P + 3) / 4 * 4;
    sc.tau_a = (float *)malloc(sizeof(float) * (size_t)n * sc.TS);
    sc.tau_b = (float *)malloc(sizeof(float) * (size_t)n * sc.TS);
    sc.mu = (float *)malloc(sizeof(float) * (size_t)n * (d + 1));
    sc.draws = draws;
    float *lw_last = (float *)malloc(sizeof(float) * (size_t)n);
    sc.lw_last = lw_last;
    double logZ = o_lg_run_impl(md, n, T, key, y, ess_threshold, scheme, ess_out, resampled_out, NULL, NULL, NULL, &sc);
    double st[4];
    o_lse_ess(lw_last, n, st);
    for (int q = 0; q < sc.P; ++q) grad[q] = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double w = exp((double)lw_last[i] - st[1]);
        for (int q = 0; q < sc.P; ++q) grad[q] += w * (double)sc.tau_a[i * sc.TS + q];
    }
    free(sc.tau_a); free(sc.tau_b); free(sc.mu); free(lw_last);
    return logZ;
}

static double o_lg_run_impl(const o_lg_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                            float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out,
                            float *x_hist, float *lw_hist, int32_t *anc_hist, o_score_ctx *sc)
{
    const int d = md->d, dy = md->dy;
    float *xa = (float *)malloc(sizeof(float) * (size_t)(n * d));
    float *xb = (float *)malloc(sizeof(float) * (size_t)(n * d));
    float *la = (float *)malloc(sizeof(float) * (size_t)n);
    float *lb = (float *)malloc(sizeof(float) * (size_t)n);
    int32_t *anc = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint32_t keys2[4], rk[2], sk[2];
    o_split(key, 2, keys2);
    rk[0] = keys2[0]; rk[1] = keys2[1];
    sk[0] = keys2[2]; sk[1] = keys2[3];

    o_lg_init(md, n, sk, y, xa, la);
    if (sc) o_score_init(sc, md, n, xa, y);
    double st[4];
    o_lse_ess(la, n, st);
    double logn = log((double)n);
    double logZ = st[1] - logn;
    double lse_prev = st[1];
    float ess_prev = (float)st[3];
    ess_out[0] = ess_prev;
    resampled_out[0] = 0;
    if (x_hist) memcpy(x_hist, xa, sizeof(float) * (size_t)(n * d));
    if (lw_hist) memcpy(lw_hist, la, sizeof(float) * (size_t)n);

    uint32_t *tkeys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)(T > 1 ? T - 1 : 1));
    if (T > 1) o_split(rk, T - 1, tkeys);
    for (int64_t t = 1; t < T; ++t) {
        const uint32_t *kt = tkeys + 2 * (t - 1);
        int res = ess_prev < ess_threshold * (float)n;
        if (res) {
            if (scheme == 0) {
                uint32_t b = o_bits_at(kt[0], kt[1], 1, 0);
                o_resample_systematic(la, n, b >> 9, anc);
            } else if (scheme == 1) {
                o_resample_multinomial(la, n, kt, anc);
            } else {
                o_resample_gumbel(la, n, n, kt, anc);
            }
        }
        if (res && anc_hist) memcpy(anc_hist + t * n, anc, sizeof(int32_t) * (size_t)n);
        o_lg_propagate(md, n, kt, y + t * dy, xa, res ? anc : NULL, res ? NULL : la, xb, lb);
        if (sc) o_score_step(sc, md, n, t, xa, xb, res ? anc : NULL, la, y + t * dy);
        o_lse_ess(lb, n, st);
        logZ += st[1] - (res ? logn : lse_prev);
        lse_prev = st[1];
        ess_prev = (float)st[3];
        ess_out[t] = ess_prev;
        resampled_out[t] = res;
        if (x_hist) memcpy(x_hist + t * n * d, xb, sizeof(float) * (size_t)(n * d));
        if (lw_hist) memcpy(lw_hist + t * n, lb, sizeof(float) * (size_t)n);
        float *tp = xa; xa = xb; xb = tp;
        tp = la; la = lb; lb = tp;
    }
    if (sc) memcpy(sc->lw_last, la, sizeof(float) * (size_t)n);
    free(tkeys);
    free(xa); free(xb); free(la); free(lb); free(anc);
    return logZ;
}

/* ------------------------------------------ optimal proposal (A6, linear f) */

typedef struct {
    int d, dy;
    const float *F;    /* transition_function x -> F x */
    const float *H;    /* dy x d */
    const float *K;    /* d x dy proposal_kalman_gain */
    const float *S;    /* d x d proposal_covariance_sqrt */
    const float *W;    /* dy x dy weight_precision_sqrt */
    float cw;          /* (dy log 2pi - log weight_precision_det) / 2 */
    const float *K0;   /* d x dy initial_kalman_gain */
    const float *C0c;  /* d x d initial_conditioned_covariance_sqrt */
    const float *m0;   /* d */
} o_opt_model;

/* initial_sample (nonlinear_gaussian.py:198-209): mean + normal(keys[0], (n, d)) @ C0c
 * with keys = split(key, n); initial weights are zero. */
void o_opt_init(const o_opt_model *md, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw)
{
    const int d = md->d, dy = md->dy;
    uint32_t k0, k1;
    o_split_at(key[0], key[1], (uint64_t)n, 0, &k0, &k1);
    float mean[64], innov[64];
    for (int j = 0; j < dy; ++j) {
        float hm = md->H[j * d] * md->m0[0];
        for (int k = 1; k < d; ++k) hm = fmaf(md->H[j * d + k], md->m0[k], hm);
        innov[j] = y0[j] - hm;
    }
    for (int r = 0; r < d; ++r) {
        float g = md->K0[r * dy] * innov[0];
        for (int j = 1; j < dy; ++j) g = fmaf(md->K0[r * dy + j], innov[j], g);
        mean[r] = md->m0[r] + g;
    }
    uint64_t tot = (uint64_t)n * (uint64_t)d;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float e[64];
        for (int j = 0; j < d; ++j) e[j] = o_bits_to_normal(o_bits_at(k0, k1, tot, (uint64_t)i * d + j));
        for (int r = 0; r < d; ++r) {
            float v = e[0] * md->C0c[r];
            for (int k = 1; k < d; ++k) v = fmaf(e[k], md->C0c[k * d + r], v);
            x[i * d + r] = mean[r] + v;
        }
        lw[i] = 0.0f;
    }
}

/* fused vectorised step (nonlinear_gaussian.py:264-281): noise from keys[0] of
 * split(k_t, n) with shape (n, d). */
void o_opt_propagate(const o_opt_model *md, int64_t n, const uint32_t *kt, const float *y, const float *x_prev,
                     const int32_t *anc, const float *lw_prev, float *x_new, float *lw_new)
{
    const int d = md->d, dy = md->dy;
    uint32_t k0, k1;
    o_split_at(kt[0], kt[1], (uint64_t)n, 0, &k0, &k1);
    uint64_t tot = (uint64_t)n * (uint64_t)d;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float mx[64], innov[64], e[64];
        const float *xs = x_prev + (int64_t)(anc ? anc[i] : i) * d;
        for (int r = 0; r < d; ++r) {
            float v = md->F[r * d] * xs[0];
            for (int k = 1; k < d; ++k) v = fmaf(md->F[r * d + k], xs[k], v);
            mx[r] = v;
        }
        for (int j = 0; j < dy; ++j) {
            float hm = mx[0] * md->H[j * d];
            for (int k = 1; k < d; ++k) hm = fmaf(mx[k], md->H[j * d + k], hm);
            innov[j] = y[j] - hm;
        }
        for (int j = 0; j < d; ++j) e[j] = o_bits_to_normal(o_bits_at(k0, k1, tot, (uint64_t)i * d + j));
        for (int r = 0; r < d; ++r) {
            float g = innov[0] * md->K[r * dy];
            for (int j = 1; j < dy; ++j) g = fmaf(innov[j], md->K[r * dy + j], g);
            float s = e[0] * md->S[r * d];
            for (int k = 1; k < d; ++k) s = fmaf(e[k], md->S[r * d + k], s);
            x_new[i * d + r] = (mx[r] + g) + s;
        }
        float quad = 0.0f;
        for (int k = 0; k < dy; ++k) {
            float v = innov[0] * md->W[k];
            for (int j = 1; j < dy; ++j) v = fmaf(innov[j], md->W[j * dy + k], v);
            quad = k == 0 ? v * v : fmaf(v, v, quad);
        }
        float lres = lw_prev ? lw_prev[i] : 0.0f;
        lw_new[i] = lres - (0.5f * quad + md->cw);
    }
}

double o_opt_run(const o_opt_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                 float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out,
                 float *x_hist, float *lw_hist)
{
    const int d = md->d, dy = md->dy;
    float *xa = (float *)malloc(sizeof(float) * (size_t)(n * d));
    float *xb = (float *)malloc(sizeof(float) * (size_t)(n * d));
    float *la = (float *)malloc(sizeof(float) * (size_t)n);
    float *lb = (float *)malloc(sizeof(float) * (size_t)n);
    int32_t *anc = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint32_t keys2[4], rk[2], sk[2];
    o_split(key, 2, keys2);
    rk[0] = keys2[0]; rk[1] = keys2[1];
    sk[0] = keys2[2]; sk[1] = keys2[3];
    o_opt_init(md, n, sk, y, xa, la);
    double st[4];
    o_lse_ess(la, n, st);
    double logn = log((double)n);
    double logZ = st[1] - logn, lse_prev = st[1];
    float ess_prev = (float)st[3];
    ess_out[0] = ess_prev;
    resampled_out[0] = 0;
    if (x_hist) memcpy(x_hist, xa, sizeof(float) * (size_t)(n * d));
    if (lw_hist) memcpy(lw_hist, la, sizeof(float) * (size_t)n);
    uint32_t *tkeys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)(T > 1 ? T - 1 : 1));
    if (T > 1) o_split(rk, T - 1, tkeys);
    for (int64_t t = 1; t < T; ++t) {
        const uint32_t *kt = tkeys + 2 * (t - 1);
        int res = ess_prev < ess_threshold * (float)n;
        if (res) {
            if (scheme == 0) o_resample_systematic(la, n, o_bits_at(kt[0], kt[1], 1, 0) >> 9, anc);
            else if (scheme == 1) o_resample_multinomial(la, n, kt, anc);
            else o_resample_gumbel(la, n, n, kt, anc);
        }
        o_opt_propagate(md, n, kt, y + t * dy, xa, res ? anc : NULL, res ? NULL : la, xb, lb);
        o_lse_ess(lb, n, st);
        logZ += st[1] - (res ? logn : lse_prev);
        lse_prev = st[1];
        ess_prev = (float)st[3];
        ess_out[t] = ess_prev;
        resampled_out[t] = res;
        if (x_hist) memcpy(x_hist + t * n * d, xb, sizeof(float) * (size_t)(n * d));
        if (lw_hist) memcpy(lw_hist + t * n, lb, sizeof(float) * (size_t)n);
        float *tp = xa; xa = xb; xb = tp;
        tp = la; la = lb; lb = tp;
    }
    free(tkeys);
    free(xa); free(xb); free(la); free(lb); free(anc);
    return logZ;
}

/* ---------------------------------------------- stochastic volatility, d = 1 */

typedef struct {
    float phi;    /* transition_matrix */
    float bsig;   /* transition_covariance_sqrt * sqrt(t_new - t_prev) */
    float r2;     /* likelihood_precision_diag_sqrt^2 = 1 / R */
    float cB;     /* (log 2pi - log r2) / 2 */
    float c0;     /* initial_covariance_sqrt */
    float m0;     /* initial_mean */
} o_sv_model;

/* likelihood_potential (stochastic_volatility.py:96-102) with
 * s = r / exp(x/2):  0.5 y^2 s^2 + 0.5 (log 2pi - log s^2)
 *                 =  (0.5 y^2 r^2) exp(-x) + (0.5 x + cB). */
static inline float o_sv_potential(const o_sv_model *md, float x, float y)
{
    float a = (0.5f * (y * y)) * md->r2;
    return fmaf(a, o_expf(-x), fmaf(0.5f, x, md->cB));
}

/* One stochastic-volatility filter; scheme as in o_lg_run.  t_all (nullable): the T
 * times, step t then takes bsig_t = md->bsig sqrt(t_t - t_{t-1}) (md->bsig being the
 * dt = 1 value), else md->bsig.  x_hist, lw_hist (nullable): (T, n).  Returns logZ. */
static double o_sv_run_impl(const o_sv_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                            const float *t_all, float ess_threshold, int scheme, float *ess_out,
                            int32_t *resampled_out, float *x_hist, float *lw_hist)
{
    float *xa = (float *)malloc(sizeof(float) * (size_t)n), *xb = (float *)malloc(sizeof(float) * (size_t)n);
    float *la = (float *)malloc(sizeof(float) * (size_t)n), *lb = (float *)malloc(sizeof(float) * (size_t)n);
    int32_t *anc = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint32_t keys2[4], rk[2], sk[2];
    o_split(key, 2, keys2);
    rk[0] = keys2[0]; rk[1] = keys2[1];
    sk[0] = keys2[2]; sk[1] = keys2[3];
    for (int64_t i = 0; i < n; ++i) {
        uint32_t a0, a1;
        o_split_at(sk[0], sk[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
        float e = o_bits_to_normal(o_bits_at(a0, a1, 1, 0));
        xa[i] = e * md->c0 + md->m0;
        la[i] = -o_sv_potential(md, xa[i], y[0]);
    }
    if (x_hist) memcpy(x_hist, xa, sizeof(float) * (size_t)n);
    if (lw_hist) memcpy(lw_hist, la, sizeof(float) * (size_t)n);
    double st[4];
    o_lse_ess(la, n, st);
    double logn = log((double)n);
    double logZ = st[1] - logn, lse_prev = st[1];
    float ess_prev = (float)st[3];
    if (ess_out) ess_out[0] = ess_prev;
    if (resampled_out) resampled_out[0] = 0;
    uint32_t *tkeys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)(T > 1 ? T - 1 : 1));
    if (T > 1) o_split(rk, T - 1, tkeys);
    for (int64_t t = 1; t < T; ++t) {
        const uint32_t *kt = tkeys + 2 * (t - 1);
        int res = ess_prev < ess_threshold * (float)n;
        if (res) {
            if (scheme == 0) o_resample_systematic(la, n, o_bits_at(kt[0], kt[1], 1, 0) >> 9, anc);
            else if (scheme == 1) o_resample_multinomial(la, n, kt, anc);
            else o_resample_gumbel(la, n, n, kt, anc);
        }
        const float bsig = t_all ? md->bsig * sqrtf(t_all[t] - t_all[t - 1]) : md->bsig;
        for (int64_t i = 0; i < n; ++i) {
            uint32_t a0, a1;
            o_split_at(kt[0], kt[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
            float e = o_bits_to_normal(o_bits_at(a0, a1, 1, 0));
            float xs = xa[res ? anc[i] : i];
            float xn = fmaf(xs, md->phi, e * bsig);
            xb[i] = xn;
            lb[i] = (res ? 0.0f : la[i]) - o_sv_potential(md, xn, y[t]);
        }
        o_lse_ess(lb, n, st);
        logZ += st[1] - (res ? logn : lse_prev);
        lse_prev = st[1];
        ess_prev = (float)st[3];
        if (ess_out) ess_out[t] = ess_prev;
        if (resampled_out) resampled_out[t] = res;
        if (x_hist) memcpy(x_hist + t * n, xb, sizeof(float) * (size_t)n);
        if (lw_hist) memcpy(lw_hist + t * n, lb, sizeof(float) * (size_t)n);
        float *tp = xa; xa = xb; xb = tp;
        tp = la; la = lb; lb = tp;
    }
    free(tkeys);
    free(xa); free(xb); free(la); free(lb); free(anc);
    return logZ;
}

double o_sv_run(const o_sv_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out)
{
    return o_sv_run_impl(md, n, T, key, y, NULL, ess_threshold, scheme, ess_out, resampled_out, NULL, NULL);
}

/* run_particle_filter_for_marginals on StochasticVolatility (dim 1) with the history */
double o_sv_run_hist(const o_sv_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                     const float *t_all, float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out,
                     float *x_hist, float *lw_hist)
{
    return o_sv_run_impl(md, n, T, key, y, t_all, ess_threshold, scheme, ess_out, resampled_out, x_hist, lw_hist);
}

/* ------------------------------------- stochastic volatility, dimension d */

/* StochasticVolatility (stochastic_volatility.py:15-108) with a diagonal likelihood
 * covariance R (likelihood_covariance_diag, a vector):
 *   initial_sample     x_0 = C0 normal(key, (d,)) + m0                         (:71-76)
 *   transition_sample  x_t = A x_{t-1} + (Lq normal(key, (d,))) sqrt(t_t - t_{t-1}) (:87-94)
 *   likelihood_potential with s_j = r_j / exp(x_j / 2), r_j^2 = 1 / R_j:
 *     sum_j 0.5 y_j^2 s_j^2 + (d log 2pi - sum_j log s_j^2) / 2
 *     = cB + sum_j (0.5 x_j + (0.5 y_j^2 r2_j) exp(-x_j)),  cB = (d log 2pi - sum log r2_j) / 2
 * accumulated j = 0, 1, ... as pot = fma(a_j, exp(-x_j), fma(0.5, x_j, pot)) from pot = cB
 * (for d = 1 the dim-1 model's formula).  Matrix-vector products are fma chains in
 * ascending column order. */
typedef struct {
    int d;
    const float *A;   /* d x d transition_matrix */
    const float *Lq;  /* d x d transition_covariance_sqrt */
    const float *C0;  /* d x d initial_covariance_sqrt */
    const float *m0;  /* d initial_mean */
    const float *r2;  /* d: 1 / likelihood_covariance_diag */
    float cB;
} o_svd_model;

static inline float o_svd_potential(const o_svd_model *md, const float *x, const float *y)
{
    float pot = md->cB;
    for (int j = 0; j < md->d; ++j) {
        float a = (0.5f * (y[j] * y[j])) * md->r2[j];
        pot = fmaf(a, o_expf(-x[j]), fmaf(0.5f, x[j], pot));
    }
    return pot;
}

static inline void o_svd_mv(const float *M, const float *v, int d, int r, float *out)
{
    const float *m = M + r * d;
    float acc = m[0] * v[0];
    for (int k = 1; k < d; ++k) acc = fmaf(m[k], v[k], acc);
    *out = acc;
}

/* x particle-major (n, d) */
void o_svd_init(const o_svd_model *md, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw)
{
    const int d = md->d;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t a0, a1;
        float e[64];
        o_split_at(key[0], key[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
        o_normal_vec(a0, a1, d, e);
        float *xi = x + i * d;
        for (int r = 0; r < d; ++r) {
            float v;
            o_svd_mv(md->C0, e, d, r, &v);
            xi[r] = v + md->m0[r];
        }
        lw[i] = y0 ? -o_svd_potential(md, xi, y0) : 0.0f;
    }
}

/* one step: x_new = A x_src + (Lq e) sdt, sdt = sqrt(dt); lw_new = lw_res - potential */
void o_svd_propagate(const o_svd_model *md, int64_t n, const uint32_t *kt, const float *y, float dt,
                     const float *x_prev, const int32_t *anc, const float *lw_prev, float *x_new, float *lw_new)
{
    const int d = md->d;
    const float sdt = sqrtf(dt);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t a0, a1;
        float e[64];
        o_split_at(kt[0], kt[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
        o_normal_vec(a0, a1, d, e);
        const float *xs = x_prev + (anc ? (int64_t)anc[i] : i) * d;
        float *xn = x_new + i * d;
        for (int r = 0; r < d; ++r) {
            float fx, le;
            o_svd_mv(md->A, xs, d, r, &fx);
            o_svd_mv(md->Lq, e, d, r, &le);
            xn[r] = fx + le * sdt;
        }
        lw_new[i] = (lw_prev ? lw_prev[i] : 0.0f) - o_svd_potential(md, xn, y);
    }
}

/* run_particle_filter_for_marginals with the bootstrap filter; t_all (nullable): the T
 * times (else unit steps); scheme as in o_lg_run; x_hist (T, n, d), lw_hist (T, n)
 * nullable.  Returns log Z. */
double o_svd_run_hist(const o_svd_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y,
                      const float *t_all, float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out,
                      float *x_hist, float *lw_hist)
{
    const int d = md->d;
    float *xa = (float *)malloc(sizeof(float) * (size_t)n * d), *xb = (float *)malloc(sizeof(float) * (size_t)n * d);
    float *la = (float *)malloc(sizeof(float) * (size_t)n), *lb = (float *)malloc(sizeof(float) * (size_t)n);
    int32_t *anc = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint32_t keys2[4], rk[2], sk[2];
    o_split(key, 2, keys2);
    rk[0] = keys2[0]; rk[1] = keys2[1];
    sk[0] = keys2[2]; sk[1] = keys2[3];
    o_svd_init(md, n, sk, y, xa, la);
    if (x_hist) memcpy(x_hist, xa, sizeof(float) * (size_t)n * d);
    if (lw_hist) memcpy(lw_hist, la, sizeof(float) * (size_t)n);
    double st[4];
    o_lse_ess(la, n, st);
    double logn = log((double)n);
    double logZ = st[1] - logn, lse_prev = st[1];
    float ess_prev = (float)st[3];
    if (ess_out) ess_out[0] = ess_prev;
    if (resampled_out) resampled_out[0] = 0;
    uint32_t *tkeys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)(T > 1 ? T - 1 : 1));
    if (T > 1) o_split(rk, T - 1, tkeys);
    for (int64_t t = 1; t < T; ++t) {
        const uint32_t *kt = tkeys + 2 * (t - 1);
        int res = ess_prev < ess_threshold * (float)n;
        if (res) {
            if (scheme == 0) o_resample_systematic(la, n, o_bits_at(kt[0], kt[1], 1, 0) >> 9, anc);
            else if (scheme == 1) o_resample_multinomial(la, n, kt, anc);
            else o_resample_gumbel(la, n, n, kt, anc);
        }
        const float dt = t_all ? t_all[t] - t_all[t - 1] : 1.0f;
        o_svd_propagate(md, n, kt, y + t * d, dt, xa, res ? anc : NULL, res ? NULL : la, xb, lb);
        o_lse_ess(lb, n, st);
        logZ += st[1] - (res ? logn : lse_prev);
        lse_prev = st[1];
        ess_prev = (float)st[3];
        if (ess_out) ess_out[t] = ess_prev;
        if (resampled_out) resampled_out[t] = res;
        if (x_hist) memcpy(x_hist + t * n * d, xb, sizeof(float) * (size_t)n * d);
        if (lw_hist) memcpy(lw_hist + t * n, lb, sizeof(float) * (size_t)n);
        float *tp = xa; xa = xb; xb = tp;
        tp = la; la = lb; lb = tp;
    }
    free(tkeys);
    free(xa); free(xb); free(la); free(lb); free(anc);
    return logZ;
}

/* Many independent SV filters (the batched workload), each with its own
 * (n_b, T_b, y_b, key_b); filters run in parallel across host threads. */
void o_sv_batch(const o_sv_model *md, int64_t B, const int64_t *n, const int64_t *T, const int64_t *y_off,
                const float *y, const uint32_t *keys, float ess_threshold, int scheme, double *logZ)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t b = 0; b < B; ++b)
        logZ[b] = o_sv_run(md, n[b], T[b], keys + 2 * b, y + y_off[b], ess_threshold, scheme, NULL, NULL);
}

/* ------------------------------- one-dimensional non-linear benchmark model */

typedef struct {
    float s0;   /* initial_sd */
    float tsd;  /* transition_sd */
    float lsd;  /* likelihood_sd */
    float c;    /* log(2 pi) / 2: gaussian_potential with unit precision (utils.py:49-105) */
} o_nl_model;

/* 8 cos(1.2 t) (nonlinear1d.py:41-46): the float32 product 1.2f t, a
 * double-precision cosine rounded to float32, an exact scaling by 8 */
float o_nl_drift(float t)
{
    return 8.0f * (float)cos((double)(1.2f * t));
}

/* _transition_mean (nonlinear1d.py:41-46), left to right in float32 */
static inline float o_nl_mean(float x, float drift)
{
    return (0.5f * x + (25.0f * x) / (1.0f + x * x)) + drift;
}

/* likelihood_potential (nonlinear1d.py:63-75): 0.5 ((y - x^2 / 20) / lsd)^2 + c */
static inline float o_nl_potential(const o_nl_model *md, float x, float y)
{
    float z = (y - (x * x) / 20.0f) / md->lsd;
    return 0.5f * (z * z) + md->c;
}

/* initiate_particles with initial_sample (nonlinear1d.py:36-39):
 * x_i = normal(split(key, n)[i], (1,)) s0, lw_i = -potential(x_i, y0) (0 without y0) */
void o_nl_init(const o_nl_model *md, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t a0, a1;
        o_split_at(key[0], key[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
        x[i] = o_bits_to_normal(o_bits_at(a0, a1, 1, 0)) * md->s0;
        lw[i] = y0 ? -o_nl_potential(md, x[i], y0[0]) : 0.0f;
    }
}

/* bootstrap propagate + weight from t_previous (filtering.py:124-139, 160-170):
 * x_new = mean(x_src, t_prev) + normal(split(k_t, n)[i], (1,)) tsd;
 * lw_new = lw_res - potential(x_new, y).  anc NULL: no resampling; lw_prev NULL: 0. */
void o_nl_propagate(const o_nl_model *md, int64_t n, const uint32_t *kt, float y, float t_prev, const float *x_prev,
                    const int32_t *anc, const float *lw_prev, float *x_new, float *lw_new)
{
    const float drift = o_nl_drift(t_prev);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t a0, a1;
        o_split_at(kt[0], kt[1], (uint64_t)n, (uint64_t)i, &a0, &a1);
        float e = o_bits_to_normal(o_bits_at(a0, a1, 1, 0));
        float xn = o_nl_mean(x_prev[anc ? anc[i] : i], drift) + e * md->tsd;
        x_new[i] = xn;
        lw_new[i] = (lw_prev ? lw_prev[i] : 0.0f) - o_nl_potential(md, xn, y);
    }
}

/* Whole bootstrap filter (filtering.py:255-324) on the model; t[T] are the
 * times, step t propagating from t[t-1].  Outputs as o_lg_run (d = 1). */
double o_nl_run(const o_nl_model *md, int64_t n, int64_t T, const uint32_t *key, const float *y, const float *t,
                float ess_threshold, int scheme, float *ess_out, int32_t *resampled_out, float *x_hist,
                float *lw_hist)
{
    float *xa = (float *)malloc(sizeof(float) * (size_t)n), *xb = (float *)malloc(sizeof(float) * (size_t)n);
    float *la = (float *)malloc(sizeof(float) * (size_t)n), *lb = (float *)malloc(sizeof(float) * (size_t)n);
    int32_t *anc = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)(T > 1 ? T : 2));
    o_lg_step_keys(key, T, keys);
    o_nl_init(md, n, keys, y, xa, la);
    double st[4];
    o_lse_ess(la, n, st);
    const double logn = log((double)n);
    double logZ = st[1] - logn, lse_prev = st[1];
    float ess_prev = (float)st[3];
    if (ess_out) ess_out[0] = ess_prev;
    if (resampled_out) resampled_out[0] = 0;
    if (x_hist) memcpy(x_hist, xa, sizeof(float) * (size_t)n);
    if (lw_hist) memcpy(lw_hist, la, sizeof(float) * (size_t)n);
    for (int64_t s = 1; s < T; ++s) {
        const uint32_t *kt = keys + 2 * s;
        int res = ess_prev < ess_threshold * (float)n;
        if (res) {
            if (scheme == 0) o_resample_systematic(la, n, o_bits_at(kt[0], kt[1], 1, 0) >> 9, anc);
            else if (scheme == 1) o_resample_multinomial(la, n, kt, anc);
            else o_resample_gumbel(la, n, n, kt, anc);
        }
        o_nl_propagate(md, n, kt, y[s], t[s - 1], xa, res ? anc : NULL, res ? NULL : la, xb, lb);
        o_lse_ess(lb, n, st);
        logZ += st[1] - (res ? logn : lse_prev);
        lse_prev = st[1];
        ess_prev = (float)st[3];
        if (ess_out) ess_out[s] = ess_prev;
        if (resampled_out) resampled_out[s] = res;
        if (x_hist) memcpy(x_hist + s * n, xb, sizeof(float) * (size_t)n);
        if (lw_hist) memcpy(lw_hist + s * n, lb, sizeof(float) * (size_t)n);
        float *tp = xa; xa = xb; xb = tp;
        tp = la; la = lb; lb = tp;
    }
    free(keys);
    free(xa); free(xb); free(la); free(lb); free(anc);
    return logZ;
}

/* ------------------------------------------- backward simulation (full FFBSi) */

typedef struct {
    int d;
    const float *F;    /* d x d transition_matrix */
    const float *Pq;   /* d x d transition_precision_sqrt */
    float cq;          /* (d log 2pi - log transition_precision_det) / 2 */
    int nl;            /* 1: the non-linear benchmark transition, 2: stochastic volatility (d = 1, F and Pq unused) */
    float tsd, c;      /* the non-linear model's transition_sd and log(2 pi) / 2 */
    float phi, pq;     /* stochastic volatility: transition_matrix, transition_precision_sqrt */
} o_ffbsi_model;

/* transition_potential(x0 -> x1):
 *   linear-Gaussian  0.5 |(x1 - F x0) @ Pq|^2 + cq
 *                    (linear_gaussian.py transition_potential via gaussian_potential, utils.py:49-105);
 *   non-linear 1-D   0.5 ((x1 - mean(x0, t_prev)) / tsd)^2 + c, drift = 8 cos(1.2 t_prev)
 *                    (nonlinear1d.py:48-54). */
static inline float o_transition_potential(const o_ffbsi_model *md, const float *x0, const float *x1, float drift)
{
    if (md->nl == 2) {
        /* stochastic volatility (stochastic_volatility.py:78-85): drift carries pq sqrt(dt);
         * 0.5 ((x1 - x0 phi) pq sqrt(dt))^2, no normaliser */
        const float v = (x1[0] - x0[0] * md->phi) * drift;
        return 0.5f * (v * v);
    }
    if (md->nl) {
        float z = (x1[0] - o_nl_mean(x0[0], drift)) / md->tsd;
        return 0.5f * (z * z) + md->c;
    }
    const int d = md->d;
    float diff[64];
    for (int r = 0; r < d; ++r) {
        const float *f = md->F + r * d;
        float fx = f[0] * x0[0];
        for (int k = 1; k < d; ++k) fx = fmaf(f[k], x0[k], fx);
        diff[r] = x1[r] - fx;
    }
    float quad = 0.0f;
    for (int k = 0; k < d; ++k) {
        float v = diff[0] * md->Pq[k];
        for (int r = 1; r < d; ++r) v = fmaf(diff[r], md->Pq[r * d + k], v);
        quad = k == 0 ? v * v : fmaf(v, v, quad);
    }
    return 0.5f * quad + md->cq;
}

/* backward_simulation_full (backward.py:217-245): t_keys = split(key, T);
 * samples at T-1: categorical(t_keys[T-1], lw_{T-1}, (M,)) (Gumbel-max over the (M, N) draw);
 * for t = T-2 .. 0, sample j: keys = split(t_keys[t], M);
 *   index_j = argmax_i gumbel(keys[j], (N,))_i + lw_{t,i} - transition_potential(x_t^i -> xs_{t+1}^j)
 * (first maximum wins, NaN skipped).  x_hist (T, N, d), lw_hist (T, N); out (T, M, d), idx (T, M). */
static void o_ffbsi(const o_ffbsi_model *md, int64_t T, int64_t N, int64_t M, const float *x_hist,
                    const float *lw_hist, const float *t_all, const uint32_t *key, float *out, int32_t *idx)
{
    const int d = md->d;
    uint32_t *tkeys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)T);
    o_split(key, T, tkeys);
    o_resample_gumbel(lw_hist + (T - 1) * N, N, M, tkeys + 2 * (T - 1), idx + (T - 1) * M);
    for (int64_t j = 0; j < M; ++j)
        memcpy(out + ((T - 1) * M + j) * d, x_hist + ((T - 1) * N + idx[(T - 1) * M + j]) * d, sizeof(float) * d);
    uint32_t *skeys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)M);
    for (int64_t t = T - 2; t >= 0; --t) {
        o_split(tkeys + 2 * t, M, skeys);
        const float drift = md->nl == 1 ? o_nl_drift(t_all[t])
                            : md->nl == 2 ? md->pq * sqrtf(t_all[t + 1] - t_all[t]) : 0.0f;
        const float *xt = x_hist + t * N * d;
        const float *lw = lw_hist + t * N;
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < M; ++j) {
            const float *x1 = out + ((t + 1) * M + j) * d;
            float best = -INFINITY;
            int32_t bi = 0;
            int have = 0;
            for (int64_t i = 0; i < N; ++i) {
                float g = o_bits_to_gumbel(o_bits_at(skeys[2 * j], skeys[2 * j + 1], (uint64_t)N, (uint64_t)i));
                float v = g + (lw[i] - o_transition_potential(md, xt + i * d, x1, drift));
                if (v == v && (!have || v > best)) { best = v; bi = (int32_t)i; have = 1; }
            }
            idx[t * M + j] = bi;
            memcpy(out + (t * M + j) * d, xt + (int64_t)bi * d, sizeof(float) * d);
        }
    }
    free(skeys);
    free(tkeys);
}

void o_ffbsi_lg(const o_ffbsi_model *md, int64_t T, int64_t N, int64_t M, const float *x_hist, const float *lw_hist,
                const uint32_t *key, float *out, int32_t *idx)
{
    o_ffbsi(md, T, N, M, x_hist, lw_hist, NULL, key, out, idx);
}

static o_ffbsi_model o_nl_transition(const o_nl_model *nm)
{
    o_ffbsi_model md = {1, NULL, NULL, 0.0f, 1, nm->tsd, nm->c};
    return md;
}

/* backward_simulation_full on the non-linear benchmark model: t_all[T] are the
 * filter's times (step t's transition leaves t_all[t]); x_hist (T, N), out (T, M) */
void o_ffbsi_nl1d(const o_nl_model *nm, int64_t T, int64_t N, int64_t M, const float *x_hist, const float *lw_hist,
                  const float *t_all, const uint32_t *key, float *out, int32_t *idx)
{
    o_ffbsi_model md = o_nl_transition(nm);
    o_ffbsi(&md, T, N, M, x_hist, lw_hist, t_all, key, out, idx);
}

/* full_stitch (online_smoothing.py:21-41): keys = split(key, M0); for each x0_j,
 * idx_j = argmax_i gumbel(keys[j], (M1,))_i + lw1_i - transition_potential(x0_j -> x1_i)
 * (first maximum wins, NaN skipped).  x0 (M0, d), x1 (M1, d) particle-major. */
static void o_stitch(const o_ffbsi_model *md, int64_t M0, int64_t M1, const float *x0, const float *x1,
                     const float *lw1, float drift, const uint32_t *key, int32_t *idx)
{
    const int d = md->d;
    uint32_t *skeys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)M0);
    o_split(key, M0, skeys);
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < M0; ++j) {
        float best = -INFINITY;
        int32_t bi = 0;
        int have = 0;
        for (int64_t i = 0; i < M1; ++i) {
            float g = o_bits_to_gumbel(o_bits_at(skeys[2 * j], skeys[2 * j + 1], (uint64_t)M1, (uint64_t)i));
            float v = g + (lw1[i] - o_transition_potential(md, x0 + j * d, x1 + i * d, drift));
            if (v == v && (!have || v > best)) { best = v; bi = (int32_t)i; have = 1; }
        }
        idx[j] = bi;
    }
    free(skeys);
}

void o_stitch_lg(const o_ffbsi_model *md, int64_t M0, int64_t M1, const float *x0, const float *x1,
                 const float *lw1, const uint32_t *key, int32_t *idx)
{
    o_stitch(md, M0, M1, x0, x1, lw1, 0.0f, key, idx);
}

/* full_stitch on the non-linear benchmark model, x0 at time t_prev */
void o_stitch_nl1d(const o_nl_model *nm, int64_t M0, int64_t M1, const float *x0, const float *x1,
                   const float *lw1, float t_prev, const uint32_t *key, int32_t *idx)
{
    o_ffbsi_model md = o_nl_transition(nm);
    o_stitch(&md, M0, M1, x0, x1, lw1, o_nl_drift(t_prev), key, idx);
}

/* the stochastic-volatility transition (d = 1): t_all the T times; stitching and pair
 * potentials take dt = t_new - t_prev */
static o_ffbsi_model o_sv_transition(float phi, float pq)
{
    o_ffbsi_model md = {1, NULL, NULL, 0.0f, 2, 0.0f, 0.0f, phi, pq};
    return md;
}

void o_ffbsi_sv(float phi, float pq, int64_t T, int64_t N, int64_t M, const float *x_hist, const float *lw_hist,
                const float *t_all, const uint32_t *key, float *out, int32_t *idx)
{
    o_ffbsi_model md = o_sv_transition(phi, pq);
    o_ffbsi(&md, T, N, M, x_hist, lw_hist, t_all, key, out, idx);
}

void o_stitch_sv(float phi, float pq, int64_t M0, int64_t M1, const float *x0, const float *x1, const float *lw1,
                 float dt, const uint32_t *key, int32_t *idx)
{
    o_ffbsi_model md = o_sv_transition(phi, pq);
    o_stitch(&md, M0, M1, x0, x1, lw1, pq * sqrtf(dt), key, idx);
}

void o_transition_potential_pairs_sv(float phi, float pq, int64_t M, const float *x0, const float *x1, float dt,
                                     float *out)
{
    o_ffbsi_model md = o_sv_transition(phi, pq);
    const float pqs = pq * sqrtf(dt);
    for (int64_t i = 0; i < M; ++i) out[i] = o_transition_potential(&md, x0 + i, x1 + i, pqs);
}

/* transition_potential(x0_i -> x1_i) for each i (vmap over pairs) */
void o_transition_potential_pairs(const o_ffbsi_model *md, int64_t M, const float *x0, const float *x1, float *out)
{
    for (int64_t i = 0; i < M; ++i) out[i] = o_transition_potential(md, x0 + i * md->d, x1 + i * md->d, 0.0f);
}

void o_transition_potential_pairs_nl1d(const o_nl_model *nm, int64_t M, const float *x0, const float *x1,
                                       float t_prev, float *out)
{
    o_ffbsi_model md = o_nl_transition(nm);
    const float drift = o_nl_drift(t_prev);
    for (int64_t i = 0; i < M; ++i) out[i] = o_transition_potential(&md, x0 + i, x1 + i, drift);
}

/* -------------------------------- backward simulation and stitching by rejection */

/* transition potential of item i against pool element j: back = 1 pool_j -> itm_i
 * (backward simulation), back = 0 itm_i -> pool_j (stitching); rows particle-major */
static inline float o_rej_pot(const o_ffbsi_model *md, int back, const float *itm, const float *pool, int64_t i,
                              int64_t j, float drift)
{
    const int d = md->d;
    return back ? o_transition_potential(md, pool + j * d, itm + i * d, drift)
                : o_transition_potential(md, itm + i * d, pool + j * d, drift);
}

/* categorical(key, w) over Np logits: argmax_j gumbel(key, (Np,))_j + w_j, with
 * w_j = lw_j - potential(i, j) when full (first maximum wins, NaN skipped) */
static int32_t o_rej_categorical(const o_ffbsi_model *md, int back, int full, const float *itm, const float *pool,
                                 int64_t i, int64_t Np, const float *lw, float drift, uint32_t k0, uint32_t k1)
{
    float best = -INFINITY;
    int32_t bi = 0;
    int have = 0;
    for (int64_t j = 0; j < Np; ++j) {
        float g = o_bits_to_gumbel(o_bits_at(k0, k1, (uint64_t)Np, (uint64_t)j));
        float w = full ? lw[j] - o_rej_pot(md, back, itm, pool, i, j, drift) : lw[j];
        float v = g + w;
        if (v == v && (!have || v > best)) { best = v; bi = (int32_t)j; have = 1; }
    }
    return bi;
}

/* max with jnp.max's NaN propagation */
static inline float o_nanmax(float m, float v) { return (v != v || v > m) ? v : m; }

/* rejection_resampling (backward.py:126-169, proposals :54-123) and rejection_stitching
 * (online_smoothing.py:129-175, proposals :59-126), one routine: n items with states itm
 * (n, d), a pool (Np, d) with log-weights lw.
 *   (c0, u0, k0) = split(key, 3); idx = categorical(c0, lw, (n,)) (one (n, Np) Gumbel draw);
 *   dens_i = exp(-pot(i, idx_i)); bound = max dens > ibp ? max dens * infl : ibp;
 *   nya_i = uniform(u0, (n,))_i > dens_i / bound; key_i = split(k0, n)_i; evals = n; iter = 1
 *   while any(nya) and iter < max_rej:
 *     evals += #nya; for nya_i: (key_i, c, u) = split(key_i, 3); idx_i = categorical(c, lw);
 *       dens_i = exp(-pot(i, idx_i)); nya_i = uniform(u) > dens_i / bound   (others dens 0, nya 0)
 *     if max dens > bound: bound = max dens * infl; nya = all; iter += 1
 *   for nya_i: idx_i = categorical(key_i, lw - pot(i, .)); evals += Np * #nya.
 * Returns evals. */
static int64_t o_rejection(const o_ffbsi_model *md, int back, int64_t n, int64_t Np, const float *itm,
                           const float *pool, const float *lw, float drift, const uint32_t *key, int32_t max_rej,
                           float ibp, float infl, int32_t *idx)
{
    uint32_t k3[6];
    o_split(key, 3, k3);
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)n);
    float *dens = (float *)malloc(sizeof(float) * (size_t)n);
    uint8_t *nya = (uint8_t *)malloc((size_t)n);
    const uint64_t tot = (uint64_t)n * (uint64_t)Np;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float best = -INFINITY;
        int32_t bi = 0;
        int have = 0;
        for (int64_t j = 0; j < Np; ++j) {
            float g = o_bits_to_gumbel(o_bits_at(k3[0], k3[1], tot, (uint64_t)i * (uint64_t)Np + (uint64_t)j));
            float v = g + lw[j];
            if (v == v && (!have || v > best)) { best = v; bi = (int32_t)j; have = 1; }
        }
        idx[i] = bi;
        dens[i] = o_expf(-o_rej_pot(md, back, itm, pool, i, bi, drift));
    }
    float mx = dens[0];
    for (int64_t i = 1; i < n; ++i) mx = o_nanmax(mx, dens[i]);
    float bound = mx > ibp ? mx * infl : ibp;
    int64_t cnt = 0;
    for (int64_t i = 0; i < n; ++i) {
        float u = o_bits_to_unit(o_bits_at(k3[2], k3[3], (uint64_t)n, (uint64_t)i));
        nya[i] = u > dens[i] / bound;
        cnt += nya[i];
        o_split_at(k3[4], k3[5], (uint64_t)n, (uint64_t)i, &keys[2 * i], &keys[2 * i + 1]);
    }
    int64_t evals = n;
    for (int32_t it = 1; cnt > 0 && it < max_rej; ++it) {
        evals += cnt;
#pragma omp parallel for schedule(dynamic, 16)
        for (int64_t i = 0; i < n; ++i) {
            if (!nya[i]) { dens[i] = 0.0f; continue; }
            uint32_t sk[6];
            o_split(keys + 2 * i, 3, sk);
            int32_t bi = o_rej_categorical(md, back, 0, itm, pool, i, Np, lw, drift, sk[2], sk[3]);
            idx[i] = bi;
            dens[i] = o_expf(-o_rej_pot(md, back, itm, pool, i, bi, drift));
            float u = o_bits_to_unit(o_bits_at(sk[4], sk[5], 1, 0));
            nya[i] = u > dens[i] / bound;
            keys[2 * i] = sk[0];
            keys[2 * i + 1] = sk[1];
        }
        mx = dens[0];
        for (int64_t i = 1; i < n; ++i) mx = o_nanmax(mx, dens[i]);
        if (mx > bound) {
            bound = mx * infl;
            memset(nya, 1, (size_t)n);
        }
        cnt = 0;
        for (int64_t i = 0; i < n; ++i) cnt += nya[i];
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i)
        if (nya[i]) idx[i] = o_rej_categorical(md, back, 1, itm, pool, i, Np, lw, drift, keys[2 * i], keys[2 * i + 1]);
    evals += Np * cnt;
    free(keys);
    free(dens);
    free(nya);
    return evals;
}

/* backward_simulation_rejection (backward.py:172-214): t_keys = split(key, T); the last step as
 * the full version; step t = T-2 .. 0 by o_rejection with items = samples at t+1, pool = x_t.
 * evals (T): evals[0] = 0, evals[t+1] = step t's count. */
static void o_ffbsi_rejection(const o_ffbsi_model *md, int64_t T, int64_t N, int64_t M, const float *x_hist,
                              const float *lw_hist, const float *t_all, const uint32_t *key, int32_t max_rej,
                              float ibp, float infl, float *out, int32_t *idx, int64_t *evals)
{
    const int d = md->d;
    uint32_t *tkeys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)T);
    o_split(key, T, tkeys);
    o_resample_gumbel(lw_hist + (T - 1) * N, N, M, tkeys + 2 * (T - 1), idx + (T - 1) * M);
    for (int64_t j = 0; j < M; ++j)
        memcpy(out + ((T - 1) * M + j) * d, x_hist + ((T - 1) * N + idx[(T - 1) * M + j]) * d, sizeof(float) * d);
    evals[0] = 0;
    for (int64_t t = T - 2; t >= 0; --t) {
        const float drift = md->nl == 1 ? o_nl_drift(t_all[t])
                            : md->nl == 2 ? md->pq * sqrtf(t_all[t + 1] - t_all[t]) : 0.0f;
        evals[t + 1] = o_rejection(md, 1, M, N, out + (t + 1) * M * d, x_hist + t * N * d, lw_hist + t * N, drift,
                                   tkeys + 2 * t, max_rej, ibp, infl, idx + t * M);
        for (int64_t j = 0; j < M; ++j)
            memcpy(out + (t * M + j) * d, x_hist + (t * N + idx[t * M + j]) * d, sizeof(float) * d);
    }
    free(tkeys);
}

void o_ffbsi_rejection_lg(const o_ffbsi_model *md, int64_t T, int64_t N, int64_t M, const float *x_hist,
                          const float *lw_hist, const uint32_t *key, int32_t max_rej, float ibp, float infl,
                          float *out, int32_t *idx, int64_t *evals)
{
    o_ffbsi_rejection(md, T, N, M, x_hist, lw_hist, NULL, key, max_rej, ibp, infl, out, idx, evals);
}

void o_ffbsi_rejection_nl1d(const o_nl_model *nm, int64_t T, int64_t N, int64_t M, const float *x_hist,
                            const float *lw_hist, const float *t_all, const uint32_t *key, int32_t max_rej,
                            float ibp, float infl, float *out, int32_t *idx, int64_t *evals)
{
    o_ffbsi_model md = o_nl_transition(nm);
    o_ffbsi_rejection(&md, T, N, M, x_hist, lw_hist, t_all, key, max_rej, ibp, infl, out, idx, evals);
}

/* rejection_stitching: items x0 (M, d) at t_prev, pool x1 (M, d) with lw1; returns evals */
int64_t o_stitch_rejection_lg(const o_ffbsi_model *md, int64_t M, const float *x0, const float *x1, const float *lw1,
                              const uint32_t *key, int32_t max_rej, float ibp, float infl, int32_t *idx)
{
    return o_rejection(md, 0, M, M, x0, x1, lw1, 0.0f, key, max_rej, ibp, infl, idx);
}

void o_ffbsi_rejection_sv(float phi, float pq, int64_t T, int64_t N, int64_t M, const float *x_hist,
                          const float *lw_hist, const float *t_all, const uint32_t *key, int32_t max_rej, float ibp,
                          float infl, float *out, int32_t *idx, int64_t *evals)
{
    o_ffbsi_model md = o_sv_transition(phi, pq);
    o_ffbsi_rejection(&md, T, N, M, x_hist, lw_hist, t_all, key, max_rej, ibp, infl, out, idx, evals);
}

int64_t o_stitch_rejection_sv(float phi, float pq, int64_t M, const float *x0, const float *x1, const float *lw1,
                              float dt, const uint32_t *key, int32_t max_rej, float ibp, float infl, int32_t *idx)
{
    o_ffbsi_model md = o_sv_transition(phi, pq);
    return o_rejection(&md, 0, M, M, x0, x1, lw1, pq * sqrtf(dt), key, max_rej, ibp, infl, idx);
}

int64_t o_stitch_rejection_nl1d(const o_nl_model *nm, int64_t M, const float *x0, const float *x1, const float *lw1,
                                float t_prev, const uint32_t *key, int32_t max_rej, float ibp, float infl,
                                int32_t *idx)
{
    o_ffbsi_model md = o_nl_transition(nm);
    return o_rejection(&md, 0, M, M, x0, x1, lw1, o_nl_drift(t_prev), key, max_rej, ibp, infl, idx);
}

/* ---------------------------------------------------------------- ABC-SMC */

typedef struct {
    int d, dy;
    const float *m0, *C0, *P0;  /* prior mean, covariance sqrt, precision sqrt */
    float c0;                   /* prior potential normaliser */
    const float *H, *L, *data;  /* likelihood matrix, covariance sqrt, observed data */
} o_abc_model;

typedef struct {
    int N, mcmc_steps, max_iter, n_schedule, adapt_stepsize;
    float retain, resample_thr, term_alpha, stepsize;
    const float *schedule;
} o_abc_config;

/* prior_potential of the ABC LinearGaussian scenario: 0.5 |(x - m0) P0|^2 + c0
 * (vectorised gaussian_potential, utils.py:90-104) */
static float o_abc_prior_pot(const o_abc_model *md, const float *x)
{
    const int d = md->d;
    float diff[16];
    for (int j = 0; j < d; ++j) diff[j] = x[j] - md->m0[j];
    float quad = 0.0f;
    for (int k = 0; k < d; ++k) {
        float v = diff[0] * md->P0[k];
        for (int j = 1; j < d; ++j) v = fmaf(diff[j], md->P0[j * d + k], v);
        quad = k == 0 ? v * v : fmaf(v, v, quad);
    }
    return 0.5f * quad + md->c0;
}

/* |H x + L normal(key, (dy,)) - data|_2 (likelihood_sample, distance_function) */
static float o_abc_sim_dist(const o_abc_model *md, const float *x, uint32_t k0, uint32_t k1)
{
    const int d = md->d, dy = md->dy;
    float e[16];
    o_normal_vec(k0, k1, dy, e);
    float s = 0.0f;
    for (int r = 0; r < dy; ++r) {
        float hx = md->H[r * d] * x[0];
        for (int k = 1; k < d; ++k) hx = fmaf(md->H[r * d + k], x[k], hx);
        float le = md->L[r * dy] * e[0];
        for (int k = 1; k < dy; ++k) le = fmaf(md->L[r * dy + k], e[k], le);
        float dv = (hx + le) - md->data[r];
        s = r == 0 ? dv * dv : s + dv * dv;
    }
    return sqrtf(s);
}

/* the GPU's fixed-order float64 block sum over 1024 thread partials (each thread's float sum
 * of its values in index order): a
 * shuffle-down tree (16, 8, 4, 2, 1) inside each warp, then the 32 warp results
 * in warp order */
#define O_ABC_TPB 1024
static double o_abc_block_sum(const double *part)
{
    double warp_res[O_ABC_TPB / 32];
    for (int w = 0; w < O_ABC_TPB / 32; ++w) {
        double v[32], t[32];
        for (int l = 0; l < 32; ++l) v[l] = part[32 * w + l];
        for (int off = 16; off > 0; off >>= 1) {
            for (int l = 0; l < 32; ++l) t[l] = v[l] + (l + off < 32 ? v[l + off] : v[l]);
            memcpy(v, t, sizeof(v));
        }
        warp_res[w] = v[0];
    }
    double s = warp_res[0];
    for (int w = 1; w < O_ABC_TPB / 32; ++w) s += warp_res[w];
    return s;
}

static int o_cmp_u32(const void *a, const void *b)
{
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : (x > y);
}

/* k-th smallest of non-negative floats by bit order (NaN last) */
static float o_abc_select(const float *v, int n, int k, uint32_t *scratch)
{
    memcpy(scratch, v, sizeof(float) * (size_t)n);
    qsort(scratch, (size_t)n, sizeof(uint32_t), o_cmp_u32);
    float r;
    memcpy(&r, &scratch[k], sizeof(float));
    return r;
}

/* MetropolisedABCSMCSampler adapt (abc/smc.py:226-245); returns 1 while active.
 * iter: the iteration just completed (0 = startup); ess_prev: the state's ess field */
static int o_abc_adapt(int d, const o_abc_config *cf, int iter, float ess_prev, float *x, float *lw,
                       const float *dist, const float *alpha, float *stepsize, float *thr_out, float *ess_out,
                       float *alpha_mean_out, uint32_t *scratch)
{
    const int N = cf->N;
    double part[O_ABC_TPB];
    int cnt = 0;
    /* each GPU thread sums its values in float in index order; the 1024 partials are added
     * in float64 in the fixed tree */
    for (int t = 0; t < O_ABC_TPB; ++t) {
        float s = 0.0f;
        for (int i = t; i < N; i += O_ABC_TPB)
            if (lw[i] > -INFINITY) { s = s + alpha[i]; ++cnt; }
        part[t] = (double)s;
    }
    const float alpha_mean = (float)(o_abc_block_sum(part) / (double)cnt);
    float thr;
    if (cf->n_schedule > 0) {
        thr = cf->schedule[iter < cf->n_schedule ? iter : cf->n_schedule - 1];
    } else {
        const float q = (cf->retain * ess_prev) / (float)N;
        const float pos = q * (float)(N - 1);
        const float lo = floorf(pos), hi = ceilf(pos);
        const float hw = pos - lo, lwt = 1.0f - hw;
        const int ilo = (int)fminf(fmaxf(lo, 0.0f), (float)(N - 1));
        const int ihi = (int)fminf(fmaxf(hi, 0.0f), (float)(N - 1));
        const float vlo = o_abc_select(dist, N, ilo, scratch);
        const float vhi = ihi == ilo ? vlo : o_abc_select(dist, N, ihi, scratch);
        thr = vlo * lwt + vhi * hw;
    }
    int alive = 0;
    for (int i = 0; i < N; ++i) {
        const int a = !(dist[i] > thr);
        lw[i] = a ? 0.0f : -INFINITY;
        alive += a;
    }
    const float ess = alive > 0 ? o_expf(o_logf((float)alive)) : NAN;
    for (int j = 0; j < d; ++j) {
        if (!cf->adapt_stepsize) { stepsize[j] = cf->stepsize; continue; }
        for (int t = 0; t < O_ABC_TPB; ++t) {
            float s = 0.0f;
            for (int i = t; i < N; i += O_ABC_TPB) s = s + x[(size_t)i * d + j];
            part[t] = (double)s;
        }
        const double mean = o_abc_block_sum(part) / (double)N;
        const float mf = (float)mean;
        for (int t = 0; t < O_ABC_TPB; ++t) {
            float s = 0.0f;
            for (int i = t; i < N; i += O_ABC_TPB) {
                const float dv = x[(size_t)i * d + j] - mf;
                s = s + dv * dv;
            }
            part[t] = (double)s;
        }
        const double var = o_abc_block_sum(part) / (double)(N - 1);
        stepsize[j] = ((float)var / (float)d) * 5.6644f;
    }
    *thr_out = thr;
    *ess_out = ess;
    *alpha_mean_out = alpha_mean;
    return !(alive == 0 || alpha_mean <= cf->term_alpha || iter >= cf->max_iter);
}


/* ------------------------------------------------ g-and-k ABC scenarios */

typedef struct {
    int d;                  /* 4 (A, B, g, k) or 1 (A only) */
    int n_raw, n_sum;       /* draws per simulation, thinned order statistics */
    float c, lo, hi, buffer;
    const float *data;      /* (n_sum) observed summary */
} o_gk_model;

/* erfc by Numerical Recipes' erfcc (Chebyshev fit, fractional error < 1.2e-7) */
static float o_gk_erfcc(float x)
{
    const float z = fabsf(x);
    const float t = 1.0f / fmaf(0.5f, z, 1.0f);
    float q = 0.17087277f;
    q = fmaf(t, q, -0.82215223f);
    q = fmaf(t, q, 1.48851587f);
    q = fmaf(t, q, -1.13520398f);
    q = fmaf(t, q, 0.27886807f);
    q = fmaf(t, q, -0.18628806f);
    q = fmaf(t, q, 0.09678418f);
    q = fmaf(t, q, 0.37409196f);
    q = fmaf(t, q, 1.00002368f);
    const float arg = fmaf(t, q, -(z * z) - 1.26551223f);
    const float ans = t * o_expf(arg);
    return x >= 0.0f ? ans : 2.0f - ans;
}

static float o_gk_ncdf(float x) { return 0.5f * o_gk_erfcc(-x * 0.70710677f); }
static float o_gk_ppf(float u) { return 1.41421354f * o_erfinvf(2.0f * u - 1.0f); }

/* constrained (A, B, g, exponent): lo + Phi(x) (hi - lo); the A-only scenario keeps
 * B = 1, g = 2 and the exponent c (gk.py:146-156) */
static void o_gk_params(const o_gk_model *md, const float *x, float q[4])
{
    const float span = md->hi - md->lo;
    if (md->d == 4) {
        for (int j = 0; j < 4; ++j) q[j] = md->lo + o_gk_ncdf(x[j]) * span;
    } else {
        q[0] = md->lo + o_gk_ncdf(x[0]) * span;
        q[1] = 1.0f; q[2] = 2.0f; q[3] = md->c;
    }
}

/* full_data_sample (gk.py:101-110): u = max(buffer, f (1 - 2 buffer) + buffer), z = Phi^-1(u),
 * v = A + ((B (1 + c (1 - e) / (1 + e))) z) (1 + z^2)^k, e = exp(-g z), (.)^k = exp(k log(.)) */
static float o_gk_value(const o_gk_model *md, const float q[4], uint32_t bits)
{
    const float range = (1.0f - md->buffer) - md->buffer;
    const float u = fmaxf(md->buffer, o_bits_to_unit(bits) * range + md->buffer);
    const float z = o_gk_ppf(u);
    const float e = o_expf(-(q[2] * z));
    const float term = 1.0f + (md->c * (1.0f - e)) / (1.0f + e);
    const float pw = o_expf(q[3] * o_logf(1.0f + z * z));
    return q[0] + ((q[1] * term) * z) * pw;
}

/* ascending order of floats with NaN last (jnp.sort) */
static uint32_t o_gk_key(float v)
{
    if (v != v) return 0xFFFFFFFEu;
    const uint32_t b = o_asu(v);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

static float o_gk_unkey(uint32_t k)
{
    if (k == 0xFFFFFFFEu) return NAN;
    return o_asf((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

/* likelihood_sample of GKThinOrder (tests/test_abc_gk.py): n_sum sorted draws at ranks
 * floor(j n_raw / n_sum); with data: the distance |summary - data|_2 summed in index order */
static float o_gk_sim(const o_gk_model *md, const float *x, uint32_t k0, uint32_t k1, float *summary)
{
    float q[4];
    o_gk_params(md, x, q);
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)md->n_raw);
    for (int i = 0; i < md->n_raw; ++i)
        keys[i] = o_gk_key(o_gk_value(md, q, o_bits_at(k0, k1, (uint64_t)md->n_raw, (uint64_t)i)));
    qsort(keys, (size_t)md->n_raw, sizeof(uint32_t), o_cmp_u32);
    float acc = 0.0f;
    for (int j = 0; j < md->n_sum; ++j) {
        const float v = o_gk_unkey(keys[(int)(((int64_t)j * md->n_raw) / md->n_sum)]);
        if (summary) summary[j] = v;
        if (md->data) {
            const float dv = v - md->data[j];
            acc = j == 0 ? dv * dv : acc + dv * dv;
        }
    }
    free(keys);
    return sqrtf(acc);
}

void o_gk_simulate(const o_gk_model *md, int64_t P, const float *x, const uint32_t *keys, float *summary,
                   float *dist)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t r = 0; r < P; ++r) {
        const float dv = o_gk_sim(md, x + r * md->d, keys[2 * r], keys[2 * r + 1],
                                  summary ? summary + r * md->n_sum : NULL);
        if (dist) dist[r] = dv;
    }
}

static float o_gk_prior_pot(int d, const float *x)
{
    float s = x[0] * x[0];
    for (int j = 1; j < d; ++j) s = s + x[j] * x[j];
    return 0.5f * s;
}

/* mocat.run of MetropolisedABCSMCSampler with RandomWalkABC moves on the ABC
 * LinearGaussian scenario (abc/smc.py:101-245, abc/mcmc.py:59-103,
 * metropolis.py:48-70, transport/smc.py:61-100, sample.py:110-148), one
 * posterior, systematic resampling.  x (N, d) receives the final particles,
 * lw / dist (N) the final log-weights and distances; hist_* (max_iter + 1)
 * entry 0 = after startup.  Returns the number of iterations. */
static int o_abc_run(const o_abc_model *md, const o_gk_model *gk, const o_abc_config *cf, const uint32_t *key,
                     float *x, float *lw, float *dist, float *stepsize, float *hist_thr, float *hist_ess,
                     float *hist_alpha, int32_t *hist_res)
{
    const int N = cf->N, d = gk ? gk->d : md->d;
    float *pp = (float *)malloc(sizeof(float) * (size_t)N), *alpha = (float *)malloc(sizeof(float) * (size_t)N);
    float *x2 = (float *)malloc(sizeof(float) * (size_t)N * d), *f2 = (float *)malloc(sizeof(float) * (size_t)N * 3);
    int32_t *anc = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    uint32_t *scratch = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)N);
    uint32_t e0, e1, s0, s1, f0, f1;
    o_split_at(key[0], key[1], 2, 0, &e0, &e1);
    o_split_at(key[0], key[1], 2, 1, &s0, &s1);
    o_split_at(e0, e1, (uint64_t)N + 1, (uint64_t)N, &f0, &f1);
#pragma omp parallel for schedule(dynamic, 8)
    for (int i = 0; i < N; ++i) {
        uint32_t a0, a1, k0, k1;
        float e[16];
        o_split_at(s0, s1, (uint64_t)N, (uint64_t)i, &a0, &a1);
        o_normal_vec(a0, a1, d, e);
        float *xi = x + (size_t)i * d;
        if (gk) {
            for (int r = 0; r < d; ++r) xi[r] = e[r];
            pp[i] = o_gk_prior_pot(d, xi);
        } else {
            for (int r = 0; r < d; ++r) {
                float v = md->C0[r * d] * e[0];
                for (int k = 1; k < d; ++k) v = fmaf(md->C0[r * d + k], e[k], v);
                xi[r] = md->m0[r] + v;
            }
            pp[i] = o_abc_prior_pot(md, xi);
        }
        o_split_at(f0, f1, (uint64_t)N + 1, (uint64_t)i, &k0, &k1);
        dist[i] = gk ? o_gk_sim(gk, xi, k0, k1, NULL) : o_abc_sim_dist(md, xi, k0, k1);
        alpha[i] = 1.0f;
        lw[i] = 0.0f;
    }
    uint32_t k[2];
    o_split_at(f0, f1, (uint64_t)N + 1, (uint64_t)N, &k[0], &k[1]);
    float thr, ess, am;
    int active = o_abc_adapt(d, cf, 0, (float)N, x, lw, dist, alpha, stepsize, &thr, &ess, &am, scratch);
    hist_thr[0] = thr; hist_ess[0] = ess; hist_alpha[0] = am; hist_res[0] = 0;
    int iter = 0;
    while (active) {
        ++iter;
        const int res = ess < cf->resample_thr * (float)N;
        if (res) {
            uint32_t r0, r1;
            o_split_at(k[0], k[1], (uint64_t)N + 2, (uint64_t)N, &r0, &r1);
            o_resample_systematic(lw, N, o_bits_at(r0, r1, 1, 0) >> 9, anc);
            for (int i = 0; i < N; ++i) {
                memcpy(x2 + (size_t)i * d, x + (size_t)anc[i] * d, sizeof(float) * d);
                f2[3 * i] = dist[anc[i]]; f2[3 * i + 1] = pp[anc[i]]; f2[3 * i + 2] = alpha[anc[i]];
            }
            memcpy(x, x2, sizeof(float) * (size_t)N * d);
            for (int i = 0; i < N; ++i) {
                dist[i] = f2[3 * i]; pp[i] = f2[3 * i + 1]; alpha[i] = f2[3 * i + 2]; lw[i] = 0.0f;
            }
            ess = (float)N;
        }
        float sq[16];
        for (int j = 0; j < d; ++j) sq[j] = sqrtf(stepsize[j]);
#pragma omp parallel for schedule(dynamic, 8)
        for (int i = 0; i < N; ++i) {
            if (!(lw[i] > -INFINITY)) continue;
            float *xi = x + (size_t)i * d;
            uint32_t k0, k1;
            o_split_at(k[0], k[1], (uint64_t)N + 2, (uint64_t)i, &k0, &k1);
            float asum = 0.0f;
            for (int st = 0; st < cf->mcmc_steps; ++st) {
                uint32_t t0, t1, n0, n1, a0, a1, c0, c1, u0, u1, v0, v1;
                o_split_at(k0, k1, 2, 0, &t0, &t1);
                o_split_at(t0, t1, 4, 0, &n0, &n1);
                o_split_at(t0, t1, 4, 1, &a0, &a1);
                o_split_at(t0, t1, 4, 3, &c0, &c1);
                float e[16], xp[16] = {0.0f};
                o_normal_vec(a0, a1, d, e);
                for (int j = 0; j < d; ++j) xp[j] = xi[j] + sq[j] * e[j];
                const float ppn = gk ? o_gk_prior_pot(d, xp) : o_abc_prior_pot(md, xp);
                const float dn = gk ? o_gk_sim(gk, xp, c0, c1, NULL) : o_abc_sim_dist(md, xp, c0, c1);
                float a = o_expf(pp[i] - ppn) * (dn < thr ? 1.0f : 0.0f);
                a = a != a ? 0.0f : fminf(1.0f, a);
                o_split_at(n0, n1, 2, 0, &u0, &u1);
                o_split_at(n0, n1, 2, 1, &v0, &v1);
                const float u = o_bits_to_unit(o_bits_at(v0, v1, 1, 0));
                if (u < a) {
                    memcpy(xi, xp, sizeof(float) * d);
                    pp[i] = ppn;
                    dist[i] = dn;
                }
                asum = st == 0 ? a : asum + a;
                k0 = u0; k1 = u1;
            }
            alpha[i] = asum / (float)cf->mcmc_steps;
        }
        active = o_abc_adapt(d, cf, iter, ess, x, lw, dist, alpha, stepsize, &thr, &ess, &am, scratch);
        uint32_t z0, z1;
        o_split_at(k[0], k[1], (uint64_t)N + 2, (uint64_t)N + 1, &z0, &z1);
        k[0] = z0; k[1] = z1;
        if (iter <= cf->max_iter) {
            hist_thr[iter] = thr; hist_ess[iter] = ess; hist_alpha[iter] = am; hist_res[iter] = res;
        }
    }
    free(pp); free(alpha); free(x2); free(f2); free(anc); free(scratch);
    return iter;
}

int o_abc_lg_run(const o_abc_model *md, const o_abc_config *cf, const uint32_t *key, float *x, float *lw,
                 float *dist, float *stepsize, float *hist_thr, float *hist_ess, float *hist_alpha, int32_t *hist_res)
{
    return o_abc_run(md, NULL, cf, key, x, lw, dist, stepsize, hist_thr, hist_ess, hist_alpha, hist_res);
}

/* VanillaABC (abc/importance.py:16-118) run as mocat.run: n prior draws with the sequential
 * key chain (K, s) = split(K) [x_0]; (K, _) = split(K) [prior potential]; (K, k) = split(K)
 * [simulation of x_0]; then (K, k1, k2, k3) = split(K, 4) per draw (x_i from k1, simulation
 * from k3).  lw = 0 where dist < threshold; rate >= 0: threshold = jnp.quantile(dist, rate)
 * (linear interpolation).  Returns the threshold. */
static float o_abc_vanilla(const o_abc_model *md, const o_gk_model *gk, int n, const uint32_t *key, float thr,
                           float rate, float *x, float *pp, float *dist, float *lw)
{
    const int d = gk ? gk->d : md->d;
    uint32_t *pk = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)n);
    uint32_t *sk = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)n);
    uint32_t K0, K1, b0, b1;
    o_split_at(key[0], key[1], 2, 1, &pk[0], &pk[1]);
    o_split_at(key[0], key[1], 2, 0, &b0, &b1);
    o_split_at(b0, b1, 2, 0, &K0, &K1);
    o_split_at(K0, K1, 2, 1, &sk[0], &sk[1]);
    o_split_at(K0, K1, 2, 0, &b0, &b1);
    K0 = b0; K1 = b1;
    for (int i = 1; i < n; ++i) {
        o_split_at(K0, K1, 4, 1, &pk[2 * i], &pk[2 * i + 1]);
        o_split_at(K0, K1, 4, 3, &sk[2 * i], &sk[2 * i + 1]);
        o_split_at(K0, K1, 4, 0, &b0, &b1);
        K0 = b0; K1 = b1;
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        float e[16];
        float *xi = x + (size_t)i * d;
        o_normal_vec(pk[2 * i], pk[2 * i + 1], d, e);
        if (gk) {
            for (int r = 0; r < d; ++r) xi[r] = e[r];
            pp[i] = o_gk_prior_pot(d, xi);
            dist[i] = o_gk_sim(gk, xi, sk[2 * i], sk[2 * i + 1], NULL);
        } else {
            for (int r = 0; r < d; ++r) {
                float v = md->C0[r * d] * e[0];
                for (int k = 1; k < d; ++k) v = fmaf(md->C0[r * d + k], e[k], v);
                xi[r] = md->m0[r] + v;
            }
            pp[i] = o_abc_prior_pot(md, xi);
            dist[i] = o_abc_sim_dist(md, xi, sk[2 * i], sk[2 * i + 1]);
        }
    }
    if (rate >= 0.0f) {
        uint32_t *scratch = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
        const float pos = rate * (float)(n - 1);
        const float lo = floorf(pos), hi = ceilf(pos);
        const float hw = pos - lo, lwt = 1.0f - hw;
        const int ilo = (int)fminf(fmaxf(lo, 0.0f), (float)(n - 1));
        const int ihi = (int)fminf(fmaxf(hi, 0.0f), (float)(n - 1));
        const float vlo = o_abc_select(dist, n, ilo, scratch);
        const float vhi = ihi == ilo ? vlo : o_abc_select(dist, n, ihi, scratch);
        thr = vlo * lwt + vhi * hw;
        free(scratch);
    }
    for (int i = 0; i < n; ++i) lw[i] = dist[i] < thr ? 0.0f : -INFINITY;
    free(pk); free(sk);
    return thr;
}

float o_abc_vanilla_lg(const o_abc_model *md, int n, const uint32_t *key, float thr, float rate, float *x, float *pp,
                       float *dist, float *lw)
{
    return o_abc_vanilla(md, NULL, n, key, thr, rate, x, pp, dist, lw);
}

float o_abc_vanilla_gk(const o_gk_model *gk, int n, const uint32_t *key, float thr, float rate, float *x, float *pp,
                       float *dist, float *lw)
{
    return o_abc_vanilla(NULL, gk, n, key, thr, rate, x, pp, dist, lw);
}

/* RandomWalkABC as an MCMC sampler (abc/mcmc.py:16-100, metropolis.py:48-70, mocat.run) on the
 * ABC linear-Gaussian scenario, fixed stepsize and threshold, one chain of n states:
 * (K, s) = split(K) [x_0]; (K, _) = split(K) [prior potential]; (K, k) = split(K) [simulation];
 * per step (K, _) = split(K); (K, k1, k2, k3) = split(K, 4); x' = x + sqrt(stepsize) normal(k1);
 * alpha = min(1, exp(pp - pp') [dist' < threshold]) (NaN -> 0); (K, ku) = split(K); accept if
 * uniform(ku) < alpha.  x (n, d), dist, pp, alpha (n). */
static void o_abc_mcmc(const o_abc_model *md, const o_gk_model *gk, int n, const uint32_t *key, float stepsize,
                       float thr, float *x, float *dist, float *pp, float *alpha)
{
    const int d = gk ? gk->d : md->d;
    uint32_t K0, K1, a0, a1, t0, t1;
    o_split_at(key[0], key[1], 2, 1, &a0, &a1);
    o_split_at(key[0], key[1], 2, 0, &t0, &t1);
    o_split_at(t0, t1, 2, 0, &K0, &K1);
    float e[16], xc[16] = {0.0f}, xp[16] = {0.0f};
    o_normal_vec(a0, a1, d, e);
    float p;
    if (gk) {
        for (int r = 0; r < d; ++r) xc[r] = e[r];
        p = o_gk_prior_pot(d, xc);
    } else {
        for (int r = 0; r < d; ++r) {
            float v = md->C0[r * d] * e[0];
            for (int k = 1; k < d; ++k) v = fmaf(md->C0[r * d + k], e[k], v);
            xc[r] = md->m0[r] + v;
        }
        p = o_abc_prior_pot(md, xc);
    }
    o_split_at(K0, K1, 2, 1, &a0, &a1);
    float ds = gk ? o_gk_sim(gk, xc, a0, a1, NULL) : o_abc_sim_dist(md, xc, a0, a1);
    o_split_at(K0, K1, 2, 0, &t0, &t1);
    K0 = t0; K1 = t1;
    const float sq = sqrtf(stepsize);
    memcpy(x, xc, sizeof(float) * d);
    dist[0] = ds; pp[0] = p; alpha[0] = 1.0f;
    for (int i = 1; i < n; ++i) {
        uint32_t n0, n1, c0, c1, u0, u1, v0, v1;
        o_split_at(K0, K1, 2, 0, &t0, &t1);
        o_split_at(t0, t1, 4, 0, &n0, &n1);
        o_split_at(t0, t1, 4, 1, &a0, &a1);
        o_split_at(t0, t1, 4, 3, &c0, &c1);
        o_normal_vec(a0, a1, d, e);
        for (int j = 0; j < d; ++j) xp[j] = xc[j] + sq * e[j];
        const float ppn = gk ? o_gk_prior_pot(d, xp) : o_abc_prior_pot(md, xp);
        const float dn = gk ? o_gk_sim(gk, xp, c0, c1, NULL) : o_abc_sim_dist(md, xp, c0, c1);
        float a = o_expf(p - ppn) * (dn < thr ? 1.0f : 0.0f);
        a = a != a ? 0.0f : fminf(1.0f, a);
        o_split_at(n0, n1, 2, 0, &u0, &u1);
        o_split_at(n0, n1, 2, 1, &v0, &v1);
        const float u = o_bits_to_unit(o_bits_at(v0, v1, 1, 0));
        if (u < a) {
            memcpy(xc, xp, sizeof(float) * d);
            p = ppn;
            ds = dn;
        }
        K0 = u0; K1 = u1;
        memcpy(x + (size_t)i * d, xc, sizeof(float) * d);
        dist[i] = ds; pp[i] = p; alpha[i] = a;
    }
}

void o_abc_mcmc_lg(const o_abc_model *md, int n, const uint32_t *key, float stepsize, float thr, float *x, float *dist,
                   float *pp, float *alpha)
{
    o_abc_mcmc(md, NULL, n, key, stepsize, thr, x, dist, pp, alpha);
}

/* the same fixed chain on a g-and-k scenario: x_0 = normal(split(key)[1], (d,)), potential 0.5 |x|^2 */
void o_abc_mcmc_gk(const o_gk_model *gk, int n, const uint32_t *key, float stepsize, float thr, float *x, float *dist,
                   float *pp, float *alpha)
{
    o_abc_mcmc(NULL, gk, n, key, stepsize, thr, x, dist, pp, alpha);
}

/* RandomWalkABC with the RMMetropolisDiagStepsize correction (abc/mcmc.py:105-140,
 * metropolis.py:73-160), the sampler's defaults: threshold and stepsize unset, so the chain starts
 * at threshold 50 and stepsize 1 per dimension, post_mean x_0, diag_post_cov = stepsize d / 2.38^2.
 * Each step as o_abc_mcmc_lg with the current threshold and per-dimension stepsize, then, with
 * rm = scale iter^-neg_exp (iter = step index, exp and log by the library's own functions):
 *   threshold <- exp(log threshold - rm (alpha - target))                (log Robbins-Monro)
 *   r = min(rm, 1 - 1e-3); diag <- (1 - r) diag + r (x - post_mean)^2; post_mean <- (1 - r) post_mean + r x;
 *   stepsize <- diag / d * 2.38^2
 * Outputs per state: x (n, d), alpha (n), threshold (n), stepsize (n, d). */
static void o_abc_mcmc_rm(const o_abc_model *md, const o_gk_model *gk, int n, const uint32_t *key, float target,
                          float scale, float neg_exp, float *x, float *alpha, float *thr_out, float *step_out)
{
    const int d = gk ? gk->d : md->d;
    uint32_t K0, K1, a0, a1, t0, t1;
    o_split_at(key[0], key[1], 2, 1, &a0, &a1);
    o_split_at(key[0], key[1], 2, 0, &t0, &t1);
    o_split_at(t0, t1, 2, 0, &K0, &K1);
    float e[16], xc[16] = {0.0f}, xp[16] = {0.0f}, st[16], pm[16], dg[16];
    o_normal_vec(a0, a1, d, e);
    float p;
    if (gk) {
        /* the transformed-uniform prior: x_0 = the normal draw itself, potential 0.5 |x|^2 */
        for (int r = 0; r < d; ++r) xc[r] = e[r];
        p = o_gk_prior_pot(d, xc);
    } else {
        for (int r = 0; r < d; ++r) {
            float v = md->C0[r * d] * e[0];
            for (int k = 1; k < d; ++k) v = fmaf(md->C0[r * d + k], e[k], v);
            xc[r] = md->m0[r] + v;
        }
        p = o_abc_prior_pot(md, xc);
    }
    /* the initial simulation takes split(K)[1]; the adaptive chain does not use its distance */
    o_split_at(K0, K1, 2, 0, &t0, &t1);
    K0 = t0; K1 = t1;
    float thr = 50.0f;
    for (int j = 0; j < d; ++j) {
        st[j] = 1.0f;
        pm[j] = xc[j];
        dg[j] = (st[j] * (float)d) / 5.6644f;
    }
    memcpy(x, xc, sizeof(float) * d);
    memcpy(step_out, st, sizeof(float) * d);
    alpha[0] = 1.0f; thr_out[0] = thr;
    for (int i = 1; i < n; ++i) {
        uint32_t n0, n1, c0, c1, u0, u1, v0, v1;
        o_split_at(K0, K1, 2, 0, &t0, &t1);
        o_split_at(t0, t1, 4, 0, &n0, &n1);
        o_split_at(t0, t1, 4, 1, &a0, &a1);
        o_split_at(t0, t1, 4, 3, &c0, &c1);
        o_normal_vec(a0, a1, d, e);
        for (int j = 0; j < d; ++j) xp[j] = xc[j] + sqrtf(st[j]) * e[j];
        const float ppn = gk ? o_gk_prior_pot(d, xp) : o_abc_prior_pot(md, xp);
        const float dn = gk ? o_gk_sim(gk, xp, c0, c1, NULL) : o_abc_sim_dist(md, xp, c0, c1);
        float a = o_expf(p - ppn) * (dn < thr ? 1.0f : 0.0f);
        a = a != a ? 0.0f : fminf(1.0f, a);
        o_split_at(n0, n1, 2, 0, &u0, &u1);
        o_split_at(n0, n1, 2, 1, &v0, &v1);
        const float u = o_bits_to_unit(o_bits_at(v0, v1, 1, 0));
        if (u < a) {
            memcpy(xc, xp, sizeof(float) * d);
            p = ppn;
        }
        K0 = u0; K1 = u1;
        const float rm = scale * o_expf(-neg_exp * o_logf((float)i));
        thr = o_expf(o_logf(thr) - rm * (a - target));
        const float r2 = fminf(rm, 0.999f);
        for (int j = 0; j < d; ++j) {
            const float dv = xc[j] - pm[j];
            dg[j] = (1.0f - r2) * dg[j] + r2 * (dv * dv);
            pm[j] = (1.0f - r2) * pm[j] + r2 * xc[j];
            st[j] = (dg[j] / (float)d) * 5.6644f;
        }
        memcpy(x + (size_t)i * d, xc, sizeof(float) * d);
        memcpy(step_out + (size_t)i * d, st, sizeof(float) * d);
        alpha[i] = a; thr_out[i] = thr;
    }
}

void o_abc_mcmc_rm_lg(const o_abc_model *md, int n, const uint32_t *key, float target, float scale, float neg_exp,
                      float *x, float *alpha, float *thr_out, float *step_out)
{
    o_abc_mcmc_rm(md, NULL, n, key, target, scale, neg_exp, x, alpha, thr_out, step_out);
}

/* the same adaptive chain on a g-and-k scenario (the reference's TestMCMCGK / TestMCMCGKOnlyA):
 * prior draws x_0 = normal(split(key)[1], (d,)), prior potential 0.5 |x|^2, one g-and-k
 * simulation per step */
void o_abc_mcmc_rm_gk(const o_gk_model *gk, int n, const uint32_t *key, float target, float scale, float neg_exp,
                      float *x, float *alpha, float *thr_out, float *step_out)
{
    o_abc_mcmc_rm(NULL, gk, n, key, target, scale, neg_exp, x, alpha, thr_out, step_out);
}

/* the same sampler on a g-and-k scenario */
int o_abc_gk_run(const o_gk_model *gk, const o_abc_config *cf, const uint32_t *key, float *x, float *lw,
                 float *dist, float *stepsize, float *hist_thr, float *hist_ess, float *hist_alpha, int32_t *hist_res)
{
    return o_abc_run(NULL, gk, cf, key, x, lw, dist, stepsize, hist_thr, hist_ess, hist_alpha, hist_res);
}

int o_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void o_set_num_threads(int k)
{
#ifdef _OPENMP
    omp_set_num_threads(k);
#else
    (void)k;
#endif
}
