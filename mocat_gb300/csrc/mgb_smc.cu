// Tempered SMC sampler with MALA moves on Bayesian logistic regression, many
// independent posteriors advanced in lockstep.
//
// Reference path: mocat.run (mocat/src/sample.py:110-148) with
// MetropolisedSMCSampler (mocat/src/transport/smc.py:229-373) over
// Underdamped(leapfrog_steps=1, friction=inf) = MALA
// (mocat/src/mcmc/standard_mcmc.py:72-153, utils.leapfrog :108-156) with the
// Metropolis correction (mocat/src/mcmc/metropolis.py:48-70):
//   startup  (smc.py:128-164, :267-296; transport/sampler.py:17-31):
//            (key, sub) = split(key); beta_j = s normal(split(sub, N)[j], (d,));
//            key = split(key, 2N + 1)[-1]; tau_1 by bisection from 0;
//            lw = -tau_1 l; log Z = LSE(lw) - log N; key = split(key, 3)[0]
//   update   (smc.py:73-99, :219-225): resample when ess <= thr N (keys_all =
//            split(key, N + 2): particle keys [:N], resample key [N], next key
//            [N + 1]); per particle k = split(k_j, 3)[0], then mcmc_steps MALA moves:
//            (k, ka) = split(k); p = normal(ka, (d,)); p_h = p - eps/2 grad U;
//            beta' = beta + eps p_h; p' = p_h - eps/2 grad U(beta');
//            alpha = min(1, exp(-U' + U - |p'|^2/2 + |p|^2/2)); k = split(k, 2)[0];
//            (k, ku) = split(k); accept if uniform(ku) < alpha;
//            then l = (U - prior) / tau (smc.py:355-358)
//   adapt    (smc.py:193-217, :311-326; utils.bisect :205-237): regula falsi on
//            log ESS(lw_res - (tau' - tau) l) = log(ess retain); lw = lw_res - (tau' - tau) l;
//            log Z += LSE(lw) - LSE(lw_res)
// Scenario: prior N(0, s^2 I): prior potential |beta|^2 / (2 s^2); likelihood
// potential l(beta) = sum_i softplus(x_i beta) - y_i x_i beta, gradient
// X^T (sigmoid(X beta) - y).
//
// Differences by design: resampling is systematic (O(N), in shared memory per
// posterior) instead of random.categorical; potentials are not re-evaluated at
// the start of each MCMC block (they are deterministic, the stored values are
// the same numbers).
//
// Layout: particle-major rows beta[(b N + j) d + k] (the K-major operand of the
// potential's GEMMs); per-posterior scalars in (B,) arrays.
#include <cmath>
#include <vector>

#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_group.cuh"
#include "mgb_smc.cuh"

namespace mgb {

constexpr int SMC_TPB = 256;
constexpr int ADAPT_TPB = 1024;
constexpr int LR_TPB = 128;
constexpr int LR_ROWS = 64;

// ------------------------------------------------------------ potential, FP32
// One thread per particle; X rows staged through shared memory in tiles of
// LR_ROWS; blockIdx.y selects a chunk of the data (partials summed afterwards).
template <int D>
__global__ void __launch_bounds__(LR_TPB) k_logreg_f32(const float *__restrict__ X, const float *__restrict__ y,
                                                        int64_t n_data, int64_t chunk,
                                                        const float *__restrict__ beta, int64_t P,
                                                        const int32_t *active, int N,
                                                        float *__restrict__ part_lik,
                                                        float *__restrict__ part_grad) {
  __shared__ float xs[LR_ROWS * D];
  __shared__ float ys[LR_ROWS];
  const int64_t p = blockIdx.x * (int64_t)LR_TPB + threadIdx.x;
  const int64_t r0 = blockIdx.y * chunk, r1 = min(r0 + chunk, n_data);
  const int64_t pb = blockIdx.x * (int64_t)LR_TPB;
  // whole block inactive: the posteriors of its particles have finished
  bool any = false;
  if (active) {
    const int64_t plast = min(pb + LR_TPB, P) - 1;
    for (int64_t b = pb / N; b <= plast / N; ++b) any |= active[b] != 0;
  } else {
    any = true;
  }
  if (!any) return;
  const bool mine = p < P && (!active || active[p / N]);
  float bt[D], g[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    bt[k] = mine ? beta[p * D + k] : 0.0f;
    g[k] = 0.0f;
  }
  float acc = 0.0f;
  for (int64_t t0 = r0; t0 < r1; t0 += LR_ROWS) {
    const int rows = (int)min((int64_t)LR_ROWS, r1 - t0);
    __syncthreads();
    for (int u = threadIdx.x; u < rows * D; u += LR_TPB) xs[u] = X[t0 * D + u];
    for (int u = threadIdx.x; u < rows; u += LR_TPB) ys[u] = y[t0 + u];
    __syncthreads();
    if (mine) {
      for (int i = 0; i < rows; ++i) {
        float z = 0.0f;
#pragma unroll
        for (int k = 0; k < D; ++k) z = fmaf(bt[k], xs[i * D + k], z);
        const float yi = ys[i];
        const float sp = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
        acc += sp - yi * z;
        const float r = 1.0f / (1.0f + expf(-z)) - yi;
#pragma unroll
        for (int k = 0; k < D; ++k) g[k] = fmaf(r, xs[i * D + k], g[k]);
      }
    }
  }
  if (p < P) {
    part_lik[blockIdx.y * P + p] = acc;
#pragma unroll
    for (int k = 0; k < D; ++k) part_grad[(blockIdx.y * P + p) * D + k] = g[k];
  }
}

__global__ void k_logreg_reduce(const float *part_lik, const float *part_grad, int64_t P, int D, int chunks,
                                float *lik, float *grad) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
    float a = 0.0f;
    for (int c = 0; c < chunks; ++c) a += part_lik[c * P + p];
    lik[p] = a;
    for (int k = 0; k < D; ++k) {
      float s = 0.0f;
      for (int c = 0; c < chunks; ++c) s += part_grad[(c * P + p) * D + k];
      grad[p * D + k] = s;
    }
  }
}

int logreg_chunks(int64_t P, int64_t n_data) {
  const int64_t bx = (P + LR_TPB - 1) / LR_TPB;
  int64_t c = (4 * kNumSMs + bx - 1) / bx;
  if (c < 1) c = 1;
  if (c > 64) c = 64;
  const int64_t max_c = (n_data + LR_ROWS - 1) / LR_ROWS;
  return (int)(c < max_c ? c : max_c);
}

size_t logreg_f32_workspace(int64_t P, int64_t n_data, int d) {
  const int c = logreg_chunks(P, n_data);
  Carver cv(nullptr);
  cv.take<float>((size_t)c * P);
  cv.take<float>((size_t)c * P * d);
  return cv.bytes();
}

template <int D>
int logreg_f32(const float *X, const float *y, int64_t n_data, const float *beta, int64_t P, const int32_t *active,
               int N, float *lik, float *grad, void *ws, size_t ws_bytes, cudaStream_t s) {
  const int chunks = logreg_chunks(P, n_data);
  Carver cv(ws);
  float *pl = cv.take<float>((size_t)chunks * P);
  float *pg = cv.take<float>((size_t)chunks * P * D);
  if (cv.bytes() > ws_bytes) return ERR_WORKSPACE;
  const int64_t chunk = (((n_data + chunks - 1) / chunks + LR_ROWS - 1) / LR_ROWS) * LR_ROWS;
  const dim3 grid((unsigned)((P + LR_TPB - 1) / LR_TPB), (unsigned)((n_data + chunk - 1) / chunk));
  k_logreg_f32<D><<<grid, LR_TPB, 0, s>>>(X, y, n_data, chunk, beta, P, active, N ? N : (int)P, pl, pg);
  int st = launch_status();
  if (st) return st;
  k_logreg_reduce<<<grid_for(P, 256), 256, 0, s>>>(pl, pg, P, D, (int)grid.y, lik, grad);
  return launch_status();
}

#define MGB_SMC_D_DISPATCH(FN, ...)          \
  switch (d) {                                \
    case 2: return FN<2>(__VA_ARGS__);        \
    case 3: return FN<3>(__VA_ARGS__);        \
    case 5: return FN<5>(__VA_ARGS__);        \
    case 10: return FN<10>(__VA_ARGS__);      \
    case 20: return FN<20>(__VA_ARGS__);      \
    case 50: return FN<50>(__VA_ARGS__);      \
    default: return ERR_UNSUPPORTED;          \
  }

// ------------------------------------------------------------ SMC kernels
// jax's split(k)[i] for a 2-way split
__device__ __forceinline__ void split2(uint32_t k0, uint32_t k1, int i, uint32_t &o0, uint32_t &o1) {
  split_at(k0, k1, 2, (uint64_t)i, o0, o1);
}

// normal(key, (D,)) in jax's counter layout
template <int D>
__device__ __forceinline__ void normal_vec(uint32_t k0, uint32_t k1, float (&e)[D]) {
  uint32_t b[D];
  bits_vec<D>(k0, k1, b);
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(b[j]);
}

// prior draws and the key schedule of the sampler's startup; msplit is the key
// split of the MCMC sampler's startup (Underdamped 3, RandomWalk 2)
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_smc_prior(SMCView v, const uint32_t *keys_in, float scale, int msplit) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P) return;
  const int b = (int)(p / v.N), j = (int)(p % v.N);
  const uint32_t k0 = keys_in[2 * b], k1 = keys_in[2 * b + 1];
  uint32_t e0, e1, s0, s1, a0, a1;
  split2(k0, k1, 0, e0, e1);
  split2(k0, k1, 1, s0, s1);
  split_at(s0, s1, (uint64_t)v.N, (uint64_t)j, a0, a1);
  float e[D];
  normal_vec<D>(a0, a1, e);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    v.beta[p * D + k] = __fmul_rn(e[k], scale);
    v.ms[p * D + k] = 0.0f;  // Underdamped.startup: momenta = zeros(d)
  }
  if (j == 0) {
    uint32_t f0, f1, g0, g1;
    split_at(e0, e1, 2 * (uint64_t)v.N + 1, 2 * (uint64_t)v.N, f0, f1);  // split(key, 2N + 1)[-1]
    split_at(f0, f1, (uint64_t)msplit, 0, g0, g1);                       // the MCMC sampler's startup
    v.key[2 * b] = g0;
    v.key[2 * b + 1] = g1;
    v.tau[b] = 0.0f;
    v.ess[b] = (float)v.N;
    v.logz[b] = 0.0;
    v.iter[b] = 0;
    v.active[b] = 1;
    v.resampled[b] = 1;  // the first adapt starts from zero log-weights
  }
}

// iteration start: resampling decision, particle keys, the next sampler key
__global__ void __launch_bounds__(SMC_TPB) k_smc_keys(SMCView v, float thr_resample, int msplit) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P) return;
  const int b = (int)(p / v.N), j = (int)(p % v.N);
  if (!v.active[b]) return;
  const uint32_t k0 = v.key[2 * b], k1 = v.key[2 * b + 1];
  const uint64_t nk = (uint64_t)v.N + 2;
  uint32_t a0, a1, c0, c1;
  split_at(k0, k1, nk, (uint64_t)j, a0, a1);
  split_at(a0, a1, (uint64_t)msplit, 0, c0, c1);  // the MCMC sampler's startup in forward_proposal
  v.pkey[2 * p] = c0;
  v.pkey[2 * p + 1] = c1;
  v.alpha[p] = 0.0f;
  if (j == 0) {
    v.resampled[b] = v.ess[b] <= __fmul_rn(thr_resample, (float)v.N) ? 1 : 0;
    uint32_t r0, r1, n0, n1;
    split_at(k0, k1, nk, (uint64_t)v.N, r0, r1);
    split_at(k0, k1, nk, (uint64_t)v.N + 1, n0, n1);
    v.rkey[2 * b] = r0;
    v.rkey[2 * b + 1] = r1;
    v.key_next[2 * b] = n0;
    v.key_next[2 * b + 1] = n1;
  }
}

// systematic ancestors per posterior, fixed-point prefixes in shared memory
__global__ void __launch_bounds__(ADAPT_TPB) k_smc_resample(SMCView v) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float red[ADAPT_TPB / 32];
  __shared__ unsigned long long wtot[ADAPT_TPB / 32];
  const int b = blockIdx.x, N = v.N, tg = threadIdx.x;
  int32_t *anc = v.anc + (int64_t)b * N;
  if (!v.active[b] || !v.resampled[b]) {
    for (int k = tg; k < N; k += ADAPT_TPB) anc[k] = k;
    return;
  }
  const float *lw = v.lw + (int64_t)b * N;
  float m = -INFINITY;
  int bad = 0;
  for (int k = tg; k < N; k += ADAPT_TPB) {
    const float x = lw[k];
    bad |= (x != x) || (x == INFINITY);
    m = fmaxf(m, x);
  }
  const float M = block_max<ADAPT_TPB>(m, red);
  bad = __syncthreads_or(bad) || !(M > -INFINITY);
  if (bad) {
    for (int k = tg; k < N; k += ADAPT_TPB) anc[k] = 0;
    return;
  }
  uint64_t *C = (uint64_t *)smem;
  const float wscale = __int_as_float((weight_shift(N) + 127) << 23);
  const int lane = tg & 31, wcta = tg >> 5;
  const uint64_t Q = group_scan(C, N, ADAPT_TPB / 32, wcta, lane, wcta, wtot, 1, ADAPT_TPB,
                                [&](int j) { return quantise_weight(lw[j], M, wscale); });
  const uint32_t r = bits_at(v.rkey[2 * b], v.rkey[2 * b + 1], 1, 0);
  group_systematic_fill(C, N, Q, r >> 9, ~0ull / (uint64_t)N, anc, tg, ADAPT_TPB);
}

// the reference's categorical resampling per posterior (random.categorical(key, lw, (N,)),
// smc.py:61-71): a_k = argmax_i gumbel(bits(key, N N)[k N + i]) + lw_i, first maximum, NaN
// ignored (as k_categorical); one warp per output (per output pair for even N), grid (., B)
__global__ void __launch_bounds__(256) k_smc_categorical(SMCView v) {
  const int b = blockIdx.y, N = v.N, lane = threadIdx.x & 31;
  int32_t *anc = v.anc + (int64_t)b * N;
  const int64_t warp = (blockIdx.x * 256LL + threadIdx.x) >> 5, nwarps = ((int64_t)gridDim.x * 256) >> 5;
  if (!v.active[b] || !v.resampled[b]) {
    for (int64_t k = blockIdx.x * 256LL + threadIdx.x; k < N; k += (int64_t)gridDim.x * 256) anc[k] = (int32_t)k;
    return;
  }
  const float *lw = v.lw + (int64_t)b * N;
  const uint32_t k0 = v.rkey[2 * b], k1 = v.rkey[2 * b + 1];
  const uint64_t tot = (uint64_t)N * (uint64_t)N;
  if (N % 2 == 0) {
    // elements (k, i) and (k + N/2, i) are the two halves of one cipher call (counters k N + i
    // and k N + i + N^2/2): one warp takes the row pair, one call per column
    const int64_t half = N >> 1;
    const uint64_t h = tot >> 1;
    for (int64_t k = warp; k < half; k += nwarps) {
      float best0 = -INFINITY, best1 = -INFINITY;
      int64_t bi0 = N, bi1 = N;
      for (int64_t i = lane; i < N; i += 32) {
        const uint64_t c = (uint64_t)k * (uint64_t)N + (uint64_t)i;
        uint32_t r0, r1;
        threefry2x32(k0, k1, (uint32_t)c, (uint32_t)(c + h), r0, r1);
        const float l = lw[i];
        const float v0 = __fadd_rn(bits_to_gumbel(r0), l), v1 = __fadd_rn(bits_to_gumbel(r1), l);
        if (v0 > best0) {
          best0 = v0;
          bi0 = i;
        }
        if (v1 > best1) {
          best1 = v1;
          bi1 = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ob0 = __shfl_xor_sync(0xffffffffu, best0, o), ob1 = __shfl_xor_sync(0xffffffffu, best1, o);
        const int64_t oi0 = __shfl_xor_sync(0xffffffffu, bi0, o), oi1 = __shfl_xor_sync(0xffffffffu, bi1, o);
        if (ob0 > best0 || (ob0 == best0 && oi0 < bi0)) {
          best0 = ob0;
          bi0 = oi0;
        }
        if (ob1 > best1 || (ob1 == best1 && oi1 < bi1)) {
          best1 = ob1;
          bi1 = oi1;
        }
      }
      if (lane == 0) {
        anc[k] = (int32_t)(bi0 < N ? bi0 : 0);
        anc[k + half] = (int32_t)(bi1 < N ? bi1 : 0);
      }
    }
    return;
  }
  for (int64_t k = warp; k < N; k += nwarps) {
    float best = -INFINITY;
    int64_t bi = N;
    for (int64_t i = lane; i < N; i += 32) {
      const float g = bits_to_gumbel(bits_at(k0, k1, tot, (uint64_t)k * (uint64_t)N + (uint64_t)i));
      const float val = __fadd_rn(g, lw[i]);
      if (val > best) {
        best = val;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) anc[k] = (int32_t)(bi < N ? bi : 0);
  }
}

// rows of every posterior gathered by its ancestors (identity when it did not resample)
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_smc_gather(SMCView v) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P) return;
  const int64_t b = p / v.N;
  const int64_t src = b * v.N + v.anc[p];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    v.beta_p[p * D + k] = v.beta[src * D + k];
    v.glik_p[p * D + k] = v.glik[src * D + k];
    v.ms_p[p * D + k] = v.ms[src * D + k];
  }
  v.lik_p[p] = v.lik[src];
}

// grad U = beta / s^2 + tau grad l
template <int D>
__device__ __forceinline__ float grad_u(const float *bt, const float *gl, int k, float inv_s2, float tau) {
  return __fadd_rn(__fmul_rn(bt[k], inv_s2), __fmul_rn(tau, gl[k]));
}

template <int D>
__device__ __forceinline__ float prior_pot(const float *bt, float inv_s2) {
  float q = 0.0f;
#pragma unroll
  for (int k = 0; k < D; ++k) q = __fmaf_rn(bt[k], bt[k], q);
  return __fmul_rn(__fmul_rn(0.5f, q), inv_s2);
}

// Underdamped, always + first leapfrog half: (k, ka) = split(k); p0 = -m c1 + c2 normal(ka, (d,))
// (c1 = exp(-f eps), c2 = sqrt(1 - exp(-2 f eps)); c1 = 0, c2 = 1 for infinite friction);
// p_h = p0 - eps/2 grad U(beta); beta' = beta + eps p_h
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_ud_pre(SMCView v, float eps, float c1, float c2, float inv_s2) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P || !v.active[p / v.N]) return;
  const float tau = v.tau[p / v.N];
  const uint32_t k0 = v.pkey[2 * p], k1 = v.pkey[2 * p + 1];
  uint32_t n0, n1, a0, a1;
  split2(k0, k1, 0, n0, n1);
  split2(k0, k1, 1, a0, a1);
  float e[D];
  normal_vec<D>(a0, a1, e);
  const float he = eps / 2.0f;
  const float *bt = v.beta + p * D, *gl = v.glik + p * D;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const float p0 = __fadd_rn(__fmul_rn(-v.ms[p * D + k], c1), __fmul_rn(c2, e[k]));
    const float ph = __fsub_rn(p0, __fmul_rn(he, grad_u<D>(bt, gl, k, inv_s2, tau)));
    v.mom[p * D + k] = p0;
    v.phalf[p * D + k] = ph;
    v.beta_p[p * D + k] = __fadd_rn(bt[k], __fmul_rn(eps, ph));
  }
  v.pkey[2 * p] = n0;
  v.pkey[2 * p + 1] = n1;
}

// between two leapfrog steps (utils.py:121-135): p = p_h - eps/2 grad U(beta');
// p_h = p - eps/2 grad U(beta'); beta'' = beta' + eps p_h
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_lf_mid(SMCView v, float eps, float inv_s2) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P || !v.active[p / v.N]) return;
  const float tau = v.tau[p / v.N];
  const float he = eps / 2.0f;
  const float *bt = v.beta_p + p * D, *gl = v.glik_p + p * D;
  float nb[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const float g = grad_u<D>(bt, gl, k, inv_s2, tau);
    const float pm = __fsub_rn(v.phalf[p * D + k], __fmul_rn(he, g));
    const float ph = __fsub_rn(pm, __fmul_rn(he, g));
    v.phalf[p * D + k] = ph;
    nb[k] = __fadd_rn(bt[k], __fmul_rn(eps, ph));
  }
#pragma unroll
  for (int k = 0; k < D; ++k) v.beta_p[p * D + k] = nb[k];
}

// Underdamped, last leapfrog half and the Metropolis correction: p_L = p_h - eps/2 grad U(beta_L);
// alpha = min(1, exp(-U' + U - |p_L|^2/2 + |p0|^2/2)); k = split(k, L + 1)[0]; (k, ku) = split(k);
// accept if uniform(ku) < alpha: the state takes beta_L and the momenta -p_L, else keeps p0
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_ud_post(SMCView v, float eps, int L, float inv_s2) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P || !v.active[p / v.N]) return;
  const float tau = v.tau[p / v.N];
  float bo[D], bn[D], pL[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    bo[k] = v.beta[p * D + k];
    bn[k] = v.beta_p[p * D + k];
  }
  const float U = __fadd_rn(prior_pot<D>(bo, inv_s2), __fmul_rn(tau, v.lik[p]));
  const float Un = __fadd_rn(prior_pot<D>(bn, inv_s2), __fmul_rn(tau, v.lik_p[p]));
  const float he = eps / 2.0f;
  float K = 0.0f, Kn = 0.0f;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const float pn = __fsub_rn(v.phalf[p * D + k], __fmul_rn(he, grad_u<D>(bn, v.glik_p + p * D, k, inv_s2, tau)));
    const float pm = v.mom[p * D + k];
    pL[k] = pn;
    K = __fmaf_rn(pm, pm, K);
    Kn = __fmaf_rn(pn, pn, Kn);
  }
  K = __fmul_rn(0.5f, K);
  Kn = __fmul_rn(0.5f, Kn);
  float alpha = expf(__fadd_rn(__fsub_rn(__fadd_rn(-Un, U), Kn), K));
  alpha = alpha != alpha ? 0.0f : fminf(1.0f, alpha);
  const uint32_t k0 = v.pkey[2 * p], k1 = v.pkey[2 * p + 1];
  uint32_t q0, q1, n0, n1, u0, u1;
  split_at(k0, k1, (uint64_t)L + 1, 0, q0, q1);
  split2(q0, q1, 0, n0, n1);
  split2(q0, q1, 1, u0, u1);
  const float u = bits_to_unit(bits_at(u0, u1, 1, 0));
  if (u < alpha) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      v.beta[p * D + k] = bn[k];
      v.glik[p * D + k] = v.glik_p[p * D + k];
      v.ms[p * D + k] = -pL[k];
    }
    v.lik[p] = v.lik_p[p];
  } else {
#pragma unroll
    for (int k = 0; k < D; ++k) v.ms[p * D + k] = v.mom[p * D + k];
  }
  v.alpha[p] += alpha;
  v.pkey[2 * p] = n0;
  v.pkey[2 * p + 1] = n1;
}

// RandomWalk proposal (standard_mcmc.py:44-57): (k, ks, _) = split(k, 3); beta' = beta + sq normal(ks, (d,)),
// sq = sqrt(stepsize)
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_rw_pre(SMCView v, float sq) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P || !v.active[p / v.N]) return;
  const uint32_t k0 = v.pkey[2 * p], k1 = v.pkey[2 * p + 1];
  uint32_t n0, n1, a0, a1;
  split_at(k0, k1, 3, 0, n0, n1);
  split_at(k0, k1, 3, 1, a0, a1);
  float e[D];
  normal_vec<D>(a0, a1, e);
#pragma unroll
  for (int k = 0; k < D; ++k) v.beta_p[p * D + k] = __fadd_rn(v.beta[p * D + k], __fmul_rn(sq, e[k]));
  v.pkey[2 * p] = n0;
  v.pkey[2 * p + 1] = n1;
}

// RandomWalk correction: alpha = min(1, exp(-U' + U)); (k, ku) = split(k); accept if uniform(ku) < alpha
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_rw_post(SMCView v, float inv_s2) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P || !v.active[p / v.N]) return;
  const float tau = v.tau[p / v.N];
  float bo[D], bn[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    bo[k] = v.beta[p * D + k];
    bn[k] = v.beta_p[p * D + k];
  }
  const float U = __fadd_rn(prior_pot<D>(bo, inv_s2), __fmul_rn(tau, v.lik[p]));
  const float Un = __fadd_rn(prior_pot<D>(bn, inv_s2), __fmul_rn(tau, v.lik_p[p]));
  float alpha = expf(__fadd_rn(-Un, U));
  alpha = alpha != alpha ? 0.0f : fminf(1.0f, alpha);
  const uint32_t k0 = v.pkey[2 * p], k1 = v.pkey[2 * p + 1];
  uint32_t n0, n1, u0, u1;
  split2(k0, k1, 0, n0, n1);
  split2(k0, k1, 1, u0, u1);
  const float u = bits_to_unit(bits_at(u0, u1, 1, 0));
  if (u < alpha) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      v.beta[p * D + k] = bn[k];
      v.glik[p * D + k] = v.glik_p[p * D + k];
    }
    v.lik[p] = v.lik_p[p];
  }
  v.alpha[p] += alpha;
  v.pkey[2 * p] = n0;
  v.pkey[2 * p + 1] = n1;
}

// Gaussian likelihood of toy_examples.Gaussian: z = (x - m) @ Ps^T, l = 0.5 |z|^2, grad = Ps^T z
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_gauss_lik(const float *__restrict__ beta, int64_t P,
                                                        const int32_t *__restrict__ active, int N,
                                                        const float *__restrict__ m, const float *__restrict__ Ps,
                                                        float *__restrict__ lik, float *__restrict__ grad) {
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P || (active && !active[p / N])) return;
  float x[D], g[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    x[k] = __fsub_rn(beta[p * D + k], __ldg(&m[k]));
    g[k] = 0.0f;
  }
  float q = 0.0f;
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float z = __fmul_rn(x[0], __ldg(&Ps[r * D]));
#pragma unroll
    for (int k = 1; k < D; ++k) z = __fmaf_rn(x[k], __ldg(&Ps[r * D + k]), z);
    q = __fmaf_rn(z, z, q);
#pragma unroll
    for (int k = 0; k < D; ++k) g[k] = __fmaf_rn(__ldg(&Ps[r * D + k]), z, g[k]);
  }
  lik[p] = __fmul_rn(0.5f, q);
#pragma unroll
  for (int k = 0; k < D; ++k) grad[p * D + k] = g[k];
}

// after the moves: likelihood potential as the sampler derives it, (U - prior) / tau
template <int D>
__global__ void __launch_bounds__(SMC_TPB) k_smc_after(SMCView v, float inv_s2) {
  const int64_t P = (int64_t)v.B * v.N;
  const int64_t p = blockIdx.x * (int64_t)SMC_TPB + threadIdx.x;
  if (p >= P || !v.active[p / v.N]) return;
  const float tau = v.tau[p / v.N];
  float bt[D];
#pragma unroll
  for (int k = 0; k < D; ++k) bt[k] = v.beta[p * D + k];
  const float pr = prior_pot<D>(bt, inv_s2);
  const float U = __fadd_rn(pr, __fmul_rn(tau, v.lik[p]));
  v.lik_w[p] = __fdiv_rn(__fsub_rn(U, pr), tau);
}

// block-wide (max, sum e, sum e^2) of v_k = base_k - dt * l_k over one posterior
struct Lse3 {
  float lse, logess;
  int nan;
};
__device__ __forceinline__ Lse3 block_lse3(const float *base, const float *l, float dt, int N, float *red) {
  float m = -INFINITY, s1 = 0.0f, s2 = 0.0f;
  int nanf = 0;
  for (int k = threadIdx.x; k < N; k += ADAPT_TPB) {
    const float b0 = base ? base[k] : 0.0f;
    const float x = dt == 0.0f ? b0 : __fsub_rn(b0, __fmul_rn(dt, l[k]));
    online_acc(x, m, s1, s2, nanf);
  }
  const LsePartial part = block_online_partial<ADAPT_TPB>(m, s1, s2, nanf, red);
  Lse3 o;
  o.nan = part.nan;
  o.lse = part.m + logf(part.s1);
  o.logess = 2.0f * logf(part.s1) - logf(part.s2);
  if (part.nan) o.lse = o.logess = __int_as_float(0x7fc00000);
  return o;
}

// next temperature (regula falsi), log-weights, ESS, log Z; one CTA per posterior
__global__ void __launch_bounds__(ADAPT_TPB) k_smc_adapt(SMCView v, const float *ell_all, SMCParams sp, int startup) {
  __shared__ float red[ADAPT_TPB / 32];
  __shared__ int nan_count;
  const int b = blockIdx.x, N = v.N;
  if (!v.active[b]) return;
  const float *ell = ell_all + (int64_t)b * N;
  float *lw = v.lw + (int64_t)b * N;
  const int res = v.resampled[b];
  const float *base = res ? nullptr : lw;
  const float ess_res = res ? (float)N : v.ess[b];
  const float tau0 = v.tau[b];
  const float target = logf(__fmul_rn(ess_res, sp.retain));
  auto f = [&](float x) { return block_lse3(base, ell, __fsub_rn(x, tau0), N, red).logess - target; };
  const int it = startup ? 0 : v.iter[b] + 1;
  float tau1;
  if (sp.sched) {
    // temperature_schedule[extra.iter] (smc.py:118-121)
    tau1 = sp.sched[it < sp.n_sched ? it : sp.n_sched - 1];
  } else {
    // utils.bisect on [tau0, max_temperature]
    float b0 = tau0, b1 = sp.max_temp;
    float e0 = f(b0), e1 = f(b1);
    const bool incr = e1 > e0;
    for (int k = 0; k < sp.max_bisect; ++k) {
      const bool conv =
          fminf(fabsf(e0), fabsf(e1)) < sp.tol || (e0 < 0.0f && e1 < 0.0f) || (e0 > 0.0f && e1 > 0.0f);
      if (conv) break;
      const float np = __fsub_rn(b0, __fdiv_rn(__fmul_rn(e0, __fsub_rn(b1, b0)), __fsub_rn(e1, e0)));
      const float ne = f(np);
      const bool up = incr ? ne > 0.0f : ne < 0.0f;
      if (up) {
        b1 = np;
        e1 = ne;
      } else {
        b0 = np;
        e0 = ne;
      }
    }
    tau1 = fabsf(e1) < fabsf(e0) ? b1 : b0;
  }
  const float dt = __fsub_rn(tau1, tau0);
  // LSE of the log-weights the step started from, then the new log-weights (in place)
  float lse_res = logf((float)N);
  if (!res) lse_res = block_lse3(base, ell, 0.0f, N, red).lse;
  for (int k = threadIdx.x; k < N; k += ADAPT_TPB) {
    const float b0 = base ? base[k] : 0.0f;
    lw[k] = dt == 0.0f ? b0 : __fsub_rn(b0, __fmul_rn(dt, ell[k]));
  }
  __syncthreads();
  const Lse3 nw = block_lse3(lw, ell, 0.0f, N, red);
  // NaN entries of the particles (termination when more than 10 %)
  if (threadIdx.x == 0) nan_count = 0;
  __syncthreads();
  int cnt = 0;
  for (int64_t u = threadIdx.x; u < (int64_t)N * v.D; u += ADAPT_TPB) {
    const float x = v.beta[(int64_t)b * N * v.D + u];
    cnt += x != x;
  }
  cnt = warp_sum(cnt);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&nan_count, cnt);
  float asum = 0.0f;
  for (int k = threadIdx.x; k < N; k += ADAPT_TPB) asum += v.alpha[(int64_t)b * N + k];
  asum = block_sum<ADAPT_TPB, float>(asum, red);
  if (threadIdx.x == 0) {
    const double lz = startup ? (double)nw.lse - (double)lse_res : v.logz[b] + (double)nw.lse - (double)lse_res;
    const float ess = expf(nw.logess);
    v.tau[b] = tau1;
    v.ess[b] = ess;
    v.logz[b] = lz;
    v.iter[b] = it;
    if (!startup) {
      v.key[2 * b] = v.key_next[2 * b];
      v.key[2 * b + 1] = v.key_next[2 * b + 1];
    }
    const bool nan_stop = (float)nan_count / ((float)N * (float)v.D) > 0.1f;
    v.active[b] = !(tau1 >= sp.max_temp || it >= sp.max_iter || nan_stop);
    if (it < v.H) {
      v.h_tau[(int64_t)b * v.H + it] = tau1;
      v.h_logz[(int64_t)b * v.H + it] = lz;
      v.h_ess[(int64_t)b * v.H + it] = ess;
      v.h_alpha[(int64_t)b * v.H + it] = startup ? 1.0f : asum / ((float)N * (float)sp.mcmc_steps);
      v.h_res[(int64_t)b * v.H + it] = startup ? 0 : res;
    }
  }
}

// d log Z / d s (prior scale) by the Fisher identity over the final weighted
// particles: E_post[|beta|^2 / s^3 - d / s], one CTA per posterior
__global__ void __launch_bounds__(ADAPT_TPB) k_smc_prior_scale_grad(SMCView v, float s, double *out) {
  __shared__ float red[ADAPT_TPB / 32];
  __shared__ double dsum[ADAPT_TPB / 32][2];
  const int b = blockIdx.x, N = v.N, D = v.D;
  const float *lw = v.lw + (int64_t)b * N;
  float m = -INFINITY;
  for (int k = threadIdx.x; k < N; k += ADAPT_TPB) m = fmaxf(m, lw[k]);
  const float M = block_max<ADAPT_TPB>(m, red);
  double w = 0.0, wq = 0.0;
  for (int k = threadIdx.x; k < N; k += ADAPT_TPB) {
    const double e = exp((double)(lw[k] - M));
    double q = 0.0;
    for (int j = 0; j < D; ++j) {
      const double x = v.beta[((int64_t)b * N + k) * D + j];
      q += x * x;
    }
    w += e;
    wq += e * q;
  }
  w = warp_sum(w);
  wq = warp_sum(wq);
  if ((threadIdx.x & 31) == 0) {
    dsum[threadIdx.x >> 5][0] = w;
    dsum[threadIdx.x >> 5][1] = wq;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double W = 0.0, WQ = 0.0;
    for (int i = 0; i < ADAPT_TPB / 32; ++i) {
      W += dsum[i][0];
      WQ += dsum[i][1];
    }
    const double sd = (double)s;
    out[b] = WQ / W / (sd * sd * sd) - (double)D / sd;
  }
}

// ------------------------------------------------------------ host side
SMCView carve_smc(Carver &c, int B, int N, int d, int H) {
  const size_t P = (size_t)B * N;
  SMCView v{};
  v.B = B;
  v.N = N;
  v.D = d;
  v.H = H;
  v.beta = c.take<float>(P * d);
  v.beta_p = c.take<float>(P * d);
  v.glik = c.take<float>(P * d);
  v.glik_p = c.take<float>(P * d);
  v.mom = c.take<float>(P * d);
  v.phalf = c.take<float>(P * d);
  v.ms = c.take<float>(P * d);
  v.ms_p = c.take<float>(P * d);
  v.lik = c.take<float>(P);
  v.lik_p = c.take<float>(P);
  v.lik_w = c.take<float>(P);
  v.lw = c.take<float>(P);
  v.alpha = c.take<float>(P);
  v.pkey = c.take<uint32_t>(2 * P);
  v.anc = c.take<int32_t>(P);
  v.tau = c.take<float>(B);
  v.ess = c.take<float>(B);
  v.logz = c.take<double>(B);
  v.key = c.take<uint32_t>(2 * (size_t)B);
  v.key_next = c.take<uint32_t>(2 * (size_t)B);
  v.rkey = c.take<uint32_t>(2 * (size_t)B);
  v.iter = c.take<int32_t>(B);
  v.active = c.take<int32_t>(B);
  v.resampled = c.take<int32_t>(B);
  v.h_tau = c.take<float>((size_t)B * H);
  v.h_logz = c.take<double>((size_t)B * H);
  v.h_ess = c.take<float>((size_t)B * H);
  v.h_alpha = c.take<float>((size_t)B * H);
  v.h_res = c.take<int32_t>((size_t)B * H);
  return v;
}

static bool smc_cfg_ok(const mgb_smc_logreg_config *cfg) {
  if (!(cfg && cfg->B >= 1 && cfg->N >= 2 && cfg->N <= MGB_SMC_MAX_N && cfg->d >= 1 && cfg->mcmc_steps >= 1 &&
        cfg->max_iter >= 1 && cfg->max_bisection_iter >= 0 && cfg->prior_scale > 0.0f && cfg->stepsize > 0.0f &&
        (cfg->precision == MGB_PREC_FP32 || cfg->precision == MGB_PREC_BF16)))
    return false;
  if (cfg->move != MGB_MOVE_UNDERDAMPED && cfg->move != MGB_MOVE_RANDOM_WALK) return false;
  if (cfg->leapfrog_steps < 0 || cfg->prior_sample_scale < 0.0f || cfg->n_schedule < 0) return false;
  if (cfg->n_schedule > 0 && !cfg->schedule_dev) return false;
  if (cfg->resampling != MGB_RESAMPLE_SYSTEMATIC && cfg->resampling != MGB_RESAMPLE_CATEGORICAL) return false;
  if (cfg->likelihood == MGB_LIK_GAUSSIAN) return cfg->gauss_mean_dev && cfg->gauss_prec_sqrt_dev;
  return cfg->likelihood == MGB_LIK_LOGISTIC;
}

static bool smc_gauss(const mgb_smc_logreg_config *cfg) { return cfg->likelihood == MGB_LIK_GAUSSIAN; }

static size_t smc_pot_ws(const mgb_smc_logreg_config *cfg, int64_t n_data) {
  if (smc_gauss(cfg)) return 0;
  const int64_t P = (int64_t)cfg->B * cfg->N;
  size_t a = logreg_f32_workspace(P, n_data, cfg->d);
  if (cfg->precision == MGB_PREC_BF16) {
    const size_t b = logreg_tc_workspace(P, n_data, cfg->d);
    if (b > a) a = b;
  }
  return a;
}

template <int D>
static int gauss_lik(const mgb_smc_logreg_config *cfg, const float *beta, int64_t P, const int32_t *active, int N,
                     float *lik, float *grad, cudaStream_t s) {
  k_gauss_lik<D><<<(unsigned)((P + SMC_TPB - 1) / SMC_TPB), SMC_TPB, 0, s>>>(
      beta, P, active, N, cfg->gauss_mean_dev, cfg->gauss_prec_sqrt_dev, lik, grad);
  return launch_status();
}

static int smc_potential(const mgb_smc_logreg_config *cfg, const SMCData &dat, const float *beta, float *lik,
                         float *grad, const int32_t *active, void *ws, size_t ws_bytes, cudaStream_t s) {
  const int64_t P = (int64_t)cfg->B * cfg->N;
  const int d = cfg->d;
  if (smc_gauss(cfg)) MGB_SMC_D_DISPATCH(gauss_lik, cfg, beta, P, active, cfg->N, lik, grad, s);
  if (cfg->precision == MGB_PREC_BF16)
    return logreg_tc(dat, beta, P, active, cfg->N, lik, grad, ws, ws_bytes, s);
  MGB_SMC_D_DISPATCH(logreg_f32, dat.X, dat.y, dat.n_data, beta, P, active, cfg->N, lik, grad, ws, ws_bytes, s);
}

static SMCParams smc_params(const mgb_smc_logreg_config *cfg) {
  return SMCParams{cfg->ess_threshold_retain, cfg->max_temperature, cfg->bisection_tol, cfg->max_bisection_iter,
                   cfg->max_iter,           cfg->mcmc_steps,      cfg->n_schedule > 0 ? cfg->schedule_dev : nullptr,
                   cfg->n_schedule};
}

// key split of the MCMC sampler's startup: Underdamped (key, prior, lik) = split(key, 3), RandomWalk 2
static int smc_msplit(const mgb_smc_logreg_config *cfg) { return cfg->move == MGB_MOVE_RANDOM_WALK ? 2 : 3; }

template <int D>
static int smc_init_t(const mgb_smc_logreg_config *cfg, const SMCData &dat, const uint32_t *keys, SMCView v,
                      void *pws, size_t pws_bytes, cudaStream_t s) {
  const int64_t P = (int64_t)cfg->B * cfg->N;
  const unsigned g = (unsigned)((P + SMC_TPB - 1) / SMC_TPB);
  const float sscale = cfg->prior_sample_scale > 0.0f ? cfg->prior_sample_scale : cfg->prior_scale;
  k_smc_prior<D><<<g, SMC_TPB, 0, s>>>(v, keys, sscale, smc_msplit(cfg));
  int st = launch_status();
  if (st) return st;
  if ((st = smc_potential(cfg, dat, v.beta, v.lik, v.glik, nullptr, pws, pws_bytes, s))) return st;
  if (cudaMemsetAsync(v.alpha, 0, sizeof(float) * P, s) != cudaSuccess) return ERR_CUDA;
  k_smc_adapt<<<cfg->B, ADAPT_TPB, 0, s>>>(v, v.lik, smc_params(cfg), 1);
  return launch_status();
}

template <int D>
static int smc_step_t(const mgb_smc_logreg_config *cfg, const SMCData &dat, SMCView v, void *pws, size_t pws_bytes,
                      cudaStream_t s) {
  const int64_t P = (int64_t)cfg->B * cfg->N;
  const unsigned g = (unsigned)((P + SMC_TPB - 1) / SMC_TPB);
  const float inv_s2 = (float)(1.0 / ((double)cfg->prior_scale * (double)cfg->prior_scale));
  int st;
  k_smc_keys<<<g, SMC_TPB, 0, s>>>(v, cfg->ess_threshold_resample, smc_msplit(cfg));
  if ((st = launch_status())) return st;
  if (cfg->resampling == MGB_RESAMPLE_CATEGORICAL) {
    const unsigned gx = (unsigned)std::min<int64_t>(((int64_t)cfg->N * 32 + 255) / 256, 1024);
    k_smc_categorical<<<dim3(gx, (unsigned)cfg->B), 256, 0, s>>>(v);
  } else {
    const size_t rs_smem = sizeof(uint64_t) * (size_t)cfg->N;
    if (cudaFuncSetAttribute(k_smc_resample, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs_smem) !=
        cudaSuccess)
      return ERR_UNSUPPORTED;
    k_smc_resample<<<cfg->B, ADAPT_TPB, rs_smem, s>>>(v);
  }
  if ((st = launch_status())) return st;
  k_smc_gather<D><<<g, SMC_TPB, 0, s>>>(v);
  if ((st = launch_status())) return st;
  // the gathered rows become the state (pointer swap inside the view copy)
  SMCView w = v;
  std::swap(w.beta, w.beta_p);
  std::swap(w.glik, w.glik_p);
  std::swap(w.lik, w.lik_p);
  std::swap(w.ms, w.ms_p);
  const float eps = cfg->stepsize;
  const bool rw = cfg->move == MGB_MOVE_RANDOM_WALK;
  const int L = cfg->leapfrog_steps > 0 ? cfg->leapfrog_steps : 1;
  // OU refresh factors exp(-f eps), sqrt(1 - exp(-2 f eps)) in float32 (standard_mcmc.py:112-118)
  float c1 = 0.0f, c2 = 1.0f;
  if (!rw && cfg->friction > 0.0f && std::isfinite(cfg->friction)) {
    c1 = std::exp(-cfg->friction * eps);
    c2 = std::sqrt(1.0f - std::exp(-2.0f * cfg->friction * eps));
  }
  const float sq = std::sqrt(eps);
  for (int m = 0; m < cfg->mcmc_steps; ++m) {
    if (rw) {
      k_rw_pre<D><<<g, SMC_TPB, 0, s>>>(w, sq);
    } else {
      k_ud_pre<D><<<g, SMC_TPB, 0, s>>>(w, eps, c1, c2, inv_s2);
    }
    if ((st = launch_status())) return st;
    if ((st = smc_potential(cfg, dat, w.beta_p, w.lik_p, w.glik_p, w.active, pws, pws_bytes, s))) return st;
    for (int l = 1; !rw && l < L; ++l) {
      k_lf_mid<D><<<g, SMC_TPB, 0, s>>>(w, eps, inv_s2);
      if ((st = launch_status())) return st;
      if ((st = smc_potential(cfg, dat, w.beta_p, w.lik_p, w.glik_p, w.active, pws, pws_bytes, s))) return st;
    }
    if (rw) {
      k_rw_post<D><<<g, SMC_TPB, 0, s>>>(w, inv_s2);
    } else {
      k_ud_post<D><<<g, SMC_TPB, 0, s>>>(w, eps, L, inv_s2);
    }
    if ((st = launch_status())) return st;
  }
  k_smc_after<D><<<g, SMC_TPB, 0, s>>>(w, inv_s2);
  if ((st = launch_status())) return st;
  k_smc_adapt<<<cfg->B, ADAPT_TPB, 0, s>>>(w, w.lik_w, smc_params(cfg), 0);
  if ((st = launch_status())) return st;
  // the state lives in the swapped buffers now: copy back so the layout stays fixed
  if (cudaMemcpyAsync(v.beta, w.beta, sizeof(float) * P * D, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(v.glik, w.glik, sizeof(float) * P * D, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(v.lik, w.lik, sizeof(float) * P, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(v.ms, w.ms, sizeof(float) * P * D, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  return OK;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

size_t mgb_logreg_workspace(int64_t P, int64_t n_data, int32_t d, int precision) {
  if (P < 1 || n_data < 1 || d < 1) return 0;
  size_t a = logreg_f32_workspace(P, n_data, d);
  if (precision == MGB_PREC_BF16) {
    const size_t b = logreg_tc_workspace(P, n_data, d);
    if (b > a) a = b;
  }
  return a;
}

int mgb_logreg_potential_grad(const float *X, const float *y, int64_t n_data, int32_t d, const float *beta,
                              int64_t P, float *lik, float *grad, int precision, const void *Xbf16, void *ws,
                              size_t ws_bytes, void *stream) {
  if (!X || !y || !beta || !lik || !grad || n_data < 1 || d < 1 || P < 1 || !ws) return ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == MGB_PREC_BF16) {
    if (!Xbf16) return ERR_BAD_ARG;
    SMCData dat{X, y, (const uint16_t *)Xbf16, n_data, d};
    return logreg_tc(dat, beta, P, nullptr, (int)P, lik, grad, ws, ws_bytes, s);
  }
  if (precision != MGB_PREC_FP32) return ERR_BAD_ARG;
  MGB_SMC_D_DISPATCH(logreg_f32, X, y, n_data, beta, P, nullptr, 0, lik, grad, ws, ws_bytes, s);
}

int mgb_smc_logreg_prior_scale_grad(const mgb_smc_logreg_config *cfg, void *ws, double *out, void *stream) {
  if (!smc_cfg_ok(cfg) || !ws || !out) return ERR_BAD_ARG;
  Carver c(ws);
  const SMCView v = carve_smc(c, cfg->B, cfg->N, cfg->d, cfg->max_iter + 1);
  k_smc_prior_scale_grad<<<cfg->B, ADAPT_TPB, 0, (cudaStream_t)stream>>>(v, cfg->prior_scale, out);
  return launch_status();
}

size_t mgb_smc_logreg_workspace(const mgb_smc_logreg_config *cfg, int64_t n_data) {
  if (!smc_cfg_ok(cfg) || n_data < 1) return 0;
  Carver c(nullptr);
  carve_smc(c, cfg->B, cfg->N, cfg->d, cfg->max_iter + 1);
  c.take<unsigned char>(smc_pot_ws(cfg, n_data));
  return c.bytes();
}

int mgb_smc_logreg_views(const mgb_smc_logreg_config *cfg, void *ws, mgb_smc_views *out) {
  if (!smc_cfg_ok(cfg) || !ws || !out) return ERR_BAD_ARG;
  Carver c(ws);
  const SMCView v = carve_smc(c, cfg->B, cfg->N, cfg->d, cfg->max_iter + 1);
  out->value = v.beta;
  out->log_weight = v.lw;
  out->likelihood_potential = v.lik;
  out->temperature = v.tau;
  out->ess = v.ess;
  out->log_norm_constant = v.logz;
  out->iter = v.iter;
  out->active = v.active;
  out->hist_temperature = v.h_tau;
  out->hist_log_norm_constant = v.h_logz;
  out->hist_ess = v.h_ess;
  out->hist_alpha = v.h_alpha;
  out->hist_resampled = v.h_res;
  out->hist_len = v.H;
  return OK;
}

static int smc_setup(const mgb_smc_logreg_config *cfg, const float *X, const float *y, const void *Xbf16,
                     int64_t n_data, void *ws, size_t ws_bytes, SMCData &dat, SMCView &v, void *&pws,
                     size_t &pws_bytes) {
  if (!smc_cfg_ok(cfg) || (!smc_gauss(cfg) && (!X || !y)) || n_data < 1 || !ws) return ERR_BAD_ARG;
  if (cfg->precision == MGB_PREC_BF16 && !smc_gauss(cfg) && !Xbf16) return ERR_BAD_ARG;
  if (ws_bytes < mgb_smc_logreg_workspace(cfg, n_data)) return ERR_WORKSPACE;
  Carver c(ws);
  v = carve_smc(c, cfg->B, cfg->N, cfg->d, cfg->max_iter + 1);
  pws_bytes = smc_pot_ws(cfg, n_data);
  pws = c.take<unsigned char>(pws_bytes);
  dat = SMCData{X, y, (const uint16_t *)Xbf16, n_data, cfg->d};
  return OK;
}

int mgb_smc_logreg_init(const mgb_smc_logreg_config *cfg, const float *X, const float *y, const void *Xbf16,
                        int64_t n_data, const uint32_t *keys, void *ws, size_t ws_bytes, void *stream) {
  SMCData dat;
  SMCView v;
  void *pws;
  size_t pb;
  int st = smc_setup(cfg, X, y, Xbf16, n_data, ws, ws_bytes, dat, v, pws, pb);
  if (st) return st;
  if (!keys) return ERR_BAD_ARG;
  const int d = cfg->d;
  MGB_SMC_D_DISPATCH(smc_init_t, cfg, dat, keys, v, pws, pb, (cudaStream_t)stream);
}

int mgb_smc_logreg_step(const mgb_smc_logreg_config *cfg, const float *X, const float *y, const void *Xbf16,
                        int64_t n_data, void *ws, size_t ws_bytes, void *stream) {
  SMCData dat;
  SMCView v;
  void *pws;
  size_t pb;
  int st = smc_setup(cfg, X, y, Xbf16, n_data, ws, ws_bytes, dat, v, pws, pb);
  if (st) return st;
  const int d = cfg->d;
  MGB_SMC_D_DISPATCH(smc_step_t, cfg, dat, v, pws, pb, (cudaStream_t)stream);
}

}  // extern "C"
