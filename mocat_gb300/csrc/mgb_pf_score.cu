// Score d log p(y) / d theta of the linear-Gaussian state-space model by
// Fisher's identity, smoothed along the bootstrap filter by PaRIS.
//
// Reference path: the log-likelihood mocat estimates with
// run_particle_filter_for_marginals (mocat/src/ssm/filtering.py:255-324) and
// BootstrapFilter (:142-170) on a TimeHomogenousLinearGaussian model
// (mocat/src/ssm/linear_gaussian/linear_gaussian.py: transition_sample :86-94,
// likelihood_potential :118-128) with H = I and diagonal covariances;
// theta = (A = F, log q, log r), q_k = Lq_kk^2, r_k = P_kk^-2.
//
// Fisher's identity: score = E[ sum_t h_t(x_{t-1}, x_t) + sum_t g_t(x_t) | y ] with
//   h_t:  dA_kl = e_k x_{t-1,l} / q_k,   dlog q_k = e_k^2 / (2 q_k) - 1/2,   e = x_t - A x_{t-1}
//   g_t:  dlog r_k = (y_t,k - x_t,k)^2 / (2 r_k) - 1/2.
// PaRIS (Olsson and Westerborn, Bernoulli 23(3), 2017) carries per particle
//   tau_t^i = (1/K) sum_k [tau_{t-1}^{J_k} + h_t(x_{t-1}^{J_k}, x_t^i)] + g_t(x_t^i)
// forward with the filter and returns sum_i W_{T-1}^i tau_{T-1}^i, a consistent
// estimate of the score whose variance grows linearly in T (the statistic is
// smoothed, not traced along the collapsing genealogy).  The K backward draws
// follow Dau and Chopin ("On backward smoothing algorithms", Ann. Statist.
// 51(5), 2023): J_1 is the particle's own ancestor, an exact draw of the
// backward kernel, and each further draw continues an independent-Metropolis
// chain over the step's source population m = 0..n-1 (the resampled particles
// x_{t-1}^{a_m}; all x_{t-1}^m with their weights when the step did not
// resample) with target exp(lb_m) f(x_t^i | mu_m), mu_m = A x_{t-1}^{src(m)},
// and uniform proposals, L proposals per draw.  Cost is O(n (K - 1) L) per
// step, with no O(n^2) term and no rejection loop of random length.
//
// Random numbers: proposal s = (k - 1) L + l of particle i at step t uses
// (w0, w1) = threefry2x32(smoothing_key, (i, (t << 12) | s)); the proposed
// index is (w0 n) >> 32 (exactly uniform for n a power of two, otherwise
// within n 2^-32 of uniform) and E = exponential(w1); the chain moves when
// (lf' - lf) + E > 0.  Every float operation is rounded as written (explicit
// _rn intrinsics) in the same order as the oracle's restatement.
//
// Layout: particles dimension-major as in the filter; the proposal rows
// (mu_m, lb_m) and the statistics tau are particle-major so that a randomly
// indexed row is a few contiguous 32-byte sectors.
#include <cmath>
#include <type_traits>

#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_kernels.cuh"
#include "mgb_lg.cuh"
#include "mgb_pf_common.cuh"
#include "mgb_lg_kernels.cuh"
#include "mgb_systematic.cuh"

namespace mgb {

constexpr int SC_TPB = 128;
constexpr int SC_KMAX = 4;

template <int D>
struct ScoreDims {
  static constexpr int P = D * D + 2 * D;       // statistics per particle
  static constexpr int TS = (P + 3) / 4 * 4;     // tau row stride (floats, 16-byte rows)
  static constexpr int MS = (D / 4 + 1) * 4;     // proposal row stride: mu (D), lb, padding
};

template <int D>
struct ScoreP {
  float F[D * D];
  float iq[D], half_iq[D], half_ir[D];  // 1/q, 1/(2q), 1/(2r), rounded from float64
};

struct ScoreStep {
  const float *x;         // x_t (D, n)
  const float *xprev;     // x_{t-1} (D, n)
  const float *mu;        // (n, MS) proposal rows
  const int32_t *anc;     // a_t (n), used when *res
  const int32_t *res;     // device flag: step t resampled
  const float *tau_prev;  // (n, TS)
  float *tau;             // (n, TS)
  const float *y;         // y_t (D)
  const uint32_t *skey;   // smoothing key (2 words)
  int32_t *draws;         // (n, K) backward draws of this step, or null
  uint32_t t;
  int K, L;
  float invK;
};

// lf = lb - 1/2 sum_r (x_r - mu_r)^2 / q_r
template <int D>
__device__ __forceinline__ float score_lf(const ScoreP<D> &c, const float (&xi)[D], const float *row) {
  float s2 = 0.0f;
#pragma unroll
  for (int r = 0; r < D; ++r) {
    const float dr = __fsub_rn(xi[r], row[r]);
    s2 = __fmaf_rn(__fmul_rn(dr, dr), c.iq[r], s2);
  }
  return __fsub_rn(row[D], __fmul_rn(0.5f, s2));
}

template <int D>
__device__ __forceinline__ void load_row(const float *base, float (&row)[ScoreDims<D>::MS]) {
  const float4 *p = reinterpret_cast<const float4 *>(base);
#pragma unroll
  for (int j = 0; j < ScoreDims<D>::MS / 4; ++j) {
    const float4 v = __ldg(p + j);
    row[4 * j] = v.x;
    row[4 * j + 1] = v.y;
    row[4 * j + 2] = v.z;
    row[4 * j + 3] = v.w;
  }
}

// tau_0^i: zero dA / dlog q blocks, g_0(x_0^i) in the dlog r block
template <int D>
__global__ void __launch_bounds__(SC_TPB) k_score_init(const __grid_constant__ ScoreP<D> c, int64_t n,
                                                        const float *__restrict__ x, const float *__restrict__ y0,
                                                        float *__restrict__ tau) {
  using S = ScoreDims<D>;
  const int64_t i = blockIdx.x * (int64_t)SC_TPB + threadIdx.x;
  if (i >= n) return;
  float *to = tau + i * S::TS;
  for (int q = 0; q < S::TS; ++q) to[q] = 0.0f;
#pragma unroll
  for (int r = 0; r < D; ++r) {
    const float dr = __fsub_rn(__ldg(&y0[r]), x[r * n + i]);
    to[D * D + D + r] = __fsub_rn(__fmul_rn(__fmul_rn(dr, dr), c.half_ir[r]), 0.5f);
  }
}

// one PaRIS step: backward draws, then tau_t^i
// KK = the number of backward draws, a compile-time constant so that only KK draws'
// residuals and sources occupy registers
template <int D, int KK>
__device__ __forceinline__ void score_step_body(const ScoreP<D> &c, int64_t n, const ScoreStep &a) {
  using S = ScoreDims<D>;
  constexpr int B = 4;  // independent proposals evaluated together (their loads overlap)
  const int64_t i = blockIdx.x * (int64_t)SC_TPB + threadIdx.x;
  if (i >= n) return;
  const int res = *a.res;
  const uint32_t k0 = __ldg(&a.skey[0]), k1 = __ldg(&a.skey[1]);
  float xi[D];
#pragma unroll
  for (int r = 0; r < D; ++r) xi[r] = a.x[r * n + i];
  int64_t mk[KK];
  {
    float row[S::MS];
    load_row<D>(a.mu + i * S::MS, row);
    float lcur = score_lf<D>(c, xi, row);
    int64_t cur = i;
    mk[0] = i;
#pragma unroll
    for (int k = 1; k < KK; ++k) {
      if (k < KK) {
        for (int l0 = 0; l0 < a.L; l0 += B) {
          float lp[B], E[B];
          int64_t prop[B];
#pragma unroll
          for (int b = 0; b < B; ++b) {
            const int l = l0 + b;
            uint32_t w0 = 0u, w1 = 0u;
            if (l < a.L)
              threefry2x32(k0, k1, (uint32_t)i, (a.t << 12) | (uint32_t)((k - 1) * a.L + l), w0, w1);
            prop[b] = (int64_t)(((uint64_t)w0 * (uint64_t)n) >> 32);
            E[b] = bits_to_exponential(w1);
            float pr[S::MS];
            load_row<D>(a.mu + prop[b] * S::MS, pr);
            lp[b] = score_lf<D>(c, xi, pr);
          }
#pragma unroll
          for (int b = 0; b < B; ++b) {
            if (l0 + b < a.L && __fadd_rn(__fsub_rn(lp[b], lcur), E[b]) > 0.0f) {
              cur = prop[b];
              lcur = lp[b];
            }
          }
        }
      }
      mk[k] = cur;
    }
  }
  // the draws' source particles, their states and residuals
  float e[KK][D], v[KK][D], xp[KK][D];
  const float4 *tp[KK];
#pragma unroll
  for (int k = 0; k < KK; ++k) {
    const int kk = k < KK ? k : 0;
    const int64_t j = res ? (int64_t)__ldg(&a.anc[mk[kk]]) : mk[kk];
    if (a.draws && k < KK) a.draws[i * KK + k] = (int32_t)j;
    float row[S::MS];
    load_row<D>(a.mu + mk[kk] * S::MS, row);
#pragma unroll
    for (int r = 0; r < D; ++r) {
      xp[k][r] = __ldg(&a.xprev[r * n + j]);
      e[k][r] = __fsub_rn(xi[r], row[r]);
      v[k][r] = __fmul_rn(e[k][r], c.iq[r]);
    }
    tp[k] = reinterpret_cast<const float4 *>(a.tau_prev + j * S::TS);
  }
  float hr[D];
#pragma unroll
  for (int r = 0; r < D; ++r) {
    const float dr = __fsub_rn(__ldg(&a.y[r]), xi[r]);
    hr[r] = __fsub_rn(__fmul_rn(__fmul_rn(dr, dr), c.half_ir[r]), 0.5f);
  }
  float4 *to = reinterpret_cast<float4 *>(a.tau + i * S::TS);
#pragma unroll
  for (int q4 = 0; q4 < S::TS / 4; ++q4) {
    float4 pv[KK];
#pragma unroll
    for (int k = 0; k < KK; ++k) pv[k] = k < KK ? __ldg(tp[k] + q4) : make_float4(0.f, 0.f, 0.f, 0.f);
    float out[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int q = 4 * q4 + u;
      float acc = 0.0f;
      if (q < D * D) {
        const int r = q / D, col = q % D;
#pragma unroll
        for (int k = 0; k < KK; ++k)
          if (k < KK) {
            const float tv = u == 0 ? pv[k].x : u == 1 ? pv[k].y : u == 2 ? pv[k].z : pv[k].w;
            acc = __fadd_rn(acc, tv);
            acc = __fadd_rn(acc, __fmul_rn(v[k][r], xp[k][col]));
          }
        out[u] = __fmul_rn(acc, a.invK);
      } else if (q < D * D + D) {
        const int r = q - D * D;
#pragma unroll
        for (int k = 0; k < KK; ++k)
          if (k < KK) {
            const float tv = u == 0 ? pv[k].x : u == 1 ? pv[k].y : u == 2 ? pv[k].z : pv[k].w;
            acc = __fadd_rn(acc, tv);
            acc = __fadd_rn(acc, __fsub_rn(__fmul_rn(__fmul_rn(e[k][r], e[k][r]), c.half_iq[r]), 0.5f));
          }
        out[u] = __fmul_rn(acc, a.invK);
      } else if (q < S::P) {
        const int r = q - D * D - D;
#pragma unroll
        for (int k = 0; k < KK; ++k)
          if (k < KK) {
            const float tv = u == 0 ? pv[k].x : u == 1 ? pv[k].y : u == 2 ? pv[k].z : pv[k].w;
            acc = __fadd_rn(acc, tv);
          }
        out[u] = __fadd_rn(__fmul_rn(acc, a.invK), hr[r]);
      } else {
        out[u] = 0.0f;
      }
    }
    to[q4] = make_float4(out[0], out[1], out[2], out[3]);
  }
}

template <int D, int KK>
__global__ void __launch_bounds__(SC_TPB) k_score_step(const __grid_constant__ ScoreP<D> c, int64_t n,
                                                        const ScoreStep a) {
  score_step_body<D, KK>(c, n, a);
}

// partial[b][q] = sum over block b's particles of W_i tau_i[q] (float64, fixed order)
constexpr int SC_SUM_TPB = 128;
constexpr int SC_SUM_CHUNK = 256;
template <int D>
__global__ void __launch_bounds__(SC_SUM_TPB) k_score_wsum(int64_t n, const float *__restrict__ lw,
                                                            const double *lse, const float *__restrict__ tau,
                                                            double *__restrict__ partial) {
  using S = ScoreDims<D>;
  __shared__ double w_s[SC_SUM_CHUNK];
  const double L = *lse;
  double acc[(S::P + SC_SUM_TPB - 1) / SC_SUM_TPB];
#pragma unroll
  for (int j = 0; j < (S::P + SC_SUM_TPB - 1) / SC_SUM_TPB; ++j) acc[j] = 0.0;
  for (int64_t c0 = (int64_t)blockIdx.x * SC_SUM_CHUNK; c0 < n; c0 += (int64_t)gridDim.x * SC_SUM_CHUNK) {
    const int cnt = n - c0 < SC_SUM_CHUNK ? (int)(n - c0) : SC_SUM_CHUNK;
    __syncthreads();
    for (int u = threadIdx.x; u < cnt; u += SC_SUM_TPB) w_s[u] = exp((double)lw[c0 + u] - L);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < (S::P + SC_SUM_TPB - 1) / SC_SUM_TPB; ++j) {
      const int q = threadIdx.x + j * SC_SUM_TPB;
      if (q < S::P)
        for (int u = 0; u < cnt; ++u) acc[j] += w_s[u] * (double)tau[(c0 + u) * S::TS + q];
    }
  }
#pragma unroll
  for (int j = 0; j < (S::P + SC_SUM_TPB - 1) / SC_SUM_TPB; ++j) {
    const int q = threadIdx.x + j * SC_SUM_TPB;
    if (q < S::P) partial[(size_t)blockIdx.x * S::P + q] = acc[j];
  }
}

__global__ void k_score_sum(const double *partial, int nb, int P, float *grad) {
  for (int q = threadIdx.x; q < P; q += blockDim.x) {
    double acc = 0.0;
    for (int b = 0; b < nb; ++b) acc += partial[(size_t)b * P + q];
    grad[q] = (float)acc;
  }
}

constexpr int SC_SUM_BLOCKS = 2 * kNumSMs;

template <int D>
static ScoreP<D> make_score_params(const LGP<D, D> &p) {
  ScoreP<D> c;
  for (int i = 0; i < D * D; ++i) c.F[i] = p.F[i];
  for (int r = 0; r < D; ++r) {
    const double q = (double)p.Lq[r * D + r] * (double)p.Lq[r * D + r];
    const double pr = (double)p.P[r * D + r];
    c.iq[r] = (float)(1.0 / q);
    c.half_iq[r] = (float)(0.5 / q);
    c.half_ir[r] = (float)(0.5 * pr * pr);
  }
  return c;
}

struct ScoreWs {
  RunWs run;
  float *tau_a, *tau_b;
  float *mu;
  double *partial;
  double *lse4;
  void *lse_ws;
  size_t lse_bytes;
};

static ScoreWs carve_score(Carver &c, int64_t n, int64_t T, int d, int scheme) {
  ScoreWs w;
  w.run = carve_run(c, n, T, d, scheme, true, true, true);
  const int P = d * d + 2 * d, TS = (P + 3) / 4 * 4, MS = (d / 4 + 1) * 4;
  w.tau_a = c.take<float>((size_t)n * TS);
  w.tau_b = c.take<float>((size_t)n * TS);
  w.mu = c.take<float>((size_t)n * MS);
  w.partial = c.take<double>((size_t)SC_SUM_BLOCKS * P);
  w.lse4 = c.take<double>(4);
  w.lse_bytes = mgb_lse_ess_workspace(n);
  w.lse_ws = c.take<unsigned char>(w.lse_bytes);
  return w;
}

template <int D>
static int score_lg(const mgb_lg_model *m, int64_t n, int64_t T, const uint32_t *key, const uint32_t *skey,
                    const float *y, float thr, int scheme, int K, int L, void *ws, size_t ws_bytes, double *logz_out,
                    float *grad_out, int32_t *resampled_out, int32_t *draws_out, cudaStream_t s) {
  using S = ScoreDims<D>;
  const LGP<D, D> p = pack_lg<D, D>(m);
  if (!p.lq_diag || !p.p_diag || !p.h_eye) return ERR_UNSUPPORTED;
  const ScoreP<D> c = make_score_params<D>(p);
  Carver cv(ws);
  ScoreWs w = carve_score(cv, n, T, D, scheme);
  if (cv.bytes() > ws_bytes) return ERR_WORKSPACE;
  RunWs &r = w.run;
  int st;
  if (cudaMemsetAsync(r.st, 0, sizeof(PFState), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(r.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(r.res_hist, 0, sizeof(int32_t) * (T + 1), s) != cudaSuccess) return ERR_CUDA;
  if ((st = reset_resample(r.rws, s))) return st;
  if ((st = launch_setup_keys(key, T, r.keys, s))) return st;
  PFCtl ctl;
  ctl.parts = r.parts;
  ctl.counter = r.counter;
  ctl.st = r.st;
  ctl.ess_hist = r.ess_hist;
  ctl.res_hist = r.res_hist;
  ctl.rctl = r.rws.ctl;
  ctl.rstatus = r.rws.status;
  ctl.rstatus2 = r.rws.status2;
  ctl.ntiles = (int)r.rws.ntiles;
  ctl.thr_n = thr * (float)n;
  ctl.logn = log((double)n);
  ctl.logz_out = nullptr;
  const unsigned grid = (unsigned)((n + PF_TPB - 1) / PF_TPB);
  const unsigned grid2 = (unsigned)((n / 2 + PF_TPB - 1) / PF_TPB);
  const unsigned gs = (unsigned)((n + SC_TPB - 1) / SC_TPB);
  float *xa = r.xa, *xb = r.xb, *la = r.la, *lb = r.lb;
  float *ta = w.tau_a, *tb = w.tau_b;
  k_lg_init<D, D, true><<<grid, PF_TPB, 0, s>>>(p, n, r.keys, y, xa, la, ctl);
  k_score_init<D><<<gs, SC_TPB, 0, s>>>(c, n, xa, y, ta);
  if ((st = launch_status())) return st;
  ScoreStep a;
  a.skey = skey;
  a.K = K;
  a.L = L;
  a.invK = (float)(1.0 / K);
  for (int64_t t = 1; t < T; ++t) {
    if ((st = launch_resample(la, n, scheme, &r.st->M, r.keys + 2 * t, 0, 0u, r.res_hist + t, r.rws, r.anc, nullptr,
                              s)))
      return st;
    // the propagate also writes the proposal rows mu (F x of each particle's source and its
    // carried log-weight) that the backward draws of this step read
    if (n % 2 == 0)
      k_lg_step2<D, D, true, S::MS><<<grid2, PF_TPB, 0, s>>>(p, n, r.keys + 2 * t, y + (size_t)t * D, xa, r.anc, la,
                                                             r.res_hist + t, xb, lb, ctl, t, w.mu);
    else
      k_lg_step<D, D, true, S::MS><<<grid, PF_TPB, 0, s>>>(p, n, r.keys + 2 * t, y + (size_t)t * D, xa, r.anc, la,
                                                           r.res_hist + t, xb, lb, ctl, t, w.mu);
    a.x = xb;
    a.xprev = xa;
    a.mu = w.mu;
    a.anc = r.anc;
    a.res = r.res_hist + t;
    a.tau_prev = ta;
    a.tau = tb;
    a.y = y + (size_t)t * D;
    a.draws = draws_out ? draws_out + (size_t)t * n * K : nullptr;
    a.t = (uint32_t)t;
    switch (K) {
      case 1: k_score_step<D, 1><<<gs, SC_TPB, 0, s>>>(c, n, a); break;
      case 2: k_score_step<D, 2><<<gs, SC_TPB, 0, s>>>(c, n, a); break;
      case 3: k_score_step<D, 3><<<gs, SC_TPB, 0, s>>>(c, n, a); break;
      default: k_score_step<D, 4><<<gs, SC_TPB, 0, s>>>(c, n, a); break;
    }
    if ((st = launch_status())) return st;
    float *tp = xa; xa = xb; xb = tp;
    tp = la; la = lb; lb = tp;
    tp = ta; ta = tb; tb = tp;
  }
  if ((st = launch_finish(r.st, r.res_hist, T, logz_out, resampled_out, s))) return st;
  if ((st = mgb_lse_ess(la, n, w.lse4, w.lse_ws, w.lse_bytes, s))) return st;
  const int64_t nchunks = (n + SC_SUM_CHUNK - 1) / SC_SUM_CHUNK;
  const unsigned nb = (unsigned)(nchunks < SC_SUM_BLOCKS ? nchunks : SC_SUM_BLOCKS);
  k_score_wsum<D><<<nb, SC_SUM_TPB, 0, s>>>(n, la, w.lse4 + 1, ta, w.partial);
  k_score_sum<<<1, 128, 0, s>>>(w.partial, (int)nb, S::P, grad_out);
  return launch_status();
}


// ------------------------------------------------------------ many filters
// mgb_pf_lg_score_batch runs B filters, each with its own workspace slab of
// `ws` bytes laid out exactly as filter 0's, so every per-filter pointer is
// filter 0's plus b * ws bytes.  The per-step kernels take filter 0's pointers
// and run one filter per grid row (blockIdx.y = b) with the same code as the
// single-filter kernels; the observations and the model are shared.
template <class T>
__device__ __forceinline__ T *slab(T *p, int64_t off) {
  return p ? reinterpret_cast<T *>(reinterpret_cast<char *>(const_cast<typename std::remove_const<T>::type *>(p)) +
                                   off)
           : nullptr;
}
__device__ __forceinline__ PFCtl slab_ctl(const PFCtl &c, int64_t o) {
  PFCtl r = c;
  r.parts = slab(c.parts, o);
  r.counter = slab(c.counter, o);
  r.st = slab(c.st, o);
  r.ess_hist = slab(c.ess_hist, o);
  r.res_hist = slab(c.res_hist, o);
  r.rctl = slab(c.rctl, o);
  r.rstatus = slab(c.rstatus, o);
  r.rstatus2 = slab(c.rstatus2, o);
  r.logz_out = nullptr;
  return r;
}

__global__ void __launch_bounds__(SCAN_TPB) k_tile_sums_b(const float *lw, int64_t n, const float *Mptr,
                                                           const uint32_t *key, const int32_t *flag, ResampleCtl *ctl,
                                                           uint64_t *tile_pfx, uint64_t *units, int64_t ws) {
  const int64_t o = (int64_t)blockIdx.y * ws;
  tile_sums_body(slab(lw, o), n, slab(Mptr, o), slab(key, o), 0, 0u, slab(flag, o), slab(ctl, o), slab(tile_pfx, o),
                 slab(units, o));
}
__global__ void __launch_bounds__(SCAN_TPB) k_systematic_b(const float *lw, int64_t n, const float *Mptr,
                                                            const int32_t *flag, const ResampleCtl *ctl,
                                                            const uint64_t *tile_pfx, const uint64_t *units,
                                                            int32_t *anc, int64_t ws) {
  const int64_t o = (int64_t)blockIdx.y * ws;
  systematic_body(slab(lw, o), n, slab(Mptr, o), slab(flag, o), slab(ctl, o), slab(tile_pfx, o), slab(units, o),
                  slab(anc, o), nullptr);
}
template <int D>
__global__ void __launch_bounds__(PF_TPB, 2) k_lg_step2_b(const __grid_constant__ LGP<D, D> p, int64_t n,
                                                           const uint32_t *key, const float *y_t, const float *x_prev,
                                                           const int32_t *anc, const float *lw_prev,
                                                           const int32_t *res_flag, float *x_new, float *lw_new,
                                                           PFCtl ctl, int64_t t, float *mu, int64_t ws) {
  const int64_t o = (int64_t)blockIdx.y * ws;
  lg_step2_body<D, D, true, ScoreDims<D>::MS>(p, n, slab(key, o), y_t, slab(x_prev, o), slab(anc, o),
                                              slab(lw_prev, o), slab(res_flag, o), slab(x_new, o), slab(lw_new, o),
                                              slab_ctl(ctl, o), t, slab(mu, o));
}
template <int D, int KK>
__global__ void __launch_bounds__(SC_TPB) k_score_step_b(const __grid_constant__ ScoreP<D> c, int64_t n,
                                                          const ScoreStep a0, int64_t ws) {
  const int64_t o = (int64_t)blockIdx.y * ws;
  ScoreStep a = a0;
  a.x = slab(a0.x, o);
  a.xprev = slab(a0.xprev, o);
  a.mu = slab(a0.mu, o);
  a.anc = slab(a0.anc, o);
  a.res = slab(a0.res, o);
  a.tau_prev = slab(a0.tau_prev, o);
  a.tau = slab(a0.tau, o);
  a.skey = slab(a0.skey, o);
  a.draws = nullptr;
  score_step_body<D, KK>(c, n, a);
}

// a filter's slab: the single-filter workspace plus its smoothing key
static size_t score_slab_bytes(int64_t n, int64_t T, int d) {
  Carver c(nullptr);
  carve_score(c, n, T, d, MGB_RESAMPLE_SYSTEMATIC);
  c.take<uint32_t>(2);
  return c.bytes();
}

template <int D>
static int score_lg_batch(const mgb_lg_model *m, int64_t n, int64_t T, int64_t B, const uint32_t *keys,
                          const uint32_t *skeys, const float *y, float thr, int K, int L, void *ws, size_t ws_bytes,
                          double *logz_out, float *grad_out, cudaStream_t s) {
  using S = ScoreDims<D>;
  const LGP<D, D> p = pack_lg<D, D>(m);
  if (!p.lq_diag || !p.p_diag || !p.h_eye) return ERR_UNSUPPORTED;
  const ScoreP<D> c = make_score_params<D>(p);
  const int64_t W = (int64_t)score_slab_bytes(n, T, D);
  if ((size_t)(W * B) > ws_bytes) return ERR_WORKSPACE;
  char *base = (char *)ws;
  Carver c0(base);
  ScoreWs w0 = carve_score(c0, n, T, D, MGB_RESAMPLE_SYSTEMATIC);
  uint32_t *sk0 = c0.take<uint32_t>(2);
  RunWs &r0 = w0.run;
  int st;
  auto ctl_of = [&](const RunWs &r) {
    PFCtl ctl;
    ctl.parts = r.parts;
    ctl.counter = r.counter;
    ctl.st = r.st;
    ctl.ess_hist = r.ess_hist;
    ctl.res_hist = r.res_hist;
    ctl.rctl = r.rws.ctl;
    ctl.rstatus = r.rws.status;
    ctl.rstatus2 = r.rws.status2;
    ctl.ntiles = (int)r.rws.ntiles;
    ctl.thr_n = thr * (float)n;
    ctl.logn = log((double)n);
    ctl.logz_out = nullptr;
    return ctl;
  };
  const unsigned grid = (unsigned)((n + PF_TPB - 1) / PF_TPB);
  const unsigned grid2 = (unsigned)((n / 2 + PF_TPB - 1) / PF_TPB);
  const unsigned gs = (unsigned)((n + SC_TPB - 1) / SC_TPB);
  const unsigned tiles = (unsigned)((n + SCAN_TILE - 1) / SCAN_TILE);
  // per-filter set-up: state, keys, initial particles and statistics
  for (int64_t b = 0; b < B; ++b) {
    Carver cb(base + b * W);
    ScoreWs w = carve_score(cb, n, T, D, MGB_RESAMPLE_SYSTEMATIC);
    uint32_t *skb = cb.take<uint32_t>(2);
    RunWs &r = w.run;
    if (cudaMemsetAsync(r.st, 0, sizeof(PFState), s) != cudaSuccess) return ERR_CUDA;
    if (cudaMemsetAsync(r.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
    if (cudaMemsetAsync(r.res_hist, 0, sizeof(int32_t) * (T + 1), s) != cudaSuccess) return ERR_CUDA;
    if ((st = reset_resample(r.rws, s))) return st;
    if (cudaMemcpyAsync(skb, skeys + 2 * b, 2 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return ERR_CUDA;
    if ((st = launch_setup_keys(keys + 2 * b, T, r.keys, s))) return st;
    k_lg_init<D, D, true><<<grid, PF_TPB, 0, s>>>(p, n, r.keys, y, r.xa, r.la, ctl_of(r));
    k_score_init<D><<<gs, SC_TPB, 0, s>>>(c, n, r.xa, y, w.tau_a);
    if ((st = launch_status())) return st;
  }
  const PFCtl ctl0 = ctl_of(r0);
  float *xa = r0.xa, *xb = r0.xb, *la = r0.la, *lb = r0.lb;
  float *ta = w0.tau_a, *tb = w0.tau_b;
  ScoreStep a;
  a.skey = sk0;
  a.K = K;
  a.L = L;
  a.invK = (float)(1.0 / K);
  a.draws = nullptr;
  const dim3 gB(1, (unsigned)B);
  for (int64_t t = 1; t < T; ++t) {
    k_tile_sums_b<<<dim3(tiles, (unsigned)B), SCAN_TPB, 0, s>>>(la, n, &r0.st->M, r0.keys + 2 * t, r0.res_hist + t,
                                                                r0.rws.ctl, r0.rws.status, r0.rws.status2, W);
    k_systematic_b<<<dim3(2 * tiles, (unsigned)B), SCAN_TPB, 0, s>>>(la, n, &r0.st->M, r0.res_hist + t, r0.rws.ctl,
                                                                     r0.rws.status, r0.rws.status2, r0.anc, W);
    k_lg_step2_b<D><<<dim3(grid2, (unsigned)B), PF_TPB, 0, s>>>(p, n, r0.keys + 2 * t, y + (size_t)t * D, xa, r0.anc,
                                                                la, r0.res_hist + t, xb, lb, ctl0, t, w0.mu, W);
    a.x = xb;
    a.xprev = xa;
    a.mu = w0.mu;
    a.anc = r0.anc;
    a.res = r0.res_hist + t;
    a.tau_prev = ta;
    a.tau = tb;
    a.y = y + (size_t)t * D;
    a.t = (uint32_t)t;
    switch (K) {
      case 1: k_score_step_b<D, 1><<<dim3(gs, (unsigned)B), SC_TPB, 0, s>>>(c, n, a, W); break;
      case 2: k_score_step_b<D, 2><<<dim3(gs, (unsigned)B), SC_TPB, 0, s>>>(c, n, a, W); break;
      case 3: k_score_step_b<D, 3><<<dim3(gs, (unsigned)B), SC_TPB, 0, s>>>(c, n, a, W); break;
      default: k_score_step_b<D, 4><<<dim3(gs, (unsigned)B), SC_TPB, 0, s>>>(c, n, a, W); break;
    }
    if ((st = launch_status())) return st;
    float *tp = xa; xa = xb; xb = tp;
    tp = la; la = lb; lb = tp;
    tp = ta; ta = tb; tb = tp;
  }
  (void)gB;
  // per-filter results: log Z, then the weighted sum of the statistics
  const int64_t off_la = (char *)la - base, off_ta = (char *)ta - base;
  for (int64_t b = 0; b < B; ++b) {
    Carver cb(base + b * W);
    ScoreWs w = carve_score(cb, n, T, D, MGB_RESAMPLE_SYSTEMATIC);
    const float *lab = (const float *)(base + b * W + off_la);
    const float *tab = (const float *)(base + b * W + off_ta);
    if ((st = launch_finish(w.run.st, w.run.res_hist, T, logz_out ? logz_out + b : nullptr, nullptr, s))) return st;
    if ((st = mgb_lse_ess(lab, n, w.lse4, w.lse_ws, w.lse_bytes, s))) return st;
    const int64_t nchunks = (n + SC_SUM_CHUNK - 1) / SC_SUM_CHUNK;
    const unsigned nb = (unsigned)(nchunks < SC_SUM_BLOCKS ? nchunks : SC_SUM_BLOCKS);
    k_score_wsum<D><<<nb, SC_SUM_TPB, 0, s>>>(n, lab, w.lse4 + 1, tab, w.partial);
    k_score_sum<<<1, 128, 0, s>>>(w.partial, (int)nb, S::P, grad_out + b * S::P);
    if ((st = launch_status())) return st;
  }
  return OK;
}
}  // namespace mgb

using namespace mgb;

extern "C" {

size_t mgb_pf_lg_score_batch_workspace(int64_t n, int64_t T, int32_t d, int64_t B) {
  if (n < 1 || T < 1 || d < 1 || B < 1) return 0;
  return score_slab_bytes(n, T, d) * (size_t)B;
}

int mgb_pf_lg_score_batch(const mgb_lg_model *m, int64_t n, int64_t T, int64_t B, const uint32_t *keys,
                          const uint32_t *smoothing_keys, const float *y, float ess_threshold, int32_t backward_draws,
                          int32_t mcmc_steps, void *ws, size_t ws_bytes, double *log_z, float *grad, void *stream) {
  if (!m || !m->F || !m->Lq || !m->H || !m->P || !m->C0 || !m->m0 || n < 2 || n > 0x7FFFFFFFll || T < 1 ||
      T > (1 << 20) || B < 1 || B > 65535 || !keys || !smoothing_keys || !y || !ws || !grad || backward_draws < 1 ||
      backward_draws > SC_KMAX || mcmc_steps < 0 || (int64_t)(backward_draws - 1) * mcmc_steps > 4096)
    return ERR_BAD_ARG;
  if (m->dy != m->d || n % 2 != 0) return ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
#define MGB_SCORE_BATCH_CASE(DD)                                                                               \
  case DD:                                                                                                     \
    return score_lg_batch<DD>(m, n, T, B, keys, smoothing_keys, y, ess_threshold, backward_draws, mcmc_steps, ws, \
                              ws_bytes, log_z, grad, s);
  switch (m->d) {
    MGB_SCORE_BATCH_CASE(1)
    MGB_SCORE_BATCH_CASE(2)
    MGB_SCORE_BATCH_CASE(3)
    MGB_SCORE_BATCH_CASE(4)
    MGB_SCORE_BATCH_CASE(5)
    MGB_SCORE_BATCH_CASE(8)
    MGB_SCORE_BATCH_CASE(10)
    default: return ERR_UNSUPPORTED;
  }
#undef MGB_SCORE_BATCH_CASE
}

size_t mgb_pf_lg_score_workspace(int64_t n, int64_t T, int32_t d) {
  if (n < 1 || T < 1 || d < 1) return 0;
  Carver c(nullptr);
  carve_score(c, n, T, d, MGB_RESAMPLE_MULTINOMIAL);
  return c.bytes();
}

int mgb_pf_lg_score(const mgb_lg_model *m, int64_t n, int64_t T, const uint32_t *key, const uint32_t *smoothing_key,
                    const float *y, float ess_threshold, int scheme, int32_t backward_draws, int32_t mcmc_steps,
                    void *ws, size_t ws_bytes, double *log_z, float *grad, int32_t *resampled, int32_t *draws,
                    void *stream) {
  if (!m || !m->F || !m->Lq || !m->H || !m->P || !m->C0 || !m->m0 || n < 2 || n > 0x7FFFFFFFll || T < 1 ||
      T > (1 << 20) || !key || !smoothing_key || !y || !ws || !grad || backward_draws < 1 ||
      backward_draws > SC_KMAX || mcmc_steps < 0 || (int64_t)(backward_draws - 1) * mcmc_steps > 4096)
    return ERR_BAD_ARG;
  if (m->dy != m->d) return ERR_UNSUPPORTED;
  if (scheme != MGB_RESAMPLE_SYSTEMATIC && scheme != MGB_RESAMPLE_MULTINOMIAL) return ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
#define MGB_SCORE_CASE(DD)                                                                                        \
  case DD:                                                                                                       \
    return score_lg<DD>(m, n, T, key, smoothing_key, y, ess_threshold, scheme, backward_draws, mcmc_steps, ws,   \
                        ws_bytes, log_z, grad, resampled, draws, s);
  switch (m->d) {
    MGB_SCORE_CASE(1)
    MGB_SCORE_CASE(2)
    MGB_SCORE_CASE(3)
    MGB_SCORE_CASE(4)
    MGB_SCORE_CASE(5)
    MGB_SCORE_CASE(8)
    MGB_SCORE_CASE(10)
    default: return ERR_UNSUPPORTED;
  }
#undef MGB_SCORE_CASE
}

}  // extern "C"
