// ABC-SMC: MetropolisedABCSMCSampler with random-walk ABC moves on the ABC
// linear-Gaussian scenario, B posteriors at once.
//
// Reference: MetropolisedABCSMCSampler (mocat/src/abc/smc.py:101-245) driven as
// mocat.run (mocat/src/sample.py:110-148) through SMCSampler.update
// (mocat/src/transport/smc.py:61-100); RandomWalkABC (mocat/src/abc/mcmc.py:59-103)
// with the Metropolis correction (mocat/src/mcmc/metropolis.py:48-70); scenario
// LinearGaussian (mocat/src/abc/scenarios/linear_gaussian.py):
//   prior_sample       m0 + C0 normal(key, (d,))
//   prior_potential    0.5 |(x - m0) P0|^2 + c0
//   likelihood_sample  H x + L normal(key, (dy,))
//   distance           sqrt(sum((sim - data)^2))            (abc/abc.py:36-39)
// Weights are 0 / -inf (distance <= threshold); ESS = exp(log(#alive)).
//
// Key flow (per posterior, extra.random_key = e):
//   startup   (e, sub) = split(e); x_i from split(sub, N)[i]; prior potentials
//             consume split(e, N + 1) (e <- last); simulations use
//             split(e, N + 1)[i] (e <- last)
//   iteration keys = split(e, N + 2): keys[N] resamples, keys[i] drives particle
//             i's moves, e <- keys[N + 1]; per move k <- split(k)[0];
//             (k, k1, k2, k3) = split(k, 4); proposal x + sqrt(s) normal(k1, (d,)),
//             simulation with k3; (k, ku) = split(k); accept if uniform(ku) < alpha,
//             alpha = min(1, exp(pp_old - pp_new) [dist_new < threshold]).
// Differences from the reference, by design: resampling is systematic (the
// reference draws random.categorical); the stepsize variance and the mean
// acceptance are float64 sums in a fixed order (the reference: float32 in XLA's
// order), so the oracle can mirror them exactly.
//
// Layout: per posterior b, particles particle-major value[(b N + i) d + j];
// distance, prior potential, alpha, log-weight (B N).  Per iteration three
// launches: k_abc_resample (one block per posterior), k_abc_move (one thread per
// particle), k_abc_adapt (one block per posterior: quantile by radix select,
// ESS, mean acceptance, stepsize, termination, history).
#include "mgb_internal.cuh"

namespace mgb {

constexpr int ABC_TPB = 1024;
constexpr int ABC_MOVE_TPB = 256;

template <int D, int DY>
struct ABCP {
  float m0[D], C0[D * D], P0[D * D], H[DY * D], L[DY * DY], data[DY];
  float c0;
  uint32_t one;
};

struct ABCCtl {
  int32_t N, mcmc_steps, max_iter, n_schedule, adapt_stepsize, hist_len;
  float retain, resample_thr, term_alpha, fixed_stepsize;
};

// workspace views of one sampler (all arrays cover the B posteriors)
struct ABCWs {
  float *value, *value_tmp;       // (B N, d)
  float *dist, *dist_tmp;         // (B N)
  float *pp, *pp_tmp;             // (B N) prior potentials
  float *alpha, *alpha_tmp;       // (B N)
  float *lw;                      // (B N) 0 / -inf
  int32_t *rank_idx;              // (B N) index of the alive particle of each rank
  uint32_t *key;                  // (B, 2) extra.random_key
  float *stepsize;                // (B, d)
  float *threshold, *ess, *alpha_mean;  // (B)
  int32_t *iter, *active, *resampled;   // (B)
  float *hist_thr, *hist_ess, *hist_alpha;  // (B, hist_len)
  int32_t *hist_res;              // (B, hist_len)
  float *schedule;                // (n_schedule)
};

inline ABCWs carve_abc(Carver &c, int64_t B, int64_t N, int d, int hist_len, int n_schedule) {
  ABCWs w;
  const size_t BN = (size_t)(B * N);
  w.value = c.take<float>(BN * d);
  w.value_tmp = c.take<float>(BN * d);
  w.dist = c.take<float>(BN);
  w.dist_tmp = c.take<float>(BN);
  w.pp = c.take<float>(BN);
  w.pp_tmp = c.take<float>(BN);
  w.alpha = c.take<float>(BN);
  w.alpha_tmp = c.take<float>(BN);
  w.lw = c.take<float>(BN);
  w.rank_idx = c.take<int32_t>(BN);
  w.key = c.take<uint32_t>(2 * (size_t)B);
  w.stepsize = c.take<float>((size_t)B * d);
  w.threshold = c.take<float>((size_t)B);
  w.ess = c.take<float>((size_t)B);
  w.alpha_mean = c.take<float>((size_t)B);
  w.iter = c.take<int32_t>((size_t)B);
  w.active = c.take<int32_t>((size_t)B);
  w.resampled = c.take<int32_t>((size_t)B);
  w.hist_thr = c.take<float>((size_t)B * hist_len);
  w.hist_ess = c.take<float>((size_t)B * hist_len);
  w.hist_alpha = c.take<float>((size_t)B * hist_len);
  w.hist_res = c.take<int32_t>((size_t)B * hist_len);
  w.schedule = c.take<float>((size_t)(n_schedule > 0 ? n_schedule : 1));
  return w;
}

template <int D, int DY>
__device__ __forceinline__ float abc_prior_potential(const ABCP<D, DY> &p, const float (&x)[D]) {
  float diff[D];
#pragma unroll
  for (int j = 0; j < D; ++j) diff[j] = __fsub_rn(x[j], p.m0[j]);
  float quad = 0.0f;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    float v = __fmul_rn(diff[0], p.P0[k]);
#pragma unroll
    for (int j = 1; j < D; ++j) v = __fmaf_rn(diff[j], p.P0[j * D + k], v);
    quad = k == 0 ? __fmul_rn(v, v) : __fmaf_rn(v, v, quad);
  }
  return __fadd_rn(__fmul_rn(0.5f, quad), p.c0);
}

// distance of a simulation H x + L normal(key, (dy,)) to the data
template <int D, int DY>
__device__ __forceinline__ float abc_sim_distance(const ABCP<D, DY> &p, const float (&x)[D], uint32_t k0,
                                                  uint32_t k1) {
  uint32_t b[DY];
  bits_vec<DY>(k0, k1, b, p.one);
  float e[DY];
#pragma unroll
  for (int j = 0; j < DY; ++j) e[j] = bits_to_normal(b[j]);
  float s = 0.0f;
#pragma unroll
  for (int r = 0; r < DY; ++r) {
    float hx = __fmul_rn(p.H[r * D], x[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) hx = __fmaf_rn(p.H[r * D + k], x[k], hx);
    float le = __fmul_rn(p.L[r * DY], e[0]);
#pragma unroll
    for (int k = 1; k < DY; ++k) le = __fmaf_rn(p.L[r * DY + k], e[k], le);
    const float dv = __fsub_rn(__fadd_rn(hx, le), p.data[r]);
    s = r == 0 ? __fmul_rn(dv, dv) : __fadd_rn(s, __fmul_rn(dv, dv));
  }
  return __fsqrt_rn(s);
}

// ---------------------------------------------------------------- startup
// one thread per particle: prior draw, prior potential, simulation, distance
template <int D, int DY>
__global__ void __launch_bounds__(ABC_MOVE_TPB) k_abc_init(const __grid_constant__ ABCP<D, DY> p, int64_t B,
                                                            int64_t N, const uint32_t *keys, ABCWs w) {
  const int64_t g = blockIdx.x * (int64_t)ABC_MOVE_TPB + threadIdx.x;
  if (g >= B * N) return;
  const int64_t b = g / N, i = g - b * N;
  uint32_t e0, e1, s0, s1;
  split2(keys[2 * b], keys[2 * b + 1], e0, e1, s0, s1);  // extra.random_key, sub_key of the prior draws
  uint32_t a0, a1;
  split_at(s0, s1, (uint64_t)N, (uint64_t)i, a0, a1);
  uint32_t bits[D];
  bits_vec<D>(a0, a1, bits, p.one);
  float e[D], x[D];
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(bits[j]);
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float v = __fmul_rn(p.C0[r * D], e[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) v = __fmaf_rn(p.C0[r * D + k], e[k], v);
    x[r] = __fadd_rn(p.m0[r], v);
    w.value[g * D + r] = x[r];
  }
  w.pp[g] = abc_prior_potential<D, DY>(p, x);
  // the prior potentials consume split(e, N + 1); the simulations use split(e', N + 1)[i]
  uint32_t f0, f1, k0, k1;
  split_at(e0, e1, (uint64_t)N + 1, (uint64_t)N, f0, f1);
  split_at(f0, f1, (uint64_t)N + 1, (uint64_t)i, k0, k1);
  w.dist[g] = abc_sim_distance<D, DY>(p, x, k0, k1);
  w.alpha[g] = 1.0f;
  w.lw[g] = 0.0f;
  if (i == 0) {
    uint32_t z0, z1;
    split_at(f0, f1, (uint64_t)N + 1, (uint64_t)N, z0, z1);
    w.key[2 * b] = z0;
    w.key[2 * b + 1] = z1;
  }
}

// ------------------------------------------------------- block primitives
// (float)(sum / denom) of the block's per-thread partials (each a float sum in index order),
// summed in float64 in a fixed order: a shuffle-down tree per warp, warp results added in warp
// order by thread 0 (the oracle mirrors it).  Thread 0 divides once and every thread reads the
// float (the FP64 pipe is slow: a division in every thread costs more than the whole sum)
__device__ __forceinline__ float abc_block_ratio(double v, double denom, double *sm) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = sm[0];
    for (int k = 1; k < ABC_TPB / 32; ++k) s += sm[k];
    sm[32] = (double)(float)(s / denom);
  }
  __syncthreads();
  const float r = (float)sm[32];
  __syncthreads();
  return r;
}

__device__ __forceinline__ int abc_block_count(int v, int *sm) {
  v = __reduce_add_sync(0xffffffffu, (unsigned)v);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < ABC_TPB / 32; ++k) s += sm[k];
    sm[32] = s;
  }
  __syncthreads();
  const int r = sm[32];
  __syncthreads();
  return r;
}

// the rank-th smallest (0-based) of the non-negative floats v[0..n) (bit order
// = value order; NaN sorts last, as jnp.sort places it): 4 passes of 8-bit digits.  Lanes of
// a warp with the same digit add to the histogram once (__match_any_sync: the values of one
// posterior mostly share their high byte), and warp 0 finds the digit of the rank, 8 bins
// per lane
__device__ __forceinline__ float abc_block_select(const float *v, int64_t n, int64_t rank, unsigned *hist,
                                                  unsigned *res) {
  unsigned prefix = 0u, mask = 0u;
  unsigned r = (unsigned)rank;  // rank < n < 2^31
  const int lane = threadIdx.x & 31;
#pragma unroll 1
  for (int pass = 0; pass < 4; ++pass) {
    const int shift = 24 - 8 * pass;
    for (int k = threadIdx.x; k < 256; k += ABC_TPB) hist[k] = 0u;
    __syncthreads();
    for (int64_t base = threadIdx.x - lane; base < n; base += ABC_TPB) {
      const int64_t i = base + lane;
      const unsigned u = i < n ? __float_as_uint(v[i]) : 0u;
      const bool want = i < n && (u & mask) == prefix;
      const unsigned wm = __ballot_sync(0xffffffffu, want);
      if (want) {
        const unsigned bin = (u >> shift) & 255u;
        const unsigned peers = __match_any_sync(wm, bin);
        if (lane == __ffs(peers) - 1) atomicAdd(&hist[bin], (unsigned)__popc(peers));
      }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      unsigned c[8], tot = 0u;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        c[k] = hist[8 * lane + k];
        tot += c[k];
      }
      unsigned incl = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const unsigned excl = incl - tot;
      const bool mine = excl <= r && r < incl;
      if (mine) {
        unsigned cum = excl, bin = 8u * lane + 7u;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          if (r < cum + c[k]) {
            bin = 8u * lane + k;
            break;
          }
          cum += c[k];
        }
        res[0] = bin;
        res[1] = r - cum;
      }
      const unsigned all = __shfl_sync(0xffffffffu, incl, 31);
      if (__ballot_sync(0xffffffffu, mine) == 0u && lane == 0) {
        res[0] = 255u;  // no bin holds the rank (not reached: rank < n)
        res[1] = r - all;
      }
    }
    __syncthreads();
    prefix |= res[0] << shift;
    mask |= 255u << shift;
    r = res[1];
    __syncthreads();
  }
  return __uint_as_float(prefix);
}

// the (rank + 1)-th smallest given vlo, the rank-th: vlo again when more than rank + 1 values
// are <= vlo, else the smallest value above it (one pass instead of a second select)
__device__ __forceinline__ float abc_block_next(const float *v, int64_t n, int64_t rank, float vlo, int *smi,
                                                unsigned *res) {
  const unsigned ub = __float_as_uint(vlo);
  int cnt = 0;
  unsigned mn = 0xFFFFFFFFu;
  for (int64_t i = threadIdx.x; i < n; i += ABC_TPB) {
    const unsigned u = __float_as_uint(v[i]);
    if (u <= ub)
      ++cnt;
    else
      mn = min(mn, u);
  }
  mn = __reduce_min_sync(0xffffffffu, mn);
  if ((threadIdx.x & 31) == 0) res[2 + (threadIdx.x >> 5)] = mn;
  cnt = abc_block_count(cnt, smi);  // its barriers order the per-warp minima
  unsigned m = 0xFFFFFFFFu;
  for (int k = 0; k < ABC_TPB / 32; ++k) m = min(m, res[2 + k]);
  __syncthreads();
  return (int64_t)cnt > rank + 1 ? vlo : __uint_as_float(m);
}

// --------------------------------------------------------------- adapt
// MetropolisedABCSMCSampler.adapt (abc/smc.py:226-245) after startup (startup = 1)
// or after an iteration's moves
template <int D>
__global__ void __launch_bounds__(ABC_TPB) k_abc_adapt(ABCCtl ctl, ABCWs w, int startup) {
  __shared__ double smd[33];
  __shared__ int smi[33];
  __shared__ unsigned hist[256], res[2 + ABC_TPB / 32];
  const int64_t b = blockIdx.x, N = ctl.N;
  if (!startup && !w.active[b]) return;
  const int64_t off = b * N;
  const int iter = startup ? 0 : w.iter[b] + 1;
  // mean acceptance over the particles alive before the moves.  Each thread sums its values
  // in float in index order; the block adds the 1024 partials in float64 in a fixed tree (the
  // FP64 pipe is slow on this GPU, so only the combination runs on it)
  float asf_ = 0.0f;
  int ac = 0;
  for (int64_t i = threadIdx.x; i < N; i += ABC_TPB)
    if (w.lw[off + i] > -INFINITY) {
      asf_ = __fadd_rn(asf_, w.alpha[off + i]);
      ++ac;
    }
  ac = abc_block_count(ac, smi);
  const float alpha_mean = abc_block_ratio((double)asf_, (double)ac, smd);
  // next threshold: the schedule (index clamped, as jax indexing is) or the quantile
  // of the distances at retain * ess / N (jnp.quantile, linear interpolation)
  float thr;
  if (ctl.n_schedule > 0) {
    thr = w.schedule[iter < ctl.n_schedule ? iter : ctl.n_schedule - 1];
  } else {
    const float ess_prev = startup ? (float)N : w.ess[b];
    const float q = __fdiv_rn(__fmul_rn(ctl.retain, ess_prev), (float)N);
    const float pos = __fmul_rn(q, (float)(N - 1));
    const float lo = floorf(pos), hi = ceilf(pos);
    const float hw = __fsub_rn(pos, lo), lwt = __fsub_rn(1.0f, hw);
    int64_t ilo = (int64_t)fminf(fmaxf(lo, 0.0f), (float)(N - 1));
    int64_t ihi = (int64_t)fminf(fmaxf(hi, 0.0f), (float)(N - 1));
    const float vlo = abc_block_select(w.dist + off, N, ilo, hist, res);
    const float vhi = ihi == ilo ? vlo : abc_block_next(w.dist + off, N, ilo, vlo, smi, res);
    thr = __fadd_rn(__fmul_rn(vlo, lwt), __fmul_rn(vhi, hw));
  }
  // log-weights and ESS
  int alive = 0;
  for (int64_t i = threadIdx.x; i < N; i += ABC_TPB) {
    const bool a = !(w.dist[off + i] > thr);
    w.lw[off + i] = a ? 0.0f : -INFINITY;
    alive += a;
  }
  alive = abc_block_count(alive, smi);
  const float ess = alive > 0 ? expf_(logf_((float)alive)) : __int_as_float(0x7fc00000);
  // stepsize: per-dimension variance (ddof 1) of all particles / d * 2.38^2
  if (ctl.adapt_stepsize) {
    // one pass per moment over the particles' rows, a float accumulator per dimension (the
    // same per-dimension sums, in the same order, as a pass per dimension)
    float s1[D], mf[D], s2[D];
#pragma unroll
    for (int j = 0; j < D; ++j) s1[j] = s2[j] = 0.0f;
    for (int64_t i = threadIdx.x; i < N; i += ABC_TPB) {
#pragma unroll
      for (int j = 0; j < D; ++j) s1[j] = __fadd_rn(s1[j], w.value[(off + i) * D + j]);
    }
#pragma unroll 1
    for (int j = 0; j < D; ++j) mf[j] = abc_block_ratio((double)s1[j], (double)N, smd);
    for (int64_t i = threadIdx.x; i < N; i += ABC_TPB) {
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const float dv = __fsub_rn(w.value[(off + i) * D + j], mf[j]);
        s2[j] = __fadd_rn(s2[j], __fmul_rn(dv, dv));
      }
    }
#pragma unroll 1
    for (int j = 0; j < D; ++j) {
      const float var = abc_block_ratio((double)s2[j], (double)(N - 1), smd);
      if (threadIdx.x == 0) w.stepsize[b * D + j] = __fmul_rn(__fdiv_rn(var, (float)D), 5.6644f);
    }
  } else if (threadIdx.x < D) {
    w.stepsize[b * D + threadIdx.x] = ctl.fixed_stepsize;
  }
  if (threadIdx.x == 0) {
    w.threshold[b] = thr;
    w.ess[b] = ess;
    w.alpha_mean[b] = alpha_mean;
    w.iter[b] = iter;
    const int done = alive == 0 || alpha_mean <= ctl.term_alpha || iter >= ctl.max_iter;
    w.active[b] = !done;
    if (iter < ctl.hist_len) {
      w.hist_thr[b * ctl.hist_len + iter] = thr;
      w.hist_ess[b * ctl.hist_len + iter] = ess;
      w.hist_alpha[b * ctl.hist_len + iter] = alpha_mean;
      w.hist_res[b * ctl.hist_len + iter] = startup ? 0 : w.resampled[b];
    }
    if (!startup) {
      // e <- split(e, N + 2)[N + 1], after the moves have used the old e
      uint32_t z0, z1;
      split_at(w.key[2 * b], w.key[2 * b + 1], (uint64_t)N + 2, (uint64_t)N + 1, z0, z1);
      w.key[2 * b] = z0;
      w.key[2 * b + 1] = z1;
    }
  }
}

// -------------------------------------------------------------- resample
// systematic resampling of 0 / -inf weights: output k takes the alive particle
// of rank floor((k 2^23 + m) A / (N 2^23)) (A alive, m the uniform's mantissa),
// the ancestor the 62-bit fixed-point systematic fill gives for these weights
template <int D>
__global__ void __launch_bounds__(ABC_TPB) k_abc_resample(ABCCtl ctl, ABCWs w) {
  __shared__ int smi[33];
  __shared__ int wsum[ABC_TPB / 32];
  const int64_t b = blockIdx.x, N = ctl.N;
  if (!w.active[b]) return;
  const int64_t off = b * N;
  const int res = w.ess[b] < __fmul_rn(ctl.resample_thr, (float)N);
  if (threadIdx.x == 0) w.resampled[b] = res;
  if (!res) return;
  // ranks of the alive particles: each thread scans a contiguous chunk
  const int64_t per = (N + ABC_TPB - 1) / ABC_TPB;
  const int64_t i0 = threadIdx.x * per, i1 = i0 + per < N ? i0 + per : N;
  int cnt = 0;
  for (int64_t i = i0; i < i1; ++i) cnt += w.lw[off + i] > -INFINITY;
  // block exclusive scan of cnt
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < ABC_TPB / 32; ++k) {
      const int t = wsum[k];
      wsum[k] = s;
      s += t;
    }
    smi[32] = s;
  }
  __syncthreads();
  int rank = wsum[warp] + incl - cnt;
  const int A = smi[32];
  if (A == 0) return;  // nothing alive: the posterior is inactive (adapt), kept as a guard
  for (int64_t i = i0; i < i1; ++i)
    if (w.lw[off + i] > -INFINITY) w.rank_idx[off + rank++] = (int32_t)i;
  __syncthreads();
  const uint32_t *kb = w.key + 2 * b;
  uint32_t r0, r1;
  split_at(kb[0], kb[1], (uint64_t)N + 2, (uint64_t)N, r0, r1);
  const uint64_t m23 = bits_at(r0, r1, 1, 0) >> 9;
  const uint64_t den = (uint64_t)N << 23;
  for (int64_t k = threadIdx.x; k < N; k += ABC_TPB) {
    const uint64_t rk = ((((uint64_t)k) << 23) + m23) * (uint64_t)A / den;
    const int64_t src = off + w.rank_idx[off + rk];
#pragma unroll
    for (int j = 0; j < D; ++j) w.value_tmp[(off + k) * D + j] = w.value[src * D + j];
    w.dist_tmp[off + k] = w.dist[src];
    w.pp_tmp[off + k] = w.pp[src];
    w.alpha_tmp[off + k] = w.alpha[src];
  }
  __syncthreads();
  for (int64_t k = threadIdx.x; k < N; k += ABC_TPB) {
#pragma unroll
    for (int j = 0; j < D; ++j) w.value[(off + k) * D + j] = w.value_tmp[(off + k) * D + j];
    w.dist[off + k] = w.dist_tmp[off + k];
    w.pp[off + k] = w.pp_tmp[off + k];
    w.alpha[off + k] = w.alpha_tmp[off + k];
    w.lw[off + k] = 0.0f;
  }
  if (threadIdx.x == 0) w.ess[b] = (float)N;
}

// ------------------------------------------------------------------ moves
// forward_proposal (abc/smc.py:172-209): mcmc_steps random-walk ABC moves of
// every alive particle with key split(e, N + 2)[i]; dead particles are kept
template <int D, int DY>
__global__ void __launch_bounds__(ABC_MOVE_TPB) k_abc_move(const __grid_constant__ ABCP<D, DY> p, ABCCtl ctl,
                                                            int64_t B, ABCWs w) {
  const int64_t N = ctl.N;
  const int64_t g = blockIdx.x * (int64_t)ABC_MOVE_TPB + threadIdx.x;
  if (g >= B * N) return;
  const int64_t b = g / N, i = g - b * N;
  if (!w.active[b] || !(w.lw[g] > -INFINITY)) return;
  const float thr = w.threshold[b];
  float sq[D], x[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    sq[j] = __fsqrt_rn(w.stepsize[b * D + j]);
    x[j] = w.value[g * D + j];
  }
  float pp = w.pp[g], dist = w.dist[g];
  uint32_t k0, k1;
  split_at(w.key[2 * b], w.key[2 * b + 1], (uint64_t)N + 2, (uint64_t)i, k0, k1);
  float asum = 0.0f;
#pragma unroll 1
  for (int s = 0; s < ctl.mcmc_steps; ++s) {
    uint32_t t0, t1;
    split_at(k0, k1, 2, 0, t0, t1);  // always(): key <- split(key)[0]
    uint32_t sk4[8];
    split4(t0, t1, sk4);
    const uint32_t n0 = sk4[0], n1 = sk4[1];  // new extra key
    const uint32_t a0 = sk4[2], a1 = sk4[3];  // proposal normals
    const uint32_t c0 = sk4[6], c1 = sk4[7];  // simulation
    uint32_t bits[D];
    bits_vec<D>(a0, a1, bits, p.one);
    float xp[D];
#pragma unroll
    for (int j = 0; j < D; ++j) xp[j] = __fadd_rn(x[j], __fmul_rn(sq[j], bits_to_normal(bits[j])));
    const float ppn = abc_prior_potential<D, DY>(p, xp);
    const float dn = abc_sim_distance<D, DY>(p, xp, c0, c1);
    // min(1, exp(pp - ppn) [dn < thr]) with NaN (inf * 0) mapped to 0 (metropolis.py:58)
    float a = __fmul_rn(expf_(__fsub_rn(pp, ppn)), dn < thr ? 1.0f : 0.0f);
    a = a != a ? 0.0f : fminf(1.0f, a);
    uint32_t u0, u1, v0, v1;
    split2(n0, n1, u0, u1, v0, v1);
    const float u = bits_to_unit(bits_at(v0, v1, 1, 0));
    if (u < a) {
#pragma unroll
      for (int j = 0; j < D; ++j) x[j] = xp[j];
      pp = ppn;
      dist = dn;
    }
    asum = s == 0 ? a : __fadd_rn(asum, a);
    k0 = u0;
    k1 = u1;
  }
#pragma unroll
  for (int j = 0; j < D; ++j) w.value[g * D + j] = x[j];
  w.pp[g] = pp;
  w.dist[g] = dist;
  w.alpha[g] = __fdiv_rn(asum, (float)ctl.mcmc_steps);
}

template <int D, int DY>
static ABCP<D, DY> pack_abc(const mgb_abc_lg_model *m) {
  ABCP<D, DY> p;
  for (int i = 0; i < D; ++i) p.m0[i] = m->m0[i];
  for (int i = 0; i < D * D; ++i) {
    p.C0[i] = m->C0[i];
    p.P0[i] = m->P0[i];
  }
  for (int i = 0; i < DY * D; ++i) p.H[i] = m->H[i];
  for (int i = 0; i < DY * DY; ++i) p.L[i] = m->L[i];
  for (int i = 0; i < DY; ++i) p.data[i] = m->data[i];
  p.c0 = m->c0;
  p.one = 1u;
  return p;
}

static int abc_hist_len(const mgb_abc_smc_config *cfg) { return cfg->max_iter + 1; }

static ABCCtl abc_ctl(const mgb_abc_smc_config *cfg) {
  ABCCtl c;
  c.N = cfg->N;
  c.mcmc_steps = cfg->mcmc_steps;
  c.max_iter = cfg->max_iter;
  c.n_schedule = cfg->n_schedule;
  c.adapt_stepsize = cfg->adapt_stepsize;
  c.hist_len = abc_hist_len(cfg);
  c.retain = cfg->ess_threshold_retain;
  c.resample_thr = cfg->ess_threshold_resample;
  c.term_alpha = cfg->termination_alpha;
  c.fixed_stepsize = cfg->stepsize;
  return c;
}

static ABCWs abc_ws(const mgb_abc_smc_config *cfg, int d, void *ws) {
  Carver c(ws);
  return carve_abc(c, cfg->B, cfg->N, d, abc_hist_len(cfg), cfg->n_schedule);
}

template <int D, int DY>
static int abc_init(const mgb_abc_smc_config *cfg, const mgb_abc_lg_model *m, const uint32_t *keys, void *ws,
                    cudaStream_t s) {
  const ABCWs w = abc_ws(cfg, D, ws);
  const ABCCtl ctl = abc_ctl(cfg);
  if (cfg->n_schedule > 0 &&
      cudaMemcpyAsync(w.schedule, cfg->schedule, sizeof(float) * cfg->n_schedule, cudaMemcpyHostToDevice, s) !=
          cudaSuccess)
    return ERR_CUDA;
  const int64_t BN = (int64_t)cfg->B * cfg->N;
  k_abc_init<D, DY><<<(unsigned)((BN + ABC_MOVE_TPB - 1) / ABC_MOVE_TPB), ABC_MOVE_TPB, 0, s>>>(
      pack_abc<D, DY>(m), cfg->B, cfg->N, keys, w);
  int st = launch_status();
  if (st) return st;
  k_abc_adapt<D><<<(unsigned)cfg->B, ABC_TPB, 0, s>>>(ctl, w, 1);
  return launch_status();
}

template <int D, int DY>
static int abc_step(const mgb_abc_smc_config *cfg, const mgb_abc_lg_model *m, void *ws, cudaStream_t s) {
  const ABCWs w = abc_ws(cfg, D, ws);
  const ABCCtl ctl = abc_ctl(cfg);
  k_abc_resample<D><<<(unsigned)cfg->B, ABC_TPB, 0, s>>>(ctl, w);
  int st = launch_status();
  if (st) return st;
  const int64_t BN = (int64_t)cfg->B * cfg->N;
  k_abc_move<D, DY><<<(unsigned)((BN + ABC_MOVE_TPB - 1) / ABC_MOVE_TPB), ABC_MOVE_TPB, 0, s>>>(
      pack_abc<D, DY>(m), ctl, cfg->B, w);
  if ((st = launch_status())) return st;
  k_abc_adapt<D><<<(unsigned)cfg->B, ABC_TPB, 0, s>>>(ctl, w, 0);
  return launch_status();
}

// ------------------------------------------------------------- g-and-k
// GKTransformedUniformPrior / GKOnlyATransformedUniformPrior (abc/scenarios/gk.py:81-175)
// with the thinned-order-statistics summary of the reference's GK tests
// (tests/test_abc_gk.py GKThinOrder):
//   prior_sample     normal(key, (d,)); prior_potential 0.5 sum x^2
//   constrain        lo + Phi(x) (hi - lo)
//   simulation       u = max(buffer, f (1 - 2 buffer) + buffer) from uniform bits f,
//                    z = Phi^-1(u), e = exp(-g z),
//                    v = A + ((B (1 + c (1 - e) / (1 + e))) z) (1 + z^2)^k
//                    (the A-only scenario: B = 1, g = 2 and the exponent c, as the reference writes it)
//   summary          sorted v at ranks floor(j n_raw / n_sum), j < n_sum; distance |summary - data|_2.
// Phi(x) = 0.5 erfc(-x / sqrt 2) with the erfc of Numerical Recipes (erfcc, a Chebyshev
// fit with fractional error below 1.2e-7); Phi^-1(u) = sqrt 2 erfinv(2u - 1) with the
// library's own erfinv; (1 + z^2)^k = exp(k log(1 + z^2)) with its own exp and log.
constexpr int GK_TPB = 256;
constexpr int GK_MAX_RAW = 2048;

struct GKP {
  int32_t d, n_raw, n_sum, p2;  // p2: sort length, the power of two >= n_raw
  float c, lo, hi, buffer;
  const float *data;
  uint32_t one;
};

__device__ __forceinline__ float gk_erfcc(float x) {
  const float z = fabsf(x);
  const float t = __fdiv_rn(1.0f, __fmaf_rn(0.5f, z, 1.0f));
  float q = 0.17087277f;
  q = __fmaf_rn(t, q, -0.82215223f);
  q = __fmaf_rn(t, q, 1.48851587f);
  q = __fmaf_rn(t, q, -1.13520398f);
  q = __fmaf_rn(t, q, 0.27886807f);
  q = __fmaf_rn(t, q, -0.18628806f);
  q = __fmaf_rn(t, q, 0.09678418f);
  q = __fmaf_rn(t, q, 0.37409196f);
  q = __fmaf_rn(t, q, 1.00002368f);
  const float arg = __fmaf_rn(t, q, __fsub_rn(-__fmul_rn(z, z), 1.26551223f));
  const float ans = __fmul_rn(t, expf_(arg));
  return x >= 0.0f ? ans : __fsub_rn(2.0f, ans);
}

__device__ __forceinline__ float gk_ncdf(float x) {
  return __fmul_rn(0.5f, gk_erfcc(__fmul_rn(-x, 0.70710677f)));
}

__device__ __forceinline__ float gk_ppf(float u) {
  return __fmul_rn(1.41421354f, erfinv_(__fsub_rn(__fmul_rn(2.0f, u), 1.0f)));
}

// (A, B, g, exponent) of a parameter row
__device__ __forceinline__ void gk_params(const GKP &p, const float *x, float (&q)[4]) {
  const float span = __fsub_rn(p.hi, p.lo);
  if (p.d == 4) {
#pragma unroll
    for (int j = 0; j < 4; ++j) q[j] = __fadd_rn(p.lo, __fmul_rn(gk_ncdf(x[j]), span));
  } else {
    q[0] = __fadd_rn(p.lo, __fmul_rn(gk_ncdf(x[0]), span));
    q[1] = 1.0f;
    q[2] = 2.0f;
    q[3] = p.c;
  }
}

__device__ __forceinline__ float gk_value(const GKP &p, const float (&q)[4], uint32_t bits) {
  const float range = __fsub_rn(__fsub_rn(1.0f, p.buffer), p.buffer);
  const float u = fmaxf(p.buffer, __fadd_rn(__fmul_rn(bits_to_unit(bits), range), p.buffer));
  const float z = gk_ppf(u);
  const float e = expf_(-__fmul_rn(q[2], z));
  const float term = __fadd_rn(1.0f, __fdiv_rn(__fmul_rn(p.c, __fsub_rn(1.0f, e)), __fadd_rn(1.0f, e)));
  const float pw = expf_(__fmul_rn(q[3], logf_(__fadd_rn(1.0f, __fmul_rn(z, z)))));
  return __fadd_rn(q[0], __fmul_rn(__fmul_rn(__fmul_rn(q[1], term), z), pw));
}

// ascending sort keys of floats (NaN of either sign after +inf, as jnp.sort)
__device__ __forceinline__ uint32_t gk_key(float v) {
  if (v != v) return 0xFFFFFFFEu;
  const uint32_t b = __float_as_uint(v);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float gk_unkey(uint32_t k) {
  if (k == 0xFFFFFFFEu) return __uint_as_float(0x7fc00000u);
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

constexpr int GK_EPT = GK_MAX_RAW / GK_TPB;  // sort elements per thread at the largest length

// bitonic sort of the P2 keys in sk (P2 a power of two, at most EPT * 256) by the whole CTA;
// thread t holds elements t + 256 m, m < EPT, in the register phases
template <int EPT>
__device__ __forceinline__ void gk_sort(uint32_t *sk, int P2, int t) {
  const bool warp_live = (t & ~31) < P2;  // the warp holds elements (all lanes join the shuffles)
  for (int kk = 2; kk <= P2; kk <<= 1) {
    int j = kk >> 1;
    for (; j >= 32; j >>= 1) {
      // pair q joins elements i (bit j clear) and i + j; the lower index of an ascending pair
      // (i & kk == 0) keeps the minimum
      for (int q = t; q < (P2 >> 1); q += GK_TPB) {
        const int i = ((q & ~(j - 1)) << 1) | (q & (j - 1));
        const uint32_t a = sk[i], b = sk[i + j];
        const bool asc = (i & kk) == 0;
        sk[i] = asc ? min(a, b) : max(a, b);
        sk[i + j] = asc ? max(a, b) : min(a, b);
      }
      __syncthreads();
    }
    // the stages j < 32 of this kk in registers.  For element e = t + 256 m the pair direction
    // (e & kk) == 0 is fixed per m over the phase, and for jj < 32 the lower-index test
    // (e & jj) == 0 is (t & jj) == 0 for every m
    if (warp_live) {
      uint32_t v[EPT];
      bool asc[EPT];
#pragma unroll
      for (int m = 0; m < EPT; ++m) {
        const int e = t + GK_TPB * m;
        v[m] = e < P2 ? sk[e] : 0xFFFFFFFFu;
        asc[m] = (e & kk) == 0;
      }
      for (int jj = j; jj > 0; jj >>= 1) {
        const bool lower = (t & jj) == 0;
#pragma unroll
        for (int m = 0; m < EPT; ++m) {
          const uint32_t o = __shfl_xor_sync(0xffffffffu, v[m], jj);
          v[m] = lower == asc[m] ? min(v[m], o) : max(v[m], o);
        }
      }
#pragma unroll
      for (int m = 0; m < EPT; ++m) {
        const int e = t + GK_TPB * m;
        if (e < P2) sk[e] = v[m];
      }
    }
    __syncthreads();
  }
}

// One g-and-k simulation by the whole CTA (every thread calls it): n_raw draws of parameters qv
// with key (k0, k1), sort, thinned order statistics into summary_row (when given) and, when
// want_dist, the distance to the data, returned in thread 0.
// Draws: element q and q + ceil(n_raw/2) of random_bits(key, (n_raw,)) are the two halves of one
// cipher call.  Sort: a bitonic network over p2 keys in shared memory; the stages with partner
// distance j < 32 run on warp shuffles (thread t holds elements t + 256 m, so e and e ^ j share
// a warp), the others through shared memory.  Distance: the order statistics and their squared
// differences are gathered in parallel, then summed in index order by one thread.
__device__ float gk_sim_cta(const GKP &p, const float (&qv)[4], uint32_t k0, uint32_t k1, uint32_t *sk, bool want_dist,
                            float *summary_row) {
  const int n_raw = p.n_raw, P2 = p.p2, t = threadIdx.x;
  const int h = (n_raw + 1) >> 1;
  for (int i = t; i < h; i += GK_TPB) {
    uint32_t r0, r1;
    threefry2x32_m(k0, k1, (uint32_t)i, i + h < n_raw ? (uint32_t)(i + h) : 0u, p.one, r0, r1);
    sk[i] = gk_key(gk_value(p, qv, r0));
    if (i + h < n_raw) sk[i + h] = gk_key(gk_value(p, qv, r1));
  }
  for (int i = n_raw + t; i < P2; i += GK_TPB) sk[i] = 0xFFFFFFFFu;
  __syncthreads();
  if (P2 <= GK_TPB)
    gk_sort<1>(sk, P2, t);
  else if (P2 <= 2 * GK_TPB)
    gk_sort<2>(sk, P2, t);
  else if (P2 <= 4 * GK_TPB)
    gk_sort<4>(sk, P2, t);
  else
    gk_sort<8>(sk, P2, t);
  // thinned order statistics j < n_sum (ranks floor(j n_raw / n_sum), below 2^22) and, for the
  // distance, their squared differences to the data, gathered in parallel
  float sv[GK_EPT], dv2[GK_EPT];
#pragma unroll
  for (int m = 0; m < GK_EPT; ++m) {
    const int j = t + GK_TPB * m;
    if (j < p.n_sum) {
      sv[m] = gk_unkey(sk[(int)(((uint32_t)j * (uint32_t)n_raw) / (uint32_t)p.n_sum)]);
      if (want_dist) {
        const float dv = __fsub_rn(sv[m], p.data[j]);
        dv2[m] = __fmul_rn(dv, dv);
      }
    }
  }
  if (summary_row) {
#pragma unroll
    for (int m = 0; m < GK_EPT; ++m) {
      const int j = t + GK_TPB * m;
      if (j < p.n_sum) summary_row[j] = sv[m];
    }
  }
  float dist = 0.0f;
  if (want_dist) {
    __syncthreads();  // every rank read before sk is reused for the squared differences
    float *sd = reinterpret_cast<float *>(sk);
#pragma unroll
    for (int m = 0; m < GK_EPT; ++m) {
      const int j = t + GK_TPB * m;
      if (j < p.n_sum) sd[j] = dv2[m];
    }
    __syncthreads();
    if (t == 0) {
      float acc = sd[0];
#pragma unroll 8
      for (int j = 1; j < p.n_sum; ++j) acc = __fadd_rn(acc, sd[j]);
      dist = __fsqrt_rn(acc);
    }
  }
  return dist;
}

// one CTA per parameter row
__global__ void __launch_bounds__(GK_TPB) k_gk_sim(const GKP p, int64_t P, const float *__restrict__ x,
                                                    const uint32_t *__restrict__ keys, const int32_t *mask,
                                                    float *__restrict__ dist, float *__restrict__ summary) {
  __shared__ uint32_t sk[GK_MAX_RAW];
  __shared__ float q[4];
  const int64_t r = blockIdx.x;
  if (r >= P || (mask && !mask[r])) return;
  if (threadIdx.x == 0) {
    float qq[4];
    gk_params(p, x + r * p.d, qq);
#pragma unroll
    for (int j = 0; j < 4; ++j) q[j] = qq[j];
  }
  __syncthreads();
  const float qv[4] = {q[0], q[1], q[2], q[3]};
  const float dv = gk_sim_cta(p, qv, keys[2 * r], keys[2 * r + 1], sk, dist != nullptr,
                              summary ? summary + r * p.n_sum : nullptr);
  if (dist && threadIdx.x == 0) dist[r] = dv;
}

template <int D>
__device__ __forceinline__ float gk_prior_pot(const float (&x)[D]) {
  float s = __fmul_rn(x[0], x[0]);
#pragma unroll
  for (int j = 1; j < D; ++j) s = __fadd_rn(s, __fmul_rn(x[j], x[j]));
  return __fmul_rn(0.5f, s);
}

// RandomWalkABC() with the RMMetropolisDiagStepsize correction on a g-and-k scenario, one CTA per
// chain (the reference's TestMCMCGK / TestMCMCGKOnlyA): thread 0 holds the chain (keys, proposal,
// Metropolis step and the Robbins-Monro updates of k_abc_mcmc_rm_lg); every step's simulation
// runs on the whole CTA.  The prior is the transformed-uniform one: x_0 = normal(split(key)[1],
// (d,)), potential 0.5 |x|^2.
template <int D>
__global__ void __launch_bounds__(GK_TPB) k_abc_mcmc_rm_gk(const GKP p, int64_t B, int64_t n, const uint32_t *keys,
                                                            float target, float scale, float neg_exp,
                                                            float *__restrict__ x_out, float *__restrict__ alpha_out,
                                                            float *__restrict__ thr_out, float *__restrict__ st_out) {
  __shared__ uint32_t sk[GK_MAX_RAW];
  __shared__ float q_s[4];
  __shared__ uint32_t ck[2];
  const int64_t b = blockIdx.x;
  if (b >= B) return;
  const bool lead = threadIdx.x == 0;
  float x[D], xp[D], st[D], pm[D], dg[D], pp = 0.0f, ppn = 0.0f, thr = 50.0f;
  uint32_t K0 = 0, K1 = 0, n0 = 0, n1 = 0;
  const int64_t base = b * n;
  if (lead) {
    uint32_t a0, a1, t0, t1;
    K0 = keys[2 * b];
    K1 = keys[2 * b + 1];
    split_at(K0, K1, 2, 1, a0, a1);
    split_at(K0, K1, 2, 0, t0, t1);
    split_at(t0, t1, 2, 0, K0, K1);  // prior potential
    uint32_t bits[D];
    bits_vec<D>(a0, a1, bits, p.one);
#pragma unroll
    for (int j = 0; j < D; ++j) x[j] = bits_to_normal(bits[j]);
    pp = gk_prior_pot<D>(x);
    split_at(K0, K1, 2, 0, t0, t1);  // the initial simulation takes split(K)[1]; its distance is unused
    K0 = t0;
    K1 = t1;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      st[j] = 1.0f;
      pm[j] = x[j];
      dg[j] = __fdiv_rn(__fmul_rn(st[j], (float)D), 5.6644f);
      x_out[base * D + j] = x[j];
      st_out[base * D + j] = st[j];
    }
    alpha_out[base] = 1.0f;
    thr_out[base] = thr;
  }
#pragma unroll 1
  for (int64_t i = 1; i < n; ++i) {
    if (lead) {
      uint32_t t0, t1;
      split_at(K0, K1, 2, 0, t0, t1);  // always
      uint32_t sk4[8];                 // split(t, 4): 0 new extra key, 1 proposal normals, 3 simulation
      split4(t0, t1, sk4);
      uint32_t bits[D];
      bits_vec<D>(sk4[2], sk4[3], bits, p.one);
#pragma unroll
      for (int j = 0; j < D; ++j) xp[j] = __fadd_rn(x[j], __fmul_rn(__fsqrt_rn(st[j]), bits_to_normal(bits[j])));
      ppn = gk_prior_pot<D>(xp);
      float qq[4];
      gk_params(p, xp, qq);
#pragma unroll
      for (int j = 0; j < 4; ++j) q_s[j] = qq[j];
      ck[0] = sk4[6];
      ck[1] = sk4[7];
      n0 = sk4[0];
      n1 = sk4[1];
    }
    __syncthreads();
    const float qv[4] = {q_s[0], q_s[1], q_s[2], q_s[3]};
    const float dn = gk_sim_cta(p, qv, ck[0], ck[1], sk, true, nullptr);
    if (lead) {
      float a = __fmul_rn(expf_(__fsub_rn(pp, ppn)), dn < thr ? 1.0f : 0.0f);
      a = a != a ? 0.0f : fminf(1.0f, a);
      uint32_t u0, u1, v0, v1;
      split2(n0, n1, u0, u1, v0, v1);
      const float u = bits_to_unit(bits_at(v0, v1, 1, 0));
      if (u < a) {
#pragma unroll
        for (int j = 0; j < D; ++j) x[j] = xp[j];
        pp = ppn;
      }
      K0 = u0;
      K1 = u1;
      const float rm = __fmul_rn(scale, expf_(__fmul_rn(-neg_exp, logf_((float)i))));
      thr = expf_(__fsub_rn(logf_(thr), __fmul_rn(rm, __fsub_rn(a, target))));
      const float r2 = fminf(rm, 0.999f), q2 = __fsub_rn(1.0f, r2);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const float dv = __fsub_rn(x[j], pm[j]);
        dg[j] = __fadd_rn(__fmul_rn(q2, dg[j]), __fmul_rn(r2, __fmul_rn(dv, dv)));
        pm[j] = __fadd_rn(__fmul_rn(q2, pm[j]), __fmul_rn(r2, x[j]));
        st[j] = __fmul_rn(__fdiv_rn(dg[j], (float)D), 5.6644f);
        x_out[(base + i) * D + j] = x[j];
        st_out[(base + i) * D + j] = st[j];
      }
      alpha_out[base + i] = a;
      thr_out[base + i] = thr;
    }
  }
}

// RandomWalkABC(stepsize, threshold) on a g-and-k scenario (the Metropolis correction), one CTA
// per chain: the key chain and Metropolis step of k_abc_mcmc_lg with the transformed-uniform
// prior, every simulation (the initial one included) on the whole CTA
template <int D>
__global__ void __launch_bounds__(GK_TPB) k_abc_mcmc_gk(const GKP p, int64_t B, int64_t n, const uint32_t *keys,
                                                         float stepsize, float thr, float *__restrict__ x_out,
                                                         float *__restrict__ dist_out, float *__restrict__ pp_out,
                                                         float *__restrict__ alpha_out) {
  __shared__ uint32_t sk[GK_MAX_RAW];
  __shared__ float q_s[4];
  __shared__ uint32_t ck[2];
  const int64_t b = blockIdx.x;
  if (b >= B) return;
  const bool lead = threadIdx.x == 0;
  const float sq = __fsqrt_rn(stepsize);
  float x[D], xp[D], pp = 0.0f, ppn = 0.0f, dist = 0.0f;
  uint32_t K0 = 0, K1 = 0, n0 = 0, n1 = 0;
  const int64_t base = b * n;
  if (lead) {
    uint32_t a0, a1, t0, t1;
    K0 = keys[2 * b];
    K1 = keys[2 * b + 1];
    split_at(K0, K1, 2, 1, a0, a1);
    split_at(K0, K1, 2, 0, t0, t1);
    split_at(t0, t1, 2, 0, K0, K1);  // prior potential
    uint32_t bits[D];
    bits_vec<D>(a0, a1, bits, p.one);
#pragma unroll
    for (int j = 0; j < D; ++j) x[j] = bits_to_normal(bits[j]);
    pp = gk_prior_pot<D>(x);
    float qq[4];
    gk_params(p, x, qq);
#pragma unroll
    for (int j = 0; j < 4; ++j) q_s[j] = qq[j];
    split2(K0, K1, t0, t1, a0, a1);  // split(K): [0] the chain key, [1] the initial simulation
    ck[0] = a0;
    ck[1] = a1;
    K0 = t0;
    K1 = t1;
  }
  __syncthreads();
  {
    const float qv[4] = {q_s[0], q_s[1], q_s[2], q_s[3]};
    const float d0 = gk_sim_cta(p, qv, ck[0], ck[1], sk, true, nullptr);
    if (lead) {
      dist = d0;
#pragma unroll
      for (int j = 0; j < D; ++j) x_out[base * D + j] = x[j];
      dist_out[base] = dist;
      pp_out[base] = pp;
      alpha_out[base] = 1.0f;
    }
  }
#pragma unroll 1
  for (int64_t i = 1; i < n; ++i) {
    if (lead) {
      uint32_t t0, t1;
      split_at(K0, K1, 2, 0, t0, t1);  // always
      uint32_t sk4[8];                 // split(t, 4): 0 new extra key, 1 proposal normals, 3 simulation
      split4(t0, t1, sk4);
      uint32_t bits[D];
      bits_vec<D>(sk4[2], sk4[3], bits, p.one);
#pragma unroll
      for (int j = 0; j < D; ++j) xp[j] = __fadd_rn(x[j], __fmul_rn(sq, bits_to_normal(bits[j])));
      ppn = gk_prior_pot<D>(xp);
      float qq[4];
      gk_params(p, xp, qq);
#pragma unroll
      for (int j = 0; j < 4; ++j) q_s[j] = qq[j];
      ck[0] = sk4[6];
      ck[1] = sk4[7];
      n0 = sk4[0];
      n1 = sk4[1];
    }
    __syncthreads();
    const float qv[4] = {q_s[0], q_s[1], q_s[2], q_s[3]};
    const float dn = gk_sim_cta(p, qv, ck[0], ck[1], sk, true, nullptr);
    if (lead) {
      float a = __fmul_rn(expf_(__fsub_rn(pp, ppn)), dn < thr ? 1.0f : 0.0f);
      a = a != a ? 0.0f : fminf(1.0f, a);
      uint32_t u0, u1, v0, v1;
      split2(n0, n1, u0, u1, v0, v1);
      const float u = bits_to_unit(bits_at(v0, v1, 1, 0));
      if (u < a) {
#pragma unroll
        for (int j = 0; j < D; ++j) x[j] = xp[j];
        pp = ppn;
        dist = dn;
      }
      K0 = u0;
      K1 = u1;
#pragma unroll
      for (int j = 0; j < D; ++j) x_out[(base + i) * D + j] = x[j];
      dist_out[base + i] = dist;
      pp_out[base + i] = pp;
      alpha_out[base + i] = a;
    }
  }
}

// per-particle state of the split moves (the simulation is a CTA per particle)
struct GKWs {
  float *xp;        // (B N, d) proposals
  float *ppn, *dn;  // (B N) proposal prior potential, distance
  float *asum;      // (B N) acceptance sums
  uint32_t *skey;   // (B N, 2) simulation keys
  uint32_t *mkey;   // (B N, 2) move keys
  int32_t *mask;    // (B N) rows to simulate
};

inline GKWs carve_gk(Carver &c, int64_t B, int64_t N, int d) {
  GKWs g;
  const size_t BN = (size_t)(B * N);
  g.xp = c.take<float>(BN * d);
  g.ppn = c.take<float>(BN);
  g.dn = c.take<float>(BN);
  g.asum = c.take<float>(BN);
  g.skey = c.take<uint32_t>(2 * BN);
  g.mkey = c.take<uint32_t>(2 * BN);
  g.mask = c.take<int32_t>(BN);
  return g;
}

// startup: prior draw, prior potential, the simulation key (the simulation itself is k_gk_sim)
template <int D>
__global__ void __launch_bounds__(ABC_MOVE_TPB) k_gk_init(int64_t B, int64_t N, const uint32_t *keys, ABCWs w,
                                                           GKWs g, uint32_t one) {
  const int64_t i0 = blockIdx.x * (int64_t)ABC_MOVE_TPB + threadIdx.x;
  if (i0 >= B * N) return;
  const int64_t b = i0 / N, i = i0 - b * N;
  uint32_t e0, e1, s0, s1, a0, a1;
  split_at(keys[2 * b], keys[2 * b + 1], 2, 0, e0, e1);
  split_at(keys[2 * b], keys[2 * b + 1], 2, 1, s0, s1);
  split_at(s0, s1, (uint64_t)N, (uint64_t)i, a0, a1);
  uint32_t bits[D];
  bits_vec<D>(a0, a1, bits, one);
  float x[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    x[j] = bits_to_normal(bits[j]);
    w.value[i0 * D + j] = x[j];
  }
  w.pp[i0] = gk_prior_pot<D>(x);
  uint32_t f0, f1, k0, k1;
  split_at(e0, e1, (uint64_t)N + 1, (uint64_t)N, f0, f1);
  split_at(f0, f1, (uint64_t)N + 1, (uint64_t)i, k0, k1);
  g.skey[2 * i0] = k0;
  g.skey[2 * i0 + 1] = k1;
  g.mask[i0] = 1;
  w.alpha[i0] = 1.0f;
  w.lw[i0] = 0.0f;
  if (i == 0) {
    uint32_t z0, z1;
    split_at(f0, f1, (uint64_t)N + 1, (uint64_t)N, z0, z1);
    w.key[2 * b] = z0;
    w.key[2 * b + 1] = z1;
  }
}

// first move of an iteration: the particle's key split(e, N + 2)[i]; every move:
// key <- split(key)[0]; (key, k1, k2, k3) = split(key, 4); proposal x + sqrt(s) normal(k1, (d,))
template <int D>
__global__ void __launch_bounds__(ABC_MOVE_TPB) k_gk_prop(ABCCtl ctl, int64_t B, ABCWs w, GKWs g, int first,
                                                           uint32_t one) {
  const int64_t N = ctl.N;
  const int64_t i0 = blockIdx.x * (int64_t)ABC_MOVE_TPB + threadIdx.x;
  if (i0 >= B * N) return;
  const int64_t b = i0 / N, i = i0 - b * N;
  const bool live = w.active[b] && (w.lw[i0] > -INFINITY);
  g.mask[i0] = live;
  if (!live) return;
  uint32_t k0, k1;
  if (first) {
    split_at(w.key[2 * b], w.key[2 * b + 1], (uint64_t)N + 2, (uint64_t)i, k0, k1);
  } else {
    k0 = g.mkey[2 * i0];
    k1 = g.mkey[2 * i0 + 1];
  }
  uint32_t t0, t1, n0, n1, a0, a1, c0, c1;
  split_at(k0, k1, 2, 0, t0, t1);
  uint32_t sk4[8];  // split(t, 4): 0 new extra key, 1 proposal normals, 3 simulation
  split4(t0, t1, sk4);
  n0 = sk4[0];
  n1 = sk4[1];
  a0 = sk4[2];
  a1 = sk4[3];
  c0 = sk4[6];
  c1 = sk4[7];
  uint32_t bits[D];
  bits_vec<D>(a0, a1, bits, one);
  float xp[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    xp[j] = __fadd_rn(w.value[i0 * D + j], __fmul_rn(__fsqrt_rn(w.stepsize[b * D + j]), bits_to_normal(bits[j])));
    g.xp[i0 * D + j] = xp[j];
  }
  g.ppn[i0] = gk_prior_pot<D>(xp);
  g.skey[2 * i0] = c0;
  g.skey[2 * i0 + 1] = c1;
  g.mkey[2 * i0] = n0;
  g.mkey[2 * i0 + 1] = n1;
}

// Metropolis correction of the move: alpha = min(1, exp(pp - ppn) [dn < threshold]) (NaN -> 0);
// (key, ku) = split(key); accept if uniform(ku) < alpha
template <int D>
__global__ void __launch_bounds__(ABC_MOVE_TPB) k_gk_accept(ABCCtl ctl, int64_t B, ABCWs w, GKWs g, int step) {
  const int64_t N = ctl.N;
  const int64_t i0 = blockIdx.x * (int64_t)ABC_MOVE_TPB + threadIdx.x;
  if (i0 >= B * N || !g.mask[i0]) return;
  const int64_t b = i0 / N;
  const float thr = w.threshold[b];
  const float pp = w.pp[i0], ppn = g.ppn[i0], dn = g.dn[i0];
  float a = __fmul_rn(expf_(__fsub_rn(pp, ppn)), dn < thr ? 1.0f : 0.0f);
  a = a != a ? 0.0f : fminf(1.0f, a);
  const uint32_t n0 = g.mkey[2 * i0], n1 = g.mkey[2 * i0 + 1];
  uint32_t u0, u1, v0, v1;
  split2(n0, n1, u0, u1, v0, v1);
  const float u = bits_to_unit(bits_at(v0, v1, 1, 0));
  if (u < a) {
#pragma unroll
    for (int j = 0; j < D; ++j) w.value[i0 * D + j] = g.xp[i0 * D + j];
    w.pp[i0] = ppn;
    w.dist[i0] = dn;
  }
  const float as = step == 0 ? a : __fadd_rn(g.asum[i0], a);
  g.asum[i0] = as;
  g.mkey[2 * i0] = u0;
  g.mkey[2 * i0 + 1] = u1;
  if (step == ctl.mcmc_steps - 1) w.alpha[i0] = __fdiv_rn(as, (float)ctl.mcmc_steps);
}

static GKP pack_gk(const mgb_abc_gk_model *m) {
  GKP p;
  p.d = m->d;
  p.n_raw = m->n_unsummarised;
  p.n_sum = m->n_summary;
  int p2 = 1;
  while (p2 < m->n_unsummarised) p2 <<= 1;
  p.p2 = p2;
  p.c = m->c;
  p.lo = m->prior_min;
  p.hi = m->prior_max;
  p.buffer = m->buffer;
  p.data = m->data_dev;
  p.one = 1u;
  return p;
}

static bool gk_ok(const mgb_abc_gk_model *m) {
  return m && (m->d == 4 || m->d == 1) && m->n_unsummarised >= 1 && m->n_unsummarised <= GK_MAX_RAW &&
         m->n_summary >= 1 && m->n_summary <= m->n_unsummarised;
}

static GKWs gk_ws(const mgb_abc_smc_config *cfg, int d, void *ws) {
  Carver c(ws);
  carve_abc(c, cfg->B, cfg->N, d, abc_hist_len(cfg), cfg->n_schedule);
  return carve_gk(c, cfg->B, cfg->N, d);
}

template <int D>
static int gk_init(const mgb_abc_smc_config *cfg, const mgb_abc_gk_model *m, const uint32_t *keys, void *ws,
                   cudaStream_t s) {
  const ABCWs w = abc_ws(cfg, D, ws);
  const GKWs g = gk_ws(cfg, D, ws);
  const ABCCtl ctl = abc_ctl(cfg);
  if (cfg->n_schedule > 0 &&
      cudaMemcpyAsync(w.schedule, cfg->schedule, sizeof(float) * cfg->n_schedule, cudaMemcpyHostToDevice, s) !=
          cudaSuccess)
    return ERR_CUDA;
  const int64_t BN = (int64_t)cfg->B * cfg->N;
  const unsigned grid = (unsigned)((BN + ABC_MOVE_TPB - 1) / ABC_MOVE_TPB);
  k_gk_init<D><<<grid, ABC_MOVE_TPB, 0, s>>>(cfg->B, cfg->N, keys, w, g, 1u);
  int st = launch_status();
  if (st) return st;
  k_gk_sim<<<(unsigned)BN, GK_TPB, 0, s>>>(pack_gk(m), BN, w.value, g.skey, nullptr, w.dist, nullptr);
  if ((st = launch_status())) return st;
  k_abc_adapt<D><<<(unsigned)cfg->B, ABC_TPB, 0, s>>>(ctl, w, 1);
  return launch_status();
}

template <int D>
static int gk_step(const mgb_abc_smc_config *cfg, const mgb_abc_gk_model *m, void *ws, cudaStream_t s) {
  const ABCWs w = abc_ws(cfg, D, ws);
  const GKWs g = gk_ws(cfg, D, ws);
  const ABCCtl ctl = abc_ctl(cfg);
  k_abc_resample<D><<<(unsigned)cfg->B, ABC_TPB, 0, s>>>(ctl, w);
  int st = launch_status();
  if (st) return st;
  const int64_t BN = (int64_t)cfg->B * cfg->N;
  const unsigned grid = (unsigned)((BN + ABC_MOVE_TPB - 1) / ABC_MOVE_TPB);
  const GKP p = pack_gk(m);
  for (int k = 0; k < cfg->mcmc_steps; ++k) {
    k_gk_prop<D><<<grid, ABC_MOVE_TPB, 0, s>>>(ctl, cfg->B, w, g, k == 0, 1u);
    if ((st = launch_status())) return st;
    k_gk_sim<<<(unsigned)BN, GK_TPB, 0, s>>>(p, BN, g.xp, g.skey, g.mask, g.dn, nullptr);
    if ((st = launch_status())) return st;
    k_gk_accept<D><<<grid, ABC_MOVE_TPB, 0, s>>>(ctl, cfg->B, w, g, k);
    if ((st = launch_status())) return st;
  }
  k_abc_adapt<D><<<(unsigned)cfg->B, ABC_TPB, 0, s>>>(ctl, w, 0);
  return launch_status();
}

// ------------------------------------------------------------ VanillaABC
// mocat.run(scenario, VanillaABC(threshold | acceptance_rate), n, key) (abc/importance.py:16-118,
// abc/abc.py:42-66, sample.py:110-148): a chain of n independent prior draws whose keys
// are sequential:
//   (K, s) = split(K): x_0 = prior_sample(s); (K, _) = split(K) (prior potential);
//   (K, k) = split(K): simulation of x_0 with k;
//   step i = 1..n-1: (K, k1, k2, k3) = split(K, 4): x_i = prior_sample(k1), simulation with k3;
//   log_weight = 0 if distance < threshold else -inf; with acceptance_rate the threshold is
//   jnp.quantile(distance, acceptance_rate) (linear interpolation) over the whole chain.
// The key chain is one thread (a serial dependency); the draws and simulations are parallel.
__global__ void k_vabc_keys(const uint32_t *key, int64_t n, uint32_t *__restrict__ pk, uint32_t *__restrict__ sk) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t K0 = key[0], K1 = key[1], a0, a1, b0, b1;
  split_at(K0, K1, 2, 1, a0, a1);
  pk[0] = a0;
  pk[1] = a1;
  split_at(K0, K1, 2, 0, b0, b1);        // after the prior draw
  split_at(b0, b1, 2, 0, K0, K1);        // after the prior potential
  split_at(K0, K1, 2, 1, a0, a1);        // the simulation key of x_0
  sk[0] = a0;
  sk[1] = a1;
  split_at(K0, K1, 2, 0, b0, b1);
  K0 = b0;
  K1 = b1;
  for (int64_t i = 1; i < n; ++i) {
    split_at(K0, K1, 4, 1, a0, a1);
    pk[2 * i] = a0;
    pk[2 * i + 1] = a1;
    split_at(K0, K1, 4, 3, a0, a1);
    sk[2 * i] = a0;
    sk[2 * i + 1] = a1;
    split_at(K0, K1, 4, 0, b0, b1);
    K0 = b0;
    K1 = b1;
  }
}

// linear-Gaussian scenario: prior draw, prior potential, simulation distance, threshold weight
template <int D, int DY>
__global__ void __launch_bounds__(ABC_MOVE_TPB) k_vabc_lg(const __grid_constant__ ABCP<D, DY> p, int64_t n,
                                                           const uint32_t *pk, const uint32_t *sk, float thr,
                                                           int weigh, float *x, float *pp, float *dist, float *lw) {
  const int64_t i = blockIdx.x * (int64_t)ABC_MOVE_TPB + threadIdx.x;
  if (i >= n) return;
  uint32_t bits[D];
  bits_vec<D>(pk[2 * i], pk[2 * i + 1], bits, p.one);
  float e[D], xv[D];
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(bits[j]);
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float v = __fmul_rn(p.C0[r * D], e[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) v = __fmaf_rn(p.C0[r * D + k], e[k], v);
    xv[r] = __fadd_rn(p.m0[r], v);
    x[i * D + r] = xv[r];
  }
  pp[i] = abc_prior_potential<D, DY>(p, xv);
  const float dv = abc_sim_distance<D, DY>(p, xv, sk[2 * i], sk[2 * i + 1]);
  dist[i] = dv;
  if (weigh) lw[i] = dv < thr ? 0.0f : -INFINITY;
}

// g-and-k scenario: prior draw and potential (the simulation is k_gk_sim)
template <int D>
__global__ void __launch_bounds__(ABC_MOVE_TPB) k_vabc_gk_prior(int64_t n, const uint32_t *pk, float *x, float *pp,
                                                                 uint32_t one) {
  const int64_t i = blockIdx.x * (int64_t)ABC_MOVE_TPB + threadIdx.x;
  if (i >= n) return;
  uint32_t bits[D];
  bits_vec<D>(pk[2 * i], pk[2 * i + 1], bits, one);
  float xv[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    xv[j] = bits_to_normal(bits[j]);
    x[i * D + j] = xv[j];
  }
  pp[i] = gk_prior_pot<D>(xv);
}

// the threshold (given, or the acceptance-rate quantile of the distances) and the weights; one block
__global__ void __launch_bounds__(ABC_TPB) k_vabc_weights(int64_t n, float thr_in, float rate, const float *dist,
                                                          float *lw, float *thr_out) {
  __shared__ unsigned hist[256], res[2 + ABC_TPB / 32];
  __shared__ int smi[33];
  float thr = thr_in;
  if (rate >= 0.0f) {
    const float pos = __fmul_rn(rate, (float)(n - 1));
    const float lo = floorf(pos), hi = ceilf(pos);
    const float hw = __fsub_rn(pos, lo), lwt = __fsub_rn(1.0f, hw);
    const int64_t ilo = (int64_t)fminf(fmaxf(lo, 0.0f), (float)(n - 1));
    const int64_t ihi = (int64_t)fminf(fmaxf(hi, 0.0f), (float)(n - 1));
    const float vlo = abc_block_select(dist, n, ilo, hist, res);
    const float vhi = ihi == ilo ? vlo : abc_block_next(dist, n, ilo, vlo, smi, res);
    thr = __fadd_rn(__fmul_rn(vlo, lwt), __fmul_rn(vhi, hw));
  }
  for (int64_t i = threadIdx.x; i < n; i += ABC_TPB) lw[i] = dist[i] < thr ? 0.0f : -INFINITY;
  if (threadIdx.x == 0) *thr_out = thr;
}

struct VABCWs {
  uint32_t *pk, *sk;
};

static VABCWs carve_vabc(Carver &c, int64_t n) {
  VABCWs v;
  v.pk = c.take<uint32_t>(2 * (size_t)n);
  v.sk = c.take<uint32_t>(2 * (size_t)n);
  return v;
}

template <int D, int DY>
static int vabc_lg(const mgb_abc_lg_model *m, int64_t n, const uint32_t *key, float thr, float rate, void *ws,
                   float *x, float *pp, float *dist, float *lw, float *thr_out, cudaStream_t s) {
  Carver c(ws);
  const VABCWs v = carve_vabc(c, n);
  k_vabc_keys<<<1, 32, 0, s>>>(key, n, v.pk, v.sk);
  int st = launch_status();
  if (st) return st;
  k_vabc_lg<D, DY><<<(unsigned)((n + ABC_MOVE_TPB - 1) / ABC_MOVE_TPB), ABC_MOVE_TPB, 0, s>>>(
      pack_abc<D, DY>(m), n, v.pk, v.sk, thr, 0, x, pp, dist, lw);
  if ((st = launch_status())) return st;
  k_vabc_weights<<<1, ABC_TPB, 0, s>>>(n, thr, rate, dist, lw, thr_out);
  return launch_status();
}

template <int D>
static int vabc_gk(const mgb_abc_gk_model *m, int64_t n, const uint32_t *key, float thr, float rate, void *ws,
                   float *x, float *pp, float *dist, float *lw, float *thr_out, cudaStream_t s) {
  Carver c(ws);
  const VABCWs v = carve_vabc(c, n);
  k_vabc_keys<<<1, 32, 0, s>>>(key, n, v.pk, v.sk);
  int st = launch_status();
  if (st) return st;
  k_vabc_gk_prior<D><<<(unsigned)((n + ABC_MOVE_TPB - 1) / ABC_MOVE_TPB), ABC_MOVE_TPB, 0, s>>>(n, v.pk, x, pp, 1u);
  if ((st = launch_status())) return st;
  k_gk_sim<<<(unsigned)n, GK_TPB, 0, s>>>(pack_gk(m), n, x, v.sk, nullptr, dist, nullptr);
  if ((st = launch_status())) return st;
  k_vabc_weights<<<1, ABC_TPB, 0, s>>>(n, thr, rate, dist, lw, thr_out);
  return launch_status();
}

// --------------------------------------------------------- RandomWalkABC chains
// mocat.run(scenario, RandomWalkABC(stepsize, threshold), n, key) (abc/mcmc.py:16-100,
// mcmc/sampler.py:32-110, metropolis.py:48-70) with a fixed stepsize and threshold, one chain
// per key:
//   startup   (K, s) = split(K): x_0 = prior_sample(s); (K, _) = split(K) (prior potential);
//             (K, k) = split(K): simulation of x_0 with k; alpha_0 = 1
//   step      (K, _) = split(K) (always); (K, k1, k2, k3) = split(K, 4);
//             x' = x + sqrt(stepsize) normal(k1, (d,)), simulation with k3;
//             alpha = min(1, exp(pp - pp') [dist' < threshold]) (NaN -> 0);
//             (K, ku) = split(K); accept if uniform(ku) < alpha
// The chain is serial: one thread per chain writes its n states.
template <int D, int DY>
__global__ void __launch_bounds__(128) k_abc_mcmc_lg(const __grid_constant__ ABCP<D, DY> p, int64_t B, int64_t n,
                                                      const uint32_t *keys, float stepsize, float thr,
                                                      float *__restrict__ x_out, float *__restrict__ dist_out,
                                                      float *__restrict__ pp_out, float *__restrict__ alpha_out) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= B) return;
  uint32_t K0 = keys[2 * b], K1 = keys[2 * b + 1], a0, a1, t0, t1;
  split_at(K0, K1, 2, 1, a0, a1);
  split_at(K0, K1, 2, 0, t0, t1);
  split_at(t0, t1, 2, 0, K0, K1);  // prior potential
  uint32_t bits[D];
  bits_vec<D>(a0, a1, bits, p.one);
  float e[D], x[D];
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(bits[j]);
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float v = __fmul_rn(p.C0[r * D], e[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) v = __fmaf_rn(p.C0[r * D + k], e[k], v);
    x[r] = __fadd_rn(p.m0[r], v);
  }
  float pp = abc_prior_potential<D, DY>(p, x);
  split_at(K0, K1, 2, 1, a0, a1);
  float dist = abc_sim_distance<D, DY>(p, x, a0, a1);
  split_at(K0, K1, 2, 0, t0, t1);
  K0 = t0;
  K1 = t1;
  const float sq = __fsqrt_rn(stepsize);
  const int64_t base = b * n;
#pragma unroll
  for (int j = 0; j < D; ++j) x_out[base * D + j] = x[j];
  dist_out[base] = dist;
  pp_out[base] = pp;
  alpha_out[base] = 1.0f;
#pragma unroll 1
  for (int64_t i = 1; i < n; ++i) {
    split_at(K0, K1, 2, 0, t0, t1);  // always
    uint32_t n0, n1, c0, c1;
    uint32_t sk4[8];  // split(t, 4): 0 new extra key, 1 proposal normals, 3 simulation
    split4(t0, t1, sk4);
    n0 = sk4[0];
    n1 = sk4[1];
    a0 = sk4[2];
    a1 = sk4[3];
    c0 = sk4[6];
    c1 = sk4[7];
    bits_vec<D>(a0, a1, bits, p.one);
    float xp[D];
#pragma unroll
    for (int j = 0; j < D; ++j) xp[j] = __fadd_rn(x[j], __fmul_rn(sq, bits_to_normal(bits[j])));
    const float ppn = abc_prior_potential<D, DY>(p, xp);
    const float dn = abc_sim_distance<D, DY>(p, xp, c0, c1);
    float a = __fmul_rn(expf_(__fsub_rn(pp, ppn)), dn < thr ? 1.0f : 0.0f);
    a = a != a ? 0.0f : fminf(1.0f, a);
    uint32_t u0, u1, v0, v1;
    split2(n0, n1, u0, u1, v0, v1);
    const float u = bits_to_unit(bits_at(v0, v1, 1, 0));
    if (u < a) {
#pragma unroll
      for (int j = 0; j < D; ++j) x[j] = xp[j];
      pp = ppn;
      dist = dn;
    }
    K0 = u0;
    K1 = u1;
#pragma unroll
    for (int j = 0; j < D; ++j) x_out[(base + i) * D + j] = x[j];
    dist_out[base + i] = dist;
    pp_out[base + i] = pp;
    alpha_out[base + i] = a;
  }
}

// RandomWalkABC with the RMMetropolisDiagStepsize correction (abc/mcmc.py:105-140,
// mcmc/metropolis.py:73-160) at the sampler's defaults (threshold and stepsize unset: 50 and 1 per
// dimension, post_mean x_0, diag_post_cov = stepsize d / 2.38^2), one thread per chain.  Each step
// is the fixed-parameter chain's step with the current threshold and per-dimension stepsize,
// followed by, with rm = scale iter^-neg_exp (iter = the step index; the library's exp and log):
//   threshold <- exp(log threshold - rm (alpha - target))       (log Robbins-Monro, increasing)
//   r = min(rm, 1 - 1e-3); diag <- (1 - r) diag + r (x - post_mean)^2; post_mean <- (1 - r) post_mean + r x;
//   stepsize <- diag / d * 2.38^2
template <int D, int DY>
__global__ void __launch_bounds__(128) k_abc_mcmc_rm_lg(const __grid_constant__ ABCP<D, DY> p, int64_t B, int64_t n,
                                                         const uint32_t *keys, float target, float scale,
                                                         float neg_exp, float *__restrict__ x_out,
                                                         float *__restrict__ alpha_out, float *__restrict__ thr_out,
                                                         float *__restrict__ st_out) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= B) return;
  uint32_t K0 = keys[2 * b], K1 = keys[2 * b + 1], a0, a1, t0, t1;
  split_at(K0, K1, 2, 1, a0, a1);
  split_at(K0, K1, 2, 0, t0, t1);
  split_at(t0, t1, 2, 0, K0, K1);  // prior potential
  uint32_t bits[D];
  bits_vec<D>(a0, a1, bits, p.one);
  float e[D], x[D];
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(bits[j]);
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float v = __fmul_rn(p.C0[r * D], e[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) v = __fmaf_rn(p.C0[r * D + k], e[k], v);
    x[r] = __fadd_rn(p.m0[r], v);
  }
  float pp = abc_prior_potential<D, DY>(p, x);
  split_at(K0, K1, 2, 0, t0, t1);  // the initial simulation takes split(K)[1]; its distance is unused
  K0 = t0;
  K1 = t1;
  float thr = 50.0f, st[D], pm[D], dg[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    st[j] = 1.0f;
    pm[j] = x[j];
    dg[j] = __fdiv_rn(__fmul_rn(st[j], (float)D), 5.6644f);
  }
  const int64_t base = b * n;
#pragma unroll
  for (int j = 0; j < D; ++j) {
    x_out[base * D + j] = x[j];
    st_out[base * D + j] = st[j];
  }
  alpha_out[base] = 1.0f;
  thr_out[base] = thr;
#pragma unroll 1
  for (int64_t i = 1; i < n; ++i) {
    split_at(K0, K1, 2, 0, t0, t1);  // always
    uint32_t sk4[8];                 // split(t, 4): 0 new extra key, 1 proposal normals, 3 simulation
    split4(t0, t1, sk4);
    bits_vec<D>(sk4[2], sk4[3], bits, p.one);
    float xp[D];
#pragma unroll
    for (int j = 0; j < D; ++j) xp[j] = __fadd_rn(x[j], __fmul_rn(__fsqrt_rn(st[j]), bits_to_normal(bits[j])));
    const float ppn = abc_prior_potential<D, DY>(p, xp);
    const float dn = abc_sim_distance<D, DY>(p, xp, sk4[6], sk4[7]);
    float a = __fmul_rn(expf_(__fsub_rn(pp, ppn)), dn < thr ? 1.0f : 0.0f);
    a = a != a ? 0.0f : fminf(1.0f, a);
    uint32_t u0, u1, v0, v1;
    split2(sk4[0], sk4[1], u0, u1, v0, v1);
    const float u = bits_to_unit(bits_at(v0, v1, 1, 0));
    if (u < a) {
#pragma unroll
      for (int j = 0; j < D; ++j) x[j] = xp[j];
      pp = ppn;
    }
    K0 = u0;
    K1 = u1;
    const float rm = __fmul_rn(scale, expf_(__fmul_rn(-neg_exp, logf_((float)i))));
    thr = expf_(__fsub_rn(logf_(thr), __fmul_rn(rm, __fsub_rn(a, target))));
    const float r2 = fminf(rm, 0.999f), q2 = __fsub_rn(1.0f, r2);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const float dv = __fsub_rn(x[j], pm[j]);
      dg[j] = __fadd_rn(__fmul_rn(q2, dg[j]), __fmul_rn(r2, __fmul_rn(dv, dv)));
      pm[j] = __fadd_rn(__fmul_rn(q2, pm[j]), __fmul_rn(r2, x[j]));
      st[j] = __fmul_rn(__fdiv_rn(dg[j], (float)D), 5.6644f);
      x_out[(base + i) * D + j] = x[j];
      st_out[(base + i) * D + j] = st[j];
    }
    alpha_out[base + i] = a;
    thr_out[base + i] = thr;
  }
}

template <int D, int DY>
static int abc_mcmc_rm_lg(const mgb_abc_lg_model *m, int64_t B, int64_t n, const uint32_t *keys, float target,
                          float scale, float neg_exp, float *x, float *alpha, float *thr, float *st, cudaStream_t s) {
  k_abc_mcmc_rm_lg<D, DY><<<(unsigned)((B + 127) / 128), 128, 0, s>>>(pack_abc<D, DY>(m), B, n, keys, target, scale,
                                                                      neg_exp, x, alpha, thr, st);
  return launch_status();
}

template <int D, int DY>
static int abc_mcmc_lg(const mgb_abc_lg_model *m, int64_t B, int64_t n, const uint32_t *keys, float stepsize,
                       float thr, float *x, float *dist, float *pp, float *alpha, cudaStream_t s) {
  k_abc_mcmc_lg<D, DY><<<(unsigned)((B + 127) / 128), 128, 0, s>>>(pack_abc<D, DY>(m), B, n, keys, stepsize, thr, x,
                                                                   dist, pp, alpha);
  return launch_status();
}

#define MGB_ABC_DISPATCH(FN, ...)                                     \
  do {                                                                \
    const int d_ = m->d, dy_ = m->dy;                                 \
    if (d_ == 1 && dy_ == 1) return FN<1, 1>(__VA_ARGS__);            \
    if (d_ == 2 && dy_ == 1) return FN<2, 1>(__VA_ARGS__);            \
    if (d_ == 2 && dy_ == 2) return FN<2, 2>(__VA_ARGS__);            \
    if (d_ == 3 && dy_ == 2) return FN<3, 2>(__VA_ARGS__);            \
    if (d_ == 3 && dy_ == 3) return FN<3, 3>(__VA_ARGS__);            \
    if (d_ == 5 && dy_ == 5) return FN<5, 5>(__VA_ARGS__);            \
    if (d_ == 10 && dy_ == 10) return FN<10, 10>(__VA_ARGS__);        \
    return ERR_UNSUPPORTED;                                           \
  } while (0)

static bool abc_ok(const mgb_abc_smc_config *cfg, const mgb_abc_lg_model *m) {
  return cfg && m && m->m0 && m->C0 && m->P0 && m->H && m->L && m->data && cfg->B >= 1 && cfg->N >= 2 &&
         cfg->N <= MGB_ABC_MAX_N && cfg->mcmc_steps >= 1 && cfg->max_iter >= 0 && cfg->max_iter <= 100000 &&
         cfg->n_schedule >= 0 && (cfg->n_schedule == 0 || cfg->schedule);
}

}  // namespace mgb

using namespace mgb;

extern "C" {

size_t mgb_abc_smc_workspace(const mgb_abc_smc_config *cfg, int32_t d) {
  if (!cfg || d < 1) return 0;
  Carver c(nullptr);
  carve_abc(c, cfg->B, cfg->N, d, abc_hist_len(cfg), cfg->n_schedule);
  return c.bytes();
}

int mgb_abc_smc_views(const mgb_abc_smc_config *cfg, int32_t d, void *ws, mgb_abc_views *out) {
  if (!cfg || !ws || !out || d < 1) return ERR_BAD_ARG;
  const ABCWs w = abc_ws(cfg, d, ws);
  out->value = w.value;
  out->distance = w.dist;
  out->log_weight = w.lw;
  out->prior_potential = w.pp;
  out->alpha = w.alpha;
  out->stepsize = w.stepsize;
  out->threshold = w.threshold;
  out->ess = w.ess;
  out->alpha_mean = w.alpha_mean;
  out->iter = w.iter;
  out->active = w.active;
  out->hist_threshold = w.hist_thr;
  out->hist_ess = w.hist_ess;
  out->hist_alpha = w.hist_alpha;
  out->hist_resampled = w.hist_res;
  out->hist_len = abc_hist_len(cfg);
  return OK;
}

int mgb_abc_smc_init(const mgb_abc_smc_config *cfg, const mgb_abc_lg_model *m, const uint32_t *keys, void *ws,
                     size_t ws_bytes, void *stream) {
  if (!abc_ok(cfg, m) || !keys || !ws) return ERR_BAD_ARG;
  if (ws_bytes < mgb_abc_smc_workspace(cfg, m->d)) return ERR_WORKSPACE;
  MGB_ABC_DISPATCH(abc_init, cfg, m, keys, ws, (cudaStream_t)stream);
}

int mgb_abc_smc_step(const mgb_abc_smc_config *cfg, const mgb_abc_lg_model *m, void *ws, size_t ws_bytes,
                     void *stream) {
  if (!abc_ok(cfg, m) || !ws) return ERR_BAD_ARG;
  if (ws_bytes < mgb_abc_smc_workspace(cfg, m->d)) return ERR_WORKSPACE;
  MGB_ABC_DISPATCH(abc_step, cfg, m, ws, (cudaStream_t)stream);
}

size_t mgb_abc_gk_workspace(const mgb_abc_smc_config *cfg, int32_t d) {
  if (!cfg || (d != 1 && d != 4)) return 0;
  Carver c(nullptr);
  carve_abc(c, cfg->B, cfg->N, d, abc_hist_len(cfg), cfg->n_schedule);
  carve_gk(c, cfg->B, cfg->N, d);
  return c.bytes();
}

static bool abc_cfg_ok(const mgb_abc_smc_config *cfg) {
  return cfg && cfg->B >= 1 && cfg->N >= 2 && cfg->N <= MGB_ABC_MAX_N && cfg->mcmc_steps >= 1 &&
         cfg->max_iter >= 0 && cfg->max_iter <= 100000 && cfg->n_schedule >= 0 &&
         (cfg->n_schedule == 0 || cfg->schedule);
}

int mgb_abc_gk_smc_init(const mgb_abc_smc_config *cfg, const mgb_abc_gk_model *m, const uint32_t *keys, void *ws,
                        size_t ws_bytes, void *stream) {
  if (!abc_cfg_ok(cfg) || !gk_ok(m) || !m->data_dev || !keys || !ws) return ERR_BAD_ARG;
  if (ws_bytes < mgb_abc_gk_workspace(cfg, m->d)) return ERR_WORKSPACE;
  if (m->d == 4) return gk_init<4>(cfg, m, keys, ws, (cudaStream_t)stream);
  return gk_init<1>(cfg, m, keys, ws, (cudaStream_t)stream);
}

int mgb_abc_gk_smc_step(const mgb_abc_smc_config *cfg, const mgb_abc_gk_model *m, void *ws, size_t ws_bytes,
                        void *stream) {
  if (!abc_cfg_ok(cfg) || !gk_ok(m) || !m->data_dev || !ws) return ERR_BAD_ARG;
  if (ws_bytes < mgb_abc_gk_workspace(cfg, m->d)) return ERR_WORKSPACE;
  if (m->d == 4) return gk_step<4>(cfg, m, ws, (cudaStream_t)stream);
  return gk_step<1>(cfg, m, ws, (cudaStream_t)stream);
}

size_t mgb_abc_vanilla_workspace(int64_t n) {
  if (n < 1) return 0;
  Carver c(nullptr);
  carve_vabc(c, n);
  return c.bytes();
}

int mgb_abc_vanilla_lg(const mgb_abc_lg_model *m, int64_t n, const uint32_t *key, float threshold,
                       float acceptance_rate, void *ws, size_t ws_bytes, float *x, float *pp, float *dist, float *lw,
                       float *threshold_out, void *stream) {
  if (!m || !m->m0 || !m->C0 || !m->P0 || !m->H || !m->L || !m->data || n < 2 || n > 0x7FFFFFFFll || !key || !ws ||
      !x || !pp || !dist || !lw || !threshold_out)
    return ERR_BAD_ARG;
  if (ws_bytes < mgb_abc_vanilla_workspace(n)) return ERR_WORKSPACE;
  MGB_ABC_DISPATCH(vabc_lg, m, n, key, threshold, acceptance_rate, ws, x, pp, dist, lw, threshold_out,
                   (cudaStream_t)stream);
}

int mgb_abc_vanilla_gk(const mgb_abc_gk_model *m, int64_t n, const uint32_t *key, float threshold,
                       float acceptance_rate, void *ws, size_t ws_bytes, float *x, float *pp, float *dist, float *lw,
                       float *threshold_out, void *stream) {
  if (!gk_ok(m) || !m->data_dev || n < 2 || n > 0x7FFFFFFFll || !key || !ws || !x || !pp || !dist || !lw ||
      !threshold_out)
    return ERR_BAD_ARG;
  if (ws_bytes < mgb_abc_vanilla_workspace(n)) return ERR_WORKSPACE;
  if (m->d == 4)
    return vabc_gk<4>(m, n, key, threshold, acceptance_rate, ws, x, pp, dist, lw, threshold_out, (cudaStream_t)stream);
  return vabc_gk<1>(m, n, key, threshold, acceptance_rate, ws, x, pp, dist, lw, threshold_out, (cudaStream_t)stream);
}

int mgb_abc_mcmc_lg(const mgb_abc_lg_model *m, int64_t B, int64_t n, const uint32_t *keys, float stepsize,
                    float threshold, float *x, float *dist, float *pp, float *alpha, void *stream) {
  if (!m || !m->m0 || !m->C0 || !m->P0 || !m->H || !m->L || !m->data || B < 1 || B > 0x7FFFFFFFll || n < 1 ||
      !keys || !x || !dist || !pp || !alpha || !(stepsize >= 0.0f))
    return ERR_BAD_ARG;
  MGB_ABC_DISPATCH(abc_mcmc_lg, m, B, n, keys, stepsize, threshold, x, dist, pp, alpha, (cudaStream_t)stream);
}

int mgb_abc_mcmc_rm_lg(const mgb_abc_lg_model *m, int64_t B, int64_t n, const uint32_t *keys, float target,
                       float scale, float neg_exp, float *x, float *alpha, float *threshold, float *stepsize,
                       void *stream) {
  if (!m || !m->m0 || !m->C0 || !m->P0 || !m->H || !m->L || !m->data || B < 1 || B > 0x7FFFFFFFll || n < 1 ||
      !keys || !x || !alpha || !threshold || !stepsize || !(target == target) || !(scale > 0.0f) ||
      !(neg_exp >= 0.0f) || scale > 3.0e38f || neg_exp > 3.0e38f)
    return ERR_BAD_ARG;
  MGB_ABC_DISPATCH(abc_mcmc_rm_lg, m, B, n, keys, target, scale, neg_exp, x, alpha, threshold, stepsize,
                   (cudaStream_t)stream);
}

int mgb_abc_mcmc_gk(const mgb_abc_gk_model *m, int64_t B, int64_t n, const uint32_t *keys, float stepsize,
                    float threshold, float *x, float *dist, float *pp, float *alpha, void *stream) {
  if (!gk_ok(m) || !m->data_dev || B < 1 || B > 0x7FFFFFFFll || n < 1 || !keys || !x || !dist || !pp || !alpha ||
      !(stepsize >= 0.0f))
    return ERR_BAD_ARG;
  const GKP p = pack_gk(m);
  if (m->d == 4)
    k_abc_mcmc_gk<4><<<(unsigned)B, GK_TPB, 0, (cudaStream_t)stream>>>(p, B, n, keys, stepsize, threshold, x, dist,
                                                                       pp, alpha);
  else
    k_abc_mcmc_gk<1><<<(unsigned)B, GK_TPB, 0, (cudaStream_t)stream>>>(p, B, n, keys, stepsize, threshold, x, dist,
                                                                       pp, alpha);
  return launch_status();
}

int mgb_abc_mcmc_rm_gk(const mgb_abc_gk_model *m, int64_t B, int64_t n, const uint32_t *keys, float target,
                       float scale, float neg_exp, float *x, float *alpha, float *threshold, float *stepsize,
                       void *stream) {
  if (!gk_ok(m) || !m->data_dev || B < 1 || B > 0x7FFFFFFFll || n < 1 || !keys || !x || !alpha || !threshold ||
      !stepsize || !(target == target) || !(scale > 0.0f) || !(neg_exp >= 0.0f) || scale > 3.0e38f ||
      neg_exp > 3.0e38f)
    return ERR_BAD_ARG;
  const GKP p = pack_gk(m);
  if (m->d == 4)
    k_abc_mcmc_rm_gk<4><<<(unsigned)B, GK_TPB, 0, (cudaStream_t)stream>>>(p, B, n, keys, target, scale, neg_exp, x,
                                                                          alpha, threshold, stepsize);
  else
    k_abc_mcmc_rm_gk<1><<<(unsigned)B, GK_TPB, 0, (cudaStream_t)stream>>>(p, B, n, keys, target, scale, neg_exp, x,
                                                                          alpha, threshold, stepsize);
  return launch_status();
}

int mgb_abc_gk_simulate(const mgb_abc_gk_model *m, int64_t P, const float *x, const uint32_t *keys, float *summary,
                        float *dist, void *stream) {
  if (!gk_ok(m) || P < 1 || P > 0x7FFFFFFFll || !x || !keys || (!summary && !dist) || (dist && !m->data_dev))
    return ERR_BAD_ARG;
  k_gk_sim<<<(unsigned)P, GK_TPB, 0, (cudaStream_t)stream>>>(pack_gk(m), P, x, keys, nullptr, dist, summary);
  return launch_status();
}

}  // extern "C"
