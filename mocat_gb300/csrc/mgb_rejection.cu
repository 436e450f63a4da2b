// Backward simulation and particle stitching by rejection sampling
// (maximum_rejections > 0), for the linear-Gaussian, the non-linear 1-D
// benchmark and the stochastic-volatility transitions.
//
// Reference: rejection_resampling (mocat/src/ssm/backward.py:54-169) driven by
// backward_simulation_rejection (:172-214), and rejection_stitching
// (mocat/src/ssm/online_smoothing.py:59-175) driven by fixed_lag_stitching
// (:178-209).  Both are one algorithm: n items, each with a fixed state, each
// draw an index into a pool of Np particles with log-weights lw; the density of
// the pair (i, j) is exp(-transition_potential):
//   backward simulation  item = sample x_{t+1}^i, pool = filter particles x_t^j,
//                        potential(x_{t+1}^i - mean(x_t^j));
//   stitching            item = x0_i, pool = x1_j, potential(x1_j - mean(x0_i)).
// With (c0, u0, k0) = split(key, 3):
//   prerun   idx_i = categorical(c0, lw, (n,))_i (one (n, Np) Gumbel draw),
//            dens_i = exp(-potential(i, idx_i)), B = max dens > ibp ? max dens * inflation : ibp,
//            nya_i = uniform(u0, (n,))_i > dens_i / B, key_i = split(k0, n)_i, evals = n, iter = 1
//   while any(nya) and iter < maximum_rejections:
//            evals += #nya; for nya_i: (key_i, c, u) = split(key_i, 3), idx_i = categorical(c, lw),
//            dens_i = exp(-potential(i, idx_i)), nya_i = uniform(u) > dens_i / B (others: dens 0);
//            if max dens > B: B = max dens * inflation and every item is unaccepted again; iter += 1
//   final    for nya_i: idx_i = categorical(key_i, lw - potential(i, .)); evals += Np * #nya.
// jnp.max propagates NaN and NaN comparisons are false; both hold here.
//
// GPU layout: one CTA per item for each draw (only unaccepted items do work);
// the loop's state between launches is a ring of three slots {max density bits
// (unsigned order, so any NaN is the maximum), unaccepted count, bound}: the
// launch for iteration k reads slot k-1, derives reset / bound / count itself
// (every CTA the same), accumulates into slot k and clears slot k+1.  A launch
// that finds the loop over sets a done flag and records the last iteration; the
// later launches return at once.  The host launches iterations in groups and
// reads the flag between groups, so these entry points synchronise their
// stream.
#include <type_traits>
#include <vector>

#include "mgb_transition.cuh"

namespace mgb {

constexpr int RJ_POLL = 8;           // iteration launches between reads of the done flag
constexpr uint32_t RJ_NAN = 0x7fc00000u;

struct RejSlot {
  uint32_t maxbits;  // max over the iteration's densities, as unsigned bits
  uint32_t count;    // items unaccepted after the iteration, before any reset
  float bound;       // the bound the iteration used
  uint32_t pad;
};

struct RejCtl {
  uint32_t pre_max;  // prerun max density bits
  int32_t done, last;
  int32_t pad;
  long long evals;
};

struct RejCfg {
  int32_t max_rej;
  float ibp, infl;
};

// iteration k's (reset, bound, unaccepted count) from iteration k-1's slot
__device__ __forceinline__ void rej_state(const RejSlot &s, float infl, int64_t n, bool &reset, float &bound,
                                          int64_t &count) {
  const float mx = asf(s.maxbits);
  reset = mx > s.bound;
  bound = reset ? __fmul_rn(mx, infl) : s.bound;
  count = reset ? n : (int64_t)s.count;
}

// transition potential of item vector u (already a mean for stitching) against pool element j
template <class TP, bool BACK>
__device__ __forceinline__ float rej_potential(const TP &p, const float *u, const float *__restrict__ pool, int64_t Np,
                                               int64_t j) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  float diff[DC];
#pragma unroll
  for (int r = 0; r < D; ++r) diff[r] = BACK ? __fsub_rn(u[r], pool[r * Np + j]) : __fsub_rn(pool[r * Np + j], u[r]);
  return p.potential(diff);
}

// argmax_j gumbel(key, (Np,))_j + lw_j (- potential(i, j) when FULL), the Gumbel bits of j and
// j + ceil(Np/2) from one cipher call
template <class TP, bool BACK, bool FULL>
__device__ __forceinline__ int32_t rej_categorical(const TP &p, uint32_t k0, uint32_t k1, int64_t Np,
                                                   const float *__restrict__ lw, const float *u,
                                                   const float *__restrict__ pool, Best *sm) {
  const int64_t h = (Np + 1) >> 1;
  Best b{-INFINITY, 0, 0};
  for (int64_t q = threadIdx.x; q < h; q += FB_TPB) {
    uint32_t r0, r1;
    threefry2x32_m(k0, k1, (uint32_t)q, q + h < Np ? (uint32_t)(q + h) : 0u, p.one, r0, r1);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int64_t j = s ? q + h : q;
      if (j >= Np) break;
      const float g = bits_to_gumbel(s ? r1 : r0);
      const float w = FULL ? __fsub_rn(lw[j], rej_potential<TP, BACK>(p, u, pool, Np, j)) : lw[j];
      best_take(b, __fadd_rn(g, w), (int32_t)j);
    }
  }
  return block_argmax<FB_TPB>(b, sm);
}

// prerun draw: item i takes row i of the (n, Np) Gumbel array of split(key, 3)[0]
template <class TP, bool BACK>
__global__ void __launch_bounds__(FB_TPB) k_rej_prerun(const __grid_constant__ TP p, int64_t n, int64_t Np,
                                                        const float *__restrict__ itm, const float *__restrict__ pool,
                                                        const float *__restrict__ lw, const uint32_t *key,
                                                        int32_t *__restrict__ idx, float *__restrict__ dens,
                                                        RejCtl *ctl) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  __shared__ Best sm[FB_TPB / 32];
  __shared__ uint32_t kc[2];
  const int64_t i = blockIdx.x;
  if (threadIdx.x == 0) split_at(key[0], key[1], 3, 0, kc[0], kc[1]);
  __syncthreads();
  const uint32_t k0 = kc[0], k1 = kc[1];
  const uint64_t tot = (uint64_t)n * (uint64_t)Np;
  Best b{-INFINITY, 0, 0};
  for (int64_t j = threadIdx.x; j < Np; j += FB_TPB) {
    const float g = bits_to_gumbel(bits_at(k0, k1, tot, (uint64_t)i * Np + j));
    best_take(b, __fadd_rn(g, lw[j]), (int32_t)j);
  }
  const int32_t bi = block_argmax<FB_TPB>(b, sm);
  if (threadIdx.x == 0) {
    float u[DC];
#pragma unroll
    for (int r = 0; r < D; ++r) u[r] = itm[r * n + i];
    const float dv = expf_(-rej_potential<TP, BACK>(p, u, pool, Np, bi));
    idx[i] = bi;
    dens[i] = dv;
    atomicMax(&ctl->pre_max, asu(dv));
  }
}

// the prerun draw for an even number of items: element (i, j) and (i + n/2, j) of the (n, Np)
// Gumbel array are the two halves of one cipher call (counters i Np + j and i Np + j + n Np / 2),
// so CTA i takes items i and i + n/2 and spends one call per pool element
template <class TP, bool BACK>
__global__ void __launch_bounds__(FB_TPB) k_rej_prerun_pairs(const __grid_constant__ TP p, int64_t n, int64_t Np,
                                                              const float *__restrict__ itm,
                                                              const float *__restrict__ pool,
                                                              const float *__restrict__ lw, const uint32_t *key,
                                                              int32_t *__restrict__ idx, float *__restrict__ dens,
                                                              RejCtl *ctl) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  __shared__ Best sm0[FB_TPB / 32], sm1[FB_TPB / 32];
  __shared__ uint32_t kc[2];
  const int64_t i = blockIdx.x, half = n >> 1;
  if (threadIdx.x == 0) split_at(key[0], key[1], 3, 0, kc[0], kc[1]);
  __syncthreads();
  const uint32_t k0 = kc[0], k1 = kc[1];
  const uint64_t h = (uint64_t)half * (uint64_t)Np;
  Best b0{-INFINITY, 0, 0}, b1{-INFINITY, 0, 0};
  for (int64_t j = threadIdx.x; j < Np; j += FB_TPB) {
    const uint64_t c = (uint64_t)i * Np + j;
    uint32_t r0, r1;
    threefry2x32_m(k0, k1, (uint32_t)c, (uint32_t)(c + h), p.one, r0, r1);
    const float l = lw[j];
    best_take(b0, __fadd_rn(bits_to_gumbel(r0), l), (int32_t)j);
    best_take(b1, __fadd_rn(bits_to_gumbel(r1), l), (int32_t)j);
  }
  const int32_t bi0 = block_argmax<FB_TPB>(b0, sm0);
  const int32_t bi1 = block_argmax<FB_TPB>(b1, sm1);
  if (threadIdx.x == 0) {
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
      const int64_t it = s ? i + half : i;
      const int32_t bi = s ? bi1 : bi0;
      float u[DC];
#pragma unroll
      for (int r = 0; r < D; ++r) u[r] = itm[r * n + it];
      const float dv = expf_(-rej_potential<TP, BACK>(p, u, pool, Np, bi));
      idx[it] = bi;
      dens[it] = dv;
      atomicMax(&ctl->pre_max, asu(dv));
    }
  }
}

// prerun acceptance: the initial bound, nya_i, the items' keys, slot 0
__global__ void k_rej_accept(int64_t n, RejCfg cfg, const uint32_t *key, const float *__restrict__ dens,
                             uint8_t *__restrict__ nya, uint32_t *__restrict__ keys, RejSlot *ring, RejCtl *ctl) {
  const float mx = asf(ctl->pre_max);
  const float bound = mx > cfg.ibp ? __fmul_rn(mx, cfg.infl) : cfg.ibp;
  uint32_t u0, u1, s0, s1;
  split_at(key[0], key[1], 3, 1, u0, u1);
  split_at(key[0], key[1], 3, 2, s0, s1);
  uint32_t cnt = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float u = bits_to_unit(bits_at(u0, u1, (uint64_t)n, (uint64_t)i));
    const bool a = u > __fdiv_rn(dens[i], bound);
    nya[i] = a;
    cnt += a;
    uint32_t a0, a1;
    split_at(s0, s1, (uint64_t)n, (uint64_t)i, a0, a1);
    keys[2 * i] = a0;
    keys[2 * i + 1] = a1;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&ring[0].count, cnt);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ring[0].bound = bound;
    ring[0].maxbits = RJ_NAN;  // no reset after the prerun
    ctl->evals = n;
  }
}

// iteration k >= 1 of the rejection loop
template <class TP, bool BACK>
__global__ void __launch_bounds__(FB_TPB) k_rej_iter(const __grid_constant__ TP p, int32_t k, int64_t n, int64_t Np,
                                                      const float *__restrict__ itm, const float *__restrict__ pool,
                                                      const float *__restrict__ lw, RejCfg cfg,
                                                      int32_t *__restrict__ idx, uint32_t *__restrict__ keys,
                                                      uint8_t *__restrict__ nya, RejSlot *ring, RejCtl *ctl) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  __shared__ Best sm[FB_TPB / 32];
  __shared__ uint32_t ks[6];
  __shared__ float sb;
  __shared__ int go;
  __shared__ float su[DC];
  const int64_t i = blockIdx.x;
  if (threadIdx.x == 0) {
    int g = 0;
    if (!ctl->done) {
      bool reset;
      float bound;
      int64_t cnt;
      rej_state(ring[(k - 1) % 3], cfg.infl, n, reset, bound, cnt);
      if (cnt == 0 || k >= cfg.max_rej) {
        if (i == 0) {
          ctl->done = 1;
          ctl->last = k - 1;
        }
      } else {
        if (i == 0) {
          ring[k % 3].bound = bound;
          ring[(k + 1) % 3] = RejSlot{0u, 0u, 0.0f, 0u};
          ctl->evals += cnt;
        }
        if (reset || nya[i]) {
          g = 1;
          sb = bound;
          const uint32_t a = keys[2 * i], b = keys[2 * i + 1];
          split_at(a, b, 3, 0, ks[0], ks[1]);
          split_at(a, b, 3, 1, ks[2], ks[3]);
          split_at(a, b, 3, 2, ks[4], ks[5]);
#pragma unroll
          for (int r = 0; r < D; ++r) su[r] = itm[r * n + i];
        }
      }
    }
    go = g;
  }
  __syncthreads();
  if (!go) return;
  const int32_t bi = rej_categorical<TP, BACK, false>(p, ks[2], ks[3], Np, lw, su, pool, sm);
  if (threadIdx.x == 0) {
    const float dv = expf_(-rej_potential<TP, BACK>(p, su, pool, Np, bi));
    const float u = bits_to_unit(bits_at(ks[4], ks[5], 1, 0));
    const bool a = u > __fdiv_rn(dv, sb);
    idx[i] = bi;
    keys[2 * i] = ks[0];
    keys[2 * i + 1] = ks[1];
    nya[i] = a;
    atomicMax(&ring[k % 3].maxbits, asu(dv));
    if (a) atomicAdd(&ring[k % 3].count, 1u);
  }
}

// items still unaccepted after the loop: the full categorical with their keys
template <class TP, bool BACK>
__global__ void __launch_bounds__(FB_TPB) k_rej_final(const __grid_constant__ TP p, int64_t n, int64_t Np,
                                                       const float *__restrict__ itm, const float *__restrict__ pool,
                                                       const float *__restrict__ lw, RejCfg cfg,
                                                       int32_t *__restrict__ idx, const uint32_t *__restrict__ keys,
                                                       const uint8_t *__restrict__ nya, const RejSlot *ring,
                                                       const RejCtl *ctl, long long *evals) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  __shared__ Best sm[FB_TPB / 32];
  __shared__ uint32_t ks[2];
  __shared__ int go;
  __shared__ float su[DC];
  const int64_t i = blockIdx.x;
  if (threadIdx.x == 0) {
    bool reset;
    float bound;
    int64_t cnt;
    rej_state(ring[ctl->last % 3], cfg.infl, n, reset, bound, cnt);
    if (i == 0) *evals = ctl->evals + (long long)Np * cnt;
    go = reset || nya[i];
    ks[0] = keys[2 * i];
    ks[1] = keys[2 * i + 1];
#pragma unroll
    for (int r = 0; r < D; ++r) su[r] = itm[r * n + i];
  }
  __syncthreads();
  if (!go) return;
  const int32_t bi = rej_categorical<TP, BACK, true>(p, ks[0], ks[1], Np, lw, su, pool, sm);
  if (threadIdx.x == 0) idx[i] = bi;
}

struct RejWs {
  uint32_t *keys;
  uint8_t *nya;
  float *dens;
  RejSlot *ring;
  RejCtl *ctl;
};

static RejWs carve_rej(Carver &c, int64_t n) {
  RejWs w;
  w.keys = c.take<uint32_t>(2 * (size_t)n);
  w.nya = c.take<uint8_t>((size_t)n);
  w.dens = c.take<float>((size_t)n);
  w.ring = c.take<RejSlot>(3);
  w.ctl = c.take<RejCtl>(1);
  return w;
}

// one rejection draw of n items from a pool of Np: idx (n), *evals the transition evaluations
template <class TP, bool BACK>
static int rej_run(const TP &p, const RejCfg &cfg, int64_t n, int64_t Np, const float *itm, const float *pool,
                   const float *lw, const uint32_t *key, int32_t *idx, long long *evals, const RejWs &w,
                   cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(w.ring, 0, 3 * sizeof(RejSlot), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.ctl, 0, sizeof(RejCtl), s);
  if (e != cudaSuccess) return ERR_CUDA;
  int st;
  if (n % 2 == 0)
    k_rej_prerun_pairs<TP, BACK><<<(unsigned)(n / 2), FB_TPB, 0, s>>>(p, n, Np, itm, pool, lw, key, idx, w.dens,
                                                                       w.ctl);
  else
    k_rej_prerun<TP, BACK><<<(unsigned)n, FB_TPB, 0, s>>>(p, n, Np, itm, pool, lw, key, idx, w.dens, w.ctl);
  if ((st = launch_status())) return st;
  k_rej_accept<<<grid_for(n, 256), 256, 0, s>>>(n, cfg, key, w.dens, w.nya, w.keys, w.ring, w.ctl);
  if ((st = launch_status())) return st;
  for (int32_t k = 1; k <= cfg.max_rej; ++k) {
    k_rej_iter<TP, BACK><<<(unsigned)n, FB_TPB, 0, s>>>(p, k, n, Np, itm, pool, lw, cfg, idx, w.keys, w.nya, w.ring,
                                                         w.ctl);
    if ((st = launch_status())) return st;
    if (k % RJ_POLL == 0 && k < cfg.max_rej) {
      int32_t done = 0;
      e = cudaMemcpyAsync(&done, &w.ctl->done, sizeof(done), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return ERR_CUDA;
      if (done) break;
    }
  }
  k_rej_final<TP, BACK><<<(unsigned)n, FB_TPB, 0, s>>>(p, n, Np, itm, pool, lw, cfg, idx, w.keys, w.nya, w.ring,
                                                        w.ctl, evals);
  return launch_status();
}

// backward_simulation_rejection: t_all (device, T) for policies with a drift
template <class TP>
static int ffbsi_rej_run(TP p, const RejCfg &cfg, const float *t_all, int64_t T, int64_t N, int64_t M,
                         const float *x_hist, const float *lw_hist, const uint32_t *key, float *out, int32_t *idx,
                         long long *evals, void *ws, size_t ws_bytes, cudaStream_t s,
                         const float *pqs_host = nullptr) {
  constexpr int TD = take_dim<TP>();
  const int D = p.dim();
  Carver c(ws);
  float *fx = c.take<float>((size_t)D * N);
  uint32_t *tkeys = c.take<uint32_t>(2 * (size_t)T);
  const RejWs w = carve_rej(c, M);
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
  if (cudaMemsetAsync(evals, 0, sizeof(long long), s) != cudaSuccess) return ERR_CUDA;
  int st = mgb_split(key, T, tkeys, s);
  if (st) return st;
  const size_t xs = (size_t)D * N;
  k_ffbsi_last<<<(unsigned)M, FB_TPB, 0, s>>>(N, M, lw_hist + (size_t)(T - 1) * N, tkeys + 2 * (T - 1),
                                              idx + (size_t)(T - 1) * M);
  if ((st = launch_status())) return st;
  k_ffbsi_take<TD><<<grid_for(M, 256), 256, 0, s>>>(N, M, x_hist + (size_t)(T - 1) * xs, idx + (size_t)(T - 1) * M,
                                                    out + (size_t)(T - 1) * D * M, D);
  if ((st = launch_status())) return st;
  for (int64_t t = T - 2; t >= 0; --t) {
    if constexpr (TP::kDrift) p.tp = t_all + t;
    if constexpr (std::is_same<TP, SVT>::value) p.pqs = pqs_host[t];
    k_ffbsi_fx<TP><<<(unsigned)((N + FB_TPB - 1) / FB_TPB), FB_TPB, 0, s>>>(p, N, x_hist + (size_t)t * xs, fx);
    if ((st = launch_status())) return st;
    st = rej_run<TP, true>(p, cfg, M, N, out + (size_t)(t + 1) * D * M, fx, lw_hist + (size_t)t * N, tkeys + 2 * t,
                           idx + (size_t)t * M, evals + t + 1, w, s);
    if (st) return st;
    k_ffbsi_take<TD><<<grid_for(M, 256), 256, 0, s>>>(N, M, x_hist + (size_t)t * xs, idx + (size_t)t * M,
                                                      out + (size_t)t * D * M, D);
    if ((st = launch_status())) return st;
  }
  return OK;
}

// rejection_stitching: M items x0 (their means first), pool x1 of M
template <class TP>
static int stitch_rej_run(const TP &p, const RejCfg &cfg, int64_t M, const float *x0, const float *x1,
                          const float *lw1, const uint32_t *key, int32_t *idx, long long *evals, void *ws,
                          size_t ws_bytes, cudaStream_t s) {
  const int D = p.dim();
  Carver c(ws);
  float *fx0 = c.take<float>((size_t)D * M);
  const RejWs w = carve_rej(c, M);
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
  k_ffbsi_fx<TP><<<(unsigned)((M + FB_TPB - 1) / FB_TPB), FB_TPB, 0, s>>>(p, M, x0, fx0);
  int st = launch_status();
  if (st) return st;
  return rej_run<TP, false>(p, cfg, M, M, fx0, x1, lw1, key, idx, evals, w, s);
}

static size_t ffbsi_rej_bytes(int64_t N, int64_t M, int64_t T, int32_t d) {
  Carver c(nullptr);
  c.take<float>((size_t)d * N);
  c.take<uint32_t>(2 * (size_t)T);
  carve_rej(c, M);
  return c.bytes();
}

static size_t stitch_rej_bytes(int64_t M, int32_t d) {
  Carver c(nullptr);
  c.take<float>((size_t)d * M);
  carve_rej(c, M);
  return c.bytes();
}

static bool rej_cfg_ok(const mgb_rejection_config *cfg, RejCfg &rc) {
  if (!cfg || cfg->maximum_rejections < 1) return false;
  rc.max_rej = cfg->maximum_rejections;
  rc.ibp = cfg->init_bound_param;
  rc.infl = cfg->bound_inflation;
  return true;
}

static bool rej_sizes_ok(int64_t T, int64_t N, int64_t M) {
  return T >= 1 && N >= 1 && N <= 0x7FFFFFFFll && M >= 1 && M <= 0x7FFFFFFFll &&
         (uint64_t)M * (uint64_t)N < (1ull << 32);
}

template <int D, bool RT = false>
static int ffbsi_rej_lg(const mgb_lg_transition *tr, const RejCfg &cfg, int64_t T, int64_t N, int64_t M,
                        const float *x_hist, const float *lw_hist, const uint32_t *key, float *out, int32_t *idx,
                        long long *evals, void *ws, size_t ws_bytes, cudaStream_t s) {
  return ffbsi_rej_run(pack_lgt<D, RT>(tr), cfg, nullptr, T, N, M, x_hist, lw_hist, key, out, idx, evals, ws, ws_bytes,
                       s);
}

template <int D, bool RT = false>
static int stitch_rej_lg(const mgb_lg_transition *tr, const RejCfg &cfg, int64_t M, const float *x0, const float *x1,
                         const float *lw1, const uint32_t *key, int32_t *idx, long long *evals, void *ws,
                         size_t ws_bytes, cudaStream_t s) {
  return stitch_rej_run(pack_lgt<D, RT>(tr), cfg, M, x0, x1, lw1, key, idx, evals, ws, ws_bytes, s);
}

}  // namespace mgb

using namespace mgb;

// compiled dimensions take their own instances; any other d up to 32 the run-time one
#define MGB_RJ_DISPATCH(FN, ...)                                                    \
  switch (tr->d) {                                                                  \
    case 1: return FN<1>(__VA_ARGS__);                                              \
    case 2: return FN<2>(__VA_ARGS__);                                              \
    case 3: return FN<3>(__VA_ARGS__);                                              \
    case 4: return FN<4>(__VA_ARGS__);                                              \
    case 5: return FN<5>(__VA_ARGS__);                                              \
    case 8: return FN<8>(__VA_ARGS__);                                              \
    case 10: return FN<10>(__VA_ARGS__);                                            \
    default:                                                                        \
      if (tr->d >= 1 && tr->d <= LGT_DMAX) return FN<LGT_DMAX, true>(__VA_ARGS__);  \
      return ERR_UNSUPPORTED;                                                       \
  }

extern "C" {

size_t mgb_ffbsi_rejection_workspace(int64_t N, int64_t M, int64_t T, int32_t d) {
  if (N < 1 || M < 1 || T < 1 || d < 1) return 0;
  return ffbsi_rej_bytes(N, M, T, d);
}

size_t mgb_stitch_rejection_workspace(int64_t M, int32_t d) {
  if (M < 1 || d < 1) return 0;
  return stitch_rej_bytes(M, d);
}

int mgb_ffbsi_rejection_lg(const mgb_lg_transition *tr, const mgb_rejection_config *cfg, int64_t T, int64_t N,
                           int64_t M, const float *x_hist, const float *lw_hist, const uint32_t *key, float *out,
                           int32_t *idx, int64_t *evals, void *ws, size_t ws_bytes, void *stream) {
  RejCfg rc;
  if (!tr || !tr->F || !tr->Pq || !rej_cfg_ok(cfg, rc) || !rej_sizes_ok(T, N, M) || !x_hist || !lw_hist || !key ||
      !out || !idx || !evals || !ws)
    return ERR_BAD_ARG;
  MGB_RJ_DISPATCH(ffbsi_rej_lg, tr, rc, T, N, M, x_hist, lw_hist, key, out, idx, (long long *)evals, ws, ws_bytes,
                  (cudaStream_t)stream);
}

int mgb_ffbsi_rejection_nl1d(const mgb_nl1d_model *m, const mgb_rejection_config *cfg, int64_t T, int64_t N,
                             int64_t M, const float *x_hist, const float *lw_hist, const float *t,
                             const uint32_t *key, float *out, int32_t *idx, int64_t *evals, void *ws, size_t ws_bytes,
                             void *stream) {
  RejCfg rc;
  if (!m || !rej_cfg_ok(cfg, rc) || !rej_sizes_ok(T, N, M) || !x_hist || !lw_hist || !t || !key || !out || !idx ||
      !evals || !ws)
    return ERR_BAD_ARG;
  return ffbsi_rej_run(pack_nlt(m, nullptr, 0.0f), rc, t, T, N, M, x_hist, lw_hist, key, out, idx,
                       (long long *)evals, ws, ws_bytes, (cudaStream_t)stream);
}

int mgb_stitch_rejection_lg(const mgb_lg_transition *tr, const mgb_rejection_config *cfg, int64_t M, const float *x0,
                            const float *x1, const float *lw1, const uint32_t *key, int32_t *idx, int64_t *evals,
                            void *ws, size_t ws_bytes, void *stream) {
  RejCfg rc;
  if (!tr || !tr->F || !tr->Pq || !rej_cfg_ok(cfg, rc) || !rej_sizes_ok(1, M, M) || !x0 || !x1 || !lw1 || !key ||
      !idx || !evals || !ws)
    return ERR_BAD_ARG;
  MGB_RJ_DISPATCH(stitch_rej_lg, tr, rc, M, x0, x1, lw1, key, idx, (long long *)evals, ws, ws_bytes,
                  (cudaStream_t)stream);
}

int mgb_stitch_rejection_nl1d(const mgb_nl1d_model *m, const mgb_rejection_config *cfg, int64_t M, const float *x0,
                              const float *x1, const float *lw1, float t_previous, const uint32_t *key, int32_t *idx,
                              int64_t *evals, void *ws, size_t ws_bytes, void *stream) {
  RejCfg rc;
  if (!m || !rej_cfg_ok(cfg, rc) || !rej_sizes_ok(1, M, M) || !x0 || !x1 || !lw1 || !key || !idx || !evals || !ws)
    return ERR_BAD_ARG;
  return stitch_rej_run(pack_nlt(m, nullptr, t_previous), rc, M, x0, x1, lw1, key, idx, (long long *)evals, ws,
                        ws_bytes, (cudaStream_t)stream);
}

int mgb_ffbsi_rejection_sv(float phi, float pq, const mgb_rejection_config *cfg, int64_t T, int64_t N, int64_t M,
                           const float *x_hist, const float *lw_hist, const float *t_host, const uint32_t *key,
                           float *out, int32_t *idx, int64_t *evals, void *ws, size_t ws_bytes, void *stream) {
  RejCfg rc;
  if (!rej_cfg_ok(cfg, rc) || !rej_sizes_ok(T, N, M) || !x_hist || !lw_hist || !t_host || !key || !out || !idx ||
      !evals || !ws)
    return ERR_BAD_ARG;
  std::vector<float> pqs((size_t)T, pq);
  for (int64_t t = 0; t + 1 < T; ++t) pqs[t] = pq * std::sqrt(t_host[t + 1] - t_host[t]);
  return ffbsi_rej_run(pack_svt(phi, pq, 1.0f), rc, nullptr, T, N, M, x_hist, lw_hist, key, out, idx,
                       (long long *)evals, ws, ws_bytes, (cudaStream_t)stream, pqs.data());
}

int mgb_stitch_rejection_sv(float phi, float pq, const mgb_rejection_config *cfg, int64_t M, const float *x0,
                            const float *x1, const float *lw1, float dt, const uint32_t *key, int32_t *idx,
                            int64_t *evals, void *ws, size_t ws_bytes, void *stream) {
  RejCfg rc;
  if (!rej_cfg_ok(cfg, rc) || !rej_sizes_ok(1, M, M) || !x0 || !x1 || !lw1 || !key || !idx || !evals || !ws)
    return ERR_BAD_ARG;
  return stitch_rej_run(pack_svt(phi, pq, dt), rc, M, x0, x1, lw1, key, idx, (long long *)evals, ws, ws_bytes,
                        (cudaStream_t)stream);
}

}  // extern "C"
