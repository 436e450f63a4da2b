// Bootstrap particle filter for the time-homogeneous linear-Gaussian SSM:
// fused propagate + weight (+ ancestor gather + online logsumexp / ESS)
// kernels and the whole-filter driver.
//
// Reference path: run_particle_filter_for_marginals
// (mocat/src/ssm/filtering.py:255-324) with BootstrapFilter (:142-170) on
// TimeHomogenousLinearGaussian (mocat/src/ssm/linear_gaussian/linear_gaussian.py:
// initial_sample :46-51, transition_sample :86-94, likelihood_potential :118-128).
//
// Data layout in HBM: particles dimension-major x[j * n + i] (each component
// row is contiguous, so a warp's loads and stores are 128-byte coalesced and
// the sorted ancestors of systematic / multinomial resampling keep the gather
// coalesced); log-weights (n) float32; ancestors (n) int32.
//
// One thread per particle.  Per step and particle the kernel
//   * derives key_i = split(k_t, n)[i] and draws eps = normal(key_i, (d,))
//     (2 + ceil(d/2) threefry2x32 evaluations),
//   * gathers x_prev[:, a_i] (a_i = i when the step did not resample),
//   * x_new = F x + Lq eps, lw_new = lw_res - 0.5 |(y - H x_new) P|^2 - c,
//   * reduces (max, sum e, sum e^2) over the block into a partial; the last
//     block combines all partials (float64) into logsumexp / ESS, accumulates
//     log Z, decides whether the next step resamples (ESS < threshold n) and
//     clears the resampling scratch for it.
// The resampling kernels of the next step read that decision from device
// memory, so a whole run is enqueued without host round trips (and can be
// captured in a CUDA graph).
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_kernels.cuh"
#include "mgb_lg.cuh"
#include "mgb_persist.cuh"
#include "mgb_pf_common.cuh"
#include "mgb_lg_kernels.cuh"

namespace mgb {

// key schedule of run_particle_filter_for_marginals: (random_key, sub_key) =
// split(key); step keys = split(random_key, T - 1).  out[0..1] = sub_key,
// out[2t..2t+1] = key of step t (t >= 1).
__global__ void k_setup_keys(const uint32_t *key, int64_t T, uint32_t *out) {
  uint32_t r0, r1, s0, s1;
  split_at(key[0], key[1], 2, 0, r0, r1);
  split_at(key[0], key[1], 2, 1, s0, s1);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x) {
    if (t == 0) {
      out[0] = s0;
      out[1] = s1;
    } else {
      uint32_t a, b;
      split_at(r0, r1, (uint64_t)(T - 1), (uint64_t)(t - 1), a, b);
      out[2 * t] = a;
      out[2 * t + 1] = b;
    }
  }
}

__global__ void k_finish(const PFState *st, const int32_t *res_hist, int64_t T, double *logz, int32_t *resampled) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x) {
    if (resampled) resampled[t] = t == 0 ? 0 : res_hist[t];
    if (t == 0 && logz) *logz = st->logz;
  }
}


int launch_setup_keys(const uint32_t *key, int64_t T, uint32_t *out, cudaStream_t s) {
  k_setup_keys<<<grid_for(T, 256), 256, 0, s>>>(key, T, out);
  return launch_status();
}

int launch_finish(const PFState *st, const int32_t *res_hist, int64_t T, double *logz, int32_t *resampled,
                  cudaStream_t s) {
  k_finish<<<grid_for(T, 256), 256, 0, s>>>(st, res_hist, T, logz, resampled);
  return launch_status();
}

template <int D, int DY>
static int run_lg(const mgb_lg_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y, float thr,
                  int scheme, bool persistent, void *ws, size_t ws_bytes, const mgb_pf_outputs *out,
                  cudaStream_t s) {
  const LGP<D, DY> p = pack_lg<D, DY>(m);
  const bool hx = out && out->x_hist, hl = out && out->lw_hist;
  Carver c(ws);
  RunWs w = carve_run(c, n, T, D, scheme, !hx, !hl, !(out && out->ess));
  PersistWs pw = carve_persist(c, n, T);
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
  float *ess = (out && out->ess) ? out->ess : w.ess_hist;
  int *err = out ? out->err : nullptr;
  if (cudaMemsetAsync(w.st, 0, sizeof(PFState), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.res_hist, 0, sizeof(int32_t) * (T + 1), s) != cudaSuccess) return ERR_CUDA;
  int st = reset_resample(w.rws, s);
  if (st) return st;
  k_setup_keys<<<grid_for(T, 256), 256, 0, s>>>(key, T, w.keys);

  if (persistent && persistent_ok(n, scheme)) {
    PersistArgs a;
    if ((st = persist_setup(w, pw, n, T, y, thr, ess, out, a, s))) return st;
    if ((st = run_lg_persistent(m, a, s))) return st;
    if ((st = persist_finish(a, D, out, s))) return st;
    return launch_status();
  }

  PFCtl ctl;
  ctl.parts = w.parts;
  ctl.counter = w.counter;
  ctl.st = w.st;
  ctl.ess_hist = ess;
  ctl.res_hist = w.res_hist;
  ctl.rctl = w.rws.ctl;
  ctl.rstatus = w.rws.status;
  ctl.rstatus2 = w.rws.status2;
  ctl.ntiles = (int)w.rws.ntiles;
  ctl.thr_n = thr * (float)n;
  ctl.logn = log((double)n);
  ctl.logz_out = nullptr;

  const unsigned grid = (unsigned)((n + PF_TPB - 1) / PF_TPB);
  const unsigned grid2 = (unsigned)((n / 2 + PF_TPB - 1) / PF_TPB);
  auto xbuf = [&](int64_t t) -> float * { return hx ? out->x_hist + (size_t)t * D * n : (t & 1 ? w.xb : w.xa); };
  auto lbuf = [&](int64_t t) -> float * { return hl ? out->lw_hist + (size_t)t * n : (t & 1 ? w.lb : w.la); };
  k_lg_init<D, DY, true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys, y, xbuf(0), lbuf(0), ctl);
  if ((st = launch_status())) return st;
  for (int64_t t = 1; t < T; ++t) {
    st = launch_resample(lbuf(t - 1), n, scheme, &w.st->M, w.keys + 2 * t, 0, 0u, w.res_hist + t, w.rws, w.anc,
                         err, s);
    if (st) return st;
    if (n % 2 == 0)
      k_lg_step2<D, DY, true><<<grid2, PF_TPB, 0, s>>>(p, n, w.keys + 2 * t, y + (size_t)t * DY, xbuf(t - 1),
                                                        w.anc, lbuf(t - 1), w.res_hist + t, xbuf(t), lbuf(t), ctl, t);
    else
      k_lg_step<D, DY, true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys + 2 * t, y + (size_t)t * DY, xbuf(t - 1), w.anc,
                                                      lbuf(t - 1), w.res_hist + t, xbuf(t), lbuf(t), ctl, t);
    if ((st = launch_status())) return st;
  }
  k_finish<<<grid_for(T, 256), 256, 0, s>>>(w.st, w.res_hist, T, out ? out->log_z : nullptr,
                                            out ? out->resampled : nullptr);
  if (out && out->x_final && cudaMemcpyAsync(out->x_final, xbuf(T - 1), sizeof(float) * D * n,
                                             cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  if (out && out->lw_final && cudaMemcpyAsync(out->lw_final, lbuf(T - 1), sizeof(float) * n,
                                              cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  return launch_status();
}

template <int D, int DY>
static int init_lg(const mgb_lg_model *m, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw,
                   cudaStream_t s) {
  const LGP<D, DY> p = pack_lg<D, DY>(m);
  PFCtl ctl{};
  k_lg_init<D, DY, false><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, s>>>(p, n, key, y0, x, lw, ctl);
  return launch_status();
}

template <int D, int DY>
static int step_lg(const mgb_lg_model *m, int64_t n, const uint32_t *key, const float *y, const float *xp,
                   const int32_t *anc, const float *lwp, float *xn, float *lwn, cudaStream_t s) {
  const LGP<D, DY> p = pack_lg<D, DY>(m);
  PFCtl ctl{};
  if (n % 2 == 0)
    k_lg_step2<D, DY, false><<<(unsigned)((n / 2 + PF_TPB - 1) / PF_TPB), PF_TPB, 0, s>>>(p, n, key, y, xp, anc, lwp,
                                                                                          nullptr, xn, lwn, ctl, 0);
  else
    k_lg_step<D, DY, false><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, s>>>(p, n, key, y, xp, anc, lwp,
                                                                                      nullptr, xn, lwn, ctl, 0);
  return launch_status();
}

// ---------------------------------------------------------------------------
// Run-time dimensions: the bootstrap filter for (d, dy) pairs without a compiled
// instance (d, dy <= LGD_MAX).  One particle per thread, the model's matrices in
// the kernel's parameter block (read through the constant cache, every thread
// at the same address), the per-particle vectors in local arrays.  Every value
// is the same float operation sequence as the templated kernels' (the fma
// chains of lg_transition / lg_potential / k_lg_init, the same draws), so the
// results are the oracle's bit for bit; only the speed differs.
constexpr int LGD_MAX = 32;
struct LGDyn {
  float F[LGD_MAX * LGD_MAX], Lq[LGD_MAX * LGD_MAX], H[LGD_MAX * LGD_MAX], P[LGD_MAX * LGD_MAX],
      C0[LGD_MAX * LGD_MAX], m0[LGD_MAX];
  float c;
  int d, dy, lq_diag, h_eye, p_diag;
};

static bool lgd_ok(const mgb_lg_model *m) { return m->d <= LGD_MAX && m->dy <= LGD_MAX; }

static LGDyn pack_lgd(const mgb_lg_model *m) {
  LGDyn p;
  const int d = m->d, dy = m->dy;
  p.d = d;
  p.dy = dy;
  for (int i = 0; i < d * d; ++i) {
    p.F[i] = m->F[i];
    p.Lq[i] = m->Lq[i];
    p.C0[i] = m->C0[i];
  }
  for (int i = 0; i < dy * d; ++i) p.H[i] = m->H[i];
  for (int i = 0; i < dy * dy; ++i) p.P[i] = m->P[i];
  for (int i = 0; i < d; ++i) p.m0[i] = m->m0[i];
  p.c = m->c;
  auto diag = [](const float *a, int k) {
    for (int r = 0; r < k; ++r)
      for (int c = 0; c < k; ++c)
        if (r != c && a[r * k + c] != 0.0f) return 0;
    return 1;
  };
  p.lq_diag = diag(p.Lq, d);
  p.p_diag = diag(p.P, dy);
  p.h_eye = 0;
  if (dy == d) {
    int eye = 1;
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) eye &= p.H[r * d + c] == (r == c ? 1.0f : 0.0f);
    p.h_eye = eye;
  }
  return p;
}

// normal(split(k, n)[i], (d,)): ceil(d / 2) cipher calls, counters (j, j + H)
__device__ __forceinline__ void lgd_normals(uint32_t k0, uint32_t k1, int64_t n, int64_t i, int d, float *e) {
  uint32_t a0, a1;
  split_at(k0, k1, (uint64_t)n, (uint64_t)i, a0, a1);
  const int H = (d + 1) / 2;
  for (int j = 0; j < H; ++j) {
    uint32_t r0, r1;
    threefry2x32(a0, a1, (uint32_t)j, (j + H < d) ? (uint32_t)(j + H) : 0u, r0, r1);
    e[j] = bits_to_normal(r0);
    if (j + H < d) e[j + H] = bits_to_normal(r1);
  }
}

__device__ __forceinline__ float lgd_potential(const LGDyn &p, const float *x, const float *y) {
  const int d = p.d, dy = p.dy;
  float diff[LGD_MAX];
  if (dy == d && p.h_eye) {
    for (int j = 0; j < dy; ++j) diff[j] = __fsub_rn(y[j], x[j]);
  } else {
    for (int j = 0; j < dy; ++j) {
      float hx = __fmul_rn(p.H[j * d], x[0]);
      for (int k = 1; k < d; ++k) hx = __fmaf_rn(p.H[j * d + k], x[k], hx);
      diff[j] = __fsub_rn(y[j], hx);
    }
  }
  float quad = 0.0f;
  for (int k = 0; k < dy; ++k) {
    float v;
    if (p.p_diag) {
      v = __fmul_rn(diff[k], p.P[k * dy + k]);
    } else {
      v = __fmul_rn(diff[0], p.P[k]);
      for (int j = 1; j < dy; ++j) v = __fmaf_rn(diff[j], p.P[j * dy + k], v);
    }
    quad = k == 0 ? __fmul_rn(v, v) : __fmaf_rn(v, v, quad);
  }
  return __fadd_rn(__fmul_rn(0.5f, quad), p.c);
}

template <bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_lgd_init(const __grid_constant__ LGDyn p, int64_t n, const uint32_t *key,
                                                      const float *y0, float *__restrict__ x,
                                                      float *__restrict__ lw, PFCtl ctl) {
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  const uint32_t k0 = key[0], k1 = key[1];
  __shared__ float y[LGD_MAX];
  if (threadIdx.x < p.dy) y[threadIdx.x] = y0 ? y0[threadIdx.x] : 0.0f;
  __syncthreads();
  float l = -INFINITY;
  const bool active = i < n;
  if (active) {
    const int d = p.d;
    float e[LGD_MAX], xv[LGD_MAX];
    lgd_normals(k0, k1, n, i, d, e);
    for (int r = 0; r < d; ++r) {
      float v = __fmul_rn(p.C0[r * d], e[0]);
      for (int k = 1; k < d; ++k) v = __fmaf_rn(p.C0[r * d + k], e[k], v);
      xv[r] = __fadd_rn(v, p.m0[r]);
      x[r * n + i] = xv[r];
    }
    l = y0 ? -lgd_potential(p, xv, y) : 0.0f;
    lw[i] = l;
  }
  if (FUSED) pf_reduce<PF_TPB>(l, active, ctl, 0);
}

// one step; res_flag (nullable) decides resampled vs identity at run time, as k_lg_step
template <bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_lgd_step(const __grid_constant__ LGDyn p, int64_t n, const uint32_t *key,
                                                      const float *y_t, const float *__restrict__ x_prev,
                                                      const int32_t *anc, const float *lw_prev,
                                                      const int32_t *res_flag, float *__restrict__ x_new,
                                                      float *__restrict__ lw_new, PFCtl ctl, int64_t t) {
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  const bool res = res_flag ? (*res_flag != 0) : (anc != nullptr);
  const uint32_t k0 = key[0], k1 = key[1];
  __shared__ float y[LGD_MAX];
  if (threadIdx.x < p.dy) y[threadIdx.x] = y_t[threadIdx.x];
  __syncthreads();
  float l = -INFINITY;
  const bool active = i < n;
  if (active) {
    const int d = p.d;
    float e[LGD_MAX], xs[LGD_MAX], xn[LGD_MAX];
    lgd_normals(k0, k1, n, i, d, e);
    const int64_t src = res ? (int64_t)anc[i] : i;
    for (int j = 0; j < d; ++j) xs[j] = __ldg(&x_prev[j * n + src]);
    for (int r = 0; r < d; ++r) {
      float fx = __fmul_rn(p.F[r * d], xs[0]);
      for (int k = 1; k < d; ++k) fx = __fmaf_rn(p.F[r * d + k], xs[k], fx);
      float le;
      if (p.lq_diag) {
        le = __fmul_rn(p.Lq[r * d + r], e[r]);
      } else {
        le = __fmul_rn(p.Lq[r * d], e[0]);
        for (int k = 1; k < d; ++k) le = __fmaf_rn(p.Lq[r * d + k], e[k], le);
      }
      xn[r] = __fadd_rn(fx, le);
      x_new[r * n + i] = xn[r];
    }
    const float *lws = res_flag ? (res ? nullptr : lw_prev) : lw_prev;
    const float lres = lws ? __ldg(&lws[i]) : 0.0f;
    l = __fsub_rn(lres, lgd_potential(p, xn, y));
    lw_new[i] = l;
  }
  if (FUSED) pf_reduce<PF_TPB>(l, active, ctl, t);
}

static int run_lgd(const mgb_lg_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y, float thr,
                   int scheme, bool, void *ws, size_t ws_bytes, const mgb_pf_outputs *out, cudaStream_t s) {
  const LGDyn p = pack_lgd(m);
  const int D = p.d, DY = p.dy;
  const bool hx = out && out->x_hist, hl = out && out->lw_hist;
  Carver c(ws);
  RunWs w = carve_run(c, n, T, D, scheme, !hx, !hl, !(out && out->ess));
  carve_persist(c, n, T);  // the layout mgb_pf_lg_workspace sizes
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
  float *ess = (out && out->ess) ? out->ess : w.ess_hist;
  int *err = out ? out->err : nullptr;
  if (cudaMemsetAsync(w.st, 0, sizeof(PFState), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.res_hist, 0, sizeof(int32_t) * (T + 1), s) != cudaSuccess) return ERR_CUDA;
  int st = reset_resample(w.rws, s);
  if (st) return st;
  k_setup_keys<<<grid_for(T, 256), 256, 0, s>>>(key, T, w.keys);
  PFCtl ctl;
  ctl.parts = w.parts;
  ctl.counter = w.counter;
  ctl.st = w.st;
  ctl.ess_hist = ess;
  ctl.res_hist = w.res_hist;
  ctl.rctl = w.rws.ctl;
  ctl.rstatus = w.rws.status;
  ctl.rstatus2 = w.rws.status2;
  ctl.ntiles = (int)w.rws.ntiles;
  ctl.thr_n = thr * (float)n;
  ctl.logn = log((double)n);
  ctl.logz_out = nullptr;
  const unsigned grid = (unsigned)((n + PF_TPB - 1) / PF_TPB);
  auto xbuf = [&](int64_t t) -> float * { return hx ? out->x_hist + (size_t)t * D * n : (t & 1 ? w.xb : w.xa); };
  auto lbuf = [&](int64_t t) -> float * { return hl ? out->lw_hist + (size_t)t * n : (t & 1 ? w.lb : w.la); };
  k_lgd_init<true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys, y, xbuf(0), lbuf(0), ctl);
  if ((st = launch_status())) return st;
  for (int64_t t = 1; t < T; ++t) {
    st = launch_resample(lbuf(t - 1), n, scheme, &w.st->M, w.keys + 2 * t, 0, 0u, w.res_hist + t, w.rws, w.anc,
                         err, s);
    if (st) return st;
    k_lgd_step<true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys + 2 * t, y + (size_t)t * DY, xbuf(t - 1), w.anc,
                                             lbuf(t - 1), w.res_hist + t, xbuf(t), lbuf(t), ctl, t);
    if ((st = launch_status())) return st;
  }
  k_finish<<<grid_for(T, 256), 256, 0, s>>>(w.st, w.res_hist, T, out ? out->log_z : nullptr,
                                            out ? out->resampled : nullptr);
  if (out && out->x_final && cudaMemcpyAsync(out->x_final, xbuf(T - 1), sizeof(float) * D * n,
                                             cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  if (out && out->lw_final && cudaMemcpyAsync(out->lw_final, lbuf(T - 1), sizeof(float) * n,
                                              cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  return launch_status();
}

static int init_lgd(const mgb_lg_model *m, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw,
                    cudaStream_t s) {
  const LGDyn p = pack_lgd(m);
  PFCtl ctl{};
  k_lgd_init<false><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, s>>>(p, n, key, y0, x, lw, ctl);
  return launch_status();
}

static int step_lgd(const mgb_lg_model *m, int64_t n, const uint32_t *key, const float *y, const float *xp,
                    const int32_t *anc, const float *lwp, float *xn, float *lwn, cudaStream_t s) {
  const LGDyn p = pack_lgd(m);
  PFCtl ctl{};
  k_lgd_step<false><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, s>>>(p, n, key, y, xp, anc, lwp, nullptr,
                                                                              xn, lwn, ctl, 0);
  return launch_status();
}

// ---------------------------------------------------------------------------
// The d-dimensional stochastic-volatility model (stochastic_volatility.py:15-108,
// diagonal likelihood covariance) on the same run-time-dimension scheme:
//   x_0 = C0 e + m0;  x_t = A x_{t-1} + (Lq e) sqrt(t_t - t_{t-1})
//   potential = cB + sum_j (0.5 x_j + (0.5 y_j^2 r2_j) exp(-x_j)),  r2 = 1 / R,
// accumulated j = 0, 1, ... from cB (for d = 1 the dim-1 kernels' formula).
struct SVDyn {
  float A[LGD_MAX * LGD_MAX], Lq[LGD_MAX * LGD_MAX], C0[LGD_MAX * LGD_MAX], m0[LGD_MAX], r2[LGD_MAX];
  float cB;
  int d, lq_diag;
};

static bool svd_model_ok(const mgb_svd_model *m) {
  return m && m->d >= 1 && m->d <= LGD_MAX && m->A && m->Lq && m->C0 && m->m0 && m->r2;
}

static SVDyn pack_svd(const mgb_svd_model *m) {
  SVDyn p;
  const int d = m->d;
  p.d = d;
  for (int i = 0; i < d * d; ++i) {
    p.A[i] = m->A[i];
    p.Lq[i] = m->Lq[i];
    p.C0[i] = m->C0[i];
  }
  for (int i = 0; i < d; ++i) {
    p.m0[i] = m->m0[i];
    p.r2[i] = m->r2[i];
  }
  p.cB = m->cB;
  int diag = 1;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c)
      if (r != c && p.Lq[r * d + c] != 0.0f) diag = 0;
  p.lq_diag = diag;
  return p;
}

__device__ __forceinline__ float svd_potential(const SVDyn &p, const float *x, const float *y) {
  float pot = p.cB;
  for (int j = 0; j < p.d; ++j) {
    const float a = __fmul_rn(__fmul_rn(0.5f, __fmul_rn(y[j], y[j])), p.r2[j]);
    pot = __fmaf_rn(a, expf_(-x[j]), __fmaf_rn(0.5f, x[j], pot));
  }
  return pot;
}

template <bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_svd_init(const __grid_constant__ SVDyn p, int64_t n, const uint32_t *key,
                                                      const float *y0, float *__restrict__ x,
                                                      float *__restrict__ lw, PFCtl ctl) {
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  const uint32_t k0 = key[0], k1 = key[1];
  __shared__ float y[LGD_MAX];
  if (threadIdx.x < p.d) y[threadIdx.x] = y0 ? y0[threadIdx.x] : 0.0f;
  __syncthreads();
  float l = -INFINITY;
  const bool active = i < n;
  if (active) {
    const int d = p.d;
    float e[LGD_MAX], xv[LGD_MAX];
    lgd_normals(k0, k1, n, i, d, e);
    for (int r = 0; r < d; ++r) {
      float v = __fmul_rn(p.C0[r * d], e[0]);
      for (int k = 1; k < d; ++k) v = __fmaf_rn(p.C0[r * d + k], e[k], v);
      xv[r] = __fadd_rn(v, p.m0[r]);
      x[r * n + i] = xv[r];
    }
    l = y0 ? -svd_potential(p, xv, y) : 0.0f;
    lw[i] = l;
  }
  if (FUSED) pf_reduce<PF_TPB>(l, active, ctl, 0);
}

// one step; dt = t_dev[t] - t_dev[t-1] when t_dev is given, else dt_arg
template <bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_svd_step(const __grid_constant__ SVDyn p, int64_t n, const uint32_t *key,
                                                      const float *y_t, const float *t_dev, float dt_arg,
                                                      const float *__restrict__ x_prev, const int32_t *anc,
                                                      const float *lw_prev, const int32_t *res_flag,
                                                      float *__restrict__ x_new, float *__restrict__ lw_new,
                                                      PFCtl ctl, int64_t t) {
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  const bool res = res_flag ? (*res_flag != 0) : (anc != nullptr);
  const uint32_t k0 = key[0], k1 = key[1];
  __shared__ float y[LGD_MAX];
  if (threadIdx.x < p.d) y[threadIdx.x] = y_t[threadIdx.x];
  __syncthreads();
  float l = -INFINITY;
  const bool active = i < n;
  if (active) {
    const int d = p.d;
    const float dt = t_dev ? __fsub_rn(__ldg(&t_dev[t]), __ldg(&t_dev[t - 1])) : dt_arg;
    const float sdt = __fsqrt_rn(dt);
    float e[LGD_MAX], xs[LGD_MAX], xn[LGD_MAX];
    lgd_normals(k0, k1, n, i, d, e);
    const int64_t src = res ? (int64_t)anc[i] : i;
    for (int j = 0; j < d; ++j) xs[j] = __ldg(&x_prev[j * n + src]);
    for (int r = 0; r < d; ++r) {
      float fx = __fmul_rn(p.A[r * d], xs[0]);
      for (int k = 1; k < d; ++k) fx = __fmaf_rn(p.A[r * d + k], xs[k], fx);
      float le;
      if (p.lq_diag) {
        le = __fmul_rn(p.Lq[r * d + r], e[r]);
      } else {
        le = __fmul_rn(p.Lq[r * d], e[0]);
        for (int k = 1; k < d; ++k) le = __fmaf_rn(p.Lq[r * d + k], e[k], le);
      }
      xn[r] = __fadd_rn(fx, __fmul_rn(le, sdt));
      x_new[r * n + i] = xn[r];
    }
    const float *lws = res_flag ? (res ? nullptr : lw_prev) : lw_prev;
    const float lres = lws ? __ldg(&lws[i]) : 0.0f;
    l = __fsub_rn(lres, svd_potential(p, xn, y));
    lw_new[i] = l;
  }
  if (FUSED) pf_reduce<PF_TPB>(l, active, ctl, t);
}

static int run_svd(const mgb_svd_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y,
                   const float *t_dev, float thr, int scheme, void *ws, size_t ws_bytes, const mgb_pf_outputs *out,
                   cudaStream_t s) {
  const SVDyn p = pack_svd(m);
  const int D = p.d;
  const bool hx = out && out->x_hist, hl = out && out->lw_hist;
  Carver c(ws);
  RunWs w = carve_run(c, n, T, D, scheme, !hx, !hl, !(out && out->ess));
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
  float *ess = (out && out->ess) ? out->ess : w.ess_hist;
  int *err = out ? out->err : nullptr;
  if (cudaMemsetAsync(w.st, 0, sizeof(PFState), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.res_hist, 0, sizeof(int32_t) * (T + 1), s) != cudaSuccess) return ERR_CUDA;
  int st = reset_resample(w.rws, s);
  if (st) return st;
  k_setup_keys<<<grid_for(T, 256), 256, 0, s>>>(key, T, w.keys);
  PFCtl ctl;
  ctl.parts = w.parts;
  ctl.counter = w.counter;
  ctl.st = w.st;
  ctl.ess_hist = ess;
  ctl.res_hist = w.res_hist;
  ctl.rctl = w.rws.ctl;
  ctl.rstatus = w.rws.status;
  ctl.rstatus2 = w.rws.status2;
  ctl.ntiles = (int)w.rws.ntiles;
  ctl.thr_n = thr * (float)n;
  ctl.logn = log((double)n);
  ctl.logz_out = nullptr;
  const unsigned grid = (unsigned)((n + PF_TPB - 1) / PF_TPB);
  auto xbuf = [&](int64_t t) -> float * { return hx ? out->x_hist + (size_t)t * D * n : (t & 1 ? w.xb : w.xa); };
  auto lbuf = [&](int64_t t) -> float * { return hl ? out->lw_hist + (size_t)t * n : (t & 1 ? w.lb : w.la); };
  k_svd_init<true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys, y, xbuf(0), lbuf(0), ctl);
  if ((st = launch_status())) return st;
  for (int64_t t = 1; t < T; ++t) {
    st = launch_resample(lbuf(t - 1), n, scheme, &w.st->M, w.keys + 2 * t, 0, 0u, w.res_hist + t, w.rws, w.anc,
                         err, s);
    if (st) return st;
    k_svd_step<true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys + 2 * t, y + (size_t)t * D, t_dev, 1.0f, xbuf(t - 1),
                                             w.anc, lbuf(t - 1), w.res_hist + t, xbuf(t), lbuf(t), ctl, t);
    if ((st = launch_status())) return st;
  }
  k_finish<<<grid_for(T, 256), 256, 0, s>>>(w.st, w.res_hist, T, out ? out->log_z : nullptr,
                                            out ? out->resampled : nullptr);
  if (out && out->x_final && cudaMemcpyAsync(out->x_final, xbuf(T - 1), sizeof(float) * D * n,
                                             cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  if (out && out->lw_final && cudaMemcpyAsync(out->lw_final, lbuf(T - 1), sizeof(float) * n,
                                              cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  return launch_status();
}

// (d, dy) dispatch over the compiled instantiations
#define MGB_LG_DISPATCH(FN, ...)                                   \
  do {                                                             \
    const int d_ = m->d, dy_ = m->dy;                              \
    if (dy_ == 1) {                                                \
      switch (d_) {                                                \
        case 1: return FN<1, 1>(__VA_ARGS__);                      \
        case 2: return FN<2, 1>(__VA_ARGS__);                      \
        case 3: return FN<3, 1>(__VA_ARGS__);                      \
        case 4: return FN<4, 1>(__VA_ARGS__);                      \
        case 5: return FN<5, 1>(__VA_ARGS__);                      \
        case 8: return FN<8, 1>(__VA_ARGS__);                      \
        case 10: return FN<10, 1>(__VA_ARGS__);                    \
        default: break;                                            \
      }                                                            \
    } else if (dy_ == d_) {                                        \
      switch (d_) {                                                \
        case 2: return FN<2, 2>(__VA_ARGS__);                      \
        case 3: return FN<3, 3>(__VA_ARGS__);                      \
        case 4: return FN<4, 4>(__VA_ARGS__);                      \
        case 5: return FN<5, 5>(__VA_ARGS__);                      \
        case 8: return FN<8, 8>(__VA_ARGS__);                      \
        case 10: return FN<10, 10>(__VA_ARGS__);                   \
        default: break;                                            \
      }                                                            \
    }                                                              \
    /* no compiled instance: the run-time-dimension kernels */     \
    if (lgd_ok(m)) return FN##d(__VA_ARGS__);                      \
    return ERR_UNSUPPORTED;                                        \
  } while (0)

static bool lg_model_ok(const mgb_lg_model *m) {
  return m && m->d >= 1 && m->dy >= 1 && m->F && m->Lq && m->H && m->P && m->C0 && m->m0;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

size_t mgb_pf_lg_workspace(int64_t n, int64_t T, int32_t d, int scheme) {
  Carver c(nullptr);
  carve_run(c, n, T < 1 ? 1 : T, d, scheme & 0xff, true, true, true);
  carve_persist(c, n, T < 1 ? 1 : T);
  return c.bytes();
}

int mgb_pf_lg_init(const mgb_lg_model *m, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw,
                   void *stream) {
  if (!lg_model_ok(m) || n < 1 || n > 0x7FFFFFFFll || !key || !x || !lw) return ERR_BAD_ARG;
  MGB_LG_DISPATCH(init_lg, m, n, key, y0, x, lw, (cudaStream_t)stream);
}

int mgb_pf_lg_propagate(const mgb_lg_model *m, int64_t n, const uint32_t *key, const float *y, const float *xp,
                        const int32_t *anc, const float *lwp, float *xn, float *lwn, void *stream) {
  if (!lg_model_ok(m) || n < 1 || n > 0x7FFFFFFFll || !key || !y || !xp || !xn || !lwn) return ERR_BAD_ARG;
  MGB_LG_DISPATCH(step_lg, m, n, key, y, xp, anc, lwp, xn, lwn, (cudaStream_t)stream);
}

int mgb_pf_lg_run(const mgb_lg_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y, float thr,
                  int scheme, void *ws, size_t ws_bytes, const mgb_pf_outputs *out, void *stream) {
  if (!lg_model_ok(m) || n < 1 || n > 0x7FFFFFFFll || T < 1 || !key || !y || !ws) return ERR_BAD_ARG;
  const bool persistent = !(scheme & MGB_RUN_LAUNCH_PER_STEP);
  scheme &= ~MGB_RUN_LAUNCH_PER_STEP;
  if (scheme < 0 || scheme > 2) return ERR_BAD_ARG;
  if (scheme == MGB_RESAMPLE_CATEGORICAL && n > 46340) return ERR_UNSUPPORTED;
  if (ws_bytes < mgb_pf_lg_workspace(n, T, m->d, scheme)) return ERR_WORKSPACE;
  MGB_LG_DISPATCH(run_lg, m, n, T, key, y, thr, scheme, persistent, ws, ws_bytes, out, (cudaStream_t)stream);
}

size_t mgb_pf_svd_workspace(int64_t n, int64_t T, int32_t d, int scheme) {
  Carver c(nullptr);
  carve_run(c, n, T < 1 ? 1 : T, d, scheme & 0xff, true, true, true);
  return c.bytes();
}

int mgb_pf_svd_init(const mgb_svd_model *m, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw,
                    void *stream) {
  if (!m || n < 1 || n > 0x7FFFFFFFll || !key || !x || !lw) return ERR_BAD_ARG;
  if (!svd_model_ok(m)) return m->d > LGD_MAX ? ERR_UNSUPPORTED : ERR_BAD_ARG;
  const SVDyn p = pack_svd(m);
  PFCtl ctl{};
  k_svd_init<false><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, (cudaStream_t)stream>>>(p, n, key, y0, x, lw,
                                                                                               ctl);
  return launch_status();
}

int mgb_pf_svd_propagate(const mgb_svd_model *m, int64_t n, const uint32_t *key, const float *y, float dt,
                         const float *xp, const int32_t *anc, const float *lwp, float *xn, float *lwn, void *stream) {
  if (!m || n < 1 || n > 0x7FFFFFFFll || !key || !y || !xp || !xn || !lwn || !(dt >= 0.0f)) return ERR_BAD_ARG;
  if (!svd_model_ok(m)) return m->d > LGD_MAX ? ERR_UNSUPPORTED : ERR_BAD_ARG;
  const SVDyn p = pack_svd(m);
  PFCtl ctl{};
  k_svd_step<false><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, (cudaStream_t)stream>>>(
      p, n, key, y, nullptr, dt, xp, anc, lwp, nullptr, xn, lwn, ctl, 0);
  return launch_status();
}

int mgb_pf_svd_run(const mgb_svd_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y,
                   const float *t, float thr, int scheme, void *ws, size_t ws_bytes, const mgb_pf_outputs *out,
                   void *stream) {
  if (!m || n < 1 || n > 0x7FFFFFFFll || T < 1 || !key || !y || !ws) return ERR_BAD_ARG;
  if (!svd_model_ok(m)) return m->d > LGD_MAX ? ERR_UNSUPPORTED : ERR_BAD_ARG;
  scheme &= ~MGB_RUN_LAUNCH_PER_STEP;
  if (scheme < 0 || scheme > 2) return ERR_BAD_ARG;
  if (scheme == MGB_RESAMPLE_CATEGORICAL && n > 46340) return ERR_UNSUPPORTED;
  if (ws_bytes < mgb_pf_svd_workspace(n, T, m->d, scheme)) return ERR_WORKSPACE;
  return run_svd(m, n, T, key, y, t, thr, scheme, ws, ws_bytes, out, (cudaStream_t)stream);
}

}  // extern "C"
