// Bootstrap particle filter for one stochastic-volatility series (dim = 1), with
// the full particle history: what run_particle_filter_for_marginals
// (mocat/src/ssm/filtering.py:255-324) with BootstrapFilter (:142-170) returns on
// StochasticVolatility (mocat/src/ssm/scenarios/stochastic_volatility.py:15-108).
// The arithmetic is the batched filters' (mgb_sv.cuh); the time step enters
// through bsig_t = transition_covariance_sqrt sqrt(t_t - t_{t-1}), one value per
// step computed once per run (k_sv_bsig), so uneven time grids are followed.
// key_i = split(k_t, n)[i] as in the other bootstrap kernels.
//
// A run with systematic resampling and even n <= 2^21 is one persistent
// cooperative launch (k_pf_persist<SVModelP>); otherwise each step launches the
// resampling kernels and the fused step kernel.
//
// Layout: particles (n) float32, log-weights (n) float32, ancestors (n) int32;
// 12-16 B per particle and step, as the non-linear benchmark filter.
#include <cmath>

#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_kernels.cuh"
#include "mgb_pf_common.cuh"
#include "mgb_sv.cuh"
#include "mgb_persist.cuh"

namespace mgb {

__device__ __forceinline__ float sv_particle(const SVParams &p, int64_t i, float e, bool res,
                                             const float *__restrict__ x_prev, const int32_t *anc, const float *lws,
                                             float y, float bsig, float *__restrict__ x_new,
                                             float *__restrict__ lw_new) {
  const float xs = __ldg(&x_prev[res ? (int64_t)__ldg(&anc[i]) : i]);
  const float xn = sv_next_x(p, xs, e, bsig);
  x_new[i] = xn;
  const float lres = lws ? lws[i] : 0.0f;
  const float l = __fsub_rn(lres, sv_potential(p, xn, y));
  lw_new[i] = l;
  return l;
}

// initiate_particles: x_0 = e c0 + m0, lw_0 = -potential(x_0, y_0) (0 without y_0)
template <bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_sv_init(const SVParams p, int64_t n, const uint32_t *key, const float *y0,
                                                     float *__restrict__ x, float *__restrict__ lw, PFCtl ctl) {
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  float m = -INFINITY, a1 = 0.0f, a2 = 0.0f;
  int nanf = 0;
  if (i < n) {
    uint32_t ka, kb;
    split_at(key[0], key[1], (uint64_t)n, (uint64_t)i, ka, kb);
    const float xv = sv_init_x(p, sv_normal(ka, kb, p.one));
    x[i] = xv;
    const float l = y0 ? -sv_potential(p, xv, __ldg(y0)) : 0.0f;
    lw[i] = l;
    online_acc(l, m, a1, a2, nanf);
  }
  if (FUSED) pf_reduce_online<PF_TPB>(m, a1, a2, nanf, ctl, 0);
}

// aux[t] = sqrtq sqrt(t_all[t] - t_all[t - 1]), the noise scale of step t (aux[0] = 0)
__global__ void k_sv_bsig(const float *t_all, int64_t T, float sqrtq, float *aux) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x)
    aux[t] = t == 0 ? 0.0f : __fmul_rn(sqrtq, __fsqrt_rn(__fsub_rn(t_all[t], t_all[t - 1])));
}

// One bootstrap step; even n pairs particles i and i + n/2 on the two halves of
// the same cipher calls.  bp (nullable) points at the step's bsig, else bsig is
// used; res_flag (nullable) decides resampled vs identity at run time.
template <bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_sv_step(const SVParams p, int64_t n, const uint32_t *key, const float *y_t,
                                                     const float *bp, float bsig, const float *__restrict__ x_prev,
                                                     const int32_t *anc, const float *lw_prev,
                                                     const int32_t *res_flag, float *__restrict__ x_new,
                                                     float *__restrict__ lw_new, PFCtl ctl, int64_t t) {
  __shared__ float sh[2];
  if (threadIdx.x == 0) {
    sh[0] = bp ? *bp : bsig;
    sh[1] = *y_t;
  }
  __syncthreads();
  const float bs = sh[0], y = sh[1];
  const bool res = res_flag ? (*res_flag != 0) : (anc != nullptr);
  const float *lws = res_flag ? (res ? nullptr : lw_prev) : lw_prev;
  const uint32_t k0 = key[0], k1 = key[1];
  float m = -INFINITY, a1 = 0.0f, a2 = 0.0f;
  int nanf = 0;
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  if (n % 2 == 0) {
    const int64_t h = n >> 1;
    if (i < h) {
      uint32_t r0, r1, s0, s1;
      threefry2x32_m(k0, k1, (uint32_t)(2 * i), (uint32_t)(2 * i + n), p.one, r0, r1);
      threefry2x32_m(k0, k1, (uint32_t)(2 * i + 1), (uint32_t)(2 * i + 1 + n), p.one, s0, s1);
      const float ea = sv_normal(r0, s0, p.one), eb = sv_normal(r1, s1, p.one);
      online_acc(sv_particle(p, i, ea, res, x_prev, anc, lws, y, bs, x_new, lw_new), m, a1, a2, nanf);
      online_acc(sv_particle(p, i + h, eb, res, x_prev, anc, lws, y, bs, x_new, lw_new), m, a1, a2, nanf);
    }
  } else if (i < n) {
    uint32_t ka, kb;
    split_at(k0, k1, (uint64_t)n, (uint64_t)i, ka, kb);
    online_acc(sv_particle(p, i, sv_normal(ka, kb, p.one), res, x_prev, anc, lws, y, bs, x_new, lw_new), m, a1, a2,
               nanf);
  }
  if (FUSED) pf_reduce_online<PF_TPB>(m, a1, a2, nanf, ctl, t);
}

inline unsigned sv_grid(int64_t n) {
  const int64_t work = n % 2 == 0 ? n / 2 : n;
  return (unsigned)((work + PF_TPB - 1) / PF_TPB);
}

static void carve_sv(Carver &c, int64_t n, int64_t T, int scheme, bool need_x, bool need_lw, bool need_ess,
                     RunWs *w, PersistWs *pw, float **aux) {
  RunWs rw = carve_run(c, n, T, 1, scheme, need_x, need_lw, need_ess);
  PersistWs p = carve_persist(c, n, T);
  float *a = c.take<float>((size_t)T);
  if (w) *w = rw;
  if (pw) *pw = p;
  if (aux) *aux = a;
}

static int run_sv(const mgb_sv_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y,
                  const float *t_all, float thr, int scheme, bool persistent, void *ws, size_t ws_bytes,
                  const mgb_pf_outputs *out, cudaStream_t s) {
  const SVParams p = pack_sv(m);
  const bool hx = out && out->x_hist, hl = out && out->lw_hist;
  Carver c(ws);
  RunWs w;
  PersistWs pw;
  float *aux;
  carve_sv(c, n, T, scheme, !hx, !hl, !(out && out->ess), &w, &pw, &aux);
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
  float *ess = (out && out->ess) ? out->ess : w.ess_hist;
  int *err = out ? out->err : nullptr;
  if (cudaMemsetAsync(w.st, 0, sizeof(PFState), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.res_hist, 0, sizeof(int32_t) * (T + 1), s) != cudaSuccess) return ERR_CUDA;
  int st = reset_resample(w.rws, s);
  if (st) return st;
  if ((st = launch_setup_keys(key, T, w.keys, s))) return st;
  k_sv_bsig<<<grid_for(T, 256), 256, 0, s>>>(t_all, T, m->bsig, aux);
  if ((st = launch_status())) return st;

  if (persistent && persistent_ok(n, scheme)) {
    PersistArgs a;
    if ((st = persist_setup(w, pw, n, T, y, thr, ess, out, a, s))) return st;
    a.aux = aux;
    if ((st = run_sv_persistent(m, a, s))) return st;
    if ((st = persist_finish(a, 1, out, s))) return st;
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
  auto xbuf = [&](int64_t t) -> float * { return hx ? out->x_hist + (size_t)t * n : (t & 1 ? w.xb : w.xa); };
  auto lbuf = [&](int64_t t) -> float * { return hl ? out->lw_hist + (size_t)t * n : (t & 1 ? w.lb : w.la); };
  k_sv_init<true><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, s>>>(p, n, w.keys, y, xbuf(0), lbuf(0), ctl);
  if ((st = launch_status())) return st;
  const unsigned grid = sv_grid(n);
  for (int64_t t = 1; t < T; ++t) {
    st = launch_resample(lbuf(t - 1), n, scheme, &w.st->M, w.keys + 2 * t, 0, 0u, w.res_hist + t, w.rws, w.anc,
                         err, s);
    if (st) return st;
    k_sv_step<true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys + 2 * t, y + t, aux + t, 0.0f, xbuf(t - 1), w.anc,
                                            lbuf(t - 1), w.res_hist + t, xbuf(t), lbuf(t), ctl, t);
    if ((st = launch_status())) return st;
  }
  if ((st = launch_finish(w.st, w.res_hist, T, out ? out->log_z : nullptr, out ? out->resampled : nullptr, s)))
    return st;
  if (out && out->x_final &&
      cudaMemcpyAsync(out->x_final, xbuf(T - 1), sizeof(float) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  if (out && out->lw_final &&
      cudaMemcpyAsync(out->lw_final, lbuf(T - 1), sizeof(float) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  return launch_status();
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_pf_sv_init(const mgb_sv_model *m, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw,
                   void *stream) {
  if (!m || n < 1 || n > 0x7FFFFFFFll || !key || !x || !lw) return ERR_BAD_ARG;
  PFCtl ctl{};
  k_sv_init<false><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, (cudaStream_t)stream>>>(pack_sv(m), n, key,
                                                                                              y0, x, lw, ctl);
  return launch_status();
}

int mgb_pf_sv_propagate(const mgb_sv_model *m, int64_t n, const uint32_t *key, const float *y, float dt,
                        const float *xp, const int32_t *anc, const float *lwp, float *xn, float *lwn, void *stream) {
  if (!m || n < 1 || n > 0x7FFFFFFFll || !key || !y || !xp || !xn || !lwn) return ERR_BAD_ARG;
  PFCtl ctl{};
  const float bs = m->bsig * std::sqrt(dt);
  k_sv_step<false><<<sv_grid(n), PF_TPB, 0, (cudaStream_t)stream>>>(pack_sv(m), n, key, y, nullptr, bs, xp, anc, lwp,
                                                                    nullptr, xn, lwn, ctl, 0);
  return launch_status();
}

size_t mgb_pf_sv_workspace(int64_t n, int64_t T, int scheme) {
  if (n < 1 || T < 1) return 0;
  Carver c(nullptr);
  carve_sv(c, n, T, scheme & 0xff, true, true, true, nullptr, nullptr, nullptr);
  return c.bytes();
}

int mgb_pf_sv_run(const mgb_sv_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y, const float *t,
                  float ess_threshold, int scheme, void *ws, size_t ws_bytes, const mgb_pf_outputs *out,
                  void *stream) {
  if (!m || n < 1 || n > 0x7FFFFFFFll || T < 1 || !key || !y || !t || !ws) return ERR_BAD_ARG;
  const bool persistent = !(scheme & MGB_RUN_LAUNCH_PER_STEP);
  scheme &= ~MGB_RUN_LAUNCH_PER_STEP;
  if (scheme != MGB_RESAMPLE_SYSTEMATIC && scheme != MGB_RESAMPLE_MULTINOMIAL && scheme != MGB_RESAMPLE_CATEGORICAL)
    return ERR_UNSUPPORTED;
  if (scheme == MGB_RESAMPLE_CATEGORICAL && n > 46340) return ERR_UNSUPPORTED;
  if (ws_bytes < mgb_pf_sv_workspace(n, T, scheme)) return ERR_WORKSPACE;
  return run_sv(m, n, T, key, y, t, ess_threshold, scheme, persistent, ws, ws_bytes, out, (cudaStream_t)stream);
}

}  // extern "C"
