// Bootstrap particle filter for the one-dimensional non-linear benchmark model.
//
// Reference path: run_particle_filter_for_marginals
// (mocat/src/ssm/filtering.py:255-324) with BootstrapFilter (:142-170) on
// NonLinear1DBenchmark (mocat/src/ssm/scenarios/nonlinear1d.py:16-80):
//   initial_sample       x_0 = normal(key_i, (1,)) * initial_sd                (:36-39)
//   transition_sample    x_t = mean(x_{t-1}, t_{t-1}) + normal(key_i, (1,)) * transition_sd
//                        mean(x, t) = 0.5 x + 25 x / (1 + x^2) + 8 cos(1.2 t)  (:41-61)
//   likelihood_potential 0.5 ((y - x^2 / 20) / likelihood_sd)^2 + c           (:63-75)
//                        c = (log 2 pi - log 1) / 2: the reference calls gaussian_potential
//                        on the standardised residual with unit precision, so the
//                        normaliser does not depend on likelihood_sd.
// key_i = split(k_t, n)[i] as in the linear-Gaussian bootstrap kernels; the
// operations are evaluated in the order the reference's expressions state them,
// each rounded to float32 (IEEE division, no contraction), so every particle and
// log-weight equals the oracle's.
//
// 8 cos(1.2 t) is a per-step constant, 8 * float(cos(double(1.2f * t))): the
// float32 product the reference forms, a double-precision cosine rounded to
// float32, and an exact scaling by 8.  A whole run computes it for every step
// once (k_nl_drifts); a single propagate call computes it in thread 0 of each block.
//
// A run with systematic resampling and even n <= 2^21 is one persistent
// cooperative launch (k_pf_persist<NLModelP>, the same kernel as the
// linear-Gaussian filter's); otherwise each step launches the resampling
// kernels and the fused step kernel.
//
// Layout: particles (n) float32, log-weights (n) float32, ancestors (n) int32.
// One step reads x_prev[a_i] (4 B), the previous log-weight when the step did
// not resample (4 B) and writes x_new, lw_new (8 B): 12-16 B per particle.
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_kernels.cuh"
#include "mgb_pf_common.cuh"
#include "mgb_nl1d.cuh"
#include "mgb_persist.cuh"

namespace mgb {

__device__ __forceinline__ float nl_particle(const NLP &p, int64_t i, float e, bool res,
                                             const float *__restrict__ x_prev, const int32_t *anc, const float *lws,
                                             float y, float drift, float *__restrict__ x_new,
                                             float *__restrict__ lw_new) {
  const float xs = __ldg(&x_prev[res ? (int64_t)__ldg(&anc[i]) : i]);
  const float xn = __fadd_rn(nl_mean(xs, drift), __fmul_rn(e, p.tsd));
  x_new[i] = xn;
  const float lres = lws ? lws[i] : 0.0f;
  const float l = __fsub_rn(lres, nl_potential(p, xn, y));
  lw_new[i] = l;
  return l;
}

// initiate_particles: x_0 = e s0, lw_0 = -potential(x_0, y_0) (0 without y_0)
template <bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_nl_init(const NLP p, int64_t n, const uint32_t *key, const float *y0,
                                                     float *__restrict__ x, float *__restrict__ lw, PFCtl ctl) {
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  float m = -INFINITY, a1 = 0.0f, a2 = 0.0f;
  int nanf = 0;
  if (i < n) {
    uint32_t ka, kb;
    split_at(key[0], key[1], (uint64_t)n, (uint64_t)i, ka, kb);
    const float xv = __fmul_rn(nl_normal(ka, kb, p.one), p.s0);
    x[i] = xv;
    const float l = y0 ? -nl_potential(p, xv, __ldg(y0)) : 0.0f;
    lw[i] = l;
    online_acc(l, m, a1, a2, nanf);
  }
  if (FUSED) pf_reduce_online<PF_TPB>(m, a1, a2, nanf, ctl, 0);
}

// aux[t] = 8 cos(1.2 t_all[t - 1]), the drift of step t (aux[0] = 0)
__global__ void k_nl_drifts(const float *t_all, int64_t T, float *aux) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x)
    aux[t] = t == 0 ? 0.0f : nl_drift(t_all[t - 1]);
}

// One bootstrap step.  Even n: a thread takes particles i and i + n/2, whose
// keys are the two halves of the same two cipher calls.  dp (nullable) points
// at the step's precomputed drift, else it is computed from t_prev; res_flag
// (nullable) decides resampled vs identity at run time (run mode: lw_res = 0
// after a resample, filtering.py:292).
template <bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_nl_step(const NLP p, int64_t n, const uint32_t *key, const float *y_t,
                                                     const float *dp, float t_prev, const float *__restrict__ x_prev,
                                                     const int32_t *anc, const float *lw_prev,
                                                     const int32_t *res_flag, float *__restrict__ x_new,
                                                     float *__restrict__ lw_new, PFCtl ctl, int64_t t) {
  __shared__ float sh[2];
  if (threadIdx.x == 0) {
    sh[0] = dp ? *dp : nl_drift(t_prev);
    sh[1] = *y_t;
  }
  __syncthreads();
  const float drift = sh[0], y = sh[1];
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
      const float ea = nl_normal(r0, s0, p.one), eb = nl_normal(r1, s1, p.one);
      online_acc(nl_particle(p, i, ea, res, x_prev, anc, lws, y, drift, x_new, lw_new), m, a1, a2, nanf);
      online_acc(nl_particle(p, i + h, eb, res, x_prev, anc, lws, y, drift, x_new, lw_new), m, a1, a2, nanf);
    }
  } else if (i < n) {
    uint32_t ka, kb;
    split_at(k0, k1, (uint64_t)n, (uint64_t)i, ka, kb);
    online_acc(nl_particle(p, i, nl_normal(ka, kb, p.one), res, x_prev, anc, lws, y, drift, x_new, lw_new), m, a1,
               a2, nanf);
  }
  if (FUSED) pf_reduce_online<PF_TPB>(m, a1, a2, nanf, ctl, t);
}

inline unsigned nl_grid(int64_t n) {
  const int64_t work = n % 2 == 0 ? n / 2 : n;
  return (unsigned)((work + PF_TPB - 1) / PF_TPB);
}

static void carve_nl(Carver &c, int64_t n, int64_t T, int scheme, bool need_x, bool need_lw, bool need_ess,
                     RunWs *w, PersistWs *pw, float **aux) {
  RunWs rw = carve_run(c, n, T, 1, scheme, need_x, need_lw, need_ess);
  PersistWs p = carve_persist(c, n, T);
  float *a = c.take<float>((size_t)T);
  if (w) *w = rw;
  if (pw) *pw = p;
  if (aux) *aux = a;
}

static int run_nl(const mgb_nl1d_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y,
                  const float *t_all, float thr, int scheme, bool persistent, void *ws, size_t ws_bytes,
                  const mgb_pf_outputs *out, cudaStream_t s) {
  const NLP p = pack_nl(m);
  const bool hx = out && out->x_hist, hl = out && out->lw_hist;
  Carver c(ws);
  RunWs w;
  PersistWs pw;
  float *aux;
  carve_nl(c, n, T, scheme, !hx, !hl, !(out && out->ess), &w, &pw, &aux);
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
  float *ess = (out && out->ess) ? out->ess : w.ess_hist;
  int *err = out ? out->err : nullptr;
  if (cudaMemsetAsync(w.st, 0, sizeof(PFState), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.res_hist, 0, sizeof(int32_t) * (T + 1), s) != cudaSuccess) return ERR_CUDA;
  int st = reset_resample(w.rws, s);
  if (st) return st;
  if ((st = launch_setup_keys(key, T, w.keys, s))) return st;
  k_nl_drifts<<<grid_for(T, 256), 256, 0, s>>>(t_all, T, aux);
  if ((st = launch_status())) return st;

  if (persistent && persistent_ok(n, scheme)) {
    PersistArgs a;
    if ((st = persist_setup(w, pw, n, T, y, thr, ess, out, a, s))) return st;
    a.aux = aux;
    if ((st = run_nl_persistent(m, a, s))) return st;
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
  k_nl_init<true><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, s>>>(p, n, w.keys, y, xbuf(0), lbuf(0), ctl);
  if ((st = launch_status())) return st;
  const unsigned grid = nl_grid(n);
  for (int64_t t = 1; t < T; ++t) {
    st = launch_resample(lbuf(t - 1), n, scheme, &w.st->M, w.keys + 2 * t, 0, 0u, w.res_hist + t, w.rws, w.anc,
                         err, s);
    if (st) return st;
    k_nl_step<true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys + 2 * t, y + t, aux + t, 0.0f, xbuf(t - 1), w.anc,
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

static bool nl_model_ok(const mgb_nl1d_model *m) { return m != nullptr; }

}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_pf_nl1d_init(const mgb_nl1d_model *m, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw,
                     void *stream) {
  if (!nl_model_ok(m) || n < 1 || n > 0x7FFFFFFFll || !key || !x || !lw) return ERR_BAD_ARG;
  PFCtl ctl{};
  k_nl_init<false><<<(unsigned)((n + PF_TPB - 1) / PF_TPB), PF_TPB, 0, (cudaStream_t)stream>>>(pack_nl(m), n, key,
                                                                                              y0, x, lw, ctl);
  return launch_status();
}

int mgb_pf_nl1d_propagate(const mgb_nl1d_model *m, int64_t n, const uint32_t *key, const float *y, float t_previous,
                          const float *xp, const int32_t *anc, const float *lwp, float *xn, float *lwn,
                          void *stream) {
  if (!nl_model_ok(m) || n < 1 || n > 0x7FFFFFFFll || !key || !y || !xp || !xn || !lwn) return ERR_BAD_ARG;
  PFCtl ctl{};
  k_nl_step<false><<<nl_grid(n), PF_TPB, 0, (cudaStream_t)stream>>>(pack_nl(m), n, key, y, nullptr, t_previous, xp,
                                                                    anc, lwp, nullptr, xn, lwn, ctl, 0);
  return launch_status();
}

size_t mgb_pf_nl1d_workspace(int64_t n, int64_t T, int scheme) {
  if (n < 1 || T < 1) return 0;
  Carver c(nullptr);
  carve_nl(c, n, T, scheme & 0xff, true, true, true, nullptr, nullptr, nullptr);
  return c.bytes();
}

int mgb_pf_nl1d_run(const mgb_nl1d_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y,
                    const float *t, float ess_threshold, int scheme, void *ws, size_t ws_bytes,
                    const mgb_pf_outputs *out, void *stream) {
  if (!nl_model_ok(m) || n < 1 || n > 0x7FFFFFFFll || T < 1 || !key || !y || !t || !ws) return ERR_BAD_ARG;
  const bool persistent = !(scheme & MGB_RUN_LAUNCH_PER_STEP);
  scheme &= ~MGB_RUN_LAUNCH_PER_STEP;
  if (scheme != MGB_RESAMPLE_SYSTEMATIC && scheme != MGB_RESAMPLE_MULTINOMIAL && scheme != MGB_RESAMPLE_CATEGORICAL)
    return ERR_UNSUPPORTED;
  if (scheme == MGB_RESAMPLE_CATEGORICAL && n > 46340) return ERR_UNSUPPORTED;
  if (ws_bytes < mgb_pf_nl1d_workspace(n, T, scheme)) return ERR_WORKSPACE;
  return run_nl(m, n, T, key, y, t, ess_threshold, scheme, persistent, ws, ws_bytes, out, (cudaStream_t)stream);
}

}  // extern "C"
