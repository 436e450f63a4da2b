// Particle filter with the optimal proposal for a linear transition and
// linear-Gaussian observations.
//
// Reference path: OptimalNonLinearGaussianParticleFilter
// (mocat/src/ssm/nonlinear_gaussian.py:134-281) with f(x) = F x, driven by
// run_particle_filter_for_marginals (mocat/src/ssm/filtering.py:255-324):
//   init (:198-209, :223-230): x_0 = (m0 + K0 (y_0 - H m0)) + eps C0c, lw_0 = 0,
//        eps = normal(split(key, n)[0], (n, d))
//   step (:264-281): mx = F x_prev[a_i]; r = y_t - H mx;
//        x_new = (mx + K r) + S eps_i,  lw = lw_res - (0.5 |r W|^2 + cw),
//        eps = normal(split(k_t, n)[0], (n, d)) -- ONE key for all particles.
// K = proposal_kalman_gain, S = proposal_covariance_sqrt, W = weight_precision_sqrt,
// cw = (dy log 2 pi - log weight_precision_det) / 2, K0 = initial_kalman_gain,
// C0c = initial_conditioned_covariance_sqrt (all computed once on the host, as
// the reference's startup does).
//
// The (n, d) draw is threefry over counters 0 .. n d - 1: for even n element
// (i, j) and (i + n/2, j) come from the two halves of one cipher call, so a
// thread takes the particle pair (i, i + n/2) and spends d cipher calls on it.
// Layout: particles dimension-major x[j * n + i]; log-weights and ancestors (n).
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_kernels.cuh"
#include "mgb_pf_common.cuh"

namespace mgb {

// CD, CDY: the arrays' capacities.  A compiled pair has RT = false and the dimensions are the
// template constants; RT = true reads them from rd, rdy (the run-time-dimension instance, d and
// dy up to 32), with every matrix packed at its run-time strides at the front of its array.
template <int CD, int CDY, bool RT = false>
struct OPTP {
  float F[CD * CD], H[CDY * CD], K[CD * CDY], S[CD * CD], W[CDY * CDY], K0[CD * CDY], C0c[CD * CD], m0[CD];
  float cw;
  uint32_t one;  // == 1, multiplier of the cipher's multiply-adds
  int rd, rdy;
  __host__ __device__ __forceinline__ int d() const { return RT ? rd : CD; }
  __host__ __device__ __forceinline__ int dy() const { return RT ? rdy : CDY; }
};

// the run-time-dimension capacity
constexpr int OPT_DMAX = 32;

template <int CD, int CDY, bool RT>
OPTP<CD, CDY, RT> pack_opt(const mgb_opt_model *m) {
  OPTP<CD, CDY, RT> p{};
  const int D = RT ? m->d : CD, DY = RT ? m->dy : CDY;
  for (int i = 0; i < D * D; ++i) {
    p.F[i] = m->F[i];
    p.S[i] = m->S[i];
    p.C0c[i] = m->C0c[i];
  }
  for (int i = 0; i < DY * D; ++i) {
    p.H[i] = m->H[i];
    p.K[i] = m->K[i];
    p.K0[i] = m->K0[i];
  }
  for (int i = 0; i < DY * DY; ++i) p.W[i] = m->W[i];
  for (int i = 0; i < D; ++i) p.m0[i] = m->m0[i];
  p.cw = m->cw;
  p.one = 1u;
  p.rd = D;
  p.rdy = DY;
  return p;
}

// eps of particles i and i + n/2 (n even): one cipher call per component
template <int CD>
__device__ __forceinline__ void pair_noise(uint32_t k0, uint32_t k1, int64_t i, int64_t h, uint32_t one, int D,
                                           float (&ea)[CD], float (&eb)[CD]) {
  const uint64_t hN = (uint64_t)h * D;
#pragma unroll
  for (int j = 0; j < D; ++j) {
    const uint64_t p = (uint64_t)i * D + j;
    uint32_t r0, r1;
    threefry2x32_m(k0, k1, (uint32_t)p, (uint32_t)(p + hN), one, r0, r1);
    ea[j] = bits_to_normal(r0);
    eb[j] = bits_to_normal(r1);
  }
}

// eps of particle i for any n: element-wise counter layout
template <int CD>
__device__ __forceinline__ void single_noise(uint32_t k0, uint32_t k1, int64_t n, int64_t i, int D, float (&e)[CD]) {
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(bits_at(k0, k1, (uint64_t)n * D, (uint64_t)i * D + j));
}

// the proposal key split(k, n)[0] for the block, in shared memory
__device__ __forceinline__ void block_noise_key(const uint32_t *key, int64_t n, uint32_t *ks) {
  if (threadIdx.x == 0) {
    uint32_t a, b;
    split_at(key[0], key[1], (uint64_t)n, 0, a, b);
    ks[0] = a;
    ks[1] = b;
  }
  __syncthreads();
}

// x_0 = mean0 + eps C0c (column sums in ascending order), mean0 = m0 + K0 (y0 - H m0)
template <int CD, int CDY, bool RT>
__device__ __forceinline__ void opt_init_particle(const OPTP<CD, CDY, RT> &p, const float *mean0,
                                                  const float (&e)[CD], int64_t n, int64_t i, float *x) {
  const int D = p.d();
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float v = __fmul_rn(e[0], p.C0c[r]);
#pragma unroll
    for (int k = 1; k < D; ++k) v = __fmaf_rn(e[k], p.C0c[k * D + r], v);
    x[r * n + i] = __fadd_rn(mean0[r], v);
  }
}

// mean0 into shared memory (thread 0; the caller synchronises)
template <int CD, int CDY, bool RT>
__device__ __forceinline__ void opt_mean0(const OPTP<CD, CDY, RT> &p, const float *y0, float *mean0) {
  const int D = p.d(), DY = p.dy();
  if (threadIdx.x == 0) {
    float innov[CDY];
#pragma unroll
    for (int j = 0; j < DY; ++j) {
      float hm = __fmul_rn(p.H[j * D], p.m0[0]);
#pragma unroll
      for (int k = 1; k < D; ++k) hm = __fmaf_rn(p.H[j * D + k], p.m0[k], hm);
      innov[j] = __fsub_rn(y0[j], hm);
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
      float g = __fmul_rn(p.K0[r * DY], innov[0]);
#pragma unroll
      for (int j = 1; j < DY; ++j) g = __fmaf_rn(p.K0[r * DY + j], innov[j], g);
      mean0[r] = __fadd_rn(p.m0[r], g);
    }
  }
}

template <int CD, int CDY, bool RT, bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_opt_init(const __grid_constant__ OPTP<CD, CDY, RT> p, int64_t n,
                                                      const uint32_t *key, const float *y0, float *__restrict__ x,
                                                      float *__restrict__ lw, PFCtl ctl) {
  const int D = p.d();
  __shared__ uint32_t ks[2];
  __shared__ float mean0[CD];
  opt_mean0(p, y0, mean0);
  block_noise_key(key, n, ks);
  const uint32_t k0 = ks[0], k1 = ks[1];
  float m = -INFINITY, a1 = 0.0f, a2 = 0.0f;
  int nanf = 0;
  if (n % 2 == 0) {
    const int64_t h = n >> 1;
    const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
    if (i < h) {
      float ea[CD], eb[CD];
      pair_noise<CD>(k0, k1, i, h, p.one, D, ea, eb);
      opt_init_particle(p, mean0, ea, n, i, x);
      opt_init_particle(p, mean0, eb, n, i + h, x);
      lw[i] = 0.0f;
      lw[i + h] = 0.0f;
      online_acc(0.0f, m, a1, a2, nanf);
      online_acc(0.0f, m, a1, a2, nanf);
    }
  } else {
    const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
    if (i < n) {
      float e[CD];
      single_noise<CD>(k0, k1, n, i, D, e);
      opt_init_particle(p, mean0, e, n, i, x);
      lw[i] = 0.0f;
      online_acc(0.0f, m, a1, a2, nanf);
    }
  }
  if (FUSED) pf_reduce_online<PF_TPB>(m, a1, a2, nanf, ctl, 0);
}

// one particle of the fused step (nonlinear_gaussian.py:264-281), oracle op order
template <int CD, int CDY, bool RT>
__device__ __forceinline__ float opt_particle(const OPTP<CD, CDY, RT> &p, int64_t n, int64_t i, const float (&e)[CD],
                                              bool res, const float *__restrict__ x_prev, const int32_t *anc,
                                              const float *lws, const float *y, float *__restrict__ x_new,
                                              float *__restrict__ lw_new) {
  const int D = p.d(), DY = p.dy();
  const int64_t src = res ? (int64_t)anc[i] : i;
  float xs[CD], mx[CD], innov[CDY];
#pragma unroll
  for (int j = 0; j < D; ++j) xs[j] = __ldg(&x_prev[j * n + src]);
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float v = __fmul_rn(p.F[r * D], xs[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) v = __fmaf_rn(p.F[r * D + k], xs[k], v);
    mx[r] = v;
  }
#pragma unroll
  for (int j = 0; j < DY; ++j) {
    float hm = __fmul_rn(mx[0], p.H[j * D]);
#pragma unroll
    for (int k = 1; k < D; ++k) hm = __fmaf_rn(mx[k], p.H[j * D + k], hm);
    innov[j] = __fsub_rn(y[j], hm);
  }
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float g = __fmul_rn(innov[0], p.K[r * DY]);
#pragma unroll
    for (int j = 1; j < DY; ++j) g = __fmaf_rn(innov[j], p.K[r * DY + j], g);
    float s = __fmul_rn(e[0], p.S[r * D]);
#pragma unroll
    for (int k = 1; k < D; ++k) s = __fmaf_rn(e[k], p.S[r * D + k], s);
    x_new[r * n + i] = __fadd_rn(__fadd_rn(mx[r], g), s);
  }
  float quad = 0.0f;
#pragma unroll
  for (int k = 0; k < DY; ++k) {
    float v = __fmul_rn(innov[0], p.W[k]);
#pragma unroll
    for (int j = 1; j < DY; ++j) v = __fmaf_rn(innov[j], p.W[j * DY + k], v);
    quad = k == 0 ? __fmul_rn(v, v) : __fmaf_rn(v, v, quad);
  }
  const float lres = lws ? lws[i] : 0.0f;
  const float l = __fsub_rn(lres, __fadd_rn(__fmul_rn(0.5f, quad), p.cw));
  lw_new[i] = l;
  return l;
}

// one step; res_flag (nullable) decides resampled vs identity at run time
template <int CD, int CDY, bool RT, bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_opt_step(const __grid_constant__ OPTP<CD, CDY, RT> p, int64_t n,
                                                      const uint32_t *key, const float *y_t,
                                                      const float *__restrict__ x_prev, const int32_t *anc,
                                                      const float *lw_prev, const int32_t *res_flag,
                                                      float *__restrict__ x_new, float *__restrict__ lw_new,
                                                      PFCtl ctl, int64_t t) {
  const int D = p.d(), DY = p.dy();
  __shared__ uint32_t ks[2];
  __shared__ float y[CDY];
  if (threadIdx.x < DY) y[threadIdx.x] = y_t[threadIdx.x];
  block_noise_key(key, n, ks);
  const uint32_t k0 = ks[0], k1 = ks[1];
  const bool res = res_flag ? (*res_flag != 0) : (anc != nullptr);
  // run mode: lw_res = 0 after a resample (filtering.py:292); standalone: lw_prev as given
  const float *lws = res_flag ? (res ? nullptr : lw_prev) : lw_prev;
  float m = -INFINITY, a1 = 0.0f, a2 = 0.0f;
  int nanf = 0;
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  if (n % 2 == 0) {
    const int64_t h = n >> 1;
    if (i < h) {
      float ea[CD], eb[CD];
      pair_noise<CD>(k0, k1, i, h, p.one, D, ea, eb);
      online_acc(opt_particle(p, n, i, ea, res, x_prev, anc, lws, y, x_new, lw_new), m, a1, a2, nanf);
      online_acc(opt_particle(p, n, i + h, eb, res, x_prev, anc, lws, y, x_new, lw_new), m, a1, a2, nanf);
    }
  } else if (i < n) {
    float e[CD];
    single_noise<CD>(k0, k1, n, i, D, e);
    online_acc(opt_particle(p, n, i, e, res, x_prev, anc, lws, y, x_new, lw_new), m, a1, a2, nanf);
  }
  if (FUSED) pf_reduce_online<PF_TPB>(m, a1, a2, nanf, ctl, t);
}

inline unsigned opt_grid(int64_t n) {
  const int64_t work = n % 2 == 0 ? n / 2 : n;
  return (unsigned)((work + PF_TPB - 1) / PF_TPB);
}

template <int CD, int CDY, bool RT = false>
static int run_opt(const mgb_opt_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y, float thr,
                   int scheme, void *ws, size_t ws_bytes, const mgb_pf_outputs *out, cudaStream_t s) {
  const OPTP<CD, CDY, RT> p = pack_opt<CD, CDY, RT>(m);
  const int D = p.d(), DY = p.dy();
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
  if ((st = launch_setup_keys(key, T, w.keys, s))) return st;
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
  auto xbuf = [&](int64_t t) -> float * { return hx ? out->x_hist + (size_t)t * D * n : (t & 1 ? w.xb : w.xa); };
  auto lbuf = [&](int64_t t) -> float * { return hl ? out->lw_hist + (size_t)t * n : (t & 1 ? w.lb : w.la); };
  const unsigned grid = opt_grid(n);
  k_opt_init<CD, CDY, RT, true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys, y, xbuf(0), lbuf(0), ctl);
  if ((st = launch_status())) return st;
  for (int64_t t = 1; t < T; ++t) {
    st = launch_resample(lbuf(t - 1), n, scheme, &w.st->M, w.keys + 2 * t, 0, 0u, w.res_hist + t, w.rws, w.anc,
                         err, s);
    if (st) return st;
    k_opt_step<CD, CDY, RT, true><<<grid, PF_TPB, 0, s>>>(p, n, w.keys + 2 * t, y + (size_t)t * DY, xbuf(t - 1),
                                                           w.anc, lbuf(t - 1), w.res_hist + t, xbuf(t), lbuf(t), ctl,
                                                           t);
    if ((st = launch_status())) return st;
  }
  if ((st = launch_finish(w.st, w.res_hist, T, out ? out->log_z : nullptr, out ? out->resampled : nullptr, s)))
    return st;
  if (out && out->x_final && cudaMemcpyAsync(out->x_final, xbuf(T - 1), sizeof(float) * D * n,
                                             cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  if (out && out->lw_final && cudaMemcpyAsync(out->lw_final, lbuf(T - 1), sizeof(float) * n,
                                              cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  return launch_status();
}

template <int CD, int CDY, bool RT = false>
static int init_opt(const mgb_opt_model *m, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw,
                    cudaStream_t s) {
  const OPTP<CD, CDY, RT> p = pack_opt<CD, CDY, RT>(m);
  PFCtl ctl{};
  k_opt_init<CD, CDY, RT, false><<<opt_grid(n), PF_TPB, 0, s>>>(p, n, key, y0, x, lw, ctl);
  return launch_status();
}

template <int CD, int CDY, bool RT = false>
static int step_opt(const mgb_opt_model *m, int64_t n, const uint32_t *key, const float *y, const float *xp,
                    const int32_t *anc, const float *lwp, float *xn, float *lwn, cudaStream_t s) {
  const OPTP<CD, CDY, RT> p = pack_opt<CD, CDY, RT>(m);
  PFCtl ctl{};
  k_opt_step<CD, CDY, RT, false><<<opt_grid(n), PF_TPB, 0, s>>>(p, n, key, y, xp, anc, lwp, nullptr, xn, lwn, ctl,
                                                                0);
  return launch_status();
}

static bool opt_model_ok(const mgb_opt_model *m) {
  return m && m->F && m->H && m->K && m->S && m->W && m->K0 && m->C0c && m->m0 && m->d >= 1 && m->dy >= 1;
}

// the (n, d) draw uses 32-bit counters
static bool opt_size_ok(const mgb_opt_model *m, int64_t n) {
  return n >= 1 && n <= 0x7FFFFFFFll && (uint64_t)n * (uint64_t)m->d < (1ull << 32);
}

// compiled pairs take their own instances; any other (d, dy) up to 32 the run-time one
#define MGB_OPT_DISPATCH(FN, ...)                                                      \
  do {                                                                                 \
    const int d_ = m->d, dy_ = m->dy;                                                  \
    if (dy_ == 1) {                                                                    \
      switch (d_) {                                                                    \
        case 1: return FN<1, 1>(__VA_ARGS__);                                          \
        case 2: return FN<2, 1>(__VA_ARGS__);                                          \
        case 3: return FN<3, 1>(__VA_ARGS__);                                          \
        case 4: return FN<4, 1>(__VA_ARGS__);                                          \
        case 5: return FN<5, 1>(__VA_ARGS__);                                          \
        case 8: return FN<8, 1>(__VA_ARGS__);                                          \
        case 10: return FN<10, 1>(__VA_ARGS__);                                        \
        default: break;                                                                \
      }                                                                                \
    } else if (dy_ == d_) {                                                            \
      switch (d_) {                                                                    \
        case 2: return FN<2, 2>(__VA_ARGS__);                                          \
        case 3: return FN<3, 3>(__VA_ARGS__);                                          \
        case 4: return FN<4, 4>(__VA_ARGS__);                                          \
        case 5: return FN<5, 5>(__VA_ARGS__);                                          \
        case 8: return FN<8, 8>(__VA_ARGS__);                                          \
        case 10: return FN<10, 10>(__VA_ARGS__);                                       \
        default: break;                                                                \
      }                                                                                \
    }                                                                                  \
    if (d_ <= OPT_DMAX && dy_ <= OPT_DMAX) return FN<OPT_DMAX, OPT_DMAX, true>(__VA_ARGS__); \
    return ERR_UNSUPPORTED;                                                            \
  } while (0)

}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_pf_opt_init(const mgb_opt_model *m, int64_t n, const uint32_t *key, const float *y0, float *x, float *lw,
                    void *stream) {
  if (!opt_model_ok(m) || !opt_size_ok(m, n) || !key || !y0 || !x || !lw) return ERR_BAD_ARG;
  MGB_OPT_DISPATCH(init_opt, m, n, key, y0, x, lw, (cudaStream_t)stream);
}

int mgb_pf_opt_propagate(const mgb_opt_model *m, int64_t n, const uint32_t *key, const float *y, const float *xp,
                         const int32_t *anc, const float *lwp, float *xn, float *lwn, void *stream) {
  if (!opt_model_ok(m) || !opt_size_ok(m, n) || !key || !y || !xp || !xn || !lwn) return ERR_BAD_ARG;
  MGB_OPT_DISPATCH(step_opt, m, n, key, y, xp, anc, lwp, xn, lwn, (cudaStream_t)stream);
}

size_t mgb_pf_opt_workspace(int64_t n, int64_t T, int32_t d, int scheme) {
  if (n < 1 || T < 1 || d < 1) return 0;
  Carver c(nullptr);
  carve_run(c, n, T, d, scheme & 0xff, true, true, true);
  return c.bytes();
}

int mgb_pf_opt_run(const mgb_opt_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y,
                   float ess_threshold, int scheme, void *ws, size_t ws_bytes, const mgb_pf_outputs *out,
                   void *stream) {
  if (!opt_model_ok(m) || !opt_size_ok(m, n) || T < 1 || !key || !y || !ws) return ERR_BAD_ARG;
  if (scheme != MGB_RESAMPLE_SYSTEMATIC && scheme != MGB_RESAMPLE_MULTINOMIAL && scheme != MGB_RESAMPLE_CATEGORICAL)
    return ERR_UNSUPPORTED;
  if (scheme == MGB_RESAMPLE_CATEGORICAL && n > 46340) return ERR_UNSUPPORTED;
  MGB_OPT_DISPATCH(run_opt, m, n, T, key, y, ess_threshold, scheme, ws, ws_bytes, out, (cudaStream_t)stream);
}

}  // extern "C"
