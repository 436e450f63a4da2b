// Adjoint of the bootstrap filter's log Z with the resampling held fixed.
//
// Reference path: jax.grad through run_particle_filter_for_marginals
// (mocat/src/ssm/filtering.py:255-324) with BootstrapFilter on a
// TimeHomogenousLinearGaussian model (mocat/src/ssm/linear_gaussian/linear_gaussian.py:
// transition_sample :86-94, likelihood_potential :118-128) whose likelihood matrix
// is the identity and whose covariances are diagonal; the ancestors and the
// resampling decisions are constants.  theta = (A, log q, log r) with
// Lq = diag(sqrt(q)), P = diag(1 / sqrt(r)).
//
// log Z = sum over segment ends e of LSE(lw_e) - (#segments) log n, where a
// segment is a run of steps without resampling and lw_e sums -pot along it, so
// d log Z / d pot_t^i = -W_e(t)^i (normalised weights at the end of t's segment).
// Backward recursion over particles j (mu = adjoint carried into step t from t+1):
//   mu_t^j    = sum_{i : a_{t+1}^i = j} lambda_{t+1}^i      (identity if t+1 did not resample)
//   lambda_t^j = -W^j d pot/dx (x_t^j) + A^T mu_t^j
//   dA       += mu_t^j x_t^j^T
//   dlog q_k += lambda_{t,k}^j eps_{t,k}^j sqrt(q_k) / 2     (t >= 1)
//   dlog r_k += -W^j (1/2 - ((y_k - x_k) P_k)^2 / 2)
// Memory: the forward pass keeps (x, lw) every `ckpt` steps and the ancestors
// of every step; the backward pass recomputes each segment of `ckpt` steps
// from its checkpoint (x_t, lw_t and the draws eps_t, bit-identical to the
// forward), then walks it backwards.  Children of parent j are the index range
// [starts_j, starts_{j+1}) of the sorted ancestor vector (systematic and
// multinomial resampling both give non-decreasing ancestors); the kernel that
// produces lambda of a resampled step stores it as warp-chunk prefixes
// restarted at each new ancestor, so a parent with many children sums one
// value per 32 of them (the order is fixed: results do not depend on timing).  Parameter
// partials accumulate per block across all steps (float32) and are summed at
// the end, so the result does not depend on scheduling.
#include <cmath>
#include <vector>

#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_kernels.cuh"
#include "mgb_lg.cuh"
#include "mgb_pf_common.cuh"
#include "mgb_lg_kernels.cuh"
#include "mgb_persist.cuh"

namespace mgb {

constexpr int ADJ_TPB = 256;

// Recompute step t (one particle per thread) with the forward's arithmetic;
// noise_only writes eps_t alone (the checkpointed step).
template <int D>
__global__ void __launch_bounds__(ADJ_TPB) k_adj_recompute(const __grid_constant__ LGP<D, D> p, int64_t n,
                                                            const uint32_t *key, const float *y_t,
                                                            const float *__restrict__ x_prev, const int32_t *anc,
                                                            const float *lw_prev, int res, int noise_only,
                                                            float *__restrict__ x_new, float *__restrict__ lw_new,
                                                            float *__restrict__ eps) {
  const int64_t i = blockIdx.x * (int64_t)ADJ_TPB + threadIdx.x;
  if (i >= n) return;
  uint32_t a0, a1;
  split_at(key[0], key[1], (uint64_t)n, (uint64_t)i, a0, a1);
  uint32_t b[D];
  bits_vec<D>(a0, a1, b, p.one);
  float e[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    e[j] = bits_to_normal(b[j]);
    eps[j * n + i] = e[j];
  }
  if (noise_only) return;
  const int64_t src = res ? (int64_t)anc[i] : i;
  float xs[D], xn[D];
#pragma unroll
  for (int j = 0; j < D; ++j) xs[j] = __ldg(&x_prev[j * n + src]);
  lg_transition<D, D>(p, xs, e, xn);
#pragma unroll
  for (int r = 0; r < D; ++r) x_new[r * n + i] = xn[r];
  const float lres = res ? 0.0f : lw_prev[i];
  lw_new[i] = __fsub_rn(lres, lg_potential<D, D>(p, xn, y_t));
}

// starts[j] = #{i : anc[i] < j} for sorted anc, j = 0..n
__global__ void k_adj_starts(const int32_t *anc, int64_t n, int32_t *starts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = i == 0 ? 0 : (int64_t)anc[i - 1] + 1;
    const int64_t hi = anc[i];
    for (int64_t j = lo; j <= hi; ++j) starts[j] = (int32_t)i;
    if (i == n - 1)
      for (int64_t j = hi + 1; j <= n; ++j) starts[j] = (int32_t)n;
  }
}

struct AdjStep {
  const float *x, *lw, *eps, *y;  // step t
  const float *lam_next;          // from step t+1 (d, n): lambda_{t+1}, or its segmented warp prefixes
                                  // when t+1 resampled; null at the last step
  const int32_t *starts;          // children of a_{t+1}, null when t+1 did not resample
  const double *lse;              // LSE(lw_t) at a segment end, else null
  const int32_t *anc;             // a_t when step t resampled (lam then holds segmented prefixes), else null
  float *lam;                     // out (d, n)
  float *W;                       // normalised weights of the current segment (n)
  float *partial;                 // (gridDim.x, d d + 2 d), accumulated
  int has_eps;                    // t >= 1
};

template <int D>
__global__ void __launch_bounds__(ADJ_TPB) k_adj_back(const __grid_constant__ LGP<D, D> p, int64_t n,
                                                       const AdjStep s) {
  constexpr int G = D * D + 2 * D;
  __shared__ float mu_s[ADJ_TPB * D], x_s[ADJ_TPB * D], lq_s[ADJ_TPB * D], lr_s[ADJ_TPB * D];
  const int64_t j = blockIdx.x * (int64_t)ADJ_TPB + threadIdx.x;
  const int tid = threadIdx.x;
  float mu[D], xv[D];
#pragma unroll
  for (int k = 0; k < D; ++k) mu[k] = xv[k] = 0.0f;
  float lq[D], lr[D];
#pragma unroll
  for (int k = 0; k < D; ++k) lq[k] = lr[k] = 0.0f;
  if (j < n) {
    if (s.lam_next) {
      if (s.starts) {
        // children [c0, c1) of parent j: lam_next holds, per warp-aligned chunk of 32
        // children, prefixes restarted at each new parent, so the sum over the range is
        // the prefix at c1 - 1 plus the chunk-end prefixes of the earlier chunks it covers
        const int32_t c0 = s.starts[j], c1 = s.starts[j + 1];
        if (c1 > c0) {
          const int32_t k0 = c0 >> 5, k1 = (c1 - 1) >> 5;
#pragma unroll
          for (int k = 0; k < D; ++k) mu[k] = __ldg(&s.lam_next[k * n + c1 - 1]);
          for (int32_t ch = k0; ch < k1; ++ch) {
#pragma unroll
            for (int k = 0; k < D; ++k) mu[k] += __ldg(&s.lam_next[k * n + ch * 32 + 31]);
          }
        }
      } else {
#pragma unroll
        for (int k = 0; k < D; ++k) mu[k] = __ldg(&s.lam_next[k * n + j]);
      }
    }
    float w;
    if (s.lse) {
      w = expf((float)((double)s.lw[j] - *s.lse));
      s.W[j] = w;
    } else {
      w = s.W[j];
    }
    const float g = -w;
#pragma unroll
    for (int k = 0; k < D; ++k) xv[k] = __ldg(&s.x[k * n + j]);
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const float P = p.P[k * D + k];
      const float diff = __ldg(&s.y[k]) - xv[k];
      const float dp = diff * P;
      // lambda_k = g dpot/dx_k + (A^T mu)_k,  dpot/dx_k = -diff P^2
      float lam = -g * diff * (P * P);
#pragma unroll
      for (int r = 0; r < D; ++r) lam = fmaf(p.F[r * D + k], mu[r], lam);
      lq[k] = lam;  // lambda_t, kept for the eps term below
      lr[k] = g * (0.5f - 0.5f * dp * dp);
    }
  }
  // lambda_t out: raw, or (step t resampled) warp prefixes restarted at each new ancestor
  {
    const int32_t key = (j < n && s.anc) ? s.anc[j] : -1;
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      float v = lq[k];
      if (s.anc) {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float u = __shfl_up_sync(full, v, o);
          const int32_t ku = __shfl_up_sync(full, key, o);
          if ((threadIdx.x & 31) >= o && ku == key) v += u;
        }
      }
      if (j < n) s.lam[k * n + j] = v;
    }
  }
  if (j < n) {
#pragma unroll
    for (int k = 0; k < D; ++k)
      lq[k] = s.has_eps ? lq[k] * __ldg(&s.eps[k * n + j]) * (0.5f * p.Lq[k * D + k]) : 0.0f;
  }
#pragma unroll
  for (int k = 0; k < D; ++k) {
    mu_s[tid * D + k] = mu[k];
    x_s[tid * D + k] = xv[k];
    lq_s[tid * D + k] = lq[k];
    lr_s[tid * D + k] = lr[k];
  }
  __syncthreads();
  // block sums of the G parameter partials: two threads per output, half the particles each
  __shared__ float half_s[2 * G];
  for (int q2 = tid; q2 < 2 * G; q2 += ADJ_TPB) {
    const int q = q2 % G, u0 = (q2 / G) * (ADJ_TPB / 2), u1 = u0 + ADJ_TPB / 2;
    float acc = 0.0f;
    if (q < D * D) {
      const int r = q / D, c = q % D;
      for (int u = u0; u < u1; ++u) acc = fmaf(mu_s[u * D + r], x_s[u * D + c], acc);
    } else if (q < D * D + D) {
      const int k = q - D * D;
      for (int u = u0; u < u1; ++u) acc += lq_s[u * D + k];
    } else {
      const int k = q - D * D - D;
      for (int u = u0; u < u1; ++u) acc += lr_s[u * D + k];
    }
    half_s[q2] = acc;
  }
  __syncthreads();
  for (int q = tid; q < G; q += ADJ_TPB) s.partial[(size_t)blockIdx.x * G + q] += half_s[q] + half_s[q + G];
}

// grad[q] = sum over blocks of partial[b][q] (float64 sum, float32 result)
__global__ void k_adj_sum(const float *partial, int nb, int G, float *grad) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < G; q += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int b = 0; b < nb; ++b) acc += (double)partial[(size_t)b * G + q];
    grad[q] = (float)acc;
  }
}

struct AdjWs {
  RunWs run;
  PersistWs pw;
  int32_t *anc_hist;
  float *ckx, *ckl;
  float *segx, *segl, *sege;
  float *lam;
  float *W;
  int32_t *starts;
  float *partial;
  double *lse4;
  void *lse_ws;
  size_t lse_bytes;
};

static AdjWs carve_adj(Carver &c, int64_t n, int64_t T, int d, int scheme, int k) {
  AdjWs w;
  w.run = carve_run(c, n, T, d, scheme, true, true, true);
  w.pw = carve_persist(c, n, T);
  const int64_t nck = (T + k - 1) / k;
  const int64_t nb = (n + ADJ_TPB - 1) / ADJ_TPB;
  w.anc_hist = c.take<int32_t>((size_t)T * n);
  w.ckx = c.take<float>((size_t)nck * d * n);
  w.ckl = c.take<float>((size_t)nck * n);
  w.segx = c.take<float>((size_t)k * d * n);
  w.segl = c.take<float>((size_t)k * n);
  w.sege = c.take<float>((size_t)k * d * n);
  w.lam = c.take<float>((size_t)2 * d * n);
  w.W = c.take<float>((size_t)n);
  w.starts = c.take<int32_t>((size_t)n + 1);
  w.partial = c.take<float>((size_t)nb * (d * d + 2 * d));
  w.lse4 = c.take<double>(4);
  w.lse_bytes = mgb_lse_ess_workspace(n);
  w.lse_ws = c.take<unsigned char>(w.lse_bytes);
  return w;
}

template <int D>
static int grad_lg(const mgb_lg_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y, float thr,
                   int scheme, bool persistent, int k, void *ws, size_t ws_bytes, double *logz_out, float *grad_out,
                   int32_t *resampled_out, cudaStream_t s) {
  const LGP<D, D> p = pack_lg<D, D>(m);
  if (!p.lq_diag || !p.p_diag || !p.h_eye) return ERR_UNSUPPORTED;
  Carver c(ws);
  AdjWs w = carve_adj(c, n, T, D, scheme, k);
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
  RunWs &r = w.run;
  int st;
  // ---- taped forward: the plain filter, keeping the ancestors of every step
  //      and (x, lw) every k steps
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
  std::vector<int32_t> res((size_t)T + 1, 0);
  if (persistent && persistent_ok(n, scheme)) {
    // one persistent launch (k_pf_persist) writing the ancestor tape and the checkpoints
    mgb_pf_outputs o = {};
    o.log_z = logz_out;
    PersistArgs a;
    if ((st = persist_setup(r, w.pw, n, T, y, thr, r.ess_hist, &o, a, s))) return st;
    a.anc_hist = w.anc_hist;
    a.ck_every = k;
    a.ckx = w.ckx;
    a.ckl = w.ckl;
    if ((st = run_lg_persistent(m, a, s))) return st;
    if (resampled_out &&
        cudaMemcpyAsync(resampled_out, a.res, sizeof(int32_t) * T, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return ERR_CUDA;
    // the backward pass is laid out on the host from the resampling decisions
    if (cudaMemcpyAsync(res.data(), a.res, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return ERR_CUDA;
  } else {
    auto xbuf = [&](int64_t t) -> float * {
      return t % k == 0 ? w.ckx + (size_t)(t / k) * D * n : (t & 1 ? r.xb : r.xa);
    };
    auto lbuf = [&](int64_t t) -> float * {
      return t % k == 0 ? w.ckl + (size_t)(t / k) * n : (t & 1 ? r.lb : r.la);
    };
    const unsigned grid = (unsigned)((n + PF_TPB - 1) / PF_TPB);
    const unsigned grid2 = (unsigned)((n / 2 + PF_TPB - 1) / PF_TPB);
    k_lg_init<D, D, true><<<grid, PF_TPB, 0, s>>>(p, n, r.keys, y, xbuf(0), lbuf(0), ctl);
    if ((st = launch_status())) return st;
    for (int64_t t = 1; t < T; ++t) {
      int32_t *anc = w.anc_hist + (size_t)t * n;
      if ((st = launch_resample(lbuf(t - 1), n, scheme, &r.st->M, r.keys + 2 * t, 0, 0u, r.res_hist + t, r.rws,
                                anc, nullptr, s)))
        return st;
      if (n % 2 == 0)
        k_lg_step2<D, D, true><<<grid2, PF_TPB, 0, s>>>(p, n, r.keys + 2 * t, y + (size_t)t * D, xbuf(t - 1), anc,
                                                        lbuf(t - 1), r.res_hist + t, xbuf(t), lbuf(t), ctl, t);
      else
        k_lg_step<D, D, true><<<grid, PF_TPB, 0, s>>>(p, n, r.keys + 2 * t, y + (size_t)t * D, xbuf(t - 1), anc,
                                                      lbuf(t - 1), r.res_hist + t, xbuf(t), lbuf(t), ctl, t);
      if ((st = launch_status())) return st;
    }
    if ((st = launch_finish(r.st, r.res_hist, T, logz_out, resampled_out, s))) return st;
    if (cudaMemcpyAsync(res.data(), r.res_hist, sizeof(int32_t) * (T + 1), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return ERR_CUDA;
  }

  // ---- backward, segment by segment from the end
  const int G = D * D + 2 * D;
  const unsigned nb = (unsigned)((n + ADJ_TPB - 1) / ADJ_TPB);
  if (cudaMemsetAsync(w.partial, 0, sizeof(float) * nb * G, s) != cudaSuccess) return ERR_CUDA;
  const int64_t nseg = (T + k - 1) / k;
  for (int64_t seg = nseg - 1; seg >= 0; --seg) {
    const int64_t c0 = seg * k, e = std::min<int64_t>(c0 + k, T) - 1;
    auto xv = [&](int64_t t) -> float * { return t == c0 ? w.ckx + (size_t)seg * D * n : w.segx + (size_t)(t - c0) * D * n; };
    auto lv = [&](int64_t t) -> float * { return t == c0 ? w.ckl + (size_t)seg * n : w.segl + (size_t)(t - c0) * n; };
    auto ev = [&](int64_t t) -> float * { return w.sege + (size_t)(t - c0) * D * n; };
    for (int64_t t = c0 == 0 ? 1 : c0; t <= e; ++t) {
      const int noise_only = t == c0;
      k_adj_recompute<D><<<nb, ADJ_TPB, 0, s>>>(p, n, r.keys + 2 * t, y + (size_t)t * D,
                                                 noise_only ? nullptr : xv(t - 1),
                                                 w.anc_hist + (size_t)t * n, noise_only ? nullptr : lv(t - 1),
                                                 res[t], noise_only, noise_only ? nullptr : xv(t),
                                                 noise_only ? nullptr : lv(t), ev(t));
      if ((st = launch_status())) return st;
    }
    for (int64_t t = e; t >= c0; --t) {
      const bool last = t == T - 1;
      const bool res_next = !last && res[t + 1];
      AdjStep a;
      a.x = xv(t);
      a.lw = lv(t);
      a.eps = t >= 1 ? ev(t) : nullptr;
      a.y = y + (size_t)t * D;
      a.lam_next = last ? nullptr : w.lam + (size_t)((t + 1) & 1) * D * n;
      a.starts = nullptr;
      a.lse = nullptr;
      a.lam = w.lam + (size_t)(t & 1) * D * n;
      a.anc = (t >= 1 && res[t]) ? w.anc_hist + (size_t)t * n : nullptr;
      a.W = w.W;
      a.partial = w.partial;
      a.has_eps = t >= 1;
      if (last || res_next) {
        if ((st = mgb_lse_ess(a.lw, n, w.lse4, w.lse_ws, w.lse_bytes, s))) return st;
        a.lse = w.lse4 + 1;
      }
      if (res_next) {
        k_adj_starts<<<grid_for(n, 256), 256, 0, s>>>(w.anc_hist + (size_t)(t + 1) * n, n, w.starts);
        a.starts = w.starts;
      }
      k_adj_back<D><<<nb, ADJ_TPB, 0, s>>>(p, n, a);
      if ((st = launch_status())) return st;
    }
  }
  k_adj_sum<<<1, 256, 0, s>>>(w.partial, (int)nb, G, grad_out);
  return launch_status();
}

}  // namespace mgb

using namespace mgb;

extern "C" {

size_t mgb_pf_lg_grad_workspace(int64_t n, int64_t T, int32_t d, int32_t ckpt_every) {
  if (n < 1 || T < 1 || d < 1 || ckpt_every < 1) return 0;
  Carver c(nullptr);
  carve_adj(c, n, T, d, MGB_RESAMPLE_MULTINOMIAL, ckpt_every);
  return c.bytes();
}

int mgb_pf_lg_grad(const mgb_lg_model *m, int64_t n, int64_t T, const uint32_t *key, const float *y,
                   float ess_threshold, int scheme, int32_t ckpt_every, void *ws, size_t ws_bytes, double *log_z,
                   float *grad, int32_t *resampled, void *stream) {
  if (!m || !m->F || !m->Lq || !m->H || !m->P || !m->C0 || !m->m0 || n < 2 || n > 0x7FFFFFFFll || T < 1 || !key ||
      !y || !ws || !grad || ckpt_every < 1)
    return ERR_BAD_ARG;
  if (m->dy != m->d) return ERR_UNSUPPORTED;
  const bool persistent = !(scheme & MGB_RUN_LAUNCH_PER_STEP);
  scheme &= ~MGB_RUN_LAUNCH_PER_STEP;
  if (scheme != MGB_RESAMPLE_SYSTEMATIC && scheme != MGB_RESAMPLE_MULTINOMIAL) return ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  switch (m->d) {
    case 1: return grad_lg<1>(m, n, T, key, y, ess_threshold, scheme, persistent, ckpt_every, ws, ws_bytes, log_z, grad,
                                    resampled, s);
    case 2: return grad_lg<2>(m, n, T, key, y, ess_threshold, scheme, persistent, ckpt_every, ws, ws_bytes, log_z, grad,
                                    resampled, s);
    case 3: return grad_lg<3>(m, n, T, key, y, ess_threshold, scheme, persistent, ckpt_every, ws, ws_bytes, log_z, grad,
                                    resampled, s);
    case 4: return grad_lg<4>(m, n, T, key, y, ess_threshold, scheme, persistent, ckpt_every, ws, ws_bytes, log_z, grad,
                                    resampled, s);
    case 5: return grad_lg<5>(m, n, T, key, y, ess_threshold, scheme, persistent, ckpt_every, ws, ws_bytes, log_z, grad,
                                    resampled, s);
    case 8: return grad_lg<8>(m, n, T, key, y, ess_threshold, scheme, persistent, ckpt_every, ws, ws_bytes, log_z, grad,
                                    resampled, s);
    case 10: return grad_lg<10>(m, n, T, key, y, ess_threshold, scheme, persistent, ckpt_every, ws, ws_bytes, log_z, grad,
                                    resampled, s);
    default: return ERR_UNSUPPORTED;
  }
}

}  // extern "C"
