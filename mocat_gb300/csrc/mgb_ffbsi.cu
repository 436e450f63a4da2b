// Backward simulation (forward filtering, backward simulation) and particle
// stitching: the full O(N M) versions, for a linear-Gaussian transition, the
// one-dimensional non-linear benchmark transition and the stochastic-volatility one.
//
// Reference: backward_simulation_full (mocat/src/ssm/backward.py:217-245),
// full_resampling / full_resample_single (:20-40):
//   t_keys = split(key, T)
//   samples at T-1:  categorical(t_keys[T-1], lw_{T-1}, (M,))  -- one (M, N) Gumbel draw
//   for t = T-2 .. 0, sample j (keys = split(t_keys[t], M)):
//     index_j = argmax_i gumbel(keys[j], (N,))_i + lw_{t,i} - transition_potential(x_t^i -> xs_{t+1}^j)
// transition_potential(x0 -> x1) = potential(x1 - mean(x0)):
//   linear-Gaussian   mean = F x0, potential(diff) = 0.5 |diff @ Pq|^2 + cq
//                     (linear_gaussian.py, gaussian_potential utils.py:49-105);
//   non-linear 1-D    mean = 0.5 x + 25 x / (1 + x^2) + 8 cos(1.2 t_prev),
//                     potential(diff) = 0.5 (diff / transition_sd)^2 + log(2 pi) / 2
//                     (nonlinear1d.py:41-61).
// The kernels are templates over a transition policy (LGT<D>, NLT, SVT) that supplies
// the two; LGT<32, true> reads its dimension (any d up to 32) from the parameter block.  First maximum wins, NaN entries are skipped.
//
// One CTA per sample: mean(x_t^i) is computed once per step by a separate kernel
// (dimension-major, read through L2 by every CTA); the Gumbel bits of element
// i and i + ceil(N/2) come from the two halves of one cipher call.  The
// argmax is reduced in the fixed order (value, then smaller index), so the
// result does not depend on scheduling.
#include <type_traits>
#include <vector>

#include "mgb_transition.cuh"

namespace mgb {

// step t: sample j conditions on its state at t + 1
template <class TP>
__global__ void __launch_bounds__(FB_TPB) k_ffbsi_step(const __grid_constant__ TP p, int64_t N, int64_t M,
                                                        const float *__restrict__ fx, const float *__restrict__ lw,
                                                        const float *__restrict__ x_next_samples,
                                                        const uint32_t *tkey, int32_t *__restrict__ idx) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  __shared__ Best sm[FB_TPB / 32];
  __shared__ float x1[DC];
  __shared__ uint32_t kj[2];
  const int64_t j = blockIdx.x;
  if (threadIdx.x < D) x1[threadIdx.x] = x_next_samples[threadIdx.x * M + j];
  if (threadIdx.x == 0) {
    uint32_t a0, a1;
    split_at(tkey[0], tkey[1], (uint64_t)M, (uint64_t)j, a0, a1);
    kj[0] = a0;
    kj[1] = a1;
  }
  __syncthreads();
  const uint32_t k0 = kj[0], k1 = kj[1];
  const int64_t h = (N + 1) >> 1;
  Best b{-INFINITY, 0, 0};
  for (int64_t q = threadIdx.x; q < h; q += FB_TPB) {
    uint32_t r0, r1;
    threefry2x32_m(k0, k1, (uint32_t)q, q + h < N ? (uint32_t)(q + h) : 0u, p.one, r0, r1);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int64_t i = s ? q + h : q;
      if (i >= N) break;
      const float g = bits_to_gumbel(s ? r1 : r0);
      float diff[DC];
#pragma unroll
      for (int r = 0; r < D; ++r) diff[r] = __fsub_rn(x1[r], fx[r * N + i]);
      best_take(b, __fadd_rn(g, __fsub_rn(lw[i], p.potential(diff))), (int32_t)i);
    }
  }
  const int32_t bi = block_argmax<FB_TPB>(b, sm);
  if (threadIdx.x == 0) idx[j] = bi;
}

// transition potential of particle pairs (x0_i -> x1_i), plus lw_i when given
// (non_interacting_log_weight of fixed_lag_stitching, online_smoothing.py:191-193)
template <class TP>
__global__ void __launch_bounds__(FB_TPB) k_pair_potential(const __grid_constant__ TP p, int64_t M,
                                                            const float *__restrict__ x0, const float *__restrict__ x1,
                                                            const float *__restrict__ lw, float *__restrict__ out) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  __shared__ float sd[1];
  const float drift = block_drift(p, sd);
  const int64_t i = blockIdx.x * (int64_t)FB_TPB + threadIdx.x;
  if (i >= M) return;
  float xv[DC], m[DC], diff[DC];
#pragma unroll
  for (int k = 0; k < D; ++k) xv[k] = x0[k * M + i];
  p.mean(xv, m, drift);
#pragma unroll
  for (int r = 0; r < D; ++r) diff[r] = __fsub_rn(x1[r * M + i], m[r]);
  const float pot = p.potential(diff);
  out[i] = lw ? __fadd_rn(lw[i], pot) : pot;
}

// full_stitch (online_smoothing.py:21-41): CTA j conditions on x0_j and draws among the x1_i
template <class TP>
__global__ void __launch_bounds__(FB_TPB) k_stitch(const __grid_constant__ TP p, int64_t M0, int64_t M1,
                                                    const float *__restrict__ x0, const float *__restrict__ x1,
                                                    const float *__restrict__ lw1, const uint32_t *key,
                                                    int32_t *__restrict__ idx) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  __shared__ Best sm[FB_TPB / 32];
  __shared__ float fx0[DC];
  __shared__ uint32_t kj[2];
  __shared__ float sd[1];
  const float drift = block_drift(p, sd);
  const int64_t j = blockIdx.x;
  if (threadIdx.x == 0) {
    float xv[DC], m[DC];
#pragma unroll
    for (int k = 0; k < D; ++k) xv[k] = x0[k * M0 + j];
    p.mean(xv, m, drift);
#pragma unroll
    for (int r = 0; r < D; ++r) fx0[r] = m[r];
    uint32_t a0, a1;
    split_at(key[0], key[1], (uint64_t)M0, (uint64_t)j, a0, a1);
    kj[0] = a0;
    kj[1] = a1;
  }
  __syncthreads();
  const uint32_t k0 = kj[0], k1 = kj[1];
  const int64_t h = (M1 + 1) >> 1;
  Best b{-INFINITY, 0, 0};
  for (int64_t q = threadIdx.x; q < h; q += FB_TPB) {
    uint32_t r0, r1;
    threefry2x32_m(k0, k1, (uint32_t)q, q + h < M1 ? (uint32_t)(q + h) : 0u, p.one, r0, r1);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int64_t i = s ? q + h : q;
      if (i >= M1) break;
      const float g = bits_to_gumbel(s ? r1 : r0);
      float diff[DC];
#pragma unroll
      for (int r = 0; r < D; ++r) diff[r] = __fsub_rn(x1[r * M1 + i], fx0[r]);
      best_take(b, __fadd_rn(g, __fsub_rn(lw1[i], p.potential(diff))), (int32_t)i);
    }
  }
  const int32_t bi = block_argmax<FB_TPB>(b, sm);
  if (threadIdx.x == 0) idx[j] = bi;
}

template <class TP>
static int stitch_run(const TP &p, int64_t M0, int64_t M1, const float *x0, const float *x1, const float *lw1,
                      const uint32_t *key, int32_t *idx, cudaStream_t s) {
  k_stitch<TP><<<(unsigned)M0, FB_TPB, 0, s>>>(p, M0, M1, x0, x1, lw1, key, idx);
  return launch_status();
}

template <class TP>
static int pairs_run(const TP &p, int64_t M, const float *x0, const float *x1, const float *lw, float *out,
                     cudaStream_t s) {
  k_pair_potential<TP><<<(unsigned)((M + FB_TPB - 1) / FB_TPB), FB_TPB, 0, s>>>(p, M, x0, x1, lw, out);
  return launch_status();
}

template <int D, bool RT = false>
static int stitch_lg(const mgb_lg_transition *tr, int64_t M0, int64_t M1, const float *x0, const float *x1,
                     const float *lw1, const uint32_t *key, int32_t *idx, cudaStream_t s) {
  return stitch_run(pack_lgt<D, RT>(tr), M0, M1, x0, x1, lw1, key, idx, s);
}

template <int D, bool RT = false>
static int pair_potential(const mgb_lg_transition *tr, int64_t M, const float *x0, const float *x1, const float *lw,
                          float *out, cudaStream_t s) {
  return pairs_run(pack_lgt<D, RT>(tr), M, x0, x1, lw, out, s);
}

// t_all (device, T times): step t's transition leaves x_t at t_all[t] (policies with a drift)
template <class TP>
static int ffbsi_run(TP p, const float *t_all, int64_t T, int64_t N, int64_t M, const float *x_hist,
                     const float *lw_hist, const uint32_t *key, float *out, int32_t *idx, void *ws, size_t ws_bytes,
                     cudaStream_t s, const float *pqs_host = nullptr) {
  constexpr int TD = take_dim<TP>();
  const int D = p.dim();
  Carver c(ws);
  float *fx = c.take<float>((size_t)D * N);
  uint32_t *tkeys = c.take<uint32_t>(2 * (size_t)T);
  if (c.bytes() > ws_bytes) return ERR_WORKSPACE;
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
    k_ffbsi_step<TP><<<(unsigned)M, FB_TPB, 0, s>>>(p, N, M, fx, lw_hist + (size_t)t * N,
                                                    out + (size_t)(t + 1) * D * M, tkeys + 2 * t,
                                                    idx + (size_t)t * M);
    if ((st = launch_status())) return st;
    k_ffbsi_take<TD><<<grid_for(M, 256), 256, 0, s>>>(N, M, x_hist + (size_t)t * xs, idx + (size_t)t * M,
                                                      out + (size_t)t * D * M, D);
    if ((st = launch_status())) return st;
  }
  return OK;
}

template <int D, bool RT = false>
static int ffbsi_lg(const mgb_lg_transition *tr, int64_t T, int64_t N, int64_t M, const float *x_hist,
                    const float *lw_hist, const uint32_t *key, float *out, int32_t *idx, void *ws, size_t ws_bytes,
                    cudaStream_t s) {
  return ffbsi_run(pack_lgt<D, RT>(tr), nullptr, T, N, M, x_hist, lw_hist, key, out, idx, ws, ws_bytes, s);
}

static bool ffbsi_sizes_ok(int64_t T, int64_t N, int64_t M) {
  return T >= 1 && N >= 1 && N <= 0x7FFFFFFFll && M >= 1 && M <= 0x7FFFFFFFll &&
         (uint64_t)M * (uint64_t)N < (1ull << 32);
}

}  // namespace mgb

using namespace mgb;

// compiled dimensions take their own instances; any other d up to 32 the run-time one
#define MGB_FB_DISPATCH(FN, ...)                                                    \
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

size_t mgb_ffbsi_workspace(int64_t N, int64_t T, int32_t d) {
  if (N < 1 || T < 1 || d < 1) return 0;
  Carver c(nullptr);
  c.take<float>((size_t)d * N);
  c.take<uint32_t>(2 * (size_t)T);
  return c.bytes();
}

int mgb_ffbsi_lg(const mgb_lg_transition *tr, int64_t T, int64_t N, int64_t M, const float *x_hist,
                 const float *lw_hist, const uint32_t *key, float *out, int32_t *idx, void *ws, size_t ws_bytes,
                 void *stream) {
  if (!tr || !tr->F || !tr->Pq || !ffbsi_sizes_ok(T, N, M) || !x_hist || !lw_hist || !key || !out || !idx || !ws)
    return ERR_BAD_ARG;
  MGB_FB_DISPATCH(ffbsi_lg, tr, T, N, M, x_hist, lw_hist, key, out, idx, ws, ws_bytes, (cudaStream_t)stream);
}

int mgb_stitch_lg(const mgb_lg_transition *tr, int64_t M0, int64_t M1, const float *x0, const float *x1,
                  const float *lw1, const uint32_t *key, int32_t *idx, void *stream) {
  if (!tr || !tr->F || !tr->Pq || M0 < 1 || M1 < 1 || M0 > 0x7FFFFFFFll || M1 > 0x7FFFFFFFll || !x0 || !x1 ||
      !lw1 || !key || !idx)
    return ERR_BAD_ARG;
  MGB_FB_DISPATCH(stitch_lg, tr, M0, M1, x0, x1, lw1, key, idx, (cudaStream_t)stream);
}

int mgb_transition_potential_pairs(const mgb_lg_transition *tr, int64_t M, const float *x0, const float *x1,
                                   const float *lw, float *out, void *stream) {
  if (!tr || !tr->F || !tr->Pq || M < 1 || !x0 || !x1 || !out) return ERR_BAD_ARG;
  MGB_FB_DISPATCH(pair_potential, tr, M, x0, x1, lw, out, (cudaStream_t)stream);
}

int mgb_ffbsi_nl1d(const mgb_nl1d_model *m, int64_t T, int64_t N, int64_t M, const float *x_hist,
                   const float *lw_hist, const float *t, const uint32_t *key, float *out, int32_t *idx, void *ws,
                   size_t ws_bytes, void *stream) {
  if (!m || !ffbsi_sizes_ok(T, N, M) || !x_hist || !lw_hist || !t || !key || !out || !idx || !ws) return ERR_BAD_ARG;
  return ffbsi_run(pack_nlt(m, nullptr, 0.0f), t, T, N, M, x_hist, lw_hist, key, out, idx, ws, ws_bytes,
                   (cudaStream_t)stream);
}

int mgb_stitch_nl1d(const mgb_nl1d_model *m, int64_t M0, int64_t M1, const float *x0, const float *x1,
                    const float *lw1, float t_previous, const uint32_t *key, int32_t *idx, void *stream) {
  if (!m || M0 < 1 || M1 < 1 || M0 > 0x7FFFFFFFll || M1 > 0x7FFFFFFFll || !x0 || !x1 || !lw1 || !key || !idx)
    return ERR_BAD_ARG;
  return stitch_run(pack_nlt(m, nullptr, t_previous), M0, M1, x0, x1, lw1, key, idx, (cudaStream_t)stream);
}

int mgb_transition_potential_pairs_nl1d(const mgb_nl1d_model *m, int64_t M, const float *x0, const float *x1,
                                        float t_previous, const float *lw, float *out, void *stream) {
  if (!m || M < 1 || !x0 || !x1 || !out) return ERR_BAD_ARG;
  return pairs_run(pack_nlt(m, nullptr, t_previous), M, x0, x1, lw, out, (cudaStream_t)stream);
}

// stochastic volatility (dim 1): t_host the T times on the host; step t's potential scales
// by sqrt(t_host[t + 1] - t_host[t])
int mgb_ffbsi_sv(float phi, float pq, int64_t T, int64_t N, int64_t M, const float *x_hist, const float *lw_hist,
                 const float *t_host, const uint32_t *key, float *out, int32_t *idx, void *ws, size_t ws_bytes,
                 void *stream) {
  if (!ffbsi_sizes_ok(T, N, M) || !x_hist || !lw_hist || !t_host || !key || !out || !idx || !ws) return ERR_BAD_ARG;
  std::vector<float> pqs((size_t)T, pq);
  for (int64_t t = 0; t + 1 < T; ++t) pqs[t] = pq * std::sqrt(t_host[t + 1] - t_host[t]);
  return ffbsi_run(pack_svt(phi, pq, 1.0f), nullptr, T, N, M, x_hist, lw_hist, key, out, idx, ws, ws_bytes,
                   (cudaStream_t)stream, pqs.data());
}

int mgb_stitch_sv(float phi, float pq, int64_t M0, int64_t M1, const float *x0, const float *x1, const float *lw1,
                  float dt, const uint32_t *key, int32_t *idx, void *stream) {
  if (M0 < 1 || M1 < 1 || M0 > 0x7FFFFFFFll || M1 > 0x7FFFFFFFll || !x0 || !x1 || !lw1 || !key || !idx)
    return ERR_BAD_ARG;
  return stitch_run(pack_svt(phi, pq, dt), M0, M1, x0, x1, lw1, key, idx, (cudaStream_t)stream);
}

int mgb_transition_potential_pairs_sv(float phi, float pq, int64_t M, const float *x0, const float *x1, float dt,
                                      const float *lw, float *out, void *stream) {
  if (M < 1 || !x0 || !x1 || !out) return ERR_BAD_ARG;
  return pairs_run(pack_svt(phi, pq, dt), M, x0, x1, lw, out, (cudaStream_t)stream);
}

}  // extern "C"
