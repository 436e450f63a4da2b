// Transition policies shared by the backward-simulation, stitching and rejection
// kernels: transition_potential(x0 -> x1) = potential(x1 - mean(x0)) for
//   linear-Gaussian   mean = F x0, potential(diff) = 0.5 |diff @ Pq|^2 + cq
//                     (linear_gaussian.py, gaussian_potential utils.py:49-105);
//   non-linear 1-D    mean = 0.5 x + 25 x / (1 + x^2) + 8 cos(1.2 t_prev),
//                     potential(diff) = 0.5 (diff / transition_sd)^2 + log(2 pi) / 2
//                     (nonlinear1d.py:41-61),
// and the block-wide argmax (first maximum wins, NaN entries skipped) that turns
// Gumbel draws plus log-weights into a categorical draw.
#pragma once
#include <cmath>

#include "mgb_internal.cuh"
#include "mgb_nl1d.cuh"

namespace mgb {

constexpr int FB_TPB = 256;

// linear-Gaussian transition; RT: D is the capacity (32) and the dimension d_ is read from the
// parameter block, F and Pq packed d_ x d_ row-major at the front of their arrays
template <int D, bool RT = false>
struct LGT {
  static constexpr int DIM = D;
  static constexpr bool kDrift = false;
  static constexpr bool kRT = RT;
  float F[D * D], Pq[D * D];
  float cq;
  uint32_t one;
  int d_;
  __host__ __device__ __forceinline__ int dim() const { return RT ? d_ : D; }
  __device__ __forceinline__ void mean(const float (&x)[D], float (&m)[D], float) const {
    const int d = dim();
#pragma unroll
    for (int r = 0; r < d; ++r) {
      float v = __fmul_rn(F[r * d], x[0]);
#pragma unroll
      for (int k = 1; k < d; ++k) v = __fmaf_rn(F[r * d + k], x[k], v);
      m[r] = v;
    }
  }
  __device__ __forceinline__ float potential(const float (&diff)[D]) const {
    const int d = dim();
    float quad = 0.0f;
#pragma unroll
    for (int k = 0; k < d; ++k) {
      float v = __fmul_rn(diff[0], Pq[k]);
#pragma unroll
      for (int r = 1; r < d; ++r) v = __fmaf_rn(diff[r], Pq[r * d + k], v);
      quad = k == 0 ? __fmul_rn(v, v) : __fmaf_rn(v, v, quad);
    }
    return __fadd_rn(__fmul_rn(0.5f, quad), cq);
  }
};

// the run-time-dimension capacity of the linear-Gaussian transition
constexpr int LGT_DMAX = 32;

// non-linear 1-D benchmark transition; t_previous from *tp (device) or tv
struct NLT {
  static constexpr int DIM = 1;
  static constexpr bool kDrift = true;
  static constexpr bool kRT = false;
  float tsd, c;
  const float *tp;
  float tv;
  uint32_t one;
  __host__ __device__ __forceinline__ int dim() const { return 1; }
  __device__ __forceinline__ void mean(const float (&x)[1], float (&m)[1], float drift) const {
    m[0] = nl_mean(x[0], drift);
  }
  __device__ __forceinline__ float potential(const float (&diff)[1]) const { return nl_gauss(diff[0], tsd, c); }
};

// stochastic-volatility transition, dim 1 (stochastic_volatility.py:78-85): mean = phi x0,
// potential(diff) = 0.5 (diff pqs)^2 with pqs = transition_precision_sqrt sqrt(t_new - t_prev)
// (the reference multiplies the precision square root by sqrt(dt)); a 2-D precision square
// root gives no normaliser (gaussian_potential without det_prec, utils.py:67-79).  pqs is set
// per launch by the host.
struct SVT {
  static constexpr int DIM = 1;
  static constexpr bool kDrift = false;
  static constexpr bool kRT = false;
  float phi, pqs;
  uint32_t one;
  __host__ __device__ __forceinline__ int dim() const { return 1; }
  __device__ __forceinline__ void mean(const float (&x)[1], float (&m)[1], float) const {
    m[0] = __fmul_rn(x[0], phi);
  }
  __device__ __forceinline__ float potential(const float (&diff)[1]) const {
    const float v = __fmul_rn(diff[0], pqs);
    return __fmul_rn(0.5f, __fmul_rn(v, v));
  }
};

inline SVT pack_svt(float phi, float pq, float dt) {
  SVT p;
  p.phi = phi;
  p.pqs = pq * std::sqrt(dt);
  p.one = 1u;
  return p;
}

// the policy's per-launch constant (8 cos(1.2 t_prev)), computed once per block
// by thread 0; every thread of the block calls this
template <class TP>
__device__ __forceinline__ float block_drift(const TP &p, float *sm) {
  if constexpr (TP::kDrift) {
    if (threadIdx.x == 0) sm[0] = nl_drift(p.tp ? *p.tp : p.tv);
    __syncthreads();
    return sm[0];
  } else {
    return 0.0f;
  }
}

// mean(x_t^i) for all i (dimension-major in and out)
template <class TP>
__global__ void __launch_bounds__(FB_TPB) k_ffbsi_fx(const __grid_constant__ TP p, int64_t N,
                                                      const float *__restrict__ x, float *__restrict__ fx) {
  constexpr int DC = TP::DIM;
  const int D = p.dim();
  __shared__ float sm[1];
  const float drift = block_drift(p, sm);
  const int64_t i = blockIdx.x * (int64_t)FB_TPB + threadIdx.x;
  if (i >= N) return;
  float xv[DC], m[DC];
#pragma unroll
  for (int k = 0; k < D; ++k) xv[k] = x[k * N + i];
  p.mean(xv, m, drift);
#pragma unroll
  for (int r = 0; r < D; ++r) fx[r * N + i] = m[r];
}

struct Best {
  float v;
  int32_t i;
  int have;
};
__device__ __forceinline__ void best_take(Best &b, float v, int32_t i) {
  if (v != v) return;
  if (!b.have || v > b.v || (v == b.v && i < b.i)) {
    b.v = v;
    b.i = i;
    b.have = 1;
  }
}
__device__ __forceinline__ void best_merge(Best &b, const Best &o) {
  if (!o.have) return;
  if (!b.have || o.v > b.v || (o.v == b.v && o.i < b.i)) b = o;
}

template <int TPB>
__device__ __forceinline__ int32_t block_argmax(Best b, Best *sm) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    Best o;
    o.v = __shfl_down_sync(0xffffffffu, b.v, off);
    o.i = __shfl_down_sync(0xffffffffu, b.i, off);
    o.have = __shfl_down_sync(0xffffffffu, b.have, off);
    best_merge(b, o);
  }
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    Best r = sm[0];
    for (int w = 1; w < TPB / 32; ++w) best_merge(r, sm[w]);
    sm[0] = r;
  }
  __syncthreads();
  return sm[0].have ? sm[0].i : 0;
}

// last step: sample j draws over the (M, N) Gumbel array of t_key
static __global__ void __launch_bounds__(FB_TPB) k_ffbsi_last(int64_t N, int64_t M, const float *__restrict__ lw,
                                                        const uint32_t *tkey, int32_t *__restrict__ idx) {
  __shared__ Best sm[FB_TPB / 32];
  const int64_t j = blockIdx.x;
  const uint32_t k0 = tkey[0], k1 = tkey[1];
  const uint64_t tot = (uint64_t)M * (uint64_t)N;
  Best b{-INFINITY, 0, 0};
  for (int64_t i = threadIdx.x; i < N; i += FB_TPB) {
    const float g = bits_to_gumbel(bits_at(k0, k1, tot, (uint64_t)j * N + i));
    best_take(b, __fadd_rn(g, lw[i]), (int32_t)i);
  }
  const int32_t bi = block_argmax<FB_TPB>(b, sm);
  if (threadIdx.x == 0) idx[j] = bi;
}

// xs_t[:, j] = x_t[:, idx_j]; DC = 0: the dimension d is a run-time argument
template <int DC>
__global__ void k_ffbsi_take(int64_t N, int64_t M, const float *__restrict__ x, const int32_t *__restrict__ idx,
                             float *__restrict__ out, int d) {
  const int D = DC ? DC : d;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx[j];
#pragma unroll
    for (int k = 0; k < D; ++k) out[k * M + j] = x[k * N + i];
  }
}

template <int D, bool RT = false>
LGT<D, RT> pack_lgt(const mgb_lg_transition *tr) {
  LGT<D, RT> p{};
  const int d = RT ? tr->d : D;
  for (int i = 0; i < d * d; ++i) {
    p.F[i] = tr->F[i];
    p.Pq[i] = tr->Pq[i];
  }
  p.cq = tr->cq;
  p.one = 1u;
  p.d_ = d;
  return p;
}

// the take kernel's compile-time dimension for policy TP (0: run-time)
template <class TP>
constexpr int take_dim() {
  return TP::kRT ? 0 : TP::DIM;
}

inline NLT pack_nlt(const mgb_nl1d_model *m, const float *tp, float tv) {
  NLT p;
  p.tsd = m->transition_sd;
  p.c = m->c;
  p.tp = tp;
  p.tv = tv;
  p.one = 1u;
  return p;
}

}  // namespace mgb
