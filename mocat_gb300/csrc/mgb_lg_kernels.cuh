// Fused bootstrap-filter kernels of the linear-Gaussian model (init, one
// particle per thread, two particles per thread); shared by the whole-filter
// driver and the adjoint's taped forward pass.
#pragma once
#include "mgb_lg.cuh"
#include "mgb_pf_common.cuh"

namespace mgb {

// initiate_particles: x_0 = C0 eps + m0, lw_0 = -potential(x_0, y_0)
template <int D, int DY, bool FUSED>
__global__ void __launch_bounds__(PF_TPB) k_lg_init(const __grid_constant__ LGP<D, DY> p, int64_t n,
                                                     const uint32_t *key, const float *y0, float *__restrict__ x,
                                                     float *__restrict__ lw, PFCtl ctl) {
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  const uint32_t k0 = key[0], k1 = key[1];
  __shared__ float y[DY];
  if (threadIdx.x < DY) y[threadIdx.x] = y0 ? y0[threadIdx.x] : 0.0f;
  __syncthreads();
  float l = -INFINITY;
  const bool active = i < n;
  if (active) {
    float e[D], xv[D];
    particle_normals<D>(k0, k1, n, i, e);
#pragma unroll
    for (int r = 0; r < D; ++r) {
      float v = __fmul_rn(p.C0[r * D], e[0]);
#pragma unroll
      for (int k = 1; k < D; ++k) v = __fmaf_rn(p.C0[r * D + k], e[k], v);
      xv[r] = __fadd_rn(v, p.m0[r]);
      x[r * n + i] = xv[r];
    }
    l = y0 ? -lg_potential<D, DY>(p, xv, y) : 0.0f;
    lw[i] = l;
  }
  if (FUSED) pf_reduce<PF_TPB>(l, active, ctl, 0);
}

// one bootstrap step; res_flag (nullable) decides resampled vs identity at run time.
// MUS > 0: also the score's proposal rows mu (lg_particle)
template <int D, int DY, bool FUSED, int MUS = 0>
__global__ void __launch_bounds__(PF_TPB) k_lg_step(const __grid_constant__ LGP<D, DY> p, int64_t n,
                                                     const uint32_t *key, const float *y_t,
                                                     const float *__restrict__ x_prev, const int32_t *anc,
                                                     const float *lw_prev, const int32_t *res_flag,
                                                     float *__restrict__ x_new, float *__restrict__ lw_new,
                                                     PFCtl ctl, int64_t t, float *__restrict__ mu = nullptr) {
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  const bool res = res_flag ? (*res_flag != 0) : (anc != nullptr);
  const uint32_t k0 = key[0], k1 = key[1];
  __shared__ float y[DY];
  if (threadIdx.x < DY) y[threadIdx.x] = y_t[threadIdx.x];
  __syncthreads();
  float l = -INFINITY;
  const bool active = i < n;
  if (active) {
    float e[D];
    particle_normals<D>(k0, k1, n, i, e);
    // run mode (res_flag set): lw_res = 0 after a resample (filtering.py:292);
    // standalone mode: lw_prev as given (NULL = 0)
    const float *lws = res_flag ? (res ? nullptr : lw_prev) : lw_prev;
    l = lg_particle_e<D, DY, false, MUS>(p, n, e, i, res, x_prev, anc, lws, y, x_new, lw_new, mu);
  }
  if (FUSED) pf_reduce<PF_TPB>(l, active, ctl, t);
}

// Two particles per thread, i and i + n/2 (n even).  In jax's split layout the
// key of particle i is (T(2i, 2i+n).x0, T(2i+1, 2i+1+n).x0) and the key of
// particle i + n/2 is the .x1 halves of the same two cipher calls, so the
// pair costs two key-split evaluations instead of four.
template <int D, int DY, bool FUSED, int MUS = 0>
__device__ __forceinline__ void lg_step2_body(const LGP<D, DY> &p, int64_t n, const uint32_t *key, const float *y_t,
                                              const float *__restrict__ x_prev, const int32_t *anc,
                                              const float *lw_prev, const int32_t *res_flag,
                                              float *__restrict__ x_new, float *__restrict__ lw_new,
                                              const PFCtl &ctl, int64_t t, float *__restrict__ mu = nullptr) {
  const int64_t h = n >> 1;
  const int64_t i = blockIdx.x * (int64_t)PF_TPB + threadIdx.x;
  const bool res = res_flag ? (*res_flag != 0) : (anc != nullptr);
  const float *lws = res_flag ? (res ? nullptr : lw_prev) : lw_prev;
  const uint32_t k0 = key[0], k1 = key[1];
  __shared__ float y[DY];
  if (threadIdx.x < DY) y[threadIdx.x] = y_t[threadIdx.x];
  __syncthreads();
  float m = -INFINITY, a1 = 0.0f, a2 = 0.0f;
  int nanf = 0;
  if (i < h) {
    uint32_t r0, r1, s0, s1;
    threefry2x32_m(k0, k1, (uint32_t)(2 * i), (uint32_t)(2 * i + n), p.one, r0, r1);
    threefry2x32_m(k0, k1, (uint32_t)(2 * i + 1), (uint32_t)(2 * i + 1 + n), p.one, s0, s1);
    // two-trip loop, not unrolled: one copy of the particle code (instruction cache)
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
      const float l = lg_particle<D, DY, false, MUS>(p, n, s ? r1 : r0, s ? s1 : s0, s ? i + h : i, res, x_prev,
                                                     anc, lws, y, x_new, lw_new, mu);
      online_acc(l, m, a1, a2, nanf);
    }
  }
  if (FUSED) pf_reduce_online<PF_TPB>(m, a1, a2, nanf, ctl, t);
}
template <int D, int DY, bool FUSED, int MUS = 0>
__global__ void __launch_bounds__(PF_TPB, 2) k_lg_step2(const __grid_constant__ LGP<D, DY> p, int64_t n,
                                                         const uint32_t *key, const float *y_t,
                                                         const float *__restrict__ x_prev, const int32_t *anc,
                                                         const float *lw_prev, const int32_t *res_flag,
                                                         float *__restrict__ x_new, float *__restrict__ lw_new,
                                                         PFCtl ctl, int64_t t, float *__restrict__ mu = nullptr) {
  lg_step2_body<D, DY, FUSED, MUS>(p, n, key, y_t, x_prev, anc, lw_prev, res_flag, x_new, lw_new, ctl, t, mu);
}

}  // namespace mgb
