// Arithmetic of the stochastic-volatility model with dim = 1
// (mocat/src/ssm/scenarios/stochastic_volatility.py:15-108), shared by the
// batched filters and the single-series filter:
//   initial_sample        x_0 = normal(key, (1,)) c0 + m0                       (:71-76)
//   transition_sample     x_t = phi x_{t-1} + normal(key, (1,)) bsig,
//                         bsig = transition_covariance_sqrt sqrt(t_new - t_prev)  (:87-94)
//   likelihood_potential  with s = r / exp(x/2): 0.5 y^2 s^2 + 0.5 (log 2 pi - log s^2)
//                         = (0.5 y^2 r^2) exp(-x) + (0.5 x + cB)                 (:96-102)
#pragma once
#include "mgb_internal.cuh"

namespace mgb {

struct SVParams {
  float phi, bsig, r2, cB, c0, m0;
  uint32_t one;  // == 1, multiplier of the cipher's multiply-adds
};

inline SVParams pack_sv(const mgb_sv_model *m) {
  return SVParams{m->phi, m->bsig, m->r2, m->cB, m->c0, m->m0, 1u};
}

__device__ __forceinline__ float sv_potential(const SVParams &p, float x, float y) {
  const float a = __fmul_rn(__fmul_rn(0.5f, __fmul_rn(y, y)), p.r2);
  return __fmaf_rn(a, expf_(-x), __fmaf_rn(0.5f, x, p.cB));
}

// normal(key, (1,)) for the particle key (ka, kb)
__device__ __forceinline__ float sv_normal(uint32_t ka, uint32_t kb, uint32_t one) {
  uint32_t b[1];
  bits_vec<1>(ka, kb, b, one);
  return bits_to_normal(b[0]);
}

__device__ __forceinline__ float sv_init_x(const SVParams &p, float e) { return __fadd_rn(__fmul_rn(e, p.c0), p.m0); }

__device__ __forceinline__ float sv_next_x(const SVParams &p, float xs, float e, float bsig) {
  return __fmaf_rn(xs, p.phi, __fmul_rn(e, bsig));
}

// the model as a particle policy of the persistent whole-filter kernel; aux is
// the step's bsig (transition_covariance_sqrt sqrt(t_t - t_{t-1}))
struct SVModelP {
  static constexpr int kD = 1, kDY = 1;
  SVParams p;
  __device__ __forceinline__ uint32_t one() const { return p.one; }
  __device__ __forceinline__ float init(int64_t, uint32_t ka, uint32_t kb, int64_t i, const float *y,
                                        float *__restrict__ x, float *__restrict__ lw) const {
    const float xv = sv_init_x(p, sv_normal(ka, kb, p.one));
    x[i] = xv;
    const float l = -sv_potential(p, xv, y[0]);
    lw[i] = l;
    return l;
  }
  __device__ __forceinline__ float step(int64_t, uint32_t ka, uint32_t kb, int64_t i, const float (&xs)[1],
                                        float lres, const float *y, float aux, float *__restrict__ x,
                                        float *__restrict__ lw) const {
    const float xn = sv_next_x(p, xs[0], sv_normal(ka, kb, p.one), aux);
    x[i] = xn;
    const float l = __fsub_rn(lres, sv_potential(p, xn, y[0]));
    lw[i] = l;
    return l;
  }
};

}  // namespace mgb
