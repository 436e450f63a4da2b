// Arithmetic of the one-dimensional non-linear benchmark model
// (mocat/src/ssm/scenarios/nonlinear1d.py:16-80), shared by the filter and the
// backward-simulation / stitching kernels.  Every operation is one float32
// rounding in the order the reference's expressions state it, so values equal
// the oracle's.
#pragma once
#include "mgb_internal.cuh"

namespace mgb {

// 8 cos(1.2 t): the float32 product 1.2f t, a double-precision cosine rounded
// to float32, an exact scaling by 8.  Called by one thread per block.
__device__ __forceinline__ float nl_drift(float t) {
  const float a = __fmul_rn(1.2f, t);
  return __fmul_rn(8.0f, __double2float_rn(cos((double)a)));
}

// _transition_mean: 0.5 x + 25 x / (1 + x^2) + drift, left to right (:41-46)
__device__ __forceinline__ float nl_mean(float x, float drift) {
  const float a = __fmul_rn(0.5f, x);
  const float b = __fdiv_rn(__fmul_rn(25.0f, x), __fadd_rn(1.0f, __fmul_rn(x, x)));
  return __fadd_rn(__fadd_rn(a, b), drift);
}

// gaussian_potential(diff / sd) with unit precision: 0.5 (diff / sd)^2 + c, c = log(2 pi) / 2
__device__ __forceinline__ float nl_gauss(float diff, float sd, float c) {
  const float z = __fdiv_rn(diff, sd);
  return __fadd_rn(__fmul_rn(0.5f, __fmul_rn(z, z)), c);
}

// likelihood_potential (:63-75): residual y - x^2 / 20
__device__ __forceinline__ float nl_lik_potential(float x, float y, float lsd, float c) {
  return nl_gauss(__fsub_rn(y, __fdiv_rn(__fmul_rn(x, x), 20.0f)), lsd, c);
}

struct NLP {
  float s0, tsd, lsd, c;
  uint32_t one;  // == 1, multiplier of the cipher's multiply-adds
};

inline NLP pack_nl(const mgb_nl1d_model *m) {
  NLP p;
  p.s0 = m->initial_sd;
  p.tsd = m->transition_sd;
  p.lsd = m->likelihood_sd;
  p.c = m->c;
  p.one = 1u;
  return p;
}

__device__ __forceinline__ float nl_potential(const NLP &p, float x, float y) {
  return nl_lik_potential(x, y, p.lsd, p.c);
}

// normal(key, (1,)) for the particle key (ka, kb)
__device__ __forceinline__ float nl_normal(uint32_t ka, uint32_t kb, uint32_t one) {
  uint32_t b[1];
  bits_vec<1>(ka, kb, b, one);
  return bits_to_normal(b[0]);
}

// the model as a particle policy of the persistent whole-filter kernel; aux is
// the step's drift 8 cos(1.2 t_prev)
struct NLModelP {
  static constexpr int kD = 1, kDY = 1;
  NLP p;
  __device__ __forceinline__ uint32_t one() const { return p.one; }
  __device__ __forceinline__ float init(int64_t, uint32_t ka, uint32_t kb, int64_t i, const float *y,
                                        float *__restrict__ x, float *__restrict__ lw) const {
    const float xv = __fmul_rn(nl_normal(ka, kb, p.one), p.s0);
    x[i] = xv;
    const float l = -nl_potential(p, xv, y[0]);
    lw[i] = l;
    return l;
  }
  __device__ __forceinline__ float step(int64_t, uint32_t ka, uint32_t kb, int64_t i, const float (&xs)[1],
                                        float lres, const float *y, float aux, float *__restrict__ x,
                                        float *__restrict__ lw) const {
    const float xn = __fadd_rn(nl_mean(xs[0], aux), __fmul_rn(nl_normal(ka, kb, p.one), p.tsd));
    x[i] = xn;
    const float l = __fsub_rn(lres, nl_potential(p, xn, y[0]));
    lw[i] = l;
    return l;
  }
};

}  // namespace mgb
