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

}  // namespace mgb
