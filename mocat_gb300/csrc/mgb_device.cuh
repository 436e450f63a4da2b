// Device building blocks shared by every kernel of libmocatgb:
//   * jax.random restatement on the GPU: threefry2x32-20 (Random123, Salmon et
//     al. SC'11) with jax's non-partitionable counter layout for split /
//     random_bits / uniform / normal / exponential / gumbel
//     (call sites in the reference: mocat/src/ssm/filtering.py:181,199,294;
//     mocat/src/ssm/linear_gaussian/linear_gaussian.py:51,94;
//     mocat/src/transport/smc.py:65,82);
//   * float maths written from textbook methods with explicit IEEE-rounded
//     intrinsics, so every value is reproducible on any IEEE host:
//       logf   -- reduction to [sqrt(1/2), sqrt(2)) + 2 atanh(s) series;
//       expf   -- Cody-Waite reduction by ln 2 + degree-7 Taylor polynomial;
//       erfinv -- M. Giles, "Approximating the erfinv function" (2011),
//                 single-precision branch;
//   * block reductions and status codes.
// Functions marked __host__ __device__ also run in the host-side driver.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define MGB_HD __host__ __device__ __forceinline__

namespace mgb {

// ------------------------------------------------------------------ status
enum Status : int {
  OK = 0,
  ERR_BAD_ARG = 1,
  ERR_UNSUPPORTED = 2,
  ERR_LAUNCH = 3,
  ERR_WORKSPACE = 4,
  ERR_DEVICE_TIMEOUT = 5,
  ERR_NONFINITE_WEIGHTS = 6,
  ERR_CUDA = 7,
};
// bits of the device-side error word
enum ErrBits : int { EB_TIMEOUT = 1, EB_DEGENERATE = 2 };

// ------------------------------------------------------------ threefry2x32
MGB_HD uint32_t rotl32(uint32_t v, int r) {
#ifdef __CUDA_ARCH__
  return __funnelshift_l(v, v, r);
#else
  return (v << r) | (v >> (32 - r));
#endif
}

MGB_HD void threefry2x32(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t &r0, uint32_t &r1) {
  const uint32_t k2 = k0 ^ k1 ^ 0x1BD11BDAu;
  uint32_t x0 = c0 + k0, x1 = c1 + k1;
#define MGB_TF_ROUND(R) { x0 += x1; x1 = rotl32(x1, R); x1 ^= x0; }
#define MGB_TF_G0 MGB_TF_ROUND(13) MGB_TF_ROUND(15) MGB_TF_ROUND(26) MGB_TF_ROUND(6)
#define MGB_TF_G1 MGB_TF_ROUND(17) MGB_TF_ROUND(29) MGB_TF_ROUND(16) MGB_TF_ROUND(24)
  MGB_TF_G0 x0 += k1; x1 += k2 + 1u;
  MGB_TF_G1 x0 += k2; x1 += k0 + 2u;
  MGB_TF_G0 x0 += k0; x1 += k1 + 3u;
  MGB_TF_G1 x0 += k1; x1 += k2 + 4u;
  MGB_TF_G0 x0 += k2; x1 += k0 + 5u;
#undef MGB_TF_G1
#undef MGB_TF_G0
#undef MGB_TF_ROUND
  r0 = x0;
  r1 = x1;
}

// Device variant with the 32-bit additions issued as multiply-adds by a
// runtime `one` (== 1, read from kernel parameters so it cannot be folded):
// integer add / xor / funnel-shift all compete for the integer ALU pipe, while
// IMAD issues to the FMA pipe.  Same values as threefry2x32.
__device__ __forceinline__ uint32_t madd(uint32_t a, uint32_t one, uint32_t b) {
  uint32_t r;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(one), "r"(b));
  return r;
}
__device__ __forceinline__ void threefry2x32_m(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t one,
                                               uint32_t &r0, uint32_t &r1) {
  const uint32_t k2 = k0 ^ k1 ^ 0x1BD11BDAu;
  uint32_t x0 = madd(c0, one, k0), x1 = madd(c1, one, k1);
#define MGB_TFM_ROUND(R) { x0 = madd(x1, one, x0); x1 = rotl32(x1, R); x1 ^= x0; }
#define MGB_TFM_G0 MGB_TFM_ROUND(13) MGB_TFM_ROUND(15) MGB_TFM_ROUND(26) MGB_TFM_ROUND(6)
#define MGB_TFM_G1 MGB_TFM_ROUND(17) MGB_TFM_ROUND(29) MGB_TFM_ROUND(16) MGB_TFM_ROUND(24)
  MGB_TFM_G0 x0 = madd(k1, one, x0); x1 = madd(k2 + 1u, one, x1);
  MGB_TFM_G1 x0 = madd(k2, one, x0); x1 = madd(k0 + 2u, one, x1);
  MGB_TFM_G0 x0 = madd(k0, one, x0); x1 = madd(k1 + 3u, one, x1);
  MGB_TFM_G1 x0 = madd(k1, one, x0); x1 = madd(k2 + 4u, one, x1);
  MGB_TFM_G0 x0 = madd(k2, one, x0); x1 = madd(k0 + 5u, one, x1);
#undef MGB_TFM_G1
#undef MGB_TFM_G0
#undef MGB_TFM_ROUND
  r0 = x0;
  r1 = x1;
}

// element p of threefry_2x32(key, iota(n)) (count padded to even length with a
// zero; outputs concatenated [first halves, second halves] and trimmed)
MGB_HD uint32_t bits_at(uint32_t k0, uint32_t k1, uint64_t n, uint64_t p) {
  const uint64_t h = (n + 1) >> 1;
  uint32_t r0, r1;
  if (p < h) {
    const uint64_t c1 = p + h;
    threefry2x32(k0, k1, (uint32_t)p, c1 < n ? (uint32_t)c1 : 0u, r0, r1);
    return r0;
  }
  threefry2x32(k0, k1, (uint32_t)(p - h), (uint32_t)p, r0, r1);
  return r1;
}

// split(key, num)[i]
MGB_HD void split_at(uint32_t k0, uint32_t k1, uint64_t num, uint64_t i, uint32_t &o0, uint32_t &o1) {
  o0 = bits_at(k0, k1, 2 * num, 2 * i);
  o1 = bits_at(k0, k1, 2 * num, 2 * i + 1);
}

// both sub-keys of split(key, 2) from the two cipher calls of random_bits(key, (4,)): call
// (0, 2) gives words 0 and 2, call (1, 3) words 1 and 3; sub-key j is words 2j, 2j + 1
MGB_HD void split2(uint32_t k0, uint32_t k1, uint32_t &a0, uint32_t &a1, uint32_t &b0, uint32_t &b1) {
  uint32_t x0, x1, y0, y1;
  threefry2x32(k0, k1, 0u, 2u, x0, x1);
  threefry2x32(k0, k1, 1u, 3u, y0, y1);
  a0 = x0;
  a1 = y0;
  b0 = x1;
  b1 = y1;
}

// the four sub-keys of split(key, 4) from the four cipher calls of random_bits(key, (8,)):
// call (q, q + 4) gives words q and q + 4; o[2j], o[2j + 1] = sub-key j
MGB_HD void split4(uint32_t k0, uint32_t k1, uint32_t (&o)[8]) {
  for (int q = 0; q < 4; ++q) threefry2x32(k0, k1, (uint32_t)q, (uint32_t)(q + 4), o[q], o[q + 4]);
}

// random_bits(key, (D,)) for a compile-time D: ceil(D/2) cipher calls
template <int D>
__device__ __forceinline__ void bits_vec(uint32_t k0, uint32_t k1, uint32_t (&b)[D], uint32_t one = 1u) {
  constexpr int H = (D + 1) / 2;
#pragma unroll
  for (int j = 0; j < H; ++j) {
    uint32_t r0, r1;
    threefry2x32_m(k0, k1, (uint32_t)j, (j + H < D) ? (uint32_t)(j + H) : 0u, one, r0, r1);
    b[j] = r0;
    if (j + H < D) b[j + H] = r1;
  }
}

// ------------------------------------------------------------- float maths
__device__ __forceinline__ float asf(uint32_t u) { return __uint_as_float(u); }
__device__ __forceinline__ uint32_t asu(float f) { return __float_as_uint(f); }

// natural log of a positive normal float
__device__ __forceinline__ float logf_(float x) {
  // x = 2^e m with m in [sqrt(1/2), sqrt(2)) split off in integer arithmetic: subtracting the
  // bits of the lower bound 0x3f3504f4 leaves e in the high bits and the mantissa offset in
  // the low 23 (the same (e, m) as taking m = 1.mantissa and halving it when above sqrt(2),
  // for every positive normal float)
  const uint32_t t = asu(x) - 0x3f3504f4u;
  const int e = (int)t >> 23;
  const float m = asf((t & 0x007fffffu) + 0x3f3504f4u);
  // log(1 + f) = f - f^2/2 + f^3 q(f), f = m - 1 (exact) in [sqrt(1/2) - 1, sqrt(2) - 1];
  // q: degree-7 weighted least-squares fit (no division on the path)
  const float f = __fsub_rn(m, 1.0f);
  const float f2 = __fmul_rn(f, f);
  float q = __fmaf_rn(f, -0x1.38b582p-4f, 0x1.055b72p-3f);
  q = __fmaf_rn(f, q, -0x1.0d8544p-3f);
  q = __fmaf_rn(f, q, 0x1.22da1cp-3f);
  q = __fmaf_rn(f, q, -0x1.547244p-3f);
  q = __fmaf_rn(f, q, 0x1.99a008p-3f);
  q = __fmaf_rn(f, q, -0x1.000226p-2f);
  q = __fmaf_rn(f, q, 0x1.555554p-2f);
  const float lm = __fadd_rn(f, __fmaf_rn(__fmul_rn(f2, f), q, __fmul_rn(-0.5f, f2)));
  const float ef = (float)e;
  return __fmaf_rn(ef, 0x1.63p-1f, __fmaf_rn(ef, -0x1.bd0106p-13f, lm));
}

// exp: 0 below -104, +inf above 88.5, NaN passes through
__device__ __forceinline__ float expf_(float x) {
  if (x != x) return x;
  if (x < -104.0f) return 0.0f;
  if (x > 88.5f) return __int_as_float(0x7f800000);
  const float kf = rintf(__fmul_rn(x, 0x1.715476p+0f));
  float r = __fmaf_rn(-kf, 0x1.63p-1f, x);
  r = __fmaf_rn(-kf, -0x1.bd0106p-13f, r);
  float p = __fmaf_rn(r, 0x1.a01a02p-13f, 0x1.6c16c2p-10f);
  p = __fmaf_rn(r, p, 0x1.111112p-7f);
  p = __fmaf_rn(r, p, 0x1.555556p-5f);
  p = __fmaf_rn(r, p, 0x1.555556p-3f);
  p = __fmaf_rn(r, p, 0.5f);
  p = __fmaf_rn(r, p, 1.0f);
  p = __fmaf_rn(r, p, 1.0f);
  const int k = (int)kf;
  if (k < -126) return __fmul_rn(__fmul_rn(p, asf((uint32_t)(k + 64 + 127) << 23)), 0x1p-64f);
  if (k > 127) return __fmul_rn(__fmul_rn(p, 2.0f), asf((uint32_t)(k - 1 + 127) << 23));
  return __fmul_rn(p, asf((uint32_t)(k + 127) << 23));
}

// Giles (2011) erfinv, single precision
__device__ __forceinline__ float erfinv_(float x) {
  float w = -logf_(__fmaf_rn(-x, x, 1.0f));
  float p;
  if (w < 5.0f) {
    w = __fsub_rn(w, 2.5f);
    p = 2.81022636e-08f;
    p = __fmaf_rn(p, w, 3.43273939e-07f);
    p = __fmaf_rn(p, w, -3.5233877e-06f);
    p = __fmaf_rn(p, w, -4.39150654e-06f);
    p = __fmaf_rn(p, w, 0.00021858087f);
    p = __fmaf_rn(p, w, -0.00125372503f);
    p = __fmaf_rn(p, w, -0.00417768164f);
    p = __fmaf_rn(p, w, 0.246640727f);
    p = __fmaf_rn(p, w, 1.50140941f);
  } else {
    w = __fsub_rn(__fsqrt_rn(w), 3.0f);
    p = -0.000200214257f;
    p = __fmaf_rn(p, w, 0.000100950558f);
    p = __fmaf_rn(p, w, 0.00134934322f);
    p = __fmaf_rn(p, w, -0.00367342844f);
    p = __fmaf_rn(p, w, 0.00573950773f);
    p = __fmaf_rn(p, w, -0.0076224613f);
    p = __fmaf_rn(p, w, 0.00943887047f);
    p = __fmaf_rn(p, w, 1.00167406f);
    p = __fmaf_rn(p, w, 2.83297682f);
  }
  return __fmul_rn(p, x);
}

__device__ __forceinline__ float bits_to_unit(uint32_t b) { return __fsub_rn(asf((b >> 9) | 0x3f800000u), 1.0f); }

// jax.random.normal from raw bits: u = max(lo, 2 f + lo), sqrt(2) erfinv(u).
// 2 f is exact, so one fused rounding of 2 f + lo equals jax's two-step
// rounding, and u >= lo always (f >= 0), so the max is the identity.
__device__ __forceinline__ float bits_to_normal(uint32_t b) {
  const float lo = -0x1.fffffep-1f;
  const float u = __fmaf_rn(bits_to_unit(b), 2.0f, lo);
  return __fmul_rn(0x1.6a09e6p+0f, erfinv_(u));
}

// jax.random.exponential: -log1p(-u) = -log(1 - u), 1 - u exact
__device__ __forceinline__ float bits_to_exponential(uint32_t b) { return -logf_(__fsub_rn(1.0f, bits_to_unit(b))); }

// jax.random.gumbel with minval = tiny
__device__ __forceinline__ float bits_to_gumbel(uint32_t b) {
  const float tiny = 0x1p-126f;
  const float u = fmaxf(__fadd_rn(bits_to_unit(b), tiny), tiny);
  return -logf_(-logf_(u));
}

// ---------------------------------------------------------- fixed point
MGB_HD int ceil_log2_u64(uint64_t n) {
  int b = 0;
  while (b < 63 && ((uint64_t)1 << b) < n) ++b;
  return b;
}
// weights exp(lw - max) in [0, 1] are quantised with 2^weight_shift(n): total < 2^62
MGB_HD int weight_shift(int64_t n) { return 61 - ceil_log2_u64((uint64_t)n); }
// exponential spacings (< 16) quantised with 2^exp_shift(n) over n + 1 draws: total < 2^60
MGB_HD int exp_shift(int64_t n) { return 56 - ceil_log2_u64((uint64_t)n + 1); }

// trunc(expf(lw - M) * 2^S) from the float's bits (integer ops only; equals
// __float2ull_rz of the exactly scaled value).  `scale` is 2^S.
__device__ __forceinline__ uint64_t quantise_weight(float lw, float M, float scale) {
  const uint32_t b = __float_as_uint(expf_(__fsub_rn(lw, M)));
  const int ex = (int)((b >> 23) & 0xffu);
  if (ex == 0 || ex == 255 || (b >> 31)) return 0ull;  // zero / subnormal, NaN / inf, negative
  const int S = (int)((__float_as_uint(scale) >> 23) & 0xffu) - 127;
  const uint64_t mant = (uint64_t)((b & 0x007fffffu) | 0x00800000u);
  const int sh = ex - 150 + S;
  return sh >= 0 ? (mant << sh) : (sh > -64 ? (mant >> -sh) : 0ull);
}

// 128-bit product comparison a*b <= c*d (all < 2^64)
__device__ __forceinline__ bool mul_le(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
  const uint64_t h1 = __umul64hi(a, b), l1 = a * b;
  const uint64_t h2 = __umul64hi(c, d), l2 = c * d;
  return h1 < h2 || (h1 == h2 && l1 <= l2);
}

// Arrival of a block at a "last block finishes" counter, by thread 0 after the
// block's results are stored: the GPU-scope acq_rel add publishes them (release) and,
// in the last block to arrive, makes every other block's visible (acquire; the block
// barrier that follows passes them on to its other threads).  True in the last block.
__device__ __forceinline__ bool last_block_arrival(unsigned int *counter) {
  unsigned int prev;
  asm volatile("atom.acq_rel.gpu.add.u32 %0, [%1], 1;" : "=r"(prev) : "l"(counter) : "memory");
  return prev == gridDim.x - 1;
}

// ---------------------------------------------------------- reductions
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_or(int v) { return __any_sync(0xffffffffu, v); }

// block-wide max of one value per thread (all threads get the result)
template <int TPB>
__device__ __forceinline__ float block_max(float v, float *sm /* >= TPB/32 */) {
  v = warp_max(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sm[w] = v;
  __syncthreads();
  float r = sm[0];
#pragma unroll
  for (int i = 1; i < TPB / 32; ++i) r = fmaxf(r, sm[i]);
  __syncthreads();
  return r;
}
template <int TPB, class T>
__device__ __forceinline__ T block_sum(T v, T *sm /* >= TPB/32 */) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sm[w] = v;
  __syncthreads();
  T r = sm[0];
#pragma unroll
  for (int i = 1; i < TPB / 32; ++i) r += sm[i];
  __syncthreads();
  return r;
}

// record an error bit in a device-side error word (never traps)
__device__ __forceinline__ void raise_err(int *err, int bit) {
  if (err) atomicOr(err, bit);
}

}  // namespace mgb
