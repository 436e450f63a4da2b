// jax.random draws on the GPU (threefry2x32, non-partitionable layout) and the
// library's float maths, exposed through the C ABI for the random module and
// for bit-level parity tests.
#include "mgb_internal.cuh"

namespace mgb {

enum DrawKind { DRAW_BITS = 0, DRAW_UNIFORM = 1, DRAW_NORMAL = 2, DRAW_EXPONENTIAL = 3, DRAW_GUMBEL = 4 };

// one thread per counter pair (p, p + h): both outputs are used, so every
// cipher evaluation is done exactly once
template <int KIND>
__global__ void k_draw(const uint32_t *__restrict__ key, int64_t n, void *__restrict__ out) {
  const uint32_t k0 = key[0], k1 = key[1];
  const int64_t h = (n + 1) >> 1;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < h; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c1 = j + h;
    uint32_t r0, r1;
    threefry2x32(k0, k1, (uint32_t)j, c1 < n ? (uint32_t)c1 : 0u, r0, r1);
    if (KIND == DRAW_BITS) {
      uint32_t *o = (uint32_t *)out;
      o[j] = r0;
      if (c1 < n) o[c1] = r1;
    } else {
      float *o = (float *)out;
      float v0, v1;
      if (KIND == DRAW_UNIFORM) { v0 = bits_to_unit(r0); v1 = bits_to_unit(r1); }
      if (KIND == DRAW_NORMAL) { v0 = bits_to_normal(r0); v1 = bits_to_normal(r1); }
      if (KIND == DRAW_EXPONENTIAL) { v0 = bits_to_exponential(r0); v1 = bits_to_exponential(r1); }
      if (KIND == DRAW_GUMBEL) { v0 = bits_to_gumbel(r0); v1 = bits_to_gumbel(r1); }
      o[j] = v0;
      if (c1 < n) o[c1] = v1;
    }
  }
}

__global__ void k_split(const uint32_t *__restrict__ key, int64_t num, uint32_t *__restrict__ out) {
  const uint32_t k0 = key[0], k1 = key[1];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < num; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t a, b;
    split_at(k0, k1, (uint64_t)num, (uint64_t)i, a, b);
    out[2 * i] = a;
    out[2 * i + 1] = b;
  }
}

__global__ void k_normal_keys(const uint32_t *__restrict__ keys, int64_t nkeys, int64_t d, float *__restrict__ out) {
  const int64_t tot = nkeys * d;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < tot; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = p / d, j = p - i * d;
    out[p] = bits_to_normal(bits_at(keys[2 * i], keys[2 * i + 1], (uint64_t)d, (uint64_t)j));
  }
}

__global__ void k_math(int op, const float *__restrict__ x, int64_t n, float *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = x[i];
    out[i] = op == 0 ? logf_(v) : (op == 1 ? expf_(v) : erfinv_(v));
  }
}

template <int KIND>
static int draw(const uint32_t *key, int64_t n, void *out, void *stream) {
  if (n < 0 || (n > 0 && (!key || !out)) || n > (int64_t)0xFFFFFFFFll) return ERR_BAD_ARG;
  if (n == 0) return OK;
  const int64_t h = (n + 1) >> 1;
  k_draw<KIND><<<grid_for(h, 256), 256, 0, (cudaStream_t)stream>>>(key, n, out);
  return launch_status();
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_random_bits(const uint32_t *key, int64_t n, uint32_t *out, void *s) { return draw<DRAW_BITS>(key, n, out, s); }
int mgb_uniform(const uint32_t *key, int64_t n, float *out, void *s) { return draw<DRAW_UNIFORM>(key, n, out, s); }
int mgb_normal(const uint32_t *key, int64_t n, float *out, void *s) { return draw<DRAW_NORMAL>(key, n, out, s); }
int mgb_exponential(const uint32_t *key, int64_t n, float *out, void *s) {
  return draw<DRAW_EXPONENTIAL>(key, n, out, s);
}
int mgb_gumbel(const uint32_t *key, int64_t n, float *out, void *s) { return draw<DRAW_GUMBEL>(key, n, out, s); }

int mgb_split(const uint32_t *key, int64_t num, uint32_t *out, void *s) {
  if (num < 0 || (num > 0 && (!key || !out)) || num > (int64_t)0x7FFFFFFFll) return ERR_BAD_ARG;
  if (num == 0) return OK;
  k_split<<<grid_for(num, 256), 256, 0, (cudaStream_t)s>>>(key, num, out);
  return launch_status();
}

int mgb_normal_keys(const uint32_t *keys, int64_t nkeys, int64_t d, float *out, void *s) {
  if (nkeys < 0 || d < 1 || (nkeys > 0 && (!keys || !out))) return ERR_BAD_ARG;
  if (nkeys == 0) return OK;
  k_normal_keys<<<grid_for(nkeys * d, 256), 256, 0, (cudaStream_t)s>>>(keys, nkeys, d, out);
  return launch_status();
}

int mgb_math_eval(int op, const float *x, int64_t n, float *out, void *s) {
  if (op < 0 || op > 2 || n < 0 || (n > 0 && (!x || !out))) return ERR_BAD_ARG;
  if (n == 0) return OK;
  k_math<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>(op, x, n, out);
  return launch_status();
}

}  // extern "C"
