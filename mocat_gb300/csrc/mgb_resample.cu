// Standalone weight-normalisation / resampling / gather kernels and their C ABI.
// The particle-filter drivers reuse the same kernels with a `flag` pointer
// that skips the work on steps that do not resample.
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_kernels.cuh"
#include "mgb_systematic.cuh"

namespace mgb {

// ------------------------------------------------------------------ LSE / ESS
template <int TPB>
__global__ void __launch_bounds__(TPB) k_lse_ess(const float *__restrict__ lw, int64_t n, LsePartial *parts,
                                                  unsigned int *counter, LseOut *out, double *out4) {
  __shared__ float smf[TPB / 32];
  __shared__ double smd[TPB / 32];
  __shared__ bool last;
  // per-thread pass 1: local max / NaN
  float m = -INFINITY;
  bool nan = false;
  const int64_t stride = (int64_t)gridDim.x * TPB;
  for (int64_t i = blockIdx.x * (int64_t)TPB + threadIdx.x; i < n; i += stride) {
    const float v = lw[i];
    if (v != v) nan = true;
    else m = fmaxf(m, v);
  }
  const float mb = block_max<TPB>(m, smf);
  float s1 = 0.0f, s2 = 0.0f;
  if (mb > -INFINITY && mb < INFINITY) {
    for (int64_t i = blockIdx.x * (int64_t)TPB + threadIdx.x; i < n; i += stride) {
      const float v = lw[i];
      if (v == v) {
        const float e = expf(v - mb);
        s1 += e;
        s2 += e * e;
      }
    }
  }
  const float d1 = block_sum<TPB, float>(s1, smf);
  const float d2 = block_sum<TPB, float>(s2, smf);
  const int nn = __syncthreads_or(nan);
  if (threadIdx.x == 0) {
    parts[blockIdx.x] = LsePartial{mb, d1, d2, nn};
    last = last_block_arrival(counter);
  }
  __syncthreads();
  if (!last) return;
  const LseOut o = combine_lse<TPB>(parts, gridDim.x, smf, smd);
  if (threadIdx.x == 0) {
    *out = o;
    if (out4) {
      out4[0] = (double)o.M;
      out4[1] = o.lse;
      out4[2] = o.lse2;
      out4[3] = o.ess;
    }
    *counter = 0u;
  }
}

constexpr int LSE_TPB = 256;
inline unsigned lse_grid(int64_t n) { return grid_for(n, LSE_TPB, 4LL * kNumSMs); }

struct LseWs {
  LsePartial *parts;
  unsigned int *counter;
  LseOut *out;
};
inline LseWs carve_lse(Carver &c, int64_t n) {
  LseWs w;
  w.parts = c.take<LsePartial>(lse_grid(n));
  w.counter = c.take<unsigned int>(1);
  w.out = c.take<LseOut>(1);
  return w;
}

int launch_lse(const float *lw, int64_t n, const LseWs &w, double *out4, cudaStream_t s) {
  k_lse_ess<LSE_TPB><<<lse_grid(n), LSE_TPB, 0, s>>>(lw, n, w.parts, w.counter, w.out, out4);
  return launch_status();
}

// ------------------------------------------------------- resampling kernels
// (bodies in mgb_systematic.cuh)
__global__ void __launch_bounds__(SCAN_TPB) k_tile_sums(const float *__restrict__ lw, int64_t n, const float *Mptr,
                                                         const uint32_t *key, int has_m23, uint32_t m23_arg,
                                                         const int32_t *flag, ResampleCtl *ctl,
                                                         uint64_t *__restrict__ tile_pfx,
                                                         uint64_t *__restrict__ units) {
  tile_sums_body(lw, n, Mptr, key, has_m23, m23_arg, flag, ctl, tile_pfx, units);
}
__global__ void __launch_bounds__(SCAN_TPB) k_systematic(const float *__restrict__ lw, int64_t n, const float *Mptr,
                                                          const int32_t *flag, const ResampleCtl *ctl,
                                                          const uint64_t *__restrict__ tile_pfx,
                                                          const uint64_t *__restrict__ units,
                                                          int32_t *__restrict__ anc, int *err) {
  systematic_body(lw, n, Mptr, flag, ctl, tile_pfx, units, anc, err);
}

// generic decoupled-lookback scan producing an inclusive u64 array:
//   mode 0: fixed-point weights of lw (len n), mode 1: exponential spacings of key (len n + 1)
__global__ void __launch_bounds__(SCAN_TPB) k_scan_store(int mode, const float *__restrict__ lw, int64_t len,
                                                          int64_t n, const float *Mptr, const uint32_t *key,
                                                          const int32_t *flag, unsigned int *tile_counter,
                                                          int *degenerate, uint64_t *status,
                                                          uint64_t *__restrict__ out, int *err) {
  if (flag && *flag == 0) return;
  __shared__ uint32_t tile_s;
  if (threadIdx.x == 0) tile_s = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const uint32_t tile = tile_s;
  const int64_t i0 = (int64_t)tile * SCAN_TILE + (int64_t)threadIdx.x * SCAN_IPT;
  uint64_t v[SCAN_IPT];
  if (mode == 0) {
    const float M = *Mptr;
    const bool ok = M > -INFINITY && M < INFINITY;
    const float scale = __int_as_float((weight_shift(n) + 127) << 23);
    int bad = !ok;
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) {
      const float x = (i0 + j < len) ? lw[i0 + j] : -INFINITY;
      const bool good = x == x && x != INFINITY;
      bad |= !good;
      v[j] = (ok && good) ? quantise_weight(x, M, scale) : 0ull;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(degenerate, 1);
  } else {
    const float sc = __int_as_float((exp_shift(n) + 127) << 23);
    const uint32_t k0 = key[0], k1 = key[1];
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j)
      v[j] = (i0 + j < len) ? __float2ull_rz(__fmul_rn(bits_to_exponential(bits_at(k0, k1, (uint64_t)len, (uint64_t)(i0 + j))), sc))
                            : 0ull;
  }
  uint64_t texcl, ttot;
  tile_scan(v, tile, status, err, texcl, ttot);
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j)
    if (i0 + j < len) out[i0 + j] = v[j];
}

// merge-path search: a_k = #{i : C_i S_n <= S_k Q}
constexpr int MP_TPB = 256, MP_IPT = 8, MP_L = MP_TPB * MP_IPT;

__device__ __forceinline__ int64_t mp_split(int64_t d, const uint64_t *A, const uint64_t *B, int64_t na, int64_t nb,
                                            uint64_t den, uint64_t Q) {
  int64_t lo = d > nb ? d - nb : 0, hi = d < na ? d : na;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (mul_le(A[mid], den, B[d - 1 - mid], Q)) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(MP_TPB) k_merge_path(const uint64_t *__restrict__ C, const uint64_t *__restrict__ S,
                                                        int64_t n, const float *Mptr, const int32_t *flag,
                                                        const int *degenerate, int32_t *__restrict__ anc, int *err) {
  if (flag && *flag == 0) return;
  __shared__ uint64_t sa[MP_L], sb[MP_L];
  __shared__ int32_t so[MP_L];
  __shared__ int64_t sp[2];
  const uint64_t Q = C[n - 1], den = S[n];
  const float M = *Mptr;
  const int64_t d0 = (int64_t)blockIdx.x * MP_L;
  const int64_t d1 = d0 + MP_L < 2 * n ? d0 + MP_L : 2 * n;
  if (Q == 0 || den == 0 || !(M > -INFINITY && M < INFINITY) || *(volatile const int *)degenerate) {
    // degenerate weights: every ancestor is 0 (the categorical draw of the
    // reference returns index 0 when every logit is -inf / NaN)
    for (int64_t k = d0 / 2 + threadIdx.x; k < d1 / 2; k += MP_TPB) anc[k] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_err(err, EB_DEGENERATE);
    return;
  }
  if (threadIdx.x < 2) sp[threadIdx.x] = mp_split(threadIdx.x == 0 ? d0 : d1, C, S, n, n, den, Q);
  __syncthreads();
  const int64_t ia = sp[0], ib = sp[1];
  const int64_t ka = d0 - ia, kb = d1 - ib;
  const int na = (int)(ib - ia), nb = (int)(kb - ka);
  for (int j = threadIdx.x; j < na; j += MP_TPB) sa[j] = C[ia + j];
  for (int j = threadIdx.x; j < nb; j += MP_TPB) sb[j] = S[ka + j];
  __syncthreads();
  // this thread's sub-diagonal
  const int dd0 = threadIdx.x * MP_IPT;
  const int dlen = na + nb;
  if (dd0 < dlen) {
    int lo = dd0 > nb ? dd0 - nb : 0, hi = dd0 < na ? dd0 : na;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (mul_le(sa[mid], den, sb[dd0 - 1 - mid], Q)) lo = mid + 1;
      else hi = mid;
    }
    int ii = lo, kk = dd0 - lo;
    const int dd1 = dd0 + MP_IPT < dlen ? dd0 + MP_IPT : dlen;
    for (int s = dd0; s < dd1; ++s) {
      if (ii < na && (kk >= nb || mul_le(sa[ii], den, sb[kk], Q))) {
        ++ii;
      } else {
        so[kk] = (int32_t)(ia + ii);
        ++kk;
      }
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nb; j += MP_TPB) anc[ka + j] = so[j];
}

// mocat's categorical: a_k = argmax_i gumbel[k, i] + lw_i (first maximum; NaN ignored)
__global__ void __launch_bounds__(256) k_categorical(const float *__restrict__ lw, int64_t n, int64_t nout,
                                                      const uint32_t *key, const int32_t *flag,
                                                      int32_t *__restrict__ anc) {
  if (flag && *flag == 0) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * 256LL + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * 256) >> 5;
  const uint32_t k0 = key[0], k1 = key[1];
  const uint64_t tot = (uint64_t)n * (uint64_t)nout;
  for (int64_t k = warp; k < nout; k += nwarps) {
    float best = -INFINITY;
    int64_t bi = n;
    for (int64_t i = lane; i < n; i += 32) {
      const float g = bits_to_gumbel(bits_at(k0, k1, tot, (uint64_t)k * (uint64_t)n + (uint64_t)i));
      const float v = __fadd_rn(g, lw[i]);
      if (v > best) { best = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane == 0) anc[k] = (int32_t)(bi < n ? bi : 0);
  }
}

// the same draw for an even number of outputs: element (k, i) and (k + nout/2, i) of the
// (nout, n) Gumbel array are the two halves of one cipher call (counter k n + i and
// k n + i + n nout / 2), so one warp takes the row pair and spends one call per column
__global__ void __launch_bounds__(256) k_categorical_pairs(const float *__restrict__ lw, int64_t n, int64_t nout,
                                                            const uint32_t *key, const int32_t *flag,
                                                            uint32_t one, int32_t *__restrict__ anc) {
  if (flag && *flag == 0) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * 256LL + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * 256) >> 5;
  const uint32_t k0 = key[0], k1 = key[1];
  const int64_t half = nout >> 1;
  const uint64_t h = (uint64_t)n * (uint64_t)half;
  for (int64_t k = warp; k < half; k += nwarps) {
    float best0 = -INFINITY, best1 = -INFINITY;
    int64_t bi0 = n, bi1 = n;
    for (int64_t i = lane; i < n; i += 32) {
      const uint64_t c = (uint64_t)k * (uint64_t)n + (uint64_t)i;
      uint32_t r0, r1;
      threefry2x32_m(k0, k1, (uint32_t)c, (uint32_t)(c + h), one, r0, r1);
      const float l = lw[i];
      const float v0 = __fadd_rn(bits_to_gumbel(r0), l), v1 = __fadd_rn(bits_to_gumbel(r1), l);
      if (v0 > best0) { best0 = v0; bi0 = i; }
      if (v1 > best1) { best1 = v1; bi1 = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob0 = __shfl_xor_sync(0xffffffffu, best0, o), ob1 = __shfl_xor_sync(0xffffffffu, best1, o);
      const int64_t oi0 = __shfl_xor_sync(0xffffffffu, bi0, o), oi1 = __shfl_xor_sync(0xffffffffu, bi1, o);
      if (ob0 > best0 || (ob0 == best0 && oi0 < bi0)) { best0 = ob0; bi0 = oi0; }
      if (ob1 > best1 || (ob1 == best1 && oi1 < bi1)) { best1 = ob1; bi1 = oi1; }
    }
    if (lane == 0) {
      anc[k] = (int32_t)(bi0 < n ? bi0 : 0);
      anc[k + half] = (int32_t)(bi1 < n ? bi1 : 0);
    }
  }
}

// out[k, :] = x[anc[k], :]
__global__ void k_gather_rows_v4(const float4 *__restrict__ x, int64_t w4, const int32_t *__restrict__ anc,
                                 int64_t n_out, float4 *__restrict__ out) {
  const int64_t tot = n_out * w4;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < tot; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = p / w4, c = p - k * w4;
    out[p] = __ldg(&x[(int64_t)anc[k] * w4 + c]);
  }
}
__global__ void k_gather_rows(const float *__restrict__ x, int64_t w, const int32_t *__restrict__ anc, int64_t n_out,
                              float *__restrict__ out) {
  const int64_t tot = n_out * w;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < tot; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = p / w, c = p - k * w;
    out[p] = __ldg(&x[(int64_t)anc[k] * w + c]);
  }
}

// ----------------------------------------------------- host-side launchers

ResampleWs carve_resample(Carver &c, int64_t n, int scheme) {
  ResampleWs w;
  w.ctl = c.take<ResampleCtl>(1);
  const int64_t tiles = (n + 1 + SCAN_TILE - 1) / SCAN_TILE;
  w.status = c.take<uint64_t>(tiles);
  w.status2 = c.take<uint64_t>(2 * tiles + 2);
  w.ntiles = tiles;
  w.C = scheme == MGB_RESAMPLE_MULTINOMIAL ? c.take<uint64_t>(n) : nullptr;
  w.S = scheme == MGB_RESAMPLE_MULTINOMIAL ? c.take<uint64_t>(n + 1) : nullptr;
  return w;
}

// Zero the control block / tile status words (async; graph-capturable).
// status and the first ntiles words of status2 hold decoupled-lookback flags
// (the tile scan of either scheme, and the multinomial scan of the n + 1
// spacings, which has exactly ntiles tiles), so they must start at zero; the
// rest of status2 (the systematic fill units) is written before it is read.
int reset_resample(const ResampleWs &w, cudaStream_t s) {
  if (cudaMemsetAsync(w.ctl, 0, sizeof(ResampleCtl), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.status, 0, sizeof(uint64_t) * w.ntiles, s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(w.status2, 0, sizeof(uint64_t) * w.ntiles, s) != cudaSuccess) return ERR_CUDA;
  return OK;
}

int launch_resample(const float *lw, int64_t n, int scheme, const float *Mptr, const uint32_t *key, int has_m23,
                    uint32_t m23, const int32_t *flag, const ResampleWs &w, int32_t *anc, int *err, cudaStream_t s) {
  const unsigned tiles = (unsigned)((n + SCAN_TILE - 1) / SCAN_TILE);
  if (scheme == MGB_RESAMPLE_SYSTEMATIC) {
    // status holds the tile prefixes, status2 the fill units (<= 2 x tiles)
    k_tile_sums<<<tiles, SCAN_TPB, 0, s>>>(lw, n, Mptr, key, has_m23, m23, flag, w.ctl, w.status, w.status2);
    k_systematic<<<2 * tiles, SCAN_TPB, 0, s>>>(lw, n, Mptr, flag, w.ctl, w.status, w.status2, anc, err);
  } else if (scheme == MGB_RESAMPLE_MULTINOMIAL) {
    const unsigned tiles_e = (unsigned)((n + 1 + SCAN_TILE - 1) / SCAN_TILE);
    k_scan_store<<<tiles, SCAN_TPB, 0, s>>>(0, lw, n, n, Mptr, key, flag, &w.ctl->tile_counter,
                                            &w.ctl->degenerate, w.status, w.C, err);
    k_scan_store<<<tiles_e, SCAN_TPB, 0, s>>>(1, lw, n + 1, n, Mptr, key, flag, &w.ctl->tile_counter2,
                                              &w.ctl->degenerate, w.status2, w.S, err);
    const unsigned g = (unsigned)((2 * n + MP_L - 1) / MP_L);
    k_merge_path<<<g, MP_TPB, 0, s>>>(w.C, w.S, n, Mptr, flag, &w.ctl->degenerate, anc, err);
  } else if (scheme == MGB_RESAMPLE_CATEGORICAL) {
    if (n % 2 == 0)
      k_categorical_pairs<<<grid_for(n * 16, 256, 8LL * kNumSMs), 256, 0, s>>>(lw, n, n, key, flag, 1u, anc);
    else
      k_categorical<<<grid_for(n * 32, 256, 8LL * kNumSMs), 256, 0, s>>>(lw, n, n, key, flag, anc);
  } else {
    return ERR_BAD_ARG;
  }
  return launch_status();
}

}  // namespace mgb

using namespace mgb;

extern "C" {

const char *mgb_status_string(int st) {
  switch (st) {
    case MGB_OK: return "ok";
    case MGB_ERR_BAD_ARG: return "bad argument";
    case MGB_ERR_UNSUPPORTED: return "unsupported configuration";
    case MGB_ERR_LAUNCH: return "kernel launch failed";
    case MGB_ERR_WORKSPACE: return "workspace too small";
    case MGB_ERR_DEVICE_TIMEOUT: return "a bounded device wait ran out";
    case MGB_ERR_NONFINITE_WEIGHTS: return "degenerate (zero / non-finite) weights";
    case MGB_ERR_CUDA: return "CUDA runtime error";
    default: return "unknown status";
  }
}

int mgb_version(void) { return 100; }

size_t mgb_lse_ess_workspace(int64_t n) {
  Carver c(nullptr);
  carve_lse(c, n);
  return c.bytes();
}

int mgb_lse_ess(const float *lw, int64_t n, double *out4, void *ws, size_t ws_bytes, void *stream) {
  if (n < 1 || !lw || !out4 || !ws) return ERR_BAD_ARG;
  if (ws_bytes < mgb_lse_ess_workspace(n)) return ERR_WORKSPACE;
  Carver c(ws);
  LseWs w = carve_lse(c, n);
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
  return launch_lse(lw, n, w, out4, s);
}

size_t mgb_resample_workspace(int64_t n, int scheme) {
  Carver c(nullptr);
  carve_lse(c, n);
  carve_resample(c, n, scheme);
  return c.bytes();
}

static int resample_common(const float *lw, int64_t n, int scheme, const uint32_t *key, int has_m23, uint32_t m23,
                           int32_t *anc, void *ws, size_t ws_bytes, int32_t *err, void *stream) {
  if (n < 1 || n > 0x7FFFFFFFll || !lw || !anc || !ws || (!has_m23 && !key)) return ERR_BAD_ARG;
  if (scheme < 0 || scheme > 2) return ERR_BAD_ARG;
  if (scheme == MGB_RESAMPLE_CATEGORICAL && n > 46340) return ERR_UNSUPPORTED;  // n^2 counters < 2^31
  if (ws_bytes < mgb_resample_workspace(n, scheme)) return ERR_WORKSPACE;
  Carver c(ws);
  LseWs lws = carve_lse(c, n);
  ResampleWs rws = carve_resample(c, n, scheme);
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(lws.counter, 0, sizeof(unsigned int), s) != cudaSuccess) return ERR_CUDA;
  int st = reset_resample(rws, s);
  if (st) return st;
  st = launch_lse(lw, n, lws, nullptr, s);
  if (st) return st;
  return launch_resample(lw, n, scheme, &lws.out->M, key, has_m23, m23, nullptr, rws, anc, (int *)err, s);
}

int mgb_resample(const float *lw, int64_t n, int scheme, const uint32_t *key, int32_t *anc, void *ws, size_t ws_bytes,
                 int32_t *err, void *stream) {
  return resample_common(lw, n, scheme, key, 0, 0u, anc, ws, ws_bytes, err, stream);
}

int mgb_resample_systematic_u(const float *lw, int64_t n, uint32_t m23, int32_t *anc, void *ws, size_t ws_bytes,
                              int32_t *err, void *stream) {
  if (m23 >= (1u << 23)) return ERR_BAD_ARG;
  return resample_common(lw, n, MGB_RESAMPLE_SYSTEMATIC, nullptr, 1, m23, anc, ws, ws_bytes, err, stream);
}

int mgb_gather_rows(const float *x, int64_t width, const int32_t *anc, int64_t n_out, float *out, void *stream) {
  if (width < 1 || n_out < 0 || (n_out > 0 && (!x || !anc || !out))) return ERR_BAD_ARG;
  if (n_out == 0) return OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (width % 4 == 0 && (((uintptr_t)x | (uintptr_t)out) & 15) == 0) {
    k_gather_rows_v4<<<grid_for(n_out * width / 4, 256), 256, 0, s>>>((const float4 *)x, width / 4, anc, n_out,
                                                                       (float4 *)out);
  } else {
    k_gather_rows<<<grid_for(n_out * width, 256), 256, 0, s>>>(x, width, anc, n_out, out);
  }
  return launch_status();
}

}  // extern "C"
