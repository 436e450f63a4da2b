// Weight normalisation and resampling building blocks (device side), shared
// by the standalone C-ABI entry points and the particle-filter drivers.
//
//  * LSE / ESS: each block reduces max and sum exp(lw - block max) (and of
//    its square) into a partial; the last block to finish combines the
//    partials in float64 (metrics.py:69-78, max-shifted logsumexp with shift 0
//    when the max is not finite).
//  * Fixed-point weights q_i = trunc(exp(lw_i - M) 2^S), S = 61 - ceil(log2 n),
//    so every prefix sum is an exact integer below 2^62 and ancestors do not
//    depend on the order of summation.
//  * Decoupled-lookback prefix scan over 2048-item tiles: a tile publishes
//    (flag | value) in one 64-bit word (flag 1 = tile aggregate, 2 = inclusive
//    prefix); its first warp sums predecessors' words until it meets an
//    inclusive prefix.  Waits are bounded: on expiry the kernel raises
//    EB_TIMEOUT and continues.
//  * Systematic: thresholds (k + u) n^-1 Q form an arithmetic progression, so
//    particle i's offspring are the k in [K(C_{i-1}), K(C_i)) with
//    K(X) = #{k : (k 2^23 + m) Q < X n 2^23}; each tile fills its output range
//    cooperatively (binary search over the tile's K values in shared memory).
//  * Multinomial: sorted uniforms S_k / S_n from n+1 exponential spacings
//    (exact integer scan); ancestors by a merge-path merge of the weight
//    prefix C with S (A_i precedes B_k iff C_i S_n <= S_k Q).
#pragma once
#include "mgb_device.cuh"

namespace mgb {

constexpr int SCAN_TPB = 256, SCAN_IPT = 8, SCAN_TILE = SCAN_TPB * SCAN_IPT;
constexpr uint64_t SFLAG_AGG = 1ull << 62, SFLAG_PFX = 2ull << 62, SVAL = (1ull << 62) - 1;
constexpr int SPIN_LIMIT = 1 << 22;

// per-resample control block (zeroed before each resample)
struct ResampleCtl {
  unsigned int tile_counter;
  int degenerate;
  unsigned long long total;  // exact sum of q_i
  unsigned int tile_counter2;
  int pad;
};

struct LsePartial {
  float m, s1, s2;
  int nan;
};

// result of a combine, stored in the workspace / filter state
struct LseOut {
  double lse, lse2, ess;
  float M;   // max log-weight (for quantisation)
  int flags; // 1 = NaN seen
};

// ------------------------------------------------------- LSE partials
// Block-level reduction of (max, sums) over a set of values, one per thread
// slot; inactive slots pass -inf.
template <int TPB>
__device__ __forceinline__ LsePartial block_lse_partial(float v, bool nan_in, float *smf, double *smd) {
  const float m = block_max<TPB>(v, smf);
  float e = 0.0f;
  if (m > -INFINITY && m < INFINITY && v == v) e = expf(v - m);
  const double s1 = block_sum<TPB, double>((double)e, smd);
  const double s2 = block_sum<TPB, double>((double)e * (double)e, smd);
  const int nn = __syncthreads_or(nan_in ? 1 : 0);
  LsePartial p;
  p.m = m;
  p.s1 = (float)s1;
  p.s2 = (float)s2;
  p.nan = nn;
  return p;
}

// Combine all partials (called by the last block, TPB threads). Returns LseOut
// in every thread.
template <int TPB>
__device__ __forceinline__ LseOut combine_lse(const LsePartial *parts, int nparts, float *smf, double *smd) {
  float m = -INFINITY;
  int nan = 0;
  for (int b = threadIdx.x; b < nparts; b += TPB) {
    const float mb = __ldcg(&parts[b].m);
    const int nb = __ldcg(&parts[b].nan);
    m = fmaxf(m, mb);
    nan |= nb;
  }
  const float M = block_max<TPB>(m, smf);
  const int anynan = __syncthreads_or(nan);
  double s1 = 0.0, s2 = 0.0;
  if (M > -INFINITY && M < INFINITY) {
    for (int b = threadIdx.x; b < nparts; b += TPB) {
      const float mb = __ldcg(&parts[b].m);
      if (mb > -INFINITY) {
        const float f = expf(mb - M);
        s1 += (double)(__ldcg(&parts[b].s1) * f);
        s2 += (double)(__ldcg(&parts[b].s2) * (f * f));
      }
    }
  }
  s1 = block_sum<TPB, double>(s1, smd);
  s2 = block_sum<TPB, double>(s2, smd);
  LseOut o;
  o.M = M;
  o.flags = anynan ? 1 : 0;
  if (anynan) {
    o.lse = o.lse2 = o.ess = __longlong_as_double(0x7ff8000000000000ll);
  } else if (M == INFINITY) {
    o.lse = o.lse2 = __longlong_as_double(0x7ff0000000000000ll);
    o.ess = __longlong_as_double(0x7ff8000000000000ll);
  } else if (M == -INFINITY) {
    o.lse = o.lse2 = -__longlong_as_double(0x7ff0000000000000ll);
    o.ess = __longlong_as_double(0x7ff8000000000000ll);
  } else {
    o.lse = (double)M + log(s1);
    o.lse2 = 2.0 * (double)M + log(s2);
    o.ess = exp(2.0 * o.lse - o.lse2);
  }
  return o;
}

// ------------------------------------------------------- scan helpers
__device__ __forceinline__ uint64_t ld_status(const uint64_t *p) { return *(volatile const uint64_t *)p; }
__device__ __forceinline__ void st_status(uint64_t *p, uint64_t v) { *(volatile uint64_t *)p = v; }

// Scan one tile: v[] are this thread's SCAN_IPT consecutive items (blocked
// layout).  On return v[] hold global inclusive prefixes; returns the tile's
// exclusive prefix and total (via refs).
__device__ __forceinline__ void tile_scan(uint64_t (&v)[SCAN_IPT], uint32_t tile, uint64_t *status, int *err,
                                          uint64_t &tile_excl, uint64_t &tile_total) {
  __shared__ uint64_t wsum[SCAN_TPB / 32];
  __shared__ uint64_t excl_s;
#pragma unroll
  for (int j = 1; j < SCAN_IPT; ++j) v[j] += v[j - 1];
  const uint64_t tsum = v[SCAN_IPT - 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t x = tsum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  uint64_t wpre = 0, btot = 0;
#pragma unroll
  for (int w = 0; w < SCAN_TPB / 32; ++w) {
    const uint64_t s = wsum[w];
    if (w < warp) wpre += s;
    btot += s;
  }
  const uint64_t texcl = wpre + x - tsum;
  if (warp == 0) {
    uint64_t run = 0;
    if (tile == 0) {
      if (lane == 0) st_status(&status[0], SFLAG_PFX | (btot & SVAL));
    } else {
      if (lane == 0) st_status(&status[tile], SFLAG_AGG | (btot & SVAL));
      int64_t pos = (int64_t)tile - 1;
      while (true) {
        const int64_t idx = pos - lane;
        uint64_t s = SFLAG_PFX;
        if (idx >= 0) {
          s = ld_status(&status[idx]);
          int polls = 0;
          while ((s >> 62) == 0) {
            if (++polls > SPIN_LIMIT) {
              raise_err(err, EB_TIMEOUT);
              s = SFLAG_PFX;
              break;
            }
            __nanosleep(32);
            s = ld_status(&status[idx]);
          }
        }
        const unsigned pm = __ballot_sync(0xffffffffu, (s >> 62) == 2);
        const int first = pm ? __ffs(pm) - 1 : 32;
        uint64_t val = (lane <= first) ? (s & SVAL) : 0;
        val = warp_sum<uint64_t>(val);
        run += val;
        if (pm) break;
        pos -= 32;
      }
      if (lane == 0) st_status(&status[tile], SFLAG_PFX | ((run + btot) & SVAL));
    }
    if (lane == 0) excl_s = run;
  }
  __syncthreads();
  tile_excl = excl_s;
  tile_total = btot;
  const uint64_t add = tile_excl + texcl;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) v[j] += add;
}

// K(X) = #{k in [0, n) : (k 2^23 + m) Q < X n 2^23}  (systematic threshold count)
__device__ __forceinline__ int64_t sys_count(uint64_t X, int64_t n, uint64_t m, uint64_t Q, float n_over_q) {
  const uint64_t den = (uint64_t)n << 23;
  float est = __fmul_rn((float)X, n_over_q) - (float)m * 0x1p-23f;
  int64_t kk = (int64_t)ceilf(est);
  if (kk < 0) kk = 0;
  if (kk > n) kk = n;
  // predicate f(k): (k 2^23 + m) Q < X den  (monotone: true then false)
  while (kk > 0 && mul_le(X, den, (((uint64_t)(kk - 1)) << 23) + m, Q)) --kk;
  while (kk < n && !mul_le(X, den, (((uint64_t)kk) << 23) + m, Q)) ++kk;
  return kk;
}

}  // namespace mgb
