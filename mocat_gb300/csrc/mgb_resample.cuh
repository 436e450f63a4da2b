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
//  * Systematic: reduce-then-scan.  Pass 1 sums each 2048-particle tile and
//    its last block scans the tile sums (the total Q must be known before any
//    threshold can be placed).  Thresholds (k + u) Q / n form an arithmetic
//    progression, so particle i's offspring are the k in [K(C_{i-1}), K(C_i))
//    with K(X) = #{k : (k 2^23 + m) Q < X n 2^23}; pass 1 also cuts each tile's
//    output range into units of <= 2048 outputs, and pass 2 runs one block per
//    unit (heavy tiles are split across blocks, so no block does more than one
//    tile of scan work plus 2048 outputs).
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
  unsigned int units;        // systematic fill units
  unsigned int m23;          // systematic uniform's mantissa
  // systematic thresholds T_k = floor((k 2^23 + m) Q / (n 2^23))
  //                          = k qn + a + floor((k rn + bh) / n)
  unsigned long long qn, rn, a, bh, magic;  // magic = floor((2^64 - 1) / n)
};

// Threshold constants from Q, n and the uniform's mantissa m:
//   Q = qn n + rn;  m qn = a1 2^23 + r1;  V = r1 n + m rn < 2^24 n
//   m Q / (n 2^23) = a1 + V / (n 2^23),  a = a1 + [V >= n 2^23],  bh = (V mod n 2^23) >> 23
__device__ __forceinline__ void sys_constants(uint64_t Q, uint64_t n, uint32_t m, ResampleCtl &c,
                                              uint64_t magic) {
  uint64_t qn = __umul64hi(Q, magic), rn = Q - qn * n;  // magic = floor((2^64 - 1) / n)
  if (rn >= n) {
    ++qn;
    rn -= n;
  }
  c.qn = qn;
  c.rn = rn;
  const uint64_t lo = (uint64_t)m * c.qn, hi = __umul64hi((uint64_t)m, c.qn);
  const uint64_t a1 = (hi << 41) | (lo >> 23), r1 = lo & ((1ull << 23) - 1);
  uint64_t V = r1 * n + (uint64_t)m * c.rn;
  const uint64_t den = n << 23;
  uint64_t a2 = 0;
  if (V >= den) { V -= den; a2 = 1; }
  c.a = a1 + a2;
  c.bh = V >> 23;
  c.magic = magic;
}

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
// slot; inactive slots pass -inf.  The sums are float shuffle trees (pairwise,
// error O(log2 TPB) ulp); float64 is used only across blocks, where there are
// few terms -- FP64 runs at a small fraction of the FP32 rate on this part.
template <int TPB>
__device__ __forceinline__ LsePartial block_lse_partial(float v, bool nan_in, float *smf, double *smd) {
  (void)smd;
  const float m = block_max<TPB>(v, smf);
  float e = 0.0f;
  if (m > -INFINITY && m < INFINITY && v == v) e = expf(v - m);
  const float s1 = block_sum<TPB, float>(e, smf);
  const float s2 = block_sum<TPB, float>(e * e, smf);
  const int nn = __syncthreads_or(nan_in ? 1 : 0);
  LsePartial p;
  p.m = m;
  p.s1 = s1;
  p.s2 = s2;
  p.nan = nn;
  return p;
}

// Combine all partials (TPB threads of one block).  The max is a block
// reduction; the float64 sums run in warp 0 only and the logarithms /
// exponential in its lane 0, then the result is broadcast through shared
// memory (FP64 throughput is low on this part, so it is kept off the other
// warps).
template <int TPB>
__device__ __forceinline__ LseOut combine_lse(const LsePartial *parts, int nparts, float *smf, double *smd) {
  (void)smd;
  __shared__ LseOut res_s;
  float m = -INFINITY;
  int nan = 0;
  for (int b = threadIdx.x; b < nparts; b += TPB) {
    m = fmaxf(m, __ldcg(&parts[b].m));
    nan |= __ldcg(&parts[b].nan);
  }
  const float M = block_max<TPB>(m, smf);
  const int anynan = __syncthreads_or(nan);
  if (threadIdx.x < 32) {
    double s1 = 0.0, s2 = 0.0;
    if (M > -INFINITY && M < INFINITY) {
      for (int b = threadIdx.x; b < nparts; b += 32) {
        const float mb = __ldcg(&parts[b].m);
        if (mb > -INFINITY) {
          const float f = expf(mb - M);
          s1 += (double)(__ldcg(&parts[b].s1) * f);
          s2 += (double)(__ldcg(&parts[b].s2) * (f * f));
        }
      }
    }
    s1 = warp_sum<double>(s1);
    s2 = warp_sum<double>(s2);
    if (threadIdx.x == 0) {
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
        // float logarithms of the float64 sums (relative error ~1e-7 of
        // log S, i.e. ~1e-7 absolute on the logsumexp); the ESS S1^2 / S2 in float64
        o.lse = (double)M + (double)logf((float)s1);
        o.lse2 = 2.0 * (double)M + (double)logf((float)s2);
        o.ess = s1 * s1 / s2;
      }
      res_s = o;
    }
  }
  __syncthreads();
  const LseOut o = res_s;
  __syncthreads();
  return o;
}

// online (max, sum exp(l - max), sum exp(2 (l - max))) of a stream of values
__device__ __forceinline__ void online_acc(float l, float &m, float &s1, float &s2, int &nanf) {
  if (l != l) {
    nanf = 1;
    return;
  }
  if (l == -INFINITY || m == INFINITY) return;
  if (l > m) {
    const float sc = m == -INFINITY ? 0.0f : expf(m - l);
    s1 = s1 * sc + 1.0f;
    s2 = s2 * (sc * sc) + 1.0f;
    m = l;
  } else {
    const float e = expf(l - m);
    s1 += e;
    s2 += e * e;
  }
}

// block partial of per-thread online accumulators
template <int TPB>
__device__ __forceinline__ LsePartial block_online_partial(float m, float s1, float s2, int nanf, float *smf) {
  const float Mb = block_max<TPB>(m, smf);
  const float f = (m > -INFINITY && Mb < INFINITY) ? expf(m - Mb) : 0.0f;
  const float b1 = block_sum<TPB, float>(s1 * f, smf);
  const float b2 = block_sum<TPB, float>(s2 * (f * f), smf);
  const int bn = __syncthreads_or(nanf);
  return LsePartial{Mb, b1, b2, bn};
}

// ------------------------------------------------------- scan helpers
__device__ __forceinline__ uint64_t ld_status(const uint64_t *p) { return *(volatile const uint64_t *)p; }
__device__ __forceinline__ void st_status(uint64_t *p, uint64_t v) { *(volatile uint64_t *)p = v; }

// Scan one tile: v[] are this thread's SCAN_IPT consecutive items (blocked
// layout).  On return v[] hold global inclusive prefixes; returns the tile's
// exclusive prefix and total (via refs).
__device__ __forceinline__ void tile_scan(uint64_t (&v)[SCAN_IPT], uint32_t tile, uint64_t *status, int *err,
                                          uint64_t &tile_excl, uint64_t &tile_total, int limit = SPIN_LIMIT) {
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
            if (++polls > limit) {
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

// Threshold cursor: T_k and the remainder of (k rn + bh) mod n, so that
// T_{k+1} = T_k + qn + carry costs four integer operations.
struct ThrCursor {
  uint64_t T, rem;
};
__device__ __forceinline__ ThrCursor thr_at(const ResampleCtl &c, uint64_t k, uint64_t n) {
  const uint64_t num = k * c.rn + c.bh;
  uint64_t q = __umul64hi(num, c.magic);
  uint64_t rem = num - q * n;
  if (rem >= n) {
    ++q;
    rem -= n;
  }
  return ThrCursor{k * c.qn + c.a + q, rem};
}
__device__ __forceinline__ void thr_next(ThrCursor &t, const ResampleCtl &c, uint64_t n) {
  t.rem += c.rn;
  const uint64_t carry = t.rem >= n ? 1ull : 0ull;
  t.rem -= carry * n;
  t.T += c.qn + carry;
}

// Offspring-run window: RUN_WINDOW consecutive outputs in shared memory.
// Every particle whose run [lo, hi) meets the window marks the window slot of
// its first output there with its tile-local number; an inclusive max-scan
// then gives every slot the particle that covers it (runs are disjoint and
// ordered by particle, so the covering particle is the largest mark at or
// before the slot).  TPB threads, RUN_WINDOW / TPB consecutive slots each.
constexpr int RUN_WINDOW = 4096;
template <int TPB = 256>
__device__ __forceinline__ void window_max_scan(int32_t *stage, int32_t *wmax /* >= TPB / 32 */) {
  constexpr int V = RUN_WINDOW / TPB / 4;  // int4 per thread
  static_assert(V * 4 * TPB == RUN_WINDOW && TPB % 32 == 0, "whole int4 slots per thread");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int4 *s4 = (int4 *)stage + threadIdx.x * V;
  int4 v[V];
#pragma unroll
  for (int j = 0; j < V; ++j) v[j] = s4[j];
  int run = -1;
#pragma unroll
  for (int j = 0; j < V; ++j) {
    run = max(run, v[j].x);
    v[j].x = run;
    run = max(run, v[j].y);
    v[j].y = run;
    run = max(run, v[j].z);
    v[j].z = run;
    run = max(run, v[j].w);
    v[j].w = run;
  }
  int x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x = max(x, y);
  }
  if (lane == 31) wmax[warp] = x;
  __syncthreads();
  int carry = -1;
#pragma unroll
  for (int w = 0; w < TPB / 32; ++w)
    if (w < warp) carry = max(carry, wmax[w]);
  const int ex = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane > 0) carry = max(carry, ex);
#pragma unroll
  for (int j = 0; j < V; ++j) {
    v[j].x = max(v[j].x, carry);
    v[j].y = max(v[j].y, carry);
    v[j].z = max(v[j].z, carry);
    v[j].w = max(v[j].w, carry);
    s4[j] = v[j];
  }
}

// block-wide exclusive scan of one u64 per thread over TPB threads (returns the
// block total too); sm holds TPB / 32 words
template <int TPB = SCAN_TPB>
__device__ __forceinline__ unsigned long long block_excl_scan_u64(unsigned long long v, unsigned long long *sm,
                                                                  unsigned long long &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) sm[warp] = x;
  __syncthreads();
  unsigned long long wpre = 0, tot = 0;
#pragma unroll
  for (int w = 0; w < TPB / 32; ++w) {
    if (w < warp) wpre += sm[w];
    tot += sm[w];
  }
  total = tot;
  return wpre + x - v;
}

// K(X) = #{k in [0, n) : (k 2^23 + m) Q < X n 2^23}  (systematic threshold count)
// The float estimate is within one of K; both neighbours are tested
// unconditionally (independent 128-bit products, no loop on the common path)
// and a walk runs only if the estimate was further off.
__device__ __forceinline__ int64_t sys_count(uint64_t X, int64_t n, uint64_t m, uint64_t Q, float n_over_q) {
  const uint64_t den = (uint64_t)n << 23;
  const float xf = __fmaf_rn(__uint2float_rn((uint32_t)(X >> 32)), 0x1p32f, __uint2float_rn((uint32_t)X));
  // the estimate lies in [-1, n] with n < 2^31: a 32-bit conversion (a float to
  // 64-bit integer conversion is a slow path on this part)
  const float est = fminf(fmaxf(__fmul_rn(xf, n_over_q) - (float)m * 0x1p-23f, -1.0f), 0x1.fffffep+30f);
  int64_t kk = (int64_t)(int)ceilf(est);
  kk = kk < 0 ? 0 : (kk > n ? n : kk);
  // f(k) := (k 2^23 + m) Q < X den, true for k < K, false from K on
  const bool f_lo = kk > 0 && !mul_le(X, den, (((uint64_t)(kk - 1)) << 23) + m, Q);
  const bool f_hi = kk < n && !mul_le(X, den, (((uint64_t)kk) << 23) + m, Q);
  if ((kk == 0 || f_lo) && !f_hi) return kk;
  while (kk > 0 && mul_le(X, den, (((uint64_t)(kk - 1)) << 23) + m, Q)) --kk;
  while (kk < n && !mul_le(X, den, (((uint64_t)kk) << 23) + m, Q)) ++kk;
  return kk;
}

// sys_count for n <= 2^21, without branches.  The float estimate est of
// Y - u (Y = X n / Q, u = m / 2^23) is within 0.8 of it: X, Q and n / Q each
// carry a relative error below 2^-23 and the product one below 2^-24, so Y
// is off by less than 2^-21.6 Y <= 0.66 for Y <= n <= 2^21, and the final
// subtraction rounds by at most 1/8.  K lies in [Y - u, Y - u + 1), so K is
// ceil(est) - 1, ceil(est) or ceil(est) + 1, and the two exact tests f(kk - 1)
// and f(kk) pick it.
constexpr int64_t SYS_COUNT_SMALL_MAX_N = 1 << 21;
__device__ __forceinline__ int32_t sys_count_small(uint64_t X, int32_t n, uint64_t m, uint64_t Q, float n_over_q) {
  const uint64_t den = (uint64_t)n << 23;
  const float xf = __fmaf_rn(__uint2float_rn((uint32_t)(X >> 32)), 0x1p32f, __uint2float_rn((uint32_t)X));
  const float est = fminf(fmaxf(__fmul_rn(xf, n_over_q) - (float)m * 0x1p-23f, -1.0f), (float)n);
  int32_t kk = (int32_t)ceilf(est);
  kk = kk < 0 ? 0 : (kk > n ? n : kk);
  // f(k) := (k 2^23 + m) Q < X den, true for k < K, false from K on
  const bool f_lo = kk == 0 || !mul_le(X, den, (((uint64_t)(uint32_t)(kk - 1)) << 23) + m, Q);
  const bool f_hi = kk < n && !mul_le(X, den, (((uint64_t)(uint32_t)kk) << 23) + m, Q);
  return kk - (f_lo ? 0 : 1) + (f_hi ? 1 : 0);
}

}  // namespace mgb
