// Thread-group primitives for kernels that run several independent problems
// in one CTA (a group = a power-of-two number of warps): a group barrier and
// an in-place group-wide inclusive scan of 64-bit integers.
#pragma once
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"

namespace mgb {

// group barrier: named barrier `id` over `nthr` threads, or the warp
__device__ __forceinline__ void gbar(int id, int nthr) {
  if (nthr <= 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthr) : "memory");
  }
}

// In-place inclusive scan of V[0..cnt) by the group's W warps (warp wg owns a
// contiguous segment, processed 32 items at a time); item j is load(j) on
// entry.  Returns the total.  Two group barriers.
template <class Load>
__device__ __forceinline__ uint64_t group_scan(uint64_t *V, int cnt, int W, int wg, int lane, int wcta,
                                               unsigned long long *wtot, int bar, int G, Load load) {
  const int seg = ((cnt + 32 * W - 1) / (32 * W)) * 32;
  const int s0 = wg * seg, s1 = min(s0 + seg, cnt);
  uint64_t carry = 0;
  for (int c = s0; c < s1; c += 32) {
    const int j = c + lane;
    uint64_t v = j < s1 ? load(j) : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    v += carry;
    if (j < s1) V[j] = v;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
  if (lane == 0) wtot[wcta] = carry;
  gbar(bar, G);
  uint64_t off = 0, tot = 0;
  for (int w = 0; w < W; ++w) {
    const uint64_t x = wtot[wcta - wg + w];
    off += w < wg ? x : 0ull;
    tot += x;
  }
  if (off)
    for (int j = s0 + lane; j < s1; j += 32) V[j] += off;
  gbar(bar, G);
  return tot;
}

// Systematic ancestors by merge path on a group: C[0..n) are the inclusive
// fixed-point weight prefixes (total Q), m the uniform's 23-bit mantissa,
// magic = floor((2^64 - 1) / n).  A[k] = #{i : C_i <= T_k} (clamped to n - 1),
// T_k = floor((k 2^23 + m) Q / (n 2^23)).  Thread tg of G merges diagonals
// [tg per, (tg + 1) per) after one partition search.  No barrier inside.
__device__ __forceinline__ void group_systematic_fill(const uint64_t *C, int n, uint64_t Q, uint32_t m, uint64_t magic,
                                                      int32_t *A, int tg, int G) {
  ResampleCtl c;
  sys_constants(Q, (uint64_t)n, m, c, magic);
  const int total = 2 * n, per = (total + G - 1) / G, d0 = tg * per;
  if (d0 >= total) return;
  int lo = d0 > n ? d0 - n : 0, hi = d0 < n ? d0 : n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (C[mid] <= thr_at(c, (uint64_t)(d0 - 1 - mid), (uint64_t)n).T) lo = mid + 1;
    else hi = mid;
  }
  int i = lo, kk = d0 - lo;
  ThrCursor cur = thr_at(c, (uint64_t)(kk < n ? kk : 0), (uint64_t)n);
  const int d1 = min(d0 + per, total);
  uint64_t ci = i < n ? C[i] : 0ull;
  for (int d = d0; d < d1; ++d) {
    if (i < n && (kk >= n || ci <= cur.T)) {
      ++i;
      ci = i < n ? C[i] : 0ull;
    } else {
      A[kk] = i < n ? i : n - 1;
      ++kk;
      thr_next(cur, c, (uint64_t)n);
    }
  }
}

}  // namespace mgb
