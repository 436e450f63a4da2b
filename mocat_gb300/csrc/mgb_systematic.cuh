// Systematic resampling's two passes as device functions: the standalone
// kernels k_tile_sums / k_systematic (mgb_resample.cu) run one filter per
// launch; the batched score driver (mgb_pf_score.cu) runs many filters per
// launch, one per grid row, with the same code.
#pragma once
#include "mgb_resample.cuh"

namespace mgb {

// Systematic resampling, pass 1: exact per-tile sums of the fixed-point
// weights; the last block to finish turns them into exclusive tile prefixes
// and the total Q (reduce-then-scan: the total is needed before any
// threshold can be placed, so pass 2 re-reads the weights anyway and no tile
// ever waits on another).
__device__ __forceinline__ void load_tile_q(const float *__restrict__ lw, int64_t n, int64_t i0, float M,
                                            float scale, uint64_t (&q)[SCAN_IPT], int &bad) {
  if (i0 + SCAN_IPT <= n && ((((uintptr_t)(lw + i0)) & 15) == 0)) {
    const float4 a = __ldg((const float4 *)(lw + i0)), b = __ldg((const float4 *)(lw + i0 + 4));
    const float f[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) {
      bad |= (f[j] != f[j]) || (f[j] == INFINITY);
      q[j] = quantise_weight(f[j], M, scale);
    }
  } else {
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) {
      const float v = (i0 + j < n) ? lw[i0 + j] : -INFINITY;
      bad |= (v != v) || (v == INFINITY);
      q[j] = quantise_weight(v, M, scale);
    }
  }
}

constexpr int SYS_UNIT = SCAN_TILE;  // outputs per fill block

// Pass 1: per-tile sums of q; the last block scans them in place into
// exclusive tile prefixes P_t, sets Q and the uniform's mantissa, and cuts
// every tile's output range [K(P_t), K(P_{t+1})) into units of at most
// SYS_UNIT outputs: units[u] = (t << 32) | first output of the unit.
__device__ __forceinline__ void tile_sums_body(const float *__restrict__ lw, int64_t n, const float *Mptr,
                                                         const uint32_t *key, int has_m23, uint32_t m23_arg,
                                                         const int32_t *flag, ResampleCtl *ctl,
                                                         uint64_t *__restrict__ tile_pfx,
                                                         uint64_t *__restrict__ units) {
  if (flag && *flag == 0) return;
  __shared__ unsigned long long sm[SCAN_TPB / 32];
  __shared__ bool last;
  const float M = *Mptr;
  const float scale = __int_as_float((weight_shift(n) + 127) << 23);
  const int64_t i0 = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_IPT;
  uint64_t q[SCAN_IPT];
  int bad = !(M > -INFINITY && M < INFINITY);
  load_tile_q(lw, n, i0, M, scale, q, bad);
  unsigned long long acc = 0;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) acc += q[j];
  acc = block_sum<SCAN_TPB, unsigned long long>(acc, sm);
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    tile_pfx[blockIdx.x] = acc;
    if (bad) atomicOr(&ctl->degenerate, 1);
    last = last_block_arrival(&ctl->tile_counter);
  }
  __syncthreads();
  if (!last) return;
  const int nt = (int)gridDim.x;
  const int per = (nt + SCAN_TPB - 1) / SCAN_TPB;
  const int b0 = threadIdx.x * per, b1 = min(b0 + per, nt);
  unsigned long long sums[32];  // per <= 32 for n <= 2^24 (8192 tiles / 256 threads)
  unsigned long long run = 0;
  for (int b = b0, j = 0; b < b1; ++b, ++j) {
    const unsigned long long v = __ldcg(&tile_pfx[b]);
    if (j < 32) sums[j] = v;
    run += v;
  }
  unsigned long long Q;
  unsigned long long pre = block_excl_scan_u64(run, sm, Q);
  unsigned long long pfx[32];
  for (int b = b0, j = 0; b < b1; ++b, ++j) {
    const unsigned long long v = j < 32 ? sums[j] : __ldcg(&tile_pfx[b]);
    if (j < 32) pfx[j] = pre;
    tile_pfx[b] = pre;
    pre += v;
  }
  const int degenerate = bad || *(volatile int *)&ctl->degenerate || Q == 0;
  if (degenerate) {
    if (threadIdx.x == 0) {
      ctl->total = Q;
      ctl->units = 0u;
      ctl->tile_counter = 0u;
    }
    return;
  }
  const uint32_t m = has_m23 ? m23_arg : (bits_at(key[0], key[1], 1, 0) >> 9);
  const float n_over_q = __fdiv_rn((float)n, (float)Q);
  // this thread's tiles b0..b1-1 have prefixes P(j) (j = b - b0) and the run ends at `pre` = P_{b1}
  auto P = [&](int j) -> uint64_t { return j < 32 ? pfx[j] : tile_pfx[b0 + j]; };
  const int cnt = b1 - b0;
  unsigned long long nu = 0;
  if (cnt > 0) {
    int64_t kcur = sys_count(P(0), n, m, Q, n_over_q);
    for (int j = 0; j < cnt; ++j) {
      const int64_t knext = sys_count(j + 1 < cnt ? P(j + 1) : pre, n, m, Q, n_over_q);
      nu += (uint64_t)((knext - kcur + SYS_UNIT - 1) / SYS_UNIT);
      kcur = knext;
    }
  }
  unsigned long long utot;
  unsigned long long uo = block_excl_scan_u64(nu, sm, utot);
  if (cnt > 0) {
    int64_t kcur = sys_count(P(0), n, m, Q, n_over_q);
    for (int j = 0; j < cnt; ++j) {
      const int64_t knext = sys_count(j + 1 < cnt ? P(j + 1) : pre, n, m, Q, n_over_q);
      for (int64_t k = kcur; k < knext; k += SYS_UNIT) units[uo++] = ((uint64_t)(b0 + j) << 32) | (uint64_t)k;
      kcur = knext;
    }
  }
  if (threadIdx.x == 0) {
    ctl->total = Q;
    ctl->units = (unsigned int)utot;
    ctl->m23 = m;
    ctl->tile_counter = 0u;
  }
}

// Pass 2: one block per unit.  The block rescans its tile into exact
// inclusive prefixes C_j (shared memory), computes every particle's offspring
// count K(C_j) (sys_count_small, branch-free, for n <= 2^21; sys_count above)
// and writes the unit's outputs [kb, ke) through a shared window: particle j's
// run [K(C_{j-1}), K(C_j)) marks its first slot in the unit, an inclusive
// max-scan gives every slot its particle, and the slots are stored coalesced.
// Output k goes to the first particle with C_j > T_k, as in a merge of the
// prefixes with the thresholds.
__device__ __forceinline__ void systematic_body(const float *__restrict__ lw, int64_t n, const float *Mptr,
                                                          const int32_t *flag, const ResampleCtl *ctl,
                                                          const uint64_t *__restrict__ tile_pfx,
                                                          const uint64_t *__restrict__ units,
                                                          int32_t *__restrict__ anc, int *err) {
  if (flag && *flag == 0) return;
  static_assert(SYS_UNIT <= RUN_WINDOW && SCAN_TPB == 256, "one window per unit");
  __shared__ unsigned long long wsum[SCAN_TPB / 32];
  __shared__ __align__(16) uint64_t cs[SCAN_TILE];  // prefixes, then the output window
  __shared__ int32_t sK[SCAN_TILE];
  __shared__ int32_t wmax[SCAN_TPB / 32];
  __shared__ int32_t k0_s;
  const int64_t ntiles_real = (n + SCAN_TILE - 1) / SCAN_TILE;
  const uint64_t Q = *(volatile const unsigned long long *)&ctl->total;
  const int degenerate = *(volatile const int *)&ctl->degenerate || Q == 0;
  if (degenerate) {
    if (blockIdx.x < ntiles_real) {
      const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
      for (int j = threadIdx.x; j < SCAN_TILE; j += SCAN_TPB)
        if (base + j < n) anc[base + j] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_err(err, EB_DEGENERATE);
    return;
  }
  if (blockIdx.x >= *(volatile const unsigned int *)&ctl->units) return;
  const uint32_t m = *(volatile const unsigned int *)&ctl->m23;
  const uint64_t ud = __ldg(&units[blockIdx.x]);
  const int64_t tile = (int64_t)(ud >> 32), kb = (int64_t)(ud & 0xffffffffu);
  const int64_t base = tile * SCAN_TILE;
  const float M = *Mptr;
  const float scale = __int_as_float((weight_shift(n) + 127) << 23);
  const int64_t i0 = base + (int64_t)threadIdx.x * SCAN_IPT;
  uint64_t q[SCAN_IPT];
  int bad = 0;
  load_tile_q(lw, n, i0, M, scale, q, bad);
  uint64_t tsum = 0;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) tsum += q[j];
  unsigned long long btot;
  const uint64_t P = __ldg(&tile_pfx[tile]);
  uint64_t cc = P + block_excl_scan_u64(tsum, wsum, btot);
  const float n_over_q = __fdiv_rn((float)n, (float)Q);
  const int64_t ke_tile = sys_count(P + btot, n, m, Q, n_over_q);
  const int64_t ke = kb + SYS_UNIT < ke_tile ? kb + SYS_UNIT : ke_tile;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) {
    cc += q[j];
    cs[threadIdx.x * SCAN_IPT + j] = cc;
  }
  __syncthreads();
  const int cnt_valid = (int)(n - base < SCAN_TILE ? n - base : SCAN_TILE);
  const bool small = n <= SYS_COUNT_SMALL_MAX_N;
  // K of the tile's particles (past n: K = n, empty runs after the last particle)
#pragma unroll
  for (int r = 0; r < SCAN_IPT; ++r) {
    const int jj = threadIdx.x + SCAN_TPB * r;
    int32_t k = (int32_t)n;
    if (jj < cnt_valid)
      k = small ? sys_count_small(cs[jj], (int32_t)n, m, Q, n_over_q) : (int32_t)sys_count(cs[jj], n, m, Q, n_over_q);
    sK[jj] = k;
  }
  if (threadIdx.x == 0)
    k0_s = small ? sys_count_small(P, (int32_t)n, m, Q, n_over_q) : (int32_t)sys_count(P, n, m, Q, n_over_q);
  __syncthreads();
  int32_t *stage = (int32_t *)cs;
  int4 *s4 = (int4 *)stage;
#pragma unroll
  for (int j = 0; j < RUN_WINDOW / 4 / SCAN_TPB; ++j) s4[threadIdx.x + SCAN_TPB * j] = make_int4(-1, -1, -1, -1);
  __syncthreads();
  const int32_t k0 = k0_s, w0 = (int32_t)kb, w1 = (int32_t)ke;
#pragma unroll
  for (int r = 0; r < SCAN_IPT; ++r) {
    const int jj = threadIdx.x + SCAN_TPB * r;
    const int32_t lo = jj ? sK[jj - 1] : k0, hi = sK[jj];
    const int32_t st = lo > w0 ? lo : w0;
    if (hi > st && st < w1) stage[st - w0] = jj;
  }
  __syncthreads();
  window_max_scan(stage, wmax);
  __syncthreads();
  // every slot is covered (slot 0 by the run through kb); the clamp only keeps a
  // wrong count from producing an out-of-range ancestor
  for (int q = threadIdx.x; q < w1 - w0; q += SCAN_TPB) anc[w0 + q] = (int32_t)(base + max(stage[q], 0));
}

}  // namespace mgb
