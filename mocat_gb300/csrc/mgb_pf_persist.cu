// Whole-filter persistent kernel: a bootstrap particle filter with
// ESS-triggered systematic resampling, all T steps in one cooperative launch
// (one CTA group resident on every SM).  The model enters as a particle policy
// (the GPU counterpart of the reference's StateSpaceModel plugin): kD, kDY,
// init() for the initial draw and weight, step() for one propagate + weight
// from a source state and a carried log-weight; LGModelP (linear-Gaussian),
// NLModelP (one-dimensional non-linear benchmark) and SVModelP (stochastic
// volatility, dim 1) are compiled here.
//
// Per step the grid runs
//   P1  propagate + weight, two particles per thread (i, i + n/2), grid-stride;
//       each block folds its log-weights into an online (max, sum e, sum e^2)
//       partial                                                  -> barrier
//   P2  every block combines all partials identically (same data, same order,
//       so every block reaches the same logsumexp / ESS / resample decision);
//       block 0 records ESS, the resample flag and log Z
//   and, when the next step resamples,
//   P3  exact fixed-point tile sums of the new log-weights, and each tile's
//       within-tile prefixes                                          -> barrier
//   P4  every block scans the tile sums in shared memory; for the particles
//       of its own tiles it computes the exact systematic offspring counts and
//       writes each particle's run of ancestor indices               -> barrier
// A non-resampling step costs one grid barrier, a resampling step three; no
// kernel launches, no host round trips.  Data written inside the kernel is
// read back through L2 (__ldcg): L1 is not coherent across SMs.  The grid
// barrier is a sense-reversing counter with a bounded wait (on expiry the
// error word gets EB_TIMEOUT and the kernel runs to completion).
//
// Results are identical to the multi-kernel path (same float op sequence per
// particle, integer resampling); only the float64 LSE reduction is grouped
// differently.
#include "mgb_internal.cuh"
#include "mgb_kernels.cuh"
#include "mgb_lg.cuh"
#include "mgb_persist.cuh"
#include "mgb_nl1d.cuh"
#include "mgb_sv.cuh"

namespace mgb {

// err is the kernel's own (never null) error word: once a wait has run out,
// later barriers stop waiting and the step loop exits, so a fault can cost at
// most one bounded wait.  Returns true (in every thread of the block) when this
// block left the barrier without every block having arrived: its wait ran out,
// or another block's had.  Only thread 0 reads the error word; the result
// reaches the other threads through shared memory at the closing __syncthreads,
// so a normal pass adds no global load.
__device__ __forceinline__ bool grid_sync(GridBar *bar, unsigned nblocks, int *err, int limit = BAR_SPIN_LIMIT) {
  __shared__ int gs_out;
  if (nblocks == 1) {  // one block: a block barrier orders its own global writes
    __syncthreads();
    return false;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // Release / acquire at GPU scope instead of full fences: the arrival (acq_rel)
    // publishes this block's writes (ordered before it by the block barrier) and, in
    // the last block to arrive, acquires every other block's; that block's release
    // of the generation passes them all on to the waiters' acquiring loads.
    int out = 0;
    unsigned int g, prev;
    asm volatile("ld.relaxed.gpu.u32 %0, [%1];" : "=r"(g) : "l"(&bar->gen) : "memory");
    asm volatile("atom.acq_rel.gpu.add.u32 %0, [%1], 1;" : "=r"(prev) : "l"(&bar->count) : "memory");
    if (prev == nblocks - 1) {
      asm volatile("st.relaxed.gpu.u32 [%0], 0;" ::"l"(&bar->count) : "memory");
      asm volatile("red.release.gpu.add.u32 [%0], 1;" ::"l"(&bar->gen) : "memory");
    } else {
      int polls = 0;
      while (true) {
        unsigned int cur;
        asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(cur) : "l"(&bar->gen) : "memory");
        if (cur != g) break;
        // another block's timeout (checked every 64 polls: one load per poll on the barrier's line)
        if ((polls & 63) == 63 && (*(volatile int *)err & EB_TIMEOUT)) {
          out = 1;
          break;
        }
        if (++polls > limit) {
          atomicOr(err, EB_TIMEOUT);
          out = 1;
          break;
        }
      }
    }
    gs_out = out;
  }
  __syncthreads();
  return gs_out != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// phase boundary stamp (block 0, thread 0 only)
__device__ __forceinline__ void stamp(const PersistArgs &a, int64_t t, int k) {
  if (a.trace && blockIdx.x == 0 && threadIdx.x == 0) a.trace[t * 10 + k] = globaltimer_ns();
}

__device__ __forceinline__ bool timed_out(const int *err) { return (*(volatile const int *)err & EB_TIMEOUT) != 0; }

// warp partial of per-lane online accumulators: lane 0's value of a fixed
// shuffle tree (each lane's order is fixed, so lane 0's result does not depend
// on timing)
__device__ __forceinline__ LsePartial warp_online_partial(float m, float s1, float s2, int nanf) {
  const float Mw = warp_max(m);
  const float f = (m > -INFINITY && Mw < INFINITY) ? expf(m - Mw) : 0.0f;
  const float b1 = warp_sum<float>(s1 * f);
  const float b2 = warp_sum<float>(s2 * (f * f));
  const int bn = __any_sync(0xffffffffu, nanf);
  return LsePartial{Mw, b1, b2, bn};
}

// combine of up to 32 partials, one per lane (inactive lanes pass m = -inf):
// lane 0's value of a fixed shuffle tree
__device__ __forceinline__ LsePartial warp_partial_combine(const LsePartial &q) {
  const float Mw = warp_max(q.m);
  const float f = (q.m > -INFINITY && Mw < INFINITY) ? expf(q.m - Mw) : 0.0f;
  const float b1 = warp_sum<float>(q.s1 * f);
  const float b2 = warp_sum<float>(q.s2 * (f * f));
  const int bn = __any_sync(0xffffffffu, q.nan);
  return LsePartial{Mw, b1, b2, bn};
}

// Fixed-order combine of the chunk partials (identical in every block): float
// shuffle trees only -- FP64 throughput is low on this part and this runs in
// every block every step.  Logarithms in float; log Z accumulates in float64.
template <int TPB>
__device__ __forceinline__ LseOut combine_chunks(const LsePartial *parts, int np, float *smf, LseOut *res_s) {
  // up to 10 partials per thread stay in registers between the max and the sums
  // (one L2 round trip); more chunks than that are read twice
  constexpr int PER = 8;
  const bool one_pass = np <= PER * TPB;
  float4 q[PER];
  float m = -INFINITY;
  int nan = 0;
  if (one_pass) {
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int b = threadIdx.x + j * TPB;
      q[j] = b < np ? __ldcg((const float4 *)&parts[b]) : make_float4(-INFINITY, 0.0f, 0.0f, 0.0f);
      m = fmaxf(m, q[j].x);
      nan |= __float_as_int(q[j].w);
    }
  } else {
    for (int b = threadIdx.x; b < np; b += TPB) {
      m = fmaxf(m, __ldcg(&parts[b].m));
      nan |= __ldcg(&parts[b].nan);
    }
  }
  const float M = block_max<TPB>(m, smf);
  const int anynan = __syncthreads_or(nan);
  float s1 = 0.0f, s2 = 0.0f;
  if (M > -INFINITY && M < INFINITY) {
    if (one_pass) {
#pragma unroll
      for (int j = 0; j < PER; ++j) {
        if (q[j].x > -INFINITY) {
          const float f = expf(q[j].x - M);
          s1 += q[j].y * f;
          s2 += q[j].z * (f * f);
        }
      }
    } else {
      for (int b = threadIdx.x; b < np; b += TPB) {
        const float4 v = __ldcg((const float4 *)&parts[b]);
        if (v.x > -INFINITY) {
          const float f = expf(v.x - M);
          s1 += v.y * f;
          s2 += v.z * (f * f);
        }
      }
    }
  }
  s1 = block_sum<TPB, float>(s1, smf);
  s2 = block_sum<TPB, float>(s2, smf);
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
      o.lse = (double)M + (double)logf(s1);
      o.lse2 = 2.0 * (double)M + (double)logf(s2);
      o.ess = (double)s1 * (double)s1 / (double)s2;
    }
    *res_s = o;
  }
  __syncthreads();
  const LseOut o = *res_s;
  __syncthreads();
  return o;
}

// log-weights lw[i0 .. i0 + SCAN_IPT) through L2 (written by other blocks this
// step); -inf past n
__device__ __forceinline__ void load_tile_lw(const float *lw, int64_t i0, int64_t n, float (&v)[SCAN_IPT]) {
  static_assert(SCAN_IPT == 8, "two float4 loads per thread");
  if (i0 + SCAN_IPT <= n && (((uintptr_t)(lw + i0)) & 15) == 0) {
    const float4 a = __ldcg((const float4 *)(lw + i0));
    const float4 b = __ldcg((const float4 *)(lw + i0) + 1);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
  } else {
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) v[j] = i0 + j < n ? __ldcg(&lw[i0 + j]) : -INFINITY;
  }
}

// within-tile inclusive prefixes of particles base + threadIdx.x + PP_TPB r
// (r < SCAN_IPT; warp-contiguous), written by other blocks this step and so
// read through L2; past n they are never used
__device__ __forceinline__ void load_tile_cloc(const uint64_t *cloc, int64_t base, int64_t n,
                                               uint64_t (&X)[SCAN_IPT]) {
#pragma unroll
  for (int r = 0; r < SCAN_IPT; ++r) {
    const int64_t i = base + threadIdx.x + PP_TPB * r;
    X[r] = i < n ? __ldcg(&cloc[i]) : 0ull;
  }
}

// the linear-Gaussian model as a particle policy
template <int D, int DY>
struct LGModelP {
  static constexpr int kD = D, kDY = DY;
  LGP<D, DY> p;
  __device__ __forceinline__ uint32_t one() const { return p.one; }
  __device__ __forceinline__ float init(int64_t n, uint32_t ka, uint32_t kb, int64_t i, const float *y,
                                        float *__restrict__ x, float *__restrict__ lw) const {
    return lg_init_particle<D, DY>(p, n, ka, kb, i, y, x, lw);
  }
  __device__ __forceinline__ float step(int64_t n, uint32_t ka, uint32_t kb, int64_t i, const float (&xs)[D],
                                        float lres, const float *y, float, float *__restrict__ x,
                                        float *__restrict__ lw) const {
    return lg_particle_regs<D, DY>(p, n, ka, kb, i, xs, lres, y, x, lw);
  }
};

// P4 of a resampling step: every block scans the tile sums (identical result
// in every block), then writes the ancestors of the outputs of its own tiles.
// Particle j, with global inclusive prefix X_j, takes the outputs
// [K(X_{j-1}), K(X_j)), K the exact systematic threshold count
// (sys_count_small, branch-free); a tile's outputs are written RUN_WINDOW at
// a time through a shared window (runs marked, max-scanned, stored
// coalesced).  All global accesses are warp-contiguous.  Out of line: its
// registers then do not shape the allocation of the propagate loop, and the
// call costs a few register saves once per resampling step.
__device__ __noinline__ void resample_fill(const PersistArgs &a, int64_t t, int64_t n, int ntiles,
                                           int32_t *__restrict__ anc_n) {
  __shared__ uint64_t sP[PP_MAX_TILES];
  __shared__ unsigned long long smu[PP_TPB / 32];
  __shared__ int32_t sKt[SCAN_TILE];
  __shared__ __align__(16) int32_t stage[RUN_WINDOW];  // int4 accesses
  __shared__ int32_t wmax_s[PP_TPB / 32];
  __shared__ int32_t k0_s;
  const int G = (int)gridDim.x;
  const int per = (ntiles + PP_TPB - 1) / PP_TPB;
  const int b0 = threadIdx.x * per, b1 = min(b0 + per, ntiles);
  unsigned long long ts[4];
  unsigned long long run = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    ts[j] = (j < per && b0 + j < b1) ? __ldcg(&a.tile_sum[b0 + j]) : 0ull;
    run += ts[j];
  }
  unsigned long long Q;
  unsigned long long pre = block_excl_scan_u64(run, smu, Q);
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (j < per && b0 + j < b1) {
      sP[b0 + j] = pre;
      pre += ts[j];
    }
  const int degenerate = __ldcg(&a.degen[t]) || Q == 0;
  if (degenerate) {
    for (int64_t i = blockIdx.x * (int64_t)PP_TPB + threadIdx.x; i < n; i += (int64_t)G * PP_TPB) anc_n[i] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.err, EB_DEGENERATE);
  } else {
    const uint32_t m23 = bits_at(__ldg(&a.keys[2 * (t + 1)]), __ldg(&a.keys[2 * (t + 1) + 1]), 1, 0) >> 9;
    const float n_over_q = __fdiv_rn((float)n, (float)Q);
    __syncthreads();                 // sP
    stamp(a, t, 6);
    for (int tile = blockIdx.x; tile < ntiles; tile += G) {
      const int64_t base = (int64_t)tile * SCAN_TILE;
      const uint64_t P = sP[tile];
      uint64_t X[SCAN_IPT];
      load_tile_cloc(a.cloc, base, n, X);
      // K of the tile's particles (particle base + threadIdx.x + PP_TPB r);
      // past n, K = n (empty runs after the last particle, whose K is n)
#pragma unroll
      for (int r = 0; r < SCAN_IPT; ++r) {
        const int jj = threadIdx.x + PP_TPB * r;
        sKt[jj] = base + jj < n ? sys_count_small(P + X[r], (int32_t)n, m23, Q, n_over_q) : (int32_t)n;
      }
      if (threadIdx.x == 0) k0_s = sys_count_small(P, (int32_t)n, m23, Q, n_over_q);
      __syncthreads();
      const int32_t k0 = k0_s, k1 = sKt[SCAN_TILE - 1];
      for (int32_t w0 = k0; w0 < k1; w0 += RUN_WINDOW) {
        int4 *s4 = (int4 *)stage;
#pragma unroll
        for (int j = 0; j < RUN_WINDOW / 4 / PP_TPB; ++j) s4[threadIdx.x + PP_TPB * j] = make_int4(-1, -1, -1, -1);
        __syncthreads();
#pragma unroll
        for (int r = 0; r < SCAN_IPT; ++r) {
          const int jj = threadIdx.x + PP_TPB * r;
          const int32_t lo = jj ? sKt[jj - 1] : k0, hi = sKt[jj];
          const int32_t st = lo > w0 ? lo : w0;
          if (hi > st && st < w0 + RUN_WINDOW) stage[st - w0] = jj;
        }
        __syncthreads();
        window_max_scan(stage, wmax_s);
        __syncthreads();
        const int cnt = k1 - w0 < RUN_WINDOW ? k1 - w0 : RUN_WINDOW;
        // every slot is covered (slot 0 by the run through w0); the clamp only keeps a
        // wrong count from producing an out-of-range ancestor
        for (int q = threadIdx.x; q < cnt; q += PP_TPB) anc_n[w0 + q] = (int32_t)(base + max(stage[q], 0));
        __syncthreads();  // the window is cleared again, or sKt rewritten by the next tile
      }
    }
  }
}

template <class MP>
__global__ void __launch_bounds__(PP_TPB, 2) k_pf_persist(const __grid_constant__ MP p,
                                                           const __grid_constant__ PersistArgs a) {
  constexpr int D = MP::kD, DY = MP::kDY;
  __shared__ float smf[PP_TPB / 32];
  __shared__ unsigned long long smu[PP_TPB / 32];
  __shared__ LseOut res_s;
  __shared__ LsePartial wp_s[PP_TPB / 32];
  __shared__ float y_s[DY];
  const unsigned G = gridDim.x;
  const int64_t n = a.n, h = n >> 1;
  const int lane = threadIdx.x & 31;
  const int64_t wid = (int64_t)blockIdx.x * (PP_TPB / 32) + (threadIdx.x >> 5);
  const int nwarps = (int)G * (PP_TPB / 32);
  const int ntiles = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
  const float scale = __int_as_float((weight_shift(n) + 127) << 23);
  int res_cur = 0;
  double logz = 0.0, lse_prev = 0.0;

  for (int64_t t = 0; t < a.T; ++t) {
    if (timed_out(a.err)) break;
    stamp(a, t, 0);
    float *xo = persist_xbuf(a, t, D);
    float *lo = persist_lbuf(a, t);
    const float *xi = t == 0 ? nullptr : persist_xbuf(a, t - 1, D);
    const float *li = t == 0 ? nullptr : persist_lbuf(a, t - 1);

    const uint32_t k0 = __ldg(&a.keys[2 * t]), k1 = __ldg(&a.keys[2 * t + 1]);
    const float aux = a.aux ? __ldg(&a.aux[t]) : 0.0f;
    // observation of the step in shared memory (broadcast reads; keeps DY
    // registers free in the particle loop)
    if (threadIdx.x < DY) y_s[threadIdx.x] = __ldg(&a.y[t * DY + threadIdx.x]);
    const float *y = y_s;
    LsePartial *parts = a.parts + (t & 1) * PP_MAX_CHUNKS;

    // ---- P1: propagate + weight.  Warp w of the W warps of the grid takes the
    // 32-pair rounds w, w + W, w + 2W, ... (a static assignment: each partial
    // covers a fixed set of particles in a fixed order, so the combine does not
    // depend on timing), each lane keeps an online (max, sum e, sum e^2) across
    // its rounds, and at the end of the phase the block combines its warps'
    // partials in warp order into one.  No block-wide barrier inside the rounds:
    // a warp never waits for the block's slowest warp.
    __syncthreads();  // y_s
    const uint64_t t0 = (a.trace && t == 1 && threadIdx.x == 0) ? globaltimer_ns() : 0;
    {
      float m = -INFINITY, s1 = 0.0f, s2 = 0.0f;
      int nanf = 0;
      for (int64_t base = wid * 32; base < h; base += nwarps * 32) {
        const int64_t i = base + lane;
        if (i < h && t == 0) {
          uint32_t r0, r1, q0, q1;
          threefry2x32_m(k0, k1, (uint32_t)(2 * i), (uint32_t)(2 * i + n), p.one(), r0, r1);
          threefry2x32_m(k0, k1, (uint32_t)(2 * i + 1), (uint32_t)(2 * i + 1 + n), p.one(), q0, q1);
#pragma unroll 1
          for (int s = 0; s < 2; ++s) {
            const float l = p.init(n, s ? r1 : r0, s ? q1 : q0, s ? i + h : i, y, xo, lo);
            online_acc(l, m, s1, s2, nanf);
          }
        } else if (i < h) {
          // both particles' ancestors and source states are requested before the
          // key-split ciphers run, so the cipher arithmetic hides the gather latency
          // ancestors of this step (from the tape when one is recorded)
          const int32_t *anc_t = a.anc_hist ? a.anc_hist + (size_t)t * n : a.anc;
          const int64_t sa = res_cur ? (int64_t)__ldcg(&anc_t[i]) : i;
          const int64_t sb = res_cur ? (int64_t)__ldcg(&anc_t[i + h]) : i + h;
          float xa_[D], xb_[D];
#pragma unroll
          for (int j = 0; j < D; ++j) {
            xa_[j] = __ldcg(&xi[j * n + sa]);
            xb_[j] = __ldcg(&xi[j * n + sb]);
          }
          const float la_ = res_cur ? 0.0f : __ldcg(&li[i]);
          const float lb_ = res_cur ? 0.0f : __ldcg(&li[i + h]);
          uint32_t r0, r1, q0, q1;
          threefry2x32_m(k0, k1, (uint32_t)(2 * i), (uint32_t)(2 * i + n), p.one(), r0, r1);
          threefry2x32_m(k0, k1, (uint32_t)(2 * i + 1), (uint32_t)(2 * i + 1 + n), p.one(), q0, q1);
          // the pair runs as a two-trip loop (not unrolled): one copy of the
          // particle code keeps the hot loop inside the instruction cache
#pragma unroll 1
          for (int s = 0; s < 2; ++s) {
            float xs[D];
#pragma unroll
            for (int j = 0; j < D; ++j) xs[j] = s ? xb_[j] : xa_[j];
            const float l = p.step(n, s ? r1 : r0, s ? q1 : q0, s ? i + h : i, xs, s ? lb_ : la_, y, aux, xo, lo);
            online_acc(l, m, s1, s2, nanf);
          }
        }
      }
      // the block's 8 warp partials, combined in warp order: one partial per block
      const LsePartial wpart = warp_online_partial(m, s1, s2, nanf);
      if (lane == 0) wp_s[threadIdx.x >> 5] = wpart;
      __syncthreads();
      if (threadIdx.x < 32) {
        const LsePartial q = lane < PP_TPB / 32 ? wp_s[lane] : LsePartial{-INFINITY, 0.0f, 0.0f, 0};
        const LsePartial part = warp_partial_combine(q);
        if (lane == 0) parts[blockIdx.x] = part;
      }
    }
    if (a.trace && t == 1 && threadIdx.x == 0) a.trace[a.T * 10 + blockIdx.x] = globaltimer_ns() - t0;
    stamp(a, t, 1);
    // no phase runs on data that a barrier which did not complete failed to order
    if (grid_sync(a.bar, G, a.err)) break;
    stamp(a, t, 2);

    // ---- P2: combine (identical in every block)
    const LseOut o = combine_chunks<PP_TPB>(parts, (int)G, smf, &res_s);
    logz = t == 0 ? o.lse - a.logn : logz + o.lse - (res_cur ? a.logn : lse_prev);
    lse_prev = o.lse;
    const int res_next = ((float)o.ess < a.thr_n) ? 1 : 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.ess[t] = (float)o.ess;
      a.res[t] = res_cur;
      if (a.logz) *a.logz = logz;
    }
    stamp(a, t, 3);
    if (t + 1 == a.T) break;

    if (res_next) {
      const float M = o.M;
      // ancestors filled for the next step (into the tape when one is recorded)
      int32_t *anc_n = a.anc_hist ? a.anc_hist + (size_t)(t + 1) * n : a.anc;
      // ---- P3: per tile, exact fixed-point weights, their within-tile
      // inclusive prefixes (stored) and the tile sum.  The next tile's
      // log-weights are requested before this tile's scan, so a block with two
      // tiles waits for one L2 round trip instead of two.
      float v[SCAN_IPT];
      if ((int)blockIdx.x < ntiles) load_tile_lw(lo, (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT, n, v);
      for (int tile = blockIdx.x; tile < ntiles; tile += G) {
        const int64_t i0 = (int64_t)tile * SCAN_TILE + (int64_t)threadIdx.x * SCAN_IPT;
        float w[SCAN_IPT];
        if (tile + (int)G < ntiles) load_tile_lw(lo, i0 + (int64_t)G * SCAN_TILE, n, w);
        uint64_t q[SCAN_IPT];
        int bad = !(M > -INFINITY && M < INFINITY);
        uint64_t tsum = 0;
#pragma unroll
        for (int j = 0; j < SCAN_IPT; ++j) {
          bad |= (v[j] != v[j]) || (v[j] == INFINITY);
          q[j] = quantise_weight(v[j], M, scale);
          tsum += q[j];
        }
        unsigned long long btot;
        uint64_t c = block_excl_scan_u64(tsum, smu, btot);
#pragma unroll
        for (int j = 0; j < SCAN_IPT; ++j) {
          c += q[j];
          q[j] = c;
        }
        if (i0 + SCAN_IPT <= n) {
          ulonglong2 *dst = (ulonglong2 *)&a.cloc[i0];
#pragma unroll
          for (int j = 0; j < SCAN_IPT / 2; ++j) dst[j] = make_ulonglong2(q[2 * j], q[2 * j + 1]);
        } else {
#pragma unroll
          for (int j = 0; j < SCAN_IPT; ++j)
            if (i0 + j < n) a.cloc[i0 + j] = q[j];
        }
        bad = __syncthreads_or(bad);
        if (threadIdx.x == 0) {
          a.tile_sum[tile] = btot;
          if (bad) atomicOr(&a.degen[t], 1);
        }
#pragma unroll
        for (int j = 0; j < SCAN_IPT; ++j) v[j] = w[j];
      }
      stamp(a, t, 4);
      if (grid_sync(a.bar, G, a.err)) break;
      stamp(a, t, 5);

      // ---- P4: offspring runs of the next step (out of line, see resample_fill)
      resample_fill(a, t, n, ntiles, anc_n);
      stamp(a, t, 7);
      if (grid_sync(a.bar, G, a.err)) break;
      stamp(a, t, 8);
    }
    res_cur = res_next;
  }
}

// Bounded-wait self-tests: each makes one of the library's device waits run
// out on purpose, with no data behind it.  The barrier counts one more arrival
// than there are blocks (the missing block never comes); the lookback scans
// tile 1 while tile 0 never publishes its prefix.
__global__ void k_wait_selftest_barrier(GridBar *bar, int *err, int limit) {
  grid_sync(bar, gridDim.x + 1, err, limit);
}
__global__ void __launch_bounds__(SCAN_TPB) k_wait_selftest_lookback(uint64_t *status, int *err, int limit) {
  uint64_t v[SCAN_IPT];
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) v[j] = 1ull;
  uint64_t excl, total;
  tile_scan(v, 1u, status, err, excl, total, limit);
}

__global__ void k_or_err(const int *src, int *dst) {
  if (dst && *src) atomicOr(dst, *src);
}

// host: occupancy-sized cooperative launch
template <class MP>
static int launch_persist(const MP &p, const PersistArgs &args, cudaStream_t s) {
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ERR_CUDA;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return ERR_UNSUPPORTED;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pf_persist<MP>, PP_TPB, 0) != cudaSuccess ||
      per_sm < 1)
    return ERR_UNSUPPORTED;
  MP pc = p;
  PersistArgs a = args;
  void *kargs[] = {(void *)&pc, (void *)&a};
  // no more blocks than there are 256-pair propagate chunks: a small filter's grid
  // barriers then span a few blocks instead of every co-resident one
  const int64_t chunks = (args.n / 2 + PP_TPB - 1) / PP_TPB;
  int64_t cap = (int64_t)sms * per_sm;
  if (cap > PP_MAX_CHUNKS) cap = PP_MAX_CHUNKS;  // one LSE partial per block
  int64_t g = chunks < cap ? (chunks > 0 ? chunks : 1) : cap;
  // a small filter (a few 256-pair chunks of a low-dimensional model) runs in one block:
  // its steps are short enough that grid barriers between blocks would dominate them
  if (chunks * MP::kD <= 4) g = 1;
  const dim3 grid((unsigned)g), block(PP_TPB);
  if (cudaLaunchCooperativeKernel((void *)k_pf_persist<MP>, grid, block, kargs, 0, s) != cudaSuccess)
    return ERR_LAUNCH;
  k_or_err<<<1, 1, 0, s>>>(args.err, args.user_err);
  return launch_status();
}

#define MGB_PERSIST_CASE(D_, DY_) \
  if (m->d == D_ && m->dy == DY_) return launch_persist(LGModelP<D_, DY_>{pack_lg<D_, DY_>(m)}, a, s);

int run_lg_persistent(const mgb_lg_model *m, const PersistArgs &a, cudaStream_t s) {
  MGB_PERSIST_CASE(1, 1)
  MGB_PERSIST_CASE(2, 1)
  MGB_PERSIST_CASE(3, 1)
  MGB_PERSIST_CASE(4, 1)
  MGB_PERSIST_CASE(5, 1)
  MGB_PERSIST_CASE(8, 1)
  MGB_PERSIST_CASE(10, 1)
  MGB_PERSIST_CASE(2, 2)
  MGB_PERSIST_CASE(3, 3)
  MGB_PERSIST_CASE(4, 4)
  MGB_PERSIST_CASE(5, 5)
  MGB_PERSIST_CASE(8, 8)
  MGB_PERSIST_CASE(10, 10)
  return ERR_UNSUPPORTED;
}

int run_nl_persistent(const mgb_nl1d_model *m, const PersistArgs &a, cudaStream_t s) {
  return launch_persist(NLModelP{pack_nl(m)}, a, s);
}

int run_sv_persistent(const mgb_sv_model *m, const PersistArgs &a, cudaStream_t s) {
  return launch_persist(SVModelP{pack_sv(m)}, a, s);
}

}  // namespace mgb

using namespace mgb;

extern "C" size_t mgb_wait_selftest_workspace(void) { return 512; }

extern "C" int mgb_wait_selftest(int which, int32_t polls, void *ws, size_t ws_bytes, void *stream) {
  if ((which != MGB_WAIT_GRID_BARRIER && which != MGB_WAIT_LOOKBACK) || polls < 1 || polls > BAR_SPIN_LIMIT || !ws ||
      ws_bytes < mgb_wait_selftest_workspace())
    return ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  char *base = (char *)ws;
  int *err = (int *)base;                        // [0, 4)
  GridBar *bar = (GridBar *)(base + 128);        // [128, 384)
  uint64_t *status = (uint64_t *)(base + 384);   // [384, 400): tiles 0 and 1
  static_assert(128 + sizeof(GridBar) <= 384, "selftest layout");
  if (cudaMemsetAsync(ws, 0, 512, s) != cudaSuccess) return ERR_CUDA;
  if (which == MGB_WAIT_GRID_BARRIER)
    k_wait_selftest_barrier<<<4, 32, 0, s>>>(bar, err, polls);
  else
    k_wait_selftest_lookback<<<1, SCAN_TPB, 0, s>>>(status, err, polls);
  if (launch_status()) return ERR_LAUNCH;
  int h = 0;
  if (cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return ERR_CUDA;
  return (h & EB_TIMEOUT) ? ERR_DEVICE_TIMEOUT : OK;
}
