// Logistic-regression likelihood potential and its gradient for many
// parameter rows on the 5th-generation tensor cores (tcgen05, bf16 operands,
// fp32 accumulation in tensor memory), fused so that the (n_data x P) matrix
// of linear predictors never reaches HBM.
//
// For 128 parameter rows beta (one CTA) and the data streamed in 128-row tiles:
//   MMA1  Z = beta X_t^T          M = 128 rows, N = 128 data rows, K = 64 features
//   epi   pot += sum softplus(z) - y z;   R = sigmoid(Z) - y  (bf16, into tensor memory)
//   MMA2  G += R X_t              M = 128 rows, N = 64 features, K = 128 data rows
// Reference computation: the vmapped likelihood_potential_and_grad that
// mocat's MALA moves call (mocat/src/mcmc/standard_mcmc.py:121-131,
// mocat/src/utils.py:121-131) for the logistic scenario.
//
// Warp roles (576 threads): warp 0 issues the TMA loads of X tiles (128B
// swizzle) into a 4-stage ring; warp 1 owns tensor memory and issues the MMAs
// from one thread; warps 2-17 are the epilogue: warp w reads lane quarter
// w % 4 and one 32-column group of each Z tile with tcgen05.ld, so four warps
// per scheduler hide the latency of the transcendental epilogue.  Z is double-buffered in
// tensor memory (2 x 128 columns) so MMA1 of tile t+1 overlaps the epilogue of
// tile t; G takes 64 more columns.  Every mbarrier wait is bounded: a wait that
// runs out sets an error bit, raises a CTA-wide abort flag and the CTA drains.
// Operand layouts (K-major / MN-major, SWIZZLE_128B, 1024-byte aligned tiles):
//   beta tile  128 x 64 bf16 K-major    (written by the CTA from fp32 rows)
//   X tile     128 x 64 bf16 row-major: K-major B of MMA1, MN-major B of MMA2
//   R tile     128 x 128 bf16 in tensor memory (lane = parameter row, two data rows per
//              32-bit column), the A operand of MMA2 read from tensor memory
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "mgb_smc.cuh"

namespace mgb {

constexpr int TC_ROWS = 128;     // parameter rows per CTA (MMA M)
constexpr int TC_DT = 128;       // data rows per tile
constexpr int TC_K = 64;         // padded feature count
constexpr int TC_STAGES = 4;
constexpr int TC_EPI_WARPS = 16;  // 4 column groups x 4 tensor-memory lane quarters
constexpr int TC_THREADS = 64 + 32 * TC_EPI_WARPS;
constexpr uint32_t TC_TMEM_COLS = 512;
// tensor-memory columns: Z buffers 0 and 128, G 256 .. 319, R buffers (bf16 pairs) 320 and 384
constexpr uint32_t TC_R_COL = 320;
constexpr uint32_t TILE_BYTES = TC_DT * TC_K * 2;  // 16 KB
// alignment slack + beta tile + X ring + one tile of guard space (R lives in tensor memory)
constexpr size_t TC_SMEM = 1024 + TILE_BYTES + TC_STAGES * TILE_BYTES + TILE_BYTES;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false when it ran out or the CTA aborted
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, volatile int *abort) {
  for (uint32_t i = 0; i < TC_WAIT_LIMIT; ++i) {
    if (mbar_try(b, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  return false;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor, SWIZZLE_128B, both byte offsets 1024
// (8-row group stride; the other offset is unused for a 128-byte-wide atom)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(1024u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version
  d |= (uint64_t)2 << 61;  // SWIZZLE_128B
  return d;
}
// instruction descriptor, kind::f16: bf16 A/B, fp32 D, M x N, operand majorness
__host__ __device__ constexpr uint32_t bf16_idesc(int M, int N, bool a_mn, bool b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// the same MMA with A read from tensor memory (row i of A in lane i, two 16-bit K elements per
// 32-bit column): a_tmem is the address of the K-step's first column
__device__ __forceinline__ void mma_bf16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                            uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
#define MGB_TMEM_LD32(taddr, v)                                                                                    \
  asm volatile(                                                                                                    \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, " \
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"              \
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),          \
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),    \
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),  \
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])   \
      : "r"(taddr))
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// 16 consecutive 32-bit columns of this thread's lane
#define MGB_TMEM_ST16(taddr, v)                                                                                  \
  asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, " \
               "%13, %14, %15, %16};" ::"r"(taddr),                                                             \
               "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), \
               "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])                \
               : "memory")
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// byte offset of element (row, col) of a 64-column bf16 K-major SWIZZLE_128B tile
__device__ __forceinline__ uint32_t sw128_off(int row, int col) {
  return (uint32_t)row * 128u + ((((uint32_t)col >> 3) ^ ((uint32_t)row & 7u)) << 4) + (((uint32_t)col & 7u) << 1);
}

__device__ __forceinline__ float exp2f_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float log2f_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *(const uint32_t *)&h;
}

// Epilogue of one pair of linear predictors z (labels y in {0, 1}):
//   potential term softplus(z) - y z = max(w, 0) + log(1 + exp(-|z|)), w = (1 - 2y) z:
//   s_lin += max(w, 0); prod *= (1 + exp(-|z|)) (one log2 of the product per 32 columns);
//   gradient operand r = sigmoid(z) - y = tanh(z / 2) / 2 + (1/2 - y), packed bf16x2.
// A padding column passes z = -inf, y = 0: it adds 0 to both sums.
// softplus(w) = max(w, 0) + log(1 + e^-|z|) with w = (1 - 2y) z, and sum_j max(w_j, 0) =
// (sum_j w_j + sum_j |z_j|) / 2 where sum_j w_j = beta . u, u = X^T (1 - 2y) (added once per
// row): per element only |z| is accumulated (a0, a1: |z| of valid columns, 0 past n_data)
// c = (0.5 - y0, 0.5 - y1) as bf16x2 comes precomputed per column pair (k_logreg_cw); the
// even and odd columns keep separate products (two independent multiply chains)
__device__ __forceinline__ void epi_pair(float z0, float z1, float a0, float a1, uint32_t c, float &s_abs,
                                         float &prod0, float &prod1, uint32_t &packed) {
  s_abs += a0 + a1;
  const float e0 = exp2f_approx(-1.4426950408889634f * fabsf(z0));
  const float e1 = exp2f_approx(-1.4426950408889634f * fabsf(z1));
  prod0 = fmaf(prod0, e0, prod0);
  prod1 = fmaf(prod1, e1, prod1);
  uint32_t zh = pack_bf16(z0, z1), h;
  asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(zh) : "r"(zh), "r"(0x3F003F00u));  // z / 2 (exact)
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(h) : "r"(zh));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(packed) : "r"(h), "r"(0x3F003F00u), "r"(c));
}

struct TCArgs {
  const float *beta;
  const float *y;
  const float *u;  // (TC_K) X^T (1 - 2y) from the bf16 rows
  const uint4 *cw;  // (tiles x 16) bf16x2 words (0.5 - y_2p, 0.5 - y_2p+1), 4 per 8 columns
  const int32_t *active;
  float *lik, *grad;
  int *err;
  int64_t P, n_data;
  int d, N;
};

__global__ void __launch_bounds__(TC_THREADS, 1) k_logreg_tc(const __grid_constant__ CUtensorMap xmap,
                                                             const __grid_constant__ TCArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_xfull[TC_STAGES], bar_xempty[TC_STAGES];
  __shared__ __align__(8) uint64_t bar_zfull[2], bar_zempty[2], bar_rfull[2], bar_rempty[2], bar_gdone;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ double pot_s[4][TC_ROWS];
  __shared__ int grad_ok_s;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row0 = (int64_t)blockIdx.x * TC_ROWS;

  // nothing to do when every posterior of this tile has finished
  if (a.active) {
    bool any = false;
    const int64_t last = min(row0 + TC_ROWS, a.P) - 1;
    for (int64_t b = row0 / a.N; b <= last / a.N; ++b) any |= a.active[b] != 0;
    if (!any) return;
  }

  unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char *sA = base;                        // beta tile
  unsigned char *sX = sA + TILE_BYTES;             // X ring

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&bar_xfull[s], 1);
      mbar_init(&bar_xempty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&bar_zfull[b], 1);
      mbar_init(&bar_zempty[b], 32 * TC_EPI_WARPS);
      mbar_init(&bar_rfull[b], 32 * TC_EPI_WARPS);
      mbar_init(&bar_rempty[b], 1);
    }
    mbar_init(&bar_gdone, 1);
    abort_flag = 0;
    grad_ok_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  // beta rows -> bf16 K-major swizzled tile (zero rows past P / of finished posteriors, zero columns past d)
  for (int u = threadIdx.x; u < TC_ROWS * (TC_K / 8); u += TC_THREADS) {
    const int r = u >> 3, ch = u & 7;
    const int64_t p = row0 + r;
    const bool live = p < a.P && (!a.active || a.active[p / a.N]);
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int c = ch * 8 + e;
      v[e] = (live && c < a.d) ? a.beta[p * a.d + c] : 0.0f;
    }
    uint4 q;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    *(uint4 *)(sA + sw128_off(r, ch * 8)) = q;
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t tg = tmem + 256u;  // Z buffers at columns 0 and 128, G at 256
  const int nt = (int)((a.n_data + TC_DT - 1) / TC_DT);

  if (warp == 0) {
    // ---------------------------------------------------------------- TMA producer
    if (lane == 0) {
      for (int t = 0; t < nt; ++t) {
        const int s = t % TC_STAGES;
        if (!mbar_wait(&bar_xempty[s], ((t / TC_STAGES) & 1) ^ 1, &abort_flag)) break;
        mbar_expect_tx(&bar_xfull[s], TILE_BYTES);
        tma_load_2d(sX + s * TILE_BYTES, &xmap, 0, t * TC_DT, &bar_xfull[s]);
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issuer
    if (lane == 0) {
      const uint32_t id1 = bf16_idesc(128, 128, false, false);
      const uint32_t id2 = bf16_idesc(128, 64, false, true);
      const uint32_t aA = smem_u32(sA);
      bool ok = true;
      for (int t = 0; t <= nt && ok; ++t) {
        if (t < nt) {
          const int s = t % TC_STAGES, zb = t & 1;
          ok = mbar_wait(&bar_xfull[s], (t / TC_STAGES) & 1, &abort_flag) &&
               mbar_wait(&bar_zempty[zb], ((t >> 1) & 1) ^ 1, &abort_flag);
          if (!ok) break;
          tc_fence_after();
          const uint32_t aX = smem_u32(sX + s * TILE_BYTES);
#pragma unroll
          for (int k = 0; k < TC_K / 16; ++k)
            mma_bf16(tmem + zb * 128u, sw128_desc(aA + k * 32), sw128_desc(aX + k * 32), id1, k > 0 ? 1u : 0u);
          mma_commit(&bar_zfull[zb]);
        }
        if (t >= 1) {
          const int u = t - 1, rb = u & 1, s = u % TC_STAGES;
          ok = mbar_wait(&bar_rfull[rb], (u >> 1) & 1, &abort_flag);
          if (!ok) break;
          tc_fence_after();
          const uint32_t tR = tmem + TC_R_COL + (uint32_t)rb * (TC_DT / 2);
          const uint32_t aX = smem_u32(sX + s * TILE_BYTES);
#pragma unroll
          for (int k = 0; k < TC_DT / 16; ++k)
            mma_bf16_ta(tg, tR + (uint32_t)k * 8u, sw128_desc(aX + k * 2048), id2, (u > 0 || k > 0) ? 1u : 0u);
          mma_commit(&bar_xempty[s]);
          mma_commit(&bar_rempty[rb]);
        }
      }
      mma_commit(&bar_gdone);
    }
  } else {
    // ---------------------------------------------------------------- epilogue
    // warp w reads lane quarter w % 4 (the hardware's rule) and column group
    // (w - 2) / 4 of 32 columns of every tile
    const int q = warp & 3;
    const int cg = (warp - 2) >> 2;
    const int row = q * 32 + lane;      // parameter row within the tile
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    double pot = 0.0;
    float pot_f = 0.0f;  // 16 tiles at a time in float, then into the double
    bool ok = true;
    // this warp's 16 label words of tile t: cw[t * 16 + cg * 4 .. + 4] (uniform across lanes)
    uint4 cnext[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) cnext[m] = __ldg(&a.cw[cg * 4 + m]);
    for (int t = 0; t < nt && ok; ++t) {
      const int zb = t & 1, rb = t & 1;
      uint4 ccur[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) ccur[m] = cnext[m];
      if (t + 1 < nt) {
#pragma unroll
        for (int m = 0; m < 4; ++m) cnext[m] = __ldg(&a.cw[(int64_t)(t + 1) * 16 + cg * 4 + m]);
      }
      ok = mbar_wait(&bar_zfull[zb], (t >> 1) & 1, &abort_flag) &&
           mbar_wait(&bar_rempty[rb], ((t >> 1) & 1) ^ 1, &abort_flag);
      if (!ok) break;
      tc_fence_after();
      uint32_t v[32];
      MGB_TMEM_LD32(tmem + zb * 128u + lane_off + (uint32_t)(cg * 32), v);
      tmem_ld_wait();
      tc_fence_before();
      mbar_arrive(&bar_zempty[zb]);
      const int64_t i0 = (int64_t)t * TC_DT + cg * 32;
      const int nvalid = (int)min((int64_t)32, a.n_data - i0);
      const uint32_t cwd[16] = {ccur[0].x, ccur[0].y, ccur[0].z, ccur[0].w, ccur[1].x, ccur[1].y, ccur[1].z, ccur[1].w,
                                ccur[2].x, ccur[2].y, ccur[2].z, ccur[2].w, ccur[3].x, ccur[3].y, ccur[3].z, ccur[3].w};
      float s_abs = 0.0f, prod0 = 1.0f, prod1 = 1.0f;
      uint32_t packed[16];
      if (nvalid == 32) {
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
          const float z0 = __uint_as_float(v[j]), z1 = __uint_as_float(v[j + 1]);
          epi_pair(z0, z1, fabsf(z0), fabsf(z1), cwd[j >> 1], s_abs, prod0, prod1, packed[j >> 1]);
        }
      } else {
        // columns past n_data: z = -inf (adds 0 to both sums), label word 0.5 (y = 0)
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
          const bool ok0 = j < nvalid, ok1 = j + 1 < nvalid;
          const float z0 = __uint_as_float(v[j]), z1 = __uint_as_float(v[j + 1]);
          epi_pair(ok0 ? z0 : -INFINITY, ok1 ? z1 : -INFINITY, ok0 ? fabsf(z0) : 0.0f, ok1 ? fabsf(z1) : 0.0f,
                   cwd[j >> 1], s_abs, prod0, prod1, packed[j >> 1]);
          if (!ok1) packed[j >> 1] &= ok0 ? 0x0000FFFFu : 0u;
        }
      }
      const float s_l2 = log2f_approx(prod0 * prod1);
      const float tsum = fmaf(0.69314718055994531f, s_l2, 0.5f * s_abs);
      // R of this lane's row, data columns cg*32 .. +32 as bf16 pairs: tensor-memory columns
      // cg*16 .. +16 of R buffer rb (the A operand of MMA2)
      MGB_TMEM_ST16(tmem + TC_R_COL + (uint32_t)rb * (TC_DT / 2) + lane_off + (uint32_t)(cg * 16), packed);
      tmem_st_wait();
      tc_fence_before();
      mbar_arrive(&bar_rfull[rb]);
      pot_f += tsum;
      if ((t & 15) == 15) {
        pot += (double)pot_f;
        pot_f = 0.0f;
      }
    }
    pot += (double)pot_f;
    pot_s[cg][row] = pot;
    if (cg == 0 && ok && mbar_wait(&bar_gdone, 0, &abort_flag)) {
      tc_fence_after();
      uint32_t g0[32], g1[32];
      MGB_TMEM_LD32(tg + lane_off, g0);
      MGB_TMEM_LD32(tg + lane_off + 32u, g1);
      tmem_ld_wait();
      grad_ok_s = 1;
      const int64_t p = row0 + row;
      if (p < a.P && (!a.active || a.active[p / a.N])) {
#pragma unroll
        for (int k = 0; k < 32; ++k) {
          if (k < a.d) a.grad[p * a.d + k] = __uint_as_float(g0[k]);
          if (k + 32 < a.d) a.grad[p * a.d + k + 32] = __uint_as_float(g1[k]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (abort_flag && threadIdx.x == 0 && a.err) atomicOr(a.err, 1);
  // potential: the four column groups of each row
  if (threadIdx.x < TC_ROWS && grad_ok_s) {
    const int64_t p = row0 + threadIdx.x;
    if (p < a.P && (!a.active || a.active[p / a.N])) {
      // 0.5 sum_j w_j = 0.5 bf16(beta_p) . u (the MMA's operands)
      float bu = 0.0f;
      for (int k = 0; k < a.d; ++k) bu = fmaf(__bfloat162float(__float2bfloat16_rn(a.beta[p * a.d + k])), a.u[k], bu);
      a.lik[p] = (float)(pot_s[0][threadIdx.x] + pot_s[1][threadIdx.x] + pot_s[2][threadIdx.x] +
                         pot_s[3][threadIdx.x] + 0.5 * (double)bu);
    }
  }
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------- host side
static int encode_xmap(CUtensorMap *map, const uint16_t *Xb, int64_t n_data) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return ERR_UNSUPPORTED;
    encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)TC_K, (cuuint64_t)n_data};
  const cuuint64_t strides[1] = {(cuuint64_t)TC_K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)TC_K, (cuuint32_t)TC_DT};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)Xb, dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? OK : ERR_BAD_ARG;
}

// u = X^T (1 - 2y) over the bf16 rows, in a fixed order: block b sums rows of its chunk
// (4 row lanes per feature, then the lanes in order), a second kernel sums the blocks in order
constexpr int TC_UBLOCKS = 64;
__global__ void __launch_bounds__(256) k_logreg_u_part(const uint16_t *Xb, const float *y, int64_t n_data,
                                                        float *partial) {
  __shared__ float sm[4][TC_K];
  const int k = threadIdx.x & (TC_K - 1), r = threadIdx.x / TC_K;
  const int64_t chunk = (n_data + TC_UBLOCKS - 1) / TC_UBLOCKS;
  const int64_t j0 = blockIdx.x * chunk, j1 = j0 + chunk < n_data ? j0 + chunk : n_data;
  float acc = 0.0f;
  for (int64_t j = j0 + r; j < j1; j += 4) {
    const float x = __uint_as_float((uint32_t)Xb[j * TC_K + k] << 16);
    acc = __ldg(&y[j]) != 0.0f ? acc - x : acc + x;
  }
  sm[r][k] = acc;
  __syncthreads();
  if (threadIdx.x < TC_K) partial[blockIdx.x * TC_K + k] = ((sm[0][k] + sm[1][k]) + sm[2][k]) + sm[3][k];
}
__global__ void k_logreg_u_sum(const float *partial, float *u) {
  float s = 0.0f;
  for (int b = 0; b < TC_UBLOCKS; ++b) s += partial[b * TC_K + threadIdx.x];
  u[threadIdx.x] = s;
}

// label words: cw[t * 64 + p] = bf16x2 (0.5 - y_{2p}, 0.5 - y_{2p+1}) of tile t's columns 2p, 2p+1
// (y = 0 past n_data), the constant of the epilogue's r = tanh(z/2)/2 + (0.5 - y)
__global__ void k_logreg_cw(const float *y, int64_t n_data, int64_t nwords, uint32_t *cw) {
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nwords; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = 2 * w;
    const uint32_t y0 = (j < n_data && y[j] != 0.0f) ? 1u : 0u;
    const uint32_t y1 = (j + 1 < n_data && y[j + 1] != 0.0f) ? 1u : 0u;
    cw[w] = 0x3F003F00u | (y0 << 15) | (y1 << 31);
  }
}

// err word, block partials of u, u, label words (one 16-byte aligned slab)
static size_t cw_offset() { return ((256 + sizeof(float) * (TC_UBLOCKS + 1) * TC_K) + 255) & ~(size_t)255; }
size_t logreg_tc_workspace(int64_t, int64_t n_data, int) {
  const int64_t nt = (n_data + TC_DT - 1) / TC_DT;
  return cw_offset() + sizeof(uint32_t) * (size_t)nt * (TC_DT / 2);
}

int logreg_tc(const SMCData &dat, const float *beta, int64_t P, const int32_t *active, int N, float *lik, float *grad,
              void *ws, size_t ws_bytes, cudaStream_t s) {
  if (dat.d > TC_K || !dat.Xb || ((uintptr_t)dat.Xb & 15u) || ws_bytes < logreg_tc_workspace(P, dat.n_data, dat.d))
    return ERR_BAD_ARG;
  CUtensorMap map;
  int st = encode_xmap(&map, dat.Xb, dat.n_data);
  if (st) return st;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_logreg_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM) != cudaSuccess)
      return ERR_UNSUPPORTED;
    attr = true;
  }
  int *err = (int *)ws;
  float *partial = (float *)((char *)ws + 256), *u = partial + TC_UBLOCKS * TC_K;
  if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return ERR_CUDA;
  k_logreg_u_part<<<TC_UBLOCKS, 256, 0, s>>>(dat.Xb, dat.y, dat.n_data, partial);
  k_logreg_u_sum<<<1, TC_K, 0, s>>>(partial, u);
  const int64_t nwords = ((dat.n_data + TC_DT - 1) / TC_DT) * (TC_DT / 2);
  uint32_t *cw = (uint32_t *)((char *)ws + cw_offset());
  k_logreg_cw<<<grid_for(nwords, 256), 256, 0, s>>>(dat.y, dat.n_data, nwords, cw);
  if ((st = launch_status())) return st;
  TCArgs a{beta, dat.y, u, (const uint4 *)cw, active, lik, grad, err, P, dat.n_data, dat.d, N > 0 ? N : (int)P};
  const unsigned grid = (unsigned)((P + TC_ROWS - 1) / TC_ROWS);
  k_logreg_tc<<<grid, TC_THREADS, TC_SMEM, s>>>(map, a);
  return launch_status();
}

}  // namespace mgb
