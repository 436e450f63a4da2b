// Whole-filter persistent kernel: arguments and workspace shared with the
// drivers of the models that run on it.
#pragma once
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_pf_common.cuh"

namespace mgb {

constexpr int PP_TPB = 256;
constexpr int PP_MAX_TILES = 1024;  // n <= 2^21 on this path
constexpr int BAR_SPIN_LIMIT = 1 << 22;  // polls of an L2 word (>= ~0.5 us each under load): seconds
constexpr int PP_MAX_CHUNKS = 4096;  // 256-pair chunks per step (n <= 2^21)

// arrival counter and generation on separate 128-byte lines: the waiters' polling loads
// of gen do not queue behind the arrivals' atomics on count
struct GridBar {
  unsigned int count;
  unsigned int pad0[31];
  unsigned int gen;
  unsigned int pad1[31];
};

struct PersistArgs {
  int64_t n, T;
  const uint32_t *keys;  // (T, 2): [0] initial sub-key, [t] key of step t
  const float *y;        // (T, dy)
  float thr_n;
  double logn;
  float *xa, *xb, *la, *lb;       // ping-pong buffers (unused slots of a history)
  float *x_hist, *lw_hist;        // (T, d, n), (T, n) or null
  int32_t *anc;
  LsePartial *parts;              // 2 * PP_MAX_CHUNKS (one per chunk, double-buffered by step parity)
  uint64_t *cloc;                 // (n,) within-tile inclusive fixed-point prefixes
  uint64_t *tile_sum;             // tiles
  int *degen;                     // (T,) degenerate-weights flag per step
  GridBar *bar;
  float *ess;                     // (T,)
  int32_t *res;                   // (T,)
  double *logz;                   // scalar (may be null)
  int *err;                       // the kernel's own error word (workspace, zeroed)
  int *user_err;                  // caller's error word (may be null): err is OR-ed into it
  unsigned long long magic;       // floor((2^64 - 1) / n)
  uint64_t *trace;                // (T, 8) phase timestamps from block 0, or null
  const float *aux;               // (T,) per-step constant of the model (may be null)
  // taped runs (the adjoint's forward pass): ancestors of every step into anc_hist
  // (T, n) instead of anc, and (x, lw) of every ck_every-th step into the
  // checkpoint slots ckx (T / ck_every, d, n) / ckl instead of the ping-pong buffers
  int32_t *anc_hist;
  int64_t ck_every;
  float *ckx, *ckl;
};

// particles / log-weights of step s: the history, a checkpoint slot, or a ping-pong buffer
__host__ __device__ inline float *persist_xbuf(const PersistArgs &a, int64_t s, int d) {
  if (a.x_hist) return a.x_hist + (size_t)s * d * a.n;
  if (a.ck_every && s % a.ck_every == 0) return a.ckx + (size_t)(s / a.ck_every) * d * a.n;
  return (s & 1) ? a.xb : a.xa;
}
__host__ __device__ inline float *persist_lbuf(const PersistArgs &a, int64_t s) {
  if (a.lw_hist) return a.lw_hist + (size_t)s * a.n;
  if (a.ck_every && s % a.ck_every == 0) return a.ckl + (size_t)(s / a.ck_every) * a.n;
  return (s & 1) ? a.lb : a.la;
}

// Persistent path: systematic resampling, even n, n <= 2^21 (tile prefixes in
// smem; the branch-free offspring count is exact up to that size).
static_assert((int64_t)PP_MAX_TILES * SCAN_TILE <= SYS_COUNT_SMALL_MAX_N, "sys_count_small bound");
inline bool persistent_ok(int64_t n, int scheme) {
  return scheme == MGB_RESAMPLE_SYSTEMATIC && n % 2 == 0 && (n + SCAN_TILE - 1) / SCAN_TILE <= PP_MAX_TILES;
}

struct PersistWs {
  LsePartial *parts;
  uint64_t *cloc;
  uint64_t *tile_sum;
  int *degen;
  GridBar *bar;
  int32_t *res;
  int *err;
};

inline PersistWs carve_persist(Carver &c, int64_t n, int64_t T) {
  PersistWs w;
  w.parts = c.take<LsePartial>(2 * PP_MAX_CHUNKS);
  w.cloc = c.take<uint64_t>((size_t)n);
  w.tile_sum = c.take<uint64_t>((size_t)((n + SCAN_TILE - 1) / SCAN_TILE));
  w.degen = c.take<int>((size_t)T);
  w.bar = c.take<GridBar>(1);
  w.res = c.take<int32_t>((size_t)T);
  w.err = c.take<int>(1);
  return w;
}

// zeroes the per-run state and fills the arguments every model shares; x_hist /
// lw_hist are used when the caller asked for histories
inline int persist_setup(const RunWs &w, const PersistWs &pw, int64_t n, int64_t T, const float *y, float thr,
                         float *ess, const mgb_pf_outputs *out, PersistArgs &a, cudaStream_t s) {
  if (cudaMemsetAsync(pw.degen, 0, sizeof(int) * T, s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(pw.bar, 0, sizeof(GridBar), s) != cudaSuccess) return ERR_CUDA;
  if (cudaMemsetAsync(pw.err, 0, sizeof(int), s) != cudaSuccess) return ERR_CUDA;
  const bool hx = out && out->x_hist, hl = out && out->lw_hist;
  a.n = n;
  a.T = T;
  a.keys = w.keys;
  a.y = y;
  a.thr_n = thr * (float)n;
  a.logn = log((double)n);
  a.xa = w.xa;
  a.xb = w.xb;
  a.la = w.la;
  a.lb = w.lb;
  a.x_hist = hx ? out->x_hist : nullptr;
  a.lw_hist = hl ? out->lw_hist : nullptr;
  a.anc = w.anc;
  a.parts = pw.parts;
  a.cloc = pw.cloc;
  a.tile_sum = pw.tile_sum;
  a.degen = pw.degen;
  a.bar = pw.bar;
  a.ess = ess;
  a.res = (out && out->resampled) ? out->resampled : pw.res;
  a.logz = out ? out->log_z : nullptr;
  a.err = pw.err;
  a.user_err = out ? out->err : nullptr;
  a.magic = ~0ull / (unsigned long long)n;
  a.trace = out ? out->trace : nullptr;
  a.aux = nullptr;
  a.anc_hist = nullptr;
  a.ck_every = 0;
  a.ckx = a.ckl = nullptr;
  return OK;
}

// copies the last step's particles / log-weights to x_final / lw_final when asked
inline int persist_finish(const PersistArgs &a, int d, const mgb_pf_outputs *out, cudaStream_t s) {
  const int64_t n = a.n, T = a.T;
  const float *xl = persist_xbuf(a, T - 1, d);
  const float *ll = persist_lbuf(a, T - 1);
  if (out && out->x_final &&
      cudaMemcpyAsync(out->x_final, xl, sizeof(float) * d * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  if (out && out->lw_final &&
      cudaMemcpyAsync(out->lw_final, ll, sizeof(float) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return ERR_CUDA;
  return OK;
}

int run_lg_persistent(const mgb_lg_model *m, const PersistArgs &a, cudaStream_t s);
// the one-dimensional non-linear benchmark model; a.aux = 8 cos(1.2 t_{t-1}) per step
int run_nl_persistent(const mgb_nl1d_model *m, const PersistArgs &a, cudaStream_t s);
// stochastic volatility, dim 1; a.aux = transition_covariance_sqrt sqrt(t_t - t_{t-1}) per step
int run_sv_persistent(const mgb_sv_model *m, const PersistArgs &a, cudaStream_t s);

}  // namespace mgb
