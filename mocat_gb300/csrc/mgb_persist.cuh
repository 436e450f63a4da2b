// Whole-filter persistent kernel: arguments shared with the driver.
#pragma once
#include "mgb_internal.cuh"

namespace mgb {

constexpr int PP_TPB = 256;
constexpr int PP_MAX_TILES = 1024;  // n <= 2^21 on this path
constexpr int BAR_SPIN_LIMIT = 1 << 22;  // polls of an L2 word (>= ~0.5 us each under load): seconds
constexpr int PP_MAX_CHUNKS = 4096;  // 256-pair chunks per step (n <= 2^21)

struct GridBar {
  unsigned int count;
  unsigned int gen;
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
  int *chunk_ctr;                 // (T,) chunk counters (zeroed)
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
};

int run_lg_persistent(const mgb_lg_model *m, const PersistArgs &a, cudaStream_t s);

}  // namespace mgb
