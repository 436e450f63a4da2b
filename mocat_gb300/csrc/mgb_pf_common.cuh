// Pieces shared by the launch-per-step particle-filter drivers (bootstrap
// linear-Gaussian, optimal proposal): running state, the fused block reduction
// whose last block finalises a step (logsumexp / ESS, log Z, next step's
// resampling decision), and the run workspace.
#pragma once
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_kernels.cuh"

namespace mgb {

struct PFState {
  double logz;
  double lse_prev;
  float M;
  int pad;
};

// per-run control block passed by value to the fused kernels
struct PFCtl {
  LsePartial *parts;
  unsigned int *counter;
  PFState *st;
  float *ess_hist;     // (T,)
  int32_t *res_hist;   // (T+1,): entry t = 1 if step t resamples
  ResampleCtl *rctl;   // cleared by the finalising block for the next step
  uint64_t *rstatus, *rstatus2;
  int ntiles;
  float thr_n;         // ess_threshold * n (float32, as the reference compares)
  double logn;
  double *logz_out;
};

constexpr int PF_TPB = 256;

// last block: combine partials, update the running state, clear scratch
template <int TPB>
__device__ __forceinline__ void pf_finalize(const PFCtl &ctl, int64_t t, float *smf, double *smd) {
  const LseOut o = combine_lse<TPB>(ctl.parts, gridDim.x, smf, smd);
  if (threadIdx.x == 0) {
    PFState *st = ctl.st;
    const int res_t = t == 0 ? 0 : ctl.res_hist[t];
    const double logz = t == 0 ? o.lse - ctl.logn : st->logz + o.lse - (res_t ? ctl.logn : st->lse_prev);
    st->logz = logz;
    st->lse_prev = o.lse;
    st->M = o.M;
    ctl.ess_hist[t] = (float)o.ess;
    ctl.res_hist[t + 1] = ((float)o.ess < ctl.thr_n) ? 1 : 0;
    if (ctl.logz_out) *ctl.logz_out = logz;
    *ctl.counter = 0u;
    ctl.rctl->tile_counter = 0u;
    ctl.rctl->tile_counter2 = 0u;
    ctl.rctl->degenerate = 0;
    ctl.rctl->total = 0ull;
  }
  for (int j = threadIdx.x; j < ctl.ntiles; j += TPB) {
    ctl.rstatus[j] = 0ull;
    ctl.rstatus2[j] = 0ull;
  }
  if (threadIdx.x == 0) ctl.rctl->units = 0u;
}

// block partial + (optionally) last-block finalize
template <int TPB>
__device__ __forceinline__ void pf_reduce(float lw, bool active, const PFCtl &ctl, int64_t t) {
  __shared__ float smf[TPB / 32];
  __shared__ double smd[TPB / 32];
  __shared__ bool last;
  const bool nan = active && lw != lw;
  const LsePartial part = block_lse_partial<TPB>(active && !nan ? lw : -INFINITY, nan, smf, smd);
  if (threadIdx.x == 0) {
    ctl.parts[blockIdx.x] = part;
    last = last_block_arrival(ctl.counter);
  }
  __syncthreads();
  if (!last) return;
  pf_finalize<TPB>(ctl, t, smf, smd);
}

template <int TPB>
__device__ __forceinline__ void pf_reduce_online(float m, float s1, float s2, int nanf, const PFCtl &ctl, int64_t t) {
  __shared__ float smf[TPB / 32];
  __shared__ double smd[TPB / 32];
  __shared__ bool last;
  const LsePartial part = block_online_partial<TPB>(m, s1, s2, nanf, smf);
  if (threadIdx.x == 0) {
    ctl.parts[blockIdx.x] = part;
    last = last_block_arrival(ctl.counter);
  }
  __syncthreads();
  if (!last) return;
  pf_finalize<TPB>(ctl, t, smf, smd);
}

// ------------------------------------------------------------- host side
struct RunWs {
  uint32_t *keys;
  PFState *st;
  LsePartial *parts;
  unsigned int *counter;
  int32_t *res_hist;
  float *ess_hist;
  float *xa, *xb, *la, *lb;
  int32_t *anc;
  ResampleWs rws;
};

inline RunWs carve_run(Carver &c, int64_t n, int64_t T, int d, int scheme, bool need_x, bool need_lw, bool need_ess) {
  RunWs w;
  w.keys = c.take<uint32_t>(2 * (size_t)T);
  w.st = c.take<PFState>(1);
  w.parts = c.take<LsePartial>((size_t)((n + PF_TPB - 1) / PF_TPB));
  w.counter = c.take<unsigned int>(1);
  w.res_hist = c.take<int32_t>((size_t)T + 1);
  w.ess_hist = need_ess ? c.take<float>((size_t)T) : nullptr;
  w.xa = need_x ? c.take<float>((size_t)d * n) : nullptr;
  w.xb = need_x ? c.take<float>((size_t)d * n) : nullptr;
  w.la = need_lw ? c.take<float>((size_t)n) : nullptr;
  w.lb = need_lw ? c.take<float>((size_t)n) : nullptr;
  w.anc = c.take<int32_t>((size_t)n);
  w.rws = carve_resample(c, n, scheme);
  return w;
}


// key schedule of run_particle_filter_for_marginals (filtering.py:267-278):
// (random_key, sub_key) = split(key); step keys = split(random_key, T - 1).
// out[0..1] = sub_key, out[2t..2t+1] = key of step t (t >= 1).
int launch_setup_keys(const uint32_t *key, int64_t T, uint32_t *out, cudaStream_t s);
// logz <- st->logz; resampled[t] <- res_hist[t] (0 at t = 0)
int launch_finish(const PFState *st, const int32_t *res_hist, int64_t T, double *logz, int32_t *resampled,
                  cudaStream_t s);

}  // namespace mgb
