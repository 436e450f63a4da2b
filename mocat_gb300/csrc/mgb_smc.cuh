// Shared declarations of the tempered-SMC translation units: the device view
// of the sampler's workspace, the per-posterior parameters and the logistic
// regression data (float32 rows and the bf16 copy used by the tensor cores).
#pragma once
#include "mgb_internal.cuh"

namespace mgb {

struct SMCView {
  int32_t B, N, D, H;
  float *beta, *beta_p;      // (B N, D) state / proposal rows
  float *glik, *glik_p;      // (B N, D) likelihood-potential gradients
  float *mom, *phalf;        // (B N, D) momentum at the move's start, half-step momentum of the proposal
  float *ms, *ms_p;          // (B N, D) Underdamped momenta kept between moves (and their gathered copy)
  float *lik, *lik_p, *lik_w;  // (B N) likelihood potential: state, proposal, (U - prior) / tau
  float *lw, *alpha;         // (B N) log-weights, acceptance-probability sums
  uint32_t *pkey;            // (B N, 2) MCMC keys
  int32_t *anc;              // (B N) ancestors within each posterior
  float *tau, *ess;          // (B)
  double *logz;              // (B) log_norm_constant
  uint32_t *key, *key_next, *rkey;  // (B, 2) sampler key, next key, resampling key
  int32_t *iter, *active, *resampled;  // (B)
  float *h_tau, *h_ess, *h_alpha;  // (B, H) per-iteration history
  double *h_logz;
  int32_t *h_res;
};

struct SMCParams {
  float retain, max_temp, tol;
  int32_t max_bisect, max_iter, mcmc_steps;
  const float *sched;  // temperature schedule (nullptr: adaptive)
  int32_t n_sched;
};

struct SMCData {
  const float *X;        // (n_data, d) row-major
  const float *y;        // (n_data) labels in {0, 1}
  const uint16_t *Xb;    // (n_data, 64) bf16 rows zero-padded to 64 features (tensor-core path)
  int64_t n_data;
  int d;
};

// tensor-core (tcgen05, bf16 operands, fp32 accumulation) potential and gradient
size_t logreg_tc_workspace(int64_t P, int64_t n_data, int d);
int logreg_tc(const SMCData &dat, const float *beta, int64_t P, const int32_t *active, int N, float *lik, float *grad,
              void *ws, size_t ws_bytes, cudaStream_t s);

}  // namespace mgb
