// Host-side declarations shared between the C-ABI translation units:
// workspace layouts and launchers of the reduction / resampling kernels.
#pragma once
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"

namespace mgb {

struct LseWs;
struct ResampleWs {
  ResampleCtl *ctl;
  uint64_t *status, *status2;
  int64_t ntiles;
  uint64_t *C, *S;  // multinomial only: weight prefix (n) and spacing prefix (n + 1)
};

ResampleWs carve_resample(Carver &c, int64_t n, int scheme);
int reset_resample(const ResampleWs &w, cudaStream_t s);
// Resample lw (n) into anc.  M: device float (max log-weight).  key: step key
// (device, 2 words).  flag (nullable): skip unless *flag != 0.
int launch_resample(const float *lw, int64_t n, int scheme, const float *Mptr, const uint32_t *key, int has_m23,
                    uint32_t m23, const int32_t *flag, const ResampleWs &w, int32_t *anc, int *err, cudaStream_t s);

}  // namespace mgb
