// Logistic-regression potential and gradient on the tensor cores (bf16
// operands, fp32 accumulation): not built yet; the entry reports
// MGB_ERR_UNSUPPORTED.
#include "mgb_smc.cuh"

namespace mgb {

size_t logreg_tc_workspace(int64_t, int64_t, int) { return 256; }

int logreg_tc(const SMCData &, const float *, int64_t, const int32_t *, int, float *, float *, void *, size_t,
              cudaStream_t) {
  return ERR_UNSUPPORTED;
}

}  // namespace mgb
