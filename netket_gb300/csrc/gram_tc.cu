// Tensor-core Gram contraction (placeholder until the tcgen05 kernel lands):
// the entry point reports VMCK_ERR_UNSUPPORTED so that no caller silently gets
// a different code path.
#include "gram_tc.cuh"

namespace vmck {

int64_t gram_tc_workspace_doubles(int M, int64_t n) {
  (void)M;
  (void)n;
  return 0;
}

int gram_tc_launch(vmck_ctx *, cudaStream_t, const float *, const uint32_t *, int, int, int,
                   int64_t, const double *, const double *, double, double, double *, float *,
                   double *) {
  set_last_error("rbm_gram: tensor-core mode not built");
  return VMCK_ERR_UNSUPPORTED;
}

}  // namespace vmck
