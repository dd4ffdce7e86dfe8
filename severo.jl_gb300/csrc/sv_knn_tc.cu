// BF16 tensor-core (tcgen05) distance tiles for the kNN candidate stage.
#include "sv_internal.cuh"

int sv_knn_tc_candidates(sv_context* ctx, const float* X32, const float* sq, int64_t n, int d,
                         int K2, int include_self, int32_t* cand) {
  (void)ctx; (void)X32; (void)sq; (void)n; (void)d; (void)K2; (void)include_self; (void)cand;
  sv_set_error("the BF16 tensor-core kNN path is not built yet");
  return SV_ERR_UNSUPPORTED;
}
