#include "split.cuh"

namespace sc {

static sc_status not_built() {
  set_error("the split-BF16 form is not available in this build");
  return SC_ERR_INVALID;
}

sc_status split_prepare(SplitState *, int, const void *, int64_t, int, double *, cudaStream_t) { return not_built(); }
sc_status split_centroids_changed(SplitState *, const double *, int, cudaStream_t) { return not_built(); }
sc_status split_assign(SplitState *, int, const void *, int64_t, int, const double *, int, int32_t *, Acc128 *,
                       unsigned long long *, int, LloydState *, cudaStream_t) { return not_built(); }
void split_free(SplitState *) {}
sc_status split_knn(SplitKnnState *, int, const void *, int64_t, int, const void *, int64_t, int, int64_t *,
                    double *, int64_t *, cudaStream_t) { return not_built(); }
void split_knn_free(SplitKnnState *) {}

}  // namespace sc
