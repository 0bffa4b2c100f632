// Split-BF16 form: -2 x.c^T on the tcgen05 tensor cores with a certified
// error bound, FP64 re-score of every decision inside the bound.
#pragma once

#include "common.cuh"

namespace sc {

struct SplitState {
  int ready = 0;
};

struct SplitKnnState {
  int ready = 0;
};

sc_status split_prepare(SplitState *s, int dtype, const void *x, int64_t n, int d,
                        double *xnorm_total, cudaStream_t st);
sc_status split_centroids_changed(SplitState *s, const double *cent, int k, cudaStream_t st);
sc_status split_assign(SplitState *s, int dtype, const void *x, int64_t n, int d,
                       const double *cent, int k, int32_t *labels, Acc128 *acc,
                       unsigned long long *cnt, int scale, LloydState *lst, cudaStream_t st);
void split_free(SplitState *s);

sc_status split_knn(SplitKnnState *s, int dtype, const void *train, int64_t n, int d,
                    const void *queries, int64_t m, int k, int64_t *idx, double *dist,
                    int64_t *rescored, cudaStream_t st);
void split_knn_free(SplitKnnState *s);

}  // namespace sc
