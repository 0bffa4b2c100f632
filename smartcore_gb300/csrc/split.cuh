// Split-BF16 form: -2 x.c^T on the tcgen05 tensor cores with a certified
// error bound, FP64 re-score of every decision inside the bound.
#pragma once

#include <vector>

#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"

namespace sc {

struct SplitState {
  int ready = 0;
  int dtype = 0;
  int64_t n = 0, n_pad = 0;
  int d = 0, d_pad = 0, kt_elems = 0, nkt = 0, row_bytes = 0;
  __nv_bfloat16 *xh = nullptr, *xl = nullptr;  // n_pad x d_pad
  float *xnrm = nullptr;                        // n_pad: upper bound of ||x||
  double *part = nullptr;                       // block partials of ||x||^2
  int k = 0, k_pad = 0, k_alloc = 0;
  int wide = 0;                                 // centroids streamed in blocks (split_wide_kernel)
  __nv_bfloat16 *ch = nullptr, *cl = nullptr;  // k_pad x d_pad
  __nv_bfloat16 *cbx = nullptr;                 // k_pad x 16: BF16 terms of -||c||^2/2
  __nv_bfloat16 *ones = nullptr;                // 128 x 16: [1, 1, 1, 0...] rows
  CUtensorMap tm_cbx, tm_ones;
  float *cn2 = nullptr;                         // k_pad: ||c||^2 rounded to f32 (+inf for padding)
  unsigned int *cmax = nullptr;                 // bits of an upper bound of max ||c||
  float *cT = nullptr;                          // d_pad x k_cols: centroids in f32, transposed
  unsigned int *list_count = nullptr;           // near ties of the last assignment: rows per CTA,
  int64_t *list_rows = nullptr;                 //   their rows (per-CTA regions),
  uint2 *cand4 = nullptr;                       //   [2][n_pad] candidate columns by row (4 x 16 bits)
  uint8_t *cmeta = nullptr;                     //   [2][n_pad] valid columns, list complete
  CUtensorMap tm_xh, tm_xl, tm_ch, tm_cl;
  int num_sms = 0;
  uint64_t wait_ns = 0;                         // bound of the assignment's pipeline waits (0: 2 s)
};

struct SplitKnnState {
  int ready = 0;
  const void *train = nullptr;  // device rows the training operand was built from
  int64_t n = 0;
  int d = 0, num_sms = 0;
  __nv_bfloat16 *th = nullptr, *tl = nullptr;  // n_pad x d_pad training halves
  __nv_bfloat16 *tbx = nullptr;                 // n_pad x 16: BF16 terms of -||t||^2/2
  __nv_bfloat16 *ones = nullptr;                // 128 x 16: [1, 1, 1, 0...] rows
  unsigned int *tmax = nullptr;                 // bits of an upper bound of max ||t||
  CUtensorMap tm_th, tm_tl, tm_tbx, tm_ones;
  __nv_bfloat16 *qh = nullptr, *ql = nullptr;  // query halves (per call)
  float *qnrm = nullptr;
  double *qn2 = nullptr;
  int64_t m_cap = 0;
  int32_t *cand = nullptr;                      // find: candidate rows, m_pad x cap
  int32_t *count = nullptr, *over = nullptr;    //   per query: candidates; queries past cap
  size_t cand_cap = 0;
  int64_t count_cap = 0;
  unsigned long long *evals = nullptr;          // [0] exact evaluations, [1] error flag, [2] queries past cap
};

sc_status split_prepare(SplitState *s, int dtype, const void *x, int64_t n, int d,
                        double *xnorm_total, cudaStream_t st);
sc_status split_centroids_changed(SplitState *s, const double *cent, int k, cudaStream_t st);
sc_status split_assign(SplitState *s, int dtype, const void *x, int64_t n, int d,
                       const double *cent, int k, int32_t *labels, LloydState *lst,
                       cudaStream_t st, cudaEvent_t *timing = nullptr);
void split_free(SplitState *s, cudaStream_t st);

sc_status split_knn(SplitKnnState *s, int dtype, const void *train, int64_t n, int d,
                    const void *queries, int64_t m, int k, int64_t *idx, double *dist,
                    int64_t *rescored, cudaStream_t st);
// Whether the split-BF16 kNN kernels serve d features and k neighbours for
// find (heaps of at most 64 entries) or for find_radius (its tiles at most
// 256 features); the entry points run the FP64 kernels, with the same
// results, otherwise.
bool split_knn_serves(int d, int k, int dtype, bool radius);
// Testing: candidate slots per query of split find (0: the default).
void split_knn_set_candidate_cap(int64_t cap);
void split_knn_set_chunk_queries(int64_t q);
// Widest rows the split-BF16 k-means kernels serve.
constexpr int kSplitKMeansMaxD = 128;
// find_radius: counting pass when idx is null (counts[q]), else filling pass
// (query q's rows from offsets[q] on); every pointer is device memory.
sc_status split_knn_radius(SplitKnnState *s, int dtype, const void *train, int64_t n, int d,
                           const void *queries, int64_t m, double radius, int64_t *counts,
                           const int64_t *offsets, int64_t *idx, double *dist, cudaStream_t st);
// find_radius lists of m device queries, usually in one pass: CSR offsets
// (m + 1, host) and device arrays idx / dist allocated here (dfree them).
// SC_ERR_INVALID with nothing allocated when m is too large for the slots;
// the caller then runs the counting and filling passes.
sc_status split_knn_radius_lists(SplitKnnState *s, int dtype, const void *train, int64_t n, int d,
                                 const void *queries, int64_t m, double radius, std::vector<int64_t> &off,
                                 int64_t **idx, double **dist, cudaStream_t st);
void split_knn_free(SplitKnnState *s, cudaStream_t st);

}  // namespace sc
