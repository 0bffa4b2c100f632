// Batched k-means: many independent KMeans::fit problems (uneven n, d, k) in
// one pass over the GPU.  Each problem keeps the semantics of KMeans::fit
// (src/cluster/kmeans.rs:254-323): k-means++ from its own draws (:354-413),
// initial means of the seeding partition (:275-292), then up to max_iter
// Lloyd iterations with the break rule `distortion <= dist` (:305-309).
//
// Device layout (one arena per call, problems sorted by k, largest first):
//   X        every problem's rows, row-major, width D = d rounded up to a
//            power of two in [8, 64], pad columns zero, problem starts
//            16-byte aligned
//   labels   int32 per row; dd / dd32: k-means++ distances (f64, f32 up)
//   part     f64 per 256-row block (k-means++ sums, ||x||^2 sums)
//   cent64   k x d f64 centroids per problem; cent32: k_pad x D f32 copies
//   acc/cnt  128-bit fixed-point cluster sums and counts per problem
//   items    the Lloyd work queue: (problem, rows [r0, r1), kernel variant),
//            largest cost first; one queue head per launch
//
// The problems are grouped by padded width D into four classes, and each
// class's work runs as one chain on its own stream (the widest on a
// high-priority stream): its rows (copied, or read in place from pinned host
// memory by a gather kernel), the scan of ||x||^2 and max |x| with the
// start values and fixed-point scales, its k-means++ draws, the initial
// means, and its Lloyd loop.  Per Lloyd iteration two launches, captured in
// one CUDA graph per class:
//   batch_assign_kernel  persistent CTAs pop items; per row an FP32
//                        expansion-form score to every centroid, a certified
//                        bound on its error, an FP64 re-score (the
//                        reference's operation order) of the rows whose best
//                        two centroids fall inside the bound, and the exact
//                        fixed-point sums of the item's rows in shared memory
//                        (the rows are read once per iteration)
//   batch_finalize_kernel one CTA per problem of the class: centroids = sums /
//                        sizes, distortion, break rule, the next f32
//                        centroid copies
// k-means++ runs a class's draw j for all its problems still seeding: one
// update launch over their rows, one selection launch (a CTA each).
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "exactsum.cuh"
#include "ppsel.cuh"

namespace sc {

// capi.cu: pinned staging buffer for results copied into caller memory
extern std::mutex g_stage_mutex;
sc_status host_stage(size_t bytes, void **out);

namespace {

constexpr int kBlk = 256;         // rows per k-means++ block (one thread each)
constexpr int kAsgThreads = 256;  // threads per assignment CTA (one row each)
constexpr int kSelT = 256;        // threads per selection CTA
constexpr int kFinT = 256;        // threads per finalize CTA
constexpr int kMaxBD = 64;        // widest padded row served
constexpr int kMaxBK = 128;       // most clusters per problem served
constexpr int kNumCU = 3;         // kernel variants: centroids per inner pass
constexpr int kCUs[kNumCU] = {2, 4, 8};
constexpr int kNumRows = 3;       // rows per work item
constexpr int kRowsOpts[kNumRows] = {1024, 2048, 4096};
constexpr int kGraphIters = 32;  // Lloyd iterations per graph launch
constexpr int kNumD = 4;         // padded widths 8, 16, 32, 64

struct BProb {
  int64_t x_off;   // element offset of row 0 in X
  int64_t row0;    // global index of row 0 (labels, dd, dd32)
  int64_t c_off;   // offset of the k x d arrays (cent64, acc, seed_x)
  int64_t c32_off; // offset of the f32 centroid copies: k_pad x D values, then k_pad ||c||^2
  int32_t n, d, D, k;
  int32_t k_off;   // offset of the per-cluster arrays
  int32_t b0, nb;  // 256-row blocks of the problem
  int32_t max_iter;
  int32_t scale;   // fixed-point scale 2^scale of the sums
  int32_t lg_d;    // ceil(log2 d)
  int32_t u_off;   // offset of the k-means++ uniforms (k - 1)
  int32_t rows;    // rows per work item
};

struct BState {
  double distortion;  // the reference's `distortion` (f64::MAX at the start)
  double last_dist;   // distortion of the latest clustering step
  double xnorm2;      // sum over rows of ||x||^2
  int64_t iters;
  int64_t pp_chosen;  // k-means++: row of the current seed
  int64_t rescored;   // rows re-scored in FP64
  int64_t pp_replays; // draws resolved by the sequential replay
  float cdelta;       // >= max over centroids of ||c - fl32(c)||
  float cmax;         // >= max over centroids of ||fl32(c)||
  int32_t done;
  int32_t pad;
};

struct BItem {
  int32_t prob, r0, r1, variant;
};

__host__ __device__ inline int pad_width(int d) {
  int D = 8;
  while (D < d) D <<= 1;
  return D;
}

// v * 2^scale rounded to the nearest integer (ties to even); the scale
// guarantees |v| * 2^scale < 2^62.
__device__ __forceinline__ long long fixed64(float v, int scale) {
  const uint32_t b = __float_as_uint(v);
  int e = (int)((b >> 23) & 0xffu);
  uint32_t m = b & 0x7fffffu;
  if (e == 0) e = 1; else m |= 0x800000u;
  if (!m) return 0;
  const int sh = e - 150 + scale;
  unsigned long long mag;
  if (sh >= 0) {
    mag = (unsigned long long)m << sh;
  } else if (sh > -25) {
    const int r = -sh;
    const uint32_t q = m >> r, rem = m & ((1u << r) - 1u), half = 1u << (r - 1);
    mag = q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
  } else {
    mag = 0;  // below half a quantum
  }
  return (b >> 31) ? -(long long)mag : (long long)mag;
}

__device__ __forceinline__ long long fixed64(double v, int scale) {
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  int e = (int)((b >> 52) & 0x7ffu);
  uint64_t m = b & 0xfffffffffffffull;
  if (e == 0) e = 1; else m |= 0x10000000000000ull;
  if (!m) return 0;
  const int sh = e - 1075 + scale;
  unsigned long long mag;
  if (sh >= 0) {
    mag = m << sh;
  } else if (sh > -54) {
    const int r = -sh;
    const uint64_t q = m >> r, rem = m & ((1ull << r) - 1ull), half = 1ull << (r - 1);
    mag = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
  } else {
    mag = 0;
  }
  return (b >> 63) ? -(long long)mag : (long long)mag;
}

__device__ __forceinline__ void atomic_add128(Acc128 *a, long long sv) {
  const unsigned __int128 v = (unsigned __int128)(__int128)sv;
  const unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)(v >> 64);
  const unsigned long long old = atomicAdd(&a->lo, lo);
  const unsigned long long h = hi + ((old + lo) < old ? 1ull : 0ull);
  if (h) atomicAdd(&a->hi, h);
}

// Correctly rounded value of a 128-bit two's-complement integer * 2^-scale.
__device__ double fixed128_to_double(unsigned long long lo, unsigned long long hi, int scale) {
  unsigned __int128 v = ((unsigned __int128)hi << 64) | lo;
  const bool neg = (hi >> 63) != 0;
  if (neg) v = (unsigned __int128)0 - v;
  const uint64_t vh = (uint64_t)(v >> 64), vl = (uint64_t)v;
  double r;
  if (vh == 0) {
    r = ldexp(__ull2double_rn(vl), -scale);
  } else {
    const int lz = __clzll((long long)vh);
    const unsigned __int128 t = v << lz;
    uint64_t top = (uint64_t)(t >> 64);
    top |= ((uint64_t)t != 0) ? 1ull : 0ull;  // sticky bit
    r = ldexp(__ull2double_rn(top), 64 - lz - scale);
  }
  return neg ? -r : r;
}

// ---------------------------------------------------------------------------
// Error bound of the FP32 difference-form distance.  With c~ = fl32(c) (and
// x~ = fl32(x) for f64 rows), t_j = fl(x~_j - c~_j) and D32 = the FMA chain
// of t_j^2 over the D (zero-padded) terms:
//   |D32 - ||x~ - c~||^2| <= g ||x~ - c~||^2 + A,  g = (d + 3) 2^-24 (1.01),
//   A = (d + 2) 2^-140 (underflow of the terms),
// and with del >= ||(x - x~) - (c - c~)||, |D~ - D| <= 2 sqrt(D~) del + del^2
// for D = ||x - c||^2, D~ = ||x~ - c~||^2 <= (1 + 2g) D32 + A.  Hence
//   |D32 - D| <= E(D32) = 2 (g D32 + 2 sqrt((1 + 2g) D32) del + 3 del^2) + A
// (a factor 2 of slack, every operation rounded up).  The reference's own
// FP64 value is within (d + 2) 2^-53 D of D, inside the slack.
// ---------------------------------------------------------------------------
struct Bound {
  float g, g2, del, del2x3, A, floor16;
};

__device__ __forceinline__ Bound make_bound(int d, float del) {
  Bound b;
  b.g = __fmul_ru((float)(d + 3), 0x1.02p-24f);
  b.g2 = __fadd_ru(1.f, __fmul_ru(2.f, b.g));
  b.del = del;
  b.del2x3 = __fmul_ru(3.f, __fmul_ru(del, del));
  b.A = __fmul_ru((float)(d + 2), 0x1p-140f);
  b.floor16 = __fmul_ru(16.f, __fmul_ru(del, del));
  return b;
}

__device__ __forceinline__ float err_bound(float v, const Bound &b) {
  const float s = __fsqrt_ru(__fmul_ru(v, b.g2));
  const float e = __fadd_ru(__fadd_ru(__fmul_ru(b.g, v), __fmul_ru(__fmul_ru(2.f, s), b.del)), b.del2x3);
  return __fadd_ru(__fmul_ru(2.f, e), b.A);
}

// FP32 difference-form distance of the row x (registers) to centroid c, in
// two interleaved FMA chains (even and odd feature pairs) added at the end:
// every term passes through at most D / 2 + 1 roundings, within the bound.
template <int D>
__device__ __forceinline__ float dist32(const float (&x)[D], const float *__restrict__ c) {
  float a = 0.f, b = 0.f;
#pragma unroll
  for (int j = 0; j < D; j += 4) {
    const float4 cc = *reinterpret_cast<const float4 *>(c + j);
    float t = __fsub_rn(x[j], cc.x);
    a = __fmaf_rn(t, t, a);
    t = __fsub_rn(x[j + 1], cc.y);
    b = __fmaf_rn(t, t, b);
    t = __fsub_rn(x[j + 2], cc.z);
    a = __fmaf_rn(t, t, a);
    t = __fsub_rn(x[j + 3], cc.w);
    b = __fmaf_rn(t, t, b);
  }
  return __fadd_rn(a, b);
}

// Expansion-form score of the row x to centroid c: ||c~||^2 - 2 x~.c~ (the
// row's own ||x~||^2, common to every centroid, is left out), the dot product
// in two FMA chains.  Against ||c~||^2 - 2 S for the exact S = x~.c~:
//   |score - (||c~||^2 - 2 S)| <= E_s = (2 g + 2u) ||x~|| cmax + 2.01 u cmax^2 + A
// with g = (D/2 + 1) u (1.02) (the roundings a product passes through),
// u = 2^-24, cn2 within 1.01 u of ||c~||^2, and A the underflow of the
// products.  Differences of two scores then bound differences of the
// D~ = ||x~ - c~||^2 within 2 E_s.
template <int D>
__device__ __forceinline__ float score32(const float (&x)[D], const float *__restrict__ c, float cn2) {
  float a = 0.f, b = 0.f;
#pragma unroll
  for (int j = 0; j < D; j += 4) {
    const float4 cc = *reinterpret_cast<const float4 *>(c + j);
    a = __fmaf_rn(x[j], cc.x, a);
    b = __fmaf_rn(x[j + 1], cc.y, b);
    a = __fmaf_rn(x[j + 2], cc.z, a);
    b = __fmaf_rn(x[j + 3], cc.w, b);
  }
  return __fmaf_rn(-2.f, __fadd_rn(a, b), cn2);
}

template <typename T, int D>
__device__ __forceinline__ void load_row(const T *__restrict__ xr, float (&x)[D]) {
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int j = 0; j < D; j += 4) {
      const float4 v = __ldg(reinterpret_cast<const float4 *>(xr + j));
      x[j] = v.x; x[j + 1] = v.y; x[j + 2] = v.z; x[j + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < D; j += 2) {
      const double2 v = __ldg(reinterpret_cast<const double2 *>(xr + j));
      x[j] = __double2float_rn(v.x); x[j + 1] = __double2float_rn(v.y);
    }
  }
}

// The label of a scored row: certain when the two best scores differ by more
// than the bound, else settled among the centroids the difference form cannot
// exclude with the reference's FP64 distance.  x: the row's f32 values, xr:
// the row as given; best / second / bi from the scores in centroid order.
template <typename T, int D>
__device__ __forceinline__ int settle_row(const float (&x)[D], const T *__restrict__ xr, const BProb &P,
                                          const double *__restrict__ cent64, const float *s_c, float best,
                                          float second, int bi, float cdelta, float cmax, long long &rescored) {
  const int d = P.d, k = P.k;
  // ||x~|| from above; for f64 rows also ||x - fl32(x)|| <= 2^-24 ||x~|| (1 + 2^-20)
  float xn = 0.f;
#pragma unroll
  for (int j = 0; j < D; ++j) xn = __fmaf_ru(x[j], x[j], xn);
  const float rn = __fsqrt_ru(xn);
  float del = cdelta;
  if constexpr (sizeof(T) == 8) del = __fadd_ru(del, __fmul_ru(rn, 0x1.00001p-24f));
  // The label is certain when the two best scores differ by more than
  // 2 (2 E_s + 2 E_d): E_s bounds each score (score32), E_d >= |D - D~|
  // for every centroid, 2 (||x~|| + cmax) del + del^2, plus the
  // reference's own FP64 rounding of D; any other centroid's D then
  // exceeds the best one's (a factor 2 of slack).
  bool certain;
  {
    const float g2 = __fadd_ru(__fmul_ru((float)(D / 2 + 1), 0x1.06p-23f), 0x1p-23f);  // 2 g + 2 u
    const float rc = __fmul_ru(rn, cmax);
    float es = __fadd_ru(__fmul_ru(g2, rc), __fmul_ru(0x1.02p-23f, __fmul_ru(cmax, cmax)));
    es = __fadd_ru(es, __fmul_ru((float)(D + 4), 0x1p-138f));
    const float rs = __fadd_ru(rn, cmax);
    float ed = __fadd_ru(__fmul_ru(__fmul_ru(2.f, rs), del), __fmul_ru(del, del));
    ed = __fadd_ru(ed, __fmul_ru(__fmul_ru((float)(d + 2), 0x1p-52f), __fmul_ru(rs, rs)));
    const float margin = __fmul_ru(4.f, __fadd_ru(es, ed));
    certain = __fsub_rd(second, best) > margin;
  }
  if (!certain) {
    // Near tie (or a non-finite value): the difference form bounds each
    // centroid's D on its own; every centroid whose FP32 distance cannot
    // be shown to exceed the best one's is scored with the reference's
    // FP64 distance (src/metrics/distance/euclidian.rs:51-63 on f64 rows,
    // kmeans.rs:338-346), strict <, lowest index first.
    const Bound bd = make_bound(d, del);
    float best32 = __int_as_float(0x7f800000);
    for (int c = 0; c < k; ++c) best32 = fminf(best32, dist32<D>(x, s_c + c * D));
    const float thr = __fadd_ru(best32, err_bound(best32, bd));
    double bdist = DBL_MAX;
    int b = 0;
    for (int c = 0; c < k; ++c) {
      const float a = dist32<D>(x, s_c + c * D);
      if (__fsub_rd(a, err_bound(a, bd)) > thr) continue;
      const double *cr = cent64 + P.c_off + (int64_t)c * d;
      double sd = 0.0;
      for (int j = 0; j < d; ++j) sd = __dadd_rn(sd, sq_term((double)xr[j], cr[j]));
      if (sd < bdist) {
        bdist = sd;
        b = c;
      }
    }
    ++rescored;
    return b;
  }
  return bi;
}

// One work item of rows in passes of 256, one row per thread for the
// distances.  mode 0: assign + sums; mode 1: sums of the given labels (the
// seeding partition).  The sums are taken warp by warp afterwards: for each
// of its 32 rows the warp adds the row's values, lane j feature j, into the
// cluster's shared accumulators, so the 64-bit shared atomics of one
// instruction hit consecutive words (no bank conflicts); the rows are read
// again from global memory, where the distance pass has just brought them
// into L1.
template <typename T, int D, int CU>
__device__ __forceinline__ void assign_rows(const BItem &it, const BProb &P, BState *st, const T *__restrict__ X,
                                            const double *__restrict__ cent64, const float *s_c, float cdelta,
                                            float cmax, unsigned long long *s_acc, unsigned *s_cnt, int *s_lab,
                                            int32_t *__restrict__ labels, int mode) {
  const int d = P.d, k = P.k, kpad = (k + 7) & ~7;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long rescored = 0;
  for (int base = it.r0; base < it.r1; base += kAsgThreads) {
    const int r = base + (int)threadIdx.x;
    int bi = -1;
    if (r < it.r1) {
      const T *xr = X + P.x_off + (int64_t)r * D;
      if (mode == 1) {
        bi = labels[P.row0 + r];
      } else {
        float x[D];
        load_row<T, D>(xr, x);
        float best = __int_as_float(0x7f800000), second = best;
        bi = 0;
        const float *s_cn2 = s_c + kpad * D;
#pragma unroll 1
        for (int c0 = 0; c0 < kpad; c0 += CU) {
          // the CU centroids' dot products in 2 CU independent FMA chains,
          // interleaved feature group by feature group (score32's order per
          // centroid, so the same roundings)
          // (a, b) of a centroid as one pair: each paired FMA is the two
          // chains' scalar FMAs, each rounded on its own
          float2 ab[CU];
#pragma unroll
          for (int u = 0; u < CU; ++u) ab[u] = make_float2(0.f, 0.f);
#pragma unroll
          for (int j = 0; j < D; j += 4) {
            float4 cc[CU];
#pragma unroll
            for (int u = 0; u < CU; ++u) cc[u] = *reinterpret_cast<const float4 *>(s_c + (c0 + u) * D + j);
            const float2 x01 = make_float2(x[j], x[j + 1]), x23 = make_float2(x[j + 2], x[j + 3]);
#pragma unroll
            for (int u = 0; u < CU; ++u) {
              ab[u] = __ffma2_rn(x01, make_float2(cc[u].x, cc[u].y), ab[u]);
              ab[u] = __ffma2_rn(x23, make_float2(cc[u].z, cc[u].w), ab[u]);
            }
          }
          float a[CU];
#pragma unroll
          for (int u = 0; u < CU; ++u) a[u] = __fmaf_rn(-2.f, __fadd_rn(ab[u].x, ab[u].y), s_cn2[c0 + u]);
#pragma unroll
          for (int u = 0; u < CU; ++u) {
            const float v = a[u];  // NaN (padding, empty clusters) never wins
            if (v < best) {
              second = best;
              best = v;
              bi = c0 + u;
            } else if (v < second) {
              second = v;
            }
          }
        }
        bi = settle_row<T, D>(x, xr, P, cent64, s_c, best, second, bi, cdelta, cmax, rescored);
        labels[P.row0 + r] = bi;
      }
    }
    s_lab[threadIdx.x] = bi;
    __syncwarp();
    // exact fixed-point sums of the warp's rows, four rows' loads in flight
    const int rw = base + w * 32;
    constexpr int JW = D > 32 ? 2 : 1;  // features per lane
    for (int q0 = 0; q0 < 32; q0 += 4) {
      int lab[4];
      T v[4][JW];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        lab[u] = s_lab[w * 32 + q0 + u];  // -1: past the item's end (uniform over the warp)
        const T *xr = X + P.x_off + (int64_t)(rw + q0 + u) * D;
#pragma unroll
        for (int h = 0; h < JW; ++h) {
          const int j = lane + 32 * h;
          v[u][h] = (lab[u] >= 0 && j < d) ? xr[j] : T(0);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (lab[u] < 0) break;
        unsigned long long *ar = s_acc + (int64_t)lab[u] * d;
#pragma unroll
        for (int h = 0; h < JW; ++h) {
          const int j = lane + 32 * h;
          const long long fv = j < d ? fixed64(v[u][h], P.scale) : 0ll;
          if (fv) atomicAdd(ar + j, (unsigned long long)fv);
        }
        if (lane == 0) atomicAdd(&s_cnt[lab[u]], 1u);
      }
      if (lab[3] < 0) break;
    }
    __syncwarp();  // s_lab is rewritten by the next pass
  }
  if (rescored) atomicAdd((unsigned long long *)&st->rescored, (unsigned long long)rescored);
}

template <typename T, int D>
__device__ __forceinline__ void assign_rows_cu(int cu, const BItem &it, const BProb &P, BState *st, const T *X,
                                               const double *cent64, const float *s_c, float cdelta, float cmax,
                                               unsigned long long *s_acc, unsigned *s_cnt, int *s_lab,
                                               int32_t *labels, int mode) {
  if (cu == 2) assign_rows<T, D, 2>(it, P, st, X, cent64, s_c, cdelta, cmax, s_acc, s_cnt, s_lab, labels, mode);
  else if (cu == 8) assign_rows<T, D, 8>(it, P, st, X, cent64, s_c, cdelta, cmax, s_acc, s_cnt, s_lab, labels, mode);
  else assign_rows<T, D, 4>(it, P, st, X, cent64, s_c, cdelta, cmax, s_acc, s_cnt, s_lab, labels, mode);
}

// Resident CTAs per SM the compiler plans registers for, by row width.
template <int D>
struct AsgOcc {
  static constexpr int value = D <= 16 ? 4 : D <= 32 ? 3 : 2;
};

// Persistent assignment (+ sums) kernel of the problems of padded width D,
// fed by the device work queue `head` over their items.
template <typename T, int D>
__global__ void __launch_bounds__(kAsgThreads, AsgOcc<D>::value)
batch_assign_kernel(const BItem *__restrict__ items, int nitems, const BProb *__restrict__ probs, BState *st,
                    const T *__restrict__ X, const float *__restrict__ cent32, const double *__restrict__ cent64,
                    int32_t *__restrict__ labels, Acc128 *__restrict__ acc, unsigned long long *__restrict__ cnt,
                    unsigned *head, const int *active, int mode) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_item, s_prob;
  __shared__ int s_lab[kAsgThreads];
  if (mode == 0 && *active == 0) return;
  if (threadIdx.x == 0) s_prob = -1;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = (int)atomicAdd(head, 1u);
    __syncthreads();
    const int iti = s_item;
    if (iti >= nitems) break;
    const BItem it = items[iti];
    if (mode == 0 && st[it.prob].done) continue;
    const BProb P = probs[it.prob];
    const int k = P.k, d = P.d, kpad = (k + 7) & ~7;
    float *s_c = reinterpret_cast<float *>(smraw);  // kpad x D values, then kpad ||c||^2
    unsigned long long *s_acc = reinterpret_cast<unsigned long long *>(smraw + (size_t)kpad * (D + 1) * 4);
    unsigned *s_cnt = reinterpret_cast<unsigned *>(s_acc + (size_t)k * d);
    const bool reload = mode == 0 && s_prob != it.prob;
    __syncthreads();  // every thread has read s_prob
    if (reload) {
      const float4 *src = reinterpret_cast<const float4 *>(cent32 + P.c32_off);
      for (int t = threadIdx.x; t < kpad * (D + 1) / 4; t += kAsgThreads) reinterpret_cast<float4 *>(s_c)[t] = src[t];
      if (threadIdx.x == 0) s_prob = it.prob;
    }
    for (int t = threadIdx.x; t < k * d; t += kAsgThreads) s_acc[t] = 0ull;
    for (int t = threadIdx.x; t < k; t += kAsgThreads) s_cnt[t] = 0u;
    __syncthreads();
    assign_rows_cu<T, D>(it.variant, it, P, st + it.prob, X, cent64, s_c, st[it.prob].cdelta, st[it.prob].cmax,
                         s_acc, s_cnt, s_lab, labels, mode);
    __syncthreads();
    for (int t = threadIdx.x; t < k * d; t += kAsgThreads) {
      const long long v = (long long)s_acc[t];
      if (v) atomic_add128(&acc[P.c_off + t], v);
    }
    for (int t = threadIdx.x; t < k; t += kAsgThreads)
      if (s_cnt[t]) atomicAdd(&cnt[P.k_off + t], (unsigned long long)s_cnt[t]);
  }
}

// End of a clustering step, one CTA per problem: centroids = sums / sizes
// (an empty cluster keeps its centroid, kmeans.rs:297-303; after seeding it
// becomes NaN, the reference's 0 / 0 at :287-291), the distortion of the
// step from the identity sum ||x||^2 - 2 c.S + n ||c||^2 over the old
// centroids, the break rule, and the f32 copies of the new centroids.
__global__ void __launch_bounds__(kFinT)
batch_finalize_kernel(const BProb *__restrict__ probs, BState *st, Acc128 *__restrict__ acc,
                      unsigned long long *__restrict__ cnt, double *__restrict__ cent64, float *__restrict__ cent32,
                      int64_t *__restrict__ sizes, int init, int *active, const int32_t *__restrict__ plist) {
  __shared__ float wd[kFinT / 32], wc[kFinT / 32];
  const int p = plist ? plist[blockIdx.x] : (int)blockIdx.x;  // plist: one width class's problems
  const BProb P = probs[p];
  BState *S = st + p;
  if (!init && S->done) return;
  const int k = P.k, d = P.d, D = P.D, kd = k * d, kpad = (k + 7) & ~7;
  double term = 0.0;
  for (int t = threadIdx.x; t < kd; t += kFinT) {
    const int c = t / d;
    const unsigned long long cn = cnt[P.k_off + c];
    Acc128 &a = acc[P.c_off + t];
    const double sum = fixed128_to_double(a.lo, a.hi, P.scale);
    const double old = cent64[P.c_off + t];
    if (cn > 0) {
      const double dn = (double)cn;
      term = __dadd_rn(term, __dmul_rn(old, __dsub_rn(__dmul_rn(dn, old), __dmul_rn(2.0, sum))));
      cent64[P.c_off + t] = __ddiv_rn(sum, dn);
    } else if (init) {
      cent64[P.c_off + t] = __longlong_as_double(0x7ff8000000000000ll);
    }
    a.lo = 0ull;
    a.hi = 0ull;
  }
  __syncthreads();  // every thread has read the counts
  for (int c = threadIdx.x; c < k; c += kFinT) {
    sizes[P.k_off + c] = (int64_t)cnt[P.k_off + c];
    cnt[P.k_off + c] = 0ull;
  }
  const double tot = block_sum_fixed<kFinT>(term);
  if (threadIdx.x == 0 && !init) {
    const double dist = __dadd_rn(S->xnorm2, tot);
    S->iters += 1;
    S->last_dist = dist;
    bool stop = false;
    if (S->distortion <= dist) stop = true;
    else S->distortion = dist;
    if (S->iters >= P.max_iter) stop = true;
    if (stop) {
      S->done = 1;
      atomicSub(active, 1);
    }
  }
  __syncthreads();  // the new centroids are visible to the whole CTA
  for (int t = threadIdx.x; t < kpad * D; t += kFinT) {
    const int c = t / D, j = t - c * D;
    float v = __int_as_float(0x7fc00000);  // padding centroids: NaN
    if (c < k) v = j < d ? __double2float_rn(cent64[P.c_off + (int64_t)c * d + j]) : 0.f;
    cent32[P.c32_off + t] = v;
  }
  // per centroid: ||c~||^2 rounded to f32 (the f64 sum of the exact squares
  // is within d 2^-53 of it), cdelta >= ||c - c~||, cmax >= ||c~|| (NaN
  // centroids skipped in both maxima)
  float mx = 0.f, mc = 0.f;
  for (int c = threadIdx.x; c < kpad; c += kFinT) {
    double s = 0.0, n2 = 0.0;
    for (int j = 0; c < k && j < d; ++j) {
      const double v = cent64[P.c_off + (int64_t)c * d + j];
      const double vf = (double)__double2float_rn(v);
      const double e = __dsub_rn(v, vf);
      s = __fma_rn(e, e, s);
      n2 = __fma_rn(vf, vf, n2);
    }
    cent32[P.c32_off + (int64_t)kpad * D + c] = c < k ? __double2float_rn(n2) : __int_as_float(0x7fc00000);
    if (c < k && s == s) mx = fmaxf(mx, __fmul_ru(__fsqrt_ru(__double2float_ru(s)), 1.0001f));
    if (c < k && n2 == n2) mc = fmaxf(mc, __fmul_ru(__fsqrt_ru(__double2float_ru(n2)), 1.0001f));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mc = fmaxf(mc, __shfl_xor_sync(0xffffffffu, mc, o));
  }
  if ((threadIdx.x & 31) == 0) {
    wd[threadIdx.x >> 5] = mx;
    wc[threadIdx.x >> 5] = mc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.f, m2 = 0.f;
    for (int w = 0; w < kFinT / 32; ++w) {
      m = fmaxf(m, wd[w]);
      m2 = fmaxf(m2, wc[w]);
    }
    S->cdelta = m;
    S->cmax = m2;
  }
}

// ||x||^2 sums and max |x|: one thread per row, one CTA per 256-row block.
template <typename T>
__global__ void __launch_bounds__(kBlk)
batch_scan_kernel(const int32_t *__restrict__ block_prob, const BProb *__restrict__ probs, const T *__restrict__ X,
                  double *__restrict__ part, unsigned long long *__restrict__ absmax_bits) {
  const int b = blockIdx.x;
  const int p = block_prob[b];
  const BProb P = probs[p];
  const int64_t il = (int64_t)(b - P.b0) * kBlk + threadIdx.x;
  double s = 0.0, m = 0.0;
  if (il < P.n) {
    const T *xr = X + P.x_off + il * P.D;
    for (int j = 0; j < P.d; ++j) {
      const double v = (double)xr[j];
      s = __fma_rn(v, v, s);
      const double a = fabs(v);
      m = (a > m || a != a) ? a : m;  // NaN propagates
    }
  }
  const double tot = block_sum_fixed<kBlk>(s);
  if (threadIdx.x == 0) part[b] = tot;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double y = __shfl_xor_sync(0xffffffffu, m, o);
    m = (y > m || y != y) ? y : m;
  }
  // nonnegative doubles (and NaN above +inf) order like their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(&absmax_bits[p], (unsigned long long)__double_as_longlong(m));
}

// The same scan for f32 rows of padded width D, the row read with 16-byte
// loads (pad columns are zero).
template <int D>
__global__ void __launch_bounds__(kBlk)
batch_scan32_kernel(const int32_t *__restrict__ cls_blocks, const int32_t *__restrict__ block_prob,
                    const BProb *__restrict__ probs, const float *__restrict__ X, double *__restrict__ part,
                    unsigned long long *__restrict__ absmax_bits) {
  const int b = cls_blocks[blockIdx.x];
  const int p = block_prob[b];
  const BProb P = probs[p];
  const int64_t il = (int64_t)(b - P.b0) * kBlk + threadIdx.x;
  double s = 0.0;
  float m = 0.f;
  if (il < P.n) {
    float x[D];
    load_row<float, D>(X + P.x_off + il * D, x);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const double v = (double)x[j];
      s = __fma_rn(v, v, s);
      const float a = fabsf(x[j]);
      m = (a > m || a != a) ? a : m;  // NaN propagates
    }
  }
  const double tot = block_sum_fixed<kBlk>(s);
  if (threadIdx.x == 0) part[b] = tot;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float y = __shfl_xor_sync(0xffffffffu, m, o);
    m = (y > m || y != y) ? y : m;
  }
  if ((threadIdx.x & 31) == 0)
    atomicMax(&absmax_bits[p], (unsigned long long)__double_as_longlong((double)m));
}

// Per problem: xnorm2 = sum of its block partials in order, the state's start
// values, the first seed (row first_index) as seed 0, and the fixed-point
// scale of the sums from max |x| < 2^e: an item's int64 partial of up to
// `rows` values stays below 2^62 (at most 2^160; a non-finite max leaves a
// scale that the call reports as an error before writing any output).
// plist: one width class's problems (else problem = block).
template <typename T>
__global__ void batch_init_kernel(BProb *__restrict__ probs, int count, BState *st, const double *__restrict__ part,
                                  const int64_t *__restrict__ first, const T *__restrict__ X, T *__restrict__ seed_x,
                                  int64_t *__restrict__ seed_idx, const unsigned long long *__restrict__ absmax_bits,
                                  const int32_t *__restrict__ plist) {
  if ((int)blockIdx.x >= count) return;
  const int p = plist ? plist[blockIdx.x] : (int)blockIdx.x;
  const BProb P = probs[p];
  if (threadIdx.x == 0) {
    const double a = __longlong_as_double((long long)absmax_bits[p]);
    int e = 0;
    if (a > 0.0 && a <= DBL_MAX) frexp(a, &e);
    int lg = 0;
    while ((1ll << lg) < (long long)P.rows + 1) ++lg;
    const int sc = 62 - e - lg;
    probs[p].scale = sc > 160 ? 160 : sc;
    double s = 0.0;
    for (int b = 0; b < P.nb; ++b) s = __dadd_rn(s, part[P.b0 + b]);
    BState z;
    memset(&z, 0, sizeof z);
    z.distortion = DBL_MAX;
    z.xnorm2 = s;
    z.pp_chosen = first[p];
    st[p] = z;
    seed_idx[P.k_off] = first[p];
  }
  const T *src = X + P.x_off + first[p] * P.D;
  for (int j = threadIdx.x; j < P.d; j += blockDim.x) seed_x[P.c_off + j] = src[j];
}

// ---------------------------------------------------------------------------
// k-means++ update of draw j (kmeans.rs:367-379, and :399-410 for the last
// seed): d[i] = min(d[i], |x_i - seed|^2) in the element type's arithmetic,
// y[i] = j - 1 when it drops, then each block's fixed-order sum of d.  One
// CTA per 256-row block of the problems with k >= j.  For f32 rows the far
// test (triangle inequality through the seed-to-seed gaps, as in the
// single-problem kernel) and an f32 lower bound skip the exact value of the
// rows whose distance cannot drop.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kBlk)
batch_pp_update_kernel(const int32_t *__restrict__ block_prob, const BProb *__restrict__ probs,
                       const BState *__restrict__ st, const T *__restrict__ X, double *__restrict__ dd,
                       float *__restrict__ dd32, int32_t *__restrict__ labels, double *__restrict__ part,
                       const float *__restrict__ seed_cc, int j, PPFar32 far) {
  __shared__ __align__(16) T s_seed[kMaxBD];
  const int b = blockIdx.x;
  const int p = block_prob[b];
  const BProb P = probs[p];
  const int64_t ci = st[p].pp_chosen;
  for (int t = threadIdx.x; t < P.D; t += kBlk) s_seed[t] = X[P.x_off + ci * P.D + t];
  __syncthreads();
  const int64_t il = (int64_t)(b - P.b0) * kBlk + threadIdx.x;
  const bool live = il < P.n;
  const int64_t gi = P.row0 + il;
  const bool first = j == 1;
  double cur = 0.0;
  if (live) {
    cur = first ? DBL_MAX : dd[gi];
    int32_t lab = first ? 0 : labels[gi];
    const int d = P.d;
    const T *xr = X + P.x_off + il * P.D;
    bool need = true;
    if constexpr (sizeof(T) == 4) {
      if (!first) {
        const float c32 = dd32[gi];
        need = !pp_far32(seed_cc[P.k_off + lab], c32, far);
        if (need) {
          // The reference's terms fl32((x_t - c_t)^2) summed in f32 bound its
          // f64 sum from below by s32 (1 - 1.05 d 2^-24).
          float s32 = 0.f;
          for (int t = 0; t < d; ++t) {
            const float r = __fsub_rn(xr[t], s_seed[t]);
            s32 = __fadd_rn(s32, __fmul_rn(r, r));
          }
          if (__fmul_rd(s32, 1.f - 1.05f * d * 0x1p-24f) > c32) need = false;
        }
      }
    }
    if (need) {
      double s = 0.0;
      bool exact = false;
      if constexpr (sizeof(T) == 4) exact = sqd_seq_f32(xr, s_seed, d, P.lg_d, s);
      if (!exact) {
        s = 0.0;
        for (int t = 0; t < d; ++t) s = __dadd_rn(s, sq_term(xr[t], s_seed[t]));
      }
      if (s < cur) {
        cur = s;
        lab = j - 1;
      }
      dd[gi] = cur;
      dd32[gi] = __double2float_ru(cur);
      labels[gi] = lab;
    }
  }
  const double tot = block_sum_fixed<kBlk>(live ? cur : 0.0);
  if (threadIdx.x == 0) part[b] = tot;
}

// The reference's f64 sequential sum of the terms fl32((x_t - c_t)^2) of an
// f32 row (zero past d, padded width D, 16-byte aligned) against the seed
// c in shared memory, given emin / emax of its nonzero terms, recomputing the
// terms from the row (a second read, from cache) instead of holding them:
// the integer sum where no running sum can round, else the sequential
// reproduction (both as sqd_terms), else the f64 additions themselves.
template <int D>
__device__ __noinline__ double pp_exact_row(const float *__restrict__ xr, const float *s_seed, int d, int lg_d,
                                            uint32_t emn, uint32_t emx) {
  if (emn == 256u) return 0.0;
  const float4 *x4 = reinterpret_cast<const float4 *>(xr);
  if (emx < 255u && emx - emn <= 24u && (int)(emx - emn) <= 29 - lg_d) {
    uint32_t lo[4] = {0u, 0u, 0u, 0u}, hi[4] = {0u, 0u, 0u, 0u};
#pragma unroll 4
    for (int q = 0; q < D / 4; ++q) {
      const float4 v = x4[q];
      const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float r = __fsub_rn(vv[c], s_seed[4 * q + c]);
        const uint32_t u = __float_as_uint(__fmul_rn(r, r));
        const uint32_t e = u >> 23;
        const uint32_t m = u ? (u & 0x7fffffu) | (e ? 0x800000u : 0u) : 0u;
        const uint32_t sh = max(e, 1u) - emn;  // <= 24 for every nonzero term (0 terms add nothing)
        lo[c] += (m << (sh & 31u)) & 0xffffffu;
        hi[c] += sh ? m >> (24u - sh) : 0u;
      }
    }
    const unsigned long long S = ((unsigned long long)(hi[0] + hi[1] + hi[2] + hi[3]) << 24) +
                                 (unsigned long long)(lo[0] + lo[1] + lo[2] + lo[3]);
    return sqd_from_units(S, emn);
  }
  if (emx < 255u && (int)(emx - emn) <= 38 - lg_d) {
    unsigned long long S = 0;
    for (int t = 0; t < d; ++t) {
      const float r = __fsub_rn(xr[t], s_seed[t]);
      const uint32_t u = __float_as_uint(__fmul_rn(r, r));
      if (u != 0u) {
        const int e = (int)(u >> 23);
        const uint32_t m = (u & 0x7fffffu) | (e ? 0x800000u : 0u);
        S += (unsigned long long)m << (max(e, 1) - (int)emn);  // stays below 2^63
        if (S >> 53) {  // more than 53 significant bits: round as the f64 addition does
          const int drop = 11 - __clzll((long long)S);
          const unsigned long long half = 1ull << (drop - 1), rem = S & ((half << 1) - 1ull);
          unsigned long long qv = S >> drop;
          if (rem > half || (rem == half && (qv & 1ull))) ++qv;
          S = qv << drop;
        }
      }
    }
    const int pbit = 63 - __clzll((long long)S);
    const unsigned long long mant = pbit <= 52 ? S << (52 - pbit) : S >> (pbit - 52);
    const int ex = pbit + (int)emn - 150 + 1023;
    return __longlong_as_double((long long)(((unsigned long long)ex << 52) | (mant & 0xfffffffffffffull)));
  }
  double s = 0.0;
  for (int t = 0; t < d; ++t) {
    const float r = __fsub_rn(xr[t], s_seed[t]);
    s = __dadd_rn(s, (double)__fmul_rn(r, r));
  }
  return s;
}

// The same update for f32 rows of padded width D: the row is read with
// 16-byte loads only when the far test leaves it, and streamed: its terms
// fl32((x_t - c_t)^2) give the f32 lower bound and the exponent range of the
// terms, and only when the bound cannot settle the row is it read again for
// the exact value (pp_exact_row).  Holding no row in registers leaves room
// for four CTAs per SM.  One CTA per 256-row block of the width's problems
// with k >= j (cls_blocks lists them, largest k first).
template <int D>
__global__ void __launch_bounds__(kBlk, 4)
batch_pp_update32_kernel(const int32_t *__restrict__ cls_blocks, const int32_t *__restrict__ block_prob,
                         const BProb *__restrict__ probs, const BState *__restrict__ st,
                         const float *__restrict__ X, double *__restrict__ dd, float *__restrict__ dd32,
                         int32_t *__restrict__ labels, double *__restrict__ part,
                         const float *__restrict__ seed_cc, int j, PPFar32 far) {
  __shared__ __align__(16) float s_seed[D];
  const int b = cls_blocks[blockIdx.x];
  const int p = block_prob[b];
  const BProb P = probs[p];
  const int64_t ci = st[p].pp_chosen;
  if (threadIdx.x < D) s_seed[threadIdx.x] = X[P.x_off + ci * D + threadIdx.x];
  __syncthreads();
  const int64_t il = (int64_t)(b - P.b0) * kBlk + threadIdx.x;
  const bool live = il < P.n;
  const int64_t gi = P.row0 + il;
  const bool first = j == 1;
  double cur = 0.0;
  if (live) {
    cur = first ? DBL_MAX : dd[gi];
    int32_t lab = first ? 0 : labels[gi];
    const int d = P.d;
    const float c32 = first ? 0.f : dd32[gi];
    if (first || !pp_far32(seed_cc[P.k_off + lab], c32, far)) {
      const float *xr = X + P.x_off + il * D;
      const float4 *x4 = reinterpret_cast<const float4 *>(xr);
      float s32 = 0.f;
      uint32_t emn = 256u, emx = 0u;
#pragma unroll 4
      for (int q = 0; q < D / 4; ++q) {
        const float4 v = __ldg(x4 + q);
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float r = __fsub_rn(vv[c], s_seed[4 * q + c]);
          const float tv = __fmul_rn(r, r);
          if (4 * q + c < d) s32 = __fadd_rn(s32, tv);
          const uint32_t u = __float_as_uint(tv), e = max(u >> 23, 1u);
          emn = min(emn, u ? e : 256u);
          emx = max(emx, u ? e : 0u);
        }
      }
      // the terms summed in f32 bound the reference's f64 sum from below by
      // s32 (1 - 1.05 d 2^-24): above the current distance, the row keeps it
      if (first || !(__fmul_rd(s32, 1.f - 1.05f * d * 0x1p-24f) > c32)) {
        const double s = pp_exact_row<D>(xr, s_seed, d, P.lg_d, emn, emx);
        if (s < cur) {
          cur = s;
          lab = j - 1;
        }
        dd[gi] = cur;
        dd32[gi] = __double2float_ru(cur);
        labels[gi] = lab;
      }
    }
  }
  const double tot = block_sum_fixed<kBlk>(live ? cur : 0.0);
  if (threadIdx.x == 0) part[b] = tot;
}

// ---------------------------------------------------------------------------
// k-means++ selection of seed j (kmeans.rs:381-396), one CTA per problem with
// k > j: sum = sequential f64 sum of d, cutoff = u * sum, index = the first
// i whose sequential prefix >= cutoff.  As in the single-problem kernel, a
// parallel prefix locates the crossing and a rigorous bound on both
// summations certifies it; a cutoff inside the rounding band is replayed
// sequentially.  Then the seed's row and its gaps to the earlier seeds.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kSelT)
batch_pp_select_kernel(const BProb *__restrict__ probs, BState *st, const T *__restrict__ X,
                       const double *__restrict__ dd_all, const double *__restrict__ part_all,
                       const double *__restrict__ uniforms, int64_t *__restrict__ seed_idx, T *__restrict__ seed_x,
                       float *__restrict__ seed_cc, int j, const int32_t *__restrict__ plist) {
  __shared__ double s_incl[kSelT];
  __shared__ double s_wtot[32];
  __shared__ int s_chunk;
  __shared__ long long s_pick;
  const int p = plist ? plist[blockIdx.x] : (int)blockIdx.x;  // plist: one width class's problems
  const BProb P = probs[p];
  BState *S = st + p;
  const double *part = part_all + P.b0;
  const double *dd = dd_all + P.row0;
  const int nb = P.nb;
  const int64_t n = P.n;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int chunk = (nb + kSelT - 1) / kSelT;
  const int b0 = min(nb, t * chunk), b1 = min(nb, b0 + chunk);
  double loc = 0.0;
  for (int b = b0; b < b1; ++b) loc = __dadd_rn(loc, part[b]);
  double v = warp_incl_scan(loc);
  if (lane == 31) s_wtot[w] = v;
  if (t == 0) s_chunk = kSelT;
  __syncthreads();
  if (w == 0) s_wtot[lane] = warp_incl_scan(lane < kSelT / 32 ? s_wtot[lane] : 0.0);
  __syncthreads();
  if (w > 0) v = __dadd_rn(v, s_wtot[w - 1]);
  s_incl[t] = v;
  __syncthreads();
  const double total = s_incl[kSelT - 1];
  const double u = uniforms[P.u_off + j - 1];
  const double cutoff = __dmul_rn(u, total);
  const double depth_q = (double)chunk + 2.0 * kSelT + 2.0 * kBlk + 64.0;
  {
    const double excl = t > 0 ? s_incl[t - 1] : 0.0;
    if (b1 > b0 && v >= cutoff && !(excl >= cutoff)) atomicMin(&s_chunk, t);
  }
  __syncthreads();
  if (w == 0) {
    const bool finite = isfinite(total) && total < DBL_MAX;
    const double tol_tot = pp_tol(total, (double)n + depth_q);
    const double cut_lo = __dmul_rn(u, __dsub_rn(total, tol_tot));
    const double cut_hi = __dmul_rn(u, __dadd_rn(total, tol_tot));
    int64_t pick = -1;
    if (finite && s_chunk < kSelT) {
      const int c = s_chunk;
      const int cb0 = c * chunk, cb1 = min(nb, cb0 + chunk);
      const Crossing cb = warp_first_crossing(part + cb0, cb1 - cb0, c > 0 ? s_incl[c - 1] : 0.0, cutoff);
      if (cb.t < cb1 - cb0) {
        const int64_t i0 = (int64_t)(cb0 + cb.t) * kBlk, i1 = min(n, i0 + kBlk);
        const Crossing ci = warp_first_crossing(dd + i0, (int)(i1 - i0), cb.qprev, cutoff);
        if (ci.t < i1 - i0) {
          const int64_t i = i0 + ci.t;
          const bool above = __dsub_rn(ci.q, pp_tol(ci.q, (double)i + depth_q)) >= cut_hi;
          const bool below = i == 0 ? (0.0 < cut_lo)
                                    : (__dadd_rn(ci.qprev, pp_tol(ci.qprev, (double)i + depth_q)) < cut_lo);
          if (above && below) pick = i;
        }
      }
    }
    if (lane == 0) s_pick = pick;
    __syncwarp();
  }
  __syncthreads();
  if (s_pick < 0) {  // inside the rounding band: the exact sequential sum and prefix, by the CTA
    double sum = 0.0;
    int64_t index = n;
    seq_exact_pass<kSelT>(dd, n, false, 0.0, &sum, nullptr);
    seq_exact_pass<kSelT>(dd, n, true, __dmul_rn(u, sum), nullptr, &index);
    if (t == 0) {
      s_pick = index < n ? index : n - 1;
      S->pp_replays += 1;
    }
    __syncthreads();
  }
  if (t == 0) {
    S->pp_chosen = s_pick;
    seed_idx[P.k_off + j] = s_pick;
  }
  const T *xp = X + P.x_off + (int64_t)s_pick * P.D;
  for (int c = t; c < P.d; c += kSelT) seed_x[P.c_off + (int64_t)j * P.d + c] = xp[c];
  if constexpr (sizeof(T) == 4) pp_seed_gaps<kSelT>(xp, P.d, seed_x + P.c_off, j, seed_cc + P.k_off);
}

// ---------------------------------------------------------------------------
// Tuning table: per (padded width D, cluster class) the centroids per inner
// pass (CU) and rows per work item of the assignment kernel.
// ---------------------------------------------------------------------------
constexpr int kNumKC = 5;
struct Tune {
  bool ready = false;
  int cu[kNumD][kNumKC];
  int rows[kNumD][kNumKC];
  float us[kNumD][kNumKC];
};
Tune g_tune;
std::mutex g_tune_mutex;

int dclass(int D) { return D <= 8 ? 0 : D <= 16 ? 1 : D <= 32 ? 2 : 3; }
int kclass(int k) { return k <= 8 ? 0 : k <= 16 ? 1 : k <= 32 ? 2 : k <= 64 ? 3 : 4; }
const int kClassK[kNumKC] = {8, 16, 32, 64, 128};
const int kClassD[kNumD] = {8, 16, 32, 64};

int g_variant_override = -1;  // sc_debug_batch_variant

void tune_choice(int D, int k, int *cu, int *rows) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  if (g_tune.ready) {
    *cu = g_tune.cu[dclass(D)][kclass(k)];
    *rows = g_tune.rows[dclass(D)][kclass(k)];
  } else {
    *cu = 4;
    *rows = 2048;
  }
  if (g_variant_override >= 0) *cu = g_variant_override;
}

int ceil_log2i(int64_t v) {
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}

size_t esz(int dtype) { return dtype == SC_F32 ? 4 : 8; }

// Arena of the device buffers of one batch.
struct Arena {
  char *base = nullptr;
  size_t off = 0, cap = 0;
  template <class U>
  U *take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    U *p = (U *)(base + off);
    off += (count ? count : 1) * sizeof(U);
    return p;
  }
};

struct CopyJob {
  const uint4 *src;
  uint4 *dst;
  int64_t n16;
};

struct Batch {
  int dtype = SC_F32;
  int count = 0;
  std::vector<BProb> probs;       // internal order (k descending)
  std::vector<int> order;         // internal index -> caller's index
  std::vector<int32_t> block_prob;
  std::vector<int32_t> cls_blocks;  // blocks of each width's problems (largest k first), classes in order
  int cls_off[kNumD + 1] = {};
  int32_t *d_cls_blocks = nullptr;
  std::vector<int32_t> cls_probs;  // each width's problems, classes in order
  int cls_poff[kNumD + 1] = {};
  int32_t *d_cls_probs = nullptr;
  std::vector<BItem> items;         // grouped by padded width, each group largest first
  int item_off[kNumD + 1] = {};     // group dc = items [item_off[dc], item_off[dc + 1])
  size_t smem_d[kNumD] = {};        // dynamic shared memory of each width's kernel
  int grid_d[kNumD] = {};           // persistent CTAs of each width's kernel
  std::vector<double> uniforms;
  std::vector<int64_t> first;
  int64_t rows = 0, xelems = 0, kd = 0, k32 = 0, ksum = 0;
  int blocks = 0, kmax = 0, max_iter = 0;
  bool needs_pad = false;
  // device
  cudaStream_t s = nullptr;
  cudaStream_t side[3] = {nullptr, nullptr, nullptr};  // streams of the width classes' parallel chains
  bool chains_open = false;  // set-up left each class's work on its own stream (no join)
  void *mem = nullptr;
  void *X = nullptr, *seed_x = nullptr;
  int32_t *labels = nullptr, *d_block_prob = nullptr;
  double *dd = nullptr, *part = nullptr, *cent64 = nullptr, *d_uniforms = nullptr;
  float *dd32 = nullptr, *cent32 = nullptr, *seed_cc = nullptr;
  Acc128 *acc = nullptr;
  unsigned long long *cnt = nullptr, *absmax = nullptr;
  int64_t *sizes = nullptr, *seed_idx = nullptr, *d_first = nullptr;
  BProb *d_probs = nullptr;
  BState *st = nullptr;
  BItem *d_items = nullptr;
  unsigned *heads = nullptr;  // one queue head per (graph iteration, width), then the seeding pass's
  int *active = nullptr;
  CopyJob *d_jobs = nullptr;  // gather table of rows read in place from host memory
};

// Phase times of one batched call, printed to stderr when the environment
// variable SMARTCORE_GB300_TRACE is set (each mark waits for the stream, so
// tracing itself serialises the phases).
struct PhaseTrace {
  bool on = std::getenv("SMARTCORE_GB300_TRACE") != nullptr;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  std::string line;
  void mark(const char *name, cudaStream_t s) {
    if (!on) return;
    if (s) cudaStreamSynchronize(s);
    const auto t = std::chrono::steady_clock::now();
    char buf[96];
    snprintf(buf, sizeof buf, " %s %.2f ms", name, std::chrono::duration<double, std::milli>(t - t0).count());
    line += buf;
    t0 = t;
  }
  ~PhaseTrace() {
    if (on) fprintf(stderr, "[smartcore_gb300] sc_kmeans_fit_batched:%s\n", line.c_str());
  }
};

// Dynamic shared memory of the assignment kernel for problem P: centroids
// (f32 and ||c||^2), 64-bit sums and counts.
size_t assign_smem(const BProb &P) {
  return (size_t)((P.k + 7) & ~7) * (P.D + 1) * 4 + (size_t)P.k * P.d * 8 + (size_t)P.k * 4 + 64;
}

// Work items of problem q with the given rows per item and variant.
void add_items(std::vector<BItem> &items, int q, int n, int rows, int cu) {
  for (int r0 = 0; r0 < n; r0 += rows) items.push_back(BItem{q, r0, std::min(n, r0 + rows), cu});
}

// Layout of the batch (host side): offsets, blocks, items sorted by cost.
void plan_batch(Batch &B, const std::vector<int64_t> &n, const std::vector<int64_t> &d, const std::vector<int64_t> &k,
                const std::vector<int64_t> &max_iter, const std::vector<int> &caller_index) {
  const int m = (int)n.size();
  std::vector<int> idx(m);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return k[a] > k[b]; });
  B.count = m;
  B.probs.resize(m);
  B.order.resize(m);
  const int align = B.dtype == SC_F32 ? 4 : 2;  // 16-byte problem starts
  int64_t xo = 0, row = 0, co = 0, c32 = 0;
  int ko = 0, uo = 0, blk = 0;
  for (int q = 0; q < m; ++q) {
    const int i = idx[q];
    BProb &P = B.probs[q];
    memset(&P, 0, sizeof P);
    P.n = (int32_t)n[i];
    P.d = (int32_t)d[i];
    P.D = pad_width(P.d);
    P.k = (int32_t)k[i];
    P.max_iter = (int32_t)std::min<int64_t>(max_iter[i], 1 << 30);
    P.x_off = xo;
    P.row0 = row;
    P.c_off = co;
    P.c32_off = c32;
    P.k_off = ko;
    P.u_off = uo;
    P.b0 = blk;
    P.nb = (int32_t)((P.n + kBlk - 1) / kBlk);
    P.lg_d = ceil_log2i(P.d);
    if (P.D != P.d) B.needs_pad = true;
    xo += ((int64_t)P.n * P.D + align - 1) / align * align;
    row += P.n;
    co += (int64_t)P.k * P.d;
    c32 += (int64_t)((P.k + 7) & ~7) * (P.D + 1);
    ko += P.k;
    uo += P.k - 1;
    blk += P.nb;
    for (int b = 0; b < P.nb; ++b) B.block_prob.push_back(q);
    B.order[q] = caller_index[i];
    B.kmax = std::max(B.kmax, P.k);
    B.max_iter = std::max(B.max_iter, P.max_iter);
    int cu, rows;
    tune_choice(P.D, P.k, &cu, &rows);
    P.rows = rows;
    B.smem_d[dclass(P.D)] = std::max(B.smem_d[dclass(P.D)], assign_smem(P));
  }
  // work items grouped by width, largest cost (rows x k) first in each group
  std::vector<BItem> groups[kNumD];
  for (int q = 0; q < m; ++q) {
    const BProb &P = B.probs[q];
    int cu, rows;
    tune_choice(P.D, P.k, &cu, &rows);
    add_items(groups[dclass(P.D)], q, P.n, P.rows, cu);
  }
  for (int dc = 0; dc < kNumD; ++dc) {
    std::stable_sort(groups[dc].begin(), groups[dc].end(), [&](const BItem &a, const BItem &b) {
      return (int64_t)(a.r1 - a.r0) * B.probs[a.prob].k > (int64_t)(b.r1 - b.r0) * B.probs[b.prob].k;
    });
    B.item_off[dc] = (int)B.items.size();
    B.items.insert(B.items.end(), groups[dc].begin(), groups[dc].end());
  }
  B.item_off[kNumD] = (int)B.items.size();
  for (int dc = 0; dc < kNumD; ++dc) {
    B.cls_off[dc] = (int)B.cls_blocks.size();
    for (int q = 0; q < m; ++q)
      if (dclass(B.probs[q].D) == dc)
        for (int b = 0; b < B.probs[q].nb; ++b) B.cls_blocks.push_back(B.probs[q].b0 + b);
  }
  B.cls_off[kNumD] = (int)B.cls_blocks.size();
  for (int dc = 0; dc < kNumD; ++dc) {
    B.cls_poff[dc] = (int)B.cls_probs.size();
    for (int q = 0; q < m; ++q)
      if (dclass(B.probs[q].D) == dc) B.cls_probs.push_back(q);
  }
  B.cls_poff[kNumD] = (int)B.cls_probs.size();
  B.xelems = xo;
  B.rows = row;
  B.kd = co;
  B.k32 = c32;
  B.ksum = ko;
  B.blocks = blk;
}

sc_status alloc_batch(Batch &B) {
  Arena A;
  auto layout = [&](Arena &a) {
    B.X = a.take<char>((size_t)B.xelems * esz(B.dtype));
    B.seed_x = a.take<char>((size_t)B.kd * esz(B.dtype));
    B.labels = a.take<int32_t>(B.rows);
    B.dd = a.take<double>(B.rows);
    B.dd32 = a.take<float>(B.rows);
    B.part = a.take<double>(B.blocks);
    B.cent64 = a.take<double>(B.kd);
    B.cent32 = a.take<float>(B.k32);
    B.acc = a.take<Acc128>(B.kd);
    B.cnt = a.take<unsigned long long>(B.ksum);
    B.sizes = a.take<int64_t>(B.ksum);
    B.seed_idx = a.take<int64_t>(B.ksum);
    B.seed_cc = a.take<float>(B.ksum);
    B.d_uniforms = a.take<double>(B.uniforms.size());
    B.d_first = a.take<int64_t>(B.count);
    B.absmax = a.take<unsigned long long>(B.count);
    B.d_probs = a.take<BProb>(B.count);
    B.st = a.take<BState>(B.count);
    B.d_block_prob = a.take<int32_t>(B.blocks);
    B.d_cls_blocks = a.take<int32_t>(B.cls_blocks.size());
    B.d_cls_probs = a.take<int32_t>(B.cls_probs.size());
    B.d_items = a.take<BItem>(B.items.size());
    B.heads = a.take<unsigned>((size_t)(kGraphIters + 1) * kNumD);
    B.active = a.take<int>(1);
  };
  layout(A);  // sizes only (base = null)
  SC_TRY(dev_alloc(&B.mem, A.off + 256, B.s));
  Arena R;
  R.base = (char *)B.mem;
  layout(R);
  return SC_OK;
}

sc_status upload_tables(Batch &B) {
  SC_CUDA(cudaMemcpyAsync(B.d_probs, B.probs.data(), B.probs.size() * sizeof(BProb), cudaMemcpyHostToDevice, B.s));
  SC_CUDA(cudaMemcpyAsync(B.d_block_prob, B.block_prob.data(), B.block_prob.size() * sizeof(int32_t),
                          cudaMemcpyHostToDevice, B.s));
  SC_CUDA(cudaMemcpyAsync(B.d_items, B.items.data(), B.items.size() * sizeof(BItem), cudaMemcpyHostToDevice, B.s));
  SC_CUDA(cudaMemcpyAsync(B.d_cls_blocks, B.cls_blocks.data(), B.cls_blocks.size() * sizeof(int32_t),
                          cudaMemcpyHostToDevice, B.s));
  SC_CUDA(cudaMemcpyAsync(B.d_cls_probs, B.cls_probs.data(), B.cls_probs.size() * sizeof(int32_t),
                          cudaMemcpyHostToDevice, B.s));
  if (!B.uniforms.empty())
    SC_CUDA(cudaMemcpyAsync(B.d_uniforms, B.uniforms.data(), B.uniforms.size() * sizeof(double),
                            cudaMemcpyHostToDevice, B.s));
  SC_CUDA(cudaMemcpyAsync(B.d_first, B.first.data(), B.first.size() * sizeof(int64_t), cudaMemcpyHostToDevice, B.s));
  return SC_OK;
}

template <typename T, int D>
sc_status launch_assign_d(Batch &B, int dc, unsigned *head, int nitems, const BItem *items, int mode,
                          cudaStream_t st = nullptr) {
  if (nitems == 0) return SC_OK;
  // shared-memory attribute set by assign_grid
  batch_assign_kernel<T, D><<<B.grid_d[dc], kAsgThreads, B.smem_d[dc], st ? st : B.s>>>(
      items, nitems, B.d_probs, B.st, (const T *)B.X, B.cent32, B.cent64, B.labels, B.acc, B.cnt, head, B.active,
      mode);
  SC_LAUNCHED();
  return SC_OK;
}

// One assignment pass over the item groups of every width; heads[dc] is the
// queue head of width dc (cleared beforehand).
template <typename T>
sc_status launch_assign(Batch &B, unsigned *heads, int mode) {
  const BItem *it = B.d_items;
  const int *o = B.item_off;
  SC_TRY((launch_assign_d<T, 64>(B, 3, heads + 3, o[4] - o[3], it + o[3], mode)));
  SC_TRY((launch_assign_d<T, 32>(B, 2, heads + 2, o[3] - o[2], it + o[2], mode)));
  SC_TRY((launch_assign_d<T, 16>(B, 1, heads + 1, o[2] - o[1], it + o[1], mode)));
  SC_TRY((launch_assign_d<T, 8>(B, 0, heads + 0, o[1] - o[0], it + o[0], mode)));
  return SC_OK;
}

// The items of one width class only (the tuner's single-problem passes).
template <typename T>
sc_status launch_assign_class(Batch &B, int dc, unsigned *head, int nitems, const BItem *items, int mode) {
  switch (dc) {
    case 0: return launch_assign_d<T, 8>(B, 0, head, nitems, items, mode);
    case 1: return launch_assign_d<T, 16>(B, 1, head, nitems, items, mode);
    case 2: return launch_assign_d<T, 32>(B, 2, head, nitems, items, mode);
    default: return launch_assign_d<T, 64>(B, 3, head, nitems, items, mode);
  }
}

template <typename T, int D>
sc_status assign_grid_d(Batch &B, int dc, int sms) {
  if (B.item_off[dc + 1] == B.item_off[dc]) return SC_OK;
  int per = 0;
  SC_CUDA(cudaFuncSetAttribute(batch_assign_kernel<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)B.smem_d[dc]));
  SC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_assign_kernel<T, D>, kAsgThreads, B.smem_d[dc]));
  B.grid_d[dc] = sms * std::max(1, per);
  return SC_OK;
}

template <typename T>
sc_status assign_grid_t(Batch &B, int sms) {
  SC_TRY((assign_grid_d<T, 8>(B, 0, sms)));
  SC_TRY((assign_grid_d<T, 16>(B, 1, sms)));
  SC_TRY((assign_grid_d<T, 32>(B, 2, sms)));
  SC_TRY((assign_grid_d<T, 64>(B, 3, sms)));
  return SC_OK;
}

sc_status assign_grid(Batch &B, int dtype) {
  int dev = 0, sms = 0;
  SC_CUDA(cudaGetDevice(&dev));
  SC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  return dtype == SC_F32 ? assign_grid_t<float>(B, sms) : assign_grid_t<double>(B, sms);
}

// Rows the device can read where they are (pinned, mapped host memory):
// copied by SM loads, 16 bytes each, every CTA striding over every job.
__global__ void __launch_bounds__(256) gather_host_rows_kernel(const CopyJob *__restrict__ jobs, int njobs) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int q = 0; q < njobs; ++q) {
    const CopyJob jb = jobs[q];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < jb.n16; i += 4 * stride) {  // four loads in flight
      const uint4 a = jb.src[i], b = jb.src[i + stride], c = jb.src[i + 2 * stride], e = jb.src[i + 3 * stride];
      jb.dst[i] = a;
      jb.dst[i + stride] = b;
      jb.dst[i + 2 * stride] = c;
      jb.dst[i + 3 * stride] = e;
    }
    for (; i < jb.n16; i += stride) jb.dst[i] = jb.src[i];
  }
}

// The side streams of a batch's parallel width-class launches.
sc_status ensure_side_streams(Batch &B) {
  for (int i = 0; i < 3; ++i)
    if (!B.side[i]) SC_CUDA(cudaStreamCreateWithFlags(&B.side[i], cudaStreamNonBlocking));
  return SC_OK;
}

// Stream of width class dc's chain: the widest on B.s, the others on the side
// streams.
cudaStream_t class_stream(const Batch &B, int dc) { return dc == kNumD - 1 ? B.s : B.side[kNumD - 2 - dc]; }

// Fork / join events (no timing), destroyed with the set.
struct EventSet {
  cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
  sc_status create() {
    for (int i = 0; i < 4; ++i) SC_CUDA(cudaEventCreateWithFlags(&e[i], cudaEventDisableTiming));
    return SC_OK;
  }
  ~EventSet() {
    for (int i = 0; i < 4; ++i)
      if (e[i]) cudaEventDestroy(e[i]);
  }
};

// Clears what the set-up accumulates (max |x|, the initial means' sums and
// queue heads, the count of running problems), then forks the side streams
// from B.s: each width class's work from here on runs on its own stream.
sc_status begin_chains(Batch &B) {
  cudaStream_t s = B.s;
  SC_CUDA(cudaMemsetAsync(B.absmax, 0, (size_t)B.count * sizeof(unsigned long long), s));
  SC_CUDA(cudaMemsetAsync(B.acc, 0, (size_t)B.kd * sizeof(Acc128), s));
  SC_CUDA(cudaMemsetAsync(B.cnt, 0, (size_t)B.ksum * sizeof(unsigned long long), s));
  SC_CUDA(cudaMemsetAsync(B.heads + (size_t)kGraphIters * kNumD, 0, kNumD * sizeof(unsigned), s));
  const int act = B.count;
  SC_CUDA(cudaMemcpyAsync(B.active, &act, sizeof act, cudaMemcpyHostToDevice, s));
  SC_TRY(ensure_side_streams(B));
  EventSet ev;
  SC_TRY(ev.create());
  SC_CUDA(cudaEventRecord(ev.e[0], s));
  for (int i = 0; i < 3; ++i) SC_CUDA(cudaStreamWaitEvent(B.side[i], ev.e[0], 0));
  B.chains_open = true;
  return SC_OK;
}

// Joins the side streams into B.s.
sc_status join_chains(Batch &B) {
  EventSet ev;
  SC_TRY(ev.create());
  for (int i = 0; i < 3; ++i)
    if (B.side[i]) {
      SC_CUDA(cudaEventRecord(ev.e[1 + i], B.side[i]));
      SC_CUDA(cudaStreamWaitEvent(B.s, ev.e[1 + i], 0));
    }
  B.chains_open = false;
  return SC_OK;
}

// Device phases of a batch: scan, scales, k-means++, initial means.
template <typename T>
sc_status run_setup(Batch &B) {
  cudaStream_t s = B.s;
  if (!B.chains_open) SC_TRY(begin_chains(B));
  const PPFar32 far = pp_far_bound32(kMaxBD);  // d = 64 bounds the far test of every width
  unsigned *seed_heads = B.heads + (size_t)kGraphIters * kNumD;
  if constexpr (sizeof(T) == 4) {
    // One chain per width class, on the class's stream after its rows (its
    // problems, largest k first, and their blocks are prefixes of the
    // class's lists at every draw): the scan of ||x||^2 and max |x|, the
    // start values and scales, each draw's update and the class's
    // selection, then the initial means of the seeding partition.  The
    // chains run side by side and stay open: the class's Lloyd loop follows
    // on the same stream.
    const float *xf = (const float *)B.X;
    for (int dc = kNumD - 1; dc >= 0; --dc) {
      const int np = B.cls_poff[dc + 1] - B.cls_poff[dc];
      if (np == 0) continue;
      const int32_t *pl = B.cls_probs.data() + B.cls_poff[dc];
      const int32_t *cb = B.d_cls_blocks + B.cls_off[dc];
      const int32_t *dpl = B.d_cls_probs + B.cls_poff[dc];
      cudaStream_t cs = class_stream(B, dc);
      int ge = np, gt = np, nb = B.cls_off[dc + 1] - B.cls_off[dc];
      switch (dc) {
        case 0: batch_scan32_kernel<8><<<nb, kBlk, 0, cs>>>(cb, B.d_block_prob, B.d_probs, xf, B.part, B.absmax); break;
        case 1: batch_scan32_kernel<16><<<nb, kBlk, 0, cs>>>(cb, B.d_block_prob, B.d_probs, xf, B.part, B.absmax); break;
        case 2: batch_scan32_kernel<32><<<nb, kBlk, 0, cs>>>(cb, B.d_block_prob, B.d_probs, xf, B.part, B.absmax); break;
        default: batch_scan32_kernel<64><<<nb, kBlk, 0, cs>>>(cb, B.d_block_prob, B.d_probs, xf, B.part, B.absmax); break;
      }
      SC_LAUNCHED();
      batch_init_kernel<T><<<np, 64, 0, cs>>>(B.d_probs, np, B.st, B.part, B.d_first, (const T *)B.X,
                                               (T *)B.seed_x, B.seed_idx, B.absmax, dpl);
      SC_LAUNCHED();
      for (int j = 1; j <= B.probs[pl[0]].k; ++j) {
        while (ge > 0 && B.probs[pl[ge - 1]].k < j) nb -= B.probs[pl[--ge]].nb;
        while (gt > 0 && B.probs[pl[gt - 1]].k <= j) --gt;
        if (nb > 0) {
          switch (dc) {
            case 0: batch_pp_update32_kernel<8><<<nb, kBlk, 0, cs>>>(cb, B.d_block_prob, B.d_probs, B.st, xf, B.dd, B.dd32, B.labels, B.part, B.seed_cc, j, far); break;
            case 1: batch_pp_update32_kernel<16><<<nb, kBlk, 0, cs>>>(cb, B.d_block_prob, B.d_probs, B.st, xf, B.dd, B.dd32, B.labels, B.part, B.seed_cc, j, far); break;
            case 2: batch_pp_update32_kernel<32><<<nb, kBlk, 0, cs>>>(cb, B.d_block_prob, B.d_probs, B.st, xf, B.dd, B.dd32, B.labels, B.part, B.seed_cc, j, far); break;
            default: batch_pp_update32_kernel<64><<<nb, kBlk, 0, cs>>>(cb, B.d_block_prob, B.d_probs, B.st, xf, B.dd, B.dd32, B.labels, B.part, B.seed_cc, j, far); break;
          }
          SC_LAUNCHED();
        }
        if (gt > 0) {
          batch_pp_select_kernel<T><<<gt, kSelT, 0, cs>>>(B.d_probs, B.st, (const T *)B.X, B.dd, B.part, B.d_uniforms,
                                                          B.seed_idx, (T *)B.seed_x, B.seed_cc, j, dpl);
          SC_LAUNCHED();
        }
      }
      const int ni = B.item_off[dc + 1] - B.item_off[dc];
      const BItem *it = B.d_items + B.item_off[dc];
      switch (dc) {
        case 0: SC_TRY((launch_assign_d<T, 8>(B, 0, seed_heads + 0, ni, it, 1, cs))); break;
        case 1: SC_TRY((launch_assign_d<T, 16>(B, 1, seed_heads + 1, ni, it, 1, cs))); break;
        case 2: SC_TRY((launch_assign_d<T, 32>(B, 2, seed_heads + 2, ni, it, 1, cs))); break;
        default: SC_TRY((launch_assign_d<T, 64>(B, 3, seed_heads + 3, ni, it, 1, cs))); break;
      }
      batch_finalize_kernel<<<np, kFinT, 0, cs>>>(B.d_probs, B.st, B.acc, B.cnt, B.cent64, B.cent32, B.sizes, 1,
                                                  B.active, dpl);
      SC_LAUNCHED();
    }
    return SC_OK;
  } else {
    SC_TRY(join_chains(B));  // the rows of every class, then the whole set-up on B.s
    batch_scan_kernel<T><<<B.blocks, kBlk, 0, s>>>(B.d_block_prob, B.d_probs, (const T *)B.X, B.part, B.absmax);
    SC_LAUNCHED();
    batch_init_kernel<T><<<B.count, 64, 0, s>>>(B.d_probs, B.count, B.st, B.part, B.d_first, (const T *)B.X,
                                               (T *)B.seed_x, B.seed_idx, B.absmax, nullptr);
    SC_LAUNCHED();
    // k-means++: problems sorted by k descending, so those still drawing at
    // step j are a prefix of the problems and their blocks a prefix of the
    // blocks
    std::vector<int> blocks_upto(B.count + 1, 0);
    for (int q = 0; q < B.count; ++q) blocks_upto[q + 1] = blocks_upto[q] + B.probs[q].nb;
    int q_ge = B.count, q_gt = B.count;
    for (int j = 1; j <= B.kmax; ++j) {
      while (q_ge > 0 && B.probs[q_ge - 1].k < j) --q_ge;
      while (q_gt > 0 && B.probs[q_gt - 1].k <= j) --q_gt;
      if (q_ge > 0) {
        batch_pp_update_kernel<T><<<blocks_upto[q_ge], kBlk, 0, s>>>(B.d_block_prob, B.d_probs, B.st,
                                                                     (const T *)B.X, B.dd, B.dd32, B.labels, B.part,
                                                                     B.seed_cc, j, far);
        SC_LAUNCHED();
      }
      if (q_gt > 0) {
        batch_pp_select_kernel<T><<<q_gt, kSelT, 0, s>>>(B.d_probs, B.st, (const T *)B.X, B.dd, B.part,
                                                         B.d_uniforms, B.seed_idx, (T *)B.seed_x, B.seed_cc, j,
                                                         nullptr);
        SC_LAUNCHED();
      }
    }
    // initial means of the seeding partition
    SC_TRY(launch_assign<T>(B, seed_heads, 1));
    batch_finalize_kernel<<<B.count, kFinT, 0, s>>>(B.d_probs, B.st, B.acc, B.cnt, B.cent64, B.cent32, B.sizes, 1,
                                                    B.active, nullptr);
    SC_LAUNCHED();
    return SC_OK;
  }
}

// The Lloyd loop: per width class a graph of G = min(max_iter, 32)
// iterations (the class's queue heads cleared, then G x (assignment,
// finalize)), launched on the class's stream so that it follows the class's
// own set-up; the classes are joined after each round of graphs, which
// repeats until every problem has stopped.  A stopped problem's items and
// finalize return at once.
template <typename T>
sc_status run_lloyd(Batch &B) {
  cudaStream_t s = B.s;
  const int G = std::min(B.max_iter, kGraphIters);
  SC_TRY(ensure_side_streams(B));
  EventSet evs;
  SC_TRY(evs.create());
  cudaEvent_t *ev = evs.e;
  if (!B.chains_open) {  // every class waits for the set-up on B.s
    SC_CUDA(cudaEventRecord(ev[0], s));
    for (int i = 0; i < 3; ++i) SC_CUDA(cudaStreamWaitEvent(B.side[i], ev[0], 0));
  }
  B.chains_open = false;
  cudaGraph_t graph[kNumD] = {};
  cudaGraphExec_t exec[kNumD] = {};
  sc_status r = SC_OK;
  for (int dc = kNumD - 1; dc >= 0 && r == SC_OK; --dc) {
    const int np = B.cls_poff[dc + 1] - B.cls_poff[dc], ni = B.item_off[dc + 1] - B.item_off[dc];
    if (np == 0) continue;
    cudaStream_t cs = class_stream(B, dc);
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "cudaStreamBeginCapture");
      break;
    }
    unsigned *heads = B.heads + (size_t)dc * kGraphIters;
    if (cudaMemsetAsync(heads, 0, (size_t)G * sizeof(unsigned), cs) != cudaSuccess)
      r = cuda_fail(cudaGetLastError(), "memset");
    const BItem *it = B.d_items + B.item_off[dc];
    for (int t = 0; t < G && r == SC_OK; ++t) {
      switch (dc) {
        case 0: r = launch_assign_d<T, 8>(B, 0, heads + t, ni, it, 0, cs); break;
        case 1: r = launch_assign_d<T, 16>(B, 1, heads + t, ni, it, 0, cs); break;
        case 2: r = launch_assign_d<T, 32>(B, 2, heads + t, ni, it, 0, cs); break;
        default: r = launch_assign_d<T, 64>(B, 3, heads + t, ni, it, 0, cs); break;
      }
      if (r != SC_OK) break;
      batch_finalize_kernel<<<np, kFinT, 0, cs>>>(B.d_probs, B.st, B.acc, B.cnt, B.cent64, B.cent32, B.sizes, 0,
                                                  B.active, B.d_cls_probs + B.cls_poff[dc]);
      note_launch();
      const cudaError_t le = cudaGetLastError();
      if (le != cudaSuccess) r = cuda_fail(le, "batch_finalize_kernel");
    }
    const cudaError_t ec = cudaStreamEndCapture(cs, &graph[dc]);
    if (r == SC_OK && ec != cudaSuccess) r = cuda_fail(ec, "cudaStreamEndCapture");
    if (r == SC_OK) {
      const cudaError_t e = cudaGraphInstantiate(&exec[dc], graph[dc], 0);
      if (e != cudaSuccess) r = cuda_fail(e, "cudaGraphInstantiate");
    }
  }
  for (int done = 0; r == SC_OK && done < B.max_iter; done += G) {
    cudaError_t e = cudaSuccess;
    for (int dc = kNumD - 1; dc >= 0 && e == cudaSuccess; --dc)
      if (exec[dc]) e = cudaGraphLaunch(exec[dc], class_stream(B, dc));
    for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
      e = cudaEventRecord(ev[1 + i], B.side[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev[1 + i], 0);
    }
    int act = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&act, B.active, sizeof act, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) r = cuda_fail(e, "Lloyd graphs");
    else if (act == 0) break;
  }
  for (int dc = 0; dc < kNumD; ++dc) {
    if (exec[dc]) cudaGraphExecDestroy(exec[dc]);
    if (graph[dc]) cudaGraphDestroy(graph[dc]);
  }
  return r;
}

void free_batch(Batch &B) {
  // the side streams' work (an error may have left a chain unjoined) ends
  // before the arena is released on B.s
  for (int i = 0; i < 3; ++i)
    if (B.side[i]) {
      cudaStreamSynchronize(B.side[i]);
      cudaStreamDestroy(B.side[i]);
      B.side[i] = nullptr;
    }
  if (B.mem) dev_free(B.mem, B.s);
  B.mem = nullptr;
  if (B.d_jobs) dev_free(B.d_jobs, B.s);
  B.d_jobs = nullptr;
  if (B.s) {
    cudaStreamSynchronize(B.s);
    cudaStreamDestroy(B.s);
    B.s = nullptr;
  }
}

// ---------------------------------------------------------------------------
// Tuner: times every variant of the assignment kernel on one synthetic
// problem per (D, cluster class) and keeps the fastest.
// ---------------------------------------------------------------------------
__global__ void tune_fill_kernel(float *x, int64_t count, uint32_t seed) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)i * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    x[i] = (float)(h & 0xffffff) * 0x1p-20f - 8.f;  // uniform in [-8, 8)
  }
}

}  // namespace
}  // namespace sc

using namespace sc;

extern "C" {

sc_status sc_kmeans_fit_batched(sc_kmeans_problem *problems, int64_t count, int32_t dtype, int32_t form) {
  if (count < 0 || (count > 0 && !problems)) { set_error("invalid problem list"); return SC_ERR_INVALID; }
  if (dtype != SC_F32 && dtype != SC_F64) { set_error("unsupported dtype %d", dtype); return SC_ERR_INVALID; }
  if (form != SC_FORM_FP64 && form != SC_FORM_SPLIT_BF16) { set_error("unknown form %d", form); return SC_ERR_INVALID; }
  if (count > (1 << 20)) { set_error("count=%lld is too large", (long long)count); return SC_ERR_INVALID; }
  // Validation of every problem first (the messages of KMeans::fit,
  // kmeans.rs:257-269), so a bad problem changes no output.
  for (int64_t i = 0; i < count; ++i) {
    sc_kmeans_problem &q = problems[i];
    q.status = SC_ERR_INVALID;
    const char *msg = nullptr;
    char buf[160];
    if (q.k < 2) { snprintf(buf, sizeof buf, "invalid number of clusters: %lld", (long long)q.k); msg = buf; }
    else if (q.max_iter == 0) { snprintf(buf, sizeof buf, "invalid maximum number of iterations: %lld", (long long)q.max_iter); msg = buf; }
    else if (q.max_iter < 0) { snprintf(buf, sizeof buf, "invalid maximum number of iterations: %lld", (long long)q.max_iter); msg = buf; }
    else if (q.n < 1 || q.d < 1 || q.d > (1 << 16) || q.n > ((int64_t)1 << 31) - 1) { snprintf(buf, sizeof buf, "invalid shape (%lld, %lld)", (long long)q.n, (long long)q.d); msg = buf; }
    else if (!q.x) msg = "null matrix pointer";
    else if (q.layout != SC_ROW_MAJOR && q.layout != SC_COL_MAJOR) msg = "unsupported layout";
    else if ((q.layout == SC_ROW_MAJOR && q.ld < q.d) || (q.layout == SC_COL_MAJOR && q.ld < q.n)) msg = "leading dimension too small";
    else if (q.first_index < 0 || q.first_index >= q.n) { snprintf(buf, sizeof buf, "first seed index %lld out of range", (long long)q.first_index); msg = buf; }
    else if (!q.uniforms) msg = "null uniforms";
    else if (q.k > (1 << 20)) { snprintf(buf, sizeof buf, "k=%lld is too large", (long long)q.k); msg = buf; }
    if (msg) {
      set_error("problem %lld: %s", (long long)i, msg);
      return SC_ERR_INVALID;
    }
  }
  for (int64_t i = 0; i < count; ++i) problems[i].status = SC_OK;
  // Problems beyond the batched kernels' limits run one by one through the
  // single-problem path (same results, still on the GPU).
  std::vector<int64_t> n, d, k, mi;
  std::vector<int> who;
  for (int64_t i = 0; i < count; ++i) {
    sc_kmeans_problem &q = problems[i];
    if (q.d <= kMaxBD && q.k <= kMaxBK) {
      n.push_back(q.n); d.push_back(q.d); k.push_back(q.k); mi.push_back(q.max_iter); who.push_back((int)i);
      continue;
    }
    q.status = sc_kmeans_fit(q.x, dtype, q.layout, q.n, q.d, q.ld, q.k, q.max_iter, q.first_index, q.uniforms, form,
                             q.centroids_out, q.sizes_out, q.labels_out, q.distortion_out, q.iters_out);
    if (q.status != SC_OK) return q.status;
  }
  if (who.empty()) return SC_OK;

  PhaseTrace trace;
  Batch B;
  B.dtype = dtype;
  plan_batch(B, n, d, k, mi, who);
  for (int q = 0; q < B.count; ++q) {
    const sc_kmeans_problem &pr = problems[B.order[q]];
    B.first.push_back(pr.first_index);
    for (int64_t a = 0; a + 1 < pr.k; ++a) B.uniforms.push_back(pr.uniforms[a]);
  }
  // the widest class's chain (on B.s) is the longest: its blocks go first
  int prio_lo = 0, prio_hi = 0;
  if (cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess ||
      cudaStreamCreateWithPriority(&B.s, cudaStreamNonBlocking, prio_hi) != cudaSuccess)
    return cuda_fail(cudaGetLastError(), "cudaStreamCreate");
  sc_status r = SC_OK;
  do {
    trace.mark("plan", nullptr);
    if ((r = alloc_batch(B)) != SC_OK) break;
    if ((r = assign_grid(B, dtype)) != SC_OK) break;
    if ((r = upload_tables(B)) != SC_OK) break;
    trace.mark("alloc", B.s);
    // Rows into the padded layout.  Column-major rows (a transpose through a
    // staging buffer) go first on B.s; then, after the fork of the width
    // classes' streams, each class's rows on its own stream, the widest
    // class first and each class's copies after the previous class's, so
    // that the widest class's set-up starts as soon as its rows are in.
    // Rows in pinned, device-mapped host memory are read in place by one
    // gather kernel per class; the others are copied.
    const size_t es = esz(dtype);
    if (B.needs_pad && cudaMemsetAsync(B.X, 0, (size_t)B.xelems * es, B.s) != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "memset"); break; }
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    std::vector<CopyJob> jobs;  // rows the device reads in place, by class
    int jb[kNumD] = {}, je[kNumD] = {};  // class dc's jobs: [jb[dc], je[dc])
    std::vector<char> copy_q(B.count, 0);  // row-major problems copied on their class's stream
    for (int dc = kNumD - 1; dc >= 0 && r == SC_OK; --dc) {
      jb[dc] = (int)jobs.size();
      for (int i = B.cls_poff[dc]; i < B.cls_poff[dc + 1] && r == SC_OK; ++i) {
        const int q = B.cls_probs[i];
        const sc_kmeans_problem &pr = problems[B.order[q]];
        const BProb &P = B.probs[q];
        char *dst = (char *)B.X + (size_t)P.x_off * es;
        const size_t pitch = (size_t)pr.ld * es, bytes = (size_t)P.n * P.d * es;
        if (pr.layout == SC_ROW_MAJOR) {
          if (P.D == P.d && pitch == (size_t)P.d * es && bytes % 16 == 0) {
            cudaPointerAttributes at;
            if (cudaPointerGetAttributes(&at, pr.x) == cudaSuccess && at.type == cudaMemoryTypeHost &&
                at.devicePointer && ((uintptr_t)at.devicePointer & 15) == 0) {
              jobs.push_back(CopyJob{(const uint4 *)at.devicePointer, (uint4 *)dst, (int64_t)(bytes / 16)});
              continue;
            }
            cudaGetLastError();  // an unregistered pointer leaves an error behind on some drivers
          }
          copy_q[q] = 1;
          continue;
        }
        // the columns as stored, then a transpose to rows on the device
        const size_t span = (size_t)((P.d - 1) * pr.ld + P.n) * es, span_al = (span + 255) & ~(size_t)255;
        const size_t need = span_al + (size_t)P.n * P.d * es;
        if (need > tmp_bytes) {
          if (tmp) dev_free(tmp, B.s);
          tmp = nullptr;
          tmp_bytes = 0;
          if ((r = dev_alloc(&tmp, need, B.s)) != SC_OK) break;
          tmp_bytes = need;
        }
        char *rm = (char *)tmp + span_al;
        if (cudaMemcpyAsync(tmp, pr.x, span, cudaMemcpyHostToDevice, B.s) != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "upload"); break; }
        if ((r = launch_to_row_major(dtype, tmp, P.n, P.d, pr.ld, rm, B.s)) != SC_OK) break;
        const cudaError_t e = P.D == P.d ? cudaMemcpyAsync(dst, rm, bytes, cudaMemcpyDeviceToDevice, B.s)
                                         : cudaMemcpy2DAsync(dst, (size_t)P.D * es, rm, (size_t)P.d * es,
                                                             (size_t)P.d * es, (size_t)P.n, cudaMemcpyDeviceToDevice, B.s);
        if (e != cudaSuccess) r = cuda_fail(e, "upload");
      }
      je[dc] = (int)jobs.size();
    }
    if (tmp) dev_free(tmp, B.s);
    if (r != SC_OK) break;
    if (!jobs.empty()) {
      if ((r = dev_alloc((void **)&B.d_jobs, jobs.size() * sizeof(CopyJob), B.s)) != SC_OK) break;
      if (cudaMemcpyAsync(B.d_jobs, jobs.data(), jobs.size() * sizeof(CopyJob), cudaMemcpyHostToDevice, B.s) !=
          cudaSuccess) { r = cuda_fail(cudaGetLastError(), "upload"); break; }
    }
    if ((r = begin_chains(B)) != SC_OK) break;
    {
      int dev = 0, sms = 0;
      EventSet ev;
      if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        r = cuda_fail(cudaGetLastError(), "upload");
        break;
      }
      if ((r = ev.create()) != SC_OK) break;
      for (int dc = kNumD - 1; dc >= 0 && r == SC_OK; --dc) {
        cudaStream_t cs = class_stream(B, dc);
        if (dc < kNumD - 1 && cudaStreamWaitEvent(cs, ev.e[0], 0) != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "upload"); break; }
        for (int i = B.cls_poff[dc]; i < B.cls_poff[dc + 1] && r == SC_OK; ++i) {
          const int q = B.cls_probs[i];
          if (!copy_q[q]) continue;
          const sc_kmeans_problem &pr = problems[B.order[q]];
          const BProb &P = B.probs[q];
          char *dst = (char *)B.X + (size_t)P.x_off * es;
          const size_t pitch = (size_t)pr.ld * es;
          const cudaError_t e = (P.D == P.d && pitch == (size_t)P.d * es)
                                    ? cudaMemcpyAsync(dst, pr.x, (size_t)P.n * P.d * es, cudaMemcpyHostToDevice, cs)
                                    : cudaMemcpy2DAsync(dst, (size_t)P.D * es, pr.x, pitch, (size_t)P.d * es,
                                                        (size_t)P.n, cudaMemcpyHostToDevice, cs);
          if (e != cudaSuccess) r = cuda_fail(e, "upload");
        }
        const int nj = je[dc] - jb[dc];
        if (r == SC_OK && nj > 0) {
          gather_host_rows_kernel<<<4 * sms, 256, 0, cs>>>(B.d_jobs + jb[dc], nj);
          note_launch();
          const cudaError_t le = cudaGetLastError();
          if (le != cudaSuccess) r = cuda_fail(le, "gather_host_rows_kernel");
        }
        if (r == SC_OK && cudaEventRecord(ev.e[0], cs) != cudaSuccess) r = cuda_fail(cudaGetLastError(), "upload");
      }
    }
    if (r != SC_OK) break;
    trace.mark("upload", B.s);
    r = dtype == SC_F32 ? run_setup<float>(B) : run_setup<double>(B);
    if (r != SC_OK) break;
    trace.mark("seeding", B.s);
    r = dtype == SC_F32 ? run_lloyd<float>(B) : run_lloyd<double>(B);
    if (r != SC_OK) break;
    trace.mark("lloyd", B.s);
    {  // non-finite input: an error, and no output written
      std::vector<unsigned long long> am(B.count);
      if (cudaMemcpyAsync(am.data(), B.absmax, am.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, B.s) !=
              cudaSuccess ||
          cudaStreamSynchronize(B.s) != cudaSuccess) {
        r = cuda_fail(cudaGetLastError(), "results");
        break;
      }
      for (int q = 0; q < B.count && r == SC_OK; ++q) {
        double a;
        memcpy(&a, &am[q], sizeof a);
        if (!(a <= DBL_MAX)) {
          set_error("problem %d: x contains NaN or infinity; the GPU path requires finite input", B.order[q]);
          r = SC_ERR_INVALID;
        }
      }
      if (r != SC_OK) break;
    }
    // results back to the callers' buffers
    std::vector<double> cent((size_t)B.kd);
    std::vector<int64_t> sizes((size_t)B.ksum);
    std::vector<BState> st((size_t)B.count);
    if (cudaMemcpyAsync(cent.data(), B.cent64, cent.size() * sizeof(double), cudaMemcpyDeviceToHost, B.s) != cudaSuccess ||
        cudaMemcpyAsync(sizes.data(), B.sizes, sizes.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, B.s) != cudaSuccess ||
        cudaMemcpyAsync(st.data(), B.st, st.size() * sizeof(BState), cudaMemcpyDeviceToHost, B.s) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "results");
      break;
    }
    std::unique_lock<std::mutex> stage_lock(g_stage_mutex);
    void *stage = nullptr;
    if ((r = host_stage((size_t)B.rows * sizeof(int32_t), &stage)) != SC_OK) break;
    if (cudaMemcpyAsync(stage, B.labels, (size_t)B.rows * sizeof(int32_t), cudaMemcpyDeviceToHost, B.s) != cudaSuccess ||
        cudaStreamSynchronize(B.s) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "results");
      break;
    }
    const int32_t *lab = (const int32_t *)stage;
    // into the callers' buffers: problems split over host threads by row
    // count (the labels widen to 64 bits on the way)
    auto fill = [&](int q0, int q1) {
      for (int q = q0; q < q1; ++q) {
        sc_kmeans_problem &pr = problems[B.order[q]];
        const BProb &P = B.probs[q];
        if (pr.centroids_out) memcpy(pr.centroids_out, cent.data() + P.c_off, (size_t)P.k * P.d * sizeof(double));
        if (pr.sizes_out) memcpy(pr.sizes_out, sizes.data() + P.k_off, (size_t)P.k * sizeof(int64_t));
        if (pr.labels_out)
          for (int64_t i = 0; i < P.n; ++i) pr.labels_out[i] = lab[P.row0 + i];
        if (pr.distortion_out) *pr.distortion_out = st[q].distortion;
        if (pr.iters_out) *pr.iters_out = st[q].iters;
        pr.rescored = st[q].rescored;
        pr.pp_replays = st[q].pp_replays;
      }
    };
    const int nth = (int)std::min<int64_t>({(int64_t)std::max(1u, std::thread::hardware_concurrency()), 16,
                                            (int64_t)B.count, B.rows / 65536 + 1});
    std::vector<int> cut(nth + 1, B.count);  // thread t: problems [cut[t], cut[t + 1])
    cut[0] = 0;
    for (int q = 0, t = 1; q < B.count && t < nth; ++q)
      if (B.probs[q].row0 + B.probs[q].n >= B.rows * t / nth) cut[t++] = q + 1;
    std::vector<std::thread> pool;
    try {
      for (int t = 1; t < nth; ++t) pool.emplace_back(fill, cut[t], cut[t + 1]);
    } catch (...) {  // no threads: the rest on this one
      fill(cut[pool.size() + 1], B.count);
    }
    fill(cut[0], cut[1]);
    for (auto &th : pool) th.join();
    trace.mark("results", nullptr);
  } while (0);
  free_batch(B);
  trace.mark("free", nullptr);
  return r;
}

static std::string device_tag() {
  int dev = 0, sms = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "";
  sms = prop.multiProcessorCount;
  std::string name(prop.name);
  for (char &c : name)
    if (c == ' ') c = '_';
  char buf[320];
  snprintf(buf, sizeof buf, "device %s sm_%d%d sms %d", name.c_str(), prop.major, prop.minor, sms);
  return buf;
}

static const char *kTuneHeader = "smartcore_gb300 batched-assignment tuning v2";  // v2: timed over repeated items

sc_status sc_batch_tune(const char *path) {
  const std::string tag = device_tag();
  if (tag.empty()) return cuda_fail(cudaGetLastError(), "device properties");
  // One synthetic problem per (D, cluster class): 32,768 rows uniform in
  // [-8, 8)^D, its own k-means++ start.
  constexpr int kTuneRows = 32768;
  std::vector<int64_t> n, d, k, mi;
  std::vector<int> who;
  for (int dc = 0; dc < kNumD; ++dc)
    for (int kc = 0; kc < kNumKC; ++kc) {
      n.push_back(kTuneRows); d.push_back(kClassD[dc]); k.push_back(kClassK[kc]); mi.push_back(1);
      who.push_back(dc * kNumKC + kc);
    }
  Batch B;
  B.dtype = SC_F32;
  plan_batch(B, n, d, k, mi, who);
  for (int q = 0; q < B.count; ++q) {
    B.first.push_back((int64_t)q * 977 % kTuneRows);
    for (int a = 0; a + 1 < B.probs[q].k; ++a) B.uniforms.push_back((double)((a * 7919 + q * 104729) % 1000) / 1000.0);
  }
  // Each timed launch runs the problem's items kTuneRepeat times over, so that
  // every persistent CTA has work, as in a full batch (the sums of the
  // repeats only grow the 128-bit totals; the labels are rewritten alike).
  constexpr int kTuneRepeat = 16;
  size_t item_cap = ((size_t)kTuneRows / kRowsOpts[0] + 1) * kTuneRepeat;
  if (cudaStreamCreateWithFlags(&B.s, cudaStreamNonBlocking) != cudaSuccess) return cuda_fail(cudaGetLastError(), "cudaStreamCreate");
  Tune T;
  sc_status r = SC_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BItem *d_items = nullptr;
  do {
    if ((r = alloc_batch(B)) != SC_OK) break;
    if ((r = dev_alloc((void **)&d_items, item_cap * sizeof(BItem), B.s)) != SC_OK) break;
    if ((r = assign_grid(B, SC_F32)) != SC_OK) break;
    if ((r = upload_tables(B)) != SC_OK) break;
    tune_fill_kernel<<<1024, 256, 0, B.s>>>((float *)B.X, B.xelems, 12345u);
    SC_LAUNCHED();
    if ((r = run_setup<float>(B)) != SC_OK) break;
    for (int i = 0; i < 3; ++i)  // the classes' set-up chains, before any timing
      if (B.side[i] && cudaStreamSynchronize(B.side[i]) != cudaSuccess) r = cuda_fail(cudaGetLastError(), "tuning set-up");
    if (r != SC_OK) break;
    const int act = B.count;
    if (cudaMemcpyAsync(B.active, &act, sizeof act, cudaMemcpyHostToDevice, B.s) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
        cudaStreamSynchronize(B.s) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "tuning set-up");
      break;
    }
    for (int q = 0; q < B.count && r == SC_OK; ++q) {
      const int cls = B.order[q], dc = cls / kNumKC, kc = cls % kNumKC;
      float best_us = 1e30f;
      for (int ci = 0; ci < kNumCU && r == SC_OK; ++ci)
        for (int ri = 0; ri < kNumRows && r == SC_OK; ++ri) {
          std::vector<BItem> items;
          for (int rp = 0; rp < kTuneRepeat; ++rp) add_items(items, q, B.probs[q].n, kRowsOpts[ri], kCUs[ci]);
          std::vector<BProb> probs = B.probs;
          const int sc = 62 - 3 - ceil_log2i(kRowsOpts[ri] + 1);  // |x| < 2^3 here
          probs[q].scale = sc;
          if (cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(BItem), cudaMemcpyHostToDevice, B.s) != cudaSuccess ||
              cudaMemcpyAsync(B.d_probs + q, &probs[q], sizeof(BProb), cudaMemcpyHostToDevice, B.s) != cudaSuccess) {
            r = cuda_fail(cudaGetLastError(), "tuning tables");
            break;
          }
          float ms_best = 1e30f;
          for (int rep = 0; rep < 4 && r == SC_OK; ++rep) {
            if (cudaMemsetAsync(B.heads, 0, sizeof(unsigned), B.s) != cudaSuccess ||
                cudaEventRecord(e0, B.s) != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "tuning"); break; }
            if ((r = launch_assign_class<float>(B, dc, B.heads, (int)items.size(), d_items, 0)) != SC_OK) break;
            float ms = 0.f;
            if (cudaEventRecord(e1, B.s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "tuning"); break; }
            if (rep > 0) ms_best = std::min(ms_best, ms);  // the first launch warms up
          }
          if (r == SC_OK && 1e3f * ms_best < best_us) {
            best_us = 1e3f * ms_best;
            T.cu[dc][kc] = kCUs[ci];
            T.rows[dc][kc] = kRowsOpts[ri];
            T.us[dc][kc] = best_us;
          }
        }
    }
  } while (0);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (d_items) dev_free(d_items, B.s);
  free_batch(B);
  if (r != SC_OK) return r;
  T.ready = true;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune = T;
  }
  if (path) {
    FILE *f = fopen(path, "w");
    if (!f) { set_error("cannot write the tuning table to %s", path); return SC_ERR_INVALID; }
    fprintf(f, "%s\n%s\n", kTuneHeader, tag.c_str());
    for (int dc = 0; dc < kNumD; ++dc)
      for (int kc = 0; kc < kNumKC; ++kc)
        fprintf(f, "%d %d %d %d %.2f\n", kClassD[dc], kClassK[kc], T.cu[dc][kc], T.rows[dc][kc], T.us[dc][kc]);
    fclose(f);
  }
  return SC_OK;
}

sc_status sc_batch_tune_load(const char *path) {
  if (!path) { set_error("null path"); return SC_ERR_INVALID; }
  FILE *f = fopen(path, "r");
  if (!f) { set_error("cannot read the tuning table %s", path); return SC_ERR_INVALID; }
  char line[400];
  std::string head, tag;
  if (fgets(line, sizeof line, f)) head = line;
  if (fgets(line, sizeof line, f)) tag = line;
  while (!head.empty() && (head.back() == '\n' || head.back() == '\r')) head.pop_back();
  while (!tag.empty() && (tag.back() == '\n' || tag.back() == '\r')) tag.pop_back();
  Tune T;
  int seen = 0;
  int D, K, cu, rows;
  float us;
  while (fgets(line, sizeof line, f)) {
    if (sscanf(line, "%d %d %d %d %f", &D, &K, &cu, &rows, &us) != 5) continue;
    int dc = -1, kc = -1;
    for (int i = 0; i < kNumD; ++i) if (kClassD[i] == D) dc = i;
    for (int i = 0; i < kNumKC; ++i) if (kClassK[i] == K) kc = i;
    bool cu_ok = false, rows_ok = false;
    for (int i = 0; i < kNumCU; ++i) cu_ok |= kCUs[i] == cu;
    for (int i = 0; i < kNumRows; ++i) rows_ok |= kRowsOpts[i] == rows;
    if (dc < 0 || kc < 0 || !cu_ok || !rows_ok) continue;
    T.cu[dc][kc] = cu;
    T.rows[dc][kc] = rows;
    T.us[dc][kc] = us;
    ++seen;
  }
  fclose(f);
  if (head != kTuneHeader) { set_error("%s is not a tuning table of this library", path); return SC_ERR_INVALID; }
  const std::string want = device_tag();
  if (tag != want) { set_error("tuning table %s was made on another device (%s)", path, tag.c_str()); return SC_ERR_INVALID; }
  if (seen != kNumD * kNumKC) { set_error("tuning table %s is incomplete", path); return SC_ERR_INVALID; }
  T.ready = true;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tune = T;
  return SC_OK;
}

sc_status sc_debug_batch_variant(int32_t variant) {
  bool ok = variant < 0;
  for (int i = 0; i < kNumCU; ++i) ok |= kCUs[i] == variant;
  if (!ok) { set_error("unknown batched assignment variant %d", variant); return SC_ERR_INVALID; }
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_variant_override = variant < 0 ? -1 : variant;
  return SC_OK;
}

sc_status sc_batch_tune_get(int32_t d, int32_t k, int32_t *cu_out, int32_t *rows_out) {
  if (d < 1 || d > kMaxBD || k < 1 || k > kMaxBK) { set_error("(d, k) = (%d, %d) is outside the batched kernels", d, k); return SC_ERR_INVALID; }
  int cu, rows;
  tune_choice(pad_width(d), k, &cu, &rows);
  if (cu_out) *cu_out = cu;
  if (rows_out) *rows_out = rows;
  return SC_OK;
}

}  // extern "C"
