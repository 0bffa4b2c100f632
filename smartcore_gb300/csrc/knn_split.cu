// Split-BF16 form of LinearKNNSearch::find (src/algorithm/neighbour/
// linear_search.rs:52-84).
//
// The queries are the A operand of a tcgen05 GEMM (128 per tile, one query
// per epilogue thread) and the training rows stream through the B operand in
// index order, 256 per tile.  From x.t_j (split-BF16, FP32 accumulate) each
// thread forms a_j = ||t_j||^2 - 2 q.t_j, which with ||q||^2 approximates the
// reference's squared distance D_j to within a certified bound E_q.  The
// thread keeps the reference's k-slot heap and replays it exactly: row j can
// only enter when D_j < root^2, so every row with a_j > root^2 - ||q||^2 + E_q
// is skipped, and every other row gets the reference distance
// sqrt(sum_t (double)((q_t - x_t)^2)) in FP64 and the reference's insertion
// test and heapify (src/algorithm/sort/heap_select.rs:42-50, :71-86).  The
// result is the reference's heap array, bit for bit.
#include <float.h>
#include <math.h>
#include <string.h>

#include "exactsum.cuh"
#include "split.cuh"
#include "splitprep.cuh"
#include "tc.cuh"

namespace sc {

namespace {

constexpr int kQM = 128;         // queries per tile (UMMA M)
constexpr int kOwnerWarps = 4;   // one query per thread: heap, exact replay
constexpr int kFilterWarps = 8;  // 2 accumulator buffers x 4 TMEM lane quarters
constexpr int kKnnThreads = 32 * (2 + kOwnerWarps + kFilterWarps);  // + warp 0 TMA, warp 1 MMA
constexpr int kMaskSlots = 4;    // candidate-mask tiles between the filters and the owners
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr int kQueue = 64;       // per owner warp: ring of pending candidates (owner lane << 27 | row);
                                 // a round runs once 32 are pending, and a column adds at most 32
constexpr int kRowBits = 27;     // training rows per handle < 2^27
constexpr int kStageFloats = 1056;  // per owner warp (f32 data): training rows, then query rows (528 floats each)

// One term of Euclidian::squared_distance (src/metrics/distance/
// euclidian.rs:56-62): r = a - b and r * r in the element type, then to_f64.
__device__ __forceinline__ double ref_term(float a, float b) {
  const float r = __fsub_rn(a, b);
  return (double)__fmul_rn(r, r);
}
__device__ __forceinline__ double ref_term(double a, double b) {
  const double r = __dsub_rn(a, b);
  return __dmul_rn(r, r);
}

// Rows of a matrix as split-BF16 operand: halves (row i of either at
// [i * stride]: separate arrays, or both halves in one row when interleaved),
// f32 upper bound of the norm, ||row||^2 rounded to f32 (+inf for padding
// rows) and in f64.
template <typename T>
__global__ void __launch_bounds__(256)
knn_prep_kernel(const T *__restrict__ x, int64_t n, int64_t n_pad, int d, int d_pad, int stride,
                __nv_bfloat16 *__restrict__ xh, __nv_bfloat16 *__restrict__ xl, float *__restrict__ nrm,
                float *__restrict__ n2f, double *__restrict__ n2d, unsigned int *__restrict__ nmax,
                __nv_bfloat16 *__restrict__ bx) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * 8 + w;
  if (i >= n_pad) return;
  double s = 0.0;
  for (int j = lane; j < d_pad; j += 32) {
    __nv_bfloat16 h = __float2bfloat16_rn(0.f), l = h;
    if (i < n && j < d) {
      const T v = x[i * d + j];
      split2<T>(v, h, l);
      s = fma((double)v, (double)v, s);
    }
    xh[i * stride + j] = h;
    xl[i * stride + j] = l;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) {
    const float r = __fsqrt_ru(__double2float_ru(s));
    const float up = __uint_as_float(__float_as_uint(r) + 1u);
    if (nrm) nrm[i] = up;
    if (n2f) n2f[i] = i < n ? __double2float_rn(s) : __int_as_float(0x7f800000);
    if (n2d) n2d[i] = s;
    if (nmax && i < n) atomicMax(nmax, __float_as_uint(up));
    if (bx) {  // norm-folding row: BF16 terms of -||row||^2/2 (padding rows never pass)
      const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
      __nv_bfloat16 h = __float2bfloat16_rn(-1e30f), mm = zero, l = zero;
      if (i < n) split3(-0.5 * s, h, mm, l);
      __nv_bfloat16 *row = bx + i * 16;
      row[0] = h;
      row[1] = mm;
      row[2] = l;
      for (int c = 3; c < 16; ++c) row[c] = zero;
    }
  }
}

struct KnnParams {
  int64_t n, m;
  int b_box;  // training rows per TMA box
  int il;     // interleaved halves (KnnPipe::il)
  int n_tiles_t, n_tiles_q;
  int nkt, kt_elems, row_bytes;
  int stages;
  int k, d, lg_d;
  const float *qnrm;
  const double *qn2;
  const unsigned int *tmax;
  float coef_xc, coef_cc, coef_ref;
  int64_t *idx_out;
  double *dist_out;
  unsigned long long *evals;
  int *err;
  // find_radius (linear_search.rs:89-108): rows with sqrt(D) <= radius, in
  // index order; counts per query (counting pass, idx_out == nullptr), the
  // rows from offsets[q] on (filling pass), or both at once (slot pass:
  // counts, and the first cap_q rows of query q from slot q * cap_q on)
  int radius_mode;
  double radius, r2up;  // r2up >= every D whose sqrt rounds to <= radius
  int64_t *counts;
  const int64_t *offsets;
  int64_t cap_q;
};

// The reference keys its heap on d = sqrt(D) (f64).  The heap here holds D
// itself: correctly rounded sqrt is monotone, so sqrt(a) < sqrt(b) exactly
// when a < b, except that values a few ulps apart may round to the same
// sqrt.  Keys are >= 0 or +inf, so their bit patterns order as their values
// (integer compares); only keys within 8 ulps take the two square roots.
__device__ __forceinline__ bool sqrt_less(double a, double b) {
  const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  if (ia >= ib) return false;
  if (ib - ia > 8) return true;
  return __dsqrt_rn(a) < __dsqrt_rn(b);
}

// sift_down of heap_select.rs:71-86 on the distances: node kk has children 2kk
// and 2kk+1.  Heap entry e of a query lives at [e * S]: S = 1 for a
// per-thread array, S = 128 for the shared-memory heaps of a query tile.
template <int S>
__device__ __forceinline__ void heap_sift(double *hD, int32_t *hi, int kk, int nn) {
  while (2 * kk <= nn) {
    int j = 2 * kk;
    if (j < nn && sqrt_less(hD[j * S], hD[(j + 1) * S])) ++j;
    const double a = hD[kk * S], b = hD[j * S];
    if (!sqrt_less(a, b)) break;  // a == b || a > b
    if (j == kk) break;
    hD[kk * S] = b;
    hD[j * S] = a;
    const int32_t t = hi[kk * S];
    hi[kk * S] = hi[j * S];
    hi[j * S] = t;
    kk = j;
  }
}

// Pulls training row j into L2 when it is queued, tiles before its exact
// distance is computed (L1 is almost all shared memory in this kernel).
template <typename T>
__device__ __forceinline__ void prefetch_row(const T *train, int64_t j, int d) {
  const char *a = (const char *)(train + j * (int64_t)d);
  const char *b = a + (size_t)d * sizeof(T) - 1;
  asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
  if (((uintptr_t)a >> 7) != ((uintptr_t)b >> 7)) asm volatile("prefetch.global.L2 [%0];" ::"l"(b));
}

__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool in) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(in ? 4 : 0)
               : "memory");
}

// Exact reference squared distances of up to 32 queued f32 entries (lane r:
// entry r).  Groups of entries are staged by asynchronous copies, coalesced
// (lane l copies features l, l + 32, ...), into the warp's slice of shared
// memory (Sx: training rows, Sq: query rows; zeros past d), so that all of a
// group's loads are in flight at once without holding registers.
//  - d <= 32 (KC = 1): 16 entries a group at a row stride of 33 floats; lane r
//    then sums its own entry from shared memory (conflict-free): branch-free
//    where no running sum can round, else the sequential form, FP64 only
//    where the exponent span is too wide for that.
//  - wider rows (KC = 2 or 8 features a lane): 16 / KC entries a group, each
//    summed across the warp by warp_sqd_terms (a lane reads back only what it
//    copied itself); fb is set where a running sum may round and the caller
//    runs the sequential form.
// Lane r gets entry r's distance in sq.
template <int KC>
__device__ __forceinline__ void round_dist_f32(const float *__restrict__ train, const float *__restrict__ queries,
                                               uint32_t e, uint32_t cnt, int64_t qbase, int64_t m, int d, int lg_d,
                                               int lane, float *Sx, float *Sq, double &sq, bool &fb) {
  constexpr int G = 16 / KC, W = KC == 1 ? 33 : 32 * KC;
  const bool live = (uint32_t)lane < cnt && qbase + (int)(e >> kRowBits) < m;
  unsigned long long S = 0ull;
  uint32_t emin = 256u;
  bool ok = true;
  for (uint32_t b0 = 0; b0 < cnt; b0 += G) {
#pragma unroll
    for (int r = 0; r < G; ++r) {
      const uint32_t er = __shfl_sync(0xffffffffu, e, (int)((b0 + r) & 31u));
      const int64_t qr = qbase + (int)(er >> kRowBits);
      const bool in_r = b0 + r < cnt && qr < m;
      const float *tr = train + (int64_t)(er & ((1u << kRowBits) - 1u)) * d;
      const float *qrow = queries + qr * d;
#pragma unroll
      for (int c = 0; c < KC; ++c) {
        const int f = 32 * c + lane;
        const bool in = in_r && f < d;
        cp_async4(Sx + r * W + f, in ? tr + f : train, in);
        cp_async4(Sq + r * W + f, in ? qrow + f : queries, in);
      }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    if constexpr (KC == 1) {
      __syncwarp();  // every lane's copies have landed
      const int r = lane - (int)b0;
      if (live && r >= 0 && r < G) {
        if (!sqd_f32_d32(Sq + r * W, Sx + r * W, d, lg_d, sq)) {
          sq = 0.0;
          for (int t = 0; t < d; ++t) sq = __dadd_rn(sq, ref_term(Sq[r * W + t], Sx[r * W + t]));
        }
      }
      __syncwarp();  // before the next group's copies
    } else {
      constexpr int NB = KC == 2 ? 2 : 1;
#pragma unroll
      for (int r0 = 0; r0 < G; r0 += NB) {
        if (b0 + r0 >= cnt) break;
        float t[NB][KC];
#pragma unroll
        for (int r = 0; r < NB; ++r)
#pragma unroll
          for (int c = 0; c < KC; ++c) {
            const int o = (r0 + r) * W + 32 * c + lane;
            const float df = __fsub_rn(Sq[o], Sx[o]);
            t[r][c] = __fmul_rn(df, df);
          }
        warp_sqd_terms<KC, NB>(t, lg_d, lane, (int)(b0 + r0), S, emin, ok);
      }
    }
  }
  if constexpr (KC != 1) {
    if (live) {
      fb = !ok;
      if (ok) sq = sqd_from_units(S, emin);
    }
  }
}

// Threshold on a_j below which a row may enter the heap: D_root - ||q||^2 + E,
// rounded up (a larger threshold only admits more rows to the exact test),
// in f32 with a margin of 2^-22 (D_root + ||q||^2) for the f32 roundings.
// qf is ||q||^2 rounded down to f32 (once per query).
__device__ __forceinline__ float knn_threshold(double droot, float qf, float eq) {
  const long long b = __double_as_longlong(droot);  // droot >= 0 or +inf: integer tests, no FP64 pipe
  if (b >= 0x7ff0000000000000ll) return __int_as_float(0x7f800000);
  // an f32 upper bound of droot: its top 23 fraction bits plus one ulp
  const int e = (int)(b >> 52) - 1023;
  const float r = e > 127 ? __int_as_float(0x7f800000)
                  : e < -126 ? 0x1p-126f
                             : __uint_as_float((((uint32_t)(e + 127) << 23) | (uint32_t)((b >> 29) & 0x7fffff)) + 1u);
  return __fadd_ru(__fadd_ru(__fsub_ru(r, qf), eq), __fmul_ru(0x1p-22f, __fadd_ru(r, qf)));
}

// The shared-memory pipeline of the split kNN kernels: the query tile (A,
// resident per query tile), training tiles (B, `stages` deep) and the two
// TMEM accumulators, with their barriers.
struct KnnPipe {
  uint8_t *sA, *sOnes, *sB;
  uint64_t *full, *empty, *afull, *aempty, *accfull, *accempty, *mma_done;
  int *s_abort;
  int a_blk, a_bytes, b_blk, b_stage;  // a_bytes: one 128-query half
  int n_tiles_q, n_tiles_t, nkt, kt_elems, row_bytes, stages;
  int qh;     // 128-query halves per query tile, each with its accumulator pair
  int b_box;  // training rows per TMA box (a tile of TN rows takes TN / b_box boxes)
  int qt0;    // first query tile (a chunk of the queries starts there)
  int il;     // interleaved halves: one row_bytes row holds the high then the low half (d_pad = 32:
              // 128-byte rows, 128-byte swizzle); else the halves are separate nkt-block operands
};

// TMA producer (one thread): per query tile its split halves once (and the
// ones tile on the first), then the training tiles in index order.  A query
// tile is qh x 128 queries; each training tile serves all of them.
template <int TN>
__device__ void knn_tma_role(const KnnPipe &P, const CUtensorMap *tm_qh, const CUtensorMap *tm_ql,
                             const CUtensorMap *tm_th, const CUtensorMap *tm_tl, const CUtensorMap *tm_ones,
                             const CUtensorMap *tm_tbx) {
  int it = 0, ql = 0;
  bool ok = true;
  for (int qt = blockIdx.x; ok && qt < P.n_tiles_q; qt += gridDim.x, ++ql) {
    if (!tc::mbar_wait(P.aempty, (uint32_t)(ql & 1) ^ 1u, kWaitNs)) { ok = false; break; }
    tc::mbar_expect_tx(P.afull, (uint32_t)(P.qh * P.a_bytes + (ql == 0 ? kQM * 32 : 0)));
    for (int h = 0; h < P.qh; ++h)
      for (int part = 0; part < (P.il ? 1 : 2); ++part)
        for (int kt = 0; kt < P.nkt; ++kt)
          tc::tma_load_2d(P.sA + h * P.a_bytes + (part * P.nkt + kt) * P.a_blk, part ? tm_ql : tm_qh, P.afull,
                          kt * P.kt_elems, ((P.qt0 + qt) * P.qh + h) * kQM);
    if (ql == 0) tc::tma_load_2d(P.sOnes, tm_ones, P.afull, 0, 0);
    for (int tt = 0; tt < P.n_tiles_t; ++tt, ++it) {
      const int s = it % P.stages;
      const uint32_t ph = (uint32_t)(it / P.stages) & 1u;
      if (!tc::mbar_wait(&P.empty[s], ph ^ 1u, kWaitNs) || *(volatile int *)P.s_abort) { ok = false; break; }
      tc::mbar_expect_tx(&P.full[s], (uint32_t)P.b_stage);
      uint8_t *dst = P.sB + (size_t)s * P.b_stage;
      const int parts = P.il ? 1 : 2;
      for (int r = 0; r < TN; r += P.b_box) {  // boxes stack rows in the K-major operand layout
        for (int part = 0; part < parts; ++part)
          for (int kt = 0; kt < P.nkt; ++kt)
            tc::tma_load_2d(dst + (part * P.nkt + kt) * P.b_blk + r * P.row_bytes, part ? tm_tl : tm_th, &P.full[s],
                            kt * P.kt_elems, tt * TN + r);
        tc::tma_load_2d(dst + parts * P.nkt * P.b_blk + r * 32, tm_tbx, &P.full[s], 0, tt * TN + r);
      }
    }
  }
  if (!ok) atomicExch(P.s_abort, 1);
  for (int j = (it > P.stages ? it - P.stages : 0); j < it; ++j)  // drain in-flight copies
    tc::mbar_wait(&P.full[j % P.stages], (uint32_t)(j / P.stages) & 1u, kWaitNs);
  if (ql > 0) tc::mbar_wait(P.afull, (uint32_t)((ql - 1) & 1), kWaitNs);
}

// MMA issuer (one thread): per training tile and query half h, into
// accumulator (h, it & 1) at TMEM column (2 h + (it & 1)) TN: -||t||^2 / 2
// (ones x norm-folding rows), then q_h.t_h + q_h.t_l + q_l.t_h.
template <int TN>
__device__ void knn_mma_role(const KnnPipe &P, uint32_t tmem) {
  const uint32_t idesc = tc::idesc_bf16_f32(kQM, TN);
  const uint32_t sA0 = tc::smem_u32(P.sA), sB0 = tc::smem_u32(P.sB);
  const uint64_t ones_desc = tc::smem_desc(tc::smem_u32(P.sOnes), 32);
  int it = 0, ql = 0;
  bool ok = true;
  for (int qt = blockIdx.x; ok && qt < P.n_tiles_q; qt += gridDim.x, ++ql) {
    if (!tc::mbar_wait(P.afull, (uint32_t)(ql & 1), kWaitNs)) { ok = false; break; }
    for (int tt = 0; tt < P.n_tiles_t; ++tt, ++it) {
      const int s = it % P.stages, acc = it & 1;
      const uint32_t ph = (uint32_t)(it / P.stages) & 1u, aph = (uint32_t)(it >> 1) & 1u;
      if (!tc::mbar_wait(&P.accempty[acc], aph ^ 1u, kWaitNs) || !tc::mbar_wait(&P.full[s], ph, kWaitNs) ||
          *(volatile int *)P.s_abort) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint32_t b0 = sB0 + (uint32_t)(s * P.b_stage);
      const int parts = P.il ? 1 : 2;
      for (int h = 0; h < P.qh; ++h) {
        const uint32_t d_tmem = tmem + (uint32_t)((2 * h + acc) * TN);
        const uint32_t a0 = sA0 + (uint32_t)(h * P.a_bytes);
        tc::mma_f16(d_tmem, ones_desc, tc::smem_desc(b0 + (uint32_t)(parts * P.nkt * P.b_blk), 32), idesc, 0u);
        for (int prod = 0; prod < 3; ++prod) {
          const int pa = prod == 2 ? 1 : 0, pb = prod == 1 ? 1 : 0;
          // a half's K slices: its own nkt-block operand, or (interleaved) its
          // 64-byte half of each 128-byte row
          const int pa_off = P.il ? pa * P.kt_elems * 2 : pa * P.nkt * P.a_blk;
          const int pb_off = P.il ? pb * P.kt_elems * 2 : pb * P.nkt * P.b_blk;
          for (int kt = 0; kt < P.nkt; ++kt)
            for (int ks = 0; ks < P.kt_elems / 16; ++ks) {
              const uint64_t ad = tc::smem_desc(a0 + (uint32_t)(pa_off + kt * P.a_blk + ks * 32), P.row_bytes);
              const uint64_t bd = tc::smem_desc(b0 + (uint32_t)(pb_off + kt * P.b_blk + ks * 32), P.row_bytes);
              tc::mma_f16(d_tmem, ad, bd, idesc, 1u);
            }
        }
      }
      tc::mma_commit(&P.empty[s]);
      tc::mma_commit(&P.accfull[acc]);
    }
    tc::mma_commit(P.aempty);  // the query tile's smem is free once these MMAs complete
  }
  if (!ok) atomicExch(P.s_abort, 1);
  tc::mma_commit(P.mma_done);
  tc::mbar_wait(P.mma_done, 0, kWaitNs);
}

// Roles: warp 0 TMA (query tile once, training tiles in index order), warp 1
// MMA (one elected thread), warps 2-5 owners (one query per thread: the
// reference heap, replayed exactly in index order), warps 6-13 filters.  A
// filter warp reads its accumulator buffer's TMEM lanes (32 queries, every
// column of the tile) and writes, per query, the bit mask of the rows a
// certified bound cannot exclude; the owners consume the masks of each tile
// in order.  A filter may
// use a threshold up to two tiles stale: the heap root only decreases, so a
// staler threshold admits more rows, never fewer.
template <typename T, int TN, bool SH>
__global__ void __launch_bounds__(kKnnThreads, 1)
knn_split_kernel(const __grid_constant__ CUtensorMap tm_qh, const __grid_constant__ CUtensorMap tm_ql,
                 const __grid_constant__ CUtensorMap tm_th, const __grid_constant__ CUtensorMap tm_tl,
                 const __grid_constant__ CUtensorMap tm_ones, const __grid_constant__ CUtensorMap tm_tbx,
                 const T *__restrict__ train, const T *__restrict__ queries, const KnnParams p) {
  constexpr int kWords = TN / 32;  // mask words per query and tile
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int a_blk = kQM * p.row_bytes;
  const int a_bytes = (p.il ? 1 : 2) * p.nkt * a_blk;
  const int b_blk = TN * p.row_bytes;
  const int b_stage = (p.il ? 1 : 2) * p.nkt * b_blk + TN * 32;  // halves + norm-folding rows
  uint8_t *sA = base;
  uint8_t *sOnes = base + a_bytes;                   // 128 x 32 B
  uint8_t *sB = sOnes + kQM * 32;
  uint32_t *sQ = (uint32_t *)(sB + (size_t)p.stages * b_stage);  // owner warps x kQueue entries
  uint32_t *sMask = sQ + kOwnerWarps * kQueue;                   // [slot][word][query]
  float *s_stage = (float *)(sMask + kMaskSlots * kQM * kWords);  // f32: owner warps x kStageFloats
  float *s_lo = s_stage + (sizeof(T) == 4 ? kOwnerWarps * kStageFloats : 0);  // per query: filter threshold on acc
  double *s_rs = (double *)(s_lo + kQM);                          // owner warps x 32: round distances
  int32_t *s_rj = (int32_t *)(s_rs + kOwnerWarps * 32);            //   rows
  uint32_t *s_rg = (uint32_t *)(s_rj + kOwnerWarps * 32);          //   entries per owner lane
  double *s_hD = (double *)(s_rg + kOwnerWarps * 32);  // SH: heaps of the tile's queries, [k][128]
  int32_t *s_hi = (int32_t *)(s_hD + (SH ? p.k * kQM : 0));
  uint64_t *bars = (uint64_t *)(s_hi + (SH ? ((p.k * kQM + 1) & ~1) : 0));
  uint64_t *full = bars, *empty = bars + p.stages, *afull = bars + 2 * p.stages;
  uint64_t *aempty = afull + 1, *accfull = afull + 2, *accempty = afull + 4, *mma_done = afull + 6;
  uint64_t *maskfull = afull + 7, *maskempty = maskfull + kMaskSlots;
  uint32_t *s_tmem = (uint32_t *)(maskempty + kMaskSlots);
  int *s_abort = (int *)(s_tmem + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < p.stages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(afull, 1);
    tc::mbar_init(aempty, 1);
    tc::mbar_init(mma_done, 1);
    for (int a = 0; a < 2; ++a) {
      tc::mbar_init(&accfull[a], 1);
      tc::mbar_init(&accempty[a], 32 * kFilterWarps / 2);
    }
    for (int s = 0; s < kMaskSlots; ++s) {
      tc::mbar_init(&maskfull[s], 32 * kFilterWarps / 2);
      tc::mbar_init(&maskempty[s], 32 * kOwnerWarps);
    }
    *s_abort = 0;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tm_qh);
    tc::prefetch_tmap(&tm_ql);
    tc::prefetch_tmap(&tm_th);
    tc::prefetch_tmap(&tm_tl);
    tc::prefetch_tmap(&tm_ones);
    tc::prefetch_tmap(&tm_tbx);
  }
  if (warp == 1) {
    tc::tmem_alloc(s_tmem, 2 * TN);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *s_tmem;

  const KnnPipe P{sA, sOnes, sB, full, empty, afull, aempty, accfull, accempty, mma_done, s_abort,
                  a_blk, a_bytes, b_blk, b_stage, p.n_tiles_q, p.n_tiles_t, p.nkt, p.kt_elems, p.row_bytes,
                  p.stages, 1, p.b_box, 0, p.il};
  if (warp == 0) {
    if (lane == 0) knn_tma_role<TN>(P, &tm_qh, &tm_ql, &tm_th, &tm_tl, &tm_ones, &tm_tbx);
  } else if (warp == 1) {
    if (lane == 0) knn_mma_role<TN>(P, tmem);
  } else if (warp < 2 + kOwnerWarps) {
    // ---------------- owners: one query per thread ----------------
    // The candidates of a tile arrive as bit masks in index order; they are
    // appended, per query in index order, to the warp's queue; whenever 32
    // are pending the warp computes their exact reference distances
    // lane-parallel and each owner replays its heap steps in order.
    const int lq = warp & 3;
    const int row = lq * 32 + lane;
    const float tmax = __uint_as_float(*p.tmax);
    uint32_t *Q = sQ + (warp - 2) * kQueue;
    double *Rs = s_rs + (warp - 2) * 32;
    int32_t *Rj = s_rj + (warp - 2) * 32;
    uint32_t *Rg = s_rg + (warp - 2) * 32;
    constexpr int HS = SH ? kQM : 1;  // heap entry stride
    double hD_l[SH ? 1 : kMaxKnnK];   // heap keys: the squared distances D
    int32_t hi_l[SH ? 1 : kMaxKnnK];
    double *hD = SH ? s_hD + row : hD_l;
    int32_t *hi = SH ? s_hi + row : hi_l;
    unsigned long long evals = 0;
    int it = 0;
    bool stop = false;
    for (int qt = blockIdx.x; !stop && qt < p.n_tiles_q; qt += gridDim.x) {
      const int64_t q = (int64_t)qt * kQM + row;
      const bool live = q < p.m;
      for (int s = 0; s < p.k; ++s) {
        hD[s * HS] = __longlong_as_double(0x7ff0000000000000ll);
        hi[s * HS] = -1;
      }
      const float qn = live ? p.qnrm[q] : 0.f;
      const float qn2f = live ? __double2float_rd(p.qn2[q]) : 0.f;
      // |a_j - (D_j - ||q||^2)| <= e, a_j = -2 acc_j (see split.cu for the terms)
      const float eq = 1.05f * (2.f * (p.coef_xc * qn * tmax + p.coef_cc * tmax * tmax) +
                                p.coef_ref * (qn + tmax) * (qn + tmax)) + 1e-30f;
      // row j can enter only if acc_j >= lo = -thr / 2 (thr = root^2 - ||q||^2 + e)
      float lo = live ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000);
      s_lo[row] = lo;
      int64_t rc = 0, rpos = 0;  // find_radius: rows found, next output position
      if (p.radius_mode && p.idx_out && live) rpos = p.offsets ? p.offsets[q] : q * p.cap_q;
      uint32_t qhead = 0, qtail = 0;  // warp-uniform queue cursors
      const int64_t qbase = (int64_t)qt * kQM + lq * 32;
      // one round: exact distances of up to 32 queued entries, then the owners' heap steps
      auto round = [&](uint32_t cnt) {
        const uint32_t e = (uint32_t)lane < cnt ? Q[(qhead + lane) & (kQueue - 1)] : 0u;
        const int owner = (int)(e >> kRowBits);
        const int64_t j = (int64_t)(e & ((1u << kRowBits) - 1u));
        double sq = __longlong_as_double(0x7ff0000000000000ll);
        bool seq = (uint32_t)lane < cnt && qbase + owner < p.m;  // this lane's entry needs the sequential form
        if constexpr (sizeof(T) == 4) {
          constexpr int KC = TN == 256 ? 1 : TN == 128 ? 2 : 8;  // d_pad <= 32, 64, 256
          bool fb = false;
          float *Sx = s_stage + (warp - 2) * kStageFloats;
          round_dist_f32<KC>((const float *)train, (const float *)queries, e, cnt, qbase, p.m, p.d, p.lg_d, lane, Sx,
                             Sx + kStageFloats / 2, sq, fb);
          seq = seq && fb;
        }
        if (seq) {
          const T *tr = train + j * (int64_t)p.d;
          const T *qrow = queries + (qbase + owner) * (int64_t)p.d;
          bool done = false;
          if constexpr (sizeof(T) == 4) {
            if (p.d <= 32) {
              done = sqd_seq_f32_d32((const float *)qrow, (const float *)tr, p.d, p.lg_d, sq);
            } else {
              done = sqd_seq_f32(qrow, tr, p.d, p.lg_d, sq);
            }
          }
          if (!done) {
            sq = 0.0;
            for (int t = 0; t < p.d; ++t) sq = __dadd_rn(sq, ref_term(qrow[t], tr[t]));
          }
        }
        // every owner replays its own entries of the round (ascending = index
        // order), all owners at once: entry r's owner learns the set of
        // entries it owns from the group of equal owners
        Rs[lane] = sq;
        Rj[lane] = (int32_t)j;
        Rg[lane] = 0u;
        const int own = (uint32_t)lane < cnt ? owner : 32;
        const uint32_t grp = __match_any_sync(0xffffffffu, own);
        __syncwarp();
        if (own < 32 && lane == __ffs(grp) - 1) Rg[own] = grp;
        __syncwarp();
        for (uint32_t mine = Rg[lane]; mine; mine &= mine - 1u) {
          const int r = __ffs(mine) - 1;
          const double sr = Rs[r];
          if (p.radius_mode) {  // linear_search.rs:100-104: d <= radius, appended in index order
            const double dist = __dsqrt_rn(sr);
            if (dist <= p.radius) {
              if (p.idx_out && (p.offsets || rc < p.cap_q)) {
                p.idx_out[rpos] = Rj[r];
                p.dist_out[rpos] = dist;
                ++rpos;
              }
              ++rc;
            }
            continue;
          }
          if (sqrt_less(sr, hD[0])) {  // sqrt(D) < root (linear_search.rs:72)
            hD[0] = sr;
            hi[0] = Rj[r];
            if (p.k > 1)
              for (int s2 = p.k / 2 - 1; s2 >= 0; --s2) heap_sift<HS>(hD, hi, s2, p.k - 1);
            lo = -0.5f * knn_threshold(hD[0], qn2f, eq);
          }
        }
        if (!p.radius_mode) s_lo[row] = lo;
        __syncwarp();
        qhead += cnt;
        evals += (uint32_t)lane < cnt ? 1u : 0u;
        __syncwarp();
      };
      for (int tt = 0; tt < p.n_tiles_t; ++tt, ++it) {
        const int slot = it % kMaskSlots;
        const bool got = tc::mbar_wait(&maskfull[slot], (uint32_t)(it / kMaskSlots) & 1u, kWaitNs);
        // (A stopped filter shows up here as a wait that runs out.)
        if (!__all_sync(0xffffffffu, got)) {
          atomicExch(s_abort, 1);
          stop = true;
          break;
        }
        const uint32_t *mcol = sMask + (size_t)slot * kWords * kQM + row;
        const int64_t j0 = (int64_t)tt * TN;
        uint32_t nzw = 0u;  // this query's words with an entry
#pragma unroll
        for (int w = 0; w < kWords; ++w) nzw |= (mcol[w * kQM] != 0u ? 1u : 0u) << w;
        // Once the tile's mask is in registers the slot is free, and the
        // filters may take the current threshold (entries still queued only
        // make it staler).  Tile 0 is released after its replay instead: the
        // thresholds of tiles 1 and 2 come from it.
        const bool early = tt != 0 || p.radius_mode;
        if (early) {
          s_lo[row] = lo;
          tc::mbar_arrive(&maskempty[slot]);
        }
        // Entries in row order, and within a row in owner order: each owner
        // still sees its rows in index order, and a round spreads over many
        // owners, so their heap replays run side by side.
        // (The filters refill this slot only after this owner has taken the
        // mask of tile tt + 2, so its words are read again here.)
        for (uint32_t words = __reduce_or_sync(0xffffffffu, nzw); words; words &= words - 1u) {
          {
            const int w = __ffs(words) - 1;
            const uint32_t mword = mcol[w * kQM];
            uint32_t cols = __reduce_or_sync(0xffffffffu, mword);  // rows of this word with an entry
            while (cols) {
              const int b = __ffs(cols) - 1;
              cols &= cols - 1u;
              const bool mine = (mword >> b) & 1u;
              const uint32_t own = __ballot_sync(0xffffffffu, mine);
              const int64_t jr = j0 + 32 * w + b;
              if (mine)
                Q[(qtail + __popc(own & ((1u << lane) - 1u))) & (kQueue - 1)] =
                    ((uint32_t)lane << kRowBits) | (uint32_t)jr;
              if (lane == __ffs(own) - 1) prefetch_row(train, jr, p.d);
              qtail += __popc(own);
              if (qtail - qhead >= 32) {
                __syncwarp();
                round(32);
              }
            }
          }
        }
        if (!early) {
          s_lo[row] = lo;
          tc::mbar_arrive(&maskempty[slot]);
        }
      }
      while (!stop && qtail != qhead) round(min(32u, qtail - qhead));
      if (p.radius_mode) {
        if (live && !stop && p.counts) p.counts[q] = rc;
      } else if (live && !stop)
        for (int s = 0; s < p.k; ++s) {
          p.idx_out[q * p.k + s] = hi[s * HS];
          p.dist_out[q * p.k + s] = __dsqrt_rn(hD[s * HS]);  // sqrt(+inf) = +inf for an empty slot
        }
    }
    if (evals) atomicAdd(p.evals, evals);
  } else {
    // ---------------- filters: candidate masks from TMEM ----------------
    const int f = warp - 2 - kOwnerWarps;  // 0 .. 7
    const int g = f >> 2, lq = warp & 3;
    const int row = lq * 32 + lane;
    constexpr int kCols = TN;
    constexpr int c_lo = 0;
    int it = 0;
    bool stop = false;
    for (int qt = blockIdx.x; !stop && qt < p.n_tiles_q; qt += gridDim.x) {
      const bool live_q = (int64_t)qt * kQM + row < p.m;
      float rad_lo = __int_as_float(0x7f800000);  // find_radius: a fixed threshold, D <= r2up
      if (p.radius_mode && live_q) {
        const int64_t q = (int64_t)qt * kQM + row;
        const float tmax = __uint_as_float(*p.tmax);
        const float qn = p.qnrm[q];
        const float eq = 1.05f * (2.f * (p.coef_xc * qn * tmax + p.coef_cc * tmax * tmax) +
                                  p.coef_ref * (qn + tmax) * (qn + tmax)) + 1e-30f;
        rad_lo = -0.5f * knn_threshold(p.r2up, __double2float_rd(p.qn2[q]), eq);
      }
      for (int tt = 0; tt < p.n_tiles_t; ++tt, ++it) {
        if ((it & 1) != g) continue;
        const int slot = it % kMaskSlots;
        bool ok = tc::mbar_wait(&accfull[g], (uint32_t)(it >> 1) & 1u, kWaitNs);
        // Every tile waits until the owners have taken the mask of tile it - 2
        // (tile 0 of the query tile for tile 1): by then they have finished
        // with tile it - 4, the slot's previous contents.  Threshold: tile 0
        // of a query tile admits every row; tile 1 uses the owners' replay of
        // tile 0; later tiles whatever the owners have published by now.
        float lo = live_q ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000);
        const int u = p.radius_mode || tt != 1 ? it - 2 : it - 1;
        if (u >= 0)
          ok = ok && tc::mbar_wait(&maskempty[u % kMaskSlots], (uint32_t)(u / kMaskSlots) & 1u, kWaitNs);
        if (p.radius_mode)
          lo = rad_lo;
        else if (tt >= 1)
          lo = *(volatile float *)&s_lo[row];
        if (!__all_sync(0xffffffffu, ok) || __any_sync(0xffffffffu, *(volatile int *)s_abort != 0)) {
          atomicExch(s_abort, 1);
          stop = true;
          break;
        }
        tc::fence_after_sync();
        const uint32_t tbase = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(g * TN);
        const uint32_t taddr = tbase + (uint32_t)c_lo;
        uint32_t *mcol = sMask + (size_t)slot * kWords * kQM + row;
        const int64_t j0 = (int64_t)tt * TN + c_lo;
        float lo_rest = lo;  // threshold for the rows after the tile's first 32
        if (tt == 0 && !p.radius_mode && p.k <= 32) {
          // No heap yet.  Once any k rows have been seen the root is at most
          // the largest of their distances, so every row after the first 32
          // needs acc_j > (k-th largest acc of those 32) - e: |acc - (||q||^2 -
          // D)/2| <= e/2 for both rows.  The 1% margin covers the f32 rounding.
          uint32_t v[32];
          tc::tmem_ld32(tbase, v);
          tc::tmem_wait_ld();
          float top[32];
          int nt = 0;
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) {  // k largest, descending (insertion)
            float x = __uint_as_float(v[jj]);
            if (nt < p.k) ++nt;
            else if (!(x > top[nt - 1])) continue;
            int pos = nt - 1;
            while (pos > 0 && top[pos - 1] < x) { top[pos] = top[pos - 1]; --pos; }
            top[pos] = x;
          }
          const int64_t q = (int64_t)qt * kQM + row;
          const float tmax = __uint_as_float(*p.tmax);
          const float qn = q < p.m ? p.qnrm[q] : 0.f;
          const float eq = 1.05f * (2.f * (p.coef_xc * qn * tmax + p.coef_cc * tmax * tmax) +
                                    p.coef_ref * (qn + tmax) * (qn + tmax)) + 1e-30f;
          lo_rest = live_q && p.n >= 32 ? top[p.k - 1] - 1.01f * eq - 1e-30f : lo;
        }
#pragma unroll 1
        for (int c1 = 0; c1 < kCols; c1 += 64) {  // 64 columns per TMEM round trip
          uint32_t v[64];
          tc::tmem_ld64(taddr + (uint32_t)c1, v);
          tc::tmem_wait_ld();
#pragma unroll
          for (int c2 = 0; c2 < 64; c2 += 32) {
            const int c0 = c1 + c2;
            if (c_lo + c0 >= 32) lo = lo_rest;
            float mx[16];  // max of the 32 columns as a tree (depth 5, not a chain of 31)
#pragma unroll
            for (int jj = 0; jj < 16; ++jj) mx[jj] = fmaxf(__uint_as_float(v[c2 + jj]), __uint_as_float(v[c2 + jj + 16]));
#pragma unroll
            for (int w2 = 8; w2 > 0; w2 >>= 1)
#pragma unroll
              for (int jj = 0; jj < w2; ++jj) mx[jj] = fmaxf(mx[jj], mx[jj + w2]);
            uint32_t mask = 0u;
            if (__any_sync(0xffffffffu, mx[0] >= lo)) {
#pragma unroll
              for (int jj = 0; jj < 32; ++jj) mask |= (__uint_as_float(v[c2 + jj]) >= lo ? 1u : 0u) << jj;
              const int64_t rem = p.n - (j0 + c0);  // rows past the end of the training set
              if (rem < 32) mask &= rem <= 0 ? 0u : ((1u << rem) - 1u);
            }
            mcol[(c_lo + c0) / 32 * kQM] = mask;
          }
        }
        tc::fence_before_sync();
        tc::mbar_arrive(&accempty[g]);
        tc::mbar_arrive(&maskfull[slot]);
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 2 * TN);
  }
  if (threadIdx.x == 0 && *s_abort) atomicExch(p.err, 4);
}

// ---------------------------------------------------------------------------
// find: a certified candidate filter on the tensor cores, then the exact
// replay per query on the CUDA cores
// ---------------------------------------------------------------------------
// The reference inserts row j exactly when D_j < root_j, the largest of the
// k smallest distances among rows 0..j-1 (+inf before k rows).  With acc_i
// the split-BF16 score, |acc_i - (||q||^2 - D_i) / 2| <= e / 2, so if T is the
// k-th largest acc among any prefix of rows 0..j-1 (-inf before k rows),
// T <= (||q||^2 - root_j) / 2 + e / 2 and D_j < root_j implies acc_j > T - e.
// Each filter lane keeps the k largest acc of its query (a min-heap in shared
// memory) and lists every row with acc_j >= T - e, in index order: a superset
// of the rows the reference inserts, found without any exact distance.  The
// refine kernel then computes the reference distances of the listed rows and
// replays the heap exactly.
// Filter CTA: warp 0 TMA, warp 1 MMA, then 4 filter warps per 128-query half.
template <int QH>
constexpr int filt_threads() { return 32 * (2 + 4 * QH); }

struct FilterParams {
  int64_t n, m;
  int b_box;
  int il;   // interleaved halves (KnnPipe::il)
  int qt0;  // the chunk's first query tile: cand and count are indexed from its first query
  int n_tiles_t, n_tiles_q;
  int nkt, kt_elems, row_bytes;
  int stages;
  int k;
  const float *qnrm;
  const unsigned int *tmax;
  float coef_xc, coef_cc, coef_ref;
  int64_t cap;                 // candidate slots per query
  int32_t *cand;               // [chunk queries][cap]: rows in index order
  int32_t *count;              // per query of the chunk: candidates, or -1 past cap
  int32_t *over;               // the queries past cap
  unsigned long long *stats;   // [1] wait timed out, [2] queries past cap
};

// Inserts x (> the root) into a lane's min-heap of its k largest scores
// (entries at stride kQM) and returns the new root, the k-th largest.
__device__ __noinline__ float topk_push(float *h, int k, float x) {
  int i = 0;
  while (true) {
    int c = 2 * i + 1;
    if (c >= k) break;
    float cv = h[c * kQM];
    if (c + 1 < k) {
      const float c2 = h[(c + 1) * kQM];
      if (c2 < cv) {
        cv = c2;
        ++c;
      }
    }
    if (!(cv < x)) break;
    h[i * kQM] = cv;
    i = c;
  }
  h[i * kQM] = x;
  return h[0];
}

__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// A filter lane's state for its query: candidates listed, the k-th largest
// score (its heap root) and the threshold root - e.
struct FiltLane {
  int64_t cnt;
  float root, lo;
};

// One block of W columns of a lane's scores (W / 8 <= 32 groups of 8), at
// TMEM address ta: the maxima of its 8-column groups against the threshold at
// the start of the block (a staler threshold only admits more) give each lane
// a mask of groups, one warp-wide OR the groups any lane needs.  Those are
// read again from TMEM, 8 columns at a time in a rolled loop (the per-column
// code exists once), and scanned: rows at or above the threshold are listed
// in index order and pushed into the top-k when above its root.
template <int W>
__device__ __forceinline__ void filt_block(FiltLane &st, const uint32_t (&v)[W], uint32_t ta, int64_t jb, int64_t n,
                                           int32_t *cq, int64_t cap, float *top, int k, float marg) {
  uint32_t lm = 0u;
#pragma unroll
  for (int g = 0; g < W / 8; ++g) {
    const float *x = (const float *)&v[8 * g];
    const float gm = fmax3(fmax3(x[0], x[1], x[2]), fmax3(x[3], x[4], x[5]), fmaxf(x[6], x[7]));
    lm |= (gm >= st.lo ? 1u : 0u) << g;
  }
#pragma unroll 1
  for (uint32_t um = __reduce_or_sync(0xffffffffu, lm); um; um &= um - 1u) {
    const int g = __ffs(um) - 1;
    uint32_t x8[8];
    tc::tmem_ld8(ta + (uint32_t)(8 * g), x8);
    tc::tmem_wait_ld();
    if ((lm >> g) & 1u) {
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const float x = __uint_as_float(x8[jj]);
        const int64_t row = jb + 8 * g + jj;
        if (x >= st.lo && row < n) {
          if (st.cnt < cap) cq[st.cnt] = (int32_t)row;
          ++st.cnt;
          if (x > st.root) {
            st.root = topk_push(top, k, x);
            st.lo = __fsub_rd(st.root, marg);
          }
        }
      }
    }
  }
}

// Roles: warp 0 TMA, warp 1 MMA (one elected thread each), warps 2 .. 4 QH + 1
// filters: warp w reads TMEM lane quarter w % 4 (32 queries) of query half
// (w - 2) / 4, every column of every tile, so each query's running top-k stays
// with one lane and is never stale.  A query tile is QH x 128 queries: every
// training tile brought on chip serves all of them.
template <int TN, int QH>
__global__ void __launch_bounds__(filt_threads<QH>(), 1)
knn_filter_kernel(const __grid_constant__ CUtensorMap tm_qh, const __grid_constant__ CUtensorMap tm_ql,
                  const __grid_constant__ CUtensorMap tm_th, const __grid_constant__ CUtensorMap tm_tl,
                  const __grid_constant__ CUtensorMap tm_ones, const __grid_constant__ CUtensorMap tm_tbx,
                  const FilterParams p) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int a_blk = kQM * p.row_bytes;
  const int a_bytes = (p.il ? 1 : 2) * p.nkt * a_blk;
  const int b_blk = TN * p.row_bytes;
  const int b_stage = (p.il ? 1 : 2) * p.nkt * b_blk + TN * 32;
  uint8_t *sA = base;
  uint8_t *sOnes = base + QH * a_bytes;
  uint8_t *sB = sOnes + kQM * 32;
  float *s_top = (float *)(sB + (size_t)p.stages * b_stage);  // [half][k][query]: min-heaps of the k largest scores
  uint64_t *bars = (uint64_t *)(s_top + QH * p.k * kQM);
  uint64_t *full = bars, *empty = bars + p.stages, *afull = bars + 2 * p.stages;
  uint64_t *aempty = afull + 1, *accfull = afull + 2, *accempty = afull + 4, *mma_done = afull + 6;
  uint32_t *s_tmem = (uint32_t *)(afull + 7);
  int *s_abort = (int *)(s_tmem + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < p.stages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(afull, 1);
    tc::mbar_init(aempty, 1);
    tc::mbar_init(mma_done, 1);
    for (int a = 0; a < 2; ++a) {
      tc::mbar_init(&accfull[a], 1);
      tc::mbar_init(&accempty[a], 32 * 4 * QH);
    }
    *s_abort = 0;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tm_qh);
    tc::prefetch_tmap(&tm_ql);
    tc::prefetch_tmap(&tm_th);
    tc::prefetch_tmap(&tm_tl);
    tc::prefetch_tmap(&tm_ones);
    tc::prefetch_tmap(&tm_tbx);
  }
  if (warp == 1) {
    tc::tmem_alloc(s_tmem, 2 * QH * TN);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *s_tmem;
  const KnnPipe P{sA, sOnes, sB, full, empty, afull, aempty, accfull, accempty, mma_done, s_abort,
                  a_blk, a_bytes, b_blk, b_stage, p.n_tiles_q, p.n_tiles_t, p.nkt, p.kt_elems, p.row_bytes,
                  p.stages, QH, p.b_box, p.qt0, p.il};
  if (warp == 0) {
    if (lane == 0) knn_tma_role<TN>(P, &tm_qh, &tm_ql, &tm_th, &tm_tl, &tm_ones, &tm_tbx);
  } else if (warp == 1) {
    if (lane == 0) knn_mma_role<TN>(P, tmem);
  } else {
    const int lq = warp & 3, half = (warp - 2) >> 2;
    const int row = lq * 32 + lane;
    const float tmax = __uint_as_float(*p.tmax);
    float *top = s_top + half * p.k * kQM + row;
    int it = 0;
    bool stop = false;
    for (int qt = blockIdx.x; !stop && qt < p.n_tiles_q; qt += gridDim.x) {
      const int64_t ql = ((int64_t)qt * QH + half) * kQM + row;  // within the chunk
      const int64_t q = (int64_t)p.qt0 * QH * kQM + ql;
      const bool live = q < p.m;
      for (int s = 0; s < p.k; ++s) top[s * kQM] = -__int_as_float(0x7f800000);
      float root = -__int_as_float(0x7f800000);
      const float qn = live ? p.qnrm[q] : 0.f;
      // e bounds |a_j - (D_j - ||q||^2)| for a_j = -2 acc_j (see split.cu for
      // the terms); the 1% covers the f32 roundings of the comparison
      const float eq = 1.05f * (2.f * (p.coef_xc * qn * tmax + p.coef_cc * tmax * tmax) +
                                p.coef_ref * (qn + tmax) * (qn + tmax)) + 1e-30f;
      const float marg = __fadd_ru(__fmul_ru(1.01f, eq), 1e-30f);
      FiltLane st{0, root, live ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000)};
      int32_t *cq = p.cand + (live ? ql : 0) * p.cap;
      for (int tt = 0; tt < p.n_tiles_t; ++tt, ++it) {
        const int acc = it & 1;
        const bool got = tc::mbar_wait(&accfull[acc], (uint32_t)(it >> 1) & 1u, kWaitNs);
        if (!__all_sync(0xffffffffu, got) || __any_sync(0xffffffffu, *(volatile int *)s_abort != 0)) {
          atomicExch(s_abort, 1);
          stop = true;
          break;
        }
        tc::fence_after_sync();
        const uint32_t taddr = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)((2 * half + acc) * TN);
        const int64_t j0 = (int64_t)tt * TN;
        // blocks of up to 128 columns: their TMEM loads issued together, then
        // one scan (a rolled loop over the blocks keeps the code small)
        constexpr int W = TN < 128 ? TN : 128;
#pragma unroll 1
        for (int c = 0; c < TN; c += W) {
          uint32_t v[W];
#pragma unroll
          for (int c2 = 0; c2 < W; c2 += 32)
            tc::tmem_ld32(taddr + (uint32_t)(c + c2), *reinterpret_cast<uint32_t(*)[32]>(&v[c2]));
          tc::tmem_wait_ld();
          filt_block<W>(st, v, taddr + (uint32_t)c, j0 + c, p.n, cq, p.cap, top, p.k, marg);
        }
        tc::fence_before_sync();
        tc::mbar_arrive(&accempty[acc]);
      }
      const int64_t cnt = st.cnt;
      if (live && !stop) {
        if (cnt <= p.cap) {
          p.count[ql] = (int32_t)cnt;
        } else {
          p.count[ql] = -1;
          p.over[atomicAdd(&p.stats[2], 1ull)] = (int32_t)q;
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 2 * QH * TN);
  }
  if (threadIdx.x == 0 && *s_abort) atomicExch(&p.stats[1], 1ull);
}

// The reference's squared distance of a query row and a training row.
template <typename T>
__device__ __forceinline__ double knn_exact_sqd(const T *__restrict__ a, const T *__restrict__ b, int d, int lg_d) {
  double sq;
  if constexpr (sizeof(T) == 4) {
    if (d <= 32 ? sqd_f32_d32(a, b, d, lg_d, sq) : sqd_seq_f32(a, b, d, lg_d, sq)) return sq;
  }
  sq = 0.0;
  for (int t = 0; t < d; ++t) sq = __dadd_rn(sq, ref_term(a[t], b[t]));
  return sq;
}

// A row of d <= 32 f32 features into registers, zeros past d: 16-byte loads
// when d % 4 == 0 (rows then start on 16-byte boundaries), else scalar.
__device__ __forceinline__ void load_row32(const float *__restrict__ p, int d, float (&x)[32]) {
  if ((d & 3) == 0) {
#pragma unroll
    for (int t = 0; t < 32; t += 4) {
      const float4 v = t < d ? __ldg(reinterpret_cast<const float4 *>(p + t)) : make_float4(0.f, 0.f, 0.f, 0.f);
      x[t] = v.x;
      x[t + 1] = v.y;
      x[t + 2] = v.z;
      x[t + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int t = 0; t < 32; ++t) x[t] = t < d ? __ldg(p + t) : 0.f;
  }
}

// One lane per query: the reference distances of its candidates in index
// order, each followed by the reference's insertion test and heapify
// (linear_search.rs:72-77, heap_select.rs:42-50, :71-86).  The reference's
// heapify after a replaced root runs sift_down from every internal node; all
// of them but the root's find their (unchanged) subtrees already in heap order
// and stop at once (the heap never holds a NaN: a NaN distance fails the
// insertion test), so one sift_down from the root leaves the same array.
// The heaps live in shared memory, entry e of lane l at [e][l].  Queries past
// the candidate capacity (count -1) are left to the FP64 kernel.
constexpr int kRefineThreads = 64;
template <typename T>
__global__ void __launch_bounds__(kRefineThreads)
knn_refine_kernel(const T *__restrict__ train, const T *__restrict__ queries, int64_t q0, int64_t m, int d, int lg_d,
                  int k, int64_t cap, const int32_t *__restrict__ cand, const int32_t *__restrict__ count,
                  int64_t *__restrict__ idx_out, double *__restrict__ dist_out, unsigned long long *evals) {
  extern __shared__ __align__(8) uint8_t refine_smem[];
  double *hD = (double *)refine_smem + threadIdx.x;
  int32_t *hi = (int32_t *)((double *)refine_smem + (size_t)k * kRefineThreads) + threadIdx.x;
  const int64_t ql = (int64_t)blockIdx.x * kRefineThreads + threadIdx.x;  // within the chunk of m queries
  const int64_t q = q0 + ql;
  unsigned long long ev = 0;
  if (ql < m) {
    const int c = count[ql];
    if (c >= 0) {
      for (int s = 0; s < k; ++s) {
        hD[s * kRefineThreads] = __longlong_as_double(0x7ff0000000000000ll);
        hi[s * kRefineThreads] = -1;
      }
      double root = __longlong_as_double(0x7ff0000000000000ll);
      const T *qrow = queries + q * d;
      const int32_t *cq = cand + ql * cap;
      // f32 rows of up to 32 features: the query row held in registers, each
      // candidate row loaded whole (16-byte loads when d % 4 == 0)
      float qv[32];
      const bool regs = sizeof(T) == 4 && d <= 32;
      if constexpr (sizeof(T) == 4) {
        if (regs) load_row32((const float *)qrow, d, qv);
      }
      for (int r = 0; r < c; ++r) {
        const int32_t j = cq[r];
        double sr;
        if constexpr (sizeof(T) == 4) {
          if (regs) {
            float xv[32];
            load_row32((const float *)(train + (int64_t)j * d), d, xv);
#pragma unroll
            for (int t = 0; t < 32; ++t) {
              const float df = __fsub_rn(qv[t], xv[t]);
              xv[t] = __fmul_rn(df, df);
            }
            if (!sqd_terms32(xv, d, lg_d, sr)) {
              sr = 0.0;
#pragma unroll
              for (int t = 0; t < 32; ++t)
                if (t < d) sr = __dadd_rn(sr, (double)xv[t]);
            }
          } else {
            sr = knn_exact_sqd<T>(qrow, train + (int64_t)j * d, d, lg_d);
          }
        } else {
          sr = knn_exact_sqd<T>(qrow, train + (int64_t)j * d, d, lg_d);
        }
        if (sqrt_less(sr, root)) {  // sqrt(D) < root (linear_search.rs:72)
          hD[0] = sr;
          hi[0] = j;
          if (k > 1) heap_sift<kRefineThreads>(hD, hi, 0, k - 1);
          root = hD[0];
        }
      }
      ev = (unsigned long long)c;
      for (int s = 0; s < k; ++s) {
        idx_out[q * k + s] = hi[s * kRefineThreads];
        dist_out[q * k + s] = __dsqrt_rn(hD[s * kRefineThreads]);  // sqrt(+inf) = +inf for an empty slot
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ev += __shfl_xor_sync(0xffffffffu, ev, o);
  if ((threadIdx.x & 31) == 0 && ev) atomicAdd(evals, ev);
}

// Queries past the candidate capacity: their rows gathered for the FP64
// kernel, and its heaps scattered back.
template <typename T>
__global__ void gather_rows_kernel(const T *__restrict__ src, const int32_t *__restrict__ rows, int64_t nr, int d,
                                   T *__restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nr * d) return;
  dst[i] = src[(int64_t)rows[i / d] * d + i % d];
}
__global__ void scatter_heaps_kernel(const int32_t *__restrict__ rows, int64_t nr, int k,
                                     const int64_t *__restrict__ isub, const double *__restrict__ dsub,
                                     int64_t *__restrict__ idx, double *__restrict__ dist) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nr * k) return;
  const int64_t q = rows[i / k];
  idx[q * k + i % k] = isub[i];
  dist[q * k + i % k] = dsub[i];
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

sc_status map2d(CUtensorMap *m, void *ptr, int64_t rows, int cols, int box_cols, int box_rows, int row_bytes) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &f, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      set_error("cuTensorMapEncodeTiled is unavailable");
      return SC_ERR_CUDA;
    }
    fn = (EncodeTiledFn)f;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUtensorMapSwizzle sw = row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                : row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                  : CU_TENSOR_MAP_SWIZZLE_32B;
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return SC_ERR_CUDA; }
  return SC_OK;
}


int knn_pad_d(int d) { return d <= 16 ? 16 : d <= 32 ? 32 : (d + 63) / 64 * 64; }

// Training rows per TMA box: 128 up to d_pad = 64, then 64 so that the
// resident query tile and two or more training stages fit in shared memory.
int knn_tile_n(int d_pad) { return d_pad <= 64 ? 128 : 64; }

size_t knn_smem(int nkt, int row_bytes, int stages, int tn, int heap_k, int dtype) {
  return 1024 + (size_t)2 * nkt * kQM * row_bytes + kQM * 32 + (size_t)stages * (2 * nkt * tn * row_bytes + tn * 32) +
         (size_t)kOwnerWarps * kQueue * 4 + (size_t)kMaskSlots * kQM * (tn / 32) * 4 +
         (dtype == SC_F32 ? (size_t)kOwnerWarps * kStageFloats * 4 : 0) + kQM * 4 +
         (size_t)kOwnerWarps * 32 * 16 + (size_t)heap_k * kQM * 12 + 8 +
         (size_t)(2 * stages + 7 + 2 * kMaskSlots) * 8 + 16;
}

// Training rows per tile of both kNN kernels: 256 up to d_pad = 32 (one
// 128 x 256 MMA per K step: the fewest MMA instructions per score), then the
// TMA box height of knn_tile_n.  One 128-query half per query tile.
int filt_tile_n(int d_pad) { return d_pad <= 32 ? 256 : knn_tile_n(d_pad); }
int filt_halves(int) { return 1; }

size_t filt_smem(int nkt, int row_bytes, int stages, int tn, int k, int qh) {
  return 1024 + (size_t)qh * 2 * nkt * kQM * row_bytes + kQM * 32 +
         (size_t)stages * (2 * nkt * tn * row_bytes + tn * 32) + (size_t)qh * k * kQM * 4 +
         (size_t)(2 * stages + 7) * 8 + 16;
}

// Training stages of the filter kernel: as many as fit, up to 6 (deeper
// queues hide DRAM latency when the training rows exceed L2).
int filt_stages(int nkt, int row_bytes, int tn, int k, int qh) {
  int st = 6;
  while (st > 2 && filt_smem(nkt, row_bytes, st, tn, k, qh) > 227 * 1024) --st;
  return st;
}

// Candidate slots per query: about 6 k (1 + ln(n / k)), the expected number
// of heap insertions k (1 + ln(n / k)) of rows in random order with room for
// ordered data, ties and the bound's slack; a query past it is served by the
// streaming kernel (exact root feedback, no capacity).
int64_t g_knn_cap_override = 0;
int64_t g_knn_chunk_override = 0;
int64_t knn_candidate_cap(int64_t n, int k) {
  if (g_knn_cap_override > 0) return g_knn_cap_override;
  const double r = (double)n / k > 1.0 ? (double)n / k : 1.0;
  int64_t c = (int64_t)(6.0 * k * (1.0 + log(r))) + 64;
  c = (c + 31) / 32 * 32;
  return c < 256 ? 256 : c;
}

template <int TN, int QH>
sc_status launch_knn_filter(int grid, size_t smem, const CUtensorMap &tm_qh, const CUtensorMap &tm_ql,
                            const SplitKnnState *s, const FilterParams &p, cudaStream_t st) {
  auto kern = knn_filter_kernel<TN, QH>;
  SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, filt_threads<QH>(), smem, st>>>(tm_qh, tm_ql, s->tm_th, s->tm_tl, s->tm_ones, s->tm_tbx, p);
  SC_LAUNCHED();
  return SC_OK;
}

template <typename T, int TN, bool SH>
sc_status launch_knn_split(int grid, size_t smem, const CUtensorMap &tm_qh, const CUtensorMap &tm_ql,
                           const SplitKnnState *s, const void *train, const void *queries, const KnnParams &p,
                           cudaStream_t st) {
  auto kern = knn_split_kernel<T, TN, SH>;
  SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, kKnnThreads, smem, st>>>(tm_qh, tm_ql, s->tm_th, s->tm_tl, s->tm_ones, s->tm_tbx, (const T *)train,
                                        (const T *)queries, p);
  SC_LAUNCHED();
  return SC_OK;
}

}  // namespace

namespace {
struct RadiusArgs {
  double radius;
  int64_t *counts;         // counting pass (idx == nullptr), or slot pass
  const int64_t *offsets;  // filling pass
  int64_t cap_q;           // slot pass: rows kept per query (offsets == nullptr)
};

struct RadiusArgs;
sc_status run_split_knn(SplitKnnState *s, int dtype, const void *train, int64_t n, int d, const void *queries,
                        int64_t m, int k, int64_t *idx, double *dist, int64_t *rescored, const RadiusArgs *rad,
                        cudaStream_t st, bool streaming = false);

// find: the candidate filter, the exact replay per query, and for the queries
// past the candidate capacity the streaming kernel (or, where its shared
// memory does not fit, the FP64 kernel).
sc_status run_split_find(SplitKnnState *s, int dtype, const void *train, int64_t n, int d, int lg_d,
                         const void *queries, int64_t m, int64_t m_pad, int k, int64_t *idx, double *dist,
                         int64_t *rescored, const CUtensorMap &tm_qh, const CUtensorMap &tm_ql, int nkt, int kt_elems,
                         int row_bytes, int il, int tn, float coef_xc, float coef_cc, float coef_ref, cudaStream_t st) {
  const int qh = filt_halves(nkt * kt_elems);
  const int b_box = knn_tile_n(nkt * kt_elems);  // rows per box of the training maps
  const int stages = filt_stages(nkt, row_bytes, tn, k, qh);
  const size_t smem = filt_smem(nkt, row_bytes, stages, tn, k, qh);
  if (smem > 227 * 1024) {
    set_error("d=%d exceeds the split-BF16 kNN kernel's shared memory", d);
    return SC_ERR_INVALID;
  }
  const int64_t cap = knn_candidate_cap(n, k);
  // queries in chunks whose candidate lists take at most 2 GB, whole query tiles
  const int64_t tile_q = (int64_t)kQM * qh;
  int64_t chunk = (g_knn_chunk_override > 0 ? g_knn_chunk_override : ((int64_t)1 << 31) / (cap * 4)) / tile_q * tile_q;
  if (chunk < tile_q) chunk = tile_q;
  if (chunk > m_pad) chunk = m_pad;
  if ((size_t)(chunk * cap) > s->cand_cap || m_pad > s->count_cap) {
    s->cand_cap = 0;
    s->count_cap = 0;
    dfree(s->cand, st); dfree(s->count, st); dfree(s->over, st);
    SC_TRY(dalloc(&s->cand, (size_t)(chunk * cap), st));
    SC_TRY(dalloc(&s->count, (size_t)m_pad, st));
    SC_TRY(dalloc(&s->over, (size_t)m_pad, st));
    s->cand_cap = (size_t)(chunk * cap);
    s->count_cap = m_pad;
  }
  FilterParams fp;
  memset(&fp, 0, sizeof fp);
  fp.n = n;
  fp.m = m;
  fp.n_tiles_t = (int)((n + tn - 1) / tn);
  fp.b_box = b_box;
  fp.n_tiles_q = 0;  // per chunk, below
  fp.nkt = nkt;
  fp.kt_elems = kt_elems;
  fp.row_bytes = il ? 2 * row_bytes : row_bytes;  // sizes above use the half width: the same bytes either way
  fp.il = il;
  fp.stages = stages;
  fp.k = k;
  fp.qnrm = s->qnrm;
  fp.tmax = s->tmax;
  fp.coef_xc = coef_xc;
  fp.coef_cc = coef_cc;
  fp.coef_ref = coef_ref;
  fp.cap = cap;
  fp.cand = s->cand;
  fp.count = s->count;
  fp.over = s->over;
  fp.stats = s->evals;
  for (int64_t q0 = 0; q0 < m; q0 += chunk) {
    const int64_t mc = m - q0 < chunk ? m - q0 : chunk;
    fp.qt0 = (int)(q0 / tile_q);
    fp.n_tiles_q = (int)((mc + tile_q - 1) / tile_q);
    const int grid = fp.n_tiles_q < s->num_sms ? fp.n_tiles_q : s->num_sms;
    if (tn == 256)
      SC_TRY((launch_knn_filter<256, 1>(grid, smem, tm_qh, tm_ql, s, fp, st)));
    else if (tn == 128)
      SC_TRY((launch_knn_filter<128, 1>(grid, smem, tm_qh, tm_ql, s, fp, st)));
    else
      SC_TRY((launch_knn_filter<64, 1>(grid, smem, tm_qh, tm_ql, s, fp, st)));
    const int rgrid = (int)((mc + kRefineThreads - 1) / kRefineThreads);
    const size_t rsmem = (size_t)k * kRefineThreads * 12;
    if (dtype == SC_F32)
      knn_refine_kernel<float><<<rgrid, kRefineThreads, rsmem, st>>>((const float *)train, (const float *)queries, q0,
                                                                      mc, d, lg_d, k, cap, s->cand, s->count, idx,
                                                                      dist, s->evals);
    else
      knn_refine_kernel<double><<<rgrid, kRefineThreads, rsmem, st>>>((const double *)train, (const double *)queries,
                                                                       q0, mc, d, lg_d, k, cap, s->cand, s->count,
                                                                       idx, dist, s->evals);
    SC_LAUNCHED();
  }
  unsigned long long host[3];
  SC_CUDA(cudaMemcpyAsync(host, s->evals, sizeof host, cudaMemcpyDeviceToHost, st));
  SC_CUDA(cudaStreamSynchronize(st));
  if (host[1]) {
    set_error("split-BF16 kNN kernel: a bounded wait timed out");
    return SC_ERR_TIMEOUT;
  }
  int64_t evals = (int64_t)host[0];
  const int64_t nover = (int64_t)host[2];
  if (nover > 0) {  // past the candidate capacity: the FP64 kernel on those queries
    const size_t es = dtype == SC_F32 ? 4 : 8;
    char *qsub = nullptr;
    int64_t *isub = nullptr;
    double *dsub = nullptr;
    sc_status r = dalloc(&qsub, (size_t)nover * d * es, st);
    if (r == SC_OK) r = dalloc(&isub, (size_t)(nover * k), st);
    if (r == SC_OK) r = dalloc(&dsub, (size_t)(nover * k), st);
    if (r == SC_OK) {
      const int64_t tot = nover * d;
      const int gb = (int)((tot + 255) / 256);
      if (dtype == SC_F32)
        gather_rows_kernel<float><<<gb, 256, 0, st>>>((const float *)queries, s->over, nover, d, (float *)qsub);
      else
        gather_rows_kernel<double><<<gb, 256, 0, st>>>((const double *)queries, s->over, nover, d, (double *)qsub);
      if (cudaGetLastError() != cudaSuccess) r = SC_ERR_CUDA;
      note_launch();
    }
    int64_t ev2 = nover * n;
    if (r == SC_OK) {
      const int d_pad = nkt * kt_elems, stn = filt_tile_n(d_pad);
      const bool sh = knn_smem(nkt, row_bytes, 2, stn, k, dtype) <= 227 * 1024;
      if (knn_smem(nkt, row_bytes, 2, stn, sh ? k : 0, dtype) <= 227 * 1024)
        r = run_split_knn(s, dtype, train, n, d, qsub, nover, k, isub, dsub, &ev2, nullptr, st, true);
      else
        r = launch_knn_fp64(dtype, train, n, d, qsub, nover, k, isub, dsub, st);
    }
    if (r == SC_OK) {
      scatter_heaps_kernel<<<(int)((nover * k + 255) / 256), 256, 0, st>>>(s->over, nover, k, isub, dsub, idx, dist);
      if (cudaGetLastError() != cudaSuccess) r = SC_ERR_CUDA;
      note_launch();
    }
    if (r == SC_OK && cudaStreamSynchronize(st) != cudaSuccess) r = SC_ERR_CUDA;
    dfree(qsub, st);
    dfree(isub, st);
    dfree(dsub, st);
    if (r != SC_OK) {
      if (r == SC_ERR_CUDA) set_error("kNN: the pass over %lld queries past the candidate capacity failed",
                                      (long long)nover);
      return r;
    }
    evals += ev2;
  }
  if (rescored) *rescored = evals;
  return SC_OK;
}

// streaming: find through the streaming kernel (each query's heap replayed as
// the tiles arrive; no candidate capacity) instead of filter + replay.
sc_status run_split_knn(SplitKnnState *s, int dtype, const void *train, int64_t n, int d, const void *queries,
                        int64_t m, int k, int64_t *idx, double *dist, int64_t *rescored, const RadiusArgs *rad,
                        cudaStream_t st, bool streaming) {
  if (rescored) *rescored = 0;
  if (m == 0 || n == 0) return SC_OK;
  if (n >= ((int64_t)1 << kRowBits)) {
    set_error("n=%lld exceeds the split-BF16 kNN kernel's limit of 2^27 training rows", (long long)n);
    return SC_ERR_INVALID;
  }
  const int d_pad = knn_pad_d(d);
  const int kt_elems = d_pad >= 64 ? 64 : d_pad, nkt = d_pad / kt_elems, row_bytes = kt_elems * 2;
  // d_pad = 32: both halves of a row in one 128-byte row (128-byte swizzle);
  // the same bytes as two 64-byte operands, so the sizes keep row_bytes
  const int il = d_pad == 32 ? 1 : 0, lay_bytes = il ? 2 * row_bytes : row_bytes;
  const int tn = filt_tile_n(d_pad), box = knn_tile_n(d_pad);
  // heaps in shared memory when they fit beside at least two training stages
  bool sh = knn_smem(nkt, row_bytes, 2, tn, k, dtype) <= 227 * 1024;
  const int heap_k = sh ? k : 0;
  int stages = 4;
  while (stages > 2 && knn_smem(nkt, row_bytes, stages, tn, heap_k, dtype) > 227 * 1024) --stages;
  const size_t smem = knn_smem(nkt, row_bytes, stages, tn, heap_k, dtype);
  if (d_pad > 256 || smem > 227 * 1024) {
    set_error("d=%d exceeds the split-BF16 kNN kernel's shared memory", d);
    return SC_ERR_INVALID;
  }
  int dev = 0;
  SC_CUDA(cudaGetDevice(&dev));
  if (!s->num_sms) SC_CUDA(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t n_pad = (n + 255) / 256 * 256;  // whole tiles of every kernel (TMA boxes never leave the operand)
  if (!s->ready || s->train != train || s->n != n || s->d != d) {  // training operand, once per handle
    s->ready = 0;  // until every buffer below exists
    dfree(s->th, st); dfree(s->tl, st); dfree(s->tbx, st); dfree(s->tmax, st); dfree(s->ones, st);
    SC_TRY(dalloc(&s->th, (size_t)n_pad * d_pad * (il ? 2 : 1), st));
    if (!il) SC_TRY(dalloc(&s->tl, (size_t)n_pad * d_pad, st));
    SC_TRY(dalloc(&s->tbx, (size_t)n_pad * 16, st));
    SC_TRY(dalloc(&s->tmax, 1, st));
    SC_TRY(dalloc(&s->ones, (size_t)kQM * 16, st));
    ones_tile_kernel<<<1, kQM, 0, st>>>(s->ones);
    SC_LAUNCHED();
    SC_TRY(map2d(&s->tm_ones, s->ones, kQM, 16, 16, kQM, 32));
    SC_CUDA(cudaMemsetAsync(s->tmax, 0, sizeof(unsigned int), st));
    const int nb = (int)((n_pad + 7) / 8);
    if (dtype == SC_F32)
      knn_prep_kernel<float><<<nb, 256, 0, st>>>((const float *)train, n, n_pad, d, d_pad, il ? 2 * d_pad : d_pad,
                                                s->th, il ? s->th + d_pad : s->tl, nullptr,
                                                nullptr, nullptr, s->tmax, s->tbx);
    else
      knn_prep_kernel<double><<<nb, 256, 0, st>>>((const double *)train, n, n_pad, d, d_pad, il ? 2 * d_pad : d_pad,
                                                 s->th, il ? s->th + d_pad : s->tl,
                                                 nullptr, nullptr, nullptr, s->tmax, s->tbx);
    SC_LAUNCHED();
    if (il) {
      SC_TRY(map2d(&s->tm_th, s->th, n_pad, 2 * d_pad, 2 * kt_elems, box, lay_bytes));
      s->tm_tl = s->tm_th;  // unused: one operand holds both halves
    } else {
      SC_TRY(map2d(&s->tm_th, s->th, n_pad, d_pad, kt_elems, box, row_bytes));
      SC_TRY(map2d(&s->tm_tl, s->tl, n_pad, d_pad, kt_elems, box, row_bytes));
    }
    SC_TRY(map2d(&s->tm_tbx, s->tbx, n_pad, 16, 16, box, 32));
    s->train = train;
    s->n = n;
    s->d = d;
    s->ready = 1;
  }
  const int64_t m_pad = (m + 2 * kQM - 1) / (2 * kQM) * (2 * kQM);  // whole 256-query tiles
  if (m_pad > s->m_cap) {
    s->m_cap = 0;  // a failed allocation leaves no stale capacity
    dfree(s->qh, st); dfree(s->ql, st); dfree(s->qnrm, st); dfree(s->qn2, st);
    SC_TRY(dalloc(&s->qh, (size_t)m_pad * d_pad * (il ? 2 : 1), st));
    if (!il) SC_TRY(dalloc(&s->ql, (size_t)m_pad * d_pad, st));
    SC_TRY(dalloc(&s->qnrm, (size_t)m_pad, st));
    SC_TRY(dalloc(&s->qn2, (size_t)m_pad, st));
    s->m_cap = m_pad;
  }
  if (!s->evals) SC_TRY(dalloc(&s->evals, 3, st));
  SC_CUDA(cudaMemsetAsync(s->evals, 0, 3 * sizeof(unsigned long long), st));
  const int nbq = (int)((m_pad + 7) / 8);
  if (dtype == SC_F32)
    knn_prep_kernel<float><<<nbq, 256, 0, st>>>((const float *)queries, m, m_pad, d, d_pad, il ? 2 * d_pad : d_pad,
                                               s->qh, il ? s->qh + d_pad : s->ql, s->qnrm,
                                               nullptr, s->qn2, nullptr, nullptr);
  else
    knn_prep_kernel<double><<<nbq, 256, 0, st>>>((const double *)queries, m, m_pad, d, d_pad, il ? 2 * d_pad : d_pad,
                                                s->qh, il ? s->qh + d_pad : s->ql,
                                                s->qnrm, nullptr, s->qn2, nullptr, nullptr);
  SC_LAUNCHED();
  CUtensorMap tm_qh, tm_ql;
  if (il) {
    SC_TRY(map2d(&tm_qh, s->qh, m_pad, 2 * d_pad, 2 * kt_elems, kQM, lay_bytes));
    tm_ql = tm_qh;
  } else {
    SC_TRY(map2d(&tm_qh, s->qh, m_pad, d_pad, kt_elems, kQM, row_bytes));
    SC_TRY(map2d(&tm_ql, s->ql, m_pad, d_pad, kt_elems, kQM, row_bytes));
  }
  const double nacc = 3.0 * d_pad + 3.0;
  const float coef_xc = (float)(3.02 * 0x1p-16 + 1.02 * nacc * 0x1p-22);
  const float coef_cc = (float)(1.01 * 0x1p-25 + 0.51 * nacc * 0x1p-22);
  const float coef_ref = (float)((d + 4) * 0x1p-52);
  int lg_d = 0;
  while ((1 << lg_d) < d) ++lg_d;
  if (!rad && !streaming)
    return run_split_find(s, dtype, train, n, d, lg_d, queries, m, m_pad, k, idx, dist, rescored, tm_qh, tm_ql, nkt,
                          kt_elems, row_bytes, il, tn, coef_xc, coef_cc, coef_ref, st);
  KnnParams p;
  memset(&p, 0, sizeof p);
  p.n = n;
  p.m = m;
  p.n_tiles_t = (int)(n_pad / tn);
  p.n_tiles_q = (int)(m_pad / kQM);
  p.b_box = box;
  p.nkt = nkt;
  p.kt_elems = kt_elems;
  p.row_bytes = lay_bytes;
  p.il = il;
  p.stages = stages;
  p.k = k;
  p.d = d;
  p.lg_d = lg_d;
  p.qnrm = s->qnrm;
  p.qn2 = s->qn2;
  p.tmax = s->tmax;
  p.coef_xc = coef_xc;
  p.coef_cc = coef_cc;
  p.coef_ref = coef_ref;
  p.idx_out = idx;
  p.dist_out = dist;
  if (rad) {
    p.radius_mode = 1;
    p.radius = rad->radius;
    p.r2up = rad->radius * rad->radius * (1.0 + 0x1p-48);  // covers every D with sqrt(D) rounding to <= radius
    p.counts = rad->counts;
    p.offsets = rad->offsets;
    p.cap_q = rad->cap_q;
  }
  p.evals = s->evals;
  p.err = (int *)(s->evals + 1);
  const int grid = p.n_tiles_q < s->num_sms ? p.n_tiles_q : s->num_sms;
  sc_status r;
#define SC_KNN_LAUNCH(TT, NN)                                                                        \
  (sh ? launch_knn_split<TT, NN, true>(grid, smem, tm_qh, tm_ql, s, train, queries, p, st)            \
      : launch_knn_split<TT, NN, false>(grid, smem, tm_qh, tm_ql, s, train, queries, p, st))
  if (dtype == SC_F32)
    r = tn == 256 ? SC_KNN_LAUNCH(float, 256) : tn == 128 ? SC_KNN_LAUNCH(float, 128) : SC_KNN_LAUNCH(float, 64);
  else
    r = tn == 256 ? SC_KNN_LAUNCH(double, 256) : tn == 128 ? SC_KNN_LAUNCH(double, 128) : SC_KNN_LAUNCH(double, 64);
#undef SC_KNN_LAUNCH
  SC_TRY(r);
  unsigned long long host[2];
  SC_CUDA(cudaMemcpyAsync(host, s->evals, sizeof host, cudaMemcpyDeviceToHost, st));
  SC_CUDA(cudaStreamSynchronize(st));
  if (host[1]) {
    set_error("split-BF16 kNN kernel: a bounded wait timed out");
    return SC_ERR_TIMEOUT;
  }
  if (rescored) *rescored = (int64_t)host[0];
  return SC_OK;
}

}  // namespace

void split_knn_set_candidate_cap(int64_t cap) { g_knn_cap_override = cap > 0 ? cap : 0; }
void split_knn_set_chunk_queries(int64_t q) { g_knn_chunk_override = q > 0 ? q : 0; }

bool split_knn_serves(int d, int k, int dtype, bool radius) {
  const int d_pad = knn_pad_d(d);
  if (d_pad > 256 || k > kMaxKnnK) return false;
  const int kt = d_pad >= 64 ? 64 : d_pad, nkt = d_pad / kt, rb = kt * 2, tn = filt_tile_n(d_pad);
  if (!radius) return filt_smem(nkt, rb, 2, filt_tile_n(d_pad), k, filt_halves(d_pad)) <= 227 * 1024;
  const bool sh = knn_smem(nkt, rb, 2, tn, k, dtype) <= 227 * 1024;
  return knn_smem(nkt, rb, 2, tn, sh ? k : 0, dtype) <= 227 * 1024;
}

sc_status split_knn(SplitKnnState *s, int dtype, const void *train, int64_t n, int d, const void *queries,
                    int64_t m, int k, int64_t *idx, double *dist, int64_t *rescored, cudaStream_t st) {
  return run_split_knn(s, dtype, train, n, d, queries, m, k, idx, dist, rescored, nullptr, st);
}

sc_status split_knn_radius(SplitKnnState *s, int dtype, const void *train, int64_t n, int d, const void *queries,
                           int64_t m, double radius, int64_t *counts, const int64_t *offsets, int64_t *idx,
                           double *dist, cudaStream_t st) {
  const RadiusArgs rad{radius, counts, offsets, 0};
  return run_split_knn(s, dtype, train, n, d, queries, m, 0, idx, dist, nullptr, &rad, st);
}

namespace {
// Row q's first min(counts[q], cap) slots of the slot pass to its place in
// the packed lists, one warp per query.
__global__ void pack_radius_kernel(const int64_t *__restrict__ pad_idx, const double *__restrict__ pad_dist,
                                   int64_t cap, const int64_t *__restrict__ counts, const int64_t *__restrict__ off,
                                   int64_t m, int64_t *__restrict__ idx, double *__restrict__ dist) {
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= m) return;
  const int64_t c = counts[q] < cap ? counts[q] : cap, o = off[q];
  for (int64_t e = lane; e < c; e += 32) {
    idx[o + e] = pad_idx[q * cap + e];
    dist[o + e] = pad_dist[q * cap + e];
  }
}
}  // namespace

// find_radius lists of m device queries in one pass in the usual case: the
// slot pass keeps each query's first kRadiusSlots rows and counts them all;
// the packed lists (CSR: off, m + 1 entries on the host; idx / dist on the
// device, allocated here) take the kept rows, and the queries with more
// rows than slots run the filling pass alone, writing their whole lists in
// place.  Returns SC_ERR_INVALID (nothing allocated) when the slots of m
// queries would take more than 2 GB; the caller then counts and fills.
sc_status split_knn_radius_lists(SplitKnnState *s, int dtype, const void *train, int64_t n, int d,
                                 const void *queries, int64_t m, double radius, std::vector<int64_t> &off,
                                 int64_t **idx_out, double **dist_out, cudaStream_t st) {
  constexpr int64_t kRadiusSlots = 128;
  *idx_out = nullptr;
  *dist_out = nullptr;
  off.assign((size_t)m + 1, 0);
  if (m == 0) return SC_OK;
  if (m * kRadiusSlots * 16 > ((int64_t)1 << 31)) return SC_ERR_INVALID;
  int64_t *pad_idx = nullptr, *cnt = nullptr, *doff = nullptr, *oidx = nullptr, *sub_off = nullptr;
  double *pad_dist = nullptr, *odist = nullptr;
  int32_t *sub_rows = nullptr;
  char *sub_q = nullptr;
  sc_status r = SC_OK;
  do {
    if ((r = dalloc(&pad_idx, (size_t)(m * kRadiusSlots), st)) != SC_OK ||
        (r = dalloc(&pad_dist, (size_t)(m * kRadiusSlots), st)) != SC_OK || (r = dalloc(&cnt, (size_t)m, st)) != SC_OK ||
        (r = dalloc(&doff, (size_t)m, st)) != SC_OK)
      break;
    if (cudaMemsetAsync(cnt, 0, (size_t)m * sizeof(int64_t), st) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "memset");
      break;
    }
    const RadiusArgs rad{radius, cnt, nullptr, kRadiusSlots};
    if ((r = run_split_knn(s, dtype, train, n, d, queries, m, 0, pad_idx, pad_dist, nullptr, &rad, st)) != SC_OK) break;
    std::vector<int64_t> c((size_t)m);
    if (cudaMemcpyAsync(c.data(), cnt, (size_t)m * sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "radius counts");
      break;
    }
    std::vector<int32_t> over;
    for (int64_t q = 0; q < m; ++q) {
      off[(size_t)q + 1] = off[(size_t)q] + c[(size_t)q];
      if (c[(size_t)q] > kRadiusSlots) over.push_back((int32_t)q);
    }
    const int64_t total = off[(size_t)m];
    if (total == 0) break;
    if ((r = dalloc(&oidx, (size_t)total, st)) != SC_OK || (r = dalloc(&odist, (size_t)total, st)) != SC_OK) break;
    if (cudaMemcpyAsync(doff, off.data(), (size_t)m * sizeof(int64_t), cudaMemcpyHostToDevice, st) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "radius offsets");
      break;
    }
    pack_radius_kernel<<<(int)((m * 32 + 255) / 256), 256, 0, st>>>(pad_idx, pad_dist, kRadiusSlots, cnt, doff, m,
                                                                     oidx, odist);
    if (cudaGetLastError() != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "pack_radius_kernel"); break; }
    note_launch();
    if (!over.empty()) {  // their whole lists, written at their offsets
      const int64_t no = (int64_t)over.size();
      const size_t es = dtype == SC_F32 ? 4 : 8;
      std::vector<int64_t> so((size_t)no);
      for (int64_t i = 0; i < no; ++i) so[(size_t)i] = off[(size_t)over[(size_t)i]];
      if ((r = dalloc(&sub_rows, (size_t)no, st)) != SC_OK || (r = dalloc(&sub_off, (size_t)no, st)) != SC_OK ||
          (r = dalloc(&sub_q, (size_t)no * d * es, st)) != SC_OK)
        break;
      if (cudaMemcpyAsync(sub_rows, over.data(), (size_t)no * sizeof(int32_t), cudaMemcpyHostToDevice, st) != cudaSuccess ||
          cudaMemcpyAsync(sub_off, so.data(), (size_t)no * sizeof(int64_t), cudaMemcpyHostToDevice, st) != cudaSuccess) {
        r = cuda_fail(cudaGetLastError(), "radius overflow");
        break;
      }
      const int gb = (int)((no * d + 255) / 256);
      if (dtype == SC_F32)
        gather_rows_kernel<float><<<gb, 256, 0, st>>>((const float *)queries, sub_rows, no, d, (float *)sub_q);
      else
        gather_rows_kernel<double><<<gb, 256, 0, st>>>((const double *)queries, sub_rows, no, d, (double *)sub_q);
      if (cudaGetLastError() != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "gather_rows_kernel"); break; }
      note_launch();
      const RadiusArgs fill{radius, nullptr, sub_off, 0};
      if ((r = run_split_knn(s, dtype, train, n, d, sub_q, no, 0, oidx, odist, nullptr, &fill, st)) != SC_OK) break;
      // sync before the host vectors above (copied from pageable memory) go
      if (cudaStreamSynchronize(st) != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "radius overflow"); break; }
    }
  } while (0);
  dfree(pad_idx, st); dfree(pad_dist, st); dfree(cnt, st); dfree(doff, st);
  dfree(sub_rows, st); dfree(sub_off, st); dfree(sub_q, st);
  if (r != SC_OK) {
    dfree(oidx, st);
    dfree(odist, st);
    return r;
  }
  *idx_out = oidx;
  *dist_out = odist;
  return SC_OK;
}

void split_knn_free(SplitKnnState *s, cudaStream_t st) {
  dfree(s->th, st); dfree(s->tl, st); dfree(s->tbx, st); dfree(s->tmax, st); dfree(s->ones, st);
  dfree(s->qh, st); dfree(s->ql, st); dfree(s->qnrm, st); dfree(s->qn2, st); dfree(s->evals, st);
  dfree(s->cand, st); dfree(s->count, st); dfree(s->over, st);
  s->ready = 0;
  s->m_cap = 0;
  s->cand_cap = 0;
  s->count_cap = 0;
}

}  // namespace sc
