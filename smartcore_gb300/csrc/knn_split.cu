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
constexpr int kQueue = 1024;     // per owner warp: ring of pending candidates (owner lane << 27 | row)
constexpr int kRowBits = 27;     // training rows per handle < 2^27

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

// Rows of a matrix as split-BF16 operand: halves, f32 upper bound of the norm,
// ||row||^2 rounded to f32 (+inf for padding rows) and in f64.
template <typename T>
__global__ void __launch_bounds__(256)
knn_prep_kernel(const T *__restrict__ x, int64_t n, int64_t n_pad, int d, int d_pad,
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
    xh[i * d_pad + j] = h;
    xl[i * d_pad + j] = l;
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
  // index order; counts per query (counting pass, idx_out == nullptr) or the
  // rows from offsets[q] on (filling pass)
  int radius_mode;
  double radius, r2up;  // r2up >= every D whose sqrt rounds to <= radius
  int64_t *counts;
  const int64_t *offsets;
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

// Pulls training row j toward L1 when it is queued, tiles before its exact
// distance is computed.
template <typename T>
__device__ __forceinline__ void prefetch_row(const T *train, int64_t j, int d) {
  const char *a = (const char *)(train + j * (int64_t)d);
  const char *b = a + (size_t)d * sizeof(T) - 1;
  asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
  if (((uintptr_t)a >> 7) != ((uintptr_t)b >> 7)) asm volatile("prefetch.global.L1 [%0];" ::"l"(b));
}

// Threshold on a_j below which a row may enter the heap: D_root - ||q||^2 + E,
// rounded up (a larger threshold only admits more rows to the exact test),
// in f32 with a margin of 2^-22 (D_root + ||q||^2) for the f32 roundings.
__device__ __forceinline__ float knn_threshold(double droot, double qn2, float eq) {
  if (!(droot < DBL_MAX)) return __int_as_float(0x7f800000);
  const float r = __double2float_ru(droot), qf = __double2float_rd(qn2);
  return __fadd_ru(__fadd_ru(__fsub_ru(r, qf), eq), __fmul_ru(0x1p-22f, __fadd_ru(r, qf)));
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
  const int a_bytes = 2 * p.nkt * a_blk;
  const int b_blk = TN * p.row_bytes;
  const int b_stage = 2 * p.nkt * b_blk + TN * 32;  // halves + norm-folding rows
  uint8_t *sA = base;
  uint8_t *sOnes = base + a_bytes;                   // 128 x 32 B
  uint8_t *sB = sOnes + kQM * 32;
  uint32_t *sQ = (uint32_t *)(sB + (size_t)p.stages * b_stage);  // owner warps x kQueue entries
  uint32_t *sMask = sQ + kOwnerWarps * kQueue;                   // [slot][query][word]
  float *s_lo = (float *)(sMask + kMaskSlots * kQM * kWords);    // per query: filter threshold on acc
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

  if (warp == 0) {
    if (lane == 0) {  // ---------------- TMA producer ----------------
      int it = 0, ql = 0;
      bool ok = true;
      for (int qt = blockIdx.x; ok && qt < p.n_tiles_q; qt += gridDim.x, ++ql) {
        if (!tc::mbar_wait(aempty, (uint32_t)(ql & 1) ^ 1u, kWaitNs)) { ok = false; break; }
        tc::mbar_expect_tx(afull, (uint32_t)(a_bytes + (ql == 0 ? kQM * 32 : 0)));
        for (int part = 0; part < 2; ++part)
          for (int kt = 0; kt < p.nkt; ++kt)
            tc::tma_load_2d(sA + (part * p.nkt + kt) * a_blk, part ? &tm_ql : &tm_qh, afull, kt * p.kt_elems,
                            qt * kQM);
        if (ql == 0) tc::tma_load_2d(sOnes, &tm_ones, afull, 0, 0);
        for (int tt = 0; tt < p.n_tiles_t; ++tt, ++it) {
          const int s = it % p.stages;
          const uint32_t ph = (uint32_t)(it / p.stages) & 1u;
          if (!tc::mbar_wait(&empty[s], ph ^ 1u, kWaitNs) || *(volatile int *)s_abort) { ok = false; break; }
          tc::mbar_expect_tx(&full[s], (uint32_t)b_stage);
          uint8_t *dst = sB + (size_t)s * b_stage;
          for (int part = 0; part < 2; ++part)
            for (int kt = 0; kt < p.nkt; ++kt)
              tc::tma_load_2d(dst + (part * p.nkt + kt) * b_blk, part ? &tm_tl : &tm_th, &full[s],
                              kt * p.kt_elems, tt * TN);
          tc::tma_load_2d(dst + 2 * p.nkt * b_blk, &tm_tbx, &full[s], 0, tt * TN);
        }
      }
      if (!ok) atomicExch(s_abort, 1);
      for (int j = (it > p.stages ? it - p.stages : 0); j < it; ++j)  // drain in-flight copies
        tc::mbar_wait(&full[j % p.stages], (uint32_t)(j / p.stages) & 1u, kWaitNs);
      if (ql > 0) tc::mbar_wait(afull, (uint32_t)((ql - 1) & 1), kWaitNs);
    }
  } else if (warp == 1) {
    if (lane == 0) {  // ---------------- MMA issuer ----------------
      const uint32_t idesc = tc::idesc_bf16_f32(kQM, TN);
      const uint32_t sA0 = tc::smem_u32(sA), sB0 = tc::smem_u32(sB);
      const uint64_t ones_desc = tc::smem_desc(tc::smem_u32(sOnes), 32);
      int it = 0, ql = 0;
      bool ok = true;
      for (int qt = blockIdx.x; ok && qt < p.n_tiles_q; qt += gridDim.x, ++ql) {
        if (!tc::mbar_wait(afull, (uint32_t)(ql & 1), kWaitNs)) { ok = false; break; }
        for (int tt = 0; tt < p.n_tiles_t; ++tt, ++it) {
          const int s = it % p.stages, acc = it & 1;
          const uint32_t ph = (uint32_t)(it / p.stages) & 1u, aph = (uint32_t)(it >> 1) & 1u;
          if (!tc::mbar_wait(&accempty[acc], aph ^ 1u, kWaitNs) || !tc::mbar_wait(&full[s], ph, kWaitNs) ||
              *(volatile int *)s_abort) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t d_tmem = tmem + (uint32_t)(acc * TN);
          const uint32_t b0 = sB0 + (uint32_t)(s * b_stage);
          // -||t||^2 / 2 first, then q_h.t_h + q_h.t_l + q_l.t_h
          tc::mma_f16(d_tmem, ones_desc, tc::smem_desc(b0 + (uint32_t)(2 * p.nkt * b_blk), 32), idesc, 0u);
          for (int prod = 0; prod < 3; ++prod) {
            const int pa = prod == 2 ? 1 : 0, pb = prod == 1 ? 1 : 0;
            for (int kt = 0; kt < p.nkt; ++kt)
              for (int ks = 0; ks < p.kt_elems / 16; ++ks) {
                const uint64_t ad = tc::smem_desc(sA0 + (uint32_t)((pa * p.nkt + kt) * a_blk + ks * 32), p.row_bytes);
                const uint64_t bd = tc::smem_desc(b0 + (uint32_t)((pb * p.nkt + kt) * b_blk + ks * 32), p.row_bytes);
                tc::mma_f16(d_tmem, ad, bd, idesc, 1u);
              }
          }
          tc::mma_commit(&empty[s]);
          tc::mma_commit(&accfull[acc]);
        }
        tc::mma_commit(aempty);  // the query tile's smem is free once these MMAs complete
      }
      if (!ok) atomicExch(s_abort, 1);
      tc::mma_commit(mma_done);
      tc::mbar_wait(mma_done, 0, kWaitNs);
    }
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
      const double qn2 = live ? p.qn2[q] : 0.0;
      // |a_j - (D_j - ||q||^2)| <= e, a_j = -2 acc_j (see split.cu for the terms)
      const float eq = 1.05f * (2.f * (p.coef_xc * qn * tmax + p.coef_cc * tmax * tmax) +
                                p.coef_ref * (qn + tmax) * (qn + tmax)) + 1e-30f;
      // row j can enter only if acc_j >= lo = -thr / 2 (thr = root^2 - ||q||^2 + e)
      float lo = live ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000);
      s_lo[row] = lo;
      int64_t rc = 0, rpos = p.radius_mode && p.idx_out && live ? p.offsets[q] : 0;  // find_radius
      uint32_t qhead = 0, qtail = 0;  // warp-uniform queue cursors
      const int64_t qbase = (int64_t)qt * kQM + lq * 32;
      // one round: exact distances of up to 32 queued entries, then the owners' heap steps
      auto round = [&](uint32_t cnt) {
        const uint32_t e = (uint32_t)lane < cnt ? Q[(qhead + lane) & (kQueue - 1)] : 0u;
        const int owner = (int)(e >> kRowBits);
        const int64_t j = (int64_t)(e & ((1u << kRowBits) - 1u));
        double sq = __longlong_as_double(0x7ff0000000000000ll);
        if ((uint32_t)lane < cnt && qbase + owner < p.m) {
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
              if (p.idx_out) {
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
            lo = -0.5f * knn_threshold(hD[0], qn2, eq);
          }
        }
        __syncwarp();
        qhead += cnt;
        evals += (uint32_t)lane < cnt ? 1u : 0u;
        __syncwarp();
      };
      for (int tt = 0; tt < p.n_tiles_t; ++tt, ++it) {
        const int slot = it % kMaskSlots;
        const bool got = tc::mbar_wait(&maskfull[slot], (uint32_t)(it / kMaskSlots) & 1u, kWaitNs);
        if (!__all_sync(0xffffffffu, got) || __any_sync(0xffffffffu, *(volatile int *)s_abort != 0)) {
          atomicExch(s_abort, 1);
          stop = true;
          break;
        }
        const uint32_t *mrow = sMask + ((size_t)slot * kQM + row) * kWords;
        const int64_t j0 = (int64_t)tt * TN;
        uint32_t mw[kWords], mcnt = 0u;
#pragma unroll
        for (int w = 0; w < kWords; ++w) {
          mw[w] = mrow[w];
          mcnt += __popc(mw[w]);
        }
        const uint32_t mtotal = __reduce_add_sync(0xffffffffu, mcnt);
        if (mtotal != 0u && mtotal <= (uint32_t)(kQueue - 32)) {
          // the whole tile at once: one scan, entries in index order per owner
          uint32_t incl = mcnt;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          uint32_t pos = qtail + incl - mcnt;
#pragma unroll
          for (int w = 0; w < kWords; ++w)
            for (uint32_t m = mw[w]; m; m &= m - 1) {
              const int64_t jr = j0 + 32 * w + __ffs(m) - 1;
              prefetch_row(train, jr, p.d);
              Q[(pos++) & (kQueue - 1)] = ((uint32_t)lane << kRowBits) | (uint32_t)jr;
            }
          qtail += mtotal;
          __syncwarp();
          while (qtail - qhead >= 32) round(32);
        }
#pragma unroll
        for (int w = 0; w < kWords && mtotal > (uint32_t)(kQueue - 32); ++w) {  // rare: a tile too large for the ring
          if (!__any_sync(0xffffffffu, mw[w] != 0u)) continue;
#pragma unroll
          for (int half = 0; half < 2; ++half) {  // <= 32 x 16 new entries per step: the ring never overflows
            const uint32_t mask = (mw[w] >> (16 * half)) & 0xffffu;
            const uint32_t cnt = __popc(mask);
            const uint32_t total = __reduce_add_sync(0xffffffffu, cnt);
            if (total == 0) continue;
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
              if (lane >= o) incl += y;
            }
            uint32_t pos = qtail + incl - cnt;
            for (uint32_t m = mask; m; m &= m - 1) {
              const int64_t jr = j0 + 32 * w + 16 * half + __ffs(m) - 1;
              prefetch_row(train, jr, p.d);
              Q[(pos++) & (kQueue - 1)] = ((uint32_t)lane << kRowBits) | (uint32_t)jr;
            }
            qtail += total;
            __syncwarp();
            while (qtail - qhead >= 32) round(32);
          }
        }
        s_lo[row] = lo;                     // threshold for the filters, published before the release
        tc::mbar_arrive(&maskempty[slot]);  // tile replayed (queued entries only make lo staler)
      }
      while (!stop && qtail != qhead) round(min(32u, qtail - qhead));
      if (p.radius_mode) {
        if (live && !stop && !p.idx_out) p.counts[q] = rc;
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
      for (int tt = 0; tt < p.n_tiles_t; ++tt, ++it) {
        if ((it & 1) != g) continue;
        const int slot = it % kMaskSlots;
        bool ok = tc::mbar_wait(&accfull[g], (uint32_t)(it >> 1) & 1u, kWaitNs);
        // threshold: tile 0 of a query tile admits every row; tile 1 waits for
        // the owners' replay of tile 0; later tiles use the replay of tile
        // tt - 2.  Either wait also frees this tile's mask slot.
        const bool live_q = (int64_t)qt * kQM + row < p.m;
        float lo = live_q ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000);
        if (p.radius_mode) {
          // a fixed threshold: D <= r2up; only the mask slot must be free
          if (it >= kMaskSlots) {
            const int u = it - kMaskSlots;
            ok = ok && tc::mbar_wait(&maskempty[u % kMaskSlots], (uint32_t)(u / kMaskSlots) & 1u, kWaitNs);
          }
          if (live_q) {
            const int64_t q = (int64_t)qt * kQM + row;
            const float tmax = __uint_as_float(*p.tmax);
            const float qn = p.qnrm[q];
            const float eq = 1.05f * (2.f * (p.coef_xc * qn * tmax + p.coef_cc * tmax * tmax) +
                                      p.coef_ref * (qn + tmax) * (qn + tmax)) + 1e-30f;
            lo = -0.5f * knn_threshold(p.r2up, p.qn2[q], eq);
          }
        } else if (tt >= 1) {
          const int u = it - (tt == 1 ? 1 : 2);
          ok = ok && tc::mbar_wait(&maskempty[u % kMaskSlots], (uint32_t)(u / kMaskSlots) & 1u, kWaitNs);
          lo = *(volatile float *)&s_lo[row];
        } else if (it >= kMaskSlots) {
          const int u = it - kMaskSlots;
          ok = ok && tc::mbar_wait(&maskempty[u % kMaskSlots], (uint32_t)(u / kMaskSlots) & 1u, kWaitNs);
        }
        if (!__all_sync(0xffffffffu, ok) || __any_sync(0xffffffffu, *(volatile int *)s_abort != 0)) {
          atomicExch(s_abort, 1);
          stop = true;
          break;
        }
        tc::fence_after_sync();
        const uint32_t tbase = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(g * TN);
        const uint32_t taddr = tbase + (uint32_t)c_lo;
        uint32_t *mrow = sMask + ((size_t)slot * kQM + row) * kWords + c_lo / 32;
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
#pragma unroll
        for (int c1 = 0; c1 < kCols; c1 += 64) {  // 64 columns per TMEM round trip
          uint32_t v[64];
          tc::tmem_ld64(taddr + (uint32_t)c1, v);
          tc::tmem_wait_ld();
#pragma unroll
          for (int c2 = 0; c2 < 64; c2 += 32) {
            const int c0 = c1 + c2;
            if (c_lo + c0 >= 32) lo = lo_rest;
            float mx = __uint_as_float(v[c2]);
#pragma unroll
            for (int jj = 1; jj < 32; ++jj) mx = fmaxf(mx, __uint_as_float(v[c2 + jj]));
            uint32_t mask = 0u;
            if (__any_sync(0xffffffffu, mx >= lo)) {
#pragma unroll
              for (int jj = 0; jj < 32; ++jj) mask |= (__uint_as_float(v[c2 + jj]) >= lo ? 1u : 0u) << jj;
              const int64_t rem = p.n - (j0 + c0);  // rows past the end of the training set
              if (rem < 32) mask &= rem <= 0 ? 0u : ((1u << rem) - 1u);
            }
            mrow[c0 / 32] = mask;
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

// Training rows per tile: 256 up to d = 32, then narrower so that the
// resident query tile and two or more training stages fit in shared memory.
int knn_tile_n(int d_pad) { return d_pad <= 32 ? 256 : d_pad <= 64 ? 128 : 64; }

size_t knn_smem(int nkt, int row_bytes, int stages, int tn, int heap_k) {
  return 1024 + (size_t)2 * nkt * kQM * row_bytes + kQM * 32 + (size_t)stages * (2 * nkt * tn * row_bytes + tn * 32) +
         (size_t)kOwnerWarps * kQueue * 4 + (size_t)kMaskSlots * kQM * (tn / 32) * 4 + kQM * 4 +
         (size_t)kOwnerWarps * 32 * 16 + (size_t)heap_k * kQM * 12 + 8 +
         (size_t)(2 * stages + 7 + 2 * kMaskSlots) * 8 + 16;
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
  int64_t *counts;         // counting pass (idx == nullptr)
  const int64_t *offsets;  // filling pass
};

sc_status run_split_knn(SplitKnnState *s, int dtype, const void *train, int64_t n, int d, const void *queries,
                        int64_t m, int k, int64_t *idx, double *dist, int64_t *rescored, const RadiusArgs *rad,
                        cudaStream_t st) {
  if (rescored) *rescored = 0;
  if (m == 0 || n == 0) return SC_OK;
  if (n >= ((int64_t)1 << kRowBits)) {
    set_error("n=%lld exceeds the split-BF16 kNN kernel's limit of 2^27 training rows", (long long)n);
    return SC_ERR_INVALID;
  }
  const int d_pad = knn_pad_d(d);
  const int kt_elems = d_pad >= 64 ? 64 : d_pad, nkt = d_pad / kt_elems, row_bytes = kt_elems * 2;
  const int tn = knn_tile_n(d_pad);
  // heaps in shared memory when they fit beside at least two training stages
  bool sh = knn_smem(nkt, row_bytes, 2, tn, k) <= 227 * 1024;
  const int heap_k = sh ? k : 0;
  int stages = 4;
  while (stages > 2 && knn_smem(nkt, row_bytes, stages, tn, heap_k) > 227 * 1024) --stages;
  const size_t smem = knn_smem(nkt, row_bytes, stages, tn, heap_k);
  if (d_pad > 256 || smem > 227 * 1024) {
    set_error("d=%d exceeds the split-BF16 kNN kernel's shared memory", d);
    return SC_ERR_INVALID;
  }
  int dev = 0;
  SC_CUDA(cudaGetDevice(&dev));
  if (!s->num_sms) SC_CUDA(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t n_pad = (n + tn - 1) / tn * tn;
  if (!s->ready || s->train != train || s->n != n || s->d != d) {  // training operand, once per handle
    s->ready = 0;  // until every buffer below exists
    dfree(s->th, st); dfree(s->tl, st); dfree(s->tbx, st); dfree(s->tmax, st); dfree(s->ones, st);
    SC_TRY(dalloc(&s->th, (size_t)n_pad * d_pad, st));
    SC_TRY(dalloc(&s->tl, (size_t)n_pad * d_pad, st));
    SC_TRY(dalloc(&s->tbx, (size_t)n_pad * 16, st));
    SC_TRY(dalloc(&s->tmax, 1, st));
    SC_TRY(dalloc(&s->ones, (size_t)kQM * 16, st));
    ones_tile_kernel<<<1, kQM, 0, st>>>(s->ones);
    SC_LAUNCHED();
    SC_TRY(map2d(&s->tm_ones, s->ones, kQM, 16, 16, kQM, 32));
    SC_CUDA(cudaMemsetAsync(s->tmax, 0, sizeof(unsigned int), st));
    const int nb = (int)((n_pad + 7) / 8);
    if (dtype == SC_F32)
      knn_prep_kernel<float><<<nb, 256, 0, st>>>((const float *)train, n, n_pad, d, d_pad, s->th, s->tl, nullptr,
                                                nullptr, nullptr, s->tmax, s->tbx);
    else
      knn_prep_kernel<double><<<nb, 256, 0, st>>>((const double *)train, n, n_pad, d, d_pad, s->th, s->tl,
                                                 nullptr, nullptr, nullptr, s->tmax, s->tbx);
    SC_LAUNCHED();
    SC_TRY(map2d(&s->tm_th, s->th, n_pad, d_pad, kt_elems, tn, row_bytes));
    SC_TRY(map2d(&s->tm_tl, s->tl, n_pad, d_pad, kt_elems, tn, row_bytes));
    SC_TRY(map2d(&s->tm_tbx, s->tbx, n_pad, 16, 16, tn, 32));
    s->train = train;
    s->n = n;
    s->d = d;
    s->ready = 1;
  }
  const int64_t m_pad = (m + kQM - 1) / kQM * kQM;
  if (m_pad > s->m_cap) {
    s->m_cap = 0;  // a failed allocation leaves no stale capacity
    dfree(s->qh, st); dfree(s->ql, st); dfree(s->qnrm, st); dfree(s->qn2, st);
    SC_TRY(dalloc(&s->qh, (size_t)m_pad * d_pad, st));
    SC_TRY(dalloc(&s->ql, (size_t)m_pad * d_pad, st));
    SC_TRY(dalloc(&s->qnrm, (size_t)m_pad, st));
    SC_TRY(dalloc(&s->qn2, (size_t)m_pad, st));
    s->m_cap = m_pad;
  }
  if (!s->evals) SC_TRY(dalloc(&s->evals, 2, st));
  SC_CUDA(cudaMemsetAsync(s->evals, 0, 2 * sizeof(unsigned long long), st));
  const int nbq = (int)((m_pad + 7) / 8);
  if (dtype == SC_F32)
    knn_prep_kernel<float><<<nbq, 256, 0, st>>>((const float *)queries, m, m_pad, d, d_pad, s->qh, s->ql, s->qnrm,
                                               nullptr, s->qn2, nullptr, nullptr);
  else
    knn_prep_kernel<double><<<nbq, 256, 0, st>>>((const double *)queries, m, m_pad, d, d_pad, s->qh, s->ql,
                                                s->qnrm, nullptr, s->qn2, nullptr, nullptr);
  SC_LAUNCHED();
  CUtensorMap tm_qh, tm_ql;
  SC_TRY(map2d(&tm_qh, s->qh, m_pad, d_pad, kt_elems, kQM, row_bytes));
  SC_TRY(map2d(&tm_ql, s->ql, m_pad, d_pad, kt_elems, kQM, row_bytes));
  KnnParams p;
  memset(&p, 0, sizeof p);
  p.n = n;
  p.m = m;
  p.n_tiles_t = (int)(n_pad / tn);
  p.n_tiles_q = (int)(m_pad / kQM);
  p.nkt = nkt;
  p.kt_elems = kt_elems;
  p.row_bytes = row_bytes;
  p.stages = stages;
  p.k = k;
  p.d = d;
  p.lg_d = 0;
  while ((1 << p.lg_d) < d) ++p.lg_d;
  p.qnrm = s->qnrm;
  p.qn2 = s->qn2;
  p.tmax = s->tmax;
  const double nacc = 3.0 * d_pad + 3.0;
  p.coef_xc = (float)(3.02 * 0x1p-16 + 1.02 * nacc * 0x1p-22);
  p.coef_cc = (float)(1.01 * 0x1p-25 + 0.51 * nacc * 0x1p-22);
  p.coef_ref = (float)((d + 4) * 0x1p-52);
  p.idx_out = idx;
  p.dist_out = dist;
  if (rad) {
    p.radius_mode = 1;
    p.radius = rad->radius;
    p.r2up = rad->radius * rad->radius * (1.0 + 0x1p-48);  // covers every D with sqrt(D) rounding to <= radius
    p.counts = rad->counts;
    p.offsets = rad->offsets;
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

bool split_knn_serves(int d, int k) {
  const int d_pad = knn_pad_d(d);
  if (d_pad > 256 || k > kMaxKnnK) return false;
  const int kt = d_pad >= 64 ? 64 : d_pad, nkt = d_pad / kt, rb = kt * 2, tn = knn_tile_n(d_pad);
  const bool sh = knn_smem(nkt, rb, 2, tn, k) <= 227 * 1024;
  return knn_smem(nkt, rb, 2, tn, sh ? k : 0) <= 227 * 1024;
}

sc_status split_knn(SplitKnnState *s, int dtype, const void *train, int64_t n, int d, const void *queries,
                    int64_t m, int k, int64_t *idx, double *dist, int64_t *rescored, cudaStream_t st) {
  return run_split_knn(s, dtype, train, n, d, queries, m, k, idx, dist, rescored, nullptr, st);
}

sc_status split_knn_radius(SplitKnnState *s, int dtype, const void *train, int64_t n, int d, const void *queries,
                           int64_t m, double radius, int64_t *counts, const int64_t *offsets, int64_t *idx,
                           double *dist, cudaStream_t st) {
  const RadiusArgs rad{radius, counts, offsets};
  return run_split_knn(s, dtype, train, n, d, queries, m, 0, idx, dist, nullptr, &rad, st);
}

void split_knn_free(SplitKnnState *s, cudaStream_t st) {
  dfree(s->th, st); dfree(s->tl, st); dfree(s->tbx, st); dfree(s->tmax, st); dfree(s->ones, st);
  dfree(s->qh, st); dfree(s->ql, st); dfree(s->qnrm, st); dfree(s->qn2, st); dfree(s->evals, st);
  s->ready = 0;
  s->m_cap = 0;
}

}  // namespace sc
