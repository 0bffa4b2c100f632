// Split-BF16 assignment (K5) and FP64 re-score (K6) for the Lloyd loop and
// KMeans::predict.
//
// For a point x and centroids c_j the label is argmin_j D_j, D_j the FP64
// squared distance in the reference's operation order.  ||x||^2 is common to
// every j, so the kernel ranks A_j = ||c_j||^2 - 2 x.c_j, with x.c_j from a
// tcgen05 GEMM on BF16 halves: x = x_h + x_l + r_x, c = c_h + c_l + r_c
// (|r| <= 2^-16 |.|), x.c ~ x_h.c_h + x_h.c_l + x_l.c_h, FP32 accumulate in
// TMEM.  A rigorous per-point bound E on |A_j - (D_j - ||x||^2)| certifies the
// label when the gap between the best and second-best A exceeds 2E.  Every
// other point is re-ranked with an FP32 CUDA-core dot product (a bound ~50x
// tighter), and the candidates that remain within that bound are re-scored
// in FP64 in the reference's operation order.
#include <float.h>
#include <math.h>
#include <string.h>

#include "split.cuh"
#include "splitprep.cuh"
#include "tc.cuh"

namespace sc {

namespace {

constexpr int kBM = 128;           // points per tile (UMMA M)
constexpr int kEpiWarps = 16;      // 2 accumulator buffers x 2 column halves x 4 lane quarters
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kAssignThreads = 64 + kEpiThreads;  // warp 0 TMA, warp 1 MMA, then epilogue
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s bound on every barrier wait

enum { kErrTimeout = 4 };

__device__ __forceinline__ double sqd_term(double a, double b) {
  const double r = __dsub_rn(a, b);
  return __dmul_rn(r, r);
}

// Centroid operand: BF16 halves of the f64 centroids, the norm-folding row
// (three BF16 terms of -||c||^2/2; padding rows -1e30 so they never win),
// ||c||^2 rounded to f32, an upper bound of max_j ||c_j||, and the
// centroids in f32, transposed, for the re-score.
__global__ void __launch_bounds__(128)
prep_c_kernel(const double *__restrict__ cent, int k, int d, int d_pad, int k_pad, int k_cols,
              __nv_bfloat16 *__restrict__ ch, __nv_bfloat16 *__restrict__ cl, __nv_bfloat16 *__restrict__ cbx,
              float *__restrict__ cn2, unsigned int *__restrict__ cmax, float *__restrict__ cT) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  __shared__ double ws[4];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int t = threadIdx.x; t < d_pad; t += 128) {
    __nv_bfloat16 h = __float2bfloat16_rn(0.f), l = h;
    if (j < k && t < d) {
      const double v = cent[(int64_t)j * d + t];
      split2<double>(v, h, l);
      s = fma(v, v, s);
    }
    if (j < k_pad) {
      ch[(int64_t)j * d_pad + t] = h;
      cl[(int64_t)j * d_pad + t] = l;
    }
    cT[(int64_t)t * k_cols + j] = (j < k && t < d) ? (float)cent[(int64_t)j * d + t] : 0.f;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    const double t = ws[0] + ws[1] + ws[2] + ws[3];
    __nv_bfloat16 zero = __float2bfloat16_rn(0.f), h = zero, m = zero, l = zero;
    if (j < k) {
      cn2[j] = __double2float_rn(t);
      const float r = __fsqrt_ru(__double2float_ru(t));
      atomicMax(cmax, __float_as_uint(r) + 1u);
      split3(-0.5 * t, h, m, l);
    } else {
      cn2[j] = __int_as_float(0x7f800000);  // padding: never the minimum
      h = __float2bfloat16_rn(-1e30f);
    }
    if (j < k_pad) {
      __nv_bfloat16 *row = cbx + (int64_t)j * 16;
      row[0] = h;
      row[1] = m;
      row[2] = l;
      for (int c = 3; c < 16; ++c) row[c] = zero;
    }
  }
}

// ---------------------------------------------------------------------------
// K5: persistent tcgen05 assignment kernel.
//   accumulator(m, j) = x_h.c_h + x_h.c_l + x_l.c_h  - ||c_j||^2 / 2
//                     ~ x.c_j - ||c_j||^2 / 2 = (||x||^2 - D_j) / 2,
// so the nearest centroid is the column with the largest accumulator.
// ---------------------------------------------------------------------------
struct AssignParams {
  int64_t n;
  int n_tiles;
  int nkt, kt_elems, row_bytes;
  int k, k_pad, k_cols;  // k_cols = k_pad rounded up to 32 (TMEM stride)
  int stages;
  uint32_t tmem_cols;
  const float *xnrm;
  const unsigned int *cmax;
  float coef_xc;    // accumulator error: coef_xc * ||x|| * ||c|| + coef_cc * ||c||^2
  float coef_cc;
  float coef_ref;   // reference rounding of D: <= coef_ref * (||x|| + ||c||)^2
  int32_t *labels;
  int64_t n_pad;
  int region;                // near-tie list entries reserved per CTA
  unsigned int *list_count;  // near-tie rows listed by each CTA
  int64_t *list_rows;        //   CTA b's rows at [b * region, ...)
  uint2 *cand4;              // [2 halves][n_pad]: up to 4 candidate columns of a listed row (16 bits each)
  uint8_t *cmeta;            // [2 halves][n_pad]: bits 0-3 valid columns of cand4, bit 4 list complete
  LloydState *st;
  uint64_t wait_ns;  // bound of the pipeline waits (the drains keep kWaitNs)
};

__global__ void __launch_bounds__(kAssignThreads, 1)
split_assign_kernel(const __grid_constant__ CUtensorMap tm_xh, const __grid_constant__ CUtensorMap tm_xl,
                    const __grid_constant__ CUtensorMap tm_ch, const __grid_constant__ CUtensorMap tm_cl,
                    const __grid_constant__ CUtensorMap tm_ones, const __grid_constant__ CUtensorMap tm_cbx,
                    const AssignParams p) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (p.st && p.st->done) return;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int a_blk = kBM * p.row_bytes;               // one (part, k-tile) block of a stage
  const int a_stage = 2 * p.nkt * a_blk;
  const int b_blk = p.k_pad * p.row_bytes;           // one (part, k-tile) block of B
  const int b_bytes = (2 * p.nkt * b_blk + 1023) & ~1023;
  const int x_bytes = (kBM * 32 + p.k_pad * 32 + 1023) & ~1023;  // norm-folding operands
  uint8_t *sB = base;
  uint8_t *sOnes = base + b_bytes;
  uint8_t *sBx = sOnes + kBM * 32;
  uint8_t *sA = base + b_bytes + x_bytes;
  float4 *s_xch = (float4 *)(sA + (size_t)p.stages * a_stage);  // [2 buffers][2 accumulators][2 halves][128 rows]
  uint64_t *bars = (uint64_t *)(s_xch + 8 * kBM);
  uint64_t *full = bars, *empty = bars + p.stages, *bfull = bars + 2 * p.stages;
  uint64_t *accfull = bfull + 1, *accempty = bfull + 3, *mma_done = bfull + 5;
  uint32_t *s_tmem = (uint32_t *)(bfull + 6);
  int *s_abort = (int *)(s_tmem + 1);
  unsigned int *s_nlist = (unsigned int *)(s_abort + 1);  // near-tie rows listed by this CTA

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < p.stages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(bfull, 1);
    tc::mbar_init(mma_done, 1);
    for (int a = 0; a < 2; ++a) {
      tc::mbar_init(&accfull[a], 1);
      tc::mbar_init(&accempty[a], kEpiThreads / 2);  // both column halves of the buffer
    }
    *s_abort = 0;
    *s_nlist = 0u;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tm_xh);
    tc::prefetch_tmap(&tm_xl);
    tc::prefetch_tmap(&tm_ch);
    tc::prefetch_tmap(&tm_cl);
    tc::prefetch_tmap(&tm_ones);
    tc::prefetch_tmap(&tm_cbx);
  }
  if (warp == 1) {
    tc::tmem_alloc(s_tmem, p.tmem_cols);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *s_tmem;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      tc::mbar_expect_tx(bfull, (uint32_t)(2 * p.nkt * b_blk + kBM * 32 + p.k_pad * 32));
      for (int part = 0; part < 2; ++part)
        for (int kt = 0; kt < p.nkt; ++kt)
          tc::tma_load_2d(sB + (part * p.nkt + kt) * b_blk, part ? &tm_cl : &tm_ch, bfull, kt * p.kt_elems, 0);
      tc::tma_load_2d(sOnes, &tm_ones, bfull, 0, 0);
      tc::tma_load_2d(sBx, &tm_cbx, bfull, 0, 0);
      int it = 0;
      for (int t = blockIdx.x; t < p.n_tiles; t += gridDim.x, ++it) {
        const int s = it % p.stages;
        const uint32_t ph = (uint32_t)(it / p.stages) & 1u;
        if (!tc::mbar_wait(&empty[s], ph ^ 1u, p.wait_ns)) { atomicExch(s_abort, 1); break; }
        if (*(volatile int *)s_abort) break;
        tc::mbar_expect_tx(&full[s], (uint32_t)a_stage);
        uint8_t *dst = sA + (size_t)s * a_stage;
        for (int part = 0; part < 2; ++part)
          for (int kt = 0; kt < p.nkt; ++kt)
            tc::tma_load_2d(dst + (part * p.nkt + kt) * a_blk, part ? &tm_xl : &tm_xh, &full[s],
                            kt * p.kt_elems, t * kBM);
      }
      // drain: every issued stage must land before the CTA may exit
      const int issued = it;
      for (int j = (issued > p.stages ? issued - p.stages : 0); j < issued; ++j)
        tc::mbar_wait(&full[j % p.stages], (uint32_t)(j / p.stages) & 1u, kWaitNs);
      tc::mbar_wait(bfull, 0, kWaitNs);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_bf16_f32(kBM, p.k_pad);
      bool ok = tc::mbar_wait(bfull, 0, p.wait_ns);
      const uint32_t sA0 = tc::smem_u32(sA), sB0 = tc::smem_u32(sB);
      const uint64_t ones_desc = tc::smem_desc(tc::smem_u32(sOnes), 32);
      const uint64_t bx_desc = tc::smem_desc(tc::smem_u32(sBx), 32);
      int it = 0;
      for (int t = blockIdx.x; ok && t < p.n_tiles; t += gridDim.x, ++it) {
        const int s = it % p.stages, acc = it & 1;
        const uint32_t ph = (uint32_t)(it / p.stages) & 1u, aph = (uint32_t)(it >> 1) & 1u;
        if (!tc::mbar_wait(&accempty[acc], aph ^ 1u, p.wait_ns) || !tc::mbar_wait(&full[s], ph, p.wait_ns)) {
          ok = false;
          break;
        }
        if (*(volatile int *)s_abort) { ok = false; break; }
        tc::fence_after_sync();
        const uint32_t d_tmem = tmem + (uint32_t)(acc * p.k_cols);
        const uint32_t a0 = sA0 + (uint32_t)(s * a_stage);
        // -||c||^2 / 2 first, then x_h.c_h + x_h.c_l + x_l.c_h
        tc::mma_f16(d_tmem, ones_desc, bx_desc, idesc, 0u);
        for (int prod = 0; prod < 3; ++prod) {
          const int pa = prod == 2 ? 1 : 0, pb = prod == 1 ? 1 : 0;
          for (int kt = 0; kt < p.nkt; ++kt)
            for (int ks = 0; ks < p.kt_elems / 16; ++ks) {
              const uint64_t ad = tc::smem_desc(a0 + (uint32_t)((pa * p.nkt + kt) * a_blk + ks * 32), p.row_bytes);
              const uint64_t bd = tc::smem_desc(sB0 + (uint32_t)((pb * p.nkt + kt) * b_blk + ks * 32), p.row_bytes);
              tc::mma_f16(d_tmem, ad, bd, idesc, 1u);
            }
        }
        tc::mma_commit(&empty[s]);
        tc::mma_commit(&accfull[acc]);
      }
      if (!ok) atomicExch(s_abort, 1);
      // every MMA of this CTA must be complete before TMEM is released
      tc::mma_commit(mma_done);
      tc::mbar_wait(mma_done, 0, kWaitNs);
    }
  } else {
    // ---------------- epilogue: 4 warpgroups ----------------
    // Warpgroup (g, h) handles the tiles of accumulator buffer g (every
    // other tile) and the column half h; warp w reads TMEM lanes 32*(w%4)..,
    // one point per thread.  Four interleaved (best, second, argmax) trackers
    // per thread; the two halves of a row meet in shared memory behind a
    // 64-thread named barrier, merged with the lowest index winning ties.
    const int ew = warp - 2;
    const int g = ew >> 3, h = (ew >> 2) & 1, q = warp & 3;
    const int row = q * 32 + lane;
    const uint32_t bar_id = 1u + (uint32_t)(g * 4 + q);
    const int split = ((p.k_pad / 2) + 15) & ~15;
    const int c_lo = h ? split : 0, c_hi = h ? p.k_pad : split;
    const float cmax = __uint_as_float(*p.cmax);
    const float ninf = -__int_as_float(0x7f800000);
    int it = 0;
    for (int t = blockIdx.x; t < p.n_tiles; t += gridDim.x, ++it) {
      if ((it & 1) != g) continue;
      const int64_t i = (int64_t)t * kBM + row;
      const bool live = i < p.n;
      const float xn = live ? __ldg(p.xnrm + i) : 0.f;
      const uint32_t aph = (uint32_t)(it >> 1) & 1u;
      const bool got = tc::mbar_wait(&accfull[g], aph, p.wait_ns);
      if (tc::bar_red_or(!got || *(volatile int *)s_abort != 0, bar_id, 64)) {  // uniform over the pair
        atomicExch(s_abort, 1);
        break;
      }
      tc::fence_after_sync();
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(g * p.k_cols);
      float m1[4] = {ninf, ninf, ninf, ninf}, m2[4] = {ninf, ninf, ninf, ninf};
      int mi[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
      for (int c0 = c_lo; c0 < c_hi;) {
        uint32_t v[64];
        int nc;
        if (c0 + 64 <= c_hi) {
          tc::tmem_ld64(taddr + (uint32_t)c0, v);
          nc = 64;
        } else if (c0 + 32 <= c_hi) {
          tc::tmem_ld32(taddr + (uint32_t)c0, *reinterpret_cast<uint32_t (*)[32]>(v));
          nc = 32;
        } else {
          tc::tmem_ld16(taddr + (uint32_t)c0, *reinterpret_cast<uint32_t (*)[16]>(v));
          nc = 16;
        }
        tc::tmem_wait_ld();
#pragma unroll
        for (int jj = 0; jj < 64; jj += 4) {
          if (jj >= nc) break;
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const float x = __uint_as_float(v[jj + r]);
            const bool gt = x > m1[r];
            m2[r] = gt ? m1[r] : fmaxf(m2[r], x);
            mi[r] = gt ? c0 + jj + r : mi[r];
            m1[r] = gt ? x : m1[r];
          }
        }
        c0 += nc;
      }
      tc::fence_before_sync();
      tc::mbar_arrive(&accempty[g]);
      // merge the four trackers: largest value, lowest index on ties
      float mm1 = m1[0], mm2 = m2[0];
      int a = mi[0];
#pragma unroll
      for (int r = 1; r < 4; ++r) {
        if (m1[r] > mm1 || (m1[r] == mm1 && mi[r] < a)) {
          mm2 = fmaxf(mm1, m2[r]);
          mm1 = m1[r];
          a = mi[r];
        } else {
          mm2 = fmaxf(mm2, m1[r]);
        }
        mm2 = fmaxf(mm2, m2[r]);
      }
      // the two halves of the row meet in shared memory; both merge them in
      // column order (lower half first), so both reach the same decision
      float4 *xs = s_xch + (((it >> 1) & 1) * 2 + g) * 2 * kBM;
      xs[h * kBM + row] = make_float4(mm1, mm2, __int_as_float(a), 0.f);
      tc::bar_sync(bar_id, 64);
      const float4 o = xs[(h ^ 1) * kBM + row];
      float b1 = h ? o.x : mm1, b2 = h ? o.y : mm2;
      int ba = h ? __float_as_int(o.z) : a;
      {
        const float u1 = h ? mm1 : o.x, u2 = h ? mm2 : o.y;
        const int ua = h ? a : __float_as_int(o.z);
        if (u1 > b1 || (u1 == b1 && ua < ba)) {
          b2 = fmaxf(b1, u2);
          b1 = u1;
          ba = ua;
        } else {
          b2 = fmaxf(b2, u1);
        }
        b2 = fmaxf(b2, u2);
      }
      // |acc_j - (x.c_j - ||c_j||^2/2)| <= E_acc, and D_j = ||x||^2 - 2 (x.c_j - ||c_j||^2/2)
      // up to the reference's own rounding: the label is certain when the
      // best and second-best D differ by more than 2 (2 E_acc + E_ref).
      // Otherwise the reference's minimum is among the columns whose score
      // is within 2 E_acc + E_ref of the best (margin 1.05): the candidates.
      const float e_acc = p.coef_xc * xn * cmax + p.coef_cc * cmax * cmax;
      const float e = 2.f * e_acc + p.coef_ref * (xn + cmax) * (xn + cmax) + 1e-30f;
      const bool flagged = live && !(2.f * (b1 - b2) > 2.1f * e);
      if (h == 0) {
        if (live) p.labels[i] = ba == 0x7fffffff ? 0 : ba;
        const uint32_t fm = __ballot_sync(0xffffffffu, flagged);
        if (fm) {
          unsigned int first = 0;
          if (lane == 0) first = atomicAdd(s_nlist, (unsigned int)__popc(fm));
          first = __shfl_sync(0xffffffffu, first, 0);
          if (flagged)
            p.list_rows[(int64_t)blockIdx.x * p.region + first + __popc(fm & ((1u << lane) - 1u))] = i;
        }
      }
      if (flagged) {
        // Tracker r saw this half's columns c with (c - c_lo) = r (mod 4).  When
        // its second value is below the threshold, only its maximum can be a
        // candidate; when every tracker's is, the maxima above the threshold
        // are this half's complete candidate list.
        const float thr = b1 - 1.05f * e;
        uint32_t cw[2] = {0u, 0u}, meta = 16u;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          if (m1[r] >= thr) { cw[r >> 1] |= (uint32_t)mi[r] << (16 * (r & 1)); meta |= 1u << r; }
          if (m2[r] >= thr) meta &= ~16u;
        }
        p.cand4[(size_t)h * p.n_pad + i] = make_uint2(cw[0], cw[1]);
        p.cmeta[(size_t)h * p.n_pad + i] = (uint8_t)meta;
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, p.tmem_cols);
  }
  if (threadIdx.x == 0) p.list_count[blockIdx.x] = *s_nlist;
  if (threadIdx.x == 0 && *s_abort && p.st) {
    // the step is void: the kernels after this one return at once
    atomicExch(&p.st->err, kErrTimeout);
    atomicExch(&p.st->done, 1);
  }
}

// ---------------------------------------------------------------------------
// K5b: assignment for many centroids (k_pad > 256, or centroids too large to
// stay resident).  The point tile (both BF16 halves) stays in shared memory
// while the centroids stream through a TMA ring in blocks of kWN; two TMEM
// accumulators alternate between blocks, and epilogue warpgroup g (4 warps,
// one row per thread) folds blocks b = g (mod 2) into its four trackers.  At
// the end of a tile the two warpgroups merge their trackers and hand near
// ties over exactly as split_assign_kernel's column halves do.
// ---------------------------------------------------------------------------
constexpr int kWN = 128;  // centroids per block (UMMA N)
constexpr int kWideThreads = 64 + 32 * 8;

__global__ void __launch_bounds__(kWideThreads, 1)
split_wide_kernel(const __grid_constant__ CUtensorMap tm_xh, const __grid_constant__ CUtensorMap tm_xl,
                  const __grid_constant__ CUtensorMap tm_ch, const __grid_constant__ CUtensorMap tm_cl,
                  const __grid_constant__ CUtensorMap tm_ones, const __grid_constant__ CUtensorMap tm_cbx,
                  const AssignParams p) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (p.st && p.st->done) return;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int nblk = p.k_pad / kWN;
  const int a_blk = kBM * p.row_bytes;   // one (part, k-tile) block of the point tile
  const int a_bytes = 2 * p.nkt * a_blk;
  const int b_blk = kWN * p.row_bytes;  // one (part, k-tile) block of a centroid block
  const int b_stage = (2 * p.nkt * b_blk + kWN * 32 + 1023) & ~1023;
  uint8_t *sA = base;
  uint8_t *sOnes = sA + a_bytes;
  uint8_t *sB = sOnes + 4096;
  float *s_xch = (float *)(sB + (size_t)p.stages * b_stage);  // [2 warpgroups][128 rows][12]
  uint64_t *bars = (uint64_t *)(s_xch + 2 * kBM * 12);
  uint64_t *bfull = bars, *bempty = bars + p.stages, *afull = bars + 2 * p.stages;
  uint64_t *aempty = afull + 1, *accfull = afull + 2, *accempty = afull + 4, *mma_done = afull + 6;
  uint32_t *s_tmem = (uint32_t *)(afull + 7);
  int *s_abort = (int *)(s_tmem + 1);
  unsigned int *s_nlist = (unsigned int *)(s_abort + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < p.stages; ++s) {
      tc::mbar_init(&bfull[s], 1);
      tc::mbar_init(&bempty[s], 1);
    }
    tc::mbar_init(afull, 1);
    tc::mbar_init(aempty, 1);
    tc::mbar_init(mma_done, 1);
    for (int a = 0; a < 2; ++a) {
      tc::mbar_init(&accfull[a], 1);
      tc::mbar_init(&accempty[a], 128);  // one warpgroup
    }
    *s_abort = 0;
    *s_nlist = 0u;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tm_xh);
    tc::prefetch_tmap(&tm_xl);
    tc::prefetch_tmap(&tm_ch);
    tc::prefetch_tmap(&tm_cl);
    tc::prefetch_tmap(&tm_ones);
    tc::prefetch_tmap(&tm_cbx);
  }
  if (warp == 1) {
    tc::tmem_alloc(s_tmem, 2 * kWN);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *s_tmem;

  if (warp == 0) {
    if (lane == 0) {  // ---------------- TMA producer ----------------
      int it = 0, ti = 0;
      bool ok = true;
      for (int t = blockIdx.x; ok && t < p.n_tiles; t += gridDim.x, ++ti) {
        if (!tc::mbar_wait(aempty, (uint32_t)(ti & 1) ^ 1u, kWaitNs)) { ok = false; break; }
        tc::mbar_expect_tx(afull, (uint32_t)(a_bytes + (ti == 0 ? kBM * 32 : 0)));
        for (int part = 0; part < 2; ++part)
          for (int kt = 0; kt < p.nkt; ++kt)
            tc::tma_load_2d(sA + (part * p.nkt + kt) * a_blk, part ? &tm_xl : &tm_xh, afull, kt * p.kt_elems,
                            t * kBM);
        if (ti == 0) tc::tma_load_2d(sOnes, &tm_ones, afull, 0, 0);
        for (int b = 0; b < nblk; ++b, ++it) {
          const int s = it % p.stages;
          const uint32_t ph = (uint32_t)(it / p.stages) & 1u;
          if (!tc::mbar_wait(&bempty[s], ph ^ 1u, kWaitNs) || *(volatile int *)s_abort) { ok = false; break; }
          tc::mbar_expect_tx(&bfull[s], (uint32_t)(2 * p.nkt * b_blk + kWN * 32));
          uint8_t *dst = sB + (size_t)s * b_stage;
          for (int part = 0; part < 2; ++part)
            for (int kt = 0; kt < p.nkt; ++kt)
              tc::tma_load_2d(dst + (part * p.nkt + kt) * b_blk, part ? &tm_cl : &tm_ch, &bfull[s],
                              kt * p.kt_elems, b * kWN);
          tc::tma_load_2d(dst + 2 * p.nkt * b_blk, &tm_cbx, &bfull[s], 0, b * kWN);
        }
      }
      if (!ok) atomicExch(s_abort, 1);
      for (int j = (it > p.stages ? it - p.stages : 0); j < it; ++j)  // drain in-flight copies
        tc::mbar_wait(&bfull[j % p.stages], (uint32_t)(j / p.stages) & 1u, kWaitNs);
      if (ti > 0) tc::mbar_wait(afull, (uint32_t)((ti - 1) & 1), kWaitNs);
    }
  } else if (warp == 1) {
    if (lane == 0) {  // ---------------- MMA issuer ----------------
      const uint32_t idesc = tc::idesc_bf16_f32(kBM, kWN);
      const uint32_t sA0 = tc::smem_u32(sA), sB0 = tc::smem_u32(sB);
      const uint64_t ones_desc = tc::smem_desc(tc::smem_u32(sOnes), 32);
      int it = 0, ti = 0;
      bool ok = true;
      for (int t = blockIdx.x; ok && t < p.n_tiles; t += gridDim.x, ++ti) {
        if (!tc::mbar_wait(afull, (uint32_t)(ti & 1), kWaitNs)) { ok = false; break; }
        for (int b = 0; b < nblk; ++b, ++it) {
          const int s = it % p.stages, acc = it & 1;
          const uint32_t ph = (uint32_t)(it / p.stages) & 1u, aph = (uint32_t)(it >> 1) & 1u;
          if (!tc::mbar_wait(&accempty[acc], aph ^ 1u, kWaitNs) || !tc::mbar_wait(&bfull[s], ph, kWaitNs) ||
              *(volatile int *)s_abort) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t d_tmem = tmem + (uint32_t)(acc * kWN);
          const uint32_t b0 = sB0 + (uint32_t)(s * b_stage);
          // -||c||^2 / 2 first, then x_h.c_h + x_h.c_l + x_l.c_h
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
          tc::mma_commit(&bempty[s]);
          tc::mma_commit(&accfull[acc]);
        }
        if (!ok) break;
        tc::mma_commit(aempty);  // the point tile's smem is free once these MMAs complete
      }
      if (!ok) atomicExch(s_abort, 1);
      tc::mma_commit(mma_done);
      tc::mbar_wait(mma_done, 0, kWaitNs);
    }
  } else {
    // ---------------- epilogue: 2 warpgroups x 4 lane quarters ----------------
    const int g = (warp - 2) >> 2, lq = warp & 3;
    const int row = lq * 32 + lane;
    const uint32_t bar_id = 1u + (uint32_t)lq;  // the two warps of this lane quarter
    const float cmax = __uint_as_float(*p.cmax);
    const float ninf = -__int_as_float(0x7f800000);
    int it = 0;
    for (int t = blockIdx.x; t < p.n_tiles; t += gridDim.x) {
      const int64_t i = (int64_t)t * kBM + row;
      const bool live = i < p.n;
      const float xn = live ? __ldg(p.xnrm + i) : 0.f;
      float m1[4] = {ninf, ninf, ninf, ninf}, m2[4] = {ninf, ninf, ninf, ninf};
      int mi[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
      bool stop = false;
      for (int b = 0; b < nblk; ++b, ++it) {
        if ((it & 1) != g || stop) continue;
        const bool got = tc::mbar_wait(&accfull[g], (uint32_t)(it >> 1) & 1u, kWaitNs);
        if (!__all_sync(0xffffffffu, got) || __any_sync(0xffffffffu, *(volatile int *)s_abort != 0)) {
          atomicExch(s_abort, 1);
          stop = true;
          continue;
        }
        tc::fence_after_sync();
        const uint32_t taddr = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(g * kWN);
#pragma unroll
        for (int c1 = 0; c1 < kWN; c1 += 64) {
          uint32_t v[64];
          tc::tmem_ld64(taddr + (uint32_t)c1, v);
          tc::tmem_wait_ld();
#pragma unroll
          for (int jj = 0; jj < 64; jj += 4) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              const float x = __uint_as_float(v[jj + r]);
              const bool gt = x > m1[r];
              m2[r] = gt ? m1[r] : fmaxf(m2[r], x);
              mi[r] = gt ? b * kWN + c1 + jj + r : mi[r];
              m1[r] = gt ? x : m1[r];
            }
          }
        }
        tc::fence_before_sync();
        tc::mbar_arrive(&accempty[g]);
      }
      // merge the two warpgroups' trackers (warpgroup 0's first, in both)
      float *mine = s_xch + ((size_t)g * kBM + row) * 12;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        mine[r] = m1[r];
        mine[4 + r] = m2[r];
        mine[8 + r] = __int_as_float(mi[r]);
      }
      if (tc::bar_red_or(stop || *(volatile int *)s_abort != 0, bar_id, 64)) break;  // uniform over the pair
      const float *w0 = s_xch + (size_t)row * 12, *w1 = s_xch + ((size_t)kBM + row) * 12;
      float b1 = w0[0], b2 = w0[4];
      int ba = __float_as_int(w0[8]);
#pragma unroll
      for (int r = 1; r < 8; ++r) {
        const float *src = r < 4 ? w0 : w1;
        const float u1 = src[r & 3], u2 = src[4 + (r & 3)];
        const int ua = __float_as_int(src[8 + (r & 3)]);
        if (u1 > b1 || (u1 == b1 && ua < ba)) {
          b2 = fmaxf(b1, u2);
          b1 = u1;
          ba = ua;
        } else {
          b2 = fmaxf(b2, u1);
        }
        b2 = fmaxf(b2, u2);
      }
      tc::bar_sync(bar_id, 64);  // both have read the exchange before the next tile writes it
      // certification and near-tie hand-over: as in split_assign_kernel
      const float e_acc = p.coef_xc * xn * cmax + p.coef_cc * cmax * cmax;
      const float e = 2.f * e_acc + p.coef_ref * (xn + cmax) * (xn + cmax) + 1e-30f;
      const bool flagged = live && !(2.f * (b1 - b2) > 2.1f * e);
      if (g == 0) {
        if (live) p.labels[i] = ba == 0x7fffffff ? 0 : ba;
        const uint32_t fm = __ballot_sync(0xffffffffu, flagged);
        if (fm) {
          unsigned int first = 0;
          if (lane == 0) first = atomicAdd(s_nlist, (unsigned int)__popc(fm));
          first = __shfl_sync(0xffffffffu, first, 0);
          if (flagged)
            p.list_rows[(int64_t)blockIdx.x * p.region + first + __popc(fm & ((1u << lane) - 1u))] = i;
        }
      }
      if (flagged) {
        const float thr = b1 - 1.05f * e;
        uint32_t cw[2] = {0u, 0u}, meta = 16u;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          if (m1[r] >= thr) { cw[r >> 1] |= (uint32_t)mi[r] << (16 * (r & 1)); meta |= 1u << r; }
          if (m2[r] >= thr) meta &= ~16u;
        }
        p.cand4[(size_t)g * p.n_pad + i] = make_uint2(cw[0], cw[1]);
        p.cmeta[(size_t)g * p.n_pad + i] = (uint8_t)meta;
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 2 * kWN);
  }
  if (threadIdx.x == 0) {
    p.list_count[blockIdx.x] = *s_nlist;
    if (*s_abort && p.st) atomicExch(&p.st->err, kErrTimeout);
  }
}

// ---------------------------------------------------------------------------
// K6: re-score of the near-tie rows the assignment kernel listed.  Block b
// takes CTA b's list in passes of up to kRsRows rows:
//   1. a_j = ||c_j||^2 - 2 x.c_j with FP32 CUDA-core dot products and the
//      rigorous bound e32 (error of the f32 conversions, the FMA chain and the
//      reference's own rounding of D), for the row's listed candidates (8
//      threads per row) or, when a list is not complete, for every centroid
//      (register-tiled: warp = 2 rows, lane = 8 centroids).
//   2. Survivors: a_j <= min_j a_j + 2 e32.  One survivor is the label.
//   3. Otherwise every (row, survivor) pair gets its own thread: D_j in FP64
//      in the reference order (kmeans.rs:338-346, bbd_tree.rs:101-111); per
//      row the minimum, lowest index on ties, is the label.
// ---------------------------------------------------------------------------
constexpr int kRsRows = 128;      // listed rows per pass
constexpr int kRsThreads = 1024;  // 8 threads per row in the listed pass
constexpr int kRsPairs = 1024;    // pairs held per pass (more: one row at a time)

template <typename T>
__device__ __forceinline__ double exact_sqd(const T *__restrict__ xr, const double *__restrict__ cj, int d) {
  double s = 0.0;
  for (int t = 0; t < d; ++t) s = __dadd_rn(s, sqd_term((double)xr[t], cj[t]));
  return s;
}

// Column of the u-th set bit (ascending) of a mask of `words` words.
__device__ __forceinline__ int nth_candidate(const uint32_t *mask, int words, int u) {
  for (int m = 0; m < words; ++m) {
    uint32_t b = mask[m];
    const int c = __popc(b);
    if (u < c) {
      for (int q = 0; q < u; ++q) b &= b - 1u;
      return 32 * m + __ffs(b) - 1;
    }
    u -= c;
  }
  return 0;
}

__device__ __forceinline__ float e32_bound(float xn, float cmax, int d) {
  return 1.05f * ((2.f * d + 8.f) * 0x1p-24f * xn * cmax + 0x1p-23f * (cmax * cmax + 2.f * xn * cmax) +
                  (float)((d + 4) * 0x1p-52) * (xn + cmax) * (xn + cmax)) + 1e-30f;
}

template <typename T>
__global__ void __launch_bounds__(kRsThreads, 1)
rescore_kernel(const T *__restrict__ x, int d, const double *__restrict__ cent, int k, int k_cols,
               const float *__restrict__ cT, const float *__restrict__ cn2,
               const unsigned int *__restrict__ cmax_bits, const float *__restrict__ xnrm,
               const int64_t *__restrict__ list_rows, const unsigned int *__restrict__ list_count, int region,
               const uint2 *__restrict__ cand4, const uint8_t *__restrict__ cmeta, int64_t n_pad,
               int32_t *__restrict__ labels, LloydState *st, int stage_ct) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (st && st->done) return;
  // dynamic: [d x k_cols centroids^T when stage_ct] [d x kRsRows rows^T] [kRsRows x mw survivor masks]
  extern __shared__ __align__(16) float dyn[];
  __shared__ int64_t s_row[kRsRows];
  __shared__ int s_cnt[kRsRows];           // survivors per row (0: resolved)
  __shared__ int s_pre[kRsRows + 1];
  __shared__ int s_full[kRsRows];          // rows whose candidate list is not complete
  __shared__ int s_nfull;
  __shared__ double q_s[kRsPairs];
  __shared__ int16_t q_j[kRsPairs];
  __shared__ unsigned long long s_best;
  __shared__ int s_bj;
  const unsigned int total = list_count[blockIdx.x];
  if (total == 0) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float *xs = dyn + (stage_ct ? d * k_cols : 0);  // xs[t * kRsRows + r]
  const int mw = k_cols >> 5;                      // mask words per row
  uint32_t *s_mask = (uint32_t *)(xs + d * kRsRows);  // s_mask[r * mw + word]
  if (stage_ct) {
    const int n_ct = d * k_cols;
    for (int t = threadIdx.x; t < n_ct; t += kRsThreads) dyn[t] = cT[t];
    cT = dyn;
  }
  const float cmax = __uint_as_float(*cmax_bits);
  const int64_t *rows = list_rows + (int64_t)blockIdx.x * region;
  for (unsigned int base = 0; base < total; base += kRsRows) {
    const int nr = (int)min((unsigned int)kRsRows, total - base);
    if (threadIdx.x < kRsRows) {
      const int r = threadIdx.x;
      s_cnt[r] = 0;
      if (r < nr) s_row[r] = rows[base + r];
    }
    for (int e = threadIdx.x; e < kRsRows * mw; e += kRsThreads) s_mask[e] = 0u;
    if (threadIdx.x == 0) s_nfull = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < kRsRows * d; e += kRsThreads) {
      const int r = e / d, t = e - r * d;
      xs[t * kRsRows + r] = r < nr ? (float)x[s_row[r] * (int64_t)d + t] : 0.f;
    }
    if (threadIdx.x < nr) {
      const int64_t i = s_row[threadIdx.x];
      if (!(cmeta[i] & cmeta[n_pad + i] & 16u)) s_full[atomicAdd(&s_nfull, 1)] = threadIdx.x;
    }
    __syncthreads();
    // ---- listed candidates: 8 threads per row (u = half * 4 + tracker)
    {
      const int r = threadIdx.x >> 3, u = threadIdx.x & 7;
      const int64_t i = r < nr ? s_row[r] : 0;
      const bool listed = r < nr && (cmeta[i] & cmeta[n_pad + i] & 16u);  // uniform over the 8 threads
      int j = -1;
      float a = __int_as_float(0x7f800000);
      if (listed && ((cmeta[(size_t)(u >> 2) * n_pad + i] >> (u & 3)) & 1u)) {
        const uint2 cw = cand4[(size_t)(u >> 2) * n_pad + i];
        j = (int)((((u & 2) ? cw.y : cw.x) >> (16 * (u & 1))) & 0xffffu);
        float dot = 0.f;
        for (int t = 0; t < d; ++t) dot = fmaf(xs[t * kRsRows + r], cT[(int64_t)t * k_cols + j], dot);
        a = fmaf(-2.f, dot, cn2[j]);
      }
      float mn = a;
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, 1));
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, 2));
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, 4));
      const float lim = listed ? mn + 2.f * e32_bound(xnrm[i], cmax, d) : 0.f;
      const bool surv = j >= 0 && a <= lim;
      const uint32_t grp = (__ballot_sync(0xffffffffu, surv) >> (lane & 24)) & 0xffu;
      if (surv) atomicOr(&s_mask[r * mw + (j >> 5)], 1u << (j & 31));
      if (listed && u == 0) s_cnt[r] = __popc(grp) > 1 ? __popc(grp) : 0;
      if (surv && __popc(grp) == 1) labels[i] = j;
    }
    // ---- rows without a complete list: every centroid (warp = 2 rows), in
    // blocks of 256 columns: the minimum first, then the survivors
    const int nfull = s_nfull;
    for (int f0 = 2 * w; f0 < nfull; f0 += 2 * (kRsThreads / 32)) {
      const int r0 = s_full[f0], r1 = f0 + 1 < nfull ? s_full[f0 + 1] : r0;
      const bool two = f0 + 1 < nfull;  // warp-uniform
      auto scores = [&](int cb, float (&acc)[2][8]) {
#pragma unroll
        for (int m = 0; m < 8; ++m) { acc[0][m] = 0.f; acc[1][m] = 0.f; }
        const int mch = min(8, (k_cols - cb) >> 5);
        for (int t = 0; t < d; ++t) {
          const float x0 = xs[t * kRsRows + r0], x1 = xs[t * kRsRows + r1];
          const float *crow = cT + (int64_t)t * k_cols + cb + lane;
#pragma unroll
          for (int m = 0; m < 8; ++m) {
            if (m < mch) {
              const float cv = crow[32 * m];
              acc[0][m] = fmaf(x0, cv, acc[0][m]);
              acc[1][m] = fmaf(x1, cv, acc[1][m]);
            }
          }
        }
#pragma unroll
        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
          for (int m = 0; m < 8; ++m) {
            const int j = cb + lane + 32 * m;
            acc[rr][m] = (m < mch && j < k) ? fmaf(-2.f, acc[rr][m], cn2[j]) : __int_as_float(0x7f800000);
          }
      };
      float acc[2][8];
      float mn[2] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000)};
      for (int cb = 0; cb < k_cols; cb += 256) {
        scores(cb, acc);
#pragma unroll
        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
          for (int m = 0; m < 8; ++m) mn[rr] = fminf(mn[rr], acc[rr][m]);
      }
#pragma unroll
      for (int rr = 0; rr < 2; ++rr)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mn[rr] = fminf(mn[rr], __shfl_xor_sync(0xffffffffu, mn[rr], o));
      const float lim0 = mn[0] + 2.f * e32_bound(xnrm[s_row[r0]], cmax, d);
      const float lim1 = mn[1] + 2.f * e32_bound(xnrm[s_row[r1]], cmax, d);
      int count[2] = {0, 0}, first[2] = {0x7fffffff, 0x7fffffff};
      for (int cb = 0; cb < k_cols; cb += 256) {
        if (k_cols > 256 || cb > 0) scores(cb, acc);  // one block: the scores are still in registers
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
          if (rr == 1 && !two) break;
          const int r = rr ? r1 : r0;
          const float lim = rr ? lim1 : lim0;
#pragma unroll
          for (int m = 0; m < 8; ++m) {
            const uint32_t bm = __ballot_sync(0xffffffffu, acc[rr][m] <= lim);
            count[rr] += __popc(bm);
            if (bm && first[rr] == 0x7fffffff) first[rr] = cb + 32 * m + __ffs(bm) - 1;
            if (lane == m && cb + 32 * m < k_cols) s_mask[r * mw + (cb >> 5) + m] = bm;
          }
        }
      }
#pragma unroll
      for (int rr = 0; rr < 2; ++rr) {
        if (rr == 1 && !two) break;
        const int r = rr ? r1 : r0;
        if (lane == 0) {
          s_cnt[r] = count[rr] > 1 ? count[rr] : 0;
          if (count[rr] <= 1) labels[s_row[r]] = first[rr] == 0x7fffffff ? 0 : first[rr];
        }
      }
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive prefix of the survivor counts
      int carry = 0;
      for (int r0 = 0; r0 < kRsRows; r0 += 32) {
        const int v = s_cnt[r0 + lane];
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        s_pre[r0 + lane] = carry + incl - v;
        carry += __shfl_sync(0xffffffffu, incl, 31);
      }
      if (lane == 0) s_pre[kRsRows] = carry;
    }
    __syncthreads();
    const int npairs = s_pre[kRsRows];
    if (npairs <= kRsPairs) {
      // ---- one thread per (row, survivor) pair
      for (int p = threadIdx.x; p < npairs; p += kRsThreads) {
        int lo = 0, hi = kRsRows - 1;  // the row: largest r with s_pre[r] <= p
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_pre[mid] <= p) lo = mid; else hi = mid - 1;
        }
        const int j = nth_candidate(s_mask + lo * mw, mw, p - s_pre[lo]);
        q_j[p] = (int16_t)j;
        q_s[p] = exact_sqd(x + s_row[lo] * (int64_t)d, cent + (int64_t)j * d, d);
      }
      __syncthreads();
      if (threadIdx.x < kRsRows && s_cnt[threadIdx.x] > 0) {
        const int r = threadIdx.x, b = s_pre[r], e = s_pre[r + 1];
        double best = q_s[b];
        int bj = q_j[b];
        for (int u = b + 1; u < e; ++u)  // ascending j: strict < keeps the lowest index
          if (q_s[u] < best) { best = q_s[u]; bj = q_j[u]; }
        labels[s_row[r]] = bj;
      }
    } else {
      // ---- many survivors: one row at a time, survivors spread over the threads
      for (int r = 0; r < kRsRows; ++r) {
        const int c = s_cnt[r];
        if (c == 0) continue;
        if (threadIdx.x == 0) { s_best = ~0ull; s_bj = 0x7fffffff; }
        __syncthreads();
        double sv = DBL_MAX;
        int j = 0x7fffffff;
        for (int u = threadIdx.x; u < c; u += kRsThreads) {  // ascending j: strict < keeps the lowest
          const int ju = nth_candidate(s_mask + r * mw, mw, u);
          const double su = exact_sqd(x + s_row[r] * (int64_t)d, cent + (int64_t)ju * d, d);
          if (su < sv) { sv = su; j = ju; }
        }
        if ((int)threadIdx.x < c)
          atomicMin(&s_best, (unsigned long long)__double_as_longlong(sv));  // sv >= 0: bits order as values
        __syncthreads();
        if ((int)threadIdx.x < c && (unsigned long long)__double_as_longlong(sv) == s_best) atomicMin(&s_bj, j);
        __syncthreads();
        if (threadIdx.x == 0) labels[s_row[r]] = s_bj;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && st) atomicAdd((unsigned long long *)&st->rescored, (unsigned long long)total);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

sc_status make_map(CUtensorMap *m, void *ptr, int64_t rows, int cols, int box_cols, int box_rows, int row_bytes) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) { set_error("cuTensorMapEncodeTiled is unavailable"); return SC_ERR_CUDA; }
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


// Feature padding: rows of 32 B (d <= 16, 32-byte swizzle), 64 B (d <= 32,
// 64-byte swizzle) or multiples of 128 B (128-byte swizzle, 64-feature tiles).
int pad_d(int d) { return d <= 16 ? 16 : d <= 32 ? 32 : (d + 63) / 64 * 64; }

size_t assign_smem(const SplitState *s, int stages, int k_pad) {
  const size_t a_stage = (size_t)2 * s->nkt * kBM * s->row_bytes;
  const size_t b_bytes = (((size_t)2 * s->nkt * k_pad * s->row_bytes) + 1023) & ~(size_t)1023;
  const size_t x_bytes = ((size_t)kBM * 32 + (size_t)k_pad * 32 + 1023) & ~(size_t)1023;
  return 1024 + b_bytes + x_bytes + (size_t)stages * a_stage + 8 * kBM * 16 + (size_t)(2 * stages + 6) * 8 + 16;
}

}  // namespace

sc_status split_prepare(SplitState *s, int dtype, const void *x, int64_t n, int d, double *xnorm_total,
                        cudaStream_t st) {
  split_free(s, st);
  s->dtype = dtype;
  s->n = n;
  s->n_pad = (n + kBM - 1) / kBM * kBM;
  if (s->n_pad == 0) s->n_pad = kBM;
  s->d = d;
  s->d_pad = pad_d(d);
  s->kt_elems = s->d_pad >= 64 ? 64 : s->d_pad;
  s->nkt = s->d_pad / s->kt_elems;
  s->row_bytes = s->kt_elems * 2;
  if (s->d_pad > 256) {
    set_error("d=%d exceeds the split-BF16 kernel's limit of 256 features", d);
    return SC_ERR_INVALID;
  }
  int dev = 0;
  SC_CUDA(cudaGetDevice(&dev));
  SC_CUDA(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev));
  SC_TRY(dalloc(&s->xh, (size_t)(s->n_pad * s->d_pad), st));
  SC_TRY(dalloc(&s->xl, (size_t)(s->n_pad * s->d_pad), st));
  SC_TRY(dalloc(&s->xnrm, (size_t)s->n_pad, st));
  const int nb = (int)((s->n_pad + 7) / 8);
  SC_TRY(dalloc(&s->part, (size_t)nb, st));
  SC_TRY(dalloc(&s->list_rows, (size_t)(s->n_pad + (int64_t)s->num_sms * kBM), st));
  SC_TRY(dalloc(&s->list_count, (size_t)s->num_sms, st));
  SC_TRY(dalloc(&s->cand4, (size_t)(2 * s->n_pad), st));  // uint2 each
  SC_TRY(dalloc(&s->cmeta, (size_t)(2 * s->n_pad), st));
  SC_TRY(dalloc(&s->cmax, 1, st));
  if (dtype == SC_F32)
    prep_x_kernel<float><<<nb, 256, 0, st>>>((const float *)x, n, s->n_pad, d, s->d_pad, s->xh, s->xl, s->xnrm, s->part);
  else
    prep_x_kernel<double><<<nb, 256, 0, st>>>((const double *)x, n, s->n_pad, d, s->d_pad, s->xh, s->xl, s->xnrm, s->part);
  SC_LAUNCHED();
  sum_parts_kernel<<<1, 1024, 0, st>>>(s->part, nb, xnorm_total);
  SC_LAUNCHED();
  SC_TRY(make_map(&s->tm_xh, s->xh, s->n_pad, s->d_pad, s->kt_elems, kBM, s->row_bytes));
  SC_TRY(make_map(&s->tm_xl, s->xl, s->n_pad, s->d_pad, s->kt_elems, kBM, s->row_bytes));
  SC_TRY(dalloc(&s->ones, (size_t)kBM * 16, st));
  ones_tile_kernel<<<1, kBM, 0, st>>>(s->ones);
  SC_LAUNCHED();
  SC_TRY(make_map(&s->tm_ones, s->ones, kBM, 16, 16, kBM, 32));
  s->ready = 1;
  return SC_OK;
}

size_t wide_smem(const SplitState *s, int stages) {
  const size_t a_bytes = (size_t)2 * s->nkt * kBM * s->row_bytes;
  const size_t b_stage = ((size_t)2 * s->nkt * kWN * s->row_bytes + kWN * 32 + 1023) & ~(size_t)1023;
  return 1024 + a_bytes + 4096 + (size_t)stages * b_stage + (size_t)2 * kBM * 12 * 4 + (size_t)(2 * stages + 7) * 8 + 16;
}

sc_status split_centroids_changed(SplitState *s, const double *cent, int k, cudaStream_t st) {
  if (!s->ready) { set_error("split-BF16 state is not prepared"); return SC_ERR_INTERNAL; }
  // up to 256 centroids resident in shared memory; more (or too large) stream in blocks of kWN
  const int k_pad16 = (k + 15) / 16 * 16;
  const bool wide = k_pad16 > 256 || assign_smem(s, 2, k_pad16) > 227 * 1024;
  const int k_pad = wide ? (k + kWN - 1) / kWN * kWN : k_pad16;
  const int k_cols = (k_pad + 31) / 32 * 32;
  if (k_pad > 65535) {
    set_error("k=%d exceeds the split-BF16 kernel's limit of 65535 clusters", k);
    return SC_ERR_INVALID;
  }
  if (wide && wide_smem(s, 2) > 227 * 1024) {
    set_error("d=%d exceeds the split-BF16 kernel's shared memory for k=%d", s->d, k);
    return SC_ERR_INVALID;
  }
  if (k_cols > s->k_alloc) {
    s->k_alloc = 0;  // a failed allocation leaves no stale capacity
    s->k_pad = 0;
    dfree(s->ch, st); dfree(s->cl, st); dfree(s->cn2, st); dfree(s->cT, st); dfree(s->cbx, st);
    SC_TRY(dalloc(&s->ch, (size_t)k_cols * s->d_pad, st));
    SC_TRY(dalloc(&s->cl, (size_t)k_cols * s->d_pad, st));
    SC_TRY(dalloc(&s->cbx, (size_t)k_cols * 16, st));
    SC_TRY(dalloc(&s->cn2, (size_t)k_cols, st));
    SC_TRY(dalloc(&s->cT, (size_t)k_cols * s->d_pad, st));
    s->k_alloc = k_cols;
    s->k_pad = 0;
  }
  if (k_pad != s->k_pad) {
    const int box = wide ? kWN : k_pad;
    SC_TRY(make_map(&s->tm_ch, s->ch, k_pad, s->d_pad, s->kt_elems, box, s->row_bytes));
    SC_TRY(make_map(&s->tm_cl, s->cl, k_pad, s->d_pad, s->kt_elems, box, s->row_bytes));
    SC_TRY(make_map(&s->tm_cbx, s->cbx, k_pad, 16, 16, box, 32));
  }
  s->wide = wide ? 1 : 0;
  s->k = k;
  s->k_pad = k_pad;
  SC_CUDA(cudaMemsetAsync(s->cmax, 0, sizeof(unsigned int), st));
  SC_TRY(launch_pdl(prep_c_kernel, k_cols, 128, 0, st, cent, k, s->d, s->d_pad, k_pad, k_cols, s->ch, s->cl, s->cbx,
                    s->cn2, s->cmax, s->cT));
  SC_LAUNCHED();
  return SC_OK;
}

sc_status split_assign(SplitState *s, int dtype, const void *x, int64_t n, int d, const double *cent, int k,
                       int32_t *labels, LloydState *lst, cudaStream_t st, cudaEvent_t *timing) {
  if (!s->ready || s->k != k) { set_error("split-BF16 centroids are not prepared"); return SC_ERR_INTERNAL; }
  if (n == 0) return SC_OK;
  const int k_cols = (s->k_pad + 31) / 32 * 32;
  uint32_t tmem_cols = 32;
  while (tmem_cols < (uint32_t)(2 * k_cols)) tmem_cols <<= 1;
  int stages = s->wide ? 4 : 6;
  if (s->wide)
    while (stages > 2 && wide_smem(s, stages) > 227 * 1024) --stages;
  else
    while (stages > 2 && assign_smem(s, stages, s->k_pad) > 227 * 1024) --stages;
  const size_t smem = s->wide ? wide_smem(s, stages) : assign_smem(s, stages, s->k_pad);
  if (smem > 227 * 1024) {
    set_error("d=%d, k=%d exceed the split-BF16 kernel's shared memory", d, k);
    return SC_ERR_INVALID;
  }
  AssignParams p;
  memset(&p, 0, sizeof p);
  p.n = n;
  p.n_tiles = (int)(s->n_pad / kBM);
  const int grid = p.n_tiles < s->num_sms ? p.n_tiles : s->num_sms;
  p.nkt = s->nkt;
  p.kt_elems = s->kt_elems;
  p.row_bytes = s->row_bytes;
  p.k = k;
  p.k_pad = s->k_pad;
  p.k_cols = k_cols;
  p.stages = stages;
  p.tmem_cols = tmem_cols;
  p.xnrm = s->xnrm;
  p.cmax = s->cmax;
  // |acc - (x.c - ||c||^2/2)|: split remainders 3.02 * 2^-16 ||x|| ||c||; three-term
  // split of ||c||^2/2 (2^-24 relative); FP32 accumulation of 3 d_pad + 3 exact
  // terms, <= 2^-22 of their absolute sum per term
  const double nacc = 3.0 * s->d_pad + 3.0;
  p.coef_xc = (float)(3.02 * 0x1p-16 + 1.02 * nacc * 0x1p-22);
  p.coef_cc = (float)(1.01 * 0x1p-25 + 0.51 * nacc * 0x1p-22);
  p.coef_ref = (float)((d + 4) * 0x1p-52);
  p.labels = labels;
  p.n_pad = s->n_pad;
  p.region = (int)((p.n_tiles + grid - 1) / grid) * kBM;
  p.list_count = s->list_count;
  p.list_rows = s->list_rows;
  p.cand4 = s->cand4;
  p.cmeta = s->cmeta;
  p.st = lst;
  p.wait_ns = s->wait_ns ? s->wait_ns : kWaitNs;
  if (s->wide) {
    SC_CUDA(cudaFuncSetAttribute(split_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (timing) SC_CUDA(cudaEventRecord(timing[0], st));
    SC_TRY(launch_pdl(split_wide_kernel, grid, kWideThreads, smem, st, s->tm_xh, s->tm_xl, s->tm_ch, s->tm_cl,
                      s->tm_ones, s->tm_cbx, p));
  } else {
    SC_CUDA(cudaFuncSetAttribute(split_assign_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (timing) SC_CUDA(cudaEventRecord(timing[0], st));
    SC_TRY(launch_pdl(split_assign_kernel, grid, kAssignThreads, smem, st, s->tm_xh, s->tm_xl, s->tm_ch, s->tm_cl,
                      s->tm_ones, s->tm_cbx, p));
  }
  SC_LAUNCHED();
  if (timing) SC_CUDA(cudaEventRecord(timing[1], st));
  // near ties: re-score the rows each CTA listed
  const size_t ct_bytes = (size_t)d * k_cols * sizeof(float);
  const size_t xs_bytes = (size_t)d * kRsRows * sizeof(float) + (size_t)kRsRows * (k_cols / 32) * sizeof(uint32_t);
  const int stage = ct_bytes + xs_bytes <= 180 * 1024 ? 1 : 0;
  const size_t rsmem = xs_bytes + (stage ? ct_bytes : 0);
  if (dtype == SC_F32) {
    auto kern = rescore_kernel<float>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem));
    SC_TRY(launch_pdl(kern, grid, kRsThreads, rsmem, st, (const float *)x, d, cent, k, k_cols, s->cT, s->cn2, s->cmax,
                      s->xnrm, s->list_rows, s->list_count, p.region, s->cand4, s->cmeta, s->n_pad, labels, lst, stage));
  } else {
    auto kern = rescore_kernel<double>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem));
    SC_TRY(launch_pdl(kern, grid, kRsThreads, rsmem, st, (const double *)x, d, cent, k, k_cols, s->cT, s->cn2, s->cmax,
                      s->xnrm, s->list_rows, s->list_count, p.region, s->cand4, s->cmeta, s->n_pad, labels, lst, stage));
  }
  SC_LAUNCHED();
  return SC_OK;
}

void split_free(SplitState *s, cudaStream_t st) {
  dfree(s->xh, st); dfree(s->xl, st); dfree(s->xnrm, st); dfree(s->part, st);
  dfree(s->ch, st); dfree(s->cl, st); dfree(s->cn2, st); dfree(s->cmax, st); dfree(s->cbx, st); dfree(s->ones, st);
  dfree(s->cT, st); dfree(s->list_rows, st); dfree(s->list_count, st); dfree(s->cand4, st); dfree(s->cmeta, st);
  s->ready = 0;
  s->k_alloc = 0;
  s->k_pad = 0;
}



}  // namespace sc
