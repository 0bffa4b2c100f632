// FP64 kernels that keep smartcore's own operation order, so every distance
// they produce is bit-identical to the reference CPU value.
//
// This translation unit is compiled with -fmad=false, and every arithmetic
// step is also spelled with an explicit round-to-nearest intrinsic: no
// multiply-add is ever fused (rustc never fuses either).
#include <float.h>

#include <algorithm>
#include <type_traits>

#include <cuda_bf16.h>

#include "common.cuh"
#include "exactsum.cuh"
#include "ppsel.cuh"

namespace sc {

// ---------------------------------------------------------------------------
// K1: assignment in FP64 — KMeans::predict (src/cluster/kmeans.rs:327-352)
// and the per-point outcome of BBDTree::clustering (src/algorithm/neighbour/
// bbd_tree.rs:101-111 at the leaves): argmin over centroids of
// sum_j (f64(x_j) - c_j)^2, strict <, lowest index wins ties; min starts at
// f64::MAX.  Also writes the block's fixed-order sum of the winning distances
// (the distortion of this step) to part[blockIdx.x].
// ---------------------------------------------------------------------------
constexpr int kAssignThreads = 128;

template <typename T>
__global__ void __launch_bounds__(kAssignThreads)
assign_fp64_kernel(const T *__restrict__ x, int64_t n, int d,
                   const double *__restrict__ cent, int k, int ktile,
                   int32_t *__restrict__ labels, double *__restrict__ part,
                   const LloydState *st) {
  if (st && st->done) return;
  extern __shared__ double cs[];  // ktile x d centroid tile
  const int64_t i = (int64_t)blockIdx.x * kAssignThreads + threadIdx.x;
  const bool live = i < n;
  const T *xr = x + (live ? i : 0) * (int64_t)d;
  double best = DBL_MAX;
  int bi = 0;
  for (int c0 = 0; c0 < k; c0 += ktile) {
    const int kt = min(ktile, k - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < kt * d; t += kAssignThreads) cs[t] = cent[(int64_t)c0 * d + t];
    __syncthreads();
    if (!live) continue;
    int c = 0;
    for (; c + 4 <= kt; c += 4) {
      const double *p = cs + c * d;
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      for (int j = 0; j < d; ++j) {
        const double xj = (double)xr[j];
        a0 = __dadd_rn(a0, sq_term(xj, p[j]));
        a1 = __dadd_rn(a1, sq_term(xj, p[d + j]));
        a2 = __dadd_rn(a2, sq_term(xj, p[2 * d + j]));
        a3 = __dadd_rn(a3, sq_term(xj, p[3 * d + j]));
      }
      if (a0 < best) { best = a0; bi = c0 + c; }
      if (a1 < best) { best = a1; bi = c0 + c + 1; }
      if (a2 < best) { best = a2; bi = c0 + c + 2; }
      if (a3 < best) { best = a3; bi = c0 + c + 3; }
    }
    for (; c < kt; ++c) {
      const double *p = cs + c * d;
      double a = 0.0;
      for (int j = 0; j < d; ++j) a = __dadd_rn(a, sq_term((double)xr[j], p[j]));
      if (a < best) { best = a; bi = c0 + c; }
    }
  }
  if (live) labels[i] = bi;
  const double tot = block_sum_fixed<kAssignThreads>(live ? best : 0.0);
  if (threadIdx.x == 0 && part) part[blockIdx.x] = tot;
}

int assign_block_count(int64_t n) { return (int)((n + kAssignThreads - 1) / kAssignThreads); }

sc_status launch_assign_fp64(int dtype, const void *x, int64_t n, int d,
                             const double *cent, int k, int32_t *labels,
                             double *part, const LloydState *st,
                             cudaStream_t s) {
  if (n == 0) return SC_OK;
  const int max_smem = 96 * 1024;
  int ktile = max_smem / (d * (int)sizeof(double));
  if (ktile < 1) {
    set_error("d=%d is too large for the FP64 assignment kernel", d);
    return SC_ERR_INVALID;
  }
  if (ktile > k) ktile = k;
  const size_t smem = (size_t)ktile * d * sizeof(double);
  const int grid = assign_block_count(n);
  if (dtype == SC_F32) {
    auto kern = assign_fp64_kernel<float>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, kAssignThreads, smem, s>>>((const float *)x, n, d, cent, k, ktile, labels, part, st);
  } else {
    auto kern = assign_fp64_kernel<double>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, kAssignThreads, smem, s>>>((const double *)x, n, d, cent, k, ktile, labels, part, st);
  }
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// K3: k-means++ D^2 update — KMeans::kmeans_plus_plus (src/cluster/
// kmeans.rs:367-379 and :399-410).  The seed row is st->pp_chosen; the
// distance uses the element type's arithmetic (a - b and its square in T,
// summed in f64).  first_pass initialises d = f64::MAX and y = 0 (:357, :364).
//
// Rows far from the new seed are not read.  A row whose current seed a
// (labels[i]) and the new seed c satisfy |c - c_a| >= 2 |x - c_a| has
// |x - c| >= |x - c_a| (triangle inequality), so the reference's strict
// `dist < d[i]` test keeps d[i].  The test is made rigorous against the
// computed values: the reference's D = computed |x - c|^2 satisfies
//   (1 - eta) r^2 - A <= D <= (1 + eta) r^2 + A
// for the real r = |x - c| (terms in T, f64 sum of d terms; eta and A below),
// so with cc_lo <= |c - c_a|^2 (pp_seed_gaps) the row keeps its distance when
//   cc_lo >= 4 (1 + 3 eta) (D + A)                     (pp_far, pp_far32)
// since then the new seed's computed distance is >= D.
// ---------------------------------------------------------------------------
constexpr int kPPThreads = 256;

// The draw and selection kernels of k-means++ alternate 2 (k - 1) times;
// they are launched as programmatic dependents (launch_pdl, common.cuh).

int pp_block_count(int64_t n) { return (int)((n + kPPThreads - 1) / kPPThreads); }

// f32 terms: fl32(fl32(x - c)^2) is within (1 +- 2^-24)^3 of (x - c)^2, or
// within 2^-149 on underflow; the f64 sum adds d 2^-53 relative.  eta =
// 2^-22 covers d <= 2^25, A = d 2^-140.  f64 terms: eta = (d + 4) 2^-52,
// A = d 2^-1070.
struct PPFar {
  double mul, abs_;  // keep when cc_lo >= mul (D + abs_)
};

PPFar pp_far_bound(int dtype, int d) {
  const double eta = dtype == SC_F32 ? 0x1p-22 : (double)(d + 4) * 0x1p-52;
  const double a = dtype == SC_F32 ? (double)d * 0x1p-140 : (double)d * 0x1p-1070;
  return PPFar{4.0 * (1.0 + 3.0 * eta), a};
}

__device__ __forceinline__ bool pp_far(double cc_lo, double D, PPFar f) {
  return cc_lo >= __dmul_rn(f.mul, __dadd_rn(D, f.abs_));
}

template <typename T>
__global__ void __launch_bounds__(kPPThreads)
pp_update_kernel(const T *__restrict__ x, int64_t n, int d, const LloydState *st,
                 int32_t label_of_seed, double *__restrict__ dd,
                 int32_t *__restrict__ labels, double *__restrict__ part,
                 int first_pass, int lg_d, const float *__restrict__ seed_cc, PPFar far) {
  extern __shared__ unsigned char smraw[];
  T *cen = reinterpret_cast<T *>(smraw);
  const int64_t ci = st->pp_chosen;
  for (int t = threadIdx.x; t < d; t += kPPThreads) cen[t] = x[ci * d + t];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * kPPThreads + threadIdx.x;
  double v = 0.0;
  if (i < n) {
    double cur = first_pass ? DBL_MAX : dd[i];
    int32_t lab = first_pass ? 0 : labels[i];
    if (first_pass || !seed_cc || !pp_far((double)seed_cc[lab], cur, far)) {
      const T *xr = x + i * (int64_t)d;
      double s = 0.0;
      bool exact = false;
      // f32 rows: the same value from the integer reproduction of the sequential sum
      if constexpr (sizeof(T) == 4) exact = sqd_seq_f32(xr, cen, d, lg_d, s);
      if (!exact) {
        s = 0.0;
        for (int j = 0; j < d; ++j) s = __dadd_rn(s, sq_term(xr[j], cen[j]));
      }
      if (s < cur) { cur = s; lab = label_of_seed; }
      dd[i] = cur;
      labels[i] = lab;
    }
    v = cur;
  }
  const double tot = block_sum_fixed<kPPThreads>(v);
  if (threadIdx.x == 0 && part) part[blockIdx.x] = tot;
}

// Row stride (floats) of the staged tiles.  vec4: a multiple of 4 with an odd
// number of 16-byte units, so 8 lanes reading float4s of 8 rows hit 8
// different 4-bank groups; scalar: d + 1.
__host__ __device__ __forceinline__ int pp_stage_ld(int d, int vec4) {
  return vec4 ? (((d >> 2) & 1) ? d + 8 : d + 4) : d + 1;
}

// ---- f32 rows, d <= 128: one launch per draw ----
// pp_draw_kernel: one warp per 256-row block of d, in three stages.
//  1. The far test, in f32 from (d32 = d rounded up, y, seed_cc): reads no row.
//  2. Split form only: the rows it leaves are bounded through their BF16 high
//     halves (half the bytes of the f32 row).
//  3. The rows still left are read coalesced (up to four 16-byte units per
//     lane) for the f32 lower bound; the rows that bound cannot settle either
//     (the rows whose distance may drop) get the reference's exact value: from
//     the integer sum of their terms across the row's lanes when that sum
//     shows that no addition of the sequential f64 sum can round (almost every
//     row), else from the sequential reproduction, one row per lane.
// The warp then writes the block's fixed-order partial sum of d for the
// selection.  The first draw (every row exact) runs pp_first_kernel, which
// stages the rows in shared memory, and then pp_partials_kernel.
constexpr int kPPWarps = kPPThreads / 32;  // 32-row groups per 256-row block
constexpr int kDrawWarps = 4, kDrawThreads = 32 * kDrawWarps;

// Fixed-order sum of the 256 values of block b: lane l adds rows 32 g + l for
// g = 0..7 in order, then the lanes by a shuffle tree (depth 8 + 5).
__device__ __forceinline__ double pp_block_partial(const double *__restrict__ dd, int64_t n, int64_t b) {
  const int lane = threadIdx.x & 31;
  double t = 0.0;
#pragma unroll
  for (int g = 0; g < kPPWarps; ++g) {
    const int64_t i = b * kPPThreads + g * 32 + lane;
    t = __dadd_rn(t, i < n ? dd[i] : 0.0);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t = __dadd_rn(t, __shfl_down_sync(0xffffffffu, t, o));
  return t;
}

// Component c4 of unit uu's term fl32((x - c)^2).
template <int VEC>
__device__ __forceinline__ float pp_term(float4 v, const float *cen, int uu, int c4) {
  const float a = c4 == 0 ? v.x : c4 == 1 ? v.y : c4 == 2 ? v.z : v.w;
  const float r = __fsub_rn(a, cen[uu * 4 + c4]);
  return __fmul_rn(r, r);
}
template <int VEC>
__device__ __forceinline__ float pp_term(float v, const float *cen, int uu, int) {
  const float r = __fsub_rn(v, cen[uu]);
  return __fmul_rn(r, r);
}

template <int VEC>
__global__ void __launch_bounds__(kDrawThreads, 7)
pp_draw_kernel(const float *__restrict__ x, int64_t n, int d, const LloydState *st, int32_t label_of_seed,
               double *__restrict__ dd, float *__restrict__ dd32, int32_t *__restrict__ labels,
               double *__restrict__ part, int64_t nb, int lg_d, const float *__restrict__ seed_cc,
               PPFar32 far, const __nv_bfloat16 *__restrict__ xh, int d_pad, const float *__restrict__ xnrm) {
  using V = typename std::conditional<VEC == 4, float4, float>::type;
  constexpr int NP = VEC == 4 ? 1 : 4;  // row passes with loads in flight together
  constexpr int UM = 4;                 // loads per lane per row (d <= 128)
  __shared__ __align__(16) float s_cen[128];
  __shared__ uint8_t s_need[kDrawWarps][kPPThreads];  // the warp's rows left by the far test
  __shared__ uint8_t s_need2[kDrawWarps][kPPThreads];  // ... and by the BF16 bound
  __shared__ float s_cur[kDrawWarps][kPPThreads];     // d32 of the block's rows
  __shared__ uint8_t s_ex[kDrawWarps][kPPThreads];    // rows that need the sequential exact sum
  __shared__ uint8_t s_valr[kDrawWarps][kPPThreads];  // rows whose exact value is known
  __shared__ double s_valv[kDrawWarps][kPPThreads];   // and that value
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // launched as a programmatic dependent of the previous draw's selection:
  // the CTAs come up while it runs and wait here for its results
  pdl_release_dependents();
  pdl_wait_prerequisite();
  const int64_t ci = st->pp_chosen;
  for (int t = threadIdx.x; t < 128; t += kDrawThreads) s_cen[t] = t < d ? x[ci * d + t] : 0.f;
  __syncthreads();
  // a row is `units` loads of VEC floats; p lanes per row (a power of two,
  // at most UM units per lane), R = 32 / p rows per pass
  const int units = d / VEC;
  int p = 1;
  while (p * UM < units) p <<= 1;
  const int R = 32 / p, seg = lane / p, unit = lane - seg * p;
  const float lbf = 1.f - 1.05f * d * 0x1p-24f;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t nw = (int64_t)gridDim.x * kDrawWarps;
  for (int64_t b = (int64_t)blockIdx.x * kDrawWarps + w; b < nb; b += nw) {
    const int64_t rb = b * kPPThreads;  // first row of the block
    // far test of the block's 8 groups, four groups' loads issued together
    int cnt = 0;  // rows listed in s_need
#pragma unroll
    for (int h = 0; h < kPPWarps; h += 4) {
      float c32[4];
      int32_t lb[4];
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        const int64_t i = rb + (h + g) * 32 + lane;
        c32[g] = i < n ? dd32[i] : 0.f;
        lb[g] = i < n ? labels[i] : 0;
      }
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        const int64_t i = rb + (h + g) * 32 + lane;
        const bool need = i < n && !pp_far32(seed_cc[lb[g]], c32[g], far);
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if (need) s_need[w][cnt + __popc(m & lt)] = (uint8_t)((h + g) * 32 + lane);
        s_cur[w][(h + g) * 32 + lane] = c32[g];
        cnt += __popc(m);
      }
    }
    __syncwarp();
    const uint8_t *need_list = s_need[w];
    if (xh) {
      // Split form: the BF16 high half x_h of the row (half the bytes) bounds
      // the real distance from below: |x - c| >= |x_h - c| - |x - x_h|, with
      // |x - x_h| <= 2^-8 |x| + sqrt(d) 2^-133 (round to nearest BF16) and
      // xnrm >= |x|.  With the f32 sum s_h of fl(fl(x_h - c)^2) (depth <= d),
      // |x_h - c|^2 >= (s_h - d 2^-147)(1 - (d + 8) 2^-23); the row keeps its
      // distance when (1 - eta) r_lo^2 - A >= d32, as in the far test.
      const int units_h = d_pad >> 3;  // 16-byte units (8 BF16) per row
      constexpr int UH = 2;  // 16-byte units per lane
      int ph = 1;
      while (ph * UH < units_h) ph <<= 1;
      const int Rh = 32 / ph, segh = lane / ph, unith = lane - segh * ph;
      const uint4 *xbh = reinterpret_cast<const uint4 *>(xh + rb * d_pad);
      const float relh = 1.f - (float)(d + 8) * 0x1p-23f, sqd = sqrtf((float)d) * 0x1p-133f;
      int cnt2 = 0;
      for (int it = 0; it < cnt; it += Rh) {
        const int idx = it + segh;
        const int rr = idx < cnt ? (int)need_list[idx] : -1;
        uint4 hv[UH];
#pragma unroll
        for (int k = 0; k < UH; ++k) {
          const int uu = unith + k * ph;
          if (rr >= 0 && uu < units_h) hv[k] = xbh[rr * units_h + uu];
        }
        const float xn = rr >= 0 && unith == 0 ? xnrm[rb + rr] : 0.f;
        float sh = 0.f;
#pragma unroll
        for (int k = 0; k < UH; ++k) {
          const int uu = unith + k * ph;
          if (rr >= 0 && uu < units_h) {
            const uint32_t wv[4] = {hv[k].x, hv[k].y, hv[k].z, hv[k].w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const float lo = __uint_as_float(wv[e] << 16), hi = __uint_as_float(wv[e] & 0xffff0000u);
              float r = __fsub_rn(lo, s_cen[uu * 8 + 2 * e]);
              sh = __fadd_rn(sh, __fmul_rn(r, r));
              r = __fsub_rn(hi, s_cen[uu * 8 + 2 * e + 1]);
              sh = __fadd_rn(sh, __fmul_rn(r, r));
            }
          }
        }
        for (int o = ph >> 1; o > 0; o >>= 1) sh = __fadd_rn(sh, __shfl_xor_sync(0xffffffffu, sh, o));
        bool left = false;
        if (rr >= 0 && unith == 0) {
          const float L = fmaxf(0.f, __fmul_rd(__fsub_rd(sh, (float)d * 0x1p-147f), relh));
          const float rlo = __fsub_rd(__fsqrt_rd(L), __fadd_ru(__fmul_ru(xn, 0x1p-8f), sqd));
          left = !(rlo > 0.f &&
                   __fsub_rd(__fmul_rd(__fmul_rd(rlo, rlo), 1.f - 0x1p-22f), far.abs_) >= s_cur[w][rr]);
        }
        const unsigned lm = __ballot_sync(0xffffffffu, left);
        if (left) s_need2[w][cnt2 + __popc(lm & lt)] = (uint8_t)rr;
        cnt2 += __popc(lm);
      }
      __syncwarp();
      need_list = s_need2[w];
      cnt = cnt2;
    }
    // f32 lower bound of the listed rows, R rows per load, NP loads in flight
    const V *xb = reinterpret_cast<const V *>(x + rb * d);
    int exn = 0;   // rows listed in s_ex
    int nval = 0;  // rows listed in s_valr / s_valv
    for (int it = 0; it < cnt; it += R * NP) {
      int rq[NP];
      V val[NP][UM];
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const int idx = it + q * R + seg;
        rq[q] = idx < cnt ? (int)need_list[idx] : -1;
#pragma unroll
        for (int k = 0; k < UM; ++k) {
          const int uu = unit + k * p;
          if (rq[q] >= 0 && uu < units) val[q][k] = xb[rq[q] * units + uu];
        }
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        // The reference's terms q_t = fl32((x_t - c_t)^2).  Summed in f32 (any
        // order, depth <= d) they bound its f64 sum from below by s32 (1 - 1.05
        // d 2^-24): when that exceeds the current distance the row keeps it.
        float s32 = 0.f;
#pragma unroll
        for (int k = 0; k < UM; ++k) {
          const int uu = unit + k * p;
          if (rq[q] >= 0 && uu < units) {
            if constexpr (VEC == 4) {
              const float4 a = val[q][k];
              const float4 c = reinterpret_cast<const float4 *>(s_cen)[uu];
              float r = __fsub_rn(a.x, c.x);
              s32 = __fadd_rn(s32, __fmul_rn(r, r));
              r = __fsub_rn(a.y, c.y);
              s32 = __fadd_rn(s32, __fmul_rn(r, r));
              r = __fsub_rn(a.z, c.z);
              s32 = __fadd_rn(s32, __fmul_rn(r, r));
              r = __fsub_rn(a.w, c.w);
              s32 = __fadd_rn(s32, __fmul_rn(r, r));
            } else {
              const float r = __fsub_rn(val[q][k], s_cen[uu]);
              s32 = __fadd_rn(s32, __fmul_rn(r, r));
            }
          }
        }
        for (int o = p >> 1; o > 0; o >>= 1) s32 = __fadd_rn(s32, __shfl_xor_sync(0xffffffffu, s32, o));
        const bool ex = rq[q] >= 0 && unit == 0 && !(__fmul_rd(s32, lbf) > s_cur[w][rq[q] >= 0 ? rq[q] : 0]);
        if (__any_sync(0xffffffffu, ex)) {
          // The exact value without the sequential sum: in units of
          // 2^(emin - 150) every term is an integer below 2^(24 + span), so
          // while span <= 38 - ceil(log2 d) the integer sum S of the terms
          // (in any order; here across the row's lanes) is below 2^62.  The
          // terms are nonnegative, so when S < 2^53 every partial sum of the
          // reference's f64 sequence is an integer below 2^53 as well: no
          // addition rounds and its result is S.
          int emn = 255, emx = 0;
#pragma unroll
          for (int k = 0; k < UM; ++k) {
            const int uu = unit + k * p;
            if (rq[q] >= 0 && uu < units) {
#pragma unroll
              for (int c4 = 0; c4 < VEC; ++c4) {
                const uint32_t u = __float_as_uint(pp_term<VEC>(val[q][k], s_cen, uu, c4));
                if (u) {
                  const int e = max((int)(u >> 23), 1);
                  emn = min(emn, e);
                  emx = max(emx, e);
                }
              }
            }
          }
          for (int o = p >> 1; o > 0; o >>= 1) {
            emn = min(emn, __shfl_xor_sync(0xffffffffu, emn, o));
            emx = max(emx, __shfl_xor_sync(0xffffffffu, emx, o));
          }
          const bool span_ok = emx < 255 && (emn == 255 || emx - emn <= 38 - lg_d);
          unsigned long long S = 0ull;
          if (span_ok && emn < 255) {
#pragma unroll
            for (int k = 0; k < UM; ++k) {
              const int uu = unit + k * p;
              if (rq[q] >= 0 && uu < units) {
#pragma unroll
                for (int c4 = 0; c4 < VEC; ++c4) {
                  const uint32_t u = __float_as_uint(pp_term<VEC>(val[q][k], s_cen, uu, c4));
                  const int e = (int)(u >> 23);
                  const uint32_t m = (u & 0x7fffffu) | (e ? 0x800000u : 0u);
                  S += u ? (unsigned long long)m << (max(e, 1) - emn) : 0ull;
                }
              }
            }
          }
          for (int o = p >> 1; o > 0; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
          const bool fits = span_ok && (S >> 53) == 0ull;
          const unsigned fm = __ballot_sync(0xffffffffu, ex && fits);
          const unsigned sm = __ballot_sync(0xffffffffu, ex && !fits);
          if (ex && fits) {
            const int pos = nval + __popc(fm & lt);
            s_valr[w][pos] = (uint8_t)rq[q];
            s_valv[w][pos] = emn == 255 ? 0.0
                                        : __dmul_rn(__ull2double_rn(S),
                                                    __longlong_as_double((long long)(emn - 150 + 1023) << 52));
          }
          if (ex && !fits) s_ex[w][exn + __popc(sm & lt)] = (uint8_t)rq[q];
          nval += __popc(fm);
          exn += __popc(sm);
        }
      }
    }
    __syncwarp();
    // rows whose exact value is known: keep the smaller distance
    for (int e = lane; e < nval; e += 32) {
      const int64_t i = rb + s_valr[w][e];
      const double v = s_valv[w][e];
      if (v < dd[i]) {
        dd[i] = v;
        dd32[i] = __double2float_ru(v);
        labels[i] = label_of_seed;
      }
    }
    // the other rows whose distance may drop: the sequential exact sum, one
    // row per lane
    for (int e = lane; e < exn; e += 32) {
      const int64_t i = rb + s_ex[w][e];
      const float *xr = x + i * d;
      double sq = 0.0;
      if (!sqd_seq_f32(xr, s_cen, d, lg_d, sq)) {
        sq = 0.0;
        for (int j = 0; j < d; ++j) sq = __dadd_rn(sq, sq_term(xr[j], s_cen[j]));
      }
      if (sq < dd[i]) {
        dd[i] = sq;
        dd32[i] = __double2float_ru(sq);
        labels[i] = label_of_seed;
      }
    }
    __syncwarp();
    if (part) {
      const double t = pp_block_partial(dd, n, b);
      if (lane == 0) part[b] = t;
    }
    __syncwarp();  // s_need / s_ex are refilled for the next block
  }
}

// First draw: every row's exact distance to the first seed (d = f64::MAX and
// y = 0 before it, kmeans.rs:357, :364), rows staged in shared memory by
// asynchronous copies (16 bytes when d % 4 == 0, else 4), one row per lane.
__global__ void __launch_bounds__(kPPThreads)
pp_first_kernel(const float *__restrict__ x, int64_t n, int d, const LloydState *st,
                double *__restrict__ dd, float *__restrict__ dd32, int32_t *__restrict__ labels,
                int lg_d, int vec4) {
  extern __shared__ __align__(16) float smf[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ld = pp_stage_ld(d, vec4);
  float *cen = smf;                                          // d (padded to 4)
  float *tile = smf + ((d + 3) & ~3) + (size_t)w * 32 * ld;  // 32 rows x ld
  const int64_t ci = st->pp_chosen;
  for (int t = threadIdx.x; t < d; t += kPPThreads) cen[t] = x[ci * d + t];
  __syncthreads();
  const int64_t groups = (n + 31) / 32;
  const int64_t nw = (int64_t)gridDim.x * kPPWarps;
  const int units = vec4 ? d >> 2 : d;
  for (int64_t g = (int64_t)blockIdx.x * kPPWarps + w; g < groups; g += nw) {
    const int64_t r0 = g * 32, row = r0 + lane;
    const int nrows = n - r0 < 32 ? (int)(n - r0) : 32;
    // (row, unit) pairs of the warp's rows spread over the lanes
    int rr = lane / units, c = lane - rr * units;
    while (rr < nrows) {
      if (vec4) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(tile + rr * ld + 4 * c);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(x + (r0 + rr) * d + 4 * c) : "memory");
      } else {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(tile + rr * ld + c);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(x + (r0 + rr) * d + c) : "memory");
      }
      c += 32;
      while (c >= units) { c -= units; ++rr; }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
    if (lane < nrows) {
      const float *xr = tile + lane * ld;
      double sq = 0.0;
      if (!sqd_seq_f32(xr, cen, d, lg_d, sq)) {
        sq = 0.0;
        for (int j = 0; j < d; ++j) sq = __dadd_rn(sq, sq_term(xr[j], cen[j]));
      }
      const double v = sq < DBL_MAX ? sq : DBL_MAX;
      dd[row] = v;
      dd32[row] = __double2float_ru(v);
      labels[row] = 0;
    }
    __syncwarp();  // the tile is refilled by the next group
  }
}

__global__ void __launch_bounds__(kPPThreads)
pp_partials_kernel(const double *__restrict__ dd, int64_t n, int64_t nb, double *__restrict__ part) {
  const int64_t b = (int64_t)blockIdx.x * kPPWarps + (threadIdx.x >> 5);
  if (b >= nb) return;
  const double t = pp_block_partial(dd, n, b);
  if ((threadIdx.x & 31) == 0) part[b] = t;
}

int device_sms() {
  static int sms[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 132;
  if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms[dev] = 132;
  return sms[dev];
}

sc_status launch_pp_update(int dtype, const void *x, int64_t n, int d,
                           const LloydState *st, int32_t label_of_seed,
                           double *dd, float *dd32, int32_t *labels, double *part,
                           int first_pass, const float *seed_cc, const __nv_bfloat16 *xh, int d_pad,
                           const float *xnrm, cudaStream_t s) {
  const int grid = pp_block_count(n);
  const size_t smem = (size_t)d * (dtype == SC_F32 ? 4 : 8);
  if (smem > 48 * 1024) {
    set_error("d=%d is too large for the k-means++ kernel", d);
    return SC_ERR_INVALID;
  }
  int lg_d = 0;
  while ((1 << lg_d) < d) ++lg_d;
  if (dtype == SC_F32 && d <= 128 && dd32) {
    const float *xf = (const float *)x;
    const int sms = device_sms();
    const int vec4 = (d % 4 == 0 && ((uintptr_t)x & 15) == 0) ? 1 : 0;
    const int warp_blocks = (grid + kPPWarps - 1) / kPPWarps;
    if (first_pass) {
      const size_t ssm = ((size_t)((d + 3) & ~3) + (size_t)kPPThreads * pp_stage_ld(d, vec4)) * sizeof(float);
      SC_CUDA(cudaFuncSetAttribute(pp_first_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
      const int per_sm = std::max(1, std::min(8, (int)((225 * 1024) / (ssm + 1024))));
      const int g1 = (int)std::min<int64_t>((int64_t)sms * per_sm, (int64_t)warp_blocks);
      pp_first_kernel<<<g1, kPPThreads, ssm, s>>>(xf, n, d, st, dd, dd32, labels, lg_d, vec4);
      SC_LAUNCHED();
      if (part) {
        pp_partials_kernel<<<warp_blocks, kPPThreads, 0, s>>>(dd, n, grid, part);
        SC_LAUNCHED();
      }
    } else {
      // one warp per 256-row block, every warp resident at once when they fit
      const int g1 = std::min((grid + kDrawWarps - 1) / kDrawWarps, sms * 7);
      const PPFar32 far = pp_far_bound32(d);
      if (vec4)
        SC_TRY(launch_pdl(pp_draw_kernel<4>, g1, kDrawThreads, 0, s, xf, n, d, st, label_of_seed, dd, dd32, labels,
                          part, (int64_t)grid, lg_d, seed_cc, far, xh, d_pad, xnrm));
      else
        SC_TRY(launch_pdl(pp_draw_kernel<1>, g1, kDrawThreads, 0, s, xf, n, d, st, label_of_seed, dd, dd32, labels,
                          part, (int64_t)grid, lg_d, seed_cc, far, xh, d_pad, xnrm));
      SC_LAUNCHED();
    }
  } else if (dtype == SC_F32) {
    pp_update_kernel<float><<<grid, kPPThreads, smem, s>>>((const float *)x, n, d, st, label_of_seed, dd, labels,
                                                           part, first_pass, lg_d, seed_cc, pp_far_bound(dtype, d));
    SC_LAUNCHED();
  } else {
    pp_update_kernel<double><<<grid, kPPThreads, smem, s>>>((const double *)x, n, d, st, label_of_seed, dd, labels,
                                                            part, first_pass, lg_d, seed_cc, pp_far_bound(dtype, d));
    SC_LAUNCHED();
  }
  return SC_OK;
}

// ---------------------------------------------------------------------------
// k-means++ seed selection (kmeans.rs:381-396): sum = sequential f64 sum of
// d, cutoff = u * sum, index = first i whose sequential prefix >= cutoff.
//
// The sequential prefix S_i is inherently serial.  Here a parallel prefix
// Q_i (block partials, a block-wide scan of chunk sums, then warp walks over
// the crossing chunk's partials and the crossing block's rows) locates the
// candidate, and the choice is certified with a rigorous bound: all d_i >= 0,
// so |S_i - P_i| <= gamma_i P_i (Higham) for the exact prefix P_i, and Q_i
// obeys the same bound with the depth of its own summation tree.  Only when
// the cutoff falls inside the uncertainty band of the crossing does the
// kernel recompute S exactly as the reference does, on one thread.
//
// The same launch then copies the seed's row to seed_x[j] and writes the
// lower bounds seed_cc[a] of |x_pick - seed_x[a]|^2 for a < j, which the next
// update uses for its far test.
// ---------------------------------------------------------------------------
constexpr int kSelThreads = 1024;

template <typename T>
__global__ void __launch_bounds__(kSelThreads)
pp_select_kernel(const T *__restrict__ x, int d, const double *__restrict__ dd,
                 const double *__restrict__ part, int64_t n, int nb,
                 const double *__restrict__ uniform, LloydState *st,
                 T *__restrict__ seed_x, float *__restrict__ seed_cc, int j) {
  // threads that sum chunks of the partials: fewer than the CTA, since the
  // scan's FP64 additions (a narrow pipe) cost more than its longer chains
  constexpr int kScan = 256;
  __shared__ double s_incl[kScan];  // inclusive prefix of the chunk sums
  __shared__ double s_wtot[32];
  __shared__ int s_chunk;
  __shared__ long long s_pick;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  pdl_release_dependents();  // the next draw's CTAs may come up now; they wait for this kernel's results
  pdl_wait_prerequisite();   // the draw's partial sums
  const int chunk = (nb + kScan - 1) / kScan;
  const int b0 = min(nb, t * chunk), b1 = min(nb, b0 + chunk);
  double v = 0.0;
  if (t < kScan) {
    double loc = 0.0;
    for (int b = b0; b < b1; b += 8) {  // eight loads in flight, added in order
      double pv[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) pv[e] = b + e < b1 ? part[b + e] : 0.0;
#pragma unroll
      for (int e = 0; e < 8; ++e)
        if (b + e < b1) loc = __dadd_rn(loc, pv[e]);
    }
    // inclusive scan: warp scans, then a scan of the warp totals
    v = warp_incl_scan(loc);
    if (lane == 31) s_wtot[w] = v;
  }
  if (t == 0) s_chunk = kScan;
  __syncthreads();
  if (w == 0) s_wtot[lane] = warp_incl_scan(lane < kScan / 32 ? s_wtot[lane] : 0.0);
  __syncthreads();
  if (t < kScan) {
    if (w > 0) v = __dadd_rn(v, s_wtot[w - 1]);
    s_incl[t] = v;
  }
  __syncthreads();
  const double total = s_incl[kScan - 1];
  const double u = *uniform;
  const double cutoff = __dmul_rn(u, total);
  const double depth_q = (double)chunk + 2.0 * kSelThreads + 2.0 * kPPThreads + 64.0;
  if (t < kScan) {
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
    if (finite && s_chunk < kScan) {
      const int c = s_chunk;
      const int cb0 = c * chunk, cb1 = min(nb, cb0 + chunk);
      const Crossing cb = warp_first_crossing(part + cb0, cb1 - cb0, c > 0 ? s_incl[c - 1] : 0.0, cutoff);
      if (cb.t < cb1 - cb0) {
        const int64_t i0 = (int64_t)(cb0 + cb.t) * kPPThreads, i1 = min(n, i0 + kPPThreads);
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
  if (s_pick < 0) {
    // The cutoff is inside the rounding band: the exact values of the
    // sequential sum and prefix of kmeans.rs:381-396, by the whole CTA.
    double sum = 0.0;
    int64_t index = n;
    seq_exact_pass<kSelThreads>(dd, n, false, 0.0, &sum, nullptr);
    seq_exact_pass<kSelThreads>(dd, n, true, __dmul_rn(u, sum), nullptr, &index);
    if (t == 0) {
      s_pick = index < n ? index : n - 1;
      st->pp_replays += 1;
    }
    __syncthreads();
  }
  if (t == 0) st->pp_chosen = s_pick;
  const T *xp = x + (int64_t)s_pick * d;
  for (int c = t; c < d; c += kSelThreads) seed_x[(int64_t)j * d + c] = xp[c];
  pp_seed_gaps<kSelThreads>(xp, d, seed_x, j, seed_cc);
}

sc_status launch_pp_select(int dtype, const void *x, int d, const double *dd, const double *part,
                           int64_t n, int nb, const double *uniform, LloydState *st,
                           void *seed_x, float *seed_cc, int j, cudaStream_t s) {
  if (dtype == SC_F32)
    SC_TRY(launch_pdl(pp_select_kernel<float>, 1, kSelThreads, 0, s, (const float *)x, d, dd, part, n, nb, uniform,
                      st, (float *)seed_x, seed_cc, j));
  else
    SC_TRY(launch_pdl(pp_select_kernel<double>, 1, kSelThreads, 0, s, (const double *)x, d, dd, part, n, nb, uniform,
                      st, (double *)seed_x, seed_cc, j));
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// K4: LinearKNNSearch::find (src/algorithm/neighbour/linear_search.rs:52-84)
// in FP64, one query per thread.  The training rows stream through shared
// memory in index order; each thread keeps the reference's k-slot heap and
// replays it exactly: a row enters iff its distance is strictly below
// heap[0], which it replaces, followed by a full heapify
// (src/algorithm/sort/heap_select.rs:42-50, :71-86).
// ---------------------------------------------------------------------------
constexpr int kKnnTile = 32;  // training rows per shared-memory tile

__device__ __forceinline__ void heap_sift_down(double *hd, int32_t *hi, int kk,
                                               int nn, int stride) {
  while (2 * kk <= nn) {
    int j = 2 * kk;
    if (j < nn && hd[j * stride] < hd[(j + 1) * stride]) ++j;
    const double a = hd[kk * stride], b = hd[j * stride];
    if (a == b || a > b) break;
    if (j == kk) break;  // only reachable with a NaN root
    hd[kk * stride] = b;
    hd[j * stride] = a;
    const int32_t ti = hi[kk * stride];
    hi[kk * stride] = hi[j * stride];
    hi[j * stride] = ti;
    kk = j;
  }
}

__device__ __forceinline__ void heap_heapify(double *hd, int32_t *hi, int k, int stride) {
  if (k <= 1) return;
  for (int s = k / 2 - 1; s >= 0; --s) heap_sift_down(hd, hi, s, k - 1, stride);
}

// SHQ: the block's queries (transposed) and each training tile are staged in
// shared memory (else read from global memory, for wide rows).  SHH: the
// heaps live in shared memory (else in global memory, slot s of local query
// t at gh*[s * gstride + t], for large k).
template <typename T, bool SHQ, bool SHH>
__global__ void knn_fp64_kernel(const T *__restrict__ train, int64_t n, int d,
                                const T *__restrict__ queries, int64_t m, int k,
                                int64_t *__restrict__ idx_out,
                                double *__restrict__ dist_out,
                                double *__restrict__ ghd, int32_t *__restrict__ ghi, int64_t gstride) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nt = blockDim.x;
  double *hd = reinterpret_cast<double *>(smraw);                          // k x nt (SHH)
  int32_t *hi = reinterpret_cast<int32_t *>(hd + (SHH ? (size_t)k * nt : 0));  // k x nt (SHH)
  T *qs = reinterpret_cast<T *>(hi + (SHH ? (size_t)k * nt + ((k * nt) & 1) : 0));  // d x nt (SHQ)
  T *ts = qs + (SHQ ? (size_t)d * nt : 0);                                  // kKnnTile x d (SHQ)
  const int tid = threadIdx.x;
  const int64_t q = (int64_t)blockIdx.x * nt + tid;
  const bool live = q < m;
  if (SHQ)
    for (int j = 0; j < d; ++j) qs[j * nt + tid] = live ? queries[q * d + j] : T(0);
  double *mh = SHH ? hd + tid : ghd + (live ? q : 0);
  int32_t *mi = SHH ? hi + tid : ghi + (live ? q : 0);
  const int hs = SHH ? nt : (int)gstride;
  if (SHH || live)
    for (int s = 0; s < k; ++s) {
      mh[s * hs] = __longlong_as_double(0x7ff0000000000000ll);  // +inf
      mi[s * hs] = -1;
    }
  const T *qg = queries + (live ? q : 0) * d;
  for (int64_t r0 = 0; r0 < n; r0 += kKnnTile) {
    const int rt = (int)min((int64_t)kKnnTile, n - r0);
    if (SHQ) {
      __syncthreads();
      for (int t = tid; t < rt * d; t += nt) ts[t] = train[r0 * d + t];
      __syncthreads();
    }
    if (!live) continue;
    for (int r = 0; r < rt; ++r) {
      double s = 0.0;
      if (SHQ) {
        const T *tr = ts + r * d;
        for (int j = 0; j < d; ++j) s = __dadd_rn(s, sq_term(qs[j * nt + tid], tr[j]));
      } else {
        const T *tr = train + (r0 + r) * d;
        for (int j = 0; j < d; ++j) s = __dadd_rn(s, sq_term(qg[j], tr[j]));
      }
      const double dist = __dsqrt_rn(s);
      if (dist < mh[0]) {
        mh[0] = dist;
        mi[0] = (int32_t)(r0 + r);
        heap_heapify(mh, mi, k, hs);
      }
    }
  }
  if (!live) return;
  for (int s = 0; s < k; ++s) {
    idx_out[q * k + s] = mi[s * hs];
    dist_out[q * k + s] = mh[s * hs];
  }
}

// ---------------------------------------------------------------------------
// FastPair::init (src/algorithm/neighbour/fastpair.rs:82-150): for each row i
// the nearest later row j > i by the reference's squared distance, scanned in
// index order with the strict `d < nbd`, where nbd is the running best kept in
// the element type (T::from(d)) and starting at T::MAX.  One thread per row;
// the later rows stream through shared memory in tiles.  Row n - 1 keeps
// neighbour n - 1 and distance T::MAX (fastpair.rs:141-143).
// ---------------------------------------------------------------------------
// Element c of a row stored with stride s (a column of a transposed tile).
struct StridedRow {
  const float *p;
  int s;
  __device__ __forceinline__ float operator[](int c) const { return p[c * s]; }
};

template <typename T>
__global__ void fastpair_kernel(const T *__restrict__ x, int64_t n, int d, int lg_d, int64_t *__restrict__ nb_out,
                                double *__restrict__ dist_out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nt = blockDim.x;
  T *qs = reinterpret_cast<T *>(smraw);  // d x nt: this block's rows, transposed
  T *ts = qs + (size_t)d * nt;           // kKnnTile x d
  const int tid = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * nt + tid;
  const bool live = i < n;
  for (int j = 0; j < d; ++j) qs[j * nt + tid] = live ? x[i * d + j] : T(0);
  const T tmax = sizeof(T) == 4 ? (T)FLT_MAX : (T)DBL_MAX;
  T best = tmax;
  int64_t idx = i + 1;
  const int64_t first = (int64_t)blockIdx.x * nt + 1;  // the block's smallest j
  for (int64_t r0 = first - (first % kKnnTile); r0 < n; r0 += kKnnTile) {
    const int rt = (int)min((int64_t)kKnnTile, n - r0);
    __syncthreads();
    for (int t = tid; t < rt * d; t += nt) ts[t] = x[r0 * d + t];
    __syncthreads();
    if (!live) continue;
    for (int r = 0; r < rt; ++r) {
      const int64_t j = r0 + r;
      if (j <= i) continue;
      const T *tr = ts + r * d;
      if constexpr (sizeof(T) == 4) {
        // The terms fl32((x_c - y_c)^2) summed in f32 bound the reference's
        // f64 sum from below by s32 (1 - 1.05 d 2^-24): at or above the
        // running best the row cannot replace it, and its exact value is
        // not needed (almost every pair once the best is close).
        float s32 = 0.f;
        for (int c = 0; c < d; ++c) {
          const float df = __fsub_rn(qs[c * nt + tid], tr[c]);
          s32 = __fadd_rn(s32, __fmul_rn(df, df));
        }
        if (__fmul_rd(s32, 1.f - 1.05f * d * 0x1p-24f) >= best) continue;
      }
      // Euclidian::squared_distance (euclidian.rs:51-63) in the reference's
      // order; f32 rows by the integer reproduction of the sequential sum
      double s = 0.0;
      bool done = false;
      if constexpr (sizeof(T) == 4) done = sqd_seq_f32(StridedRow{qs + tid, nt}, tr, d, lg_d, s);
      if (!done) {
        s = 0.0;
        for (int c = 0; c < d; ++c) s = __dadd_rn(s, sq_term(qs[c * nt + tid], tr[c]));
      }
      if (s < (double)best) {
        best = (T)s;  // T::from(d): round to nearest
        idx = j;
      }
    }
  }
  if (!live) return;
  if (i == n - 1) {
    nb_out[i] = n - 1;
    dist_out[i] = (double)tmax;
  } else {
    nb_out[i] = idx;
    dist_out[i] = (double)best;
  }
}

sc_status launch_fastpair(int dtype, const void *x, int64_t n, int d, int64_t *nb, double *dist, cudaStream_t s) {
  if (n == 0) return SC_OK;
  const int es = dtype == SC_F32 ? 4 : 8;
  int nt = 128;
  size_t smem = 0;
  for (; nt >= 32; nt >>= 1) {
    smem = (size_t)d * nt * es + (size_t)kKnnTile * d * es;
    if (smem <= 200 * 1024) break;
  }
  if (nt < 32) {
    set_error("d=%d exceeds the FastPair kernel's shared memory", d);
    return SC_ERR_INVALID;
  }
  int lg_d = 0;
  while ((1 << lg_d) < d) ++lg_d;
  const int grid = (int)((n + nt - 1) / nt);
  if (dtype == SC_F32) {
    SC_CUDA(cudaFuncSetAttribute(fastpair_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fastpair_kernel<float><<<grid, nt, smem, s>>>((const float *)x, n, d, lg_d, nb, dist);
  } else {
    SC_CUDA(cudaFuncSetAttribute(fastpair_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fastpair_kernel<double><<<grid, nt, smem, s>>>((const double *)x, n, d, lg_d, nb, dist);
  }
  SC_LAUNCHED();
  return SC_OK;
}

template <typename T, bool SHQ, bool SHH>
static sc_status knn_fp64_launch(const T *train, int64_t n, int d, const T *queries, int64_t m, int k,
                                 int64_t *idx, double *dist, int nt, size_t smem, double *ghd, int32_t *ghi,
                                 int64_t gstride, cudaStream_t s) {
  auto kern = knn_fp64_kernel<T, SHQ, SHH>;
  SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<(unsigned)((m + nt - 1) / nt), nt, smem, s>>>(train, n, d, queries, m, k, idx, dist, ghd, ghi, gstride);
  SC_LAUNCHED();
  return SC_OK;
}

template <typename T>
static sc_status knn_fp64_typed(const T *train, int64_t n, int d, const T *queries, int64_t m, int k,
                                int64_t *idx, double *dist, cudaStream_t s) {
  constexpr size_t es = sizeof(T), kLimit = 200 * 1024;
  const size_t rows = (size_t)kKnnTile * d * es + 16;
  // everything in shared memory, widest block first
  for (int nt = 128; nt >= 32; nt >>= 1) {
    const size_t smem = (size_t)k * nt * 12 + 8 + (size_t)d * nt * es + rows;
    if (smem <= kLimit) return knn_fp64_launch<T, true, true>(train, n, d, queries, m, k, idx, dist, nt, smem,
                                                               nullptr, nullptr, 0, s);
  }
  // Heaps in global memory, queries in chunks of bounded heap storage.
  const bool shq = (size_t)d * 64 * es + rows <= kLimit;
  const int nt = shq ? 64 : 128;
  const size_t smem = shq ? (size_t)d * nt * es + rows : 0;
  int64_t chunk = std::max<int64_t>(nt, (int64_t)(((size_t)256 << 20) / ((size_t)k * 12)) / nt * nt);
  chunk = std::min<int64_t>(chunk, (m + nt - 1) / nt * nt);
  double *ghd = nullptr;
  int32_t *ghi = nullptr;
  SC_TRY(dalloc(&ghd, (size_t)chunk * k, s));
  sc_status r = dalloc(&ghi, (size_t)chunk * k, s);
  for (int64_t q0 = 0; r == SC_OK && q0 < m; q0 += chunk) {
    const int64_t mc = std::min(chunk, m - q0);
    r = shq ? knn_fp64_launch<T, true, false>(train, n, d, queries + q0 * d, mc, k, idx + q0 * k, dist + q0 * k, nt,
                                              smem, ghd, ghi, chunk, s)
            : knn_fp64_launch<T, false, false>(train, n, d, queries + q0 * d, mc, k, idx + q0 * k, dist + q0 * k,
                                               nt, 0, ghd, ghi, chunk, s);
  }
  dfree(ghd, s);
  dfree(ghi, s);
  return r;
}

sc_status launch_knn_fp64(int dtype, const void *train, int64_t n, int d,
                          const void *queries, int64_t m, int k, int64_t *idx,
                          double *dist, cudaStream_t s) {
  if (m == 0) return SC_OK;
  if (dtype == SC_F32)
    return knn_fp64_typed<float>((const float *)train, n, d, (const float *)queries, m, k, idx, dist, s);
  return knn_fp64_typed<double>((const double *)train, n, d, (const double *)queries, m, k, idx, dist, s);
}

// ---------------------------------------------------------------------------
// LinearKNNSearch::find_radius (src/algorithm/neighbour/linear_search.rs:89-
// 108) in FP64, one query per thread: every training row i in index order
// with d = sqrt(D) <= radius.  Pass 1 (out == nullptr) counts per query; pass
// 2 writes each query's rows from offsets[q] on.
// ---------------------------------------------------------------------------
// SHQ: queries and training tiles staged in shared memory (else read from
// global memory, for rows too wide to stage).
template <typename T, bool SHQ>
__global__ void knn_radius_fp64_kernel(const T *__restrict__ train, int64_t n, int d,
                                       const T *__restrict__ queries, int64_t m, double radius,
                                       int64_t *__restrict__ counts, const int64_t *__restrict__ offsets,
                                       int64_t *__restrict__ idx_out, double *__restrict__ dist_out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nt = blockDim.x;
  T *qs = reinterpret_cast<T *>(smraw);  // d x nt (SHQ)
  T *ts = qs + (SHQ ? (size_t)d * nt : 0);  // kKnnTile x d (SHQ)
  const int tid = threadIdx.x;
  const int64_t q = (int64_t)blockIdx.x * nt + tid;
  const bool live = q < m;
  if (SHQ)
    for (int j = 0; j < d; ++j) qs[j * nt + tid] = live ? queries[q * d + j] : T(0);
  const T *qg = queries + (live ? q : 0) * d;
  int64_t c = 0, pos = live && idx_out ? offsets[q] : 0;
  for (int64_t r0 = 0; r0 < n; r0 += kKnnTile) {
    const int rt = (int)min((int64_t)kKnnTile, n - r0);
    if (SHQ) {
      __syncthreads();
      for (int t = tid; t < rt * d; t += nt) ts[t] = train[r0 * d + t];
      __syncthreads();
    }
    if (!live) continue;
    for (int r = 0; r < rt; ++r) {
      double sq = 0.0;
      if (SHQ) {
        const T *tr = ts + r * d;
        for (int j = 0; j < d; ++j) sq = __dadd_rn(sq, sq_term(qs[j * nt + tid], tr[j]));
      } else {
        const T *tr = train + (r0 + r) * d;
        for (int j = 0; j < d; ++j) sq = __dadd_rn(sq, sq_term(qg[j], tr[j]));
      }
      const double dist = __dsqrt_rn(sq);
      if (dist <= radius) {
        if (idx_out) {
          idx_out[pos] = r0 + r;
          dist_out[pos] = dist;
          ++pos;
        }
        ++c;
      }
    }
  }
  if (live && !idx_out) counts[q] = c;
}

template <typename T>
static sc_status knn_radius_typed(const T *train, int64_t n, int d, const T *queries, int64_t m, double radius,
                                  int64_t *counts, const int64_t *offsets, int64_t *idx, double *dist,
                                  cudaStream_t s) {
  constexpr size_t es = sizeof(T);
  for (int nt = 128; nt >= 32; nt >>= 1) {
    const size_t smem = (size_t)d * nt * es + (size_t)kKnnTile * d * es + 16;
    if (smem > 200 * 1024) continue;
    auto kern = knn_radius_fp64_kernel<T, true>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<(unsigned)((m + nt - 1) / nt), nt, smem, s>>>(train, n, d, queries, m, radius, counts, offsets, idx,
                                                         dist);
    SC_LAUNCHED();
    return SC_OK;
  }
  knn_radius_fp64_kernel<T, false><<<(unsigned)((m + 127) / 128), 128, 0, s>>>(train, n, d, queries, m, radius,
                                                                                counts, offsets, idx, dist);
  SC_LAUNCHED();
  return SC_OK;
}

sc_status launch_knn_radius_fp64(int dtype, const void *train, int64_t n, int d, const void *queries, int64_t m,
                                 double radius, int64_t *counts, const int64_t *offsets, int64_t *idx,
                                 double *dist, cudaStream_t s) {
  if (m == 0) return SC_OK;
  if (dtype == SC_F32)
    return knn_radius_typed<float>((const float *)train, n, d, (const float *)queries, m, radius, counts, offsets,
                                   idx, dist, s);
  return knn_radius_typed<double>((const double *)train, n, d, (const double *)queries, m, radius, counts, offsets,
                                  idx, dist, s);
}

// ---------------------------------------------------------------------------
// KNNWeightFunction::calc_weights (src/neighbors/mod.rs:62-78) and the
// classifier vote (src/neighbors/knn_classifier.rs:279-299): weights in heap
// order over the entries whose index is Some, w_sum summed in that order,
// c[y] += w / w_sum, argmax by strict > scanned in heap order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int knn_weights(const int64_t *qi, const double *qd,
                                           int k, int weight, double *w,
                                           int *pos) {
  int c = 0;
  bool any_zero = false;
  for (int s = 0; s < k; ++s)
    if (qi[s] >= 0) {
      pos[c++] = s;
      any_zero |= qd[s] == 0.0;
    }
  for (int t = 0; t < c; ++t) {
    const double e = qd[pos[t]];
    w[t] = weight == SC_KNN_UNIFORM ? 1.0 : (any_zero ? (e == 0.0 ? 1.0 : 0.0) : __ddiv_rn(1.0, e));
  }
  return c;
}

// Per-query work arrays of the aggregation: in local memory for k <= 64,
// else slices of a global scratch (k entries per query of the launch).
struct VoteScratch {
  double *w = nullptr, *cv = nullptr;
  int *pos = nullptr;
  int64_t *cls = nullptr;
};

template <bool LOCAL>
__global__ void knn_vote_kernel(const int64_t *__restrict__ idx,
                                const double *__restrict__ dist, int64_t m,
                                int k, int weight,
                                const int64_t *__restrict__ y_class,
                                int64_t *__restrict__ out, VoteScratch sc) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  double wl[LOCAL ? kMaxKnnK : 1], cvl[LOCAL ? kMaxKnnK : 1];
  int posl[LOCAL ? kMaxKnnK : 1];
  int64_t clsl[LOCAL ? kMaxKnnK : 1];
  double *w = LOCAL ? wl : sc.w + q * k, *cv = LOCAL ? cvl : sc.cv + q * k;
  int *pos = LOCAL ? posl : sc.pos + q * k;
  int64_t *cls = LOCAL ? clsl : sc.cls + q * k;
  const int c = knn_weights(idx + q * k, dist + q * k, k, weight, w, pos);
  double w_sum = 0.0;
  for (int t = 0; t < c; ++t) w_sum = __dadd_rn(w_sum, w[t]);
  int ncls = 0;
  double max_c = 0.0;
  int64_t max_i = 0;
  for (int t = 0; t < c; ++t) {
    const int64_t y = y_class[idx[q * k + pos[t]]];
    int slot = 0;
    while (slot < ncls && cls[slot] != y) ++slot;
    if (slot == ncls) { cls[ncls] = y; cv[ncls] = 0.0; ++ncls; }
    cv[slot] = __dadd_rn(cv[slot], __ddiv_rn(w[t], w_sum));
    if (cv[slot] > max_c) { max_c = cv[slot]; max_i = y; }
  }
  out[q] = max_i;
}

// KNNRegressor::predict_for_row (src/neighbors/knn_regressor.rs:268-282).
template <bool LOCAL>
__global__ void knn_regress_kernel(const int64_t *__restrict__ idx,
                                   const double *__restrict__ dist, int64_t m,
                                   int k, int weight,
                                   const double *__restrict__ y,
                                   double *__restrict__ out, VoteScratch sc) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  double wl[LOCAL ? kMaxKnnK : 1];
  int posl[LOCAL ? kMaxKnnK : 1];
  double *w = LOCAL ? wl : sc.w + q * k;
  int *pos = LOCAL ? posl : sc.pos + q * k;
  const int c = knn_weights(idx + q * k, dist + q * k, k, weight, w, pos);
  double w_sum = 0.0;
  for (int t = 0; t < c; ++t) w_sum = __dadd_rn(w_sum, w[t]);
  double r = 0.0;
  for (int t = 0; t < c; ++t)
    r = __dadd_rn(r, __dmul_rn(y[idx[q * k + pos[t]]], __ddiv_rn(w[t], w_sum)));
  out[q] = r;
}

// Labels widened to the reference's usize-sized indices for the host copy.
__global__ void widen_labels_kernel(const int32_t *__restrict__ in, int64_t *__restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

sc_status launch_widen_labels(const int32_t *in, int64_t *out, int64_t n, cudaStream_t s) {
  if (n == 0) return SC_OK;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  widen_labels_kernel<<<grid, 256, 0, s>>>(in, out, n);
  SC_LAUNCHED();
  return SC_OK;
}

// Queries per launch of the scratch form: at most 256 MB of work arrays.
static int64_t vote_chunk(int64_t m, int k) {
  return std::min<int64_t>(m, std::max<int64_t>(128, (int64_t)(((size_t)256 << 20) / ((size_t)k * 28))));
}

sc_status launch_knn_vote(const int64_t *idx, const double *dist, int64_t m,
                          int k, int weight, const int64_t *y_class,
                          int64_t *out, cudaStream_t s) {
  if (m == 0) return SC_OK;
  if (k <= kMaxKnnK) {
    knn_vote_kernel<true><<<(unsigned)((m + 127) / 128), 128, 0, s>>>(idx, dist, m, k, weight, y_class, out,
                                                                       VoteScratch());
    SC_LAUNCHED();
    return SC_OK;
  }
  const int64_t chunk = vote_chunk(m, k);
  VoteScratch sc;
  sc_status r = dalloc(&sc.w, (size_t)chunk * k, s);
  if (r == SC_OK) r = dalloc(&sc.cv, (size_t)chunk * k, s);
  if (r == SC_OK) r = dalloc(&sc.pos, (size_t)chunk * k, s);
  if (r == SC_OK) r = dalloc(&sc.cls, (size_t)chunk * k, s);
  for (int64_t q0 = 0; r == SC_OK && q0 < m; q0 += chunk) {
    const int64_t mc = std::min(chunk, m - q0);
    knn_vote_kernel<false><<<(unsigned)((mc + 127) / 128), 128, 0, s>>>(idx + q0 * k, dist + q0 * k, mc, k, weight,
                                                                         y_class, out + q0, sc);
    note_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) r = cuda_fail(e, "knn_vote_kernel");
  }
  dfree(sc.w, s); dfree(sc.cv, s); dfree(sc.pos, s); dfree(sc.cls, s);
  return r;
}

sc_status launch_knn_regress(const int64_t *idx, const double *dist,
                             int64_t m, int k, int weight, const double *y,
                             double *out, cudaStream_t s) {
  if (m == 0) return SC_OK;
  if (k <= kMaxKnnK) {
    knn_regress_kernel<true><<<(unsigned)((m + 127) / 128), 128, 0, s>>>(idx, dist, m, k, weight, y, out,
                                                                         VoteScratch());
    SC_LAUNCHED();
    return SC_OK;
  }
  const int64_t chunk = vote_chunk(m, k);
  VoteScratch sc;
  sc_status r = dalloc(&sc.w, (size_t)chunk * k, s);
  if (r == SC_OK) r = dalloc(&sc.pos, (size_t)chunk * k, s);
  for (int64_t q0 = 0; r == SC_OK && q0 < m; q0 += chunk) {
    const int64_t mc = std::min(chunk, m - q0);
    knn_regress_kernel<false><<<(unsigned)((mc + 127) / 128), 128, 0, s>>>(idx + q0 * k, dist + q0 * k, mc, k,
                                                                           weight, y, out + q0, sc);
    note_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) r = cuda_fail(e, "knn_regress_kernel");
  }
  dfree(sc.w, s); dfree(sc.pos, s);
  return r;
}

}  // namespace sc
