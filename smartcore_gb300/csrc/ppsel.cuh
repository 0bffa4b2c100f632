// Device helpers shared by the k-means++ kernels of the single-problem path
// (exact.cu) and of the batched path (batch.cu): the reference's squared-
// distance term, the f32 far test, and the certified prefix search of the
// seed selection.  Both translation units are compiled with -fmad=false.
#pragma once

#include <cuda_runtime.h>

namespace sc {

// One term of Euclidian::squared_distance (src/metrics/distance/
// euclidian.rs:56-62): r = a - b and r * r in the element type, then to_f64.
__device__ __forceinline__ double sq_term(float a, float b) {
  float r = __fsub_rn(a, b);
  return (double)__fmul_rn(r, r);
}
__device__ __forceinline__ double sq_term(double a, double b) {
  double r = __dsub_rn(a, b);
  return __dmul_rn(r, r);
}

// f32 form of the far test: keep when cc >= mul (D32 + abs_), both roundings
// upward, with D32 >= D.
struct PPFar32 {
  float mul, abs_;
};

inline PPFar32 pp_far_bound32(int d) {
  // eta = 2^-22: 4 (1 + 3 eta) is exact in f32; A = d 2^-140 is an f32 subnormal
  return PPFar32{4.0f * (1.0f + 3.0f * 0x1p-22f), (float)d * 0x1p-140f};
}

__device__ __forceinline__ bool pp_far32(float cc, float D32, PPFar32 f) {
  return cc >= __fmul_ru(f.mul, __fadd_ru(D32, f.abs_));
}

__device__ __forceinline__ double pp_tol(double q, double depth) {
  // (depth) * 2^-53 * q, inflated by 1% to absorb the rounding of this bound
  return depth * 1.1102230246251565e-16 * 1.01 * q;
}

__device__ __forceinline__ double warp_incl_scan(double v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v = __dadd_rn(v, y);
  }
  return v;
}

struct Crossing {
  int t;         // first index whose prefix reaches the cutoff (len: none)
  double q;      // prefix through t (the total when none)
  double qprev;  // prefix before t
};

// Whole warp: prefixes base + v[0] + ... + v[t] of len values, 8 consecutive
// values per lane (sequential within the lane, a shuffle scan across lanes,
// summation depth <= 8 + 5 + 2 per 256 values).
static __device__ Crossing warp_first_crossing(const double *__restrict__ v, int len, double base, double cutoff) {
  constexpr int E = 8;
  const int lane = threadIdx.x & 31;
  for (int r0 = 0; r0 < len; r0 += 32 * E) {
    const int s0 = r0 + lane * E;
    double a[E];
#pragma unroll
    for (int e = 0; e < E; ++e) a[e] = s0 + e < len ? v[s0 + e] : 0.0;
    double run = 0.0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      run = __dadd_rn(run, a[e]);
      a[e] = run;
    }
    const double incl = warp_incl_scan(run);
    const double prev = __shfl_up_sync(0xffffffffu, incl, 1);
    const double off = lane ? __dadd_rn(base, prev) : base;
    int first = E;
    double q = 0.0, qp = 0.0;
#pragma unroll
    for (int e = E - 1; e >= 0; --e) {
      const double qe = __dadd_rn(off, a[e]);
      if (s0 + e < len && qe >= cutoff) {
        first = e;
        q = qe;
        qp = e ? __dadd_rn(off, a[e - 1]) : off;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, first < E);
    if (m) {
      const int L = __ffs(m) - 1;
      Crossing r;
      r.t = __shfl_sync(0xffffffffu, s0 + first, L);
      r.q = __shfl_sync(0xffffffffu, q, L);
      r.qprev = __shfl_sync(0xffffffffu, qp, L);
      return r;
    }
    base = __dadd_rn(base, __shfl_sync(0xffffffffu, incl, 31));
  }
  return Crossing{len, base, base};
}

// Fixed-order block sum (warp shuffle tree, then warps in index order).
// Every thread passes a value; thread 0 returns the total.
template <int kThreads>
__device__ __forceinline__ double block_sum_fixed(double v) {
  __shared__ double ws[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kThreads / 32; ++i) t = __dadd_rn(t, ws[i]);
  return t;
}

// Lower bound (an f32 value) of the real |x_p - x_a|^2 for every earlier seed
// a < j (rows seed_x[a]), one warp per seed, four seeds per pass of the
// kThreads threads; each lane sums its strided terms in order, then a shuffle
// tree (depth m <= d + 5).
//   f32 rows, f32 arithmetic: g = fl(x_p - x_a) is within 2^-24 |x_p - x_a|
//     (exact when subnormal), fl(g^2) within 2^-24 relative or 2^-150, and each
//     addition of nonnegative terms within 2^-24, so the real value is at least
//     (s - d 2^-149)(1 - (d + 10) 2^-23), evaluated with downward rounding.
//   f64 rows, f64 arithmetic: at least s (1 - (d + 16) 2^-52) - d 2^-1068,
//     rounded down to f32.
template <int kThreads, typename T>
__device__ void pp_seed_gaps(const T *__restrict__ xp, int d, const T *__restrict__ seed_x, int j,
                             float *__restrict__ seed_cc) {
  constexpr int kW = kThreads / 32, kQ = 4;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int a0 = w; a0 < j; a0 += kW * kQ) {
    T s[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) s[q] = (T)0;
    for (int t = lane; t < d; t += 32) {
      const T xv = xp[t];
#pragma unroll
      for (int q = 0; q < kQ; ++q) {
        const int a = a0 + q * kW;
        if (a < j) {
          if constexpr (sizeof(T) == 4) {
            const float g = __fsub_rn(xv, seed_x[(int64_t)a * d + t]);
            s[q] = __fadd_rn(s[q], __fmul_rn(g, g));
          } else {
            const double g = __dsub_rn(xv, seed_x[(int64_t)a * d + t]);
            s[q] = __dadd_rn(s[q], __dmul_rn(g, g));
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      T v = s[q];
      float lo;
      if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
        const float rel = 1.0f - (float)(d + 10) * 0x1p-23f;  // exact for d <= 2^13
        lo = __fmul_rd(__fsub_rd(v, (float)d * 0x1p-149f), rel);
      } else {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
        lo = __double2float_rd(__dsub_rn(__dmul_rn(v, 1.0 - (double)(d + 16) * 0x1p-52), (double)d * 0x1p-1068));
      }
      const int a = a0 + q * kW;
      if (lane == 0 && a < j) seed_cc[a] = fmaxf(0.f, lo);
    }
  }
}

}  // namespace sc
