// Device helpers shared by the k-means++ kernels of the single-problem path
// (exact.cu) and of the batched path (batch.cu): the reference's squared-
// distance term, the f32 far test, and the certified prefix search of the
// seed selection.  Both translation units are compiled with -fmad=false.
#pragma once

#include <cfloat>
#include <climits>

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

// ---------------------------------------------------------------------------
// Exact sequential f64 sum of nonnegative doubles by a whole CTA: the values
// the reference's loops `sum += d[i]` and `cost += d[index]` take, bit for
// bit, in parallel.  While the running sum S stays inside one binade, every
// addition rounds to the same grid q (the binade's ulp): with S = N q,
// S + v rounds to (N + r) q, where r is v / q rounded to an integer; only
// an exact tie depends on S, through the parity of N (ties to even).  So an
// addend is a function of the parity: (grid steps added, parity after), and
// these compose associatively: a CTA scan gives every prefix's N.  The first
// element whose sum leaves the binade (N reaches 2^53) is added with one real
// f64 addition, and the scan resumes after it on the new grid.  Binades only
// grow, so a pass rescans at most one chunk per binade change.
// ---------------------------------------------------------------------------
struct SeqFn {
  unsigned long long d0, d1;  // grid steps added for parity 0 / 1 of N (saturating at 2^62)
  int f0, f1;                 // parity of N after the addend, for parity 0 / 1 before
};
constexpr unsigned long long kSeqCap = 1ull << 62;

__device__ __forceinline__ SeqFn seq_identity() { return SeqFn{0ull, 0ull, 0, 1}; }

__device__ __forceinline__ SeqFn seq_compose(const SeqFn &a, const SeqFn &b) {  // a, then b
  SeqFn r;
  r.d0 = min(a.d0 + (a.f0 ? b.d1 : b.d0), kSeqCap);
  r.d1 = min(a.d1 + (a.f1 ? b.d1 : b.d0), kSeqCap);
  r.f0 = a.f0 ? b.f1 : b.f0;
  r.f1 = a.f1 ? b.f1 : b.f0;
  return r;
}

// The addend v >= 0 on the grid 2^qe.
__device__ __forceinline__ SeqFn seq_elem(double v, int qe) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int ef = (int)((b >> 52) & 0x7ff);
  const unsigned long long M = (b & 0xfffffffffffffull) | (ef ? (1ull << 52) : 0ull);
  const int e = (ef ? ef : 1) - 1075;  // v = M 2^e
  unsigned long long m = 0;
  int cls = 1;  // 0 below half, 1 exact, 2 above half, 3 tie
  if (M != 0) {
    const int s = qe - e;
    if (s <= 0) {
      const int sh = -s;
      m = (sh >= 62 || (M >> (62 - sh)) != 0ull) ? kSeqCap : (M << sh);
    } else if (s >= 64) {
      cls = 0;
    } else {
      m = M >> s;
      const unsigned long long rem = M & ((1ull << s) - 1ull), half = 1ull << (s - 1);
      cls = rem == 0ull ? 1 : (rem < half ? 0 : (rem > half ? 2 : 3));
    }
  }
  SeqFn f;
  if (cls == 3) {  // the result is even whatever the parity before
    f.d0 = m + (m & 1ull);
    f.d1 = m + ((m + 1ull) & 1ull);
    f.f0 = 0;
    f.f1 = 0;
  } else {
    const unsigned long long r = m + (cls == 2 ? 1ull : 0ull);
    f.d0 = r;
    f.d1 = r;
    f.f0 = (int)(r & 1ull);
    f.f1 = (int)((r + 1ull) & 1ull);
  }
  return f;
}

__device__ __forceinline__ SeqFn seq_shfl_up(const SeqFn &f, int o) {
  SeqFn r;
  r.d0 = __shfl_up_sync(0xffffffffu, f.d0, o);
  r.d1 = __shfl_up_sync(0xffffffffu, f.d1, o);
  r.f0 = __shfl_up_sync(0xffffffffu, f.f0, o);
  r.f1 = __shfl_up_sync(0xffffffffu, f.f1, o);
  return r;
}

// Whole CTA of NT threads.  find = false: *sum_out = the sequential sum of
// v[0..n).  find = true: *index_out = the first i whose sequential prefix
// through v[i] is >= cutoff (n when none).
template <int NT>
__device__ void seq_exact_pass(const double *__restrict__ v, int64_t n, bool find, double cutoff, double *sum_out,
                               int64_t *index_out) {
  constexpr int E = 4, NW = NT / 32;
  constexpr int64_t CH = (int64_t)NT * E;
  constexpr unsigned long long kTop = 1ull << 53;
  __shared__ unsigned long long s_d0[NW], s_d1[NW];
  __shared__ int s_f0[NW], s_f1[NW];
  __shared__ double s_S, s_Snew;
  __shared__ long long s_j, s_ovf, s_crs;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) {
    s_S = 0.0;
    s_j = 0;
  }
  __syncthreads();
  int64_t found = -1;
  for (;;) {
    const double S = s_S;
    const int64_t j = s_j;
    if (j >= n) break;
    if (t == 0) {
      s_ovf = LLONG_MAX;
      s_crs = LLONG_MAX;
    }
    const unsigned long long sb = (unsigned long long)__double_as_longlong(S);
    const int ef = (int)((sb >> 52) & 0x7ff);
    const int qe = (ef ? ef : 1) - 1075;
    const unsigned long long N0 = (sb & 0xfffffffffffffull) | (ef ? (1ull << 52) : 0ull);
    const int p0 = (int)(N0 & 1ull);
    const int64_t e0 = j + (int64_t)t * E;
    SeqFn fe[E];
    SeqFn F = seq_identity();
#pragma unroll
    for (int e = 0; e < E; ++e) {
      fe[e] = e0 + e < n ? seq_elem(v[e0 + e], qe) : seq_identity();
      F = seq_compose(F, fe[e]);
    }
    // inclusive warp scan, then the warps' totals in order
    SeqFn G = F;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const SeqFn y = seq_shfl_up(G, o);
      if (lane >= o) G = seq_compose(y, G);
    }
    if (lane == 31) {
      s_d0[w] = G.d0;
      s_d1[w] = G.d1;
      s_f0[w] = G.f0;
      s_f1[w] = G.f1;
    }
    __syncthreads();
    SeqFn P = seq_identity();  // everything before this warp
    for (int q = 0; q < w; ++q) P = seq_compose(P, SeqFn{s_d0[q], s_d1[q], s_f0[q], s_f1[q]});
    SeqFn Gx = seq_shfl_up(G, 1);  // exclusive within the warp
    if (lane == 0) Gx = seq_identity();
    P = seq_compose(P, Gx);
    unsigned long long N = min(N0 + (p0 ? P.d1 : P.d0), kSeqCap);
    int par = p0 ? P.f1 : P.f0;
    long long my_ovf = LLONG_MAX, my_crs = LLONG_MAX;
    unsigned long long n_before = N;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if (e0 + e >= n) break;
      const unsigned long long Ne = min(N + (par ? fe[e].d1 : fe[e].d0), kSeqCap);
      if (Ne >= kTop) {  // this addend leaves the binade
        my_ovf = e0 + e;
        n_before = N;
        break;
      }
      if (find && my_crs == LLONG_MAX && ldexp((double)Ne, qe) >= cutoff) my_crs = e0 + e;
      N = Ne;
      par = par ? fe[e].f1 : fe[e].f0;
    }
    if (my_ovf != LLONG_MAX) atomicMin(&s_ovf, my_ovf);
    if (my_crs != LLONG_MAX) atomicMin(&s_crs, my_crs);
    __syncthreads();
    const long long ovf = s_ovf, crs = s_crs;
    if (ovf != LLONG_MAX && my_ovf == ovf)  // the one real addition of the segment
      s_Snew = __dadd_rn(ldexp((double)n_before, qe), v[ovf]);
    // the sum after the chunk when nothing left the binade
    const int64_t last = min(n, j + CH) - 1;
    if (ovf == LLONG_MAX && e0 <= last && last < e0 + E) s_Snew = ldexp((double)N, qe);
    __syncthreads();
    const double Sn = s_Snew;
    __syncthreads();
    if (find && crs != LLONG_MAX && crs < ovf) { found = crs; break; }
    if (ovf != LLONG_MAX && !(Sn <= DBL_MAX)) {  // the sum overflowed: it stays +inf from here on
      if (find) found = Sn >= cutoff ? ovf : n;
      else if (t == 0) s_S = Sn;
      __syncthreads();
      break;
    }
    if (ovf != LLONG_MAX) {
      if (find && Sn >= cutoff) { found = ovf; break; }
      if (t == 0) {
        s_S = Sn;
        s_j = ovf + 1;
      }
    } else if (t == 0) {
      s_S = Sn;
      s_j = j + CH;
    }
    __syncthreads();
  }
  if (sum_out) *sum_out = s_S;
  if (index_out) *index_out = found < 0 ? n : found;
  __syncthreads();
}

}  // namespace sc
