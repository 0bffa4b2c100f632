// Centroid update and end-of-iteration step of the Lloyd loop.
//
// Cluster sums are accumulated in 128-bit two's-complement fixed point with a
// per-dataset scale 2^scale chosen so that no sum can overflow.  Integer
// addition is associative, so the sums are identical whatever order the
// atomics land in: the result is deterministic and equals the exact sum of
// the (scaled, rounded-to-nearest) inputs, rounded once to f64.  For the
// data sizes served (|x| < 2^E, n points) the quantum is 2^-(126-E-log2 n),
// far below one f64 ulp of any input, so this is at least as accurate as the
// reference's tree-ordered f64 sums (src/algorithm/neighbour/bbd_tree.rs:
// 151-155) and (src/cluster/kmeans.rs:297-303).
#include <float.h>
#include <math.h>

#include <algorithm>
#include <type_traits>

#include "common.cuh"

namespace sc {

__device__ __forceinline__ unsigned __int128 fixed_mag(uint64_t mant, int sh) {
  // mant * 2^sh rounded to an integer (half to even); sh <= 127 - 53.
  if (sh >= 0) return (unsigned __int128)mant << sh;
  if (sh <= -64) return 0;
  const int r = -sh;
  uint64_t q = mant >> r;
  const uint64_t rem = mant & ((1ull << r) - 1ull), half = 1ull << (r - 1);
  if (rem > half || (rem == half && (q & 1ull))) ++q;
  return q;
}

__device__ __forceinline__ unsigned __int128 to_fixed(float v, int scale) {
  const uint32_t b = __float_as_uint(v);
  int e = (int)((b >> 23) & 0xffu);
  uint64_t m = b & 0x7fffffu;
  if (e == 0) e = 1; else m |= 0x800000u;
  unsigned __int128 mag = m ? fixed_mag(m, e - 150 + scale) : 0;
  return (b >> 31) ? (unsigned __int128)0 - mag : mag;
}

__device__ __forceinline__ unsigned __int128 to_fixed(double v, int scale) {
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  int e = (int)((b >> 52) & 0x7ffu);
  uint64_t m = b & 0xfffffffffffffull;
  if (e == 0) e = 1; else m |= 0x10000000000000ull;
  unsigned __int128 mag = m ? fixed_mag(m, e - 1075 + scale) : 0;
  return (b >> 63) ? (unsigned __int128)0 - mag : mag;
}

__device__ __forceinline__ void atomic_add128(Acc128 *a, unsigned __int128 v) {
  const unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)(v >> 64);
  const unsigned long long old = atomicAdd(&a->lo, lo);
  const unsigned long long carry = (old + lo) < old ? 1ull : 0ull;
  const unsigned long long h = hi + carry;
  if (h) atomicAdd(&a->hi, h);
}

// Correctly rounded conversion of a 128-bit two's-complement value * 2^-scale.
__device__ double fixed_to_double(unsigned long long lo, unsigned long long hi, int scale) {
  unsigned __int128 v = ((unsigned __int128)hi << 64) | lo;
  const bool neg = (hi >> 63) != 0;
  if (neg) v = (unsigned __int128)0 - v;
  const uint64_t vh = (uint64_t)(v >> 64), vl = (uint64_t)v;
  double r;
  if (vh == 0) {
    r = __ull2double_rn(vl);
    r = ldexp(r, -scale);
  } else {
    const int lz = __clzll((long long)vh);
    const unsigned __int128 t = v << lz;  // top bit at 127
    uint64_t top = (uint64_t)(t >> 64);
    top |= ((uint64_t)t != 0) ? 1ull : 0ull;  // sticky bit below the rounding point
    r = ldexp(__ull2double_rn(top), 64 - lz - scale);
  }
  return neg ? -r : r;
}

// ---------------------------------------------------------------------------
// K2: sums and counts per cluster.  One warp per point, lane = coordinate:
// coalesced row reads and atomics on adjacent accumulator words.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256)
update_fixed_kernel(const T *__restrict__ x, int64_t n, int d,
                    const int32_t *__restrict__ labels, Acc128 *__restrict__ acc,
                    unsigned long long *__restrict__ cnt, int scale,
                    const LloydState *st) {
  if (st && st->done) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < n; i += nw) {
    const int c = labels[i];
    if (lane == 0) atomicAdd(&cnt[c], 1ull);
    const T *xr = x + i * (int64_t)d;
    Acc128 *ar = acc + (int64_t)c * d;
    for (int j = lane; j < d; j += 32) atomic_add128(&ar[j], to_fixed(xr[j], scale));
  }
}

sc_status launch_update_fixed(int dtype, const void *x, int64_t n, int d,
                              const int32_t *labels, Acc128 *acc,
                              unsigned long long *cnt, int scale,
                              const LloydState *st, cudaStream_t s) {
  if (n == 0) return SC_OK;
  int64_t blocks = (n + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (dtype == SC_F32)
    update_fixed_kernel<float><<<(unsigned)blocks, 256, 0, s>>>((const float *)x, n, d, labels, acc, cnt, scale, st);
  else
    update_fixed_kernel<double><<<(unsigned)blocks, 256, 0, s>>>((const double *)x, n, d, labels, acc, cnt, scale, st);
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// K2, partial form: each CTA owns a contiguous chunk of points.  It sorts the
// chunk's point indices by label in shared memory (32-bit counting sort),
// then each warp sums whole clusters in int64 fixed-point registers (lane =
// feature), with no atomics on the data path, and writes one partial per
// (CTA, cluster, feature).  The scale keeps every partial below 2^63:
// |x| < 2^E, chunk < 2^C points, scale = 62 - E - C.
// ---------------------------------------------------------------------------
// v * 2^scale rounded to the nearest integer (ties to even), integer ALU only
// (a 64-bit float-to-int conversion would run on the FP64 pipe).  The scale
// guarantees |v| * 2^scale < 2^62.  Normal values whose scaled mantissa is an
// integer (the common case) take the short path.
__device__ __noinline__ long long to_fixed64_slow(uint32_t b, int scale) {
  const int e = (int)((b >> 23) & 0xffu);
  const uint32_t m = (b & 0x7fffffu) | (e ? 0x800000u : 0u);
  const int sh = (e ? e : 1) - 150 + scale;
  long long mag;
  if (sh >= 0) {
    mag = (long long)((unsigned long long)m << sh);
  } else if (sh > -25) {
    const int r = -sh;
    const uint32_t q = m >> r, rem = m & ((1u << r) - 1u), half = 1u << (r - 1);
    mag = (long long)(q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u));
  } else {
    mag = 0;  // |v| * 2^scale < 2^-1
  }
  return (b >> 31) ? -mag : mag;
}

// Fast path of the conversion: a normal value whose scaled mantissa is an
// integer shifted left by sh in [0, 30] (exponent field e in [lo, lo + span]),
// so that v * 2^scale = (signed mantissa) * 2^sh is one 32 x 32 -> 64-bit
// multiply-add on the FMA pipe.  The partial-form scales keep sh <= 38 - C
// for chunks of 2^C rows, so chunks of 128 rows or more never leave it.
struct FixedConv {
  uint32_t lo, span;
  int sh0, scale;
};

__device__ __forceinline__ FixedConv fixed_conv(int scale) {
  FixedConv f;
  const int lo = max(1, 150 - scale), hi = 180 - scale;  // sh = e - 150 + scale in [0, 30], e >= 1
  f.lo = hi >= lo ? (uint32_t)lo : 0xffffffffu;
  f.span = hi >= lo ? (uint32_t)(hi - lo) : 0u;
  f.sh0 = lo - 150 + scale;
  f.scale = scale;
  return f;
}

__device__ __forceinline__ void add_fixed64(long long &acc, float v, const FixedConv &f) {
  const uint32_t b = __float_as_uint(v);
  const uint32_t de = ((b >> 23) & 0xffu) - f.lo;
  if (de <= f.span) {
    const int m = (int)((b & 0x7fffffu) | 0x800000u);
    const int sm = (int)b < 0 ? -m : m;
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(acc) : "r"(sm), "r"(1 << ((int)de + f.sh0)));
    return;
  }
  if ((b << 1) == 0u) return;  // +-0
  acc += to_fixed64_slow(b, f.scale);  // subnormal, below the integer grid, or sh > 30: rare
}

// Packed fixed-point form of an f32 value for a given scale, made once per
// dataset: bits 25..31 hold sh = e - 150 + scale in [0, 30] and bits 0..24 the
// signed 25-bit mantissa, so v * 2^scale = mantissa * 2^sh.  sh = 31 marks a
// value outside that form (subnormal, below the integer grid, or sh > 30),
// converted from the f32 value itself.  +-0 packs to 0.
constexpr uint32_t kPackSlow = 31u << 25;

__global__ void pack_fixed_kernel(const float *__restrict__ x, int64_t count, uint32_t *__restrict__ xq, int scale,
                                  unsigned int *__restrict__ slow) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = __float_as_uint(x[i]);
    const int e = (int)((b >> 23) & 0xffu);
    uint32_t q;
    if (e == 0) {
      q = (b << 1) == 0u ? 0u : kPackSlow;
    } else {
      const int sh = e - 150 + scale;
      if (sh < 0 || sh > 30) {
        q = kPackSlow;
      } else {
        const int m = (int)((b & 0x7fffffu) | 0x800000u);
        q = ((uint32_t)sh << 25) | ((uint32_t)((int)b < 0 ? -m : m) & 0x1ffffffu);
      }
    }
    if (q == kPackSlow) atomicAdd(slow, 1u);
    xq[i] = q;
  }
}

// The same sum as add_fixed64 from the packed form: one shift pair and one
// 32 x 32 -> 64-bit multiply-add per value.
// SLOW = false: the dataset has no value outside the packed form (counted
// when it was packed), so no value needs the check.
template <bool SLOW>
__device__ __forceinline__ void add_packed64(long long &acc, uint32_t q, const float *xe, int scale) {
  const uint32_t sh = q >> 25;
  if (!SLOW || sh != 31u) {
    const int sm = ((int)(q << 7)) >> 7;
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(acc) : "r"(sm), "r"(1 << sh));
  } else {
    acc += to_fixed64_slow(__float_as_uint(*xe), scale);
  }
}

// The step updates the persistent totals from its moved rows alone when they
// hold the previous labels' sums and at most mcap rows changed label; else
// the full pass runs.  Every kernel of the step reads the same two values.
__device__ __forceinline__ bool incremental_step(const LloydState *st, int64_t mcap) {
  return st && st->sums_valid && st->moved <= mcap;
}

// Counting sort of a CTA's chunk by label (shared memory): cnt[c] points of
// cluster c, off[c] .. off[c + 1] their positions in idx (chunk-relative rows).
__device__ __forceinline__ void sort_chunk_by_label(const int32_t *__restrict__ labels, int64_t i0, int len, int k,
                                                    int *cnt, int *off, int *cur, int *idx) {
  for (int t = threadIdx.x; t < k; t += blockDim.x) cnt[t] = 0;
  __syncthreads();
  for (int t = threadIdx.x; t < len; t += blockDim.x) atomicAdd(&cnt[labels[i0 + t]], 1);
  __syncthreads();
  if (threadIdx.x < 32) {  // exclusive scan of the counts by one warp
    int carry = 0;
    for (int base = 0; base < k; base += 32) {
      const int c = base + threadIdx.x;
      const int v = c < k ? cnt[c] : 0;
      int incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)threadIdx.x >= o) incl += y;
      }
      if (c < k) { off[c] = carry + incl - v; cur[c] = carry + incl - v; }
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (threadIdx.x == 0) off[k] = carry;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < len; t += blockDim.x) idx[atomicAdd(&cur[labels[i0 + t]], 1)] = t;
}

// K2, balanced partial form: after the counting sort, warp w sums the w-th
// equal slice of the label-sorted rows (lane = feature) in int64 registers
// and flushes them into a k x d shared accumulator whenever the cluster
// changes, so every warp gathers the same number of rows whatever the
// cluster sizes.  Same partials as update_sorted_kernel.
template <int MAXJ, bool PACKED, bool SLOW>
__global__ void __launch_bounds__(1024)
update_balanced_kernel(const float *__restrict__ x, const uint32_t *__restrict__ xq, int64_t n, int d,
                       const int32_t *__restrict__ labels, int k, long long *__restrict__ part,
                       unsigned int *__restrict__ cpart, int scale, const LloydState *st, int64_t mcap) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (st && (st->done || incremental_step(st, mcap))) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  unsigned long long *acc = reinterpret_cast<unsigned long long *>(smraw);  // k x d
  const int kd = k * d;
  int *cnt = reinterpret_cast<int *>(acc + kd);  // k
  int *off = cnt + k;                            // k + 1
  int *cur = off + k + 1;                        // k
  int *idx = cur + k;                            // chunk
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  const int len = i1 > i0 ? (int)(i1 - i0) : 0;
  for (int t = threadIdx.x; t < kd; t += blockDim.x) acc[t] = 0ull;
  sort_chunk_by_label(labels, i0, len, k, cnt, off, cur, idx);
  for (int t = threadIdx.x; t < k; t += blockDim.x) cpart[(size_t)blockIdx.x * k + t] = (unsigned int)cnt[t];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  constexpr int kRows = (PACKED && MAXJ == 1) ? 12 : 16 / MAXJ;  // rows in flight per warp
  const FixedConv fc = fixed_conv(scale);
  const int seg = (len + nw - 1) / nw;
  const int s_begin = min(len, w * seg), s_end = min(len, s_begin + seg);
  if (s_begin < s_end) {
    int lo = 0, hi = k - 1;  // cluster of position s_begin: the largest c with off[c] <= s_begin
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= s_begin) lo = mid; else hi = mid - 1;
    }
    int c = lo, next = off[lo + 1];
    long long a[MAXJ];
#pragma unroll
    for (int q = 0; q < MAXJ; ++q) a[q] = 0;
    for (int s = s_begin; s < s_end; s += kRows) {
      using E = typename std::conditional<PACKED, uint32_t, float>::type;
      E v[kRows][MAXJ];
      int rt[kRows];  // chunk-relative rows
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        const bool ok = s + r < s_end;
        rt[r] = ok ? idx[s + r] : 0;
        const int64_t ro = (i0 + rt[r]) * (int64_t)d;
        if constexpr (PACKED) {  // lane = features MAXJ * lane ... + MAXJ - 1, one vector load
          const bool live = ok && lane * MAXJ < d;
          if constexpr (MAXJ == 4) {
            const uint4 t = live ? __ldg(reinterpret_cast<const uint4 *>(xq + ro) + lane) : make_uint4(0, 0, 0, 0);
            v[r][0] = t.x; v[r][1] = t.y; v[r][2] = t.z; v[r][3] = t.w;
          } else if constexpr (MAXJ == 2) {
            const uint2 t = live ? __ldg(reinterpret_cast<const uint2 *>(xq + ro) + lane) : make_uint2(0, 0);
            v[r][0] = t.x; v[r][1] = t.y;
          } else {
            v[r][0] = live ? __ldg(xq + ro + lane) : 0u;
          }
        } else {
#pragma unroll
          for (int q = 0; q < MAXJ; ++q) {
            const int j = lane + 32 * q;
            v[r][q] = (ok && j < d) ? __ldg(x + ro + j) : 0.f;
          }
        }
      }
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        if (s + r >= s_end) break;
        while (s + r >= next) {  // cluster boundary: flush
#pragma unroll
          for (int q = 0; q < MAXJ; ++q) {
            const int j = PACKED ? lane * MAXJ + q : lane + 32 * q;
            if (j < d && a[q] != 0) atomicAdd(acc + c * d + j, (unsigned long long)a[q]);
            a[q] = 0;
          }
          ++c;
          next = off[c + 1];
        }
#pragma unroll
        for (int q = 0; q < MAXJ; ++q) {
          if constexpr (PACKED)
            add_packed64<SLOW>(a[q], v[r][q], x + (i0 + rt[r]) * (int64_t)d + lane * MAXJ + q, scale);
          else
            add_fixed64(a[q], v[r][q], fc);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < MAXJ; ++q) {
      const int j = PACKED ? lane * MAXJ + q : lane + 32 * q;
      if (j < d && a[q] != 0) atomicAdd(acc + c * d + j, (unsigned long long)a[q]);
    }
  }
  __syncthreads();
  long long *pc = part + (size_t)blockIdx.x * kd;
  for (int t = threadIdx.x; t < kd; t += blockDim.x) pc[t] = (long long)acc[t];
}

template <typename T, int MAXJ>
__global__ void __launch_bounds__(1024)
update_sorted_kernel(const T *__restrict__ x, int64_t n, int d, const int32_t *__restrict__ labels, int k,
                     long long *__restrict__ part, unsigned int *__restrict__ cpart, int scale,
                     const LloydState *st, int64_t mcap) {
  if (st && (st->done || incremental_step(st, mcap))) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  int *cnt = reinterpret_cast<int *>(smraw);  // k
  int *off = cnt + k;                         // k + 1
  int *cur = off + k + 1;                     // k
  int *idx = cur + k;                         // chunk
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  const int len = i1 > i0 ? (int)(i1 - i0) : 0;
  sort_chunk_by_label(labels, i0, len, k, cnt, off, cur, idx);
  for (int t = threadIdx.x; t < k; t += blockDim.x) cpart[(size_t)blockIdx.x * k + t] = (unsigned int)cnt[t];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  constexpr int kRows = MAXJ >= 16 ? 1 : 16 / MAXJ;  // rows in flight per warp (memory-level parallelism)
  const FixedConv fc = fixed_conv(scale);
  for (int c = w; c < k; c += nw) {
    long long acc[MAXJ];
#pragma unroll
    for (int q = 0; q < MAXJ; ++q) acc[q] = 0;
    const int s0 = off[c], s1 = off[c + 1];
    for (int s = s0; s < s1; s += kRows) {
      T v[kRows][MAXJ];
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        const bool ok = s + r < s1;
        const T *xr = x + (i0 + (ok ? idx[s + r] : 0)) * (int64_t)d;
#pragma unroll
        for (int q = 0; q < MAXJ; ++q) {
          const int j = lane + 32 * q;
          v[r][q] = (ok && j < d) ? __ldg(xr + j) : T(0);
        }
      }
#pragma unroll
      for (int r = 0; r < kRows; ++r)
#pragma unroll
        for (int q = 0; q < MAXJ; ++q) add_fixed64(acc[q], v[r][q], fc);
    }
    long long *pc = part + ((size_t)blockIdx.x * k + c) * d;
#pragma unroll
    for (int q = 0; q < MAXJ; ++q) {
      const int j = lane + 32 * q;
      if (j < d) pc[j] = acc[q];
    }
  }
}

// New centroids from the per-CTA partials.  A block handles 32 (cluster,
// feature) elements with 8 threads each; thread g adds the partials b = g
// (mod 8) exactly in 128 bits, the 8 sums meet in shared memory.  Also the
// distortion-identity term n_c c_j^2 - 2 c_j S_j of the element (with the
// centroid used for the assignment); terms[b] is block b's sum of them.
__global__ void __launch_bounds__(256)
finalize_partials_kernel(const long long *__restrict__ part, const unsigned int *__restrict__ cpart,
                         int nparts, int k, double *__restrict__ cent, int64_t *__restrict__ sizes, int d,
                         int scale, double *__restrict__ terms, int empty_nan, const LloydState *st,
                         Acc128 *__restrict__ tot, unsigned long long *__restrict__ tcnt, int64_t mcap) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (st && (st->done || incremental_step(st, mcap))) return;
  __shared__ unsigned long long s_lo[8][32], s_hi[8][32];
  __shared__ unsigned long long s_cn[8][32];
  const int64_t kd = (int64_t)k * d;
  const int e = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int64_t t = (int64_t)blockIdx.x * 32 + e;
  unsigned __int128 v = 0;
  unsigned long long cn = 0;
  if (t < kd) {
    const int c = (int)(t / d);
    for (int b = g; b < nparts; b += 8) {
      v += (unsigned __int128)(__int128)part[b * kd + t];
      cn += cpart[(size_t)b * k + c];
    }
  }
  s_lo[g][e] = (unsigned long long)v;
  s_hi[g][e] = (unsigned long long)(v >> 64);
  s_cn[g][e] = cn;
  __syncthreads();
  if (g != 0) return;
  double term = 0.0;
  if (t < kd) {
    for (int q = 1; q < 8; ++q) {
      v += ((unsigned __int128)s_hi[q][e] << 64) | s_lo[q][e];
      cn += s_cn[q][e];
    }
    const int c = (int)(t / d);
    if (tot) {  // the totals of these labels, for the next step's incremental path
      tot[t].lo = (unsigned long long)v;
      tot[t].hi = (unsigned long long)(v >> 64);
      if (t % d == 0) tcnt[c] = cn;
    }
    const double sum = fixed_to_double((unsigned long long)v, (unsigned long long)(v >> 64), scale);
    const double dn = (double)cn;
    const double old = cent[t];
    term = __fma_rn(old, __fma_rn(dn, old, -2.0 * sum), 0.0);
    if (cn > 0) cent[t] = __ddiv_rn(sum, dn);
    else if (empty_nan) cent[t] = __longlong_as_double(0x7ff8000000000000ll);
    if (sizes && t % d == 0) sizes[c] = (int64_t)cn;
  }
  if (terms) {  // the block's 32 terms summed here: the scalar step adds one value per block
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) term += __shfl_down_sync(0xffffffffu, term, o);
    if (e == 0) terms[blockIdx.x] = term;
  }
}

// ---------------------------------------------------------------------------
// Incremental path of a step.  label_diff_kernel lists the rows whose label
// differs from the one the totals were summed for (and records the new one);
// moved_rows_kernel moves each listed row's fixed-point values from its old
// cluster's totals to its new one's; finalize_total_kernel makes the
// centroids and the distortion terms from the totals, element for element
// and block for block as finalize_partials_kernel does, so both paths give
// the same bits.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
label_diff_kernel(const int32_t *__restrict__ labels, int32_t *__restrict__ prev, int64_t n,
                  int64_t *__restrict__ mrows, int32_t *__restrict__ mold, int64_t mcap, LloydState *st) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (st->done) return;
  const int lane = threadIdx.x & 31;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = i0 + threadIdx.x;
    int32_t l = 0, p = 0;
    if (i < n) {
      l = labels[i];
      p = prev[i];
    }
    const bool moved = i < n && l != p;
    const unsigned m = __ballot_sync(0xffffffffu, moved);
    if (!m) continue;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd((unsigned long long *)&st->moved, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (moved) {
      prev[i] = l;
      const int64_t pos = (int64_t)base + __popc(m & ((1u << lane) - 1u));
      if (pos < mcap) {
        mrows[pos] = i;
        mold[pos] = p;
      }
    }
  }
}

__device__ __forceinline__ void atomic_sub128(Acc128 *a, unsigned __int128 v) {
  atomic_add128(a, (unsigned __int128)0 - v);
}

// One warp per moved row, lane = feature.
__global__ void __launch_bounds__(256)
moved_rows_kernel(const float *__restrict__ x, int d, const int32_t *__restrict__ labels,
                  const int64_t *__restrict__ mrows, const int32_t *__restrict__ mold, int64_t mcap,
                  Acc128 *__restrict__ tot, unsigned long long *__restrict__ tcnt, int scale, const LloydState *st) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (st->done || !incremental_step(st, mcap)) return;
  const int64_t nm = st->moved;
  const int lane = threadIdx.x & 31;
  for (int64_t m = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; m < nm;
       m += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t i = mrows[m];
    const int cn = labels[i], co = mold[m];
    const float *xr = x + i * (int64_t)d;
    for (int j = lane; j < d; j += 32) {
      const long long v = to_fixed64_slow(__float_as_uint(xr[j]), scale);
      if (v) {
        const unsigned __int128 w = (unsigned __int128)(__int128)v;
        atomic_add128(&tot[(int64_t)cn * d + j], w);
        atomic_sub128(&tot[(int64_t)co * d + j], w);
      }
    }
    if (lane == 0) {
      atomicAdd(&tcnt[cn], 1ull);
      atomicAdd(&tcnt[co], ~0ull);  // minus one
    }
  }
}

__global__ void __launch_bounds__(32)
finalize_total_kernel(const Acc128 *__restrict__ tot, const unsigned long long *__restrict__ tcnt, int k,
                      double *__restrict__ cent, int64_t *__restrict__ sizes, int d, int scale,
                      double *__restrict__ terms, LloydState *st, int64_t mcap) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (st->done || !incremental_step(st, mcap)) return;
  const int64_t kd = (int64_t)k * d;
  const int e = threadIdx.x;
  const int64_t t = (int64_t)blockIdx.x * 32 + e;
  double term = 0.0;
  if (t < kd) {
    const int c = (int)(t / d);
    const unsigned long long cn = tcnt[c];
    const double sum = fixed_to_double(tot[t].lo, tot[t].hi, scale);
    const double dn = (double)cn;
    const double old = cent[t];
    term = __fma_rn(old, __fma_rn(dn, old, -2.0 * sum), 0.0);
    if (cn > 0) cent[t] = __ddiv_rn(sum, dn);
    if (sizes && t % d == 0) sizes[c] = (int64_t)cn;
  }
  if (terms) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) term += __shfl_down_sync(0xffffffffu, term, o);
    if (e == 0) terms[blockIdx.x] = term;
  }
  if (blockIdx.x == 0 && e == 0) st->incremental_steps += 1;
}

// ---------------------------------------------------------------------------
// New centroids (kmeans.rs:297-303: c = sums / size when size > 0, else the
// old centroid; the initial means of :288-292 divide unconditionally, so an
// empty cluster becomes NaN there: empty_nan = 1).  One block per cluster.
// Also writes the per-cluster term of the distortion identity
//   sum_{i in c} ||x_i - c||^2 = sum ||x_i||^2 - 2 c.S_c + n_c ||c||^2
// (with the centroid used for the assignment), then clears the accumulators.
// ---------------------------------------------------------------------------
constexpr int kFinThreads = 128;

__global__ void __launch_bounds__(kFinThreads)
finalize_centroids_kernel(Acc128 *__restrict__ acc, unsigned long long *__restrict__ cnt,
                          double *__restrict__ cent, int64_t *__restrict__ sizes,
                          int d, int scale, double *__restrict__ cluster_terms,
                          int empty_nan, const LloydState *st) {
  if (st && st->done) return;
  __shared__ double ws[kFinThreads / 32];
  const int c = blockIdx.x;
  const unsigned long long cn = cnt[c];
  const double dn = (double)cn;
  double term = 0.0;
  for (int j = threadIdx.x; j < d; j += kFinThreads) {
    const int64_t t = (int64_t)c * d + j;
    const double s = fixed_to_double(acc[t].lo, acc[t].hi, scale);
    const double old = cent[t];
    term = __fma_rn(old, __fma_rn(dn, old, -2.0 * s), term);
    if (cn > 0) cent[t] = __ddiv_rn(s, dn);
    else if (empty_nan) cent[t] = __longlong_as_double(0x7ff8000000000000ll);
    acc[t].lo = 0ull;
    acc[t].hi = 0ull;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) term += __shfl_down_sync(0xffffffffu, term, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = term;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tt = 0.0;
    for (int w = 0; w < kFinThreads / 32; ++w) tt += ws[w];
    if (cluster_terms) cluster_terms[c] = tt;
    if (sizes) sizes[c] = (int64_t)cn;
    cnt[c] = 0ull;
  }
}

sc_status launch_finalize_centroids(Acc128 *acc, unsigned long long *cnt,
                                    double *cent, int64_t *sizes, int k, int d,
                                    int scale, double *cluster_terms,
                                    int empty_nan, const LloydState *st,
                                    cudaStream_t s) {
  finalize_centroids_kernel<<<k, kFinThreads, 0, s>>>(acc, cnt, cent, sizes, d, scale, cluster_terms, empty_nan, st);
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// Distortion of the step (fixed-order sum of the block partials, or the
// identity above) and the break rule of kmeans.rs:305-309:
//   if distortion <= dist { break } else { distortion = dist }.
// ---------------------------------------------------------------------------
constexpr int kScalarThreads = 1024;

__global__ void __launch_bounds__(kScalarThreads)
finalize_scalar_kernel(const double *__restrict__ part, int nparts,
                       const double *__restrict__ cluster_terms, int64_t k,
                       const double *__restrict__ xnorm_total, LloydState *st) {
  pdl_release_dependents();  // launched as a programmatic dependent in the Lloyd step
  pdl_wait_prerequisite();
  if (st->done) return;
  __shared__ double ws[kScalarThreads / 32];
  const double *a = part ? part : cluster_terms;
  const int64_t cnt = part ? (int64_t)nparts : k;
  double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;  // four loads in flight per thread
  int64_t i = threadIdx.x;
  for (; i + 3 * kScalarThreads < cnt; i += 4 * kScalarThreads) {
    v0 += a[i];
    v1 += a[i + kScalarThreads];
    v2 += a[i + 2 * kScalarThreads];
    v3 += a[i + 3 * kScalarThreads];
  }
  for (; i < cnt; i += kScalarThreads) v0 += a[i];
  double v = (v0 + v1) + (v2 + v3);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x != 0) return;
  double dist = 0.0;
  for (int w = 0; w < kScalarThreads / 32; ++w) dist += ws[w];
  if (!part) dist += *xnorm_total;
  st->iters += 1;
  st->last_dist = dist;
  if (st->stop && st->distortion <= dist) st->done = 1;
  else st->distortion = dist;
  st->sums_valid = 1;  // either path left the totals of this step's labels
  st->moved = 0;
}

sc_status launch_finalize_scalar(const double *part, int nparts,
                                 const double *cluster_terms, int64_t k,
                                 const double *xnorm_total, LloydState *st,
                                 cudaStream_t s) {
  SC_TRY(launch_pdl(finalize_scalar_kernel, 1, kScalarThreads, 0, s, part, nparts, cluster_terms, k, xnorm_total, st));
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// Helpers: max |x| as the bit pattern of a non-negative double (NaN / inf
// map above every finite value), and a column-major to row-major copy.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void absmax_kernel(const T *__restrict__ x, int64_t count,
                              unsigned long long *__restrict__ out) {
  unsigned long long best = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double a = fabs((double)x[i]);
    unsigned long long b = (unsigned long long)__double_as_longlong(a);
    if (a != a) b = 0x7ff8000000000000ull;
    best = best > b ? best : b;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_down_sync(0xffffffffu, best, o);
    best = best > other ? best : other;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

sc_status launch_absmax(int dtype, const void *x, int64_t count,
                        unsigned long long *out_bits, cudaStream_t s) {
  SC_CUDA(cudaMemsetAsync(out_bits, 0, sizeof(unsigned long long), s));
  if (count == 0) return SC_OK;
  int64_t blocks = (count + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (dtype == SC_F32)
    absmax_kernel<float><<<(unsigned)blocks, 256, 0, s>>>((const float *)x, count, out_bits);
  else
    absmax_kernel<double><<<(unsigned)blocks, 256, 0, s>>>((const double *)x, count, out_bits);
  SC_LAUNCHED();
  return SC_OK;
}

template <typename T>
__global__ void to_row_major_kernel(const T *__restrict__ src, int64_t n, int64_t d,
                                    int64_t ld, T *__restrict__ dst) {
  __shared__ T tile[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {  // read: column j0+r, rows i0+tx
    const int64_t i = i0 + threadIdx.x, j = j0 + r;
    if (i < n && j < d) tile[r][threadIdx.x] = src[j * ld + i];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {  // write: row i0+r, columns j0+tx
    const int64_t i = i0 + r, j = j0 + threadIdx.x;
    if (i < n && j < d) dst[i * d + j] = tile[threadIdx.x][r];
  }
}

sc_status launch_to_row_major(int dtype, const void *src, int64_t n, int64_t d,
                              int64_t ld, void *dst, cudaStream_t s) {
  if (n == 0 || d == 0) return SC_OK;
  dim3 grid((unsigned)((n + 31) / 32), (unsigned)((d + 31) / 32)), block(32, 8);
  if (dtype == SC_F32)
    to_row_major_kernel<float><<<grid, block, 0, s>>>((const float *)src, n, d, ld, (float *)dst);
  else
    to_row_major_kernel<double><<<grid, block, 0, s>>>((const double *)src, n, d, ld, (double *)dst);
  SC_LAUNCHED();
  return SC_OK;
}

}  // namespace sc

namespace sc {

static int ceil_log2(int64_t v) {
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}

UpdatePlan update_plan(int dtype, int64_t n, int d, int k, double absmax, int num_sms) {
  UpdatePlan p;
  int e = 0;
  if (absmax > 0) frexp(absmax, &e);  // |x| < 2^e
  int grid = num_sms;
  int64_t chunk = (n + grid - 1) / grid;
  if (chunk > 40000) {  // keep the per-CTA index list in shared memory
    grid = (int)((n + 39999) / 40000);
    chunk = (n + grid - 1) / grid;
  }
  const size_t smem = (size_t)(3 * k + 1 + chunk) * 4;
  const size_t part_bytes = (size_t)grid * k * d * sizeof(long long);
  if (dtype == SC_F32 && d <= 256 && smem <= 200 * 1024 && part_bytes <= ((size_t)512 << 20) && n > 0) {
    p.mode = 1;
    p.grid = grid;
    p.smem = smem;
    p.scale = 62 - e - ceil_log2(chunk + 1);
    if (p.scale > 160) p.scale = 160;  // values below 2^-160 contribute 0
    return p;
  }
  p.mode = 0;
  p.scale = 125 - e - ceil_log2(n + 1);
  return p;
}

sc_status update_alloc(UpdateBuf *u, int dtype, int64_t n, int d, int k, double absmax, int num_sms,
                       cudaStream_t s) {
  update_free(u, s);
  const UpdatePlan p = update_plan(dtype, n, d, k, absmax, num_sms);
  u->mode = p.mode;
  u->scale = p.scale;
  if (p.mode == 1) {
    u->grid = p.grid;
    u->threads = 1024;
    u->smem = p.smem;
    const size_t bal = p.smem + (size_t)k * d * sizeof(long long);
    u->balanced_smem = (d <= 128 && bal <= 200 * 1024) ? bal : 0;
    SC_TRY(dalloc(&u->part, (size_t)p.grid * k * d, s));
    SC_TRY(dalloc(&u->cpart, (size_t)p.grid * k, s));
    // incremental sums: totals, the labels they hold, the moved-row list
    u->mcap = std::min<int64_t>(n, n / 32 + 1);
    SC_TRY(dalloc(&u->tot, (size_t)k * d, s));
    SC_TRY(dalloc(&u->tcnt, (size_t)k, s));
    SC_TRY(dalloc(&u->prev, (size_t)n, s));
    SC_TRY(dalloc(&u->mrows, (size_t)u->mcap, s));
    SC_TRY(dalloc(&u->mold, (size_t)u->mcap, s));
    return SC_OK;
  }
  SC_TRY(dalloc(&u->acc, (size_t)k * d, s));
  SC_TRY(dalloc(&u->cnt, (size_t)k, s));
  SC_CUDA(cudaMemsetAsync(u->acc, 0, (size_t)k * d * sizeof(Acc128), s));
  SC_CUDA(cudaMemsetAsync(u->cnt, 0, (size_t)k * sizeof(unsigned long long), s));
  return SC_OK;
}

void update_free(UpdateBuf *u, cudaStream_t s) {
  dfree(u->tot, s);
  dfree(u->tcnt, s);
  dfree(u->prev, s);
  dfree(u->mrows, s);
  dfree(u->mold, s);
  dfree(u->xq, s);
  dfree(u->acc, s);
  dfree(u->cnt, s);
  dfree(u->part, s);
  dfree(u->cpart, s);
  *u = UpdateBuf();
}

template <int MAXJ>
static sc_status launch_balanced(const UpdateBuf *u, const float *x, int64_t n, int d, const int32_t *labels, int k,
                                 const LloydState *st, cudaStream_t s) {
  const bool packed = u->xq && u->xq_src == (const void *)x && d % MAXJ == 0;
  auto kern = !packed ? update_balanced_kernel<MAXJ, false, false>
              : u->xq_slow ? update_balanced_kernel<MAXJ, true, true> : update_balanced_kernel<MAXJ, true, false>;
  SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)u->balanced_smem));
  SC_TRY(launch_pdl(kern, u->grid, 1024, u->balanced_smem, s, x, u->xq, n, d, labels, k, u->part, u->cpart, u->scale,
                    st, u->mcap));
  SC_LAUNCHED();
  return SC_OK;
}

sc_status update_pack(UpdateBuf *u, const float *x, int64_t n, int d, cudaStream_t s) {
  if (u->mode != 1 || !u->balanced_smem || n == 0) return SC_OK;
  if (!u->xq) SC_TRY(dalloc(&u->xq, (size_t)n * d, s));
  const int64_t count = n * d;
  unsigned int *slow = nullptr;
  SC_TRY(dalloc(&slow, 1, s));
  SC_CUDA(cudaMemsetAsync(slow, 0, sizeof(unsigned int), s));
  pack_fixed_kernel<<<(int)std::min<int64_t>((count + 255) / 256, 65536), 256, 0, s>>>(x, count, u->xq, u->scale,
                                                                                     slow);
  SC_LAUNCHED();
  unsigned int hs = 0;
  SC_CUDA(cudaMemcpyAsync(&hs, slow, sizeof hs, cudaMemcpyDeviceToHost, s));
  SC_CUDA(cudaStreamSynchronize(s));
  dfree(slow, s);
  u->xq_slow = hs != 0;
  u->xq_src = x;
  return SC_OK;
}

template <int MAXJ>
static sc_status launch_sorted(const UpdateBuf *u, const float *x, int64_t n, int d, const int32_t *labels, int k,
                               const LloydState *st, cudaStream_t s) {
  auto kern = update_sorted_kernel<float, MAXJ>;
  SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)u->smem));
  kern<<<u->grid, u->threads, u->smem, s>>>(x, n, d, labels, k, u->part, u->cpart, u->scale, st, u->mcap);
  SC_LAUNCHED();
  return SC_OK;
}

sc_status launch_update(const UpdateBuf *u, int dtype, const void *x, int64_t n, int d,
                        const int32_t *labels, int k, const LloydState *st, cudaStream_t s) {
  if (n == 0) return SC_OK;
  if (u->mode == 0) return launch_update_fixed(dtype, x, n, d, labels, u->acc, u->cnt, u->scale, st, s);
  if (dtype != SC_F32) {  // the partial form scales f32 values exactly with one FMUL
    set_error("internal: partial update form needs f32 data");
    return SC_ERR_INTERNAL;
  }
  const float *xf = (const float *)x;
  // a Lloyd step (st set): the rows that changed label, then the full pass or
  // the moved rows, whichever the step's count selects on the device
  LloydState *ms = const_cast<LloydState *>(st);
  const int sms = u->grid > 0 ? u->grid : 1;
  if (ms) {
    SC_TRY(launch_pdl(label_diff_kernel, sms * 8, 256, 0, s, labels, u->prev, n, u->mrows, u->mold, u->mcap, ms));
    SC_LAUNCHED();
  }
  if (u->balanced_smem) {
    if (d <= 32) SC_TRY(launch_balanced<1>(u, xf, n, d, labels, k, st, s));
    else if (d <= 64) SC_TRY(launch_balanced<2>(u, xf, n, d, labels, k, st, s));
    else SC_TRY(launch_balanced<4>(u, xf, n, d, labels, k, st, s));
  } else {
    if (d <= 32) SC_TRY(launch_sorted<1>(u, xf, n, d, labels, k, st, s));
    else if (d <= 64) SC_TRY(launch_sorted<2>(u, xf, n, d, labels, k, st, s));
    else if (d <= 128) SC_TRY(launch_sorted<4>(u, xf, n, d, labels, k, st, s));
    else SC_TRY(launch_sorted<8>(u, xf, n, d, labels, k, st, s));
  }
  if (ms) {
    SC_TRY(launch_pdl(moved_rows_kernel, sms * 4, 256, 0, s, xf, d, labels, u->mrows, u->mold, u->mcap, u->tot,
                      u->tcnt, u->scale, ms));
    SC_LAUNCHED();
  }
  return SC_OK;
}

sc_status update_mark_sums(const UpdateBuf *u, const int32_t *labels, int64_t n, LloydState *st, cudaStream_t s) {
  if (u->mode != 1 || !u->prev || n == 0) return SC_OK;
  SC_CUDA(cudaMemcpyAsync(u->prev, labels, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  static const int32_t one = 1;
  static const int64_t zero = 0;
  SC_CUDA(cudaMemcpyAsync(&st->sums_valid, &one, sizeof one, cudaMemcpyHostToDevice, s));
  SC_CUDA(cudaMemcpyAsync(&st->moved, &zero, sizeof zero, cudaMemcpyHostToDevice, s));
  return SC_OK;
}

sc_status launch_finalize(const UpdateBuf *u, double *cent, int64_t *sizes, int k, int d,
                          double *terms, int empty_nan, const LloydState *st, cudaStream_t s) {
  if (u->mode == 0)
    return launch_finalize_centroids(u->acc, u->cnt, cent, sizes, k, d, u->scale, terms, empty_nan, st, s);
  const int64_t kd = (int64_t)k * d;
  const int blocks = (int)((kd + 31) / 32);
  SC_TRY(launch_pdl(finalize_partials_kernel, blocks, 256, 0, s, u->part, u->cpart, u->grid, k, cent, sizes, d,
                    u->scale, terms, empty_nan, st, u->tot, u->tcnt, u->mcap));
  SC_LAUNCHED();
  if (st) {
    SC_TRY(launch_pdl(finalize_total_kernel, blocks, 32, 0, s, u->tot, u->tcnt, k, cent, sizes, d, u->scale, terms,
                      const_cast<LloydState *>(st), u->mcap));
    SC_LAUNCHED();
  }
  return SC_OK;
}

}  // namespace sc
