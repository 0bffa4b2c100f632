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
                       const double *__restrict__ cluster_terms, int k,
                       const double *__restrict__ xnorm_total, LloydState *st) {
  if (st->done) return;
  __shared__ double ws[kScalarThreads / 32];
  double v = 0.0;
  if (part) {
    for (int i = threadIdx.x; i < nparts; i += kScalarThreads) v += part[i];
  } else {
    for (int i = threadIdx.x; i < k; i += kScalarThreads) v += cluster_terms[i];
  }
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
}

sc_status launch_finalize_scalar(const double *part, int nparts,
                                 const double *cluster_terms, int k,
                                 const double *xnorm_total, LloydState *st,
                                 cudaStream_t s) {
  finalize_scalar_kernel<<<1, kScalarThreads, 0, s>>>(part, nparts, cluster_terms, k, xnorm_total, st);
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
