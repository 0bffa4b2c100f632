// Shared preparation kernels of the split-BF16 operands: BF16 halves of
// each row, an f32 upper bound of its norm, and block sums of ||row||^2.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace sc {
namespace {

// ---------------------------------------------------------------------------
// Preparation of the point operand: BF16 halves (row-major, d padded to
// d_pad), an upper bound of ||x|| in f32, and block sums of ||x||^2 in f64.
// One warp per point.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void split2(T v, __nv_bfloat16 &h, __nv_bfloat16 &l);
template <>
__device__ __forceinline__ void split2<float>(float v, __nv_bfloat16 &h, __nv_bfloat16 &l) {
  h = __float2bfloat16_rn(v);
  l = __float2bfloat16_rn(v - __bfloat162float(h));  // v - h is exact in f32
}
template <>
__device__ __forceinline__ void split2<double>(double v, __nv_bfloat16 &h, __nv_bfloat16 &l) {
  h = __double2bfloat16(v);
  l = __double2bfloat16(v - (double)__bfloat162float(h));  // exact in f64
}

template <typename T>
__global__ void __launch_bounds__(256)
prep_x_kernel(const T *__restrict__ x, int64_t n, int64_t n_pad, int d, int d_pad,
              __nv_bfloat16 *__restrict__ xh, __nv_bfloat16 *__restrict__ xl,
              float *__restrict__ xnrm, double *__restrict__ part) {
  __shared__ double ws[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * 8 + w;
  double s = 0.0;
  if (i < n_pad) {
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
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) {
    if (i < n_pad) {
      // sqrt rounded up, then one more f32 ulp: an upper bound of ||x||
      const float r = __fsqrt_ru(__double2float_ru(s));
      xnrm[i] = __uint_as_float(__float_as_uint(r) + 1u);
    }
    ws[w] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < 8; ++q) t += ws[q];
    part[blockIdx.x] = t;
  }
}

// Three BF16 terms h + m + l of v (|v - (h + m + l)| <= 2^-24 |v|).
__device__ __forceinline__ void split3(double v, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
  h = __double2bfloat16(v);
  const double r1 = v - (double)__bfloat162float(h);
  m = __double2bfloat16(r1);
  l = __double2bfloat16(r1 - (double)__bfloat162float(m));
}

// The constant A operand of the norm-folding MMA: 128 rows of 16 BF16
// columns, [1, 1, 1, 0, ..., 0].  Paired with a B operand whose row j holds
// the three BF16 terms of -||c_j||^2 / 2, one extra K=16 step adds
// -||c_j||^2 / 2 to every x.c_j of the accumulator.
__global__ void ones_tile_kernel(__nv_bfloat16 *__restrict__ ones) {
  const int t = threadIdx.x;  // 128 x 16 elements, 16 per thread
  for (int c = 0; c < 16; ++c) ones[t * 16 + c] = __float2bfloat16_rn(c < 3 ? 1.f : 0.f);
}

__global__ void sum_parts_kernel(const double *__restrict__ part, int nparts, double *__restrict__ out) {
  __shared__ double ws[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += part[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    *out = t;
  }
}


}  // namespace
}  // namespace sc
