// Exact reference squared distances of f32 rows without FP64 instructions.
#pragma once

#include <stdint.h>

namespace sc {

// Squared distance of the reference (src/metrics/distance/euclidian.rs:56-63)
// for f32 rows: terms q_t = fl32((a_t - b_t)^2), summed in f64 from t = 0,
// reproduced without FP64 instructions.  Every term is an integer in units of
// 2^(emin - 150) (emin: the smallest exponent among the nonzero terms).
// While the exponents span at most 38 - ceil(log2 d), every term is below
// 2^(62 - ceil(log2 d)), so the running sum S is an exact 64-bit integer below
// 2^63; after each term it is rounded to 53 significant bits (nearest, ties to
// even) exactly as the f64 addition rounds.  A wider span (or inf/NaN) returns
// false and the caller runs the FP64 sequence.

// d <= 32: each pass streams the rows in two chunks of 16 terms with the
// chunk's loads issued together (the second pass hits L1).
__device__ __forceinline__ float sq_term32(const float *__restrict__ a, const float *__restrict__ b, int t, int d) {
  const float r = t < d ? __fsub_rn(__ldg(a + t), __ldg(b + t)) : 0.f;
  return __fmul_rn(r, r);
}

__device__ __forceinline__ bool sqd_seq_f32_d32(const float *__restrict__ a, const float *__restrict__ b, int d,
                                                int lg_d, double &out) {
  int emin = 256, emax = 0;
#pragma unroll
  for (int c = 0; c < 32; c += 16) {
    float q[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) q[t] = sq_term32(a, b, c + t, d);
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const uint32_t u = __float_as_uint(q[t]);
      if (u != 0u) {
        const int e = max((int)(u >> 23), 1);
        emin = min(emin, e);
        emax = max(emax, e);
      }
    }
  }
  if (emin == 256) { out = 0.0; return true; }
  if (emax >= 255 || emax - emin > 38 - lg_d) return false;
  unsigned long long S = 0;
#pragma unroll
  for (int c = 0; c < 32; c += 16) {
    float q[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) q[t] = sq_term32(a, b, c + t, d);
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const uint32_t u = __float_as_uint(q[t]);
      const int e = (int)(u >> 23);
      const uint32_t m = (u & 0x7fffffu) | (e ? 0x800000u : 0u);
      S += u ? (unsigned long long)m << (max(e, 1) - emin) : 0ull;  // stays below 2^63
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
  const unsigned long long mant = pbit <= 52 ? S << (52 - pbit) : S >> (pbit - 52);  // exact: S has <= 53 significant bits
  const int ex = pbit + emin - 150 + 1023;
  out = __longlong_as_double((long long)(((unsigned long long)ex << 52) | (mant & 0xfffffffffffffull)));
  return true;
}

// Any d, each pass in chunks of 16 terms with the chunk's loads issued
// together.  a and b may point to global or shared memory.
template <typename PA, typename PB>
__device__ __forceinline__ bool sqd_seq_f32(PA a, PB b, int d, int lg_d, double &out) {
  int emin = 256, emax = 0;
  for (int c = 0; c < d; c += 16) {
    float q[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const float r = c + t < d ? __fsub_rn(a[c + t], b[c + t]) : 0.f;
      q[t] = __fmul_rn(r, r);
    }
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const uint32_t u = __float_as_uint(q[t]);
      if (u != 0u) {
        const int e = max((int)(u >> 23), 1);
        emin = min(emin, e);
        emax = max(emax, e);
      }
    }
  }
  if (emin == 256) { out = 0.0; return true; }
  if (emax >= 255 || emax - emin > 38 - lg_d) return false;
  unsigned long long S = 0;
  for (int c = 0; c < d; c += 16) {
    float q[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const float r = c + t < d ? __fsub_rn(a[c + t], b[c + t]) : 0.f;
      q[t] = __fmul_rn(r, r);
    }
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const uint32_t u = __float_as_uint(q[t]);
      const int e = (int)(u >> 23);
      const uint32_t m = (u & 0x7fffffu) | (e ? 0x800000u : 0u);
      S += u ? (unsigned long long)m << (max(e, 1) - emin) : 0ull;  // stays below 2^63
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
  const int ex = pbit + emin - 150 + 1023;
  out = __longlong_as_double((long long)(((unsigned long long)ex << 52) | (mant & 0xfffffffffffffull)));
  return true;
}

}  // namespace sc

namespace sc {

// The same reproduction from terms already in registers: q[t] =
// fl32((a_t - b_t)^2) for t < d (entries t >= d are ignored), D a compile-
// time bound so that q stays in registers.
template <int D>
__device__ __forceinline__ bool sqd_seq_terms(const float (&q)[D], int d, int lg_d, double &out) {
  int emin = 256, emax = 0;
#pragma unroll
  for (int t = 0; t < D; ++t) {
    const uint32_t u = __float_as_uint(q[t]);
    if (t < d && u != 0u) {
      const int e = max((int)(u >> 23), 1);
      emin = min(emin, e);
      emax = max(emax, e);
    }
  }
  if (emin == 256) { out = 0.0; return true; }
  if (emax >= 255 || emax - emin > 38 - lg_d) return false;
  unsigned long long S = 0;
#pragma unroll
  for (int t = 0; t < D; ++t) {
    const uint32_t u = __float_as_uint(q[t]);
    if (t < d && u != 0u) {
      const int e = (int)(u >> 23);
      const uint32_t m = (u & 0x7fffffu) | (e ? 0x800000u : 0u);
      S += (unsigned long long)m << (max(e, 1) - emin);  // stays below 2^63
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
  const int ex = pbit + emin - 150 + 1023;
  out = __longlong_as_double((long long)(((unsigned long long)ex << 52) | (mant & 0xfffffffffffffull)));
  return true;
}

}  // namespace sc
