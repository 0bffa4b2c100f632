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

// The f64 value of an exact total from warp_sqd_terms, S 2^(emin - 150) with
// 0 < S < 2^53 (0 when every term was zero), built from its bits: S fits the
// significand, so no rounding, and no FP64 instruction.
__device__ __forceinline__ double sqd_from_units(unsigned long long S, uint32_t emin) {
  if (emin == 256u || S == 0ull) return 0.0;
  const int pbit = 63 - __clzll((long long)S);
  const unsigned long long mant = S << (52 - pbit);
  const unsigned long long ex = (unsigned long long)(pbit + (int)emin - 150 + 1023);
  return __longlong_as_double((long long)((ex << 52) | (mant & 0xfffffffffffffull)));
}

// Warp-cooperative form for NB row pairs at once: lane l holds, for entry r,
// the terms t[r][c] of features 32 c + l (c < KC; zero past d).  When the
// total S_r, in units of 2^(emin_r - 150), is below 2^53, every running sum of
// the reference is an integer multiple of that unit below 2^53, so no f64
// addition rounds and the sequential sum is the exact total, in any order.
// The common case (span <= 29 - ceil(log2 d): S < 2^53 by construction) takes
// two 32-bit warp reductions; spans up to 29 sum 64-bit parts over the warp
// and test S.  The NB entries' reductions are issued back to back.  Lane
// base + r receives entry r's total as (S, emin) for sqd_from_units; ok[r] is
// false where a running sum may round or a term is inf/NaN (the caller runs
// the sequential form), true with emin = 256 when every term is zero.
template <int KC, int NB>
__device__ __forceinline__ void warp_sqd_terms(const float (&t)[NB][KC], int lg_d, int lane, int base,
                                               unsigned long long &S_out, uint32_t &e_out, bool &ok_out) {
  uint32_t emn[NB], emx[NB];
#pragma unroll
  for (int r = 0; r < NB; ++r) {
    emn[r] = 256u;
    emx[r] = 0u;
#pragma unroll
    for (int c = 0; c < KC; ++c) {
      const uint32_t u = __float_as_uint(t[r][c]);
      if (u != 0u) {
        const uint32_t e = max(u >> 23, 1u);
        emn[r] = min(emn[r], e);
        emx[r] = max(emx[r], e);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < NB; ++r) {
    emn[r] = __reduce_min_sync(0xffffffffu, emn[r]);
    emx[r] = __reduce_max_sync(0xffffffffu, emx[r]);
  }
  uint32_t lo[NB], hi[NB];
#pragma unroll
  for (int r = 0; r < NB; ++r) {
    lo[r] = 0u;  // S = hi 2^24 + lo; both sums stay below 2^32 for d <= 256
    hi[r] = 0u;
    const uint32_t e0 = min(emn[r], 254u);
#pragma unroll
    for (int c = 0; c < KC; ++c) {
      const uint32_t u = __float_as_uint(t[r][c]);
      const uint32_t e = u >> 23;
      const uint32_t sh = min(max(e, 1u) - e0, 40u);  // clamped: spans past 29 - lg_d are redone below
      const unsigned long long v = u ? (unsigned long long)((u & 0x7fffffu) | (e ? 0x800000u : 0u)) << sh : 0ull;
      lo[r] += (uint32_t)(v & 0xffffffull);
      hi[r] += (uint32_t)(v >> 24);
    }
  }
#pragma unroll
  for (int r = 0; r < NB; ++r) {
    lo[r] = __reduce_add_sync(0xffffffffu, lo[r]);
    hi[r] = __reduce_add_sync(0xffffffffu, hi[r]);
  }
#pragma unroll
  for (int r = 0; r < NB; ++r) {
    bool ok = true;
    unsigned long long S = ((unsigned long long)hi[r] << 24) + lo[r];
    if (emn[r] != 256u) {
      if (emx[r] >= 255u || emx[r] - emn[r] > 29u) {  // a term alone reaches 2^53 units, or inf/NaN
        ok = false;
      } else if ((int)(emx[r] - emn[r]) > 29 - lg_d) {  // rare: the exact 64-bit total decides
        unsigned long long v = 0ull;  // each term < 2^53, KC <= 8 per lane: the warp total < 2^61
#pragma unroll
        for (int c = 0; c < KC; ++c) {
          const uint32_t u = __float_as_uint(t[r][c]);
          const uint32_t e = u >> 23;
          v += u ? (unsigned long long)((u & 0x7fffffu) | (e ? 0x800000u : 0u)) << (max(e, 1u) - emn[r]) : 0ull;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        S = v;
        ok = (v >> 53) == 0ull;
      }
    }
    if (lane == base + r) {
      S_out = S;
      e_out = emn[r];
      ok_out = ok;
    }
  }
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

// d <= 32 rows, one lane per row pair, branch-free where no running sum can
// round: after the exponent range (pass 1), a span of at most min(24, 29 -
// ceil(log2 d)) bounds the total below 2^53 units of 2^(emin - 150), so the reference's
// sequential f64 sum is the exact total and the terms are summed in any order,
// as 32-bit parts (hi 2^24 + lo, each part well below 2^32) with independent
// chains.  Wider spans take the sequential form above (sqd_seq_f32).
template <typename PA, typename PB>
__device__ __forceinline__ bool sqd_f32_d32(PA a, PB b, int d, int lg_d, double &out) {
  uint32_t emn0 = 256u, emn1 = 256u, emx0 = 0u, emx1 = 0u;
#pragma unroll
  for (int t = 0; t < 32; t += 2) {
    const float r0 = t < d ? __fsub_rn(a[t], b[t]) : 0.f, r1 = t + 1 < d ? __fsub_rn(a[t + 1], b[t + 1]) : 0.f;
    const uint32_t u0 = __float_as_uint(__fmul_rn(r0, r0)), u1 = __float_as_uint(__fmul_rn(r1, r1));
    const uint32_t e0 = max(u0 >> 23, 1u), e1 = max(u1 >> 23, 1u);
    emn0 = min(emn0, u0 ? e0 : 256u);
    emn1 = min(emn1, u1 ? e1 : 256u);
    emx0 = max(emx0, u0 ? e0 : 0u);
    emx1 = max(emx1, u1 ? e1 : 0u);
  }
  const uint32_t emn = min(emn0, emn1), emx = max(emx0, emx1);
  if (emn == 256u) { out = 0.0; return true; }
  if (emx >= 255u || emx - emn > 24u || (int)(emx - emn) > 29 - lg_d) return sqd_seq_f32(a, b, d, lg_d, out);
  uint32_t lo[4] = {0u, 0u, 0u, 0u}, hi[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int t = 0; t < 32; ++t) {
    const float r = t < d ? __fsub_rn(a[t], b[t]) : 0.f;
    const uint32_t u = __float_as_uint(__fmul_rn(r, r));
    const uint32_t e = u >> 23;
    const uint32_t m = u ? (u & 0x7fffffu) | (e ? 0x800000u : 0u) : 0u;
    const uint32_t sh = max(e, 1u) - emn;  // <= 24 for every nonzero term (0 terms add nothing)
    lo[t & 3] += (m << (sh & 31u)) & 0xffffffu;
    hi[t & 3] += sh ? m >> (24u - sh) : 0u;
  }
  const unsigned long long S = ((unsigned long long)(hi[0] + hi[1] + hi[2] + hi[3]) << 24) +
                               (unsigned long long)(lo[0] + lo[1] + lo[2] + lo[3]);
  out = sqd_from_units(S, emn);
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

// Register terms of d <= D features (zero past d), branch-free where no
// running sum can round (the span test of sqd_f32_d32), else sqd_seq_terms.
// Four 32-bit accumulator pairs: each takes D / 4 <= 16 terms of < 2^24, so
// none can overflow.
template <int D>
__device__ __forceinline__ bool sqd_terms(const float (&q)[D], int d, int lg_d, double &out) {
  static_assert(D % 4 == 0 && D <= 64, "four accumulators of at most 16 terms");
  uint32_t emn0 = 256u, emn1 = 256u, emx0 = 0u, emx1 = 0u;
#pragma unroll
  for (int t = 0; t < D; t += 2) {
    const uint32_t u0 = __float_as_uint(q[t]), u1 = __float_as_uint(q[t + 1]);
    const uint32_t e0 = max(u0 >> 23, 1u), e1 = max(u1 >> 23, 1u);
    emn0 = min(emn0, u0 ? e0 : 256u);
    emn1 = min(emn1, u1 ? e1 : 256u);
    emx0 = max(emx0, u0 ? e0 : 0u);
    emx1 = max(emx1, u1 ? e1 : 0u);
  }
  const uint32_t emn = min(emn0, emn1), emx = max(emx0, emx1);
  if (emn == 256u) { out = 0.0; return true; }
  if (emx >= 255u || emx - emn > 24u || (int)(emx - emn) > 29 - lg_d) return sqd_seq_terms<D>(q, d, lg_d, out);
  uint32_t lo[4] = {0u, 0u, 0u, 0u}, hi[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int t = 0; t < D; ++t) {
    const uint32_t u = __float_as_uint(q[t]);
    const uint32_t e = u >> 23;
    const uint32_t m = u ? (u & 0x7fffffu) | (e ? 0x800000u : 0u) : 0u;
    const uint32_t sh = max(e, 1u) - emn;  // <= 24 for every nonzero term (0 terms add nothing)
    lo[t & 3] += (m << (sh & 31u)) & 0xffffffu;
    hi[t & 3] += sh ? m >> (24u - sh) : 0u;
  }
  const unsigned long long S = ((unsigned long long)(hi[0] + hi[1] + hi[2] + hi[3]) << 24) +
                               (unsigned long long)(lo[0] + lo[1] + lo[2] + lo[3]);
  out = sqd_from_units(S, emn);
  return true;
}

__device__ __forceinline__ bool sqd_terms32(const float (&q)[32], int d, int lg_d, double &out) {
  return sqd_terms<32>(q, d, lg_d, out);
}

}  // namespace sc
