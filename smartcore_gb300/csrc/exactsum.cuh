// Exact reference squared distances of f32 rows without FP64 instructions.
#pragma once

#include <stdint.h>

namespace sc {

// Squared distance of the reference (src/metrics/distance/euclidian.rs:56-63)
// for f32 rows: terms q_t = fl32((a_t - b_t)^2), summed in f64 from t = 0.
// When the terms' exponents span less than 2^(29 - ceil(log2 d)), no partial
// sum of that sequence can round (all are integers below 2^53 in units of the
// smallest term's last bit), so the sequence's value is the exact sum, which
// is computed here in 64-bit integers: no FP64 instruction.  Returns false
// when that condition fails (the caller then runs the FP64 sequence).
template <typename PA, typename PB>
__device__ __forceinline__ bool sqd_exact_f32(PA a, PB b, int d, int lg_d, double &out) {
  int emin = 256, emax = 0;
  for (int t = 0; t < d; ++t) {
    const float r = __fsub_rn(a[t], b[t]);
    const uint32_t q = __float_as_uint(__fmul_rn(r, r));
    if (q == 0u) continue;
    const int e = max((int)(q >> 23), 1);
    emin = min(emin, e);
    emax = max(emax, e);
  }
  if (emin == 256) { out = 0.0; return true; }
  if (emax >= 255 || emax - emin > 29 - lg_d) return false;  // inf/NaN, or a partial sum might round
  unsigned long long S = 0;
  for (int t = 0; t < d; ++t) {
    const float r = __fsub_rn(a[t], b[t]);
    const uint32_t q = __float_as_uint(__fmul_rn(r, r));
    if (q == 0u) continue;
    const int e = (int)(q >> 23);
    const uint32_t m = (q & 0x7fffffu) | (e ? 0x800000u : 0u);
    S += (unsigned long long)m << (max(e, 1) - emin);
  }
  const int pbit = 63 - __clzll((long long)S);  // S < 2^53
  const unsigned long long mant = S << (52 - pbit);
  const int ex = pbit + emin - 150 + 1023;
  out = __longlong_as_double((long long)(((unsigned long long)ex << 52) | (mant & 0xfffffffffffffull)));
  return true;
}


}  // namespace sc
