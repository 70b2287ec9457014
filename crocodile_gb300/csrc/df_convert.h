// FP64 <-> double-float conversions by integer operations.
//
// GB300 executes FP64 arithmetic, including the F64 <-> F32 conversions, at
// a small fraction of its FP32 and integer rates, so a pipeline that keeps
// complex128 data as double-float pairs (hi + lo floats) spends most of its
// conversion time on the FP64 pipe.  These helpers compute the same results
// from the IEEE-754 bit patterns with 32/64-bit integer operations:
//
//   split(v) = (hi, lo) with hi = RN_float(v) (round to nearest, ties to
//              even, on the bit pattern: add 0x0FFFFFFF plus the lowest kept
//              bit, then truncate 29 mantissa bits) and lo = RN_float(v - hi)
//              (v - hi is the integer difference of the patterns times the
//              ulp of v's binade, exact; then one int -> float rounding);
//   join(hi, lo) = RN_double(hi + lo): both significands aligned in a 64-bit
//              integer with 10 guard bits and a sticky flag, summed, then
//              rounded to 53 bits, ties to even.
//
// Both are bit-identical to the FP64 forms ((float)v, (float)(v - (double)hi)
// and (double)hi + (double)lo) wherever the fast path applies: |v| in
// [2^-74, 2^127) for split; hi normal and finite, lo finite and at most 2^15
// units of hi's 53-bit extension for join.  Anything else (zero excepted,
// which is handled by bits) takes the FP64 form.
//
// Plain C++ shared by the device code and a host test (no CUDA types).
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define CG_DF_HD __host__ __device__ __forceinline__
#else
#define CG_DF_HD inline
#endif

namespace cg {

CG_DF_HD uint64_t f64_bits(double v) {
  uint64_t u;
  memcpy(&u, &v, 8);
  return u;
}
CG_DF_HD double f64_from(uint64_t u) {
  double v;
  memcpy(&v, &u, 8);
  return v;
}
CG_DF_HD uint32_t f32_bits(float v) {
  uint32_t u;
  memcpy(&u, &v, 4);
  return u;
}
CG_DF_HD float f32_from(uint32_t u) {
  float v;
  memcpy(&v, &u, 4);
  return v;
}

// v -> (hi, lo)
CG_DF_HD void f64_split(double v, float &hi, float &lo) {
  const uint64_t b = f64_bits(v);
  const uint32_t sgn = (uint32_t)(b >> 63);
  const uint64_t a = b & 0x7FFFFFFFFFFFFFFFull;
  const int E = (int)(a >> 52);
  if (a == 0) {  // +-0
    hi = f32_from(sgn << 31);
    lo = 0.0f;
    return;
  }
  if (E < 949 || E > 1149) {  // outside the range the bit path covers
    hi = (float)v;
    lo = (float)(v - (double)hi);
    return;
  }
  const uint64_t t = (a + 0x0FFFFFFFull + ((a >> 29) & 1)) & ~0x1FFFFFFFull;  // RNE to 24 bits
  const int Et = (int)(t >> 52);                                             // E or E + 1
  hi = f32_from((sgn << 31) | ((uint32_t)(Et - 896) << 23) |
                ((uint32_t)(t >> 29) & 0x7FFFFFu));
  const int32_t d = (int32_t)(int64_t)(a - t);          // |d| <= 2^28: (|v| - |hi|) / ulp
  const float p = f32_from((uint32_t)(E - 948) << 23);  // ulp of v's binade, 2^(E - 1075)
  lo = (float)(sgn ? -d : d) * p;                       // exact scaling of RN(d); +0 if d = 0
}

// (hi, lo) -> RN(hi + lo)
CG_DF_HD double f64_join(float hi, float lo) {
  const uint32_t hb = f32_bits(hi), lb = f32_bits(lo);
  const uint32_t ha = hb & 0x7FFFFFFFu, la = lb & 0x7FFFFFFFu;
  const int eh = (int)(ha >> 23), el = (int)(la >> 23);
  if (ha == 0 && la == 0) return f64_from((uint64_t)(hb & lb & 0x80000000u) << 32);  // +-0
  const int e_eff = el ? el : 1;
  // lo in units of 2^(eh - 189): hi's 24-bit significand shifted left 39
  // (53 bits and 10 guard bits)
  const int sh = e_eff - eh + 39;
  if (eh == 0 || eh == 255 || el == 255 || sh > 15) return (double)hi + (double)lo;
  const uint64_t mh = (uint64_t)((ha & 0x7FFFFFu) | 0x800000u);
  const uint64_t ml = (uint64_t)((la & 0x7FFFFFu) | (el ? 0x800000u : 0u));
  const bool same = ((hb ^ lb) & 0x80000000u) == 0;
  // S = floor(|hi| + (+-|lo|)) in those units, S in (2^62 - 2^39, 2^63 + 2^39);
  // the true magnitude is S + f with f in [0, 1), f > 0 iff sticky
  uint64_t S = mh << 39;
  bool sticky = false;
  if (ml != 0) {
    if (sh >= 0) {
      S = same ? S + (ml << sh) : S - (ml << sh);
    } else if (sh > -40) {
      const int r = -sh;
      const uint64_t q = ml >> r;
      sticky = (ml & (((uint64_t)1 << r) - 1)) != 0;
      S = same ? S + q : S - q - (sticky ? 1 : 0);
    } else {  // |lo| under 2^-16 units: only its sign matters
      if (!same) S -= 1;
      sticky = true;
    }
  }
  int ex = eh + 896;  // hi's exponent as a biased double exponent
  if (S >> 63) {      // >= 2^63: one bit right
    sticky = sticky || (S & 1);
    S >>= 1;
    ++ex;
  } else if (!(S >> 62)) {  // < 2^62: one bit left (f moves into the free bit)
    S <<= 1;
    --ex;
  }
  // S in [2^62, 2^63): 53 significant bits over 10 guard bits
  uint64_t m = S >> 10;
  const uint32_t rem = (uint32_t)(S & 1023);
  if (rem > 512 || (rem == 512 && (sticky || (m & 1)))) ++m;
  if (m >> 53) {  // rounding carried into the next binade
    m >>= 1;
    ++ex;
  }
  return f64_from(((uint64_t)(hb & 0x80000000u) << 32) | ((uint64_t)ex << 52) |
                  (m & 0xFFFFFFFFFFFFFull));
}

}  // namespace cg
