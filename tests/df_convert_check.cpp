// Host check of crocodile_gb300/csrc/df_convert.h: the integer FP64 <->
// double-float conversions against the FP64 forms they replace, bit for bit,
// on random bit patterns and on the edge cases of each path (ties of the
// split, carries into the next binade, cancelling and tiny or subnormal lo
// parts, zeros, infinities, NaNs).  Exit status 0 when everything matches.
// Built with: g++ -O2 -ffp-contract=off -I crocodile_gb300/csrc
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "df_convert.h"

using namespace cg;

static uint64_t state = 0x9E3779B97F4A7C15ull;
static uint64_t next() {  // splitmix64
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static bool same_f(float a, float b) {
  if (std::isnan(a) || std::isnan(b)) return std::isnan(a) && std::isnan(b);
  return f32_bits(a) == f32_bits(b);
}
static bool same_d(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return std::isnan(a) && std::isnan(b);
  return f64_bits(a) == f64_bits(b);
}

static long bad_split = 0, bad_join = 0, n_split = 0, n_join = 0;

static void check_split(double v) {
  float hi, lo;
  f64_split(v, hi, lo);
  const float rh = (float)v;
  const float rl = (float)(v - (double)rh);
  ++n_split;
  if (!same_f(hi, rh) || (!std::isnan(rh) && !std::isinf(rh) && !same_f(lo, rl))) {
    if (bad_split++ < 10)
      printf("split %a: got (%a, %a) want (%a, %a)\n", v, hi, lo, rh, rl);
  }
}

static void check_join(float hi, float lo) {
  const double got = f64_join(hi, lo);
  const double want = (double)hi + (double)lo;
  ++n_join;
  if (!same_d(got, want)) {
    if (bad_join++ < 10) printf("join (%a, %a): got %a want %a\n", hi, lo, got, want);
  }
}

int main() {
  // split: random bit patterns, then values in the fast range with chosen
  // low bits (exact ties, just above and below, all ones)
  for (int i = 0; i < 4000000; ++i) check_split(f64_from(next()));
  const uint64_t lows[] = {0x10000000ull, 0x0FFFFFFFull, 0x10000001ull, 0x1FFFFFFFull, 0ull, 1ull};
  for (int i = 0; i < 2000000; ++i) {
    const uint64_t e = 940 + next() % 220;  // around both ends of the fast range
    uint64_t m = next() & 0xFFFFFFFFFFFFFull;
    m = (m & ~0x1FFFFFFFull) | lows[i % 6];
    if (i % 7 == 0) m |= 0xFFFFFE0000000ull;  // kept bits all ones: carry into the exponent
    check_split(f64_from(((next() & 1) << 63) | (e << 52) | m));
  }
  const double specials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, -1.0, 0x1p-74, 0x1p-75,
                             0x1.fffffffffffffp126, 0x1p127, 0x1.ffffffp-75, 4.9e-324,
                             0x1.fffffffp-1};
  for (double v : specials) check_split(v);
  // join: pairs from splits of random doubles (normalised double-floats)
  for (int i = 0; i < 3000000; ++i) {
    const uint64_t e = 900 + next() % 300;
    const double v = f64_from(((next() & 1) << 63) | (e << 52) | (next() & 0xFFFFFFFFFFFFFull));
    float hi, lo;
    f64_split(v, hi, lo);
    check_join(hi, lo);
  }
  // hi random, lo at or below half an ulp of hi with either sign, down to
  // subnormals; hi powers of two with negative lo (the left renormalisation)
  for (int i = 0; i < 4000000; ++i) {
    uint32_t hb = (uint32_t)next();
    if (i % 5 == 0) hb &= 0xFF800000u;  // a power of two
    const int eh = (int)((hb >> 23) & 0xFF);
    const int back = 24 + (int)(next() % 50);  // lo exponent below hi's
    const int el = eh - back;
    uint32_t lb = (uint32_t)next() & 0x807FFFFFu;
    if (el > 0)
      lb |= (uint32_t)el << 23;
    else if (i % 3)
      lb &= 0x80000000u | (0x7FFFFFu >> std::min(23, -el + 1));  // subnormal or zero
    else
      lb &= 0x80000000u;
    if (i % 5 == 0) lb |= 0x80000000u ^ (hb & 0x80000000u);
    check_join(f32_from(hb), f32_from(lb));
  }
  // arbitrary pairs (mostly the FP64 fallback) and specials
  for (int i = 0; i < 2000000; ++i) check_join(f32_from((uint32_t)next()), f32_from((uint32_t)next()));
  const float fs[] = {0.f, -0.f, INFINITY, -INFINITY, NAN, 1.f, -1.f, 0x1p-126f, 0x1p-149f,
                      0x1.fffffep127f, 0x1p-24f, -0x1p-25f, 0x1p-25f};
  for (float a : fs)
    for (float b : fs) check_join(a, b);
  printf("split: %ld of %ld differ; join: %ld of %ld differ\n", bad_split, n_split, bad_join,
         n_join);
  return (bad_split || bad_join) ? 1 : 0;
}
