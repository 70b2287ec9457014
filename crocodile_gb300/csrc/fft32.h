// Register-blocked Stockham FFT of power-of-two lines (N = 2^logn, 64..8192)
// in FP32: the arithmetic shared by the kernels of fft32.cu and the host
// check tests/fft32_check.cpp.  Plain C++ apart from the qualifiers.
//
// Every stage is radix 16 except one first stage of radix 2^(logn mod 4)
// when logn is not a multiple of 4.  A line is worked by T = N / 16
// threads, each holding 16 values in registers per stage: 16 / R
// butterflies of radix R.  Stage with span p (the length of the
// subsequences already transformed: 1 at the first stage, then times R):
// butterfly b (b < N / R), k = b mod p,
//   inputs  x[b + r N/R]                (r < R), times the twiddle w_N^(r k N/(pR)),
//   an R-point DFT (w_R = exp(sign 2 pi i / R)),
//   outputs y[(b - k) R + k + r p].
// The last stage has p = N / R, so its outputs y[b + r p] are in natural
// order, and every stage's inputs x[b + r N/R] are contiguous across b:
// the first stage can read global memory and the last stage write it
// directly, coalesced across threads.  Between stages all threads read their inputs
// before any thread writes, so one buffer holds the line throughout.
#pragma once

#ifdef __CUDACC__
#define CG_FHD __host__ __device__ __forceinline__
#else
#define CG_FHD inline
#endif

namespace cg {
namespace f32 {

struct cf {
  float x, y;
};

CG_FHD cf cf_add(cf a, cf b) { return {a.x + b.x, a.y + b.y}; }
CG_FHD cf cf_sub(cf a, cf b) { return {a.x - b.x, a.y - b.y}; }
CG_FHD cf cf_mul(cf a, cf b) {
#ifdef __CUDACC__
  return {fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x)};
#else
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
#endif
}
// times (sign i): sign > 0: i (x + iy) = -y + ix; sign < 0: -i (x + iy) = y - ix
CG_FHD cf cf_mul_si(cf a, int sign) { return sign > 0 ? cf{-a.y, a.x} : cf{a.y, -a.x}; }

// stages of a 2^logn transform: count, log2 radix and log2 span of stage s
CG_FHD constexpr int stage_count(int logn) { return (logn + 3) / 4; }
CG_FHD constexpr int stage_logr(int logn, int s) { return ((logn & 3) && s == 0) ? (logn & 3) : 4; }
CG_FHD constexpr int stage_logp(int logn, int s) {
  const int rem = logn & 3;
  return s == 0 ? 0 : (rem ? rem + 4 * (s - 1) : 4 * s);
}

// R-point DFTs in place, X[k] = sum_n v[n] w_R^(n k)
CG_FHD void dft2(cf *v) {
  const cf a = v[0], b = v[1];
  v[0] = cf_add(a, b);
  v[1] = cf_sub(a, b);
}
CG_FHD void dft4(cf *v, int sign) {
  const cf a0 = cf_add(v[0], v[2]), a1 = cf_sub(v[0], v[2]);
  const cf b0 = cf_add(v[1], v[3]), b1 = cf_mul_si(cf_sub(v[1], v[3]), sign);
  v[0] = cf_add(a0, b0);
  v[2] = cf_sub(a0, b0);
  v[1] = cf_add(a1, b1);
  v[3] = cf_sub(a1, b1);
}
// w_8^j for the sign
CG_FHD cf w8(int j, int sign) {
  const float h = 0.70710678118654752f, s = (float)sign;
  switch (j & 7) {
    case 0: return {1.f, 0.f};
    case 1: return {h, s * h};
    case 2: return {0.f, s};
    case 3: return {-h, s * h};
    case 4: return {-1.f, 0.f};
    case 5: return {-h, -s * h};
    case 6: return {0.f, -s};
    default: return {h, -s * h};
  }
}
// w_16^j for the sign
CG_FHD cf w16(int j, int sign) {
  const float c = 0.92387953251128676f, q = 0.38268343236508977f, s = (float)sign;
  switch (j & 15) {
    case 1: return {c, s * q};
    case 3: return {q, s * c};
    case 5: return {-q, s * c};
    case 7: return {-c, s * q};
    case 9: return {-c, -s * q};
    case 11: return {-q, -s * c};
    case 13: return {q, -s * c};
    case 15: return {c, -s * q};
    default: return w8((j & 15) >> 1, sign);
  }
}
// Radix-8 and radix-16 DFTs in place with their outputs left permuted:
// X[r] ends in v[out_slot(logr, r)] (the stage's store reads that slot), so
// that no copy between register arrays is needed.
// 8 = 2 x 4: n = b + 4a (b < 4, a < 2), k = k1 + 2 k2:
//   X[k1 + 2 k2] = sum_b w_4^(b k2) [w_8^(b k1) sum_a v[b + 4a] w_2^(a k1)];
//   after the pass over a, v[b + 4 k1] holds the bracket; X[k1 + 2 k2] in
//   v[4 k1 + k2].
CG_FHD void dft8(cf *v, int sign) {
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const cf x = v[b], y = v[b + 4];
    v[b] = cf_add(x, y);
    v[b + 4] = b ? cf_mul(cf_sub(x, y), w8(b, sign)) : cf_sub(x, y);
  }
  dft4(v, sign);
  dft4(v + 4, sign);
}
// 16 = 4 x 4: n = a + 4b, k = c + 4d:
//   X[c + 4d] = sum_a w_4^(a d) [w_16^(a c) sum_b v[a + 4b] w_4^(b c)];
//   after the pass over b, v[a + 4c] holds the bracket; X[c + 4d] in v[4c + d].
CG_FHD void dft16(cf *v, int sign) {
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    cf t[4] = {v[a], v[a + 4], v[a + 8], v[a + 12]};
    dft4(t, sign);
#pragma unroll
    for (int c = 0; c < 4; ++c) v[a + 4 * c] = (a && c) ? cf_mul(t[c], w16(a * c, sign)) : t[c];
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    cf t[4] = {v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]};
    dft4(t, sign);
#pragma unroll
    for (int d = 0; d < 4; ++d) v[4 * c + d] = t[d];
  }
}
CG_FHD void dft_r(cf *v, int logr, int sign) {
  if (logr == 1) dft2(v);
  else if (logr == 2) dft4(v, sign);
  else if (logr == 3) dft8(v, sign);
  else dft16(v, sign);
}
// register slot holding output r of a radix-2^logr DFT
CG_FHD int out_slot(int logr, int r) {
  if (logr == 3) return 4 * (r & 1) + (r >> 1);
  if (logr == 4) return 4 * (r & 3) + (r >> 2);
  return r;
}

// Twiddles of stage s (s >= 1), w_N^(r k N / (p R)) for r < R, k < p, from a
// table laid out per stage so that a warp's lookups do not conflict in
// shared-memory banks: with k = k_lo + 32 k_hi (k_lo < 32),
//   L_s[r][k_lo] = w^(r k_lo N / (p R))      (R x min(p, 32) entries)
//   H_s[r][k_hi] = w^(r 32 k_hi N / (p R))   (R x p / 32 entries, p > 32)
// and the twiddle is L_s[r][k] for p <= 32 (the correctly rounded value)
// or L_s[r][k_lo] H_s[r][k_hi] (one complex product more).  The threads of
// a warp share k_hi and hold consecutive k_lo (or few distinct k), so L
// reads are contiguous or broadcast and H reads are broadcast.
CG_FHD constexpr int tw_stage_entries(int logn, int s) {
  const int logr = stage_logr(logn, s), logp = stage_logp(logn, s);
  const int p = 1 << logp, lo = p < 32 ? p : 32, hi = p > 32 ? p >> 5 : 0;
  return (1 << logr) * (lo + hi);
}
CG_FHD constexpr int tw_stage_offset(int logn, int s) {
  int off = 0;
  for (int q = 1; q < s; ++q) off += tw_stage_entries(logn, q);
  return off;
}
CG_FHD constexpr int tw_table_entries(int logn) {
  return tw_stage_offset(logn, stage_count(logn));
}
// fills the table; w(j) gives the exact w_N^j (j < N) rounded to FP32
template <class W>
inline void tw_table_fill(int logn, const W &w, cf *out) {
  for (int s = 1; s < stage_count(logn); ++s) {
    const int logr = stage_logr(logn, s), logp = stage_logp(logn, s);
    const int R = 1 << logr, p = 1 << logp, lo = p < 32 ? p : 32;
    const int sh = logn - logp - logr;  // N / (p R) = 2^sh
    cf *L = out + tw_stage_offset(logn, s), *H = L + R * lo;
    for (int r = 0; r < R; ++r) {
      for (int k = 0; k < lo; ++k) L[r * lo + k] = w(((long long)r * k << sh) & ((1 << logn) - 1));
      for (int kh = 0; kh < (p >> 5) && p > 32; ++kh)
        H[r * (p >> 5) + kh] = w(((long long)r * 32 * kh << sh) & ((1 << logn) - 1));
    }
  }
}
// the twiddle of input r of a butterfly with k, at stage s; tb(i) reads entry i
template <class TB>
CG_FHD cf tw_lookup(int logn, int s, int r, int k, const TB &tb) {
  const int logr = stage_logr(logn, s), logp = stage_logp(logn, s);
  const int R = 1 << logr, p = 1 << logp;
  const int base = tw_stage_offset(logn, s);
  if (p <= 32) return tb(base + r * p + k);
  return cf_mul(tb(base + r * 32 + (k & 31)), tb(base + R * 32 + r * (p >> 5) + (k >> 5)));
}

// One thread's share of stage s: 16 / R butterflies b = t + m T (m < 16/R,
// T = N / 16), in three steps so that a kernel can put a barrier between
// every thread's reads and every thread's writes.  ld(e) / st(e, v) access
// element e of the line; tw(s, r, k) gives w_N^(r k N / (p R)) of stage s.
template <class LD, class TW>
CG_FHD void stage_load(int logn, int s, int t, const LD &ld, const TW &tw, cf *v) {
  const int logr = stage_logr(logn, s), logp = stage_logp(logn, s);
  const int R = 1 << logr, nb = 16 >> logr, T = 1 << (logn - 4);
  const int NR = 1 << (logn - logr);  // N / R
#pragma unroll
  for (int m = 0; m < nb; ++m) {
    const int b = t + m * T;
    const int k = b & ((1 << logp) - 1);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      cf x = ld(b + r * NR);
      if (r && k) x = cf_mul(x, tw(s, r, k));  // w_N^(r k N/(pR))
      v[m * R + r] = x;
    }
  }
}
CG_FHD void stage_dft(int logn, int s, int sign, cf *v) {
  const int logr = stage_logr(logn, s), nb = 16 >> logr;
#pragma unroll
  for (int m = 0; m < nb; ++m) dft_r(v + (m << logr), logr, sign);
}
// Output index of butterfly m's output r at stage s for thread t, and the
// register slot holding it: slot q = m R + r is output out_index(q).
CG_FHD int out_index(int logn, int s, int t, int m, int r) {
  const int logr = stage_logr(logn, s), logp = stage_logp(logn, s);
  const int b = t + m * (1 << (logn - 4));
  const int k = b & ((1 << logp) - 1);
  return ((b - k) << logr) + k + (r << logp);
}
template <class ST>
CG_FHD void stage_store(int logn, int s, int t, const ST &st, const cf *v) {
  const int logr = stage_logr(logn, s);
  const int R = 1 << logr, nb = 16 >> logr;
#pragma unroll
  for (int m = 0; m < nb; ++m) {
#pragma unroll
    for (int r = 0; r < R; ++r) st(out_index(logn, s, t, m, r), v[m * R + out_slot(logr, r)]);
  }
}

}  // namespace f32
}  // namespace cg
