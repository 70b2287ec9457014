// In-place radix-4 decimation-in-time FFT of one line of N = 2^logn complex
// values held in an indexable buffer (shared memory on the device; plain
// arrays in tests/fft32_check.cpp, which checks it on the host against a
// direct DFT).  Plain C++ apart from the qualifiers.
//
// The line is loaded in bit-reversed order (element i at position
// bitrev(i)); the stages then leave X[k] at position k.  Radix-2 DIT stage
// with half-span h (h = 1, 2, 4, ..., N/2): for groups of 2h and j < h,
//   (x[a], x[a + h]) <- (x[a] + w^j x[a + h], x[a] - w^j x[a + h]),
//   w = w_N^(N / 2h), w_N = exp(sign 2 pi i / N).
// Two consecutive stages h, 2h form one radix-4 butterfly on a0 = g 4h + j,
// a1 = a0 + h, a2 = a0 + 2h, a3 = a0 + 3h (j < h):
//   stage h:  b0,1 = x0 +- w1 x1,  b2,3 = x2 +- w1 x3,   w1 = w_N^(j N / 2h)
//   stage 2h: c0,2 = b0 +- w2 b2,  c1,3 = b1 +- w3 b3,   w2 = w_N^(j N / 4h),
//             w3 = w2 w_N^(N/4) = w2 * (sign i)
// With odd logn one radix-2 stage (h = 1, twiddle 1) comes first.  The
// twiddle table holds w_N^k for k < N / 2.
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
// times (sign i): sign > 0: i (a.x, a.y) = (-a.y, a.x); sign < 0: -i -> (a.y, -a.x)
CG_FHD cf cf_mul_si(cf a, int sign) { return sign > 0 ? cf{-a.y, a.x} : cf{a.y, -a.x}; }

CG_FHD unsigned bitrev(unsigned i, int logn) {
#ifdef __CUDA_ARCH__
  return __brev(i) >> (32 - logn);
#else
  unsigned r = 0;
  for (int b = 0; b < logn; ++b) r |= ((i >> b) & 1u) << (logn - 1 - b);
  return r;
#endif
}

// Butterfly q of the odd-logn radix-2 first stage (q < N / 2): pair (2q, 2q + 1).
template <class BUF>
CG_FHD void radix2_first(BUF &x, int q) {
  const cf u = x.get(2 * q), v = x.get(2 * q + 1);
  x.set(2 * q, cf_add(u, v));
  x.set(2 * q + 1, cf_sub(u, v));
}

// Radix-4 butterfly q (q < N / 4) of the stage pair (h, 2h), h = 2^lh.
template <class BUF, class TW>
CG_FHD void radix4(BUF &x, const TW &tw, int logn, int lh, int q, int sign) {
  const int h = 1 << lh;
  const int j = q & (h - 1), g = q >> lh;
  const int a0 = (g << (lh + 2)) + j;
  const cf x0 = x.get(a0), x1 = x.get(a0 + h), x2 = x.get(a0 + 2 * h), x3 = x.get(a0 + 3 * h);
  // w1 = w_N^(j N / 2h), w2 = w_N^(j N / 4h)
  const cf w1 = tw.get(j << (logn - 1 - lh)), w2 = tw.get(j << (logn - 2 - lh));
  const cf t1 = cf_mul(w1, x1), t3 = cf_mul(w1, x3);
  const cf b0 = cf_add(x0, t1), b1 = cf_sub(x0, t1), b2 = cf_add(x2, t3), b3 = cf_sub(x2, t3);
  const cf u2 = cf_mul(w2, b2), u3 = cf_mul_si(cf_mul(w2, b3), sign);
  x.set(a0, cf_add(b0, u2));
  x.set(a0 + 2 * h, cf_sub(b0, u2));
  x.set(a0 + h, cf_add(b1, u3));
  x.set(a0 + 3 * h, cf_sub(b1, u3));
}

// The whole line in one thread (host reference of the stage sequence; the
// kernels run the same butterflies spread over threads with a barrier
// between stages).
template <class BUF, class TW>
CG_FHD void line_serial(BUF &x, const TW &tw, int logn, int sign) {
  const int N = 1 << logn;
  int lh = 0;
  if (logn & 1) {
    for (int q = 0; q < N / 2; ++q) radix2_first(x, q);
    lh = 1;
  }
  for (; lh + 1 < logn; lh += 2)
    for (int q = 0; q < N / 4; ++q) radix4(x, tw, logn, lh, q, sign);
}

}  // namespace f32
}  // namespace cg
