// Facet -> subgrid recombination (examples/grid/recombine.c, the 2-D
// algorithm of examples/notebooks/facet-subgrid-impl.ipynb cells 24-30).
//
// One facet [yB, yB] becomes the contributions NMBF_NMBF[i0][i1]
// [xM_yN, xM_yN] to every requested subgrid in one call:
//   1. k_rc_prep_rows   : BF[r][k] = Fb[t] F[r][t] / yP, zero-padded to yP
//                         (prepare_facet along axis 1; rows leave in raw order)
//      inverse FFT of yB rows of length yP
//   2. k_rc_window      : per subgrid column offset, the xMxN_yP samples around
//                         it times m, margins folded onto xM_yP (extract_subgrid)
//      forward FFT of n1 * yB rows of length xM_yP
//   3. k_rc_crop_prep_T : crop to xM_yN times Fn, transpose, prepare_facet along
//                         axis 0 (times Fb, zero-pad to yP), via a 32x32 tile
//      inverse FFT of n1 * xM_yN rows of length yP
//   4. k_rc_window      : per subgrid row offset, as 2.
//      forward FFT of n0 * n1 * xM_yN rows of length xM_yP
//   5. k_rc_crop_T      : crop times Fn, transpose to [i0][i1][axis 0][axis 1]
// Every FFT runs over contiguous rows.  The caller's arrays are complex128 as
// the reference.  When both transform lengths are powers of two 64..2048 the
// double-float pipeline runs (facet_to_subgrids_df / subgrids_to_facet_df):
// stage arrays of double-float pairs (about 48 significant bits, arithmetic
// on the FP32 units, df.cuh), double-float FFTs (dfft.cuh), and steps 1, 2,
// 4 and 5 done inside the loads and stores of the neighbouring transforms
// (prepare in the loads of the first, the windows in the loads of the
// xM_yP transforms, the final crop in the stores of the last), so that per
// facet four transform launches and the transpose of step 3 remain.
// Otherwise complex128 with FP64 cuFFT and the separate stage kernels.
// Arrays are in the C prototype's raw
// layout (centre at index 0, FFTW sign conventions: backward = e^{+2 pi i},
// unnormalised) except where a `centred` flag maps the facet in or the
// result out in numpy's fftshift layout (the notebook's).
//
// k_rc_add_facet is recombine2d_af0_af1 (recombine.c:504-544): the facet's
// contribution rolled to the facet offset and added into the subgrid,
// divided by xM^2 in the raw form (an unnormalised backward FFT follows);
// the centred form is the notebook's `approx += roll(pad_mid(...))`
// (a normalised centred ifft follows).

#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "cg_internal.cuh"
#include "df.cuh"
#include "dfft.cuh"

namespace cg {
int fft_plan(int batch, int H, int W, cufftType type, cufftHandle *out);
bool dfft_supported(int n);
bool dfft_long_supported(int n);
int dfft_rows(double2 *data, int64_t batch, int n, int inverse, cudaStream_t st);
int dfft_rows_df(float4 *data, int64_t batch, int n, int inverse, cudaStream_t st);
}

struct cg_recombine {
  int N, subgrid_spacing, facet_spacing;
  int yB, yN, yP, xA, xM, xMxN_yP;
  int xM_yP, xM_yN, yP_spacing, xM_spacing;
  int fft_mode;  // 0: double-float FFTs for power-of-two rows, cuFFT Z2Z otherwise; 1: cuFFT Z2Z
  double *d_Fb, *d_Fn, *d_m;
  float2 *d_Fb2, *d_Fn2, *d_m2;  // the same split into double-float (hi, lo)
};

namespace {

using namespace cg;

__host__ __device__ inline int pmod(long long a, int n) {
  long long r = a % n;
  return (int)(r < 0 ? r + n : r);
}

// a mod n for a in [-n, 2n) (one conditional add or subtract, 32-bit)
__device__ __forceinline__ int wrap1(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// Element policies of the stage arrays.  P64: complex128 with FP64
// arithmetic.  PDF: double-float pairs (float4 = re.hi, re.lo, im.hi, im.lo,
// the same 16 bytes) with arithmetic on the FP32 units, window weights as
// float2 (hi, lo); conversions from and to complex128 only where the
// pipeline reads the caller's arrays or writes its results.  The divisors
// passed to wdiv are transform lengths, powers of two in the PDF pipeline.
struct P64 {
  typedef double2 S;  // stored element
  typedef double2 V;  // element in registers
  typedef double W;   // weight in registers
  typedef double WS;  // weight as stored
  __device__ static V in(double2 a) { return a; }
  __device__ static double2 out(V a) { return a; }
  __device__ static V ld(const S &s) { return s; }
  __device__ static S st(const V &v) { return v; }
  __device__ static V zero() { return make_double2(0.0, 0.0); }
  __device__ static W w(const WS *a, int i) { return a[i]; }
  __device__ static W one() { return 1.0; }
  __device__ static W wmul(W a, W b) { return a * b; }
  __device__ static W wdiv(W a, int n) { return a / (double)n; }
  __device__ static V scale(V a, W s) {
    a.x *= s;
    a.y *= s;
    return a;
  }
  __device__ static V madd(V acc, W w, const V &b) {  // acc + w b
    acc.x += w * b.x;
    acc.y += w * b.y;
    return acc;
  }
};

struct PDF {
  typedef float4 S;
  typedef cdf V;
  typedef df W;
  typedef float2 WS;
  __device__ static V in(double2 a) { return cdf_from(a); }
  __device__ static double2 out(const V &a) { return cdf_to(a); }
  __device__ static V ld(const S &s) { return cdf_load(s); }
  __device__ static S st(const V &v) { return cdf_store(v); }
  __device__ static V zero() { return {{0.f, 0.f}, {0.f, 0.f}}; }
  __device__ static W w(const WS *a, int i) {
    const float2 t = a[i];
    return {t.x, t.y};
  }
  __device__ static W one() { return {1.f, 0.f}; }
  __device__ static W wmul(W a, W b) { return df_mul(a, b); }
  __device__ static W wdiv(W a, int n) {  // n a power of two: exact
    const float r = 1.0f / (float)n;
    return {a.hi * r, a.lo * r};
  }
  __device__ static V scale(const V &a, W s) { return cdf_scale(a, s); }
  __device__ static V madd(const V &acc, W w, const V &b) { return cdf_add(acc, cdf_scale(b, w)); }
};

// prepare_facet along the rows: out[r][k], k < yP.  With `centred`, the input
// facet is in fftshift layout on both axes and row r of the output is raw row r.
template <class P>
__global__ void k_rc_prep_rows(const double2 *__restrict__ in, int rows, int yB, int yP,
                               const typename P::WS *__restrict__ Fb, int centred,
                               typename P::S *__restrict__ out) {
  const int h = yB / 2;
  const size_t total = (size_t)rows * yP;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / yP), k = (int)(e % yP);
    int t = -1;
    if (k < h)
      t = k;
    else if (k >= yP - h)
      t = k - yP + yB;
    typename P::V v = P::zero();
    if (t >= 0) {
      const int rs = centred ? (r + h) % yB : r;
      const int ts = centred ? (t + h) % yB : t;
      v = P::scale(P::in(in[(size_t)rs * yB + ts]), P::wdiv(P::w(Fb, t), yP));
    }
    out[e] = P::st(v);
  }
}

// Subgrid offsets in grid cells -> yP samples; an offset that is not a
// multiple of the subgrid spacing is counted as an index error and taken as 0.
__global__ void k_rc_offsets(const int32_t *__restrict__ off0, int n0,
                             const int32_t *__restrict__ off1, int n1, int spacing,
                             int yP_spacing, int yP, int32_t *__restrict__ out,
                             int32_t *status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n0 + n1) return;
  const int o = i < n0 ? off0[i] : off1[i - n0];
  if (pmod(o, spacing) != 0) {
    atomicAdd(&status[ST_INDEX], 1);
    out[i] = 0;
    return;
  }
  out[i] = pmod((long long)(o - pmod(o, spacing)) / spacing * yP_spacing, yP);
}

// extract_subgrid's window: out[o][r][i] from row r of bf at offset offs[o]
// (in yP samples).
template <class P>
__global__ void k_rc_window(const typename P::S *__restrict__ bf, int rows, int yP,
                            const int32_t *__restrict__ offs, int noff, int xM_yP, int xMxN_yP,
                            const typename P::WS *__restrict__ m,
                            typename P::S *__restrict__ out) {
  const int xN_yP = xMxN_yP - xM_yP;
  const size_t total = (size_t)noff * rows * xM_yP;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % xM_yP);
    const size_t orow = e / xM_yP;
    const int r = (int)(orow % rows);
    const int off = offs[orow / rows];
    const typename P::S *row = bf + (size_t)r * yP;
    typename P::V v = P::zero();
    // off < yP and i < xM_yP <= yP, so both sums lie within one period
    if (i < (xMxN_yP + 1) / 2) v = P::madd(v, P::w(m, i), P::ld(row[wrap1(i + off, yP)]));
    if (i >= xM_yP - xMxN_yP / 2)
      v = P::madd(v, P::w(m, xN_yP + i), P::ld(row[wrap1(i + off - xM_yP, yP)]));
    out[e] = P::st(v);
  }
}

__device__ __forceinline__ int crop_src(int c, int xM_yN, int xM_yP) {
  return c < xM_yN / 2 ? c : xM_yP - xM_yN + c;
}

// Crop (times Fn) along the rows of mbf [n1][yB][xM_yP], transpose and
// prepare along the former row axis: out[i1][c][k], k < yP.
// Block: 32 x 8 threads; tile of 32 columns c by 32 output positions k.
template <class P>
__global__ void k_rc_crop_prep_T(const typename P::S *__restrict__ mbf, int yB, int xM_yP,
                                 int xM_yN, const typename P::WS *__restrict__ Fn,
                                 const typename P::WS *__restrict__ Fb, int yP,
                                 typename P::S *__restrict__ out) {
  __shared__ typename P::S tile[32][33];
  const int i1 = blockIdx.z;
  const int c0 = blockIdx.y * 32;
  const int k0 = blockIdx.x * 32;
  const int h = yB / 2;
  const typename P::S *src = mbf + (size_t)i1 * yB * xM_yP;
  // load: tile[kk][cc] = Fb[t] Fn[c] mbf[t][crop(c)] / yP for k = k0 + kk
  for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
    const int k = k0 + kk;
    const int c = c0 + threadIdx.x;
    int t = -1;
    if (k < yP) {
      if (k < h)
        t = k;
      else if (k >= yP - h)
        t = k - yP + yB;
    }
    typename P::V v = P::zero();
    if (t >= 0 && c < xM_yN)
      v = P::scale(P::ld(src[(size_t)t * xM_yP + crop_src(c, xM_yN, xM_yP)]),
                   P::wdiv(P::wmul(P::w(Fn, c), P::w(Fb, t)), yP));
    tile[kk][threadIdx.x] = P::st(v);
  }
  __syncthreads();
  for (int cc = threadIdx.y; cc < 32; cc += blockDim.y) {
    const int c = c0 + cc;
    const int k = k0 + threadIdx.x;
    if (c < xM_yN && k < yP) out[((size_t)i1 * xM_yN + c) * yP + k] = tile[threadIdx.x][cc];
  }
}

// Final crop (times Fn) along the rows of mbf2 [n0][n1][xM_yN (axis 1)][xM_yP]
// and transpose: out[i0][i1][a0][a1].  With `centred`, both output axes in
// fftshift layout.
template <class P>
__global__ void k_rc_crop_T(const typename P::S *__restrict__ mbf2, int n1, int xM_yP, int xM_yN,
                            const typename P::WS *__restrict__ Fn, int centred,
                            double2 *__restrict__ out) {
  __shared__ typename P::S tile[32][33];
  const int pair = blockIdx.z;  // i0 * n1 + i1
  const int a10 = blockIdx.y * 32;
  const int a00 = blockIdx.x * 32;
  const typename P::S *src = mbf2 + (size_t)pair * xM_yN * xM_yP;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int a1 = a10 + yy;
    const int a0 = a00 + threadIdx.x;
    typename P::V v = P::zero();
    if (a1 < xM_yN && a0 < xM_yN)
      v = P::scale(P::ld(src[(size_t)a1 * xM_yP + crop_src(a0, xM_yN, xM_yP)]), P::w(Fn, a0));
    tile[yy][threadIdx.x] = P::st(v);
  }
  __syncthreads();
  const int h = xM_yN / 2;
  double2 *dst = out + (size_t)pair * xM_yN * xM_yN;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int a0 = a00 + yy;
    const int a1 = a10 + threadIdx.x;
    if (a0 < xM_yN && a1 < xM_yN) {
      const int d0 = centred ? (a0 + h) % xM_yN : a0;
      const int d1 = centred ? (a1 + h) % xM_yN : a1;
      dst[(size_t)d0 * xM_yN + d1] = P::out(P::ld(tile[threadIdx.x][yy]));
    }
  }
}

// subgrids[s] += nmbf[s] rolled to (fo0, fo1) (in xM samples).  Raw: both in
// raw layout, divided by xM^2; centred: both in fftshift layout, unscaled.
__global__ void k_rc_add_facet(const double2 *__restrict__ nmbf, int xM_yN, int xM, int fo0,
                               int fo1, int centred, double2 *__restrict__ sub) {
  const int j1 = blockIdx.x * blockDim.x + threadIdx.x;
  const int j0 = blockIdx.y;
  const int s = blockIdx.z;
  if (j1 >= xM_yN || j0 >= xM_yN) return;
  const int h = xM_yN / 2;
  // j is the frequency index offset by h: signed frequency f = j - h
  int src0, src1, dst0, dst1;
  if (centred) {
    src0 = j0;
    src1 = j1;
    // pad_mid puts centred index j at xM/2 - h + j; roll adds the facet offset
    dst0 = wrap1(xM / 2 - h + j0 + fo0, xM);
    dst1 = wrap1(xM / 2 - h + j1 + fo1, xM);
  } else {
    src0 = wrap1(j0 + h, xM_yN);
    src1 = wrap1(j1 + h, xM_yN);
    dst0 = wrap1(j0 - h + fo0, xM);
    dst1 = wrap1(j1 - h + fo1, xM);
  }
  double2 v = nmbf[((size_t)s * xM_yN + src0) * xM_yN + src1];
  if (!centred) {
    const double sc = 1.0 / ((double)xM * (double)xM);
    v.x *= sc;
    v.y *= sc;
  }
  double2 *d = sub + ((size_t)s * xM + dst0) * xM + dst1;
  double2 a = *d;
  a.x += v.x;
  a.y += v.y;
  *d = a;
}

// ---------------------------------------------------- subgrid -> facet
// The adjoint direction (notebook cell 18, 2-D by separability): for one
// facet and n0 x n1 subgrids whose spectra FS [n0][n1][xM][xM] are given.

__device__ __forceinline__ int signed_freq(int c, int n) { return c < n / 2 ? c : c - n; }

// inverse of the crop: padded index k (length np) -> cropped index, or -1
__device__ __forceinline__ int uncrop(int k, int n, int np) {
  if (k < n / 2) return k;
  if (k >= np - n / 2) return k - np + n;
  return -1;
}

// A[(i0 n1 + i1) xM_yN + a0][k]: the facet's xM_yN^2 block of each subgrid
// spectrum (rolled by the facet offset), times Fn on both axes, padded to
// xM_yP along axis 1 and divided by xM_yP (the inverse FFT that follows is
// unnormalised).  `centred`: FS in fftshift layout.
template <class P>
__global__ void k_rcT_split(const double2 *__restrict__ fs, int npair, int xM, int xM_yN,
                            int xM_yP, int fo0, int fo1, const typename P::WS *__restrict__ Fn,
                            int centred, typename P::S *__restrict__ out) {
  const size_t total = (size_t)npair * xM_yN * xM_yP;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % xM_yP);
    const size_t row = e / xM_yP;
    const int a0 = (int)(row % xM_yN);
    const size_t pair = row / xM_yN;
    const int c1 = uncrop(k, xM_yN, xM_yP);
    typename P::V v = P::zero();
    if (c1 >= 0) {
      // |signed frequency| <= xM_yN / 2 <= xM and 0 <= fo < xM
      int s0 = wrap1(signed_freq(a0, xM_yN) + fo0, xM);
      int s1 = wrap1(signed_freq(c1, xM_yN) + fo1, xM);
      if (centred) {
        s0 = (s0 + xM / 2) % xM;
        s1 = (s1 + xM / 2) % xM;
      }
      v = P::scale(P::in(fs[(pair * xM + s0) * xM + s1]),
                   P::wdiv(P::wmul(P::w(Fn, a0), P::w(Fn, c1)), xM_yP));
    }
    out[e] = P::st(v);
  }
}

// out[o][r][k] (k < yP) = sum over j < noff of the window of in[o][j][r][.]
// placed at offset offs[j]: position p (|p| within xMxN_yP / 2) of the
// periodic extension of the xM_yP samples, times m, lands at (p + off) mod yP.
// Grid-stride over the outputs; I is the index type (32-bit while the
// outputs fit, its divisions being a fraction of the 64-bit ones).
template <class P, typename I>
__global__ void k_rcT_scatter(const typename P::S *__restrict__ in, int outer, int noff,
                              int inner, int xM_yP, int xMxN_yP, int yP,
                              const int32_t *__restrict__ offs,
                              const typename P::WS *__restrict__ m,
                              typename P::S *__restrict__ out) {
  const I total = (I)outer * (I)inner * (I)yP;
  const int half = xMxN_yP / 2;
  for (I e = (I)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (I)gridDim.x * blockDim.x) {
    const int k = (int)(e % (I)yP);
    const I orow = e / (I)yP;
    const int r = (int)(orow % (I)inner);
    const I o = orow / (I)inner;
    typename P::V v = P::zero();
    for (int j = 0; j < noff; ++j) {
      // k, offs[j] in [0, yP): the signed distance in [-yP/2, yP/2)
      int p = k - offs[j];
      if (p >= yP / 2) p -= yP;
      if (p < -(yP / 2)) p += yP;
      if (p < -half || p >= xMxN_yP - half) continue;
      // |p| <= xMxN_yP / 2 <= xM_yP: one wrap each
      v = P::madd(v, P::w(m, p < 0 ? p + xMxN_yP : p),
                  P::ld(in[(((size_t)o * noff + j) * inner + r) * xM_yP +
                           (p < 0 ? p + xM_yP : p)]));
    }
    out[e] = P::st(v);
  }
}

// B[t][i0][k0]: rows (i0, a0) of acc [n0][xM_yN][yP] cropped to the yB facet
// positions t, transposed so that a0 runs along the rows, padded to xM_yP
// and divided by xM_yP.  Block 32 x 8: a tile of 32 positions t by 32 k0.
template <class P>
__global__ void k_rcT_crop_T_pad(const typename P::S *__restrict__ acc, int n0, int xM_yN,
                                 int yP, int yB, int xM_yP, typename P::S *__restrict__ out) {
  __shared__ typename P::S tile[32][33];
  const int i0 = blockIdx.z;
  const int t0 = blockIdx.y * 32;
  const int k00 = blockIdx.x * 32;
  // load tile[kk][tt] = acc[i0][a0(k0)][crop(t)]
  for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
    const int k0 = k00 + kk;
    const int t = t0 + threadIdx.x;
    typename P::V v = P::zero();
    const int a0 = k0 < xM_yP ? uncrop(k0, xM_yN, xM_yP) : -1;
    if (a0 >= 0 && t < yB) {
      const int kt = t < yB / 2 ? t : yP - yB + t;
      v = P::scale(P::ld(acc[((size_t)i0 * xM_yN + a0) * yP + kt]), P::wdiv(P::one(), xM_yP));
    }
    tile[kk][threadIdx.x] = P::st(v);
  }
  __syncthreads();
  for (int tt = threadIdx.y; tt < 32; tt += blockDim.y) {
    const int t = t0 + tt;
    const int k0 = k00 + threadIdx.x;
    if (t < yB && k0 < xM_yP)
      out[((size_t)t * n0 + i0) * xM_yP + k0] = tile[threadIdx.x][tt];
  }
}

// facet[s][t] (+)= acc2[t][crop(s)] Fb[s] Fb[t], transposed; `centred`:
// facet in fftshift layout.  Block 32 x 8: a tile of 32 t by 32 s.
template <class P>
__global__ void k_rcT_final(const typename P::S *__restrict__ acc2, int yP, int yB,
                            const typename P::WS *__restrict__ Fb, int centred, int accumulate,
                            double2 *__restrict__ facet) {
  __shared__ typename P::S tile[32][33];
  const int t0 = blockIdx.y * 32;
  const int s0 = blockIdx.x * 32;
  for (int tt = threadIdx.y; tt < 32; tt += blockDim.y) {
    const int t = t0 + tt;
    const int s = s0 + threadIdx.x;
    typename P::V v = P::zero();
    if (t < yB && s < yB) {
      const int ks = s < yB / 2 ? s : yP - yB + s;
      v = P::scale(P::ld(acc2[(size_t)t * yP + ks]), P::wmul(P::w(Fb, s), P::w(Fb, t)));
    }
    tile[tt][threadIdx.x] = P::st(v);
  }
  __syncthreads();
  const int h = yB / 2;
  for (int ss = threadIdx.y; ss < 32; ss += blockDim.y) {
    const int s = s0 + ss;
    const int t = t0 + threadIdx.x;
    if (s < yB && t < yB) {
      const int d0 = centred ? (s + h) % yB : s;
      const int d1 = centred ? (t + h) % yB : t;
      double2 *d = facet + (size_t)d0 * yB + d1;
      const double2 v = P::out(P::ld(tile[threadIdx.x][ss]));
      if (accumulate) {
        double2 a = *d;
        a.x += v.x;
        a.y += v.y;
        *d = a;
      } else {
        *d = v;
      }
    }
  }
}

// ------------------------------------------------ fused double-float passes
// I/O policies of the double-float row transforms (dfft.cuh) that take over
// the stage kernels above in the double-float pipeline: each window, prepare
// or crop step runs inside the loads or the stores of the transform next to
// it, with the same arithmetic as the stage kernel it replaces, so that stage
// array is neither written nor read.

// prepare_facet along the rows (k_rc_prep_rows) as the load of the yP inverse
// transforms; rows r < yB
struct IoPrep {
  const double2 *facet;
  const float2 *Fb;
  float4 *out;
  int yB, yP, centred;
  __device__ cdf ld(int64_t row, int k) const {
    const int t = uncrop(k, yB, yP);
    if (t < 0) return PDF::zero();
    const int r = (int)row, h = yB / 2;
    const int rs = centred ? (r + h) % yB : r;
    const int ts = centred ? (t + h) % yB : t;
    return PDF::scale(PDF::in(facet[(size_t)rs * yB + ts]), PDF::wdiv(PDF::w(Fb, t), yP));
  }
  __device__ void st(int64_t row, int k, const cdf &v) const {
    out[row * yP + k] = PDF::st(v);
  }
};

// extract_subgrid's window (k_rc_window): element i of transform row
// o * rows + r is the window of bf row r at offset offs[o]
struct WindowSrc {
  const float4 *bf;
  const int32_t *offs;
  const float2 *m;
  int rows, yP, xM_yP, xMxN_yP;
  __device__ cdf ld(int64_t row, int i) const {
    const int o = (int)row / rows, r = (int)row - ((int)row / rows) * rows;
    const int off = offs[o];
    const float4 *src = bf + (size_t)r * yP;
    cdf v = PDF::zero();
    if (i < (xMxN_yP + 1) / 2) v = PDF::madd(v, PDF::w(m, i), PDF::ld(src[wrap1(i + off, yP)]));
    if (i >= xM_yP - xMxN_yP / 2)
      v = PDF::madd(v, PDF::w(m, xMxN_yP - xM_yP + i),
                    PDF::ld(src[wrap1(i + off - xM_yP, yP)]));
    return v;
  }
};

struct IoWindowDF {  // the window in, double-float rows out
  WindowSrc w;
  float4 *out;
  __device__ cdf ld(int64_t row, int i) const { return w.ld(row, i); }
  __device__ void st(int64_t row, int i, const cdf &v) const {
    out[row * w.xM_yP + i] = PDF::st(v);
  }
};

// the window in; the final crop times Fn and transpose (k_rc_crop_T) out:
// transform row pair * xM_yN + a1, element crop_src(a0) -> out[pair][a0][a1]
struct IoWindowCrop {
  WindowSrc w;
  const float2 *Fn;
  double2 *out;
  int xM_yN, centred;
  __device__ cdf ld(int64_t row, int i) const { return w.ld(row, i); }
  __device__ void st(int64_t row, int i, const cdf &v) const {
    const int a0 = uncrop(i, xM_yN, w.xM_yP);
    if (a0 < 0) return;
    const int pair = (int)row / xM_yN, a1 = (int)row - ((int)row / xM_yN) * xM_yN;
    const int h = xM_yN / 2;
    const int d0 = centred ? (a0 + h) % xM_yN : a0;
    const int d1 = centred ? (a1 + h) % xM_yN : a1;
    out[((size_t)pair * xM_yN + d0) * xM_yN + d1] = PDF::out(PDF::scale(v, PDF::w(Fn, a0)));
  }
};

// the window in; the crop times Fn (k_rc_crop_T) and the sum into the
// subgrids (k_rc_add_facet) out: element (a0, a1) of subgrid pair's
// contribution lands at (off + f0 + fo0, off + f1 + fo1) mod xM, f the signed
// frequency of the raw index and off = xM/2 for centred subgrids (0 raw,
// where the contribution is also divided by xM^2) -- the same FP64 values
// and additions as k_rc_crop_T followed by k_rc_add_facet
struct IoWindowCropAdd {
  WindowSrc w;
  const float2 *Fn;
  double2 *sub;
  int xM_yN, xM, fo0, fo1, centred;
  __device__ cdf ld(int64_t row, int i) const { return w.ld(row, i); }
  __device__ void st(int64_t row, int i, const cdf &v) const {
    const int a0 = uncrop(i, xM_yN, w.xM_yP);
    if (a0 < 0) return;
    const int pair = (int)row / xM_yN, a1 = (int)row - ((int)row / xM_yN) * xM_yN;
    const int base = centred ? xM / 2 : 0;
    const int d0 = wrap1(base + signed_freq(a0, xM_yN) + fo0, xM);
    const int d1 = wrap1(base + signed_freq(a1, xM_yN) + fo1, xM);
    double2 o = PDF::out(PDF::scale(v, PDF::w(Fn, a0)));
    if (!centred) {
      const double sc = 1.0 / ((double)xM * (double)xM);
      o.x *= sc;
      o.y *= sc;
    }
    double2 *d = sub + ((size_t)pair * xM + d0) * xM + d1;
    double2 a = *d;
    a.x += o.x;
    a.y += o.y;
    *d = a;
  }
};

// subgrid -> facet: the split of each subgrid spectrum (k_rcT_split) as the
// load of the xM_yP inverse transforms; rows pair * xM_yN + a0
struct IoSplit {
  const double2 *fs;
  const float2 *Fn;
  float4 *out;
  int xM, xM_yN, xM_yP, fo0, fo1, centred;
  __device__ cdf ld(int64_t row, int k) const {
    const int c1 = uncrop(k, xM_yN, xM_yP);
    if (c1 < 0) return PDF::zero();
    const int pair = (int)row / xM_yN, a0 = (int)row - ((int)row / xM_yN) * xM_yN;
    int s0 = wrap1(signed_freq(a0, xM_yN) + fo0, xM);
    int s1 = wrap1(signed_freq(c1, xM_yN) + fo1, xM);
    if (centred) {
      s0 = (s0 + xM / 2) % xM;
      s1 = (s1 + xM / 2) % xM;
    }
    return PDF::scale(PDF::in(fs[((size_t)pair * xM + s0) * xM + s1]),
                      PDF::wdiv(PDF::wmul(PDF::w(Fn, a0), PDF::w(Fn, c1)), xM_yP));
  }
  __device__ void st(int64_t row, int k, const cdf &v) const {
    out[row * xM_yP + k] = PDF::st(v);
  }
};

// the windows of every subgrid summed into place (k_rcT_scatter): element k
// of transform row o * inner + r
struct ScatterSrc {
  const float4 *in;
  const int32_t *offs;
  const float2 *m;
  int noff, inner, xM_yP, xMxN_yP, yP;
  __device__ cdf ld(int64_t row, int k) const {
    const int o = (int)row / inner, r = (int)row - ((int)row / inner) * inner;
    const int half = xMxN_yP / 2;
    cdf v = PDF::zero();
    for (int j = 0; j < noff; ++j) {
      int p = k - offs[j];
      if (p >= yP / 2) p -= yP;
      if (p < -(yP / 2)) p += yP;
      if (p < -half || p >= xMxN_yP - half) continue;
      v = PDF::madd(v, PDF::w(m, p < 0 ? p + xMxN_yP : p),
                    PDF::ld(in[(((size_t)o * noff + j) * inner + r) * xM_yP +
                               (p < 0 ? p + xM_yP : p)]));
    }
    return v;
  }
};

// the scatter in; the facet crop times Fb x Fb and transpose (k_rcT_final)
// out: transform row t, element ks -> facet[s][t]
struct IoScatterFinal {
  ScatterSrc s;
  const float2 *Fb;
  double2 *facet;
  int yB, centred, accumulate;
  __device__ cdf ld(int64_t row, int k) const { return s.ld(row, k); }
  __device__ void st(int64_t row, int k, const cdf &v) const {
    const int sx = uncrop(k, yB, s.yP);
    if (sx < 0) return;
    const int t = (int)row, h = yB / 2;
    const int d0 = centred ? (sx + h) % yB : sx;
    const int d1 = centred ? (t + h) % yB : t;
    const double2 o = PDF::out(PDF::scale(v, PDF::wmul(PDF::w(Fb, sx), PDF::w(Fb, t))));
    double2 *d = facet + (size_t)d0 * yB + d1;
    if (accumulate) {
      double2 a = *d;
      a.x += o.x;
      a.y += o.y;
      *d = a;
    } else {
      *d = o;
    }
  }
};

// ------------------------------------------------------------------ host side

// the window tables of the complex128 pipeline (the double-float one reads
// the split copies d_Fb2, d_Fn2, d_m2)
template <class P>
struct Tab;
template <>
struct Tab<P64> {
  static const double *Fb(const cg_recombine *h) { return h->d_Fb; }
  static const double *Fn(const cg_recombine *h) { return h->d_Fn; }
  static const double *m(const cg_recombine *h) { return h->d_m; }
};
template <>
struct Tab<PDF> {
  static const float2 *Fb(const cg_recombine *h) { return h->d_Fb2; }
  static const float2 *Fn(const cg_recombine *h) { return h->d_Fn2; }
  static const float2 *m(const cg_recombine *h) { return h->d_m2; }
};

// complex128 only: Fb = 1 / PSWF spans many decades at the facet edge (6.4e6
// for the 512 / 128 / 140 test set), and the contributions come out of
// intermediates 1e3 times larger than their peak, so single-precision FFTs
// lose 1e-3 of the result (measured) where the method delivers 1e-7.
int rows_fft(const cg_recombine *h, double2 *data, int batch, int len, int dir, cudaStream_t st) {
  // power-of-two rows in double-float arithmetic on the FP32 units: the FP64
  // transforms are bound by GB300's FP64 rate
  if (h->fft_mode == 0 && dfft_supported(len))
    return dfft_rows(data, batch, len, dir == CUFFT_INVERSE, st);
  cufftHandle plan;
  int rc = fft_plan(batch, 1, len, CUFFT_Z2Z, &plan);
  if (rc) return rc;
  if (cufftSetStream(plan, st) != CUFFT_SUCCESS)
    return set_error(CG_ERR_CUDA, "cufftSetStream failed");
  const cufftResult r =
      cufftExecZ2Z(plan, (cufftDoubleComplex *)data, (cufftDoubleComplex *)data, dir);
  return r == CUFFT_SUCCESS ? CG_OK : set_error(CG_ERR_CUDA, "cufftExec failed: %d", (int)r);
}

int rows_fft(const cg_recombine *, float4 *data, int batch, int len, int dir, cudaStream_t st) {
  return dfft_rows_df(data, batch, len, dir == CUFFT_INVERSE, st);
}

// The pipeline of a configuration (unless FP64 cuFFT was asked for): both
// transform lengths within one CTA's double-float FFT (64..2048): the fused
// double-float passes; yP up to 8192 (the four-step double-float rows): the
// double-float stage kernels; otherwise complex128 and FP64 cuFFT.
enum { PIPE_C128 = 0, PIPE_DF_FUSED = 1, PIPE_DF = 2 };
int pipeline(const cg_recombine *h) {
  if (h->fft_mode != 0) return PIPE_C128;
  if (dfft_supported(h->yP) && dfft_supported(h->xM_yP)) return PIPE_DF_FUSED;
  if (dfft_long_supported(h->yP) && dfft_long_supported(h->xM_yP)) return PIPE_DF;
  return PIPE_C128;
}

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

inline unsigned grid_for(size_t n);

template <class P>
void launch_scatter(const typename P::S *in, int outer, int noff, int inner, int xM_yP,
                    int xMxN_yP, int yP, const int32_t *offs, const typename P::WS *m,
                    typename P::S *out, cudaStream_t st) {
  const size_t total = (size_t)outer * inner * yP;
  if (total < ((size_t)1 << 31))
    k_rcT_scatter<P, uint32_t><<<grid_for(total), 256, 0, st>>>(in, outer, noff, inner, xM_yP,
                                                                xMxN_yP, yP, offs, m, out);
  else
    k_rcT_scatter<P, size_t><<<grid_for(total), 256, 0, st>>>(in, outer, noff, inner, xM_yP,
                                                              xMxN_yP, yP, offs, m, out);
}

// grid-stride launches: enough 256-thread blocks to fill the GPU a few times
inline unsigned grid_for(size_t n) {
  const size_t want = (n + 255) / 256;
  return (unsigned)std::max<size_t>(1, std::min<size_t>(want, (size_t)num_sms() * 16));
}

struct WsLayout {
  size_t bf, mbf, bf2, mbf2, offs, nm, total;
};

// subgrid -> facet: A [n0 n1 xM_yN][xM_yP], acc [n0 xM_yN][yP], B [yB n0][xM_yP],
// acc2 [yB][yP], the offsets
struct WsLayoutT {
  size_t a, acc, b, acc2, offs, total;
};

WsLayoutT ws_layout_t(const cg_recombine *h, int n0, int n1) {
  const size_t e = sizeof(double2);
  WsLayoutT L;
  L.a = 0;
  L.acc = L.a + align256((size_t)n0 * n1 * h->xM_yN * h->xM_yP * e);
  L.b = L.acc + align256((size_t)n0 * h->xM_yN * h->yP * e);
  L.acc2 = L.b + align256((size_t)h->yB * n0 * h->xM_yP * e);
  L.offs = L.acc2 + align256((size_t)h->yB * h->yP * e);
  L.total = L.offs + align256((size_t)(n0 + n1) * sizeof(int32_t));
  return L;
}

template <class P>
int subgrids_to_facet(cg_recombine *h, const void *fs, int centred, int n0, int n1, int fo0,
                      int fo1, void *facet, int out_centred, int accumulate, char *ws,
                      const WsLayoutT &L, cudaStream_t st) {
  typedef typename P::S S;
  S *A = (S *)(ws + L.a);
  S *acc = (S *)(ws + L.acc);
  S *B = (S *)(ws + L.b);
  S *acc2 = (S *)(ws + L.acc2);
  const int32_t *offs0 = (const int32_t *)(ws + L.offs);
  const int32_t *offs1 = offs0 + n0;
  const int yB = h->yB, yP = h->yP, xM = h->xM, xM_yP = h->xM_yP, xM_yN = h->xM_yN;
  int rc;
  k_rcT_split<P><<<grid_for((size_t)n0 * n1 * xM_yN * xM_yP), 256, 0, st>>>(
      (const double2 *)fs, n0 * n1, xM, xM_yN, xM_yP, fo0, fo1, Tab<P>::Fn(h), centred, A);
  CG_LAUNCH("recombine split subgrids");
  if ((rc = rows_fft(h, A, n0 * n1 * xM_yN, xM_yP, CUFFT_INVERSE, st))) return rc;
  launch_scatter<P>(A, n0, n1, xM_yN, xM_yP, h->xMxN_yP, yP, offs1, Tab<P>::m(h), acc, st);
  CG_LAUNCH("recombine subgrid windows (axis 1)");
  if ((rc = rows_fft(h, acc, n0 * xM_yN, yP, CUFFT_FORWARD, st))) return rc;
  k_rcT_crop_T_pad<P><<<dim3((xM_yP + 31) / 32, (yB + 31) / 32, n0), dim3(32, 8), 0, st>>>(
      acc, n0, xM_yN, yP, yB, xM_yP, B);
  CG_LAUNCH("recombine crop to the facet (axis 1)");
  if ((rc = rows_fft(h, B, yB * n0, xM_yP, CUFFT_INVERSE, st))) return rc;
  launch_scatter<P>(B, yB, n0, 1, xM_yP, h->xMxN_yP, yP, offs0, Tab<P>::m(h), acc2, st);
  CG_LAUNCH("recombine subgrid windows (axis 0)");
  if ((rc = rows_fft(h, acc2, yB, yP, CUFFT_FORWARD, st))) return rc;
  k_rcT_final<P><<<dim3((yB + 31) / 32, (yB + 31) / 32), dim3(32, 8), 0, st>>>(
      acc2, yP, yB, Tab<P>::Fb(h), out_centred, accumulate, (double2 *)facet);
  CG_LAUNCH("recombine facet");
  return CG_OK;
}

WsLayout ws_layout(const cg_recombine *h, int n0, int n1) {
  const size_t e = sizeof(double2);
  WsLayout L;
  L.bf = 0;
  L.mbf = L.bf + align256((size_t)h->yB * h->yP * e);
  L.bf2 = L.mbf + align256((size_t)n1 * h->yB * h->xM_yP * e);
  L.mbf2 = L.bf2 + align256((size_t)n1 * h->xM_yN * h->yP * e);
  L.offs = L.mbf2 + align256((size_t)n0 * n1 * h->xM_yN * h->xM_yP * e);
  // the contributions, for cg_recombine_facet_add on the complex128 pipeline
  L.nm = L.offs + align256((size_t)(n0 + n1) * sizeof(int32_t));
  L.total = L.nm + align256((size_t)n0 * n1 * h->xM_yN * h->xM_yN * e);
  return L;
}

template <class P>
int facet_to_subgrids(cg_recombine *h, const void *facet, int centred, int n0, int n1,
                      void *nmbf, int out_centred, char *ws, const WsLayout &L,
                      cudaStream_t st) {
  typedef typename P::S S;
  S *bf = (S *)(ws + L.bf);
  S *mbf = (S *)(ws + L.mbf);
  S *bf2 = (S *)(ws + L.bf2);
  S *mbf2 = (S *)(ws + L.mbf2);
  const int32_t *offs0 = (const int32_t *)(ws + L.offs);
  const int32_t *offs1 = offs0 + n0;
  const int yB = h->yB, yP = h->yP, xM_yP = h->xM_yP, xM_yN = h->xM_yN;
  int rc;
  const unsigned g1 = grid_for((size_t)yB * yP);
  k_rc_prep_rows<P><<<g1, 256, 0, st>>>((const double2 *)facet, yB, yB, yP, Tab<P>::Fb(h),
                                         centred, bf);
  CG_LAUNCH("recombine prepare facet (axis 1)");
  if ((rc = rows_fft(h, bf, yB, yP, CUFFT_INVERSE, st))) return rc;
  k_rc_window<P><<<grid_for((size_t)n1 * yB * xM_yP), 256, 0, st>>>(
      bf, yB, yP, offs1, n1, xM_yP, h->xMxN_yP, Tab<P>::m(h), mbf);
  CG_LAUNCH("recombine extract subgrid (axis 1)");
  if ((rc = rows_fft(h, mbf, n1 * yB, xM_yP, CUFFT_FORWARD, st))) return rc;
  k_rc_crop_prep_T<P><<<dim3((yP + 31) / 32, (xM_yN + 31) / 32, n1), dim3(32, 8), 0, st>>>(
      mbf, yB, xM_yP, xM_yN, Tab<P>::Fn(h), Tab<P>::Fb(h), yP, bf2);
  CG_LAUNCH("recombine prepare facet (axis 0)");
  if ((rc = rows_fft(h, bf2, n1 * xM_yN, yP, CUFFT_INVERSE, st))) return rc;
  k_rc_window<P><<<grid_for((size_t)n0 * n1 * xM_yN * xM_yP), 256, 0, st>>>(
      bf2, n1 * xM_yN, yP, offs0, n0, xM_yP, h->xMxN_yP, Tab<P>::m(h), mbf2);
  CG_LAUNCH("recombine extract subgrid (axis 0)");
  if ((rc = rows_fft(h, mbf2, n0 * n1 * xM_yN, xM_yP, CUFFT_FORWARD, st))) return rc;
  k_rc_crop_T<P><<<dim3((xM_yN + 31) / 32, (xM_yN + 31) / 32, n0 * n1), dim3(32, 8), 0, st>>>(
      mbf2, n1, xM_yP, xM_yN, Tab<P>::Fn(h), out_centred, (double2 *)nmbf);
  CG_LAUNCH("recombine crop");
  return CG_OK;
}

// The double-float pipelines with the fused passes: per facet, four
// transform launches and one transpose kernel each way (and the scatter
// kernel of the first axis on the way back).
// the last transforms' stores: the contributions (IoWindowCrop) or their sum
// into the subgrids (IoWindowCropAdd)
template <class LastIO>
int facet_df_passes(cg_recombine *h, const void *facet, int centred, int n0, int n1,
                    LastIO last, char *ws, const WsLayout &L, cudaStream_t st);

int facet_to_subgrids_df(cg_recombine *h, const void *facet, int centred, int n0, int n1,
                         void *nmbf, int out_centred, char *ws, const WsLayout &L,
                         cudaStream_t st) {
  const int32_t *offs0 = (const int32_t *)(ws + L.offs);
  const WindowSrc w2{(const float4 *)(ws + L.bf2), offs0, h->d_m2, n1 * h->xM_yN, h->yP,
                     h->xM_yP, h->xMxN_yP};
  return facet_df_passes(h, facet, centred, n0, n1,
                         IoWindowCrop{w2, h->d_Fn2, (double2 *)nmbf, h->xM_yN, out_centred}, ws,
                         L, st);
}

int facet_add_df(cg_recombine *h, const void *facet, int centred, int n0, int n1, int fo0,
                 int fo1, void *sub, int sub_centred, char *ws, const WsLayout &L,
                 cudaStream_t st) {
  const int32_t *offs0 = (const int32_t *)(ws + L.offs);
  const WindowSrc w2{(const float4 *)(ws + L.bf2), offs0, h->d_m2, n1 * h->xM_yN, h->yP,
                     h->xM_yP, h->xMxN_yP};
  return facet_df_passes(h, facet, centred, n0, n1,
                         IoWindowCropAdd{w2, h->d_Fn2, (double2 *)sub, h->xM_yN, h->xM, fo0,
                                         fo1, sub_centred},
                         ws, L, st);
}

template <class LastIO>
int facet_df_passes(cg_recombine *h, const void *facet, int centred, int n0, int n1,
                    LastIO last, char *ws, const WsLayout &L, cudaStream_t st) {
  float4 *bf = (float4 *)(ws + L.bf);
  float4 *mbf = (float4 *)(ws + L.mbf);
  float4 *bf2 = (float4 *)(ws + L.bf2);
  const int32_t *offs0 = (const int32_t *)(ws + L.offs);
  const int32_t *offs1 = offs0 + n0;
  const int yB = h->yB, yP = h->yP, xM_yP = h->xM_yP, xM_yN = h->xM_yN, xMxN = h->xMxN_yP;
  int rc;
  // prepare along axis 1 in the loads of the yP inverse transforms
  if ((rc = dfft_rows_io(IoPrep{(const double2 *)facet, h->d_Fb2, bf, yB, yP, centred}, yB, yP,
                         1, st)))
    return rc;
  // each subgrid column offset's window in the loads of the xM_yP transforms
  if ((rc = dfft_rows_io(IoWindowDF{WindowSrc{bf, offs1, h->d_m2, yB, yP, xM_yP, xMxN}, mbf},
                         (int64_t)n1 * yB, xM_yP, 0, st)))
    return rc;
  k_rc_crop_prep_T<PDF><<<dim3((yP + 31) / 32, (xM_yN + 31) / 32, n1), dim3(32, 8), 0, st>>>(
      mbf, yB, xM_yP, xM_yN, h->d_Fn2, h->d_Fb2, yP, bf2);
  CG_LAUNCH("recombine prepare facet (axis 0)");
  if ((rc = dfft_rows_df(bf2, (int64_t)n1 * xM_yN, yP, 1, st))) return rc;
  // each subgrid row offset's window in the loads, the crop in the stores
  return dfft_rows_io(last, (int64_t)n0 * n1 * xM_yN, xM_yP, 0, st);
}

int subgrids_to_facet_df(cg_recombine *h, const void *fs, int centred, int n0, int n1, int fo0,
                         int fo1, void *facet, int out_centred, int accumulate, char *ws,
                         const WsLayoutT &L, cudaStream_t st) {
  float4 *A = (float4 *)(ws + L.a);
  float4 *acc = (float4 *)(ws + L.acc);
  float4 *B = (float4 *)(ws + L.b);
  const int32_t *offs0 = (const int32_t *)(ws + L.offs);
  const int32_t *offs1 = offs0 + n0;
  const int yB = h->yB, yP = h->yP, xM = h->xM, xM_yP = h->xM_yP, xM_yN = h->xM_yN;
  const int xMxN = h->xMxN_yP;
  int rc;
  // each subgrid spectrum's share of the facet in the loads of the xM_yP inverse transforms
  if ((rc = dfft_rows_io(IoSplit{(const double2 *)fs, h->d_Fn2, A, xM, xM_yN, xM_yP, fo0, fo1,
                                 centred},
                         (int64_t)n0 * n1 * xM_yN, xM_yP, 1, st)))
    return rc;
  // the subgrid column windows summed by a separate kernel: in the loads of
  // the yP transforms (ScatterSrc) the 2048-point kernel's occupancy leaves
  // the offset loop's dependent loads exposed (measured 193 us against 158
  // for the pair on the 8192 / 1280 / 512 set)
  launch_scatter<PDF>(A, n0, n1, xM_yN, xM_yP, xMxN, yP, offs1, h->d_m2, acc, st);
  CG_LAUNCH("recombine subgrid windows (axis 1)");
  if ((rc = dfft_rows_df(acc, (int64_t)n0 * xM_yN, yP, 0, st))) return rc;
  k_rcT_crop_T_pad<PDF><<<dim3((xM_yP + 31) / 32, (yB + 31) / 32, n0), dim3(32, 8), 0, st>>>(
      acc, n0, xM_yN, yP, yB, xM_yP, B);
  CG_LAUNCH("recombine crop to the facet (axis 1)");
  if ((rc = dfft_rows_df(B, (int64_t)yB * n0, xM_yP, 1, st))) return rc;
  // the subgrid row windows summed in the loads, the facet crop in the stores
  return dfft_rows_io(
      IoScatterFinal{ScatterSrc{B, offs0, h->d_m2, n0, 1, xM_yP, xMxN, yP}, h->d_Fb2,
                     (double2 *)facet, yB, out_centred, accumulate},
      yB, yP, 0, st);
}

// generate_m (recombine.c:35-67): the PSWF times the sinc of the xM box, then
// the DCT-I of length yP/2 + 1 (X_j = 0 from yN/2 on), mirrored to xMxN_yP.
std::vector<double> generate_m(int N, int yP, int yN, int xM, int xMxN_yP, const double *pswf) {
  const int n = yP / 2 + 1;
  std::vector<double> X(n, 0.0);
  X[0] = pswf[0] * xM / N;
  for (int i = 1; i < yN / 2 && i < n; ++i) {
    const double x = (double)i * xM / N;
    X[i] = pswf[i] * (std::sin(x * M_PI) / x / M_PI) * xM / N;
  }
  const int half = xMxN_yP / 2;
  std::vector<double> Y(half + 1);
  for (int k = 0; k <= half; ++k) {
    double s = X[0] + ((k & 1) ? -X[n - 1] : X[n - 1]);
    for (int j = 1; j < n - 1; ++j)
      if (X[j] != 0.0) s += 2 * X[j] * std::cos(M_PI * (double)j * k / (double)(n - 1));
    Y[k] = s;
  }
  std::vector<double> m(xMxN_yP);
  for (int i = 0; i <= half; ++i) m[i] = Y[i];
  for (int i = half + 1; i < xMxN_yP; ++i) m[i] = Y[xMxN_yP - i];
  return m;
}

int upload(const std::vector<double> &v, double **d) {
  CG_CUDA(cudaMalloc(d, v.size() * sizeof(double)));
  CG_CUDA(cudaMemcpy(*d, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
  return CG_OK;
}

int upload_df(const std::vector<double> &v, float2 **d) {
  std::vector<float2> s(v.size());
  for (size_t i = 0; i < v.size(); ++i) {
    const float hi = (float)v[i];
    s[i] = make_float2(hi, (float)(v[i] - (double)hi));
  }
  CG_CUDA(cudaMalloc(d, s.size() * sizeof(float2)));
  CG_CUDA(cudaMemcpy(*d, s.data(), s.size() * sizeof(float2), cudaMemcpyHostToDevice));
  return CG_OK;
}

}  // namespace

extern "C" {

int cg_recombine_create(int image_size, int subgrid_spacing, const double *pswf, int yB, int yN,
                        int yP, int xA, int xM, int xMxN_yP, cg_recombine **out) {
  CG_REQUIRE(out && pswf, "bad recombine_create arguments");
  *out = nullptr;
  CG_REQUIRE(image_size > 0 && subgrid_spacing > 0 && yB > 0 && yN > 0 && yP > 0 && xA > 0 &&
                 xM > 0 && xMxN_yP > 0,
             "recombine sizes must be positive");
  // the side conditions of recombine2d_set_config (recombine.c:139-172)
  CG_REQUIRE(image_size % subgrid_spacing == 0, "image_size %% subgrid_spacing != 0");
  const int facet_spacing = image_size / subgrid_spacing;
  CG_REQUIRE(image_size % xM == 0, "image_size %% xM_size != 0");
  const int xM_step = image_size / xM;
  CG_REQUIRE(facet_spacing % xM_step == 0, "facet spacing not a multiple of image/xM");
  CG_REQUIRE(((long long)subgrid_spacing * yP) % image_size == 0,
             "subgrid_spacing * yP_size not a multiple of image_size");
  CG_REQUIRE(yB % facet_spacing == 0, "yB_size not a multiple of the facet spacing");
  CG_REQUIRE(xA % subgrid_spacing == 0, "xA_size not a multiple of subgrid_spacing");
  CG_REQUIRE(((long long)xM * yP) % image_size == 0, "xM_size * yP_size not a multiple of image");
  CG_REQUIRE(((long long)xM * yN) % image_size == 0, "xM_size * yN_size not a multiple of image");
  const int xM_yP = (int)((long long)xM * yP / image_size);
  const int xM_yN = (int)((long long)xM * yN / image_size);
  CG_REQUIRE(yN % xM_yN == 0, "yN_size not a multiple of xM_yN_size");  // generate_Fn
  CG_REQUIRE((xMxN_yP - xM_yP) % 2 == 0 && xMxN_yP >= xM_yP && xMxN_yP <= 2 * xM_yP,
             "xMxN_yP_size - xM_yP_size must be even, xM_yP <= xMxN_yP <= 2 xM_yP");
  CG_REQUIRE(yB % 2 == 0 && xM_yN % 2 == 0 && yB <= yP && yB <= yN && xM_yN <= xM_yP &&
                 xM_yN <= xM,
             "need even yB, xM_yN and yB <= yP, yN; xM_yN <= xM_yP, xM");
  cg_recombine *h = new cg_recombine();
  h->N = image_size;
  h->subgrid_spacing = subgrid_spacing;
  h->facet_spacing = facet_spacing;
  h->yB = yB;
  h->yN = yN;
  h->yP = yP;
  h->xA = xA;
  h->xM = xM;
  h->xMxN_yP = xMxN_yP;
  h->xM_yP = xM_yP;
  h->xM_yN = xM_yN;
  h->fft_mode = 0;
  h->yP_spacing = (int)((long long)subgrid_spacing * yP / image_size);
  h->xM_spacing = (int)((long long)facet_spacing * xM / image_size);
  // generate_Fb / generate_Fn (recombine.c:12-33) from the raw PSWF [yN]
  std::vector<double> Fb(yB), Fn(xM_yN);
  for (int i = 0; i <= yB / 2; ++i) Fb[i] = 1 / pswf[i];
  for (int i = yB / 2 + 1; i < yB; ++i) Fb[i] = Fb[yB - i];
  for (int i = 0; i < xM_yN; ++i) Fn[i] = pswf[(size_t)i * (yN / xM_yN)];
  const std::vector<double> m = generate_m(image_size, yP, yN, xM, xMxN_yP, pswf);
  int rc;
  if ((rc = upload(Fb, &h->d_Fb)) || (rc = upload(Fn, &h->d_Fn)) || (rc = upload(m, &h->d_m)) ||
      (rc = upload_df(Fb, &h->d_Fb2)) || (rc = upload_df(Fn, &h->d_Fn2)) ||
      (rc = upload_df(m, &h->d_m2))) {
    cg_recombine_destroy(h);
    return rc;
  }
  *out = h;
  return CG_OK;
}

int cg_recombine_destroy(cg_recombine *h) {
  if (!h) return CG_OK;
  cudaFree(h->d_Fb);
  cudaFree(h->d_Fn);
  cudaFree(h->d_m);
  cudaFree(h->d_Fb2);
  cudaFree(h->d_Fn2);
  cudaFree(h->d_m2);
  delete h;
  return CG_OK;
}

int cg_recombine_set_fft(cg_recombine *h, int mode) {
  CG_REQUIRE(h && (mode == 0 || mode == 1), "fft mode 0 (double-float) or 1 (FP64 cuFFT)");
  h->fft_mode = mode;
  return CG_OK;
}

int cg_recombine_sizes(const cg_recombine *h, int32_t *sizes) {
  CG_REQUIRE(h && sizes, "bad recombine_sizes arguments");
  sizes[0] = h->xM_yP;
  sizes[1] = h->xM_yN;
  sizes[2] = h->facet_spacing;
  sizes[3] = h->yP_spacing;
  sizes[4] = h->xM_spacing;
  return CG_OK;
}

int cg_recombine_windows(const cg_recombine *h, double *Fb, double *Fn, double *m) {
  CG_REQUIRE(h, "bad recombine_windows arguments");
  if (Fb) CG_CUDA(cudaMemcpy(Fb, h->d_Fb, h->yB * sizeof(double), cudaMemcpyDeviceToHost));
  if (Fn) CG_CUDA(cudaMemcpy(Fn, h->d_Fn, h->xM_yN * sizeof(double), cudaMemcpyDeviceToHost));
  if (m) CG_CUDA(cudaMemcpy(m, h->d_m, h->xMxN_yP * sizeof(double), cudaMemcpyDeviceToHost));
  return CG_OK;
}

size_t cg_recombine_workspace_bytes(const cg_recombine *h, int n0, int n1) {
  if (!h || n0 < 0 || n1 < 0) return 0;
  return std::max(ws_layout(h, n0, n1).total, ws_layout_t(h, n0, n1).total);
}

int cg_recombine_facet_to_subgrids(cg_recombine *h, const void *facet, int centred,
                                   const int32_t *subgrid_off0, int n0,
                                   const int32_t *subgrid_off1, int n1, void *nmbf,
                                   int out_centred, void *ws, size_t ws_bytes, int32_t *d_status,
                                   cg_stream_t stream) {
  CG_REQUIRE(h && facet && d_status && n0 >= 0 && n1 >= 0,
             "bad recombine_facet_to_subgrids arguments");
  if (n0 == 0 || n1 == 0) return CG_OK;
  CG_REQUIRE(nmbf && subgrid_off0 && subgrid_off1, "bad recombine_facet_to_subgrids arguments");
  CG_REQUIRE(n1 <= 65535 && (long long)n0 * n1 <= 65535,
             "at most 65535 subgrids (n0 * n1) per call; split the offsets");
  const WsLayout L = ws_layout(h, n0, n1);
  if (!ws || ws_bytes < L.total)
    return set_error(CG_ERR_WORKSPACE, "recombine needs %zu workspace bytes", L.total);
  cudaStream_t st = (cudaStream_t)stream;
  char *w = (char *)ws;
  k_rc_offsets<<<(n0 + n1 + 255) / 256, 256, 0, st>>>(subgrid_off0, n0, subgrid_off1, n1,
                                                      h->subgrid_spacing, h->yP_spacing, h->yP,
                                                      (int32_t *)(w + L.offs), d_status);
  CG_LAUNCH("recombine offsets");
  switch (pipeline(h)) {
    case PIPE_DF_FUSED:
      return facet_to_subgrids_df(h, facet, centred, n0, n1, nmbf, out_centred, w, L, st);
    case PIPE_DF:
      return facet_to_subgrids<PDF>(h, facet, centred, n0, n1, nmbf, out_centred, w, L, st);
  }
  return facet_to_subgrids<P64>(h, facet, centred, n0, n1, nmbf, out_centred, w, L, st);
}

int cg_recombine_facet_add(cg_recombine *h, const void *facet, int centred,
                           const int32_t *subgrid_off0, int n0, const int32_t *subgrid_off1,
                           int n1, int facet_off0, int facet_off1, void *subgrids,
                           int sub_centred, void *ws, size_t ws_bytes, int32_t *d_status,
                           cg_stream_t stream) {
  CG_REQUIRE(h && facet && d_status && n0 >= 0 && n1 >= 0, "bad recombine_facet_add arguments");
  if (n0 == 0 || n1 == 0) return CG_OK;
  CG_REQUIRE(subgrids && subgrid_off0 && subgrid_off1, "bad recombine_facet_add arguments");
  CG_REQUIRE(n1 <= 65535 && (long long)n0 * n1 <= 65535,
             "at most 65535 subgrids (n0 * n1) per call; split the offsets");
  CG_REQUIRE(pmod(facet_off0, h->facet_spacing) == 0 && pmod(facet_off1, h->facet_spacing) == 0,
             "facet offsets must be multiples of the facet spacing %d", h->facet_spacing);
  const WsLayout L = ws_layout(h, n0, n1);
  if (!ws || ws_bytes < L.total)
    return set_error(CG_ERR_WORKSPACE, "recombine needs %zu workspace bytes", L.total);
  cudaStream_t st = (cudaStream_t)stream;
  char *w = (char *)ws;
  k_rc_offsets<<<(n0 + n1 + 255) / 256, 256, 0, st>>>(subgrid_off0, n0, subgrid_off1, n1,
                                                      h->subgrid_spacing, h->yP_spacing, h->yP,
                                                      (int32_t *)(w + L.offs), d_status);
  CG_LAUNCH("recombine offsets");
  // facet offsets in xM samples, reduced to [0, xM) (the kernels wrap once)
  const int fo0 = pmod((long long)facet_off0 / h->facet_spacing * h->xM_spacing, h->xM);
  const int fo1 = pmod((long long)facet_off1 / h->facet_spacing * h->xM_spacing, h->xM);
  const int pipe = pipeline(h);
  if (pipe == PIPE_DF_FUSED)
    return facet_add_df(h, facet, centred, n0, n1, fo0, fo1, subgrids, sub_centred, w, L, st);
  double2 *nm = (double2 *)(w + L.nm);
  int rc = pipe == PIPE_DF
               ? facet_to_subgrids<PDF>(h, facet, centred, n0, n1, nm, sub_centred, w, L, st)
               : facet_to_subgrids<P64>(h, facet, centred, n0, n1, nm, sub_centred, w, L, st);
  if (rc) return rc;
  const dim3 grid((h->xM_yN + 127) / 128, h->xM_yN, n0 * n1);
  k_rc_add_facet<<<grid, 128, 0, st>>>(nm, h->xM_yN, h->xM, fo0, fo1, sub_centred,
                                       (double2 *)subgrids);
  CG_LAUNCH("recombine add facet");
  return CG_OK;
}

int cg_recombine_subgrids_to_facet(cg_recombine *h, const void *fs, int centred,
                                   const int32_t *subgrid_off0, int n0,
                                   const int32_t *subgrid_off1, int n1, int facet_off0,
                                   int facet_off1, void *facet, int out_centred, int accumulate,
                                   void *ws, size_t ws_bytes, int32_t *d_status,
                                   cg_stream_t stream) {
  CG_REQUIRE(h && facet && d_status && n0 >= 0 && n1 >= 0,
             "bad recombine_subgrids_to_facet arguments");
  CG_REQUIRE(pmod(facet_off0, h->facet_spacing) == 0 && pmod(facet_off1, h->facet_spacing) == 0,
             "facet offsets must be multiples of the facet spacing %d", h->facet_spacing);
  cudaStream_t st = (cudaStream_t)stream;
  if (n0 == 0 || n1 == 0) {
    if (!accumulate)
      CG_CUDA(cudaMemsetAsync(facet, 0, (size_t)h->yB * h->yB * sizeof(double2), st));
    return CG_OK;
  }
  CG_REQUIRE(fs && subgrid_off0 && subgrid_off1, "bad recombine_subgrids_to_facet arguments");
  CG_REQUIRE(n0 <= 65535 && (long long)n0 * n1 * h->xM_yN <= (1ll << 31) - 1,
             "too many subgrids for one call; split the offsets");
  const WsLayoutT L = ws_layout_t(h, n0, n1);
  if (!ws || ws_bytes < L.total)
    return set_error(CG_ERR_WORKSPACE, "recombine needs %zu workspace bytes", L.total);
  char *w = (char *)ws;
  k_rc_offsets<<<(n0 + n1 + 255) / 256, 256, 0, st>>>(subgrid_off0, n0, subgrid_off1, n1,
                                                      h->subgrid_spacing, h->yP_spacing, h->yP,
                                                      (int32_t *)(w + L.offs), d_status);
  CG_LAUNCH("recombine offsets");
  // facet offsets in xM samples, reduced to [0, xM) (the kernels wrap once)
  const int fo0 = pmod((long long)facet_off0 / h->facet_spacing * h->xM_spacing, h->xM);
  const int fo1 = pmod((long long)facet_off1 / h->facet_spacing * h->xM_spacing, h->xM);
  switch (pipeline(h)) {
    case PIPE_DF_FUSED:
      return subgrids_to_facet_df(h, fs, centred, n0, n1, fo0, fo1, facet, out_centred,
                                  accumulate, w, L, st);
    case PIPE_DF:
      return subgrids_to_facet<PDF>(h, fs, centred, n0, n1, fo0, fo1, facet, out_centred,
                                    accumulate, w, L, st);
  }
  return subgrids_to_facet<P64>(h, fs, centred, n0, n1, fo0, fo1, facet, out_centred,
                                accumulate, w, L, st);
}

int cg_recombine_add_facet(const cg_recombine *h, const void *nmbf, int n, int facet_off0,
                           int facet_off1, int centred, void *subgrids, cg_stream_t stream) {
  CG_REQUIRE(h && n >= 0 && (n == 0 || (nmbf && subgrids)), "bad recombine_add_facet arguments");
  if (n == 0) return CG_OK;
  CG_REQUIRE(pmod(facet_off0, h->facet_spacing) == 0 && pmod(facet_off1, h->facet_spacing) == 0,
             "facet offsets must be multiples of the facet spacing %d", h->facet_spacing);
  CG_REQUIRE(n <= 65535, "too many subgrids for one call");
  // facet offsets in xM samples, reduced to [0, xM) (the kernel wraps once)
  const int fo0 = pmod((long long)facet_off0 / h->facet_spacing * h->xM_spacing, h->xM);
  const int fo1 = pmod((long long)facet_off1 / h->facet_spacing * h->xM_spacing, h->xM);
  const dim3 grid((h->xM_yN + 127) / 128, h->xM_yN, n);
  cudaStream_t st = (cudaStream_t)stream;
  k_rc_add_facet<<<grid, 128, 0, st>>>((const double2 *)nmbf, h->xM_yN, h->xM, fo0, fo1,
                                                centred, (double2 *)subgrids);
  CG_LAUNCH("recombine add facet");
  return CG_OK;
}

}  // extern "C"
