// Kernel generation on the GPU (K5, K6).
//
// kernel_oversample (crocodile/synthesis.py:330-354):
//   extract_oversampled(fft(pad_mid(ff, N*Q)), Q, s)
// runs as one fill pass (pad + ifftshift folded into the write index), a
// batched cuFFT Z2Z and one extract pass (fftshift folded into the read
// index).  w_kernel (:357-377) computes its far field
// exp(2 pi i w (1 - sqrt(1 - l^2 - m^2))) (:273-293) inside the fill pass
// in FP64, with every product and sum explicitly rounded so the phase is
// the one numpy evaluates.  aw_kernel_fn (:701-734) convolves two A kernels
// and then the result with every oversampled w sub-kernel ('same' crops as
// scipy.signal.convolve2d), on CUDA cores: complex64 tables of 16 x 16
// kernels by 32 x 32 FFTs (aw_fft.cu), other sizes and complex128 output by
// the direct sums below.
#include <cufft.h>

#include <algorithm>

#include "cg_internal.cuh"

namespace cg {

int fft_plan(int batch, int H, int W, cufftType type, cufftHandle *out);
bool aw_fft_supported(int SA, int S);
size_t aw_fft_workspace_bytes(int nk, int nW, int Q);
int aw_fft_launch(const float2 *akern, int nk, const void *W, int nW, int Q, int S,
                  const int32_t *wi, void *out, int out_c64, void *ws, size_t ws_bytes,
                  int32_t *d_status, cudaStream_t st);
int aw_fft_launch64(const double2 *akern, int nk, const void *W, int nW, int Q, int S,
                    const int32_t *wi, void *out, void *ws, size_t ws_bytes, int32_t *d_status,
                    cudaStream_t st);

struct FarField {
  int kind;  // 0: from ff array, 1: w-kernel phase
  const double2 *ff;
  int N0, ndim, Q, M;
  // w-kernel parameters
  double theta, dl, dm, T00, T01, T10, T11;
  int useT, invert;
  const double *w;  // device, per batch entry
};

// numpy's complex reciprocal 1 / (c + i d) (Smith's algorithm).
__device__ __forceinline__ double2 crecip(double c, double d) {
  if (fabs(c) >= fabs(d)) {
    const double rat = __ddiv_rn(d, c);
    const double scl = __ddiv_rn(1.0, __dadd_rn(c, __dmul_rn(d, rat)));
    return make_double2(scl, __dmul_rn(-rat, scl));
  }
  const double rat = __ddiv_rn(c, d);
  const double scl = __ddiv_rn(1.0, __dadd_rn(d, __dmul_rn(c, rat)));
  return make_double2(__dmul_rn(rat, scl), -scl);
}

// Far-field value at pixel (r, c) of an N0 x N0 pattern.
__device__ double2 far_value(const FarField &F, int b, int r, int c, int *bad) {
  if (F.kind == 0) {
    const size_t plane = F.ndim == 2 ? (size_t)F.N0 * F.N0 : (size_t)F.N0;
    return F.ff[(size_t)b * plane + (F.ndim == 2 ? (size_t)r * F.N0 + c : (size_t)c)];
  }
  const int N2 = F.N0 / 2;
  // kernel_coordinates (synthesis.py:250-270): l, m = coordinates2(N) * theta
  double l = __dmul_rn(__ddiv_rn((double)(c - N2), (double)F.N0), F.theta);
  double m = __dmul_rn(__ddiv_rn((double)(r - N2), (double)F.N0), F.theta);
  if (F.useT) {
    const double l2 = __dadd_rn(__dmul_rn(F.T00, l), __dmul_rn(F.T10, m));
    const double m2 = __dadd_rn(__dmul_rn(F.T01, l), __dmul_rn(F.T11, m));
    l = l2;
    m = m2;
  }
  l = __dadd_rn(l, F.dl);
  m = __dadd_rn(m, F.dm);
  const double r2 = __dadd_rn(__dmul_rn(l, l), __dmul_rn(m, m));
  if (!(r2 < 1.0)) *bad = 1;
  const double ph = __dadd_rn(1.0, -sqrt(__dadd_rn(1.0, -r2)));
  const double phase = __dmul_rn(__dmul_rn(2.0 * 3.141592653589793, F.w[b]), ph);
  double sn, cs;
  sincos(phase, &sn, &cs);
  return F.invert ? crecip(cs, sn) : make_double2(cs, sn);
}

// B[b, i, j] = pad_mid(ff)[(i + M/2) % M, (j + M/2) % M]
__global__ void k_ko_fill(FarField F, int batch, double2 *__restrict__ B, int32_t *status) {
  const int M = F.M;
  const int o = M / 2 - F.N0 / 2;
  const int64_t plane = F.ndim == 2 ? (int64_t)M * M : (int64_t)M;
  const int64_t total = plane * batch;
  int bad = 0;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total;
       L += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(L / plane);
    const int64_t q = L - (int64_t)b * plane;
    int i = 0, j;
    if (F.ndim == 2) {
      i = (int)(q / M);
      j = (int)(q - (int64_t)i * M);
    } else {
      j = (int)q;
    }
    const int r = (F.ndim == 2) ? (i + M / 2) % M - o : 0;
    const int c = (j + M / 2) % M - o;
    double2 v = make_double2(0.0, 0.0);
    if (c >= 0 && c < F.N0 && r >= 0 && r < F.N0) v = far_value(F, b, r, c, &bad);
    B[L] = v;
  }
  if (bad && status) atomicAdd(&status[ST_RANGE], 1);
}

// out[b, yf, xf, iy, ix] = fftshift(B)[my + Q*iy, mx + Q*ix]
template <typename C>
__global__ void k_ko_extract(const double2 *__restrict__ B, int batch, int ndim, int M,
                             int Q, int s, C *__restrict__ out) {
  const int64_t per = ndim == 2 ? (int64_t)Q * Q * s * s : (int64_t)Q * s;
  const int64_t total = per * batch;
  const int64_t plane = ndim == 2 ? (int64_t)M * M : (int64_t)M;
  const int base = M / 2 - Q * (s / 2);
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total;
       L += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(L / per);
    int64_t q = L - (int64_t)b * per;
    double2 v;
    if (ndim == 2) {
      const int ix = (int)(q % s);
      q /= s;
      const int iy = (int)(q % s);
      q /= s;
      const int xf = (int)(q % Q);
      const int yf = (int)(q / Q);
      const int ky = base + yf + Q * iy, kx = base + xf + Q * ix;
      const int sy = (ky - M / 2 + M) % M, sx = (kx - M / 2 + M) % M;
      v = B[(int64_t)b * plane + (int64_t)sy * M + sx];
    } else {
      const int ix = (int)(q % s);
      const int xf = (int)(q / s);
      const int kx = base + xf + Q * ix;
      v = B[(int64_t)b * plane + (kx - M / 2 + M) % M];
    }
    C o;
    o.x = v.x;
    o.y = v.y;
    out[L] = o;
  }
}

static unsigned blocks_for(int64_t count) {
  int64_t b = (count + 255) / 256;
  int64_t cap = (int64_t)num_sms() * 16;
  return (unsigned)std::max<int64_t>(1, std::min(b, cap));
}

static int oversample_run(FarField F, int batch, int s, void *out, bool out_c64,
                          void *ws, size_t ws_bytes, int32_t *status, cudaStream_t st) {
  const int M = F.M;
  const size_t per = (size_t)(F.ndim == 2 ? (int64_t)M * M : M) * sizeof(double2);
  CG_REQUIRE(s >= 1 && s <= F.N0, "kernel size %d must lie in [1, %d]", s, F.N0);
  if (!ws || ws_bytes < per)
    return set_error(CG_ERR_WORKSPACE, "kernel generation needs >= %zu workspace bytes", per);
  const int chunk = (int)std::min<size_t>((size_t)batch, ws_bytes / per);
  const int64_t out_per = F.ndim == 2 ? (int64_t)F.Q * F.Q * s * s : (int64_t)F.Q * s;
  const size_t esz = out_c64 ? sizeof(float2) : sizeof(double2);
  for (int b0 = 0; b0 < batch; b0 += chunk) {
    const int nb = std::min(chunk, batch - b0);
    FarField Fb = F;
    if (F.kind == 0) Fb.ff = F.ff + (size_t)b0 * (F.ndim == 2 ? (size_t)F.N0 * F.N0 : F.N0);
    else Fb.w = F.w + b0;
    const int64_t fill = (int64_t)nb * (per / sizeof(double2));
    k_ko_fill<<<blocks_for(fill), 256, 0, st>>>(Fb, nb, (double2 *)ws, status);
    CG_LAUNCH("kernel fill");
    if (M > 1) {  // a length-1 transform is the identity
      cufftHandle plan;
      int rc = fft_plan(nb, F.ndim == 2 ? M : 1, M, CUFFT_Z2Z, &plan);
      if (rc) return rc;
      if (cufftSetStream(plan, st) != CUFFT_SUCCESS ||
          cufftExecZ2Z(plan, (cufftDoubleComplex *)ws, (cufftDoubleComplex *)ws,
                       CUFFT_FORWARD) != CUFFT_SUCCESS)
        return set_error(CG_ERR_CUDA, "kernel FFT failed");
    }
    char *o = (char *)out + (size_t)b0 * out_per * esz;
    if (out_c64)
      k_ko_extract<float2><<<blocks_for(nb * out_per), 256, 0, st>>>(
          (const double2 *)ws, nb, F.ndim, M, F.Q, s, (float2 *)o);
    else
      k_ko_extract<double2><<<blocks_for(nb * out_per), 256, 0, st>>>(
          (const double2 *)ws, nb, F.ndim, M, F.Q, s, (double2 *)o);
    CG_LAUNCH("kernel extract");
  }
  return CG_OK;
}

// ---------------------------------------------------------------- AW kernels
// akern[k] = convolve2d(A[a1], A[a2], 'same'), FP64: one CTA per AW kernel.
// Then aw[k, f] = convolve2d(akern[k], W[wi, f], 'same') for the Q*Q
// sub-kernels f, FP32 products with FP32 accumulation, one CTA per (k, f).
// 'same' keeps the size of the first operand, centred on the full output:
//   same[i, j] = sum_{p, q} a[p, q] * b[i + o - p, j + o - q],  o = (nb - 1) / 2.
// R: the accumulation type, C: the stored type.  double / double2 for
// complex128 output (the reference's FP64 throughout); float / float2 for the
// complex64 tables, whose convolutions that follow run in FP32 anyway.
template <typename R, typename C>
__global__ void k_aw_akern(const double2 *__restrict__ A, int SA,
                           const int32_t *__restrict__ a1, const int32_t *__restrict__ a2,
                           int nA, C *__restrict__ akern, int32_t *status) {
  const int k = blockIdx.x;
  const int i1 = a1[k], i2 = a2[k];
  if (i1 < 0 || i1 >= nA || i2 < 0 || i2 >= nA) {
    if (threadIdx.x == 0) atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  // both A kernels staged in shared memory in the accumulation type
  extern __shared__ unsigned char aw_sh[];
  R *sp = (R *)aw_sh, *sr = sp + 2 * SA * SA;
  for (int t = threadIdx.x; t < SA * SA; t += blockDim.x) {
    const double2 u = A[(size_t)i1 * SA * SA + t], v = A[(size_t)i2 * SA * SA + t];
    sp[2 * t] = (R)u.x;
    sp[2 * t + 1] = (R)u.y;
    sr[2 * t] = (R)v.x;
    sr[2 * t + 1] = (R)v.y;
  }
  __syncthreads();
  const int o = (SA - 1) / 2;
  for (int t = threadIdx.x; t < SA * SA; t += blockDim.x) {
    const int i = t / SA, j = t - (t / SA) * SA;
    R ax = 0, ay = 0;
    for (int p = 0; p < SA; ++p) {
      const int y = i + o - p;
      if (y < 0 || y >= SA) continue;
      for (int q = 0; q < SA; ++q) {
        const int x = j + o - q;
        if (x < 0 || x >= SA) continue;
        const R ux = sp[2 * (p * SA + q)], uy = sp[2 * (p * SA + q) + 1];
        const R vx = sr[2 * (y * SA + x)], vy = sr[2 * (y * SA + x) + 1];
        ax += ux * vx - uy * vy;
        ay += ux * vy + uy * vx;
      }
    }
    C r;
    r.x = ax;
    r.y = ay;
    akern[(size_t)k * SA * SA + t] = r;
  }
}

template <typename C>
__global__ void k_aw_conv(const float2 *__restrict__ akern, int SA,
                          const float2 *__restrict__ Wk, int nW, int Q, int S,
                          const int32_t *__restrict__ wi, C *__restrict__ out,
                          int32_t *status) {
  extern __shared__ float2 sh[];
  float2 *sa = sh, *sw = sh + SA * SA;
  const int k = blockIdx.y, f = blockIdx.x;  // f = yf*Q + xf
  const int w = wi[k];
  if (w < 0 || w >= nW) {
    if (threadIdx.x == 0 && f == 0) atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  if ((status[ST_RANGE] | status[ST_INDEX]) != 0) return;
  const float2 *ak = akern + (size_t)k * SA * SA;
  const float2 *wk = Wk + ((size_t)w * Q * Q + f) * S * S;
  for (int t = threadIdx.x; t < SA * SA; t += blockDim.x) sa[t] = ak[t];
  for (int t = threadIdx.x; t < S * S; t += blockDim.x) sw[t] = wk[t];
  __syncthreads();
  const int o = (S - 1) / 2;
  C *dst = out + ((size_t)k * Q * Q + f) * SA * SA;
  for (int t = threadIdx.x; t < SA * SA; t += blockDim.x) {
    const int i = t / SA, j = t - (t / SA) * SA;
    float ax = 0.f, ay = 0.f;
    const int p_lo = max(0, i + o - (S - 1)), p_hi = min(SA - 1, i + o);
    const int q_lo = max(0, j + o - (S - 1)), q_hi = min(SA - 1, j + o);
    for (int p = p_lo; p <= p_hi; ++p) {
      const float2 *wrow = sw + (i + o - p) * S;
      for (int q = q_lo; q <= q_hi; ++q) {
        const float2 u = sa[p * SA + q], v = wrow[j + o - q];
        ax = fmaf(u.x, v.x, ax);
        ax = fmaf(-u.y, v.y, ax);
        ay = fmaf(u.x, v.y, ay);
        ay = fmaf(u.y, v.x, ay);
      }
    }
    C r;
    r.x = ax;
    r.y = ay;
    dst[t] = r;
  }
}

// The same convolution for SA x SA = SAC x SAC outputs with register blocking:
// a thread computes JB neighbouring outputs (i, j0 .. j0+JB-1) of one row, and
// for each A row p holds the SAC + JB - 1 w values that row needs in
// registers, so a loaded A tap feeds JB complex multiply-adds (the
// one-output-per-thread form is bound by shared-memory loads).
template <typename C, int SAC, int JB>
__global__ void __launch_bounds__(SAC *(SAC / JB)) k_aw_conv_blocked(
    const float2 *__restrict__ akern, const float2 *__restrict__ Wk, int nW, int Q, int S,
    const int32_t *__restrict__ wi, C *__restrict__ out, int32_t *status) {
  extern __shared__ float2 sh[];
  float2 *sa = sh, *sw = sh + SAC * SAC;
  const int k = blockIdx.y, f = blockIdx.x;  // f = yf*Q + xf
  const int w = wi[k];
  if (w < 0 || w >= nW) {
    if (threadIdx.x == 0 && f == 0) atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  if ((status[ST_RANGE] | status[ST_INDEX]) != 0) return;
  const float2 *ak = akern + (size_t)k * SAC * SAC;
  const float2 *wk = Wk + ((size_t)w * Q * Q + f) * S * S;
  for (int t = threadIdx.x; t < SAC * SAC; t += blockDim.x) sa[t] = ak[t];
  // w rows at an odd pitch (S + 1): a warp's lanes read 8 different rows, and a
  // 16-element row is 128 B, so an even pitch would put them all on one bank set
  const int SP = S + 1;
  for (int t = threadIdx.x; t < S * S; t += blockDim.x) {
    const int r = t / S, c = t - (t / S) * S;
    sw[r * SP + c] = wk[t];
  }
  __syncthreads();
  const int o = (S - 1) / 2;
  const int i = threadIdx.x / (SAC / JB), j0 = (threadIdx.x % (SAC / JB)) * JB;
  // (re, im) accumulators as pairs for the paired FP32 FMA: acc += (u.x, u.x) *
  // (v.x, v.y), then acc += (-u.y, u.y) * (v.y, v.x) -- per component the same
  // FMA sequence as the scalar form
  float2 acc[JB];
#pragma unroll
  for (int d = 0; d < JB; ++d) acc[d] = make_float2(0.f, 0.f);
  const int p_lo = max(0, i + o - (S - 1)), p_hi = min(SAC - 1, i + o);
  const int c0 = j0 + o - (SAC - 1);  // w column of register m = c0 + m
  for (int p = p_lo; p <= p_hi; ++p) {
    const float2 *wrow = sw + (i + o - p) * SP;
    float2 wv[SAC + JB - 1], ws[SAC + JB - 1];
#pragma unroll
    for (int m = 0; m < SAC + JB - 1; ++m) {
      const int c = c0 + m;
      wv[m] = (c >= 0 && c < S) ? wrow[c] : make_float2(0.f, 0.f);
      ws[m] = make_float2(wv[m].y, wv[m].x);
    }
    const float2 *arow = sa + p * SAC;
#pragma unroll
    for (int q = 0; q < SAC; ++q) {
      const float2 u = arow[q];
      const float2 ux = make_float2(u.x, u.x), uy = make_float2(-u.y, u.y);
#pragma unroll
      for (int d = 0; d < JB; ++d) {  // w column j0 + d + o - q is register d + SAC - 1 - q
        acc[d] = __ffma2_rn(ux, wv[d + SAC - 1 - q], acc[d]);
        acc[d] = __ffma2_rn(uy, ws[d + SAC - 1 - q], acc[d]);
      }
    }
  }
  C *dst = out + ((size_t)k * Q * Q + f) * SAC * SAC + i * SAC + j0;
#pragma unroll
  for (int d = 0; d < JB; ++d) {
    C r;
    r.x = acc[d].x;
    r.y = acc[d].y;
    dst[d] = r;
  }
}

// The complex128 AW kernels in FP64 throughout: A1 (*) A2 and the w
// sub-kernels as double2, products and sums in FP64 (the reference's
// scipy.signal.convolve2d of complex128 arrays).  A thread computes JB
// neighbouring outputs of one row; for each A row p it holds the S + JB - 1
// w values that row needs in registers (columns outside [0, S) read as
// zero), so one A tap feeds JB complex multiply-adds.  SA = SAC, S <= SAC.
template <int SAC, int JB>
__global__ void __launch_bounds__(SAC *(SAC / JB)) k_aw_conv64(
    const double2 *__restrict__ akern, const double2 *__restrict__ Wk, int nW, int Q, int S,
    const int32_t *__restrict__ wi, double2 *__restrict__ out, int32_t *status) {
  extern __shared__ double2 sh64[];
  double2 *sa = sh64, *sw = sh64 + SAC * SAC;
  const int k = blockIdx.y, f = blockIdx.x;  // f = yf*Q + xf
  const int w = wi[k];
  if (w < 0 || w >= nW) {
    if (threadIdx.x == 0 && f == 0) atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  if ((status[ST_RANGE] | status[ST_INDEX]) != 0) return;
  const double2 *ak = akern + (size_t)k * SAC * SAC;
  const double2 *wk = Wk + ((size_t)w * Q * Q + f) * S * S;
  for (int t = threadIdx.x; t < SAC * SAC; t += blockDim.x) sa[t] = ak[t];
  const int SP = S + 1;  // odd pitch against bank conflicts
  for (int t = threadIdx.x; t < S * S; t += blockDim.x) {
    const int r = t / S, c = t - (t / S) * S;
    sw[r * SP + c] = wk[t];
  }
  __syncthreads();
  const int o = (S - 1) / 2;
  const int i = threadIdx.x / (SAC / JB), j0 = (threadIdx.x % (SAC / JB)) * JB;
  double ax[JB], ay[JB];
#pragma unroll
  for (int d = 0; d < JB; ++d) ax[d] = ay[d] = 0.0;
  const int p_lo = max(0, i + o - (S - 1)), p_hi = min(SAC - 1, i + o);
  const int c0 = j0 + o - (SAC - 1);  // w column of register m = c0 + m
  for (int p = p_lo; p <= p_hi; ++p) {
    const double2 *wrow = sw + (i + o - p) * SP;
    double2 wv[SAC + JB - 1];
#pragma unroll
    for (int m = 0; m < SAC + JB - 1; ++m) {
      const int c = c0 + m;
      wv[m] = (c >= 0 && c < S) ? wrow[c] : make_double2(0.0, 0.0);
    }
    const double2 *arow = sa + p * SAC;
#pragma unroll
    for (int q = 0; q < SAC; ++q) {
      const double2 u = arow[q];
#pragma unroll
      for (int d = 0; d < JB; ++d) {  // w column j0 + d + o - q is register d + SAC - 1 - q
        const double2 v = wv[d + SAC - 1 - q];
        ax[d] = fma(u.x, v.x, ax[d]);
        ax[d] = fma(-u.y, v.y, ax[d]);
        ay[d] = fma(u.x, v.y, ay[d]);
        ay[d] = fma(u.y, v.x, ay[d]);
      }
    }
  }
  double2 *dst = out + ((size_t)k * Q * Q + f) * SAC * SAC + i * SAC + j0;
#pragma unroll
  for (int d = 0; d < JB; ++d) dst[d] = make_double2(ax[d], ay[d]);
}

// Any SA: one output per thread, FP64 sums over the 'same' support.
__global__ void k_aw_conv64_any(const double2 *__restrict__ akern, int SA,
                                const double2 *__restrict__ Wk, int nW, int Q, int S,
                                const int32_t *__restrict__ wi, double2 *__restrict__ out,
                                int32_t *status) {
  extern __shared__ double2 sh64[];
  double2 *sa = sh64, *sw = sh64 + SA * SA;
  const int k = blockIdx.y, f = blockIdx.x;
  const int w = wi[k];
  if (w < 0 || w >= nW) {
    if (threadIdx.x == 0 && f == 0) atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  if ((status[ST_RANGE] | status[ST_INDEX]) != 0) return;
  const double2 *ak = akern + (size_t)k * SA * SA;
  const double2 *wk = Wk + ((size_t)w * Q * Q + f) * S * S;
  for (int t = threadIdx.x; t < SA * SA; t += blockDim.x) sa[t] = ak[t];
  for (int t = threadIdx.x; t < S * S; t += blockDim.x) sw[t] = wk[t];
  __syncthreads();
  const int o = (S - 1) / 2;
  double2 *dst = out + ((size_t)k * Q * Q + f) * SA * SA;
  for (int t = threadIdx.x; t < SA * SA; t += blockDim.x) {
    const int i = t / SA, j = t - (t / SA) * SA;
    double ax = 0.0, ay = 0.0;
    const int p_lo = max(0, i + o - (S - 1)), p_hi = min(SA - 1, i + o);
    const int q_lo = max(0, j + o - (S - 1)), q_hi = min(SA - 1, j + o);
    for (int p = p_lo; p <= p_hi; ++p) {
      const double2 *wrow = sw + (i + o - p) * S;
      for (int q = q_lo; q <= q_hi; ++q) {
        const double2 u = sa[p * SA + q], v = wrow[j + o - q];
        ax = fma(u.x, v.x, ax);
        ax = fma(-u.y, v.y, ax);
        ay = fma(u.x, v.y, ay);
        ay = fma(u.y, v.x, ay);
      }
    }
    dst[t] = make_double2(ax, ay);
  }
}

}  // namespace cg

using namespace cg;

extern "C" {

size_t cg_kernel_oversample_workspace_bytes(int batch, int ndim, int N0, int Q) {
  const int64_t M = (int64_t)N0 * Q;
  return (size_t)batch * (size_t)(ndim == 2 ? M * M : M) * sizeof(double2);
}

int cg_kernel_oversample(const void *ff, int batch, int ndim, int N0, int Q, int s,
                         void *out, int out_c64, void *ws, size_t ws_bytes,
                         cg_stream_t stream) {
  CG_REQUIRE(ff && out && batch >= 1 && (ndim == 1 || ndim == 2) && N0 >= 1 && Q >= 1,
             "bad kernel_oversample arguments");
  FarField F = {};
  F.kind = 0;
  F.ff = (const double2 *)ff;
  F.N0 = N0;
  F.ndim = ndim;
  F.Q = Q;
  F.M = N0 * Q;
  return oversample_run(F, batch, s, out, out_c64 != 0, ws, ws_bytes, nullptr,
                        (cudaStream_t)stream);
}

size_t cg_w_kernels_workspace_bytes(int nw, int NpixFF, int Q) {
  const int64_t M = (int64_t)NpixFF * Q;
  return (size_t)nw * (size_t)(M * M) * sizeof(double2) + 256 + (size_t)nw * 8;
}

int cg_w_kernels(double theta, const double *w_host, int nw, int NpixFF, int S, int Q,
                 int invert, double dl, double dm, const double *T, void *out, int out_c64,
                 void *ws, size_t ws_bytes, int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(w_host && out && nw >= 1 && NpixFF >= 1 && S >= 1 && Q >= 1 && d_status,
             "bad w_kernels arguments");
  // w_kernel's precondition (synthesis.py:371)
  CG_REQUIRE(NpixFF > S || (NpixFF == S && Q == 1),
             "AssertionError: NpixFF %d must exceed NpixKern %d (or equal it with Qpx 1)",
             NpixFF, S);
  cudaStream_t st = (cudaStream_t)stream;
  // the w values go to the head of the workspace
  const size_t wbytes = ((size_t)nw * 8 + 255) & ~size_t(255);
  CG_REQUIRE(ws && ws_bytes > wbytes, "w_kernels workspace too small");
  double *d_w = (double *)ws;
  CG_CUDA(cudaMemcpyAsync(d_w, w_host, (size_t)nw * 8, cudaMemcpyHostToDevice, st));
  FarField F = {};
  F.kind = 1;
  F.N0 = NpixFF;
  F.ndim = 2;
  F.Q = Q;
  F.M = NpixFF * Q;
  F.theta = theta;
  F.dl = dl;
  F.dm = dm;
  F.useT = T != nullptr;
  if (T) {
    F.T00 = T[0];
    F.T01 = T[1];
    F.T10 = T[2];
    F.T11 = T[3];
  }
  F.invert = invert;
  F.w = d_w;
  return oversample_run(F, nw, S, out, out_c64 != 0, (char *)ws + wbytes, ws_bytes - wbytes,
                        d_status, st);
}

__global__ void k_c128_to_c64(const double2 *__restrict__ in, int64_t n, float2 *__restrict__ out) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    out[t] = make_float2((float)in[t].x, (float)in[t].y);
}

// Workspace: the A1 (*) A2 kernels [nk, SA, SA] (FP32 for complex64 tables,
// FP64 for complex128 ones; room for FP64), then for complex64 tables the w
// sub-kernels converted once to FP32 [nW, Q, Q, S, S] (the convolution blocks
// read both many times; converting per block would load the narrow FP64 pipe)
// or the FFT form's spectra.
static size_t aw_ws_akern_bytes(int nk, int SA) {
  return ((size_t)std::max(nk, 1) * SA * SA * sizeof(double2) + 255) & ~(size_t)255;
}

size_t cg_aw_kernels_workspace_bytes(int nk, int SA, int nW, int Q, int S) {
  size_t rest = (size_t)std::max(nW, 1) * Q * Q * S * S * sizeof(float2);
  if (aw_fft_supported(SA, S)) rest = std::max(rest, aw_fft_workspace_bytes(nk, nW, Q));
  return aw_ws_akern_bytes(nk, SA) + rest;
}

int cg_aw_kernels(const void *A, int nA, int SA, const void *Wk, int nW, int Q, int S,
                  const int32_t *a1, const int32_t *a2, const int32_t *wi, int nk, void *out,
                  int out_c64, void *ws, size_t ws_bytes, int32_t *d_status,
                  cg_stream_t stream) {
  CG_REQUIRE(A && Wk && a1 && a2 && wi && out && d_status && nA >= 1 && nW >= 1 && SA >= 1 &&
                 S >= 1 && Q >= 1 && nk >= 0,
             "bad aw_kernels arguments");
  CG_REQUIRE(SA <= 64 && S <= 64, "AW kernel sizes above 64 are not supported");
  if (nk == 0) return CG_OK;
  const size_t need = cg_aw_kernels_workspace_bytes(nk, SA, nW, Q, S);
  if (!ws || ws_bytes < need)
    return set_error(CG_ERR_WORKSPACE, "aw_kernels needs %zu workspace bytes", need);
  cudaStream_t st = (cudaStream_t)stream;
  if (!out_c64) {  // complex128 tables: FP64 throughout
    double2 *akern64 = (double2 *)ws;
    const size_t sh_a = 4 * (size_t)SA * SA * sizeof(double);
    if (sh_a > 48 * 1024)
      CG_CUDA(cudaFuncSetAttribute(k_aw_akern<double, double2>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh_a));
    k_aw_akern<double, double2><<<nk, 256, sh_a, st>>>((const double2 *)A, SA, a1, a2, nA,
                                                       akern64, d_status);
    CG_LAUNCH("aw akern (FP64)");
    if (aw_fft_supported(SA, S))  // the 32 x 32 FFT form in FP64
      return aw_fft_launch64(akern64, nk, Wk, nW, Q, S, wi, out,
                             (char *)ws + aw_ws_akern_bytes(nk, SA),
                             ws_bytes - aw_ws_akern_bytes(nk, SA), d_status, st);
    dim3 grid(Q * Q, nk);
    if (SA == 16 && S <= 16) {
      const size_t smem = (size_t)(SA * SA + S * (S + 1)) * sizeof(double2);
      k_aw_conv64<16, 4><<<grid, 64, smem, st>>>(akern64, (const double2 *)Wk, nW, Q, S, wi,
                                                 (double2 *)out, d_status);
    } else {
      const size_t smem = (size_t)(SA * SA + S * S) * sizeof(double2);
      if (smem > 48 * 1024)
        CG_CUDA(cudaFuncSetAttribute(k_aw_conv64_any, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
      k_aw_conv64_any<<<grid, 256, smem, st>>>(akern64, SA, (const double2 *)Wk, nW, Q, S, wi,
                                               (double2 *)out, d_status);
    }
    CG_LAUNCH("aw conv (FP64)");
    return CG_OK;
  }
  float2 *akern = (float2 *)ws;
  float2 *wk32 = (float2 *)((char *)ws + aw_ws_akern_bytes(nk, SA));
  const bool fft_form = aw_fft_supported(SA, S);
  // shared staging of the two A kernels in FP32: up to 64 KB at SA = 64
  const size_t sh_a = 4 * (size_t)SA * SA * sizeof(float);
  if (sh_a > 48 * 1024)
    CG_CUDA(cudaFuncSetAttribute(k_aw_akern<float, float2>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh_a));
  k_aw_akern<float, float2><<<nk, 256, sh_a, st>>>((const double2 *)A, SA, a1, a2, nA, akern,
                                                   d_status);
  CG_LAUNCH("aw akern");
  if (fft_form)  // complex64 tables: the FFT form
    return aw_fft_launch(akern, nk, Wk, nW, Q, S, wi, out, 1,
                         (char *)ws + aw_ws_akern_bytes(nk, SA),
                         ws_bytes - aw_ws_akern_bytes(nk, SA), d_status, st);
  const int64_t nwk = (int64_t)nW * Q * Q * S * S;
  k_c128_to_c64<<<(unsigned)std::min<int64_t>((nwk + 255) / 256, (int64_t)num_sms() * 16), 256, 0,
                  st>>>((const double2 *)Wk, nwk, wk32);
  CG_LAUNCH("aw w kernels to FP32");
  const size_t smem = (size_t)(SA * SA + S * S) * sizeof(float2);
  dim3 grid(Q * Q, nk);
  if (SA == 16) {  // the AW kernels' size: register-blocked form, 4 outputs per thread
    const size_t smem_b = (size_t)(SA * SA + S * (S + 1)) * sizeof(float2);
    k_aw_conv_blocked<float2, 16, 4><<<grid, 64, smem_b, st>>>(akern, wk32, nW, Q, S, wi,
                                                               (float2 *)out, d_status);
    CG_LAUNCH("aw conv");
    return CG_OK;
  }
  k_aw_conv<float2><<<grid, 256, smem, st>>>(akern, SA, wk32, nW, Q, S, wi, (float2 *)out,
                                             d_status);
  CG_LAUNCH("aw conv");
  return CG_OK;
}

}  // extern "C"
