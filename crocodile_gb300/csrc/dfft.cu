// Batched complex FFTs computed in double-float arithmetic.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, and a batched FP64
// FFT is bound by that rate, not by memory.  Here each complex value is
// carried as two unevaluated float sums (hi + lo, about 48 significant bits)
// and every butterfly uses error-free transformations on the FP32 units
// (df.cuh; sloppy pair sums in the butterflies, normwise error about 2u^2
// per stage, u = 2^-24).  Transforms are power-of-two lengths 64 .. 2048 in
// shared memory by the Stockham (self-sorting) algorithm in radix 4, with one
// radix-2 stage first when log2 n is odd: the stage with stride s reads
// x[q + s (p + k m)] (m = n/(4s), k < 4, t = p s + q) and writes
// y[q + s (4p + k)] = (the 4-point DFT of those four)_k w^(k p s), so the
// output is in natural order; half the shared-memory passes and a quarter
// fewer twiddle products than radix 2.  Twiddles w^k = exp(-+2 pi i k / n),
// k < 3n/4, come from an FP64 host table split into hi + lo.
// Unnormalised, as cuFFT.
//
// Elements reach the kernels through an I/O policy, so one transform serves
//   - complex128 rows in place (converted on load and store),
//   - double-float rows (float4 = re.hi, re.lo, im.hi, im.lo) in place,
//   - the two passes of a centred 2-D transform of complex128 planes: rows
//     with the (-1)^(i+j) pre-modulation, complex128 in and double-float out;
//     then columns, double-float in and complex128 out with the post-
//     modulation and the 1 / (H W) of an inverse.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "cg_internal.cuh"
#include "df.cuh"
#include "dfft.cuh"

namespace cg {

namespace {

using dfk::AtCol;
using dfk::radix2_first;
using dfk::radix4;

// ---------------------------------------------------------------- I/O policies
// ld(row, i) / st(row, i, v): element i of transform row `row`

struct IoC128 {
  double2 *d;
  int n;
  __device__ cdf ld(int64_t row, int i) const { return cdf_from(d[row * n + i]); }
  __device__ void st(int64_t row, int i, const cdf &v) const { d[row * n + i] = cdf_to(v); }
};

struct IoDF {
  float4 *d;
  int n;
  __device__ cdf ld(int64_t row, int i) const { return cdf_load(d[row * n + i]); }
  __device__ void st(int64_t row, int i, const cdf &v) const { d[row * n + i] = cdf_store(v); }
};

__device__ __forceinline__ cdf cdf_neg(const cdf &v) { return {df_neg(v.re), df_neg(v.im)}; }

// centred 2-D, pass over rows: complex128 plane rows in, the sign (-1)^(i+j)
// of the pre-modulation (i = row within its plane of H rows), double-float out
// in place (same 16 bytes per element)
struct IoRowsCentred {
  double2 *d;
  int n, H;
  __device__ cdf ld(int64_t row, int i) const {
    const cdf v = cdf_from(d[row * n + i]);
    return (((int)(row % H) + i) & 1) ? cdf_neg(v) : v;
  }
  __device__ void st(int64_t row, int i, const cdf &v) const {
    ((float4 *)d)[row * n + i] = cdf_store(v);
  }
};

// ---------------------------------------------------------------- column transforms
// Planes [nplanes][N][W] of double-float, transformed along N (the columns);
// each CTA takes C adjacent columns of one plane (C * 16 bytes per row read),
// T threads; then the centred post-modulation (-1)^(l + k + phase) * scale and
// complex128 out in place.
template <int LOGN, int C, int T>
__global__ void __launch_bounds__(T)
    k_dfft_cols_centred(double2 *d, int64_t nplanes, int W, int phase, float scale,
                        const float4 *__restrict__ tw, int inverse) {
  constexpr int N = 1 << LOGN;
  constexpr int Q = N / 4;
  extern __shared__ float dsm[];
  cdf *buf0 = (cdf *)dsm;    // [N][C]
  cdf *buf1 = buf0 + N * C;  // [N][C]
  cdf *stw = buf1 + N * C;   // [3N/4]
  for (int k = threadIdx.x; k < 3 * Q; k += T) stw[k] = cdf_load(tw[k]);
  const bool inv = inverse != 0;
  const int groups = W / C;
  const int64_t jobs = nplanes * groups;
  for (int64_t job = blockIdx.x; job < jobs; job += gridDim.x) {
    const int64_t plane = job / groups;
    const int c0 = (int)(job - plane * groups) * C;
    const float4 *src = (const float4 *)(d + plane * N * W) + c0;
    for (int e = threadIdx.x; e < N * C; e += T) {
      const int i = e / C, c = e - (e / C) * C;
      buf0[e] = cdf_load(src[(int64_t)i * W + c]);
    }
    __syncthreads();
    cdf *x = buf0, *y = buf1;
    if (LOGN & 1) {
      for (int b = threadIdx.x; b < N / 2 * C; b += T)
        radix2_first<N>(x, y, stw, b / C, AtCol<C>{b % C});
      __syncthreads();
      cdf *tmp = x;
      x = y;
      y = tmp;
    }
#pragma unroll
    for (int ls = (LOGN & 1); ls < LOGN; ls += 2) {
      for (int b = threadIdx.x; b < Q * C; b += T)
        radix4<N>(x, y, stw, b / C, 1 << ls, inv, AtCol<C>{b % C});
      __syncthreads();
      cdf *tmp = x;
      x = y;
      y = tmp;
    }
    double2 *dst = d + plane * N * W + c0;
    for (int e = threadIdx.x; e < N * C; e += T) {
      const int l = e / C, c = e - (e / C) * C;
      const float sg = ((l + c0 + c + phase) & 1) ? -scale : scale;  // a power of two
      const cdf v = x[e];
      const cdf w = {{v.re.hi * sg, v.re.lo * sg}, {v.im.hi * sg, v.im.lo * sg}};
      dst[(int64_t)l * W + c] = cdf_to(w);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- long rows
// n = N1 * 2048 (N1 = 2, 4) in three passes, the four-step factorisation
//   X[k1 + N1 k2] = sum_n2 w_n^(n2 k1) [sum_n1 x[n2 + 2048 n1] w_N1^(n1 k1)] w_2048^(n2 k2):
// k_dfft_long_pre forms the bracket times w_n^(n2 k1) in place (row position
// k1 * 2048 + n2), the 2048-point kernel transforms the N1 sub-rows, and
// k_dfft_long_T puts X back in natural order through shared memory.
constexpr int DF_LONG_N2 = 2048;

template <int N1>
__global__ void k_dfft_long_pre(float4 *d, int64_t batch, const float4 *__restrict__ tw,
                                int inverse) {
  constexpr int N2 = DF_LONG_N2, N = N1 * N2;
  const int64_t total = batch * N2;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / N2;
    const int n2 = (int)(e - b * N2);
    float4 *row = d + b * N;
    cdf x[N1], y[N1];
#pragma unroll
    for (int j = 0; j < N1; ++j) x[j] = cdf_load(row[n2 + N2 * j]);
    if (N1 == 2) {
      y[0] = cdf_add_f(x[0], x[1]);
      y[1] = cdf_sub_f(x[0], x[1]);
    } else {
      const cdf a0 = cdf_add_f(x[0], x[N1 > 2 ? 2 : 0]), a1 = cdf_sub_f(x[0], x[N1 > 2 ? 2 : 0]);
      const cdf b0 = cdf_add_f(x[1], x[N1 > 3 ? 3 : 1]);
      const cdf b1 = dfk::cdf_mul_j(cdf_sub_f(x[1], x[N1 > 3 ? 3 : 1]), inverse != 0);
      y[0] = cdf_add_f(a0, b0);
      y[1] = cdf_add_f(a1, b1);
      y[N1 > 2 ? 2 : 0] = cdf_sub_f(a0, b0);
      y[N1 > 3 ? 3 : 1] = cdf_sub_f(a1, b1);
    }
    row[n2] = cdf_store(y[0]);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1)
      row[k1 * N2 + n2] = cdf_store(n2 == 0 ? y[k1] : cdf_mul_f(y[k1], cdf_load(tw[n2 * k1])));
  }
}

// X[k1 + N1 k2] = Z[k1][k2] for each row, in place; one CTA per row, the sub-
// rows padded by one element in shared memory
template <int N1>
__global__ void __launch_bounds__(1024) k_dfft_long_T(float4 *d, int64_t batch) {
  constexpr int N2 = DF_LONG_N2, N = N1 * N2, P = N2 + 1;
  extern __shared__ float dsm[];
  float4 *buf = (float4 *)dsm;  // [N1][P]
  for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
    float4 *row = d + b * N;
    for (int e = threadIdx.x; e < N; e += blockDim.x) buf[(e / N2) * P + (e % N2)] = row[e];
    __syncthreads();
    for (int k = threadIdx.x; k < N; k += blockDim.x) row[k] = buf[(k % N1) * P + k / N1];
    __syncthreads();
  }
}

// complex128 <-> double-float in place (the same 16 bytes per element)
__global__ void k_c128_to_df(double2 *d, int64_t count) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x)
    ((float4 *)d)[e] = cdf_store(cdf_from(d[e]));
}
__global__ void k_df_to_c128(double2 *d, int64_t count) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x)
    d[e] = cdf_to(cdf_load(((float4 *)d)[e]));
}

// ---------------------------------------------------------------- twiddles
}  // namespace

std::mutex g_tw_mu;
std::map<std::pair<int, int>, float4 *> g_tw;  // (device, n * sign) -> table

int dfft_twiddles(int n, int sign, const float4 **out) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(g_tw_mu);
  auto key = std::make_pair(dev, n * sign);
  auto it = g_tw.find(key);
  if (it != g_tw.end()) {
    *out = it->second;
    return CG_OK;
  }
  std::vector<float4> h(3 * n / 4);
  for (int k = 0; k < 3 * n / 4; ++k) {
    const double a = 2.0 * M_PI * (double)k / (double)n;
    const double c = std::cos(a), s = sign * std::sin(a);
    const float ch = (float)c, sh = (float)s;
    h[k] = make_float4(ch, (float)(c - (double)ch), sh, (float)(s - (double)sh));
  }
  float4 *d = nullptr;
  CG_CUDA(cudaMalloc(&d, h.size() * sizeof(float4)));
  CG_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice));
  g_tw[key] = d;
  *out = d;
  return CG_OK;
}

namespace {

template <int LOGN, int C>
int launch_cols(double2 *d, int64_t nplanes, int W, int phase, float scale, const float4 *tw,
                int inverse, cudaStream_t st) {
  constexpr int N = 1 << LOGN;
  constexpr int T = 256;
  const size_t smem = (size_t)(2 * N * C + 3 * N / 4) * sizeof(cdf);
  if (smem > 48 * 1024)
    CG_CUDA(cudaFuncSetAttribute(k_dfft_cols_centred<LOGN, C, T>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t jobs = nplanes * (W / C);
  const unsigned grid = (unsigned)std::min<int64_t>(jobs, (int64_t)num_sms() * 8);
  k_dfft_cols_centred<LOGN, C, T><<<grid, T, smem, st>>>(d, nplanes, W, phase, scale, tw,
                                                         inverse);
  CG_LAUNCH("double-float column FFT");
  return CG_OK;
}

}  // namespace

bool dfft_supported(int n) { return n >= 64 && n <= 2048 && (n & (n - 1)) == 0; }

// In-place batched FFT of `batch` contiguous complex128 rows of length n
// (a power of two, 64..2048); inverse: exp(+2 pi i), unnormalised.
int dfft_rows(double2 *data, int64_t batch, int n, int inverse, cudaStream_t st) {
  return dfft_rows_io(IoC128{data, n}, batch, n, inverse, st);
}

bool dfft_long_supported(int n) { return dfft_supported(n) || n == 4096 || n == 8192; }

namespace {
template <int N1>
int dfft_long(float4 *data, int64_t batch, int inverse, cudaStream_t st) {
  const int n = N1 * DF_LONG_N2;
  const float4 *tw;
  int rc = dfft_twiddles(n, inverse ? 1 : -1, &tw);
  if (rc) return rc;
  const int64_t total = batch * DF_LONG_N2;
  const unsigned g = (unsigned)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
  k_dfft_long_pre<N1><<<g, 256, 0, st>>>(data, batch, tw, inverse);
  CG_LAUNCH("double-float long FFT (first pass)");
  if ((rc = dfft_rows_io(IoDF{data, DF_LONG_N2}, batch * N1, DF_LONG_N2, inverse, st)))
    return rc;
  const size_t smem = (size_t)N1 * (DF_LONG_N2 + 1) * sizeof(float4);
  CG_CUDA(cudaFuncSetAttribute(k_dfft_long_T<N1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  const unsigned gt = (unsigned)std::min<int64_t>(batch, (int64_t)num_sms() * 4);
  k_dfft_long_T<N1><<<gt, 1024, smem, st>>>(data, batch);
  CG_LAUNCH("double-float long FFT (transpose)");
  return CG_OK;
}
}  // namespace

// The same on rows stored as double-float (float4 per element); lengths up to
// 8192 (4096 and 8192 by the four-step passes).
int dfft_rows_df(float4 *data, int64_t batch, int n, int inverse, cudaStream_t st) {
  if (batch <= 0) return CG_OK;
  if (n == 4096) return dfft_long<2>(data, batch, inverse, st);
  if (n == 8192) return dfft_long<4>(data, batch, inverse, st);
  return dfft_rows_io(IoDF{data, n}, batch, n, inverse, st);
}

// In-place centred 2-D FFT of `batch` complex128 planes [H][W] (numpy's
// fftshift(fft2(ifftshift(x))), or the normalised ifft2 for inverse), H and W
// powers of two 64..2048.  The fftshifts are the checkerboard modulations
// (-1)^(i+j) before and (-1)^(k+l+H/2+W/2) after the transform.
int dfft2_centred(double2 *data, int64_t batch, int H, int W, int inverse, cudaStream_t st) {
  CG_REQUIRE(dfft_supported(H) && dfft_supported(W),
             "double-float 2-D FFT sides are powers of two 64..2048");
  if (batch <= 0) return CG_OK;
  int rc = dfft_rows_io(IoRowsCentred{data, W, H}, batch * H, W, inverse, st);
  if (rc) return rc;
  const float4 *tw;
  if ((rc = dfft_twiddles(H, inverse ? 1 : -1, &tw))) return rc;
  const int phase = (H / 2 + W / 2) & 1;
  const float scale = inverse ? 1.0f / ((float)H * (float)W) : 1.0f;  // a power of two
  switch (H) {  // columns per CTA: measured best for 512 at 2 (38 KB, 5 CTAs per SM)
    case 64: return launch_cols<6, 16>(data, batch, W, phase, scale, tw, inverse, st);
    case 128: return launch_cols<7, 16>(data, batch, W, phase, scale, tw, inverse, st);
    case 256: return launch_cols<8, 8>(data, batch, W, phase, scale, tw, inverse, st);
    case 512: return launch_cols<9, 2>(data, batch, W, phase, scale, tw, inverse, st);
    case 1024: return launch_cols<10, 4>(data, batch, W, phase, scale, tw, inverse, st);
    case 2048: return launch_cols<11, 2>(data, batch, W, phase, scale, tw, inverse, st);
  }
  return set_error(CG_ERR_ARG, "unsupported double-float FFT length %d", H);
}

}  // namespace cg

extern "C" int cg_fft_rows_df(void *data_c128, int64_t batch, int n, int inverse,
                              cg_stream_t stream) {
  CG_REQUIRE(data_c128 && batch >= 0, "bad double-float FFT arguments");
  if (n == 4096 || n == 8192) {  // converted in place around the double-float passes
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t count = batch * n;
    if (count == 0) return CG_OK;
    const unsigned g =
        (unsigned)std::min<int64_t>((count + 255) / 256, (int64_t)cg::num_sms() * 16);
    cg::k_c128_to_df<<<g, 256, 0, st>>>((double2 *)data_c128, count);
    CG_LAUNCH("complex128 to double-float");
    const int rc = cg::dfft_rows_df((float4 *)data_c128, batch, n, inverse, st);
    if (rc) return rc;
    cg::k_df_to_c128<<<g, 256, 0, st>>>((double2 *)data_c128, count);
    CG_LAUNCH("double-float to complex128");
    return CG_OK;
  }
  return cg::dfft_rows((double2 *)data_c128, batch, n, inverse, (cudaStream_t)stream);
}

extern "C" int cg_fft2_centred_df(void *data_c128, int64_t batch, int H, int W, int inverse,
                                  cg_stream_t stream) {
  CG_REQUIRE(data_c128 && batch >= 0, "bad double-float 2-D FFT arguments");
  return cg::dfft2_centred((double2 *)data_c128, batch, H, W, inverse, (cudaStream_t)stream);
}
