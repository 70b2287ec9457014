// Batched complex FFTs of FP64 rows computed in double-float arithmetic.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, and a batched FP64
// FFT is bound by that rate, not by memory.  Here each complex128 element is
// carried as two unevaluated float sums (hi + lo, about 48 significant bits)
// and every butterfly uses error-free transformations on the FP32 units:
//   two_sum (Knuth), two_prod by FMA, the double-float sum with both
//   components' errors (the accurate pair sum of Joldes, Muller and Popescu,
//   "Tight and rigorous error bounds for basic building blocks of
//   double-word arithmetic", 2017) and the double-float product with FMA.
// Rows are power-of-two lengths 64 .. 2048, contiguous in memory, one or more
// rows per CTA, transformed in shared memory by the radix-2 Stockham
// (self-sorting) algorithm: stage s reads x[q + s p], x[q + s (p + m)] and
// writes y[q + s 2p] = a + b, y[q + s (2p + 1)] = (a - b) w^(p s), m = n/(2s),
// so the output is in natural order.  Twiddles w^k = exp(-+2 pi i k / n) come
// from an FP64 host table split into hi + lo.  Unnormalised, as cuFFT.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "cg_internal.cuh"

namespace cg {

namespace {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  const df t = two_sum(x.lo, y.lo);
  df v = fast_two_sum(s.hi, s.lo + t.hi);
  return fast_two_sum(v.hi, t.lo + v.lo);
}

__device__ __forceinline__ df df_neg(df x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ df df_mul(df x, df y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return fast_two_sum(p, e);
}

struct cdf {
  df re, im;
};

__device__ __forceinline__ cdf cdf_add(const cdf &a, const cdf &b) {
  return {df_add(a.re, b.re), df_add(a.im, b.im)};
}
__device__ __forceinline__ cdf cdf_sub(const cdf &a, const cdf &b) {
  return {df_add(a.re, df_neg(b.re)), df_add(a.im, df_neg(b.im))};
}
__device__ __forceinline__ cdf cdf_mul(const cdf &a, const cdf &w) {
  return {df_add(df_mul(a.re, w.re), df_neg(df_mul(a.im, w.im))),
          df_add(df_mul(a.re, w.im), df_mul(a.im, w.re))};
}

__device__ __forceinline__ df split(double v) {
  const float hi = (float)v;
  return {hi, (float)(v - (double)hi)};
}

__device__ __forceinline__ cdf to_cdf(double2 v) { return {split(v.x), split(v.y)}; }

__device__ __forceinline__ double2 from_cdf(const cdf &v) {
  return make_double2((double)v.re.hi + (double)v.re.lo, (double)v.im.hi + (double)v.im.lo);
}

// ROWS rows of length N per CTA, N/2 threads per row; two cdf buffers
template <int LOGN, int ROWS>
__global__ void __launch_bounds__((1 << LOGN) / 2 * ROWS)
    k_dfft_rows(double2 *__restrict__ data, int64_t batch, const double2 *__restrict__ tw) {
  constexpr int N = 1 << LOGN;
  constexpr int H = N / 2;
  extern __shared__ float dsm[];
  cdf *buf0 = (cdf *)dsm;                 // [ROWS][N]
  cdf *buf1 = buf0 + ROWS * N;            // [ROWS][N]
  cdf *stw = buf1 + ROWS * N;             // [N/2] twiddles, as double-float
  const int r = threadIdx.x / H, t = threadIdx.x - (threadIdx.x / H) * H;
  for (int k = threadIdx.x; k < H; k += blockDim.x) stw[k] = to_cdf(tw[k]);
  for (int64_t row0 = (int64_t)blockIdx.x * ROWS; row0 < batch;
       row0 += (int64_t)gridDim.x * ROWS) {
    const int64_t row = row0 + r;
    const bool live = row < batch;
    double2 *src = data + row * N;
    cdf *x = buf0 + r * N, *y = buf1 + r * N;
    if (live) {
      x[t] = to_cdf(src[t]);
      x[t + H] = to_cdf(src[t + H]);
    }
    __syncthreads();
#pragma unroll
    for (int ls = 0; ls < LOGN; ++ls) {
      const int s = 1 << ls;                  // stride
      const int p = t >> ls, q = t & (s - 1);  // t = p s + q, p < m = N / (2s)
      if (live) {
        const cdf a = x[q + s * p], b = x[q + s * p + H];
        y[q + s * 2 * p] = cdf_add(a, b);
        const cdf d = cdf_sub(a, b);
        y[q + s * (2 * p + 1)] = (p == 0) ? d : cdf_mul(d, stw[p * s]);
      }
      __syncthreads();
      cdf *tmp = x;
      x = y;
      y = tmp;
    }
    if (live) {
      src[t] = from_cdf(x[t]);
      src[t + H] = from_cdf(x[t + H]);
    }
    __syncthreads();
  }
}

std::mutex g_tw_mu;
std::map<std::pair<int, int>, double2 *> g_tw;  // (device, n * sign) -> table

int twiddles(int n, int sign, const double2 **out) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(g_tw_mu);
  auto key = std::make_pair(dev, n * sign);
  auto it = g_tw.find(key);
  if (it != g_tw.end()) {
    *out = it->second;
    return CG_OK;
  }
  std::vector<double2> h(n / 2);
  for (int k = 0; k < n / 2; ++k) {
    const double a = 2.0 * M_PI * (double)k / (double)n;
    h[k] = make_double2(std::cos(a), sign * std::sin(a));
  }
  double2 *d = nullptr;
  CG_CUDA(cudaMalloc(&d, h.size() * sizeof(double2)));
  CG_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice));
  g_tw[key] = d;
  *out = d;
  return CG_OK;
}

template <int LOGN, int ROWS>
int launch(double2 *data, int64_t batch, const double2 *tw, cudaStream_t st) {
  constexpr int N = 1 << LOGN;
  const size_t smem = (size_t)(2 * ROWS * N + N / 2) * sizeof(cdf);
  if (smem > 48 * 1024)  // set on every launch: the attribute is per device
    CG_CUDA(cudaFuncSetAttribute(k_dfft_rows<LOGN, ROWS>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t ctas = (batch + ROWS - 1) / ROWS;
  const unsigned grid = (unsigned)std::min<int64_t>(ctas, (int64_t)num_sms() * 8);
  k_dfft_rows<LOGN, ROWS><<<grid, N / 2 * ROWS, smem, st>>>(data, batch, tw);
  CG_LAUNCH("double-float FFT");
  return CG_OK;
}

}  // namespace

bool dfft_supported(int n) { return n >= 64 && n <= 2048 && (n & (n - 1)) == 0; }

// In-place batched FFT of `batch` contiguous complex128 rows of length n
// (a power of two, 64..2048); inverse: exp(+2 pi i), unnormalised.
int dfft_rows(double2 *data, int64_t batch, int n, int inverse, cudaStream_t st) {
  CG_REQUIRE(dfft_supported(n), "double-float FFT lengths are powers of two 64..2048");
  if (batch <= 0) return CG_OK;
  const double2 *tw;
  int rc = twiddles(n, inverse ? 1 : -1, &tw);
  if (rc) return rc;
  switch (n) {
    case 64: return launch<6, 8>(data, batch, tw, st);
    case 128: return launch<7, 4>(data, batch, tw, st);
    case 256: return launch<8, 2>(data, batch, tw, st);
    case 512: return launch<9, 1>(data, batch, tw, st);
    case 1024: return launch<10, 1>(data, batch, tw, st);
    case 2048: return launch<11, 1>(data, batch, tw, st);
  }
  return set_error(CG_ERR_ARG, "unsupported double-float FFT length %d", n);
}

}  // namespace cg

extern "C" int cg_fft_rows_df(void *data_c128, int64_t batch, int n, int inverse,
                              cg_stream_t stream) {
  CG_REQUIRE(data_c128 && batch >= 0, "bad double-float FFT arguments");
  return cg::dfft_rows((double2 *)data_c128, batch, n, inverse, (cudaStream_t)stream);
}
