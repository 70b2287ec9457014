// Double-float FFT building blocks shared by the transforms of dfft.cu and
// the fused recombination passes of recombine.cu: the radix-2 / radix-4
// Stockham butterflies (dfft.cu has the algorithm), the row-transform kernel
// over an element I/O policy, and its launcher.
//
// An I/O policy is a small struct passed by value with
//   __device__ cdf ld(int64_t row, int i) const;            // element i of row
//   __device__ void st(int64_t row, int i, const cdf &v) const;
// so a transform can gather its input (a window, a crop, a conversion) and
// scatter its output (a crop, a transpose, a weighting) without a separate
// pass over HBM.
#pragma once

#include <algorithm>

#include "cg_internal.cuh"
#include "df.cuh"

namespace cg {

bool dfft_supported(int n);
// device table of w^k = exp(sign 2 pi i k / n), k < 3n/4, as double-float
// (cached per device, n and sign)
int dfft_twiddles(int n, int sign, const float4 **out);

namespace dfk {

// ---------------------------------------------------------------- butterflies
// One radix-2 butterfly of the first stage (stride 1, m = N/2) on element t2
// and one radix-4 butterfly of the stage with stride s (m = N/(4s)) for
// t = p s + q: inputs x[t + k N/4], outputs y[q + s (4p + k)], twiddles
// w^(k p s) from the table (k p s < 3N/4).  x[.] indexes through `at`, so the
// same code serves rows (at(i) = i) and column tiles (at(i) = i C + c).

__device__ __forceinline__ cdf cdf_mul_j(const cdf &v, bool inverse) {  // times -i (+i)
  return inverse ? cdf{df_neg(v.im), v.re} : cdf{v.im, df_neg(v.re)};
}

template <int N, class AT>
__device__ __forceinline__ void radix2_first(const cdf *x, cdf *y, const cdf *stw, int t2,
                                             AT at) {
  const cdf a = x[at(t2)], b = x[at(t2 + N / 2)];
  y[at(2 * t2)] = cdf_add_f(a, b);
  const cdf d = cdf_sub_f(a, b);
  y[at(2 * t2 + 1)] = t2 == 0 ? d : cdf_mul_f(d, stw[t2]);
}

template <int N, class AT>
__device__ __forceinline__ void radix4(const cdf *x, cdf *y, const cdf *stw, int t, int s,
                                       bool inverse, AT at) {
  constexpr int Q = N / 4;
  const int q = t & (s - 1), ps = t - q;  // p s
  const cdf x0 = x[at(t)], x1 = x[at(t + Q)], x2 = x[at(t + 2 * Q)], x3 = x[at(t + 3 * Q)];
  const cdf a0 = cdf_add_f(x0, x2), a1 = cdf_sub_f(x0, x2);
  const cdf b0 = cdf_add_f(x1, x3), b1 = cdf_mul_j(cdf_sub_f(x1, x3), inverse);
  const int o = q + 4 * ps;
  y[at(o)] = cdf_add_f(a0, b0);
  if (ps == 0) {
    y[at(o + s)] = cdf_add_f(a1, b1);
    y[at(o + 2 * s)] = cdf_sub_f(a0, b0);
    y[at(o + 3 * s)] = cdf_sub_f(a1, b1);
  } else {
    y[at(o + s)] = cdf_mul_f(cdf_add_f(a1, b1), stw[ps]);
    y[at(o + 2 * s)] = cdf_mul_f(cdf_sub_f(a0, b0), stw[2 * ps]);
    y[at(o + 3 * s)] = cdf_mul_f(cdf_sub_f(a1, b1), stw[3 * ps]);
  }
}

struct AtRow {
  __device__ int operator()(int i) const { return i; }
};
template <int C>
struct AtCol {
  int c;
  __device__ int operator()(int i) const { return i * C + c; }
};

// ---------------------------------------------------------------- row transforms
// ROWS rows of length N per CTA, N/4 threads per row; two cdf buffers and
// the 3N/4 twiddles in shared memory.  Odd log2 N: one radix-2 stage first.
template <int LOGN, int ROWS, class IO>
__global__ void __launch_bounds__((1 << LOGN) / 4 * ROWS)
    k_dfft_rows(IO io, int64_t batch, const float4 *__restrict__ tw, int inverse) {
  constexpr int N = 1 << LOGN;
  constexpr int Q = N / 4;
  extern __shared__ float dsm[];
  cdf *buf0 = (cdf *)dsm;       // [ROWS][N]
  cdf *buf1 = buf0 + ROWS * N;  // [ROWS][N]
  cdf *stw = buf1 + ROWS * N;   // [3N/4] twiddles
  const int r = threadIdx.x / Q, t = threadIdx.x - (threadIdx.x / Q) * Q;
  for (int k = threadIdx.x; k < 3 * Q; k += blockDim.x) stw[k] = cdf_load(tw[k]);
  const bool inv = inverse != 0;
  for (int64_t row0 = (int64_t)blockIdx.x * ROWS; row0 < batch;
       row0 += (int64_t)gridDim.x * ROWS) {
    const int64_t row = row0 + r;
    const bool live = row < batch;
    cdf *x = buf0 + r * N, *y = buf1 + r * N;
    if (live) {
#pragma unroll
      for (int k = 0; k < 4; ++k) x[t + k * Q] = io.ld(row, t + k * Q);
    }
    __syncthreads();
    if (LOGN & 1) {
      if (live) {
        radix2_first<N>(x, y, stw, t, AtRow());
        radix2_first<N>(x, y, stw, t + Q, AtRow());
      }
      __syncthreads();
      cdf *tmp = x;
      x = y;
      y = tmp;
    }
#pragma unroll
    for (int ls = (LOGN & 1); ls < LOGN; ls += 2) {
      if (live) radix4<N>(x, y, stw, t, 1 << ls, inv, AtRow());
      __syncthreads();
      cdf *tmp = x;
      x = y;
      y = tmp;
    }
    if (live) {
#pragma unroll
      for (int k = 0; k < 4; ++k) io.st(row, t + k * Q, x[t + k * Q]);
    }
    __syncthreads();
  }
}

template <int LOGN, int ROWS, class IO>
int launch_rows(IO io, int64_t batch, const float4 *tw, int inverse, cudaStream_t st) {
  constexpr int N = 1 << LOGN;
  const size_t smem = (size_t)(2 * ROWS * N + 3 * N / 4) * sizeof(cdf);
  if (smem > 48 * 1024)  // set on every launch: the attribute is per device
    CG_CUDA(cudaFuncSetAttribute(k_dfft_rows<LOGN, ROWS, IO>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t ctas = (batch + ROWS - 1) / ROWS;
  const unsigned grid = (unsigned)std::min<int64_t>(ctas, (int64_t)num_sms() * 8);
  k_dfft_rows<LOGN, ROWS, IO><<<grid, N / 4 * ROWS, smem, st>>>(io, batch, tw, inverse);
  CG_LAUNCH("double-float FFT");
  return CG_OK;
}

template <class IO>
int launch_any(IO io, int64_t batch, int n, int inverse, cudaStream_t st) {
  CG_REQUIRE(dfft_supported(n), "double-float FFT lengths are powers of two 64..2048");
  if (batch <= 0) return CG_OK;
  const float4 *tw;
  int rc = dfft_twiddles(n, inverse ? 1 : -1, &tw);
  if (rc) return rc;
  switch (n) {  // N/4 threads per row, 256 threads per CTA up to 1024
    case 64: return launch_rows<6, 16>(io, batch, tw, inverse, st);
    case 128: return launch_rows<7, 8>(io, batch, tw, inverse, st);
    case 256: return launch_rows<8, 4>(io, batch, tw, inverse, st);
    case 512: return launch_rows<9, 2>(io, batch, tw, inverse, st);
    case 1024: return launch_rows<10, 1>(io, batch, tw, inverse, st);
    case 2048: return launch_rows<11, 1>(io, batch, tw, inverse, st);
  }
  return set_error(CG_ERR_ARG, "unsupported double-float FFT length %d", n);
}

}  // namespace dfk

// In-place batched transforms of `batch` rows of length n (a power of two,
// 64..2048) through the I/O policy io; inverse: exp(+2 pi i), unnormalised.
template <class IO>
int dfft_rows_io(IO io, int64_t batch, int n, int inverse, cudaStream_t st) {
  return dfk::launch_any(io, batch, n, inverse, st);
}

}  // namespace cg
