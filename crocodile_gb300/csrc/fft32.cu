// Hand-written FP32 FFTs of power-of-two complex64 planes: the centred
// fft / ifft of crocodile/synthesis.py:83-106 (fftshift(fft2(ifftshift(a))),
// 1 / (H W) on the inverse), the unshifted transform of the sub-grid stacks,
// and the dirty image of do_imaging (real part of the centred ifft, :903-906),
// for sides 64 .. 8192.
//
// Two passes over HBM per plane, both in place:
//   rows:    each CTA loads whole rows (bit-reversed into shared memory),
//            transforms them with the radix-4 DIT of fft32.h and stores them;
//   columns: each CTA loads a tile of C adjacent columns (C x 8 bytes of every
//            row, H x C <= 16384 elements), transforms every column of the
//            tile and stores it.
// Neither needs a second buffer (the DIT runs in place on the bit-reversed
// line), so even 8192-long columns fit two to a CTA.  The centring of the
// centred transform is the checkerboard identity for even sides,
//   fftshift(F(ifftshift x))[k] = (-1)^(k + H/2 + W/2) F((-1)^n x)[k],
// folded into the row pass's loads and the column pass's stores together
// with the 1 / (H W) of the inverse; the dirty image's real part, sign and
// scale and its maximum are the column pass's store.
#include <float.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "cg_internal.cuh"
#include "fft32.h"

namespace cg {
namespace f32 {

constexpr int MIN_LOG = 6, MAX_LOG = 13;
constexpr int ROW_THREADS = 512, COL_THREADS = 1024;

__device__ __forceinline__ int pad(int i) { return i + (i >> 5); }  // bank spread

// A line in shared memory: element p at base[pad(p) * C + c] (C lines interleaved).
struct SmLine {
  float2 *base;
  int C, c;
  __device__ cf get(int p) const {
    const float2 v = base[pad(p) * C + c];
    return {v.x, v.y};
  }
  __device__ void set(int p, cf v) const { base[pad(p) * C + c] = make_float2(v.x, v.y); }
};
struct SmTw {
  const float2 *t;
  __device__ cf get(int k) const {
    const float2 v = t[k];
    return {v.x, v.y};
  }
};

// w_N^k = exp(sign 2 pi i k / N), k < N / 2, cached per device, log N and sign
std::mutex g_mu;
std::map<std::tuple<int, int, int>, float2 *> g_tw;

int twiddles(int logn, int sign, const float2 **out) {
  int dev = 0;
  CG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_mu);
  const auto key = std::make_tuple(dev, logn, sign);
  auto it = g_tw.find(key);
  if (it != g_tw.end()) {
    *out = it->second;
    return CG_OK;
  }
  const int n = 1 << logn;
  std::vector<float2> h(n / 2);
  for (int k = 0; k < n / 2; ++k) {
    const double a = 2.0 * M_PI * (double)k / (double)n;
    h[k] = make_float2((float)std::cos(a), (float)(sign * std::sin(a)));
  }
  float2 *d = nullptr;
  CG_CUDA(cudaMalloc(&d, h.size() * sizeof(float2)));
  CG_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice));
  g_tw[key] = d;
  *out = d;
  return CG_OK;
}

// ---------------------------------------------------------------- I/O policies
// Row pass: rows of all planes, row index = plane * H + r.
struct RowIO {
  float2 *d;
  int W, H;
  int modulate;  // multiply element (r, i) by (-1)^(r + i) on the way in
  int post;      // rows-only transforms: times scale (-1)^(k + phase) on the way out
  int phase;
  float scale;
  __device__ float2 ld(int64_t row, int i) const {
    float2 v = d[row * W + i];
    if (modulate && (((int)(row % H) + i) & 1)) v = make_float2(-v.x, -v.y);
    return v;
  }
  __device__ void st(int64_t row, int i, float2 v) const {
    if (post) {
      const float s = ((i + phase) & 1) ? -scale : scale;
      v = make_float2(v.x * s, v.y * s);
    }
    d[row * W + i] = v;
  }
};

// Column pass, complex output: times s = scale (and (-1)^(k + c + phase) if centred).
struct ColIO {
  float2 *d;
  int W, H;
  int centred, phase;
  float scale;
  __device__ float2 ld(int64_t plane, int i, int c) const {
    return d[(plane * H + i) * (int64_t)W + c];
  }
  __device__ void st(int64_t plane, int i, int c, float2 v, float &) const {
    float s = scale;
    if (centred && ((i + c + phase) & 1)) s = -s;
    d[(plane * H + i) * (int64_t)W + c] = make_float2(v.x * s, v.y * s);
  }
  static constexpr bool kMax = false;
};

// Column pass of the dirty image: the real part, demodulated and scaled, into a
// float image, and its maximum.
struct ColImageIO {
  const float2 *d;
  float *img;
  int W, H, phase;
  float scale;
  __device__ float2 ld(int64_t, int i, int c) const { return d[(int64_t)i * W + c]; }
  __device__ void st(int64_t, int i, int c, float2 v, float &mx) const {
    const float r = v.x * (((i + c + phase) & 1) ? -scale : scale);
    img[(int64_t)i * W + c] = r;
    mx = fmaxf(mx, r);
  }
  static constexpr bool kMax = true;
};

__device__ __forceinline__ void atomic_max_f(float *addr, float v) {
  if (v >= 0.f)
    atomicMax((int *)addr, __float_as_int(v));
  else
    atomicMin((unsigned int *)addr, __float_as_uint(v));
}

// ---------------------------------------------------------------- kernels
// R = 2048 / N rows per CTA for short rows (at least 512 butterflies a stage).
template <int LOGN>
__global__ void __launch_bounds__(ROW_THREADS) k_fft32_rows(RowIO io, int64_t nrows,
                                                            const float2 *__restrict__ tw,
                                                            int sign) {
  constexpr int N = 1 << LOGN;
  constexpr int R = N >= 2048 ? 1 : 2048 / N;
  constexpr int P = N + N / 32;  // padded row
  extern __shared__ float2 f32_sm[];
  float2 *stw = f32_sm;
  float2 *rows = f32_sm + N / 2;
  const int tid = threadIdx.x;
  for (int k = tid; k < N / 2; k += ROW_THREADS) stw[k] = tw[k];
  const SmTw T{stw};
  for (int64_t row0 = (int64_t)blockIdx.x * R; row0 < nrows; row0 += (int64_t)gridDim.x * R) {
    __syncthreads();  // twiddles staged; the previous rows' stores have read smem
    for (int e = tid; e < R * N; e += ROW_THREADS) {
      const int r = e >> LOGN, i = e & (N - 1);
      const int64_t row = row0 + r;
      rows[r * P + pad((int)bitrev((unsigned)i, LOGN))] =
          row < nrows ? io.ld(row, i) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    int lh = 0;
    if (LOGN & 1) {
      for (int b = tid; b < R * N / 2; b += ROW_THREADS) {
        SmLine x{rows + (b >> (LOGN - 1)) * P, 1, 0};
        radix2_first(x, b & (N / 2 - 1));
      }
      __syncthreads();
      lh = 1;
    }
#pragma unroll 1
    for (; lh + 1 < LOGN; lh += 2) {
      for (int b = tid; b < R * N / 4; b += ROW_THREADS) {
        SmLine x{rows + (b >> (LOGN - 2)) * P, 1, 0};
        radix4(x, T, LOGN, lh, b & (N / 4 - 1), sign);
      }
      __syncthreads();
    }
    for (int e = tid; e < R * N; e += ROW_THREADS) {
      const int r = e >> LOGN, i = e & (N - 1);
      const int64_t row = row0 + r;
      if (row < nrows) io.st(row, i, rows[r * P + pad(i)]);
    }
  }
}

// Tiles of C columns of one plane; units = planes * (W / C).
template <int LOGH, int C, class IO>
__global__ void __launch_bounds__(COL_THREADS) k_fft32_cols(IO io, int64_t nplanes, int W,
                                                            const float2 *__restrict__ tw,
                                                            int sign, float *max_out) {
  constexpr int H = 1 << LOGH;
  extern __shared__ float2 f32_sm[];
  float2 *stw = f32_sm;
  float2 *cols = f32_sm + H / 2;
  const int tid = threadIdx.x;
  for (int k = tid; k < H / 2; k += COL_THREADS) stw[k] = tw[k];
  const SmTw T{stw};
  const int per_plane = W / C;
  float mx = -FLT_MAX;
  for (int64_t unit = blockIdx.x; unit < nplanes * per_plane; unit += gridDim.x) {
    const int64_t plane = unit / per_plane;
    const int c0 = (int)(unit - plane * per_plane) * C;
    __syncthreads();
    for (int e = tid; e < H * C; e += COL_THREADS) {
      const int i = e / C, c = e - (e / C) * C;
      cols[pad((int)bitrev((unsigned)i, LOGH)) * C + c] = io.ld(plane, i, c0 + c);
    }
    __syncthreads();
    int lh = 0;
    if (LOGH & 1) {
      for (int b = tid; b < C * H / 2; b += COL_THREADS) {
        SmLine x{cols, C, b % C};
        radix2_first(x, b / C);
      }
      __syncthreads();
      lh = 1;
    }
#pragma unroll 1
    for (; lh + 1 < LOGH; lh += 2) {
      for (int b = tid; b < C * H / 4; b += COL_THREADS) {
        SmLine x{cols, C, b % C};
        radix4(x, T, LOGH, lh, b / C, sign);
      }
      __syncthreads();
    }
    for (int e = tid; e < H * C; e += COL_THREADS) {
      const int i = e / C, c = e - (e / C) * C;
      io.st(plane, i, c0 + c, cols[pad(i) * C + c], mx);
    }
  }
  if (IO::kMax && max_out) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) atomic_max_f(max_out, mx);
  }
}

__global__ void k_fft32_init_max(float *m) { *m = -FLT_MAX; }

int log2_exact(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return (1 << l) == n ? l : -1;
}

template <int LOGN>
int launch_rows(const RowIO &io, int64_t nrows, int sign, cudaStream_t st) {
  constexpr int N = 1 << LOGN;
  constexpr int R = N >= 2048 ? 1 : 2048 / N;
  const float2 *tw;
  int rc = twiddles(LOGN, sign, &tw);
  if (rc) return rc;
  const size_t smem = (size_t)(N / 2 + R * (N + N / 32)) * sizeof(float2);
  CG_CUDA(cudaFuncSetAttribute(k_fft32_rows<LOGN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  const int64_t ctas = (nrows + R - 1) / R;
  const unsigned grid = (unsigned)std::min<int64_t>(ctas, (int64_t)num_sms() * 4);
  k_fft32_rows<LOGN><<<grid, ROW_THREADS, smem, st>>>(io, nrows, tw, sign);
  CG_LAUNCH("FP32 FFT rows");
  return CG_OK;
}

// columns per tile: H * C <= 16384 elements (128 KB), at most 32
constexpr int cols_for(int logh) { return logh >= 13 ? 2 : logh >= 9 ? (1 << (14 - logh)) : 32; }

template <int LOGH, class IO>
int launch_cols(const IO &io, int64_t nplanes, int W, int sign, float *max_out, cudaStream_t st) {
  constexpr int H = 1 << LOGH, C = cols_for(LOGH);
  CG_REQUIRE(W % C == 0, "FP32 FFT: width %d is not a multiple of the column tile %d", W, C);
  const float2 *tw;
  int rc = twiddles(LOGH, sign, &tw);
  if (rc) return rc;
  const size_t smem = (size_t)(H / 2 + (H + H / 32) * C) * sizeof(float2);
  CG_CUDA(cudaFuncSetAttribute(k_fft32_cols<LOGH, C, IO>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t units = nplanes * (W / C);
  const unsigned grid = (unsigned)std::min<int64_t>(units, (int64_t)num_sms() * 2);
  k_fft32_cols<LOGH, C, IO><<<grid, COL_THREADS, smem, st>>>(io, nplanes, W, tw, sign, max_out);
  CG_LAUNCH("FP32 FFT columns");
  return CG_OK;
}

template <class IO>
int dispatch_cols(int logh, const IO &io, int64_t nplanes, int W, int sign, float *max_out,
                  cudaStream_t st) {
  switch (logh) {
    case 6: return launch_cols<6>(io, nplanes, W, sign, max_out, st);
    case 7: return launch_cols<7>(io, nplanes, W, sign, max_out, st);
    case 8: return launch_cols<8>(io, nplanes, W, sign, max_out, st);
    case 9: return launch_cols<9>(io, nplanes, W, sign, max_out, st);
    case 10: return launch_cols<10>(io, nplanes, W, sign, max_out, st);
    case 11: return launch_cols<11>(io, nplanes, W, sign, max_out, st);
    case 12: return launch_cols<12>(io, nplanes, W, sign, max_out, st);
    case 13: return launch_cols<13>(io, nplanes, W, sign, max_out, st);
  }
  return set_error(CG_ERR_ARG, "FP32 FFT: unsupported column length 2^%d", logh);
}

int dispatch_rows(int logw, const RowIO &io, int64_t nrows, int sign, cudaStream_t st) {
  switch (logw) {
    case 6: return launch_rows<6>(io, nrows, sign, st);
    case 7: return launch_rows<7>(io, nrows, sign, st);
    case 8: return launch_rows<8>(io, nrows, sign, st);
    case 9: return launch_rows<9>(io, nrows, sign, st);
    case 10: return launch_rows<10>(io, nrows, sign, st);
    case 11: return launch_rows<11>(io, nrows, sign, st);
    case 12: return launch_rows<12>(io, nrows, sign, st);
    case 13: return launch_rows<13>(io, nrows, sign, st);
  }
  return set_error(CG_ERR_ARG, "FP32 FFT: unsupported row length 2^%d", logw);
}

}  // namespace f32

// Sides the hand-written FP32 transform takes: powers of two 64..8192 (H may
// be 1 for a batch of rows).
bool fft32_supported(int H, int W) {
  const int lw = f32::log2_exact(W), lh = f32::log2_exact(H);
  return lw >= f32::MIN_LOG && lw <= f32::MAX_LOG &&
         (H == 1 || (lh >= f32::MIN_LOG && lh <= f32::MAX_LOG));
}

// In place on batch planes of H x W complex64: centred (fft / ifft of
// synthesis.py, 1 / (H W) on the inverse) or raw (unshifted, unscaled).
int fft32_planes(float2 *data, int64_t batch, int H, int W, bool inverse, bool centred,
                 cudaStream_t st) {
  CG_REQUIRE(fft32_supported(H, W), "FP32 FFT sides must be powers of two 64..8192 (%dx%d)", H,
             W);
  const int sign = inverse ? 1 : -1;
  const int lw = f32::log2_exact(W), lh = H == 1 ? 0 : f32::log2_exact(H);
  const double scale = inverse && centred ? 1.0 / ((double)H * W) : 1.0;
  const int phase = (H == 1 ? 0 : H / 2) + W / 2;
  if (H == 1) {  // rows only: modulation on the way in, sign and scale on the way out
    f32::RowIO io{data, W, 1, centred ? 1 : 0, centred ? 1 : 0, phase & 1, (float)scale};
    return f32::dispatch_rows(lw, io, batch, sign, st);
  }
  f32::RowIO rio{data, W, H, centred ? 1 : 0, 0, 0, 1.f};
  int rc = f32::dispatch_rows(lw, rio, batch * H, sign, st);
  if (rc) return rc;
  f32::ColIO cio{data, W, H, centred ? 1 : 0, phase & 1, (float)scale};
  return f32::dispatch_cols(lh, cio, batch, W, sign, nullptr, st);
}

// The dirty image of a pre-modulated hermitian grid (k_hermitian with the
// checkerboard): rows, then columns storing the real part times
// (-1)^(i + j + H/2 + W/2) / (H W) and the image maximum.
int fft32_image(const float2 *grid_premod, int H, int W, float *image, float *max_out,
                cudaStream_t st) {
  CG_REQUIRE(fft32_supported(H, W) && H > 1, "FP32 FFT sides must be powers of two 64..8192");
  const int lw = f32::log2_exact(W), lh = f32::log2_exact(H);
  f32::RowIO rio{(float2 *)grid_premod, W, H, 0, 0, 0, 1.f};
  int rc = f32::dispatch_rows(lw, rio, H, 1, st);
  if (rc) return rc;
  if (max_out) {
    f32::k_fft32_init_max<<<1, 1, 0, st>>>(max_out);
    CG_LAUNCH("image max init");
  }
  f32::ColImageIO io{grid_premod, image, W, H, (H / 2 + W / 2) & 1,
                     (float)(1.0 / ((double)H * W))};
  return f32::dispatch_cols(lh, io, 1, W, 1, max_out, st);
}

}  // namespace cg
