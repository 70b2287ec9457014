// Hand-written FP32 FFTs of power-of-two complex64 planes: the centred
// fft / ifft of crocodile/synthesis.py:83-106 (fftshift(fft2(ifftshift(a))),
// 1 / (H W) on the inverse), the unshifted transform of the sub-grid stacks,
// and the dirty image of do_imaging (real part of the centred ifft, :903-906),
// for sides 64 .. 8192.
//
// Two passes over HBM per plane, both in place:
//   rows:    512 threads per CTA transform 512 / (N / 16) whole rows;
//   columns: up to 512 threads per CTA transform a tile of C adjacent
//            columns (C x 8 bytes of every row, H x C <= 8192 elements).
// Each line runs the register-blocked Stockham stages of fft32.h (radix 16,
// 16 values per thread): the first stage reads global memory and the last
// writes it, coalesced; the stages between exchange through one padded
// shared-memory buffer (every thread reads, barrier, every thread writes),
// so a line makes one or two round trips through shared memory.  The
// centring of the centred transform is the checkerboard identity for even
// sides,
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
constexpr int ROW_THREADS = 512, COL_THREADS = 512;
// square planes from this side on run their columns as rows between two
// in-place transposes (the column tiles hold only 1 or 2 columns there)
constexpr int TRANSPOSE_MIN = 4096;

__device__ __forceinline__ int pad(int e) { return e + (e >> 5); }  // bank spread

// Twiddles w_N^j = exp(sign 2 pi i j / N), j < N, as a two-level table:
// w_N^j = A[j mod TWB] * C[j / TWB], A[a] = w_N^a (a < TWB), C[c] = w_N^(c TWB)
// (c < N / TWB); TWB + N / TWB entries (192 for N = 8192), staged in shared
// memory by every CTA.  Each twiddle costs one complex product more than a
// full table (within about 1.5 units of FP32 rounding).  Cached per device,
// log N and sign.
constexpr int TWB_LOG = 6, TWB = 1 << TWB_LOG;
constexpr int tw_entries(int logn) {
  return logn > TWB_LOG ? TWB + (1 << (logn - TWB_LOG)) : (1 << logn) + 1;
}
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
  const int nb = logn > TWB_LOG ? TWB : n, nc = logn > TWB_LOG ? n / TWB : 1;
  std::vector<float2> h(tw_entries(logn));
  auto w = [&](long j) {
    const double a = 2.0 * M_PI * (double)j / (double)n;
    return make_float2((float)std::cos(a), (float)(sign * std::sin(a)));
  };
  for (int a = 0; a < nb; ++a) h[a] = w(a);
  for (int c = 0; c < nc; ++c) h[nb + c] = w((long)c * nb);
  float2 *d = nullptr;
  CG_CUDA(cudaMalloc(&d, h.size() * sizeof(float2)));
  CG_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice));
  g_tw[key] = d;
  *out = d;
  return CG_OK;
}

// the two-level table in shared memory
template <int LOGN>
struct SmTw2 {
  const float2 *t;
  __device__ cf operator()(int j) const {
    if (LOGN <= TWB_LOG) {
      const float2 v = t[j];
      return cf{v.x, v.y};
    }
    const float2 a = t[j & (TWB - 1)], c = t[TWB + (j >> TWB_LOG)];
    return cf_mul(cf{a.x, a.y}, cf{c.x, c.y});
  }
};

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
  // column `c` of plane `plane`: element i at base[i * W]
  __device__ const float2 *src(int64_t plane, int c) const { return d + plane * H * (int64_t)W + c; }
  __device__ float2 *dst(int64_t plane, int c) const { return d + plane * H * (int64_t)W + c; }
  __device__ void st(float2 *base, int i, int c, float2 v, float &) const {
    float s = scale;
    if (centred && ((i + c + phase) & 1)) s = -s;
    base[i * W] = make_float2(v.x * s, v.y * s);
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
  __device__ const float2 *src(int64_t, int c) const { return d + c; }
  __device__ float *dst(int64_t, int c) const { return img + c; }
  __device__ void st(float *base, int i, int c, float2 v, float &mx) const {
    const float r = v.x * (((i + c + phase) & 1) ? -scale : scale);
    base[i * W] = r;
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
// T = N / 16 threads per line.  Rows: 512 / T lines per CTA.
template <int LOGN>
__global__ void __launch_bounds__(ROW_THREADS, 2) k_fft32_rows(RowIO io, int64_t nrows,
                                                            const float2 *__restrict__ tw,
                                                            int sign) {
  constexpr int N = 1 << LOGN, T = N / 16, LPC = ROW_THREADS / T, P = N + N / 32;
  constexpr int NS = (LOGN + 3) / 4;
  extern __shared__ float2 f32_sm[];
  const int line = threadIdx.x / T, t = threadIdx.x % T;
  float2 *buf = f32_sm + line * P;
  float2 *stw = f32_sm + LPC * P;
  for (int k = threadIdx.x; k < tw_entries(LOGN); k += ROW_THREADS) stw[k] = tw[k];
  __syncthreads();
  const SmTw2<LOGN> twf{stw};
  auto lds = [&](int e) {
    const float2 v = buf[pad(e)];
    return cf{v.x, v.y};
  };
  auto sts = [&](int e, cf v) { buf[pad(e)] = make_float2(v.x, v.y); };
  for (int64_t row0 = (int64_t)blockIdx.x * LPC; row0 < nrows; row0 += (int64_t)gridDim.x * LPC) {
    const int64_t row = row0 + line;
    const bool live = row < nrows;
    cf v[16];
    stage_load(LOGN, 0, t, [&](int e) {
      const float2 x = live ? io.ld(row, e) : make_float2(0.f, 0.f);
      return cf{x.x, x.y};
    }, twf, v);
    stage_dft(LOGN, 0, sign, v);
    stage_store(LOGN, 0, t, sts, v);
#pragma unroll
    for (int s = 1; s < NS; ++s) {
      // a row of N <= 512 is one warp's (T <= 32 threads): warp barriers suffice
      if (T <= 32) __syncwarp(); else __syncthreads();  // previous stores visible
      stage_load(LOGN, s, t, lds, twf, v);
      if (T <= 32) __syncwarp(); else __syncthreads();  // all reads before any write
      stage_dft(LOGN, s, sign, v);
      if (s + 1 < NS) {
        stage_store(LOGN, s, t, sts, v);
      } else if (live) {
        stage_store(LOGN, s, t, [&](int e, cf x) { io.st(row, e, make_float2(x.x, x.y)); }, v);
      }
    }
  }
}

// Tiles of C columns of one plane (units = planes * W / C), T = H / 16
// threads per column, thread (t, c) with c fastest for coalesced rows.
template <int LOGH, int C, class IO>
__global__ void __launch_bounds__(COL_THREADS) k_fft32_cols(IO io, int64_t nplanes, int W,
                                                            const float2 *__restrict__ tw,
                                                            int sign, float *max_out) {
  constexpr int H = 1 << LOGH, T = H / 16;
  constexpr int NS = (LOGH + 3) / 4;
  extern __shared__ float2 f32_sm[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  float2 *stw = f32_sm + (H + H / 32) * C;
  for (int k = threadIdx.x; k < tw_entries(LOGH); k += C * T) stw[k] = tw[k];
  __syncthreads();
  const SmTw2<LOGH> twf{stw};
  auto lds = [&](int e) {
    const float2 v = f32_sm[pad(e) * C + c];
    return cf{v.x, v.y};
  };
  auto sts = [&](int e, cf v) { f32_sm[pad(e) * C + c] = make_float2(v.x, v.y); };
  const int per_plane = W / C;
  float mx = -FLT_MAX;
  for (int64_t unit = blockIdx.x; unit < nplanes * per_plane; unit += gridDim.x) {
    const int64_t plane = unit / per_plane;
    const int col = (int)(unit - plane * per_plane) * C + c;
    const float2 *src = io.src(plane, col);
    auto dst = io.dst(plane, col);
    cf v[16];
    __syncthreads();  // the previous tile's last reads of shared memory are done
    stage_load(LOGH, 0, t, [&](int e) {
      const float2 x = src[e * W];
      return cf{x.x, x.y};
    }, twf, v);
    stage_dft(LOGH, 0, sign, v);
    stage_store(LOGH, 0, t, sts, v);
#pragma unroll
    for (int s = 1; s < NS; ++s) {
      __syncthreads();
      stage_load(LOGH, s, t, lds, twf, v);
      __syncthreads();
      stage_dft(LOGH, s, sign, v);
      if (s + 1 < NS)
        stage_store(LOGH, s, t, sts, v);
      else
        stage_store(LOGH, s, t, [&](int e, cf x) { io.st(dst, e, col, make_float2(x.x, x.y), mx); },
                    v);
    }
  }
  if (IO::kMax && max_out) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomic_max_f(max_out, mx);
  }
}

// ---------------------------------------------------------------- square transposes
// In place on nplanes N x N planes: the CTA of tile pair (I, J), I <= J, of
// 32 x 32 tiles reads both tiles into shared memory and writes each to the
// other's place (a diagonal tile to itself).  The store policy takes the
// final position (r, c); the last transpose of a centred transform applies
// (-1)^(r + c + phase) and the scale there, or writes the dirty image.
struct TpPlain {
  __device__ void st(float2 *d, int64_t off, int, int, float2 v, float &) const { d[off] = v; }
  static constexpr bool kMax = false;
};
struct TpCentred {
  int phase;
  float scale;
  __device__ void st(float2 *d, int64_t off, int r, int c, float2 v, float &) const {
    const float s = ((r + c + phase) & 1) ? -scale : scale;
    d[off] = make_float2(v.x * s, v.y * s);
  }
  static constexpr bool kMax = false;
};
struct TpImage {
  float *img;
  int phase;
  float scale;
  __device__ void st(float2 *, int64_t off, int r, int c, float2 v, float &mx) const {
    const float x = v.x * (((r + c + phase) & 1) ? -scale : scale);
    img[off] = x;
    mx = fmaxf(mx, x);
  }
  static constexpr bool kMax = true;
};

template <class ST>
__global__ void __launch_bounds__(256) k_fft32_transpose(float2 *d, int N, ST st, float *max_out) {
  __shared__ float2 ta[32][33], tb[32][33];
  const int nt = N / 32;
  const int I = blockIdx.x / nt, J = blockIdx.x - (blockIdx.x / nt) * nt;
  float mx = -FLT_MAX;
  if (I <= J) {
    float2 *p = d + (int64_t)blockIdx.y * N * N;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
#pragma unroll
    for (int k = 0; k < 32; k += 8) {
      ta[ty + k][tx] = p[(int64_t)(I * 32 + ty + k) * N + J * 32 + tx];
      if (I != J) tb[ty + k][tx] = p[(int64_t)(J * 32 + ty + k) * N + I * 32 + tx];
    }
    __syncthreads();
    const int64_t plane = (int64_t)blockIdx.y * N * N;
#pragma unroll
    for (int k = 0; k < 32; k += 8) {
      // tile (J, I) receives ta transposed; tile (I, J) receives tb transposed
      const int r1 = J * 32 + ty + k, c1 = I * 32 + tx;
      st.st(d, plane + (int64_t)r1 * N + c1, r1, c1, ta[tx][ty + k], mx);
      if (I != J) {
        const int r2 = I * 32 + ty + k, c2 = J * 32 + tx;
        st.st(d, plane + (int64_t)r2 * N + c2, r2, c2, tb[tx][ty + k], mx);
      }
    }
  }
  if (ST::kMax && max_out) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomic_max_f(max_out, mx);
  }
}

template <class ST>
int launch_transpose(float2 *d, int64_t nplanes, int N, const ST &st, float *max_out,
                     cudaStream_t s) {
  CG_REQUIRE(N % 32 == 0 && nplanes <= 65535, "transpose needs N a multiple of 32");
  const int nt = N / 32;
  k_fft32_transpose<ST><<<dim3((unsigned)(nt * nt), (unsigned)nplanes), 256, 0, s>>>(d, N, st,
                                                                                      max_out);
  CG_LAUNCH("FP32 FFT transpose");
  return CG_OK;
}

__global__ void k_fft32_init_max(float *m) { *m = -FLT_MAX; }

int log2_exact(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return (1 << l) == n ? l : -1;
}

template <int LOGN>
int launch_rows(const RowIO &io, int64_t nrows, int sign, cudaStream_t st) {
  constexpr int N = 1 << LOGN, T = N / 16, LPC = ROW_THREADS / T;
  const float2 *tw;
  int rc = twiddles(LOGN, sign, &tw);
  if (rc) return rc;
  const size_t smem = (size_t)(LPC * (N + N / 32) + tw_entries(LOGN)) * sizeof(float2);
  CG_CUDA(cudaFuncSetAttribute(k_fft32_rows<LOGN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  const int64_t ctas = (nrows + LPC - 1) / LPC;
  const unsigned grid = (unsigned)std::min<int64_t>(ctas, (int64_t)num_sms() * 3);
  k_fft32_rows<LOGN><<<grid, ROW_THREADS, smem, st>>>(io, nrows, tw, sign);
  CG_LAUNCH("FP32 FFT rows");
  return CG_OK;
}

// columns per tile: 512 threads (T = H / 16 per column), at most 32 columns
constexpr int cols_for(int logh) {
  return (COL_THREADS >> (logh - 4)) < 32 ? (COL_THREADS >> (logh - 4)) : 32;
}

template <int LOGH, class IO>
int launch_cols(const IO &io, int64_t nplanes, int W, int sign, float *max_out, cudaStream_t st) {
  constexpr int H = 1 << LOGH, C = cols_for(LOGH), T = H / 16;
  CG_REQUIRE(W % C == 0, "FP32 FFT: width %d is not a multiple of the column tile %d", W, C);
  const float2 *tw;
  int rc = twiddles(LOGH, sign, &tw);
  if (rc) return rc;
  const size_t smem = (size_t)((H + H / 32) * C + tw_entries(LOGH)) * sizeof(float2);
  CG_CUDA(cudaFuncSetAttribute(k_fft32_cols<LOGH, C, IO>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t units = nplanes * (W / C);
  const unsigned grid = (unsigned)std::min<int64_t>(units, (int64_t)num_sms() * 2);
  k_fft32_cols<LOGH, C, IO><<<grid, C * T, smem, st>>>(io, nplanes, W, tw, sign, max_out);
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
  if (H == W && H >= f32::TRANSPOSE_MIN && batch <= 65535) {
    // long columns: transpose, transform rows, transpose back (all coalesced)
    if ((rc = f32::launch_transpose(data, batch, H, f32::TpPlain{}, nullptr, st))) return rc;
    f32::RowIO r2{data, W, H, 0, 0, 0, 1.f};
    if ((rc = f32::dispatch_rows(lw, r2, batch * H, sign, st))) return rc;
    if (centred)
      return f32::launch_transpose(data, batch, H, f32::TpCentred{phase & 1, (float)scale},
                                   nullptr, st);
    return f32::launch_transpose(data, batch, H, f32::TpPlain{}, nullptr, st);
  }
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
  if (H == W && H >= f32::TRANSPOSE_MIN) {
    float2 *g = (float2 *)grid_premod;
    if ((rc = f32::launch_transpose(g, 1, H, f32::TpPlain{}, nullptr, st))) return rc;
    if ((rc = f32::dispatch_rows(lw, rio, H, 1, st))) return rc;
    return f32::launch_transpose(g, 1, H, f32::TpImage{image, (H / 2 + W / 2) & 1,
                                                       (float)(1.0 / ((double)H * W))},
                                 max_out, st);
  }
  f32::ColImageIO io{grid_premod, image, W, H, (H / 2 + W / 2) & 1,
                     (float)(1.0 / ((double)H * W))};
  return f32::dispatch_cols(lh, io, 1, W, 1, max_out, st);
}

}  // namespace cg
