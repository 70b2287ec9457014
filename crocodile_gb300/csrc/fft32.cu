// Hand-written FP32 FFTs of power-of-two complex64 planes: the centred
// fft / ifft of crocodile/synthesis.py:83-106 (fftshift(fft2(ifftshift(a))),
// 1 / (H W) on the inverse), the unshifted transform of the sub-grid stacks,
// and the dirty image of do_imaging (real part of the centred ifft, :903-906),
// for sides 64 .. 8192.
//
// Passes over HBM per plane:
//   rows:    N / 16 threads per row, whole rows per CTA, in place;
//   columns up to 1024: up to 512 threads per CTA transform a tile of C
//            adjacent columns (C x 8 bytes of every row, H x C <= 8192
//            elements), in place;
//   columns from 2048: two four-step passes over tiles of 32 columns
//            (H = H1 x H2, lines of H1 then H2 elements), the second out of
//            place (through a scratch stack, or into the dirty image); each
//            unit's 32 x H1 (or H2) input tile arrives by one tiled tensor
//            copy (TMA), double-buffered against the previous unit's stages.
// Each line runs the register-blocked Stockham stages of fft32.h (radix 16,
// 16 values per thread): the first stage reads global memory and the last
// writes it, coalesced; the stages between exchange through one padded
// shared-memory buffer (every thread reads, barrier, every thread writes).  The
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
#include "mbar.cuh"

#include <cudaTypedefs.h>

namespace cg {
namespace f32 {

constexpr int MIN_LOG = 6, MAX_LOG = 13;
constexpr int COL_THREADS = 512;
// columns from this length on run as the four-step passes (lines of
// H1 >= 64 and H2 >= 32 elements; at 1024 the column tiles are faster:
// 0.032 against 0.039 ms for a 1024^2 plane, at 2048 the four-step passes:
// 0.064 against 0.066 ms)
constexpr int STEP_MIN = 2048;

__device__ __forceinline__ int pad(int e) { return e + (e >> 5); }  // bank spread

// Twiddles: the per-stage tables of fft32.h (tw_table_fill / tw_lookup),
// correctly rounded entries computed in double on the host, staged in
// shared memory by every CTA (1312 entries for N = 8192).  Cached per
// device, log N and sign.
constexpr int tw_entries(int logn) { return tw_table_entries(logn) + 1; }
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
  std::vector<cf> h(tw_entries(logn));
  tw_table_fill(logn, [&](long long j) {
    const double a = 2.0 * M_PI * (double)j / (double)n;
    return cf{(float)std::cos(a), (float)(sign * std::sin(a))};
  }, h.data());
  float2 *d = nullptr;
  CG_CUDA(cudaMalloc(&d, h.size() * sizeof(float2)));
  CG_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice));
  g_tw[key] = d;
  *out = d;
  return CG_OK;
}

// the table in shared memory
template <int LOGN>
struct SmTw {
  const float2 *t;
  __device__ cf operator()(int s, int r, int k) const {
    return tw_lookup(LOGN, s, r, k, [this](int i) {
      const float2 v = t[i];
      return cf{v.x, v.y};
    });
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
  __device__ const float2 *src(int64_t row) const { return d + row * W; }
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
// Rows: T = N / 16 threads per row, TPC = max(T, 256) threads and TPC / T
// rows per CTA at a time (small CTAs: each barrier holds fewer warps); the
// first stage loads global memory straight into registers and the last
// stage writes it from registers.  (Copying the next row into a
// second shared buffer by cp.async while a row is transformed, at the cost
// of half the CTAs per SM, measured slower: 0.088 against 0.078 ms for the
// rows of a 4096^2 plane, 0.350 against 0.300 ms at 8192^2.)
template <int LOGN>
struct RowShape {
  static constexpr int N = 1 << LOGN, T = N / 16;
  static constexpr int TPC = T > 256 ? T : 256, LPC = TPC / T, MINB = 1024 / TPC;
  static constexpr int P = N + N / 32;  // padded row
};

template <int LOGN>
__global__ void __launch_bounds__(RowShape<LOGN>::TPC, RowShape<LOGN>::MINB)
    k_fft32_rows(RowIO io, int64_t nrows, const float2 *__restrict__ tw, int sign) {
  using RS = RowShape<LOGN>;
  constexpr int T = RS::T, LPC = RS::LPC, P = RS::P;
  constexpr int NS = (LOGN + 3) / 4;
  extern __shared__ float2 f32_sm[];
  const int line = threadIdx.x / T, t = threadIdx.x % T;
  float2 *buf = f32_sm + line * P;
  float2 *stw = f32_sm + LPC * P;
  for (int k = threadIdx.x; k < tw_entries(LOGN); k += RS::TPC) stw[k] = tw[k];
  __syncthreads();
  const SmTw<LOGN> twf{stw};
  // a row of N <= 512 is one warp's (T <= 32 threads): warp barriers suffice
  auto sync = [] {
    if (T <= 32) __syncwarp(); else __syncthreads();
  };
  auto lds = [&](int e) {
    const float2 x = buf[pad(e)];
    return cf{x.x, x.y};
  };
  auto sts = [&](int e, cf x) { buf[pad(e)] = make_float2(x.x, x.y); };
  for (int64_t row0 = (int64_t)blockIdx.x * LPC; row0 < nrows; row0 += (int64_t)gridDim.x * LPC) {
    const int64_t row = row0 + line;
    const bool live = row < nrows;
    const int rpar = io.modulate ? (int)(row % io.H) & 1 : 0;
    const float2 *src = io.src(row);
    cf v[16];
    stage_load(LOGN, 0, t, [&](int e) {
      if (!live) return cf{0.f, 0.f};
      const float2 x = src[e];
      return (io.modulate && ((rpar + e) & 1)) ? cf{-x.x, -x.y} : cf{x.x, x.y};
    }, twf, v);
    stage_dft(LOGN, 0, sign, v);
    stage_store(LOGN, 0, t, sts, v);
#pragma unroll
    for (int s = 1; s < NS; ++s) {
      sync();  // previous stores visible
      stage_load(LOGN, s, t, lds, twf, v);
      sync();  // all reads before any write
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
  const SmTw<LOGH> twf{stw};
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

// ---------------------------------------------------------------- four-step columns
// Columns of length H = H1 x H2 (H1, H2 >= 64) in two passes over tiles of
// 32 adjacent columns (256 contiguous bytes of every row touched), with
// n = n1 H2 + n2 and k = k1 + H1 k2:
//   A: for each n2, Y[k1, n2] = w_H^(n2 k1) sum_n1 x[n1 H2 + n2] w_H1^(n1 k1),
//      stored at row k1 H2 + n2 (the rows it read: A may run in place);
//   B: for each k1, X[k1 + H1 k2] = sum_n2 Y[k1, n2] w_H2^(n2 k2), reading the
//      block of rows k1 H2 .. k1 H2 + H2 - 1 and writing row k1 + H1 k2 (out
//      of place: the rows it writes belong to other blocks).
// A unit is (plane, n2 or k1, tile), the tile fastest, so neighbouring CTAs
// touch neighbouring 256-byte segments of the same rows.  The twiddles of A
// come from a full table of w_H^j in global memory (the 32 lanes of a warp
// share k1: one broadcast load).
struct StepShape {
  int W, H1, H2, tiles;  // tiles = W / 32
  int nj;                // units per plane and tile: H2 (pass A) or H1 (pass B)
  int64_t plane;         // elements per plane
  __device__ void unit(int64_t u, int64_t &pl, int &j, int &col0) const {
    const int64_t per = (int64_t)tiles * nj;
    pl = u / per;
    const int64_t r = u - pl * per;
    j = (int)(r / tiles);
    col0 = (int)(r - (int64_t)j * tiles) * 32;
  }
};

// Per unit and column: ctx(u, c) gives the input column (element i at
// src[i * stride]) and what the store needs; st(x, i, v, mx) stores output i.
struct StepCtx {
  const float2 *src;
  int64_t stride;
  float2 *dst;   // complex output column (pass A, B)
  float *fdst;   // image column (pass B of the dirty image)
  int j, col;
};

struct StepA {
  StepShape sh;
  const float2 *in;
  float2 *out;
  const float2 *twH;  // w_H^j, j < H
  __device__ StepCtx ctx(int64_t u, int c) const {
    int64_t pl;
    int j, col0;
    sh.unit(u, pl, j, col0);
    const int64_t base = pl * sh.plane + (int64_t)j * sh.W + col0 + c;
    return StepCtx{in + base, (int64_t)sh.H2 * sh.W, out + base, nullptr, j, col0 + c};
  }
  __device__ void st(const StepCtx &x, int k1, cf v, float &) const {
    const float2 w = twH[x.j * k1];
    x.dst[(int64_t)k1 * x.stride] = make_float2(fmaf(v.x, w.x, -v.y * w.y),
                                                fmaf(v.x, w.y, v.y * w.x));
  }
  static constexpr bool kMax = false;
};

// B into complex planes: times scale, and (-1)^(row + col + phase) if centred
struct StepB {
  StepShape sh;
  const float2 *in;
  float2 *out;
  int centred, phase;
  float scale;
  __device__ StepCtx ctx(int64_t u, int c) const {
    int64_t pl;
    int j, col0;
    sh.unit(u, pl, j, col0);
    const int64_t pb = pl * sh.plane + col0 + c;
    return StepCtx{in + pb + (int64_t)j * sh.H2 * sh.W, sh.W, out + pb + (int64_t)j * sh.W,
                   nullptr, j, col0 + c};
  }
  __device__ void st(const StepCtx &x, int k2, cf v, float &) const {
    float s = scale;
    if (centred && ((x.j + sh.H1 * k2 + x.col + phase) & 1)) s = -s;
    x.dst[(int64_t)k2 * sh.H1 * sh.W] = make_float2(v.x * s, v.y * s);
  }
  static constexpr bool kMax = false;
};

// B of the dirty image: the real part, demodulated and scaled, and its maximum
struct StepBImage {
  StepShape sh;
  const float2 *in;
  float *img;
  int phase;
  float scale;
  __device__ StepCtx ctx(int64_t u, int c) const {
    int64_t pl;
    int j, col0;
    sh.unit(u, pl, j, col0);
    const int col = col0 + c;
    return StepCtx{in + (int64_t)j * sh.H2 * sh.W + col, sh.W, nullptr,
                   img + (int64_t)j * sh.W + col, j, col};
  }
  __device__ void st(const StepCtx &x, int k2, cf v, float &mx) const {
    const float r = v.x * (((x.j + sh.H1 * k2 + x.col + phase) & 1) ? -scale : scale);
    x.fdst[(int64_t)k2 * sh.H1 * sh.W] = r;
    mx = fmaxf(mx, r);
  }
  static constexpr bool kMax = true;
};

// One pass of the four-step columns: lines of L = 2^LOGL, 32 columns per
// tile, T = L / 16 threads per column (thread (t, c), c fastest).
// CTAs per SM the step kernels are built for (80 registers a thread)
constexpr int step_minb(int logl) { return 768 / (32 << (logl - 4)); }

template <int LOGL, class IO>
__global__ void __launch_bounds__(32 * (1 << (LOGL - 4)), step_minb(LOGL))
    k_fft32_step(IO io, int64_t units, const float2 *__restrict__ tw, int sign,
                 float *max_out) {
  constexpr int L = 1 << LOGL, T = L / 16, C = 32, NS = (LOGL + 3) / 4;
  extern __shared__ float2 f32_sm[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  float2 *stw = f32_sm + (L + L / 32) * C;
  for (int k = threadIdx.x; k < tw_entries(LOGL); k += C * T) stw[k] = tw[k];
  __syncthreads();
  const SmTw<LOGL> twf{stw};
  auto lds = [&](int e) {
    const float2 v = f32_sm[pad(e) * C + c];
    return cf{v.x, v.y};
  };
  auto sts = [&](int e, cf v) { f32_sm[pad(e) * C + c] = make_float2(v.x, v.y); };
  float mx = -FLT_MAX;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const StepCtx x = io.ctx(u, c);
    cf v[16];
    __syncthreads();  // the previous unit's last reads of shared memory are done
    stage_load(LOGL, 0, t, [&](int e) {
      const float2 y = x.src[e * x.stride];
      return cf{y.x, y.y};
    }, twf, v);
    stage_dft(LOGL, 0, sign, v);
    stage_store(LOGL, 0, t, sts, v);
#pragma unroll
    for (int s = 1; s < NS; ++s) {
      __syncthreads();
      stage_load(LOGL, s, t, lds, twf, v);
      __syncthreads();
      stage_dft(LOGL, s, sign, v);
      if (s + 1 < NS)
        stage_store(LOGL, s, t, sts, v);
      else
        stage_store(LOGL, s, t, [&](int e, cf y) { io.st(x, e, y, mx); }, v);
    }
  }
  if (IO::kMax && max_out) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomic_max_f(max_out, mx);
  }
}

// The column passes with their input tiles brought by the tensor-memory
// accelerator: the 32-column x L-row box of a unit is one tiled tensor copy
// (cp.async.bulk.tensor) into shared memory, double-buffered, so that the
// next unit's tile is in flight while this one's stages run; the stages
// work in place in the tile (its rows are 256 contiguous bytes and a warp
// always touches one row: no bank conflicts without padding) and the last
// stage writes global memory as in k_fft32_step.  The tensor map spans the
// planes as (W, H2, H1, planes); pass A's box is (32, 1, H1, 1) at (col0, n2,
// 0, plane), pass B's (32, H2, 1, 1) at (col0, 0, k1, plane).  Every wait is
// bounded by the process-wide wait limit (cg_set_wait_limit; 0 polls once
// without blocking); on expiry the CTA counts the timeout in
// g_fft32_timeouts (cg_fft_timeouts), waits for its copies in flight (at
// most the default limit each) and stops, leaving its units' output undefined.
constexpr long long FFT_WAIT_CYCLES = 4000000000ll;
__device__ int g_fft32_timeouts;

__device__ __forceinline__ bool tile_wait(uint64_t *bar, uint32_t parity, long long cycles) {
  return cycles ? mbar_wait_cycles(bar, parity, cycles) : mbar_test(bar, parity);
}

template <int LOGL>
struct TmaShape {
  static constexpr int L = 1 << LOGL, C = 32, THREADS = C * (L / 16);
  static constexpr size_t tile_bytes() { return (size_t)L * C * sizeof(float2); }
  static constexpr size_t smem() {  // 128 bytes of alignment slack, two tiles, twiddles, bars
    return 128 + 2 * tile_bytes() + (size_t)tw_entries(LOGL) * sizeof(float2) + 16;
  }
};

template <int LOGL, class IO>
__global__ void __launch_bounds__(TmaShape<LOGL>::THREADS, step_minb(LOGL))
    k_fft32_step_tma(const __grid_constant__ CUtensorMap tmap, IO io, int64_t units,
                     int box_a, const float2 *__restrict__ tw, int sign, float *max_out,
                     long long wait) {
  using TS = TmaShape<LOGL>;
  constexpr int L = TS::L, T = L / 16, C = TS::C, NS = (LOGL + 3) / 4;
  extern __shared__ unsigned char f32_tsm[];
  float2 *tiles = (float2 *)(((uintptr_t)f32_tsm + 127) & ~(uintptr_t)127);
  float2 *stw = tiles + 2 * L * C;
  uint64_t *bar = (uint64_t *)(stw + tw_entries(LOGL));
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  for (int k = threadIdx.x; k < tw_entries(LOGL); k += TS::THREADS) stw[k] = tw[k];
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  const SmTw<LOGL> twf{stw};
  auto issue = [&](int64_t u, int b) {  // one thread
    int64_t pl;
    int j, col0;
    io.sh.unit(u, pl, j, col0);
    if (box_a)
      tma_load_4d(tiles + b * L * C, &tmap, col0, j, 0, (int)pl, &bar[b], (uint32_t)TS::tile_bytes());
    else
      tma_load_4d(tiles + b * L * C, &tmap, col0, 0, j, (int)pl, &bar[b], (uint32_t)TS::tile_bytes());
  };
  float mx = -FLT_MAX;
  int64_t u = blockIdx.x;
  if (threadIdx.x == 0 && u < units) issue(u, 0);
  for (int it = 0; u < units; u += gridDim.x, ++it) {
    const int b = it & 1;
    const bool next = u + gridDim.x < units;
    // the other tile's last reads were before the previous unit's last barrier
    if (threadIdx.x == 0 && next) issue(u + gridDim.x, b ^ 1);
    const bool ok = tile_wait(&bar[b], (it >> 1) & 1, wait);
    if (__syncthreads_or(!ok)) {
      // let this tile's copy and the next one's land before the CTA (and its
      // shared memory) goes away
      if (threadIdx.x == 0) {
        atomicAdd(&g_fft32_timeouts, 1);
        mbar_wait_cycles(&bar[b], (it >> 1) & 1, FFT_WAIT_CYCLES);
        if (next) mbar_wait_cycles(&bar[b ^ 1], ((it + 1) >> 1) & 1, FFT_WAIT_CYCLES);
      }
      __syncthreads();
      return;
    }
    float2 *buf = tiles + b * L * C;
    auto lds = [&](int e) {
      const float2 v = buf[e * C + c];
      return cf{v.x, v.y};
    };
    auto sts = [&](int e, cf v) { buf[e * C + c] = make_float2(v.x, v.y); };
    const StepCtx x = io.ctx(u, c);
    cf v[16];
    stage_load(LOGL, 0, t, lds, twf, v);
    __syncthreads();  // all reads before any write
    stage_dft(LOGL, 0, sign, v);
    stage_store(LOGL, 0, t, sts, v);
#pragma unroll
    for (int s = 1; s < NS; ++s) {
      __syncthreads();
      stage_load(LOGL, s, t, lds, twf, v);
      __syncthreads();
      stage_dft(LOGL, s, sign, v);
      if (s + 1 < NS)
        stage_store(LOGL, s, t, sts, v);
      else
        stage_store(LOGL, s, t, [&](int e, cf y) { io.st(x, e, y, mx); }, v);
    }
  }
  if (IO::kMax && max_out) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomic_max_f(max_out, mx);
  }
}

// w_H^j for j < H, correctly rounded, cached per device, log H and sign
std::map<std::tuple<int, int, int>, float2 *> g_twfull;

int twiddles_full(int logn, int sign, const float2 **out) {
  int dev = 0;
  CG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_mu);
  const auto key = std::make_tuple(dev, logn, sign);
  auto it = g_twfull.find(key);
  if (it != g_twfull.end()) {
    *out = it->second;
    return CG_OK;
  }
  const int n = 1 << logn;
  std::vector<float2> h(n);
  for (int j = 0; j < n; ++j) {
    const double a = 2.0 * M_PI * (double)j / (double)n;
    h[j] = make_float2((float)std::cos(a), (float)(sign * std::sin(a)));
  }
  float2 *d = nullptr;
  CG_CUDA(cudaMalloc(&d, h.size() * sizeof(float2)));
  CG_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice));
  g_twfull[key] = d;
  *out = d;
  return CG_OK;
}

template <int LOGL, class IO>
int launch_step_as(const IO &io, int64_t units, int sign, float *max_out, cudaStream_t st) {
  constexpr int L = 1 << LOGL, threads = 32 * (L / 16);
  const float2 *tw;
  int rc = twiddles(LOGL, sign, &tw);
  if (rc) return rc;
  const size_t smem = (size_t)((L + L / 32) * 32 + tw_entries(LOGL)) * sizeof(float2);
  CG_CUDA(cudaFuncSetAttribute(k_fft32_step<LOGL, IO>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft32_step<LOGL, IO>, threads,
                                                        smem));
  CG_REQUIRE(per_sm > 0, "FP32 FFT column step does not fit on an SM (smem %zu)", smem);
  const unsigned grid = (unsigned)std::min<int64_t>(units, (int64_t)num_sms() * per_sm);
  k_fft32_step<LOGL, IO><<<grid, threads, smem, st>>>(io, units, tw, sign, max_out);
  CG_LAUNCH("FP32 FFT column step");
  return CG_OK;
}

// cuTensorMapEncodeTiled from the driver (no link against libcuda)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)p;
  }();
  return fn;
}

// The TMA-fed column pass over `in` (nplanes planes of H1 H2 x W): box_a for
// pass A.  *used = false (and nothing launched) when the tensor map cannot
// describe the input: an unaligned base, an odd width, or no encoder.
template <int LOGL, class IO>
int launch_step_tma_as(const IO &io, const float2 *in, int W, int H1, int H2, int64_t nplanes,
                       bool box_a, int64_t units, int sign, float *max_out, cudaStream_t st,
                       bool *used) {
  using TS = TmaShape<LOGL>;
  *used = false;
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || ((uintptr_t)in & 15) || W % 2 || nplanes < 1 || nplanes > INT32_MAX) return CG_OK;
  if ((box_a ? H1 : H2) != TS::L) return CG_OK;
  CUtensorMap map;
  const cuuint64_t dims[4] = {(cuuint64_t)W, (cuuint64_t)H2, (cuuint64_t)H1, (cuuint64_t)nplanes};
  const cuuint64_t strides[3] = {(cuuint64_t)W * 8, (cuuint64_t)H2 * W * 8,
                                 (cuuint64_t)H1 * H2 * W * 8};
  const cuuint32_t box[4] = {32, box_a ? 1u : (cuuint32_t)H2, box_a ? (cuuint32_t)H1 : 1u, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_INT64, 4, (void *)in, dims, strides, box, es,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return CG_OK;
  const float2 *tw;
  int rc = twiddles(LOGL, sign, &tw);
  if (rc) return rc;
  const size_t smem = TS::smem();
  CG_CUDA(cudaFuncSetAttribute(k_fft32_step_tma<LOGL, IO>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft32_step_tma<LOGL, IO>,
                                                        TS::THREADS, smem));
  if (per_sm < 1) return CG_OK;
  const unsigned grid = (unsigned)std::min<int64_t>(units, (int64_t)num_sms() * per_sm);
  k_fft32_step_tma<LOGL, IO><<<grid, TS::THREADS, smem, st>>>(map, io, units, box_a ? 1 : 0, tw,
                                                              sign, max_out, wait_cycles());
  CG_LAUNCH("FP32 FFT column step (TMA)");
  *used = true;
  return CG_OK;
}

template <class IO>
int launch_step_tma(int logl, const IO &io, const float2 *in, int W, int H1, int H2,
                    int64_t nplanes, bool box_a, int64_t units, int sign, float *max_out,
                    cudaStream_t st, bool *used) {
  switch (logl) {
    case 5:
      return launch_step_tma_as<5>(io, in, W, H1, H2, nplanes, box_a, units, sign, max_out, st,
                                   used);
    case 6:
      return launch_step_tma_as<6>(io, in, W, H1, H2, nplanes, box_a, units, sign, max_out, st,
                                   used);
    case 7:
      return launch_step_tma_as<7>(io, in, W, H1, H2, nplanes, box_a, units, sign, max_out, st,
                                   used);
  }
  *used = false;
  return CG_OK;
}

template <class IO>
int launch_step(int logl, const IO &io, int64_t units, int sign, float *max_out,
                cudaStream_t st) {
  switch (logl) {
    case 5: return launch_step_as<5>(io, units, sign, max_out, st);
    case 6: return launch_step_as<6>(io, units, sign, max_out, st);
    case 7: return launch_step_as<7>(io, units, sign, max_out, st);
  }
  return set_error(CG_ERR_ARG, "FP32 FFT: unsupported column step length 2^%d", logl);
}

// The scratch stacks of pass B come from a memory pool of the library's own
// per device, which keeps what it has mapped (release threshold: unlimited),
// so that repeated transforms neither map nor touch fresh pages; stream
// ordering keeps concurrent transforms on different streams apart.
std::map<int, cudaMemPool_t> g_pools;

int scratch_pool(cudaMemPool_t *out) {
  int dev = 0;
  CG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_pools.find(dev);
  if (it != g_pools.end()) {
    *out = it->second;
    return CG_OK;
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool;
  CG_CUDA(cudaMemPoolCreate(&pool, &props));
  uint64_t keep = ~0ull;
  CG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  g_pools[dev] = pool;
  *out = pool;
  return CG_OK;
}

// lengths of the two passes: H1 = 2^ceil(log H / 2) (A), H2 = H / H1 (B)
void step_split(int logh, int &logh1, int &logh2) {
  logh1 = (logh + 1) / 2;
  logh2 = logh - logh1;
}

__global__ void k_fft32_init_max(float *m) { *m = -FLT_MAX; }

int log2_exact(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return (1 << l) == n ? l : -1;
}

template <int LOGN>
int launch_rows(const RowIO &io, int64_t nrows, int sign, cudaStream_t st) {
  using RS = RowShape<LOGN>;
  const float2 *tw;
  int rc = twiddles(LOGN, sign, &tw);
  if (rc) return rc;
  const size_t smem = (size_t)(RS::LPC * RS::P + tw_entries(LOGN)) * sizeof(float2);
  CG_CUDA(cudaFuncSetAttribute(k_fft32_rows<LOGN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft32_rows<LOGN>, RS::TPC,
                                                        smem));
  CG_REQUIRE(per_sm > 0, "FP32 FFT rows do not fit on an SM (smem %zu)", smem);
  const int64_t ctas = (nrows + RS::LPC - 1) / RS::LPC;
  const unsigned grid = (unsigned)std::min<int64_t>(ctas, (int64_t)num_sms() * per_sm);
  k_fft32_rows<LOGN><<<grid, RS::TPC, smem, st>>>(io, nrows, tw, sign);
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
  if (H >= f32::STEP_MIN && W % 32 == 0) {
    // long columns: the four-step passes A (into a scratch stack of at most
    // 1 GiB, a few planes at a time) and B (back into the planes)
    int l1, l2;
    f32::step_split(lh, l1, l2);
    const int64_t plane = (int64_t)H * W;
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(batch, (1LL << 27) / plane));
    float2 *scratch = nullptr;
    cudaMemPool_t pool;
    if ((rc = f32::scratch_pool(&pool))) return rc;
    CG_CUDA(cudaMallocFromPoolAsync((void **)&scratch, (size_t)(chunk * plane) * sizeof(float2),
                                    pool, st));
    const float2 *twH;
    if ((rc = f32::twiddles_full(lh, sign, &twH))) {
      cudaFreeAsync(scratch, st);
      return rc;
    }
    for (int64_t b0 = 0; b0 < batch && !rc; b0 += chunk) {
      const int64_t nb = std::min(chunk, batch - b0);
      float2 *d = data + b0 * plane;
      f32::StepShape sa{W, 1 << l1, 1 << l2, W / 32, 1 << l2, plane};
      f32::StepA A{sa, d, scratch, twH};
      bool used;
      rc = f32::launch_step_tma(l1, A, d, W, 1 << l1, 1 << l2, nb, true, nb * sa.nj * sa.tiles,
                                sign, nullptr, st, &used);
      if (!rc && !used) rc = f32::launch_step(l1, A, nb * sa.nj * sa.tiles, sign, nullptr, st);
      if (rc) break;
      f32::StepShape sb = sa;
      sb.nj = 1 << l1;
      f32::StepB B{sb, scratch, d, centred ? 1 : 0, phase & 1, (float)scale};
      rc = f32::launch_step_tma(l2, B, scratch, W, 1 << l1, 1 << l2, nb, false,
                                nb * sb.nj * sb.tiles, sign, nullptr, st, &used);
      if (!rc && !used) rc = f32::launch_step(l2, B, nb * sb.nj * sb.tiles, sign, nullptr, st);
    }
    const cudaError_t fe = cudaFreeAsync(scratch, st);
    if (rc) return rc;
    CG_CUDA(fe);
    return CG_OK;
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
  if (H >= f32::STEP_MIN && W % 32 == 0) {
    // four-step columns: A in place on the grid, B into the image
    int l1, l2;
    f32::step_split(lh, l1, l2);
    const float2 *twH;
    if ((rc = f32::twiddles_full(lh, 1, &twH))) return rc;
    float2 *g = (float2 *)grid_premod;
    f32::StepShape sa{W, 1 << l1, 1 << l2, W / 32, 1 << l2, (int64_t)H * W};
    f32::StepA A{sa, g, g, twH};
    bool used;
    if ((rc = f32::launch_step_tma(l1, A, g, W, 1 << l1, 1 << l2, 1, true,
                                   (int64_t)sa.nj * sa.tiles, 1, nullptr, st, &used)))
      return rc;
    if (!used && (rc = f32::launch_step(l1, A, (int64_t)sa.nj * sa.tiles, 1, nullptr, st)))
      return rc;
    f32::StepShape sb = sa;
    sb.nj = 1 << l1;
    f32::StepBImage B{sb, g, image, (H / 2 + W / 2) & 1, (float)(1.0 / ((double)H * W))};
    if ((rc = f32::launch_step_tma(l2, B, g, W, 1 << l1, 1 << l2, 1, false,
                                   (int64_t)sb.nj * sb.tiles, 1, max_out, st, &used)))
      return rc;
    if (used) return CG_OK;
    return f32::launch_step(l2, B, (int64_t)sb.nj * sb.tiles, 1, max_out, st);
  }
  f32::ColImageIO io{grid_premod, image, W, H, (H / 2 + W / 2) & 1,
                     (float)(1.0 / ((double)H * W))};
  return f32::dispatch_cols(lh, io, 1, W, 1, max_out, st);
}

}  // namespace cg

extern "C" int cg_fft_timeouts(int32_t *count, int reset) {
  CG_REQUIRE(count, "NULL argument");
  int v = 0;
  CG_CUDA(cudaMemcpyFromSymbol(&v, cg::f32::g_fft32_timeouts, sizeof(int)));
  *count = v;
  if (reset) {
    const int zero = 0;
    CG_CUDA(cudaMemcpyToSymbol(cg::f32::g_fft32_timeouts, &zero, sizeof(int)));
  }
  return CG_OK;
}
