// w-towers: w-stacking on sub-grids (examples/grid/grid.c:482-710,
// examples/notebooks/wtowers.ipynb code cell 16), batched over every sub-grid.
//
// Visibilities fall into uv chunks of C = subgrid - margin cells and w-planes
// of width wincrement:
//   ub = floor(u*theta / C), vb = floor(v*theta / C), wp = rint(w / wincrement)
// A chunk's sub-grid (s x s cells) is centred on xmid = (C*ub + C*(ub+1)) // 2
// cells from the grid centre (likewise ymid).  Each (chunk, plane) pair with
// visibilities becomes one layer of a stack of sub-grids, gridded in one
// launch (a layered plan on the chunk-relative coordinates with the residual-w
// kernels), inverse-transformed by one batched FFT; this file then forms, per
// chunk, image = sum over its planes of layer / w_kernel_function(l, m,
// wp*wincrement) (the Fresnel transfer between planes in closed form), and,
// after a batched forward FFT, adds each chunk's sub-grid into the grid.
//
// The chunk and plane of a visibility and its chunk-relative coordinates are
// IEEE double operations in the same order as the numpy restatement, so the
// binning is bit-identical to it.
#include <algorithm>

#include "cg_internal.cuh"

namespace cg {

__device__ __forceinline__ int64_t floor_div_ll(int64_t a, int64_t b) {
  int64_t q, r;
  q = a / b;
  r = a - q * b;
  if (r != 0 && ((r < 0) != (b < 0))) --q;
  return q;
}

// floor(t / C) as numpy evaluates it (IEEE quotient, then floor), filtered as
// in w_bin_fast: F = round(t * (1/C) * 2^20) from one FMA decides unless the
// quotient lies within FIX_MARGIN units of an integer, where the exact
// quotient is formed.  |t / C| < 2^30 on the fast path.
__device__ __forceinline__ double floor_div_fast(double t, double C, double invC) {
  const double e = fma(t, invC, FIX_MAGIC);
  const long long F = (long long)((unsigned long long)__double_as_longlong(e) - FIX_MAGIC_BITS);
  if (F > -(1ll << 50) && F < (1ll << 50)) {
    const long long fr = F & (FIX_ONE - 1);
    if (fr > FIX_MARGIN && fr < FIX_ONE - FIX_MARGIN) return (double)(F >> FIX_BITS);
  }
  return floor(__ddiv_rn(t, C));
}

// Pass 1: bins (ub, vb, wp) of every visibility, their ranges, and the bins
// stored as three int32 at the start of the visibility's rel row (pass 2
// reads them back before overwriting the row).
__global__ void k_tower_bounds(const double *__restrict__ uvw, int64_t stride, int64_t n,
                               double theta, int C, double invC, double winc, double inv_winc,
                               int32_t *mm, double *__restrict__ rel, int32_t *status) {
  int mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  int bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double *row = uvw + i * stride;
    const double fu = floor_div_fast(__dmul_rn(row[0], theta), (double)C, invC);
    const double fv = floor_div_fast(__dmul_rn(row[1], theta), (double)C, invC);
    const double fw = w_bin_fast(row[2], winc, inv_winc);
    int32_t *bins = (int32_t *)(rel + 3 * i);
    if (!(fabs(fu) < 1e9 && fabs(fv) < 1e9 && fabs(fw) < 1e9)) {  // NaN too
      ++bad;
      bins[0] = bins[1] = bins[2] = INT32_MIN;
      continue;
    }
    const int b[3] = {(int)fu, (int)fv, (int)fw};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      bins[d] = b[d];
      mn[d] = min(mn[d], b[d]);
      mx[d] = max(mx[d], b[d]);
    }
  }
  if (bad) atomicAdd(&status[ST_RANGE], bad);
#pragma unroll
  for (int d = 0; d < 3; ++d) block_atomic_min_max(&mm[2 * d], &mm[2 * d + 1], mn[d], mx[d]);
}

__global__ void k_tower_mm_init(int32_t *mm) {
  if (threadIdx.x < 6) mm[threadIdx.x] = (threadIdx.x & 1) ? INT32_MIN : INT32_MAX;
}

// Pass 2: key = ((vb - vbmin) * nub + (ub - ubmin)) * nwp + (wp - wpmin) (sorted
// keys group a chunk's planes together, in increasing w) and the coordinates
// relative to the chunk centre xmid / theta (IEEE quotient, as numpy) and the
// plane wp * wincrement.
constexpr int TOWER_MID_TABLE = 1024;  // chunk columns / rows whose centres a block tabulates

__device__ __forceinline__ double tower_mid_over_theta(int b, int C, double theta) {
  const int64_t mid = floor_div_ll((int64_t)C * b + (int64_t)C * (b + 1), 2);
  return __ddiv_rn((double)mid, theta);
}

__global__ void k_tower_keys(const double *__restrict__ uvw, int64_t stride, int64_t n,
                             double theta, int C, double winc, int ubmin, int vbmin, int wpmin,
                             int nub, int nvb, int nwp, int32_t *__restrict__ key,
                             double *__restrict__ rel) {
  // xmid / theta of every chunk column and row, once per block instead of two
  // FP64 divisions per visibility (the same IEEE quotients)
  __shared__ double s_mid[2][TOWER_MID_TABLE];
  const bool tu = nub <= TOWER_MID_TABLE, tv = nvb <= TOWER_MID_TABLE;
  for (int t = threadIdx.x; t < TOWER_MID_TABLE; t += blockDim.x) {
    if (tu && t < nub) s_mid[0][t] = tower_mid_over_theta(ubmin + t, C, theta);
    if (tv && t < nvb) s_mid[1][t] = tower_mid_over_theta(vbmin + t, C, theta);
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t *bins = (const int32_t *)(rel + 3 * i);
  const int ub = bins[0], vb = bins[1], wp = bins[2];
  const double *row = uvw + i * stride;
  if (ub == INT32_MIN) {  // counted as a range error by pass 1
    key[i] = 0;
    rel[3 * i] = rel[3 * i + 1] = rel[3 * i + 2] = 0.0;
    return;
  }
  const double mu = tu ? s_mid[0][ub - ubmin] : tower_mid_over_theta(ub, C, theta);
  const double mv = tv ? s_mid[1][vb - vbmin] : tower_mid_over_theta(vb, C, theta);
  const double ru = __dadd_rn(row[0], -mu);
  const double rv = __dadd_rn(row[1], -mv);
  const double rw = __dadd_rn(row[2], -__dmul_rn((double)wp, winc));
  key[i] = (int32_t)(((vb - vbmin) * nub + (ub - ubmin)) * nwp + (wp - wpmin));
  rel[3 * i] = ru;
  rel[3 * i + 1] = rv;
  rel[3 * i + 2] = rw;
}

// out[c] = sum over the layers L of chunk c of image_L / exp(2 pi i w_L ph),
// ph = 1 - sqrt(1 - l^2 - m^2) on the sub-grid's l, m = theta * coordinates2(S).
// The layers arrive as unshifted, unnormalised inverse transforms F_L of the
// sub-grids, and the centred image is image_L[k] = (-1)^(kx+ky) F_L[k + S/2] /
// S^2 (indices mod S, S even); out is written rolled by S/2 (ifftshift), so an
// unshifted forward transform of it is the centred fft up to the final roll,
// which cg_towers_add applies.  The turns w_L * ph are a double-float product
// reduced to a fraction of a turn before the FP32 sincospi.
static constexpr int TOWER_CHUNKS_PER_BLOCK = 8;  // chunks sharing one cell's FP64 phase
static constexpr int TOWER_SMEM_LAYERS = 2048;    // layers whose w split a block caches

// w as an FP32 hi + lo pair (hi = w rounded, lo = the rest)
__device__ __forceinline__ float2 split_w(double w) {
  const float hi = (float)w;
  return make_float2(hi, (float)(w - (double)hi));
}

// The four mirror cells (i, j), (S-i, j), (i, S-j), (S-i, S-j) have
// coordinates of equal magnitude, hence the same ph, factors and sign: one
// thread takes all four (those that exist), with one FP64 ph and one
// sincospi per layer, and gives each the value it would get alone.
struct MirrorCells {
  int64_t kr[4];  // rolled index of each cell, -1 where the mirror does not exist
  int i, j;       // the representative, 0 <= i, j <= S/2
  __device__ MirrorCells(int64_t rep, int S) {
    const int half = S / 2, M = half + 1;
    i = (int)(rep / M);
    j = (int)(rep - (int64_t)i * M);
    const int i2 = S - i, j2 = S - j;
    const bool hi = i2 < S && i2 != i, hj = j2 < S && j2 != j;
    auto roll = [&](int x) { return x + half >= S ? x + half - S : x + half; };
    kr[0] = (int64_t)roll(i) * S + roll(j);
    kr[1] = hj ? (int64_t)roll(i) * S + roll(j2) : -1;
    kr[2] = hi ? (int64_t)roll(i2) * S + roll(j) : -1;
    kr[3] = hi && hj ? (int64_t)roll(i2) * S + roll(j2) : -1;
  }
};

__global__ void k_towers_combine(const float2 *__restrict__ stack, int S, double theta,
                                 const double *__restrict__ layer_w,
                                 const int32_t *__restrict__ chunk_first, int nchunks,
                                 float2 *__restrict__ out, int32_t *status) {
  extern __shared__ float2 s_w[];  // the block's layers' w, split once (FP64 is slow here)
  const int c0 = blockIdx.y * TOWER_CHUNKS_PER_BLOCK;
  const int c1 = min(nchunks, c0 + TOWER_CHUNKS_PER_BLOCK);
  const int Lb0 = chunk_first[c0], Lb1 = chunk_first[c1];
  const bool cached = Lb1 - Lb0 <= TOWER_SMEM_LAYERS;
  if (cached)
    for (int L = Lb0 + (int)threadIdx.x; L < Lb1; L += blockDim.x) s_w[L - Lb0] = split_w(layer_w[L]);
  __syncthreads();
  const int64_t cells = (int64_t)S * S;
  const int half = S / 2;
  const int64_t reps = (int64_t)(half + 1) * (half + 1);
  const float scale = 1.0f / (float)cells;
  int bad = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < reps;
       k += (int64_t)gridDim.x * blockDim.x) {
    const MirrorCells mc(k, S);
    // the cells' phase, once for every chunk of the block (FP64 is slow here)
    const double l = __dmul_rn(theta, centred_coord(mc.j, half, S));
    const double m = __dmul_rn(theta, centred_coord(mc.i, half, S));
    const double r2 = __dadd_rn(__dmul_rn(l, l), __dmul_rn(m, m));
    if (!(r2 < 1.0)) bad = 1;
    const double ph = 1.0 - sqrt(1.0 - r2);
    const float ph_h = (float)ph, ph_l = (float)(ph - (double)ph_h);
    const float sg = ((mc.i + mc.j) & 1) ? -scale : scale;  // S even: mirrors alike
    for (int c = c0; c < c1; ++c) {
      const int L0 = chunk_first[c], L1 = chunk_first[c + 1];
      float ax[4] = {0.f, 0.f, 0.f, 0.f}, ay[4] = {0.f, 0.f, 0.f, 0.f};
      for (int L = L0; L < L1; L += 2) {
        float2 g[2][4], w2[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {  // two layers' loads of four cells in flight
          const bool in = L + q < L1;
          const float2 *layer = stack + (int64_t)(L + q) * cells;
#pragma unroll
          for (int e = 0; e < 4; ++e)
            g[q][e] = in && mc.kr[e] >= 0 ? layer[mc.kr[e]] : make_float2(0.f, 0.f);
          w2[q] = !in ? make_float2(0.f, 0.f) : cached ? s_w[L + q - Lb0] : split_w(layer_w[L + q]);
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float wh = w2[q].x, wl = w2[q].y;
          const float hi = wh * ph_h;
          const float lo = fmaf(wh, ph_h, -hi) + fmaf(wh, ph_l, wl * ph_h);
          const float f = (hi - rintf(hi)) + lo;
          float sn, cs;
          sincospif(2.0f * f, &sn, &cs);
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            ax[e] += g[q][e].x * cs + g[q][e].y * sn;
            ay[e] += g[q][e].y * cs - g[q][e].x * sn;
          }
        }
      }
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (mc.kr[e] >= 0) out[(int64_t)c * cells + mc.kr[e]] = make_float2(ax[e] * sg, ay[e] * sg);
    }
  }
  if (bad && status) atomicAdd(&status[ST_RANGE], 1);
}

// grid[y0 + i, x0 + j] += sub[c, i, j] inside the grid, where sub is the
// centred transform: the unshifted forward transform G of the rolled image
// read at the rolled index, sub[i, j] = G[i + S/2, j + S/2] (indices mod S).
// Sub-grids overlap by the margin, hence the atomics.
__global__ void k_towers_add(const float2 *__restrict__ sub, int S, const int32_t *__restrict__ origin,
                             int N, float2 *__restrict__ grid) {
  const int c = blockIdx.y;
  const int x0 = origin[2 * c], y0 = origin[2 * c + 1];
  const int64_t cells = (int64_t)S * S;
  const int half = S / 2;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cells;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / S), j = (int)(k - (int64_t)i * S);
    const int y = y0 + i, x = x0 + j;
    if (y < 0 || y >= N || x < 0 || x >= N) continue;
    const int ir = i + half >= S ? i + half - S : i + half;
    const int jr = j + half >= S ? j + half - S : j + half;
    const float2 v = sub[(int64_t)c * cells + (int64_t)ir * S + jr];
    if (v.x != 0.f || v.y != 0.f) atomicAdd(&grid[(int64_t)y * N + x], v);
  }
}

// Predict, the reverse pass.  cut: out[c, roll(k)] = grid[origin_c + k] (zeros
// outside the grid), roll(k) = (k + S/2) mod S per axis: the ifftshift, so an
// unshifted inverse transform Y of it gives the centred image Y[roll(k)] / S^2.
__global__ void k_towers_cut(const float2 *__restrict__ grid, int N,
                             const int32_t *__restrict__ origin, int S,
                             float2 *__restrict__ out) {
  const int c = blockIdx.y;
  const int x0 = origin[2 * c], y0 = origin[2 * c + 1];
  const int64_t cells = (int64_t)S * S;
  const int half = S / 2;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cells;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / S), j = (int)(k - (int64_t)i * S);
    const int y = y0 + i, x = x0 + j;
    const int ir = i + half >= S ? i + half - S : i + half;
    const int jr = j + half >= S ? j + half - S : j + half;
    out[(int64_t)c * cells + (int64_t)ir * S + jr] =
        (y >= 0 && y < N && x >= 0 && x < N) ? grid[(int64_t)y * N + x] : make_float2(0.f, 0.f);
  }
}

// expand: layer L (chunk c, plane w_L) = image_c / exp(2 pi i w_L ph), written
// at the rolled index times (-1)^(kx+ky), so that an unshifted forward
// transform of it is the centred sub-grid in natural order; image_c[k] =
// Y_c[roll(k)] / S^2.  Rolls are involutions for even S, so each thread reads
// and writes index n = roll(k).
__global__ void k_towers_expand(const float2 *__restrict__ images, int S, double theta,
                                const double *__restrict__ layer_w,
                                const int32_t *__restrict__ chunk_first, int nchunks,
                                float2 *__restrict__ out, int32_t *status) {
  extern __shared__ float2 s_w[];
  const int c0 = blockIdx.y * TOWER_CHUNKS_PER_BLOCK;
  const int c1 = min(nchunks, c0 + TOWER_CHUNKS_PER_BLOCK);
  const int Lb0 = chunk_first[c0], Lb1 = chunk_first[c1];
  const bool cached = Lb1 - Lb0 <= TOWER_SMEM_LAYERS;
  if (cached)
    for (int L = Lb0 + (int)threadIdx.x; L < Lb1; L += blockDim.x) s_w[L - Lb0] = split_w(layer_w[L]);
  __syncthreads();
  const int64_t cells = (int64_t)S * S;
  const int half = S / 2;
  const int64_t reps = (int64_t)(half + 1) * (half + 1);
  const float scale = 1.0f / (float)cells;
  int bad = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < reps;
       k += (int64_t)gridDim.x * blockDim.x) {
    const MirrorCells mc(k, S);
    const double l = __dmul_rn(theta, centred_coord(mc.j, half, S));
    const double m = __dmul_rn(theta, centred_coord(mc.i, half, S));
    const double r2 = __dadd_rn(__dmul_rn(l, l), __dmul_rn(m, m));
    if (!(r2 < 1.0)) bad = 1;
    const double ph = 1.0 - sqrt(1.0 - r2);
    const float ph_h = (float)ph, ph_l = (float)(ph - (double)ph_h);
    const float sg = ((mc.i + mc.j) & 1) ? -scale : scale;  // S even: mirrors alike
    for (int c = c0; c < c1; ++c) {
      float2 a[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        a[e] = mc.kr[e] >= 0 ? images[(int64_t)c * cells + mc.kr[e]] : make_float2(0.f, 0.f);
        a[e].x *= sg;
        a[e].y *= sg;
      }
      for (int L = chunk_first[c]; L < chunk_first[c + 1]; ++L) {
        const float2 w2 = cached ? s_w[L - Lb0] : split_w(layer_w[L]);
        const float hi = w2.x * ph_h;
        const float lo = fmaf(w2.x, ph_h, -hi) + fmaf(w2.x, ph_l, w2.y * ph_h);
        const float f = (hi - rintf(hi)) + lo;
        float sn, cs;
        sincospif(2.0f * f, &sn, &cs);
        float2 *layer = out + (int64_t)L * cells;
        // a / (cs + i sn) = a * (cs - i sn)
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (mc.kr[e] >= 0)
            layer[mc.kr[e]] = make_float2(a[e].x * cs + a[e].y * sn, a[e].y * cs - a[e].x * sn);
      }
    }
  }
  if (bad && status) atomicAdd(&status[ST_RANGE], 1);
}

}  // namespace cg

using namespace cg;

extern "C" {

int cg_tower_keys(const double *uvw, int64_t stride, int64_t n, double theta, int chunk,
                  double wincrement, int32_t *key_out, double *rel_out, int32_t *d_minmax,
                  int32_t *h_bounds, int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(n >= 1 && uvw && stride >= 3 && key_out && rel_out && d_minmax && h_bounds &&
                 d_status,
             "bad tower key arguments");
  CG_REQUIRE(chunk >= 1 && theta > 0.0 && wincrement > 0.0, "bad chunk, theta or wincrement");
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_tower_mm_init<<<1, 32, 0, s>>>(d_minmax);
  k_tower_bounds<<<stride_blocks(n, 256), 256, 0, s>>>(uvw, stride, n, theta, chunk,
                                                      1.0 / (double)chunk,
                                        wincrement, 1.0 / wincrement, d_minmax, rel_out,
                                        d_status);
  CG_LAUNCH("tower bounds");
  CG_CUDA(cudaMemcpyAsync(h_bounds, d_minmax, 6 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  if (h_bounds[0] > h_bounds[1]) return CG_OK;  // every coordinate out of range
  const int64_t nub = (int64_t)h_bounds[1] - h_bounds[0] + 1;
  const int64_t nvb = (int64_t)h_bounds[3] - h_bounds[2] + 1;
  const int64_t nwp = (int64_t)h_bounds[5] - h_bounds[4] + 1;
  CG_REQUIRE(nub * nvb * nwp < ((int64_t)1 << 31), "too many (chunk, plane) keys");
  k_tower_keys<<<blocks, 256, 0, s>>>(uvw, stride, n, theta, chunk, wincrement, h_bounds[0],
                                      h_bounds[2], h_bounds[4], (int)nub, (int)nvb, (int)nwp,
                                      key_out, rel_out);
  CG_LAUNCH("tower keys");
  return CG_OK;
}

int cg_towers_combine(const void *stack_c64, int layers, int S, double theta,
                      const double *layer_w, const int32_t *chunk_first, int nchunks,
                      void *out_c64, int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(stack_c64 && layer_w && chunk_first && out_c64 && layers >= 1 && S >= 2 &&
                 S % 2 == 0 && nchunks >= 1,
             "bad w-towers combine arguments (even sub-grid size)");
  const int64_t reps = (int64_t)(S / 2 + 1) * (S / 2 + 1);  // mirror-cell sets
  const unsigned bx = (unsigned)std::min<int64_t>((reps + 255) / 256, 1024);
  const unsigned by = (unsigned)((nchunks + TOWER_CHUNKS_PER_BLOCK - 1) / TOWER_CHUNKS_PER_BLOCK);
  k_towers_combine<<<dim3(bx, by), 256, TOWER_SMEM_LAYERS * sizeof(float2),
                     (cudaStream_t)stream>>>(
      (const float2 *)stack_c64, S, theta, layer_w, chunk_first, nchunks, (float2 *)out_c64,
      d_status);
  CG_LAUNCH("w-towers combine");
  return CG_OK;
}

int cg_towers_add(const void *sub_c64, int nchunks, int S, const int32_t *origin, int N,
                  void *grid_c64, cg_stream_t stream) {
  CG_REQUIRE(sub_c64 && origin && grid_c64 && S >= 2 && S % 2 == 0 && N >= 1 &&
                 nchunks >= 1 && nchunks <= 65535,
             "bad w-towers add arguments (even sub-grid size)");
  const int64_t cells = (int64_t)S * S;
  const unsigned bx = (unsigned)std::min<int64_t>((cells + 255) / 256, 64);
  k_towers_add<<<dim3(bx, nchunks), 256, 0, (cudaStream_t)stream>>>(
      (const float2 *)sub_c64, S, origin, N, (float2 *)grid_c64);
  CG_LAUNCH("w-towers add");
  return CG_OK;
}

int cg_towers_cut(const void *grid_c64, int N, const int32_t *origin, int nchunks, int S,
                  void *out_c64, cg_stream_t stream) {
  CG_REQUIRE(grid_c64 && origin && out_c64 && N >= 1 && S >= 2 && S % 2 == 0 && nchunks >= 1 &&
                 nchunks <= 65535,
             "bad w-towers cut arguments (even sub-grid size)");
  const int64_t cells = (int64_t)S * S;
  const unsigned bx = (unsigned)std::min<int64_t>((cells + 255) / 256, 64);
  k_towers_cut<<<dim3(bx, nchunks), 256, 0, (cudaStream_t)stream>>>(
      (const float2 *)grid_c64, N, origin, S, (float2 *)out_c64);
  CG_LAUNCH("w-towers cut");
  return CG_OK;
}

int cg_towers_expand(const void *images_c64, int S, double theta, const double *layer_w,
                     const int32_t *chunk_first, int nchunks, void *out_c64, int32_t *d_status,
                     cg_stream_t stream) {
  CG_REQUIRE(images_c64 && layer_w && chunk_first && out_c64 && S >= 2 && S % 2 == 0 &&
                 nchunks >= 1,
             "bad w-towers expand arguments (even sub-grid size)");
  const int64_t reps = (int64_t)(S / 2 + 1) * (S / 2 + 1);  // mirror-cell sets
  const unsigned bx = (unsigned)std::min<int64_t>((reps + 255) / 256, 1024);
  const unsigned by = (unsigned)((nchunks + TOWER_CHUNKS_PER_BLOCK - 1) / TOWER_CHUNKS_PER_BLOCK);
  k_towers_expand<<<dim3(bx, by), 256, TOWER_SMEM_LAYERS * sizeof(float2),
                    (cudaStream_t)stream>>>((const float2 *)images_c64, S, theta, layer_w,
                                            chunk_first, nchunks, (float2 *)out_c64, d_status);
  CG_LAUNCH("w-towers expand");
  return CG_OK;
}

}  // extern "C"
