// w-stacking (K9): the per-plane loop of examples/notebooks/wstacking.ipynb
// (code cell 10) with convolutional gridding, batched over all planes.
//
//   for each w-plane p with visibilities:
//       midw = mean(w of the plane's visibilities)
//       image += ifft(grid_p) / w_kernel_function(l, m, midw)
//
// The planes are gridded in one launch into a stack of grids (a layered
// plan), transformed as one batch of centred inverse FFTs, and combined here
// in one pass over the stack.  w_kernel_function (crocodile/synthesis.py:273-293) is
// exp(2 pi i w ph) with ph = 1 - sqrt(1 - l^2 - m^2); ph is computed in FP64
// once per pixel, the turns w ph of each plane are formed in double-float
// arithmetic and reduced to a fraction of a turn before the FP32 sincospi,
// so the FP32 factor is accurate to ~1e-7 for any w.
#include "cg_internal.cuh"

namespace cg {

// Mean of w over each layer's visibilities (the plan's sorted order keeps a
// layer's visibilities contiguous).  Grid (chunk, layer): every block sums up
// to LMW_CHUNK of its layer's visibilities and adds its sum to the layer's
// total (FP64 atomics, so the order of the partial sums varies between runs);
// k_layer_mean_finish divides by the counts.  Empty layers get mean 0, count 0.
constexpr int LMW_CHUNK = 8192;

__global__ void k_layer_sum_w(const double *__restrict__ uvw, int64_t stride,
                              const int32_t *__restrict__ perm, const int32_t *__restrict__ counts,
                              const int32_t *__restrict__ offsets, int buckets_per_layer,
                              double *__restrict__ sum_out) {
  const int l = blockIdx.y;
  const int b0 = l * buckets_per_layer, b1 = b0 + buckets_per_layer - 1;
  const int start = offsets[b0] + blockIdx.x * LMW_CHUNK;
  const int end = min(offsets[b1] + counts[b1], start + LMW_CHUNK);
  if (start >= end) return;
  double sum = 0.0;
  for (int j = start + threadIdx.x; j < end; j += blockDim.x) sum += uvw[(int64_t)perm[j] * stride + 2];
  __shared__ double s[32];
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? s[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) atomicAdd(&sum_out[l], t);
  }
}

__global__ void k_layer_mean_finish(int layers, const int32_t *__restrict__ counts,
                                    const int32_t *__restrict__ offsets, int buckets_per_layer,
                                    double *__restrict__ mean, int32_t *__restrict__ count_out) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= layers) return;
  const int b0 = l * buckets_per_layer, b1 = b0 + buckets_per_layer - 1;
  const int c = offsets[b1] + counts[b1] - offsets[b0];
  mean[l] = c ? mean[l] / (double)c : 0.0;
  if (count_out) count_out[l] = c;
}

// image[i, j] = sum_p planes[p, i, j] / exp(2 pi i midw_p ph(i, j)).
// The turns t = midw_p * ph are formed as a double-float product (midw and ph
// split into FP32 hi + lo parts, exact FMA residual), so their fraction keeps
// ~2^-44 relative precision for any w without 32 FP64 products per pixel.
// ph depends on l^2 + m^2 only, and the coordinates (k - N/2) / N of column
// k and of its mirror 2 (N/2) - k are negatives of each other, so the pixels
// (i, j), (i', j), (i, j'), (i', j') share ph and every plane's factor: one
// thread takes all four (those that exist), with one FP64 ph and one
// sincospi per plane, and gives each the same result as alone.  Consecutive
// threads take consecutive j, so the four row segments stay coalesced.
__global__ void k_wstack_combine(const float2 *__restrict__ planes, int layers, int N,
                                 double theta, const double *__restrict__ midw,
                                 const int32_t *__restrict__ counts, float2 *__restrict__ out,
                                 int32_t *status) {
  // (hi, lo) of midw for the layers with visibilities, in layer order, and
  // their count
  extern __shared__ float2 s_w[];
  int *s_pl = (int *)(s_w + layers);  // their layer numbers
  __shared__ int s_np;
  if (threadIdx.x == 0) {
    int np = 0;
    for (int p = 0; p < layers; ++p)
      if (counts[p]) {
        const double w = midw[p];
        const float hi = (float)w;
        s_pl[np] = p;
        s_w[np++] = make_float2(hi, (float)(w - (double)hi));
      }
    s_np = np;
  }
  __syncthreads();
  const int np = s_np;
  const int64_t total = (int64_t)N * N;
  const int half = N / 2, M = half + 1, mirror = 2 * half;  // representatives 0 .. N/2
  const int64_t reps = (int64_t)M * M;
  int bad = 0;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < reps;
       L += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(L / M), j = (int)(L - (int64_t)i * M);
    const int i2 = mirror - i, j2 = mirror - j;
    const bool hasi = i2 < N && i2 != i, hasj = j2 < N && j2 != j;
    int64_t off[4];
    off[0] = (int64_t)i * N + j;
    off[1] = hasj ? (int64_t)i * N + j2 : -1;
    off[2] = hasi ? (int64_t)i2 * N + j : -1;
    off[3] = hasi && hasj ? (int64_t)i2 * N + j2 : -1;
    // theta * coordinates2(N): l along columns (x), m along rows (y)
    const double l = __dmul_rn(theta, centred_coord(j, half, N));
    const double m = __dmul_rn(theta, centred_coord(i, half, N));
    const double r2 = __dadd_rn(__dmul_rn(l, l), __dmul_rn(m, m));
    if (!(r2 < 1.0)) bad = 1;
    const double ph = 1.0 - sqrt(1.0 - r2);
    const float ph_h = (float)ph, ph_l = (float)(ph - (double)ph_h);
    float ax[4] = {0.f, 0.f, 0.f, 0.f}, ay[4] = {0.f, 0.f, 0.f, 0.f};
    // two planes per pass: eight loads in flight before the first use
    for (int t = 0; t < np; t += 2) {
      float2 g[2][4];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const bool in = t + u < np;
        const float2 *plane = planes + (int64_t)(in ? s_pl[t + u] : 0) * total;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          g[u][q] = in && off[q] >= 0 ? plane[off[q]] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (t + u >= np) break;
        const float2 w = s_w[t + u];
        const float hi = w.x * ph_h;
        const float lo = fmaf(w.x, ph_h, -hi) + fmaf(w.x, ph_l, w.y * ph_h);
        const float f = (hi - rintf(hi)) + lo;
        float sn, cs;
        sincospif(2.0f * f, &sn, &cs);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          // g / (cs + i sn) = g * (cs - i sn) for |e| = 1
          ax[q] += g[u][q].x * cs + g[u][q].y * sn;
          ay[q] += g[u][q].y * cs - g[u][q].x * sn;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (off[q] >= 0) out[off[q]] = make_float2(ax[q], ay[q]);
  }
  if (bad && status) atomicAdd(&status[ST_RANGE], 1);
}

}  // namespace cg

using namespace cg;

extern "C" {

int cg_plan_layer_mean_w(const cg_plan *p, const double *uvw, int64_t stride, double *mean_out,
                         int32_t *count_out, cg_stream_t stream) {
  CG_REQUIRE(p && p->mode == CG_PLAN_TILED, "needs a CG_PLAN_TILED plan");
  CG_REQUIRE(uvw && stride >= 3 && mean_out, "NULL argument");
  if (p->n == 0) {
    CG_CUDA(cudaMemsetAsync(mean_out, 0, sizeof(double) * p->layers, (cudaStream_t)stream));
    if (count_out)
      CG_CUDA(cudaMemsetAsync(count_out, 0, sizeof(int32_t) * p->layers, (cudaStream_t)stream));
    return CG_OK;
  }
  const int bpl = p->tpl << (2 * p->sublog);
  cudaStream_t st = (cudaStream_t)stream;
  CG_REQUIRE(p->layers <= 65535, "at most 65535 layers");
  CG_CUDA(cudaMemsetAsync(mean_out, 0, sizeof(double) * p->layers, st));
  const dim3 grid((unsigned)((p->n + LMW_CHUNK - 1) / LMW_CHUNK), (unsigned)p->layers);
  k_layer_sum_w<<<grid, 256, 0, st>>>(uvw, stride, p->perm, p->counts, p->offsets, bpl, mean_out);
  CG_LAUNCH("layer sum w");
  k_layer_mean_finish<<<(p->layers + 255) / 256, 256, 0, st>>>(p->layers, p->counts, p->offsets,
                                                                bpl, mean_out, count_out);
  CG_LAUNCH("layer mean w");
  return CG_OK;
}

int cg_wstack_combine(const void *planes_c64, int layers, int N, double theta,
                      const double *mean_w, const int32_t *counts, void *image_c64,
                      int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(planes_c64 && mean_w && counts && image_c64 && layers >= 1 && N >= 1,
             "bad w-stacking arguments");
  const int64_t reps = (int64_t)(N / 2 + 1) * (N / 2 + 1);  // mirror-symmetric pixel sets
  int64_t blocks = (reps + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (blocks > cap) blocks = cap;
  CG_REQUIRE(layers <= 4096, "at most 4096 w-planes");
  k_wstack_combine<<<(unsigned)blocks, 256, layers * (sizeof(float2) + sizeof(int)),
                     (cudaStream_t)stream>>>(
      (const float2 *)planes_c64, layers, N, theta, mean_w, counts, (float2 *)image_c64,
      d_status);
  CG_LAUNCH("w-stack combine");
  return CG_OK;
}

}  // extern "C"
