// AW-towers imaging (examples/notebooks/awtowers.ipynb cells 17-22): the
// w-towers scheme with direction-dependent antenna terms applied per baseline
// in the sub-grid's image space.
//
// A visibility falls into the uv chunk and w-plane
//   ub = floor(u*theta / C + 1/2), vb = floor(v*theta / C + 1/2), wp = rint(w / wstep)
// (C = subgrid - margin) and is gridded, per (chunk, plane, baseline) layer,
// relative to the chunk centre (C*ub/theta, C*vb/theta) and the plane's w with
// the anti-aliasing kernel onto a 2s x 2s grid at twice the field of view.
// After one batched inverse FFT of all layers, the combine forms each chunk's
// image
//   image_c = sum over layers L of c: cut_s(layer_L) * corr * aimage[a2_L] /
//             aimage[a1_L] / w_kernel_function(l, m, wp_L * wstep)
// (corr = aa_s x aa_s / aa_2s x aa_2s on the cut: the notebook's kernel
// correction; the Fresnel transfer between planes in closed form), which a
// batched forward FFT and cg_towers_add put into the grid.
//
// The bins and chunk-relative coordinates are IEEE double operations in the
// order numpy evaluates the notebook's expressions, so they are bit-identical.

#include <algorithm>

#include "cg_internal.cuh"

namespace {

using namespace cg;

constexpr int AWT_CHUNKS_PER_BLOCK = 4;  // chunks sharing one pixel's FP64 phase

__device__ __forceinline__ float2 awt_split(double w) {
  const float hi = (float)w;
  return make_float2(hi, (float)(w - (double)hi));
}

// ub, vb, wp of one visibility (false if not finite or beyond 1e9 bins)
__device__ __forceinline__ bool awt_bins(const double *row, double theta, int C, double wstep,
                                         int64_t &ub, int64_t &vb, int64_t &wp) {
  const double fu = floor(__dadd_rn(__ddiv_rn(__dmul_rn(row[0], theta), (double)C), 0.5));
  const double fv = floor(__dadd_rn(__ddiv_rn(__dmul_rn(row[1], theta), (double)C), 0.5));
  const double fw = rint(__ddiv_rn(row[2], wstep));
  if (!(fabs(fu) < 1e9 && fabs(fv) < 1e9 && fabs(fw) < 1e9)) return false;
  ub = (int64_t)fu;
  vb = (int64_t)fv;
  wp = (int64_t)fw;
  return true;
}

__global__ void k_awt_mm_init(int32_t *mm) {
  if (threadIdx.x < 6) mm[threadIdx.x] = (threadIdx.x & 1) ? INT32_MIN : INT32_MAX;
}

__global__ void k_awt_bounds(const double *__restrict__ uvw, int64_t stride, int64_t n,
                             double theta, int C, double wstep, const int32_t *__restrict__ a1,
                             const int32_t *__restrict__ a2, int nant, int32_t *mm,
                             int32_t *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t ub, vb, wp;
  if (!awt_bins(uvw + i * stride, theta, C, wstep, ub, vb, wp)) {
    atomicAdd(&status[ST_RANGE], 1);
    return;
  }
  if ((unsigned)a1[i] >= (unsigned)nant || (unsigned)a2[i] >= (unsigned)nant) {
    atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  atomicMin(&mm[0], (int)ub);
  atomicMax(&mm[1], (int)ub);
  atomicMin(&mm[2], (int)vb);
  atomicMax(&mm[3], (int)vb);
  atomicMin(&mm[4], (int)wp);
  atomicMax(&mm[5], (int)wp);
}

// key = (((vb - vbmin) nub + (ub - ubmin)) nwp + (wp - wpmin)) nant^2 + a1 nant + a2;
// rel = (u - C*ub/theta, v - C*vb/theta, w - wp*wstep)
__global__ void k_awt_keys(const double *__restrict__ uvw, int64_t stride, int64_t n,
                           double theta, int C, double wstep, const int32_t *__restrict__ a1,
                           const int32_t *__restrict__ a2, int nant, int ubmin, int vbmin,
                           int wpmin, int nub, int nwp, int32_t *__restrict__ key,
                           double *__restrict__ rel) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *row = uvw + i * stride;
  int64_t ub, vb, wp;
  if (!awt_bins(row, theta, C, wstep, ub, vb, wp) || (unsigned)a1[i] >= (unsigned)nant ||
      (unsigned)a2[i] >= (unsigned)nant) {
    key[i] = -1;  // counted in the bounds pass
    rel[3 * i] = rel[3 * i + 1] = rel[3 * i + 2] = 0.0;
    return;
  }
  const int64_t k = (((vb - vbmin) * nub + (ub - ubmin)) * nwp + (wp - wpmin)) * nant * nant +
                    (int64_t)a1[i] * nant + a2[i];
  key[i] = (int32_t)k;
  // the notebook's uv_mid = (xy_max + xy_min) // 2 / theta is C*ub / theta exactly
  rel[3 * i] = __dadd_rn(row[0], -__ddiv_rn((double)C * (double)ub, theta));
  rel[3 * i + 1] = __dadd_rn(row[1], -__ddiv_rn((double)C * (double)vb, theta));
  rel[3 * i + 2] = __dadd_rn(row[2], -__dmul_rn((double)wp, wstep));
}

// out[c] (s x s, written rolled by s/2 for an unshifted forward FFT and
// cg_towers_add) = sum over the layers L of chunk c of the centred image of
// layer L cut to s x s, times corr, the antenna ratio and the Fresnel factor.
// The layers arrive as unshifted, unnormalised inverse transforms of the
// 2s x 2s grids: the centred image at centred index k is (-1)^(kx+ky)
// F_L[k + s] / (2s)^2 (indices mod 2s), and the cut takes k = (i, j) + s/2.
__global__ void k_awtowers_combine(const float2 *__restrict__ stack, int s, double theta,
                                   const float *__restrict__ corr,
                                   const float2 *__restrict__ aimage, int nant,
                                   const int32_t *__restrict__ la1,
                                   const int32_t *__restrict__ la2,
                                   const double *__restrict__ layer_w,
                                   const int32_t *__restrict__ chunk_first, int nchunks,
                                   float2 *__restrict__ out, int32_t *status) {
  const int c0 = blockIdx.y * AWT_CHUNKS_PER_BLOCK;
  const int c1 = min(nchunks, c0 + AWT_CHUNKS_PER_BLOCK);
  const int64_t cells = (int64_t)s * s;
  const int s2 = 2 * s;
  const int64_t cells2 = (int64_t)s2 * s2;
  const int half = s / 2;
  const float scale = 1.0f / (float)cells2;
  int bad = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cells;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / s), j = (int)(k - (int64_t)i * s);
    const double l = __dmul_rn(theta, __ddiv_rn((double)(j - half), (double)s));
    const double m = __dmul_rn(theta, __ddiv_rn((double)(i - half), (double)s));
    const double r2 = __dadd_rn(__dmul_rn(l, l), __dmul_rn(m, m));
    if (!(r2 < 1.0)) bad = 1;
    const double ph = 1.0 - sqrt(1.0 - r2);
    const float ph_h = (float)ph, ph_l = (float)(ph - (double)ph_h);
    // centred index in the 2s grid, then its place in the unshifted transform
    const int A = i + half, B = j + half;
    const int Ar = A + s >= s2 ? A + s - s2 : A + s;
    const int Br = B + s >= s2 ? B + s - s2 : B + s;
    const int64_t kr2 = (int64_t)Ar * s2 + Br;
    const float sg = (((A + B) & 1) ? -scale : scale) * corr[k];
    const int ir = i + half >= s ? i + half - s : i + half;
    const int jr = j + half >= s ? j + half - s : j + half;
    for (int c = c0; c < c1; ++c) {
      float ax = 0.f, ay = 0.f;
      for (int L = chunk_first[c]; L < chunk_first[c + 1]; ++L) {
        const float2 g = stack[(int64_t)L * cells2 + kr2];
        const float2 p2 = aimage[(int64_t)la2[L] * cells + k];
        const float2 p1 = aimage[(int64_t)la1[L] * cells + k];
        // ratio p2 / p1 = p2 conj(p1) / |p1|^2
        const float inv = 1.0f / (p1.x * p1.x + p1.y * p1.y);
        const float rx = (p2.x * p1.x + p2.y * p1.y) * inv;
        const float ry = (p2.y * p1.x - p2.x * p1.y) * inv;
        const float gx = g.x * rx - g.y * ry, gy = g.x * ry + g.y * rx;
        // divide by the Fresnel factor exp(2 pi i w ph): multiply by its conjugate
        const float2 w2 = awt_split(layer_w[L]);
        const float hi = w2.x * ph_h;
        const float lo = fmaf(w2.x, ph_h, -hi) + fmaf(w2.x, ph_l, w2.y * ph_h);
        const float f = (hi - rintf(hi)) + lo;
        float sn, cs;
        sincospif(2.0f * f, &sn, &cs);
        ax += gx * cs + gy * sn;
        ay += gy * cs - gx * sn;
      }
      out[(int64_t)c * cells + (int64_t)ir * s + jr] = make_float2(ax * sg, ay * sg);
    }
  }
  if (bad && status) atomicAdd(&status[ST_RANGE], 1);
}

}  // namespace

extern "C" {

int cg_awtower_keys(const double *uvw, int64_t stride, int64_t n, double theta, int chunk,
                    double wstep, const int32_t *a1, const int32_t *a2, int nant,
                    int32_t *key_out, double *rel_out, int32_t *d_minmax, int32_t *h_bounds,
                    int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(n >= 1 && uvw && stride >= 3 && a1 && a2 && key_out && rel_out && d_minmax &&
                 h_bounds && d_status,
             "bad AW-tower key arguments");
  CG_REQUIRE(chunk >= 1 && theta > 0.0 && wstep > 0.0 && nant >= 1 && nant <= 46340,
             "bad chunk, theta, wstep or antenna count");
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_awt_mm_init<<<1, 32, 0, s>>>(d_minmax);
  k_awt_bounds<<<blocks, 256, 0, s>>>(uvw, stride, n, theta, chunk, wstep, a1, a2, nant,
                                      d_minmax, d_status);
  CG_LAUNCH("AW-tower bounds");
  CG_CUDA(cudaMemcpyAsync(h_bounds, d_minmax, 6 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  if (h_bounds[0] > h_bounds[1]) return CG_OK;  // nothing in range
  const int64_t nub = (int64_t)h_bounds[1] - h_bounds[0] + 1;
  const int64_t nvb = (int64_t)h_bounds[3] - h_bounds[2] + 1;
  const int64_t nwp = (int64_t)h_bounds[5] - h_bounds[4] + 1;
  CG_REQUIRE(nub * nvb * nwp * (int64_t)nant * nant < ((int64_t)1 << 31),
             "too many (chunk, plane, baseline) keys");
  k_awt_keys<<<blocks, 256, 0, s>>>(uvw, stride, n, theta, chunk, wstep, a1, a2, nant,
                                    h_bounds[0], h_bounds[2], h_bounds[4], (int)nub, (int)nwp,
                                    key_out, rel_out);
  CG_LAUNCH("AW-tower keys");
  return CG_OK;
}

int cg_awtowers_combine(const void *stack_c64, int layers, int s, double theta, const float *corr,
                        const void *aimage_c64, int nant, const int32_t *layer_a1,
                        const int32_t *layer_a2, const double *layer_w,
                        const int32_t *chunk_first, int nchunks, void *out_c64,
                        int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(stack_c64 && corr && aimage_c64 && layer_a1 && layer_a2 && layer_w && chunk_first &&
                 out_c64 && layers >= 1 && s >= 2 && s % 2 == 0 && nchunks >= 1 && nant >= 1,
             "bad AW-towers combine arguments (even sub-grid size)");
  const int64_t cells = (int64_t)s * s;
  const unsigned bx = (unsigned)std::min<int64_t>((cells + 255) / 256, 1024);
  const unsigned by = (unsigned)((nchunks + AWT_CHUNKS_PER_BLOCK - 1) / AWT_CHUNKS_PER_BLOCK);
  CG_REQUIRE(by <= 65535, "too many chunks for one call");
  k_awtowers_combine<<<dim3(bx, by), 256, 0, (cudaStream_t)stream>>>(
      (const float2 *)stack_c64, s, theta, corr, (const float2 *)aimage_c64, nant, layer_a1,
      layer_a2, layer_w, chunk_first, nchunks, (float2 *)out_c64, d_status);
  CG_LAUNCH("AW-towers combine");
  return CG_OK;
}

}  // extern "C"
