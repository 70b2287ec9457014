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
#include <cmath>
#include <vector>

#include "cg_internal.cuh"
#include "tiled.cuh"

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
  int mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  int bad_range = 0, bad_index = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t ub, vb, wp;
    if (!awt_bins(uvw + i * stride, theta, C, wstep, ub, vb, wp)) {
      ++bad_range;
      continue;
    }
    if ((unsigned)a1[i] >= (unsigned)nant || (unsigned)a2[i] >= (unsigned)nant) {
      ++bad_index;
      continue;
    }
    const int b[3] = {(int)ub, (int)vb, (int)wp};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      mn[d] = min(mn[d], b[d]);
      mx[d] = max(mx[d], b[d]);
    }
  }
  if (bad_range) atomicAdd(&status[ST_RANGE], bad_range);
  if (bad_index) atomicAdd(&status[ST_INDEX], bad_index);
#pragma unroll
  for (int d = 0; d < 3; ++d) block_atomic_min_max(&mm[2 * d], &mm[2 * d + 1], mn[d], mx[d]);
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
    const double l = __dmul_rn(theta, centred_coord(j, half, s));
    const double m = __dmul_rn(theta, centred_coord(i, half, s));
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

// ------------------------------------------------ layer bookkeeping
// From the ascending distinct keys of the layers: each layer's antennas and
// plane index, and a flag where a new chunk starts; then, from the flags'
// exclusive scan, each chunk's first layer and its sub-grid origin
//   (N/2 + C ub - C/2 - (margin + 1)/2, N/2 + C vb - C/2 - (margin + 1)/2),
// the notebook's xy_min = C (ub - 1/2) - (margin + 1) // 2 (C even).
__global__ void k_awt_layers(const int32_t *__restrict__ used, int nl, int nant, int nwp,
                             int32_t *__restrict__ la1, int32_t *__restrict__ la2,
                             int32_t *__restrict__ lplane, int32_t *__restrict__ flag) {
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nl) return;
  const int nn = nant * nant;
  const int k = used[L];
  const int bl = k % nn, rest = k / nn;
  la1[L] = bl / nant;
  la2[L] = bl % nant;
  lplane[L] = rest % nwp;
  flag[L] = (L == 0 || rest / nwp != (used[L - 1] / nn) / nwp) ? 1 : 0;
}

__global__ void k_awt_chunks(const int32_t *__restrict__ used, int nl, int nant, int nwp,
                             const int32_t *__restrict__ flag, const int32_t *__restrict__ scan,
                             int nub, int ubmin, int vbmin, int C, int margin, int N,
                             int32_t *__restrict__ chunk_first, int32_t *__restrict__ origin) {
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nl) return;
  if (L == nl - 1) chunk_first[scan[L] + flag[L]] = nl;
  if (!flag[L]) return;
  const int c = scan[L];
  const int ch = (used[L] / (nant * nant)) / nwp;
  const int ub = ch % nub + ubmin, vb = ch / nub + vbmin;
  const int corner = C / 2 + (margin + 1) / 2;
  chunk_first[c] = L;
  origin[2 * c] = N / 2 + C * ub - corner;
  origin[2 * c + 1] = N / 2 + C * vb - corner;
}

// ------------------------------------------------ direct layer images
// The layers' values at the cut without the 2s x 2s grids and their FFTs.
// The anti-aliasing kernel is separable, so the unshifted inverse transform
// of a layer's grid at (Ar, Br) is the sum over its visibilities of
//   vis * Av(Ar) * Au(Br),  Av(Ar) = sum_a ky[a] w^((y0 + a) Ar),
//                           Au(Br) = sum_b kx[b] w^((x0 + b) Br),
// w = exp(+2 pi i / 2s), with (x0, y0, ky, kx) the plan's footprint and tap
// rows of that visibility (the values cuFFT would produce there, summed in
// another order).  Only the s x s cut is formed: Ar = (i + 3s/2) mod 2s,
// Br = (j + 3s/2) mod 2s.  A layer of a few visibilities costs a few
// thousand complex products instead of a 2s x 2s grid, its zeroing and its
// transform.  Each CTA takes chunks in turn; per layer the visibilities'
// A-vectors go through shared memory in batches of AWT_NB, each thread
// accumulates its pixels (column j = tid mod s, rows i = tid / s + k 256/s),
// then multiplies by the combine's factor (antenna ratio, conjugate Fresnel
// factor) into its chunk sums, which leave times corr x sign / (2s)^2 rolled
// as k_awtowers_combine writes them.

constexpr int AWT_NB = 32;    // visibilities per shared-memory batch
constexpr int AWT_MAXS = 16;  // largest kernel support of the direct form

bool awtowers_direct_supported(int s) { return s == 16 || s == 32 || s == 64; }

// per cut pixel: the Fresnel phase 1 - sqrt(1 - l^2 - m^2) as hi + lo floats
// and corr x (-1)^(A+B) / (2s)^2
__global__ void k_awt_pixels(int s, double theta, const float *__restrict__ corr,
                             float4 *__restrict__ pix, int32_t *status) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= s * s) return;
  const int i = k / s, j = k - (k / s) * s, half = s / 2;
  const double l = __dmul_rn(theta, centred_coord(j, half, s));
  const double m = __dmul_rn(theta, centred_coord(i, half, s));
  const double r2 = __dadd_rn(__dmul_rn(l, l), __dmul_rn(m, m));
  if (!(r2 < 1.0) && status) atomicAdd(&status[ST_RANGE], 1);
  const double ph = 1.0 - sqrt(1.0 - r2);
  const float ph_h = (float)ph, ph_l = (float)(ph - (double)ph_h);
  const float scale = 1.0f / ((float)(2 * s) * (float)(2 * s));
  const float sg = ((((i + half) + (j + half)) & 1) ? -scale : scale) * corr[k];
  pix[k] = make_float4(ph_h, ph_l, sg, 0.f);
}

// per w-plane and cut pixel the conjugate Fresnel factor exp(-2 pi i w ph)
// (the phase formed as k_awtowers_combine forms it), and per antenna and
// pixel conj(aimage) / |aimage|^2: the per-layer factor becomes two products
__global__ void k_awt_tables(int cells, const float4 *__restrict__ pix,
                             const double *__restrict__ plane_w, int nplanes,
                             const float2 *__restrict__ aimage, int nant,
                             float2 *__restrict__ fres, float2 *__restrict__ ainv) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nf = (int64_t)nplanes * cells;
  if (e < nf) {
    const int pl = (int)(e / cells), k = (int)(e - (int64_t)pl * cells);
    const float4 px = pix[k];
    const float2 w2 = awt_split(plane_w[pl]);
    const float hi = w2.x * px.x;
    const float lo = fmaf(w2.x, px.x, -hi) + fmaf(w2.x, px.y, w2.y * px.x);
    const float f = (hi - rintf(hi)) + lo;
    float sn, cs;
    sincospif(2.0f * f, &sn, &cs);
    fres[e] = make_float2(cs, -sn);
  } else if (e < nf + (int64_t)nant * cells) {
    const int64_t a = e - nf;
    const float2 p = aimage[a];
    const float inv = 1.0f / (p.x * p.x + p.y * p.y);
    ainv[a] = make_float2(p.x * inv, -p.y * inv);
  }
}

template <int SUB>
__global__ void __launch_bounds__(256)
    k_awtowers_direct(TiledArgs A, int bpl, int nbuckets, int layers,
                      const int32_t *__restrict__ offsets, const int32_t *__restrict__ counts,
                      const float2 *__restrict__ ktab, const float2 *__restrict__ vis,
                      const float4 *__restrict__ pix, const float2 *__restrict__ tw,
                      const float2 *__restrict__ aimage, const float2 *__restrict__ ainv,
                      const float2 *__restrict__ fres, const int32_t *__restrict__ la1,
                      const int32_t *__restrict__ la2, const int32_t *__restrict__ lplane,
                      const int32_t *__restrict__ chunk_first, int nchunks,
                      float2 *__restrict__ out) {
  constexpr int s2 = 2 * SUB, cells = SUB * SUB;
  constexpr int PPT = cells / 256;  // pixels per thread
  constexpr int RSTEP = 256 / SUB;  // rows between a thread's pixels
  __shared__ float2 sAv[AWT_NB][SUB];
  __shared__ float2 sAu[AWT_NB][SUB];
  __shared__ float2 stw[s2];
  __shared__ float2 sTap[AWT_NB][2][AWT_MAXS];
  __shared__ float2 sVis[AWT_NB];
  __shared__ int2 sOrg[AWT_NB];
  if (status_failed(A.status)) return;
  for (int t = threadIdx.x; t < s2; t += blockDim.x) stw[t] = tw[t];
  const int j = threadIdx.x % SUB, i0 = threadIdx.x / SUB;
  const int S = A.S;
  __syncthreads();
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    float2 acc[PPT];
#pragma unroll
    for (int t = 0; t < PPT; ++t) acc[t] = make_float2(0.f, 0.f);
    for (int L = chunk_first[c]; L < chunk_first[c + 1]; ++L) {
      const int rb = offsets[(int64_t)L * bpl];
      const int re = L + 1 < layers ? offsets[(int64_t)(L + 1) * bpl]
                                    : offsets[nbuckets - 1] + counts[nbuckets - 1];
      // the layer's antennas and plane, loaded before its batches
      const int pa1 = la1[L], pa2 = la2[L], pl = lplane[L];
      float2 lac[PPT];
#pragma unroll
      for (int t = 0; t < PPT; ++t) lac[t] = make_float2(0.f, 0.f);
      for (int b = rb; b < re; b += AWT_NB) {
        const int nb = min(AWT_NB, re - b);
        // stage the batch: footprints, visibilities and both tap rows, one
        // round of independent loads
        for (int e = threadIdx.x; e < nb * (2 + 2 * AWT_MAXS); e += blockDim.x) {
          const int r = e / (2 + 2 * AWT_MAXS), q = e - r * (2 + 2 * AWT_MAXS);
          if (q == 0) {
            const VisRec rec = A.recs[b + r];
            sOrg[r] = make_int2(rec.x0, rec.y0);
          } else if (q == 1) {
            sVis[r] = vis[A.perm[b + r]];
          } else {
            const int t = q - 2, axis = t / AWT_MAXS, tap = t - axis * AWT_MAXS;
            if (tap < S) {
              const VisRec rec = A.recs[b + r];
              sTap[r][axis][tap] = __ldg(&ktab[(int64_t)(axis ? rec.k1 : rec.k0) * S + tap]);
            }
          }
        }
        __syncthreads();
        // the A-vectors of this batch: Av (times the visibility) over the cut
        // rows, Au over the cut columns
        for (int e = threadIdx.x; e < 2 * nb * SUB; e += blockDim.x) {
          const int r = e / s2, rem = e - (e / s2) * s2;
          const int axis = rem / SUB, idx = rem - (rem / SUB) * SUB;
          const int rot = (idx + 3 * SUB / 2) & (s2 - 1);  // Ar or Br
          const int o = axis ? sOrg[r].x : sOrg[r].y;
          float2 a = make_float2(0.f, 0.f);
          for (int q = 0; q < S; ++q) cfma(a, sTap[r][axis][q], stw[((o + q) * rot) & (s2 - 1)]);
          if (axis) {
            sAu[r][idx] = a;
          } else {
            sAv[r][idx] = cmul(a, sVis[r]);
          }
        }
        __syncthreads();
        for (int r = 0; r < nb; ++r) {
          const float2 au = sAu[r][j];
#pragma unroll
          for (int t = 0; t < PPT; ++t) cfma(lac[t], sAv[r][i0 + RSTEP * t], au);
        }
        __syncthreads();
      }
      // the combine's factor: aimage[a2] / aimage[a1] times the conjugate
      // Fresnel factor of the layer's plane (tables)
      const float2 *p2b = aimage + (int64_t)pa2 * cells;
      const float2 *i1b = ainv + (int64_t)pa1 * cells;
      const float2 *fb = fres + (int64_t)pl * cells;
#pragma unroll
      for (int t = 0; t < PPT; ++t) {
        const int k = (i0 + RSTEP * t) * SUB + j;
        const float2 r = cmul(__ldg(&p2b[k]), __ldg(&i1b[k]));
        cfma(acc[t], cmul(lac[t], r), __ldg(&fb[k]));
      }
    }
    // out[c] rolled by s/2 (for an unshifted forward FFT and cg_towers_add)
#pragma unroll
    for (int t = 0; t < PPT; ++t) {
      const int i = i0 + RSTEP * t;
      const int k = i * SUB + j;
      const float sg = __ldg(&pix[k]).z;
      const int ir = (i + SUB / 2) & (SUB - 1), jr = (j + SUB / 2) & (SUB - 1);
      out[(int64_t)c * cells + ir * SUB + jr] = make_float2(acc[t].x * sg, acc[t].y * sg);
    }
  }
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
  k_awt_bounds<<<stride_blocks(n, 256), 256, 0, s>>>(uvw, stride, n, theta, chunk, wstep, a1,
                                                    a2, nant, d_minmax, d_status);
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


// workspace: the pixel table, the twiddles, the Fresnel table, the A-image reciprocals
static size_t awt_ws_part(size_t b) { return (b + 255) & ~(size_t)255; }

size_t cg_awtowers_direct_workspace_bytes(int s, int nant, int nplanes) {
  if (s < 2 || nant < 1 || nplanes < 1) return 0;
  const size_t cells = (size_t)s * s;
  return awt_ws_part(cells * sizeof(float4)) + awt_ws_part(2 * (size_t)s * sizeof(float2)) +
         awt_ws_part((size_t)nplanes * cells * sizeof(float2)) +
         awt_ws_part((size_t)nant * cells * sizeof(float2));
}

int cg_awtowers_direct(const cg_plan *plan, const void *ktab_c64, const void *vis_c64, int s,
                       double theta, const float *corr, const void *aimage_c64, int nant,
                       const int32_t *layer_a1, const int32_t *layer_a2,
                       const int32_t *layer_plane, const double *plane_w, int nplanes,
                       const int32_t *chunk_first, int nchunks, void *out_c64, void *ws,
                       size_t ws_bytes, int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(plan && ktab_c64 && vis_c64 && corr && aimage_c64 && layer_a1 && layer_a2 &&
                 layer_plane && plane_w && chunk_first && out_c64 && d_status && nchunks >= 1 &&
                 nant >= 1 && nplanes >= 1,
             "bad AW-towers direct arguments");
  CG_REQUIRE(awtowers_direct_supported(s), "the direct AW-towers layers need s of 16, 32 or 64");
  CG_REQUIRE(plan->kd.S >= 1 && plan->kd.S <= AWT_MAXS,
             "the direct AW-towers layers take kernel supports up to %d", AWT_MAXS);
  CG_REQUIRE(plan->mode == CG_PLAN_TILED && plan->kd.sep && plan->H == 2 * s &&
                 plan->W == 2 * s && plan->layers >= 1,
             "the direct AW-towers layers need a tiled plan of a separable kernel on 2s x 2s "
             "layers");
  if (!ws || ws_bytes < cg_awtowers_direct_workspace_bytes(s, nant, nplanes))
    return set_error(CG_ERR_WORKSPACE, "AW-towers direct workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t cells = (size_t)s * s;
  char *w = (char *)ws;
  float4 *pix = (float4 *)w;
  w += awt_ws_part(cells * sizeof(float4));
  float2 *tw = (float2 *)w;
  w += awt_ws_part(2 * (size_t)s * sizeof(float2));
  float2 *fres = (float2 *)w;
  w += awt_ws_part((size_t)nplanes * cells * sizeof(float2));
  float2 *ainv = (float2 *)w;
  std::vector<float2> h_tw(2 * s);
  for (int t = 0; t < 2 * s; ++t) {
    const double a = 2.0 * M_PI * (double)t / (2.0 * s);
    h_tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  CG_CUDA(cudaMemcpyAsync(tw, h_tw.data(), h_tw.size() * sizeof(float2), cudaMemcpyHostToDevice,
                          st));
  k_awt_pixels<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(s, theta, corr, pix, d_status);
  const int64_t nt = (int64_t)(nplanes + nant) * (int64_t)cells;
  k_awt_tables<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(
      (int)cells, pix, plane_w, nplanes, (const float2 *)aimage_c64, nant, fres, ainv);
  CG_LAUNCH("AW-towers pixel, Fresnel and A-image tables");
  if (plan->n == 0) {
    CG_CUDA(cudaMemsetAsync(out_c64, 0, (size_t)nchunks * cells * sizeof(float2), st));
    return CG_OK;
  }
  const int bpl = plan->tpl << (2 * plan->sublog);
  CG_REQUIRE((int64_t)bpl * plan->layers == plan->nbuckets, "unexpected plan bucket layout");
  const TiledArgs A = tiled_args(plan);
  const unsigned grid = (unsigned)std::min<int64_t>(nchunks, (int64_t)num_sms() * 8);
#define CG_AWT_DIRECT(SS)                                                                      \
  k_awtowers_direct<SS><<<grid, 256, 0, st>>>(                                                 \
      A, bpl, plan->nbuckets, plan->layers, plan->offsets, plan->counts,                       \
      (const float2 *)ktab_c64, (const float2 *)vis_c64, pix, tw, (const float2 *)aimage_c64,  \
      ainv, fres, layer_a1, layer_a2, layer_plane, chunk_first, nchunks, (float2 *)out_c64)
  if (s == 16) CG_AWT_DIRECT(16);
  else if (s == 32) CG_AWT_DIRECT(32);
  else CG_AWT_DIRECT(64);
#undef CG_AWT_DIRECT
  CG_LAUNCH("AW-towers direct layers");
  return CG_OK;
}


size_t cg_awtower_layers_workspace_bytes(int nlayers) {
  const int n = std::max(nlayers, 1);
  return (2 * (size_t)n + scan_scratch_words(n) + 64) * sizeof(int32_t);
}

int cg_awtower_layers(const int32_t *used, int nlayers, int nant, int nwp, int nub, int ubmin,
                      int vbmin, int chunk, int margin, int N, int32_t *layer_a1,
                      int32_t *layer_a2, int32_t *layer_plane, int32_t *chunk_first,
                      int32_t *origin, int32_t *h_nchunks, void *ws, size_t ws_bytes,
                      cg_stream_t stream) {
  CG_REQUIRE(used && nlayers >= 1 && nant >= 1 && nwp >= 1 && nub >= 1 && chunk >= 2 &&
                 chunk % 2 == 0 && margin >= 0 && layer_a1 && layer_a2 && layer_plane &&
                 chunk_first && origin && h_nchunks,
             "bad AW-tower layer arguments");
  if (!ws || ws_bytes < cg_awtower_layers_workspace_bytes(nlayers))
    return set_error(CG_ERR_WORKSPACE, "AW-tower layer workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  int32_t *flag = (int32_t *)ws, *scan = flag + nlayers, *scratch = scan + nlayers;
  const unsigned g = (unsigned)((nlayers + 255) / 256);
  k_awt_layers<<<g, 256, 0, st>>>(used, nlayers, nant, nwp, layer_a1, layer_a2, layer_plane,
                                  flag);
  CG_LAUNCH("AW-tower layers");
  int rc = launch_scan(flag, scan, nlayers, scratch, st);
  if (rc) return rc;
  k_awt_chunks<<<g, 256, 0, st>>>(used, nlayers, nant, nwp, flag, scan, nub, ubmin, vbmin, chunk,
                                  margin, N, chunk_first, origin);
  CG_LAUNCH("AW-tower chunks");
  int32_t last[2];
  CG_CUDA(cudaMemcpyAsync(&last[0], scan + nlayers - 1, 4, cudaMemcpyDeviceToHost, st));
  CG_CUDA(cudaMemcpyAsync(&last[1], flag + nlayers - 1, 4, cudaMemcpyDeviceToHost, st));
  CG_CUDA(cudaStreamSynchronize(st));
  *h_nchunks = last[0] + last[1];
  return CG_OK;
}

}  // extern "C"
