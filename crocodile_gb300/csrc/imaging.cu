// Imaging-side kernels: uniform weights (K8), mirror_uvw, make_grid_hermitian,
// the centred FFTs and the fused dirty-image pass (K7).
//
// Replaces doweight (crocodile/synthesis.py:535-549), mirror_uvw (:831-852),
// make_grid_hermitian (:855-880), fft/ifft (:83-106) and the image half of
// do_imaging (:904-911).  FFTs run in the library's own transforms (FP32,
// fft32.cu, for complex64 planes with power-of-two sides 64..8192;
// double-float, dfft.cu, for complex128 planes 64..2048) and in cuFFT for
// other shapes; the shifts of the centred transform are folded into the
// neighbouring passes: for even sizes
//   fftshift(F(ifftshift(a)))[k, l] = (-1)^(k + l + (H + W)/2) F(a * (-1)^(m + n))[k, l]
// so no data movement is spent on them.
#include <cufft.h>
#include <float.h>

#include <map>
#include <mutex>
#include <tuple>

#include "cg_internal.cuh"

namespace cg {

// ---------------------------------------------------------------- cuFFT plans (other shapes)
static std::mutex g_fft_mu;
static std::map<std::tuple<int, int, int, int, int>, cufftHandle> g_fft_plans;

bool fft32_supported(int H, int W);
int fft32_planes(float2 *data, int64_t batch, int H, int W, bool inverse, bool centred,
                 cudaStream_t st);
int fft32_image(const float2 *grid_premod, int H, int W, float *image, float *max_out,
                cudaStream_t st);
bool dfft_supported(int n);
int dfft2_centred(double2 *data, int64_t batch, int H, int W, int inverse, cudaStream_t st);

int fft_plan(int batch, int H, int W, cufftType type, cufftHandle *out) {
  int dev = 0;
  cudaGetDevice(&dev);
  auto key = std::make_tuple(dev, batch, H, W, (int)type);
  std::lock_guard<std::mutex> lock(g_fft_mu);
  auto it = g_fft_plans.find(key);
  if (it != g_fft_plans.end()) {
    *out = it->second;
    return CG_OK;
  }
  cufftHandle h;
  cufftResult r;
  if (H == 1) {
    int n[1] = {W};
    r = cufftPlanMany(&h, 1, n, nullptr, 1, W, nullptr, 1, W, type, batch);
  } else {
    int n[2] = {H, W};
    r = cufftPlanMany(&h, 2, n, nullptr, 1, H * W, nullptr, 1, H * W, type, batch);
  }
  if (r != CUFFT_SUCCESS)
    return set_error(CG_ERR_CUDA, "cufftPlanMany(%d x %d, batch %d) failed: %d", H, W,
                     batch, (int)r);
  g_fft_plans[key] = h;
  *out = h;
  return CG_OK;
}

template <typename C>
struct CT;
template <>
struct CT<float2> {
  typedef float R;
};
template <>
struct CT<double2> {
  typedef double R;
};

template <typename C>
__device__ __forceinline__ C cconj_add(C a, C b) {  // a + conj(b)
  C r;
  r.x = a.x + b.x;
  r.y = a.y - b.y;
  return r;
}

// ---------------------------------------------------------------- weights
__global__ void k_weight_count(const double *uvw, int64_t stride, double lam, AxisConst k,
                               int64_t n, int N, int32_t *counts, int32_t *status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double u = uvw[i * stride], v = uvw[i * stride + 1];
  int x, xf, y, yf;
  const bool inx = coord_fast(u, lam, k, N, 1, x, xf);
  const bool iny = coord_fast(v, lam, k, N, 1, y, yf);
  if (!(inx && iny)) {
    atomicAdd(&status[ST_RANGE], 1);
    return;
  }
  if (x < 0 || x >= N || y < 0 || y >= N) {
    atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  atomicAdd(&counts[(size_t)x * N + y], 1);  // gw[x, y] as the reference indexes it
}

__global__ void k_weight_apply(const double *uvw, int64_t stride, double lam, AxisConst k,
                               int64_t n, int N, const int32_t *counts,
                               const double *v_in, double *w_out,
                               const int32_t *status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if ((status[ST_RANGE] | status[ST_INDEX]) != 0) return;
  int x, xf, y, yf;
  if (!(coord_fast(uvw[i * stride], lam, k, N, 1, x, xf) &&
        coord_fast(uvw[i * stride + 1], lam, k, N, 1, y, yf)))
    return;
  const double v = v_in ? v_in[i] : 1.0;
  w_out[i] = v / (double)counts[(size_t)x * N + y];
}

// ---------------------------------------------------------------- mirror
template <typename C>
__global__ void k_mirror(double *uvw, int64_t stride, int64_t n, C *vis) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *row = uvw + i * stride;
  if (row[1] < 0) {
    const int nc = stride < 3 ? (int)stride : 3;
    for (int c = 0; c < nc; ++c) row[c] = -row[c];
    if (vis) vis[i].y = -vis[i].y;
  }
}

// ---------------------------------------------------------------- hermitian
// In place: every cell is paired with its mirror and both are written by
// the thread that owns the lower linear index.  MOD multiplies by the
// checkerboard (-1)^(i+j) on the way (pre-modulation of the centred ifft).
template <typename C, bool MOD>
__global__ void k_hermitian(C *g, int H, int W) {
  const int64_t total = (int64_t)H * W;
  const bool even = (H % 2) == 0;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total;
       L += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(L / W), j = (int)(L - (int64_t)i * W);
    typedef typename CT<C>::R R;
    const R s = (MOD && ((i + j) & 1)) ? R(-1) : R(1);
    if (even && (i == 0 || j == 0)) {
      if (MOD) {
        C a = g[L];
        a.x *= s;
        a.y *= s;
        g[L] = a;
      }
      continue;
    }
    const int mi = even ? H - i : H - 1 - i, mj = even ? W - j : W - 1 - j;
    const int64_t M = (int64_t)mi * W + mj;
    if (M < L) continue;
    const C a = g[L], b = g[M];
    C na = cconj_add(a, b), nb = cconj_add(b, a);
    if (MOD) {
      const R sm = ((mi + mj) & 1) ? R(-1) : R(1);
      na.x *= s;
      na.y *= s;
      nb.x *= sm;
      nb.y *= sm;
    }
    g[L] = na;
    if (M != L) g[M] = nb;
  }
}

// ---------------------------------------------------------------- centred FFT helpers
template <typename C>
__global__ void k_checker(C *a, int64_t count, int H, int W, double scale, int phase) {
  typedef typename CT<C>::R R;
  const int64_t plane = (int64_t)H * W;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < count;
       L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = L % plane;
    const int i = (int)(q / W), j = (int)(q - (int64_t)i * W);
    const R s = (((i + j + phase) & 1) ? R(-1) : R(1)) * (R)scale;
    C v = a[L];
    v.x *= s;
    v.y *= s;
    a[L] = v;
  }
}

// dst[b, i, j] = src[b, (i + sh) mod H, (j + sw) mod W] * scale
template <typename C>
__global__ void k_roll(const C *src, C *dst, int64_t count, int H, int W, int sh,
                       int sw, double scale) {
  typedef typename CT<C>::R R;
  const int64_t plane = (int64_t)H * W;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < count;
       L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = L / plane, q = L - b * plane;
    const int i = (int)(q / W), j = (int)(q - (int64_t)i * W);
    const int si = (i + sh) % H, sj = (j + sw) % W;
    C v = src[b * plane + (int64_t)si * W + sj];
    v.x *= (R)scale;
    v.y *= (R)scale;
    dst[L] = v;
  }
}

static unsigned grid_for(int64_t count) {
  int64_t b = (count + 255) / 256;
  int64_t cap = (int64_t)num_sms() * 16;
  return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
}

int centred_fft(void *data, int batch, int H, int W, bool c64, bool inverse,
                void *workspace, cudaStream_t s) {
  CG_REQUIRE(data && batch >= 1 && H >= 1 && W >= 1, "bad fft arguments");
  if (H == 1 && W == 1) return CG_OK;  // the 1 x 1 transform is the identity (scale 1)
  // the hand-written transforms: FP32 for complex64 planes with power-of-two
  // sides 64..8192, double-float (about 48 significant bits) for complex128
  // planes with sides 64..2048; cuFFT for the other shapes
  if (c64 && fft32_supported(H, W))
    return fft32_planes((float2 *)data, batch, H, W, inverse, true, s);
  if (!c64 && H > 1 && dfft_supported(H) && dfft_supported(W))
    return dfft2_centred((double2 *)data, batch, H, W, inverse ? 1 : 0, s);
  cufftHandle plan;
  int rc = fft_plan(batch, H, W, c64 ? CUFFT_C2C : CUFFT_Z2Z, &plan);
  if (rc) return rc;
  if (cufftSetStream(plan, s) != CUFFT_SUCCESS)
    return set_error(CG_ERR_CUDA, "cufftSetStream failed");
  const int64_t count = (int64_t)batch * H * W;
  const double scale = inverse ? 1.0 / ((double)H * W) : 1.0;
  const int dir = inverse ? CUFFT_INVERSE : CUFFT_FORWARD;
  auto exec = [&](void *p) -> int {
    cufftResult r = c64 ? cufftExecC2C(plan, (cufftComplex *)p, (cufftComplex *)p, dir)
                        : cufftExecZ2Z(plan, (cufftDoubleComplex *)p,
                                       (cufftDoubleComplex *)p, dir);
    return r == CUFFT_SUCCESS ? CG_OK : set_error(CG_ERR_CUDA, "cufftExec failed: %d", (int)r);
  };
  const bool even = (H == 1 || H % 2 == 0) && (W % 2 == 0);
  const unsigned g = grid_for(count);
  if (even) {
    const int phase = (H / 2 + W / 2) & 1;
    if (c64) k_checker<float2><<<g, 256, 0, s>>>((float2 *)data, count, H, W, 1.0, 0);
    else k_checker<double2><<<g, 256, 0, s>>>((double2 *)data, count, H, W, 1.0, 0);
    CG_LAUNCH("fft checker");
    rc = exec(data);
    if (rc) return rc;
    if (c64) k_checker<float2><<<g, 256, 0, s>>>((float2 *)data, count, H, W, scale, phase);
    else k_checker<double2><<<g, 256, 0, s>>>((double2 *)data, count, H, W, scale, phase);
    CG_LAUNCH("fft checker");
    return CG_OK;
  }
  CG_REQUIRE(workspace, "odd-sized centred FFT needs a workspace of one array");
  // ifftshift into the workspace, transform there, fftshift back.
  const int ih = H / 2, iw = W / 2;            // ifftshift: src index i + n//2
  const int fh = H - H / 2, fw = W - W / 2;    // fftshift:  src index i - n//2 == i + (n - n//2)
  if (c64) k_roll<float2><<<g, 256, 0, s>>>((float2 *)data, (float2 *)workspace, count, H, W, ih, iw, 1.0);
  else k_roll<double2><<<g, 256, 0, s>>>((double2 *)data, (double2 *)workspace, count, H, W, ih, iw, 1.0);
  CG_LAUNCH("fft roll");
  rc = exec(workspace);
  if (rc) return rc;
  if (c64) k_roll<float2><<<g, 256, 0, s>>>((float2 *)workspace, (float2 *)data, count, H, W, fh, fw, scale);
  else k_roll<double2><<<g, 256, 0, s>>>((double2 *)workspace, (double2 *)data, count, H, W, fh, fw, scale);
  CG_LAUNCH("fft roll");
  return CG_OK;
}

// ---------------------------------------------------------------- dirty image
__device__ __forceinline__ void atomic_max_float(float *addr, float v) {
  if (v >= 0.f)
    atomicMax((int *)addr, __float_as_int(v));
  else
    atomicMin((unsigned int *)addr, __float_as_uint(v));
}

__global__ void k_init_max(float *m) { *m = -FLT_MAX; }

__global__ void k_real_demod(const float2 *__restrict__ F, float *__restrict__ img,
                             int H, int W, float scale, int phase, float *max_out) {
  const int64_t total = (int64_t)H * W;
  float local = -FLT_MAX;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total;
       L += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(L / W), j = (int)(L - (int64_t)i * W);
    const float s = ((i + j + phase) & 1) ? -scale : scale;
    const float v = F[L].x * s;
    img[L] = v;
    local = fmaxf(local, v);
  }
  if (max_out) {
    for (int o = 16; o > 0; o >>= 1) local = fmaxf(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0) atomic_max_float(max_out, local);
  }
}

__global__ void k_scale(float *img, int64_t count, const float *d_scale) {
  const float d = *d_scale;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < count;
       L += (int64_t)gridDim.x * blockDim.x)
    img[L] = img[L] / d;
}

}  // namespace cg

using namespace cg;

extern "C" {

int cg_weights(const double *uvw, int64_t stride, double lam, int64_t n, int N,
               const double *v_in, double *w_out, int32_t *counts, int32_t *d_status,
               cg_stream_t stream) {
  CG_REQUIRE(N > 1, "weighting grid size %d must exceed 1", N);
  CG_REQUIRE(n == 0 || (uvw && w_out && counts && d_status && stride >= 2), "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) return CG_OK;
  CG_CUDA(cudaMemsetAsync(counts, 0, (size_t)N * N * sizeof(int32_t), s));
  const unsigned blocks = (unsigned)((n + 255) / 256);
  const AxisConst k = axis_const(N, 1, lam);
  k_weight_count<<<blocks, 256, 0, s>>>(uvw, stride, lam, k, n, N, counts, d_status);
  k_weight_apply<<<blocks, 256, 0, s>>>(uvw, stride, lam, k, n, N, counts, v_in, w_out,
                                        d_status);
  CG_LAUNCH("weights");
  return CG_OK;
}

int cg_mirror_uvw(double *uvw, int64_t stride, int64_t n, void *vis, int vis_is_c64,
                  cg_stream_t stream) {
  CG_REQUIRE(n == 0 || (uvw && stride >= 2), "NULL argument");
  if (n == 0) return CG_OK;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (vis_is_c64)
    k_mirror<float2><<<blocks, 256, 0, (cudaStream_t)stream>>>(uvw, stride, n, (float2 *)vis);
  else
    k_mirror<double2><<<blocks, 256, 0, (cudaStream_t)stream>>>(uvw, stride, n, (double2 *)vis);
  CG_LAUNCH("mirror_uvw");
  return CG_OK;
}

int cg_make_hermitian(void *grid, int H, int W, int is_c64, cg_stream_t stream) {
  CG_REQUIRE(grid && H >= 1 && W >= 1, "bad hermitian arguments");
  const unsigned g = grid_for((int64_t)H * W);
  if (is_c64)
    k_hermitian<float2, false><<<g, 256, 0, (cudaStream_t)stream>>>((float2 *)grid, H, W);
  else
    k_hermitian<double2, false><<<g, 256, 0, (cudaStream_t)stream>>>((double2 *)grid, H, W);
  CG_LAUNCH("hermitian");
  return CG_OK;
}

int cg_fft(void *data, int batch, int H, int W, int is_c64, int inverse, void *workspace,
           cg_stream_t stream) {
  return centred_fft(data, batch, H, W, is_c64 != 0, inverse != 0, workspace,
                     (cudaStream_t)stream);
}

int cg_fft_raw(void *data, int batch, int H, int W, int is_c64, int inverse,
               cg_stream_t stream) {
  CG_REQUIRE(data && batch >= 1 && H >= 1 && W >= 1, "bad fft arguments");
  cudaStream_t s = (cudaStream_t)stream;
  if (is_c64 && fft32_supported(H, W))
    return fft32_planes((float2 *)data, batch, H, W, inverse != 0, false, s);
  cufftHandle plan;
  int rc = fft_plan(batch, H, W, is_c64 ? CUFFT_C2C : CUFFT_Z2Z, &plan);
  if (rc) return rc;
  if (cufftSetStream(plan, s) != CUFFT_SUCCESS)
    return set_error(CG_ERR_CUDA, "cufftSetStream failed");
  const int dir = inverse ? CUFFT_INVERSE : CUFFT_FORWARD;
  const cufftResult r =
      is_c64 ? cufftExecC2C(plan, (cufftComplex *)data, (cufftComplex *)data, dir)
             : cufftExecZ2Z(plan, (cufftDoubleComplex *)data, (cufftDoubleComplex *)data, dir);
  return r == CUFFT_SUCCESS ? CG_OK : set_error(CG_ERR_CUDA, "cufftExec failed: %d", (int)r);
}

int cg_image_from_grid(void *grid, int H, int W, float *image, float *max_out,
                       cg_stream_t stream) {
  CG_REQUIRE(grid && image, "NULL argument");
  CG_REQUIRE(H % 2 == 0 && W % 2 == 0, "cg_image_from_grid needs even sizes, got %dx%d", H, W);
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned g = grid_for((int64_t)H * W);
  k_hermitian<float2, true><<<g, 256, 0, s>>>((float2 *)grid, H, W);
  CG_LAUNCH("image hermitian");
  if (fft32_supported(H, W))  // rows, then columns storing the demodulated real part
    return fft32_image((const float2 *)grid, H, W, image, max_out, s);
  cufftHandle plan;
  int rc = fft_plan(1, H, W, CUFFT_C2C, &plan);
  if (rc) return rc;
  if (cufftSetStream(plan, s) != CUFFT_SUCCESS)
    return set_error(CG_ERR_CUDA, "cufftSetStream failed");
  if (cufftExecC2C(plan, (cufftComplex *)grid, (cufftComplex *)grid, CUFFT_INVERSE) !=
      CUFFT_SUCCESS)
    return set_error(CG_ERR_CUDA, "cufftExecC2C failed");
  if (max_out) k_init_max<<<1, 1, 0, s>>>(max_out);
  k_real_demod<<<g, 256, 0, s>>>((const float2 *)grid, image, H, W,
                                 (float)(1.0 / ((double)H * W)), (H / 2 + W / 2) & 1, max_out);
  CG_LAUNCH("image demod");
  return CG_OK;
}

int cg_scale_image(float *image, int64_t count, const float *d_scale, cg_stream_t stream) {
  CG_REQUIRE(image && d_scale, "NULL argument");
  if (count == 0) return CG_OK;
  k_scale<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(image, count, d_scale);
  CG_LAUNCH("scale image");
  return CG_OK;
}

}  // extern "C"
