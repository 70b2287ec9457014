// Sze-Tan optimal gridding functions: the table- and image-sized evaluations
// of crocodile/antialias.py in FP64 on the device.
//
// calc_gridding_fine (antialias.py:189-213): for each offset nu_m,
//   rhs[rp] = trap(h_ext * cos(2 pi (lp - nu_m) x), dx),  x = x0 * k / N, k = 0..N
//   C[:, m] = Kinv . rhs,   lp = rp - R + 1, rp = 0..2R-1
// (Kinv, the inverse of the 2R x 2R Gram matrix of h_ext^2, is formed on the
// host: it is 4R^2 sums of N+1 terms.)
//
// calc_gridding_correction_fine (antialias.py:229-246): for each image
// coordinate x_n, with dnu = 1 / (2M) and nu_m = (m + 0.5) / (2M),
//   d(x) = sum_{rp, r} sum_m C[rp, m] C[r, m] cos(2 pi (lp - l) x) dnu
//   c(x) = sum_rp sum_m C[rp, m] cos(2 pi (lp - nu_m) x) dnu
//   hfine = c / d
// d only needs the Gram sums G[rp, r] = sum_m C[rp, m] C[r, m], formed once
// (one block per pair); c is one block per coordinate reducing over m, with
// the cosine split by angle subtraction: nx * M FP64 sincos and nx * M * 2R
// products (8192-pixel axis, M 8192: 6.7e7 sincos).

#include "cg_internal.cuh"

namespace {

constexpr double TWO_PI = 6.283185307179586;  // 2 * numpy.pi, as the reference forms it
constexpr int SZT_MAXR = 16;                   // largest R of the correction sweep

// Block-wide FP64 sum; every thread gets the total.
__device__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0;
  const int nw = (blockDim.x + 31) >> 5;
  for (int i = 0; i < nw; ++i) t += red[i];
  return t;
}

// One warp per offset: lane rp (< 2R) integrates rhs[rp], then lane r forms
// row r of Kinv . rhs.
__global__ void k_szetan_gridding(const double *__restrict__ h_ext, int nh1, double x0, int R,
                                  const double *__restrict__ kinv, const double *__restrict__ nu,
                                  int M, double *__restrict__ C) {
  __shared__ double rhs[8][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m = blockIdx.x * 8 + warp;
  if (m >= M) return;
  const int R2 = 2 * R;
  const int N = nh1 - 1;
  const double dx = x0 / N;
  const double nv = nu[m];
  if (lane < R2) {
    const double lp = (double)(lane - R + 1);
    const double a = TWO_PI * (lp - nv);
    double s = 0;
    for (int k = 0; k <= N; ++k) {
      const double x = x0 * (double)k / (double)N;
      s += h_ext[k] * cos(a * x);
    }
    const double e0 = h_ext[0] * cos(a * 0.0);
    const double e1 = h_ext[N] * cos(a * (x0 * (double)N / (double)N));
    rhs[warp][lane] = dx * (s - 0.5 * (e0 + e1));
  }
  __syncwarp();
  if (lane < R2) {
    double c = 0;
    for (int rp = 0; rp < R2; ++rp) c += kinv[lane * R2 + rp] * rhs[warp][rp];
    C[(size_t)lane * M + m] = c;
  }
}

// G[rp, r] = sum_m C[rp, m] C[r, m]; one block per (rp, r).
__global__ void k_szetan_gram(const double *__restrict__ C, int R2, int M, double *__restrict__ G) {
  __shared__ double red[32];
  const int rp = blockIdx.x / R2, r = blockIdx.x % R2;
  double s = 0;
  for (int m = threadIdx.x; m < M; m += blockDim.x)
    s += C[(size_t)rp * M + m] * C[(size_t)r * M + m];
  s = block_sum(s, red);
  if (threadIdx.x == 0) G[blockIdx.x] = s;
}

// One block per image coordinate.  cos(2 pi (lp - nu) x) is evaluated as
// cos(2 pi lp x) cos(2 pi nu x) + sin(2 pi lp x) sin(2 pi nu x): one sincos
// per offset instead of 2R cosines (GB300's FP64 rate bounds this sweep), the
// 2R values of the first factors once per block.
__global__ void k_szetan_correction(const double *__restrict__ C, const double *__restrict__ G,
                                    int R, int M, const double *__restrict__ x, int nx,
                                    double *__restrict__ hfine) {
  __shared__ double red[32];
  __shared__ double cl[2 * SZT_MAXR], sl[2 * SZT_MAXR];
  const int n = blockIdx.x;
  if (n >= nx) return;
  const int R2 = 2 * R;
  const double xv = x[n];
  const double dnu = 1.0 / (2.0 * M);
  if (threadIdx.x < R2) {
    const double lp = (double)((int)threadIdx.x - R + 1);
    sincos(TWO_PI * lp * xv, &sl[threadIdx.x], &cl[threadIdx.x]);
  }
  __syncthreads();
  double s = 0;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const double nv = ((double)m + 0.5) / (2.0 * M);
    double sn, cs;
    sincos(TWO_PI * nv * xv, &sn, &cs);
    for (int rp = 0; rp < R2; ++rp) s += C[(size_t)rp * M + m] * (cl[rp] * cs + sl[rp] * sn);
  }
  const double c = block_sum(s, red) * dnu;
  if (threadIdx.x == 0) {
    double d = 0;
    for (int rp = 0; rp < R2; ++rp)
      for (int r = 0; r < R2; ++r)
        d += G[rp * R2 + r] * cos(TWO_PI * (double)(rp - r) * xv);
    hfine[n] = c / (d * dnu);
  }
}

}  // namespace

using namespace cg;

extern "C" {

int cg_szetan_gridding(const double *h_ext, int nh1, double x0, int R, const double *kinv,
                       const double *nu, int M, double *C, cg_stream_t stream) {
  CG_REQUIRE(h_ext && kinv && nh1 >= 2 && R >= 1 && 2 * R <= 32 && M >= 0,
             "bad szetan_gridding arguments (2R must be <= 32, N >= 1)");
  if (M == 0) return CG_OK;
  CG_REQUIRE(nu && C, "bad szetan_gridding arguments (null offsets or output)");
  k_szetan_gridding<<<(M + 7) / 8, 256, 0, (cudaStream_t)stream>>>(h_ext, nh1, x0, R, kinv, nu,
                                                                    M, C);
  CG_LAUNCH("szetan gridding");
  return CG_OK;
}

size_t cg_szetan_correction_workspace_bytes(int R) {
  return (size_t)4 * R * R * sizeof(double);
}

int cg_szetan_correction(const double *C, int R, int M, const double *x, int nx, double *hfine,
                         void *ws, size_t ws_bytes, cg_stream_t stream) {
  CG_REQUIRE(C && R >= 1 && 2 * R <= 32 && M >= 1 && nx >= 0, "bad szetan_correction arguments");
  if (nx == 0) return CG_OK;
  CG_REQUIRE(x && hfine, "bad szetan_correction arguments (null coordinates or output)");
  if (!ws || ws_bytes < cg_szetan_correction_workspace_bytes(R))
    return set_error(CG_ERR_WORKSPACE, "szetan_correction needs %zu workspace bytes",
                     cg_szetan_correction_workspace_bytes(R));
  cudaStream_t st = (cudaStream_t)stream;
  double *G = (double *)ws;
  k_szetan_gram<<<4 * R * R, 256, 0, st>>>(C, 2 * R, M, G);
  CG_LAUNCH("szetan gram");
  k_szetan_correction<<<nx, 256, 0, st>>>(C, G, R, M, x, nx, hfine);
  CG_LAUNCH("szetan correction");
  return CG_OK;
}

}  // extern "C"
