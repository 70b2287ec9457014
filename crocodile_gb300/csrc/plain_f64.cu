// Plain FP64 gridding/degridding (K10) and boxcar gridding.
//
// The plain form is the accuracy and speed comparator of the FP32 tiled
// path: complex128 data, one thread per (visibility, tap) with FP64
// atomicAdd into the grid, one launch per kernel group (w-plane or AW
// group), no tiling, no shared memory, no register accumulation.  It
// consumes a CG_PLAN_GROUPS plan, whose records are the same bit-exact cell
// assignment as the tiled path.  Replaces convgrid/convdegrid
// (crocodile/synthesis.py:464-503) at full reference precision.
//
// Boxcar gridding replaces grid/degrid (synthesis.py:389-416).
#include "cg_internal.cuh"

namespace cg {

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ bool any_failed(const int32_t *st) {
  return (st[ST_RANGE] | st[ST_BOUNDS] | st[ST_INDEX]) != 0;
}

struct PlainArgs {
  const VisRec *recs;
  const int32_t *perm;
  const int32_t *status;
  int W, S, Q, sep;
};

__device__ __forceinline__ double2 plain_kernel(const PlainArgs &A,
                                                const double2 *__restrict__ ktab,
                                                const VisRec &r, int dy, int dx) {
  if (A.sep)
    return zmul(ktab[(long long)r.k0 * A.S + dy], ktab[(long long)r.k1 * A.S + dx]);
  const long long SS = (long long)A.S * A.S;
  return ktab[(long long)r.k0 * A.Q * A.Q * SS + (long long)r.k1 * SS + dy * A.S + dx];
}

__global__ void k_grid_plain(PlainArgs A, int start, int count,
                             const double2 *__restrict__ ktab,
                             const double2 *__restrict__ vis,
                             double *__restrict__ grid) {  // grid of this bucket's layer
  if (any_failed(A.status)) return;
  const int SS = A.S * A.S;
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)count * SS) return;
  const int j = (int)(idx / SS), t = (int)(idx - (int64_t)j * SS);
  const int dy = t / A.S, dx = t - dy * A.S;
  const VisRec r = A.recs[start + j];
  const double2 v = vis[A.perm[start + j]];
  const double2 val = zmul(plain_kernel(A, ktab, r, dy, dx), v);
  const size_t cell = (size_t)(r.y0 + dy) * A.W + (r.x0 + dx);
  atomicAdd(&grid[2 * cell], val.x);
  atomicAdd(&grid[2 * cell + 1], val.y);
}

__global__ void k_degrid_plain(PlainArgs A, int start, int count,
                               const double2 *__restrict__ ktab,
                               const double2 *__restrict__ grid,
                               double2 *__restrict__ out) {
  if (any_failed(A.status)) return;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= count) return;
  const VisRec r = A.recs[start + j];
  double2 sum = make_double2(0.0, 0.0);
  for (int dy = 0; dy < A.S; ++dy)
    for (int dx = 0; dx < A.S; ++dx) {
      const double2 g = grid[(size_t)(r.y0 + dy) * A.W + (r.x0 + dx)];
      const double2 p = zmul(g, plain_kernel(A, ktab, r, dy, dx));
      sum.x += p.x;
      sum.y += p.y;
    }
  out[A.perm[start + j]] = sum;
}

// Boxcar cell: N//2 + floor(0.5 + N*p) with numpy's wrap of indices in [-N, 0).
__device__ __forceinline__ bool boxcar_cell(double p, int N, int extent, int &c) {
  double f = floor(__dadd_rn(0.5, __dmul_rn((double)N, p)));
  long long v = (long long)(N / 2) + (long long)f;
  if (v < 0) v += extent;
  c = (int)v;
  return v >= 0 && v < extent;
}

// The reference asserts max(p) < 0.5 over every column of p (u, v and w).
__device__ __forceinline__ bool boxcar_below_half(const double *uvw, int64_t stride,
                                                  int64_t i, double lam) {
  const int ncol = stride < 3 ? (int)stride : 3;
  bool ok = true;
  for (int c = 0; c < ncol; ++c) ok = ok && (vis_coord(uvw, stride, i, c, lam) < 0.5);
  return ok;
}

// check = true: count errors only; check = false: grid unless any error was
// counted, so that a failing call leaves the grid untouched.
__global__ void k_grid_boxcar(const double *uvw, int64_t stride, double lam,
                              int64_t n, const double2 *__restrict__ vis,
                              double *__restrict__ grid, int H, int W,
                              int32_t *status, bool check) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!check && any_failed(status)) return;
  if (!boxcar_below_half(uvw, stride, i, lam)) {
    if (check) atomicAdd(&status[ST_RANGE], 1);
    return;
  }
  const double pu = vis_coord(uvw, stride, i, 0, lam);
  const double pv = vis_coord(uvw, stride, i, 1, lam);
  int x, y;
  bool okx = boxcar_cell(pu, H, W, x), oky = boxcar_cell(pv, H, H, y);
  if (!(okx && oky)) {
    if (check) atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  if (check) return;
  const double2 v = vis[i];
  atomicAdd(&grid[2 * ((size_t)y * W + x)], v.x);
  atomicAdd(&grid[2 * ((size_t)y * W + x) + 1], v.y);
}

__global__ void k_degrid_boxcar(const double *uvw, int64_t stride, double lam,
                                int64_t n, const double2 *__restrict__ grid,
                                double2 *__restrict__ out, int H, int W,
                                int32_t *status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!boxcar_below_half(uvw, stride, i, lam)) {
    atomicAdd(&status[ST_RANGE], 1);
    out[i] = make_double2(0.0, 0.0);
    return;
  }
  const double pu = vis_coord(uvw, stride, i, 0, lam);
  const double pv = vis_coord(uvw, stride, i, 1, lam);
  int x, y;
  bool okx = boxcar_cell(pu, H, W, x), oky = boxcar_cell(pv, H, H, y);
  if (!(okx && oky)) {
    atomicAdd(&status[ST_INDEX], 1);
    out[i] = make_double2(0.0, 0.0);
    return;
  }
  out[i] = grid[(size_t)y * W + x];
}

static PlainArgs plain_args(const cg_plan *p) {
  PlainArgs A;
  A.recs = p->recs;
  A.perm = p->perm;
  A.status = p->status;
  A.W = p->W;
  A.S = p->kd.S;
  A.Q = p->kd.Q;
  A.sep = p->kd.sep;
  return A;
}

}  // namespace cg

using namespace cg;

extern "C" {

int cg_grid_fp64(const cg_plan *p, const void *ktab, const void *vis, void *grid,
                 cg_stream_t stream) {
  CG_REQUIRE(p && p->mode == CG_PLAN_GROUPS, "cg_grid_fp64 needs a CG_PLAN_GROUPS plan");
  if (p->n == 0) return CG_OK;
  CG_REQUIRE(ktab && vis && grid, "NULL argument");
  PlainArgs A = plain_args(p);
  const int SS = p->kd.S * p->kd.S;
  for (int g = 0; g < p->nbuckets; ++g) {
    const int c = p->h_counts[g];
    if (!c) continue;
    const int64_t threads = (int64_t)c * SS;
    double *layer_grid = (double *)grid + 2 * (size_t)(g / p->gper) * p->H * p->W;
    k_grid_plain<<<(unsigned)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        A, p->h_offsets[g], c, (const double2 *)ktab, (const double2 *)vis, layer_grid);
  }
  CG_LAUNCH("grid_fp64");
  return CG_OK;
}

int cg_degrid_fp64(const cg_plan *p, const void *ktab, const void *grid, void *out,
                   cg_stream_t stream) {
  CG_REQUIRE(p && p->mode == CG_PLAN_GROUPS, "cg_degrid_fp64 needs a CG_PLAN_GROUPS plan");
  if (p->n == 0) return CG_OK;
  CG_REQUIRE(ktab && grid && out, "NULL argument");
  PlainArgs A = plain_args(p);
  for (int g = 0; g < p->nbuckets; ++g) {
    const int c = p->h_counts[g];
    if (!c) continue;
    const double2 *layer_grid = (const double2 *)grid + (size_t)(g / p->gper) * p->H * p->W;
    k_degrid_plain<<<(unsigned)((c + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
        A, p->h_offsets[g], c, (const double2 *)ktab, layer_grid, (double2 *)out);
  }
  CG_LAUNCH("degrid_fp64");
  return CG_OK;
}

int cg_grid_boxcar(const double *uvw, int64_t stride, double lam, int64_t n,
                   const void *vis, void *grid, int H, int W, int32_t *d_status,
                   cg_stream_t stream) {
  CG_REQUIRE(H >= 1 && W >= 1, "bad grid");
  CG_REQUIRE(n == 0 || (uvw && vis && grid && d_status && stride >= 2), "NULL argument");
  if (n == 0) return CG_OK;
  for (int pass = 0; pass < 2; ++pass)
    k_grid_boxcar<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        uvw, stride, lam, n, (const double2 *)vis, (double *)grid, H, W, d_status,
        pass == 0);
  CG_LAUNCH("grid_boxcar");
  return CG_OK;
}

int cg_degrid_boxcar(const double *uvw, int64_t stride, double lam, int64_t n,
                     const void *grid, void *out, int H, int W, int32_t *d_status,
                     cg_stream_t stream) {
  CG_REQUIRE(H >= 1 && W >= 1, "bad grid");
  CG_REQUIRE(n == 0 || (uvw && out && grid && d_status && stride >= 2), "NULL argument");
  if (n == 0) return CG_OK;
  k_degrid_boxcar<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      uvw, stride, lam, n, (const double2 *)grid, (double2 *)out, H, W, d_status);
  CG_LAUNCH("degrid_boxcar");
  return CG_OK;
}

}  // extern "C"
