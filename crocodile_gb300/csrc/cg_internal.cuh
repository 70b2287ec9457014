// Internal declarations shared by the translation units of libcrocodile_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/crocodile_gb300.h"

namespace cg {

// ---------------------------------------------------------------- errors
int set_error(int code, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *where);

#define CG_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess) return ::cg::cuda_error(_e, #call);                 \
  } while (0)
#define CG_LAUNCH(where)                                                       \
  do {                                                                         \
    cudaError_t _e = cudaGetLastError();                                       \
    if (_e != cudaSuccess) return ::cg::cuda_error(_e, where);                 \
  } while (0)
#define CG_REQUIRE(cond, ...)                                                  \
  do {                                                                         \
    if (!(cond)) return ::cg::set_error(CG_ERR_ARG, __VA_ARGS__);              \
  } while (0)

enum { ST_RANGE = 0, ST_BOUNDS = 1, ST_INDEX = 2, ST_TIMEOUT = 3 };

int num_sms();
cg_tuning tuning();  // current process-wide launch-shape tuning

// ---------------------------------------------------------------- device helpers
// Python-style floor division / modulo of an integer by a positive divisor.
__device__ __forceinline__ void floordivmod(long long a, int b, long long &q,
                                            long long &r) {
  q = a / b;
  r = a - q * b;
  if (r < 0) {
    r += b;
    q -= 1;
  }
}

// frac_coord (synthesis.py:419-435) for one coordinate p already divided by
// lam.  Every operation is an explicitly rounded IEEE double operation so
// that no FMA contraction changes the bits:
//   x = N//2 + p*N ; fx = rint((-x) * Q) ; (-(fx // Q), fx % Q)
__device__ __forceinline__ void frac_coord(double p, int N, int Q, int &xi,
                                           int &xf) {
  double x = __dadd_rn((double)(N / 2), __dmul_rn(p, (double)N));
  double fxd = rint(__dmul_rn(-x, (double)Q));
  long long q, r;
  floordivmod((long long)fxd, Q, q, r);
  xi = (int)(-q);
  xf = (int)r;
}

__device__ __forceinline__ bool in_unit_range(double p) {
  return p >= -0.5 && p < 0.5;  // false for NaN, as numpy's assert
}

// Filtered exact evaluation.  GB300 runs FP64 at a small fraction of its FP32
// rate and an IEEE division costs many FP64 operations, so coordinates are
// first estimated with one FMA from constants prepared on the host, and the
// exact sequence above runs only when the estimate cannot decide:
//   c~ = fma(-u, NQ_over_lam, -(N//2)*Q)   estimates (-(N//2 + (u/lam)*N)) * Q
// Each of the two evaluations is within a few ulp of the real value, i.e.
// within ~2^-49 * N * Q (< 1e-9 for N*Q <= 2^20) of each other, so rint()
// agrees whenever c~ is further than 1e-6 from a half-integer.  The range
// test p in [-0.5, 0.5) likewise uses u * (1/lam) except within 1e-9 of the
// ends.  Results are bit-identical to frac_coord/in_unit_range on u / lam.
struct AxisConst {
  double nq_over_lam;  // N * Q / lam
  double n2q;          // (N // 2) * Q
  double inv_lam;      // 1 / lam
};

__device__ __forceinline__ bool near_half(double c) {
  const double f = c - floor(c);
  return fabs(f - 0.5) < 1e-6;
}

// p = u / lam in range?  (exact decision)
__device__ __forceinline__ bool unit_range_fast(double u, double lam, double inv_lam) {
  const double pe = u * inv_lam;
  if (pe > -0.5 + 1e-9 && pe < 0.5 - 1e-9) return true;
  if (!(pe > -0.5 - 1e-9 && pe < 0.5 + 1e-9)) return false;  // NaN lands here too
  return in_unit_range(__ddiv_rn(u, lam));
}

__device__ __forceinline__ void frac_coord_fast(double u, double lam, const AxisConst &k, int N,
                                                int Q, int &xi, int &xf) {
  const double ce = fma(-u, k.nq_over_lam, -k.n2q);
  long long fx;
  if (!near_half(ce)) {
    fx = (long long)rint(ce);
  } else {
    const double p = __ddiv_rn(u, lam);
    const double x = __dadd_rn((double)(N / 2), __dmul_rn(p, (double)N));
    fx = (long long)rint(__dmul_rn(-x, (double)Q));
  }
  long long q, r;
  floordivmod(fx, Q, q, r);
  xi = (int)(-q);
  xf = (int)r;
}

// w bin k = rint(w / wstep) (w_cache_imaging, synthesis.py:793), filtered likewise.
__device__ __forceinline__ double w_bin_fast(double w, double wstep, double inv_wstep) {
  const double ke = w * inv_wstep;
  if (!near_half(ke)) return rint(ke);
  return rint(__ddiv_rn(w, wstep));
}

inline AxisConst axis_const(int N, int Q, double lam) {
  AxisConst k;
  k.nq_over_lam = ((double)N * (double)Q) / lam;
  k.n2q = (double)(N / 2) * (double)Q;
  k.inv_lam = 1.0 / lam;
  return k;
}

// Visibility coordinate p = uvw[i*stride + axis] / lam (IEEE division).
__device__ __forceinline__ double vis_coord(const double *uvw, int64_t stride,
                                            int64_t i, int axis, double lam) {
  return __ddiv_rn(uvw[i * stride + axis], lam);
}

// ---------------------------------------------------------------- plan
// One visibility after cell assignment: footprint origin (x0, y0) = (x - S//2,
// y - S//2) and kernel table rows.  sep: k0 = g*Q + yf, k1 = g*Q + xf
// (rows of the [G*Q, S] table); 4-D: k0 = g, k1 = yf*Q + xf.
struct __align__(16) VisRec {
  int32_t x0, y0, k0, k1;
};

struct __align__(16) WorkItem {
  int32_t tile, start, count, pad;
};

}  // namespace cg

struct cg_plan {
  int mode;
  cg_kernel_desc kd;
  int H, W;
  int64_t n;
  int T;        // tile edge in cells (tiled mode)
  int ntx, nty; // tiles per row / column
  int win;      // window edge = T + S - 1
  int pitch;    // smem row pitch (even)
  int nbuckets;
  int layers;   // stacked grids (w-stacking planes); a grid of H*W cells each
  int gper;     // groups mode: buckets per layer (launch groups, or kernel groups)
  int tpl;      // tiles per layer (ntx * nty)
  int ntiles;   // tiled mode: tiles of all layers; each holds 4^sublog sub-tile buckets
  int sublog;   // 2^sublog sub-tiles per tile edge, ordered along a Morton curve
  int subshift; // sub-tile edge = 1 << subshift cells (4, or more for huge grid stacks)
  int64_t max_items;
  int chunk;    // visibilities per work item
  // device arrays inside the caller's workspace
  cg::VisRec *recs;   // sorted records [n]
  int32_t *perm;      // sorted position -> original index [n]
  int32_t *counts;    // [nbuckets]
  int32_t *offsets;   // [nbuckets]
  cg::WorkItem *items;
  int32_t *nitems;    // device counter
  int32_t *ticket;    // device counter for the persistent kernels (2 words)
  int32_t *status;    // caller's status block
  // group mode: host copies of group ranges
  int32_t *h_offsets;
  int32_t *h_counts;
};

// Internal entry points shared across translation units.
namespace cg {
int launch_scan(const int32_t *in, int32_t *out, int n, int32_t *scratch,
                cudaStream_t s);
size_t scan_scratch_words(int n);
}  // namespace cg
