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
