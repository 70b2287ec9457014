// Internal declarations shared by the translation units of libcrocodile_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/crocodile_gb300.h"
#include "tile_order.h"

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
long long wait_cycles();  // clock limit of the bounded waits on bulk copies
int layout_for(const cg_kernel_desc &kd);  // gridder layout used for this kernel table

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
// rate (and an IEEE division costs many FP64 operations), so each coordinate
// costs ONE FP64 operation on the fast path:
//   t = fma(-u, N*Q/lam, M - (N//2)*Q),  M = 1.5 * 2^32
// For |c| < 2^31 the sum lies in [2^32, 2^33), where doubles are spaced 2^-20
// apart, so the single rounding of the FMA leaves F = bits(t) - bits(M) =
// round(c * 2^20), c = -(N//2 + (u/lam)*N) * Q, as a fixed-point integer.
// F is within 2^-21 (+ a few ulp of N*Q) of the value the exact sequence of
// frac_coord rounds, so rint() of the exact value is known unless the
// fraction of F lies within FIX_MARGIN units (2.9e-6) of one half, and the
// range test p in [-0.5, 0.5) (c in (-(N//2 + N/2)*Q, (N/2 - N//2)*Q]) is
// known unless F lies within FIX_MARGIN of an end.  Only those undecided
// cases run the exact IEEE sequence, so results are bit-identical to
// frac_coord/in_unit_range on u / lam.  Non-finite t maps to |F| >= 2^51 and
// tests out of range, as NaN/inf do in the exact test.
constexpr int FIX_BITS = 20;
constexpr long long FIX_ONE = 1ll << FIX_BITS;
constexpr long long FIX_HALF = FIX_ONE >> 1;
constexpr long long FIX_MARGIN = 3;
constexpr unsigned long long FIX_MAGIC_BITS = 0x41F8000000000000ull;  // bits of 1.5 * 2^32
constexpr double FIX_MAGIC = 6442450944.0;                          // 1.5 * 2^32

struct AxisConst {
  double nq_over_lam;  // N * Q / lam
  double c0;           // M - (N//2) * Q  (exact)
  long long lo, hi;    // range ends in fixed point: p < 0.5 <=> F > lo, p >= -0.5 <=> F <= hi
  int qshift;          // log2(Q) when Q is a power of two, else -1
  int fast;            // 0: |c| may reach 2^31 (N*Q >= 2^30); exact sequence only
};

__device__ __forceinline__ long long fixed_coord(double u, const AxisConst &k) {
  const double t = fma(-u, k.nq_over_lam, k.c0);
  return (long long)((unsigned long long)__double_as_longlong(t) - FIX_MAGIC_BITS);
}

// floor division / modulo of fx (|fx| < 2^31) by Q
__device__ __forceinline__ void split_q(long long fx, int Q, int qshift, int &xi, int &xf) {
  if (qshift >= 0) {
    const int f = (int)fx;
    xi = -(f >> qshift);
    xf = f & (Q - 1);
  } else {
    long long q, r;
    floordivmod(fx, Q, q, r);
    xi = (int)(-q);
    xf = (int)r;
  }
}

// Range test and frac_coord of one axis.  Returns false (and leaves xi, xf
// unset) when p = u / lam is outside [-0.5, 0.5) or NaN.
__device__ __forceinline__ bool coord_fast(double u, double lam, const AxisConst &k, int N, int Q,
                                           int &xi, int &xf) {
  long long fx;
  if (k.fast) {
    const long long F = fixed_coord(u, k);
    if (F > k.hi + FIX_MARGIN || F < k.lo - FIX_MARGIN) return false;
    if (F > k.hi - FIX_MARGIN || F < k.lo + FIX_MARGIN) {
      if (!in_unit_range(__ddiv_rn(u, lam))) return false;
    }
    const long long fr = F & (FIX_ONE - 1);
    if (fr < FIX_HALF - FIX_MARGIN || fr > FIX_HALF + FIX_MARGIN) {
      fx = (F >> FIX_BITS) + (fr > FIX_HALF ? 1 : 0);
      split_q(fx, Q, k.qshift, xi, xf);
      return true;
    }
  } else if (!in_unit_range(__ddiv_rn(u, lam))) {
    return false;
  }
  const double p = __ddiv_rn(u, lam);
  const double x = __dadd_rn((double)(N / 2), __dmul_rn(p, (double)N));
  fx = (long long)rint(__dmul_rn(-x, (double)Q));
  split_q(fx, Q, k.qshift, xi, xf);
  return true;
}

// w bin k = rint(w / wstep) (w_cache_imaging, synthesis.py:793), filtered the
// same way: F = round(w * (1/wstep) * 2^20) from one FMA; the estimate is within
// 2^-21 + 2^-22 of w / wstep while |w / wstep| < 2^31 (|F| < 2^51).
__device__ __forceinline__ double w_bin_fast(double w, double wstep, double inv_wstep) {
  const double t = fma(w, inv_wstep, FIX_MAGIC);
  const long long F =
      (long long)((unsigned long long)__double_as_longlong(t) - FIX_MAGIC_BITS);
  if (F > -(1ll << 50) && F < (1ll << 50)) {
    const long long fr = F & (FIX_ONE - 1);
    if (fr < FIX_HALF - FIX_MARGIN || fr > FIX_HALF + FIX_MARGIN)
      return (double)((F >> FIX_BITS) + (fr > FIX_HALF ? 1 : 0));
  }
  return rint(__ddiv_rn(w, wstep));
}

// (k - half) / S, the centred image coordinate of pixel k (coordinates2 of
// synthesis.py): for power-of-two S a multiplication by the exact reciprocal
// (the quotient is exact, so the bits are the division's) instead of an FP64
// division per pixel.
__device__ __forceinline__ double centred_coord(int k, int half, int S) {
  return (S & (S - 1)) == 0 ? __dmul_rn((double)(k - half), 1.0 / (double)S)
                            : __ddiv_rn((double)(k - half), (double)S);
}

// Running minimum and maximum over a grid in mn / mx: the block reduces its
// threads' values (warp reductions, then one warp over the warps' results)
// and one thread applies them, so each address takes one atomic per block
// (atomics of every warp on one address serialise in L2: about 4 ns each).
// Every thread of the block must call it (blockDim.x a multiple of 32); a
// thread without a value passes INT32_MAX and INT32_MIN.
__device__ __forceinline__ void block_atomic_min_max(int32_t *mn, int32_t *mx, int vmin,
                                                     int vmax) {
  __shared__ int s_mm[2][32];
  vmin = __reduce_min_sync(0xffffffffu, vmin);
  vmax = __reduce_max_sync(0xffffffffu, vmax);
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_mm[0][warp] = vmin;
    s_mm[1][warp] = vmax;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    int a = threadIdx.x < nwarps ? s_mm[0][threadIdx.x] : INT32_MAX;
    int b = threadIdx.x < nwarps ? s_mm[1][threadIdx.x] : INT32_MIN;
    a = __reduce_min_sync(0xffffffffu, a);
    b = __reduce_max_sync(0xffffffffu, b);
    if (threadIdx.x == 0) {
      if (a != INT32_MAX) atomicMin(mn, a);
      if (b != INT32_MIN) atomicMax(mx, b);
    }
  }
  __syncthreads();  // s_mm free for the next call
}

// blocks for a grid-stride pass over n items: enough to fill the GPU, few
// enough that per-block atomics stay cheap
inline unsigned stride_blocks(int64_t n, int threads) {
  const int64_t need = (n + threads - 1) / threads, cap = (int64_t)num_sms() * 8;
  return (unsigned)(need < cap ? (need > 0 ? need : 1) : cap);
}

inline AxisConst axis_const(int N, int Q, double lam) {
  AxisConst k;
  k.nq_over_lam = ((double)N * (double)Q) / lam;
  k.c0 = FIX_MAGIC - (double)(N / 2) * (double)Q;
  // p = 0.5 <=> c = -(N//2 + N/2) * Q ; p = -0.5 <=> c = (N/2 - N//2) * Q
  const double half_n = 0.5 * (double)N;
  k.lo = (long long)(-((double)(N / 2) + half_n) * (double)Q * (double)FIX_ONE);
  k.hi = (long long)((half_n - (double)(N / 2)) * (double)Q * (double)FIX_ONE);
  k.qshift = -1;
  for (int b = 0; b < 31; ++b)
    if (Q == (1 << b)) k.qshift = b;
  // fixed point needs |c| < 2^31 for every in-range u and a finite, non-zero
  // scale; otherwise every coordinate takes the exact sequence
  const double nq = (double)N * (double)Q;
  k.fast = (nq < (double)(1 << 30) && lam == lam && lam != 0.0 &&
            k.nq_over_lam - k.nq_over_lam == 0.0) ? 1 : 0;
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
  int tile_req; // requested tile edge (0: tuning / automatic)
  int T;        // tile edge in cells (tiled mode)
  int ntx, nty; // tiles per row / column
  int win;      // window edge = T + S - 1
  int pitch;    // smem row pitch (even)
  int nbuckets;
  int layers;   // stacked grids (w-stacking planes); a grid of H*W cells each
  int gper;     // groups mode: buckets per layer (launch groups, or kernel groups)
  int tblog;    // tiles are numbered in Morton order inside blocks of 2^tblog x 2^tblog tiles
  int nbx;      // tile blocks per row
  int tpl;      // tile numbers per layer (whole blocks: nbx * nby * 4^tblog >= ntx * nty)
  int ntiles;   // tiled mode: tiles of all layers; each holds 4^sublog sub-tile buckets
  int sublog;   // 2^sublog sub-tiles per tile edge, ordered along a Morton curve
  int subshift; // sub-tile edge = 1 << subshift cells (4, or more for huge grid stacks)
  int64_t max_items;
  int chunk;    // visibilities per work item
  int slice_stride;  // lane layout: elements between S x S slices of the table it reads
  int64_t kpad_slices;  // lane layout, slices padded to a 16-byte multiple: slices to copy
  // device arrays inside the caller's workspace
  cg::VisRec *recs;   // sorted records [n]
  int32_t *perm;      // sorted position -> original index [n]
  int32_t *counts;    // [nbuckets]
  int32_t *offsets;   // [nbuckets]
  cg::WorkItem *items;
  float2 *kpad;       // lane layout, odd S * S: the table with padded slices (workspace)
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
