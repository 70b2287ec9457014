// Plan construction: bit-exact cell assignment of every visibility (K1),
// counting sort into grid tiles or kernel groups (K2), and the work list of
// the persistent gridding kernels.
//
// Replaces the per-visibility coordinate work of convgrid/convdegrid
// (crocodile/synthesis.py:476-479, 497-499 via frac_coords :438-449) and the
// w ordering of sort_vis_w (:506-515).
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>

#include "cg_internal.cuh"

namespace cg {

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// ---------------------------------------------------------------- scan
// Exclusive scan of int32 counts (bucket histograms).  Three phases:
// per-block scan + block totals, scan of the totals, add-back.
static constexpr int SCAN_THREADS = 1024;
static constexpr int SCAN_PER_THREAD = 4;
static constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;

__device__ __forceinline__ int block_exclusive_scan(int v, int *s_warp,
                                                    int &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int nw = blockDim.x >> 5;
    int w = lane < nw ? s_warp[lane] : 0;
    int winc = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, winc, o);
      if (lane >= o) winc += t;
    }
    if (lane < nw) s_warp[lane] = winc - w;
    if (lane == 31) s_warp[32] = winc;
  }
  __syncthreads();
  total = s_warp[32];
  int r = s_warp[warp] + inc - v;
  __syncthreads();
  return r;
}

__global__ void k_scan_tiles(const int32_t *__restrict__ in,
                             int32_t *__restrict__ out, int n,
                             int32_t *__restrict__ block_sums) {
  __shared__ int s_warp[33];
  const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
  int v[SCAN_PER_THREAD];
  int sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_PER_THREAD; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    sum += v[k];
  }
  int total;
  int run = block_exclusive_scan(sum, s_warp, total);
#pragma unroll
  for (int k = 0; k < SCAN_PER_THREAD; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0 && block_sums) block_sums[blockIdx.x] = total;
}

__global__ void k_scan_add(int32_t *__restrict__ out, int n,
                           const int32_t *__restrict__ block_offsets) {
  const int i = blockIdx.x * SCAN_TILE + threadIdx.x;
  const int add = block_offsets[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_PER_THREAD; ++k) {
    int j = i + k * SCAN_THREADS;
    if (j < n && j < (blockIdx.x + 1) * SCAN_TILE) out[j] += add;
  }
}

// Scratch of the recursive scan: per level the block totals and their scan.
size_t scan_scratch_words(int n) {
  const int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb <= 1) return 0;
  return 2 * (size_t)(nb + 1) + scan_scratch_words(nb);
}

int launch_scan(const int32_t *in, int32_t *out, int n, int32_t *scratch,
                cudaStream_t s) {
  if (n <= 0) return CG_OK;
  const int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 1) {
    k_scan_tiles<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr);
    CG_LAUNCH("scan");
    return CG_OK;
  }
  int32_t *sums = scratch, *sums_off = scratch + nb + 1;
  k_scan_tiles<<<nb, SCAN_THREADS, 0, s>>>(in, out, n, sums);
  CG_LAUNCH("scan");
  const int rc = launch_scan(sums, sums_off, nb, scratch + 2 * (nb + 1), s);
  if (rc) return rc;
  k_scan_add<<<nb, SCAN_THREADS, 0, s>>>(out, n, sums_off);
  CG_LAUNCH("scan");
  return CG_OK;
}

// ---------------------------------------------------------------- K1 coordinates
struct CoordParams {
  const double *uvw;
  int64_t stride;
  double lam;
  int64_t n;
  int H, W, Q, S, G, sep;
  const int32_t *kidx;
  int mode, T, tblog, nbx, nbuckets, sublog, subshift;
  const int32_t *layer;  // per-visibility layer (grid of the stack), or NULL
  int layers, tpl;
  const int32_t *group;  // groups mode: per-visibility launch group, or NULL (= kernel group)
  int ngroups;
  AxisConst ax, ay;    // filtered-exact constants for x (width W) and y (height H)
  double wstep, inv_wstep;  // wstep != 0: the kernel group is the w bin - kmin
  int kmin, nk;
  VisRec *rec;
  int32_t *key;
  int32_t *rank;
  int32_t *hist;
  int32_t *status;
};

// Warp-aggregated increment of hist[key]; returns this lane's slot.  All 32
// lanes of the warp must call it (invalid lanes pass valid = false).
__device__ __forceinline__ int aggregated_slot(int32_t *hist, int key,
                                               bool valid) {
  const int lane = threadIdx.x & 31;
  unsigned peers = __match_any_sync(0xffffffffu, valid ? key : -1);
  int leader = __ffs(peers) - 1;
  int base = 0;
  if (valid && lane == leader) base = atomicAdd(&hist[key], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

// Interleave the low 8 bits of x and y (Morton / Z order).
__device__ __forceinline__ int morton2(int x, int y) {
  return (int)(spread_bits((unsigned)x) | (spread_bits((unsigned)y) << 1));
}

// Tiled-mode bucket: tile (numbered along the blocked Morton curve), then the
// 4x4-cell sub-tile of the footprint origin along a Morton curve, so that
// consecutive visibilities of a work item are spatial neighbours.
__device__ __forceinline__ int tile_bucket(const CoordParams &P, int lyr, int x0, int y0) {
  const int ty = y0 / P.T, tx = x0 / P.T;
  const int ly = y0 - ty * P.T, lx = x0 - tx * P.T;
  return ((lyr * P.tpl + tile_index(tx, ty, P.tblog, P.nbx)) << (2 * P.sublog)) |
         morton2(lx >> P.subshift, ly >> P.subshift);
}

__global__ void k_plan_coords(CoordParams P) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool live = i < P.n;
  bool ok = live;
  int key = -1;
  VisRec r = {0, 0, 0, 0};
  if (live) {
    const double u = P.uvw[i * P.stride], v = P.uvw[i * P.stride + 1];
    int x, xf, y, yf;
    const bool inx = coord_fast(u, P.lam, P.ax, P.W, P.Q, x, xf);
    const bool iny = coord_fast(v, P.lam, P.ay, P.H, P.Q, y, yf);
    if (!(inx && iny)) {
      atomicAdd(&P.status[ST_RANGE], 1);
      ok = false;
    } else {
      int x0 = x - P.S / 2, y0 = y - P.S / 2;
      if (x0 < 0 || y0 < 0 || x0 + P.S > P.W || y0 + P.S > P.H) {
        atomicAdd(&P.status[ST_BOUNDS], 1);
        ok = false;
      }
      int g = 0;
      if (P.wstep != 0.0) {
        const double j = w_bin_fast(P.uvw[i * P.stride + 2], P.wstep, P.inv_wstep) - P.kmin;
        g = (j >= 0.0 && j < (double)P.nk) ? (int)j : -1;
      } else if (P.kidx) {
        g = P.kidx[i];
      }
      if (g < 0 || g >= P.G) {
        atomicAdd(&P.status[ST_INDEX], 1);
        ok = false;
      }
      const int lyr = P.layer ? P.layer[i] : 0;
      if (lyr < 0 || lyr >= P.layers) {
        atomicAdd(&P.status[ST_INDEX], 1);
        ok = false;
      }
      r.x0 = x0;
      r.y0 = y0;
      if (P.sep) {
        r.k0 = g * P.Q + yf;
        r.k1 = g * P.Q + xf;
      } else {
        r.k0 = g;
        r.k1 = yf * P.Q + xf;
      }
      int grp = g, gper = P.G;
      if (P.mode == CG_PLAN_GROUPS && P.group) {
        grp = P.group[i];
        gper = P.ngroups;
        if (grp < 0 || grp >= gper) {
          atomicAdd(&P.status[ST_INDEX], 1);
          ok = false;
        }
      }
      if (ok) key = (P.mode == CG_PLAN_TILED) ? tile_bucket(P, lyr, x0, y0) : lyr * gper + grp;
      if (ok && (unsigned)key >= (unsigned)P.nbuckets) {  // never: a bucket outside the histogram
        atomicAdd(&P.status[ST_INDEX], 1);
        ok = false;
        key = -1;
      }
    }
  }
  int slot = aggregated_slot(P.hist, key, ok);
  if (live) {
    P.rec[i] = r;
    P.key[i] = ok ? key : -1;
    P.rank[i] = slot;
  }
}

__global__ void k_plan_scatter(int64_t n, const VisRec *__restrict__ rec,
                               const int32_t *__restrict__ key,
                               const int32_t *__restrict__ rank,
                               const int32_t *__restrict__ offsets,
                               VisRec *__restrict__ out, int32_t *__restrict__ perm) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int k = key[i];
  if (k < 0) return;
  int pos = offsets[k] + rank[i];
  out[pos] = rec[i];
  perm[pos] = (int32_t)i;
}

// Work items: each tile's sorted range (its 4^sublog sub-tile buckets are
// contiguous) cut into pieces of at most `chunk` visibilities.  First the
// number of pieces per tile, then (after an exclusive scan of those numbers)
// the items at their scanned positions, so that the work list follows the
// tile numbering exactly and the persistent kernels, which take items in list
// order, visit the tiles in that order.
__global__ void k_plan_item_counts(int ntiles, int sublog, const int32_t *__restrict__ counts,
                                   const int32_t *__restrict__ offsets, int chunk,
                                   int32_t *__restrict__ nch) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const int b0 = t << (2 * sublog), b1 = b0 + (1 << (2 * sublog)) - 1;
  const int c = offsets[b1] + counts[b1] - offsets[b0];
  nch[t] = (c + chunk - 1) / chunk;
}

__global__ void k_plan_items(int ntiles, int sublog, const int32_t *__restrict__ counts,
                             const int32_t *__restrict__ offsets, int chunk,
                             const int32_t *__restrict__ nch, const int32_t *__restrict__ ioff,
                             WorkItem *__restrict__ items, int32_t *__restrict__ nitems) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  if (t == ntiles - 1) *nitems = ioff[t] + nch[t];
  const int m = nch[t];
  if (m == 0) return;
  const int b0 = t << (2 * sublog), b1 = b0 + (1 << (2 * sublog)) - 1;
  const int off = offsets[b0];
  const int c = offsets[b1] + counts[b1] - off;
  const int base = ioff[t];
  for (int j = 0; j < m; ++j) {
    WorkItem w;
    w.tile = t;
    w.start = off + j * chunk;
    w.count = min(chunk, c - j * chunk);
    w.pad = 0;
    items[base + j] = w;
  }
}

__global__ void k_frac_coords(const double *uvw, int64_t stride, double lam,
                              int64_t n, int H, int W, int Q, AxisConst ax, AxisConst ay,
                              int32_t *x, int32_t *xf, int32_t *y, int32_t *yf,
                              int32_t *status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double u = uvw[i * stride], v = uvw[i * stride + 1];
  int a = 0, b = 0, c = 0, d = 0;
  const bool inx = coord_fast(u, lam, ax, W, Q, a, b);
  const bool iny = coord_fast(v, lam, ay, H, Q, c, d);
  if (!(inx && iny)) atomicAdd(&status[ST_RANGE], 1);
  x[i] = a;
  xf[i] = b;
  y[i] = c;
  yf[i] = d;
}

// ---------------------------------------------------------------- w bins
// w_cache_imaging's bin (synthesis.py:793): wbin = wstep * round(w / wstep),
// half-to-even.  k = rint(w / wstep) is the bin number.
__global__ void k_w_bins(const double *uvw, int64_t stride, int64_t n, double wstep,
                         double inv_wstep, int32_t *kidx, int32_t *minmax, int32_t *status) {
  int lo = INT32_MAX, hi = INT32_MIN, bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double k = w_bin_fast(uvw[i * stride + 2], wstep, inv_wstep);
    if (!(k > -1.0e9 && k < 1.0e9)) {
      ++bad;
      kidx[i] = 0;
    } else {
      const int ki = (int)k;
      kidx[i] = ki;
      lo = min(lo, ki);
      hi = max(hi, ki);
    }
  }
  if (bad) atomicAdd(&status[ST_RANGE], bad);
  block_atomic_min_max(&minmax[0], &minmax[1], lo, hi);
}

__global__ void k_w_bins_rebase(int32_t *kidx, int64_t n, const int32_t *minmax) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) kidx[i] -= minmax[0];
}

// Bins against a known table range [kmin, kmin + nk): no host round trip.
__global__ void k_w_bins_fixed(const double *uvw, int64_t stride, int64_t n, double wstep,
                               double inv_wstep, int kmin, int nk, int32_t *kidx,
                               int32_t *status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double k = w_bin_fast(uvw[i * stride + 2], wstep, inv_wstep);
  const double j = k - (double)kmin;
  if (!(j >= 0.0 && j < (double)nk)) {
    atomicAdd(&status[ST_INDEX], 1);
    kidx[i] = 0;
    return;
  }
  kidx[i] = (int32_t)j;
}

__global__ void k_minmax_init(int32_t *mm) {
  mm[0] = INT32_MAX;
  mm[1] = INT32_MIN;
}

// ---------------------------------------------------------------- key compaction
// The keys in use as a bitmap (one bit per possible key), the rank of a key
// = the prefix of the words' popcounts + the bits below it in its word: the
// key space of the tower schemes (chunks x planes x antenna pairs) runs to
// hundreds of millions of keys for a few hundred thousand visibilities, and
// a bit per key keeps the passes over it 32 times smaller than a flag word.
// Bits of the keys in use.  Small key spaces (at most KEY_SMEM_WORDS words:
// the w-towers' chunk x plane keys) collect in a shared-memory copy of the
// bitmap that each block ORs into the global one at the end, one atomic per
// non-zero word per block: the keys of a few thousand words take atomics
// from every warp of the grid otherwise, and atomics on one address
// serialise.  Larger key spaces set their bits directly, the lanes of a warp
// that set bits of one word merging them first.
constexpr int KEY_SMEM_WORDS = 8192;

__global__ void k_key_bits(const int32_t *__restrict__ key, int64_t n, int nkeys,
                           uint32_t *__restrict__ bits, int32_t *status) {
  extern __shared__ uint32_t s_bits[];
  const int nw = (nkeys + 31) >> 5;
  const bool local = nw <= KEY_SMEM_WORDS;
  if (local) {
    for (int w = threadIdx.x; w < nw; w += blockDim.x) s_bits[w] = 0u;
    __syncthreads();
  }
  int bad = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // whole warps walk the range together (the merge below needs all 32 lanes)
  const int64_t nround = (n + 31) & ~(int64_t)31;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += stride) {
    const int k = i < n ? key[i] : -1;
    const bool ok = k >= 0 && k < nkeys;
    if (i < n && !ok) ++bad;
    if (local) {
      if (ok) atomicOr(&s_bits[k >> 5], 1u << (k & 31));
      continue;
    }
    const int word = ok ? k >> 5 : -1;
    const uint32_t bit = ok ? 1u << (k & 31) : 0u;
    const uint32_t same = __match_any_sync(0xffffffffu, word);
    uint32_t acc = 0;
#pragma unroll
    for (int l = 0; l < 32; ++l) {
      const uint32_t b = __shfl_sync(0xffffffffu, bit, l);
      if (same & (1u << l)) acc |= b;
    }
    if (ok && (threadIdx.x & 31) == __ffs(same) - 1) atomicOr(&bits[word], acc);
  }
  if (bad) atomicAdd(&status[ST_INDEX], bad);
  if (local) {
    __syncthreads();
    for (int w = threadIdx.x; w < nw; w += blockDim.x)
      if (s_bits[w]) atomicOr(&bits[w], s_bits[w]);
  }
}

__global__ void k_key_popc(const uint32_t *__restrict__ bits, int nw, int32_t *__restrict__ cnt) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nw) cnt[w] = __popc(bits[w]);
}

__global__ void k_key_rows(const int32_t *__restrict__ key, int64_t n, int nkeys,
                           const uint32_t *__restrict__ bits, const int32_t *__restrict__ wpre,
                           int32_t *__restrict__ row) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = key[i];
  if (k < 0 || k >= nkeys) {
    row[i] = 0;
    return;
  }
  const uint32_t below = (1u << (k & 31)) - 1u;
  row[i] = wpre[k >> 5] + __popc(bits[k >> 5] & below);
}

__global__ void k_key_of_row(int nw, const uint32_t *__restrict__ bits,
                             const int32_t *__restrict__ wpre, int32_t *__restrict__ key_of_row) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  uint32_t b = bits[w];
  int r = wpre[w];
  while (b) {
    const int t = __ffs(b) - 1;
    key_of_row[r++] = (w << 5) + t;
    b &= b - 1u;
  }
}

// Kernel-cache key of every visibility for w_cache_imaging with src columns
// (synthesis.py:793-794: kernel_cache(theta, wbin, *src[i])): the w bin and
// the integer src columns of the row packed in mixed radix,
//   key = ((wbin - kmin) * r0 + (c0 - m0)) * r1 + (c1 - m1) ...
// A column value outside [m, m + r) is an index error (key 0).
struct RowKeyCols {
  int ncols;
  int32_t mins[8], ranges[8];
};

__global__ void k_row_keys(const double *__restrict__ uvw, int64_t stride, int64_t n,
                           double wstep, double inv_wstep, int kmin, int nbins,
                           const int32_t *__restrict__ cols, RowKeyCols C,
                           int32_t *__restrict__ key, int32_t *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double j = w_bin_fast(uvw[i * stride + 2], wstep, inv_wstep) - (double)kmin;
  bool ok = j >= 0.0 && j < (double)nbins;
  int64_t k = ok ? (int64_t)j : 0;
  for (int c = 0; c < C.ncols; ++c) {
    const int v = cols[i * C.ncols + c] - C.mins[c];
    ok = ok && v >= 0 && v < C.ranges[c];
    k = k * C.ranges[c] + (ok ? v : 0);
  }
  if (!ok) {
    atomicAdd(&status[ST_INDEX], 1);
    k = 0;
  }
  key[i] = (int32_t)k;
}

// AW kernel key of every visibility: (a1 * nant + a2) * nbins + w bin - kmin, the
// (wbin, a1, a2) key of the AW kernel cache (scripts/image_dataset.py:153-171,
// synthesis.py:793).
__global__ void k_aw_keys(const double *__restrict__ uvw, int64_t stride,
                          const int32_t *__restrict__ a1, const int32_t *__restrict__ a2,
                          int64_t n, int nant, double wstep, double inv_wstep, int kmin,
                          int nbins, int32_t *__restrict__ key, int32_t *status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double j = w_bin_fast(uvw[i * stride + 2], wstep, inv_wstep) - (double)kmin;
  const int p = a1[i], q = a2[i];
  if (!(j >= 0.0 && j < (double)nbins) || p < 0 || p >= nant || q < 0 || q >= nant) {
    atomicAdd(&status[ST_INDEX], 1);
    key[i] = 0;
    return;
  }
  key[i] = (p * nant + q) * nbins + (int)j;
}

// ---------------------------------------------------------------- sizing
struct Layout {
  size_t rec_tmp, key, rank, recs, perm, counts, offsets, scan, items, tnch, tioff, ctr, kpad,
      total;
};

static int tile_edge(const cg_kernel_desc &kd, int req) {
  const cg_tuning t = tuning();
  const int S = kd.S;
  if (req > 0) return std::max(4, std::min(64, req & ~3));
  if (t.tile > 0) return std::max(4, std::min(64, t.tile & ~3));
  if (layout_for(kd) == CG_LAYOUT_LANE) return 16;  // per-warp windows stay small
  if (S <= 8) return 32;
  if (S <= 16) return 48;
  return 64;
}

static void plan_geometry(cg_plan &p) {
  if (p.mode == CG_PLAN_TILED) {
    p.T = tile_edge(p.kd, p.tile_req);
    p.ntx = (p.W + p.T - 1) / p.T;
    p.nty = (p.H + p.T - 1) / p.T;
    // Morton blocks of up to 32 x 32 tiles (no larger than the grid needs)
    p.tblog = tile_block_log(p.ntx, p.nty);
    p.nbx = (p.ntx + (1 << p.tblog) - 1) >> p.tblog;
    const int nby = (p.nty + (1 << p.tblog) - 1) >> p.tblog;
    p.tpl = (p.nbx * nby) << (2 * p.tblog);
    p.ntiles = p.tpl * p.layers;
    const cg_tuning t = tuning();
    // 4x4-cell sub-tiles, 2^sublog per tile edge (4 << full >= T), except for the
    // lane layout, whose private windows need no order inside a tile (tile
    // buckets only).  The sub-tile edge is 1 << subshift cells, so that an
    // in-tile coordinate shifted by subshift is always below 2^sublog.
    int full = 0;
    while ((4 << full) < p.T) ++full;
    p.sublog = layout_for(p.kd) == CG_LAYOUT_LANE ? 0 : full;
    p.subshift = 2 + full - p.sublog;
    // keep the histogram (4 B per bucket) within 2^24 buckets: coarser sub-tiles
    // for very large grid stacks
    while (p.sublog > 0 && ((int64_t)p.ntiles << (2 * p.sublog)) > (1 << 24)) {
      --p.sublog;
      ++p.subshift;
    }
    p.nbuckets = p.ntiles << (2 * p.sublog);
    p.win = p.T + p.kd.S - 1;
    // pitch = S (mod 16): the taps t = dy*S + dx of consecutive lanes fall on
    // consecutive 8-byte bank pairs of the window (no bank conflicts)
    p.pitch = p.win;
    while ((p.pitch - p.kd.S) % 16 != 0) ++p.pitch;
    int64_t want = p.n / (int64_t)(num_sms() * 16) + 1;
    // lane layout: one warp per item, ~12 warps per SM, so shorter items
    p.chunk = t.chunk > 0                              ? t.chunk
              : layout_for(p.kd) == CG_LAYOUT_LANE ? 512
                                                   : (int)std::min<int64_t>(
                                                         2048, std::max<int64_t>(256, want));
    p.max_items = (p.n + p.chunk - 1) / p.chunk + p.ntiles;
    // The lane gridder streams each visibility's S x S slice with one bulk copy,
    // which needs a multiple of 16 bytes: for odd S * S it reads a copy of the
    // table whose slices are padded by one element (made in the workspace by
    // every gridding call).
    const int SS = p.kd.S * p.kd.S;
    p.slice_stride = SS;
    p.kpad_slices = 0;
    if (layout_for(p.kd) == CG_LAYOUT_LANE && !p.kd.sep && (SS & 1)) {
      p.slice_stride = SS + 1;
      p.kpad_slices = (int64_t)p.kd.G * p.kd.Q * p.kd.Q;
    }
  } else {
    p.T = 0;
    p.ntx = p.nty = 0;
    p.tblog = 0;
    p.nbx = 1;
    p.tpl = 1;
    p.nbuckets = p.gper * p.layers;
    p.win = p.pitch = 0;
    p.chunk = 0;
    p.max_items = 0;
    p.slice_stride = p.kd.sep ? p.kd.S : p.kd.S * p.kd.S;
    p.kpad_slices = 0;
  }
}

static Layout layout_of(const cg_plan &p) {
  Layout L;
  size_t o = 0;
  size_t n = (size_t)std::max<int64_t>(p.n, 1);
  L.rec_tmp = o; o = align256(o + n * sizeof(VisRec));
  L.key = o;     o = align256(o + n * 4);
  L.rank = o;    o = align256(o + n * 4);
  L.recs = o;    o = align256(o + n * sizeof(VisRec));
  L.perm = o;    o = align256(o + n * 4);
  L.counts = o;  o = align256(o + (size_t)p.nbuckets * 4);
  L.offsets = o; o = align256(o + (size_t)p.nbuckets * 4);
  L.scan = o;    o = align256(o + scan_scratch_words(p.nbuckets) * 4);
  L.items = o;   o = align256(o + (size_t)std::max<int64_t>(p.max_items, 1) * sizeof(WorkItem));
  const size_t nt = p.mode == CG_PLAN_TILED ? (size_t)p.ntiles : 0;  // items per tile, scanned
  L.tnch = o;    o = align256(o + nt * 4);
  L.tioff = o;   o = align256(o + nt * 4);
  L.ctr = o;     o = align256(o + 4 * 4);
  L.kpad = o;    o = align256(o + (size_t)p.kpad_slices * p.slice_stride * sizeof(float2));
  L.total = o;
  return L;
}

static int check_desc(const cg_kernel_desc *kd, int H, int W) {
  CG_REQUIRE(kd, "kernel descriptor is NULL");
  CG_REQUIRE(kd->Q >= 1 && kd->S >= 1 && kd->G >= 1,
             "bad kernel descriptor Q=%d S=%d G=%d", kd->Q, kd->S, kd->G);
  CG_REQUIRE(kd->S <= 32, "support %d exceeds the supported maximum 32", kd->S);
  CG_REQUIRE(H >= 1 && W >= 1 && H <= 65536 && W <= 65536, "bad grid %dx%d", H, W);
  return CG_OK;
}

// Plan built into a caller-provided struct (no host or device allocation):
// geometry, workspace layout, coordinates + histogram, scan, scatter and (tiled
// mode) the work list.  wstep != 0 derives each visibility's kernel group
// from its w bin (round(w / wstep) - kmin, synthesis.py:793) in the same pass.
int plan_build_into(cg_plan *p, int mode, const cg_kernel_desc *kd, int H, int W,
                    const double *uvw, int64_t stride, double lam, const int32_t *kidx,
                    double wstep, int kmin, int layers, const int32_t *layer,
                    const int32_t *group, int ngroups, int64_t n, void *workspace,
                    size_t workspace_bytes, int32_t *d_status, cudaStream_t s, int tile_req = 0) {
  int rc = check_desc(kd, H, W);
  CG_REQUIRE(!group || (mode == CG_PLAN_GROUPS && ngroups >= 1),
             "launch groups need a CG_PLAN_GROUPS plan and ngroups >= 1");
  if (rc) return rc;
  CG_REQUIRE(layers >= 1 && (layers == 1 || layer || n == 0), "bad layer arguments");
  CG_REQUIRE((int64_t)layers * H * W < ((int64_t)1 << 40), "grid stack too large");
  CG_REQUIRE(mode == CG_PLAN_TILED || mode == CG_PLAN_GROUPS, "bad plan mode %d", mode);
  CG_REQUIRE(n >= 0 && n < (int64_t)INT32_MAX, "visibility count %lld unsupported",
             (long long)n);
  CG_REQUIRE(n == 0 || (uvw && stride >= (wstep != 0.0 ? 3 : 2)), "uvw is NULL or stride too small");
  CG_REQUIRE(d_status, "status block is NULL");
  CG_REQUIRE(kd->G == 1 || kidx || wstep != 0.0 || n == 0,
             "G > 1 needs per-visibility kernel indices");
  memset(p, 0, sizeof(*p));
  p->mode = mode;
  p->kd = *kd;
  p->H = H;
  p->W = W;
  p->n = n;
  p->layers = layers;
  p->gper = group ? ngroups : kd->G;
  p->tile_req = tile_req;
  plan_geometry(*p);
  CG_REQUIRE((int64_t)p->nbuckets < (int64_t)INT32_MAX / 2, "too many tiles");
  const Layout L = layout_of(*p);
  if (!workspace || workspace_bytes < L.total)
    return set_error(CG_ERR_WORKSPACE, "plan needs %zu workspace bytes, got %zu", L.total,
                     workspace_bytes);
  char *ws = (char *)workspace;
  VisRec *rec_tmp = (VisRec *)(ws + L.rec_tmp);
  int32_t *key = (int32_t *)(ws + L.key);
  int32_t *rank = (int32_t *)(ws + L.rank);
  p->recs = (VisRec *)(ws + L.recs);
  p->perm = (int32_t *)(ws + L.perm);
  p->counts = (int32_t *)(ws + L.counts);
  p->offsets = (int32_t *)(ws + L.offsets);
  p->items = (WorkItem *)(ws + L.items);
  p->kpad = p->kpad_slices ? (float2 *)(ws + L.kpad) : nullptr;
  int32_t *ctr = (int32_t *)(ws + L.ctr);
  p->nitems = ctr;
  p->ticket = ctr + 1;
  p->status = d_status;
  // everything later kernels accumulate into starts at zero on every call
  CG_CUDA(cudaMemsetAsync(p->counts, 0, (size_t)p->nbuckets * 4, s));
  CG_CUDA(cudaMemsetAsync(ctr, 0, 16, s));
  if (n == 0) return CG_OK;
  CoordParams P;
  P.uvw = uvw;
  P.stride = stride;
  P.lam = lam;
  P.n = n;
  P.H = H;
  P.W = W;
  P.Q = kd->Q;
  P.S = kd->S;
  P.G = kd->G;
  P.sep = kd->sep;
  P.kidx = kidx;
  P.mode = mode;
  P.T = p->T;
  P.tblog = p->tblog;
  P.nbx = p->nbx;
  P.nbuckets = p->nbuckets;
  P.sublog = p->sublog;
  P.subshift = p->subshift;
  P.layer = layer;
  P.layers = layers;
  P.group = group;
  P.ngroups = ngroups;
  P.tpl = p->tpl;
  P.ax = axis_const(W, kd->Q, lam);
  P.ay = axis_const(H, kd->Q, lam);
  P.wstep = wstep;
  P.inv_wstep = wstep != 0.0 ? 1.0 / wstep : 0.0;
  P.kmin = kmin;
  P.nk = kd->G;
  P.rec = rec_tmp;
  P.key = key;
  P.rank = rank;
  P.hist = p->counts;
  P.status = d_status;
  const int blocks = (int)((n + 255) / 256);
  k_plan_coords<<<blocks, 256, 0, s>>>(P);
  CG_LAUNCH("coords");
  rc = launch_scan(p->counts, p->offsets, p->nbuckets, (int32_t *)(ws + L.scan), s);
  if (rc) return rc;
  k_plan_scatter<<<blocks, 256, 0, s>>>(n, rec_tmp, key, rank, p->offsets, p->recs, p->perm);
  CG_LAUNCH("plan sort");
  if (mode == CG_PLAN_TILED) {
    int32_t *tnch = (int32_t *)(ws + L.tnch), *tioff = (int32_t *)(ws + L.tioff);
    const unsigned tb = (unsigned)((p->ntiles + 255) / 256);
    k_plan_item_counts<<<tb, 256, 0, s>>>(p->ntiles, p->sublog, p->counts, p->offsets, p->chunk,
                                          tnch);
    CG_LAUNCH("plan item counts");
    // the bucket scan's scratch is free again (ntiles <= nbuckets)
    rc = launch_scan(tnch, tioff, p->ntiles, (int32_t *)(ws + L.scan), s);
    if (rc) return rc;
    k_plan_items<<<tb, 256, 0, s>>>(p->ntiles, p->sublog, p->counts, p->offsets, p->chunk, tnch,
                                    tioff, p->items, p->nitems);
  }
  CG_LAUNCH("plan sort");
  return CG_OK;
}

int plan_build_tiled_into(cg_plan *p, const cg_kernel_desc *kd, int H, int W,
                          const double *uvw, int64_t stride, double lam,
                          const int32_t *kidx, int64_t n, void *workspace,
                          size_t workspace_bytes, int32_t *d_status, cudaStream_t s) {
  return plan_build_into(p, CG_PLAN_TILED, kd, H, W, uvw, stride, lam, kidx, 0.0, 0, 1, nullptr,
                         nullptr, 0, n, workspace, workspace_bytes, d_status, s);
}

// Heap plan; the groups form also copies the group ranges to the host.
static int plan_create_heap(cg_plan **out, int mode, const cg_kernel_desc *kd, int H, int W,
                            const double *uvw, int64_t stride, double lam, const int32_t *kidx,
                            double wstep, int kmin, int layers, const int32_t *layer,
                            const int32_t *group, int ngroups, int64_t n, void *workspace,
                            size_t workspace_bytes, int32_t *d_status, cudaStream_t s, int tile_req = 0) {
  CG_REQUIRE(out, "plan output pointer is NULL");
  *out = nullptr;
  cg_plan *p = new (std::nothrow) cg_plan;
  CG_REQUIRE(p, "out of host memory");
  int rc = plan_build_into(p, mode, kd, H, W, uvw, stride, lam, kidx, wstep, kmin, layers, layer,
                           group, ngroups, n, workspace, workspace_bytes, d_status, s, tile_req);
  if (rc) {
    delete p;
    return rc;
  }
  if (mode == CG_PLAN_GROUPS) {
    p->h_counts = (int32_t *)malloc((size_t)p->nbuckets * 4);
    p->h_offsets = (int32_t *)malloc((size_t)p->nbuckets * 4);
    cudaError_t e = cudaSuccess;
    if (!p->h_counts || !p->h_offsets) {
      rc = set_error(CG_ERR_ARG, "out of host memory");
    } else if (n == 0) {
      memset(p->h_counts, 0, (size_t)p->nbuckets * 4);
      memset(p->h_offsets, 0, (size_t)p->nbuckets * 4);
    } else if ((e = cudaMemcpyAsync(p->h_counts, p->counts, (size_t)p->nbuckets * 4,
                                    cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync(p->h_offsets, p->offsets, (size_t)p->nbuckets * 4,
                                    cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
               (e = cudaStreamSynchronize(s)) != cudaSuccess) {
      rc = cuda_error(e, "plan group readback");
    }
    if (rc) {
      free(p->h_counts);
      free(p->h_offsets);
      delete p;
      return rc;
    }
  }
  *out = p;
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" {

size_t cg_plan_workspace_bytes(int mode, int64_t n, int H, int W,
                               const cg_kernel_desc *kd) {
  if (check_desc(kd, H, W) != CG_OK) return 0;
  cg_plan p;
  memset(&p, 0, sizeof(p));
  p.mode = mode;
  p.kd = *kd;
  p.H = H;
  p.W = W;
  p.n = n;
  p.layers = 1;
  p.gper = kd->G;
  plan_geometry(p);
  return layout_of(p).total;
}

int cg_plan_create(cg_plan **out, int mode, const cg_kernel_desc *kd, int H,
                   int W, const double *uvw, int64_t stride, double lam,
                   const int32_t *kidx, int64_t n, void *workspace,
                   size_t workspace_bytes, int32_t *d_status,
                   cg_stream_t stream) {
  return plan_create_heap(out, mode, kd, H, W, uvw, stride, lam, kidx, 0.0, 0, 1, nullptr, nullptr,
                          0, n, workspace, workspace_bytes, d_status, (cudaStream_t)stream);
}

static void opts_or_default(const cg_plan_opts *o, cg_plan_opts &r) {
  r.layers = 1;
  r.layer = nullptr;
  r.wstep = 0.0;
  r.kmin = 0;
  r.group = nullptr;
  r.ngroups = 0;
  r.tile = 0;
  if (o) r = *o;
  if (r.layers < 1) r.layers = 1;
}

size_t cg_plan_workspace_bytes_ex(int mode, int64_t n, int H, int W, const cg_kernel_desc *kd,
                                  const cg_plan_opts *opts) {
  if (check_desc(kd, H, W) != CG_OK) return 0;
  cg_plan_opts o;
  opts_or_default(opts, o);
  cg_plan p;
  memset(&p, 0, sizeof(p));
  p.mode = mode;
  p.kd = *kd;
  p.H = H;
  p.W = W;
  p.n = n;
  p.layers = o.layers;
  p.gper = o.group ? o.ngroups : kd->G;
  p.tile_req = o.tile;
  plan_geometry(p);
  return layout_of(p).total;
}

int cg_plan_create_ex(cg_plan **out, int mode, const cg_kernel_desc *kd, int H, int W,
                      const double *uvw, int64_t stride, double lam, const int32_t *kidx,
                      int64_t n, const cg_plan_opts *opts, void *workspace,
                      size_t workspace_bytes, int32_t *d_status, cg_stream_t stream) {
  cg_plan_opts o;
  opts_or_default(opts, o);
  return plan_create_heap(out, mode, kd, H, W, uvw, stride, lam, kidx, o.wstep, o.kmin, o.layers,
                          o.layer, o.group, o.ngroups, n, workspace, workspace_bytes, d_status,
                          (cudaStream_t)stream, o.tile);
}

int cg_plan_create_wbins(cg_plan **out, int mode, const cg_kernel_desc *kd, int H, int W,
                         const double *uvw, int64_t stride, double lam, double wstep, int kmin,
                         int64_t n, void *workspace, size_t workspace_bytes,
                         int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(wstep != 0.0, "wstep must be non-zero");
  return plan_create_heap(out, mode, kd, H, W, uvw, stride, lam, nullptr, wstep, kmin, 1, nullptr,
                          nullptr, 0, n, workspace, workspace_bytes, d_status,
                          (cudaStream_t)stream);
}

int cg_plan_destroy(cg_plan *p) {
  if (p) {
    free(p->h_counts);
    free(p->h_offsets);
    delete p;
  }
  return CG_OK;
}

int cg_plan_info(const cg_plan *p, int64_t *info) {
  CG_REQUIRE(p && info, "NULL argument");
  info[0] = p->T;
  info[1] = p->max_items;
  info[2] = p->chunk;
  info[3] = p->nbuckets;
  return CG_OK;
}

int cg_plan_export(const cg_plan *p, int32_t *recs, int32_t *perm, int32_t *counts,
                   cg_stream_t stream) {
  CG_REQUIRE(p, "NULL plan");
  cudaStream_t s = (cudaStream_t)stream;
  if (recs && p->n > 0)
    CG_CUDA(cudaMemcpyAsync(recs, p->recs, (size_t)p->n * sizeof(VisRec),
                            cudaMemcpyDeviceToDevice, s));
  if (perm && p->n > 0)
    CG_CUDA(cudaMemcpyAsync(perm, p->perm, (size_t)p->n * 4, cudaMemcpyDeviceToDevice, s));
  if (counts)
    CG_CUDA(cudaMemcpyAsync(counts, p->counts, (size_t)p->nbuckets * 4, cudaMemcpyDeviceToDevice,
                            s));
  return CG_OK;
}

int cg_w_bins(const double *uvw, int64_t stride, int64_t n, double wstep, int32_t *kidx,
              int32_t *d_minmax, int32_t *h_minmax, int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(n >= 1 && uvw && stride >= 3 && kidx && d_minmax && h_minmax && d_status,
             "bad w_bins arguments");
  CG_REQUIRE(wstep != 0.0, "wstep must be non-zero");
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_minmax_init<<<1, 1, 0, s>>>(d_minmax);
  k_w_bins<<<stride_blocks(n, 256), 256, 0, s>>>(uvw, stride, n, wstep, 1.0 / wstep, kidx,
                                                 d_minmax, d_status);
  k_w_bins_rebase<<<blocks, 256, 0, s>>>(kidx, n, d_minmax);
  CG_LAUNCH("w_bins");
  CG_CUDA(cudaMemcpyAsync(h_minmax, d_minmax, 8, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  return CG_OK;
}

int cg_w_bins_fixed(const double *uvw, int64_t stride, int64_t n, double wstep, int kmin,
                    int nk, int32_t *kidx, int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(n >= 0 && (n == 0 || (uvw && stride >= 3 && kidx && d_status)) && nk >= 1,
             "bad w_bins_fixed arguments");
  CG_REQUIRE(wstep != 0.0, "wstep must be non-zero");
  if (n == 0) return CG_OK;
  k_w_bins_fixed<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      uvw, stride, n, wstep, 1.0 / wstep, kmin, nk, kidx, d_status);
  CG_LAUNCH("w_bins_fixed");
  return CG_OK;
}

size_t cg_compact_keys_workspace_bytes(int nkeys) {
  const int nw = (std::max(nkeys, 1) + 31) / 32;
  return (3 * (size_t)nw + scan_scratch_words(nw) + 64) * 4;
}

int cg_compact_keys(const int32_t *key, int64_t n, int nkeys, int32_t *row, int32_t *key_of_row,
                    int32_t *h_nrows, void *ws, size_t ws_bytes, int32_t *d_status,
                    cg_stream_t stream) {
  CG_REQUIRE(nkeys >= 1 && h_nrows && d_status && (n == 0 || (key && row && key_of_row)),
             "bad compact_keys arguments");
  if (!ws || ws_bytes < cg_compact_keys_workspace_bytes(nkeys))
    return set_error(CG_ERR_WORKSPACE, "compact_keys needs %zu workspace bytes",
                     cg_compact_keys_workspace_bytes(nkeys));
  cudaStream_t s = (cudaStream_t)stream;
  const int nw = (nkeys + 31) / 32;
  uint32_t *bits = (uint32_t *)ws;
  int32_t *cnt = (int32_t *)(bits + nw), *wpre = cnt + nw, *scratch = wpre + nw;
  CG_CUDA(cudaMemsetAsync(bits, 0, (size_t)nw * 4, s));
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (n > 0)
    k_key_bits<<<stride_blocks(n, 256), 256, nw <= KEY_SMEM_WORDS ? (size_t)nw * 4 : 0, s>>>(
        key, n, nkeys, bits, d_status);
  k_key_popc<<<(nw + 255) / 256, 256, 0, s>>>(bits, nw, cnt);
  CG_LAUNCH("key bits");
  int rc = launch_scan(cnt, wpre, nw, scratch, s);
  if (rc) return rc;
  if (n > 0) k_key_rows<<<blocks, 256, 0, s>>>(key, n, nkeys, bits, wpre, row);
  k_key_of_row<<<(nw + 255) / 256, 256, 0, s>>>(nw, bits, wpre, key_of_row);
  CG_LAUNCH("key rows");
  int32_t last[2];
  CG_CUDA(cudaMemcpyAsync(&last[0], wpre + nw - 1, 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaMemcpyAsync(&last[1], cnt + nw - 1, 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  *h_nrows = last[0] + last[1];
  return CG_OK;
}

int cg_aw_keys(const double *uvw, int64_t stride, const int32_t *a1, const int32_t *a2, int64_t n,
               int nant, double wstep, int kmin, int nbins, int32_t *key, int32_t *d_status,
               cg_stream_t stream) {
  CG_REQUIRE(nant >= 1 && nbins >= 1 && wstep != 0.0 && d_status &&
                 (n == 0 || (uvw && stride >= 3 && a1 && a2 && key)),
             "bad aw_keys arguments");
  CG_REQUIRE((int64_t)nant * nant * nbins < (int64_t)INT32_MAX, "too many AW keys");
  if (n == 0) return CG_OK;
  k_aw_keys<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      uvw, stride, a1, a2, n, nant, wstep, 1.0 / wstep, kmin, nbins, key, d_status);
  CG_LAUNCH("aw keys");
  return CG_OK;
}

int cg_row_keys(const double *uvw, int64_t stride, int64_t n, double wstep, int kmin, int nbins,
                const int32_t *cols, int ncols, const int32_t *col_min, const int32_t *col_range,
                int32_t *key, int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(nbins >= 1 && wstep != 0.0 && d_status && ncols >= 0 && ncols <= 8 &&
                 (ncols == 0 || (col_min && col_range)) &&
                 (n == 0 || (uvw && stride >= 3 && key && (ncols == 0 || cols))),
             "bad row_keys arguments");
  RowKeyCols C;
  C.ncols = ncols;
  int64_t space = nbins;
  for (int c = 0; c < ncols; ++c) {
    CG_REQUIRE(col_range[c] >= 1, "column %d has an empty range", c);
    C.mins[c] = col_min[c];
    C.ranges[c] = col_range[c];
    space *= col_range[c];
    CG_REQUIRE(space < (int64_t)INT32_MAX, "key space of %lld keys or more is too large",
               (long long)space);
  }
  if (n == 0) return CG_OK;
  k_row_keys<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      uvw, stride, n, wstep, 1.0 / wstep, kmin, nbins, cols, C, key, d_status);
  CG_LAUNCH("row keys");
  return CG_OK;
}

int cg_frac_coords(const double *uvw, int64_t stride, double lam, int64_t n,
                   int H, int W, int Q, int32_t *x, int32_t *xf, int32_t *y,
                   int32_t *yf, int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(Q >= 1 && H >= 1 && W >= 1, "bad frac_coords arguments");
  CG_REQUIRE(n == 0 || (uvw && x && xf && y && yf && d_status && stride >= 2),
             "NULL argument");
  if (n == 0) return CG_OK;
  k_frac_coords<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      uvw, stride, lam, n, H, W, Q, axis_const(W, Q, lam), axis_const(H, Q, lam), x, xf, y,
      yf, d_status);
  CG_LAUNCH("frac_coords");
  return CG_OK;
}

}  // extern "C"
