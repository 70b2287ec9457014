// FP32 tiled convolutional gridder (K3) and degridder (K4).
//
// Gridder, replacing convgrid (crocodile/synthesis.py:464-481):
//   grid[y0+dy, x0+dx] += K[g, yf, xf, dy, dx] * v   for each visibility.
// Visibilities arrive sorted by grid tile, and inside a tile by 4x4 sub-tile
// along a Morton curve.  A persistent CTA takes one work item (<= chunk
// visibilities of one tile), accumulates into a shared-memory window of
// (T+S-1)^2 cells and flushes the window to HBM with vectorised float2
// atomics once per item.  Inside the window every cell belongs to one thread
// of a thread group (ownership by position mod S), which keeps a running sum
// in registers while consecutive visibilities hit the same cell and writes it
// back only when the cell changes; spatially sorted visibilities make that
// rare.
//
// Degridder, replacing convdegrid (synthesis.py:484-503):
//   out[i] = sum_{dy,dx} grid[y0+dy, x0+dx] * K[g, yf, xf, dy, dx]
// A persistent CTA stages the item's grid window in shared memory; one warp
// per visibility pair sums the S*S taps (fixed per lane) and reduces with
// shuffles.
#include <algorithm>

#include "cg_internal.cuh"
#include "tiled.cuh"

namespace cg {

// ---------------------------------------------------------------- gridder
static constexpr int GRID_STAGE = 256;  // visibilities staged per batch

// A thread group has S * ceil(S / R) threads: thread (tx, yg) owns window
// column residue tx and row residues yg*R + r (r < R), i.e. for every
// visibility it updates the R cells of its residues inside the footprint,
// decoding the visibility once for R updates.  With one group per CTA each
// window cell has a single owner and the running sums are written back with
// plain read-modify-writes; with several groups sharing the window
// (shared = true) the write-backs are shared-memory atomics.
// mode 0: vis, 1: vis * weight, 2: weight only (the PSF pass).
template <bool SEP, int R>
__global__ void __launch_bounds__(256) k_grid_tiled(
    TiledArgs A, int gsize, int ngroups, int mode, bool shared,
    const float2 *__restrict__ ktab, const float2 *__restrict__ vis,
    const float *__restrict__ weight, float2 *__restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  if (status_failed(A.status)) return;
  const int S = A.S, SS = S * S, pitch = A.pitch;
  float2 *win = (float2 *)smem;
  int *s_base = (int *)(win + (size_t)pitch * A.win);
  int *s_mxy = s_base + GRID_STAGE;
  long long *s_k0 = (long long *)(s_mxy + GRID_STAGE);
  long long *s_k1 = s_k0 + GRID_STAGE;
  float2 *s_v = (float2 *)(s_k1 + GRID_STAGE);

  const int tid = threadIdx.x;
  const int gpad = (gsize + 31) & ~31;  // groups start on warp boundaries
  const int grp = tid / gpad, lt = tid - grp * gpad;
  const bool active = grp < ngroups && lt < gsize;
  const int tx = lt % S, yg = lt / S;
  const int wcells = A.win * A.win;
  const long long KSZ = (long long)A.Q * A.Q * SS;

  int it;
  while ((it = next_item(A, &s_item)) >= 0) {
    const WorkItem w = A.items[it];
    const TileOrigin org = tile_origin(A, w.tile);
    const int wx0 = org.wx0, wy0 = org.wy0;
    for (int c = tid; c < pitch * A.win; c += blockDim.x) win[c] = make_float2(0.f, 0.f);

    int cur[R];
    float2 acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      cur[r] = -1;
      acc[r] = make_float2(0.f, 0.f);
    }
    for (int b = 0; b < w.count; b += GRID_STAGE) {
      const int nb = min(GRID_STAGE, w.count - b);
      __syncthreads();
      for (int j = tid; j < nb; j += blockDim.x) {
        const int pos = w.start + b + j;
        const VisRec rec = A.recs[pos];
        const int lx0 = rec.x0 - wx0, ly0 = rec.y0 - wy0;
        s_base[j] = ly0 * pitch + lx0;
        s_mxy[j] = (lx0 % S) | ((ly0 % S) << 16);
        if (SEP) {
          s_k0[j] = (long long)rec.k0 * S;
          s_k1[j] = (long long)rec.k1 * S;
        } else {
          s_k0[j] = (long long)rec.k0 * KSZ + (long long)rec.k1 * SS;
        }
        const int src = A.perm[pos];
        float2 v;
        if (mode == 2) {
          v = make_float2(weight[src], 0.f);
        } else {
          v = vis[src];
          if (mode == 1) {
            const float wt = weight[src];
            v.x *= wt;
            v.y *= wt;
          }
        }
        s_v[j] = v;
      }
      __syncthreads();
      if (active) {
        for (int j = grp; j < nb; j += ngroups) {
          const int base = s_base[j], mxy = s_mxy[j];
          const float2 v = s_v[j];
          int dx = tx - (mxy & 0xffff);
          dx += (dx >> 31) & S;
          const int my = mxy >> 16;
          const int cb = base + dx;
          const float2 *kp;
          float2 kx = make_float2(0.f, 0.f);
          if (SEP) {
            kp = ktab + s_k0[j];
            kx = __ldg(&ktab[s_k1[j] + dx]);
          } else {
            kp = ktab + s_k0[j] + dx;
          }
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int res = yg * R + r;
            if (res < S) {
              int dy = res - my;
              dy += (dy >> 31) & S;
              const int cell = cb + dy * pitch;
              const float2 k = SEP ? cmul(__ldg(&kp[dy]), kx) : __ldg(&kp[dy * S]);
              if (cell != cur[r]) {
                if (cur[r] >= 0) {
                  if (shared) {
                    atomicAdd(&win[cur[r]].x, acc[r].x);
                    atomicAdd(&win[cur[r]].y, acc[r].y);
                  } else {
                    float2 o = win[cur[r]];
                    o.x += acc[r].x;
                    o.y += acc[r].y;
                    win[cur[r]] = o;
                  }
                }
                cur[r] = cell;
                acc[r] = make_float2(0.f, 0.f);
              }
              cfma(acc[r], k, v);
            }
          }
        }
      }
    }
    if (active) {
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (cur[r] >= 0) {
          if (shared) {
            atomicAdd(&win[cur[r]].x, acc[r].x);
            atomicAdd(&win[cur[r]].y, acc[r].y);
          } else {
            float2 o = win[cur[r]];
            o.x += acc[r].x;
            o.y += acc[r].y;
            win[cur[r]] = o;
          }
        }
    }
    __syncthreads();
    for (int c = tid; c < wcells; c += blockDim.x) {
      const int r = c / A.win, q = c - r * A.win;
      const float2 val = win[r * pitch + q];
      if (val.x != 0.f || val.y != 0.f) {
        const int gy = wy0 + r, gx = wx0 + q;
        if (gy < A.H && gx < A.W) atomicAdd(&grid[org.layer_off + (size_t)gy * A.W + gx], val);
      }
    }
  }
}

// Warp layout: one warp per visibility; lane l adds taps l, l+32, ... of the
// S x S footprint (kernel taps read coalesced) into the shared window with
// shared-memory atomic adds, so the warps of a CTA share one window freely.
template <bool SEP, int MAXT>
__global__ void __launch_bounds__(256) k_grid_warp(
    TiledArgs A, int mode, const float2 *__restrict__ ktab, const float2 *__restrict__ vis,
    const float *__restrict__ weight, float2 *__restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  if (status_failed(A.status)) return;
  const int S = A.S, SS = S * S, pitch = A.pitch;
  float2 *win = (float2 *)smem;
  int *s_base = (int *)(win + (size_t)pitch * A.win);
  long long *s_k0 = (long long *)(s_base + 2 * GRID_STAGE);
  long long *s_k1 = s_k0 + GRID_STAGE;
  float2 *s_v = (float2 *)(s_k1 + GRID_STAGE);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int wcells = A.win * A.win;
  const long long KSZ = (long long)A.Q * A.Q * SS;

  int soff[MAXT], kdy[MAXT], kdx[MAXT];
#pragma unroll
  for (int i = 0; i < MAXT; ++i) {
    const int t = lane + 32 * i;
    const int dy = t / S, dx = t - (t / S) * S;
    soff[i] = (t < SS) ? dy * pitch + dx : -1;
    kdy[i] = dy;
    kdx[i] = dx;
  }

  int it;
  while ((it = next_item(A, &s_item)) >= 0) {
    const WorkItem w = A.items[it];
    const TileOrigin org = tile_origin(A, w.tile);
    const int wx0 = org.wx0, wy0 = org.wy0;
    for (int c = tid; c < pitch * A.win; c += blockDim.x) win[c] = make_float2(0.f, 0.f);
    for (int b = 0; b < w.count; b += GRID_STAGE) {
      const int nb = min(GRID_STAGE, w.count - b);
      __syncthreads();
      for (int j = tid; j < nb; j += blockDim.x) {
        const int pos = w.start + b + j;
        const VisRec rec = A.recs[pos];
        s_base[j] = (rec.y0 - wy0) * pitch + (rec.x0 - wx0);
        if (SEP) {
          s_k0[j] = (long long)rec.k0 * S;
          s_k1[j] = (long long)rec.k1 * S;
        } else {
          s_k0[j] = (long long)rec.k0 * KSZ + (long long)rec.k1 * SS;
        }
        const int src = A.perm[pos];
        float2 v;
        if (mode == 2) {
          v = make_float2(weight[src], 0.f);
        } else {
          v = vis[src];
          if (mode == 1) {
            const float wt = weight[src];
            v.x *= wt;
            v.y *= wt;
          }
        }
        s_v[j] = v;
      }
      __syncthreads();
      // Software pipeline: the taps of the warp's next visibility are loaded
      // before the current one's are added, so two slices are in flight.
      float2 k[MAXT];
      auto load_taps = [&](int j) {
        const float2 *kk = ktab + s_k0[j];
        const float2 *kx = ktab + s_k1[j];
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (soff[i] >= 0)
            k[i] = SEP ? cmul(__ldg(&kk[kdy[i]]), __ldg(&kx[kdx[i]])) : __ldg(&kk[lane + 32 * i]);
      };
      int j = warp;
      if (j < nb) load_taps(j);
      for (; j < nb; j += nwarps) {
        float2 kc[MAXT];
#pragma unroll
        for (int i = 0; i < MAXT; ++i) kc[i] = k[i];
        if (j + nwarps < nb) load_taps(j + nwarps);
        const int base = s_base[j];
        const float2 v = s_v[j];
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (soff[i] >= 0) {
            const float2 u = cmul(kc[i], v);
            atomicAdd(&win[base + soff[i]].x, u.x);
            atomicAdd(&win[base + soff[i]].y, u.y);
          }
      }
    }
    __syncthreads();
    for (int c = tid; c < wcells; c += blockDim.x) {
      const int r = c / A.win, q = c - r * A.win;
      const float2 val = win[r * pitch + q];
      if (val.x != 0.f || val.y != 0.f) {
        const int gy = wy0 + r, gx = wx0 + q;
        if (gy < A.H && gx < A.W) atomicAdd(&grid[org.layer_off + (size_t)gy * A.W + gx], val);
      }
    }
  }
}

// ---------------------------------------------------------------- fused pass
// Degridding and gridding of the same visibilities in one traversal: every
// kernel tap is read once for both directions.  Per work item the CTA stages
// the input grid's window (for degridding) and accumulates an output window;
// one warp per visibility forms out[i] = sum(grid_in[footprint] * K) and adds
// K * u into the output window, with u = vis_in[i] (mode 0) or the residual
// vis_in[i] - out[i] (mode 1, the predict-subtract-invert step of an imaging
// major cycle).  Both windows are conflict-free thanks to the plan's pitch.
template <bool SEP, int MAXT>
__global__ void __launch_bounds__(256) k_degrid_grid_warp(
    TiledArgs A, int mode, const float2 *__restrict__ ktab, const float2 *__restrict__ grid_in,
    const float2 *__restrict__ vis_in, float2 *__restrict__ vis_out,
    float2 *__restrict__ grid_out) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  if (status_failed(A.status)) return;
  const int S = A.S, SS = S * S, pitch = A.pitch;
  const size_t wsz = (size_t)pitch * A.win;
  float2 *win_in = (float2 *)smem;
  float2 *win_out = win_in + wsz;
  int *s_base = (int *)(win_out + wsz);
  int *s_dst = s_base + GRID_STAGE;
  long long *s_k0 = (long long *)(s_dst + GRID_STAGE);
  long long *s_k1 = s_k0 + GRID_STAGE;
  float2 *s_v = (float2 *)(s_k1 + GRID_STAGE);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int wcells = A.win * A.win;
  const long long KSZ = (long long)A.Q * A.Q * SS;

  int soff[MAXT], kdy[MAXT], kdx[MAXT];
#pragma unroll
  for (int i = 0; i < MAXT; ++i) {
    const int t = lane + 32 * i;
    const int dy = t / S, dx = t - (t / S) * S;
    soff[i] = (t < SS) ? dy * pitch + dx : -1;
    kdy[i] = dy;
    kdx[i] = dx;
  }

  int it;
  while ((it = next_item(A, &s_item)) >= 0) {
    const WorkItem w = A.items[it];
    const TileOrigin org = tile_origin(A, w.tile);
    const int wx0 = org.wx0, wy0 = org.wy0;
    for (int c = tid; c < (int)wsz; c += blockDim.x) win_out[c] = make_float2(0.f, 0.f);
    for (int c = tid; c < wcells; c += blockDim.x) {
      const int r = c / A.win, q = c - r * A.win;
      const int gy = wy0 + r, gx = wx0 + q;
      win_in[r * pitch + q] = (gy < A.H && gx < A.W)
                                  ? __ldg(&grid_in[org.layer_off + (size_t)gy * A.W + gx])
                                  : make_float2(0.f, 0.f);
    }
    for (int b = 0; b < w.count; b += GRID_STAGE) {
      const int nb = min(GRID_STAGE, w.count - b);
      __syncthreads();
      for (int j = tid; j < nb; j += blockDim.x) {
        const int pos = w.start + b + j;
        const VisRec rec = A.recs[pos];
        s_base[j] = (rec.y0 - wy0) * pitch + (rec.x0 - wx0);
        if (SEP) {
          s_k0[j] = (long long)rec.k0 * S;
          s_k1[j] = (long long)rec.k1 * S;
        } else {
          s_k0[j] = (long long)rec.k0 * KSZ + (long long)rec.k1 * SS;
        }
        const int src = A.perm[pos];
        s_dst[j] = src;
        s_v[j] = vis_in ? vis_in[src] : make_float2(0.f, 0.f);
      }
      __syncthreads();
      float2 k[MAXT];
      auto load_taps = [&](int j) {
        const float2 *kk = ktab + s_k0[j];
        const float2 *kx = ktab + s_k1[j];
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (soff[i] >= 0)
            k[i] = SEP ? cmul(__ldg(&kk[kdy[i]]), __ldg(&kx[kdx[i]])) : __ldg(&kk[lane + 32 * i]);
      };
      int j = warp;
      if (j < nb) load_taps(j);
      for (; j < nb; j += nwarps) {
        float2 kc[MAXT];
#pragma unroll
        for (int i = 0; i < MAXT; ++i) kc[i] = k[i];
        if (j + nwarps < nb) load_taps(j + nwarps);
        const int base = s_base[j];
        float2 sum = make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (soff[i] >= 0) cfma(sum, win_in[base + soff[i]], kc[i]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          sum.x += __shfl_xor_sync(0xffffffffu, sum.x, o);
          sum.y += __shfl_xor_sync(0xffffffffu, sum.y, o);
        }
        if (lane == 0 && vis_out) vis_out[s_dst[j]] = sum;
        float2 u = s_v[j];
        if (mode == 1) {
          u.x -= sum.x;
          u.y -= sum.y;
        }
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (soff[i] >= 0) {
            const float2 c = cmul(kc[i], u);
            atomicAdd(&win_out[base + soff[i]].x, c.x);
            atomicAdd(&win_out[base + soff[i]].y, c.y);
          }
      }
    }
    __syncthreads();
    for (int c = tid; c < wcells; c += blockDim.x) {
      const int r = c / A.win, q = c - r * A.win;
      const float2 val = win_out[r * pitch + q];
      if (val.x != 0.f || val.y != 0.f) {
        const int gy = wy0 + r, gx = wx0 + q;
        if (gy < A.H && gx < A.W)
          atomicAdd(&grid_out[org.layer_off + (size_t)gy * A.W + gx], val);
      }
    }
  }
}

// ---------------------------------------------------------------- degridder
// Each warp sums the S*S taps of V visibilities at a time (taps fixed per
// lane, interleaved so that all V visibilities' kernel loads are in flight
// together) and reduces them with shuffles.
template <bool SEP, int MAXT, int V>
__global__ void __launch_bounds__(256) k_degrid_tiled(
    TiledArgs A, const float2 *__restrict__ ktab, const float2 *__restrict__ grid,
    float2 *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  if (status_failed(A.status)) return;
  const int S = A.S, SS = S * S, pitch = A.pitch;
  float2 *win = (float2 *)smem;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const long long KSZ = (long long)A.Q * A.Q * SS;

  int soff[MAXT], kdy[MAXT], kdx[MAXT];
#pragma unroll
  for (int i = 0; i < MAXT; ++i) {
    const int t = lane + 32 * i;
    const int dy = t / S, dx = t - (t / S) * S;
    soff[i] = (t < SS) ? dy * pitch + dx : -1;
    kdy[i] = dy;
    kdx[i] = dx;
  }

  int it;
  while ((it = next_item(A, &s_item)) >= 0) {
    const WorkItem w = A.items[it];
    const TileOrigin org = tile_origin(A, w.tile);
    const int wx0 = org.wx0, wy0 = org.wy0;
    for (int c = threadIdx.x; c < A.win * A.win; c += blockDim.x) {
      const int r = c / A.win, q = c - r * A.win;
      const int gy = wy0 + r, gx = wx0 + q;
      win[r * pitch + q] = (gy < A.H && gx < A.W)
                               ? __ldg(&grid[org.layer_off + (size_t)gy * A.W + gx])
                               : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int j = V * warp; j < w.count; j += V * nwarps) {
      int base[V];
      const float2 *kk[V], *ky[V], *kx[V];
      float2 sum[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        // past the item's end: repeat its first visibility (summed, not written)
        const VisRec r = A.recs[w.start + (j + v < w.count ? j + v : j)];
        base[v] = (r.y0 - wy0) * pitch + (r.x0 - wx0);
        kk[v] = ktab + (SEP ? 0 : (long long)r.k0 * KSZ + (long long)r.k1 * SS);
        ky[v] = ktab + (long long)r.k0 * S;
        kx[v] = ktab + (long long)r.k1 * S;
        sum[v] = make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int i = 0; i < MAXT; ++i)
        if (soff[i] >= 0) {
          float2 k[V];
#pragma unroll
          for (int v = 0; v < V; ++v)
            k[v] = SEP ? cmul(__ldg(&ky[v][kdy[i]]), __ldg(&kx[v][kdx[i]]))
                       : __ldg(&kk[v][lane + 32 * i]);
#pragma unroll
          for (int v = 0; v < V; ++v) cfma(sum[v], win[base[v] + soff[i]], k[v]);
        }
#pragma unroll
      for (int v = 0; v < V; ++v)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          sum[v].x += __shfl_xor_sync(0xffffffffu, sum[v].x, o);
          sum[v].y += __shfl_xor_sync(0xffffffffu, sum[v].y, o);
        }
      if (lane == 0) {
#pragma unroll
        for (int v = 0; v < V; ++v)
          if (j + v < w.count) out[A.perm[w.start + j + v]] = sum[v];
      }
    }
  }
}


// Row residues per thread: the smallest R in {2, 3, 4} dividing S, else 4
// (1 for S = 1); overridable by the tuning.
static int pick_rows(int S) {
  const cg_tuning t = tuning();
  if (t.rows > 0) return t.rows;
  if (S == 1) return 1;
  for (int r = 2; r <= 4; ++r)
    if (S % r == 0) return r;
  return S < 4 ? S : 4;
}

template <bool SEP>
static void *grid_kernel_for(int R) {
  switch (R) {
    case 1: return (void *)k_grid_tiled<SEP, 1>;
    case 2: return (void *)k_grid_tiled<SEP, 2>;
    case 3: return (void *)k_grid_tiled<SEP, 3>;
    case 4: return (void *)k_grid_tiled<SEP, 4>;
    case 5: return (void *)k_grid_tiled<SEP, 5>;
    case 6: return (void *)k_grid_tiled<SEP, 6>;
    case 8: return (void *)k_grid_tiled<SEP, 8>;
    default: return nullptr;
  }
}

// Sparse gridder: for stacks of grids holding few visibilities per tile (the
// sub-grids of w-towers), where staging and flushing a window per work item
// costs more than the visibilities' own taps.  No shared memory: each warp
// takes work items in turn, loads 32 records at a time (one per lane) and, for
// each visibility, lane l adds taps l + 32 i straight into the grid with
// float2 atomics.  Full occupancy hides the latency of the small items.
template <bool SEP, int MAXT>
__global__ void __launch_bounds__(256) k_grid_sparse(TiledArgs A, const float2 *__restrict__ ktab,
                                                     const float2 *__restrict__ vis,
                                                     float2 *__restrict__ grid) {
  if (status_failed(A.status)) return;
  const int S = A.S, SS = S * S;
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const long long KSZ = (long long)A.Q * A.Q * SS;
  int tdy[MAXT], tdx[MAXT];
#pragma unroll
  for (int i = 0; i < MAXT; ++i) {
    const int t = lane + 32 * i;
    tdy[i] = t / S;
    tdx[i] = t - tdy[i] * S;
  }
  const int nitems = *A.nitems;
  for (int64_t it = gw; it < nitems; it += nw) {
    const WorkItem w = A.items[it];
    const TileOrigin org = tile_origin(A, w.tile);
    float2 *g0 = grid + org.layer_off;
    for (int b = 0; b < w.count; b += 32) {
      const int nb = min(32, w.count - b);
      VisRec r = {0, 0, 0, 0};
      float2 v = make_float2(0.f, 0.f);
      if (lane < nb) {
        r = A.recs[w.start + b + lane];
        v = vis[A.perm[w.start + b + lane]];
      }
      for (int q = 0; q < nb; ++q) {
        const int x0 = __shfl_sync(0xffffffffu, r.x0, q), y0 = __shfl_sync(0xffffffffu, r.y0, q);
        const int k0 = __shfl_sync(0xffffffffu, r.k0, q), k1 = __shfl_sync(0xffffffffu, r.k1, q);
        const float2 u = make_float2(__shfl_sync(0xffffffffu, v.x, q),
                                     __shfl_sync(0xffffffffu, v.y, q));
        const float2 *kk = SEP ? ktab + (long long)k0 * S : ktab + (long long)k0 * KSZ + (long long)k1 * SS;
        const float2 *kx = ktab + (long long)k1 * S;
        float2 *gp = g0 + (size_t)y0 * A.W + x0;
#pragma unroll
        for (int i = 0; i < MAXT; ++i) {
          if (lane + 32 * i < SS) {
            const float2 k = SEP ? cmul(__ldg(&kk[tdy[i]]), __ldg(&kx[tdx[i]])) : __ldg(&kk[lane + 32 * i]);
            atomicAdd(&gp[(size_t)tdy[i] * A.W + tdx[i]], cmul(k, u));
          }
        }
      }
    }
  }
}

template <bool SEP>
static void *grid_warp_kernel_for(int maxt) {
  switch (maxt) {
    case 1: return (void *)k_grid_warp<SEP, 1>;
    case 2: return (void *)k_grid_warp<SEP, 2>;
    case 4: return (void *)k_grid_warp<SEP, 4>;
    case 8: return (void *)k_grid_warp<SEP, 8>;
    case 16: return (void *)k_grid_warp<SEP, 16>;
    case 32: return (void *)k_grid_warp<SEP, 32>;
    default: return nullptr;
  }
}

static int grid_launch(const cg_plan *p, const void *ktab, const void *vis,
                       const float *weight, int mode, void *grid, cudaStream_t s) {
  CG_REQUIRE(p && p->mode == CG_PLAN_TILED, "cg_grid needs a CG_PLAN_TILED plan");
  if (p->n == 0) return CG_OK;
  CG_REQUIRE(ktab && grid, "NULL kernel table or grid");
  CG_REQUIRE(mode == 2 || vis, "NULL visibilities");
  CG_REQUIRE(mode == 0 || weight, "NULL weights");
  TiledArgs A = tiled_args(p);
  const int S = p->kd.S;
  const cg_tuning t = tuning();
  const float2 *kt = (const float2 *)ktab;
  const float2 *vv = (const float2 *)vis;
  float2 *gg = (float2 *)grid;
  const size_t wbytes = (size_t)p->pitch * p->win * sizeof(float2);
  void *fn = nullptr;
  int threads = 0;
  size_t smem = 0;
  void *args[12];
  int gsize = 0, ngroups = 0;
  bool shared = false;
  const int layout = layout_for(p->kd);
  if (layout == CG_LAYOUT_LANE)
    return lane_launch(p, kt, vv, weight, mode, gg, nullptr, nullptr, 0, false, s);
  if (layout != CG_LAYOUT_OWNER) {
    const int need = (S * S + 31) / 32;
    int maxt = 1;
    while (maxt < need) maxt *= 2;
    fn = p->kd.sep ? grid_warp_kernel_for<true>(maxt) : grid_warp_kernel_for<false>(maxt);
    CG_REQUIRE(fn, "no warp gridder for support %d", S);
    threads = 32 * (t.groups > 0 ? std::min(t.groups, 8) : 8);
    smem = wbytes + (size_t)GRID_STAGE * (8 + 8 + 8 + 8);
    args[0] = &A;
    args[1] = &mode;
    args[2] = &kt;
    args[3] = &vv;
    args[4] = (void *)&weight;
    args[5] = &gg;
  } else {
    int R = t.rows > 0 ? t.rows : pick_rows(S);
    if (R > S) R = S;
    if (R == 7) R = 8;
    gsize = S * ((S + R - 1) / R);
    const int gpad = (gsize + 31) & ~31;
    ngroups = t.groups > 0 ? t.groups : std::max(1, 256 / gpad);
    ngroups = std::max(1, std::min(ngroups, 256 / gpad));
    threads = gpad * ngroups;
    CG_REQUIRE(threads <= 256 && threads > 0,
               "gridder thread group too large (S=%d, rows=%d)", S, R);
    smem = wbytes + (size_t)GRID_STAGE * (4 + 4 + 8 + 8 + 8);
    fn = p->kd.sep ? grid_kernel_for<true>(R) : grid_kernel_for<false>(R);
    CG_REQUIRE(fn, "no gridder for %d rows per thread", R);
    shared = ngroups > 1;
    args[0] = &A;
    args[1] = &gsize;
    args[2] = &ngroups;
    args[3] = &mode;
    args[4] = &shared;
    args[5] = &kt;
    args[6] = &vv;
    args[7] = (void *)&weight;
    args[8] = &gg;
  }
  CG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  CG_REQUIRE(per_sm > 0, "gridder does not fit on an SM (smem %zu)", smem);
  int64_t blocks = std::min<int64_t>((int64_t)per_sm * num_sms(), p->max_items);
  CG_CUDA(cudaMemsetAsync(p->ticket, 0, sizeof(int32_t), s));
  CG_CUDA(cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(threads), args, smem, s));
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" {

int cg_grid(const cg_plan *p, const void *ktab, const void *vis, void *grid,
            cg_stream_t stream) {
  return grid_launch(p, ktab, vis, nullptr, 0, grid, (cudaStream_t)stream);
}

int cg_grid_weighted(const cg_plan *p, const void *ktab, const void *vis,
                     const float *weight, void *grid, cg_stream_t stream) {
  return grid_launch(p, ktab, vis, weight, vis ? 1 : 2, grid, (cudaStream_t)stream);
}

int cg_grid_sparse(const cg_plan *p, const void *ktab, const void *vis, void *grid,
                   cg_stream_t stream) {
  CG_REQUIRE(p && p->mode == CG_PLAN_TILED, "cg_grid_sparse needs a CG_PLAN_TILED plan");
  if (p->n == 0) return CG_OK;
  CG_REQUIRE(ktab && vis && grid, "NULL argument");
  const int SS = p->kd.S * p->kd.S;
  const int need = (SS + 31) / 32;
  void (*fn)(TiledArgs, const float2 *, const float2 *, float2 *) = nullptr;
#define PICK(M)                                                                \
  if (!fn && need <= M) fn = p->kd.sep ? k_grid_sparse<true, M> : k_grid_sparse<false, M>;
  PICK(1) PICK(2) PICK(4) PICK(8) PICK(16) PICK(32)
#undef PICK
  CG_REQUIRE(fn, "support too large for the sparse gridder");
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0));
  const int64_t blocks = std::max<int64_t>(
      1, std::min<int64_t>((int64_t)std::max(per_sm, 1) * num_sms(), (p->max_items + 7) / 8));
  fn<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(tiled_args(p), (const float2 *)ktab,
                                                         (const float2 *)vis, (float2 *)grid);
  CG_LAUNCH("sparse grid");
  return CG_OK;
}

int cg_degrid(const cg_plan *p, const void *ktab, const void *grid, void *out,
              cg_stream_t stream) {
  CG_REQUIRE(p && p->mode == CG_PLAN_TILED, "cg_degrid needs a CG_PLAN_TILED plan");
  if (p->n == 0) return CG_OK;
  CG_REQUIRE(ktab && grid && out, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  const int dvis = tuning().dvis;
  // dvis 1: lane-layout plans through the lane kernel's degridding traversal
  // (slices by bulk copies, no output grid); everything else through the
  // tiled degridder, which is the faster of the two at S 16
  if (dvis == 1 && layout_for(p->kd) == CG_LAYOUT_LANE)
    return lane_launch(p, (const float2 *)ktab, nullptr, nullptr, 0, nullptr,
                       (const float2 *)grid, (float2 *)out, 0, true, s);
  // dvis 3: the shared window with per-warp slice rings, where the table streams
  if (dvis == 3) {
    const int rc = ring_degrid_launch(p, (const float2 *)ktab, (const float2 *)grid,
                                      (float2 *)out, s);
    if (rc != CG_ERR_ARG) return rc;
  }
  TiledArgs A = tiled_args(p);
  const int SS = p->kd.S * p->kd.S;
  const int need = (SS + 31) / 32;
  const int threads = 256;
  const size_t smem = (size_t)p->pitch * p->win * sizeof(float2);
  const bool four = dvis == 4;  // visibilities per warp step: 4, or 2
  void (*fn)(TiledArgs, const float2 *, const float2 *, float2 *) = nullptr;
#define PICK(M)                                                                \
  if (!fn && need <= M)                                                        \
    fn = four ? (p->kd.sep ? k_degrid_tiled<true, M, 4> : k_degrid_tiled<false, M, 4>)  \
              : (p->kd.sep ? k_degrid_tiled<true, M, 2> : k_degrid_tiled<false, M, 2>);
  PICK(1) PICK(2) PICK(4) PICK(8) PICK(16) PICK(32)
#undef PICK
  CG_REQUIRE(fn, "support too large for the degridder");
  CG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  CG_REQUIRE(per_sm > 0, "degridder does not fit on an SM (smem %zu)", smem);
  int64_t blocks = std::min<int64_t>((int64_t)per_sm * num_sms(), p->max_items);
  CG_CUDA(cudaMemsetAsync(p->ticket, 0, sizeof(int32_t), s));
  fn<<<(unsigned)blocks, threads, smem, s>>>(A, (const float2 *)ktab, (const float2 *)grid,
                                              (float2 *)out);
  CG_LAUNCH("degrid");
  return CG_OK;
}

int cg_degrid_grid(const cg_plan *p, const void *ktab, const void *grid_in, const void *vis_in,
                   int residual, void *vis_out, void *grid_out, cg_stream_t stream) {
  CG_REQUIRE(p && p->mode == CG_PLAN_TILED, "cg_degrid_grid needs a CG_PLAN_TILED plan");
  if (p->n == 0) return CG_OK;
  CG_REQUIRE(ktab && grid_in && grid_out, "NULL kernel table or grid");
  CG_REQUIRE(vis_in || !residual, "the residual mode needs input visibilities");
  CG_REQUIRE(grid_in != grid_out, "input and output grids must differ");
  cudaStream_t s = (cudaStream_t)stream;
  const int S = p->kd.S;
  const cg_tuning t = tuning();
  if (layout_for(p->kd) == CG_LAYOUT_LANE)
    return lane_launch(p, (const float2 *)ktab, (const float2 *)vis_in, nullptr, 0,
                       (float2 *)grid_out, (const float2 *)grid_in, (float2 *)vis_out, residual,
                       true, s);
  TiledArgs A = tiled_args(p);
  const int need = (S * S + 31) / 32;
  int maxt = 1;
  while (maxt < need) maxt *= 2;
  void *fn = nullptr;
#define PICK(M)                                                                      \
  if (maxt == M) fn = p->kd.sep ? (void *)k_degrid_grid_warp<true, M>                 \
                                : (void *)k_degrid_grid_warp<false, M>;
  PICK(1) PICK(2) PICK(4) PICK(8) PICK(16) PICK(32)
#undef PICK
  CG_REQUIRE(fn, "no fused kernel for support %d", S);
  const int threads = 32 * (t.groups > 0 ? std::min(t.groups, 8) : 8);
  const size_t smem = 2 * (size_t)p->pitch * p->win * sizeof(float2) +
                      (size_t)GRID_STAGE * (4 + 4 + 8 + 8 + 8);
  CG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  CG_REQUIRE(per_sm > 0, "fused kernel does not fit on an SM (smem %zu)", smem);
  int64_t blocks = std::min<int64_t>((int64_t)per_sm * num_sms(), p->max_items);
  CG_CUDA(cudaMemsetAsync(p->ticket, 0, sizeof(int32_t), s));
  int mode = residual ? 1 : 0;
  const float2 *kt = (const float2 *)ktab, *gi = (const float2 *)grid_in,
               *vi = (const float2 *)vis_in;
  float2 *vo = (float2 *)vis_out, *go = (float2 *)grid_out;
  void *args[] = {&A, &mode, &kt, &gi, &vi, &vo, &go};
  CG_CUDA(cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(threads), args, smem, s));
  return CG_OK;
}

}  // extern "C"
