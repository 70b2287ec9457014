// FP32 tiled convolutional gridder (K3) and degridder (K4).
//
// Gridder, replacing convgrid (crocodile/synthesis.py:464-481):
//   grid[y0+dy, x0+dx] += K[g, yf, xf, dy, dx] * v   for each visibility.
// Visibilities arrive sorted by the grid tile of their footprint origin.  A
// persistent CTA takes one work item (<= chunk visibilities of one tile),
// accumulates into a shared-memory window of (T+S-1)^2 cells and flushes the
// window to HBM with vectorised float2 atomics once per item.  Inside the
// window, thread (tx, ty) of the S x S thread group owns every cell whose
// window coordinates are congruent to (tx, ty) mod S: each visibility's
// footprint holds exactly one such cell, so every thread updates exactly
// one cell per visibility, no two threads ever touch the same cell, and the
// running sum stays in registers while consecutive visibilities hit the
// same cell (it is written back to shared memory only when the cell
// changes).  No shared-memory atomics are needed.
//
// Degridder, replacing convdegrid (synthesis.py:484-503):
//   out[i] = sum_{dy,dx} grid[y0+dy, x0+dx] * K[g, yf, xf, dy, dx]
// A persistent CTA stages the item's grid window in shared memory; one warp
// per visibility sums its S*S taps (fixed per lane) and reduces with shuffles.
#include <algorithm>

#include "cg_internal.cuh"

namespace cg {

struct TiledArgs {
  const VisRec *recs;
  const int32_t *perm;
  const WorkItem *items;
  const int32_t *nitems;
  int32_t *ticket;
  const int32_t *status;
  int H, W, S, Q, T, ntx, win, pitch;
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ void cfma(float2 &acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

__device__ __forceinline__ bool status_failed(const int32_t *st) {
  return (st[ST_RANGE] | st[ST_BOUNDS] | st[ST_INDEX]) != 0;
}

// Next work item for the whole CTA, or -1.
__device__ __forceinline__ int next_item(const TiledArgs &A, int *s_item) {
  __syncthreads();
  if (threadIdx.x == 0) *s_item = atomicAdd(A.ticket, 1);
  __syncthreads();
  int it = *s_item;
  return it < *A.nitems ? it : -1;
}

// ---------------------------------------------------------------- gridder
static constexpr int GRID_STAGE = 256;  // visibilities staged per batch

template <bool SEP, int MODE>  // MODE 0: vis, 1: vis * weight, 2: weight only
__global__ void __launch_bounds__(1024) k_grid_tiled(
    TiledArgs A, const float2 *__restrict__ ktab, const float2 *__restrict__ vis,
    const float *__restrict__ weight, float2 *__restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  if (status_failed(A.status)) return;
  const int S = A.S, SS = S * S, pitch = A.pitch;
  float2 *win = (float2 *)smem;
  int *s_lxy = (int *)(win + (size_t)pitch * A.win);
  int *s_mxy = s_lxy + GRID_STAGE;
  long long *s_k0 = (long long *)(s_mxy + GRID_STAGE);
  long long *s_k1 = s_k0 + GRID_STAGE;
  float2 *s_v = (float2 *)(s_k1 + GRID_STAGE);

  const int tid = threadIdx.x;
  const bool active = tid < SS;
  const int tx = tid % S, ty = tid / S;
  const int wcells = A.win * A.win;
  const long long KSZ = (long long)A.Q * A.Q * SS;

  int it;
  while ((it = next_item(A, &s_item)) >= 0) {
    const WorkItem w = A.items[it];
    const int wx0 = (w.tile % A.ntx) * A.T, wy0 = (w.tile / A.ntx) * A.T;
    for (int c = tid; c < pitch * A.win; c += blockDim.x) win[c] = make_float2(0.f, 0.f);

    int cur = -1;
    float2 acc = make_float2(0.f, 0.f);
    for (int b = 0; b < w.count; b += GRID_STAGE) {
      const int nb = min(GRID_STAGE, w.count - b);
      __syncthreads();
      for (int j = tid; j < nb; j += blockDim.x) {
        const int pos = w.start + b + j;
        const VisRec r = A.recs[pos];
        const int lx0 = r.x0 - wx0, ly0 = r.y0 - wy0;
        s_lxy[j] = lx0 | (ly0 << 16);
        s_mxy[j] = (lx0 % S) | ((ly0 % S) << 16);
        if (SEP) {
          s_k0[j] = (long long)r.k0 * S;
          s_k1[j] = (long long)r.k1 * S;
        } else {
          s_k0[j] = (long long)r.k0 * KSZ + (long long)r.k1 * SS;
          s_k1[j] = 0;
        }
        const int src = A.perm[pos];
        float2 v;
        if (MODE == 2) {
          v = make_float2(weight[src], 0.f);
        } else {
          v = vis[src];
          if (MODE == 1) {
            const float wt = weight[src];
            v.x *= wt;
            v.y *= wt;
          }
        }
        s_v[j] = v;
      }
      __syncthreads();
      if (active) {
#pragma unroll 4
        for (int j = 0; j < nb; ++j) {
          const int lxy = s_lxy[j], mxy = s_mxy[j];
          const int lx0 = lxy & 0xffff, ly0 = lxy >> 16;
          int dx = tx - (mxy & 0xffff);
          dx += (dx >> 31) & S;
          int dy = ty - (mxy >> 16);
          dy += (dy >> 31) & S;
          const int cell = (ly0 + dy) * pitch + lx0 + dx;
          float2 k;
          if (SEP)
            k = cmul(__ldg(&ktab[s_k0[j] + dy]), __ldg(&ktab[s_k1[j] + dx]));
          else
            k = __ldg(&ktab[s_k0[j] + dy * S + dx]);
          if (cell != cur) {
            if (cur >= 0) {
              float2 o = win[cur];
              o.x += acc.x;
              o.y += acc.y;
              win[cur] = o;
            }
            cur = cell;
            acc = make_float2(0.f, 0.f);
          }
          cfma(acc, k, s_v[j]);
        }
      }
    }
    if (active && cur >= 0) {
      float2 o = win[cur];
      o.x += acc.x;
      o.y += acc.y;
      win[cur] = o;
    }
    __syncthreads();
    for (int c = tid; c < wcells; c += blockDim.x) {
      const int r = c / A.win, q = c - r * A.win;
      const float2 val = win[r * pitch + q];
      if (val.x != 0.f || val.y != 0.f) {
        const int gy = wy0 + r, gx = wx0 + q;
        if (gy < A.H && gx < A.W) atomicAdd(&grid[(size_t)gy * A.W + gx], val);
      }
    }
  }
}

// ---------------------------------------------------------------- degridder
template <bool SEP, int MAXT>
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
    const int wx0 = (w.tile % A.ntx) * A.T, wy0 = (w.tile / A.ntx) * A.T;
    for (int c = threadIdx.x; c < A.win * A.win; c += blockDim.x) {
      const int r = c / A.win, q = c - r * A.win;
      const int gy = wy0 + r, gx = wx0 + q;
      win[r * pitch + q] = (gy < A.H && gx < A.W) ? __ldg(&grid[(size_t)gy * A.W + gx])
                                                  : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int j = warp; j < w.count; j += nwarps) {
      const VisRec r = A.recs[w.start + j];
      const int base = (r.y0 - wy0) * pitch + (r.x0 - wx0);
      float2 sum = make_float2(0.f, 0.f);
      if (SEP) {
        const float2 *ky = ktab + (long long)r.k0 * S;
        const float2 *kx = ktab + (long long)r.k1 * S;
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (soff[i] >= 0)
            cfma(sum, win[base + soff[i]], cmul(__ldg(&ky[kdy[i]]), __ldg(&kx[kdx[i]])));
      } else {
        const float2 *kk = ktab + (long long)r.k0 * KSZ + (long long)r.k1 * SS;
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (soff[i] >= 0) cfma(sum, win[base + soff[i]], __ldg(&kk[lane + 32 * i]));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sum.x += __shfl_xor_sync(0xffffffffu, sum.x, o);
        sum.y += __shfl_xor_sync(0xffffffffu, sum.y, o);
      }
      if (lane == 0) out[A.perm[w.start + j]] = sum;
    }
  }
}

static TiledArgs tiled_args(const cg_plan *p) {
  TiledArgs A;
  A.recs = p->recs;
  A.perm = p->perm;
  A.items = p->items;
  A.nitems = p->nitems;
  A.ticket = p->ticket;
  A.status = p->status;
  A.H = p->H;
  A.W = p->W;
  A.S = p->kd.S;
  A.Q = p->kd.Q;
  A.T = p->T;
  A.ntx = p->ntx;
  A.win = p->win;
  A.pitch = p->pitch;
  return A;
}

static int grid_launch(const cg_plan *p, const void *ktab, const void *vis,
                       const float *weight, int mode, void *grid, cudaStream_t s) {
  CG_REQUIRE(p && p->mode == CG_PLAN_TILED, "cg_grid needs a CG_PLAN_TILED plan");
  if (p->n == 0) return CG_OK;
  CG_REQUIRE(ktab && grid, "NULL kernel table or grid");
  CG_REQUIRE(mode == 2 || vis, "NULL visibilities");
  CG_REQUIRE(mode == 0 || weight, "NULL weights");
  TiledArgs A = tiled_args(p);
  const int SS = p->kd.S * p->kd.S;
  const int threads = (SS + 31) / 32 * 32;
  const size_t smem = (size_t)p->pitch * p->win * sizeof(float2) +
                      (size_t)GRID_STAGE * (4 + 4 + 8 + 8 + 8);
  void (*fn)(TiledArgs, const float2 *, const float2 *, const float *, float2 *);
  if (p->kd.sep)
    fn = mode == 0 ? k_grid_tiled<true, 0> : mode == 1 ? k_grid_tiled<true, 1> : k_grid_tiled<true, 2>;
  else
    fn = mode == 0 ? k_grid_tiled<false, 0> : mode == 1 ? k_grid_tiled<false, 1> : k_grid_tiled<false, 2>;
  CG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  CG_REQUIRE(per_sm > 0, "gridder does not fit on an SM (smem %zu)", smem);
  int64_t blocks = std::min<int64_t>((int64_t)per_sm * num_sms(), p->max_items);
  CG_CUDA(cudaMemsetAsync(p->ticket, 0, sizeof(int32_t), s));
  fn<<<(unsigned)blocks, threads, smem, s>>>(A, (const float2 *)ktab, (const float2 *)vis,
                                              weight, (float2 *)grid);
  CG_LAUNCH("grid");
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

int cg_degrid(const cg_plan *p, const void *ktab, const void *grid, void *out,
              cg_stream_t stream) {
  CG_REQUIRE(p && p->mode == CG_PLAN_TILED, "cg_degrid needs a CG_PLAN_TILED plan");
  if (p->n == 0) return CG_OK;
  CG_REQUIRE(ktab && grid && out, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  TiledArgs A = tiled_args(p);
  const int SS = p->kd.S * p->kd.S;
  const int need = (SS + 31) / 32;
  const int threads = 256;
  const size_t smem = (size_t)p->pitch * p->win * sizeof(float2);
  void (*fn)(TiledArgs, const float2 *, const float2 *, float2 *) = nullptr;
#define PICK(M)                                                                \
  if (!fn && need <= M) fn = p->kd.sep ? k_degrid_tiled<true, M> : k_degrid_tiled<false, M>;
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

}  // extern "C"
