// Shared pieces of the tiled FP32 kernels: launch arguments, tile origins,
// complex helpers and the work-item ticket.
#pragma once

#include "cg_internal.cuh"

namespace cg {

struct TiledArgs {
  const VisRec *recs;
  const int32_t *perm;
  const WorkItem *items;
  const int32_t *nitems;
  int32_t *ticket;
  const int32_t *status;
  int H, W, S, Q, T, tblog, nbx, tpl, win, pitch;
};

// Window origin of a work item's tile and the offset of its layer's grid.
struct TileOrigin {
  int wx0, wy0;
  size_t layer_off;
};
__device__ __forceinline__ TileOrigin tile_origin(const TiledArgs &A, int tile) {
  const int lyr = tile / A.tpl, t = tile - lyr * A.tpl;
  int tx, ty;
  tile_xy(t, A.tblog, A.nbx, tx, ty);
  TileOrigin o;
  o.wx0 = tx * A.T;
  o.wy0 = ty * A.T;
  o.layer_off = (size_t)lyr * A.H * A.W;
  return o;
}

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

inline TiledArgs tiled_args(const cg_plan *p) {
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
  A.tblog = p->tblog;
  A.nbx = p->nbx;
  A.tpl = p->tpl;
  A.win = p->win;
  A.pitch = p->pitch;
  return A;
}

// Lane-layout launches (grid_lane.cu): gridding (fused = false; gmode 0 vis,
// 1 vis * weight, 2 weight) or the fused degrid+grid pass (fused = true).
int lane_launch(const cg_plan *p, const float2 *ktab, const float2 *vis, const float *weight,
                int gmode, float2 *grid, const float2 *grid_in, float2 *vis_out, int residual,
                bool fused, cudaStream_t s);

// Degridding of lane-layout plans with per-warp slice rings (grid_lane.cu);
// CG_ERR_ARG (nothing launched) when the plan's table cannot stream by bulk
// copies (separable, S > 16, or a table that is not 16-byte aligned).
int ring_degrid_launch(const cg_plan *p, const float2 *ktab, const float2 *grid, float2 *out,
                       cudaStream_t s);

}  // namespace cg
