// Update-rate microbenchmarks: the measured peaks that the gridders'
// grid-point update rate (2 * n * S^2 updates per grid + degrid) is compared
// with.  Neither has a counterpart in the reference; both are measurement
// utilities.
//
// kind 0, k_peak_smem_update: the lane gridder's inner loop without its HBM
//   traffic.  Every warp owns a private 31 x 32 float2 window and a 16 x 16
//   tap slice in shared memory and applies synthetic visibilities at
//   pseudo-random footprint origins: lane l reads its taps l + 32 i
//   (i < 8), reads the window cell under each, multiplies and adds in FP32
//   and writes the cell back, then the warp synchronises (one visibility =
//   256 cell updates).  16 warps per CTA, one CTA per SM.
// kind 1, k_peak_red: float2 atomic additions into an L2-resident buffer
//   (red.global.add of 32 consecutive cells per warp instruction, the form of
//   the gridders' window flushes), at pseudo-random 256-byte-aligned rows.
#include "cg_internal.cuh"

namespace cg {

namespace {

constexpr int PK_WIN = 31, PK_PITCH = 32, PK_WARPS = 16;
constexpr int PK_WARP_ELEMS = PK_WIN * PK_PITCH + 256;  // window, then the tap slice

__global__ void __launch_bounds__(PK_WARPS * 32) k_peak_smem_update(int nvis, float2 *sink) {
  extern __shared__ float2 pk_sh[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *win = pk_sh + (size_t)warp * PK_WARP_ELEMS;
  float2 *slice = win + PK_WIN * PK_PITCH;
  for (int c = lane; c < PK_WIN * PK_PITCH; c += 32) win[c] = make_float2(0.f, 0.f);
  for (int t = lane; t < 256; t += 32) slice[t] = make_float2(1e-3f * t, 1e-3f * (255 - t));
  __syncwarp();
  unsigned s = 2654435761u * (blockIdx.x * PK_WARPS + warp + 1);
  const float2 u = make_float2(0.5f, -0.25f);
  for (int j = 0; j < nvis; ++j) {
    s = s * 1664525u + 1013904223u;
    const int base = (int)((s >> 8) & 15) * PK_PITCH + (int)((s >> 16) & 15);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int t = lane + 32 * i;
      const float2 k = slice[t];
      float2 *c = &win[base + (t >> 4) * PK_PITCH + (t & 15)];
      float2 o = *c;
      o.x = fmaf(k.x, u.x, o.x);
      o.x = fmaf(-k.y, u.y, o.x);
      o.y = fmaf(k.x, u.y, o.y);
      o.y = fmaf(k.y, u.x, o.y);
      *c = o;
    }
    __syncwarp();
  }
  // keep the window live: one value per warp to global memory
  float2 acc = make_float2(0.f, 0.f);
  for (int c = lane; c < PK_WIN * PK_PITCH; c += 32) {
    acc.x += win[c].x;
    acc.y += win[c].y;
  }
  if (lane == 0) sink[blockIdx.x * PK_WARPS + warp] = acc;
}

__global__ void __launch_bounds__(256) k_peak_red(float2 *buf, unsigned rows_mask, int iters) {
  const int lane = threadIdx.x & 31;
  unsigned s = 2654435761u * (blockIdx.x * 8 + (threadIdx.x >> 5) + 1);
  const float2 v = make_float2(1.f, -1.f);
  for (int j = 0; j < iters; ++j) {
    s = s * 1664525u + 1013904223u;
    const size_t row = (s >> 4) & rows_mask;
    atomicAdd(&buf[row * 32 + lane], v);  // result unused: red.global.add.v2.f32
  }
}

}  // namespace

}  // namespace cg

using namespace cg;

extern "C" int cg_update_peak(int kind, int work, void *buf, size_t buf_bytes, double *updates,
                              cg_stream_t stream) {
  CG_REQUIRE((kind == 0 || kind == 1) && work >= 1 && buf && updates,
             "bad update-peak arguments");
  cudaStream_t st = (cudaStream_t)stream;
  const int sms = num_sms();
  if (kind == 0) {
    CG_REQUIRE(buf_bytes >= (size_t)sms * PK_WARPS * sizeof(float2),
               "update peak: sink buffer needs %zu bytes", (size_t)sms * PK_WARPS * 8);
    const size_t smem = (size_t)PK_WARPS * PK_WARP_ELEMS * sizeof(float2);
    CG_CUDA(cudaFuncSetAttribute(k_peak_smem_update, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    k_peak_smem_update<<<sms, PK_WARPS * 32, smem, st>>>(work, (float2 *)buf);
    CG_LAUNCH("shared-memory update peak");
    *updates = (double)sms * PK_WARPS * work * 256.0;
    return CG_OK;
  }
  // rows of 32 float2 cells (256 B); a power-of-two row count within the
  // buffer, at most 32 MiB so that the cells stay in L2
  size_t rows = 1;
  while (rows * 2 * 256 <= buf_bytes && rows * 2 <= ((size_t)1 << 17)) rows *= 2;
  CG_REQUIRE(rows >= 1024, "update peak: atomics buffer needs >= 256 KiB");
  const int blocks = sms * 8;
  k_peak_red<<<blocks, 256, 0, st>>>((float2 *)buf, (unsigned)(rows - 1), work);
  CG_LAUNCH("atomic update peak");
  *updates = (double)blocks * 8 * 32 * (double)work;
  return CG_OK;
}
