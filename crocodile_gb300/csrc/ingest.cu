// Visibility ingest: per-baseline blocks (the vis/[a1]/[a2] groups of the
// reference's HDF5 visibility files: frequency [nchan], time [nrow],
// uvw [nrow, 3] in metres, vis [nrow, nchan, npol]) flattened into the rows
// the gridder reads, in the order of collect_blocks
// (scripts/image_dataset.py:75-87): block by block, row by row, channel by
// channel, with
//   uvw_lambda = uvw * frequency / c        (arl/data_models.py:198-202)
//   src        = (antenna1, antenna2, time, frequency)
//   vis        = vis[row, chan, pol]
// One CTA per block (grid-stride over blocks), threads over its rows x
// channels; every product and quotient is an explicitly rounded IEEE
// operation, so uvw_lambda is bit-identical to numpy's.

#include <algorithm>

#include "cg_internal.cuh"

namespace {

using namespace cg;

constexpr double C_LIGHT = 299792458.0;  // m/s (SI definition; astropy's const.c)

template <typename VO>
__device__ __forceinline__ VO vis_out(double2 v);
template <>
__device__ __forceinline__ float2 vis_out<float2>(double2 v) {
  return make_float2((float)v.x, (float)v.y);
}
template <>
__device__ __forceinline__ double2 vis_out<double2>(double2 v) {
  return v;
}

template <typename VO>
__global__ void k_ingest(const cg_vis_block *__restrict__ blocks, int nblocks,
                         const double *__restrict__ uvw_m, const double *__restrict__ time,
                         const int32_t *__restrict__ a1, const int32_t *__restrict__ a2,
                         const double *__restrict__ freq, const double2 *__restrict__ vis, int pol,
                         double *__restrict__ uvw_lambda, double *__restrict__ src,
                         int32_t *__restrict__ a1_out, int32_t *__restrict__ a2_out,
                         VO *__restrict__ vout, int32_t *status) {
  for (int b = blockIdx.x; b < nblocks; b += gridDim.x) {
    const cg_vis_block B = blocks[b];
    if (pol >= B.npol) {
      if (threadIdx.x == 0) atomicAdd(&status[ST_INDEX], 1);
      continue;
    }
    const int64_t n64 = (int64_t)B.nrow * B.nchan;
    if (B.nrow < 0 || B.nchan <= 0 || n64 >= (1ll << 31)) {  // 32-bit row/channel split below
      if (threadIdx.x == 0 && n64 != 0) atomicAdd(&status[ST_INDEX], 1);
      continue;
    }
    const int n = (int)n64;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      const int row = e / B.nchan, chan = e - row * B.nchan;
      const int64_t r = B.row_start + row;
      const double f = freq[B.freq_start + chan];
      const int64_t o = B.out_start + e;
      for (int d = 0; d < 3; ++d)
        uvw_lambda[o * 3 + d] = __ddiv_rn(__dmul_rn(uvw_m[r * 3 + d], f), C_LIGHT);
      if (src) {
        src[o * 4 + 0] = (double)a1[r];
        src[o * 4 + 1] = (double)a2[r];
        src[o * 4 + 2] = time[r];
        src[o * 4 + 3] = f;
      }
      if (a1_out) a1_out[o] = a1[r];
      if (a2_out) a2_out[o] = a2[r];
      if (vout) vout[o] = vis_out<VO>(vis[B.vis_start + (int64_t)e * B.npol + pol]);
    }
  }
}

}  // namespace

extern "C" {

int cg_ingest_blocks(const cg_vis_block *blocks, int nblocks, const double *uvw_m,
                     const double *time, const int32_t *a1, const int32_t *a2, const double *freq,
                     const void *vis_c128, int pol, double *uvw_lambda, double *src,
                     int32_t *a1_out, int32_t *a2_out, void *vis_out, int vis_c64,
                     int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(nblocks >= 0 && pol >= 0 && d_status, "bad ingest arguments");
  if (nblocks == 0) return CG_OK;
  CG_REQUIRE(blocks && uvw_m && freq && uvw_lambda && (!src || (time && a1 && a2)) &&
                 (!a1_out || a1) && (!a2_out || a2) && (!vis_out || vis_c128),
             "bad ingest arguments (null input for a requested output)");
  const unsigned grid = (unsigned)std::min(nblocks, num_sms() * 32);
  cudaStream_t st = (cudaStream_t)stream;
  if (vis_c64)
    k_ingest<float2><<<grid, 256, 0, st>>>(blocks, nblocks, uvw_m, time, a1, a2, freq,
                                           (const double2 *)vis_c128, pol, uvw_lambda, src, a1_out,
                                           a2_out, (float2 *)vis_out, d_status);
  else
    k_ingest<double2><<<grid, 256, 0, st>>>(blocks, nblocks, uvw_m, time, a1, a2, freq,
                                            (const double2 *)vis_c128, pol, uvw_lambda, src,
                                            a1_out, a2_out, (double2 *)vis_out, d_status);
  CG_LAUNCH("ingest");
  return CG_OK;
}

}  // extern "C"
