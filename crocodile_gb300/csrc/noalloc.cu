// Convolutional gridding for callers that cannot allocate device memory.
//
// Some hosts of this library cannot hand it scratch memory: a C or Fortran
// imaging pipeline that reserves all device memory at start-up in its own
// pool and forbids cudaMalloc/cudaFree afterwards (both synchronise the device
// and can fail mid-observation once memory is fragmented), or a plug-in host
// that passes only its input and output buffers across an FFI and has no
// allocator to offer.  cg_grid_noalloc serves them: it is cg_plan_create +
// cg_grid with the plan's scratch (visibility records, sort buffers, work
// list) taken from a fixed array in device memory that is part of this
// library, so the call allocates nothing, neither on the host nor on the
// device.
//
// The array costs CG_NOALLOC_SCRATCH_BYTES of device memory on every GPU that
// loads the library, for the life of the process.  All calls share it, and
// it keeps what the last call left there: each call re-zeroes the counters and
// histograms it accumulates into before using them, and calls that overlap on
// the GPU (different streams, or different host threads on one device) race
// on it and must be serialised by the caller.  The device address of the
// array is looked up once per device and cached; cudaDeviceReset in the same
// process invalidates it, so calls after a device reset are not supported.
#include <string.h>

#include <mutex>

#include "cg_internal.cuh"

namespace cg {
int plan_build_tiled_into(cg_plan *p, const cg_kernel_desc *kd, int H, int W,
                          const double *uvw, int64_t stride, double lam,
                          const int32_t *kidx, int64_t n, void *workspace,
                          size_t workspace_bytes, int32_t *d_status, cudaStream_t s);
}

static __device__ __align__(256) unsigned char g_noalloc_scratch[CG_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch, looked up once per device.  In host
// code the array's name is only a host-side stand-in, never a device address.
static constexpr int kMaxDevices = 128;
static std::mutex g_scratch_mu;
static void *g_scratch_ptr[kMaxDevices];

static int scratch_address(void **out) {
  int dev = 0;
  CG_CUDA(cudaGetDevice(&dev));
  CG_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cg::cuda_error(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return CG_OK;
}

extern "C" int cg_grid_noalloc(const cg_kernel_desc *kd, int H, int W, const double *uvw,
                               int64_t stride, double lam, const int32_t *kidx, int64_t n,
                               const void *ktab_c64, const void *vis_c64, void *grid_c64,
                               int32_t *d_status, cg_stream_t stream) {
  const size_t need = cg_plan_workspace_bytes(CG_PLAN_TILED, n, H, W, kd);
  if (need == 0) return CG_ERR_ARG;  // message set by the size query
  if (need > (size_t)CG_NOALLOC_SCRATCH_BYTES)
    return cg::set_error(CG_ERR_WORKSPACE,
                         "cg_grid_noalloc: %lld visibilities on a %dx%d grid need %zu scratch "
                         "bytes, more than the %zu-byte static scratch; use cg_plan_create "
                         "with a caller workspace",
                         (long long)n, H, W, need, (size_t)CG_NOALLOC_SCRATCH_BYTES);
  void *ws = nullptr;
  int rc = scratch_address(&ws);
  if (rc) return rc;
  cg_plan plan;
  // the whole array as the workspace: the build re-derives the layout from the
  // current tuning and checks its own need against this size
  rc = cg::plan_build_tiled_into(&plan, kd, H, W, uvw, stride, lam, kidx, n, ws,
                                 (size_t)CG_NOALLOC_SCRATCH_BYTES, d_status,
                                 (cudaStream_t)stream);
  if (rc) return rc;
  return cg_grid(&plan, ktab_c64, vis_c64, grid_c64, stream);
}
