// Error state, status block and small utilities of the C ABI.
#include <stdarg.h>
#include <string.h>

#include <mutex>

#include "cg_internal.cuh"

namespace cg {

static thread_local char g_msg[512] = "";

int set_error(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_error(cudaError_t e, const char *where) {
  return set_error(CG_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

int num_sms() {
  static int sms = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  });
  return sms;
}

}  // namespace cg

extern "C" {

const char *cg_last_error(void) { return cg::g_msg; }

int cg_version(void) { return 100; }

int cg_status_reset(int32_t *d_status, cg_stream_t stream) {
  CG_REQUIRE(d_status, "status block is NULL");
  CG_CUDA(cudaMemsetAsync(d_status, 0, CG_STATUS_WORDS * sizeof(int32_t),
                          (cudaStream_t)stream));
  return CG_OK;
}

int cg_status_check(const int32_t *d_status, int32_t *counts_out,
                    cg_stream_t stream) {
  CG_REQUIRE(d_status, "status block is NULL");
  int32_t h[CG_STATUS_WORDS];
  CG_CUDA(cudaMemcpyAsync(h, d_status, sizeof(h), cudaMemcpyDeviceToHost,
                          (cudaStream_t)stream));
  CG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  if (counts_out) memcpy(counts_out, h, sizeof(h));
  if (h[cg::ST_RANGE])
    return cg::set_error(CG_ERR_RANGE,
                         "%d coordinates outside [-0.5, 0.5) of the grid",
                         h[cg::ST_RANGE]);
  if (h[cg::ST_BOUNDS])
    return cg::set_error(CG_ERR_BOUNDS,
                         "%d visibilities have kernel footprints outside the grid",
                         h[cg::ST_BOUNDS]);
  if (h[cg::ST_INDEX])
    return cg::set_error(CG_ERR_INDEX, "%d kernel or cell indices out of range",
                         h[cg::ST_INDEX]);
  if (h[cg::ST_TIMEOUT])
    return cg::set_error(CG_ERR_TIMEOUT, "%d bounded device waits gave up",
                         h[cg::ST_TIMEOUT]);
  return CG_OK;
}

}  // extern "C"
