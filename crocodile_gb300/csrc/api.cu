// Error state, status block and small utilities of the C ABI.
#include <stdarg.h>
#include <string.h>

#include <atomic>
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

static std::mutex g_tuning_mu;
static cg_tuning g_tuning = {0, 0, 0, 0, 0, 0};

cg_tuning tuning() {
  std::lock_guard<std::mutex> lock(g_tuning_mu);
  return g_tuning;
}

// Clock-cycle limit of the gridders' bounded waits on bulk copies (about two
// seconds at 2 GHz); lowered only by tests that make a wait run out.
static std::atomic<long long> g_wait_cycles{4000000000ll};

long long wait_cycles() { return g_wait_cycles.load(std::memory_order_relaxed); }

// The tuned layout, or automatically the lane layout for tables whose S x S
// slices stream by bulk copies (non-separable, even S <= 16) and the warp
// layout otherwise.  The lane layout needs S <= 16.
int layout_for(const cg_kernel_desc &kd) {
  const int l = tuning().layout;
  if (l == CG_LAYOUT_LANE) return kd.S <= 16 ? CG_LAYOUT_LANE : CG_LAYOUT_WARP;
  if (l > 0) return l;
  return (!kd.sep && kd.S <= 16 && kd.S % 2 == 0) ? CG_LAYOUT_LANE : CG_LAYOUT_WARP;
}

}  // namespace cg

extern "C" {

int cg_set_tuning(const cg_tuning *t) {
  CG_REQUIRE(t, "tuning is NULL");
  CG_REQUIRE(t->tile >= 0 && t->tile <= 64 && t->tile % 4 == 0, "tile %d must be a multiple of 4 "
             "in [0, 64]", t->tile);
  CG_REQUIRE(t->chunk >= 0 && t->chunk <= (1 << 20), "chunk %d out of range", t->chunk);
  CG_REQUIRE(t->rows >= 0 && t->rows <= 8, "rows %d out of range [0, 8]", t->rows);
  CG_REQUIRE(t->layout >= 0 && t->layout <= CG_LAYOUT_LANE, "layout %d unknown", t->layout);
  CG_REQUIRE(t->dvis >= 0 && t->dvis <= 4, "dvis %d must be 0..4", t->dvis);
  const int gmax = t->layout == CG_LAYOUT_LANE ? 16 : 8;
  CG_REQUIRE(t->groups >= 0 && t->groups <= gmax, "groups %d out of range [0, %d]", t->groups,
             gmax);
  std::lock_guard<std::mutex> lock(cg::g_tuning_mu);
  cg::g_tuning = *t;
  return CG_OK;
}

int cg_set_wait_limit(long long cycles) {
  CG_REQUIRE(cycles >= 0, "wait limit %lld must be >= 0", cycles);
  cg::g_wait_cycles.store(cycles, std::memory_order_relaxed);
  return CG_OK;
}

long long cg_get_wait_limit(void) { return cg::wait_cycles(); }

int cg_get_tuning(cg_tuning *out) {
  CG_REQUIRE(out, "output is NULL");
  *out = cg::tuning();
  return CG_OK;
}

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
