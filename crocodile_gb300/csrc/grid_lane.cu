// Lane-layout FP32 gridder and fused degrid+grid pass: no shared-memory atomics.
//
// Gridding replaces convgrid (crocodile/synthesis.py:464-481); the fused pass
// is convdegrid (synthesis.py:484-503) followed by convgrid of the same
// visibilities, reading every kernel tap once for both.
//
// One warp takes one work item (<= chunk visibilities of one grid tile) at a
// time and owns a private (T+S-1)^2 window in shared memory, so no other warp
// ever writes its cells.  Lane l owns the kernel taps t = l + 32 i of every
// visibility (footprint cell (t / S, t mod S)); the taps of one visibility are
// distinct cells, so each lane adds its products with a plain read-modify-write
// and the warp synchronises once per visibility: no shared-memory atomics.
// Each item's window is flushed to HBM with float2 atomics and left zeroed for
// the next one; an item with fewer taps than half its window's cells adds its
// taps straight into the grid with float2 atomics instead.
//
// Non-separable tables stream every visibility's slice (padded to a 16-byte
// multiple for odd S * S) into a per-warp ring of D shared-memory stages (D =
// 2..4, 3 by default) with bulk asynchronous copies (cp.async.bulk;
// completion counted in bytes on one mbarrier per stage), issued D - 1
// visibilities ahead by lane 0, so that ~D slices per warp are in flight
// without holding registers.  Other tables load their taps from global memory one visibility
// ahead.  Visibility records are staged 32 at a time in a per-warp ring of 64,
// the next batch being loaded while the current one runs.  Every mbarrier
// wait is bounded (about two seconds); on expiry the warp sets the timeout
// status word, waits (bounded) for its copies in flight and stops.
#include <algorithm>

#include "mbar.cuh"
#include "tiled.cuh"

namespace cg {

static constexpr int LANE_DEPTH = 4;                          // bulk-copy stages per warp (max)
static constexpr int LANE_RING = 64;                          // staged visibility records per warp
static constexpr long long LANE_WAIT_CYCLES = 4000000000ll;   // ~2 s at 2 GHz
static constexpr unsigned FULL_MASK = 0xffffffffu;

struct LaneArgs {
  const float2 *ktab;
  const float2 *vis;      // gridding: values to grid; fused: input visibilities (may be NULL)
  const float *weight;    // gridding modes 1 and 2
  float2 *grid;           // output grid
  const float2 *grid_in;  // fused: grid to degrid
  float2 *vis_out;        // fused: degridded visibilities (may be NULL)
  int mode;               // gridding: 0 vis, 1 vis * weight, 2 weight; fused: 0 plain, 1 residual
  long long wait_cycles;  // limit of a consumer's wait for a slice (the drain keeps LANE_WAIT_CYCLES)
  int kstride;            // elements between slices in ktab and in the stage ring (4-D tables)
  int depth;              // bulk-copy stages per warp, 2..LANE_DEPTH
  int degrid_only;        // fused form without an output grid: the degridder alone
  int warp_bytes;         // shared memory per warp
  int stage_off, meta_off, val_off, bar_off;  // byte offsets inside a warp's region
};

// On lanes with p set: one bulk copy of `bytes` (multiple of 16, both
// addresses 16-byte aligned) from global to shared memory completing on `bar`.
// Predicated rather than branched, so the warp does not diverge.  No proxy
// fence before it: generic code only ever reads the stages these copies fill
// (nothing generic writes them), and every read of a stage has returned its
// value, which the reading lane has consumed, before the warp barrier that
// precedes the copy reusing the stage; a fence here measured 4.33 against
// 4.13 ms for the AW gridder and 3.79 against 3.66 ms for the ring degridder.
__device__ __forceinline__ void bulk_load_if(bool p, void *dst, const void *src, uint32_t bytes,
                                             uint64_t *bar) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "@p mbarrier.arrive.expect_tx.shared::cta.b64 _, [%3], %2;\n\t"
      "@p cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      "\n\t}" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "r"((int)p)
      : "memory");
}

// Waits for the phase of `bar` with the given parity; false after ~2 s.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  return mbar_wait_cycles(bar, parity, LANE_WAIT_CYCLES);
}

// FULLT: S * S == 32 * MAXT, every lane owns MAXT taps (no per-tap checks).
// SC, PC: support and window pitch fixed at compile time (0: read at run
// time); with S dividing 32 a lane's taps then sit at immediate offsets.
template <bool SEP, bool BULK, bool FUSED, int MAXT, bool FULLT, int SC = 0, int PC = 0>
__global__ void __launch_bounds__(512) k_lane(TiledArgs A, LaneArgs P) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (status_failed(A.status)) return;
  const int S = SC ? SC : A.S, SS = S * S, pitch = PC ? PC : A.pitch, win = A.win;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char *region = smem + (size_t)warp * P.warp_bytes;
  float2 *wbuf = (float2 *)region;
  float2 *stages = (float2 *)(region + P.stage_off);
  int4 *meta = (int4 *)(region + P.meta_off);
  float2 *mval = (float2 *)(region + P.val_off);
  uint64_t *bar = (uint64_t *)(region + P.bar_off);
  const int QQ = A.Q * A.Q;
  const float2 zero = make_float2(0.f, 0.f);
  const int KS = P.kstride;  // S * S, or S * S + 1 for padded odd slices
  const uint32_t slice_bytes = (uint32_t)KS * 8u;

  // lane l owns taps t = l + 32 i: footprint cell (dy, dx) = (t / S, t % S)
  int soff[MAXT], goff[MAXT], tdy[MAXT], tdx[MAXT];
  bool own[MAXT];
  constexpr bool STEP = SC > 0 && 32 % (SC > 0 ? SC : 1) == 0;  // t + 32 is 32 / S rows down
#pragma unroll
  for (int i = 0; i < MAXT; ++i) {
    const int t = lane + 32 * i;
    tdy[i] = STEP ? lane / S + i * (32 / S) : t / S;
    tdx[i] = STEP ? lane % S : t - tdy[i] * S;
    own[i] = FULLT || t < SS;
    soff[i] = STEP ? (lane / S) * pitch + lane % S + i * (32 / S) * pitch : tdy[i] * pitch + tdx[i];
    goff[i] = tdy[i] * A.W + tdx[i];
  }

  for (int c = lane; c < pitch * win; c += 32) wbuf[c] = zero;
  if (BULK && lane == 0) {
    for (int d = 0; d < P.depth; ++d) mbar_init(&bar[d], 1);
    mbar_fence_init();
  }
  __syncwarp();

  // consumer position in the stage ring: stage and phase parity of the next
  // visibility this warp reads (persisting across items)
  int cst = 0;
  uint32_t cpar = 0;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(A.ticket, 1);
    it = __shfl_sync(FULL_MASK, it, 0);
    if (it >= *A.nitems) break;
    const WorkItem w = A.items[it];
    const TileOrigin org = tile_origin(A, w.tile);
    const int n = w.count;
    // An item whose taps are fewer than half its window's cells skips the
    // window: staging and flushing the window would cost more than per-tap
    // global atomics (sparse tiles, e.g. the many small sub-grids of w-towers).
    const bool direct = (int64_t)n * SS * 2 < (int64_t)win * win;
    const bool gout = !FUSED || !P.degrid_only;  // this traversal grids
    const float2 *gin = FUSED ? P.grid_in + org.layer_off + (size_t)org.wy0 * A.W + org.wx0
                              : nullptr;

    // Record of item visibility j, packed for the ring: x = lx0 | ly0 << 16 (the
    // footprint origin in the window), y = slice (or kernel row k0), z = k1
    // (separable), w = original index.
    auto pack = [&](const VisRec &rec, int src) {
      int4 m;
      m.x = (rec.x0 - org.wx0) | ((rec.y0 - org.wy0) << 16);
      m.y = SEP ? rec.k0 : rec.k0 * QQ + rec.k1;
      m.z = rec.k1;
      m.w = src;
      return m;
    };
    auto value = [&](int src) {
      if (FUSED) return P.vis ? P.vis[src] : zero;
      if (P.mode == 2) return make_float2(P.weight[src], 0.f);
      float2 v = P.vis[src];
      if (P.mode == 1) {
        const float wt = P.weight[src];
        v.x *= wt;
        v.y *= wt;
      }
      return v;
    };

    if (lane < n) {
      const int src = A.perm[w.start + lane];
      meta[lane] = pack(A.recs[w.start + lane], src);
      mval[lane] = value(src);
    }
    __syncwarp();

    // Bulk copies run LANE_DEPTH - 1 visibilities ahead of the consumer: the
    // copy of visibility j + LANE_DEPTH - 1 goes into the stage that visibility
    // j - 1 used.
    int issued = 0;
    if (BULK) {
      int ist = cst;
      for (; issued < min(n, P.depth - 1); ++issued) {
        const int4 m = meta[issued];
        bulk_load_if(lane == 0, stages + (size_t)ist * KS, P.ktab + (size_t)m.y * KS,
                     slice_bytes, &bar[ist]);
        ist = ist + 1 == P.depth ? 0 : ist + 1;
      }
    }

    // taps from global memory (tables that are not streamed) and, fused, the
    // input grid under the footprint: loaded one visibility ahead
    float2 kn[MAXT], gn[MAXT];
#pragma unroll
    for (int i = 0; i < MAXT; ++i) kn[i] = gn[i] = zero;
    auto load_global = [&](int j) {
      const int4 m = meta[j & (LANE_RING - 1)];
      const int lx0 = m.x & 0xffff, ly0 = m.x >> 16;
      const float2 *kk = SEP ? P.ktab + (size_t)m.y * S : P.ktab + (size_t)m.y * KS;
      const float2 *kx = P.ktab + (size_t)m.z * S;
#pragma unroll
      for (int i = 0; i < MAXT; ++i)
        if (own[i]) {
          if (!BULK)
            kn[i] = SEP ? cmul(__ldg(&kk[tdy[i]]), __ldg(&kx[tdx[i]]))
                        : __ldg(&kk[lane + 32 * i]);
          if (FUSED) gn[i] = __ldg(&gin[(size_t)ly0 * A.W + lx0 + goff[i]]);
        }
    };
    if (!BULK || FUSED) load_global(0);

    bool failed = false;
    // one visibility; false when a bulk copy did not arrive in time
    auto body = [&](int j) -> bool {
      float2 kc[MAXT], gc[MAXT];
      if (BULK) {
        if (issued < n) {
          const int4 mi = meta[issued & (LANE_RING - 1)];
          const int ist = cst == 0 ? P.depth - 1 : cst - 1;
          bulk_load_if(lane == 0, stages + (size_t)ist * KS, P.ktab + (size_t)mi.y * KS,
                       slice_bytes, &bar[ist]);
          ++issued;
        }
        // a limit of 0 (a test of the timeout path) polls without blocking
        bool ok = P.wait_cycles ? mbar_try(&bar[cst], cpar) : mbar_test(&bar[cst], cpar);
        if (!__all_sync(FULL_MASK, ok)) {  // warp-uniform slow path, bounded
          const long long t0 = clock64();
          while (!ok && clock64() - t0 <= P.wait_cycles) ok = mbar_try(&bar[cst], cpar);
          if (__any_sync(FULL_MASK, !ok)) return false;
        }
        const float2 *kp = stages + (size_t)cst * KS + lane;
#pragma unroll
        for (int i = 0; i < MAXT; ++i) kc[i] = own[i] ? kp[32 * i] : zero;
        if (++cst == P.depth) {
          cst = 0;
          cpar ^= 1u;
        }
      } else {
#pragma unroll
        for (int i = 0; i < MAXT; ++i) kc[i] = kn[i];
      }
#pragma unroll
      for (int i = 0; i < MAXT; ++i) gc[i] = gn[i];
      if ((!BULK || FUSED) && j + 1 < n) load_global(j + 1);

      const int4 m = meta[j & (LANE_RING - 1)];
      float2 u = mval[j & (LANE_RING - 1)];
      const int base = (m.x >> 16) * pitch + (m.x & 0xffff);
      if (FUSED) {
        float2 sum = zero;
#pragma unroll
        for (int i = 0; i < MAXT; ++i) cfma(sum, gc[i], kc[i]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          sum.x += __shfl_xor_sync(FULL_MASK, sum.x, o);
          sum.y += __shfl_xor_sync(FULL_MASK, sum.y, o);
        }
        if (lane == 0 && P.vis_out) P.vis_out[m.w] = sum;
        if (P.mode == 1) {
          u.x -= sum.x;
          u.y -= sum.y;
        }
      }
      if (!gout) {
        // degridding only: nothing to add
      } else if (direct) {
        // sparse item: the taps go straight to the grid (float2 atomics)
        float2 *gp = P.grid + org.layer_off + (size_t)(org.wy0 + (m.x >> 16)) * A.W +
                     org.wx0 + (m.x & 0xffff);
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (own[i]) atomicAdd(&gp[(size_t)tdy[i] * A.W + tdx[i]], cmul(kc[i], u));
      } else {
        // distinct taps of one visibility are distinct cells: plain read-modify-write
#pragma unroll
        for (int i = 0; i < MAXT; ++i)
          if (own[i]) {
            float2 *c = &wbuf[base + soff[i]];
            float2 o = *c;
            cfma(o, kc[i], u);
            *c = o;
          }
      }
      __syncwarp();  // this visibility's updates (and stage reads) before the next one
      return true;
    };

    // Batches of 32 records: the next batch's indices are loaded before the
    // first 8 visibilities, its values before the next 8, and it enters the
    // ring before the last 16 (which may issue copies from it).
    int j = 0;
    for (int b0 = 0; b0 < n && !failed; b0 += 32) {
      const int nb = min(32, n - b0);
      const bool more = b0 + 32 < n;
      const int jn = b0 + 32 + lane;
      VisRec nrec;
      int nsrc = 0;
      float2 nval = zero;
      if (more && jn < n) {
        nrec = A.recs[w.start + jn];
        nsrc = A.perm[w.start + jn];
      }
      for (int seg = 0; seg < 3 && !failed; ++seg) {
        const int jend = b0 + min(nb, seg == 0 ? 8 : seg == 1 ? 16 : 32);
        for (; j < jend; ++j)
          if (!body(j)) {
            failed = true;
            break;
          }
        if (seg == 0 && more && jn < n) nval = value(nsrc);
        if (seg == 1 && more) {
          if (jn < n) {
            meta[jn & (LANE_RING - 1)] = pack(nrec, nsrc);
            mval[jn & (LANE_RING - 1)] = nval;
          }
          __syncwarp();
        }
      }
    }
    if (failed) {
      // record the timeout, let this warp's copies in flight land, stop
      if (lane == 0) {
        atomicAdd((int32_t *)&A.status[ST_TIMEOUT], 1);
        int st = cst;
        uint32_t par = cpar;
        for (int jx = j; jx < issued; ++jx) {
          mbar_wait(&bar[st], par);
          if (++st == P.depth) {
            st = 0;
            par ^= 1u;
          }
        }
      }
      __syncwarp();
      return;
    }
    for (int row = 0; row < (direct || !gout ? 0 : win); ++row) {
      const int gy = org.wy0 + row;
      for (int q = lane; q < win; q += 32) {
        const int c = row * pitch + q;
        const float2 val = wbuf[c];
        if (val.x != 0.f || val.y != 0.f) {
          const int gx = org.wx0 + q;
          if (gy < A.H && gx < A.W)
            atomicAdd(&P.grid[org.layer_off + (size_t)gy * A.W + gx], val);
          wbuf[c] = zero;
        }
      }
    }
    __syncwarp();
  }
}

// dst[s][t] = src[s][t] for t < SS, 0 for SS <= t < KS: slices padded to KS elements
__global__ void k_pad_slices(const float2 *__restrict__ src, int64_t nslices, int SS, int KS,
                             float2 *__restrict__ dst) {
  const int64_t total = nslices * KS;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sl = e / KS;
    const int t = (int)(e - sl * KS);
    dst[e] = t < SS ? src[sl * SS + t] : make_float2(0.f, 0.f);
  }
}

// Odd S * S: the table with slices padded to an even element count (a
// 16-byte multiple), copied into the plan's workspace; ktab then points at it.
static int padded_table(const cg_plan *p, const float2 *&ktab, cudaStream_t s) {
  const int SS = p->kd.S * p->kd.S, KS = p->kd.sep ? p->kd.S : p->slice_stride;
  if (p->kd.sep || KS == SS) return CG_OK;
  CG_REQUIRE(p->kpad && KS == SS + 1, "plan has no padded kernel table");
  const int64_t total = p->kpad_slices * KS;
  const unsigned blocks = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16));
  k_pad_slices<<<blocks, 256, 0, s>>>(ktab, p->kpad_slices, SS, KS, p->kpad);
  CG_LAUNCH("kernel slice padding");
  ktab = p->kpad;
  return CG_OK;
}

template <bool SEP, bool BULK, bool FUSED>
static void *lane_kernel_for(int maxt, int SS, int pitch) {
  if (maxt == 8 && SS == 256 && pitch == 32) return (void *)k_lane<SEP, BULK, FUSED, 8, true, 16, 32>;
  if (maxt == 8 && SS == 256 && pitch == 48) return (void *)k_lane<SEP, BULK, FUSED, 8, true, 16, 48>;
  if (maxt == 8 && SS == 256) return (void *)k_lane<SEP, BULK, FUSED, 8, true>;
  if (maxt == 2 && SS == 64) return (void *)k_lane<SEP, BULK, FUSED, 2, true>;
  switch (maxt) {
    case 1: return (void *)k_lane<SEP, BULK, FUSED, 1, false>;
    case 2: return (void *)k_lane<SEP, BULK, FUSED, 2, false>;
    case 4: return (void *)k_lane<SEP, BULK, FUSED, 4, false>;
    case 8: return (void *)k_lane<SEP, BULK, FUSED, 8, false>;
    default: return nullptr;
  }
}

int lane_launch(const cg_plan *p, const float2 *ktab, const float2 *vis, const float *weight,
                int gmode, float2 *grid, const float2 *grid_in, float2 *vis_out, int residual,
                bool fused, cudaStream_t s) {
  const int S = p->kd.S, SS = S * S;
  CG_REQUIRE(S <= 16, "the lane layout supports S <= 16 (S = %d)", S);
  CG_REQUIRE(p->kd.sep || (int64_t)p->kd.G * p->kd.Q * p->kd.Q < (int64_t)1 << 31,
             "kernel table has too many slices for the lane layout");
  const int need = (SS + 31) / 32;
  int maxt = 1;
  while (maxt < need) maxt *= 2;
  const int KS = p->kd.sep ? S : p->slice_stride;
  const int prc = padded_table(p, ktab, s);
  if (prc) return prc;
  const bool bulk = !p->kd.sep && (KS * 8) % 16 == 0 && ((uintptr_t)ktab & 15) == 0;

  const cg_tuning t = tuning();
  LaneArgs P;
  P.ktab = ktab;
  P.vis = vis;
  P.weight = weight;
  P.grid = grid;
  P.grid_in = grid_in;
  P.vis_out = vis_out;
  P.mode = fused ? (residual ? 1 : 0) : gmode;
  P.wait_cycles = wait_cycles();
  P.kstride = KS;
  P.degrid_only = fused && grid == nullptr;
  auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  size_t off = up16((size_t)p->pitch * p->win * sizeof(float2));
  P.stage_off = (int)off;
  // stages: the tuning's rows field (2..4) for the lane layout, 3 by default
  // (14 warps per SM instead of 12 with 4 stages: 8.77 against 8.99 ms per
  // grid + degrid step of the 16.1M-visibility AW workload)
  const int depth = t.rows >= 2 && t.rows <= LANE_DEPTH ? t.rows : 3;
  P.depth = depth;
  if (bulk) off += (size_t)depth * KS * sizeof(float2);
  P.meta_off = (int)off;
  off += LANE_RING * sizeof(int4);
  P.val_off = (int)off;
  off += LANE_RING * sizeof(float2);
  P.bar_off = (int)off;
  off = up16(off + depth * sizeof(uint64_t));
  P.warp_bytes = (int)off;

  // warps per CTA: as asked (or as many as fill ~220 KB), at most what fits in 227 KB
  const int fit = (int)std::min<size_t>(16, (227u << 10) / off);
  CG_REQUIRE(fit >= 1, "lane-layout window does not fit in shared memory (%zu bytes per warp)",
             off);
  const int warps = std::min(fit, t.groups > 0 ? t.groups
                                               : (int)std::max<size_t>(1, (220u << 10) / off));
  void *fn = p->kd.sep ? (fused ? lane_kernel_for<true, false, true>(maxt, SS, p->pitch)
                                : lane_kernel_for<true, false, false>(maxt, SS, p->pitch))
                       : bulk ? (fused ? lane_kernel_for<false, true, true>(maxt, SS, p->pitch)
                                       : lane_kernel_for<false, true, false>(maxt, SS, p->pitch))
                              : (fused ? lane_kernel_for<false, false, true>(maxt, SS, p->pitch)
                                       : lane_kernel_for<false, false, false>(maxt, SS, p->pitch));
  CG_REQUIRE(fn, "no lane-layout kernel for support %d", S);
  const size_t smem = (size_t)warps * off;
  const int threads = 32 * warps;
  CG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  CG_REQUIRE(per_sm > 0, "lane-layout kernel does not fit on an SM (smem %zu)", smem);
  const int64_t need_blocks = (p->max_items + warps - 1) / warps;
  const int64_t blocks = std::max<int64_t>(
      1, std::min<int64_t>((int64_t)per_sm * num_sms(), need_blocks));
  TiledArgs A = tiled_args(p);
  CG_CUDA(cudaMemsetAsync(p->ticket, 0, sizeof(int32_t), s));
  void *args[] = {&A, &P};
  CG_CUDA(cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(threads), args, smem, s));
  return CG_OK;
}

// ---------------------------------------------------------------- ring degridder
// Degridding (convdegrid, synthesis.py:484-503) of lane-layout plans with the
// tiled degridder's CTA-shared window and the lane gridder's slice streaming:
// the CTA stages one work item's grid window in shared memory, warp w takes
// the item's visibilities w, w + warps, ..., and each warp streams its
// visibilities' S x S slices through its own ring of D shared-memory stages
// (bulk copies issued D - 1 visibilities ahead by lane 0, completion counted
// in bytes on one mbarrier per stage), so ~D slices per warp are in flight
// without holding registers.  Lane l sums taps l + 32 i against the window
// and the warp reduces with shuffles.  The item's records are staged per warp
// in shared memory before its first copies are issued.  Waits are bounded: a
// warp whose copy does not land in time counts the timeout, lets its copies
// in flight land, and the whole CTA stops at the next item boundary.
struct RingArgs {
  const float2 *ktab;
  const float2 *grid;
  float2 *out;
  long long wait_cycles;
  int kstride;                   // elements between slices
  int depth;                     // stages per warp
  int win_bytes;                 // window region (16-byte multiple)
  int warp_bytes;                // per-warp region: stages, records, barriers
  int meta_off, bar_off;         // offsets inside a warp's region
};

template <int MAXT, bool FULLT, int SC = 0, int PC = 0>
__global__ void __launch_bounds__(256) k_degrid_ring(TiledArgs A, RingArgs R) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item, s_fail;
  if (status_failed(A.status)) return;
  const int S = SC ? SC : A.S, SS = S * S, pitch = PC ? PC : A.pitch;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float2 *win = (float2 *)smem;
  unsigned char *region = smem + R.win_bytes + (size_t)warp * R.warp_bytes;
  float2 *stages = (float2 *)region;
  int4 *meta = (int4 *)(region + R.meta_off);
  uint64_t *bar = (uint64_t *)(region + R.bar_off);
  const int QQ = A.Q * A.Q, KS = R.kstride, D = R.depth;
  const uint32_t slice_bytes = (uint32_t)KS * 8u;
  const float2 zero = make_float2(0.f, 0.f);

  int soff[MAXT];
  bool own[MAXT];
  constexpr bool STEP = SC > 0 && 32 % (SC > 0 ? SC : 1) == 0;
#pragma unroll
  for (int i = 0; i < MAXT; ++i) {
    const int t = lane + 32 * i;
    const int dy = STEP ? lane / S + i * (32 / S) : t / S;
    const int dx = STEP ? lane % S : t - dy * S;
    own[i] = FULLT || t < SS;
    soff[i] = dy * pitch + dx;
  }
  if (lane == 0) {
    for (int d = 0; d < D; ++d) mbar_init(&bar[d], 1);
    mbar_fence_init();
  }
  if (threadIdx.x == 0) s_fail = 0;

  // consumer position in this warp's ring (persists across items)
  int cst = 0;
  uint32_t cpar = 0;
  for (;;) {
    __syncthreads();  // the last item's window reads; s_fail
    if (threadIdx.x == 0) s_item = atomicAdd(A.ticket, 1);
    __syncthreads();
    if (s_fail) return;  // a warp's wait ran out: its copies have landed
    const int it = s_item;
    if (it >= *A.nitems) break;
    const WorkItem w = A.items[it];
    const TileOrigin org = tile_origin(A, w.tile);
    const int n = w.count;
    const int mine = n > warp ? (n - warp + nw - 1) / nw : 0;

    // this warp's records: footprint base in the window, slice, destination
    for (int q = lane; q < mine; q += 32) {
      const int j = w.start + warp + q * nw;
      const VisRec r = A.recs[j];
      meta[q] = make_int4((r.y0 - org.wy0) * pitch + (r.x0 - org.wx0), r.k0 * QQ + r.k1,
                          A.perm[j], 0);
    }
    __syncwarp();
    int issued = 0;
    for (int ist = cst; issued < min(mine, D - 1); ++issued) {
      bulk_load_if(lane == 0, stages + (size_t)ist * KS, R.ktab + (size_t)meta[issued].y * KS,
                   slice_bytes, &bar[ist]);
      ist = ist + 1 == D ? 0 : ist + 1;
    }
    // the window, while the first copies are in flight
    for (int c = threadIdx.x; c < A.win * A.win; c += blockDim.x) {
      const int r = c / A.win, q = c - r * A.win;
      const int gy = org.wy0 + r, gx = org.wx0 + q;
      win[r * pitch + q] = (gy < A.H && gx < A.W)
                               ? __ldg(&R.grid[org.layer_off + (size_t)gy * A.W + gx])
                               : zero;
    }
    __syncthreads();

    int q = 0;
    bool failed = false;
    for (; q < mine; ++q) {
      if (issued < mine) {  // into the stage visibility q - 1 used
        const int ist = cst == 0 ? D - 1 : cst - 1;
        bulk_load_if(lane == 0, stages + (size_t)ist * KS, R.ktab + (size_t)meta[issued].y * KS,
                     slice_bytes, &bar[ist]);
        ++issued;
      }
      // a limit of 0 (a test of the timeout path) polls without blocking
      bool ok = R.wait_cycles ? mbar_try(&bar[cst], cpar) : mbar_test(&bar[cst], cpar);
      if (!__all_sync(FULL_MASK, ok)) {  // warp-uniform slow path, bounded
        const long long t0 = clock64();
        while (!ok && clock64() - t0 <= R.wait_cycles) ok = mbar_try(&bar[cst], cpar);
        if (__any_sync(FULL_MASK, !ok)) {
          failed = true;
          break;
        }
      }
      const int4 m = meta[q];
      const float2 *kp = stages + (size_t)cst * KS + lane;
      float2 sum = zero;
#pragma unroll
      for (int i = 0; i < MAXT; ++i)
        if (own[i]) cfma(sum, win[m.x + soff[i]], kp[32 * i]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sum.x += __shfl_xor_sync(FULL_MASK, sum.x, o);
        sum.y += __shfl_xor_sync(FULL_MASK, sum.y, o);
      }
      if (lane == 0) R.out[m.z] = sum;
      if (++cst == D) {
        cst = 0;
        cpar ^= 1u;
      }
      __syncwarp();  // this stage's reads before a copy reuses it
    }
    if (failed) {
      // record the timeout, let this warp's copies in flight land; the CTA
      // stops at the next item boundary
      if (lane == 0) {
        atomicAdd((int32_t *)&A.status[ST_TIMEOUT], 1);
        s_fail = 1;
        int st = cst;
        uint32_t par = cpar;
        for (int jx = q; jx < issued; ++jx) {
          mbar_wait(&bar[st], par);
          if (++st == D) {
            st = 0;
            par ^= 1u;
          }
        }
      }
      __syncwarp();
    }
  }
}

int ring_degrid_launch(const cg_plan *p, const float2 *ktab, const float2 *grid, float2 *out,
                       cudaStream_t s) {
  const int S = p->kd.S, SS = S * S;
  if (p->kd.sep || S > 16) return CG_ERR_ARG;
  const int KS = p->slice_stride;
  const int prc = padded_table(p, ktab, s);
  if (prc) return prc;
  if ((KS * 8) % 16 != 0 || ((uintptr_t)ktab & 15) != 0) return CG_ERR_ARG;
  const int need = (SS + 31) / 32;
  int maxt = 1;
  while (maxt < need) maxt *= 2;
  // 8 warps and 2 stages: 4 CTAs per SM with 512-visibility items, which
  // measured fastest on the AW set (3.79 ms against 3.86 with 5 CTAs, 4.29
  // with 3 stages and 3 CTAs, 4.95 with 16 warps per CTA)
  const int warps = 8;
  auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  RingArgs R;
  R.ktab = ktab;
  R.grid = grid;
  R.out = out;
  R.wait_cycles = wait_cycles();
  R.kstride = KS;
  R.depth = 2;
  R.win_bytes = (int)up16((size_t)p->pitch * p->win * sizeof(float2));
  const int per_warp = (p->chunk + warps - 1) / warps;
  size_t off = (size_t)R.depth * KS * sizeof(float2);
  R.meta_off = (int)off;
  off += (size_t)per_warp * sizeof(int4);
  R.bar_off = (int)off;
  R.warp_bytes = (int)up16(off + R.depth * sizeof(uint64_t));
  const size_t smem = (size_t)R.win_bytes + (size_t)warps * R.warp_bytes;
  CG_REQUIRE(smem <= (227u << 10), "ring degridder does not fit in shared memory (%zu bytes)",
             smem);
  void *fn = nullptr;
  if (maxt == 8 && SS == 256 && p->pitch == 32) fn = (void *)k_degrid_ring<8, true, 16, 32>;
  else if (maxt == 8 && SS == 256) fn = (void *)k_degrid_ring<8, true>;
  else if (maxt == 2 && SS == 64) fn = (void *)k_degrid_ring<2, true>;
  else if (maxt == 1) fn = (void *)k_degrid_ring<1, false>;
  else if (maxt == 2) fn = (void *)k_degrid_ring<2, false>;
  else if (maxt == 4) fn = (void *)k_degrid_ring<4, false>;
  else if (maxt == 8) fn = (void *)k_degrid_ring<8, false>;
  CG_REQUIRE(fn, "no ring degridder for support %d", S);
  const int threads = 32 * warps;
  CG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  CG_REQUIRE(per_sm > 0, "ring degridder does not fit on an SM (smem %zu)", smem);
  const int64_t blocks =
      std::max<int64_t>(1, std::min<int64_t>((int64_t)per_sm * num_sms(), p->max_items));
  TiledArgs A = tiled_args(p);
  CG_CUDA(cudaMemsetAsync(p->ticket, 0, sizeof(int32_t), s));
  void *args[] = {&A, &R};
  CG_CUDA(cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(threads), args, smem, s));
  return CG_OK;
}

}  // namespace cg
