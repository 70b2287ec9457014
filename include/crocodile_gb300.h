/*
 * crocodile_gb300 -- C ABI of the GB300 (sm_103a) convolutional gridding path.
 *
 * Each entry point replaces one function of crocodile's gridding path
 * (crocodile/synthesis.py in the SKA-ScienceDataProcessor/crocodile
 * reference); the replaced function is cited beside it.  All array
 * arguments are DEVICE pointers owned by the caller unless stated
 * otherwise; the library never frees caller memory.  Complex arrays are
 * interleaved (re, im): "c64" = 2 x float32, "c128" = 2 x float64.
 * Every call is ordered on the given stream (NULL = legacy default stream).
 *
 * Return value: CG_OK (0) or a negative CG_ERR_* code; cg_last_error()
 * gives a message for the calling thread.  No exception crosses the ABI
 * and no kernel traps: data errors found on the device (coordinates out of
 * range, footprints outside the grid, bad kernel indices) are counted in a
 * caller-visible status block and every later kernel of the same call
 * leaves its outputs untouched.  cg_status_check() reads the block.
 */
#ifndef CROCODILE_GB300_H
#define CROCODILE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *cg_stream_t; /* == cudaStream_t */

#define CG_OK 0
#define CG_ERR_ARG (-1)       /* bad argument: shape, null pointer, unsupported size */
#define CG_ERR_RANGE (-2)     /* p outside [-0.5, 0.5): AssertionError at synthesis.py:432 */
#define CG_ERR_BOUNDS (-3)    /* footprint outside the grid: ValueError at synthesis.py:480 */
#define CG_ERR_INDEX (-4)     /* kernel group / weighting cell out of range: IndexError */
#define CG_ERR_CUDA (-5)      /* CUDA or cuFFT error */
#define CG_ERR_WORKSPACE (-6) /* workspace smaller than the *_workspace_bytes query */
#define CG_ERR_TIMEOUT (-7)   /* a bounded device wait gave up */

/* Status block: CG_STATUS_WORDS int32 counters in device memory, zeroed by
 * cg_status_reset.  [0] range errors, [1] footprint errors, [2] index
 * errors, [3] timeouts. */
#define CG_STATUS_WORDS 4

const char *cg_last_error(void);
int cg_version(void);
int cg_status_reset(int32_t *d_status, cg_stream_t stream);
/* Synchronises the stream, copies the block to counts_out (may be NULL)
 * and returns the CG_ERR_* code of the first non-zero counter. */
int cg_status_check(const int32_t *d_status, int32_t *counts_out, cg_stream_t stream);

/* ------------------------------------------------------------------ */
/* Visibility coordinates.  Throughout, visibility i has coordinates
 * p = (uvw[i*stride+0], uvw[i*stride+1]) / lam as a fraction of the grid
 * (pass lam = 1 for coordinates already in grid fractions). */

/* frac_coords (synthesis.py:419-449): x, xf from p[:,0] over the width W,
 * y, yf from p[:,1] over the height H; bit-exact with numpy (FP64, IEEE
 * rounding, half-to-even, floor division).  Outputs are int32 device
 * arrays of length n.  Range errors are counted in d_status[0]. */
int cg_frac_coords(const double *uvw, int64_t stride, double lam, int64_t n,
                   int H, int W, int Q, int32_t *x, int32_t *xf, int32_t *y,
                   int32_t *yf, int32_t *d_status, cg_stream_t stream);

/* w bins of w_cache_imaging / w_cache_predict (synthesis.py:793, 825):
 * k_i = round(w_i / wstep) (half-to-even; w = uvw[i*stride+2], stride >= 3).
 * Writes kidx[i] = k_i - min(k) (a kernel-table row), stores (min k, max k)
 * in h_minmax (host, 2 ints) and synchronises the stream.  d_minmax is a
 * 2-int device scratch.  The kernel of row j is the one for
 * w = wstep * (min k + j). */
int cg_w_bins(const double *uvw, int64_t stride, int64_t n, double wstep,
              int32_t *kidx, int32_t *d_minmax, int32_t *h_minmax,
              int32_t *d_status, cg_stream_t stream);
/* Same bins against a kernel table that already covers k in [kmin, kmin+nk):
 * kidx[i] = k_i - kmin, bins outside the table are index errors.  Fully
 * stream-ordered (no synchronisation), for steady-state imaging loops. */
int cg_w_bins_fixed(const double *uvw, int64_t stride, int64_t n, double wstep,
                    int kmin, int nk, int32_t *kidx, int32_t *d_status,
                    cg_stream_t stream);

/* ------------------------------------------------------------------ */
/* Kernel (GCF) tables, as built by make_gcf (synthesis.py:451-461):
 *   sep = 1: [G, Q, S] table, footprint = outer(K[g,yf], K[g,xf])
 *   sep = 0: [G, Q, Q, S, S] table, footprint = K[g, yf, xf]
 * G counts the flattened leading "src" dimensions; the per-visibility
 * group index kidx (int32, may be NULL for G = 1) selects one. */
typedef struct {
  int sep;
  int Q;
  int S;
  int G;
} cg_kernel_desc;

/* Launch-shape tuning of the tiled kernels (no reference counterpart; the
 * autotuner in crocodile_gb300/autotune.py sets it).  Zero fields mean
 * "automatic".  tile: grid tile edge in cells (multiple of 4, <= 64; read
 * when a plan is created); chunk: visibilities per work item (plan
 * creation); layout: gridder layout, CG_LAYOUT_WARP (one warp per
 * visibility, shared-memory atomics), CG_LAYOUT_OWNER (threads own window
 * cells by position mod S and keep running sums in registers) or
 * CG_LAYOUT_LANE (one warp per work item with a private window, lanes own
 * cells by position mod S, kernel slices streamed by bulk copies; S <= 16;
 * also selects the lane form of cg_degrid_grid; odd S * S slices stream
 * from a padded copy of the table in the plan's workspace); rows: row
 * residues per owner-layout thread (1..8), or bulk-copy stages per
 * lane-layout warp (2..4; other values: 3); groups: owner-layout thread
 * groups, or warp-layout warps, per CTA (1..8), or lane-layout warps per
 * CTA (1..16); dvis: the degridder: 0 (automatic) or 2 runs the tiled
 * degridder with 2 visibilities per warp step, 4 with 4; 1 runs lane-layout
 * plans through the lane kernel's degridding traversal (others as 0); 3 runs
 * plans whose table streams by bulk copies (non-separable, S <= 16, 16-byte
 * slices) through the ring degridder: the item's window in shared memory,
 * each warp's slices by bulk copies through a 2-stage ring (others as 0).  layout 0 picks CG_LAYOUT_LANE (with 16-cell tiles) for
 * non-separable tables with even S <= 16, whose slices stream by bulk
 * copies as they are, and CG_LAYOUT_WARP otherwise.  Process-wide. */
#define CG_LAYOUT_WARP 1
#define CG_LAYOUT_OWNER 2
#define CG_LAYOUT_LANE 3
typedef struct {
  int tile;
  int chunk;
  int rows;
  int groups;
  int layout;
  int dvis;
} cg_tuning;
int cg_set_tuning(const cg_tuning *t);
int cg_get_tuning(cg_tuning *out);

/* The lane gridders wait for each kernel slice's bulk copy for at most this
 * many SM clock cycles (default 4e9, about two seconds); a wait that runs out
 * counts CG_ERR_TIMEOUT in the status block, the warp lets its copies in
 * flight land (waiting at most the default limit) and stops, and the call
 * returns.  The FP32 FFT's column passes wait for their tensor copies under
 * the same limit; a wait that runs out there is counted in a device-wide
 * counter that cg_fft_timeouts reads (after synchronising the device; reset
 * nonzero: set it back to 0), and the transform's output is undefined.  No
 * counterpart in the reference: a test hook that makes a wait run out on
 * purpose (a limit of 0 fails every copy not yet landed when it is first
 * polled).  Process-wide. */
int cg_set_wait_limit(long long cycles);
long long cg_get_wait_limit(void);
int cg_fft_timeouts(int32_t *count, int reset);

/* A plan holds the visibilities' bit-exact cell assignment, their order
 * (sorted into grid tiles, or into kernel groups for the plain FP64 form)
 * and the work list of the gridding kernels.  It lives in a caller-owned
 * workspace and is reused by any number of grid/degrid calls on the same
 * coordinates (imaging and its PSF, predict, the adjoint pair). */
typedef struct cg_plan cg_plan;

#define CG_PLAN_TILED 0  /* FP32 tiled gridder/degridder (cg_grid, cg_degrid) */
#define CG_PLAN_GROUPS 1 /* plain FP64 form, one launch per kernel group */

size_t cg_plan_workspace_bytes(int mode, int64_t n, int H, int W,
                               const cg_kernel_desc *kd);
/* Builds the plan on `stream`.  CG_PLAN_GROUPS synchronises once to learn
 * the group sizes.  A data error leaves the plan marked failed (see
 * cg_status_check); grid/degrid then do nothing. */
int cg_plan_create(cg_plan **plan, int mode, const cg_kernel_desc *kd, int H,
                   int W, const double *uvw, int64_t stride, double lam,
                   const int32_t *kidx, int64_t n, void *workspace,
                   size_t workspace_bytes, int32_t *d_status,
                   cg_stream_t stream);
/* Same, with each visibility's kernel group taken from its w bin:
 * g = round(w / wstep) - kmin (w = uvw[i*stride+2], stride >= 3), the
 * binning of w_cache_imaging (synthesis.py:793) fused into the plan's
 * coordinate pass; kd->G is the number of bins in the kernel table and bins
 * outside [kmin, kmin + G) are index errors. */
int cg_plan_create_wbins(cg_plan **plan, int mode, const cg_kernel_desc *kd,
                         int H, int W, const double *uvw, int64_t stride,
                         double lam, double wstep, int kmin, int64_t n,
                         void *workspace, size_t workspace_bytes,
                         int32_t *d_status, cg_stream_t stream);
/* Extended plan options (no reference counterpart beyond the functions
 * cited): layers > 1 grids each visibility into grid layer[i] of a stack of
 * `layers` H x W grids laid out one after another (the per-plane grids of
 * w-stacking, examples/notebooks/wstacking.ipynb cell 10), all in one launch;
 * wstep != 0 takes kernel groups from w bins as cg_plan_create_wbins. */
typedef struct {
  int layers;
  const int32_t *layer; /* device int32 [n], or NULL when layers == 1 */
  double wstep;
  int kmin;
  /* CG_PLAN_GROUPS only: launch group per visibility (device int32 [n]) in
   * [0, ngroups), e.g. the w-plane, when each visibility's kernel row (kidx)
   * is finer than the launches (AW kernels: one launch per w-plane). */
  const int32_t *group;
  int ngroups;
  /* Tiled mode: grid tile edge for this plan (multiple of 4, <= 64), or 0 for
   * the process-wide tuning / automatic choice.  Sparse stacks of small grids
   * (the sub-grids of w-towers) want large tiles: more visibilities per item. */
  int tile;
} cg_plan_opts;
size_t cg_plan_workspace_bytes_ex(int mode, int64_t n, int H, int W,
                                  const cg_kernel_desc *kd,
                                  const cg_plan_opts *opts);
int cg_plan_create_ex(cg_plan **plan, int mode, const cg_kernel_desc *kd,
                      int H, int W, const double *uvw, int64_t stride,
                      double lam, const int32_t *kidx, int64_t n,
                      const cg_plan_opts *opts, void *workspace,
                      size_t workspace_bytes, int32_t *d_status,
                      cg_stream_t stream);
int cg_plan_destroy(cg_plan *plan);
/* Tile edge (cells) and number of work items upper bound, for reports. */
int cg_plan_info(const cg_plan *plan, int64_t *info_out /* [4] */);
/* Copies of a plan's sort into caller device buffers, for checks (no
 * reference counterpart; the reference grids in input order): recs_out [n x 4]
 * int32 {x0, y0, k0, k1} (footprint origin and kernel rows, sorted by
 * bucket), perm_out [n] (sorted position -> input index), counts_out
 * [nbuckets] (visibilities per bucket: grid tile, or tile and sub-tile along a
 * Morton curve; kernel group in CG_PLAN_GROUPS mode; nbuckets = info[3] of
 * cg_plan_info).  Any output may be NULL.  Stream-ordered. */
int cg_plan_export(const cg_plan *plan, int32_t *recs_out, int32_t *perm_out,
                   int32_t *counts_out, cg_stream_t stream);

/* convgrid (synthesis.py:464-481): grid[H,W] (c64) += K * vis (c64).
 * FP32 products and accumulation; persistent tiled kernel; CG_PLAN_TILED. */
int cg_grid(const cg_plan *plan, const void *ktab_c64, const void *vis_c64,
            void *grid_c64, cg_stream_t stream);
/* Same, with the visibilities multiplied by a real per-visibility weight
 * (do_imaging's wt * vis, synthesis.py:901-906); vis_c64 may be NULL for
 * the PSF pass (vis = 1). */
int cg_grid_weighted(const cg_plan *plan, const void *ktab_c64,
                     const void *vis_c64, const float *weight,
                     void *grid_c64, cg_stream_t stream);
/* convgrid (synthesis.py:464-481) for sparse grid stacks: the same sums as
 * cg_grid, without shared-memory windows — every tap is a float2 atomic into
 * the grid.  For plans with few visibilities per tile (the many sub-grids of
 * w-towers), where cg_grid's per-item window costs more than the taps. */
int cg_grid_sparse(const cg_plan *plan, const void *ktab_c64, const void *vis_c64,
                   void *grid_c64, cg_stream_t stream);
/* convdegrid (synthesis.py:484-503): out[i] = sum(grid[footprint] * K). */
int cg_degrid(const cg_plan *plan, const void *ktab_c64, const void *grid_c64,
              void *vis_out_c64, cg_stream_t stream);
/* Degridding and gridding in one pass over the plan (each kernel tap read
 * once for both): vis_out = convdegrid(grid_in) (synthesis.py:484-503) and
 * grid_out += convgrid of u (:464-481) with u = vis_in, or, with
 * residual != 0, u = vis_in - vis_out (predict, subtract and invert: the
 * major-cycle step of do_predict followed by do_imaging's gridding).
 * vis_in may be NULL without residual (grids zeros); vis_out may be NULL.
 * grid_in and grid_out must differ.  FP32, c64 data. */
int cg_degrid_grid(const cg_plan *plan, const void *ktab_c64,
                   const void *grid_in_c64, const void *vis_in_c64, int residual,
                   void *vis_out_c64, void *grid_out_c64, cg_stream_t stream);

/* cg_update_peak: no counterpart in the reference (a measurement utility).
 * One launch of an update-rate microbenchmark, the peaks that the gridders'
 * grid-point update rate is compared with.  kind 0: shared-memory
 * read-modify-write updates of float2 cells, the lane gridder's inner loop
 * without its HBM traffic (per warp a private 31 x 32 window and a 16 x 16
 * tap slice in shared memory; `work` synthetic visibilities of 256 updates
 * per warp; buf receives one value per warp, >= 8 * 16 * SMs bytes).
 * kind 1: float2 atomic additions into an L2-resident buffer (red.global.add
 * of 32 consecutive cells per warp instruction; `work` instructions per warp;
 * buf >= 256 KiB, at most 32 MiB of it used).  *updates receives the cell
 * updates the launch performs; time it with events on `stream`. */
int cg_update_peak(int kind, int work, void *buf, size_t buf_bytes, double *updates,
                   cg_stream_t stream);

/* cg_grid_noalloc: no counterpart in the reference.  For callers that
 * cannot allocate device memory (a pipeline that owns all GPU memory in its
 * own pool and may not call cudaMalloc/cudaFree while it runs, or an FFI
 * host with nothing but its input and output buffers to pass): the same
 * result as cg_plan_create + cg_grid (FP32, grid += K * vis), with the
 * plan's scratch in a static device array of CG_NOALLOC_SCRATCH_BYTES that
 * the library holds on every GPU that loads it until the process exits.
 * Allocates nothing, on the host or the device.  Inputs and outputs are the
 * caller's device buffers, as for cg_grid; d_status is the caller's status
 * block.  Returns CG_ERR_WORKSPACE, writing nothing, when n visibilities on
 * an H x W grid need more scratch than that.  The need depends on n, the grid
 * and the gridder layout; cg_plan_workspace_bytes(CG_PLAN_TILED, ...) gives
 * it.  It is about 44 B per visibility plus the bucket tables and work
 * list: about H * W / 8 bytes for the lane layout (non-separable tables,
 * even S <= 16), but H * W / 2 bytes for the warp and owner layouts (4 x
 * 4-cell sub-tile buckets), which alone exceed the array above about
 * 5800 x 5800.  So a 512 x 512 grid takes up to about 380 000 visibilities,
 * a 4096 x 4096 grid about 330 000 with the lane layout but only about
 * 190 000 with the others.
 * The first call on a device looks up the array's device address, once per
 * device, with that device current; make that first call before any stream
 * capture.  The address stays cached, so calls after cudaDeviceReset in the
 * same process are not supported.  All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. */
#define CG_NOALLOC_SCRATCH_BYTES (16u << 20)
int cg_grid_noalloc(const cg_kernel_desc *kd, int H, int W, const double *uvw,
                    int64_t stride, double lam, const int32_t *kidx, int64_t n,
                    const void *ktab_c64, const void *vis_c64, void *grid_c64,
                    int32_t *d_status, cg_stream_t stream);

/* Plain FP64 form of the same two operations (c128 data, FP64 atomics,
 * one launch per kernel group): the accuracy and speed comparator.
 * Needs a CG_PLAN_GROUPS plan. */
int cg_grid_fp64(const cg_plan *plan, const void *ktab_c128,
                 const void *vis_c128, void *grid_c128, cg_stream_t stream);
int cg_degrid_fp64(const cg_plan *plan, const void *ktab_c128,
                   const void *grid_c128, void *vis_out_c128,
                   cg_stream_t stream);

/* ------------------------------------------------------------------ */
/* Boxcar gridding, grid/degrid (synthesis.py:389-416): nearest cell
 * N//2 + floor(0.5 + N*p), N = H (as the reference uses a.shape[0]).
 * Coordinates not below 0.5 in any of the first min(stride, 3) columns are
 * range errors (the reference asserts max(p) < 0.5 over u, v and w).
 * c128 data, FP64. */
int cg_grid_boxcar(const double *uvw, int64_t stride, double lam, int64_t n,
                   const void *vis_c128, void *grid_c128, int H, int W,
                   int32_t *d_status, cg_stream_t stream);
int cg_degrid_boxcar(const double *uvw, int64_t stride, double lam, int64_t n,
                     const void *grid_c128, void *vis_out_c128, int H, int W,
                     int32_t *d_status, cg_stream_t stream);

/* doweight (synthesis.py:535-549): w_out[i] = v_in[i] / count(cell(i)) on
 * an N x N grid (v_in NULL = ones).  counts is an int32 N*N scratch array. */
int cg_weights(const double *uvw, int64_t stride, double lam, int64_t n,
               int N, const double *v_in, double *w_out, int32_t *counts,
               int32_t *d_status, cg_stream_t stream);

/* mirror_uvw (synthesis.py:831-852), in place: rows with v < 0 become
 * (-u, -v, -w) and their visibility is conjugated (vis may be NULL). */
int cg_mirror_uvw(double *uvw, int64_t stride, int64_t n, void *vis,
                  int vis_is_c64, cg_stream_t stream);

/* make_grid_hermitian (synthesis.py:855-880), in place. */
int cg_make_hermitian(void *grid, int H, int W, int is_c64,
                      cg_stream_t stream);

/* fft / ifft (synthesis.py:83-106): centred 2-D transform of `batch`
 * H x W arrays (H = 1: 1-D), in place; the inverse includes 1/(H*W).
 * Grids with H and W even need no workspace; otherwise workspace must hold
 * one array of the same size.  complex64 with power-of-two sides 64..8192
 * run the library's own FP32 FFT; from H = 2048 its column passes go
 * through a scratch stack of at most 1 GiB taken from a memory pool the
 * library keeps per device (stream-ordered, retained after the first use). */
int cg_fft(void *data, int batch, int H, int W, int is_c64, int inverse,
           void *workspace, cg_stream_t stream);
/* The same transforms unshifted and unnormalised (cuFFT's own convention):
 * for callers that fold the centring shifts and the 1/(H W) of the inverse
 * into neighbouring passes (the w-towers pipeline). */
int cg_fft_raw(void *data, int batch, int H, int W, int is_c64, int inverse,
               cg_stream_t stream);
/* batch contiguous complex128 rows of length n (a power of two, 64..8192;
 * 4096 and 8192 by a four-step factorisation over the 2048-point transform)
 * transformed in place, unshifted and unnormalised (inverse: exp(+2 pi i)),
 * in double-float arithmetic (hi + lo pairs of floats, about 48 significant
 * bits) on the FP32 units: GB300's FP64 rate bounds an FP64 FFT. */
int cg_fft_rows_df(void *data_c128, int64_t batch, int n, int inverse, cg_stream_t stream);
/* cg_fft's centred 2-D transform (fft / ifft of synthesis.py) of batch
 * complex128 planes H x W in place, H and W powers of two 64..2048, in the
 * same double-float arithmetic: a row pass with the (-1)^(i+j) modulation
 * that stands for ifftshift, then a column pass with the fftshift modulation
 * and the 1/(H W) of the inverse. */
int cg_fft2_centred_df(void *data_c128, int64_t batch, int H, int W, int inverse,
                       cg_stream_t stream);

/* Dirty image / PSF of a grid (synthesis.py:904-907): image = Re(ifft(
 * make_grid_hermitian(grid))), written as float32 H x W; the grid is
 * consumed (overwritten).  If max_out is not NULL the image maximum is
 * stored there (float, device).  Even H and W only. */
int cg_image_from_grid(void *grid_c64, int H, int W, float *image_out,
                       float *max_out, cg_stream_t stream);
/* image *= 1 / *d_scale (do_imaging's normalisation, synthesis.py:909-911) */
int cg_scale_image(float *image, int64_t count, const float *d_scale,
                   cg_stream_t stream);

/* Distinct keys: for keys in [0, nkeys), row[i] = rank of key[i] among the
 * distinct keys present (ascending), key_of_row[r] = the r-th distinct key
 * (room for min(n, nkeys) entries), *h_nrows (host) = their number;
 * synchronises the stream.  The keys in use are a bitmap (nkeys / 8 bytes
 * of the workspace).  Replaces the kernel cache lookup of w_cache_imaging
 * (synthesis.py:788, 794) with one table row per distinct cache key. */
size_t cg_compact_keys_workspace_bytes(int nkeys);
int cg_compact_keys(const int32_t *key, int64_t n, int nkeys, int32_t *row,
                    int32_t *key_of_row, int32_t *h_nrows, void *workspace,
                    size_t workspace_bytes, int32_t *d_status,
                    cg_stream_t stream);
/* Kernel-cache keys of w_cache_imaging with integer src columns (the
 * kernel_cache(theta, wbin, *src[i]) lookup of synthesis.py:793-794):
 * key[i] = ((round(w_i / wstep) - kmin) * r0 + (c0 - m0)) * r1 + (c1 - m1) ...
 * over the ncols (<= 8) int32 columns cols[i * ncols + c], with the minima
 * m and ranges r given on the host; the key space nbins * r0 * r1 ... must
 * stay below 2^31.  Values outside [m, m + r) count CG_ERR_INDEX.  The keys
 * feed cg_compact_keys. */
int cg_row_keys(const double *uvw, int64_t stride, int64_t n, double wstep, int kmin, int nbins,
                const int32_t *cols, int ncols, const int32_t *col_min, const int32_t *col_range,
                int32_t *key, int32_t *d_status, cg_stream_t stream);
/* AW cache keys (the (wbin, a1, a2) arguments of aw_kernel_fn through
 * w_cache_imaging, synthesis.py:719, 793-794; scripts/image_dataset.py:153-171):
 * key[i] = (a1[i] * nant + a2[i]) * nbins + round(w_i / wstep) - kmin. */
int cg_aw_keys(const double *uvw, int64_t stride, const int32_t *a1,
               const int32_t *a2, int64_t n, int nant, double wstep, int kmin,
               int nbins, int32_t *key, int32_t *d_status, cg_stream_t stream);

/* ------------------------------------------------------------------ */
/* w-stacking (examples/notebooks/wstacking.ipynb code cell 10, with
 * convolutional gridding): after gridding every plane into one layer of a
 * layered plan (cg_plan_create_ex) and an inverse centred cg_fft of the
 * stack, image = sum_p plane_p / w_kernel_function(l, m, mean w of plane p)
 * (synthesis.py:273-293).  cg_plan_layer_mean_w writes the mean w (double)
 * and visibility count (int32, may be NULL) of each layer (FP64 sums over
 * chunks of the layer, the chunk sums added in an order that varies between
 * runs); cg_wstack_combine forms the complex64 N x N image (planes
 * without visibilities are skipped, as in the notebook). */
int cg_plan_layer_mean_w(const cg_plan *plan, const double *uvw, int64_t stride,
                         double *mean_out, int32_t *count_out,
                         cg_stream_t stream);
int cg_wstack_combine(const void *planes_c64, int layers, int N, double theta,
                      const double *mean_w, const int32_t *counts,
                      void *image_c64, int32_t *d_status, cg_stream_t stream);

/* w-towers: w-stacking on sub-grids (examples/grid/grid.c:482-710,
 * examples/notebooks/wtowers.ipynb code cell 16).  Visibility i falls into
 * the uv chunk ub = floor(u*theta / chunk), vb = floor(v*theta / chunk)
 * (chunk = sub-grid size - margin) and the w-plane wp = rint(w / wincrement);
 * the chunk's sub-grid is centred xmid = (chunk*ub + chunk*(ub+1)) // 2 cells
 * from the grid centre (likewise ymid).
 * cg_tower_keys writes key_out[i] = ((vb - vbmin)*nub + (ub - ubmin))*nwp +
 * (wp - wpmin) and rel_out[i] = (u - xmid/theta, v - ymid/theta,
 * w - wp*wincrement) (IEEE double, as numpy); h_bounds (host) = {ubmin,
 * ubmax, vbmin, vbmax, wpmin, wpmax}; d_minmax is 6 int32 of device scratch;
 * synchronises the stream.  The (chunk, plane) layers are then gridded with a
 * layered plan on rel_out (lam = sub-grid size / theta, residual-w kernels)
 * and inverse-transformed (cg_fft).
 * cg_towers_combine: out[c] = sum over layers L in [chunk_first[c],
 * chunk_first[c+1]) of stack[L] / w_kernel_function(l, m, layer_w[L]) on the
 * sub-grid's l, m (the Fresnel transfer between w-planes, grid.c:598-622).
 * cg_towers_add: after a forward cg_fft of out, grid[origin[2c+1] + i,
 * origin[2c] + j] += out[c, i, j] inside the N x N grid (grid.c:640-656). */
int cg_tower_keys(const double *uvw, int64_t stride, int64_t n, double theta, int chunk,
                  double wincrement, int32_t *key_out, double *rel_out, int32_t *d_minmax,
                  int32_t *h_bounds, int32_t *d_status, cg_stream_t stream);
int cg_towers_combine(const void *stack_c64, int layers, int S, double theta,
                      const double *layer_w, const int32_t *chunk_first, int nchunks,
                      void *out_c64, int32_t *d_status, cg_stream_t stream);
int cg_towers_add(const void *sub_c64, int nchunks, int S, const int32_t *origin, int N,
                  void *grid_c64, cg_stream_t stream);
/* w-towers predict (examples/notebooks/wtowers-predict.ipynb), the reverse:
 * cg_towers_cut copies each chunk's S x S sub-grid of the N x N grid at origin
 * (zeros outside), rolled by S/2 for an unshifted inverse cg_fft_raw;
 * cg_towers_expand forms each layer's sub-grid image, chunk image /
 * w_kernel_function(l, m, layer_w[L]), rolled and sign-modulated so that an
 * unshifted forward cg_fft_raw of the stack gives the centred sub-grids, which a
 * layered plan's cg_degrid then degrids with the residual-w kernels. */
int cg_towers_cut(const void *grid_c64, int N, const int32_t *origin, int nchunks, int S,
                  void *out_c64, cg_stream_t stream);
int cg_towers_expand(const void *images_c64, int S, double theta, const double *layer_w,
                     const int32_t *chunk_first, int nchunks, void *out_c64, int32_t *d_status,
                     cg_stream_t stream);

/* ------------------------------------------------------------------ */
/* Kernel generation (FP64 arithmetic; outputs c64 or c128). */

/* kernel_oversample (synthesis.py:330-354) of `batch` far fields ff
 * (c128, batch x N0 (ndim 1) or batch x N0 x N0 (ndim 2)) into
 * batch x [Q, s] or batch x [Q, Q, s, s]. */
size_t cg_kernel_oversample_workspace_bytes(int batch, int ndim, int N0, int Q);
int cg_kernel_oversample(const void *ff_c128, int batch, int ndim, int N0,
                         int Q, int s, void *out, int out_c64, void *workspace,
                         size_t workspace_bytes, cg_stream_t stream);

/* w_kernel (synthesis.py:357-377) for nw w values (host array): each
 * output is [Q, Q, S, S].  T (host, row-major 2x2) may be NULL. */
size_t cg_w_kernels_workspace_bytes(int nw, int NpixFF, int Q);
int cg_w_kernels(double theta, const double *w_host, int nw, int NpixFF,
                 int S, int Q, int invert, double dl, double dm,
                 const double *T_host, void *out, int out_c64,
                 void *workspace, size_t workspace_bytes, int32_t *d_status,
                 cg_stream_t stream);

/* aw_kernel_fn (synthesis.py:701-734): for each of nk AW kernels k,
 *   akern = convolve2d(A[a1[k]], A[a2[k]], 'same')        (SA x SA)
 *   out[k, yf, xf] = convolve2d(akern, W[wi[k], yf, xf], 'same')
 * A: [nA, SA, SA] c128, W: [nW, Q, Q, S, S] c128, out: [nk, Q, Q, SA, SA]
 * c64 or c128.  a1, a2, wi: int32 device arrays.  A kernels are combined
 * in FP64 and rounded once to FP32; W is rounded once to FP32 into the
 * workspace; the Q*Q sub-kernel convolutions use FP32 arithmetic: direct
 * sums, or for complex64 output of 16 x 16 kernels with S <= 16 the exact
 * circular convolution of the zero-padded kernels by 32 x 32 FFTs.
 * Workspace: cg_aw_kernels_workspace_bytes(nk, SA, nW, Q, S) bytes. */
size_t cg_aw_kernels_workspace_bytes(int nk, int SA, int nW, int Q, int S);
int cg_aw_kernels(const void *A_c128, int nA, int SA, const void *W_c128,
                  int nW, int Q, int S, const int32_t *a1, const int32_t *a2,
                  const int32_t *wi, int nk, void *out, int out_c64,
                  void *workspace, size_t workspace_bytes, int32_t *d_status,
                  cg_stream_t stream);

/* AW-towers (examples/notebooks/awtowers.ipynb cells 17-22): w-towers with
 * per-baseline antenna terms applied in each sub-grid's image space.
 * cg_awtower_keys bins visibilities into centred uv chunks, w-planes and
 * baselines, as the notebook (IEEE double, bit-identical to numpy):
 *   ub = floor(u*theta/chunk + 1/2), vb likewise, wp = rint(w / wstep),
 *   key = (((vb-vbmin)*nub + (ub-ubmin))*nwp + (wp-wpmin))*nant^2 + a1*nant + a2,
 *   rel = (u - chunk*ub/theta, v - chunk*vb/theta, w - wp*wstep);
 * h_bounds (host) = {ubmin, ubmax, vbmin, vbmax, wpmin, wpmax}; synchronises
 * the stream.  The (chunk, plane, baseline) layers are then gridded with the
 * anti-aliasing kernel on 2s x 2s grids (a layered plan on rel with lam =
 * s / theta) and inverse-transformed by an unshifted cg_fft_raw.
 * cg_awtowers_combine: out[c] = sum over layers L in [chunk_first[c],
 * chunk_first[c+1]) of the centred image of layer L cut to its middle s x s,
 * times corr [s, s], times aimage[layer_a2[L]] / aimage[layer_a1[L]]
 * ([nant, s, s] complex64), divided by w_kernel_function(l, m, layer_w[L]);
 * written rolled for a forward cg_fft_raw and cg_towers_add. */
int cg_awtower_keys(const double *uvw, int64_t stride, int64_t n, double theta, int chunk,
                    double wstep, const int32_t *a1, const int32_t *a2, int nant,
                    int32_t *key_out, double *rel_out, int32_t *d_minmax, int32_t *h_bounds,
                    int32_t *d_status, cg_stream_t stream);
int cg_awtowers_combine(const void *stack_c64, int layers, int s, double theta,
                        const float *corr, const void *aimage_c64, int nant,
                        const int32_t *layer_a1, const int32_t *layer_a2,
                        const double *layer_w, const int32_t *chunk_first, int nchunks,
                        void *out_c64, int32_t *d_status, cg_stream_t stream);
/* The layer bookkeeping on the device, from used [nlayers], the ascending
 * distinct keys of cg_awtower_keys (cg_compact_keys): each layer's antennas
 * (layer_a1, layer_a2) and plane index key / nant^2 mod nwp (layer_plane),
 * chunk_first [nchunks + 1] (room for nlayers + 1) and each chunk's sub-grid
 * origin [nchunks][2] = N/2 + chunk*(ub, vb) - chunk/2 - (margin+1)/2 (room for
 * 2 nlayers), *h_nchunks (host); synchronises the stream. */
size_t cg_awtower_layers_workspace_bytes(int nlayers);
int cg_awtower_layers(const int32_t *used, int nlayers, int nant, int nwp, int nub, int ubmin,
                      int vbmin, int chunk, int margin, int N, int32_t *layer_a1,
                      int32_t *layer_a2, int32_t *layer_plane, int32_t *chunk_first,
                      int32_t *origin, int32_t *h_nchunks, void *ws, size_t ws_bytes,
                      cg_stream_t stream);
/* The same out[] without the 2s x 2s layer grids and their transforms, for
 * s = 16, 32 or 64: the anti-aliasing kernel being separable, the unshifted
 * inverse transform of a layer at the cut pixel (Ar, Br) is the sum over its
 * visibilities of vis * Av(Ar) * Au(Br), Av / Au the visibility's taps times
 * exp(+2 pi i (origin + tap) Ar / 2s) summed; plan is the layered tiled plan
 * of the gridding (lam = s / theta, 2s x 2s layers, separable ktab, support
 * <= 16) whose sorted records give each layer's visibilities.  Layer L lies
 * in w-plane layer_plane[L] of nplanes, whose w is plane_w[plane] (the
 * Fresnel factor is tabulated per plane, aimage's reciprocal per antenna).
 * ws: at least cg_awtowers_direct_workspace_bytes(s, nant, nplanes) bytes of
 * device memory. */
size_t cg_awtowers_direct_workspace_bytes(int s, int nant, int nplanes);
int cg_awtowers_direct(const cg_plan *plan, const void *ktab_c64, const void *vis_c64, int s,
                       double theta, const float *corr, const void *aimage_c64, int nant,
                       const int32_t *layer_a1, const int32_t *layer_a2,
                       const int32_t *layer_plane, const double *plane_w, int nplanes,
                       const int32_t *chunk_first, int nchunks, void *out_c64, void *ws,
                       size_t ws_bytes, int32_t *d_status, cg_stream_t stream);

/* ---------------------------------------------------------------- ingest
 * Visibility blocks as the reference's HDF5 files hold them (a vis/[a1]/[a2]
 * group per baseline: frequency [nchan] Hz, time [nrow], uvw [nrow, 3]
 * metres, vis [nrow, nchan, npol] complex128) and the arl Visibility table
 * (antenna1, antenna2 per row), flattened into the gridder's rows in the
 * order of collect_blocks (scripts/image_dataset.py:75-87): block by block,
 * row by row, channel by channel.  Per output row o:
 *   uvw_lambda[o] = uvw[r] * frequency[c] / 299792458  (data_models.py:198-202;
 *                   IEEE-rounded, bit-identical to numpy)
 *   src[o]        = (antenna1[r], antenna2[r], time[r], frequency[c])  (FP64)
 *   vis_out[o]    = vis[r, c, pol]  (complex64 or complex128)
 * blocks: device array; the inputs are the blocks' columns concatenated
 * (row_start, freq_start, vis_start index them).  Any output may be NULL.  A
 * block with pol >= npol, nchan <= 0 or nrow * nchan >= 2^31 counts an
 * index error in d_status and is skipped. */
typedef struct {
  int64_t row_start;  /* first row of the block in uvw_m / time / a1 / a2 */
  int64_t freq_start; /* first channel of the block in freq */
  int64_t vis_start;  /* first element of the block's vis [nrow][nchan][npol] */
  int64_t out_start;  /* first output row of the block */
  int32_t nrow, nchan, npol, pad;
} cg_vis_block;
int cg_ingest_blocks(const cg_vis_block *blocks, int nblocks, const double *uvw_m,
                     const double *time, const int32_t *a1, const int32_t *a2,
                     const double *freq, const void *vis_c128, int pol,
                     double *uvw_lambda, double *src, int32_t *a1_out,
                     int32_t *a2_out, void *vis_out, int vis_c64, int32_t *d_status,
                     cg_stream_t stream);

/* ---------------------------------------------------------------- Sze-Tan
 * Optimal gridding functions (crocodile/antialias.py).  All arrays are FP64
 * device arrays; R is the half support (2R <= 32).
 *
 * calc_gridding_fine (antialias.py:189-213): C [2R, M] (row-major) of the
 * gridding function at offsets nu [M], from h_ext = [1, h...] ([N+1],
 * sampled at x0 * k / N) and kinv, the inverse of the 2R x 2R Gram matrix
 * K[rp, r] = trap(h_ext^2 cos(2 pi (rp - r) x), x0 / N) (row-major). */
int cg_szetan_gridding(const double *h_ext, int nh1, double x0, int R,
                       const double *kinv, const double *nu, int M, double *C,
                       cg_stream_t stream);

/* calc_gridding_correction_fine (antialias.py:229-246): hfine[n] = c(x_n) /
 * d(x_n) for nx coordinates x, from C [2R, M] evaluated at nu_m = (m + 0.5)
 * / (2M).  Workspace: cg_szetan_correction_workspace_bytes(R) bytes. */
size_t cg_szetan_correction_workspace_bytes(int R);
int cg_szetan_correction(const double *C, int R, int M, const double *x,
                         int nx, double *hfine, void *workspace,
                         size_t workspace_bytes, cg_stream_t stream);

/* ---------------------------------------------------------------- facets
 * Facet -> subgrid recombination (examples/grid/recombine.h/.c; the 2-D
 * algorithm of examples/notebooks/facet-subgrid-impl.ipynb cells 24-30).
 * Layout: the C prototype's raw layout (centre at index 0, as numpy's
 * ifftshift) unless a `centred` flag selects numpy's fftshift layout.
 *
 * recombine2d_set_config (recombine.c:135-196): sizes as there, pswf [yN]
 * the PSWF in raw layout (host array; the reference reads it from a file).
 * Fb, Fn and m are generated as generate_Fb/Fn/m (recombine.c:12-67) and kept
 * on the device.  Arrays and FFTs are complex128, as the reference's.
 * Returns CG_ERR_ARG when a side condition of the reference does not hold. */
typedef struct cg_recombine cg_recombine;
int cg_recombine_create(int image_size, int subgrid_spacing, const double *pswf_host,
                        int yB_size, int yN_size, int yP_size, int xA_size,
                        int xM_size, int xMxN_yP_size, cg_recombine **out);
int cg_recombine_destroy(cg_recombine *h);
/* FFTs of the recombination: mode 0 (default) runs double-float arithmetic
 * on the FP32 units (complex128 only in the caller's arrays) when the
 * transform lengths allow: yP_size and xM_yP_size powers of two 64..2048, the
 * fused pipeline (prepare / window / crop steps inside the transforms); yP up
 * to 8192 (four-step rows), the double-float stage kernels; otherwise power-
 * of-two rows up to 2048 in double-float on complex128 stage arrays and other
 * lengths with cuFFT Z2Z.  Mode 1 uses complex128 and cuFFT Z2Z throughout. */
int cg_recombine_set_fft(cg_recombine *h, int mode);
/* sizes[0..4] = xM_yP_size, xM_yN_size, facet_spacing, yP_spacing, xM_spacing */
int cg_recombine_sizes(const cg_recombine *h, int32_t *sizes);
/* host copies of Fb [yB], Fn [xM_yN], m [xMxN_yP] (raw layout; NULL skips) */
int cg_recombine_windows(const cg_recombine *h, double *Fb, double *Fn, double *m);
size_t cg_recombine_workspace_bytes(const cg_recombine *h, int n0, int n1);
/* recombine2d_pf1_ft1_es1 + pf0_ft0 + es0 (recombine.c:242-459) for one facet
 * [yB, yB] and every pair of n0 x n1 subgrid offsets (device arrays, grid
 * cells, multiples of subgrid_spacing; others count CG_ERR_INDEX in d_status):
 * nmbf [n0][n1][xM_yN][xM_yN].  centred / out_centred: facet / nmbf layout. */
int cg_recombine_facet_to_subgrids(cg_recombine *h, const void *facet, int centred,
                                   const int32_t *subgrid_off0, int n0,
                                   const int32_t *subgrid_off1, int n1, void *nmbf,
                                   int out_centred, void *workspace,
                                   size_t workspace_bytes, int32_t *d_status,
                                   cg_stream_t stream);
/* cg_recombine_facet_to_subgrids and cg_recombine_add_facet in one call: the
 * facet's contributions to the n0 x n1 subgrids summed straight into
 * subgrids [n0][n1][xM][xM] at the facet offsets (sub_centred: both layouts
 * as cg_recombine_add_facet's centred flag), the same values and additions,
 * without the intermediate contributions array on the double-float pipeline.
 * Workspace: cg_recombine_workspace_bytes(h, n0, n1). */
int cg_recombine_facet_add(cg_recombine *h, const void *facet, int centred,
                           const int32_t *subgrid_off0, int n0, const int32_t *subgrid_off1,
                           int n1, int facet_off0, int facet_off1, void *subgrids,
                           int sub_centred, void *ws, size_t ws_bytes, int32_t *d_status,
                           cg_stream_t stream);
/* Subgrid -> facet (the notebook's cell 18 in 2-D, by separability; the
 * adjoint of the above): facet [yB, yB] (+)= Fb x Fb times the sum over
 * n0 x n1 subgrids of their contributions, from the subgrids' spectra fs
 * [n0][n1][xM][xM] (the centred or raw FFT of each subgrid padded to xM),
 * subgrid offsets as above, the facet's offsets in grid pixels.  The facet
 * mask of the notebook is left to the caller.  accumulate: add into facet
 * instead of overwriting it (to split the subgrids over several calls).
 * Workspace: cg_recombine_workspace_bytes(h, n0, n1). */
int cg_recombine_subgrids_to_facet(cg_recombine *h, const void *fs, int centred,
                                   const int32_t *subgrid_off0, int n0,
                                   const int32_t *subgrid_off1, int n1,
                                   int facet_off0, int facet_off1, void *facet,
                                   int out_centred, int accumulate, void *workspace,
                                   size_t workspace_bytes, int32_t *d_status,
                                   cg_stream_t stream);
/* recombine2d_af0_af1 (recombine.c:504-544) for n subgrids: subgrids[s]
 * [xM, xM] += nmbf[s] rolled to the facet offsets (grid pixels, multiples of
 * the facet spacing).  Raw: divided by xM^2 (an unnormalised backward FFT
 * of the subgrid follows, cg_fft_raw); centred: the notebook's sum, unscaled
 * (a centred ifft follows, cg_fft). */
int cg_recombine_add_facet(const cg_recombine *h, const void *nmbf, int n,
                           int facet_off0, int facet_off1, int centred,
                           void *subgrids, cg_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* CROCODILE_GB300_H */
