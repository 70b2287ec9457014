"""Throughput and accuracy of every benchmark configuration on the current GPU.

    python -m crocodile_gb300.bench_configs [--only plain,wproj,...,recombine,szetan]
                                            [--steps K]

For each configuration (see configs.py) it times, with CUDA events on the
current stream after warm-up, the FP32 batched form and the plain FP64 form
(or the one-plane-per-launch form for w-stacking), and reports the relative
L2 error of the FP32 result against the FP64 one.  Prints one JSON object.
"""

import argparse
import json
import statistics
import time

import numpy
import torch

from . import _lib as L
from . import autotune
from . import configs
from . import engine as E
from . import synthesis


def _time(fn, steps, warmup=2):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return statistics.median(times)


def _graph_time(fn, steps, ms_eager):
    """(median ms of the step captured once in a CUDA graph and replayed, "CUDA graph"),
    or the eager time if the capture is refused."""
    try:
        cap = E.CapturedStep(fn)
    except RuntimeError as e:
        return ms_eager, "eager (graph capture failed: %s)" % str(e).splitlines()[0][:100]
    ms = _time(cap.replay, steps)
    del cap
    return ms, "CUDA graph"


def _rel(a, b):
    a, b = a.to(torch.complex128), b.to(torch.complex128)
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def _aa_kernel(N, Q=8, S=8, c=8):
    from . import synthesis
    return synthesis.kernel_oversample(synthesis.anti_aliasing_function(N, 0, c), Q, S)


def _drivers(theta, lam, uvw, vis, imgfn, predfn, steps=3, **kw):
    """do_imaging and do_predict (synthesis.py:883-927) end to end from numpy,
    the FP32 form against the FP64 form: rel-L2 of the dirty image, the PSF
    and the predicted visibilities (of the FP64 dirty image as the model), and
    the FP32 drivers' times (host arrays in and out)."""
    from . import synthesis as S
    d, p, _ = S.do_imaging(theta, lam, uvw, None, vis, imgfn, precision="fp32", **kw)
    d64, p64, _ = S.do_imaging(theta, lam, uvw, None, vis, imgfn, precision="fp64", **kw)
    v = S.do_predict(theta, lam, uvw, None, d64, predfn, precision="fp32", **kw)
    v64 = S.do_predict(theta, lam, uvw, None, d64, predfn, precision="fp64", **kw)

    def rel(a, b):
        return float(numpy.linalg.norm(numpy.asarray(a) - b) / numpy.linalg.norm(b))

    def host_ms(fn):
        fn()
        ts = []
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(1e3 * (time.perf_counter() - t0))
        return statistics.median(ts)

    return {"rel_err_dirty_image": rel(d, d64), "rel_err_psf": rel(p, p64),
            "rel_err_predict": rel(v, v64),
            "do_imaging_ms": host_ms(lambda: S.do_imaging(theta, lam, uvw, None, vis, imgfn,
                                                          precision="fp32", **kw)),
            "do_predict_ms": host_ms(lambda: S.do_predict(theta, lam, uvw, None, d64, predfn,
                                                          precision="fp32", **kw))}


def measure_plain(steps=20):
    """conv_imaging + conv_predict, 1024^2, 200k visibilities, separable AA kernel S 8 Q 8."""
    w = configs.plain()
    n, N = len(w.uvw), w.N
    kv = _aa_kernel(N)
    kt, kt64 = E.KernelTable.from_gcf(kv, 0, E.CF), E.KernelTable.from_gcf(kv, 0, E.CD)
    uvw = E.cuda_tensor(w.uvw, torch.float64)
    vis, vis64 = E.cuda_tensor(w.vis, E.CF), E.cuda_tensor(w.vis, E.CD)
    autotune.tune(uvw, w.lam, (N, N), kt, None, vis, cands=autotune.candidates(8, quick=True),
                  use_cache=False)
    g = torch.zeros((N, N), dtype=E.CF, device="cuda")
    g64 = torch.zeros((N, N), dtype=E.CD, device="cuda")
    out = {}

    def fp32():
        plan = E.Plan(uvw, w.lam, (N, N), kt)
        g.zero_()
        plan.grid(kt, vis, g)
        out["v"] = plan.degrid(kt, g)

    def fp64():
        plan = E.Plan(uvw, w.lam, (N, N), kt64, mode=L.CG_PLAN_GROUPS)
        g64.zero_()
        plan.grid_fp64(kt64, vis64, g64)
        out["v64"] = plan.degrid_fp64(kt64, g64)

    ms_eager, ms64 = _time(fp32, steps), _time(fp64, max(3, steps // 4))
    ms, launch = _graph_time(fp32, steps, ms_eager)
    return {"workload": w.name, "n_vis": n, "ms": ms, "mvis_s": n / ms / 1e3, "launch": launch,
            "ms_eager": ms_eager,
            "plain_fp64_ms": ms64, "plain_fp64_mvis_s": n / ms64 / 1e3, "speedup": ms64 / ms,
            "rel_err_grid": _rel(g, g64), "rel_err_degrid": _rel(out["v"], out["v64"]),
            "drivers": _drivers(w.theta, w.lam, w.uvw, w.vis, synthesis.conv_imaging,
                                synthesis.conv_predict, kv=kv)}


def measure_wproj(steps=20):
    """w_cache_imaging + w_cache_predict, 4096^2, 2M visibilities, S 15 Q 8, 101 w-kernels:
    plan (fused w binning) + grid + degrid, and the plain FP64 form."""
    w = configs.wproj()
    n, N = len(w.uvw), w.N
    wstep, npff = w.params["wstep"], w.params["NpixFF"]
    uvw = E.cuda_tensor(w.uvw, torch.float64)
    vis, vis64 = E.cuda_tensor(w.vis, E.CF), E.cuda_tensor(w.vis, E.CD)
    st = E.Status()
    kidx, kmin, kmax = E.w_bins(uvw, wstep, st)
    ws_ = wstep * numpy.arange(kmin, kmax + 1).astype(float)
    kt = E.KernelTable(E.w_kernels(w.theta, ws_, npff, w.S, w.Q).reshape(-1), False, w.Q, w.S)
    kt = kt.padded_even(uvw, w.lam, (N, N))  # S 15 -> 16 with a zero row and column
    kt64 = E.KernelTable(E.w_kernels(w.theta, ws_, npff, w.S, w.Q, dtype=E.CD).reshape(-1),
                         False, w.Q, w.S)
    tuned, _ = autotune.tune(uvw, w.lam, (N, N), kt, kidx, vis,
                             cands=autotune.candidates(kt.S, quick=True), use_cache=False)
    g = torch.zeros((N, N), dtype=E.CF, device="cuda")
    g64 = torch.zeros((N, N), dtype=E.CD, device="cuda")
    out = {}

    def fp32():
        plan = E.Plan(uvw, w.lam, (N, N), kt, status=st, wbins=(wstep, kmin))
        g.zero_()
        plan.grid(kt, vis, g)
        out["v"] = plan.degrid(kt, g)

    def fp64():
        plan = E.Plan(uvw, w.lam, (N, N), kt64, kidx, mode=L.CG_PLAN_GROUPS, status=st)
        g64.zero_()
        plan.grid_fp64(kt64, vis64, g64)
        out["v64"] = plan.degrid_fp64(kt64, g64)

    ms_eager, ms64 = _time(fp32, steps), _time(fp64, 2, 1)
    ms, launch = _graph_time(fp32, steps, ms_eager)
    st.check()
    return {"workload": w.name, "n_vis": n, "ms": ms, "mvis_s": n / ms / 1e3, "tuning": tuned,
            "kernel_table": "S %d kernels run as S %d (zero first row and column)" % (w.S, kt.S)
                            if kt.S != w.S else "S %d" % w.S,
            "launch": launch, "ms_eager": ms_eager,
            "plain_fp64_ms": ms64, "plain_fp64_mvis_s": n / ms64 / 1e3, "speedup": ms64 / ms,
            "rel_err_grid": _rel(g, g64),
            "drivers": _drivers(w.theta, w.lam, w.uvw, w.vis, synthesis.w_cache_imaging,
                                synthesis.w_cache_predict, wstep=w.params["wstep"],
                                NpixFF=w.params["NpixFF"], NpixKern=w.S, Qpx=w.Q)}


def measure_diff(steps=20):
    """Predict (FFT + degrid) and its adjoint (grid + N^2 ifft) of a 2048^2 image, 1M vis."""
    from . import autograd as AG
    w = configs.diff()
    n, N = len(w.uvw), w.N
    kv = _aa_kernel(N)
    op = AG.GriddingOperator(w.uvw, w.lam, (N, N), E.KernelTable.from_gcf(kv, 0, E.CF))
    img = torch.from_numpy(w.params["image"]).cuda().requires_grad_(True)
    obs = op.predict(img).detach() * 1.01

    def step():
        loss = (torch.abs(op.predict(img) - obs) ** 2).sum()
        torch.autograd.grad(loss, img)

    ms = _time(step, steps)
    return {"workload": w.name, "n_vis": n, "ms_forward_backward": ms,
            "mvis_s": n / ms / 1e3}


def measure_wstack(steps=5):
    """All 32 w-planes in one gridding launch + one batched FFT vs one plane per launch."""
    from . import synthesis as S
    w = configs.wstack()
    n = len(w.uvw)
    kv = _aa_kernel(w.N)
    uvw = torch.from_numpy(w.uvw).cuda()
    vis = torch.from_numpy(w.vis).cuda()
    plane = w.params["plane"]
    res = {}

    def batched():
        res["a"] = S.w_stack_imaging(w.theta, w.lam, uvw, None, vis, kv, plane)

    def per_plane():
        res["b"] = S.w_stack_imaging(w.theta, w.lam, uvw, None, vis, kv, plane, per_plane=True)

    ms, ms1 = _time(batched, steps, 1), _time(per_plane, steps, 1)
    return {"workload": w.name, "n_vis": n, "planes": int(plane.max()) + 1, "ms": ms,
            "mvis_s": n / ms / 1e3, "per_plane_ms": ms1, "per_plane_mvis_s": n / ms1 / 1e3,
            "speedup": ms1 / ms, "rel_err_batched_vs_per_plane": _rel(res["a"], res["b"]),
            "note": "times include gridding, FFTs of all planes and the Fresnel combine"}


def measure_aw(steps=5, nvis=None, fp64=True):
    """AW gridding + degridding, 8192^2, 16.1M visibilities, S 16 Q 16 (nvis: only the
    first nvis visibilities, for profiling)."""
    from . import awproj
    w = configs.aw()
    if nvis:
        w = configs.wproj_subset(w, nvis)
        w.params = dict(w.params, a1=w.params["a1"][:nvis], a2=w.params["a2"][:nvis])
    n = len(w.uvw)
    t0 = time.perf_counter()
    op = awproj.AWProjection(w.theta, w.lam, w.uvw, w.params["a1"], w.params["a2"],
                             w.params["beams"], w.params["wstep"], w.params["NpixFF"], fp64=fp64)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    vis = torch.from_numpy(w.vis.astype(numpy.complex64)).cuda()
    tuned = op.tune(vis)
    vis64 = torch.from_numpy(w.vis).cuda() if fp64 else None
    N = w.N
    g = torch.zeros((N, N), dtype=E.CF, device="cuda")
    g64 = torch.zeros((N, N), dtype=E.CD, device="cuda") if fp64 else None
    out = {}

    def run32():
        g.zero_()
        op.grid(vis, g)
        out["v"] = op.degrid(g)

    def run64():
        g64.zero_()
        op.grid_fp64(vis64, g64)
        out["v64"] = op.degrid_fp64(g64)

    ms = _time(run32, steps)
    gf = torch.zeros((N, N), dtype=E.CF, device="cuda")

    def fused():
        gf.zero_()
        out["vf"] = op.degrid_grid(g, vis, gf)

    ms_fused = _time(fused, steps)
    if not fp64:
        return {"workload": w.name, "n_vis": n, "aw_kernels": op.nkernels, "ms": ms,
                "mvis_s": n / ms / 1e3, "tuning": tuned}
    ms64 = _time(run64, max(2, steps // 2), 1)
    return {"workload": w.name, "n_vis": n, "aw_kernels": op.nkernels, "tuning": tuned,
            "kernel_table_gb": op.ktab.table.numel() * 8 / 1e9, "setup_s": setup_s,
            "ms": ms, "mvis_s": n / ms / 1e3, "plain_fp64_ms": ms64,
            "plain_fp64_mvis_s": n / ms64 / 1e3, "speedup": ms64 / ms,
            "fused_ms": ms_fused, "fused_mvis_s": n / ms_fused / 1e3,
            "fused_speedup": ms64 / ms_fused,
            "plain_form": "complex128, FP64 atomics, one launch per w-plane (%d)" % op.nbins,
            "rel_err_grid": _rel(g, g64), "rel_err_degrid": _rel(out["v"], out["v64"])}


def measure_wtowers(steps=5, variants=True):
    """w-towers (examples/grid/grid.c:482-710) on the w-projection workload (4096^2,
    2M visibilities, |w| <= 500): 256^2 sub-grids with a 16-cell margin, w-planes of
    100 wavelengths, last-mile w-kernels S 8 Q 8 of the residual w (|w| <= 50), the
    sparse gridder (with variants over gridder, tile and plane width).  Timed
    end to end (binning, key compaction, plan, one gridder launch over every
    sub-grid, batched FFTs, Fresnel combine, sub-grid add), next to w-projection
    of the same visibilities with S 15 kernels over the full w range."""
    from . import synthesis
    w = configs.wproj()
    n, N = len(w.uvw), w.N
    s, margin, winc = 256, 16, 100.0
    kw = dict(NpixFF=w.params["NpixFF"], NpixKern=8, Qpx=8)
    uvw = E.cuda_tensor(w.uvw, torch.float64)
    vis = E.cuda_tensor(w.vis, E.CF)
    ms = _time(lambda: synthesis.w_towers_imaging(w.theta, w.lam, uvw, None, vis, s, margin,
                                                  winc, 10.0, tile=32, gridder="sparse", **kw),
               steps)
    grid = synthesis.w_towers_imaging(w.theta, w.lam, uvw, None, vis, s, margin, winc, 10.0,
                                      tile=32, gridder="sparse", **kw)
    ms_pred = _time(lambda: synthesis.w_towers_predict(w.theta, w.lam, uvw, None, grid, s,
                                                       margin, winc, 10.0, tile=32, **kw), steps)
    var = {}
    for gridder, tile in ((("sparse", 32), ("tiled", 32), ("tiled", 64)) if variants else ()):
        for wi in (50.0, 100.0):
            var["%s_tile%d_winc%d" % (gridder, tile, wi)] = _time(
                lambda: synthesis.w_towers_imaging(w.theta, w.lam, uvw, None, vis, s, margin,
                                                   wi, 10.0, tile=tile, gridder=gridder, **kw),
                steps)
    st = E.Status()
    key, _, b = E.tower_keys(uvw, w.theta, s - margin, winc, st)
    row, used = E.compact_keys(key, (b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1),
                               st)
    layers = int(used.shape[0])
    chunks = len(numpy.unique(used.cpu().numpy() // (b[5] - b[4] + 1)))
    kwp = dict(NpixFF=w.params["NpixFF"], NpixKern=w.S, Qpx=w.Q)
    ms_wp = _time(lambda: synthesis.w_cache_imaging(w.theta, w.lam, uvw, None, vis,
                                                    wstep=w.params["wstep"], **kwp), steps)
    ms_wpp = _time(lambda: synthesis.w_cache_predict(w.theta, w.lam, uvw, None, grid,
                                                     wstep=w.params["wstep"], **kwp), steps)
    return {"workload": "w-towers 4096^2 2M vis, 256^2 sub-grids margin 16, w-planes of 100, "
                        "S 8 Q 8 last mile, sparse gridder", "n_vis": n, "ms": ms, "mvis_s": n / ms / 1e3,
            "chunks": chunks, "layers": layers, "ms_by_gridder_tile_and_plane_width": var,
            "predict_ms": ms_pred, "predict_mvis_s": n / ms_pred / 1e3,
            "w_projection_s15_ms": ms_wp, "w_projection_s15_mvis_s": n / ms_wp / 1e3,
            "w_projection_s15_predict_ms": ms_wpp,
            "note": "ms = imaging (grid), predict_ms = predict (visibilities from the grid), "
                    "each end to end; parity with the oracle's w-towers <= 1e-5 in "
                    "tests/test_gpu_towers.py"}


# "tiny" parameter set of examples/grid/bench_recombine.c ("8k-2k-512"): image,
# subgrid spacing, yB, yN, yP, xA, xM, xMxN_yP
RECOMBINE_TINY = (8192, 128, 1280, 1536, 2048, 384, 512, 144)


def recombine_layout(image_size, subgrid_spacing, yB, xA):
    """Facet and subgrid offsets covering the image: ceil(N / yB) facets and
    ceil(N / xA) subgrids per axis, centres rounded to the allowed spacings."""
    facet_spacing = image_size // subgrid_spacing
    nf = -(-image_size // yB)
    ns = -(-image_size // xA)
    fo = [facet_spacing * int(round(j * image_size / nf / facet_spacing)) for j in range(nf)]
    so = [subgrid_spacing * int(round(i * image_size / ns / subgrid_spacing)) for i in range(ns)]
    return fo, so


def recombine_flops_bytes(rc, n0, n1):
    """FP64 FFT flops (5 n log2 n per transform) and stage bytes (each array
    written once and read once) of one facet_to_subgrids call."""
    import math
    yB, yP, xM_yP, xM_yN = rc.yB_size, rc.yP_size, rc.xM_yP_size, rc.xM_yN_size
    ffts = [(yP, yB), (xM_yP, n1 * yB), (yP, n1 * xM_yN), (xM_yP, n0 * n1 * xM_yN)]
    flops = sum(5 * n * math.log2(n) * b for n, b in ffts)
    elems = yB * yB + 3 * yB * yP + 3 * n1 * yB * xM_yP + 3 * n1 * xM_yN * yP \
        + 3 * n0 * n1 * xM_yN * xM_yP + n0 * n1 * xM_yN ** 2
    return flops, elems * 16


def measure_recombine(steps=3, nfacets=None):
    """Facet -> subgrid recombination of a whole image, the "tiny" (8k-2k-512)
    set of examples/grid/bench_recombine.c: 8192^2 image as 7 x 7 facets of
    1280^2, 22 x 22 subgrids of 384^2 (xM 512), complex128 throughout.  A step
    is every facet's contributions to every subgrid, their sum, and the
    subgrids' inverse FFTs."""
    from .recombine import Recombine
    N, sp, yB, yN, yP, xA, xM, xMxN = RECOMBINE_TINY
    rc = Recombine(N, sp, yB, yN, yP, xA, xM, xMxN)
    fo, so = recombine_layout(N, sp, yB, xA)
    nf = len(fo) if nfacets is None else nfacets
    g = torch.Generator(device="cuda").manual_seed(11)
    facets = torch.randn((nf, len(fo), yB, yB), dtype=E.CD, device="cuda", generator=g)
    o = E.cuda_tensor(numpy.asarray(so), torch.int32)
    ns = len(so)
    approx = torch.zeros((ns, ns, xM, xM), dtype=E.CD, device="cuda")

    def per_facet(j0, j1):
        rc.facet_add(approx, facets[j0, j1], o, o, fo[j0], fo[j1], check=False)

    def step():
        approx.zero_()
        rc.status.reset()
        for j0 in range(nf):
            for j1 in range(len(fo)):
                per_facet(j0, j1)
        rc.finish_subgrids(approx, crop=False)

    ms = _time(step, steps, warmup=1)
    rc.status.check()
    ms_facet = _time(lambda: per_facet(0, 0), max(steps, 5))
    flops, nbytes = recombine_flops_bytes(rc, ns, ns)
    nfac = nf * len(fo)
    # the other direction: every facet from the 484 subgrids (their spectra
    # once, then one subgrids_to_facet call per facet)
    step()
    del facets
    fo_rows = fo[:nf]
    ms_split = _time(lambda: rc.split(approx, so, so, fo_rows, fo), steps, warmup=1)
    fs = rc.subgrid_spectra(approx)
    fout = torch.empty((yB, yB), dtype=E.CD, device="cuda")
    ms_split_facet = _time(lambda: rc.subgrids_to_facet(fs, o, o, fo[0], fo[0], out=fout,
                                                        check=False), max(steps, 5))
    rc.status.check()
    return {"workload": "facet->subgrid recombination, bench_recombine.c 'tiny' (8k-2k-512): "
                        "8192^2 image, %d x %d facets of %d^2, %d x %d subgrids (xA %d, xM %d), "
                        "complex128" % (nf, len(fo), yB, ns, ns, xA, xM),
            "facets": nfac, "subgrids": ns * ns, "ms": ms,
            "contributions_per_s": nfac * ns * ns / (ms * 1e-3),
            "ms_per_facet": ms_facet,
            "fft_gflop_per_facet": flops / 1e9, "fp64_fft_tflop_s": flops / (ms_facet * 1e-3) / 1e12,
            "stage_gb_per_facet": nbytes / 1e9,
            "stage_gb_s": nbytes / (ms_facet * 1e-3) / 1e9,
            "subgrids_to_facets_ms": ms_split, "subgrids_to_facet_ms_per_facet": ms_split_facet,
            "note": "ms: facets -> subgrids (per facet, cg_recombine_facet_add: 4 "
                    "row-transform launches with the prepare, window, crop and sum-into-the-"
                    "subgrids steps in their loads and stores, 1 transpose kernel; "
                    "stage arrays and FFTs in "
                    "double-float arithmetic on the FP32 units, complex128 in and out; then "
                    "the subgrid sums' 512^2 inverse FFTs, double-float too); "
                    "fp64_fft_tflop_s counts 5 n log2 n per transform; "
                    "subgrids_to_facets_ms: the other direction for the "
                    "whole image (the subgrids' spectra, then every facet); parity with the "
                    "reference notebook in tests/test_gpu_recombine.py"}


RECOMBINE_SMALL = (16384, 32, 5120, 5632, 8192, 416, 512, 280)


def measure_recombine_small(steps=3):
    """One facet of bench_recombine.c's "small" set (16k-8k-512: 16384^2 image,
    4 x 4 facets of 5120^2, 40 x 40 subgrids of xM 512) summed into all 1600
    subgrids (cg_recombine_facet_add): yP 8192 runs the double-float stage
    kernels with the four-step rows, against complex128 with FP64 cuFFT."""
    from .recombine import Recombine
    N, sp, yB, yN, yP, xA, xM, xMxN = RECOMBINE_SMALL
    fo, so = recombine_layout(N, sp, yB, xA)
    g = torch.Generator(device="cuda").manual_seed(13)
    facet = torch.randn((yB, yB), dtype=E.CD, device="cuda", generator=g)
    o = E.cuda_tensor(numpy.asarray(so), torch.int32)
    ns = len(so)
    approx = torch.zeros((ns, ns, xM, xM), dtype=E.CD, device="cuda")
    out = {}
    for mode in ("auto", "fp64"):
        rc = Recombine(N, sp, yB, yN, yP, xA, xM, xMxN, fft=mode)
        rc.status.reset()
        out[mode] = _time(lambda: rc.facet_add(approx, facet, o, o, fo[0], fo[0], check=False),
                          steps, warmup=1)
        rc.status.check()
        del rc
        torch.cuda.empty_cache()
    nf = len(fo) ** 2
    return {"workload": "facet->subgrid recombination, bench_recombine.c 'small' (16k-8k-512): "
                        "16384^2 image, %d facets of %d^2, %d x %d subgrids (xA %d, xM %d), "
                        "complex128" % (nf, yB, ns, ns, xA, xM),
            "facets": nf, "subgrids": ns * ns, "ms_per_facet": out["auto"],
            "ms_per_facet_fp64_cufft": out["fp64"], "speedup": out["fp64"] / out["auto"],
            "note": "one facet's contributions summed into every subgrid; yP 8192: "
                    "double-float stage arrays and four-step double-float rows (auto) "
                    "against complex128 stage arrays and FP64 cuFFT; parity of the two in "
                    "tests/test_gpu_dfft.py"}


def measure_szetan(steps=5):
    """Sze-Tan gridder evaluation (crocodile/antialias.py): the grid correction
    of an 8192-pixel axis (the gridder sampled at 8192 offsets, as
    sze_tan_grid_correction does) and a kernel table oversampled 16384 times,
    for R = 3 with h fitted here at N = 16, M = 16 points (host least squares)."""
    from . import antialias as A
    t0 = time.perf_counter()
    h = A.optimal_grid(3, 0.3, 16, 16)[0]
    fit_s = time.perf_counter() - t0
    x = (numpy.arange(8192) - 4096) / 8192
    ms_corr = _time(lambda: A.calc_gridding_correction_fine(x, h, 0.3, 8192, 3), steps)
    nu = numpy.arange(16384) / 16384
    ms_table = _time(lambda: A.calc_gridding_fine(h, 0.3, nu, 3), steps)
    return {"workload": "Sze-Tan R 3 x0 0.3: grid correction of 8192 pixels (M 8192), "
                        "gridder table at 16384 offsets", "ms_correction": ms_corr,
            "ms_table": ms_table, "host_fit_s": fit_s, "h": [float(v) for v in h],
            "note": "host round trip included (numpy in and out); FP64"}


def awtowers_workload(nant=16, ntime=125, nchan=16, s=64, seed=8):
    """AW-towers input of the AW workload's kind: Earth-rotation tracks of 16
    antennas (120 baselines x 125 hour angles x 16 channels, 240,000
    visibilities) on the 8192^2 grid, 64^2 sub-grids, per-antenna A-images
    (smooth random phase screens)."""
    w = configs.aw(nant=nant, ntime=ntime, nchan=nchan)
    rng = numpy.random.default_rng(seed)
    c = (numpy.arange(s) - s // 2) / s
    m, l = numpy.meshgrid(c, c, indexing="ij")
    aimage = numpy.array([(1 + 0.1 * rng.random()) * numpy.exp(
        2j * numpy.pi * 0.2 * (rng.normal() * l + rng.normal() * m + rng.normal() * l * m))
        for _ in range(nant)])
    src = numpy.column_stack([w.params["a1"], w.params["a2"]])
    return w, src, aimage


def measure_awtowers(steps=3):
    """AW-towers imaging (awtowers.ipynb cells 17-22) of awtowers_workload(): 64^2
    sub-grids with a 16-cell margin, w-planes of the workload's w step, the
    anti-aliasing kernel (support 6, oversampled 4096 times) on 128^2 layer
    grids.  Timed end to end (binning, key compaction, plan, one gridder
    launch over every (chunk, plane, baseline) layer, batched FFTs, combine
    with the antenna ratios and Fresnel factors, sub-grid add)."""
    w, src_h, aimage_h = awtowers_workload()
    n = len(w.uvw)
    uvw = E.cuda_tensor(w.uvw, torch.float64)
    vis = E.cuda_tensor(w.vis, E.CF)
    src = E.cuda_tensor(src_h, torch.int32)
    aimage = E.cuda_tensor(aimage_h, E.CF)
    s, margin, wstep = 64, 16, w.params["wstep"]
    run = lambda: synthesis.aw_towers_imaging(w.theta, w.lam, uvw, src, vis, s, margin, wstep,
                                              aimage)
    ms = _time(run, steps, warmup=1)
    st = E.Status()
    key, _, b = E.awtower_keys(uvw, w.theta, s - margin, wstep, src[:, 0], src[:, 1],
                               len(aimage), st)
    nk = (b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1) * len(aimage) ** 2
    _, used = E.compact_keys(key, nk, st)
    return {"workload": "AW-towers, %d visibilities (16 antennas, 125 hour angles x 16 "
                        "channels), 8192^2, 64^2 sub-grids margin 16, w step %.0f" % (n, wstep),
            "n_vis": n, "ms": ms, "mvis_s": n / ms / 1e3, "layers": int(used.shape[0]),
            "note": "end to end from device-resident uvw, vis, antenna pairs and A-images; "
                    "parity with the reference notebook and the oracle in "
                    "tests/test_gpu_awtowers.py"}


def ingest_blocks(seed=5, nant=64, ntime=125, nchan=64, npol=1):
    """Synthetic per-baseline blocks of the AW workload's shape: 2016 baselines
    x 125 times x 64 channels (16,128,000 visibilities), uvw in metres."""
    from .ingest import VisibilityBlock
    rng = numpy.random.default_rng(seed)
    freq = 1.0e8 * (1 + 0.3 * numpy.arange(nchan) / max(nchan - 1, 1))
    time = 58000.0 + numpy.arange(ntime) / 1440.0
    blocks = []
    for a1 in range(nant):
        for a2 in range(a1 + 1, nant):
            uvw = rng.normal(0, 1500.0, (ntime, 3))
            vis = (rng.standard_normal((ntime, nchan, npol), dtype=numpy.float32) + 1j *
                   rng.standard_normal((ntime, nchan, npol), dtype=numpy.float32))
            blocks.append(VisibilityBlock(freq, time, uvw, numpy.full(ntime, a1),
                                          numpy.full(ntime, a2), vis.astype(numpy.complex128)))
    return blocks


def measure_ingest(steps=3, blocks=None):
    """Visibility ingest of the AW workload's shape (2016 baseline blocks, 125
    times, 64 channels, 1 polarisation; 16.1M visibilities, 258 MB of
    complex128 vis): host blocks -> device uvw (wavelengths), complex64 vis
    and int32 antennas, through the pinned double buffer (host packing, copy
    and conversion overlapped), and the conversion kernel alone on resident
    inputs."""
    from .ingest import Ingest
    blocks = blocks or ingest_blocks()
    n = sum(b.nrow * b.nchan for b in blocks)
    ing = Ingest()
    for _ in range(2):
        ing.run(blocks, dtype=E.CF, want_src=False, want_antennas=True)
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        ing.run(blocks, dtype=E.CF, want_src=False, want_antennas=True)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    s_e2e = statistics.median(ts)
    # the kernel alone: one chunk holding everything, inputs already on the device
    big = Ingest(chunk_bytes=1 << 40)
    big.run(blocks, dtype=E.CF, want_src=False, want_antennas=True)
    out = {"uvw": torch.empty((n, 3), dtype=torch.float64, device="cuda"),
           "vis": torch.empty(n, dtype=E.CF, device="cuda"),
           "a1": torch.empty(n, dtype=torch.int32, device="cuda"),
           "a2": torch.empty(n, dtype=torch.int32, device="cuda")}
    rows, nfreq, nvis, off, pos = big._layout(blocks)
    d = big._dev[0].data_ptr()
    import ctypes
    cp = ctypes.c_void_p

    def kernel():
        L.call("cg_ingest_blocks", cp(d + off["blocks"]), len(blocks), cp(d + off["uvw"]),
               cp(d + off["time"]), cp(d + off["a1"]), cp(d + off["a2"]), cp(d + off["freq"]),
               cp(d + off["vis"]), 0, E._p(out["uvw"]), None, E._p(out["a1"]), E._p(out["a2"]),
               E._p(out["vis"]), 1, E._p(big.status.t), E.stream())

    ms_k = _time(kernel, max(steps, 5))
    big.status.check()
    nbytes = nvis * 16 + rows * 32 + n * (24 + 8 + 8)
    return {"workload": "ingest of 2016 baseline blocks x 125 times x 64 channels x 1 "
                        "polarisation (16,128,000 visibilities)", "n_vis": n,
            "e2e_ms": s_e2e * 1e3, "e2e_mvis_s": n / s_e2e / 1e6,
            "kernel_ms": ms_k, "kernel_mvis_s": n / ms_k / 1e3,
            "kernel_gb_s": nbytes / (ms_k * 1e-3) / 1e9,
            "note": "e2e: host blocks (numpy) to device arrays, host packing into pinned "
                    "buffers included; kernel: uvw metres -> wavelengths (bit-exact), vis "
                    "complex128 -> complex64, antennas, inputs resident"}


def measure_fft(steps=10):
    """The hand-written FP32 FFTs of the imaging path against cuFFT (torch.fft) on the
    same complex64 planes: the centred inverse transform (ifft of synthesis.py,
    checkerboard and 1/N^2 folded into the first and last passes), the unshifted unscaled
    inverse (cuFFT's own operation, out of place), and the dirty image of a grid
    (hermitian + transform + real part + maximum)."""
    out = {}
    for N in (1024, 2048, 4096, 8192):
        rng = numpy.random.default_rng(N)
        g = torch.from_numpy((rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N)))
                             .astype(numpy.complex64)).cuda()
        t = g.clone()
        y = torch.empty_like(g)
        ms_c = _time(lambda: E.fft_(t, True), steps)
        ms_r = _time(lambda: E.fft_raw(t, True), steps)
        ms_cu = _time(lambda: torch.fft.ifft2(t, norm="forward", out=y), steps)
        rows = t.view(N, 1, N)  # the row pass alone: N rows of N
        ms_rows = _time(lambda: E.fft_raw(rows, True), steps)

        def image():
            t.copy_(g)
            E.image_from_grid(t, want_max=True)

        ms_img = _time(image, steps) - _time(lambda: t.copy_(g), steps)
        nbytes = N * N * 8
        passes = 2 if N <= 1024 else 3
        out["%d" % N] = {"centred_ifft_ms": ms_c, "raw_ifft_ms": ms_r, "row_pass_ms": ms_rows,
                         "cufft_ifft2_ms": ms_cu,
                         "raw_vs_cufft": ms_cu / ms_r, "dirty_image_ms": ms_img,
                         "passes": passes,
                         "gb_s": 2 * passes * nbytes / (ms_r * 1e-3) / 1e9}
        del g, t, y
        torch.cuda.empty_cache()
    # a stack of small planes, the w-towers shape (2371 sub-grids of 256^2)
    st = torch.zeros((2371, 256, 256), dtype=E.CF, device="cuda")
    ys = torch.empty_like(st)
    out["256x2371"] = {"raw_ifft_ms": _time(lambda: E.fft_raw(st, True), steps),
                       "cufft_ifft2_ms": _time(lambda: torch.fft.ifft2(st, norm="forward", out=ys),
                                               steps)}
    del st, ys
    torch.cuda.empty_cache()
    out["note"] = ("complex64 N^2 planes; ours: the row pass, then columns in place as tiles "
                   "of adjacent columns up to 1024, or as two four-step passes from 2048 (the "
                   "first into a scratch stack, the second back), register-blocked radix-16 "
                   "Stockham stages; cuFFT: torch.fft.ifft2 out of place, no normalisation; "
                   "gb_s counts one read and one write of the plane per pass")
    return out


MEASURES = {"plain": measure_plain, "wproj": measure_wproj, "diff": measure_diff,
            "wstack": measure_wstack, "aw": measure_aw, "wtowers": measure_wtowers,
            "recombine": measure_recombine, "recombine_small": measure_recombine_small,
            "szetan": measure_szetan, "ingest": measure_ingest,
            "awtowers": measure_awtowers, "fft": measure_fft}


def run(only=None, steps=None):
    res = {}
    for name, fn in MEASURES.items():
        if only and name not in only:
            continue
        autotune.set_tuning()
        res[name] = fn() if steps is None else fn(steps)
        torch.cuda.empty_cache()
    autotune.set_tuning()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="")
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--no-variants", action="store_true",
                    help="w-towers only: time the measured shape alone (profiling runs)")
    ap.add_argument("--aw-nvis", type=int, default=0,
                    help="AW only: the first N visibilities, FP32 only (profiling runs)")
    ap.add_argument("--recombine-facets", type=int, default=0,
                    help="recombination only: the first N rows of facets (profiling runs)")
    a = ap.parse_args()
    if a.recombine_facets:
        print(json.dumps(measure_recombine(a.steps or 2, nfacets=a.recombine_facets)))
        return
    if a.no_variants:
        print(json.dumps(measure_wtowers(a.steps or 5, variants=False)))
        return
    if a.aw_nvis:
        print(json.dumps(measure_aw(a.steps or 2, nvis=a.aw_nvis, fp64=False)))
        return
    print(json.dumps(run([s for s in a.only.split(",") if s] or None, a.steps)))


if __name__ == "__main__":
    main()
