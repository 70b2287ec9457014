"""AW-projection at scale (8192^2, theta 0.05, 64 antennas, 16.1M visibilities,
AW kernels S 16 / Q 16): the device AW path against the oracle's w-cache loop
with aw_kernel_fn on all visibilities of 16 baselines, and at full size the
FP32 tiled form (complex64 kernels) against the plain FP64 form (complex128
kernels generated in FP64 throughout, one launch per w-plane), so that the
full-size error includes kernel generation."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def aw_workload():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import configs
    return configs.aw()


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - numpy.asarray(b)) / numpy.linalg.norm(b)


def test_aw_subset_matches_oracle(aw_workload):
    import torch
    from crocodile_gb300 import awproj
    from oracle import crocodile_oracle as O
    w = aw_workload
    a1, a2 = w.params["a1"], w.params["a2"]
    # all visibilities of 16 baselines (about 128k), short and long ones
    pairs = [(0, 1), (3, 17), (10, 40), (25, 63), (5, 6), (31, 32), (2, 50), (7, 44),
             (12, 13), (15, 60), (20, 21), (33, 48), (38, 39), (45, 58), (50, 51), (61, 62)]
    sel = numpy.zeros(len(a1), bool)
    for p, q in pairs:
        sel |= (a1 == p) & (a2 == q)
    uvw, vis = w.uvw[sel], w.vis[sel]
    src = numpy.column_stack([a1[sel], a2[sel]])
    beams, wstep, npff = w.params["beams"], w.params["wstep"], w.params["NpixFF"]

    op = awproj.AWProjection(w.theta, w.lam, uvw, a1[sel], a2[sel], beams, wstep, npff)
    g = op.grid(vis)
    v = op.degrid(g)
    g_host = g.cpu().numpy().astype(complex)

    akern = lambda theta, a: O.kernel_oversample(beams[a], 1, 16)[0, 0]
    wkern = lambda theta, ww: O.w_kernel(theta, ww, npff, 16, 16)
    memo = {}
    gen = O.aw_kernel_fn(akern, wkern)

    def fn(theta, ww, p, q):  # the reference's kernel cache: one generation per key
        key = (theta, float(ww), int(p), int(q))
        if key not in memo:
            memo[key] = gen(theta, ww, p, q)
        return memo[key]

    assert len(uvw) == 16 * 125 * 64
    ref = O.w_cache_imaging(w.theta, w.lam, uvw, src, vis, wstep=wstep, kernel_cache=fn)
    assert rel(g_host, ref) < 1e-5
    vref = O.w_cache_predict(w.theta, w.lam, uvw, src, ref, wstep=wstep, kernel_cache=fn)
    assert rel(v.cpu().numpy(), vref) < 1e-5
    from crocodile_gb300 import autotune
    autotune.set_tuning(dvis=3)  # the ring degridder
    try:
        vr = op.degrid(g)
    finally:
        autotune.set_tuning()
    assert rel(vr.cpu().numpy(), vref) < 1e-5


def test_aw_full_size_fp32_vs_fp64(aw_workload):
    import torch
    from crocodile_gb300 import awproj
    w = aw_workload
    assert len(w.uvw) == 16_128_000
    op = awproj.AWProjection(w.theta, w.lam, w.uvw, w.params["a1"], w.params["a2"],
                             w.params["beams"], w.params["wstep"], w.params["NpixFF"], fp64=True)
    vis = torch.from_numpy(w.vis).cuda()
    g32 = op.grid(vis)
    g64 = op.grid_fp64(vis)
    err = float(torch.linalg.vector_norm(g32.to(torch.complex128) - g64) /
                torch.linalg.vector_norm(g64))
    assert err < 1e-5, err
    v32 = op.degrid(g64.to(torch.complex64))
    v64 = op.degrid_fp64(g64)
    err = float(torch.linalg.vector_norm(v32.to(torch.complex128) - v64) /
                torch.linalg.vector_norm(v64))
    assert err < 1e-5, err
    # the ring degridder (dvis 3, the autotuner's pick for this workload)
    from crocodile_gb300 import autotune
    autotune.set_tuning(dvis=3)
    try:
        vr = op.degrid(g64.to(torch.complex64))
    finally:
        autotune.set_tuning()
    err = float(torch.linalg.vector_norm(vr.to(torch.complex128) - v64) /
                torch.linalg.vector_norm(v64))
    assert err < 1e-5, err
    # the fused pass (each AW slice read once) gives both results at once
    gf = torch.zeros_like(g32)
    vf = op.degrid_grid(g64.to(torch.complex64), vis, gf)
    err = float(torch.linalg.vector_norm(gf.to(torch.complex128) - g64) /
                torch.linalg.vector_norm(g64))
    assert err < 1e-5, err
    err = float(torch.linalg.vector_norm(vf.to(torch.complex128) - v64) /
                torch.linalg.vector_norm(v64))
    assert err < 1e-5, err
    op.status.check()


def _aw_reference_case(w, pairs):
    from oracle import crocodile_oracle as O
    a1, a2 = w.params["a1"], w.params["a2"]
    sel = numpy.zeros(len(a1), bool)
    for p, q in pairs:
        sel |= (a1 == p) & (a2 == q)
    beams, wstep, npff = w.params["beams"], w.params["wstep"], w.params["NpixFF"]
    akern = {}

    def a_fn(theta, a):  # host A kernels, as the reference reads them from its file
        if a not in akern:
            akern[a] = O.kernel_oversample(beams[a], 1, 16)[0, 0]
        return akern[a]

    memo = {}
    gen = O.aw_kernel_fn(a_fn, lambda theta, ww: O.w_kernel(theta, ww, npff, 16, 16))

    def oracle_fn(theta, ww, p, q):
        key = (theta, float(ww), int(p), int(q))
        if key not in memo:
            memo[key] = gen(theta, ww, p, q)
        return memo[key]

    src = numpy.column_stack([a1[sel], a2[sel]])
    return w.uvw[sel], w.vis[sel], src, wstep, npff, a_fn, oracle_fn


def test_reference_api_aw_matches_oracle(aw_workload):
    """The reference's own AW call (scripts/image_dataset.py:162-187):
    w_cache_imaging / w_cache_predict / do_imaging with src = [a1, a2] and
    kernel_cache = aw_kernel_fn(a_kernel_fn, w_kernel_fn).  The drop-in keys the
    visibilities on the device (cg_row_keys + cg_compact_keys) and generates every
    key's AW kernel in one batched pass; a plain callable as kernel_cache is called
    once per distinct device key.  Both against the oracle's complex128 loop."""
    from crocodile_gb300 import synthesis as S
    from oracle import crocodile_oracle as O
    w = aw_workload
    uvw, vis, src, wstep, npff, a_fn, oracle_fn = _aw_reference_case(
        w, [(0, 1), (3, 17), (10, 40), (25, 63)])
    fn = S.aw_kernel_fn(a_fn, lambda theta, ww: S.w_kernel(theta, ww, npff, 16, 16))
    ref = O.w_cache_imaging(w.theta, w.lam, uvw, src, vis, wstep=wstep, kernel_cache=oracle_fn)
    got = S.w_cache_imaging(w.theta, w.lam, uvw, src, vis, wstep=wstep, kernel_cache=fn)
    assert rel(got, ref) < 1e-5
    assert len(fn._tables) == 1  # one batched table, cached on the callable
    got2 = S.w_cache_imaging(w.theta, w.lam, uvw, src, vis, wstep=wstep, kernel_cache=oracle_fn)
    assert rel(got2, ref) < 1e-5  # generic callable, device-keyed
    vref = O.w_cache_predict(w.theta, w.lam, uvw, src, ref, wstep=wstep, kernel_cache=oracle_fn)
    vgot = S.w_cache_predict(w.theta, w.lam, uvw, src, ref, wstep=wstep, kernel_cache=fn)
    assert rel(vgot, vref) < 1e-5
    assert len(fn._tables) == 1  # predict reused the cached table
    d, p, pm = S.do_imaging(w.theta, w.lam, uvw, src, vis, S.w_cache_imaging, wstep=wstep,
                            kernel_cache=fn)
    dr, pr, pmr = O.do_imaging(w.theta, w.lam, uvw, src, vis, O.w_cache_imaging, wstep=wstep,
                               kernel_cache=oracle_fn)
    assert rel(d, dr) < 1e-5 and rel(p, pr) < 1e-5 and abs(pm / pmr - 1) < 1e-5
