"""GPU checks of the kernels' internal choices: the filtered-exact coordinate
path at rounding boundaries, every gridder launch shape, and the fused w-bin
plan, each against the CPU oracle."""

import ctypes

import numpy
import pytest
from numpy.testing import assert_array_equal

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import autotune, engine, synthesis
    from oracle import crocodile_oracle
    yield torch, engine, synthesis, autotune, crocodile_oracle
    autotune.set_tuning()


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - numpy.asarray(b)) / numpy.linalg.norm(b)


def test_frac_coord_at_rounding_boundaries(env):
    """Coordinates whose scaled value (-(N//2 + p*N))*Q lies exactly on, or one ulp
    around, a half-integer: the fast estimate must defer to the exact sequence."""
    torch, E, S, A, O = env
    for N, Q, lam in ((1024, 8, 12800.0), (4096, 8, 40960.0), (8192, 16, 163840.0),
                      (97, 3, 1212.5), (5, 4, 6.0)):
        k = numpy.arange(-N * Q // 2, N * Q // 2, max(1, N * Q // 4096))
        p = (k + 0.5) / (N * Q)          # exact half-steps of the oversampled grid
        p = numpy.concatenate([p, numpy.nextafter(p, 1), numpy.nextafter(p, -1), k / (N * Q)])
        p = p[(p >= -0.5) & (p < 0.5)]
        q = numpy.random.default_rng(N).permutation(p)
        pq = numpy.column_stack([p, q, numpy.zeros_like(p)])
        got = S.frac_coords((N, N), Q, pq)
        exp = O.frac_coords((N, N), Q, pq)
        for g, e in zip(got, exp):
            assert_array_equal(g, e)
        # and through lam (device division) in the plan path, for the rows whose
        # u / lam and v / lam stay inside [-0.5, 0.5)
        uvw = pq * lam
        inside = ((uvw[:, :2] / lam >= -0.5) & (uvw[:, :2] / lam < 0.5)).all(axis=1)
        uvw = uvw[inside]
        st = E.Status()
        got = E.frac_coords(uvw, lam, (N, N), Q, st)
        st.check()
        exp = O.frac_coords((N, N), Q, uvw / lam)
        for g, e in zip(got, exp):
            assert_array_equal(g.cpu().numpy(), e)


def test_w_bins_at_rounding_boundaries(env):
    torch, E, S, A, O = env
    wstep = 10.0
    w = numpy.concatenate([(numpy.arange(-60, 60) + 0.5) * wstep,
                           numpy.nextafter((numpy.arange(-60, 60) + 0.5) * wstep, 1e9),
                           numpy.random.default_rng(1).uniform(-600, 600, 1000)])
    uvw = numpy.column_stack([numpy.zeros_like(w), numpy.zeros_like(w), w])
    st = E.Status()
    kidx, kmin, kmax = E.w_bins(uvw, wstep, st)
    st.check()
    k = numpy.round(w / wstep).astype(int)
    assert (kmin, kmax) == (k.min(), k.max())
    assert_array_equal(kidx.cpu().numpy(), k - k.min())


def _wproj_case(O, n=20000, N=256, seed=5):
    rng = numpy.random.default_rng(seed)
    theta = 0.1
    lam = N / theta
    r = rng.uniform(0, 0.45 * lam, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), rng.uniform(-200, 200, n)])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    return theta, lam, uvw, vis


@pytest.mark.parametrize("cfg", [
    {"layout": 1, "groups": 8, "tile": 32},
    {"layout": 1, "groups": 4, "tile": 16, "chunk": 64},
    {"layout": 2, "rows": 1, "groups": 1, "tile": 48},
    {"layout": 2, "rows": 3, "groups": 2, "tile": 32},
    {"layout": 2, "rows": 4, "groups": 4, "tile": 24, "chunk": 100},
    {"layout": 2, "rows": 5, "groups": 1, "tile": 64},
    {"layout": 2, "rows": 8, "groups": 1, "tile": 32},
    {"layout": 3, "tile": 32},
    {"layout": 3, "groups": 3, "tile": 16, "chunk": 40},
    {"layout": 3, "groups": 16, "tile": 24},
    {"layout": 3, "rows": 2, "tile": 16},            # two bulk-copy stages per warp
    {"layout": 3, "rows": 3, "groups": 14, "tile": 16, "chunk": 64},
    {"layout": 3, "tile": 16, "dvis": 4},            # degridder: four visibilities a warp
    {"layout": 3, "tile": 16, "dvis": 1},            # degridder: the lane kernel's traversal
    {"layout": 3, "tile": 16, "dvis": 3},            # degridder: window + slice rings
    {"layout": 3, "tile": 16, "rows": 2, "chunk": 40, "dvis": 3},
    {"layout": 1, "tile": 32, "chunk": 100, "dvis": 3},  # warp layout, odd S: tiled
    {"layout": 1, "groups": 8, "tile": 32, "chunk": 100, "dvis": 4},
])
def test_gridder_shapes_match_oracle(env, cfg):
    torch, E, S, A, O = env
    theta, lam, uvw, vis = _wproj_case(O)
    kw = dict(NpixFF=32, NpixKern=15, Qpx=4)
    ref = O.w_cache_imaging(theta, lam, uvw, None, vis, wstep=20.0, **kw)
    vref = O.w_cache_predict(theta, lam, uvw, None, ref, wstep=20.0, **kw)
    A.set_tuning(**cfg)
    try:
        got = S.w_cache_imaging(theta, lam, uvw, None, vis, wstep=20.0, **kw)
        vgot = S.w_cache_predict(theta, lam, uvw, None, ref, wstep=20.0, **kw)
    finally:
        A.set_tuning()
    assert rel(got, ref) < FP32_TOL
    assert rel(vgot, vref) < FP32_TOL


@pytest.mark.parametrize("layout", [1, 2, 3])
def test_odd_support_unpadded_and_padded(env, layout):
    """An S 15 table straight through a plan (lane layout: slices padded to a
    16-byte multiple) and its zero-padded S 16 form (padded_even, which the FP32
    drivers use), each against the oracle; a footprint reaching the grid edge
    keeps the table as it is."""
    torch, E, S, A, O = env
    theta, lam, uvw, vis = _wproj_case(O, n=8000)
    N = int(round(theta * lam))
    kw = dict(NpixFF=32, NpixKern=15, Qpx=4)
    ref = O.w_cache_imaging(theta, lam, uvw, None, vis, wstep=20.0, **kw)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    st = E.Status()
    kidx, kmin, kmax = E.w_bins(uvw_t, 20.0, st)
    ws_ = 20.0 * numpy.arange(kmin, kmax + 1).astype(float)
    kt = E.KernelTable(E.w_kernels(theta, ws_, 32, 15, 4).reshape(-1), False, 4, 15)
    kt16 = kt.padded_even(uvw_t, lam, (N, N))
    assert kt16.S == 16 and kt16 is not kt
    v = E.cuda_tensor(vis, E.CF)
    A.set_tuning(layout=layout)
    try:
        for table in (kt, kt16):
            g = torch.zeros((N, N), dtype=E.CF, device="cuda")
            plan = E.Plan(uvw_t, lam, (N, N), table, kidx, status=st)
            plan.grid(table, v, g)
            plan.check()
            assert rel(g.cpu().numpy(), ref) < FP32_TOL, (layout, table.S)
    finally:
        A.set_tuning()
    edge = uvw_t.clone()
    edge[0, 0] = -0.5 * lam * (1 - 8.0 / N)  # footprint starts 4 cells from the edge
    assert kt.padded_even(edge, lam, (N, N)) is kt


@pytest.mark.parametrize("S_,sep", [(8, True), (8, False), (7, False), (16, False), (16, True),
                                    (3, False), (12, False)])
def test_supports_and_separable(env, S_, sep):
    torch, E, S, A, O = env
    rng = numpy.random.default_rng(S_)
    N, n, theta, Q = 128, 5000, 0.1, 4
    lam = N / theta
    uvw = numpy.column_stack([rng.uniform(-0.4, 0.4, (n, 2)) * lam, numpy.zeros(n)])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    aa = O.anti_aliasing_function(N, 0, 6)
    kv = O.kernel_oversample(aa, Q, S_) if sep else \
        O.kernel_oversample(numpy.outer(aa, aa), Q, S_)
    for layout in (1, 2, 3):
        A.set_tuning(layout=layout)
        try:
            g = S.conv_imaging(theta, lam, uvw, None, vis, kv)
            v = S.conv_predict(theta, lam, uvw, None, g, kv)
        finally:
            A.set_tuning()
        assert rel(g, O.conv_imaging(theta, lam, uvw, None, vis, kv)) < FP32_TOL
        assert rel(v, O.conv_predict(theta, lam, uvw, None, g, kv)) < FP32_TOL


def test_fused_wbin_plan(env):
    torch, E, S, A, O = env
    theta, lam, uvw, vis = _wproj_case(O, n=30000, N=512, seed=9)
    kw = dict(NpixFF=32, NpixKern=9, Qpx=4)
    N = int(round(theta * lam))
    ref = O.w_cache_imaging(theta, lam, uvw, None, vis, wstep=15.0, **kw)
    st = E.Status()
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    kidx, kmin, kmax = E.w_bins(uvw_t, 15.0, st)
    table = E.w_kernels(theta, 15.0 * numpy.arange(kmin, kmax + 1).astype(float), 32, 9, 4)
    kt = E.KernelTable(table.reshape(-1), False, 4, 9)
    plan = E.Plan(uvw_t, lam, (N, N), kt, status=st, wbins=(15.0, kmin))
    g = torch.zeros((N, N), dtype=E.CF, device="cuda")
    plan.grid(kt, E.cuda_tensor(vis, E.CF), g)
    plan.check()
    assert rel(g.cpu().numpy(), ref) < FP32_TOL
    # a table that misses bins is an index error and leaves the grid untouched
    st2 = E.Status()
    small = E.KernelTable(table[1:].reshape(-1), False, 4, 9)
    plan = E.Plan(uvw_t, lam, (N, N), small, status=st2, wbins=(15.0, kmin + 1))
    g2 = torch.zeros((N, N), dtype=E.CF, device="cuda")
    plan.grid(small, E.cuda_tensor(vis, E.CF), g2)
    with pytest.raises(IndexError):
        plan.check()
    assert float(g2.abs().sum()) == 0.0


@pytest.mark.parametrize("sep,S_,layout,rows", [(False, 7, 1, 0), (True, 7, 1, 0),
                                                (False, 7, 3, 0), (True, 7, 3, 0),
                                                (False, 8, 3, 0), (False, 16, 3, 0),
                                                (False, 16, 3, 2)])
def test_fused_degrid_grid_matches_separate(env, sep, S_, layout, rows):
    torch, E, S, A, O = env
    theta, lam, uvw, vis = _wproj_case(O, n=30000, N=256, seed=13)
    N = int(round(theta * lam))
    aa = O.anti_aliasing_function(N, 0, 7)
    kv = O.kernel_oversample(aa, 4, S_) if sep else \
        O.kernel_oversample(numpy.outer(aa, aa), 4, S_)
    kt = E.KernelTable.from_gcf(kv, 0, E.CF)
    A.set_tuning(layout=layout, rows=rows)
    try:
        _fused_checks(torch, E, kt, uvw, lam, N, vis)
    finally:
        A.set_tuning()


def _fused_checks(torch, E, kt, uvw, lam, N, vis):
    plan = E.Plan(uvw, lam, (N, N), kt)
    rng = numpy.random.default_rng(3)
    model = E.cuda_tensor(rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N)), E.CF)
    v_in = E.cuda_tensor(vis, E.CF)
    ref_v = plan.degrid(kt, model)
    ref_g = plan.grid(kt, v_in, torch.zeros((N, N), dtype=E.CF, device="cuda"))
    g = torch.zeros((N, N), dtype=E.CF, device="cuda")
    v = plan.degrid_grid(kt, model, v_in, g)
    plan.check()
    r = lambda a, b: float(torch.linalg.vector_norm((a - b).to(torch.complex128)) /
                           torch.linalg.vector_norm(b.to(torch.complex128)))
    assert r(v, ref_v) < 1e-6 and r(g, ref_g) < 1e-6
    # residual mode: grid(vis - degrid(model))
    ref_res = plan.grid(kt, v_in - ref_v, torch.zeros((N, N), dtype=E.CF, device="cuda"))
    g2 = torch.zeros((N, N), dtype=E.CF, device="cuda")
    plan.degrid_grid(kt, model, v_in, g2, residual=True)
    assert r(g2, ref_res) < 1e-5


@pytest.mark.parametrize("S_", [8, 15, 16])
def test_lane_layout_weighted_modes(env, S_):
    """Weighted gridding (vis * weight) and the weights-only PSF pass in the lane
    layout against the warp layout on the same plan."""
    torch, E, S, A, O = env
    theta, lam, uvw, vis = _wproj_case(O, n=20000, N=256, seed=21)
    N = int(round(theta * lam))
    aa = O.anti_aliasing_function(N, 0, 7)
    kt = E.KernelTable.from_gcf(O.kernel_oversample(numpy.outer(aa, aa), 4, S_), 0, E.CF)
    plan = E.Plan(uvw, lam, (N, N), kt)
    v = E.cuda_tensor(vis, E.CF)
    wt = torch.rand(len(vis), device="cuda", dtype=torch.float32) + 0.5
    out = {}
    for layout in (1, 3):
        A.set_tuning(layout=layout)
        try:
            g1 = plan.grid_weighted(kt, v, wt, torch.zeros((N, N), dtype=E.CF, device="cuda"))
            g2 = plan.grid_weighted(kt, None, wt, torch.zeros((N, N), dtype=E.CF, device="cuda"))
        finally:
            A.set_tuning()
        out[layout] = (g1, g2)
    plan.check()
    for a, b in zip(out[3], out[1]):
        err = float(torch.linalg.vector_norm((a - b).to(torch.complex128)) /
                    torch.linalg.vector_norm(b.to(torch.complex128)))
        assert err < 1e-6, err


@pytest.mark.parametrize("S_,sep", [(7, True), (8, False), (15, False), (16, False)])
def test_sparse_gridder_matches_oracle(env, S_, sep):
    """cg_grid_sparse (per-tap atomics, no windows) grids the same sums as convgrid."""
    torch, E, S, A, O = env
    theta, lam, uvw, vis = _wproj_case(O, n=20000, N=256, seed=61)
    N = int(round(theta * lam))
    aa = O.anti_aliasing_function(N, 0, 7)
    kv = O.kernel_oversample(aa, 4, S_) if sep else O.kernel_oversample(numpy.outer(aa, aa), 4, S_)
    kt = E.KernelTable.from_gcf(kv, 0, E.CF)
    plan = E.Plan(uvw, lam, (N, N), kt)
    g = plan.grid_sparse(kt, E.cuda_tensor(vis, E.CF), torch.zeros((N, N), dtype=E.CF,
                                                                    device="cuda"))
    plan.check()
    assert rel(g.cpu().numpy(), O.conv_imaging(theta, lam, uvw, None, vis, kv)) < FP32_TOL
