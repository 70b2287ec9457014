"""The CPU oracle against vectors produced by the real reference (CPU only)."""

import numpy
from numpy.testing import assert_allclose, assert_array_equal

from oracle import crocodile_oracle as O


def test_frac_coord_c_table(golden):
    # examples/grid/test_recombine.c:378-412 (N=4, Q=4) as produced by the Python reference
    x, xf = O.frac_coord(4, 4, golden["fc_t05_p"])
    assert_array_equal(x, golden["fc_t05_x"])
    assert_array_equal(xf, golden["fc_t05_xf"])
    # the C test's 3/5 banker's-rounding pattern: first ten (x, xf) pairs
    assert list(zip(x[:10], xf[:10])) == [(0, 0), (0, 0), (0, 0), (1, 3), (1, 3), (1, 3),
                                          (1, 2), (1, 2), (1, 2), (1, 2)]


def test_frac_coord_sweep(golden):
    p, N, Q = golden["fc_p"], golden["fc_N"], golden["fc_Q"]
    for n_, q_ in set(zip(N.tolist(), Q.tolist())):
        sel = (N == n_) & (Q == q_)
        x, xf = O.frac_coord(n_, q_, p[sel])
        assert_array_equal(x, golden["fc_x"][sel])
        assert_array_equal(xf, golden["fc_xf"][sel])


def test_frac_coord_property():
    # tests/test_synthesis.py:393-409
    for Q in range(1, 6):
        p = numpy.arange(-2 * Q, 2 * Q) / 4 / Q
        x, xf = O.frac_coord(2, Q, p)
        assert (xf >= 0).all() and (xf < Q).all()
        assert_allclose(x - xf / Q, numpy.around(numpy.arange(0, 4 * Q) / 2) / Q)


def test_kernels(golden):
    assert_allclose(O.anti_aliasing_function(32, 0, 8), golden["aa32"], rtol=1e-15)
    assert_allclose(O.kernel_oversample(golden["aa32"], 4, 8), golden["ko_1d"], rtol=0, atol=1e-13)
    assert_allclose(O.kernel_oversample(golden["ko_2d_ff"], 3, 7), golden["ko_2d"], atol=1e-12)
    assert_allclose(O.kernel_oversample(golden["ko_2d_ff"], 4, 8), golden["ko_2d_even"], atol=1e-12)
    assert_allclose(O.w_kernel(0.1, 37.5, 32, 7, 4), golden["wk_inv"], atol=1e-13)
    assert_allclose(O.w_kernel(0.1, -120.0, 32, 7, 4, invert=False), golden["wk_fwd"], atol=1e-13)
    assert_allclose(O.w_kernel(0.05, 80.0, 24, 9, 2, dl=0.003, dm=-0.002, T=golden["wk_T"]),
                    golden["wk_shift"], atol=1e-13)


def test_convgrid_bitexact(golden):
    uvw, vis, lam = golden["cg_uvw"], golden["cg_vis"], float(golden["cg_lam"])
    N = golden["cg_grid4"].shape[0]
    for key, k in (("cg_grid4", golden["cg_k4"]), ("cg_grid1", golden["cg_k1"])):
        a = numpy.zeros((N, N), dtype=complex)
        O.convgrid(k, a, uvw / lam, None, vis)
        assert_array_equal(a, golden[key])
    a = numpy.zeros((N, N), dtype=complex)
    O.convgrid(golden["cg_kg"], a, uvw / lam, golden["cg_src"], vis)
    assert_array_equal(a, golden["cg_gridsrc"])


def test_convdegrid(golden):
    uvw, lam, model = golden["cg_uvw"], float(golden["cg_lam"]), golden["cg_model"]
    assert_allclose(O.convdegrid(golden["cg_k4"], model, uvw / lam), golden["cd_vis4"], rtol=1e-13)
    assert_allclose(O.convdegrid(golden["cg_k1"], model, uvw / lam), golden["cd_vis1"], rtol=1e-13)
    assert_allclose(O.convdegrid(golden["cg_kg"], model, uvw / lam, golden["cg_src"]),
                    golden["cd_vissrc"], rtol=1e-13)


def test_drivers(golden):
    uvw, vis, lam = golden["cg_uvw"], golden["cg_vis"], float(golden["cg_lam"])
    theta = float(golden["di_theta"])
    d, psf, pmax = O.do_imaging(theta, lam, uvw, None, vis, O.conv_imaging, kv=golden["cg_k4"])
    assert_allclose(d, golden["di_dirty"], atol=1e-13)
    assert_allclose(psf, golden["di_psf"], atol=1e-13)
    assert_allclose(pmax, golden["di_pmax"], rtol=1e-14)
    pv = O.do_predict(theta, lam, uvw, None, golden["dp_image"], O.conv_predict, kv=golden["cg_k4"])
    assert_allclose(pv, golden["dp_vis"], rtol=1e-12)
    assert_array_equal(O.doweight(theta, lam, uvw, numpy.ones(len(uvw))), golden["wt"])
    mu, mv = O.mirror_uvw(uvw, vis)
    assert_array_equal(mu, golden["mirror_uvw"])
    assert_array_equal(mv, golden["mirror_vis"])


def test_hermitian_fft(golden):
    for n in (8, 9):
        assert_array_equal(O.make_grid_hermitian(golden["herm_in_%d" % n].copy()),
                           golden["herm_out_%d" % n])
    for sfx in ("", "_odd"):
        assert_array_equal(O.fft(golden["fft_in" + sfx]), golden["fft_out" + sfx])
        assert_array_equal(O.ifft(golden["fft_in" + sfx]), golden["ifft_out" + sfx])


def test_boxcar(golden):
    uvw, vis, lam = golden["cg_uvw"], golden["cg_vis"], float(golden["cg_lam"])
    N = golden["box_grid"].shape[0]
    a = numpy.zeros((N, N), dtype=complex)
    O.grid(a, uvw / lam, vis)
    assert_array_equal(a, golden["box_grid"])
    assert_array_equal(O.degrid(golden["cg_model"], uvw / lam), golden["box_degrid"])


def test_w_cache_imaging(golden):
    uvw, vis = golden["wc_uvw"], golden["wc_vis"]
    lam, theta = float(golden["wc_lam"]), float(golden["wc_theta"])
    g = O.w_cache_imaging(theta, lam, uvw, numpy.zeros((len(uvw), 0)), vis, wstep=10.0,
                          NpixFF=16, NpixKern=7, Qpx=4)
    assert_array_equal(g, golden["wc_grid"])


def test_aw_kernel(golden):
    ak = golden["aw_akerns"]
    fn = O.aw_kernel_fn(lambda theta, a: ak[a], lambda theta, w: O.w_kernel(theta, w, 16, 6, 2))
    assert_allclose(fn(0.1, 25.0, 0, 1), golden["aw_k01"], rtol=1e-13)
    assert_allclose(fn(0.1, -40.0, 1, 2), golden["aw_k12"], rtol=1e-13)


def test_simulate_point(golden):
    assert_allclose(O.simulate_point(golden["wc_uvw"], 0.013, -0.007), golden["sp_vis"], rtol=1e-15)


def test_fixed_functions_agree_with_cache_path(golden):
    # w_slice_* and w_cache_predict are broken as shipped; their restatements must agree
    # with the working w_cache_imaging / convdegrid paths when every slice shares one w.
    uvw = golden["cg_uvw"].copy()
    vis, lam = golden["cg_vis"], float(golden["cg_lam"])
    N = golden["cg_grid4"].shape[0]
    theta = N / lam
    k = golden["cg_k4"]
    kfn = lambda th, w, **kw: k
    g1 = O.w_slice_imaging(theta, lam, uvw, None, vis, wstep=97, kernel_fn=kfn)
    assert_allclose(g1, golden["cg_grid4"], atol=1e-12)
    v1 = O.w_slice_predict(theta, lam, uvw, None, golden["cg_model"], wstep=97, kernel_fn=kfn)
    assert_allclose(v1, golden["cd_vis4"], rtol=1e-12)
    v2 = O.w_cache_predict(theta, lam, uvw, None, golden["cg_model"], wstep=1e9, kernel_fn=kfn)
    assert_allclose(v2, golden["cd_vis4"], rtol=1e-12)


def test_aw_kernel_fft_equals_aw_kernel_fn(golden):
    ak = golden["aw_akerns"]
    wk = O.w_kernel(0.1, 25.0, 16, 6, 2)
    ref = O.aw_kernel_fn(lambda th, a: ak[a], lambda th, w: wk)(0.1, 25.0, 0, 1)
    assert_allclose(O.aw_kernel_fft(ak[0], ak[1], wk), ref, rtol=1e-12, atol=1e-12)
    assert_allclose(ref, golden["aw_k01"], rtol=1e-13)


def test_w_towers_single_plane_is_the_reference_w_cache_grid(golden):
    """w-towers with one w-plane (every |w| < wincrement / 2) is w-projection itself:
    the oracle's restatement reproduces the reference's own w_cache_imaging grid
    (stored by tests/golden/make_golden.py) up to summation order, for several
    sub-grid sizes and margins."""
    uvw, vis = golden["wc_uvw"], golden["wc_vis"]
    lam, theta = float(golden["wc_lam"]), float(golden["wc_theta"])
    ref = golden["wc_grid"]
    winc = 4 * float(numpy.abs(uvw[:, 2]).max()) + 1.0
    for s, margin in ((32, 8), (48, 16), (40, 10)):
        g = O.w_towers_imaging(theta, lam, uvw, None, vis, s, margin, winc, 10.0,
                               NpixFF=16, NpixKern=7, Qpx=4)
        assert numpy.linalg.norm(g - ref) <= 1e-12 * numpy.linalg.norm(ref)


def test_w_towers_bins():
    """Chunk, plane and relative coordinates of tower_bins on hand-picked values."""
    theta, C, winc = 0.1, 48, 60.0
    uvw = numpy.array([[0.0, 0.0, 0.0], [479.9, -480.0, 29.9], [-0.001, 960.0, -30.0],
                       [4800.0, -4799.5, 90.0]])
    ub, vb, wp, xmid, ymid, rel = O.tower_bins(theta, uvw, 64, 16, winc)
    assert_array_equal(ub, [0, 0, -1, 10])
    assert_array_equal(vb, [0, -1, 2, -10])
    assert_array_equal(wp, [0, 0, -0, 2])     # around: half to even (-0.5 -> -0, 1.5 -> 2)
    assert_array_equal(xmid, [24, 24, -24, 504])
    assert_array_equal(ymid, [24, -24, 120, -456])
    assert_allclose(rel[:, 0], uvw[:, 0] - xmid / theta)
    assert_allclose(rel[:, 2], uvw[:, 2] - wp * winc)


def test_w_towers_predict_single_plane_is_the_reference_predict(golden):
    """One w-plane: the oracle's w-towers predict is w_cache_predict, which the
    reference's fixed-kernel predict pins (cd_vis4, synthesis.py:484-503)."""
    uvw, vis = golden["wc_uvw"], golden["wc_vis"]
    lam, theta = float(golden["wc_lam"]), float(golden["wc_theta"])
    N = golden["wc_grid"].shape[0]
    guv = numpy.random.default_rng(4).normal(size=(N, N)) + 0j
    winc = 4 * float(numpy.abs(uvw[:, 2]).max()) + 1.0
    ref = O.w_cache_predict(theta, lam, uvw, None, guv, wstep=10.0, NpixFF=16, NpixKern=7, Qpx=4)
    for s, margin in ((32, 8), (48, 16)):
        got = O.w_towers_predict(theta, lam, uvw, None, guv, s, margin, winc, 10.0,
                                 NpixFF=16, NpixKern=7, Qpx=4)
        assert numpy.linalg.norm(got - ref) <= 1e-12 * numpy.linalg.norm(ref)


def test_simulate_helpers_match_reference():
    """simulate_point, visibility_shift and uvw_transform against the reference's
    own outputs (tests/golden/make_simulate.py)."""
    import os
    g = numpy.load(os.path.join(os.path.dirname(__file__), "golden", "simulate_golden.npz"))
    uvw, vis = g["uvw"], g["vis"]
    assert_array_equal(O.simulate_point(uvw, 0.013, -0.021), g["point"])
    assert_array_equal(O.visibility_shift(uvw, vis, 0.01, -0.03), g["shift"])
    for T, ref in zip(g["Ts"], g["transformed"]):
        assert_array_equal(O.uvw_transform(uvw, T), ref)
