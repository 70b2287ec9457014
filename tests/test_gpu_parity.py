"""GPU parity: the drop-in module (C ABI kernels) against the reference's golden
vectors and the CPU oracle.  Index work is bit-exact; FP32 gridding is held to
relative L2 <= 1e-5 against complex128; the FP64 plain form to 1e-12."""

import numpy
import pytest
from numpy.testing import assert_allclose, assert_array_equal

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5
FP64_TOL = 1e-12


@pytest.fixture(scope="module")
def S():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import synthesis
    synthesis.set_precision("fp32")
    return synthesis


@pytest.fixture(scope="module")
def O():
    from oracle import crocodile_oracle
    return crocodile_oracle


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - numpy.asarray(b)) / numpy.linalg.norm(b)


# ---------------------------------------------------------------- coordinates

def test_frac_coord_bitexact(S, golden):
    x, xf = S.frac_coord(4, 4, golden["fc_t05_p"])
    assert_array_equal(x, golden["fc_t05_x"])
    assert_array_equal(xf, golden["fc_t05_xf"])
    p, N, Q = golden["fc_p"], golden["fc_N"], golden["fc_Q"]
    for n_, q_ in sorted(set(zip(N.tolist(), Q.tolist()))):
        sel = (N == n_) & (Q == q_)
        x, xf = S.frac_coord(n_, q_, p[sel])
        assert_array_equal(x, golden["fc_x"][sel])
        assert_array_equal(xf, golden["fc_xf"][sel])


def test_frac_coord_property(S):
    # tests/test_synthesis.py:393-409
    for Q in range(1, 6):
        p = numpy.arange(-2 * Q, 2 * Q) / 4 / Q
        x, xf = S.frac_coord(2, Q, p)
        assert (xf >= 0).all() and (xf < Q).all()
        assert_allclose(x - xf / Q, numpy.around(numpy.arange(0, 4 * Q) / 2) / Q)


def test_frac_coords_random_large_lam(S, O):
    rng = numpy.random.default_rng(3)
    for lam in (6.0, 1e15, 163840.0):
        uvw = rng.uniform(-0.5, 0.5, (5000, 3)) * lam * 0.999
        p = uvw / lam
        for shape, Q in (((1024, 1024), 8), ((8192, 8192), 16), ((97, 64), 3)):
            got = S.frac_coords(shape, Q, p)
            exp = O.frac_coords(shape, Q, p)
            for g, e in zip(got, exp):
                assert_array_equal(g, e)


def test_frac_coord_range_error(S):
    with pytest.raises(AssertionError):
        S.frac_coord(8, 4, numpy.array([0.1, 0.5]))
    with pytest.raises(AssertionError):
        S.frac_coord(8, 4, numpy.array([numpy.nan]))


# ---------------------------------------------------------------- kernels

def test_kernel_generation(S, golden):
    assert_allclose(S.kernel_oversample(golden["aa32"], 4, 8), golden["ko_1d"], atol=1e-12)
    assert_allclose(S.kernel_oversample(golden["ko_2d_ff"], 3, 7), golden["ko_2d"], atol=1e-11)
    assert_allclose(S.kernel_oversample(golden["ko_2d_ff"], 4, 8), golden["ko_2d_even"], atol=1e-11)
    assert_allclose(S.w_kernel(0.1, 37.5, 32, 7, 4), golden["wk_inv"], atol=1e-12)
    assert_allclose(S.w_kernel(0.1, -120.0, 32, 7, 4, invert=False), golden["wk_fwd"], atol=1e-12)
    assert_allclose(S.w_kernel(0.05, 80.0, 24, 9, 2, dl=0.003, dm=-0.002, T=golden["wk_T"]),
                    golden["wk_shift"], atol=1e-12)


def test_kernel_oversampled_subgrid(S):
    # tests/test_synthesis.py:77-91
    for N in range(3, 20):
        pat = S.coordinates2(N)[1] + S.coordinates2(N)[0] * 1j
        kern = S.kernel_oversample(pat, 1, N - 2)
        kern2 = S.kernel_oversample(pat, 2, N - 2)
        assert_allclose(kern[0, 0], kern2[0, 0], atol=1e-13)
        kern4 = S.kernel_oversample(pat, 4, N - 2)
        for ux in range(2):
            for uy in range(2):
                assert_allclose(kern2[uy, ux], kern4[2 * uy, 2 * ux], atol=1e-13)


def test_aw_kernels(S, golden):
    ak = golden["aw_akerns"]
    fn = S.aw_kernel_fn(lambda theta, a: ak[a], lambda theta, w: S.w_kernel(theta, w, 16, 6, 2))
    for args, key in (((0.1, 25.0, 0, 1), "aw_k01"), ((0.1, -40.0, 1, 2), "aw_k12")):
        assert rel(fn(*args), golden[key]) < FP64_TOL  # complex128: FP64 throughout


def test_aw_kernels_headline_shape(S, O):
    """16 x 16 A kernels, w sub-kernels of support 16 at oversampling 16 (the AW
    configuration's shape): the complex128 table (FP64 throughout) and the
    complex64 table (32 x 32 FFT form) against the oracle's aw_kernel_fn."""
    from crocodile_gb300 import configs, engine as E
    rng = numpy.random.default_rng(17)
    theta = 0.05
    beams = configs.a_beams(rng, 3, 32, theta)
    A = numpy.array([O.kernel_oversample(b, 1, 16)[0, 0] for b in beams])
    ws = [37.0, -118.0]
    Wk = numpy.array([O.w_kernel(theta, w, 32, 16, 16) for w in ws])
    a1 = numpy.array([0, 1, 0], dtype=numpy.int32)
    a2 = numpy.array([1, 2, 2], dtype=numpy.int32)
    wi = numpy.array([0, 1, 1], dtype=numpy.int32)
    k64 = E.aw_kernels(A, Wk, a1, a2, wi, dtype=E.CD).cpu().numpy()
    k32 = E.aw_kernels(A, Wk, a1, a2, wi, dtype=E.CF).cpu().numpy()
    for k in range(3):
        fn = O.aw_kernel_fn(lambda t, a: A[a], lambda t, w: Wk[wi[k]])
        ref = fn(theta, 0.0, a1[k], a2[k])
        assert rel(k64[k], ref) < FP64_TOL, k
        assert rel(k32[k], ref) < 1e-6, k


# ---------------------------------------------------------------- gridding

@pytest.mark.parametrize("precision,tol", [("fp32", FP32_TOL), ("fp64", FP64_TOL)])
def test_convgrid(S, golden, precision, tol):
    uvw, vis, lam = golden["cg_uvw"], golden["cg_vis"], float(golden["cg_lam"])
    N = golden["cg_grid4"].shape[0]
    for key, k in (("cg_grid4", golden["cg_k4"]), ("cg_grid1", golden["cg_k1"])):
        a = numpy.zeros((N, N), dtype=complex)
        S.convgrid(k, a, uvw / lam, None, vis, precision=precision)
        assert rel(a, golden[key]) < tol, key
    a = numpy.zeros((N, N), dtype=complex)
    S.convgrid(golden["cg_kg"], a, uvw / lam, golden["cg_src"], vis, precision=precision)
    assert rel(a, golden["cg_gridsrc"]) < tol


@pytest.mark.parametrize("precision,tol", [("fp32", FP32_TOL), ("fp64", FP64_TOL)])
def test_convdegrid(S, golden, precision, tol):
    uvw, lam, model = golden["cg_uvw"], float(golden["cg_lam"]), golden["cg_model"]
    assert rel(S.convdegrid(golden["cg_k4"], model, uvw / lam, precision=precision),
               golden["cd_vis4"]) < tol
    assert rel(S.convdegrid(golden["cg_k1"], model, uvw / lam, precision=precision),
               golden["cd_vis1"]) < tol
    assert rel(S.convdegrid(golden["cg_kg"], model, uvw / lam, golden["cg_src"],
                            precision=precision), golden["cd_vissrc"]) < tol


@pytest.mark.parametrize("precision,tol", [("fp32", FP32_TOL), ("fp64", 1e-11)])
def test_drivers(S, golden, precision, tol):
    uvw, vis, lam = golden["cg_uvw"], golden["cg_vis"], float(golden["cg_lam"])
    theta = float(golden["di_theta"])
    d, psf, pmax = S.do_imaging(theta, lam, uvw, None, vis, S.conv_imaging, kv=golden["cg_k4"],
                                precision=precision)
    assert rel(d, golden["di_dirty"]) < tol
    assert rel(psf, golden["di_psf"]) < tol
    assert abs(pmax / golden["di_pmax"] - 1) < tol
    pv = S.do_predict(theta, lam, uvw, None, golden["dp_image"], S.conv_predict,
                      kv=golden["cg_k4"], precision=precision)
    assert rel(pv, golden["dp_vis"]) < tol


def test_weights_mirror_bitexact(S, golden):
    uvw, vis, lam = golden["cg_uvw"], golden["cg_vis"], float(golden["cg_lam"])
    theta = float(golden["di_theta"])
    assert_array_equal(S.doweight(theta, lam, uvw, numpy.ones(len(uvw))), golden["wt"])
    mu, mv = S.mirror_uvw(uvw, vis)
    assert_array_equal(mu, golden["mirror_uvw"])
    assert_array_equal(mv, golden["mirror_vis"])


def test_hermitian_fft(S, golden):
    for n in (8, 9):
        assert_array_equal(S.make_grid_hermitian(golden["herm_in_%d" % n].copy()),
                           golden["herm_out_%d" % n])
    for sfx in ("", "_odd"):
        assert_allclose(S.fft(golden["fft_in" + sfx]), golden["fft_out" + sfx], atol=1e-12)
        assert_allclose(S.ifft(golden["fft_in" + sfx]), golden["ifft_out" + sfx], atol=1e-14)


def test_boxcar(S, golden):
    uvw, vis, lam = golden["cg_uvw"], golden["cg_vis"], float(golden["cg_lam"])
    N = golden["box_grid"].shape[0]
    a = numpy.zeros((N, N), dtype=complex)
    S.grid(a, uvw / lam, vis)
    assert_allclose(a, golden["box_grid"], atol=1e-12)
    assert_array_equal(S.degrid(golden["cg_model"], uvw / lam), golden["box_degrid"])


@pytest.mark.parametrize("precision,tol", [("fp32", FP32_TOL), ("fp64", FP64_TOL)])
def test_w_cache_imaging(S, golden, precision, tol):
    uvw, vis = golden["wc_uvw"], golden["wc_vis"]
    lam, theta = float(golden["wc_lam"]), float(golden["wc_theta"])
    kw = dict(NpixFF=16, NpixKern=7, Qpx=4)
    g = S.w_cache_imaging(theta, lam, uvw, numpy.zeros((len(uvw), 0)), vis, wstep=10.0,
                          precision=precision, **kw)
    assert rel(g, golden["wc_grid"]) < tol
    # a host kernel callable takes the generic path and must agree
    g2 = S.w_cache_imaging(theta, lam, uvw, None, vis, wstep=10.0,
                           kernel_fn=lambda th, w, **k: S.w_kernel(th, w, **k),
                           precision=precision, **kw)
    assert rel(g2, golden["wc_grid"]) < tol


def test_w_cache_predict_matches_oracle(S, O, golden):
    uvw = golden["wc_uvw"]
    lam, theta = float(golden["wc_lam"]), float(golden["wc_theta"])
    kw = dict(NpixFF=16, NpixKern=7, Qpx=4)
    rng = numpy.random.default_rng(1)
    N = int(round(theta * lam))
    guv = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    ref = O.w_cache_predict(theta, lam, uvw, None, guv, wstep=10.0, **kw)
    for prec, tol in (("fp32", FP32_TOL), ("fp64", FP64_TOL)):
        got = S.w_cache_predict(theta, lam, uvw, None, guv, wstep=10.0, precision=prec, **kw)
        assert rel(got, ref) < tol


def test_w_slice_matches_oracle(S, O, golden):
    uvw, vis = golden["wc_uvw"], golden["wc_vis"]
    lam, theta = float(golden["wc_lam"]), float(golden["wc_theta"])
    kw = dict(NpixFF=16, NpixKern=7, Qpx=4)
    ref = O.w_slice_imaging(theta, lam, uvw, None, vis, wstep=37, **kw)
    got = S.w_slice_imaging(theta, lam, uvw, None, vis, wstep=37, **kw)
    assert rel(got, ref) < FP32_TOL
    rng = numpy.random.default_rng(2)
    N = int(round(theta * lam))
    guv = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    ref = O.w_slice_predict(theta, lam, uvw, None, guv, wstep=37, **kw)
    got = S.w_slice_predict(theta, lam, uvw, None, guv, wstep=37, **kw)
    assert rel(got, ref) < FP32_TOL


# ---------------------------------------------------------------- errors leave outputs untouched

def test_out_of_range_coordinates(S, golden):
    k = golden["cg_k4"]
    N = 96
    p = numpy.array([[0.1, 0.2, 0.0], [0.5, 0.0, 0.0]])
    for prec in ("fp32", "fp64"):
        a = numpy.full((N, N), 3 + 1j)
        with pytest.raises(AssertionError):
            S.convgrid(k, a, p, None, numpy.ones(2), precision=prec)
        assert (a == 3 + 1j).all()


def test_footprint_outside_grid(S, golden):
    k = golden["cg_k4"]  # support 6
    N = 96
    p = numpy.array([[0.1, 0.2, 0.0], [-0.5, 0.0, 0.0]])
    for prec in ("fp32", "fp64"):
        a = numpy.full((N, N), 2 - 1j)
        with pytest.raises(ValueError):
            S.convgrid(k, a, p, None, numpy.ones(2), precision=prec)
        assert (a == 2 - 1j).all()
        with pytest.raises(ValueError):
            S.convdegrid(k, a, p, precision=prec)


def test_empty_visibility_set(S, golden):
    a = numpy.zeros((32, 32), dtype=complex)
    S.convgrid(golden["cg_k4"], a, numpy.zeros((0, 3)), None, numpy.zeros(0, complex))
    assert (a == 0).all()
    assert S.convdegrid(golden["cg_k4"], a, numpy.zeros((0, 3))).shape == (0,)
