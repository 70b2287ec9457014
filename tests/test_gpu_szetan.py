"""Sze-Tan optimal gridder on the device: the FP64 gridding-function and
grid-correction kernels against the reference's vectors and the oracle, and
imaging with a Sze-Tan kernel table through the FP32 gridder (within 1e-5 of
the oracle).

Tolerance of the FP64 kernels: C = Kinv . rhs solves against the Gram matrix
K of h_ext^2, whose condition number grows with the support (62 at R=2, 120 at
R=4, 1.1e5 at R=5, x0=0.4375).  The device sums rhs in another order than
numpy, and a relative perturbation of K of one unit roundoff already moves C
by about cond(K) * eps (4.6e-13 at R=5), so the bound on C is
max(1e-13, cond(K) * eps) absolute.  The correction c(x) / d(x) adds the
cancellation of its two sums: kappa(x) = sum|terms| / |sum| of c plus that of
d reaches 62 at R=2, 1.4e5 at R=4 and 3.1e8 at R=5 (near |x| = 1/2, where d
sums terms of alternating sign), so each point is held to
10 eps (cond(K) + kappa(x)) relative (observed: 5e-15, 1.4e-11 and 9.4e-9
against 2.8e-13, 3.1e-10 and 6.8e-7)."""

import os

import numpy
import pytest
from numpy.testing import assert_allclose

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import antialias, synthesis
    from oracle import crocodile_oracle
    sz = dict(numpy.load(os.path.join(HERE, "golden", "szetan_golden.npz")))
    saved = dict(antialias.KERNEL_CACHE)
    for i in range(3):
        R, x0 = sz["case_%d" % i]
        antialias.KERNEL_CACHE[(int(R), float(x0), 64, 32)] = {
            "R": int(R), "x0": float(x0), "h": sz["h_%d" % i]}
    yield torch, antialias, synthesis, crocodile_oracle, sz
    antialias.KERNEL_CACHE.clear()
    antialias.KERNEL_CACHE.update(saved)


def cases(sz):
    for i in range(3):
        R, x0 = sz["case_%d" % i]
        yield i, int(R), float(x0), sz["h_%d" % i]


def c_tol(A, R, x0, h):
    x, dx, h_ext = A._h_grid(h, x0)
    return max(1e-13, numpy.linalg.cond(A._gram(h_ext, x, dx, R)) * numpy.finfo(float).eps)


def corr_tol(A, O, R, x0, h, x, M):
    """Per-point relative bound 10 eps (cond(K) + kappa(x)) of c(x) / d(x)."""
    xg, dx, h_ext = A._h_grid(h, x0)
    cond = numpy.linalg.cond(A._gram(h_ext, xg, dx, R))
    nu = (numpy.arange(M) + 0.5) / (2 * M)
    C = O.sze_gridding_fine(h, x0, nu, R)
    G = C @ C.T
    l = numpy.arange(2 * R) - R + 1
    kap = []
    for xv in numpy.atleast_1d(x):
        td = G * numpy.cos(2 * numpy.pi * (l[:, None] - l[None, :]) * xv)
        tc = C * numpy.cos(2 * numpy.pi * (l[:, None] - nu[None, :]) * xv)
        kap.append(numpy.abs(td).sum() / abs(td.sum()) + numpy.abs(tc).sum() / abs(tc.sum()))
    return 10 * numpy.finfo(float).eps * (cond + numpy.array(kap))


def assert_corr(got, want, tol):
    got, want = numpy.asarray(got), numpy.asarray(want)
    rel = numpy.abs(got - want) / numpy.abs(want)
    assert numpy.all(rel <= tol), "worst %.3g > bound %.3g at %d" % (
        rel.max(), tol[numpy.argmax(rel / tol)], numpy.argmax(rel / tol))


def test_gridder_table(env):
    torch, A, S, O, sz = env
    for i, R, x0, h in cases(sz):
        tol = c_tol(A, R, x0, h)
        assert_allclose(A.sze_tan_gridder(R, x0, 16), sz["gridder_%d" % i], rtol=0, atol=tol)
        nu = numpy.linspace(-0.7, 1.3, 203)
        assert_allclose(A.calc_gridding_fine(h, x0, nu, R), O.sze_gridding_fine(h, x0, nu, R),
                        rtol=0, atol=tol)


def test_grid_correction(env):
    torch, A, S, O, sz = env
    for i, R, x0, h in cases(sz):
        x = numpy.arange(-32, 32) / 64
        # 1 / hfine has the relative error of hfine
        assert_corr(A.sze_tan_grid_correction(R, x0, 64), sz["corr_%d" % i],
                    corr_tol(A, O, R, x0, h, x, 64))
        xs = numpy.linspace(0, 0.5, 37)
        assert_corr(A.calc_gridding_correction_fine(xs, h, x0, 48, R), sz["fine_corr_%d" % i],
                    corr_tol(A, O, R, x0, h, xs, 48))
        assert_allclose(A.sze_tan_mean_error(R, x0), sz["mean_err_%d" % i], rtol=1e-6)


def test_grid_correction_large(env):
    # an image axis of 4096 (the gridder sampled at 4096 offsets): every 97th
    # coordinate against the oracle with the same M
    torch, A, S, O, sz = env
    i, R, x0, h = list(cases(sz))[1]
    x = S.coordinates(4096)
    got = A.sze_tan_grid_correction(R, x0, 4096)
    pick = numpy.arange(0, 4096, 97)
    want = 1 / O.sze_gridding_correction_fine(x[pick], h, x0, 4096, R)
    assert_corr(got[pick], want, corr_tol(A, O, R, x0, h, x[pick], 4096))
    assert numpy.all(numpy.isfinite(got))


def test_odd_sizes_and_edges(env):
    torch, A, S, O, sz = env
    i, R, x0, h = list(cases(sz))[0]
    for n in (1, 7, 33):
        x = S.coordinates(n)
        assert_corr(A.sze_tan_grid_correction_gen(R, x0, x),
                    O.sze_tan_grid_correction_gen(h, x0, R, x), corr_tol(A, O, R, x0, h, x, n))
    assert A.calc_gridding_fine(h, x0, numpy.zeros(0), R).shape == (2 * R, 0)
    with pytest.raises(Exception):
        A.calc_gridding_fine(h, x0, numpy.zeros(3), 17)  # 2R > 32


def test_imaging_with_szetan_table(env):
    # aaf-szetan-schwab.ipynb: conv_imaging with kv = sze_tan_gridder(support//2, x0, over)
    torch, A, S, O, sz = env
    i, R, x0, h = list(cases(sz))[1]
    over = 64
    kv = A.sze_tan_gridder(R, x0, over)
    assert kv.shape == (over, 2 * R)
    rng = numpy.random.default_rng(17)
    N, n, theta = 256, 20000, 0.1
    lam = N / theta
    r = rng.uniform(0, 0.45 * lam, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), numpy.zeros(n)])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    g = S.conv_imaging(theta, lam, uvw, None, vis, kv)
    g_ref = O.conv_imaging(theta, lam, uvw, None, vis, kv)
    assert numpy.linalg.norm(g - g_ref) / numpy.linalg.norm(g_ref) < 1e-5
    v = S.conv_predict(theta, lam, uvw, None, g_ref, kv)
    v_ref = O.conv_predict(theta, lam, uvw, None, g_ref, kv)
    assert numpy.linalg.norm(v - v_ref) / numpy.linalg.norm(v_ref) < 1e-5
    # the dirty image, and the image divided by the grid correction inside
    # |x| <= x0 (the region the gridder is optimised for; beyond it the
    # correction falls towards 4e-3 and 1/corr^2 amplifies any rounding)
    d, p, pmax = S.do_imaging(theta, lam, uvw, None, vis, S.conv_imaging, kv=kv)
    d_ref, p_ref, pmax_ref = O.do_imaging(theta, lam, uvw, None, vis, O.conv_imaging, kv=kv)
    assert numpy.linalg.norm(d - d_ref) / numpy.linalg.norm(d_ref) < 1e-5
    corr = A.sze_tan_grid_correction(R, x0, N)
    inner = numpy.abs(S.coordinates(N)) <= x0
    dc = (d / numpy.outer(corr, corr))[numpy.ix_(inner, inner)]
    dc_ref = (d_ref / numpy.outer(corr, corr))[numpy.ix_(inner, inner)]
    assert numpy.linalg.norm(dc - dc_ref) / numpy.linalg.norm(dc_ref) < 1e-5
