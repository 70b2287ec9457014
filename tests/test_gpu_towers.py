"""w-towers (examples/grid/grid.c:482-710): the device path against the
oracle's restatement — bit-exact chunk/plane keys and chunk-relative
coordinates, and grids within 1e-5 — for separable-free w-kernels of odd and
even support (warp and lane gridder layouts), sub-grids clipped at the grid
edge, and the single-plane case against w_cache_imaging."""

import numpy
import pytest
from numpy.testing import assert_array_equal

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import engine, synthesis
    from oracle import crocodile_oracle
    return torch, engine, synthesis, crocodile_oracle


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - numpy.asarray(b)) / numpy.linalg.norm(b)


def _case(n=30000, N=256, wmax=300.0, seed=51, rmax=0.45):
    rng = numpy.random.default_rng(seed)
    theta = 0.1
    lam = N / theta
    r = rng.uniform(0, rmax * lam, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), rng.uniform(-wmax, wmax, n)])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    return theta, lam, uvw, vis


def test_tower_keys_bitexact(env):
    torch, E, S, O = env
    theta, lam, uvw, vis = _case()
    # rows on chunk and plane boundaries
    C, winc = 48, 60.0
    edge = numpy.array([[C / theta * k, -C / theta * k, winc * (k + 0.5)] for k in range(-3, 4)])
    uvw = numpy.vstack([uvw, edge, numpy.nextafter(edge, 1e9), numpy.nextafter(edge, -1e9)])
    st = E.Status()
    key, relt, (ubmin, ubmax, vbmin, vbmax, wpmin, wpmax) = E.tower_keys(uvw, theta, C, winc, st)
    st.check()
    ub, vb, wp, xmid, ymid, rel_ref = O.tower_bins(theta, uvw, 64, 16, winc)
    assert (ubmin, ubmax, vbmin, vbmax, wpmin, wpmax) == (ub.min(), ub.max(), vb.min(), vb.max(),
                                                           wp.min(), wp.max())
    nub, nwp = ubmax - ubmin + 1, wpmax - wpmin + 1
    assert_array_equal(key.cpu().numpy(), ((vb - vbmin) * nub + (ub - ubmin)) * nwp + wp - wpmin)
    assert_array_equal(relt.cpu().numpy(), rel_ref)


@pytest.mark.parametrize("s,margin,winc,kern,tile", [(64, 16, 60.0, 7, 32), (64, 16, 40.0, 8, 32),
                                                      (96, 24, 100.0, 15, 32),
                                                      (48, 16, 25.0, 4, 32), (64, 16, 40.0, 8, 16),
                                                      (64, 16, 40.0, 8, 64), (96, 24, 60.0, 7, 64)])
def test_w_towers_imaging_matches_oracle(env, s, margin, winc, kern, tile):
    torch, E, S, O = env
    theta, lam, uvw, vis = _case()
    kw = dict(NpixFF=32, NpixKern=kern, Qpx=4)
    ref = O.w_towers_imaging(theta, lam, uvw, None, vis, s, margin, winc, 10.0, **kw)
    for gridder in ("tiled", "sparse"):
        got = S.w_towers_imaging(theta, lam, uvw, None, vis, s, margin, winc, 10.0, tile=tile,
                                 gridder=gridder, **kw)
        assert rel(got, ref) < TOL, gridder


def test_w_towers_single_plane_is_w_projection(env):
    torch, E, S, O = env
    theta, lam, uvw, vis = _case(wmax=40.0, seed=52)
    kw = dict(NpixFF=32, NpixKern=8, Qpx=4)
    got = S.w_towers_imaging(theta, lam, uvw, None, vis, 64, 16, 100.0, 10.0, **kw)
    ref = S.w_cache_imaging(theta, lam, uvw, None, vis, wstep=10.0, **kw)
    assert rel(got, ref) < TOL
    assert rel(got, O.w_cache_imaging(theta, lam, uvw, None, vis, wstep=10.0, **kw)) < TOL


def test_w_towers_errors(env):
    torch, E, S, O = env
    theta, lam, uvw, vis = _case(n=1000, seed=53)
    kw = dict(NpixFF=32, NpixKern=15, Qpx=4)
    with pytest.raises(ValueError):       # margin smaller than the kernel support
        S.w_towers_imaging(theta, lam, uvw, None, vis, 64, 8, 60.0, 10.0, **kw)
    bad = uvw.copy()
    bad[3, 0] = numpy.nan
    with pytest.raises(AssertionError):   # coordinates out of range, as the reference
        S.w_towers_imaging(theta, lam, bad, None, vis, 64, 16, 60.0, 10.0, **kw)


@pytest.mark.parametrize("s,margin,winc,kern", [(64, 16, 60.0, 7), (64, 16, 40.0, 8),
                                                 (96, 24, 100.0, 15)])
def test_w_towers_predict_matches_oracle(env, s, margin, winc, kern):
    torch, E, S, O = env
    theta, lam, uvw, vis = _case(n=20000, seed=54)
    N = int(round(theta * lam))
    rng = numpy.random.default_rng(7)
    guv = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    kw = dict(NpixFF=32, NpixKern=kern, Qpx=4)
    got = S.w_towers_predict(theta, lam, uvw, None, guv, s, margin, winc, 10.0, **kw)
    ref = O.w_towers_predict(theta, lam, uvw, None, guv, s, margin, winc, 10.0, **kw)
    assert rel(got, ref) < TOL


def test_w_towers_predict_single_plane_is_w_cache_predict(env):
    torch, E, S, O = env
    theta, lam, uvw, vis = _case(n=20000, wmax=40.0, seed=55)
    N = int(round(theta * lam))
    guv = numpy.random.default_rng(8).normal(size=(N, N)).astype(complex)
    kw = dict(NpixFF=32, NpixKern=8, Qpx=4)
    got = S.w_towers_predict(theta, lam, uvw, None, guv, 64, 16, 100.0, 10.0, **kw)
    ref = O.w_cache_predict(theta, lam, uvw, None, guv, wstep=10.0, **kw)
    assert rel(got, ref) < TOL


@pytest.mark.parametrize("kern", [7, 8])
def test_w_towers_predict_ring_degridder_matches_oracle(env, kern):
    """The layered (chunk, plane) plans of w-towers predict through the ring
    degridder (tuning dvis 3): layer offsets, sparse items, padded odd slices."""
    torch, E, S, O = env
    from crocodile_gb300 import autotune
    theta, lam, uvw, vis = _case(n=20000, seed=55)
    N = int(round(theta * lam))
    rng = numpy.random.default_rng(8)
    guv = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    kw = dict(NpixFF=32, NpixKern=kern, Qpx=4)
    autotune.set_tuning(dvis=3)
    try:
        got = S.w_towers_predict(theta, lam, uvw, None, guv, 64, 16, 60.0, 10.0, **kw)
    finally:
        autotune.set_tuning()
    ref = O.w_towers_predict(theta, lam, uvw, None, guv, 64, 16, 60.0, 10.0, **kw)
    assert rel(got, ref) < TOL
