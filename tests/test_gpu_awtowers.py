"""AW-towers on the device against the reference notebook's own grid_towers
(tests/golden/make_awtowers.py) and the oracle: the grid within 1e-5 (FP32
gridding and FFTs), the notebook's image from it, a denser case with many
planes and baselines per chunk, both gridders and both layer methods (the
direct layer images against the gridded and transformed ones), and argument
errors."""

import os

import numpy
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import synthesis
    from oracle import crocodile_oracle
    g = dict(numpy.load(os.path.join(HERE, "golden", "awtowers_golden.npz")))
    return torch, synthesis, crocodile_oracle, g


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - b) / numpy.linalg.norm(b)


@pytest.mark.parametrize("method", ["direct", "fft"])
def test_notebook_golden(env, method):
    torch, S, O, g = env
    grid = S.aw_towers_imaging(float(g["theta"]), float(g["lam"]), g["uvw"], g["src"], g["vis"],
                               int(g["subgrid"]), int(g["margin"]), float(g["wstep"]),
                               g["aimage"], method=method)
    assert rel(grid, g["grid_sum"]) < 1e-5
    aa = O.anti_aliasing_function(grid.shape[0], 0, int(g["aa_support"]))
    image = numpy.real(O.ifft(grid)) / numpy.outer(aa, aa) / len(g["vis"])
    assert rel(image, g["image"]) < 1e-5


def dense_case(seed=4, nant=6, n=1500):
    rng = numpy.random.default_rng(seed)
    theta, lam = 0.1, 1280.0
    i1, i2 = numpy.triu_indices(nant, 1)
    b = rng.integers(0, len(i1), n)
    r = rng.uniform(0, 0.42 * lam, n)
    ph = rng.uniform(0, numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), rng.uniform(-90, 90, n)])
    src = numpy.column_stack([i1[b], i2[b]])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    s = 32
    l, m = O_coords(s, theta)
    aimage = numpy.array([(1 + 0.2 * rng.random()) * numpy.exp(
        2j * numpy.pi * (rng.normal() * l / theta + rng.normal() * m / theta) * 0.3)
        for _ in range(nant)])
    return theta, lam, uvw, src, vis, s, aimage


def O_coords(s, theta):
    c = numpy.arange(-(s // 2), -(s // 2) + s) / s
    m, l = numpy.meshgrid(c, c, indexing="ij")
    return l * theta, m * theta


@pytest.mark.parametrize("gridder,method", [("sparse", "fft"), ("tiled", "fft"),
                                            ("auto", "direct")])
def test_dense_vs_oracle(env, gridder, method):
    torch, S, O, g = env
    theta, lam, uvw, src, vis, s, aimage = dense_case()
    for margin, wstep in ((8, 25.0), (10, 60.0)):
        grid = S.aw_towers_imaging(theta, lam, uvw, src, vis, s, margin, wstep, aimage,
                                   gridder=gridder, method=method)
        ref, _ = O.aw_towers_imaging(theta, lam, uvw, src, vis, s, margin, wstep, aimage)
        assert rel(grid, ref) < 1e-5, (margin, wstep)


@pytest.mark.parametrize("s", [16, 64])
def test_direct_vs_fft_layers(env, s):
    """The direct layer images (no 2s x 2s grids, no layer FFTs) against the
    gridded and transformed layers on the same plan, at the other supported
    sub-grid sizes: FP32 sums in another order."""
    torch, S, O, g = env
    theta, lam, uvw, src, vis, _, _ = dense_case(seed=9)
    rng = numpy.random.default_rng(3)
    l, m = O_coords(s, theta)
    aimage = numpy.array([(1 + 0.2 * rng.random()) * numpy.exp(
        2j * numpy.pi * 0.3 * (rng.normal() * l / theta + rng.normal() * m / theta))
        for _ in range(6)])
    margin = 8 if s == 16 else 16
    a = S.aw_towers_imaging(theta, lam, uvw, src, vis, s, margin, 40.0, aimage, method="direct")
    b = S.aw_towers_imaging(theta, lam, uvw, src, vis, s, margin, 40.0, aimage, method="fft")
    assert rel(a, b) < 2e-6


def test_errors(env):
    torch, S, O, g = env
    theta, lam, uvw, src, vis, s, aimage = dense_case(n=50)
    with pytest.raises(ValueError):
        S.aw_towers_imaging(theta, lam, uvw, src, vis, s, 7, 25.0, aimage)  # odd margin
    with pytest.raises(ValueError):
        S.aw_towers_imaging(theta, lam, uvw, src, vis, s, 8, 25.0, aimage[:, :-1])
    bad = src.copy()
    bad[3, 1] = 99  # antenna beyond the A-images
    with pytest.raises(IndexError):
        S.aw_towers_imaging(theta, lam, uvw, bad, vis, s, 8, 25.0, aimage)
    with pytest.raises(ValueError):  # the direct form takes s of 16, 32 or 64
        S.aw_towers_imaging(0.1, 1280.0, uvw, src, vis, 24, 8, 25.0,
                            numpy.ones((6, 24, 24), complex), method="direct")
    empty = S.aw_towers_imaging(theta, lam, uvw[:0], src[:0], vis[:0], s, 8, 25.0, aimage)
    assert not numpy.any(empty)
