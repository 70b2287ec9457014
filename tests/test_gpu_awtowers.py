"""AW-towers on the device against the reference notebook's own grid_towers
(tests/golden/make_awtowers.py) and the oracle: the grid within 1e-5 (FP32
gridding and FFTs), the notebook's image from it, a denser case with many
planes and baselines per chunk, both gridders, and argument errors."""

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


def test_notebook_golden(env):
    torch, S, O, g = env
    grid = S.aw_towers_imaging(float(g["theta"]), float(g["lam"]), g["uvw"], g["src"], g["vis"],
                               int(g["subgrid"]), int(g["margin"]), float(g["wstep"]),
                               g["aimage"])
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


@pytest.mark.parametrize("gridder", ["sparse", "tiled"])
def test_dense_vs_oracle(env, gridder):
    torch, S, O, g = env
    theta, lam, uvw, src, vis, s, aimage = dense_case()
    for margin, wstep in ((8, 25.0), (10, 60.0)):
        grid = S.aw_towers_imaging(theta, lam, uvw, src, vis, s, margin, wstep, aimage,
                                   gridder=gridder)
        ref, _ = O.aw_towers_imaging(theta, lam, uvw, src, vis, s, margin, wstep, aimage)
        assert rel(grid, ref) < 1e-5, (margin, wstep)


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
    empty = S.aw_towers_imaging(theta, lam, uvw[:0], src[:0], vis[:0], s, 8, 25.0, aimage)
    assert not numpy.any(empty)
