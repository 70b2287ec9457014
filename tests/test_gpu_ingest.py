"""Visibility ingest on the device: bit-exact against the reference's own
collect_blocks (tests/golden/make_ingest.py) and the oracle, for one and many
chunks through the pinned double buffer, complex64 and complex128 output,
another polarisation, errors, and the ingested arrays gridded by
conv_imaging against the oracle."""

import os

import numpy
import pytest
from numpy.testing import assert_array_equal

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import ingest, synthesis, engine
    from oracle import crocodile_oracle
    ig = dict(numpy.load(os.path.join(HERE, "golden", "ingest_golden.npz")))
    return torch, ingest, synthesis, engine, crocodile_oracle, ig


def golden_blocks(I, ig):
    cols = ("frequency", "time", "uvw", "antenna1", "antenna2", "vis")
    return [I.VisibilityBlock(**{c: ig["b%d_%s" % (b, c)] for c in cols})
            for b in range(int(ig["nblocks"]))]


def random_blocks(I, seed, nb=40, npol=2):
    rng = numpy.random.default_rng(seed)
    out = []
    for b in range(nb):
        nrow, nchan = int(rng.integers(0, 40)), int(rng.integers(1, 9))
        out.append(I.VisibilityBlock(
            1.4e8 + 1e5 * numpy.arange(nchan) + rng.random(), 58000 + rng.random(nrow),
            rng.normal(0, 2000.0, (nrow, 3)), numpy.full(nrow, b % 7),
            numpy.full(nrow, 7 + b % 5),
            rng.normal(size=(nrow, nchan, npol)) + 1j * rng.normal(size=(nrow, nchan, npol))))
    return out


def test_golden_bit_exact(env):
    torch, I, S, E, O, ig = env
    r = I.Ingest().run(golden_blocks(I, ig))
    assert_array_equal(r["uvw"].cpu().numpy(), ig["uvw_lambda"])
    assert_array_equal(r["src"].cpu().numpy(), ig["src"])
    assert_array_equal(r["vis"].cpu().numpy(), ig["vis"])
    r32 = I.Ingest().run(golden_blocks(I, ig), dtype=E.CF, want_src=False, want_antennas=True)
    assert_array_equal(r32["vis"].cpu().numpy(), ig["vis"].astype(numpy.complex64))
    assert_array_equal(r32["a1"].cpu().numpy(), ig["src"][:, 0].astype(numpy.int32))
    assert_array_equal(r32["a2"].cpu().numpy(), ig["src"][:, 1].astype(numpy.int32))
    assert "src" not in r32


def test_chunks_and_polarisation(env):
    torch, I, S, E, O, ig = env
    blocks = random_blocks(I, 3)
    uvw, src, vis = O.collect_blocks(blocks, pol=1)
    one = I.Ingest(chunk_bytes=1 << 30).run(blocks, pol=1)
    many = I.Ingest(chunk_bytes=4096).run(blocks, pol=1)  # one or two blocks per chunk
    for r in (one, many):
        assert_array_equal(r["uvw"].cpu().numpy(), uvw)
        assert_array_equal(r["src"].cpu().numpy(), src)
        assert_array_equal(r["vis"].cpu().numpy(), vis)
    # the same Ingest reused (buffers kept) gives the same result
    ing = I.Ingest(chunk_bytes=8192)
    for _ in range(2):
        assert_array_equal(ing.run(blocks, pol=1)["vis"].cpu().numpy(), vis)


def test_errors_and_empty(env):
    torch, I, S, E, O, ig = env
    blocks = random_blocks(I, 4, nb=3, npol=1)
    with pytest.raises(IndexError):
        I.Ingest().run(blocks, pol=1)
    r = I.Ingest().run([])
    assert r["uvw"].shape == (0, 3)


def test_ingest_then_grid(env):
    # the path of scripts/image_dataset.py: blocks -> collect -> conv_imaging
    torch, I, S, E, O, ig = env
    rng = numpy.random.default_rng(8)
    N, theta = 256, 0.1
    lam = N / theta
    blocks = []
    for b in range(30):
        nrow, nchan = 20, 4
        freq = 1.0e8 * (1 + 0.05 * numpy.arange(nchan))
        # metres such that |uv| stays within 0.4 lam at the top channel
        r = rng.uniform(0, 0.4 * lam * I.C_LIGHT / freq[-1], nrow)
        ph = rng.uniform(0, 2 * numpy.pi, nrow)
        uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), numpy.zeros(nrow)])
        vis = rng.normal(size=(nrow, nchan, 1)) + 1j * rng.normal(size=(nrow, nchan, 1))
        blocks.append(I.VisibilityBlock(freq, 58000 + rng.random(nrow), uvw, numpy.zeros(nrow),
                                        numpy.ones(nrow), vis))
    d = I.Ingest().run(blocks, dtype=E.CF)
    kv = O.kernel_oversample(numpy.outer(O.anti_aliasing_function(N, 0, 7),
                                         O.anti_aliasing_function(N, 0, 7)), 8, 8)
    g = S.conv_imaging(theta, lam, d["uvw"], None, d["vis"], kv)
    g = g.cpu().numpy() if isinstance(g, torch.Tensor) else g
    uvw, src, vis = O.collect_blocks(blocks)
    g_ref = O.conv_imaging(theta, lam, uvw, None, vis, kv)
    assert numpy.linalg.norm(g - g_ref) / numpy.linalg.norm(g_ref) < 1e-5
