"""Distinct-key compaction (cg_compact_keys, the bitmap form) against
numpy.unique: row ranks and ascending distinct keys for dense and very
sparse key spaces, key spaces that are not a multiple of 32, the first and
last key, all-equal keys, no keys, and out-of-range keys counted as index
errors."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import engine
    return torch, engine


def check(E, keys, nkeys):
    st = E.Status()
    row, used = E.compact_keys(numpy.asarray(keys, numpy.int32), nkeys, st)
    st.check()
    want_used, want_row = numpy.unique(keys, return_inverse=True)
    numpy.testing.assert_array_equal(used.cpu().numpy(), want_used)
    numpy.testing.assert_array_equal(row.cpu().numpy(), want_row)


@pytest.mark.parametrize("nkeys,n", [(1, 5), (31, 100), (33, 1000), (4096, 50000),
                                     (300_000_001, 240_000), (1000, 1)])
def test_matches_unique(env, nkeys, n):
    torch, E = env
    rng = numpy.random.default_rng(nkeys % 1000 + n)
    keys = rng.integers(0, nkeys, n).astype(numpy.int32)
    keys[0] = 0
    keys[-1] = nkeys - 1
    check(E, keys, nkeys)


def test_all_equal_and_empty(env):
    torch, E = env
    check(E, numpy.full(777, 64, numpy.int32), 65)
    st = E.Status()
    row, used = E.compact_keys(numpy.zeros(0, numpy.int32), 100, st)
    st.check()
    assert row.numel() == 0 and used.numel() == 0


def test_out_of_range_counted(env):
    torch, E = env
    st = E.Status()
    E.compact_keys(numpy.array([0, 5, 10, -1], numpy.int32), 10, st)
    with pytest.raises(IndexError):
        st.check()
