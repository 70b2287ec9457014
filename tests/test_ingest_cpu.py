"""Visibility ingest on the CPU: the oracle's collect_blocks against the
reference's own (scripts/image_dataset.py:75-87 executed with arl's
Visibility, tests/golden/make_ingest.py), bit for bit; the directory
container's round trip and walk order; an h5py-like group tree."""

import os

import numpy
import pytest
from numpy.testing import assert_array_equal

from oracle import crocodile_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ig():
    return dict(numpy.load(os.path.join(HERE, "golden", "ingest_golden.npz")))


def golden_blocks(ig):
    cols = ("frequency", "time", "uvw", "antenna1", "antenna2", "vis")
    return [{c: ig["b%d_%s" % (b, c)] for c in cols} for b in range(int(ig["nblocks"]))]


def test_oracle_bit_exact(ig):
    uvw, src, vis = O.collect_blocks(golden_blocks(ig))
    assert_array_equal(uvw, ig["uvw_lambda"])
    assert_array_equal(src, ig["src"])
    assert_array_equal(vis, ig["vis"])


def test_container_round_trip(ig, tmp_path):
    from crocodile_gb300 import ingest as I
    blocks = [I.VisibilityBlock(**b) for b in golden_blocks(ig)]
    paths = I.write_blocks(str(tmp_path), blocks)
    assert all(os.path.isdir(p) for p in paths)
    back = I.read_blocks(str(tmp_path))
    # name order of the group walk: vis/<a1>/<a2>, names compared as strings
    key = sorted(range(len(blocks)), key=lambda i: (str(int(blocks[i].antenna1[0])),
                                                    str(int(blocks[i].antenna2[0]))))
    assert len(back) == len(blocks)
    for b, i in zip(back, key):
        for col in ("frequency", "time", "uvw", "antenna1", "antenna2", "vis"):
            assert_array_equal(getattr(b, col), getattr(blocks[i], col))


class FakeGroup(dict):
    """An h5py-like group: a mapping with attrs, members iterated in name order."""

    def __init__(self, attrs=None, **members):
        super().__init__(members)
        self.attrs = attrs or {}

    def __iter__(self):
        return iter(sorted(dict.keys(self)))


def test_group_walk_like_hdf5(ig):
    from crocodile_gb300 import ingest as I
    bl = golden_blocks(ig)

    def grp(b):
        return FakeGroup({"type": "Visibility"}, **b)

    tree = FakeGroup(vis=FakeGroup(**{"10": FakeGroup(**{"2": grp(bl[0])}),
                                      "2": FakeGroup(**{"3": grp(bl[1]), "11": grp(bl[2])})}),
                     other=FakeGroup({"type": "Configuration"}))
    got = I.read_blocks(tree)
    # name order: "10" < "2"; within "2": "11" < "3"
    want = [bl[0], bl[2], bl[1]]
    assert len(got) == 3
    for g, w in zip(got, want):
        assert_array_equal(g.vis, w["vis"])


def test_block_validation():
    from crocodile_gb300 import ingest as I
    with pytest.raises(ValueError):
        I.VisibilityBlock([1e8], [0.0, 1.0], numpy.zeros((2, 3)), [0, 0], [1, 1],
                          numpy.zeros((2, 2, 1)))
