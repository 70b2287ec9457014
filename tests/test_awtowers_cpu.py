"""AW-towers on the CPU: the oracle's restatement against the reference
notebook's own grid_towers (awtowers.ipynb, tests/golden/make_awtowers.py)."""

import os

import numpy
from numpy.testing import assert_allclose

from oracle import crocodile_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_matches_notebook():
    g = dict(numpy.load(os.path.join(HERE, "golden", "awtowers_golden.npz")))
    grid, image = O.aw_towers_imaging(float(g["theta"]), float(g["lam"]), g["uvw"], g["src"],
                                      g["vis"], int(g["subgrid"]), int(g["margin"]),
                                      float(g["wstep"]), g["aimage"], int(g["aa_support"]),
                                      int(g["aa_over"]))
    # the notebook carries a chunk's image from plane to plane by repeated
    # products with wkern; the oracle divides each plane by its own Fresnel
    # factor: equal up to rounding
    assert_allclose(grid, g["grid_sum"], rtol=0, atol=1e-10 * numpy.abs(g["grid_sum"]).max())
    # the notebook's image is also divided by sum(wt) (ones here: the count)
    assert_allclose(image / len(g["vis"]), g["image"], rtol=0,
                    atol=1e-10 * numpy.abs(g["image"]).max())
