"""Sze-Tan optimal gridder (crocodile/antialias.py) on the CPU: the oracle's
loop-for-loop restatement pinned to vectors of the real reference
(tests/golden/make_szetan.py), and the product's host-side design functions
(the least-squares residuals, the C fit, the kernel-cache lookup and file
format) against the same vectors."""

import json
import os

import numpy
import pytest
from numpy.testing import assert_allclose, assert_array_equal

from oracle import crocodile_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def sz():
    return dict(numpy.load(os.path.join(HERE, "golden", "szetan_golden.npz")))


def cases(sz):
    for i in range(3):
        R, x0 = sz["case_%d" % i]
        yield i, int(R), float(x0), sz["h_%d" % i]


def test_oracle_gridder(sz):
    for i, R, x0, h in cases(sz):
        assert_allclose(O.sze_tan_gridder(h, x0, R, 16), sz["gridder_%d" % i], rtol=0, atol=1e-15)


def test_oracle_correction(sz):
    for i, R, x0, h in cases(sz):
        x = numpy.arange(-32, 32) / 64
        assert_allclose(O.sze_tan_grid_correction_gen(h, x0, R, x), sz["corr_%d" % i], rtol=1e-14)
        xs = numpy.linspace(0, 0.5, 37)
        assert_allclose(O.sze_gridding_correction_fine(xs, h, x0, 48, R), sz["fine_corr_%d" % i],
                        rtol=1e-14)


def test_oracle_mean_error_and_fit(sz):
    for i, R, x0, h in cases(sz):
        assert_allclose(O.sze_mean_map_error(x0, 64, 32, R, h), sz["mean_err_%d" % i], rtol=1e-12)
        assert_allclose(O.sze_func_to_min(h, x0, 32, R), sz["ftm_%d" % i], rtol=0, atol=1e-13)
        nu = (numpy.arange(32, dtype=float) + 0.5) / 64
        assert_allclose(O.sze_gridder_as_C(h, x0, nu, R), sz["gac_%d" % i], rtol=0, atol=1e-14)
    assert_allclose(O.sze_mean_map_error(0.25, 8, 8, 2, sz["fit_h"]), sz["fit_mean_err"],
                    rtol=1e-12)


def test_host_design_functions(sz):
    from crocodile_gb300 import antialias as A
    for i, R, x0, h in cases(sz):
        assert_allclose(A.func_to_min(h, x0, 32, R), sz["ftm_%d" % i], rtol=0, atol=1e-12)
        nu = (numpy.arange(32, dtype=float) + 0.5) / 64
        assert_allclose(A.calc_gridder_as_C(h, x0, nu, R), sz["gac_%d" % i], rtol=0, atol=1e-12)
        nu2, x = A.make_evaluation_grids(R, 32, 64)
        assert_allclose(A.calc_gridder(h, x0, nu2, 32, R), O.sze_gridder(h, x0, nu2, 32, R),
                        rtol=0, atol=1e-12)
        g = O.sze_gridder(h, x0, nu2, 32, R)
        assert_array_equal(A.gridder_to_C(g, R), O.sze_gridder_to_C(g, R))
        corr = O.sze_gridding_correction_fine(x, h, x0, 32, R)
        assert_allclose(A.calc_map_error(g, corr, nu2, x, R), O.sze_map_error(g, corr, nu2, x, R),
                        rtol=1e-10, atol=1e-18)


def test_host_least_squares_fit(sz):
    from crocodile_gb300 import antialias as A
    h, cov, info, mesg, ler = A.optimal_grid(2, 0.25, 8, 8)
    assert ler in (1, 2, 3, 4)
    assert_allclose(h, sz["fit_h"], rtol=1e-7)


def _write_cache(path, sz):
    entries = []
    for k in sz["cache_keys"]:
        R, x0, N, M = int(k[0]), float(k[1]), int(k[2]), int(k[3])
        entries.append([[[R, x0, N, M], []],
                        {"R": R, "x0": x0, "h": {"__ndarray__": [1.0] * N, "dtype": "float64",
                                                 "shape": [N]}}])
    with open(path, "w") as f:
        json.dump(entries, f)


def test_kernel_cache_file_and_lookup(sz, tmp_path):
    from crocodile_gb300 import antialias as A
    saved = dict(A.KERNEL_CACHE)
    try:
        A.KERNEL_CACHE.clear()
        path = str(tmp_path / "gridder.json")
        _write_cache(path, sz)
        assert A.load_kernel_cache(path) == len(sz["cache_keys"])
        k = next(iter(A.KERNEL_CACHE))
        assert A.KERNEL_CACHE[k]["h"].shape == (k[2],)
        for q, want in zip(sz["queries"], sz["query_results"]):
            q = (int(q[0]), float(q[1]), int(q[2]), int(q[3]))
            got = A.find_cached_kernel(*q)
            if numpy.isnan(want[0]):
                assert got is None
            else:
                assert got == (int(want[0]), float(want[1]), int(want[2]), int(want[3]))
        # a cached kernel good enough for the request is returned as is
        entry = A.optimal_grid_cached(3, 0.25, 64, 32)
        assert entry is A.KERNEL_CACHE[(3, 0.25, 64, 32)]
    finally:
        A.KERNEL_CACHE.clear()
        A.KERNEL_CACHE.update(saved)
