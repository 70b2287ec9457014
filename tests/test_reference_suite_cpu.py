"""The reference's own synthesis tests (tests/test_synthesis.py) whose functions
are host helpers of the drop-in, restated against crocodile_gb300.synthesis.
Each test cites the reference test it follows and keeps its tolerances.  No
kernel runs; the device functions' tests are in test_gpu_reference_suite.py."""

import numpy
import pytest
from numpy.testing import assert_allclose


@pytest.fixture(scope="module")
def S():
    from crocodile_gb300 import synthesis
    return synthesis


def _pattern(S, N):
    # tests/test_synthesis.py:30-31
    return S.coordinates2(N)[1] + S.coordinates2(N)[0] * 1j


def _uvw(S, N, uw=0, vw=0):
    # tests/test_synthesis.py:102-107
    u, v = S.coordinates2(N)
    u = numpy.hstack(u)
    v = numpy.hstack(v)
    return numpy.transpose([u, v, uw * u + vw * v])


def test_coordinates(S):
    # tests/test_synthesis.py:14-28
    for N in [4, 5, 6, 7, 8, 9, 1000, 1001, 1002, 1003]:
        low, high = S.coordinateBounds(N)
        c = S.coordinates(N)
        cx, cy = S.coordinates2(N)
        for arr in (c, cx, cy):
            assert numpy.min(arr) == pytest.approx(low, abs=5e-8)  # assertAlmostEqual: 7 places
            assert numpy.max(arr) == pytest.approx(high, abs=5e-8)  # assertAlmostEqual: 7 places
        assert c[N // 2] == 0
        assert (cx[:, N // 2] == 0).all()
        assert (cy[N // 2, :] == 0).all()


def test_pad_extract(S):
    # tests/test_synthesis.py:33-44
    for N, N2 in [(1, 1), (1, 2), (2, 3), (3, 4), (2, 5), (4, 6)]:
        cs = 1 + _pattern(S, N)
        cs_pad = S.pad_mid(cs, N2)
        cs2 = 1 + _pattern(S, N2) * N2 / N
        # every field of cs_pad either equals cs2 or is zero
        equal = numpy.abs(cs_pad - cs2) < 1e-15
        zero = numpy.abs(cs_pad) < 1e-15
        assert numpy.all(equal + zero)
        # extracting the middle recovers the original data
        assert_allclose(S.extract_mid(cs_pad, N), cs)


def test_anti_aliasing(S):
    # tests/test_synthesis.py:46-50
    for shape in [(4, 4), (5, 5), (4, 6), (7, 3)]:
        aaf = S.anti_aliasing_function(shape, 0, 10)
        assert aaf.shape == shape
        assert aaf[shape[0] // 2, shape[1] // 2] == pytest.approx(1, abs=5e-8)  # assertAlmostEqual: 7 places


def test_w_kernel_function(S):
    # tests/test_synthesis.py:52-58
    l, m = S.kernel_coordinates(5, 0.1)
    assert_allclose(S.w_kernel_function(l, m, 0), 1)
    assert S.w_kernel_function(l, m, 100)[2, 2] == pytest.approx(1, abs=5e-8)  # assertAlmostEqual: 7 places
    l, m = S.kernel_coordinates(10, 0.1)
    assert S.w_kernel_function(l, m, 100)[5, 5] == pytest.approx(1, abs=5e-8)  # assertAlmostEqual: 7 places
    assert S.w_kernel_function(l, m, 1000)[5, 5] == pytest.approx(1, abs=5e-8)  # assertAlmostEqual: 7 places


def test_slice_vis(S):
    # tests/test_synthesis.py:235-240
    for N in range(2, 10):
        for step in range(1, 10):
            cs = _uvw(S, N)
            slices = S.slice_vis(step, cs)
            assert_allclose(cs, numpy.vstack(slices))
