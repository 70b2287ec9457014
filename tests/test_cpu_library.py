"""CPU-only checks: the C-ABI library loads and exports every symbol that
include/crocodile_gb300.h declares, the ctypes binding covers them, and the
host-side argument logic matches the reference's semantics.  No kernel runs."""

import ctypes
import os
import re

import numpy
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            syms |= set(re.findall(r"^\s*(?:const\s+char\s*\*|int|size_t|long\s+long)\s*\**\s*(cg_\w+)\s*\(",
                                   text, re.M))
    return syms


@pytest.fixture(scope="module")
def libpath():
    from crocodile_gb300 import build
    try:
        return build.build()
    except RuntimeError as e:  # no nvcc in this environment
        pytest.skip(str(e))


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header(libpath):
    from crocodile_gb300 import _lib
    assert set(_lib.SIGNATURES) == declared_symbols()
    L = _lib.lib()
    assert L.cg_version() >= 100


def test_workspace_queries_need_no_gpu(libpath):
    from crocodile_gb300 import _lib
    L = _lib.lib()
    kd = _lib.KernelDesc(0, 8, 15, 101)
    n = L.cg_plan_workspace_bytes(0, 2_000_000, 4096, 4096, ctypes.byref(kd))
    assert n > 2_000_000 * 40
    kd_bad = _lib.KernelDesc(0, 8, 64, 1)  # support above the supported maximum
    assert L.cg_plan_workspace_bytes(0, 10, 64, 64, ctypes.byref(kd_bad)) == 0
    assert L.cg_w_kernels_workspace_bytes(101, 64, 8) >= 101 * 512 * 512 * 16
    assert L.cg_kernel_oversample_workspace_bytes(1, 1, 1024, 8) == 8192 * 16


def test_error_mapping(libpath):
    from crocodile_gb300 import _lib
    with pytest.raises(AssertionError):
        _lib.raise_for(_lib.CG_ERR_RANGE)
    with pytest.raises(ValueError):
        _lib.raise_for(_lib.CG_ERR_BOUNDS)
    with pytest.raises(IndexError):
        _lib.raise_for(_lib.CG_ERR_INDEX)
    with pytest.raises(RuntimeError):
        _lib.raise_for(_lib.CG_ERR_CUDA)


def test_kernel_layout_and_groups():
    from crocodile_gb300 import engine as E
    # make_gcf (synthesis.py:451-461): rank minus src columns decides the layout
    k4 = numpy.zeros((3, 2, 8, 8, 7, 7), complex)
    kg = E.kernel_groups(k4.shape[:2], numpy.array([[0, 1], [2, 0], [-1, -2]]), 3)
    assert kg.tolist() == [1, 4, 4]
    with pytest.raises(IndexError):
        E.kernel_groups((3,), numpy.array([[3]]), 1)
    assert E.kernel_groups((), None, 5) is None


def test_src_columns_counted_from_the_shape():
    """The src argument's column count (the reference's src[:, i] indexing),
    from numpy, lists or tensors without a host copy; a size that is not a
    multiple of the rows is refused."""
    import torch
    from crocodile_gb300 import synthesis as S
    assert S._src_cols(None, 4) == 0
    assert S._src_cols(numpy.ndarray((4, 0)), 4) == 0
    assert S._src_cols(numpy.zeros((4, 2)), 4) == 2
    assert S._src_cols([[1, 2, 3]] * 4, 4) == 3
    assert S._src_cols(numpy.zeros(4), 4) == 1
    assert S._src_cols(torch.zeros(4, 2, dtype=torch.int32), 4) == 2
    with pytest.raises(ValueError):
        S._src_cols(numpy.zeros(7), 4)


def test_host_helpers_match_oracle():
    from crocodile_gb300 import synthesis as S
    from oracle import crocodile_oracle as O
    for N in (4, 5, 1000, 1001):
        assert numpy.array_equal(S.coordinates(N), O.coordinates(N))
        assert numpy.array_equal(S.coordinates2(N), O.coordinates2(N))
        assert S.coordinateBounds(N) == O.coordinateBounds(N)
    a = numpy.arange(36.0).reshape(6, 6) + 1j
    assert numpy.array_equal(S.pad_mid(a, 9), O.pad_mid(a, 9))
    assert numpy.array_equal(S.extract_mid(S.pad_mid(a, 9), 6), a)
    big = numpy.arange(64.0 * 64).reshape(64, 64) * (1 + 1j)
    assert numpy.array_equal(S.extract_oversampled(big, 4, 7), O.extract_oversampled(big, 4, 7))
    l, m = S.kernel_coordinates(16, 0.1, 0.01, -0.02, numpy.array([[1, .1], [.2, 1]]))
    lo, mo = O.kernel_coordinates(16, 0.1, 0.01, -0.02, numpy.array([[1, .1], [.2, 1]]))
    assert numpy.array_equal(l, lo) and numpy.array_equal(m, mo)
    assert numpy.array_equal(S.anti_aliasing_function(16, 0, 5), O.anti_aliasing_function(16, 0, 5))


def test_tuning_roundtrip_and_validation(libpath):
    from crocodile_gb300 import _lib, autotune
    try:
        autotune.set_tuning(tile=32, chunk=700, rows=3, groups=2, layout=_lib.CG_LAYOUT_OWNER,
                            dvis=4)
        assert autotune.get_tuning() == {"tile": 32, "chunk": 700, "rows": 3, "groups": 2,
                                         "layout": 2, "dvis": 4}
        for bad in ({"tile": 30}, {"tile": 68}, {"rows": 9}, {"groups": 9}, {"layout": 4},
                    {"layout": 3, "groups": 17}, {"dvis": 5}):
            with pytest.raises(ValueError):
                autotune.set_tuning(**bad)
    finally:
        autotune.set_tuning()
    assert autotune.get_tuning() == {"tile": 0, "chunk": 0, "rows": 0, "groups": 0, "layout": 0,
                                     "dvis": 0}
    cands = autotune.candidates(15)
    assert any(c["layout"] == 1 for c in cands) and any(c["layout"] == 2 for c in cands)
    assert any(c["layout"] == 3 for c in cands)
    # every lane-layout shape is tried with the tiled and the ring degridder
    lane = [c for c in cands if c["layout"] == 3]
    assert {c.get("dvis", 0) for c in lane} == {0, 3}
    assert all(c.get("dvis", 0) == 0 for c in cands if c["layout"] != 3)
    assert not any(c["layout"] == 3 for c in autotune.candidates(24))
    for c in cands:
        if c["layout"] == 2:
            gpad = (15 * ((15 + c["rows"] - 1) // c["rows"]) + 31) // 32 * 32
            assert gpad * c["groups"] <= 256
