"""The tiled plans' tile numbering (crocodile_gb300/csrc/tile_order.h, plain
C++ compiled for the host): a bijection onto [0, tpl) with tile_xy as its
inverse for a range of grid shapes (tests/tile_order_check.cpp), and equal to
the Python replica the GPU plan tests use to recompute bucket keys."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def tile_block_log(ntx, nty):
    big, b = max(ntx, nty), 0
    while b < 5 and (1 << b) < big:
        b += 1
    return b


def _spread(a):
    a = a & 0xFF
    a = (a | (a << 4)) & 0x0F0F
    a = (a | (a << 2)) & 0x3333
    return (a | (a << 1)) & 0x5555


def tile_index(tx, ty, ntx, nty):
    """Blocked Morton number of tile (tx, ty) of an ntx x nty layer (numpy arrays or ints)."""
    b = tile_block_log(ntx, nty)
    nbx = (ntx + (1 << b) - 1) >> b
    m = (1 << b) - 1
    return ((((ty >> b) * nbx + (tx >> b)) << (2 * b)) |
            (_spread(tx & m) | (_spread(ty & m) << 1)))


def tiles_per_layer(ntx, nty):
    b = tile_block_log(ntx, nty)
    return (((ntx + (1 << b) - 1) >> b) * ((nty + (1 << b) - 1) >> b)) << (2 * b)


def test_tile_numbering_host(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "tile_order_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "crocodile_gb300", "csrc"),
                    os.path.join(HERE, "tile_order_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 bad of " in r.stdout
    probes = [ln.split()[1:] for ln in r.stdout.splitlines() if ln.startswith("probe")]
    assert len(probes) == 9
    for ntx, nty, tx, ty, t in (map(int, p) for p in probes):
        assert tile_index(tx, ty, ntx, nty) == t
