"""Facet <-> subgrid recombination on the CPU: the oracle's restatement
against vectors of the reference notebook (facet-subgrid-impl.ipynb, run by
tests/golden/make_recombine.py), and the C prototype's raw-layout primitives
(examples/grid/recombine.c) against the notebook's centred forms."""

import os

import numpy
import pytest
from numpy.testing import assert_allclose

from oracle import crocodile_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def rg():
    return dict(numpy.load(os.path.join(HERE, "golden", "recombine_golden.npz")))


def config(rg):
    return O.RecombineConfig(int(rg["N"]), int(rg["yB_size"]), int(rg["yN_size"]),
                             int(rg["yP_size"]), int(rg["xA_size"]), int(rg["xM_size"]),
                             int(rg["xMxN_yP_size"]), rg["pswf"])


def test_windows(rg):
    cfg = config(rg)
    assert (cfg.xM_yP, cfg.xM_yN) == (int(rg["xM_yP_size"]), int(rg["xM_yN_size"]))
    assert_allclose(cfg.Fb, rg["Fb"], rtol=1e-15)
    assert_allclose(cfg.Fn, rg["Fn"], rtol=1e-15)
    assert_allclose(cfg.m0, rg["facet_m0_trunc"], rtol=0, atol=1e-16)


def test_facet_to_subgrid_1d(rg):
    cfg = config(rg)
    for i, so in enumerate(rg["subgrid_off"]):
        approx = numpy.zeros(cfg.xM, dtype=complex)
        for j, fo in enumerate(rg["facet_off"]):
            r = O.rc_facet_to_subgrid_1d(cfg, rg["facet"][j], int(so))
            assert_allclose(r, rg["RNjMiBjFj"][i, j], rtol=0, atol=1e-12)
            approx += numpy.roll(O.pad_mid(r, cfg.xM), int(fo) * cfg.xM // cfg.N)
        sub = rg["subgrid_A"][i] * O.extract_mid(O.ifft(approx), cfg.xA)
        assert_allclose(sub, rg["approx_subgrid_1d"][i], rtol=0, atol=1e-14)


def test_subgrid_to_facet_1d(rg):
    cfg = config(rg)
    fn = numpy.array([O.rc_split_subgrid(cfg, rg["subgrid"][i], rg["facet_off"])
                      for i in range(len(rg["subgrid_off"]))])
    assert_allclose(fn, rg["FNjSi"], rtol=0, atol=1e-12)
    for j in range(len(rg["facet_off"])):
        acc = sum(O.rc_subgrid_to_facet_axis(cfg, fn[i, j], int(so), 0)
                  for i, so in enumerate(rg["subgrid_off"]))
        assert_allclose(acc * cfg.Fb * rg["facet_B"][j], rg["approx_facet_1d"][j], rtol=0,
                        atol=1e-12)


def test_facet_to_subgrids_2d(rg):
    cfg = config(rg)
    offs = rg["subgrid_off"]
    for f, facet in enumerate(rg["facet2"]):
        out = O.rc_facet_to_subgrids(cfg, facet, offs, offs)
        for s, (i0, i1) in enumerate(rg["subgrid2_idx"]):
            assert_allclose(out[i0, i1], rg["nmbf2"][f, s], rtol=0, atol=1e-11)


def test_subgrid_to_facet_2d_separable(rg):
    # the 2-D composition on an outer-product subgrid is the outer product of
    # the 1-D reference results
    cfg = config(rg)
    a, b = rg["subgrid"][1], rg["subgrid"][2]
    fo = rg["facet_off"]
    so = rg["subgrid_off"]
    fn2 = O.rc_split_subgrid(cfg, numpy.outer(a, b), [(fo[3], fo[1])])[0]
    got = O.rc_subgrids_to_facet(cfg, fn2[None, None], [so[1]], [so[2]])
    fa = O.rc_subgrid_to_facet_axis(cfg, O.rc_split_subgrid(cfg, a, [fo[3]])[0], int(so[1]), 0)
    fb = O.rc_subgrid_to_facet_axis(cfg, O.rc_split_subgrid(cfg, b, [fo[1]])[0], int(so[2]), 0)
    assert_allclose(got, numpy.outer(fa, fb), rtol=0, atol=1e-12)


def test_raw_primitives_match_centred(rg):
    cfg = config(rg)
    sh = numpy.fft.ifftshift
    pswf_raw = sh(cfg.pswf)
    Fb = O.rc_generate_Fb(cfg.yB, pswf_raw)
    Fn = O.rc_generate_Fn(cfg.yN, cfg.xM_yN, pswf_raw)
    m = O.rc_generate_m(cfg.N, cfg.yP, cfg.yN, cfg.xM, cfg.xMxN_yP, pswf_raw)
    assert_allclose(Fb, sh(cfg.Fb), rtol=1e-15)
    assert_allclose(Fn, sh(cfg.Fn), rtol=1e-15)
    assert_allclose(m, sh(cfg.m0), rtol=0, atol=1e-15)
    facet = rg["facet"][2]
    bf = O.rc_prepare_facet_raw(cfg.yB, cfg.yP, Fb, sh(facet))
    want = sh(O.rc_prepare_facet(cfg, facet, 0))
    assert_allclose(bf, want, rtol=0, atol=1e-14 * numpy.abs(want).max())
    approx = numpy.zeros(cfg.xM, dtype=complex)
    for so in rg["subgrid_off"]:
        nm = O.rc_extract_subgrid_raw(cfg.yP, cfg.xM_yP, cfg.xMxN_yP, cfg.xM_yN,
                                      int(so) * cfg.yP // cfg.N, m, Fn, bf)
        want = O.rc_extract_subgrid(cfg, O.rc_prepare_facet(cfg, facet, 0), int(so), 0)
        # windowed sums of xMxN_yP inputs up to max|bf| (5e5 here) that cancel
        # to outputs near 800: rounding scales with the inputs
        assert_allclose(nm, sh(want), rtol=0, atol=1e-15 * cfg.xMxN_yP * numpy.abs(bf).max())
    nm = O.rc_extract_subgrid_raw(cfg.yP, cfg.xM_yP, cfg.xMxN_yP, cfg.xM_yN, 0, m, Fn, bf)
    fo = int(rg["facet_off"][3])
    O.rc_add_facet_raw(cfg.xM, cfg.xM_yN, fo * cfg.xM // cfg.N, nm, approx)
    want = numpy.roll(O.pad_mid(numpy.fft.fftshift(nm), cfg.xM), fo * cfg.xM // cfg.N) / cfg.xM
    assert_allclose(approx, sh(want), rtol=0, atol=1e-15 * numpy.abs(want).max())


def test_recombination_accuracy_2d(rg):
    # the notebook's own accuracy figure (cell 30) from the oracle on the
    # notebook's test image regenerated with its seed
    cfg = config(rg)
    N = cfg.N
    numpy.random.seed(0)
    numpy.random.rand(N)  # the 1-D test grid of cell 12
    G2 = numpy.exp(2j * numpy.pi * numpy.random.rand(N, N)) * numpy.random.rand(N, N) / 2
    FG2 = O.fft(G2)
    sa = rg["subgrid_A"]
    fb = rg["facet_B"]
    so, fo = rg["subgrid_off"], rg["facet_off"]
    facets = {}
    for j0 in range(len(fo)):
        for j1 in range(len(fo)):
            f = O.extract_mid(numpy.roll(FG2, (-fo[j0], -fo[j1]), (0, 1)), cfg.yB)
            facets[j0, j1] = f * numpy.outer(fb[j0], fb[j1])
    assert_allclose(facets[2, 1], rg["facet2"][1], rtol=0, atol=1e-12)
    nm = {j: O.rc_facet_to_subgrids(cfg, f, so, so) for j, f in facets.items()}
    err = 0
    for i0 in range(len(so)):
        for i1 in range(len(so)):
            approx = numpy.zeros((cfg.xM, cfg.xM), dtype=complex)
            for (j0, j1), n in nm.items():
                O.rc_add_facet(cfg, approx, n[i0, i1], fo[j0], fo[j1])
            sub = O.rc_finish_subgrid(cfg, approx) * numpy.outer(sa[i0], sa[i1])
            ref = O.extract_mid(numpy.roll(G2, (-so[i0], -so[i1]), (0, 1)), cfg.xA)
            ref = ref * numpy.outer(sa[i0], sa[i1])
            err += numpy.abs(sub - ref) ** 2 / len(so) ** 2
    assert_allclose(numpy.sqrt(numpy.mean(err)), rg["rmse2"], rtol=1e-6)
