"""Facet -> subgrid recombination on the device against the oracle and the
reference notebook's vectors, the C prototype's raw layout through the C
ABI, the whole transform's accuracy on the notebook's test image, and
degridding from recombined subgrids (notebook cells 32-44).

Tolerance of the FP64 path: Fb = 1 / PSWF reaches 6.4e6 at the facet edge
of this configuration (yB 128 of yN 140), so the intermediates reach 8.6e8
while the contributions peak at 2e6; a perturbation of the intermediates by
one unit roundoff moves the contributions by 5e-6 = 2.5e-12 of their peak
(oracle).  The device's FFTs and sums run in another order than numpy's, so
FP64 results are held to 1e-11 of the peak."""

import ctypes
import os

import numpy
import pytest
from numpy.testing import assert_allclose

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import recombine, synthesis, engine, _lib
    from oracle import crocodile_oracle
    rg = dict(numpy.load(os.path.join(HERE, "golden", "recombine_golden.npz")))
    return torch, recombine, synthesis, engine, _lib, crocodile_oracle, rg


def sizes(rg):
    return dict(image_size=int(rg["N"]), subgrid_spacing=128, yB_size=int(rg["yB_size"]),
                yN_size=int(rg["yN_size"]), yP_size=int(rg["yP_size"]),
                xA_size=int(rg["xA_size"]), xM_size=int(rg["xM_size"]),
                xMxN_yP_size=int(rg["xMxN_yP_size"]))


def ocfg(O, rg):
    return O.RecombineConfig(int(rg["N"]), int(rg["yB_size"]), int(rg["yN_size"]),
                             int(rg["yP_size"]), int(rg["xA_size"]), int(rg["xM_size"]),
                             int(rg["xMxN_yP_size"]), rg["pswf"])


def test_windows(env):
    torch, R, S, E, L, O, rg = env
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    assert (rc.xM_yP_size, rc.xM_yN_size) == (int(rg["xM_yP_size"]), int(rg["xM_yN_size"]))
    assert (rc.facet_spacing, rc.yP_spacing, rc.xM_spacing) == (4, 54, 2)
    Fb, Fn, m = rc.windows()
    sh = numpy.fft.ifftshift
    assert_allclose(Fb, sh(rg["Fb"]), rtol=1e-15)
    assert_allclose(Fn, sh(rg["Fn"]), rtol=1e-15)
    assert_allclose(m, sh(rg["facet_m0_trunc"]), rtol=0, atol=1e-15)
    # the default PSWF is the notebook's (same c up to rounding; scipy's
    # pro_ang1 tail at 1e-11 is sensitive to the last bits of c)
    assert_allclose(R.default_pswf(512, 140, 128, 256), rg["pswf"], rtol=0, atol=1e-12)


def test_facet_to_subgrids_fp64(env):
    torch, R, S, E, L, O, rg = env
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    so = rg["subgrid_off"]
    cfg = ocfg(O, rg)
    for f, facet in enumerate(rg["facet2"]):
        got = rc.facet_to_subgrids(facet, so, so).cpu().numpy()
        want = O.rc_facet_to_subgrids(cfg, facet, so, so)
        tol = 1e-11 * numpy.abs(want).max()
        for s, (i0, i1) in enumerate(rg["subgrid2_idx"]):
            assert_allclose(got[i0, i1], rg["nmbf2"][f, s], rtol=0, atol=tol)
        assert_allclose(got, want, rtol=0, atol=tol)
    # unequal offset lists, repeated and wrapped offsets
    o0, o1 = [384, 0, 128], [256, 640, 256 - 512]
    got = rc.facet_to_subgrids(rg["facet2"][1], o0, o1).cpu().numpy()
    want = O.rc_facet_to_subgrids(cfg, rg["facet2"][1], [o % 512 for o in o0],
                                  [o % 512 for o in o1])
    assert_allclose(got, want, rtol=0, atol=1e-11 * numpy.abs(want).max())


def test_raw_layout_c_abi(env):
    # the C prototype's layout: facet and NMBF_NMBF ifftshifted, add_facet
    # dividing by xM^2 before an unnormalised backward FFT
    torch, R, S, E, L, O, rg = env
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    cfg = ocfg(O, rg)
    sh = numpy.fft.ifftshift
    facet = rg["facet2"][1]
    so = rg["subgrid_off"]
    f = E.cuda_tensor(sh(facet), E.CD)
    o = E.cuda_tensor(so, torch.int32)
    n = rc.xM_yN_size
    out = torch.empty((4, 4, n, n), dtype=E.CD, device="cuda")
    ws = torch.empty(L.lib().cg_recombine_workspace_bytes(rc._h, 4, 4), dtype=torch.uint8,
                     device="cuda")
    st = E.Status()
    st.reset()
    L.call("cg_recombine_facet_to_subgrids", rc._h, E._p(f), 0, E._p(o), 4, E._p(o), 4,
           E._p(out), 0, E._p(ws), ws.numel(), E._p(st.t), E.stream())
    st.check()
    want = O.rc_facet_to_subgrids(cfg, facet, so, so)
    assert_allclose(out.cpu().numpy(), sh(want, axes=(2, 3)), rtol=0,
                    atol=1e-11 * numpy.abs(want).max())
    sub = torch.zeros((16, cfg.xM, cfg.xM), dtype=E.CD, device="cuda")
    L.call("cg_recombine_add_facet", rc._h, E._p(out), 16, 256, 128, 0, E._p(sub), E.stream())
    E.fft_raw(sub, inverse=True)
    approx = numpy.zeros((16, cfg.xM, cfg.xM), dtype=complex)
    for s in range(16):
        O.rc_add_facet(cfg, approx[s], want[s // 4, s % 4], 256, 128)
    want_sub = numpy.array([sh(O.ifft(a)) for a in approx])
    assert_allclose(sub.cpu().numpy(), want_sub, rtol=0, atol=1e-11 * numpy.abs(want_sub).max())


def _test_image(O, rg):
    N = int(rg["N"])
    numpy.random.seed(0)
    numpy.random.rand(N)
    G2 = numpy.exp(2j * numpy.pi * numpy.random.rand(N, N)) * numpy.random.rand(N, N) / 2
    return G2


def _facets(O, rg, FG, cfg):
    fo, fb = rg["facet_off"], rg["facet_B"]
    return [[O.extract_mid(numpy.roll(FG, (-fo[j0], -fo[j1]), (0, 1)), cfg.yB) *
             numpy.outer(fb[j0], fb[j1]) for j1 in range(len(fo))] for j0 in range(len(fo))]


def test_recombine_accuracy(env):
    # the notebook's 2-D test (cells 20, 29, 30): RMSE of the recombined
    # subgrids against the image's own subgrids
    torch, R, S, E, L, O, rg = env
    cfg = ocfg(O, rg)
    G2 = _test_image(O, rg)
    facets = _facets(O, rg, O.fft(G2), cfg)
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    so, fo, sa = rg["subgrid_off"], rg["facet_off"], rg["subgrid_A"]
    subs = rc.recombine(facets, fo, fo, so, so).cpu().numpy()
    err = 0
    for i0 in range(4):
        for i1 in range(4):
            mask = numpy.outer(sa[i0], sa[i1])
            ref = O.extract_mid(numpy.roll(G2, (-so[i0], -so[i1]), (0, 1)), cfg.xA) * mask
            err += numpy.abs(subs[i0, i1] * mask - ref) ** 2 / 16
    rmse = numpy.sqrt(numpy.mean(err))
    assert_allclose(rmse, rg["rmse2"], rtol=1e-3)


def test_degrid_from_recombined_subgrids(env):
    # notebook cells 32-44: facets of a grid-corrected image, recombined into
    # subgrids, degridded; against degridding the whole grid (oracle)
    torch, R, S, E, L, O, rg = env
    cfg = ocfg(O, rg)
    N, xM = cfg.N, cfg.xM
    so, fo = rg["subgrid_off"], rg["facet_off"]
    rng = numpy.random.default_rng(3)
    G2 = numpy.exp(2j * numpy.pi * rng.random((N, N))) * rng.random((N, N)) / 2
    support, x0 = 10, 0.35
    gc_pswf = O.anti_aliasing_function(N, 0, numpy.pi * support / 2)
    gc = O.pad_mid(O.extract_mid(1 / gc_pswf, int(N * x0 * 2)), N)
    FGgc = O.fft(G2) * numpy.outer(gc, gc)
    Ggc = O.ifft(FGgc)
    kern = O.kernel_oversample(gc_pswf, 1024, support).real
    kern /= numpy.sum(kern[0])
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    subs = rc.recombine(_facets(O, rg, FGgc, cfg), fo, fo, so, so, crop=False)
    border = (so + numpy.hstack([so[1:], [N]])) // 2
    nv = 2000
    us = (N - support) / N * (rng.random(nv) - 0.5)
    vs = (N - support) / N * (rng.random(nv) - 0.5)
    deg = O.conv_predict(N, 1, numpy.column_stack([us, vs, numpy.zeros(nv)]), None, Ggc, kern)
    su = numpy.sum((us[:, None] * N + N) % N >= border, axis=1) % 4
    sv = numpy.sum((vs[:, None] * N + N) % N >= border, axis=1) % 4
    xMf = xM / (2 * N)
    errs = []
    for a in range(4):
        for b in range(4):
            sel = numpy.where((su == b) & (sv == a))[0]
            sou = (((so[b] + N // 2) % N) - N // 2) / N
            sov = (((so[a] + N // 2) % N) - N // 2) / N
            u = numpy.column_stack([us[sel] - sou, vs[sel] - sov, numpy.zeros(len(sel))])
            u[numpy.abs(u[:, 0] / 2 / xMf) >= 0.5, 0] -= 1
            u[numpy.abs(u[:, 1] / 2 / xMf) >= 0.5, 1] -= 1
            d = S.conv_predict(N, 2 * xMf, u, None, subs[a, b].contiguous(), kern,
                               precision="fp64")
            d = d.cpu().numpy() if isinstance(d, torch.Tensor) else d
            errs.append(numpy.abs(d - deg[sel]))
    e = numpy.concatenate(errs)
    # the method's own error on this set is 1.4e-7 rms (oracle, FP64)
    assert numpy.sqrt(numpy.mean(e ** 2)) < 2.5e-7
    assert e.max() < 1e-6


def test_errors(env):
    torch, R, S, E, L, O, rg = env
    kw = sizes(rg)
    with pytest.raises(ValueError):
        R.Recombine(pswf=rg["pswf"], **dict(kw, yP_size=217))  # xM * yP not a multiple of N
    with pytest.raises(ValueError):
        R.Recombine(pswf=rg["pswf"][:-1], **kw)
    rc = R.Recombine(pswf=rg["pswf"], **kw)
    with pytest.raises(IndexError):
        rc.facet_to_subgrids(rg["facet2"][0], [0, 64], [0])  # not a multiple of 128
    with pytest.raises(ValueError):
        rc.facet_to_subgrids(rg["facet2"][0][:-2], [0], [0])
    approx = torch.zeros((1, cfg_xM(rg), cfg_xM(rg)), dtype=E.CD, device="cuda")
    nm = rc.facet_to_subgrids(rg["facet2"][0], [0], [0])
    with pytest.raises(ValueError):
        rc.add_facet(approx, nm, 2, 0)  # not a multiple of the facet spacing 4
    assert rc.facet_to_subgrids(rg["facet2"][0], [], [0]).shape[0] == 0


def cfg_xM(rg):
    return int(rg["xM_size"])


# ------------------------------------------------------------ subgrid -> facet

def _subgrids(O, rg, G2, cfg):
    so, sa = rg["subgrid_off"], rg["subgrid_A"]
    return numpy.array([[O.extract_mid(numpy.roll(G2, (-so[i0], -so[i1]), (0, 1)), cfg.xA) *
                         numpy.outer(sa[i0], sa[i1]) for i1 in range(len(so))]
                        for i0 in range(len(so))])


def test_subgrids_to_facet_vs_oracle(env):
    torch, R, S, E, L, O, rg = env
    cfg = ocfg(O, rg)
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    rng = numpy.random.default_rng(5)
    subs = rng.standard_normal((4, 4, cfg.xA, cfg.xA)) + 1j * rng.standard_normal(
        (4, 4, cfg.xA, cfg.xA))
    so, fo = rg["subgrid_off"], rg["facet_off"]
    fs = rc.subgrid_spectra(subs)
    fs_ref = numpy.array([[O.rc_split_subgrid(cfg, subs[i0, i1], [(0, 0)])[0] for i1 in range(4)]
                          for i0 in range(4)])
    # rc_split_subgrid crops to xM_yN; compare the full spectrum's middle
    c = cfg.xM // 2 - cfg.xM_yN // 2
    assert_allclose(fs.cpu().numpy()[:, :, c:c + cfg.xM_yN, c:c + cfg.xM_yN], fs_ref, rtol=0,
                    atol=1e-12 * numpy.abs(fs_ref).max())
    Fbb = numpy.outer(cfg.Fb, cfg.Fb)
    for (j0, j1) in ((0, 0), (2, 1), (3, 3)):
        got = rc.subgrids_to_facet(fs, so, so, fo[j0], fo[j1]).cpu().numpy() / Fbb
        fn = numpy.array([[O.rc_split_subgrid(cfg, subs[i0, i1], [(fo[j0], fo[j1])])[0]
                           for i1 in range(4)] for i0 in range(4)])
        want = O.rc_subgrids_to_facet(cfg, fn, so, so)
        assert_allclose(got, want, rtol=0, atol=1e-12 * numpy.abs(want).max())
    # split over two calls with accumulate = one call (compared before the
    # Fb x Fb weighting, which reaches 4e13 at the facet corners)
    fo0, fo1 = fo[1], fo[2]
    one = rc.subgrids_to_facet(fs, so, so, fo0, fo1).cpu().numpy() / Fbb
    two = rc.subgrids_to_facet(fs[:2], so[:2], so, fo0, fo1)
    rc.subgrids_to_facet(fs[2:].contiguous(), so[2:], so, fo0, fo1, out=two, accumulate=True)
    assert_allclose(two.cpu().numpy() / Fbb, one, rtol=0, atol=1e-12 * numpy.abs(one).max())


def test_split_accuracy(env):
    # the notebook's subgrid -> facet check (cell 18) in 2-D on its test image:
    # the device's error against the true facets equals the oracle's
    torch, R, S, E, L, O, rg = env
    cfg = ocfg(O, rg)
    G2 = _test_image(O, rg)
    FG2 = O.fft(G2)
    subs = _subgrids(O, rg, G2, cfg)
    facets = _facets(O, rg, FG2, cfg)
    so, fo, fb = rg["subgrid_off"], rg["facet_off"], rg["facet_B"]
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    got = rc.split(subs, so, so, fo, fo).cpu().numpy()
    err = err_ref = 0
    for j0 in (0, 2):
        for j1 in (1, 3):
            mask = numpy.outer(fb[j0], fb[j1])
            fn = numpy.array([[O.rc_split_subgrid(cfg, subs[i0, i1], [(fo[j0], fo[j1])])[0]
                               for i1 in range(4)] for i0 in range(4)])
            ref = O.rc_subgrids_to_facet(cfg, fn, so, so) * numpy.outer(cfg.Fb, cfg.Fb) * mask
            err += numpy.abs(got[j0, j1] * mask - facets[j0][j1]) ** 2
            err_ref += numpy.abs(ref - facets[j0][j1]) ** 2
    rmse, rmse_ref = numpy.sqrt(numpy.mean(err)), numpy.sqrt(numpy.mean(err_ref))
    assert rmse_ref < 1e-4 * numpy.sqrt(numpy.mean(numpy.abs(facets[0][1]) ** 2))
    assert_allclose(rmse, rmse_ref, rtol=1e-3)


def test_subgrids_to_facet_raw_layout(env):
    torch, R, S, E, L, O, rg = env
    cfg = ocfg(O, rg)
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    rng = numpy.random.default_rng(6)
    subs = rng.standard_normal((2, 3, cfg.xA, cfg.xA)) + 0j
    so = rg["subgrid_off"]
    fs = rc.subgrid_spectra(subs)
    want = rc.subgrids_to_facet(fs, so[:2], so[1:], 128, 256).cpu().numpy()
    sh = numpy.fft.ifftshift
    fs_raw = E.cuda_tensor(sh(fs.cpu().numpy(), axes=(2, 3)), E.CD)
    o0 = E.cuda_tensor(so[:2], torch.int32)
    o1 = E.cuda_tensor(so[1:], torch.int32)
    out = torch.zeros((cfg.yB, cfg.yB), dtype=E.CD, device="cuda")
    ws = torch.empty(L.lib().cg_recombine_workspace_bytes(rc._h, 2, 3), dtype=torch.uint8,
                     device="cuda")
    st = E.Status()
    st.reset()
    L.call("cg_recombine_subgrids_to_facet", rc._h, E._p(fs_raw), 0, E._p(o0), 2, E._p(o1), 3,
           128, 256, E._p(out), 0, 0, E._p(ws), ws.numel(), E._p(st.t), E.stream())
    st.check()
    assert_allclose(out.cpu().numpy(), sh(want), rtol=0, atol=1e-13 * numpy.abs(want).max())


@pytest.mark.parametrize("pow2", [False, True])
@pytest.mark.parametrize("centred", [1, 0])
def test_facet_add_equals_two_calls(env, pow2, centred):
    """cg_recombine_facet_add (the contributions summed into the subgrids by
    the last transforms' stores on the double-float pipeline, the two calls
    inside on the complex128 one) equals facet_to_subgrids + add_facet bit for
    bit, on the T05 set (yP 216: complex128 pipeline) and on a power-of-two set
    (double-float pipeline), in both layouts, at facet offsets that wrap."""
    torch, R, S, E, L, O, rg = env
    if pow2:
        kw = dict(image_size=512, subgrid_spacing=128, yB_size=128, yN_size=160, yP_size=256,
                  xA_size=128, xM_size=256, xMxN_yP_size=160)
        rc = R.Recombine(**kw)
    else:
        kw = sizes(rg)
        rc = R.Recombine(pswf=rg["pswf"], **kw)
    xM, n = rc.xM_size, rc.xM_yN_size
    yB = rc.yB_size
    rng = numpy.random.default_rng(11)
    so = numpy.array([0, 128, 256, 384], dtype=numpy.int32)
    o = E.cuda_tensor(so, torch.int32)
    ws = torch.empty(L.lib().cg_recombine_workspace_bytes(rc._h, 4, 4), dtype=torch.uint8,
                     device="cuda")
    st = E.Status()
    for fo0, fo1 in ((256, 128), (-128, 384)):
        f = E.cuda_tensor(rng.normal(size=(yB, yB)) + 1j * rng.normal(size=(yB, yB)), E.CD)
        base = E.cuda_tensor(rng.normal(size=(16, xM, xM)) + 0j, E.CD)
        two = base.clone()
        nm = torch.empty((4, 4, n, n), dtype=E.CD, device="cuda")
        st.reset()
        L.call("cg_recombine_facet_to_subgrids", rc._h, E._p(f), centred, E._p(o), 4, E._p(o),
               4, E._p(nm), centred, E._p(ws), ws.numel(), E._p(st.t), E.stream())
        L.call("cg_recombine_add_facet", rc._h, E._p(nm), 16, fo0, fo1, centred, E._p(two),
               E.stream())
        one = base.clone()
        L.call("cg_recombine_facet_add", rc._h, E._p(f), centred, E._p(o), 4, E._p(o), 4, fo0,
               fo1, E._p(one), centred, E._p(ws), ws.numel(), E._p(st.t), E.stream())
        st.check()
        assert torch.equal(one, two), (pow2, centred, fo0, fo1)


def test_recombine_uses_facet_add(env):
    # Recombine.recombine sums through facet_add: the same subgrids as the
    # two-call form
    torch, R, S, E, L, O, rg = env
    rc = R.Recombine(pswf=rg["pswf"], **sizes(rg))
    rng = numpy.random.default_rng(5)
    yB = rc.yB_size
    facets = [[rng.normal(size=(yB, yB)) + 0j for _ in range(2)] for _ in range(2)]
    fo, so = [0, 128], [0, 128, 256]
    got = rc.recombine(facets, fo, fo, so, so, crop=False)
    approx = torch.zeros_like(got)
    for j0 in range(2):
        for j1 in range(2):
            rc.add_facet(approx, rc.facet_to_subgrids(facets[j0][j1], so, so), fo[j0], fo[j1])
    assert torch.equal(got, rc.finish_subgrids(approx, crop=False))
