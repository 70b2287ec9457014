"""Double-float FFTs of complex128 rows (cg_fft_rows_df) and centred 2-D
planes (cg_fft2_centred_df) against numpy's FP64 FFT, and the recombination
with power-of-two rows (double-float stage arrays and transforms) against the
FP64 cuFFT form and the oracle."""

import ctypes

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import engine, _lib, recombine
    from oracle import crocodile_oracle
    return torch, engine, _lib, recombine, crocodile_oracle


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, 2048, 4096, 8192])
def test_rows_match_numpy(env, n):
    torch, E, L, R, O = env
    rng = numpy.random.default_rng(n)
    for batch in (1, 7, 37):
        x = rng.normal(size=(batch, n)) + 1j * rng.normal(size=(batch, n))
        for inverse in (0, 1):
            t = E.cuda_tensor(x, E.CD)
            L.call("cg_fft_rows_df", E._p(t), batch, n, inverse, E.stream())
            want = numpy.fft.ifft(x, axis=1) * n if inverse else numpy.fft.fft(x, axis=1)
            got = t.cpu().numpy()
            # double-float carries about 48 bits: rounding ~1e-15 per stage
            # (4096 and 8192: the four-step passes, 12 and 13 stages)
            err = numpy.abs(got - want).max() / numpy.abs(want).max()
            assert err < (2e-14 if n <= 2048 else 4e-14), (n, batch, inverse, err)


def test_bad_lengths(env):
    torch, E, L, R, O = env
    t = torch.zeros((2, 96), dtype=E.CD, device="cuda")
    with pytest.raises(ValueError):
        L.call("cg_fft_rows_df", E._p(t), 2, 96, 0, E.stream())


def pow2_config():
    return dict(image_size=512, subgrid_spacing=128, yB_size=128, yN_size=160, yP_size=256,
                xA_size=128, xM_size=256, xMxN_yP_size=160)


def test_recombination_double_float_vs_fp64_and_oracle(env):
    torch, E, L, R, O = env
    kw = pow2_config()
    rc = R.Recombine(**kw)
    rc64 = R.Recombine(fft="fp64", **kw)
    assert rc.xM_yP_size == 128
    cfg = O.RecombineConfig(512, 128, 160, 256, 128, 256, 160, R.default_pswf(512, 160, 128, 256))
    rng = numpy.random.default_rng(2)
    facet = rng.normal(size=(128, 128)) + 1j * rng.normal(size=(128, 128))
    offs = [0, 128, 256, 384]
    a = rc.facet_to_subgrids(facet, offs, offs).cpu().numpy()
    b = rc64.facet_to_subgrids(facet, offs, offs).cpu().numpy()
    want = O.rc_facet_to_subgrids(cfg, facet, offs, offs)
    peak = numpy.abs(want).max()
    # observed: double-float 1.4e-11 of the peak from the oracle, FP64 cuFFT
    # 1.1e-12 -- the method's own error is ~1e-7
    assert numpy.abs(b - want).max() / peak < 1e-11
    assert numpy.abs(a - want).max() / peak < 1e-10
    subs = rng.normal(size=(4, 4, 128, 128)) + 0j
    fs = rc.subgrid_spectra(subs)
    Fbb = numpy.outer(cfg.Fb, cfg.Fb)  # compared before the Fb x Fb weighting
    fa = rc.subgrids_to_facet(fs, offs, offs, 128, 256).cpu().numpy() / Fbb
    fb = rc64.subgrids_to_facet(fs, offs, offs, 128, 256).cpu().numpy() / Fbb
    assert numpy.abs(fa - fb).max() / numpy.abs(fb).max() < 1e-10


def centred(x, inverse):
    ax = (-2, -1)
    f = numpy.fft.ifft2 if inverse else numpy.fft.fft2
    return numpy.fft.fftshift(f(numpy.fft.ifftshift(x, axes=ax), axes=ax), axes=ax)


@pytest.mark.parametrize("H,W", [(64, 64), (512, 512), (64, 2048), (2048, 128), (256, 1024),
                                 (1024, 64), (128, 256)])
def test_fft2_centred_matches_numpy(env, H, W):
    torch, E, L, R, O = env
    rng = numpy.random.default_rng(H * 7 + W)
    for batch in (1, 3):
        x = rng.normal(size=(batch, H, W)) + 1j * rng.normal(size=(batch, H, W))
        for inverse in (False, True):
            t = E.cuda_tensor(x, E.CD)
            E.fft_df_(t, inverse)
            want = centred(x, inverse)
            err = numpy.abs(t.cpu().numpy() - want).max() / numpy.abs(want).max()
            # log2(H W) <= 22 double-float stages, ~1e-15 each
            assert err < 5e-14, (H, W, batch, inverse, err)


def test_fft2_centred_bad_sizes(env):
    torch, E, L, R, O = env
    t = torch.zeros((96, 128), dtype=E.CD, device="cuda")
    with pytest.raises(ValueError):
        E.fft_df_(t, True)
    with pytest.raises(ValueError):
        L.call("cg_fft2_centred_df", E._p(t), 1, 96, 128, 1, E.stream())


def test_recombination_tiny_double_float_vs_fp64(env):
    """The 8192 / 1280 / 512 configuration (every transform a power of two:
    double-float stage arrays and FFTs) against complex128 with FP64 cuFFT,
    both directions and the subgrids' finishing transforms."""
    torch, E, L, R, O = env
    from crocodile_gb300.bench_configs import RECOMBINE_TINY, recombine_layout
    N, sp, yB, yN, yP, xA, xM, xMxN = RECOMBINE_TINY
    rc = R.Recombine(N, sp, yB, yN, yP, xA, xM, xMxN)
    rc64 = R.Recombine(N, sp, yB, yN, yP, xA, xM, xMxN, fft="fp64")
    fo, so = recombine_layout(N, sp, yB, xA)
    g = torch.Generator(device="cuda").manual_seed(5)
    facet = torch.randn((yB, yB), dtype=E.CD, device="cuda", generator=g)
    a = rc.facet_to_subgrids(facet, so, so)
    b = rc64.facet_to_subgrids(facet, so, so)
    peak = b.abs().max().item()
    # observed on the 256 / 128 set: double-float 1.4e-11 of the peak
    assert (a - b).abs().max().item() / peak < 1e-10
    ns = len(so)
    approx = torch.zeros((ns, 2, xM, xM), dtype=E.CD, device="cuda")
    rc.add_facet(approx, b[:, :2].contiguous(), fo[1], fo[2])
    approx64 = approx.clone()
    fa = rc.finish_subgrids(approx, crop=False)
    fb = rc64.finish_subgrids(approx64, crop=False)
    assert (fa - fb).abs().max().item() / fb.abs().max().item() < 5e-14
    # the other direction, compared before the Fb x Fb weighting
    spec = rc.subgrid_spectra(fb)
    spec64 = rc64.subgrid_spectra(fb)
    assert (spec - spec64).abs().max().item() / spec64.abs().max().item() < 5e-14
    Fb = rc.windows()[0]
    Fbb = torch.as_tensor(numpy.fft.fftshift(numpy.outer(Fb, Fb)), device="cuda")
    x = rc.subgrids_to_facet(spec64, so, so[:2], fo[1], fo[2]) / Fbb
    y = rc64.subgrids_to_facet(spec64, so, so[:2], fo[1], fo[2]) / Fbb
    assert (x - y).abs().max().item() / y.abs().max().item() < 1e-10


LONG_SETS = {
    # bench_recombine.c's "small" (16k-8k-512) and the same at half scale: yP
    # of 8192 and 4096, the four-step double-float rows
    "small": (16384, 32, 5120, 5632, 8192, 416, 512, 280),
    "half-small": (8192, 16, 2560, 2816, 4096, 208, 256, 140),
}


@pytest.mark.parametrize("name", ["half-small", "small"])
def test_recombination_long_rows_vs_fp64(env, name):
    """Sets whose yP is beyond one CTA's transform (4096, 8192): the
    double-float stage kernels with the four-step rows against complex128
    with FP64 cuFFT, both directions, and facet_add against the two calls."""
    torch, E, L, R, O = env
    N, sp, yB, yN, yP, xA, xM, xMxN = LONG_SETS[name]
    rc = R.Recombine(N, sp, yB, yN, yP, xA, xM, xMxN)
    rc64 = R.Recombine(N, sp, yB, yN, yP, xA, xM, xMxN, fft="fp64")
    offs = [0, xA, N - xA]
    g = torch.Generator(device="cuda").manual_seed(7)
    facet = torch.randn((yB, yB), dtype=E.CD, device="cuda", generator=g)
    a = rc.facet_to_subgrids(facet, offs, offs)
    b = rc64.facet_to_subgrids(facet, offs, offs)
    assert (a - b).abs().max().item() / b.abs().max().item() < 1e-10
    approx = torch.zeros((3, 3, xM, xM), dtype=E.CD, device="cuda")
    two = rc.add_facet(approx.clone(), a, sp * (N // sp // 4), 0)
    one = rc.facet_add(approx.clone(), facet, offs, offs, sp * (N // sp // 4), 0)
    assert torch.equal(one, two)
    subs = torch.randn((3, 3, xM, xM), dtype=E.CD, device="cuda", generator=g)
    spec = rc64.subgrid_spectra(subs)
    Fb = rc.windows()[0]
    Fbb = torch.as_tensor(numpy.fft.fftshift(numpy.outer(Fb, Fb)), device="cuda")
    x = rc.subgrids_to_facet(spec, offs, offs, 0, 0) / Fbb
    y = rc64.subgrids_to_facet(spec, offs, offs, 0, 0) / Fbb
    assert (x - y).abs().max().item() / y.abs().max().item() < 1e-10
