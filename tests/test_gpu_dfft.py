"""Double-float FFTs of complex128 rows (cg_fft_rows_df) against numpy's FP64
FFT, and the recombination with power-of-two rows (double-float transforms)
against the FP64 cuFFT form and the oracle."""

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


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, 2048])
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
            err = numpy.abs(got - want).max() / numpy.abs(want).max()
            assert err < 2e-14, (n, batch, inverse, err)


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
