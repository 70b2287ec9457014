"""AW kernel generation: the FFT form (complex64 tables of 16 x 16 kernels,
32 x 32 circular convolutions of the zero-padded kernels) against the direct
sums (complex128 output) and the oracle's aw_kernel_fn (scipy convolve2d in
FP64), for odd and even w supports."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import engine
    from oracle import crocodile_oracle
    return torch, engine, crocodile_oracle


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - b) / numpy.linalg.norm(b)


@pytest.mark.parametrize("S", [16, 15, 8, 5])
def test_fft_form_matches_direct_and_oracle(env, S):
    torch, E, O = env
    rng = numpy.random.default_rng(S)
    nA, nW, Q, SA, nk = 4, 3, 4, 16, 40
    c = (numpy.arange(SA) - SA // 2) / SA
    A = numpy.array([numpy.exp(-((c[:, None] / 0.2) ** 2 + (c[None, :] / 0.25) ** 2)) *
                     numpy.exp(2j * numpy.pi * rng.normal() * (c[:, None] + c[None, :]))
                     for _ in range(nA)])
    W = rng.normal(size=(nW, Q, Q, S, S)) + 1j * rng.normal(size=(nW, Q, Q, S, S))
    a1 = rng.integers(0, nA, nk).astype(numpy.int32)
    a2 = rng.integers(0, nA, nk).astype(numpy.int32)
    wi = rng.integers(0, nW, nk).astype(numpy.int32)
    fft_form = E.aw_kernels(A, W, a1, a2, wi, dtype=E.CF).cpu().numpy()
    direct = E.aw_kernels(A, W, a1, a2, wi, dtype=E.CD).cpu().numpy()
    assert fft_form.shape == (nk, Q, Q, SA, SA)
    assert rel(fft_form, direct) < 2e-6
    fn = O.aw_kernel_fn(lambda theta, a: A[a], lambda theta, w: W[int(w)])
    for k in (0, 7, 39):
        ref = fn(0.1, wi[k], a1[k], a2[k])
        assert rel(fft_form[k], ref) < 2e-6, k
