"""The hand-written FFTs of the imaging path (crocodile_gb300/csrc/fft32.cu,
FP32, power-of-two sides 64..8192) against numpy: the centred fft / ifft of
crocodile/synthesis.py:83-106 on complex64 planes and rows, batched planes,
the unshifted transform of the sub-grid stacks, and the dirty image of a
hermitian grid (do_imaging's real(ifft(make_grid_hermitian(g)))).  FP32
transforms are held to 2e-6 relative L2 against the complex128 result; the
complex128 centred transform (double-float, sides 64..2048) to 1e-13."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import engine as E
    from crocodile_gb300 import synthesis as S
    from oracle import crocodile_oracle as O
    return torch, E, S, O


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - numpy.asarray(b)) / numpy.linalg.norm(b)


def _rand(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


@pytest.mark.parametrize("H,W", [(64, 64), (128, 512), (1024, 1024), (2048, 256), (4096, 4096),
                                 (8192, 8192), (4096, 256), (8192, 64), (1, 4096), (1, 64)])
def test_centred_fft32_matches_numpy(env, H, W):
    torch, E, S, O = env
    rng = numpy.random.default_rng(H + W)
    a = _rand(rng, (W,) if H == 1 else (H, W))
    for inverse, ref in ((False, O.fft(a)), (True, O.ifft(a))):
        t = E.cuda_tensor(a, E.CF)
        E.fft_(t, inverse)
        assert rel(t.cpu().numpy(), ref) < 2e-6, (H, W, inverse)


@pytest.mark.parametrize("shape", [(3, 256, 512), (3, 4096, 512), (9, 4096, 4096)])
def test_batched_and_raw_fft32(env, shape):
    """Column tiles (256 x 512) and, for columns of 2048 and up, the four-step
    column passes (9 planes of 4096^2 go through the 1 GiB scratch stack in
    two chunks)."""
    torch, E, S, O = env
    rng = numpy.random.default_rng(3)
    a = _rand(rng, shape)
    H, W = shape[1], shape[2]
    t = E.cuda_tensor(a, E.CF)
    E.fft_(t, True)
    ref = numpy.array([O.ifft(p) for p in a])
    assert rel(t.cpu().numpy(), ref) < 2e-6
    for inverse in (False, True):
        t = E.cuda_tensor(a, E.CF)
        E.fft_raw(t, inverse)
        ref = numpy.fft.ifft2(a) * H * W if inverse else numpy.fft.fft2(a)
        assert rel(t.cpu().numpy(), ref) < 2e-6


@pytest.mark.parametrize("N", [256, 4096, 8192])
def test_image_from_grid_fft32(env, N):
    torch, E, S, O = env
    rng = numpy.random.default_rng(N)
    g = _rand(rng, (N, N))
    ref = numpy.real(O.ifft(O.make_grid_hermitian(g.copy())))
    t = E.cuda_tensor(g, E.CF)
    img, mx = E.image_from_grid(t, want_max=True)
    got = img.cpu().numpy()
    assert rel(got, ref) < 2e-6
    assert abs(float(mx.item()) - got.max()) <= 1e-6 * abs(got.max())


@pytest.mark.parametrize("N", [64, 512, 2048])
def test_centred_fft_complex128_double_float(env, N):
    torch, E, S, O = env
    rng = numpy.random.default_rng(N + 1)
    a = _rand(rng, (N, N))
    assert rel(S.fft(a), O.fft(a)) < 1e-13
    assert rel(S.ifft(a), O.ifft(a)) < 1e-13
