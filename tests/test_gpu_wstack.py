"""Batched w-stacking (all planes in one gridding launch and one batched FFT)
against the oracle's per-plane loop (examples/notebooks/wstacking.ipynb cell 10
with conv_imaging), at a small size and at the full 4096^2 / 32-plane /
4M-visibility size of the w-stacking configuration, and at full size against
the one-plane-per-launch form."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import configs
    from crocodile_gb300 import synthesis as S
    from oracle import crocodile_oracle as O
    return torch, configs, S, O


def rel(a, b):
    return numpy.linalg.norm(numpy.asarray(a) - numpy.asarray(b)) / numpy.linalg.norm(b)


def test_wstack_matches_oracle(env):
    torch, configs, S, O = env
    w = configs.wstack(n=40000, planes=8, wmax=300.0)
    N = 512
    theta = w.theta
    lam = N / theta
    # same uv distribution scaled onto the smaller grid
    uvw = w.uvw.copy()
    uvw[:, :2] *= N / w.N
    kv = O.kernel_oversample(O.anti_aliasing_function(N, 0, 8), 8, 8)
    plane = w.params["plane"]
    ref = O.w_stack_imaging(theta, lam, uvw, None, w.vis, kv, plane)
    got = S.w_stack_imaging(theta, lam, uvw, None, w.vis, kv, plane)
    assert rel(got, ref) < 1e-5
    for gridder in ("tiled", "sparse"):  # both gridders of the stack
        got = S.w_stack_imaging(theta, lam, uvw, None, w.vis, kv, plane, gridder=gridder)
        assert rel(got, ref) < 1e-5, gridder
    got1 = S.w_stack_imaging(theta, lam, uvw, None, w.vis, kv, plane, per_plane=True)
    assert rel(got1, ref) < 1e-5


def test_wstack_empty_planes_skipped(env):
    torch, configs, S, O = env
    rng = numpy.random.default_rng(4)
    N, theta, n = 256, 0.1, 5000
    lam = N / theta
    uvw = numpy.column_stack([rng.uniform(-0.4, 0.4, (n, 2)) * lam, rng.uniform(-50, 50, n)])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    plane = numpy.where(uvw[:, 2] < 0, 0, 3)  # planes 1 and 2 stay empty
    kv = O.kernel_oversample(O.anti_aliasing_function(N, 0, 8), 8, 8)
    ref = O.w_stack_imaging(theta, lam, uvw, None, vis, kv, plane)
    assert rel(S.w_stack_imaging(theta, lam, uvw, None, vis, kv, plane), ref) < 1e-5


def test_wstack_full_size_batched_vs_per_plane(env):
    torch, configs, S, O = env
    w = configs.wstack()
    kv = O.kernel_oversample(O.anti_aliasing_function(w.N, 0, 8), 8, 8)
    uvw = torch.from_numpy(w.uvw).cuda()
    vis = torch.from_numpy(w.vis).cuda()
    plane = w.params["plane"]
    a = S.w_stack_imaging(w.theta, w.lam, uvw, None, vis, kv, plane)
    b = S.w_stack_imaging(w.theta, w.lam, uvw, None, vis, kv, plane, per_plane=True)
    err = float(torch.linalg.vector_norm((a - b).to(torch.complex128)) /
                torch.linalg.vector_norm(b.to(torch.complex128)))
    assert err < 1e-6, err


def test_wstack_full_size_matches_oracle(env):
    """The w-stacking configuration in full (4096^2, 32 planes, 4,000,000
    visibilities, S 8, Q 8 anti-aliasing kernel) against the oracle's complex128
    per-plane loop (examples/notebooks/wstacking.ipynb:190-226): about two minutes
    of host time for the oracle."""
    torch, configs, S, O = env
    w = configs.wstack()
    assert len(w.uvw) == 4_000_000 and w.N == 4096
    kv = O.kernel_oversample(O.anti_aliasing_function(w.N, 0, 8), 8, 8)
    plane = w.params["plane"]
    assert len(numpy.unique(plane)) == 32
    got = S.w_stack_imaging(w.theta, w.lam, w.uvw, None, w.vis, kv, plane)
    ref = O.w_stack_imaging(w.theta, w.lam, w.uvw, None, w.vis, kv, plane)
    assert rel(got, ref) < 1e-5


def test_wstack_fused_8192_matches_oracle(env):
    """8192^2 planes (four-step columns of 128 x 64 in the batched FFT); three
    planes, one of them empty, against the oracle."""
    torch, configs, S, O = env
    rng = numpy.random.default_rng(81)
    N, theta, n = 8192, 0.05, 20000
    lam = N / theta
    r = rng.uniform(0, 0.4 * lam, n)
    ph = rng.uniform(0, 2 * numpy.pi, n)
    uvw = numpy.column_stack([r * numpy.cos(ph), r * numpy.sin(ph), rng.uniform(-400, 400, n)])
    vis = rng.normal(size=n) + 1j * rng.normal(size=n)
    plane = numpy.where(uvw[:, 2] < 0, 0, 2)  # plane 1 stays empty
    kv = O.kernel_oversample(O.anti_aliasing_function(N, 0, 8), 8, 8)
    ref = O.w_stack_imaging(theta, lam, uvw, None, vis, kv, plane)
    got = S.w_stack_imaging(theta, lam, uvw, None, vis, kv, plane)
    assert rel(got, ref) < 1e-5
