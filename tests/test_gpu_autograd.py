"""Differentiable predict/invert (the 2048^2, 1M-visibility configuration):
adjoint dot-product tests, agreement of the backward pass with the oracle's
adjoint pair, and central finite differences on 64 random pixels evaluated
in FP64 on the device."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crocodile_gb300 import autograd as AG
    from crocodile_gb300 import configs
    from crocodile_gb300 import engine as E
    from crocodile_gb300 import synthesis as S
    from oracle import crocodile_oracle as O
    return torch, AG, configs, E, S, O


def _kernel(O, N):
    aa = O.anti_aliasing_function(N, 0, 8)
    return O.kernel_oversample(aa, 8, 8)  # separable [Q, S] = [8, 8]


def _problem(env, n=None, N=None):
    torch, AG, configs, E, S, O = env
    w = configs.diff()
    uvw, image = w.uvw, w.params["image"]
    N = N or w.N
    if n is not None:
        uvw = uvw[:n]
    if N != w.N:  # a smaller image of the same construction, uv scaled onto its grid
        uvw = uvw.copy()
        uvw[:, :2] *= N / w.N
        rng = numpy.random.default_rng(7)
        image = numpy.zeros((N, N), numpy.float32)
        ix = rng.integers(N // 4, 3 * N // 4, (50, 2))
        image[ix[:, 1], ix[:, 0]] = rng.normal(size=50)
    lam = N / w.theta
    kv = _kernel(O, N)
    kt = E.KernelTable.from_gcf(kv, 0, E.CF)
    op = AG.GriddingOperator(uvw, lam, (N, N), kt)
    return w, uvw, image, lam, kv, kt, op


def _cdot(a, b):  # <a, b> = sum(conj(a) b), in complex128
    return complex((a.conj().to(__import__("torch").complex128) *
                    b.to(__import__("torch").complex128)).sum())


def test_dot_product_adjoints(env):
    torch = env[0]
    w, uvw, image, lam, kv, kt, op = _problem(env)
    gen = torch.Generator(device="cuda").manual_seed(3)
    N = image.shape[0]
    g = torch.randn((N, N), dtype=torch.complex64, device="cuda", generator=gen)
    v = torch.randn(op.n, dtype=torch.complex64, device="cuda", generator=gen)
    lhs, rhs = _cdot(op.D(g), v), _cdot(g, op.DH(v))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    lhs, rhs = _cdot(op.G(v), g), _cdot(v, op.GH(g))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    # FFT: <F x, y> = <x, F^H y> for real x
    from crocodile_gb300 import autograd as AG
    x = torch.randn((N, N), dtype=torch.float32, device="cuda", generator=gen)
    y = torch.randn((N, N), dtype=torch.complex64, device="cuda", generator=gen)
    x.requires_grad_(True)
    Fx = AG.image_fft(x)
    (gx,) = torch.autograd.grad(Fx, x, grad_outputs=y)
    lhs = _cdot(Fx.detach(), y).real
    rhs = float((x.detach().double() * gx.double()).sum())
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_predict_and_backward_match_oracle(env):
    torch, AG, configs, E, S, O = env
    w, uvw, image, lam, kv, kt, op = _problem(env, n=20000, N=256)
    theta = w.theta
    img = torch.from_numpy(image).cuda().requires_grad_(True)
    pred = op.predict(img)
    ref = O.do_predict(theta, lam, uvw, None, image.astype(float), O.conv_predict, kv=kv)
    assert numpy.linalg.norm(pred.detach().cpu().numpy() - ref) / numpy.linalg.norm(ref) < 1e-5
    rng = numpy.random.default_rng(11)
    r = (rng.normal(size=len(uvw)) + 1j * rng.normal(size=len(uvw))) * 0.1
    loss = (torch.abs(pred - torch.from_numpy(r).cuda().to(torch.complex64)) ** 2).sum()
    (grad,) = torch.autograd.grad(loss, img)
    # oracle adjoint pair: dL/dx = 2 Re(N^2 ifft(convgrid(conj K, pred - r)))
    resid = ref - r
    a = numpy.zeros((256, 256), complex)
    O.convgrid(numpy.conj(kv), a, uvw / lam, None, resid)
    g_ref = 2 * numpy.real(256 * 256 * O.ifft(a))
    err = numpy.linalg.norm(grad.cpu().numpy() - g_ref) / numpy.linalg.norm(g_ref)
    assert err < 1e-5, err


def test_finite_differences_full_size(env):
    """Config: 2048^2 image, 1M visibilities, loss ||pred - vis_obs||^2 with vis_obs the
    prediction of a perturbed image plus complex noise (sigma 0.01).  The gradient from
    the FP32 adjoint kernels matches central differences of the loss evaluated with the
    FP64 plain form to 1e-4 on 64 random pixels, each relative to its own derivative
    or to 1e-2 of the largest sampled one, whichever is larger."""
    torch, AG, configs, E, S, O = env
    w, uvw, image, lam, kv, kt, op = _problem(env)
    N = image.shape[0]
    rng = numpy.random.default_rng(5)
    src = w.params["sources"]
    perturbed = image.copy()
    perturbed[src[:, 1], src[:, 0]] *= (1 + 0.1 * rng.normal(size=len(src))).astype(numpy.float32)
    kt64 = E.KernelTable.from_gcf(kv, 0, E.CD)
    plan64 = E.Plan(uvw, lam, (N, N), kt64, mode=1)  # CG_PLAN_GROUPS: the plain FP64 form

    def predict64(x):
        g = E.cuda_tensor(x, E.CD)
        E.fft_(g, False)
        return plan64.degrid_fp64(kt64, g)

    noise = (rng.normal(size=len(uvw)) + 1j * rng.normal(size=len(uvw))) * 0.01
    vis_obs = predict64(perturbed) + torch.from_numpy(noise).cuda()
    img = torch.from_numpy(image).cuda().requires_grad_(True)
    pred = op.predict(img)
    loss = (torch.abs(pred - vis_obs.to(torch.complex64)) ** 2).sum()
    (grad,) = torch.autograd.grad(loss, img)
    grad = grad.cpu().numpy()

    def loss64(x):
        return float((torch.abs(predict64(x) - vis_obs) ** 2).sum())

    h = 1e-3
    pix = rng.integers(0, N, (64, 2))
    fd = []
    base = image.astype(numpy.float64)
    for (py, px) in pix:
        e = numpy.zeros_like(base)
        e[py, px] = h
        fd.append((loss64(base + e) - loss64(base - e)) / (2 * h))
    fd = numpy.array(fd)
    an = grad[pix[:, 0], pix[:, 1]].astype(numpy.float64)
    # per pixel, relative to that pixel's own derivative; a pixel whose derivative
    # is below 1e-2 of the largest sampled one is held to 1e-4 of that floor,
    # i.e. to 1e-6 of the largest derivative, about 16 FP32 ulps of it: the
    # FP32 residual and adjoint round relative to the whole gradient, not to
    # one small entry of it (the loss is quadratic, so the FP64 central
    # differences themselves carry no truncation error)
    top = numpy.max(numpy.abs(fd))
    floor = 1e-2 * top
    rel = numpy.abs(an - fd) / numpy.maximum(numpy.abs(fd), floor)
    assert numpy.max(rel) < 1e-4, "worst pixel %s: analytic %g, central difference %g (%g)" % (
        tuple(pix[numpy.argmax(rel)]), an[numpy.argmax(rel)], fd[numpy.argmax(rel)],
        numpy.max(rel))
    assert numpy.count_nonzero(numpy.abs(fd) >= 1e-3 * top) >= 48  # most pixels are not tiny
