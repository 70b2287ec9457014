"""Differentiable gridding: autograd Functions whose backward is the adjoint kernel.

With the complex inner product <a, b> = sum(conj(a) b):

* degridding D (convdegrid with kernel K, crocodile/synthesis.py:484-503) has
  the adjoint D^H = convgrid with conj(K) (:464-481), and vice versa;
* the centred FFT F (fft, :83-93) has the adjoint F^H = N^2 * ifft (:96-106).

PyTorch's complex gradients follow the same convention (for a linear y = A x
the backward is A^H grad_y), so the backward passes below are exactly those
adjoint kernels, run by the same tiled CUDA kernels as the forward passes.
Gradients flow to visibilities, grids and real images; not to uvw or kernels.
"""

import torch

from . import engine as E


class GriddingOperator:
    """Grid/degrid operator for fixed coordinates and kernels (one shared plan).

    uvw: [n, 3] (wavelengths), lam: uv-grid width, shape: (H, W),
    ktab: an engine.KernelTable (complex64), kidx: per-visibility kernel rows."""

    def __init__(self, uvw, lam, shape, ktab, kidx=None, wbins=None):
        self.shape = (int(shape[0]), int(shape[1]))
        self.ktab = ktab.to(E.CF)
        self.ktab_conj = E.KernelTable(torch.conj(self.ktab.table).resolve_conj().contiguous(),
                                       ktab.sep, ktab.Q, ktab.S)
        self.plan = E.Plan(uvw, lam, self.shape, self.ktab, kidx, wbins=wbins)
        self.plan.check()
        self.n = self.plan.n

    # raw operators (no autograd)
    def D(self, grid):
        return self.plan.degrid(self.ktab, grid.contiguous())

    def DH(self, vis):
        g = torch.zeros(self.shape, dtype=E.CF, device="cuda")
        return self.plan.grid(self.ktab_conj, vis.contiguous(), g)

    def G(self, vis):
        g = torch.zeros(self.shape, dtype=E.CF, device="cuda")
        return self.plan.grid(self.ktab, vis.contiguous(), g)

    def GH(self, grid):
        return self.plan.degrid(self.ktab_conj, grid.contiguous())

    # autograd-enabled
    def degrid(self, grid):
        return Degrid.apply(grid, self)

    def grid(self, vis):
        return Grid.apply(vis, self)

    def predict(self, image):
        """Visibilities of a real image: degrid(fft(image)) (do_predict, :914-927)."""
        return self.degrid(image_fft(image))


class Degrid(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid, op):
        ctx.op = op
        return op.D(grid.to(E.CF))

    @staticmethod
    def backward(ctx, gv):
        return ctx.op.DH(gv.to(E.CF)), None


class Grid(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vis, op):
        ctx.op = op
        return op.G(vis.to(E.CF))

    @staticmethod
    def backward(ctx, gg):
        return ctx.op.GH(gg.to(E.CF)), None


class ImageFFT(torch.autograd.Function):
    """Real image -> centred FFT grid; backward N^2 * ifft, real part."""

    @staticmethod
    def forward(ctx, image):
        ctx.real = not image.is_complex()
        ctx.dtype = image.dtype
        t = image.to(E.CF).clone()
        return E.fft_(t, False)

    @staticmethod
    def backward(ctx, gy):
        H, W = gy.shape[-2], gy.shape[-1]
        t = gy.to(E.CF).clone()
        E.fft_(t, True)
        t = t * (H * W)
        return (t.real if ctx.real else t).to(ctx.dtype)


def image_fft(image):
    return ImageFFT.apply(image)
