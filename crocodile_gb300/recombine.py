"""Facet -> subgrid recombination on the device.

The algorithm of examples/notebooks/facet-subgrid-impl.ipynb (cells 24-30)
as optimised in the C prototype examples/grid/recombine.c: an image split
into facets of yB_size pixels is turned, facet by facet, into its
contributions to subgrids of xA_size cells of the image's grid (uv plane),
using PSWF windows so that each facet/subgrid pair only exchanges
xM_yN_size^2 values.  Summing a subgrid's contributions over all facets and
inverse-transforming gives the subgrid, which the degridder then reads
(``conv_predict`` on the subgrid, notebook cell 44).

``Recombine`` holds the configuration of ``recombine2d_set_config``
(recombine.c:135-196) on the device (``cg_recombine_create``); its methods
take numpy arrays or CUDA tensors in numpy's centred (fftshift) layout, as
the notebook, and return CUDA tensors:

* ``facet_to_subgrids(facet, offs0, offs1)``: NMBF_NMBF[i0, i1] of one facet
  for every pair of subgrid offsets (notebook cell 29; recombine.c
  pf1_ft1_es1 + pf0_ft0 + es0): two batched FFT passes per axis on the device;
* ``add_facet(approx, nmbf, facet_off0, facet_off1)``: approx += the
  contributions rolled to the facet (cell 30; recombine2d_af0_af1);
* ``facet_add(approx, facet, offs0, offs1, facet_off0, facet_off1)``: the two
  above in one call;
* ``finish_subgrids(approx)``: ifft and the middle xA_size (cell 30);
* ``recombine(facets, facet_offs0, facet_offs1, offs0, offs1)``: all of it.

and the other direction (notebook cell 18, in 2-D by separability):

* ``subgrid_spectra(subgrids)``: FFT of each subgrid padded to xM_size;
* ``subgrids_to_facet(fs, offs0, offs1, facet_off0, facet_off1)``: the facet
  approximation Fb x Fb x the sum of every subgrid's contribution;
* ``split(subgrids, offs0, offs1, facet_offs0, facet_offs1)``: all facets.

With ``fft="auto"`` and power-of-two transform lengths (yP and xM_yP in
64..2048) the whole pipeline runs in double-float arithmetic on the FP32
units (hi + lo float pairs, about 48 significant bits; GB300's FP64 rate
bounds FP64 work): the stage arrays, the row FFTs with the prepare, window
and crop steps in their loads and stores, and the subgrids' centred xM^2
transforms (``finish_subgrids``, ``subgrid_spectra``).  Other lengths and
``fft="fp64"`` keep complex128 stage arrays and FP64 cuFFT.  The arrays the
caller sees are complex128, as in the reference: Fb = 1 / PSWF spans
many decades towards the facet edge, and the contributions come out of
intermediates a thousand times larger than their peak, which single
precision cannot carry (measured: 6e-4 relative error per facet, the
recombined subgrids wrong at order one, where the method gives 2e-7).
"""

import ctypes

import numpy
import torch

from . import _lib as L
from . import engine as E
from .synthesis import anti_aliasing_function


def default_pswf(image_size, yN_size, xA_size, xM_size):
    """The PSWF the notebook derives its windows from (cell 14):
    anti_aliasing_function(yN_size, 0, 2 pi yN xN) with yN = yN_size / 2 and
    xN = (xM - xA) / 2 in image fractions (xM = xM_size / (2 image_size))."""
    c = numpy.pi * yN_size * (xM_size - xA_size) / (4.0 * image_size)
    return numpy.real(anti_aliasing_function(yN_size, 0, c))


class Recombine:
    """recombine2d_config on the device.  pswf: the PSWF [yN_size] in the
    notebook's centred layout (default: ``default_pswf``)."""

    def __init__(self, image_size, subgrid_spacing, yB_size, yN_size, yP_size, xA_size, xM_size,
                 xMxN_yP_size, pswf=None, fft="auto"):
        E.require_cuda()
        if pswf is None:
            pswf = default_pswf(image_size, yN_size, xA_size, xM_size)
        pswf = numpy.asarray(pswf, dtype=numpy.float64)
        if pswf.shape != (yN_size,):
            raise ValueError("pswf must have yN_size = %d samples" % yN_size)
        raw = numpy.ascontiguousarray(numpy.fft.ifftshift(pswf))
        self.image_size, self.subgrid_spacing = int(image_size), int(subgrid_spacing)
        self.yB_size, self.yN_size, self.yP_size = int(yB_size), int(yN_size), int(yP_size)
        self.xA_size, self.xM_size, self.xMxN_yP_size = int(xA_size), int(xM_size), \
            int(xMxN_yP_size)
        self.dtype = E.CD
        h = ctypes.c_void_p()
        L.call("cg_recombine_create", self.image_size, self.subgrid_spacing,
               raw.ctypes.data_as(ctypes.c_void_p), self.yB_size, self.yN_size, self.yP_size,
               self.xA_size, self.xM_size, self.xMxN_yP_size, ctypes.byref(h))
        self._h = h
        if fft not in ("auto", "fp64"):
            raise ValueError("fft must be 'auto' (double-float for power-of-two rows) or 'fp64'")
        L.call("cg_recombine_set_fft", h, 0 if fft == "auto" else 1)
        self.fft = fft
        sizes = (ctypes.c_int32 * 5)()
        L.call("cg_recombine_sizes", h, sizes)
        (self.xM_yP_size, self.xM_yN_size, self.facet_spacing, self.yP_spacing,
         self.xM_spacing) = [int(v) for v in sizes]
        self._ws = {}
        self.status = E.Status()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                L.lib().cg_recombine_destroy(h)
            except Exception:
                pass
            self._h = None

    def windows(self):
        """(Fb [yB], Fn [xM_yN], m [xMxN_yP]) in the C prototype's raw layout."""
        Fb = numpy.empty(self.yB_size)
        Fn = numpy.empty(self.xM_yN_size)
        m = numpy.empty(self.xMxN_yP_size)
        L.call("cg_recombine_windows", self._h, Fb.ctypes.data_as(ctypes.c_void_p),
               Fn.ctypes.data_as(ctypes.c_void_p), m.ctypes.data_as(ctypes.c_void_p))
        return Fb, Fn, m

    def _workspace(self, n0, n1):
        key = (n0, n1)
        if key not in self._ws:
            nbytes = L.lib().cg_recombine_workspace_bytes(self._h, n0, n1)
            self._ws = {key: torch.empty(nbytes, dtype=torch.uint8, device="cuda")}
        return self._ws[key]

    def facet_to_subgrids(self, facet, offs0, offs1, out=None, check=True):
        """NMBF_NMBF [n0, n1, xM_yN, xM_yN] (centred) of one centred facet
        [yB, yB] for every pair of subgrid offsets (grid cells, multiples of
        subgrid_spacing)."""
        f = E.cuda_tensor(facet, self.dtype)
        if tuple(f.shape) != (self.yB_size, self.yB_size):
            raise ValueError("facet must be %d x %d" % (self.yB_size, self.yB_size))
        o0 = E.cuda_tensor(numpy.atleast_1d(offs0) if not isinstance(offs0, torch.Tensor)
                           else offs0, torch.int32)
        o1 = E.cuda_tensor(numpy.atleast_1d(offs1) if not isinstance(offs1, torch.Tensor)
                           else offs1, torch.int32)
        n0, n1 = int(o0.numel()), int(o1.numel())
        n = self.xM_yN_size
        if out is None:
            out = torch.empty((n0, n1, n, n), dtype=self.dtype, device="cuda")
        ws = self._workspace(n0, n1)
        if check:
            self.status.reset()
        L.call("cg_recombine_facet_to_subgrids", self._h, E._p(f), 1, E._p(o0), n0, E._p(o1), n1,
               E._p(out), 1, E._p(ws), ws.numel(), E._p(self.status.t), E.stream())
        if check:
            self.status.check()
        return out

    def add_facet(self, approx, nmbf, facet_off0, facet_off1):
        """approx [..., xM, xM] += nmbf [..., xM_yN, xM_yN] padded and rolled to
        the facet offsets (grid pixels, multiples of the facet spacing)."""
        n = nmbf.numel() // (self.xM_yN_size ** 2)
        if approx.numel() != n * self.xM_size ** 2 or approx.dtype != self.dtype:
            raise ValueError("approx must hold %d subgrids of %d^2 %s" % (n, self.xM_size,
                                                                          self.dtype))
        L.call("cg_recombine_add_facet", self._h, E._p(nmbf.contiguous()), n, int(facet_off0),
               int(facet_off1), 1, E._p(approx), E.stream())
        return approx

    def _fft2_(self, t, inverse):
        # the double-float 2-D transform where its sizes allow ("auto"), else
        # FP64 cuFFT
        if self.fft == "auto" and E.dfft2_supported(self.xM_size, self.xM_size) \
                and t.is_contiguous():
            return E.fft_df_(t, inverse)
        return E.fft_(t, inverse)

    def facet_add(self, approx, facet, offs0, offs1, facet_off0, facet_off1, check=True):
        """approx [n0, n1, xM, xM] (centred) += the contributions of one centred
        facet at (facet_off0, facet_off1) to the subgrids at offs0 x offs1:
        facet_to_subgrids and add_facet in one call (cg_recombine_facet_add), the
        same values, without the contributions array on the double-float
        pipeline."""
        f = E.cuda_tensor(facet, self.dtype)
        if tuple(f.shape) != (self.yB_size, self.yB_size):
            raise ValueError("facet must be %d x %d" % (self.yB_size, self.yB_size))
        o0 = E.cuda_tensor(numpy.atleast_1d(offs0) if not isinstance(offs0, torch.Tensor)
                           else offs0, torch.int32)
        o1 = E.cuda_tensor(numpy.atleast_1d(offs1) if not isinstance(offs1, torch.Tensor)
                           else offs1, torch.int32)
        n0, n1 = int(o0.numel()), int(o1.numel())
        if approx.numel() != n0 * n1 * self.xM_size ** 2 or approx.dtype != self.dtype \
                or not approx.is_contiguous():
            raise ValueError("approx must be contiguous %d x %d subgrids of %d^2 %s"
                             % (n0, n1, self.xM_size, self.dtype))
        ws = self._workspace(n0, n1)
        if check:
            self.status.reset()
        L.call("cg_recombine_facet_add", self._h, E._p(f), 1, E._p(o0), n0, E._p(o1), n1,
               int(facet_off0), int(facet_off1), E._p(approx), 1, E._p(ws), ws.numel(),
               E._p(self.status.t), E.stream())
        if check:
            self.status.check()
        return approx

    def finish_subgrids(self, approx, crop=True):
        """The subgrids from their summed contributions: centred ifft (in place)
        and, with crop, the middle xA_size (a view)."""
        self._fft2_(approx, inverse=True)
        if not crop:
            return approx
        c = self.xM_size // 2 - self.xA_size // 2
        return approx[..., c:c + self.xA_size, c:c + self.xA_size]

    def recombine(self, facets, facet_offs0, facet_offs1, offs0, offs1, crop=True):
        """All subgrids [n0, n1, xA, xA] (or [.., xM, xM] without crop) of the
        facets [nf0, nf1, yB, yB] at facet_offs0 x facet_offs1."""
        n0, n1 = len(offs0), len(offs1)
        approx = torch.zeros((n0, n1, self.xM_size, self.xM_size), dtype=self.dtype,
                             device="cuda")
        o0 = E.cuda_tensor(numpy.asarray(offs0), torch.int32)
        o1 = E.cuda_tensor(numpy.asarray(offs1), torch.int32)
        self.status.reset()
        for j0, fo0 in enumerate(facet_offs0):
            for j1, fo1 in enumerate(facet_offs1):
                self.facet_add(approx, facets[j0][j1], o0, o1, fo0, fo1, check=False)
        self.status.check()
        return self.finish_subgrids(approx, crop=crop)

    # ------------------------------------------------------ subgrid -> facet

    def subgrid_spectra(self, subgrids):
        """FS [..., xM, xM]: centred FFT of each centred subgrid [..., xA, xA]
        (or already [..., xM, xM]) zero-padded to xM_size."""
        s = E.cuda_tensor(subgrids, self.dtype)
        xA = s.shape[-1]
        if xA != self.xM_size:
            lo = self.xM_size // 2 - xA // 2
            fs = torch.zeros(tuple(s.shape[:-2]) + (self.xM_size, self.xM_size),
                             dtype=self.dtype, device="cuda")
            fs[..., lo:lo + xA, lo:lo + xA] = s
        else:
            fs = s.clone()
        return self._fft2_(fs, inverse=False)

    def subgrids_to_facet(self, fs, offs0, offs1, facet_off0, facet_off1, out=None,
                          accumulate=False, check=True):
        """The facet [yB, yB] (centred) from the spectra fs [n0, n1, xM, xM] of
        the subgrids at offs0 x offs1: Fb x Fb times the sum of their
        contributions (notebook cell 18; the facet mask is left to the caller)."""
        fs = E.cuda_tensor(fs, self.dtype)
        o0 = E.cuda_tensor(numpy.atleast_1d(offs0) if not isinstance(offs0, torch.Tensor)
                           else offs0, torch.int32)
        o1 = E.cuda_tensor(numpy.atleast_1d(offs1) if not isinstance(offs1, torch.Tensor)
                           else offs1, torch.int32)
        n0, n1 = int(o0.numel()), int(o1.numel())
        if fs.numel() != n0 * n1 * self.xM_size ** 2:
            raise ValueError("fs must hold %d x %d subgrid spectra of %d^2" % (n0, n1, self.xM_size))
        if out is None:
            out = torch.zeros((self.yB_size, self.yB_size), dtype=self.dtype, device="cuda")
        ws = self._workspace(n0, n1)
        if check:
            self.status.reset()
        L.call("cg_recombine_subgrids_to_facet", self._h, E._p(fs), 1, E._p(o0), n0, E._p(o1),
               n1, int(facet_off0), int(facet_off1), E._p(out), 1, int(bool(accumulate)),
               E._p(ws), ws.numel(), E._p(self.status.t), E.stream())
        if check:
            self.status.check()
        return out

    def split(self, subgrids, offs0, offs1, facet_offs0, facet_offs1):
        """All facets [nf0, nf1, yB, yB] from the subgrids [n0, n1, xA, xA]."""
        fs = self.subgrid_spectra(subgrids)
        o0 = E.cuda_tensor(numpy.asarray(offs0), torch.int32)
        o1 = E.cuda_tensor(numpy.asarray(offs1), torch.int32)
        out = torch.empty((len(facet_offs0), len(facet_offs1), self.yB_size, self.yB_size),
                          dtype=self.dtype, device="cuda")
        self.status.reset()
        for j0, fo0 in enumerate(facet_offs0):
            for j1, fo1 in enumerate(facet_offs1):
                self.subgrids_to_facet(fs, o0, o1, fo0, fo1, out=out[j0, j1], check=False)
        self.status.check()
        return out
