"""Drop-in replacement for crocodile.synthesis on a GB300.

Same function names, argument meanings, defaults and exceptions as the
reference module (crocodile/synthesis.py; cited per function).  Grids,
visibilities and kernels given as numpy arrays come back as numpy arrays of
the reference's dtypes (complex128 / float64 / int64); given as CUDA torch
tensors they stay on the device.  The visibility hot path -- coordinates,
binning, sorting, convolutional gridding and degridding, weighting,
hermitian symmetry, FFTs and kernel generation -- runs in the hand-written
sm_103a kernels of libcrocodile_gb300.so; there is no CPU fallback.

Precision: the default ``precision="fp32"`` grids complex64 visibilities with
FP32 products and accumulation in the tiled persistent kernels, while cell
assignment and w binning stay bit-exact FP64 and kernels are generated in
FP64.  ``precision="fp64"`` selects the plain complex128 form (FP64 atomics,
one launch per kernel group).  Drivers accept ``precision=`` as an extra
keyword; ``set_precision`` changes the module default.

Small host-side helpers that only reshape or describe arrays (coordinates,
pad/extract, the prolate spheroidal taper from scipy, slicing) are plain
numpy, as in the reference.
"""

import functools

import numpy
import scipy.special
import torch

from . import _lib
from . import engine as E

_PRECISION = "fp32"


def set_precision(p):
    """Module default for the gridding precision: "fp32" (tiled) or "fp64" (plain)."""
    global _PRECISION
    if p not in ("fp32", "fp64"):
        raise ValueError("precision must be 'fp32' or 'fp64'")
    _PRECISION = p


def _prec(p):
    p = _PRECISION if p is None else p
    if p not in ("fp32", "fp64"):
        raise ValueError("precision must be 'fp32' or 'fp64'")
    return p


def _is_dev(x):
    return isinstance(x, torch.Tensor) and x.is_cuda


def _host(t, like=None, dtype=None):
    """Device tensor -> numpy (complex128 / float64 / int64 as the reference returns)."""
    if like is not None and _is_dev(like):
        return t
    a = t.detach().cpu().numpy()
    if dtype is not None:
        return a.astype(dtype)
    if numpy.iscomplexobj(a):
        return a.astype(numpy.complex128)
    if a.dtype.kind == "f":
        return a.astype(numpy.float64)
    if a.dtype.kind == "i":
        return a.astype(numpy.int64)
    return a


def _nrows(x):
    return x.shape[0]


def _src_cols(src, n):
    """Columns of src as an [n, k] array (0 for None or empty); a tensor's shape is
    read without copying it to the host."""
    if src is None:
        return 0
    size = src.numel() if isinstance(src, torch.Tensor) else numpy.size(src)
    if size == 0:
        return 0
    if n == 0 or size % n:
        raise ValueError("src has %d values, not a multiple of the %d rows" % (size, n))
    return size // n


# --------------------------------------------------------------------------
# coordinates, FFT conventions, padding (synthesis.py:38-197)

def coordinateBounds(N):
    """Lowest and highest coordinate of an N grid (synthesis.py:38-55)."""
    if N % 2 == 0:
        return -0.5, 0.5 * (N - 2) / N
    return -0.5 * (N - 1) / N, 0.5 * (N - 1) / N


def coordinates(N):
    """1-D coordinates spanning [-0.5, 0.5) with 0 at N//2 (synthesis.py:57-63)."""
    lo = -(N // 2)
    return numpy.arange(lo, lo + N) / N


def coordinates2(N):
    """(x, y) coordinate grids with (0, 0) at (N//2, N//2) (synthesis.py:66-80)."""
    c = numpy.arange(-(N // 2), -(N // 2) + N)
    rows, cols = numpy.meshgrid(c, c, indexing="ij")
    return numpy.array([cols, rows]) / N


def _centred_fft(a, inverse):
    dev = _is_dev(a)
    if not dev:
        a = numpy.asarray(a)
        if a.ndim not in (1, 2):
            raise AssertionError("Unsupported shape for FFT!")
    t = E.cuda_tensor(a, E.CD if not dev or a.dtype != E.CF else E.CF)
    if t.dim() not in (1, 2):
        raise AssertionError("Unsupported shape for FFT!")
    E.fft_(t, inverse)
    return t if dev else _host(t)


def fft(a):
    """Image -> grid: fftshift(fft2(ifftshift(a))) on the device (synthesis.py:83-93)."""
    return _centred_fft(a, False)


def ifft(a):
    """Grid -> image, normalised by 1/N^2, on the device (synthesis.py:96-106)."""
    return _centred_fft(a, True)


def pad_mid(ff, N):
    """Zero-pad a far field to N around its middle (synthesis.py:109-129)."""
    N0 = ff.shape[0]
    if N == N0:
        return ff
    assert N > N0
    lo, hi = N // 2 - N0 // 2, (N + 1) // 2 - (N0 + 1) // 2
    if ff.ndim == 2:
        assert N0 == ff.shape[1]
        return numpy.pad(ff, [(lo, hi), (lo, hi)], mode="constant")
    return numpy.pad(ff, [(lo, hi)], mode="constant")


def extract_mid(a, N):
    """Centre section of size N (synthesis.py:131-158)."""
    assert N <= a.shape[0]
    h, odd, cx = N // 2, N % 2, a.shape[0] // 2
    if a.ndim == 2:
        assert N <= a.shape[1]
        cy = a.shape[1] // 2
        return a[cx - h:cx + h + odd, cy - h:cy + h + odd]
    assert a.ndim == 1, "Unsupported grid shape for extract_mid!"
    return a[cx - h:cx + h + odd]


def extract_oversampled(a, Qpx, N):
    """Sub-kernels of an oversampled pattern (synthesis.py:160-197)."""
    Na = a.shape[0]
    start = Na // 2 - Qpx * (N // 2)
    if a.ndim == 1:
        return numpy.array([a[start + f:start + f + Qpx * N:Qpx] for f in range(Qpx)],
                           dtype=complex)
    assert a.ndim == 2, "Unsupported grid shape for extract_oversampled!"
    out = numpy.empty((Qpx, Qpx, N, N), dtype=complex)
    for fy in range(Qpx):
        for fx in range(Qpx):
            out[fy, fx] = a[start + fy:start + fy + Qpx * N:Qpx,
                            start + fx:start + fx + Qpx * N:Qpx]
    return out


# --------------------------------------------------------------------------
# kernels (synthesis.py:199-377, 682-734)

def anti_aliasing_function(shape, m, c):
    """Prolate spheroidal taper via scipy.special.pro_ang1 (synthesis.py:199-218).

    Host-side kernel preparation, as in the reference."""
    if numpy.ndim(shape) == 0:
        return scipy.special.pro_ang1(m, m, c, (2 - 1 / shape / 4) * coordinates(shape))[0]
    return numpy.outer(anti_aliasing_function(shape[0], m, c),
                       anti_aliasing_function(shape[1], m, c))


def kernel_transform(dl, dm):
    """2x2 transform keeping w-kernel coordinates stable under a shift (synthesis.py:220-248)."""
    dn = numpy.sqrt(1 - dl ** 2 - dm ** 2)
    f = (dn - 1) / (dl ** 2 + dm ** 2) if (dl != 0 or dm != 0) else 0
    return numpy.array([[dn - dm * dm * f, dl * dm * f],
                        [dl * dm * f, dn - dl * dl * f]])


def kernel_coordinates(N, theta, dl=0, dm=0, T=None):
    """(l, m) far-field coordinates, optionally transformed and shifted (synthesis.py:250-270)."""
    l, m = coordinates2(N) * theta
    if T is not None:
        l, m = T[0, 0] * l + T[1, 0] * m, T[0, 1] * l + T[1, 1] * m
    return l + dl, m + dm


def w_kernel_function(l, m, w):
    """Fresnel pattern exp(2 pi i w (1 - sqrt(1 - l^2 - m^2))) (synthesis.py:273-293)."""
    r2 = l ** 2 + m ** 2
    assert numpy.all(r2 < 1.0), "Error in image coordinate system: l %s, m %s" % (l, m)
    return numpy.exp(2j * numpy.pi * w * (1 - numpy.sqrt(1.0 - r2)))


def kernel_recentre(cp, theta, w, dl, dm):
    """Phase ramp re-centring a kernel in grid space (synthesis.py:296-311)."""
    l, m = coordinates2(cp.shape[0]) * theta
    return cp * numpy.exp(-2j * numpy.pi * w * (dl * l + dm * m))


def visibility_recentre(uvw, dl, dm):
    """Counterpart of kernel_recentre on visibility coordinates (synthesis.py:314-327)."""
    u, v, w = numpy.hsplit(uvw, 3)
    return numpy.hstack([u - w * dl, v - w * dm, w])


def invert_kernel(a):
    """Pseudo-inverse conj(a)/|a|^2 (synthesis.py:380-386; unused by the reference)."""
    return numpy.conj(a) / (numpy.abs(a) ** 2)


def kernel_oversample(ff, Qpx, s=None):
    """Oversampled convolution kernel from a far field, FP64 on the device (synthesis.py:330-354)."""
    dev = _is_dev(ff)
    ffa = ff if dev else numpy.asarray(ff)
    if ffa.ndim not in (1, 2):
        raise AssertionError("Unsupported grid shape for kernel_oversample!")
    out = E.kernel_oversample(ffa, int(Qpx), s, dtype=E.CD)
    return out if dev else _host(out)


def w_kernel(theta, w, NpixFF, NpixKern, Qpx, invert=True, **kwargs):
    """[Qpx, Qpx, S, S] w-kernel, FP64 phase + cuFFT on the device (synthesis.py:357-377)."""
    assert NpixFF > NpixKern or (NpixFF == NpixKern and Qpx == 1)
    out = E.w_kernels(theta, [w], NpixFF, NpixKern, Qpx, invert=invert,
                      dl=kwargs.get("dl", 0.0), dm=kwargs.get("dm", 0.0), T=kwargs.get("T"),
                      dtype=E.CD)
    return _host(out[0])


def w_conj_kernel_fn(kernel_fn):
    """Kernel function using K(-w) = conj(K(w)) (synthesis.py:682-699)."""
    def fn(theta, w, *args, **kw):
        if w < 0:
            return numpy.conj(kernel_fn(theta, -w, *args, **kw))
        return kernel_fn(theta, w, *args, **kw)
    return fn


class AWKernelFn:
    """The AW kernel function of aw_kernel_fn (synthesis.py:701-734): called with
    (theta, w, a1, a2, *src) it returns (A1 conv A2) conv W[yf, xf] for one key,
    computed on the device in FP64 as the reference does in complex128.

    w_cache_imaging / w_cache_predict / do_imaging / do_predict recognise it as
    their kernel_cache and, instead of one call per key, generate the kernels of
    every distinct key in one batched device pass (cg_aw_kernels): the A kernels
    once per distinct (antenna, *src) and the w kernels once per w bin, from the
    two callables given here.  Batched tables stay cached on the object (keyed by
    theta, the keys and the precision), as the reference's kernel cache keeps its
    kernels between calls."""

    def __init__(self, a_kernel_fn, w_kernel_fn, cache_size=2):
        self.a_kernel_fn, self.w_kernel_fn = a_kernel_fn, w_kernel_fn
        self.cache_size = cache_size
        self._tables = {}

    def __call__(self, theta, w, a1, a2, *src):
        A = numpy.array([self.a_kernel_fn(theta, a1, *src), self.a_kernel_fn(theta, a2, *src)])
        Wk = numpy.asarray(self.w_kernel_fn(theta, w))[None]
        one = numpy.zeros(1, dtype=numpy.int32)
        out = E.aw_kernels(A, Wk, one, one + 1, one, dtype=E.CD)
        return _host(out[0])

    def batch(self, theta, wbins, src_rows, dtype):
        """Device table [nk, Q, Q, SA, SA] of the kernels of keys (wbins[k],
        *src_rows[k]) with src_rows[k] = (a1, a2, *rest)."""
        key = (float(theta), numpy.asarray(wbins, numpy.float64).tobytes(),
               numpy.asarray(src_rows).tobytes(), dtype)
        if key in self._tables:
            t = self._tables.pop(key)
            self._tables[key] = t
            return t
        src_rows = numpy.asarray(src_rows)
        rest = [tuple(r[2:]) for r in src_rows]
        ants = {}
        ia = numpy.empty((len(src_rows), 2), dtype=numpy.int32)
        for k, r in enumerate(src_rows):
            for j in (0, 1):
                a = (r[j],) + rest[k]
                if a not in ants:
                    ants[a] = len(ants)
                ia[k, j] = ants[a]
        A = numpy.array([numpy.asarray(self.a_kernel_fn(theta, a[0], *a[1:]))
                         for a in ants])
        wu, wi = numpy.unique(numpy.asarray(wbins, numpy.float64), return_inverse=True)
        Wk = numpy.array([numpy.asarray(self.w_kernel_fn(theta, w)) for w in wu])
        t = E.aw_kernels(A, Wk, ia[:, 0], ia[:, 1], wi.astype(numpy.int32).ravel(), dtype=dtype)
        self._tables[key] = t
        while len(self._tables) > self.cache_size:
            self._tables.pop(next(iter(self._tables)))
        return t


def aw_kernel_fn(a_kernel_fn, w_kernel_fn=w_kernel):
    """AW kernel function: (A1 conv A2) conv W[yf, xf] on the device (synthesis.py:701-734)."""
    return AWKernelFn(a_kernel_fn, w_kernel_fn)


# --------------------------------------------------------------------------
# visibility coordinates (synthesis.py:419-449)

def frac_coord(N, Qpx, p):
    """Whole and fractional grid coordinate, bit-exact on the device (synthesis.py:419-435)."""
    scalar = numpy.ndim(p) == 0
    pa = numpy.atleast_1d(numpy.asarray(p, dtype=numpy.float64))
    uv = numpy.column_stack([pa, pa])
    st = E.Status()
    x, xf, _, _ = E.frac_coords(uv, 1.0, (N, N), Qpx, st)
    st.check()
    x, xf = _host(x), _host(xf)
    return (x[0], xf[0]) if scalar else (x.reshape(numpy.shape(p)), xf.reshape(numpy.shape(p)))


def frac_coords(shape, Qpx, p):
    """(x, xf, y, yf) with x over the width and y over the height (synthesis.py:438-449)."""
    st = E.Status()
    out = E.frac_coords(p, 1.0, shape, Qpx, st)
    st.check()
    return tuple(_host(o) for o in out)


# --------------------------------------------------------------------------
# boxcar gridding (synthesis.py:389-416)

def grid(a, p, v):
    """Boxcar gridding into a, in place, FP64 on the device (synthesis.py:389-401)."""
    st = E.Status()
    uvw = E.cuda_tensor(p, torch.float64)
    g = a if (_is_dev(a) and a.dtype == E.CD) else E.cuda_tensor(a, E.CD)
    E.grid_boxcar(uvw, 1.0, E.cuda_tensor(v, E.CD), g, st)
    st.check()
    if g is not a:
        if _is_dev(a):
            a.copy_(g)
        else:
            a[...] = g.cpu().numpy()


def degrid(a, p):
    """Boxcar degridding (synthesis.py:404-416)."""
    st = E.Status()
    out = E.degrid_boxcar(E.cuda_tensor(p, torch.float64), 1.0, E.cuda_tensor(a, E.CD), st)
    st.check()
    return _host(out, like=a)


# --------------------------------------------------------------------------
# convolutional gridding (synthesis.py:451-503)

def _table_and_groups(gcf, src, n, dtype):
    nsrc = _src_cols(src, n)
    ktab = E.KernelTable.from_gcf(gcf, nsrc, dtype)
    kidx = None
    if nsrc:
        s = src.cpu().numpy() if isinstance(src, torch.Tensor) else numpy.asarray(src)
        kidx = E.kernel_groups(tuple(gcf.shape[:nsrc]), s.reshape(n, nsrc), n)
    return ktab, kidx


def _grid_into(ktab, kidx, uvw, lam, shape, vis, prec, weight=None, out=None, status=None):
    """Grid on the device; returns the device grid (c64 or c128) and the plan (which
    also takes ``ktab`` when it was built for the table's even-support padding)."""
    mode = _lib.CG_PLAN_TILED if prec == "fp32" else _lib.CG_PLAN_GROUPS
    src = ktab
    if prec == "fp32":
        uvw = E.cuda_tensor(uvw, torch.float64)
        ktab = ktab.padded_even(uvw, lam, shape)  # same results, lane gridder
    plan = E.Plan(uvw, lam, shape, ktab, kidx, mode, status)
    if ktab is not src:
        plan.accept(src, ktab)
    if prec == "fp32":
        g = out if out is not None else torch.zeros(shape, dtype=E.CF, device="cuda")
        if weight is None:
            plan.grid(ktab, E.cuda_tensor(vis, E.CF), g)
        else:
            plan.grid_weighted(ktab, None if vis is None else E.cuda_tensor(vis, E.CF),
                               E.cuda_tensor(weight, torch.float32), g)
    else:
        g = out if out is not None else torch.zeros(shape, dtype=E.CD, device="cuda")
        v = E.cuda_tensor(vis, E.CD) if vis is not None else None
        if weight is not None:
            w = E.cuda_tensor(weight, torch.float64)
            v = w.to(E.CD) if v is None else v * w
        plan.grid_fp64(ktab, v, g)
    return g, plan


def _degrid_from(ktab, kidx, uvw, lam, guv, prec):
    mode = _lib.CG_PLAN_TILED if prec == "fp32" else _lib.CG_PLAN_GROUPS
    dt = E.CF if prec == "fp32" else E.CD
    g = E.cuda_tensor(guv, dt)
    if prec == "fp32":
        uvw = E.cuda_tensor(uvw, torch.float64)
        ktab = ktab.padded_even(uvw, lam, tuple(g.shape))  # same results, lane gridder
    plan = E.Plan(uvw, lam, tuple(g.shape), ktab, kidx, mode)
    out = plan.degrid(ktab, g) if prec == "fp32" else plan.degrid_fp64(ktab, g)
    plan.check()
    return out


def convgrid(gcf, a, p, src, v, precision=None):
    """Convolutional gridding into a, in place (synthesis.py:464-481)."""
    prec = _prec(precision)
    n = _nrows(p)
    ktab, kidx = _table_and_groups(gcf, src, n, E.CF if prec == "fp32" else E.CD)
    shape = tuple(a.shape)
    dev_inplace = _is_dev(a) and a.dtype == (E.CF if prec == "fp32" else E.CD)
    g, plan = _grid_into(ktab, kidx, p, 1.0, shape, v, prec, out=a if dev_inplace else None)
    plan.check()
    if not dev_inplace:
        if _is_dev(a):
            a += g.to(a.dtype)
        else:
            a += g.cpu().numpy()


def convdegrid(gcf, a, p, src=None, precision=None):
    """Convolutional degridding (synthesis.py:484-503)."""
    prec = _prec(precision)
    n = _nrows(p)
    ktab, kidx = _table_and_groups(gcf, src, n, E.CF if prec == "fp32" else E.CD)
    return _host(_degrid_from(ktab, kidx, p, 1.0, a, prec), like=a)


# --------------------------------------------------------------------------
# ordering and weighting (synthesis.py:506-549, 831-852)

def sort_vis_w(p, v=None):
    """Sort by w; stable order for ties (synthesis.py:506-515)."""
    zs = numpy.argsort(p[:, 2], kind="stable")
    return (p[zs], v[zs]) if v is not None else p[zs]


def slice_vis(step, uvw, v=None):
    """Chunks of at most step rows (synthesis.py:518-532)."""
    ii = range(0, len(uvw), step)
    if v is None:
        return [uvw[i:i + step] for i in ii]
    return [(uvw[i:i + step], v[i:i + step]) for i in ii]


def doweight(theta, lam, p, v):
    """Uniform re-weighting v / count(cell), counted on the device (synthesis.py:535-549)."""
    N = int(round(theta * lam))
    assert N > 1
    st = E.Status()
    uvw = E.cuda_tensor(p, torch.float64)
    vt = v if _is_dev(v) else numpy.asarray(v)
    if numpy.iscomplexobj(vt) if not _is_dev(vt) else vt.is_complex():
        w = E.weights(uvw, lam, N, st)
        st.check()
        out = E.cuda_tensor(vt, E.CD) * w
    else:
        out = E.weights(uvw, lam, N, st, E.cuda_tensor(vt, torch.float64))
        st.check()
    return _host(out, like=v)


def mirror_uvw(uvw, vis):
    """Flip baselines with v < 0 and conjugate their visibilities (synthesis.py:831-852)."""
    u = E.cuda_tensor(uvw, torch.float64).clone()
    cplx = torch.is_tensor(vis) and vis.is_complex() or (not torch.is_tensor(vis)
                                                        and numpy.iscomplexobj(vis))
    vt = E.cuda_tensor(vis, E.CD if not (_is_dev(vis) and vis.dtype == E.CF) else E.CF).clone() \
        if cplx else E.cuda_tensor(vis, torch.float64).clone()
    E.mirror_uvw(u, vt if cplx else None)
    if _is_dev(uvw):
        return u, vt
    return _host(u), _host(vt, dtype=numpy.asarray(vis).dtype)


def make_grid_hermitian(guv):
    """guv + conj(mirrored guv), in place, on the device (synthesis.py:855-880)."""
    if _is_dev(guv):
        return E.make_hermitian(guv)
    t = E.cuda_tensor(guv, E.CD)
    E.make_hermitian(t)
    guv[...] = t.cpu().numpy()
    return guv


# --------------------------------------------------------------------------
# kernel specifications of the imaging drivers
#
# A "spec" turns (uvw, src) into a device kernel table and per-visibility
# table rows.  All drivers share it, so imaging, PSF and predict on the same
# visibilities reuse one plan.

class _DeviceWKernels:
    """Device-resident w-kernel tables keyed by their parameters (LRU).

    Replaces pylru.FunctionCacheManager(w_kernel, size) of w_cache_imaging
    (synthesis.py:785-788) with whole tables generated in one batched pass."""

    def __init__(self, size=8):
        self.size = size
        self.tables = {}

    def get(self, theta, wstep, kmin, kmax, NpixFF, NpixKern, Qpx, invert, dl, dm, T, dtype):
        key = (float(theta), float(wstep), kmin, kmax, NpixFF, NpixKern, Qpx, bool(invert),
               float(dl), float(dm), None if T is None else numpy.asarray(T, float).tobytes(),
               dtype)
        if key in self.tables:
            t = self.tables.pop(key)
            self.tables[key] = t
            return t
        ws = wstep * numpy.arange(kmin, kmax + 1).astype(numpy.float64)
        t = E.w_kernels(theta, ws, NpixFF, NpixKern, Qpx, invert=invert, dl=dl, dm=dm, T=T,
                        dtype=dtype)
        self.tables[key] = t
        while len(self.tables) > self.size:
            self.tables.pop(next(iter(self.tables)))
        return t


W_KERNEL_TABLES = _DeviceWKernels()


def _is_w_kernel(fn):
    return fn is w_kernel


def _wkw(kwargs):
    kw = dict(kwargs)
    NpixFF, NpixKern, Qpx = kw.pop("NpixFF"), kw.pop("NpixKern"), kw.pop("Qpx")
    invert = kw.pop("invert", True)
    dl, dm, T = kw.pop("dl", 0.0), kw.pop("dm", 0.0), kw.pop("T", None)
    if kw:
        raise TypeError("unexpected w_kernel arguments %s" % sorted(kw))
    return NpixFF, NpixKern, Qpx, invert, dl, dm, T


def _spec_w_cache(theta, uvw_t, uvw_host, src, wstep, kernel_cache, kernel_fn, kwargs, dtype):
    n = uvw_t.shape[0]
    nsrc = _src_cols(src, n)
    if kernel_cache is None and _is_w_kernel(kernel_fn) and nsrc == 0:
        st = E.Status()
        kidx, kmin, kmax = E.w_bins(uvw_t, wstep, st)
        st.check()
        NpixFF, NpixKern, Qpx, invert, dl, dm, T = _wkw(kwargs)
        t = W_KERNEL_TABLES.get(theta, wstep, kmin, kmax, NpixFF, NpixKern, Qpx, invert, dl,
                                dm, T, dtype)
        return E.KernelTable(t.reshape(-1), False, Qpx, NpixKern), kidx
    fn = kernel_cache if kernel_cache is not None else kernel_fn
    dev = _device_keys(theta, uvw_t, src, nsrc, wstep, fn, kwargs, dtype)
    if dev is not None:
        return dev
    # Generic kernel callables are host functions: call each once per distinct
    # (wbin, *src_row) key, in first-use order, and upload the table.
    uh = uvw_host if uvw_host is not None else uvw_t.cpu().numpy()
    wbin = wstep * numpy.round(uh[:, 2] / wstep)
    s = numpy.zeros((n, 0)) if nsrc == 0 else numpy.asarray(
        src.cpu().numpy() if isinstance(src, torch.Tensor) else src).reshape(n, nsrc)
    keys = numpy.column_stack([wbin, s]) if nsrc else wbin[:, None]
    _, first, inv = numpy.unique(keys, axis=0, return_index=True, return_inverse=True)
    order = numpy.argsort(first)
    rank = numpy.empty_like(order)
    rank[order] = numpy.arange(len(order))
    kerns = [numpy.asarray(fn(theta, wbin[first[k]], *s[first[k]], **kwargs)) for k in order]
    table = numpy.array(kerns)
    Q, S = table.shape[1], table.shape[-1]
    return (E.KernelTable(E.cuda_tensor(table, dtype).reshape(-1), False, Q, S),
            rank[inv.ravel()].astype(numpy.int32))


def _int_columns(src, n, nsrc):
    """The src columns as an int32 [n, nsrc] device tensor with per-column minima
    and ranges (host int64 arrays), or None when a column is not integer-valued or
    the ranges are too wide for packed keys.  The integrality test and the column
    minima and maxima run on the device (on the host they took most of a 16M-row
    do_imaging call)."""
    if isinstance(src, torch.Tensor):
        t = src.reshape(n, nsrc)
        if t.dtype == torch.bool or t.dtype.is_complex:
            return None
    else:
        a = numpy.asarray(src).reshape(n, nsrc)
        if a.dtype.kind == "u":
            if a.dtype.itemsize == 8 and a.size and a.max() >= 2 ** 63:
                return None
            a = a.astype(numpy.int64)  # unsigned tensors have partial support in torch
        elif a.dtype.kind not in "if":
            return None
        t = torch.from_numpy(numpy.ascontiguousarray(a))
    t = t.to("cuda")
    if t.dtype.is_floating_point:
        if not bool(torch.isfinite(t).all()) or not bool((torch.floor(t) == t).all()):
            return None
    lo, hi = torch.aminmax(t, dim=0)
    lo, hi = lo.double().cpu().numpy(), hi.double().cpu().numpy()
    if numpy.any(lo < -2 ** 31) or numpy.any(hi >= 2 ** 31):
        return None
    lo, hi = lo.astype(numpy.int64), hi.astype(numpy.int64)
    return t.to(torch.int32), lo, hi - lo + 1


def _device_keys(theta, uvw_t, src, nsrc, wstep, fn, kwargs, dtype):
    """(ktab, kidx) with the distinct (wbin, *src_row) keys found on the device: the
    w bins and integer src columns packed into one key per visibility
    (cg_row_keys), compacted to the keys in use (cg_compact_keys); then one call
    of the kernel callable per distinct key, or, for an AWKernelFn, one batched
    generation of all of them.  None when the src columns are not integers or
    the key space is too large (the host path then handles the call)."""
    n = uvw_t.shape[0]
    if nsrc == 0 or n == 0:
        return None
    cols = _int_columns(src, n, nsrc)
    if cols is None:
        return None
    si, lo, rng = cols
    st = E.Status()
    _, kmin, kmax = E.w_bins(uvw_t, wstep, st)
    st.check()
    nb = kmax - kmin + 1
    space = int(nb) * int(numpy.prod(rng))
    if space >= 2 ** 31 - 1 or space > 64 * n + (1 << 24):
        return None
    key = E.row_keys(uvw_t, wstep, kmin, nb, si, lo, rng, st)
    rows, kor = E.compact_keys(key, space, st)
    st.check()
    kor = kor.cpu().numpy().astype(numpy.int64)
    digits = []
    r = kor
    for c in range(nsrc - 1, -1, -1):
        digits.append(r % rng[c] + lo[c])
        r = r // rng[c]
    wbins = wstep * (r + kmin).astype(numpy.float64)
    srow = numpy.column_stack(digits[::-1])
    if isinstance(fn, AWKernelFn) and nsrc >= 2 and not kwargs:
        t = fn.batch(theta, wbins, srow, dtype)
    else:
        t = E.cuda_tensor(numpy.array([numpy.asarray(fn(theta, wbins[k], *srow[k], **kwargs))
                                       for k in range(len(kor))]), dtype)
    Q, S = t.shape[1], t.shape[-1]
    return E.KernelTable(t.reshape(-1), False, Q, S), rows


def _spec_w_slice(theta, uvw_t, uvw_host, wstep, kernel_fn, kwargs, dtype):
    uh = uvw_host if uvw_host is not None else uvw_t.cpu().numpy()
    n = len(uh)
    order = numpy.argsort(uh[:, 2], kind="stable")
    nsl = (n + wstep - 1) // wstep
    means = numpy.array([numpy.mean(uh[order[i:i + wstep], 2]) for i in range(0, n, wstep)])
    kidx = numpy.empty(n, dtype=numpy.int32)
    kidx[order] = numpy.arange(n) // wstep
    if _is_w_kernel(kernel_fn):
        NpixFF, NpixKern, Qpx, invert, dl, dm, T = _wkw(kwargs)
        t = E.w_kernels(theta, means, NpixFF, NpixKern, Qpx, invert=invert, dl=dl, dm=dm, T=T,
                        dtype=dtype)
    else:
        t = E.cuda_tensor(numpy.array([numpy.asarray(kernel_fn(theta, w, **kwargs))
                                       for w in means]), dtype)
    assert t.shape[0] == nsl
    return E.KernelTable(t.reshape(-1), False, t.shape[1], t.shape[-1]), kidx


def _grid_size(theta, lam):
    N = int(round(theta * lam))
    assert N > 1
    return N


# --------------------------------------------------------------------------
# imaging / predict drivers (synthesis.py:552-679, 757-828, 883-927)

def simple_imaging(theta, lam, uvw, src, vis):
    """Boxcar imaging (synthesis.py:552-562)."""
    N = _grid_size(theta, lam)
    st = E.Status()
    g = torch.zeros((N, N), dtype=E.CD, device="cuda")
    E.grid_boxcar(E.cuda_tensor(uvw, torch.float64), lam, E.cuda_tensor(vis, E.CD), g, st)
    st.check()
    return _host(g, like=uvw)


def simple_predict(theta, lam, uvw, src, guv):
    """Boxcar predict (synthesis.py:565-580)."""
    _grid_size(theta, lam)
    st = E.Status()
    out = E.degrid_boxcar(E.cuda_tensor(uvw, torch.float64), lam, E.cuda_tensor(guv, E.CD), st)
    st.check()
    return _host(out, like=uvw)


def conv_imaging(theta, lam, uvw, src, vis, kv, precision=None):
    """Convolve and grid with a user kernel (synthesis.py:583-598)."""
    prec = _prec(precision)
    N = _grid_size(theta, lam)
    ktab, kidx = _table_and_groups(kv, src, _nrows(uvw), E.CF if prec == "fp32" else E.CD)
    g, plan = _grid_into(ktab, kidx, uvw, lam, (N, N), vis, prec)
    plan.check()
    return _host(g, like=uvw)


def conv_predict(theta, lam, uvw, src, guv, kv, precision=None):
    """Convolutional predict (synthesis.py:600-613)."""
    prec = _prec(precision)
    ktab, kidx = _table_and_groups(kv, src, _nrows(uvw), E.CF if prec == "fp32" else E.CD)
    return _host(_degrid_from(ktab, kidx, uvw, lam, guv, prec), like=uvw)


def w_slice_imaging(theta, lam, uvw, src, vis, wstep=2000, kernel_fn=w_kernel, precision=None,
                    **kwargs):
    """w-sliced imaging (synthesis.py:616-644), with the reference's undefined names
    (``p, v`` at :638) read as ``uvw, vis``.  All slices grid in one launch."""
    prec = _prec(precision)
    N = _grid_size(theta, lam)
    uh = None if _is_dev(uvw) else numpy.asarray(uvw)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    ktab, kidx = _spec_w_slice(theta, uvw_t, uh, wstep, kernel_fn, kwargs,
                               E.CF if prec == "fp32" else E.CD)
    g, plan = _grid_into(ktab, kidx, uvw_t, lam, (N, N), vis, prec)
    plan.check()
    return _host(g, like=uvw)


def w_slice_predict(theta, lam, uvw, src, guv, wstep=2000, kernel_fn=w_kernel, precision=None,
                    **kwargs):
    """w-sliced predict (synthesis.py:647-679), undefined ``p`` (:672) read as ``uvw``."""
    prec = _prec(precision)
    _grid_size(theta, lam)
    uh = None if _is_dev(uvw) else numpy.asarray(uvw)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    ktab, kidx = _spec_w_slice(theta, uvw_t, uh, wstep, kernel_fn, kwargs,
                               E.CF if prec == "fp32" else E.CD)
    return _host(_degrid_from(ktab, kidx, uvw_t, lam, guv, prec), like=uvw)


def w_cache_imaging(theta, lam, uvw, src, vis, wstep=2000, kernel_cache=None, kernel_fn=w_kernel,
                    precision=None, **kwargs):
    """w-projection with one kernel per w-bin (synthesis.py:757-796).

    With the default kernel function the bins are found and the kernels
    generated on the device, and every visibility grids in one persistent
    launch; other kernel callables are evaluated once per distinct key."""
    prec = _prec(precision)
    N = int(round(theta * lam))
    uh = None if _is_dev(uvw) else numpy.asarray(uvw)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    ktab, kidx = _spec_w_cache(theta, uvw_t, uh, src, wstep, kernel_cache, kernel_fn, kwargs,
                               E.CF if prec == "fp32" else E.CD)
    g, plan = _grid_into(ktab, kidx, uvw_t, lam, (N, N), vis, prec)
    plan.check()
    return _host(g, like=uvw)


def w_cache_predict(theta, lam, uvw, src, guv, wstep=2000, kernel_cache=None, kernel_fn=w_kernel,
                    precision=None, **kwargs):
    """w-projection predict (synthesis.py:799-828), with the reference's undefined
    ``nv``/``ixs`` (:823, :827) read as the number of rows and the row index."""
    prec = _prec(precision)
    uh = None if _is_dev(uvw) else numpy.asarray(uvw)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    ktab, kidx = _spec_w_cache(theta, uvw_t, uh, src, wstep, kernel_cache, kernel_fn, kwargs,
                               E.CF if prec == "fp32" else E.CD)
    return _host(_degrid_from(ktab, kidx, uvw_t, lam, guv, prec), like=uvw)


def _device_spec(imgfn, theta, uvw_t, uvw_host, src, kwargs, dtype):
    """(ktab, kidx) for one of this module's imaging/predict functions, or None."""
    n = uvw_t.shape[0]
    if imgfn in (conv_imaging, conv_predict):
        return _table_and_groups(kwargs["kv"], src, n, dtype)
    if imgfn in (w_cache_imaging, w_cache_predict):
        kw = dict(kwargs)
        wstep = kw.pop("wstep", 2000)
        cache = kw.pop("kernel_cache", None)
        fn = kw.pop("kernel_fn", w_kernel)
        return _spec_w_cache(theta, uvw_t, uvw_host, src, wstep, cache, fn, kw, dtype)
    if imgfn in (w_slice_imaging, w_slice_predict):
        kw = dict(kwargs)
        wstep = kw.pop("wstep", 2000)
        fn = kw.pop("kernel_fn", w_kernel)
        return _spec_w_slice(theta, uvw_t, uvw_host, wstep, fn, kw, dtype)
    return None


def do_imaging(theta, lam, uvw, src, vis, imgfn, **kwargs):
    """Dirty image and PSF (synthesis.py:883-911).

    For this module's imaging functions the whole chain runs on the device
    with one plan shared by the image and the PSF pass."""
    prec = _prec(kwargs.pop("precision", None))
    n = len(vis)
    if src is None:
        src = numpy.ndarray((n, 0))
    uvw_t = E.cuda_tensor(uvw, torch.float64).clone()
    cplx = E.CF if prec == "fp32" else E.CD
    vis_t = E.cuda_tensor(vis, E.CD).clone()
    E.mirror_uvw(uvw_t, vis_t)
    N = _grid_size(theta, lam)
    st = E.Status()
    wt = E.weights(uvw_t, lam, N, st)
    st.check()
    spec = None
    if imgfn is not simple_imaging:
        # (the host copy of the mirrored uvw is fetched only by the paths that need it)
        spec = _device_spec(imgfn, theta, uvw_t, None, src, kwargs, cplx)
    if spec is None and imgfn is not simple_imaging:
        # a caller-supplied imaging function: run it as the reference does
        uh = uvw_t.cpu().numpy()
        wh = wt.cpu().numpy()
        vh = vis_t.cpu().numpy()
        cdrt = numpy.asarray(imgfn(theta, lam, uh, src, wh * vh, **kwargs))
        c = numpy.asarray(imgfn(theta, lam, uh, src, wh, **kwargs))
        drt = numpy.real(ifft(make_grid_hermitian(cdrt)))
        psf = numpy.real(ifft(make_grid_hermitian(c)))
        pmax = psf.max()
        assert pmax > 0.0
        return drt / pmax, psf / pmax, pmax
    if imgfn is simple_imaging:
        g1 = torch.zeros((N, N), dtype=E.CD, device="cuda")
        g2 = torch.zeros((N, N), dtype=E.CD, device="cuda")
        E.grid_boxcar(uvw_t, lam, vis_t * wt, g1, st)
        E.grid_boxcar(uvw_t, lam, wt.to(E.CD), g2, st)
        st.check()
        if prec == "fp32":
            g1, g2 = g1.to(E.CF), g2.to(E.CF)
    else:
        ktab, kidx = spec
        g1, plan = _grid_into(ktab, kidx, uvw_t, lam, (N, N), vis_t, prec, weight=wt)
        g2, _ = _grid_into(ktab, kidx, uvw_t, lam, (N, N), None, prec, weight=wt) \
            if prec == "fp64" else (None, None)
        if prec == "fp32":
            g2 = torch.zeros((N, N), dtype=E.CF, device="cuda")
            plan.grid_weighted(ktab, None, wt.to(torch.float32), g2)
        plan.check()
    if prec == "fp32" and N % 2 == 0:
        img, _ = E.image_from_grid(g1)
        psf, pmax = E.image_from_grid(g2, want_max=True)
        pm = float(pmax.item())
        assert pm > 0.0
        E.scale_image(img, pmax)
        E.scale_image(psf, pmax)
        return img.double().cpu().numpy(), psf.double().cpu().numpy(), pm
    # complex128 (or odd-sized) images: hermitian + centred ifft + real part
    g1, g2 = g1.to(E.CD), g2.to(E.CD)
    for g in (g1, g2):
        E.make_hermitian(g)
        E.fft_(g, True)
    drt, psf = g1.real.cpu().numpy(), g2.real.cpu().numpy()
    pmax = psf.max()
    assert pmax > 0.0
    return drt / pmax, psf / pmax, pmax


def do_predict(theta, lam, uvw, src, modelimage, predfn, **kwargs):
    """Predict visibilities of a model image (synthesis.py:914-927)."""
    prec = _prec(kwargs.pop("precision", None))
    img = modelimage if _is_dev(modelimage) else numpy.asarray(modelimage)
    # the FP32 path transforms the model in complex64 (its degridding is FP32);
    # the boxcar and FP64 paths in complex128
    fp32_fft = prec == "fp32" and predfn in (conv_predict, w_cache_predict, w_slice_predict)
    ximage = E.cuda_tensor(img, E.CF if fp32_fft else E.CD)
    E.fft_(ximage, False)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    if predfn is simple_predict:
        st = E.Status()
        out = E.degrid_boxcar(uvw_t, lam, ximage, st)
        st.check()
        return _host(out, like=uvw)
    cplx = E.CF if prec == "fp32" else E.CD
    spec = _device_spec(predfn, theta, uvw_t, None if _is_dev(uvw) else numpy.asarray(uvw),
                        src, kwargs, cplx)
    if spec is None:
        return predfn(theta, lam, uvw, src, _host(ximage), **kwargs)
    ktab, kidx = spec
    return _host(_degrid_from(ktab, kidx, uvw_t, lam, ximage, prec), like=uvw)


def w_stack_imaging(theta, lam, uvw, src, vis, kv, plane, precision=None, per_plane=False,
                    gridder="auto"):
    """w-stacking (examples/notebooks/wstacking.ipynb, code cell 10, with conv_imaging in
    place of the notebook's boxcar gridding): for each w-plane p holding visibilities,
    ifft(grid_p) / w_kernel_function(l, m, mean w of the plane), summed; returns the
    complex image (the notebook shows 2 Re of it).  ``plane`` is each visibility's plane
    index.  All planes grid in one launch into a stack of grids and transform in one
    batched FFT; ``per_plane=True`` grids and transforms one plane per launch instead
    (the comparator).  ``gridder``: "tiled" (cg_grid), "sparse" (cg_grid_sparse, per-tap
    atomics) or "auto", sparse when the stack's tiles average fewer than 16 visibilities
    (4M visibilities over 32 planes of 4096^2: 1.4 ms sparse against 2.4 ms tiled).
    FP32 only."""
    if _prec(precision) != "fp32":
        raise ValueError("w_stack_imaging runs the FP32 tiled path only")
    N = _grid_size(theta, lam)
    n = _nrows(uvw)
    ptab = numpy.asarray(plane.cpu().numpy() if isinstance(plane, torch.Tensor) else plane)
    layers = int(ptab.max()) + 1 if n else 1
    ktab, kidx = _table_and_groups(kv, src, n, E.CF)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    vis_t = E.cuda_tensor(vis, E.CF)
    planes = torch.zeros((layers, N, N), dtype=E.CF, device="cuda")
    st = E.Status()
    if not per_plane:
        plan = E.Plan(uvw_t, lam, (N, N), ktab, kidx, status=st,
                      layers=(layers, ptab.astype(numpy.int32)))
        tiles = layers * (-(-N // plan.info()["tile"])) ** 2
        if gridder == "sparse" or (gridder == "auto" and n < 16 * tiles):
            plan.grid_sparse(ktab, vis_t, planes)
        elif gridder in ("auto", "tiled"):
            plan.grid(ktab, vis_t, planes)
        else:
            raise ValueError("gridder must be 'auto', 'tiled' or 'sparse'")
        mean_w, counts = plan.layer_mean_w()
        E.fft_(planes, True)
    else:
        mean_w = torch.zeros(layers, dtype=torch.float64, device="cuda")
        counts = torch.zeros(layers, dtype=torch.int32, device="cuda")
        for p in range(layers):
            sel = numpy.nonzero(ptab == p)[0]
            if len(sel) == 0:
                continue
            idx = torch.from_numpy(sel).cuda()
            sub = E.Plan(uvw_t[idx], lam, (N, N), ktab,
                         None if kidx is None else kidx[sel], status=st,
                         layers=(1, numpy.zeros(len(sel), numpy.int32)))
            sub.grid(ktab, vis_t[idx], planes[p])
            m, c = sub.layer_mean_w()
            mean_w[p], counts[p] = m[0], c[0]
            E.fft_(planes[p], True)
    image = E.wstack_combine(planes, theta, mean_w, counts, st)
    st.check()
    return _host(image, like=uvw)


def _tower_setup(theta, N, uvw_t, s, C, wincrement, st):
    """(chunk/plane-relative uvw, layer per visibility, used (chunk, plane) keys, plane
    of each layer, first layer of each chunk (+ end), sub-grid origin of each chunk)."""
    key, rel, (ubmin, ubmax, vbmin, vbmax, wpmin, wpmax) = E.tower_keys(uvw_t, theta, C,
                                                                        wincrement, st)
    st.check()
    nub, nvb, nwp = ubmax - ubmin + 1, vbmax - vbmin + 1, wpmax - wpmin + 1
    row, used = E.compact_keys(key, nub * nvb * nwp, st)
    used = used.cpu().numpy().astype(numpy.int64)
    plane = used % nwp + wpmin
    chunk, first = numpy.unique(used // nwp, return_index=True)
    chunk_first = numpy.append(first, len(used)).astype(numpy.int32)
    ub, vb = chunk % nub + ubmin, chunk // nub + vbmin
    xmid, ymid = (C * ub + C * (ub + 1)) // 2, (C * vb + C * (vb + 1)) // 2
    origin = numpy.column_stack([N // 2 + xmid - s // 2, N // 2 + ymid - s // 2])
    return rel, row, used, plane, chunk_first, origin.astype(numpy.int32)


def w_towers_imaging(theta, lam, uvw, src, vis, subgrid_size, margin, wincrement, wstep=2000,
                     kernel_cache=None, kernel_fn=w_kernel, precision=None, tile=32,
                     gridder="auto", **kwargs):
    """w-towers imaging: w-stacking on sub-grids (examples/grid/grid.c:482-710,
    examples/notebooks/wtowers.ipynb code cell 16).  Visibilities are binned into uv
    chunks of ``subgrid_size - margin`` cells and w-planes of width ``wincrement``;
    each (chunk, plane) is w-projected relative to the chunk centre and the plane's w
    with the kernels of w_cache_imaging (``wstep``, ``kernel_cache``/``kernel_fn``,
    ``**kwargs``) into a ``subgrid_size``^2 sub-grid, the planes of a chunk are moved to
    w = 0 in image space (division by w_kernel_function(l, m, w_plane)) and summed, and
    the chunk's sub-grid is added into the grid.  Returns the grid, the quantity
    w_cache_imaging returns.  All sub-grids grid in one launch and transform in batched
    FFTs (``tile``: the gridder's tile edge inside the sub-grids; ``gridder``: "tiled"
    (cg_grid), "sparse" (cg_grid_sparse, per-tap atomics) or "auto", sparse when the
    sub-grids average fewer than 16 visibilities per tile).  FP32 only; needs an even
    subgrid_size and margin >= the kernel support."""
    if _prec(precision) != "fp32":
        raise ValueError("w_towers_imaging runs the FP32 tiled path only")
    N = _grid_size(theta, lam)
    s, C = int(subgrid_size), int(subgrid_size) - int(margin)
    if C < 1 or margin < 0 or s % 2:
        raise ValueError("need an even subgrid_size and 0 <= margin < subgrid_size")
    n = _nrows(uvw)
    grid = torch.zeros((N, N), dtype=E.CF, device="cuda")
    if n == 0:
        return _host(grid, like=uvw)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    vis_t = E.cuda_tensor(vis, E.CF)
    st = E.Status()
    rel, row, used, plane, chunk_first, origin = _tower_setup(theta, N, uvw_t, s, C,
                                                              wincrement, st)
    ktab, kidx = _spec_w_cache(theta, rel, None, src, wstep, kernel_cache, kernel_fn, kwargs,
                               E.CF)
    stack = torch.zeros((len(used), s, s), dtype=E.CF, device="cuda")
    plan = E.Plan(rel, s / theta, (s, s), ktab, kidx, status=st, layers=(len(used), row),
                  tile=tile)
    tiles = len(used) * (-(-s // plan.info()["tile"])) ** 2
    if gridder == "sparse" or (gridder == "auto" and n < 16 * tiles):
        plan.grid_sparse(ktab, vis_t, stack)
    elif gridder in ("auto", "tiled"):
        plan.grid(ktab, vis_t, stack)
    else:
        raise ValueError("gridder must be 'auto', 'tiled' or 'sparse'")
    # unshifted transforms: the centring rolls, signs and 1/s^2 are folded into
    # the combine and add passes
    E.fft_raw(stack, True)
    sub = E.towers_combine(stack, theta, plane * float(wincrement), chunk_first, st)
    del stack
    E.fft_raw(sub, False)
    E.towers_add(sub, origin, grid)
    st.check()
    return _host(grid, like=uvw)


@functools.lru_cache(maxsize=8)
def _aw_towers_tables(N, s, aa_support, aa_over):
    """The anti-aliasing kernel table (kernel_oversample of the grid's PSWF, as the
    notebook's aa_gcf) and the correction of a cut layer image, aa_s x aa_s /
    aa_2s x aa_2s on the cut: built once per (grid, sub-grid, support, oversampling)."""
    aa = anti_aliasing_function(N, 0, aa_support)
    aa_s = anti_aliasing_function(s, 0, aa_support)
    aa_2s = anti_aliasing_function(2 * s, 0, aa_support)
    cut = aa_2s[s // 2:s // 2 + s]
    corr = E.cuda_tensor((numpy.outer(aa_s, aa_s) / numpy.outer(cut, cut)).astype(numpy.float32),
                         torch.float32)
    ktab = E.KernelTable.from_gcf(kernel_oversample(numpy.real(aa), aa_over, aa_support), 0,
                                  E.CF)
    return ktab, corr


def aw_towers_imaging(theta, lam, uvw, src, vis, subgrid_size, margin, wstep, aimage,
                      aa_support=6, aa_over=4096, precision=None, tile=32, gridder="auto",
                      method="auto"):
    """AW-towers imaging (examples/notebooks/awtowers.ipynb cells 17-22, without a
    phase-centre shift): visibilities binned into centred uv chunks of ``subgrid_size
    - margin`` cells (floor(u theta / C + 1/2)), w-planes of width ``wstep`` and
    baselines ``src[:, 0:2]`` (antenna indices into ``aimage``); each (chunk, plane,
    baseline) gridded with the anti-aliasing kernel (``aa_support``, oversampled
    ``aa_over`` times) relative to the chunk centre and the plane's w on a 2s x 2s grid
    at 2 theta; its image cut to s x s and corrected for the kernel, times
    aimage[a2] / aimage[a1]; each plane moved to w = 0 (divided by
    w_kernel_function(l, m, w_plane)); each chunk's FFT added into the grid.  Returns
    the grid; real(ifft(grid)) / aa x aa / sum(weights) is the notebook's image.  All
    layers grid in one launch and transform in batched FFTs.  FP32 only; needs even
    subgrid_size and margin, margin >= aa_support.

    method "direct" (the default for subgrid_size 16, 32 or 64) forms each layer's
    cut image straight from its visibilities (cg_awtowers_direct: the kernel is
    separable, so per visibility two s-point sums of its taps and an outer product)
    instead of gridding 2s x 2s layers and transforming them ("fft")."""
    if _prec(precision) != "fp32":
        raise ValueError("aw_towers_imaging runs the FP32 path only")
    N = int(numpy.ceil(theta * lam))
    s, C = int(subgrid_size), int(subgrid_size) - int(margin)
    if C < 1 or margin < aa_support or s % 2 or margin % 2:
        raise ValueError("need even subgrid_size and margin, aa_support <= margin < subgrid_size")
    if method not in ("auto", "direct", "fft"):
        raise ValueError("method must be 'auto', 'direct' or 'fft'")
    direct = method == "direct" or (method == "auto" and s in (16, 32, 64))
    if direct and s not in (16, 32, 64):
        raise ValueError("the direct AW-towers layers need subgrid_size 16, 32 or 64")
    grid = torch.zeros((N, N), dtype=E.CF, device="cuda")
    n = _nrows(uvw)
    if n == 0:
        return _host(grid, like=uvw)
    ai = numpy.asarray(aimage) if not _is_dev(aimage) else aimage
    nant = int(ai.shape[0])
    if tuple(ai.shape[1:]) != (s, s):
        raise ValueError("aimage must be [antennas, subgrid_size, subgrid_size]")
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    srcn = src if _is_dev(src) else numpy.asarray(src)
    a1 = E.cuda_tensor(srcn[:, 0], torch.int32)
    a2 = E.cuda_tensor(srcn[:, 1], torch.int32)
    vis_t = E.cuda_tensor(vis, E.CF)
    st = E.Status()
    key, rel, (ubmin, ubmax, vbmin, vbmax, wpmin, wpmax) = E.awtower_keys(
        uvw_t, theta, C, wstep, a1, a2, nant, st)
    st.check()
    nub, nvb, nwp = ubmax - ubmin + 1, vbmax - vbmin + 1, wpmax - wpmin + 1
    row, used = E.compact_keys(key, nub * nvb * nwp * nant * nant, st)
    # per layer its antennas and plane index, per chunk (a run of layers: used
    # ascends) its first layer and the notebook's sub-grid corner
    # xy_min = C (ub - 1/2) - (margin + 1) // 2, on the device
    la1, la2, lplane, chunk_first, origin = E.awtower_layers(used, nant, nwp, nub, ubmin,
                                                             vbmin, C, margin, N)
    plane_w = (numpy.arange(nwp) + wpmin) * float(wstep)
    ktab, corr = _aw_towers_tables(N, s, int(aa_support), int(aa_over))
    plan = E.Plan(rel, s / theta, (2 * s, 2 * s), ktab, None, status=st,
                  layers=(len(used), row), tile=tile)
    if direct:
        sub = E.awtowers_direct(plan, ktab, vis_t, s, theta, corr, ai, la1, la2, lplane,
                                plane_w, chunk_first, st)
        E.fft_raw(sub, False)
        E.towers_add(sub, origin, grid)
        st.check()
        return _host(grid, like=uvw)
    stack = torch.zeros((len(used), 2 * s, 2 * s), dtype=E.CF, device="cuda")
    tiles = len(used) * (-(-2 * s // plan.info()["tile"])) ** 2
    if gridder == "sparse" or (gridder == "auto" and n < 16 * tiles):
        plan.grid_sparse(ktab, vis_t, stack)
    elif gridder in ("auto", "tiled"):
        plan.grid(ktab, vis_t, stack)
    else:
        raise ValueError("gridder must be 'auto', 'tiled' or 'sparse'")
    E.fft_raw(stack, True)
    layer_w = E.cuda_tensor(plane_w, torch.float64)[lplane.long()]
    sub = E.awtowers_combine(stack, s, theta, corr, ai, la1, la2, layer_w, chunk_first, st)
    del stack
    E.fft_raw(sub, False)
    E.towers_add(sub, origin, grid)
    st.check()
    return _host(grid, like=uvw)


def w_towers_predict(theta, lam, uvw, src, guv, subgrid_size, margin, wincrement, wstep=2000,
                     kernel_cache=None, kernel_fn=w_kernel, precision=None, tile=32, **kwargs):
    """w-towers predict (examples/notebooks/wtowers-predict.ipynb), the reverse of
    w_towers_imaging: each chunk's sub-grid of ``guv`` goes to image space, each of the
    chunk's w-planes gets its image / w_kernel_function(l, m, w_plane) back in uv, and
    the visibilities are degridded from their plane's sub-grid with the residual-w
    kernels of w_cache_predict.  All sub-grids transform in batched FFTs and degrid in
    one launch.  Returns the visibilities.  FP32 only."""
    if _prec(precision) != "fp32":
        raise ValueError("w_towers_predict runs the FP32 tiled path only")
    s, C = int(subgrid_size), int(subgrid_size) - int(margin)
    if C < 1 or margin < 0 or s % 2:
        raise ValueError("need an even subgrid_size and 0 <= margin < subgrid_size")
    grid_t = E.cuda_tensor(guv, E.CF)
    N = grid_t.shape[-1]
    n = _nrows(uvw)
    if n == 0:
        return _host(torch.zeros(0, dtype=E.CF, device="cuda"), like=uvw)
    uvw_t = E.cuda_tensor(uvw, torch.float64)
    st = E.Status()
    rel, row, used, plane, chunk_first, origin = _tower_setup(theta, N, uvw_t, s, C,
                                                              wincrement, st)
    ktab, kidx = _spec_w_cache(theta, rel, None, src, wstep, kernel_cache, kernel_fn, kwargs,
                               E.CF)
    images = E.towers_cut(grid_t, origin, s)
    E.fft_raw(images, True)
    stack = E.towers_expand(images, theta, plane * float(wincrement), chunk_first, st)
    del images
    E.fft_raw(stack, False)
    plan = E.Plan(rel, s / theta, (s, s), ktab, kidx, status=st, layers=(len(used), row),
                  tile=tile)
    out = plan.degrid(ktab, stack)
    st.check()
    return _host(out, like=uvw)


def sample_image(image, x, y):
    """Bilinear sample relative to the image middle (synthesis.py:736-755)."""
    x = x + image.shape[0] / 2
    y = y + image.shape[1] / 2
    ix = numpy.floor(x).astype(int)
    dx = x - ix
    iy = numpy.floor(y).astype(int)
    dy = y - iy
    return numpy.sum([image[iy, ix] * ((1 - dx) * (1 - dy)),
                      image[iy, ix + 1] * (dx * (1 - dy)),
                      image[iy + 1, ix] * ((1 - dx) * dy),
                      image[iy + 1, ix + 1] * (dx * dy)], axis=0)
