"""CPU oracle of crocodile's convolutional gridding path -- TEST INFRASTRUCTURE ONLY.

A numpy (complex128) restatement of ``crocodile/synthesis.py`` written for
this project.  It is the parity checker for the CUDA product: only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import it.  The product never routes through it.

Parity pin: ``tests/golden/make_golden.py`` imports the real reference
(Python, importable in the build container) and stores its outputs as
``tests/golden/*.npz``; ``tests/test_oracle_golden.py`` checks every
function here against those fixtures and against the C golden table of
``examples/grid/test_recombine.c:378-412``.

Each function cites the reference lines whose behaviour it restates.  Three
reference functions are broken as shipped (NameError) and are restated with
the minimal fix, documented at each one: ``w_slice_imaging``,
``w_slice_predict``, ``w_cache_predict``.

Sections beyond synthesis.py, each pinned the same way: the Sze-Tan
gridder (crocodile/antialias.py; tests/golden/make_szetan.py), facet <->
subgrid recombination (examples/notebooks/facet-subgrid-impl.ipynb executed
by tests/golden/make_recombine.py; the raw-layout primitives of
examples/grid/recombine.c are tied to it by tests/test_recombine_cpu.py),
visibility ingest (scripts/image_dataset.py's collect_blocks run with arl's
Visibility by tests/golden/make_ingest.py), and w-towers (pinned by
reduction to w_cache_imaging).

Vectorisation note: ``convgrid`` here adds the S x S footprints with
``numpy.add.at`` in visibility order, which performs exactly the same
sequence of complex128 additions per grid cell as the reference's per-row
Python loop (``synthesis.py:479-481``), so grids agree bit for bit.
"""

import numpy
import scipy.special
import scipy.signal


# --------------------------------------------------------------------------
# coordinates and FFT conventions (synthesis.py:38-106)

def coordinateBounds(N):
    """Lowest/highest coordinate of an N grid (synthesis.py:38-55)."""
    if N % 2 == 0:
        return -0.5, 0.5 * (N - 2) / N
    return -0.5 * (N - 1) / N, 0.5 * (N - 1) / N


def coordinates(N):
    """1-D coordinates, zero at N//2, step 1/N (synthesis.py:57-63)."""
    lo = -(N // 2)
    return numpy.arange(lo, lo + N) / N


def coordinates2(N):
    """(x, y) 2-D coordinate grids, x varying along axis 1 (synthesis.py:66-80)."""
    c = numpy.arange(-(N // 2), -(N // 2) + N)
    cy, cx = numpy.meshgrid(c, c, indexing="ij")
    return numpy.array([cx, cy]) / N


def fft(a):
    """Centred forward FFT: fftshift(fft(ifftshift(a))) (synthesis.py:83-93)."""
    if a.ndim == 1:
        return numpy.fft.fftshift(numpy.fft.fft(numpy.fft.ifftshift(a)))
    assert a.ndim == 2, "Unsupported image shape for FFT!"
    return numpy.fft.fftshift(numpy.fft.fft2(numpy.fft.ifftshift(a)))


def ifft(a):
    """Centred inverse FFT incl. 1/N normalisation (synthesis.py:96-106)."""
    if a.ndim == 1:
        return numpy.fft.fftshift(numpy.fft.ifft(numpy.fft.ifftshift(a)))
    assert a.ndim == 2, "Unsupported grid shape for iFFT!"
    return numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.ifftshift(a)))


# --------------------------------------------------------------------------
# padding / extraction (synthesis.py:109-197)

def pad_mid(ff, N):
    """Zero-pad a far field to N (per axis) around N//2 (synthesis.py:109-129)."""
    N0 = ff.shape[0]
    if N == N0:
        return ff
    assert N > N0
    before = N // 2 - N0 // 2
    after = (N + 1) // 2 - (N0 + 1) // 2
    if ff.ndim == 2:
        assert ff.shape[1] == N0
        return numpy.pad(ff, [(before, after)] * 2, mode="constant")
    return numpy.pad(ff, [(before, after)], mode="constant")


def extract_mid(a, N):
    """Centre crop of size N around shape//2 (synthesis.py:131-158)."""
    assert N <= a.shape[0]
    h = N // 2
    odd = N % 2
    cx = a.shape[0] // 2
    if a.ndim == 2:
        assert N <= a.shape[1]
        cy = a.shape[1] // 2
        return a[cx - h:cx + h + odd, cy - h:cy + h + odd]
    assert a.ndim == 1, "Unsupported grid shape for extract_mid!"
    return a[cx - h:cx + h + odd]


def extract_oversampled(a, Qpx, N):
    """Every Qpx-th sample from offset Na//2 - Qpx*(N//2) + f (synthesis.py:160-197)."""
    Na = a.shape[0]
    base = Na // 2 - Qpx * (N // 2)
    taps = Qpx * numpy.arange(N)
    if a.ndim == 1:
        out = numpy.empty((Qpx, N), dtype=complex)
        for f in range(Qpx):
            out[f] = a[base + f + taps]
        return out
    assert a.ndim == 2, "Unsupported grid shape for extract_oversampled!"
    out = numpy.empty((Qpx, Qpx, N, N), dtype=complex)
    for fy in range(Qpx):
        rows = base + fy + taps
        for fx in range(Qpx):
            cols = base + fx + taps
            out[fy, fx] = a[numpy.ix_(rows, cols)]
    return out


# --------------------------------------------------------------------------
# kernels (synthesis.py:199-377, 682-734)

def anti_aliasing_function(shape, m, c):
    """PSWF pro_ang1(m, m, c, (2 - 1/N/4) * coordinates(N)) (synthesis.py:199-218)."""
    if numpy.ndim(shape) == 0:
        mult = 2 - 1 / shape / 4
        return scipy.special.pro_ang1(m, m, c, mult * coordinates(shape))[0]
    return numpy.outer(anti_aliasing_function(shape[0], m, c),
                       anti_aliasing_function(shape[1], m, c))


def kernel_coordinates(N, theta, dl=0, dm=0, T=None):
    """(l, m) of an N far field, optionally transformed by T and shifted (synthesis.py:250-270)."""
    l, m = coordinates2(N) * theta
    if T is not None:
        l, m = T[0, 0] * l + T[1, 0] * m, T[0, 1] * l + T[1, 1] * m
    return l + dl, m + dm


def w_kernel_function(l, m, w):
    """Fresnel pattern exp(2 pi i w (1 - sqrt(1 - l^2 - m^2))) (synthesis.py:273-293)."""
    r2 = l ** 2 + m ** 2
    assert numpy.all(r2 < 1.0), "Error in image coordinate system"
    ph = 1 - numpy.sqrt(1.0 - r2)
    return numpy.exp(2j * numpy.pi * w * ph)


def kernel_oversample(ff, Qpx, s=None):
    """Oversampled GCF: extract_oversampled(fft(pad_mid(ff, N*Qpx)), Qpx, s) (synthesis.py:330-354)."""
    N = ff.shape[0]
    if s is None:
        s = N
    return extract_oversampled(fft(pad_mid(ff, N * Qpx)), Qpx, s)


def w_kernel(theta, w, NpixFF, NpixKern, Qpx, invert=True, **kwargs):
    """[Qpx,Qpx,S,S] w-kernel, inverted for imaging by default (synthesis.py:357-377)."""
    assert NpixFF > NpixKern or (NpixFF == NpixKern and Qpx == 1)
    l, m = kernel_coordinates(NpixFF, theta, **kwargs)
    kern = w_kernel_function(l, m, w)
    if invert:
        kern = 1 / kern
    return kernel_oversample(kern, Qpx, NpixKern)


def w_conj_kernel_fn(kernel_fn):
    """K(-w) = conj(K(w)) wrapper (synthesis.py:682-699)."""
    def fn(theta, w, *args, **kw):
        if w < 0:
            return numpy.conj(kernel_fn(theta, -w, *args, **kw))
        return kernel_fn(theta, w, *args, **kw)
    return fn


def aw_kernel_fn(a_kernel_fn, w_kernel_fn=w_kernel):
    """AW kernel = (A1 conv A2) conv W[yf,xf], 'same' crops (synthesis.py:701-734)."""
    def fn(theta, w, a1, a2, *src):
        akern = scipy.signal.convolve2d(a_kernel_fn(theta, a1, *src),
                                        a_kernel_fn(theta, a2, *src), mode="same")
        wkern = w_kernel_fn(theta, w)
        return numpy.array([[scipy.signal.convolve2d(akern, wk, mode="same")
                             for wk in row] for row in wkern])
    return fn


def aw_kernel_fft(akern_a, akern_b, wkern):
    """aw_kernel_fn's result for one key, computed with scipy.signal.fftconvolve
    batched over the Q x Q sub-kernels (same 'same' crops as convolve2d, equal to
    aw_kernel_fn to rounding).  Used to prepare large CPU-baseline kernel tables;
    tests/test_oracle_golden.py pins it against aw_kernel_fn."""
    akern = scipy.signal.convolve2d(akern_a, akern_b, mode="same")
    akern = numpy.broadcast_to(akern, wkern.shape[:-2] + akern.shape)
    return scipy.signal.fftconvolve(akern, wkern, mode="same", axes=(-2, -1))


# --------------------------------------------------------------------------
# coordinates of visibilities (synthesis.py:419-449)

def frac_coord(N, Qpx, p):
    """Whole and fractional (1/Qpx) grid coordinate, banker's rounding (synthesis.py:419-435)."""
    p = numpy.asarray(p)
    assert (p >= -0.5).all() and (p < 0.5).all()
    x = N // 2 + p * N
    fx = numpy.around(-x * Qpx).astype(int)
    return -(fx // Qpx), fx % Qpx


def frac_coords(shape, Qpx, p):
    """x from p[:,0] over the width, y from p[:,1] over the height (synthesis.py:438-449)."""
    h, w = shape
    x, xf = frac_coord(w, Qpx, p[:, 0])
    y, yf = frac_coord(h, Qpx, p[:, 1])
    return x, xf, y, yf


# --------------------------------------------------------------------------
# boxcar gridding (synthesis.py:389-416)

def grid(a, p, v):
    """Nearest-cell gridding N//2 + floor(0.5 + N p) (synthesis.py:389-401)."""
    assert numpy.max(p) < 0.5
    N = a.shape[0]
    xy = N // 2 + numpy.floor(0.5 + N * p[:, 0:2]).astype(int)
    numpy.add.at(a, (xy[:, 1], xy[:, 0]), v)


def degrid(a, p):
    """Nearest-cell degridding (synthesis.py:404-416)."""
    assert numpy.max(p) < 0.5
    N = a.shape[0]
    xy = N // 2 + numpy.floor(0.5 + p[:, 0:2] * N).astype(int)
    return a[xy[:, 1], xy[:, 0]]


# --------------------------------------------------------------------------
# convolutional gridding (synthesis.py:451-503)

def gcf_layout(gcf, nsrc):
    """(separable?, Qpx, S) from the kernel rank vs the src columns (synthesis.py:451-461)."""
    extra = gcf.ndim - nsrc
    if extra == 2:
        return True, gcf.shape[-2], gcf.shape[-1]
    if extra == 4:
        assert gcf.shape[-1] == gcf.shape[-2], "non-square kernels are not supported"
        return False, gcf.shape[-3], gcf.shape[-1]
    raise AssertionError("kernel rank does not match the src columns")


def kernel_groups(gcf, src, n):
    """Flat kernel-group index of each row of src into gcf's leading dims."""
    src = numpy.zeros((n, 0)) if src is None else numpy.asarray(src)
    lead = gcf.shape[:src.shape[1]]
    if src.shape[1] == 0:
        return src, numpy.zeros(n, dtype=numpy.int64)
    idx = src.astype(numpy.int64)
    for k, d in enumerate(lead):
        col = idx[:, k]
        if ((col < -d) | (col >= d)).any():
            raise IndexError("src column %d out of range for kernel dimension %d" % (k, d))
        idx[:, k] = numpy.where(col < 0, col + d, col)
    return src, numpy.ravel_multi_index(tuple(idx.T), lead)


def _footprints(shape, S, x, y):
    x0 = x - S // 2
    y0 = y - S // 2
    bad = (x0 < 0) | (y0 < 0) | (x0 + S > shape[1]) | (y0 + S > shape[0])
    if bad.any():
        raise ValueError("%d visibilities have footprints outside the %dx%d grid"
                         % (int(bad.sum()), shape[0], shape[1]))
    return x0, y0


def _kernel_block(kt, sep, g, xf, yf):
    if sep:
        return kt[g, yf][:, :, None] * kt[g, xf][:, None, :]
    return kt[g, yf, xf]


def convgrid_indexed(kt, sep, a, x, xf, y, yf, g, v, chunk=1 << 14):
    """a[y-S//2 : y+(S+1)//2, x-S//2 : x+(S+1)//2] += K[g,yf,xf] * v, in visibility order.

    kt is the kernel table flattened to [G, Q, (Q,) S(, S)].  Restates the
    loop of synthesis.py:479-481.
    """
    S = kt.shape[-1]
    x0, y0 = _footprints(a.shape, S, x, y)
    taps = numpy.arange(S)
    for s in range(0, len(x), chunk):
        e = s + chunk
        vals = _kernel_block(kt, sep, g[s:e], xf[s:e], yf[s:e]) * v[s:e, None, None]
        iy = y0[s:e, None, None] + taps[None, :, None]
        ix = x0[s:e, None, None] + taps[None, None, :]
        numpy.add.at(a, (iy, ix), vals)


def convdegrid_indexed(kt, sep, a, x, xf, y, yf, g, chunk=1 << 14):
    """sum(a[footprint] * K[g,yf,xf]) per visibility (restates synthesis.py:500-503)."""
    S = kt.shape[-1]
    x0, y0 = _footprints(a.shape, S, x, y)
    taps = numpy.arange(S)
    out = numpy.empty(len(x), dtype=complex)
    for s in range(0, len(x), chunk):
        e = s + chunk
        iy = y0[s:e, None, None] + taps[None, :, None]
        ix = x0[s:e, None, None] + taps[None, None, :]
        prod = a[iy, ix] * _kernel_block(kt, sep, g[s:e], xf[s:e], yf[s:e])
        out[s:e] = prod.reshape(prod.shape[0], -1).sum(axis=1)
    return out


def _flat_table(gcf, nsrc):
    sep, Q, S = gcf_layout(gcf, nsrc)
    tail = (Q, S) if sep else (Q, Q, S, S)
    return gcf.reshape((-1,) + tail), sep, Q


def convgrid(gcf, a, p, src, v):
    """Convolutional gridding into a, in place (synthesis.py:464-481)."""
    n = p.shape[0]
    src, g = kernel_groups(gcf, src, n)
    kt, sep, Q = _flat_table(gcf, src.shape[1])
    x, xf, y, yf = frac_coords(a.shape, Q, p)
    convgrid_indexed(kt, sep, a, x, xf, y, yf, g, numpy.asarray(v))


def convdegrid(gcf, a, p, src=None):
    """Convolutional degridding (synthesis.py:484-503)."""
    n = p.shape[0]
    src, g = kernel_groups(gcf, src, n)
    kt, sep, Q = _flat_table(gcf, src.shape[1])
    x, xf, y, yf = frac_coords(a.shape, Q, p)
    return convdegrid_indexed(kt, sep, a, x, xf, y, yf, g)


# --------------------------------------------------------------------------
# ordering and weighting (synthesis.py:506-549, 831-852)

def sort_vis_w(p, v=None):
    """Order by w (stable argsort; the reference's default sort ties arbitrarily) (synthesis.py:506-515)."""
    zs = numpy.argsort(p[:, 2], kind="stable")
    return (p[zs], v[zs]) if v is not None else p[zs]


def slice_vis(step, uvw, v=None):
    """Fixed-size chunks (synthesis.py:518-532)."""
    starts = range(0, len(uvw), step)
    if v is None:
        return [uvw[i:i + step] for i in starts]
    return [(uvw[i:i + step], v[i:i + step]) for i in starts]


def doweight(theta, lam, p, v):
    """Uniform weighting: v / count(cell) on an N = round(theta*lam) grid (synthesis.py:535-549)."""
    N = int(round(theta * lam))
    assert N > 1
    x, _, y, _ = frac_coords((N, N), 1, p / lam)
    if ((x >= N) | (y >= N)).any():
        raise IndexError("visibility falls outside the weighting grid")
    counts = numpy.zeros((N, N))
    numpy.add.at(counts, (x, y), 1)
    return v / counts[x, y]


def mirror_uvw(uvw, vis):
    """Flip rows with v < 0 to (-uvw, conj(vis)) (synthesis.py:831-852)."""
    flip = uvw[:, 1] < 0
    uvw = numpy.copy(uvw)
    vis = numpy.copy(vis)
    uvw[flip] = -uvw[flip]
    vis[flip] = numpy.conj(vis[flip])
    return uvw, vis


def make_grid_hermitian(guv):
    """guv + conj(mirror(guv)), mirrored on the zero point (synthesis.py:855-880).

    Out-of-place right-hand side, as numpy buffers the overlapping operands
    of the reference's in-place update."""
    if guv.shape[0] % 2 == 0:
        guv[1:, 1:] += numpy.conj(guv[:0:-1, :0:-1]).copy()
    else:
        guv += numpy.conj(guv[::-1, ::-1]).copy()
    return guv


# --------------------------------------------------------------------------
# imaging / predict drivers (synthesis.py:552-679, 757-828, 883-927)

def grid_size(theta, lam):
    N = int(round(theta * lam))
    assert N > 1
    return N


def simple_imaging(theta, lam, uvw, src, vis):
    """Boxcar imaging (synthesis.py:552-562)."""
    N = grid_size(theta, lam)
    guv = numpy.zeros([N, N], dtype=complex)
    grid(guv, uvw / lam, vis)
    return guv


def simple_predict(theta, lam, uvw, src, guv):
    """Boxcar predict (synthesis.py:565-580)."""
    grid_size(theta, lam)
    return degrid(guv, uvw / lam)


def conv_imaging(theta, lam, uvw, src, vis, kv):
    """Convolutional imaging (synthesis.py:583-598)."""
    N = grid_size(theta, lam)
    guv = numpy.zeros([N, N], dtype=complex)
    convgrid(kv, guv, uvw / lam, src, vis)
    return guv


def conv_predict(theta, lam, uvw, src, guv, kv):
    """Convolutional predict (synthesis.py:600-613)."""
    return convdegrid(kv, guv, uvw / lam, src)


def w_slice_imaging(theta, lam, uvw, src, vis, wstep=2000, kernel_fn=w_kernel, **kwargs):
    """w-sliced imaging (synthesis.py:616-644).

    Minimal fix: the reference sorts undefined names ``p, v`` (:638); this
    sorts ``uvw, vis``.  ``src`` is ignored per slice as in the reference's
    kernel call (``kernel_fn(theta, w, **kwargs)``, :642) and convgrid gets
    ``None`` (the reference passes the full ``src``, which only works when it
    has no columns)."""
    N = grid_size(theta, lam)
    guv = numpy.zeros([N, N], dtype=complex)
    for ps, vs in slice_vis(wstep, *sort_vis_w(uvw, vis)):
        wg = kernel_fn(theta, numpy.mean(ps[:, 2]), **kwargs)
        convgrid(wg, guv, ps / lam, None, vs)
    return guv


def w_slice_predict(theta, lam, uvw, src, guv, wstep=2000, kernel_fn=w_kernel, **kwargs):
    """w-sliced predict (synthesis.py:647-679).  Minimal fix: ``p`` -> ``uvw`` (:672-673)."""
    grid_size(theta, lam)
    nv = len(uvw)
    v = numpy.ndarray(nv, dtype=complex)
    for ps, ixs in slice_vis(wstep, *sort_vis_w(uvw, numpy.arange(nv))):
        wg = kernel_fn(theta, numpy.mean(ps[:, 2]), **kwargs)
        v[ixs] = convdegrid(wg, guv, ps / lam)
    return v


def _w_cache_table(theta, uvw, src, wstep, kernel_cache, kernel_fn, kwargs):
    """Kernel table over the distinct (wbin, *src_row) keys, in first-use order,
    and the per-visibility table index.  wbin = wstep * round(w / wstep)
    (synthesis.py:793)."""
    if kernel_cache is None:
        kernel_cache = kernel_fn
    src = numpy.zeros((len(uvw), 0)) if src is None else numpy.asarray(src)
    wbin = wstep * numpy.round(uvw[:, 2] / wstep)
    keys = numpy.column_stack([wbin, src]) if src.shape[1] else wbin[:, None]
    uniq, first, inv = numpy.unique(keys, axis=0, return_index=True, return_inverse=True)
    order = numpy.argsort(first)
    rank = numpy.empty_like(order)
    rank[order] = numpy.arange(len(order))
    kerns = []
    for k in order:
        i = first[k]
        kerns.append(numpy.asarray(kernel_cache(theta, wbin[i], *src[i], **kwargs)))
    return numpy.array(kerns), rank[inv.ravel()]


def w_cache_imaging(theta, lam, uvw, src, vis, wstep=2000, kernel_cache=None,
                    kernel_fn=w_kernel, **kwargs):
    """w-projection with one kernel per w-bin (and src key) (synthesis.py:757-796).

    The reference grids one visibility at a time; here the kernels of all
    keys are gathered first and one convgrid pass runs in visibility order,
    which performs the same additions in the same order."""
    N = int(round(theta * lam))
    guv = numpy.zeros([N, N], dtype=complex)
    kt, g = _w_cache_table(theta, uvw, src, wstep, kernel_cache, kernel_fn, kwargs)
    Q = kt.shape[1]
    x, xf, y, yf = frac_coords(guv.shape, Q, uvw / lam)
    convgrid_indexed(kt, False, guv, x, xf, y, yf, g, numpy.asarray(vis))
    return guv


def w_cache_predict(theta, lam, uvw, src, guv, wstep=2000, kernel_cache=None,
                    kernel_fn=w_kernel, **kwargs):
    """w-projection predict (synthesis.py:799-828).

    Minimal fix: the reference uses undefined ``nv`` (:823) and ``ixs``
    (:827); this sizes the output by ``len(uvw)`` and writes row i."""
    kt, g = _w_cache_table(theta, uvw, src, wstep, kernel_cache, kernel_fn, kwargs)
    Q = kt.shape[1]
    x, xf, y, yf = frac_coords(guv.shape, Q, uvw / lam)
    return convdegrid_indexed(kt, False, guv, x, xf, y, yf, g)


def do_imaging(theta, lam, uvw, src, vis, imgfn, **kwargs):
    """Mirror, weight, grid, hermitian, FFT; PSF likewise; normalise (synthesis.py:883-911)."""
    if src is None:
        src = numpy.ndarray((len(vis), 0))
    uvw, vis = mirror_uvw(uvw, vis)
    wt = doweight(theta, lam, uvw, numpy.ones(len(uvw)))
    cdrt = imgfn(theta, lam, uvw, src, wt * vis, **kwargs)
    drt = numpy.real(ifft(make_grid_hermitian(cdrt)))
    c = imgfn(theta, lam, uvw, src, wt, **kwargs)
    psf = numpy.real(ifft(make_grid_hermitian(c)))
    pmax = psf.max()
    assert pmax > 0.0
    return drt / pmax, psf / pmax, pmax


def do_predict(theta, lam, uvw, src, modelimage, predfn, **kwargs):
    """FFT of the model image, then predfn (synthesis.py:914-927)."""
    return predfn(theta, lam, uvw, src, fft(modelimage.astype(complex)), **kwargs)


# --------------------------------------------------------------------------
# w-stacking (examples/notebooks/wstacking.ipynb, code cell 10), with
# convolutional gridding in place of the notebook's boxcar gridding.

def w_stack_imaging(theta, lam, uvw, src, vis, kv, plane):
    """Sum over planes of ifft(conv_imaging(plane vis)) / w_kernel_function(l, m, mean w).

    ``plane`` is each visibility's w-plane index; w-planes without
    visibilities are skipped, as in the notebook."""
    N = grid_size(theta, lam)
    l, m = theta * coordinates2(N)
    image = numpy.zeros((N, N), dtype=complex)
    src = numpy.zeros((len(uvw), 0)) if src is None else src
    for wp in numpy.unique(plane):
        sel = plane == wp
        midw = numpy.mean(uvw[sel, 2])
        g = conv_imaging(theta, lam, uvw[sel], src[sel], vis[sel], kv)
        image += ifft(g) / w_kernel_function(l, m, midw)
    return image


# --------------------------------------------------------------------------
# w-towers: w-stacking on sub-grids (examples/grid/grid.c:482-710,
# examples/notebooks/wtowers.ipynb code cell 16), in crocodile's Python
# conventions.  Neither reference form runs here (the C prototype needs
# FFTW/HDF5 headers; the notebook grids nearest-cell with no last-mile
# kernel), so this restatement defines the algorithm the GPU path matches:
#
#   chunk (ub, vb) = floor(u*theta / C), floor(v*theta / C)   C = subgrid - margin
#   plane wp = around(w / wincrement)                            (notebook cell 16)
#   chunk centre xmid = (C*ub + C*(ub+1)) // 2 cells, u_mid = xmid / theta
#   per (chunk, plane): w_cache_imaging of the visibilities relative to
#       (u_mid, v_mid, wp*wincrement) into an s x s sub-grid (lam_sub = s / theta),
#       i.e. the last mile w-projected with w-kernels of the residual w (grid.c:277-305)
#   per chunk: image = sum over planes of ifft(sub-grid) / w_kernel_function(l, m, wp*wincrement)
#       on the sub-grid's l, m (the Fresnel transfer of grid.c:418-480, 598-622 in closed form)
#   grid[N//2 + ymid - s//2 + i, N//2 + xmid - s//2 + j] += fft(image)[i, j], cells
#       outside the grid dropped (grid.c:640-656)
#
# With one plane and every |w| < wincrement / 2 this is w_cache_imaging itself
# (fft(ifft(x)) = x), which pins it to the reference (tests/test_oracle_golden.py).

def tower_bins(theta, uvw, subgrid_size, margin, wincrement):
    """(ub, vb, wp, xmid, ymid, uvw_rel) of every visibility."""
    C = subgrid_size - margin
    ub = numpy.floor(uvw[:, 0] * theta / C).astype(numpy.int64)
    vb = numpy.floor(uvw[:, 1] * theta / C).astype(numpy.int64)
    wp = numpy.around(uvw[:, 2] / wincrement)
    xmid = (C * ub + C * (ub + 1)) // 2
    ymid = (C * vb + C * (vb + 1)) // 2
    rel = numpy.column_stack([uvw[:, 0] - xmid / theta, uvw[:, 1] - ymid / theta,
                              uvw[:, 2] - wp * wincrement])
    return ub, vb, wp.astype(numpy.int64), xmid, ymid, rel


def w_towers_imaging(theta, lam, uvw, src, vis, subgrid_size, margin, wincrement, wstep,
                     kernel_fn=w_kernel, **kwargs):
    """w-towers imaging: returns the N x N grid (the same quantity as w_cache_imaging)."""
    N = int(round(theta * lam))
    s = subgrid_size
    guv = numpy.zeros((N, N), dtype=complex)
    src = numpy.zeros((len(uvw), 0)) if src is None else src
    ub, vb, wp, xmid, ymid, rel = tower_bins(theta, uvw, s, margin, wincrement)
    l, m = theta * coordinates2(s)
    chunks = sorted(set(zip(vb.tolist(), ub.tolist())))
    for cv, cu in chunks:
        in_chunk = (vb == cv) & (ub == cu)
        image = numpy.zeros((s, s), dtype=complex)
        for p in numpy.unique(wp[in_chunk]):
            sel = in_chunk & (wp == p)
            sub = w_cache_imaging(theta, s / theta, rel[sel], src[sel], vis[sel], wstep=wstep,
                                  kernel_fn=kernel_fn, **kwargs)
            image += ifft(sub) / w_kernel_function(l, m, p * wincrement)
        sub = fft(image)
        i = numpy.nonzero(in_chunk)[0][0]
        y0, x0 = N // 2 + ymid[i] - s // 2, N // 2 + xmid[i] - s // 2
        ya, yb, xa, xb = max(y0, 0), min(y0 + s, N), max(x0, 0), min(x0 + s, N)
        if ya < yb and xa < xb:
            guv[ya:yb, xa:xb] += sub[ya - y0:yb - y0, xa - x0:xb - x0]
    return guv


def w_towers_predict(theta, lam, uvw, src, guv, subgrid_size, margin, wincrement, wstep,
                     kernel_fn=w_kernel, **kwargs):
    """w-towers predict (examples/notebooks/wtowers-predict.ipynb; the reverse of
    w_towers_imaging): for each chunk, the s x s sub-grid of guv at the chunk's
    origin (zeros outside the grid) is taken to image space; for each w-plane of the
    chunk, fft(image / w_kernel_function(l, m, wp*wincrement)) is degridded with the
    residual-w kernels (w_cache_predict) at the chunk-relative coordinates.  With one
    plane this is w_cache_predict itself."""
    N = guv.shape[0]
    s = subgrid_size
    src = numpy.zeros((len(uvw), 0)) if src is None else src
    out = numpy.zeros(len(uvw), dtype=complex)
    ub, vb, wp, xmid, ymid, rel = tower_bins(theta, uvw, s, margin, wincrement)
    l, m = theta * coordinates2(s)
    for cv, cu in sorted(set(zip(vb.tolist(), ub.tolist()))):
        in_chunk = (vb == cv) & (ub == cu)
        i = numpy.nonzero(in_chunk)[0][0]
        y0, x0 = N // 2 + ymid[i] - s // 2, N // 2 + xmid[i] - s // 2
        crop = numpy.zeros((s, s), dtype=complex)
        ya, yb, xa, xb = max(y0, 0), min(y0 + s, N), max(x0, 0), min(x0 + s, N)
        if ya < yb and xa < xb:
            crop[ya - y0:yb - y0, xa - x0:xb - x0] = guv[ya:yb, xa:xb]
        image = ifft(crop)
        for p in numpy.unique(wp[in_chunk]):
            sel = in_chunk & (wp == p)
            sub = fft(image / w_kernel_function(l, m, p * wincrement))
            out[sel] = w_cache_predict(theta, s / theta, rel[sel], src[sel], sub, wstep=wstep,
                                       kernel_fn=kernel_fn, **kwargs)
    return out


# --------------------------------------------------------------------------
# point-source visibilities (crocodile/simulate.py:210-230)

def simulate_point(dist_uvw, l, m):
    """exp(-2 pi i (u l + v m + w (sqrt(1 - l^2 - m^2) - 1))) (simulate.py:210-230)."""
    s = numpy.array([l, m, numpy.sqrt(1 - l ** 2 - m ** 2) - 1.0])
    return numpy.exp(-2j * numpy.pi * numpy.dot(dist_uvw, s))


def visibility_shift(uvw, vis, dl, dm):
    """vis * exp(-2 pi i (u dl + v dm)): the image shifted by (dl, dm)
    (simulate.py:259-274)."""
    s = numpy.array([dl, dm])
    return vis * numpy.exp(-2j * numpy.pi * numpy.dot(uvw[:, 0:2], s))


def uvw_transform(uvw, T):
    """uv multiplied by inv(T^T), w kept: the image transformed by the 2x2 matrix T
    (simulate.py:278-298, after Sault, Staveley-Smith and Brouw 1996)."""
    Tt = numpy.linalg.inv(numpy.transpose(T))
    return numpy.hstack([numpy.dot(uvw[:, 0:2], Tt), uvw[:, 2:3]])


# --------------------------------------------------------------------------
# Sze-Tan optimal gridding functions (crocodile/antialias.py), loop for loop.
# The reference reads its optimised h vectors from a json cache; these
# functions take h explicitly.

def sze_trap(vec, dx):
    """antialias.py:22-24."""
    return dx * (numpy.sum(vec) - 0.5 * (vec[0] + vec[-1]))


def sze_gridder_as_C(h, x0, nu, R):
    """calc_gridder_as_C (antialias.py:139-164): per offset, lstsq against the
    Gram matrix with rcond 1e-14."""
    M = len(nu)
    C = numpy.zeros((2 * R, M))
    K = numpy.zeros((2 * R, 2 * R))
    N = len(h)
    x = x0 * numpy.arange(0, N + 1, dtype=float) / N
    dx = x0 / N
    h_ext = numpy.concatenate(([1.0], h))
    for rp in range(2 * R):
        lp = rp - R + 1
        for r in range(2 * R):
            l = r - R + 1
            K[rp, r] = sze_trap((h_ext ** 2) * numpy.cos(2 * numpy.pi * (lp - l) * x), dx)
    rhs = numpy.zeros(2 * R)
    for m, nu_val in enumerate(nu):
        for rp in range(2 * R):
            lp = rp - R + 1
            rhs[rp] = sze_trap(h_ext * numpy.cos(2 * numpy.pi * (lp - nu_val) * x), dx)
        C[:, m] = numpy.linalg.lstsq(K, rhs, 1e-14)[0]
    return C


def sze_func_to_min(h, x0, M, R):
    """func_to_min (antialias.py:26-44)."""
    N = len(h)
    nu = (numpy.arange(M, dtype=float) + 0.5) / (2 * M)
    x = x0 * numpy.arange(N + 1, dtype=float) / N
    C = sze_gridder_as_C(h, x0, nu, R)
    h_ext = numpy.concatenate(([1.0], h))
    loss = numpy.zeros((len(h_ext), 2, M))
    for n, x_val in enumerate(x):
        one_app = 0
        for r in range(2 * R):
            l = r - R + 1
            one_app += h_ext[n] * C[r, :] * numpy.exp(2j * numpy.pi * (l - nu) * x_val)
        loss[n, 0, :] = 1.0 - numpy.real(one_app)
        loss[n, 1, :] = numpy.imag(one_app)
        if n in [0, N]:
            loss[n, :, :] /= numpy.sqrt(2)
    return loss.reshape(2 * M * (N + 1))


def sze_gridding_fine(h, x0, nu, R):
    """calc_gridding_fine (antialias.py:189-213): inverse Gram matrix."""
    M = len(nu)
    C = numpy.zeros((2 * R, M))
    K = numpy.zeros((2 * R, 2 * R))
    N = len(h)
    x = x0 * numpy.arange(0, N + 1, dtype=float) / N
    dx = x0 / N
    h_ext = numpy.concatenate(([1.0], h))
    for rp in range(2 * R):
        lp = rp - R + 1
        for r in range(2 * R):
            l = r - R + 1
            K[rp, r] = sze_trap((h_ext ** 2) * numpy.cos(2 * numpy.pi * (lp - l) * x), dx)
    Kinv = numpy.linalg.inv(K)
    rhs = numpy.zeros(2 * R)
    for m, nu_val in enumerate(nu):
        for rp in range(2 * R):
            lp = rp - R + 1
            rhs[rp] = sze_trap(h_ext * numpy.cos(2 * numpy.pi * (lp - nu_val) * x), dx)
        C[:, m] = numpy.dot(Kinv, rhs)
    return C


def sze_gridding_correction_fine(x, h, x0, M, R):
    """calc_gridding_correction_fine (antialias.py:229-246)."""
    nu = (numpy.arange(M, dtype=float) + 0.5) / (2 * M)
    C = sze_gridding_fine(h, x0, nu, R)
    dnu = 1.0 / (2 * M)
    c = numpy.zeros(numpy.shape(x))
    d = numpy.zeros(numpy.shape(x))
    for n, x_val in enumerate(x):
        for rp in range(2 * R):
            lp = rp - R + 1
            for r in range(2 * R):
                l = r - R + 1
                d[n] += numpy.sum(C[rp, :] * C[r, :] * numpy.cos(2 * numpy.pi * (lp - l) * x_val)) \
                    * dnu
            c[n] += numpy.sum(C[rp, :] * numpy.cos(2 * numpy.pi * (lp - nu) * x_val)) * dnu
    return c / d


def sze_gridder(h, x0, nu, M, R):
    """calc_gridder (antialias.py:176-187)."""
    C = sze_gridder_as_C(h, x0, nu, R)
    gridder = numpy.zeros(2 * M * R)
    for m in range(M):
        for rp in range(2 * R):
            lp = rp - R + 1
            indx = m - 2 * lp * M
            if indx >= 0:
                gridder[indx] = C[rp, m]
            else:
                gridder[-indx - 1] = C[rp, m]
    return gridder


def sze_gridder_to_C(gridder, R):
    """gridder_to_C (antialias.py:215-227)."""
    M = len(gridder) // (2 * R)
    C = numpy.zeros((2 * R, M))
    for r in range(2 * R):
        l = r - R + 1
        indx = numpy.arange(M) - 2 * M * l
        indx[indx < 0] = -indx[indx < 0] - 1
        C[r, :] = gridder[indx]
    return C


def sze_map_error(gridder, grid_correction, nu, x, R):
    """calc_map_error (antialias.py:248-263)."""
    M = len(nu) // (2 * R)
    dnu = nu[1] - nu[0]
    C = sze_gridder_to_C(gridder, R)
    loss = numpy.zeros((len(x), 2, M))
    for n, x_val in enumerate(x):
        one_app = 0
        for r in range(2 * R):
            l = r - R + 1
            one_app += grid_correction[n] * C[r, :] * numpy.exp(2j * numpy.pi * (l - nu[:M]) * x_val)
        loss[n, 0, :] = 1.0 - numpy.real(one_app)
        loss[n, 1, :] = numpy.imag(one_app)
    map_error = numpy.zeros(len(x))
    for i in range(len(x)):
        map_error[i] = 2 * numpy.sum((loss[i, :, :].flatten()) ** 2) * dnu
    return map_error


def sze_mean_map_error(x0, N, M, R, h):
    """calc_mean_map_error (antialias.py:265-271)."""
    nu = (numpy.arange(2 * R * M, dtype=float) + 0.5) / (2 * M)
    x = numpy.arange(N + 1, dtype=float) / (2 * N)
    gridder = sze_gridder(h, x0, nu, M, R)
    grid_correction = sze_gridding_correction_fine(x, h, x0, M, R)
    map_err = sze_map_error(gridder, grid_correction, nu, x, R)
    which = numpy.digitize(x0, x)
    return numpy.sqrt(sze_trap(map_err[:which], 1.0 / (2 * N)) / x[which])


def sze_tan_gridder(h, x0, R, over):
    """sze_tan_gridder (antialias.py:299-306) for the cached (h, x0)."""
    nu = numpy.arange(over, dtype=float) / over
    return numpy.transpose(sze_gridding_fine(h, x0, nu, R)[::-1])


def sze_tan_grid_correction_gen(h, x0, R, x):
    """sze_tan_grid_correction_gen (antialias.py:285-297) for the cached (h, x0)."""
    return 1 / sze_gridding_correction_fine(numpy.array(x), h, x0, len(x), R)


# --------------------------------------------------------------------------
# Facet <-> subgrid recombination (examples/notebooks/facet-subgrid-impl.ipynb,
# examples/grid/recombine.c).  Two conventions:
#   * centred (the notebook): arrays with their centre at n//2, transforms
#     fft/ifft of this module;
#   * raw (the C prototype): centre at index 0 (numpy.fft.ifftshift of the
#     centred array), unnormalised FFTW transforms.

def _pad_mid_axis(a, n, axis):
    n0 = a.shape[axis]
    if n == n0:
        return a
    pad = [(0, 0)] * a.ndim
    pad[axis] = (n // 2 - n0 // 2, (n + 1) // 2 - (n0 + 1) // 2)
    return numpy.pad(a, pad, mode='constant', constant_values=0.0)


def _extract_mid_axis(a, n, axis):
    c = a.shape[axis] // 2
    idx = [slice(None)] * a.ndim
    idx[axis] = slice(c - n // 2, c - n // 2 + n)
    return a[tuple(idx)]


def _fft_axis(a, axis, inverse=False):
    f = numpy.fft.ifft if inverse else numpy.fft.fft
    return numpy.fft.fftshift(f(numpy.fft.ifftshift(a, axis), axis=axis), axis)


def _along(v, ndim, axis):
    shape = [1] * ndim
    shape[axis] = len(v)
    return numpy.reshape(v, shape)


class RecombineConfig:
    """Sizes and the three PSWF-derived windows of the recombination
    (facet-subgrid-impl.ipynb cells 11 and 14): Fb = 1 / the facet's PSWF,
    Fn = the PSWF sampled at the xM rate, m0 = the truncated mask."""

    def __init__(self, N, yB, yN, yP, xA, xM, xMxN_yP, pswf):
        self.N, self.yB, self.yN, self.yP, self.xA, self.xM = N, yB, yN, yP, xA, xM
        self.xMxN_yP = xMxN_yP
        self.xM_yP = xM * yP // N
        self.xM_yN = xM * yN // N
        self.xM_step = N // xM
        self.pswf = numpy.asarray(pswf, dtype=float)
        self.Fb = 1 / extract_mid(self.pswf, yB)
        self.Fn = self.pswf[(yN // 2) % self.xM_step::self.xM_step]
        m0 = self.pswf * numpy.sinc(coordinates(yN) * xM / N * yN)
        self.m0 = xM * yP / N * extract_mid(ifft(pad_mid(m0, yP)), xMxN_yP).real


def rc_prepare_facet(cfg, facet, axis):
    """b * F along one axis: multiply by Fb, pad to yP, inverse FFT (cell 24)."""
    bf = _pad_mid_axis(facet * _along(cfg.Fb, facet.ndim, axis), cfg.yP, axis)
    return _fft_axis(bf, axis, inverse=True)


def rc_extract_subgrid(cfg, bf, subgrid_off, axis):
    """n * m(b * F) along one axis for the subgrid at subgrid_off (grid cells):
    window of xMxN_yP around the subgrid in the yP image, times m0, margins
    folded onto xM_yP, FFT, middle xM_yN times Fn (cell 24)."""
    xN_yP = cfg.xMxN_yP - cfg.xM_yP
    mid = _extract_mid_axis(numpy.roll(bf, -subgrid_off * cfg.yP // cfg.N, axis), cfg.xMxN_yP,
                            axis)
    mbf = _along(cfg.m0, bf.ndim, axis) * mid
    s = numpy.array(_extract_mid_axis(mbf, cfg.xM_yP, axis))
    lo = [slice(None)] * bf.ndim
    hi = [slice(None)] * bf.ndim
    lo[axis] = slice(xN_yP // 2)
    hi[axis] = slice(-xN_yP // 2, None)   # Python floor division, as the notebook writes it
    s[tuple(lo)] += mbf[tuple(hi)]
    s[tuple(hi)] += mbf[tuple(lo)]
    return _along(cfg.Fn, bf.ndim, axis) * _extract_mid_axis(_fft_axis(s, axis), cfg.xM_yN, axis)


def rc_facet_to_subgrids(cfg, facet, offs0, offs1):
    """NMBF_NMBF[i0, i1] of one 2-D facet for subgrid offsets offs0 x offs1
    (cell 29: axis 1 first, then axis 0)."""
    out = numpy.empty((len(offs0), len(offs1), cfg.xM_yN, cfg.xM_yN), dtype=complex)
    f_bf = rc_prepare_facet(cfg, facet, 1)
    for i1, o1 in enumerate(offs1):
        bf_nmbf = rc_prepare_facet(cfg, rc_extract_subgrid(cfg, f_bf, o1, 1), 0)
        for i0, o0 in enumerate(offs0):
            out[i0, i1] = rc_extract_subgrid(cfg, bf_nmbf, o0, 0)
    return out


def rc_add_facet(cfg, approx, nmbf, facet_off0, facet_off1):
    """approx += nmbf padded to xM and rolled to the facet (cell 30)."""
    approx += numpy.roll(pad_mid(nmbf, cfg.xM), (facet_off0 * cfg.xM // cfg.N,
                                                 facet_off1 * cfg.xM // cfg.N), (0, 1))
    return approx


def rc_finish_subgrid(cfg, approx):
    """The subgrid from its summed facet contributions: ifft, middle xA (cell 30)."""
    return extract_mid(ifft(approx), cfg.xA)


def rc_facet_to_subgrid_1d(cfg, facet, subgrid_off):
    """1-D facet -> subgrid contribution RNjMiBjFj (cell 16)."""
    return rc_extract_subgrid(cfg, rc_prepare_facet(cfg, facet, 0), subgrid_off, 0)


def rc_split_subgrid(cfg, subgrid, facet_offs):
    """FNjSi: the subgrid's FFT cut at each facet (cell 18, 1-D or 2-D)."""
    fs = numpy.fft.fftshift(numpy.fft.fftn(numpy.fft.ifftshift(pad_mid(subgrid, cfg.xM))))
    out = []
    for fo in facet_offs:
        shift = tuple(-f * cfg.xM // cfg.N for f in numpy.atleast_1d(fo))
        out.append(extract_mid(numpy.roll(fs, shift, tuple(range(fs.ndim))), cfg.xM_yN))
    return numpy.array(out)


def rc_subgrid_to_facet_axis(cfg, fn, subgrid_off, axis):
    """One subgrid's contribution to a facet along one axis (cell 18): Fn,
    pad to xM_yP, inverse FFT, wrap onto xMxN_yP, m0, pad to yP, roll to the
    subgrid, FFT, middle yB (Fb and the facet mask are applied by the caller
    after the sum over subgrids)."""
    xN_yP = cfg.xMxN_yP - cfg.xM_yP
    nd = fn.ndim
    mid = _fft_axis(_pad_mid_axis(_along(cfg.Fn, nd, axis) * fn, cfg.xM_yP, axis), axis,
                    inverse=True)
    shape = list(fn.shape)
    shape[axis] = cfg.xMxN_yP
    nj = numpy.zeros(shape, dtype=complex)
    c = cfg.xMxN_yP // 2
    idx = [slice(None)] * nd
    idx[axis] = slice(c - cfg.xM_yP // 2, c - cfg.xM_yP // 2 + cfg.xM_yP)
    nj[tuple(idx)] = mid
    lo = [slice(None)] * nd
    hi = [slice(None)] * nd
    lo[axis] = slice(xN_yP // 2)
    hi[axis] = slice(-xN_yP // 2, None)
    # the margins wrap: NjSi[-xN//2:] = mid[:xN//2], NjSi[:xN//2] = mid[-xN//2:]
    nj[tuple(hi)] = mid[tuple(lo)]
    nj[tuple(lo)] = mid[tuple(hi)]
    p = _pad_mid_axis(_along(cfg.m0, nd, axis) * nj, cfg.yP, axis)
    p = numpy.roll(p, subgrid_off * cfg.yP // cfg.N, axis)
    return _extract_mid_axis(_fft_axis(p, axis), cfg.yB, axis)


def rc_subgrids_to_facet(cfg, fnjsi, offs0, offs1):
    """Facet approximation (before Fb and the facet mask) from the FNjSi of
    subgrids at offs0 x offs1 for one facet: axis 1 per subgrid, summed over
    i1, then axis 0 per row of subgrids, summed over i0 (the 2-D form of cell
    18 by separability).  fnjsi: [n0, n1, xM_yN, xM_yN]."""
    acc = numpy.zeros((cfg.yB, cfg.yB), dtype=complex)
    for i0, o0 in enumerate(offs0):
        row = numpy.zeros((cfg.xM_yN, cfg.yB), dtype=complex)
        for i1, o1 in enumerate(offs1):
            row += rc_subgrid_to_facet_axis(cfg, fnjsi[i0, i1], o1, 1)
        acc += rc_subgrid_to_facet_axis(cfg, row, o0, 0)
    return acc


# raw convention: the C prototype's primitives (examples/grid/recombine.c)

def rc_generate_Fb(yB, pswf_raw):
    """generate_Fb (recombine.c:12-22)."""
    Fb = numpy.empty(yB)
    for i in range(yB // 2 + 1):
        Fb[i] = 1 / pswf_raw[i]
    for i in range(yB // 2 + 1, yB):
        Fb[i] = Fb[yB - i]
    return Fb


def rc_generate_Fn(yN, xM_yN, pswf_raw):
    """generate_Fn (recombine.c:24-33)."""
    assert yN % xM_yN == 0
    step = yN // xM_yN
    return numpy.array([pswf_raw[i * step] for i in range(xM_yN)])


def rc_generate_m(image_size, yP, yN, xM, xMxN_yP, pswf_raw):
    """generate_m (recombine.c:35-67): the sinc-truncated PSWF, DCT-I of
    length yP/2+1 (FFTW REDFT00: Y_k = X_0 + (-1)^k X_{n-1} + 2 sum X_j
    cos(pi j k / (n-1))), mirrored to xMxN_yP."""
    n = yP // 2 + 1
    m = numpy.zeros(n)
    m[0] = pswf_raw[0] * xM / image_size
    for i in range(1, yN // 2):
        x = i * xM / image_size
        m[i] = pswf_raw[i] * (numpy.sin(x * numpy.pi) / x / numpy.pi) * xM / image_size
    j = numpy.arange(1, n - 1)
    y = numpy.array([m[0] + (-1) ** k * m[n - 1] + 2 * numpy.sum(m[1:n - 1] *
                     numpy.cos(numpy.pi * j * k / (n - 1))) for k in range(n)])
    out = numpy.empty(xMxN_yP)
    for i in range(xMxN_yP // 2 + 1):
        out[i] = y[i]
    for i in range(xMxN_yP // 2 + 1, xMxN_yP):
        out[i] = y[xMxN_yP - i]
    return out


def rc_prepare_facet_raw(yB, yP, Fb, facet):
    """prepare_facet (recombine.c:69-85) then FFTW_BACKWARD of length yP."""
    bf = numpy.zeros(yP, dtype=complex)
    for i in range(yB // 2):
        bf[i] = Fb[i] * facet[i] / yP
    for i in range(yP - yB // 2, yP):
        bf[i] = Fb[yB - yP + i] * facet[yB - yP + i] / yP
    return numpy.fft.ifft(bf) * yP


def rc_extract_subgrid_raw(yP, xM_yP, xMxN_yP, xM_yN, subgrid_offset, m_trunc, Fn, bf):
    """extract_subgrid (recombine.c:87-119); subgrid_offset in yP samples."""
    xN_yP = xMxN_yP - xM_yP
    off = subgrid_offset + 2 * yP
    mbf = numpy.zeros(xM_yP, dtype=complex)
    for i in range(xM_yP):
        if i < (xMxN_yP + 1) // 2:
            mbf[i] += m_trunc[i] * bf[(i + off) % yP]
        if i >= xM_yP - xMxN_yP // 2:
            mbf[i] += m_trunc[xN_yP + i] * bf[(i + off - xM_yP) % yP]
    mbf = numpy.fft.fft(mbf)
    nmbf = numpy.empty(xM_yN, dtype=complex)
    for i in range(xM_yN // 2):
        nmbf[i] = mbf[i] * Fn[i]
    for i in range(xM_yN // 2, xM_yN):
        nmbf[i] = mbf[xM_yP - xM_yN + i] * Fn[i]
    return nmbf


def rc_add_facet_raw(xM, xM_yN, facet_offset, nmbf, out):
    """add_facet (recombine.c:122-133); facet_offset in xM samples."""
    off = facet_offset + 2 * xM
    for i in range(xM_yN):
        out[(i - xM_yN // 2 + off) % xM] += nmbf[(i + xM_yN // 2) % xM_yN] / xM
    return out


# --------------------------------------------------------------------------
# visibility ingest: collect_blocks (scripts/image_dataset.py:75-87) over
# per-baseline blocks, uvw_lambda as arl/data_models.py:198-202 (c = the SI
# value astropy's const.c holds).  Each block: dict or object with
# frequency [nchan], time [nrow], uvw [nrow, 3], antenna1, antenna2 [nrow],
# vis [nrow, nchan, npol].

C_LIGHT = 299792458.0


def _col(b, name):
    return numpy.asarray(b[name] if isinstance(b, dict) else getattr(b, name))


def collect_blocks(blocks, pol=0):
    """(uvw_lambda [n, 3], src [n, 4], vis [n]) in block, row, channel order,
    whole blocks at a time as the reference's numpy code (the same
    elementwise operations: (uvw * f) / c)."""
    uvw, src, vis = [], [], []
    for b in blocks:
        freq, time = _col(b, "frequency"), _col(b, "time")
        u, v = _col(b, "uvw"), _col(b, "vis")
        a1, a2 = _col(b, "antenna1"), _col(b, "antenna2")
        nrow, nchan = len(time), len(freq)
        uvw.append((u[:, None, :] * freq[None, :, None] / C_LIGHT).reshape(-1, 3))
        s = numpy.empty((nrow, nchan, 4))
        s[:, :, 0] = a1[:, None]
        s[:, :, 1] = a2[:, None]
        s[:, :, 2] = time[:, None]
        s[:, :, 3] = freq[None, :]
        src.append(s.reshape(-1, 4))
        vis.append(v[:, :, pol].reshape(-1))
    if not uvw:
        return numpy.zeros((0, 3)), numpy.zeros((0, 4)), numpy.zeros(0, dtype=complex)
    return (numpy.concatenate(uvw), numpy.concatenate(src),
            numpy.concatenate(vis).astype(complex))


# --------------------------------------------------------------------------
# AW-towers imaging (examples/notebooks/awtowers.ipynb cells 17-22) with no
# phase-centre shift (dl = dm = 0, T = identity).  Per uv chunk (centred
# bins floor(u theta / C + 1/2), C = subgrid - margin), per w-plane
# (around(w / wstep)) and per baseline, the visibilities are gridded with the
# anti-aliasing kernel relative to the chunk centre on a 2s x 2s grid at 2
# theta (pregrid_tower_plane), transformed, corrected for the kernel, cut to
# s x s and multiplied by aimage[a2] / aimage[a1] (grid_tower_plane); each
# plane is moved to w = 0 by dividing by w_kernel_function(l, m, wp wstep)
# (the closed form of the notebook's wkern ** (wp - last_wp) chain; the
# notebook skips one step of that chain after a chunk's first plane when it
# is the data set's lowest, which the golden data avoids); the chunk's FFT
# is added into the grid (grid_tower, grid_towers).

def aw_towers_imaging(theta, lam, uvw, src, vis, subgrid_size, margin, wstep, aimage,
                      aa_support=6, aa_over=4096):
    """(grid_sum, image): the uv grid and real(ifft(grid_sum)) / aa x aa."""
    s, C = int(subgrid_size), int(subgrid_size) - int(margin)
    N = int(numpy.ceil(theta * lam))
    aa = anti_aliasing_function(N, 0, aa_support)
    aa_sub = anti_aliasing_function(s, 0, aa_support)
    aa_sub2 = anti_aliasing_function(2 * s, 0, aa_support)
    aa_gcf = kernel_oversample(aa, aa_over, aa_support)
    l, m = kernel_coordinates(s, theta)
    uvw = numpy.asarray(uvw, dtype=float)
    src = numpy.asarray(src)
    vis = numpy.asarray(vis)
    ubin = numpy.floor(uvw[:, 0] * theta / C + 0.5).astype(int)
    vbin = numpy.floor(uvw[:, 1] * theta / C + 0.5).astype(int)
    wplane = numpy.around(uvw[:, 2] / wstep).astype(int)
    grid = numpy.zeros((N, N), dtype=complex)
    uvw_size = s / theta
    for ub in range(ubin.min(), ubin.max() + 1):
        for vb in range(vbin.min(), vbin.max() + 1):
            sel = (ubin == ub) & (vbin == vb)
            if not numpy.any(sel):
                continue
            xy_min = C * numpy.array([ub - 0.5, vb - 0.5])
            xy_max = C * numpy.array([ub + 0.5, vb + 0.5])
            uv_mid = (xy_max + xy_min) // 2 / theta
            xy_min -= (margin + 1) // 2
            img = numpy.zeros((s, s), dtype=complex)
            for wp in numpy.unique(wplane[sel]):
                slc = sel & (wplane == wp)
                uvw_mid = numpy.hstack([uv_mid, [wp * wstep]])
                plane = numpy.zeros((s, s), dtype=complex)
                for a1, a2 in numpy.unique(src[slc], axis=0):
                    b = slc & (src[:, 0] == a1) & (src[:, 1] == a2)
                    pg = conv_imaging(2 * theta, uvw_size, uvw[b] - uvw_mid,
                                      numpy.empty((int(b.sum()), 0)), vis[b], aa_gcf)
                    pim = ifft(pg) / numpy.outer(aa_sub2, aa_sub2)
                    pim = extract_mid(pim, s) * numpy.outer(aa_sub, aa_sub)
                    plane += pim * aimage[a2] / aimage[a1]
                img += plane / w_kernel_function(l, m, wp * wstep)
            sub = fft(img)
            x0, y0 = N // 2 + xy_min.astype(int)
            x1, y1 = x0 + s, y0 + s
            x0b, y0b, x1b, y1b = max(x0, 0), max(y0, 0), min(x1, N), min(y1, N)
            grid[y0b:y1b, x0b:x1b] += sub[y0b - y0:y1b - y0, x0b - x0:x1b - x0]
    image = numpy.real(ifft(grid)) / numpy.outer(aa, aa)
    return grid, image
