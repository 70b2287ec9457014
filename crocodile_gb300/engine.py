"""Device-level engine: HBM-resident torch tensors in, C-ABI kernels underneath.

PyTorch only provides device memory, streams and the current device here;
every computation on the gridding path is a kernel of libcrocodile_gb300.so.
All functions take and return CUDA tensors and run on the current stream.
"""

import ctypes
import weakref

import numpy
import torch

from . import _lib as L

CF = torch.complex64
CD = torch.complex128


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("crocodile_gb300 needs a CUDA GPU (sm_103a); none is visible")
    L.lib()


def cuda_tensor(x, dtype):
    """x (numpy array or tensor) as a contiguous CUDA tensor of dtype."""
    if isinstance(x, torch.Tensor):
        t = x.to(device="cuda", dtype=dtype)
    else:
        a = numpy.asarray(x)
        if dtype.is_complex:
            a = a.astype(numpy.complex128 if dtype == CD else numpy.complex64, copy=False)
        t = torch.as_tensor(numpy.ascontiguousarray(a)).to(device="cuda", dtype=dtype)
    return t.contiguous()


class Status:
    """The CG_STATUS_WORDS device counters shared by a sequence of calls."""

    def __init__(self):
        self.t = torch.zeros(L.CG_STATUS_WORDS, dtype=torch.int32, device="cuda")

    def reset(self):
        L.call("cg_status_reset", _p(self.t), stream())

    def check(self):
        """Synchronise and raise the reference's exception for any counted error."""
        L.raise_for(L.lib().cg_status_check(_p(self.t), None, stream()))

    def counts(self):
        return self.t.cpu().tolist()


# --------------------------------------------------------------------------
# kernel tables

class KernelTable:
    """A GCF table on the device, flattened to [G, Q, (Q,) S(, S)] (synthesis.py:451-461)."""

    def __init__(self, table, sep, Q, S):
        self.table = table.contiguous()
        self.sep = bool(sep)
        self.Q, self.S = int(Q), int(S)
        per = Q * S if sep else Q * Q * S * S
        self.G = self.table.numel() // per
        if self.G * per != self.table.numel():
            raise ValueError("kernel table size does not match Q=%d S=%d" % (Q, S))

    @property
    def dtype(self):
        return self.table.dtype

    def desc(self):
        return L.KernelDesc(int(self.sep), self.Q, self.S, self.G)

    def to(self, dtype):
        return self if dtype == self.dtype else KernelTable(self.table.to(dtype), self.sep,
                                                            self.Q, self.S)

    def padded_even(self, uvw, lam, shape):
        """For a complex64 non-separable table of odd support S = 13 or 15, the same
        kernels zero-padded to S + 1 (a zero first row and column, so that tap j + 1
        of the padded kernel sits where tap j of the original did: footprints start
        at x - (S + 1) / 2 instead of x - S // 2).  Gridding and degridding with it
        give the same results (the extra taps add zeros), and the lane-layout
        gridder, which streams even-support slices by bulk copies, takes it: the
        w-projection step at 4096^2, 2M visibilities, S 15 runs in 1.24-1.27 ms
        against 1.40 ms with the S 15 table.  Returns self when the table does not
        qualify or a footprint could leave the grid (the padded one reaches one
        cell lower): uvw [n, 3] device coordinates in wavelengths, lam the scale
        (grid cells = N u / lam), shape the grid (H, W)."""
        if self.sep or self.dtype != CF or self.S not in (13, 15) or uvw.shape[0] == 0:
            return self
        N = min(int(shape[-2]), int(shape[-1]))
        lo, hi = torch.aminmax(uvw[:, :2])
        lo, hi = float(lo) / lam * N + N // 2, float(hi) / lam * N + N // 2
        margin = self.S // 2 + 2
        if not (lo >= margin and hi <= N - 1 - margin):
            return self
        S, Q = self.S, self.Q
        t = torch.zeros((self.G, Q, Q, S + 1, S + 1), dtype=CF, device=self.table.device)
        t[..., 1:, 1:] = self.table.view(self.G, Q, Q, S, S)
        return KernelTable(t.reshape(-1), False, Q, S + 1)

    @classmethod
    def from_gcf(cls, gcf, nsrc, dtype=CF):
        """Layout from the kernel rank against the src columns, as make_gcf decides it."""
        shape = tuple(gcf.shape)
        extra = len(shape) - nsrc
        if extra == 2:
            sep, Q, S = True, shape[-2], shape[-1]
        elif extra == 4:
            if shape[-1] != shape[-2]:
                raise ValueError("non-square kernels are not supported")
            sep, Q, S = False, shape[-3], shape[-1]
        else:
            raise AssertionError("kernel rank %d does not match %d src columns"
                                 % (len(shape), nsrc))
        if not sep and shape[-3] != shape[-4]:
            raise ValueError("kernel oversampling must be equal along both axes")
        return cls(cuda_tensor(gcf, dtype).reshape(-1), sep, Q, S)


def kernel_groups(lead_shape, src, n):
    """Flat group index of each src row into the kernel's leading dims (numpy indexing,
    negative indices wrap); int32 numpy array, or None when there are no src columns."""
    if src is None:
        return None
    src = numpy.asarray(src)
    if src.ndim != 2 or src.shape[1] == 0:
        return None
    if src.shape[1] != len(lead_shape):
        raise AssertionError("src has %d columns, kernel has %d leading dims"
                             % (src.shape[1], len(lead_shape)))
    idx = src.astype(numpy.int64)
    for k, d in enumerate(lead_shape):
        col = idx[:, k]
        if ((col < -d) | (col >= d)).any():
            raise IndexError("src column %d out of range for kernel dimension %d" % (k, d))
        idx[:, k] = numpy.where(col < 0, col + d, col)
    return numpy.ravel_multi_index(tuple(idx.T), lead_shape).astype(numpy.int32)


# --------------------------------------------------------------------------
# plans and gridding

class Plan:
    """Sorted, bit-exact cell assignment of a visibility set (cg_plan_create).

    ``uvw`` is a float64 CUDA tensor [n, >=2] (rows in units such that
    uvw / lam is the fraction of the grid), ``shape`` the grid (H, W)."""

    def __init__(self, uvw, lam, shape, ktab, kidx=None, mode=L.CG_PLAN_TILED, status=None,
                 wbins=None, layers=None, groups=None, tile=0):
        """wbins=(wstep, kmin): take each visibility's kernel group from its w bin
        (round(w / wstep) - kmin) inside the plan's coordinate pass.
        layers=(L, layer): grid visibility i into grid layer[i] of a stack of L grids.
        groups=(G, group): plain form only, one launch per group[i] in [0, G).
        tile: this plan's grid tile edge (0: the tuning / automatic choice)."""
        require_cuda()
        self.uvw = cuda_tensor(uvw, torch.float64)
        if self.uvw.dim() != 2 or self.uvw.shape[1] < 2:
            raise ValueError("uvw must be [n, >=2]")
        self.n = self.uvw.shape[0]
        self.kidx = None if kidx is None else cuda_tensor(kidx, torch.int32)
        self.shape = (int(shape[0]), int(shape[1]))
        self.mode = mode
        self.sep, self.Q, self.S, self.G = ktab.sep, ktab.Q, ktab.S, ktab.G
        kd = ktab.desc()
        self._kd = kd
        self.layers = 1 if layers is None else int(layers[0])
        self.layer = None if layers is None else cuda_tensor(layers[1], torch.int32)
        self.group = None if groups is None else cuda_tensor(groups[1], torch.int32)
        opts = L.PlanOpts(self.layers, None if self.layer is None else self.layer.data_ptr(),
                          0.0 if wbins is None else float(wbins[0]),
                          0 if wbins is None else int(wbins[1]),
                          None if self.group is None else self.group.data_ptr(),
                          0 if groups is None else int(groups[0]), int(tile))
        nbytes = L.lib().cg_plan_workspace_bytes_ex(mode, self.n, self.shape[0], self.shape[1],
                                                    ctypes.byref(kd), ctypes.byref(opts))
        if nbytes == 0:
            L.raise_for(L.CG_ERR_ARG, "cg_plan_workspace_bytes_ex")
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        self.status = status or Status()
        if status is None:
            self.status.reset()
        h = ctypes.c_void_p()
        L.call("cg_plan_create_ex", ctypes.byref(h), mode, ctypes.byref(kd), self.shape[0],
               self.shape[1], _p(self.uvw), self.uvw.stride(0), float(lam), _p(self.kidx),
               self.n, ctypes.byref(opts), _p(self.ws), nbytes, _p(self.status.t), stream())
        self.handle = h
        self._fin = weakref.finalize(self, L.lib().cg_plan_destroy, h)

    def info(self):
        out = (ctypes.c_int64 * 4)()
        L.call("cg_plan_info", self.handle, out)
        return {"tile": out[0], "max_items": out[1], "chunk": out[2], "buckets": out[3]}

    def export(self):
        """(recs [n, 4] int32 {x0, y0, k0, k1} in sorted order, perm [n] sorted
        position -> input index, counts [buckets]) as CUDA tensors."""
        nb = self.info()["buckets"]
        recs = torch.empty((self.n, 4), dtype=torch.int32, device="cuda")
        perm = torch.empty(self.n, dtype=torch.int32, device="cuda")
        counts = torch.empty(nb, dtype=torch.int32, device="cuda")
        L.call("cg_plan_export", self.handle, _p(recs), _p(perm), _p(counts), stream())
        return recs, perm, counts

    def check(self):
        self.status.check()

    def accept(self, src, table):
        """Take ``table`` wherever ``src`` is passed (a plan built for src's
        padded_even form)."""
        self._aliases = getattr(self, "_aliases", {})
        self._aliases[id(src)] = (src, table)

    def _table(self, ktab, dtype):
        alias = getattr(self, "_aliases", {}).get(id(ktab))
        if alias is not None and alias[0] is ktab:
            ktab = alias[1]
        if (ktab.sep, ktab.Q, ktab.S, ktab.G) != (self.sep, self.Q, self.S, self.G):
            raise ValueError("kernel table does not match the plan's kernel layout")
        return ktab.to(dtype).table

    def layer_mean_w(self):
        """(mean w [layers] float64, visibility count [layers] int32) per grid layer."""
        mean = torch.empty(self.layers, dtype=torch.float64, device="cuda")
        count = torch.empty(self.layers, dtype=torch.int32, device="cuda")
        L.call("cg_plan_layer_mean_w", self.handle, _p(self.uvw), self.uvw.stride(0), _p(mean),
               _p(count), stream())
        return mean, count

    def grid(self, ktab, vis, grid):
        """grid (c64 [H, W], or [layers, H, W]) += convgrid of vis (c64 [n])."""
        t = self._table(ktab, CF)
        L.call("cg_grid", self.handle, _p(t), _p(vis), _p(grid), stream())
        return grid

    def grid_sparse(self, ktab, vis, grid):
        """grid += convgrid(vis) with per-tap atomics (cg_grid_sparse): for plans with
        few visibilities per tile."""
        t = self._table(ktab, CF)
        L.call("cg_grid_sparse", self.handle, _p(t), _p(vis), _p(grid), stream())
        return grid

    def grid_weighted(self, ktab, vis, weight, grid):
        """grid += convgrid of vis * weight (vis None: weight alone, the PSF pass)."""
        t = self._table(ktab, CF)
        L.call("cg_grid_weighted", self.handle, _p(t), _p(vis), _p(weight), _p(grid), stream())
        return grid

    def degrid(self, ktab, grid, out=None):
        t = self._table(ktab, CF)
        if out is None:
            out = torch.empty(self.n, dtype=CF, device="cuda")
        L.call("cg_degrid", self.handle, _p(t), _p(grid), _p(out), stream())
        return out

    def degrid_grid(self, ktab, grid_in, vis_in, grid_out, residual=False, vis_out=None):
        """One pass: vis_out = degrid(grid_in); grid_out += grid(vis_in, or vis_in - vis_out
        when residual).  Returns vis_out."""
        t = self._table(ktab, CF)
        if vis_out is None:
            vis_out = torch.empty(self.n, dtype=CF, device="cuda")
        L.call("cg_degrid_grid", self.handle, _p(t), _p(grid_in), _p(vis_in), int(bool(residual)),
               _p(vis_out), _p(grid_out), stream())
        return vis_out

    def grid_fp64(self, ktab, vis, grid):
        t = self._table(ktab, CD)
        L.call("cg_grid_fp64", self.handle, _p(t), _p(vis), _p(grid), stream())
        return grid

    def degrid_fp64(self, ktab, grid, out=None):
        t = self._table(ktab, CD)
        if out is None:
            out = torch.empty(self.n, dtype=CD, device="cuda")
        L.call("cg_degrid_fp64", self.handle, _p(t), _p(grid), _p(out), stream())
        return out


def frac_coords(uvw, lam, shape, Q, status):
    uvw = cuda_tensor(uvw, torch.float64)
    n = uvw.shape[0]
    outs = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(4)]
    L.call("cg_frac_coords", _p(uvw), uvw.stride(0), float(lam), n, int(shape[0]),
           int(shape[1]), int(Q), *[_p(o) for o in outs], _p(status.t), stream())
    return outs


def w_bins(uvw, wstep, status):
    """(kidx int32 [n] = bin - min bin, min bin, max bin) of w_cache_imaging's bins."""
    uvw = cuda_tensor(uvw, torch.float64)
    n = uvw.shape[0]
    kidx = torch.empty(n, dtype=torch.int32, device="cuda")
    dmm = torch.empty(2, dtype=torch.int32, device="cuda")
    hmm = (ctypes.c_int32 * 2)()
    L.call("cg_w_bins", _p(uvw), uvw.stride(0), n, float(wstep), _p(kidx), _p(dmm), hmm,
           _p(status.t), stream())
    return kidx, int(hmm[0]), int(hmm[1])


def compact_keys(key, nkeys, status):
    """(row per element, distinct keys ascending) of int32 keys in [0, nkeys)."""
    key = cuda_tensor(key, torch.int32)
    n = key.shape[0]
    row = torch.empty(n, dtype=torch.int32, device="cuda")
    kor = torch.empty(max(1, min(n, int(nkeys))), dtype=torch.int32, device="cuda")
    nbytes = L.lib().cg_compact_keys_workspace_bytes(int(nkeys))
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    nrows = ctypes.c_int32()
    L.call("cg_compact_keys", _p(key), n, int(nkeys), _p(row), _p(kor), ctypes.byref(nrows),
           _p(ws), nbytes, _p(status.t), stream())
    return row, kor[:nrows.value]


def row_keys(uvw, wstep, kmin, nbins, cols, mins, ranges, status):
    """int32 kernel-cache key per row: (w bin - kmin, integer src columns) packed in
    mixed radix (cg_row_keys); cols is an int32 [n, k] tensor, mins / ranges host ints."""
    uvw = cuda_tensor(uvw, torch.float64)
    n = uvw.shape[0]
    k = len(mins)
    cols = None if k == 0 else cuda_tensor(cols, torch.int32).reshape(n, k).contiguous()
    key = torch.empty(n, dtype=torch.int32, device="cuda")
    cm = (ctypes.c_int32 * max(k, 1))(*[int(m) for m in mins])
    cr = (ctypes.c_int32 * max(k, 1))(*[int(r) for r in ranges])
    L.call("cg_row_keys", _p(uvw), uvw.stride(0), n, float(wstep), int(kmin), int(nbins),
           _p(cols), k, cm, cr, _p(key), _p(status.t), stream())
    return key


def aw_keys(uvw, a1, a2, nant, wstep, kmin, nbins, status):
    uvw = cuda_tensor(uvw, torch.float64)
    a1, a2 = cuda_tensor(a1, torch.int32), cuda_tensor(a2, torch.int32)
    key = torch.empty(uvw.shape[0], dtype=torch.int32, device="cuda")
    L.call("cg_aw_keys", _p(uvw), uvw.stride(0), _p(a1), _p(a2), uvw.shape[0], int(nant),
           float(wstep), int(kmin), int(nbins), _p(key), _p(status.t), stream())
    return key


def grid_boxcar(uvw, lam, vis, grid, status):
    L.call("cg_grid_boxcar", _p(uvw), uvw.stride(0), float(lam), uvw.shape[0], _p(vis),
           _p(grid), grid.shape[0], grid.shape[1], _p(status.t), stream())
    return grid


def degrid_boxcar(uvw, lam, grid, status):
    out = torch.empty(uvw.shape[0], dtype=CD, device="cuda")
    L.call("cg_degrid_boxcar", _p(uvw), uvw.stride(0), float(lam), uvw.shape[0], _p(grid),
           _p(out), grid.shape[0], grid.shape[1], _p(status.t), stream())
    return out


def wstack_combine(planes, theta, mean_w, counts, status):
    """sum_p planes[p] / w_kernel_function(l, m, mean_w[p]) as a complex64 image."""
    layers, N = planes.shape[0], planes.shape[-1]
    out = torch.empty((N, N), dtype=CF, device="cuda")
    L.call("cg_wstack_combine", _p(planes), layers, N, float(theta), _p(mean_w), _p(counts),
           _p(out), _p(status.t), stream())
    return out


# --------------------------------------------------------------------------
# imaging helpers

def weights(uvw, lam, N, status, v_in=None):
    """doweight on the device: float64 [n] weights."""
    n = uvw.shape[0]
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    counts = torch.empty(N * N, dtype=torch.int32, device="cuda")
    L.call("cg_weights", _p(uvw), uvw.stride(0), float(lam), n, int(N), _p(v_in), _p(out),
           _p(counts), _p(status.t), stream())
    return out


def mirror_uvw(uvw, vis):
    """In place on the device tensors (mirror_uvw)."""
    L.call("cg_mirror_uvw", _p(uvw), uvw.stride(0), uvw.shape[0], _p(vis),
           int(vis is not None and vis.dtype == CF), stream())


def make_hermitian(grid):
    L.call("cg_make_hermitian", _p(grid), grid.shape[-2], grid.shape[-1],
           int(grid.dtype == CF), stream())
    return grid


def fft_(t, inverse):
    """Centred (i)fft of the last one or two dims of t, in place."""
    if t.dim() == 1:
        H, W, batch = 1, t.shape[0], 1
    else:
        H, W = t.shape[-2], t.shape[-1]
        batch = t.numel() // (H * W)
    ws = None
    if not ((H == 1 or H % 2 == 0) and W % 2 == 0):
        ws = torch.empty_like(t)
    L.call("cg_fft", _p(t), batch, H, W, int(t.dtype == CF), int(inverse), _p(ws), stream())
    return t


def dfft2_supported(H, W):
    """Sides the double-float 2-D transform takes: powers of two 64..2048."""
    return all(64 <= n <= 2048 and n & (n - 1) == 0 for n in (H, W))


def fft_df_(t, inverse):
    """Centred (i)fft of the last two dims of a complex128 t, in place, in
    double-float arithmetic on the FP32 units (about 48 significant bits)."""
    H, W = t.shape[-2], t.shape[-1]
    if t.dtype != CD or not t.is_contiguous() or not dfft2_supported(H, W):
        raise ValueError("fft_df_ takes contiguous complex128 planes with power-of-two "
                         "sides 64..2048")
    L.call("cg_fft2_centred_df", _p(t), t.numel() // (H * W), H, W, int(inverse), stream())
    return t


def fft_timeouts(reset=True):
    """Waits of the FP32 FFT's column passes that ran out (cg_fft_timeouts), since
    the last reset; synchronises the device."""
    c = (ctypes.c_int32 * 1)()
    L.call("cg_fft_timeouts", c, int(bool(reset)))
    return int(c[0])


def fft_raw(t, inverse):
    """Unshifted, unnormalised (i)fft of the last two dims of t, in place."""
    H, W = t.shape[-2], t.shape[-1]
    L.call("cg_fft_raw", _p(t), t.numel() // (H * W), H, W, int(t.dtype == CF), int(inverse),
           stream())
    return t


def image_from_grid(grid, want_max=False):
    """Re(ifft(make_grid_hermitian(grid))) as float32; consumes grid (c64, even sizes)."""
    H, W = grid.shape
    img = torch.empty((H, W), dtype=torch.float32, device="cuda")
    mx = torch.empty(1, dtype=torch.float32, device="cuda") if want_max else None
    L.call("cg_image_from_grid", _p(grid), H, W, _p(img), _p(mx), stream())
    return img, mx


def scale_image(img, d_scale):
    L.call("cg_scale_image", _p(img), img.numel(), _p(d_scale), stream())
    return img


# --------------------------------------------------------------------------
# kernel generation

def kernel_oversample(ff, Qpx, s=None, dtype=CD, ndim=None):
    """kernel_oversample of one far field, or of a batch along leading dims
    (then ``ndim`` says whether each far field is 1-D or 2-D), on the device."""
    ff = cuda_tensor(ff, CD)
    if ndim is None:
        ndim = ff.dim()
    if ndim not in (1, 2) or ff.dim() < ndim:
        raise AssertionError("Unsupported grid shape for kernel_oversample")
    if ndim == 2 and ff.shape[-1] != ff.shape[-2]:
        raise AssertionError("2-D far fields must be square")
    N0 = ff.shape[-1]
    s = N0 if s is None else int(s)
    batch_shape = tuple(ff.shape[:-ndim])
    batch = int(numpy.prod(batch_shape)) if batch_shape else 1
    nbytes = L.lib().cg_kernel_oversample_workspace_bytes(batch, ndim, N0, int(Qpx))
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    tail = (Qpx, Qpx, s, s) if ndim == 2 else (Qpx, s)
    out = torch.empty(batch_shape + tail, dtype=dtype, device="cuda")
    L.call("cg_kernel_oversample", _p(ff), batch, ndim, N0, int(Qpx), s, _p(out),
           int(dtype == CF), _p(ws), nbytes, stream())
    return out


def w_kernels(theta, ws_list, NpixFF, NpixKern, Qpx, invert=True, dl=0.0, dm=0.0, T=None,
              dtype=CF, status=None, max_workspace=1 << 31):
    """w_kernel for every w in ws_list: [nw, Q, Q, S, S] on the device."""
    assert NpixFF > NpixKern or (NpixFF == NpixKern and Qpx == 1)
    w = numpy.ascontiguousarray(numpy.asarray(ws_list, dtype=numpy.float64).ravel())
    nw = len(w)
    st = status or Status()
    if status is None:
        st.reset()
    per = L.lib().cg_w_kernels_workspace_bytes(1, int(NpixFF), int(Qpx))
    full = L.lib().cg_w_kernels_workspace_bytes(nw, int(NpixFF), int(Qpx))
    nbytes = int(min(full, max(per + 256 + 8 * nw, max_workspace)))
    wsb = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = torch.empty((nw, Qpx, Qpx, NpixKern, NpixKern), dtype=dtype, device="cuda")
    Tm = None
    if T is not None:
        Tm = numpy.ascontiguousarray(numpy.asarray(T, dtype=numpy.float64).reshape(4))
    L.call("cg_w_kernels", float(theta), w.ctypes.data_as(ctypes.c_void_p), nw, int(NpixFF),
           int(NpixKern), int(Qpx), int(bool(invert)), float(dl), float(dm),
           None if Tm is None else Tm.ctypes.data_as(ctypes.c_void_p), _p(out),
           int(dtype == CF), _p(wsb), nbytes, _p(st.t), stream())
    if status is None:
        st.check()
    return out


def aw_kernels(A, Wk, a1, a2, wi, dtype=CF, status=None):
    """AW kernels [nk, Q, Q, SA, SA] from A kernels [nA, SA, SA] and w kernels [nW, Q, Q, S, S]."""
    A = cuda_tensor(A, CD)
    Wk = cuda_tensor(Wk, CD)
    a1, a2, wi = (cuda_tensor(x, torch.int32) for x in (a1, a2, wi))
    nA, SA = A.shape[0], A.shape[-1]
    nW, Q, S = Wk.shape[0], Wk.shape[1], Wk.shape[-1]
    nk = a1.shape[0]
    st = status or Status()
    if status is None:
        st.reset()
    nbytes = L.lib().cg_aw_kernels_workspace_bytes(nk, SA, nW, Q, S)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = torch.empty((nk, Q, Q, SA, SA), dtype=dtype, device="cuda")
    L.call("cg_aw_kernels", _p(A), nA, SA, _p(Wk), nW, Q, S, _p(a1), _p(a2), _p(wi), nk,
           _p(out), int(dtype == CF), _p(ws), nbytes, _p(st.t), stream())
    if status is None:
        st.check()
    return out


class CapturedStep:
    """A stream-ordered sequence of library calls (e.g. plan + grid + degrid of
    one batch, or a major cycle's plan + fused degrid/grid) captured once in a
    CUDA graph and replayed: every w-plane or AW-kernel group is already one
    persistent launch, and the graph removes the host launch cost of the ~10
    launches per step.  ``fn`` must issue its work on the current stream and
    must not synchronise with the host (the tiled plan does not); its tensors
    are the graph's fixed inputs and outputs."""

    def __init__(self, fn, warmup=1):
        require_cuda()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(warmup):
                fn()
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="thread_local"):
            fn()

    def replay(self):
        self.graph.replay()


# --------------------------------------------------------------------------
# w-towers (examples/grid/grid.c:482-710)

def tower_keys(uvw, theta, chunk, wincrement, status):
    """(key int32 [n], chunk/plane-relative uvw float64 [n, 3], (ubmin, ubmax, vbmin,
    vbmax, wpmin, wpmax)) of cg_tower_keys."""
    uvw = cuda_tensor(uvw, torch.float64)
    n = uvw.shape[0]
    key = torch.empty(n, dtype=torch.int32, device="cuda")
    rel = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    dmm = torch.empty(6, dtype=torch.int32, device="cuda")
    hb = (ctypes.c_int32 * 6)()
    L.call("cg_tower_keys", _p(uvw), uvw.stride(0), n, float(theta), int(chunk),
           float(wincrement), _p(key), _p(rel), _p(dmm), hb, _p(status.t), stream())
    return key, rel, tuple(int(x) for x in hb)


def towers_combine(stack, theta, layer_w, chunk_first, status):
    """Per chunk, the sum of its layers' images / w_kernel_function(l, m, layer_w)."""
    S = stack.shape[-1]
    # keep the uploaded tables referenced until the launch is queued: a freed
    # temporary's block is handed to the next allocation
    lw = cuda_tensor(layer_w, torch.float64)
    cf = cuda_tensor(chunk_first, torch.int32)
    nchunks = int(cf.shape[0]) - 1
    out = torch.empty((nchunks, S, S), dtype=CF, device="cuda")
    L.call("cg_towers_combine", _p(stack), int(stack.shape[0]), S, float(theta), _p(lw),
           _p(cf), nchunks, _p(out), _p(status.t), stream())
    return out


def towers_add(sub, origin, grid):
    """grid += each chunk's sub-grid at its origin (x0, y0), inside the grid."""
    org = cuda_tensor(origin, torch.int32)
    L.call("cg_towers_add", _p(sub), int(sub.shape[0]), int(sub.shape[-1]), _p(org),
           int(grid.shape[-1]), _p(grid), stream())
    return grid


def towers_cut(grid, origin, S):
    """Each chunk's S x S sub-grid of grid at its origin, rolled for cg_fft_raw."""
    org = cuda_tensor(origin, torch.int32)
    nchunks = int(org.shape[0])
    out = torch.empty((nchunks, S, S), dtype=CF, device="cuda")
    L.call("cg_towers_cut", _p(grid), int(grid.shape[-1]), _p(org), nchunks, int(S), _p(out),
           stream())
    return out


def towers_expand(images, theta, layer_w, chunk_first, status):
    """Per layer, its chunk's image / w_kernel_function(l, m, layer_w), ready for a
    forward cg_fft_raw."""
    S = images.shape[-1]
    lw = cuda_tensor(layer_w, torch.float64)
    cf = cuda_tensor(chunk_first, torch.int32)
    out = torch.empty((int(lw.shape[0]), S, S), dtype=CF, device="cuda")
    L.call("cg_towers_expand", _p(images), S, float(theta), _p(lw), _p(cf),
           int(cf.shape[0]) - 1, _p(out), _p(status.t), stream())
    return out


# --------------------------------------------------------------------------
# AW-towers (examples/notebooks/awtowers.ipynb cells 17-22)

def awtower_keys(uvw, theta, chunk, wstep, a1, a2, nant, status):
    """(key int32 [n], chunk/plane-relative uvw [n, 3], (ubmin, ubmax, vbmin, vbmax,
    wpmin, wpmax)) of cg_awtower_keys."""
    uvw = cuda_tensor(uvw, torch.float64)
    a1 = cuda_tensor(a1, torch.int32)
    a2 = cuda_tensor(a2, torch.int32)
    n = uvw.shape[0]
    key = torch.empty(n, dtype=torch.int32, device="cuda")
    rel = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    dmm = torch.empty(6, dtype=torch.int32, device="cuda")
    hb = (ctypes.c_int32 * 6)()
    L.call("cg_awtower_keys", _p(uvw), uvw.stride(0), n, float(theta), int(chunk), float(wstep),
           _p(a1), _p(a2), int(nant), _p(key), _p(rel), _p(dmm), hb, _p(status.t), stream())
    return key, rel, tuple(int(x) for x in hb)


def awtowers_combine(stack, s, theta, corr, aimage, layer_a1, layer_a2, layer_w, chunk_first,
                     status):
    """Per chunk, the sum of its layers' cut images times corr, the antenna ratio and
    the inverse Fresnel factor (rolled, for fft_raw and towers_add)."""
    co = cuda_tensor(corr, torch.float32)
    ai = cuda_tensor(aimage, CF)
    a1 = cuda_tensor(layer_a1, torch.int32)
    a2 = cuda_tensor(layer_a2, torch.int32)
    lw = cuda_tensor(layer_w, torch.float64)
    cf = cuda_tensor(chunk_first, torch.int32)
    nchunks = int(cf.shape[0]) - 1
    out = torch.empty((nchunks, s, s), dtype=CF, device="cuda")
    L.call("cg_awtowers_combine", _p(stack), int(stack.shape[0]), int(s), float(theta), _p(co),
           _p(ai), int(ai.shape[0]), _p(a1), _p(a2), _p(lw), _p(cf), nchunks, _p(out),
           _p(status.t), stream())
    return out


def awtower_layers(used, nant, nwp, nub, ubmin, vbmin, chunk, margin, N):
    """(layer_a1, layer_a2, layer_plane [nlayers], chunk_first [nchunks + 1], origin
    [nchunks, 2]) as int32 CUDA tensors from the layers' ascending keys
    (cg_awtower_layers)."""
    used = cuda_tensor(used, torch.int32)
    nl = int(used.shape[0])
    a1, a2, lp = (torch.empty(nl, dtype=torch.int32, device="cuda") for _ in range(3))
    cf = torch.empty(nl + 1, dtype=torch.int32, device="cuda")
    org = torch.empty((nl, 2), dtype=torch.int32, device="cuda")
    ws = torch.empty(L.lib().cg_awtower_layers_workspace_bytes(nl), dtype=torch.uint8,
                     device="cuda")
    nc = ctypes.c_int32()
    L.call("cg_awtower_layers", _p(used), nl, int(nant), int(nwp), int(nub), int(ubmin),
           int(vbmin), int(chunk), int(margin), int(N), _p(a1), _p(a2), _p(lp), _p(cf), _p(org),
           ctypes.byref(nc), _p(ws), ws.numel(), stream())
    n = nc.value
    return a1, a2, lp, cf[:n + 1], org[:n]


def awtowers_direct(plan, ktab, vis, s, theta, corr, aimage, layer_a1, layer_a2, layer_plane,
                    plane_w, chunk_first, status):
    """awtowers_combine's output formed directly from the plan's sorted visibilities
    (cg_awtowers_direct; s = 16, 32 or 64): no layer grids, no layer transforms.
    layer_plane: each layer's index into plane_w, the w of each plane."""
    co = cuda_tensor(corr, torch.float32)
    ai = cuda_tensor(aimage, CF)
    a1 = cuda_tensor(layer_a1, torch.int32)
    a2 = cuda_tensor(layer_a2, torch.int32)
    lp = cuda_tensor(layer_plane, torch.int32)
    pw = cuda_tensor(plane_w, torch.float64)
    cf = cuda_tensor(chunk_first, torch.int32)
    nchunks = int(cf.shape[0]) - 1
    nant, nplanes = int(ai.shape[0]), int(pw.shape[0])
    out = torch.empty((nchunks, s, s), dtype=CF, device="cuda")
    ws = torch.empty(L.lib().cg_awtowers_direct_workspace_bytes(int(s), nant, nplanes),
                     dtype=torch.uint8, device="cuda")
    t = plan._table(ktab, CF)
    L.call("cg_awtowers_direct", plan.handle, _p(t), _p(vis), int(s), float(theta), _p(co),
           _p(ai), nant, _p(a1), _p(a2), _p(lp), _p(pw), nplanes, _p(cf), nchunks, _p(out),
           _p(ws), ws.numel(), _p(status.t), stream())
    return out


# --------------------------------------------------------------------------
# Sze-Tan optimal gridding functions

def szetan_gridding(h_ext, x0, R, kinv, nu):
    """calc_gridding_fine on the device: C [2R, M] (float64) at offsets nu."""
    h = cuda_tensor(h_ext, torch.float64)
    k = cuda_tensor(kinv, torch.float64)
    n = cuda_tensor(nu, torch.float64)
    M = int(n.shape[0])
    C = torch.empty((2 * R, M), dtype=torch.float64, device="cuda")
    L.call("cg_szetan_gridding", _p(h), int(h.shape[0]), float(x0), int(R), _p(k), _p(n), M,
           _p(C), stream())
    return C


def szetan_correction(C, R, x):
    """calc_gridding_correction_fine's c / d on the device for coordinates x, from C
    [2R, M] evaluated at nu_m = (m + 0.5) / (2M)."""
    Ct = cuda_tensor(C, torch.float64)
    xt = cuda_tensor(x, torch.float64)
    nx = int(xt.numel())
    out = torch.empty(nx, dtype=torch.float64, device="cuda")
    nbytes = L.lib().cg_szetan_correction_workspace_bytes(int(R))
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    L.call("cg_szetan_correction", _p(Ct), int(R), int(Ct.shape[1]), _p(xt), nx, _p(out), _p(ws),
           nbytes, stream())
    return out
