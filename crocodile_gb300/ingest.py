"""Visibility ingest: per-baseline blocks to the gridder's device arrays.

The reference keeps visibilities in HDF5 files with a group per baseline,
"vis/[a1]/[a2]", each holding ``frequency`` [nchan] (Hz), ``time`` [nrow],
``uvw`` [nrow, 3] (metres), ``antenna1``/``antenna2`` [nrow] and ``vis``
[nrow, nchan, npol] (KERNEL_WORK.md "Visibilities"; written by
arl/test_support.py:292-305, read by import_visibility_baselines_from_hdf5,
:368-394).  scripts/image_dataset.py:75-87 then flattens the blocks with
``collect_blocks``: block by block, row by row, channel by channel, uvw in
wavelengths (``Visibility.uvw_lambda``: uvw * frequency / c), src columns
(antenna1, antenna2, time, frequency) and the first polarisation.

Here:

* ``read_blocks(source)`` walks any h5py-like group tree (an ``h5py.File``
  where h5py is installed, or the directory container below) the way
  import_visibility_baselines_from_hdf5 does: members in name order, groups
  whose ``attrs['type'] == 'Visibility'`` are blocks, other groups are
  descended into.
* ``write_blocks(path, blocks)`` writes the same tree as directories with one
  ``.npy`` file per dataset and the group attributes in ``attrs.json`` (HDF5
  itself is not available in this build's image).
* ``Ingest`` flattens blocks on the device (``cg_ingest_blocks``): chunks of
  blocks are packed into two pinned host buffers in turn, copied on a copy
  stream and converted on the compute stream, so packing chunk i+1 on the
  host overlaps the copy and conversion of chunk i.  The result (device
  tensors) is bit-identical to collect_blocks: uvw_lambda by IEEE-rounded
  FP64 multiply and divide, src and vis copied.
"""

import concurrent.futures
import ctypes
import json
import os

import numpy
import torch

from . import _lib as L
from . import engine as E

C_LIGHT = 299792458.0  # m/s


class VisibilityBlock:
    """The columns of one arl Visibility (data_models.py:114-202) the
    imaging path reads."""

    def __init__(self, frequency, time, uvw, antenna1, antenna2, vis, weight=None, name=None):
        self.frequency = numpy.asarray(frequency, dtype=numpy.float64)
        self.time = numpy.asarray(time, dtype=numpy.float64)
        self.uvw = numpy.asarray(uvw, dtype=numpy.float64)
        self.antenna1 = numpy.asarray(antenna1)
        self.antenna2 = numpy.asarray(antenna2)
        self.vis = numpy.asarray(vis)
        self.weight = None if weight is None else numpy.asarray(weight)
        self.name = name
        nrow = self.uvw.shape[0]
        if self.uvw.shape != (nrow, 3) or self.vis.ndim != 3 or self.vis.shape[0] != nrow or \
                self.vis.shape[1] != len(self.frequency) or len(self.time) != nrow or \
                len(self.antenna1) != nrow or len(self.antenna2) != nrow:
            raise ValueError("inconsistent visibility block shapes")

    @property
    def nrow(self):
        return self.uvw.shape[0]

    @property
    def nchan(self):
        return len(self.frequency)

    @property
    def npol(self):
        return self.vis.shape[2]


# ------------------------------------------------------------------ container

class DirGroup:
    """A directory read like an h5py group: sub-directories are groups,
    ``<name>.npy`` files are datasets, ``attrs.json`` the attributes."""

    def __init__(self, path):
        self.path = path
        a = os.path.join(path, "attrs.json")
        self.attrs = json.load(open(a)) if os.path.exists(a) else {}

    def __iter__(self):
        names = []
        for n in os.listdir(self.path):
            p = os.path.join(self.path, n)
            if os.path.isdir(p):
                names.append(n)
            elif n.endswith(".npy"):
                names.append(n[:-4])
        return iter(sorted(names))

    def __contains__(self, name):
        return os.path.isdir(os.path.join(self.path, name)) or \
            os.path.exists(os.path.join(self.path, name + ".npy"))

    def __getitem__(self, name):
        p = os.path.join(self.path, name)
        if os.path.isdir(p):
            return DirGroup(p)
        return numpy.load(p + ".npy", mmap_mode="r")

    @property
    def name(self):
        return self.path


def _is_group(x):
    return hasattr(x, "attrs") and hasattr(x, "__iter__") and hasattr(x, "__getitem__") and \
        not hasattr(x, "shape")


def _read_block(grp, name):
    cols = {c: numpy.asarray(grp[c]) for c in ("frequency", "time", "uvw", "antenna1",
                                                "antenna2", "vis")}
    w = numpy.asarray(grp["weight"]) if "weight" in grp else None
    return VisibilityBlock(cols["frequency"], cols["time"], cols["uvw"], cols["antenna1"],
                           cols["antenna2"], cols["vis"], w, name=name)


def read_blocks(source):
    """Every visibility block under a group tree (an h5py File/Group, a
    DirGroup or a directory path), in the order of
    import_visibility_baselines_from_hdf5 (arl/test_support.py:368-394)."""
    grp = DirGroup(source) if isinstance(source, (str, os.PathLike)) else source
    out = []
    for name in grp:
        item = grp[name]
        if not _is_group(item):
            continue
        if item.attrs.get("type", "") == "Visibility":
            out.append(_read_block(item, getattr(item, "name", name)))
        else:
            out.extend(read_blocks(item))
    return out


def write_blocks(path, blocks):
    """Write blocks as vis/<antenna1>/<antenna2> groups (the reference's
    layout; the baseline's antennas from its first row) of a directory
    container; returns the group paths."""
    paths = []
    for b in blocks:
        p = os.path.join(path, "vis", str(int(b.antenna1[0])), str(int(b.antenna2[0])))
        os.makedirs(p, exist_ok=True)
        with open(os.path.join(p, "attrs.json"), "w") as f:
            json.dump({"type": "Visibility"}, f)
        for col in ("frequency", "time", "uvw", "antenna1", "antenna2", "vis"):
            numpy.save(os.path.join(p, col + ".npy"), getattr(b, col))
        if b.weight is not None and not numpy.all(b.weight == 1.0):
            numpy.save(os.path.join(p, "weight.npy"), b.weight)
        paths.append(p)
    return paths


# ------------------------------------------------------------------ device ingest

class VisBlockDesc(ctypes.Structure):
    _fields_ = [("row_start", ctypes.c_int64), ("freq_start", ctypes.c_int64),
                ("vis_start", ctypes.c_int64), ("out_start", ctypes.c_int64),
                ("nrow", ctypes.c_int32), ("nchan", ctypes.c_int32), ("npol", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


# cg_vis_block as a numpy record (filled for a whole chunk at once)
DESC_DTYPE = numpy.dtype([("row_start", "<i8"), ("freq_start", "<i8"), ("vis_start", "<i8"),
                          ("out_start", "<i8"), ("nrow", "<i4"), ("nchan", "<i4"),
                          ("npol", "<i4"), ("pad", "<i4")])
assert DESC_DTYPE.itemsize == ctypes.sizeof(VisBlockDesc)


def _align(n, a=256):
    return (n + a - 1) // a * a


class Ingest:
    """Device flattening of visibility blocks in chunks of about
    ``chunk_bytes`` of input, double-buffered through pinned host memory."""

    def __init__(self, chunk_bytes=64 << 20, workers=None):
        E.require_cuda()
        self.chunk_bytes = int(chunk_bytes)
        self.workers = int(workers or min(16, os.cpu_count() or 1))
        self._pool = concurrent.futures.ThreadPoolExecutor(self.workers)
        self._pinned = [None, None]
        self._dev = [None, None]
        self.copy_stream = torch.cuda.Stream()
        self.status = E.Status()

    def _buffers(self, nbytes):
        """Both pinned/device buffer pairs, at least nbytes each.  Grown only
        between runs (with the device idle): the kernels read the device
        buffers through raw pointers, which torch does not track."""
        if self._pinned[0] is None or self._pinned[0].numel() < nbytes:
            torch.cuda.synchronize()
            self._pinned = [torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
                            for _ in range(2)]
            self._dev = [torch.empty(nbytes, dtype=torch.uint8, device="cuda") for _ in range(2)]

    @staticmethod
    def _layout(bl):
        rows = sum(b.nrow for b in bl)
        nfreq = sum(b.nchan for b in bl)
        nvis = sum(b.vis.size for b in bl)
        off, pos = {}, 0
        for name, nbytes in (("uvw", rows * 24), ("time", rows * 8), ("a1", rows * 4),
                             ("a2", rows * 4), ("freq", nfreq * 8), ("vis", nvis * 16),
                             ("blocks", len(bl) * ctypes.sizeof(VisBlockDesc))):
            off[name] = pos
            pos += _align(max(nbytes, 1))
        return rows, nfreq, nvis, off, pos

    @staticmethod
    def _chunks(blocks, limit):
        chunk, size = [], 0
        for i, b in enumerate(blocks):
            nb = b.vis.size * 16 + b.nrow * 40 + b.nchan * 8
            if chunk and size + nb > limit:
                yield chunk
                chunk, size = [], 0
            chunk.append(i)
            size += nb
        if chunk:
            yield chunk

    def run(self, blocks, pol=0, dtype=E.CD, want_src=True, want_antennas=False):
        """dict of device tensors: uvw [n, 3] (wavelengths), vis [n] (dtype), and
        src [n, 4] (antenna1, antenna2, time, frequency) and/or int32 a1, a2."""
        counts = numpy.array([b.nrow * b.nchan for b in blocks], dtype=numpy.int64)
        starts = numpy.concatenate([[0], numpy.cumsum(counts)])
        n = int(starts[-1])
        out = {"uvw": torch.empty((n, 3), dtype=torch.float64, device="cuda"),
               "vis": torch.empty(n, dtype=dtype, device="cuda")}
        if want_src:
            out["src"] = torch.empty((n, 4), dtype=torch.float64, device="cuda")
        if want_antennas:
            out["a1"] = torch.empty(n, dtype=torch.int32, device="cuda")
            out["a2"] = torch.empty(n, dtype=torch.int32, device="cuda")
        comp = torch.cuda.current_stream()
        chunks = list(self._chunks(blocks, self.chunk_bytes))
        layouts = [self._layout([blocks[i] for i in idx]) for idx in chunks]
        if not chunks:
            return out
        self._buffers(max(lay[4] for lay in layouts))
        self.status.reset()
        h2d_done = [None, None]
        used = [None, None]
        for ci, idx in enumerate(chunks):
            k = ci % 2
            bl = [blocks[i] for i in idx]
            rows, nfreq, nvis, off, pos = layouts[ci]
            pinned, dev = self._pinned[k], self._dev[k]
            if h2d_done[k] is not None:
                h2d_done[k].synchronize()  # the copy out of this pinned buffer has finished
            hv = pinned.numpy()

            def view(name, dt, count):
                return hv[off[name]:off[name] + count * numpy.dtype(dt).itemsize].view(dt)

            nrow = numpy.array([b.nrow for b in bl], dtype=numpy.int64)
            nchan = numpy.array([b.nchan for b in bl], dtype=numpy.int64)
            nv = numpy.array([b.vis.size for b in bl], dtype=numpy.int64)
            desc = numpy.zeros(len(bl), dtype=DESC_DTYPE)
            desc["row_start"][1:] = numpy.cumsum(nrow)[:-1]
            desc["freq_start"][1:] = numpy.cumsum(nchan)[:-1]
            desc["vis_start"][1:] = numpy.cumsum(nv)[:-1]
            desc["out_start"] = starts[idx]
            desc["nrow"], desc["nchan"] = nrow, nchan
            desc["npol"] = [b.npol for b in bl]
            # the small columns: one concatenate each (a C loop over the blocks)
            numpy.concatenate([b.uvw.reshape(-1) for b in bl],
                              out=view("uvw", numpy.float64, rows * 3))
            numpy.concatenate([b.time for b in bl], out=view("time", numpy.float64, rows))
            numpy.concatenate([b.antenna1 for b in bl], out=view("a1", numpy.int32, rows),
                              casting="unsafe")
            numpy.concatenate([b.antenna2 for b in bl], out=view("a2", numpy.int32, rows),
                              casting="unsafe")
            numpy.concatenate([b.frequency for b in bl], out=view("freq", numpy.float64, nfreq))
            # the visibilities: one concatenate per worker over a range of blocks
            # (numpy releases the GIL inside the copy)
            vs = view("vis", numpy.complex128, nvis)
            vstart = numpy.concatenate([[0], numpy.cumsum(nv)])
            edges = numpy.linspace(0, len(bl), self.workers + 1).astype(int)

            def pack(lo, hi, bl=bl, vs=vs, vstart=vstart):
                if hi > lo:
                    numpy.concatenate([b.vis.reshape(-1) for b in bl[lo:hi]],
                                      out=vs[vstart[lo]:vstart[hi]], casting="unsafe")

            list(self._pool.map(lambda ab: pack(*ab), zip(edges[:-1], edges[1:])))
            view("blocks", numpy.uint8, desc.nbytes)[:] = desc.view(numpy.uint8)
            with torch.cuda.stream(self.copy_stream):
                if used[k] is not None:
                    self.copy_stream.wait_event(used[k])  # the kernel reading dev[k] is done
                dev[:pos].copy_(pinned[:pos], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(self.copy_stream)
            h2d_done[k] = ev
            comp.wait_event(ev)
            d = dev.data_ptr()
            vp = out["vis"].data_ptr()
            L.call("cg_ingest_blocks", ctypes.c_void_p(d + off["blocks"]), len(bl),
                   ctypes.c_void_p(d + off["uvw"]), ctypes.c_void_p(d + off["time"]),
                   ctypes.c_void_p(d + off["a1"]), ctypes.c_void_p(d + off["a2"]),
                   ctypes.c_void_p(d + off["freq"]), ctypes.c_void_p(d + off["vis"]), int(pol),
                   E._p(out["uvw"]), E._p(out.get("src")), E._p(out.get("a1")),
                   E._p(out.get("a2")), ctypes.c_void_p(vp), int(dtype == E.CF),
                   E._p(self.status.t), E.stream())
            u = torch.cuda.Event()
            u.record(comp)
            used[k] = u
        self.status.check()
        return out


def collect(blocks, pol=0, dtype=E.CD):
    """(uvw_lambda, src, vis) as numpy arrays, like collect_blocks of
    scripts/image_dataset.py:75-87, computed on the device."""
    r = Ingest().run(blocks, pol=pol, dtype=dtype)
    return r["uvw"].cpu().numpy(), r["src"].cpu().numpy(), r["vis"].cpu().numpy()
