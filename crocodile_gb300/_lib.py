"""ctypes binding of libcrocodile_gb300.so (the C ABI in include/crocodile_gb300.h).

There is no fallback: if the shared library is missing or cannot be loaded,
every entry point raises.  Build it with ``crocodile_gb300.build.build()``
(or ``__graft_entry__.build()``).
"""

import ctypes
import os
import threading

from . import build as _build

c_int, c_int32, c_int64, c_double, c_size_t, c_void_p = (
    ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_size_t,
    ctypes.c_void_p)
P = c_void_p

CG_OK = 0
CG_ERR_ARG = -1
CG_ERR_RANGE = -2
CG_ERR_BOUNDS = -3
CG_ERR_INDEX = -4
CG_ERR_CUDA = -5
CG_ERR_WORKSPACE = -6
CG_ERR_TIMEOUT = -7
CG_STATUS_WORDS = 4
CG_NOALLOC_SCRATCH_BYTES = 16 << 20  # include/crocodile_gb300.h
CG_PLAN_TILED = 0
CG_PLAN_GROUPS = 1
CG_LAYOUT_WARP = 1
CG_LAYOUT_OWNER = 2
CG_LAYOUT_LANE = 3


class PlanOpts(ctypes.Structure):
    _fields_ = [("layers", c_int), ("layer", c_void_p), ("wstep", c_double), ("kmin", c_int),
                ("group", c_void_p), ("ngroups", c_int), ("tile", c_int)]


class KernelDesc(ctypes.Structure):
    _fields_ = [("sep", c_int), ("Q", c_int), ("S", c_int), ("G", c_int)]


class Tuning(ctypes.Structure):
    _fields_ = [("tile", c_int), ("chunk", c_int), ("rows", c_int), ("groups", c_int),
                ("layout", c_int), ("dvis", c_int)]


# name -> (restype, argtypes); the declarations of include/crocodile_gb300.h
SIGNATURES = {
    "cg_last_error": (ctypes.c_char_p, []),
    "cg_version": (c_int, []),
    "cg_status_reset": (c_int, [P, P]),
    "cg_status_check": (c_int, [P, P, P]),
    "cg_frac_coords": (c_int, [P, c_int64, c_double, c_int64, c_int, c_int, c_int, P, P, P, P,
                               P, P]),
    "cg_plan_workspace_bytes": (c_size_t, [c_int, c_int64, c_int, c_int,
                                           ctypes.POINTER(KernelDesc)]),
    "cg_plan_create": (c_int, [ctypes.POINTER(P), c_int, ctypes.POINTER(KernelDesc), c_int, c_int,
                               P, c_int64, c_double, P, c_int64, P, c_size_t, P, P]),
    "cg_plan_create_wbins": (c_int, [ctypes.POINTER(P), c_int, ctypes.POINTER(KernelDesc), c_int,
                                     c_int, P, c_int64, c_double, c_double, c_int, c_int64, P,
                                     c_size_t, P, P]),
    "cg_plan_workspace_bytes_ex": (c_size_t, [c_int, c_int64, c_int, c_int,
                                              ctypes.POINTER(KernelDesc), ctypes.POINTER(PlanOpts)]),
    "cg_plan_create_ex": (c_int, [ctypes.POINTER(P), c_int, ctypes.POINTER(KernelDesc), c_int,
                                  c_int, P, c_int64, c_double, P, c_int64,
                                  ctypes.POINTER(PlanOpts), P, c_size_t, P, P]),
    "cg_plan_layer_mean_w": (c_int, [P, P, c_int64, P, P, P]),
    "cg_compact_keys_workspace_bytes": (c_size_t, [c_int]),
    "cg_compact_keys": (c_int, [P, c_int64, c_int, P, P, P, P, c_size_t, P, P]),
    "cg_row_keys": (c_int, [P, c_int64, c_int64, c_double, c_int, c_int, P, c_int, P, P, P, P,
                            P]),
    "cg_aw_keys": (c_int, [P, c_int64, P, P, c_int64, c_int, c_double, c_int, c_int, P, P, P]),
    "cg_wstack_combine": (c_int, [P, c_int, c_int, c_double, P, P, P, P, P]),
    "cg_tower_keys": (c_int, [P, c_int64, c_int64, c_double, c_int, c_double, P, P, P, P, P, P]),
    "cg_towers_combine": (c_int, [P, c_int, c_int, c_double, P, P, c_int, P, P, P]),
    "cg_towers_add": (c_int, [P, c_int, c_int, P, c_int, P, P]),
    "cg_towers_cut": (c_int, [P, c_int, P, c_int, c_int, P, P]),
    "cg_towers_expand": (c_int, [P, c_int, c_double, P, P, c_int, P, P, P]),
    "cg_awtower_keys": (c_int, [P, c_int64, c_int64, c_double, c_int, c_double, P, P, c_int, P,
                                P, P, P, P, P]),
    "cg_awtowers_combine": (c_int, [P, c_int, c_int, c_double, P, P, c_int, P, P, P, P, c_int, P,
                                    P, P]),
    "cg_awtower_layers_workspace_bytes": (c_size_t, [c_int]),
    "cg_awtower_layers": (c_int, [P, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                  c_int, P, P, P, P, P, P, P, c_size_t, P]),
    "cg_awtowers_direct_workspace_bytes": (c_size_t, [c_int, c_int, c_int]),
    "cg_awtowers_direct": (c_int, [P, P, P, c_int, c_double, P, P, c_int, P, P, P, P, c_int, P,
                                   c_int, P, P, c_size_t, P, P]),
    "cg_ingest_blocks": (c_int, [P, c_int, P, P, P, P, P, P, c_int, P, P, P, P, P, c_int, P, P]),
    "cg_szetan_gridding": (c_int, [P, c_int, c_double, c_int, P, P, c_int, P, P]),
    "cg_szetan_correction_workspace_bytes": (c_size_t, [c_int]),
    "cg_szetan_correction": (c_int, [P, c_int, c_int, P, c_int, P, P, c_size_t, P]),
    "cg_recombine_create": (c_int, [c_int, c_int, P, c_int, c_int, c_int, c_int, c_int, c_int,
                                    P]),
    "cg_recombine_destroy": (c_int, [P]),
    "cg_recombine_sizes": (c_int, [P, P]),
    "cg_recombine_windows": (c_int, [P, P, P, P]),
    "cg_recombine_workspace_bytes": (c_size_t, [P, c_int, c_int]),
    "cg_recombine_facet_add": (c_int, [P, P, c_int, P, c_int, P, c_int, c_int, c_int, P, c_int,
                                       P, c_size_t, P, P]),
    "cg_recombine_facet_to_subgrids": (c_int, [P, P, c_int, P, c_int, P, c_int, P, c_int, P,
                                               c_size_t, P, P]),
    "cg_recombine_add_facet": (c_int, [P, P, c_int, c_int, c_int, c_int, P, P]),
    "cg_recombine_subgrids_to_facet": (c_int, [P, P, c_int, P, c_int, P, c_int, c_int, c_int, P,
                                               c_int, c_int, P, c_size_t, P, P]),
    "cg_plan_destroy": (c_int, [P]),
    "cg_set_tuning": (c_int, [ctypes.POINTER(Tuning)]),
    "cg_get_tuning": (c_int, [ctypes.POINTER(Tuning)]),
    "cg_plan_info": (c_int, [P, P]),
    "cg_plan_export": (c_int, [P, P, P, P, P]),
    "cg_grid": (c_int, [P, P, P, P, P]),
    "cg_grid_sparse": (c_int, [P, P, P, P, P]),
    "cg_grid_weighted": (c_int, [P, P, P, P, P, P]),
    "cg_degrid": (c_int, [P, P, P, P, P]),
    "cg_degrid_grid": (c_int, [P, P, P, P, c_int, P, P, P]),
    "cg_update_peak": (c_int, [c_int, c_int, P, c_size_t, ctypes.POINTER(c_double), P]),
    "cg_set_wait_limit": (c_int, [ctypes.c_longlong]),
    "cg_fft_timeouts": (c_int, [P, c_int]),
    "cg_get_wait_limit": (ctypes.c_longlong, []),
    "cg_grid_noalloc": (c_int, [ctypes.POINTER(KernelDesc), c_int, c_int, P, c_int64, c_double,
                                P, c_int64, P, P, P, P, P]),
    "cg_grid_fp64": (c_int, [P, P, P, P, P]),
    "cg_degrid_fp64": (c_int, [P, P, P, P, P]),
    "cg_grid_boxcar": (c_int, [P, c_int64, c_double, c_int64, P, P, c_int, c_int, P, P]),
    "cg_degrid_boxcar": (c_int, [P, c_int64, c_double, c_int64, P, P, c_int, c_int, P, P]),
    "cg_weights": (c_int, [P, c_int64, c_double, c_int64, c_int, P, P, P, P, P]),
    "cg_mirror_uvw": (c_int, [P, c_int64, c_int64, P, c_int, P]),
    "cg_make_hermitian": (c_int, [P, c_int, c_int, c_int, P]),
    "cg_fft": (c_int, [P, c_int, c_int, c_int, c_int, c_int, P, P]),
    "cg_fft_raw": (c_int, [P, c_int, c_int, c_int, c_int, c_int, P]),
    "cg_fft_rows_df": (c_int, [P, c_int64, c_int, c_int, P]),
    "cg_fft2_centred_df": (c_int, [P, c_int64, c_int, c_int, c_int, P]),
    "cg_recombine_set_fft": (c_int, [P, c_int]),
    "cg_image_from_grid": (c_int, [P, c_int, c_int, P, P, P]),
    "cg_scale_image": (c_int, [P, c_int64, P, P]),
    "cg_kernel_oversample_workspace_bytes": (c_size_t, [c_int, c_int, c_int, c_int]),
    "cg_kernel_oversample": (c_int, [P, c_int, c_int, c_int, c_int, c_int, P, c_int, P, c_size_t,
                                     P]),
    "cg_w_kernels_workspace_bytes": (c_size_t, [c_int, c_int, c_int]),
    "cg_w_kernels": (c_int, [c_double, P, c_int, c_int, c_int, c_int, c_int, c_double, c_double,
                             P, P, c_int, P, c_size_t, P, P]),
    "cg_aw_kernels_workspace_bytes": (c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    "cg_aw_kernels": (c_int, [P, c_int, c_int, P, c_int, c_int, c_int, P, P, P, c_int, P, c_int,
                              P, c_size_t, P, P]),
    "cg_w_bins": (c_int, [P, c_int64, c_int64, c_double, P, P, P, P, P]),
    "cg_w_bins_fixed": (c_int, [P, c_int64, c_int64, c_double, c_int, c_int, P, P, P]),
}

_lib = None
_lock = threading.Lock()


def library_path():
    return _build.LIB


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = library_path()
            if not os.path.exists(path):
                raise RuntimeError("libcrocodile_gb300.so is not built (%s); run "
                                   "crocodile_gb300.build.build() first" % path)
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def raise_for(rc, what=""):
    """Map a CG_ERR_* code to the exception the reference raises in that case."""
    if rc == CG_OK:
        return
    msg = lib().cg_last_error().decode(errors="replace")
    if what:
        msg = "%s: %s" % (what, msg)
    if rc == CG_ERR_RANGE:
        raise AssertionError(msg)
    if rc == CG_ERR_BOUNDS:
        raise ValueError(msg)
    if rc == CG_ERR_INDEX:
        raise IndexError(msg)
    if rc == CG_ERR_ARG:
        raise ValueError(msg)
    raise RuntimeError("%s (code %d)" % (msg, rc))


def call(name, *args):
    rc = getattr(lib(), name)(*args)
    raise_for(rc, name)
    return rc
