"""Autotuner of the tiled gridder/degridder launch shape.

Sweeps the grid tile edge, visibilities per work item, row residues per
gridder thread and thread groups per gridder CTA (``cg_tuning``) on the
caller's own visibilities, timing plan + grid + degrid with CUDA events, and
keeps the fastest.  Results are cached in a JSON file keyed by GPU name and a
workload signature (grid size, support, oversampling, kernel layout and the
visibility count rounded to a power of two), so later runs start tuned.
"""

import ctypes
import itertools
import json
import os
import threading

import torch

from . import _lib as L
from . import engine as E

CACHE = os.environ.get("CROCODILE_GB300_TUNING",
                       os.path.join(os.path.expanduser("~"), ".cache", "crocodile_gb300",
                                    "tuning.json"))
_lock = threading.Lock()


def set_tuning(tile=0, chunk=0, rows=0, groups=0, layout=0, dvis=0):
    t = L.Tuning(int(tile), int(chunk), int(rows), int(groups), int(layout), int(dvis))
    L.call("cg_set_tuning", ctypes.byref(t))


def get_tuning():
    t = L.Tuning()
    L.call("cg_get_tuning", ctypes.byref(t))
    return {"tile": t.tile, "chunk": t.chunk, "rows": t.rows, "groups": t.groups,
            "layout": t.layout, "dvis": t.dvis}


def effective_layout(ktab):
    """The gridder layout the library uses for this kernel table under the
    current tuning (the rule of layout_for in csrc/api.cu): the tuned layout
    (the lane layout only for S <= 16), or automatically the lane layout for
    non-separable tables with even S <= 16 and the warp layout otherwise."""
    lay = get_tuning()["layout"]
    if lay == L.CG_LAYOUT_LANE:
        return lay if ktab.S <= 16 else L.CG_LAYOUT_WARP
    if lay:
        return lay
    return L.CG_LAYOUT_LANE if (not ktab.sep and ktab.S <= 16 and ktab.S % 2 == 0) \
        else L.CG_LAYOUT_WARP


def signature(shape, ktab, n):
    n2 = 1 << max(0, int(n - 1).bit_length())
    return "H%d_W%d_S%d_Q%d_%s_n%d" % (shape[0], shape[1], ktab.S, ktab.Q,
                                       "sep" if ktab.sep else "4d", n2)


def _key(sig):
    return "%s|%s" % (torch.cuda.get_device_name(), sig)


def load_cached(sig):
    try:
        with open(CACHE) as f:
            return json.load(f).get(_key(sig))
    except (OSError, ValueError):
        return None


def _store(sig, entry):
    with _lock:
        try:
            with open(CACHE) as f:
                data = json.load(f)
        except (OSError, ValueError):
            data = {}
        data[_key(sig)] = entry
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = CACHE + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, CACHE)


def candidates(S, quick=False):
    """Launch shapes to try: the warp layout over tile edge, work-item size and
    warps per CTA; the owner layout over tile edge, rows per thread and groups;
    the lane layout (S <= 16) over tile edge, work-item size and degridder."""
    tiles = [t for t in ((32, 48) if quick else (16, 24, 32, 48, 64)) if t >= min(S, 16)]
    chunks = (0, 1024) if quick else (0, 512, 2048)
    out = []
    if S <= 16:
        # the lane layout, each with the tiled degridder (dvis 0) and the ring
        # degridder (dvis 3)
        for tile, chunk, dvis in itertools.product((16, 32) if quick else (16, 24, 32),
                                                   (512, 1024) if quick else (0, 512, 1024),
                                                   (0, 3)):
            out.append({"tile": tile, "chunk": chunk, "rows": 0, "groups": 0,
                        "layout": L.CG_LAYOUT_LANE, "dvis": dvis})
    for tile, chunk in itertools.product(tiles, chunks):
        for warps in ((8,) if quick else (4, 8)):
            out.append({"tile": tile, "chunk": chunk, "rows": 0, "groups": warps,
                        "layout": L.CG_LAYOUT_WARP})
        for r in (1, 2, 3, 4, 5, 8):
            if r > S:
                continue
            gpad = (S * ((S + r - 1) // r) + 31) // 32 * 32
            if gpad > 256:
                continue
            for groups in sorted({1, max(1, 256 // gpad)}):
                out.append({"tile": tile, "chunk": chunk, "rows": r, "groups": groups,
                            "layout": L.CG_LAYOUT_OWNER})
    return out


def time_config(cfg, uvw, lam, shape, ktab, kidx, vis, repeats=3):
    """Median device ms of plan + grid + degrid (CUDA events around plan creation
    and the two launches) with this tuning, or None if the shape does not run."""
    set_tuning(**cfg)
    grid = torch.zeros(shape, dtype=E.CF, device="cuda")
    out = torch.empty(uvw.shape[0], dtype=E.CF, device="cuda")
    times = []
    try:
        for i in range(repeats + 1):
            grid.zero_()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[0].record()
            plan = E.Plan(uvw, lam, shape, ktab, kidx)
            ev[1].record()
            plan.grid(ktab, vis, grid)
            ev[2].record()
            plan.degrid(ktab, grid, out)
            ev[3].record()
            torch.cuda.synchronize()
            plan.check()
            if i:
                times.append(tuple(ev[k].elapsed_time(ev[k + 1]) for k in range(3)))
            del plan
    except (RuntimeError, ValueError):
        return None
    times.sort(key=sum)
    p, g, d = times[len(times) // 2]
    return {"plan": p, "grid": g, "degrid": d, "total": p + g + d}


def tune(uvw, lam, shape, ktab, kidx, vis, cands=None, repeats=3, use_cache=True, verbose=False):
    """Best tuning for this workload; sets it process-wide and returns (config, table)."""
    sig = signature(shape, ktab, uvw.shape[0])
    if use_cache:
        hit = load_cached(sig)
        if hit:
            set_tuning(**hit["config"])
            return hit["config"], hit.get("table", [])
    table = []
    best, best_ms = None, float("inf")
    for cfg in (cands or candidates(ktab.S)):
        t = time_config(cfg, uvw, lam, shape, ktab, kidx, vis, repeats)
        table.append({"config": cfg, "ms": t})
        if verbose:
            print(cfg, t, flush=True)
        if t is not None and t["total"] < best_ms:
            best, best_ms = cfg, t["total"]
    if best is None:
        best = {"tile": 0, "chunk": 0, "rows": 0, "groups": 0, "layout": 0}
    set_tuning(**best)
    _store(sig, {"config": best, "ms": best_ms, "table": table})
    return best, table
