"""A small, self-contained run of the w-projection grid + degrid step, for profiling.

    python -m crocodile_gb300.bench_case [--nvis N] [--steps K] [--workload wproj|plain|aw]

Sets up the seeded workload (kernels generated once), then runs K steps of
plan (with fused w binning) + FP32 gridding + FP32 degridding on the current
GPU and prints the per-step time.  --tune runs the autotuner first.  Meant to run under ncu with a visibility count
that keeps the capture small.
"""

import argparse
import ctypes
import time

import numpy
import torch

from . import _lib as L
from . import configs
from . import engine as E
from . import synthesis


def setup(workload="wproj", nvis=500_000, seed=None):
    if workload == "aw":
        from . import awproj
        w = configs.aw() if seed is None else configs.aw(seed=seed)
        if nvis and nvis < len(w.uvw):
            w = configs.wproj_subset(w, nvis)
            w.params = dict(w.params, a1=w.params["a1"][:nvis], a2=w.params["a2"][:nvis])
        op = awproj.AWProjection(w.theta, w.lam, w.uvw, w.params["a1"], w.params["a2"],
                                 w.params["beams"], w.params["wstep"], w.params["NpixFF"])
        vis = torch.from_numpy(w.vis.astype(numpy.complex64)).to(op.uvw.device)
        return dict(w=w, uvw=op.uvw, vis=vis, st=op.status, kt=op.ktab, kmin=0, nk=0,
                    wstep=None, rows=op.rows)
    if workload == "wproj":
        w = configs.wproj(n=nvis) if seed is None else configs.wproj(seed=seed, n=nvis)
        wstep, npixff = w.params["wstep"], w.params["NpixFF"]
    else:
        w = configs.plain(n=nvis) if seed is None else configs.plain(seed=seed, n=nvis)
        wstep, npixff = None, None
    dev = torch.device("cuda", torch.cuda.current_device())
    uvw = torch.from_numpy(w.uvw).to(dev)
    vis = torch.from_numpy(w.vis.astype(numpy.complex64)).to(dev)
    st = E.Status()
    if wstep is not None:
        _, kmin, kmax = E.w_bins(uvw, wstep, st)
        table = E.w_kernels(w.theta, wstep * numpy.arange(kmin, kmax + 1).astype(float), npixff,
                            w.S, w.Q, dtype=E.CF)
        kt = E.KernelTable(table.reshape(-1), False, w.Q, w.S)
    else:
        kmin = kmax = 0
        aa = synthesis.anti_aliasing_function(w.N, 0, w.params["aa_c"])
        k1 = synthesis.kernel_oversample(aa, w.Q, w.S)
        kt = E.KernelTable.from_gcf(numpy.asarray(k1), 0, E.CF)
    return dict(w=w, uvw=uvw, vis=vis, st=st, kt=kt, kmin=kmin, nk=kmax - kmin + 1, wstep=wstep)


class Step:
    """One plan + grid + degrid step through the C ABI, reusing one workspace."""

    def __init__(self, ctx, fused=False):
        self.c = ctx
        self.fused = fused
        self.model = None
        w = ctx["w"]
        self.n = w.uvw.shape[0]
        self.N = w.N
        dev = ctx["uvw"].device
        self.kd = ctx["kt"].desc()
        lib = L.lib()
        self.ws_bytes = lib.cg_plan_workspace_bytes(L.CG_PLAN_TILED, self.n, self.N, self.N,
                                                    ctypes.byref(self.kd))
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.grid = torch.zeros((self.N, self.N), dtype=torch.complex64, device=dev)
        self.out = torch.empty(self.n, dtype=torch.complex64, device=dev)

    def __call__(self, uvw=None, vis=None, events=None):
        c = self.c
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        uvw = c["uvw"] if uvw is None else uvw
        vis = c["vis"] if vis is None else vis
        h = ctypes.c_void_p()
        if c["wstep"] is not None:
            L.call("cg_plan_create_wbins", ctypes.byref(h), L.CG_PLAN_TILED,
                   ctypes.byref(self.kd), self.N, self.N, P(uvw), uvw.stride(0), c["w"].lam,
                   c["wstep"], c["kmin"], self.n, P(self.ws), self.ws_bytes, P(c["st"].t), sp)
        else:
            rows = c.get("rows")
            L.call("cg_plan_create", ctypes.byref(h), L.CG_PLAN_TILED, ctypes.byref(self.kd),
                   self.N, self.N, P(uvw), uvw.stride(0), c["w"].lam,
                   None if rows is None else P(rows), self.n, P(self.ws), self.ws_bytes,
                   P(c["st"].t), sp)
        try:
            self.grid.zero_()
            if self.fused:
                if self.model is None:
                    self.model = torch.randn_like(self.grid)
                L.call("cg_degrid_grid", h, P(c["kt"].table), P(self.model), P(vis), 0,
                       P(self.out), P(self.grid), sp)
                return
            if events:
                events[0].record()
            L.call("cg_grid", h, P(c["kt"].table), P(vis), P(self.grid), sp)
            if events:
                events[1].record()
            L.call("cg_degrid", h, P(c["kt"].table), P(self.grid), P(self.out), sp)
            if events:
                events[2].record()
        finally:
            L.lib().cg_plan_destroy(h)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nvis", type=int, default=500_000)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--workload", default="wproj",
                    choices=["wproj", "plain", "aw", "fft", "wstack"],
                    help="fft: one --nvis x --nvis complex64 plane, centred inverse FFTs; "
                         "wstack: w-stacking imaging of 4096^2, 32 planes, 4M visibilities "
                         "(--nvis ignored)")
    ap.add_argument("--tune", action="store_true", help="autotune the launch shape first")
    ap.add_argument("--fused", action="store_true",
                    help="one degrid+grid pass (cg_degrid_grid) instead of two calls")
    ap.add_argument("--tuning", default="",
                    help="explicit launch shape tile,chunk,rows,groups,layout[,dvis] "
                         "(no autotuning)")
    a = ap.parse_args()
    if a.workload == "fft":  # one N x N complex64 plane (N = --nvis), centred inverse FFTs
        N = a.nvis
        rng = numpy.random.default_rng(N)
        g = torch.from_numpy((rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N)))
                             .astype(numpy.complex64)).cuda()
        E.fft_(g, True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            E.fft_(g, True)
        torch.cuda.synchronize()
        print("fft %d^2: %.3f ms per transform" % (N, 1e3 * (time.perf_counter() - t0) / a.steps))
        return
    if a.workload == "wstack":  # one batched w-stacking imaging call per step
        w = configs.wstack()
        aa = synthesis.anti_aliasing_function(w.N, 0, 8)
        kv = numpy.asarray(synthesis.kernel_oversample(aa, 8, 8))
        uvw = torch.from_numpy(w.uvw).cuda()
        vis = torch.from_numpy(w.vis).cuda()
        plane = w.params["plane"]
        synthesis.w_stack_imaging(w.theta, w.lam, uvw, None, vis, kv, plane)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            synthesis.w_stack_imaging(w.theta, w.lam, uvw, None, vis, kv, plane)
        torch.cuda.synchronize()
        print("wstack %s: %.3f ms per call" % (w.name, 1e3 * (time.perf_counter() - t0) / a.steps))
        return
    ctx = setup(a.workload, a.nvis)
    if a.tuning:
        from . import autotune
        autotune.set_tuning(*(int(x) for x in a.tuning.split(",")))
    elif a.tune:
        from . import autotune
        w = ctx["w"]
        kidx = ctx.get("rows")
        if ctx["wstep"] is not None:
            kidx, _, _ = E.w_bins(ctx["uvw"], ctx["wstep"], ctx["st"])
        best, _ = autotune.tune(ctx["uvw"], w.lam, (w.N, w.N), ctx["kt"], kidx, ctx["vis"],
                                cands=autotune.candidates(w.S, quick=True), use_cache=False)
        print("tuning", best)
    step = Step(ctx, a.fused)
    step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        step()
    torch.cuda.synchronize()
    ctx["st"].check()
    print("%s%s n=%d: %.3f ms/step" % (a.workload, " fused" if a.fused else "", a.nvis,
                                        1e3 * (time.perf_counter() - t0) / a.steps))


if __name__ == "__main__":
    main()
