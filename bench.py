#!/usr/bin/env python
"""Benchmark: grid + degrid throughput (Mvis/s) of the w-projection workload on GB300.

Workload (seeded synthetic, the w_cache_imaging configuration): 4096^2 grid,
theta 0.1, 2M visibilities with 1/r radial uv density inside 0.45 lam and
|w| <= 500, w-kernels support 15, oversampling 8, w-step 10 (101 kernels,
NpixFF 64).  One step = w binning + plan (bit-exact coordinates, tile sort,
work list) + FP32 tiled gridding (w_cache_imaging) + FP32 tiled degridding
(w_cache_predict) of all visibilities, inputs resident in HBM.  Kernels are
generated once (a kernel cache, as the reference's pylru cache) and reported
separately.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU oracle (a numpy restatement of the
reference's algorithm) on the host cores over a bounded sample.
Prints one JSON line (rank 0).
"""

import argparse
import ctypes
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid+degrid Mvis/s per GB300, FP32 batched vs plain, at <=1e-5 rel err vs FP64"
WSTEP, NPIXFF = 10.0, 64


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nvis", type=int, default=2_000_000)
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-sample", type=int, default=400_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# --------------------------------------------------------------------------- CPU (oracle) arm

_CPU = {}


def _cpu_init(table, kmin, theta, lam, shared, lock):
    os.environ["OMP_NUM_THREADS"] = "1"
    _CPU.update(table=table, kmin=kmin, theta=theta, lam=lam, shared=shared, lock=lock)


def _cpu_shard(job):
    """Oracle grid + degrid of one visibility shard; the shard grid is added into
    the shared grid under its lock (the pattern of scripts/image_dataset.py:190-219)."""
    uvw, vis = job
    from oracle import crocodile_oracle as O
    table, kmin, lam = _CPU["table"], _CPU["kmin"], _CPU["lam"]
    N = int(round(_CPU["theta"] * lam))
    g = numpy.zeros((N, N), dtype=complex)
    k = numpy.round(uvw[:, 2] / WSTEP).astype(int) - kmin
    x, xf, y, yf = O.frac_coords(g.shape, table.shape[1], uvw / lam)
    O.convgrid_indexed(table, False, g, x, xf, y, yf, k, vis)
    v = O.convdegrid_indexed(table, False, g, x, xf, y, yf, k)
    if _CPU["shared"] is not None:
        with _CPU["lock"]:
            numpy.frombuffer(_CPU["shared"].get_obj(), dtype=complex).reshape(N, N)[...] += g
    return len(v)


class CpuArm:
    """The numpy oracle on `procs` host processes (spawned once, before timing)."""

    def __init__(self, w, sample, procs):
        from oracle import crocodile_oracle as O
        self.w, self.sample, self.procs = w, sample, procs
        self.uvw, self.vis = w.uvw[:sample], w.vis[:sample]
        k = numpy.round(self.uvw[:, 2] / WSTEP).astype(int)
        self.kmin, kmax = int(k.min()), int(k.max())
        self.table = numpy.array([O.w_kernel(w.theta, WSTEP * kk, NPIXFF, w.S, w.Q)
                                  for kk in range(self.kmin, kmax + 1)])
        self.pool = None
        if procs > 1:
            ctx = mp.get_context("spawn")
            self.shared = ctx.Array(ctypes.c_double, 2 * w.N * w.N)
            self.pool = ctx.Pool(procs, _cpu_init, (self.table, self.kmin, w.theta, w.lam,
                                                     self.shared, ctx.Lock()))
            self.pool.map(_cpu_shard, [(self.uvw[:8], self.vis[:8])] * procs)
        else:
            _cpu_init(self.table, self.kmin, w.theta, w.lam, None, None)

    def measure(self):
        shards = numpy.array_split(numpy.arange(self.sample), self.procs)
        jobs = [(self.uvw[s], self.vis[s]) for s in shards]
        t0 = time.perf_counter()
        if self.pool is None:
            _cpu_shard(jobs[0])
        else:
            self.pool.map(_cpu_shard, jobs)
        dt = time.perf_counter() - t0
        return self.sample / dt / 1e6, dt

    def close(self):
        if self.pool is not None:
            self.pool.close()
            self.pool.join()


def cpu_measure(w, sample, procs):
    arm = CpuArm(w, sample, procs)
    try:
        return arm.measure()
    finally:
        arm.close()


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from crocodile_gb300 import configs
    w = configs.wproj(n=args.nvis)
    procs = os.cpu_count() or 1
    # size each step's sample so that all K steps take about 90 s of host time
    probe = CpuArm(w, min(args.nvis, 4000 * procs), procs)
    probe.measure()
    rate, _ = probe.measure()
    probe.close()
    sample = int(min(args.nvis, max(2000 * procs, rate * 1e6 * 90.0 / max(args.steps, 1))))
    arm = CpuArm(w, sample, procs)
    rates, secs = [], []
    for i in range(args.steps + 1):
        r, dt = arm.measure()
        if i:  # the first pass is a warm-up
            rates.append(r)
            secs.append(dt)
    arm.close()
    value = statistics.median(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mvis/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.median(secs) * args.nvis / sample,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded)",
        "config": {"workload": w.name, "n_vis": args.nvis, "N": w.N, "S": w.S, "Q": w.Q,
                   "wstep": WSTEP, "NpixFF": NPIXFF},
        "cpu_baseline": {"value": value, "unit": "Mvis/s", "cores": procs, "kind": "port",
                         "sample": "%d of %d visibilities per step, grid+degrid, numpy oracle, "
                                   "%d spawned processes over visibility shards, shard grids "
                                   "summed into a shared grid under a lock"
                                   % (sample, args.nvis, procs)},
        "e2e": {"value": value, "unit": "Mvis/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- GPU arm

class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in out.strip().splitlines():
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, val in zip(names, f[3:7]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def run_ours(args):
    import torch
    import __graft_entry__
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    __graft_entry__.build()
    from crocodile_gb300 import _lib as L
    from crocodile_gb300 import configs
    from crocodile_gb300 import engine as E

    lib = L.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    w = configs.wproj(seed=20261204 + rank, n=args.nvis)
    n = w.uvw.shape[0]
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None

    uvw = torch.from_numpy(w.uvw).to(dev)
    vis = torch.from_numpy(w.vis.astype(numpy.complex64)).to(dev)
    st = E.Status()
    # kernel table for the bins present (generated once, reported separately)
    _, kmin, kmax = E.w_bins(uvw, WSTEP, st)
    nk = kmax - kmin + 1
    t0 = time.perf_counter()
    table = E.w_kernels(w.theta, WSTEP * numpy.arange(kmin, kmax + 1).astype(float), NPIXFF, w.S,
                        w.Q, dtype=E.CF)
    torch.cuda.synchronize()
    kgen_ms = 1e3 * (time.perf_counter() - t0)
    kt = E.KernelTable(table.reshape(-1), False, w.Q, w.S)
    kd = kt.desc()
    N = w.N
    kidx = torch.empty(n, dtype=torch.int32, device=dev)
    grid = torch.zeros((N, N), dtype=torch.complex64, device=dev)
    out = torch.empty(n, dtype=torch.complex64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    # launch-shape autotuning on this workload (outside the timed region)
    from crocodile_gb300 import autotune
    kidx_t, _, _ = E.w_bins(uvw, WSTEP, st)
    t0 = time.perf_counter()
    tuned, _ = autotune.tune(uvw, w.lam, (w.N, w.N), kt, kidx_t, vis,
                             cands=autotune.candidates(w.S, quick=True), use_cache=False)
    tune_s = time.perf_counter() - t0
    del kidx_t
    ws_bytes = lib.cg_plan_workspace_bytes(L.CG_PLAN_TILED, n, N, N, ctypes.byref(kd))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)

    def step(uvw_t, vis_t, kev=None):
        h = ctypes.c_void_p()
        L.call("cg_plan_create_wbins", ctypes.byref(h), L.CG_PLAN_TILED, ctypes.byref(kd), N, N,
               P(uvw_t), 3, w.lam, WSTEP, kmin, n, P(ws), ws_bytes, P(st.t), sp)
        grid.zero_()
        if kev:
            kev[0].record(stream)
        L.call("cg_grid", h, P(kt.table), P(vis_t), P(grid), sp)
        if kev:
            kev[1].record(stream)
        L.call("cg_degrid", h, P(kt.table), P(grid), P(out), sp)
        if kev:
            kev[2].record(stream)
        lib.cg_plan_destroy(h)

    info_plan = E.Plan(uvw, w.lam, (N, N), kt, status=st, wbins=(WSTEP, kmin)).info()
    st.reset()
    for _ in range(max(args.warmup, 3)):
        step(uvw, vis)
    torch.cuda.synchronize()
    st.check()

    # ---- timed region (device-resident inputs)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    times, tg, td = [], [], []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = ev(), ev()
        kev = [ev(), ev(), ev()]
        e0.record(stream)
        step(uvw, vis, kev)
        e1.record(stream)
        times.append((e0, e1))
        tg.append((kev[0], kev[1]))
        td.append((kev[1], kev[2]))
    torch.cuda.synchronize()
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
    ms = statistics.mean(a.elapsed_time(b) for a, b in times)
    ms_grid = statistics.mean(a.elapsed_time(b) for a, b in tg)
    ms_degrid = statistics.mean(a.elapsed_time(b) for a, b in td)
    st.check()
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n / (ms * 1e-3) / 1e6

    # ---- end to end through the C ABI with host buffers (pinned), copies timed
    h_uvw = torch.from_numpy(w.uvw).pin_memory()
    h_vis = torch.from_numpy(w.vis.astype(numpy.complex64)).pin_memory()
    h_grid = torch.empty((N, N), dtype=torch.complex64).pin_memory()
    h_out = torch.empty(n, dtype=torch.complex64).pin_memory()
    d_uvw = torch.empty_like(uvw)
    d_vis = torch.empty_like(vis)
    e2e_times = []
    for i in range(min(args.steps, 20) + 1):
        flush.zero_()
        e0, e1 = ev(), ev()
        e0.record(stream)
        d_uvw.copy_(h_uvw, non_blocking=True)
        d_vis.copy_(h_vis, non_blocking=True)
        step(d_uvw, d_vis)
        h_grid.copy_(grid, non_blocking=True)
        h_out.copy_(out, non_blocking=True)
        e1.record(stream)
        if i:
            e2e_times.append((e0, e1))
    torch.cuda.synchronize()
    ms_e2e = statistics.mean(a.elapsed_time(b) for a, b in e2e_times)
    e2e = {"value": world * n / (ms_e2e * 1e-3) / 1e6, "unit": "Mvis/s",
           "h2d_bytes_per_step": h_uvw.numel() * 8 + h_vis.numel() * 8,
           "d2h_bytes_per_step": h_grid.numel() * 8 + h_out.numel() * 8}

    # ---- plain FP64 form (one launch per w-plane) and accuracy of FP32 vs FP64
    kt64 = E.KernelTable(E.w_kernels(w.theta, WSTEP * numpy.arange(kmin, kmax + 1).astype(float),
                                     NPIXFF, w.S, w.Q, dtype=E.CD).reshape(-1), False, w.Q, w.S)
    vis64 = torch.from_numpy(w.vis).to(dev)
    g64 = torch.zeros((N, N), dtype=torch.complex128, device=dev)
    plain_ms = []
    for i in range(args.plain_steps + 1):
        e0, e1 = ev(), ev()
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        L.call("cg_w_bins_fixed", P(uvw), 3, n, WSTEP, kmin, nk, P(kidx), P(st.t), sp)
        plan64 = E.Plan(uvw, w.lam, (N, N), kt64, kidx, L.CG_PLAN_GROUPS, status=st)
        g64.zero_()
        plan64.grid_fp64(kt64, vis64, g64)
        o64 = plan64.degrid_fp64(kt64, g64)
        e1.record(stream)
        torch.cuda.synchronize()
        if i:
            plain_ms.append(1e3 * (time.perf_counter() - t0))
    st.check()
    plain_value = n / (statistics.mean(plain_ms) * 1e-3) / 1e6
    step(uvw, vis)
    torch.cuda.synchronize()
    err_grid = float(torch.linalg.vector_norm(grid.to(torch.complex128) - g64) /
                     torch.linalg.vector_norm(g64))
    o_ref = plan64.degrid_fp64(kt64, g64)
    o32 = E.Plan(uvw, w.lam, (N, N), kt, kidx, status=st).degrid(kt, g64.to(torch.complex64))
    err_degrid = float(torch.linalg.vector_norm(o32.to(torch.complex128) - o_ref) /
                       torch.linalg.vector_norm(o_ref))

    # ---- roofline of the gridder (dominant kernel): algorithmic bytes per launch
    S, Q = w.S, w.Q
    table_bytes = nk * Q * Q * S * S * 8
    grid_bytes = n * (16 + 4 + 8) + N * N * 8 + table_bytes
    degrid_bytes = n * (16 + 4 + 8) + N * N * 8 + table_bytes
    dom = "grid" if ms_grid >= ms_degrid else "degrid"
    dom_ms = max(ms_grid, ms_degrid)
    dom_bytes = grid_bytes if dom == "grid" else degrid_bytes
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tf):
        traffic = json.load(open(tf)).get("k_%s_tiled" % dom)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, dt = cpu_measure(w, min(args.cpu_sample, n), 1)
        cpu = {"value": rate, "unit": "Mvis/s", "cores": 1, "kind": "port",
               "sample": "%d of %d visibilities, grid+degrid, numpy oracle, 1 process, %.1f s"
                         % (min(args.cpu_sample, n), n, dt)}

    # kernels of ours per step: coords (with w bins), scan (1 or 3), scatter, work items,
    # grid, degrid
    per_step = 1 + (3 if info_plan["buckets"] > 4096 else 1) + 1 + 1 + 2
    line = {
        "metric": METRIC, "value": value, "unit": "Mvis/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded numpy point-source visibilities)",
        "config": {"workload": w.name, "n_vis": n, "N": N, "S": S, "Q": Q, "wstep": WSTEP,
                   "NpixFF": NPIXFF, "w_kernels": nk, "coordinates": "fp64 bit-exact",
                   "l2": "256 MiB written between timed steps (outside the step events)",
                   "tile": info_plan["tile"], "chunk": info_plan["chunk"],
                   "tuning": tuned, "tuning_seconds": round(tune_s, 2)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": "k_%s_tiled" % dom,
                     "algorithmic_bytes": dom_bytes, "ms": dom_ms,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks
                     else "fallback 6800 GB/s"},
        "kernel_ms": {"grid": ms_grid, "degrid": ms_degrid, "plan_and_bins": ms - ms_grid - ms_degrid,
                      "kernel_generation_once": kgen_ms},
        "updates_per_s": 2 * n * S * S / (ms * 1e-3),
        "plain_fp64": {"value": plain_value, "unit": "Mvis/s", "ms_per_step": statistics.mean(plain_ms),
                       "form": "complex128, FP64 atomics, one launch per w-plane (%d)" % nk},
        "speedup_vs_plain": value / plain_value,
        "rel_err_vs_fp64": {"grid": err_grid, "degrid": err_degrid},
        "e2e": e2e,
        "gpu_launches": args.steps * per_step,
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
