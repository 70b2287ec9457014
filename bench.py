#!/usr/bin/env python
"""Benchmark: convolutional grid + degrid throughput (Mvis/s) on one GB300.

Default workload (--workload aw, the AW-projection configuration the target
is stated on): 8192^2 grid, theta 0.05, 16,128,000 visibilities of 64
antennas (2016 baselines x 125 hour angles x 64 channels, Earth-rotation
uvw), AW kernels = (A1 conv A2) conv W (support 16, oversampling 16) for
every distinct (w bin, antenna pair) -- 27,751 kernels, 14.5 GB resident in
HBM, generated once as the reference's kernel cache does and reported
separately.  --workload wproj: 4096^2 w-projection, 2M visibilities, S 15,
Q 8, 101 w-kernels.

One step = plan (bit-exact FP64 cell assignment, tile sort, work list) + FP32
tiled gridding + FP32 tiled degridding of all visibilities, inputs resident
in HBM.  The same line reports the plain FP64 form (complex128, FP64
atomics, one launch per w-plane), FP32-vs-FP64 errors, the fused
degrid+grid pass, end to end with host buffers, the roofline of the dominant
kernel, the other configurations and a single-core CPU baseline.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload aw|wproj]

--impl reference times the CPU oracle (a numpy restatement of the
reference's algorithm) on the host cores over bounded samples.
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

# One hardware work queue per stream for this process (read when CUDA
# initialises): with the default 8, the end-to-end pipeline's kernel stream
# and copy-out stream can share a queue, and each step's kernels then wait
# behind the last step's copy-out.  A value the caller set is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid+degrid Mvis/s per GB300, FP32 batched vs plain, at <=1e-5 rel err vs FP64"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="aw", choices=["aw", "wproj"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations' measurements")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(ms, world, device):
    """The slowest rank's time (each rank processes its own shard; the job is done when
    the last one is), by an all-reduce over the process group; ms itself at N = 1."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([float(ms)], device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def make_workload(name, rank=0):
    from crocodile_gb300 import configs
    if name == "aw":
        return configs.aw(seed=20261207 + rank)
    return configs.wproj(seed=20261204 + rank)


# --------------------------------------------------------------------------- CPU (oracle) arm

_CPU = {}


def _cpu_init(table, theta, lam, shared, lock):
    os.environ["OMP_NUM_THREADS"] = "1"
    _CPU.update(table=table, theta=theta, lam=lam, shared=shared, lock=lock)


def _cpu_shard(job):
    """Oracle grid + degrid of one visibility shard with a prepared kernel table; the
    shard grid is added into the shared grid under its lock (the pattern of
    scripts/image_dataset.py:190-219)."""
    uvw, vis, rows = job
    from oracle import crocodile_oracle as O
    table, lam = _CPU["table"], _CPU["lam"]
    N = int(round(_CPU["theta"] * lam))
    g = numpy.zeros((N, N), dtype=complex)
    x, xf, y, yf = O.frac_coords(g.shape, table.shape[1], uvw / lam)
    O.convgrid_indexed(table, False, g, x, xf, y, yf, rows, vis)
    v = O.convdegrid_indexed(table, False, g, x, xf, y, yf, rows)
    if _CPU["shared"] is not None:
        with _CPU["lock"]:
            numpy.frombuffer(_CPU["shared"].get_obj(), dtype=complex).reshape(N, N)[...] += g
    return len(v)


def recombine_cpu_facet_s():
    """Seconds of the numpy oracle's facet -> subgrid recombination per facet of
    the 'tiny' set (8192^2, facets 1280^2, 22 x 22 subgrids), 1 core: one facet
    with 1 and with 4 subgrid columns (all 22 rows each), per facet =
    t1 + 21 (t4 - t1) / 3 (the per-facet preparation once, then linear in columns)."""
    from oracle import crocodile_oracle as O
    from crocodile_gb300 import bench_configs as BC
    from crocodile_gb300.recombine import default_pswf
    N, sp, yB, yN, yP, xA, xM, xMxN = BC.RECOMBINE_TINY
    cfg = O.RecombineConfig(N, yB, yN, yP, xA, xM, xMxN, default_pswf(N, yN, xA, xM))
    fo, so = BC.recombine_layout(N, sp, yB, xA)
    rng = numpy.random.default_rng(11)
    facet = rng.standard_normal((yB, yB)) + 1j * rng.standard_normal((yB, yB))
    t = []
    for n1 in (1, 4):
        t0 = time.perf_counter()
        O.rc_facet_to_subgrids(cfg, facet, so, so[:n1])
        t.append(time.perf_counter() - t0)
    return t[0] + (len(so) - 1) * (t[1] - t[0]) / 3, "one 1280^2 facet with 1 and 4 of 22 " \
        "subgrid columns (%.2f s, %.2f s), extrapolated to 22 columns" % tuple(t)


def szetan_cpu_correction_s(h):
    """Seconds of the oracle's calc_gridding_correction_fine over 8192 pixels
    (gridder at 8192 offsets, R 3, x0 0.3), 1 core: 32 and 64 pixels timed,
    extrapolated linearly in pixels."""
    from oracle import crocodile_oracle as O
    x = (numpy.arange(8192) - 4096) / 8192
    t = []
    for k in (32, 64):
        t0 = time.perf_counter()
        O.sze_gridding_correction_fine(x[:k], numpy.asarray(h), 0.3, 8192, 3)
        t.append(time.perf_counter() - t0)
    per = (t[1] - t[0]) / 32
    return t[0] + (8192 - 32) * per, "32 and 64 of 8192 pixels (%.2f s, %.2f s), " \
        "extrapolated" % tuple(t)


def oracle_sample(name, w, sample):
    """(uvw, vis, rows, kernel table) of a bounded sample, kernels from the oracle.

    wproj: the first `sample` visibilities, one w-kernel per bin.  aw: all
    visibilities of the first baselines up to `sample`, one AW kernel per
    distinct (w bin, a1, a2) from the oracle's aw_kernel_fft (equal to
    aw_kernel_fn to rounding, batched over sub-kernels so large samples are
    affordable)."""
    from oracle import crocodile_oracle as O
    if name == "wproj":
        wstep, npff = w.params["wstep"], w.params["NpixFF"]
        uvw, vis = w.uvw[:sample], w.vis[:sample]
        k = numpy.round(uvw[:, 2] / wstep).astype(int)
        table = numpy.array([O.w_kernel(w.theta, wstep * kk, npff, w.S, w.Q)
                             for kk in range(k.min(), k.max() + 1)])
        return uvw, vis, k - k.min(), table
    a1, a2 = w.params["a1"], w.params["a2"]
    bl = a1.astype(numpy.int64) * w.params["nant"] + a2
    order = numpy.unique(bl)
    take = numpy.zeros(len(bl), bool)
    for b in order:
        take |= bl == b
        if take.sum() >= sample:
            break
    uvw, vis = w.uvw[take], w.vis[take]
    wstep, npff, beams = w.params["wstep"], w.params["NpixFF"], w.params["beams"]
    wbin = wstep * numpy.round(uvw[:, 2] / wstep)
    keys = numpy.column_stack([wbin, a1[take], a2[take]])
    uniq, rows = numpy.unique(keys, axis=0, return_inverse=True)
    akern = {a: O.kernel_oversample(beams[a], 1, 16)[0, 0]
             for a in numpy.unique(numpy.concatenate([a1[take], a2[take]]))}
    wkern = {kw: O.w_kernel(w.theta, kw, npff, 16, 16) for kw in numpy.unique(wbin)}
    table = numpy.array([O.aw_kernel_fft(akern[int(p)], akern[int(q)], wkern[kw])
                         for kw, p, q in uniq])
    return uvw, vis, rows.ravel(), table


class CpuArm:
    """The numpy oracle on `procs` host processes (spawned once, before timing)."""

    def __init__(self, name, w, sample, procs):
        self.uvw, self.vis, self.rows, table = oracle_sample(name, w, sample)
        self.sample, self.procs = len(self.uvw), procs
        self.pool = None
        if procs > 1:
            ctx = mp.get_context("spawn")
            shared = ctx.Array(ctypes.c_double, 2 * w.N * w.N)
            self.pool = ctx.Pool(procs, _cpu_init, (table, w.theta, w.lam, shared, ctx.Lock()))
            self.pool.map(_cpu_shard, [(self.uvw[:8], self.vis[:8], self.rows[:8])] * procs)
        else:
            _cpu_init(table, w.theta, w.lam, None, None)

    def measure(self):
        shards = numpy.array_split(numpy.arange(self.sample), self.procs)
        jobs = [(self.uvw[s], self.vis[s], self.rows[s]) for s in shards]
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


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    w = make_workload(args.workload)
    n = len(w.uvw)
    procs = os.cpu_count() or 1
    # size each step's sample so that all steps take about 90 s of host time
    probe = CpuArm(args.workload, w, min(n, 8000 * procs), procs)
    probe.measure()
    rate, _ = probe.measure()
    probe.close()
    steps, warm = min(args.steps, 20), max(args.warmup, 3)
    sample = int(min(n, max(2000 * procs, rate * 1e6 * 90.0 / max(steps + warm, 1))))
    arm = CpuArm(args.workload, w, sample, procs)
    rates, secs = [], []
    for i in range(steps + warm):
        r, dt = arm.measure()
        if i >= warm:
            rates.append(r)
            secs.append(dt)
    arm.close()
    value = statistics.median(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mvis/s",
        "n_gpus": args.gpus, "steps": len(rates), "warmup": warm,
        # one step is one bounded sample of the workload (its time as measured);
        # the whole set's time at the same rate is given beside it
        "ms_per_step": 1e3 * statistics.median(secs),
        "ms_full_set_at_this_rate": 1e3 * statistics.median(secs) * n / arm.sample,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded)",
        "config": {"workload": w.name, "n_vis": n, "N": w.N, "S": w.S, "Q": w.Q},
        "cpu_baseline": {"value": value, "unit": "Mvis/s", "cores": procs, "kind": "port",
                         "sample": "%d of %d visibilities per step (%s), grid+degrid, numpy "
                                   "oracle, %d spawned processes over visibility shards, shard "
                                   "grids summed into a shared grid under a lock; kernels "
                                   "generated once before timing"
                                   % (arm.sample, n, "all visibilities of the first baselines"
                                      if args.workload == "aw" else "first visibilities",
                                      procs)},
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
                 "--format=csv,noheader,nounits", "-lms", "20"],
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


class GpuWorkload:
    """Device-resident inputs, kernel table and the step closures of one workload."""

    def __init__(self, name, w):
        import torch
        from crocodile_gb300 import _lib as L
        from crocodile_gb300 import engine as E
        self.torch, self.L, self.E = torch, L, E
        self.name, self.w = name, w
        self.n, self.N, self.S, self.Q = len(w.uvw), w.N, w.S, w.Q
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.uvw = torch.from_numpy(w.uvw).to(self.dev)
        self.vis = torch.from_numpy(w.vis.astype(numpy.complex64)).to(self.dev)
        self.st = E.Status()
        self.stream = torch.cuda.current_stream()
        self.sp = ctypes.c_void_p(self.stream.cuda_stream)
        t0 = time.perf_counter()
        self._prepare()
        torch.cuda.synchronize()
        self.kgen_ms = 1e3 * (time.perf_counter() - t0)
        self.grid = torch.zeros((self.N, self.N), dtype=torch.complex64, device=self.dev)
        self.grid_out = torch.zeros_like(self.grid)
        self.out = torch.empty(self.n, dtype=torch.complex64, device=self.dev)

    @staticmethod
    def P(t):
        return ctypes.c_void_p(t.data_ptr()) if t is not None else None

    def _alloc_ws(self):
        kd = self.kt.desc()
        self.kd = kd
        self.ws_bytes = self.L.lib().cg_plan_workspace_bytes(self.L.CG_PLAN_TILED, self.n, self.N,
                                                             self.N, ctypes.byref(kd))
        self.ws = self.torch.empty(self.ws_bytes, dtype=self.torch.uint8, device=self.dev)

    def tune(self):
        from crocodile_gb300 import autotune
        t0 = time.perf_counter()
        self.tuned, _ = autotune.tune(self.uvw, self.w.lam, (self.N, self.N), self.kt,
                                      self.tune_kidx(), self.vis,
                                      cands=autotune.candidates(self.S, quick=True),
                                      use_cache=False)
        self.tune_s = time.perf_counter() - t0
        self._alloc_ws()

    def step(self, uvw, vis, kev=None, grid=None, out=None):
        """plan + grid + degrid, all stream-ordered (no host synchronisation), into
        self.grid / self.out or the given buffers."""
        L, P = self.L, self.P
        grid = self.grid if grid is None else grid
        out = self.out if out is None else out
        cur = self.torch.cuda.current_stream()  # the capture stream inside a CUDA graph
        self.sp = ctypes.c_void_p(cur.cuda_stream)
        h = ctypes.c_void_p()
        self.create_plan(h, uvw)
        grid.zero_()
        if kev:
            kev[0].record(cur)
        L.call("cg_grid", h, P(self.kt.table), P(vis), P(grid), self.sp)
        if kev:
            kev[1].record(cur)
        L.call("cg_degrid", h, P(self.kt.table), P(grid), P(out), self.sp)
        if kev:
            kev[2].record(cur)
        L.lib().cg_plan_destroy(h)

    def fused_step(self):
        L, P = self.L, self.P
        h = ctypes.c_void_p()
        self.create_plan(h, self.uvw)
        self.grid_out.zero_()
        L.call("cg_degrid_grid", h, P(self.kt.table), P(self.grid), P(self.vis), 0, P(self.out),
               P(self.grid_out), self.sp)
        L.lib().cg_plan_destroy(h)

    def kernel_bytes_per_vis(self):
        return 0

    def kernel_input_bytes(self):
        """Bytes of the kernel inputs the step starts from, as complex64."""
        return self.kt.table.numel() * 8

    def algorithmic_bytes_step(self):
        """Algorithmic bytes of one grid + degrid step, from the configuration's
        parameters rather than this implementation's traffic: per visibility its
        uvw (24 B), value in (8 B), kernel index (4 B) and predicted value out
        (8 B); the N^2 complex64 grid written once and read once; the kernel
        inputs."""
        return self.n * (24 + 8 + 4 + 8) + 2 * self.N * self.N * 8 + self.kernel_input_bytes()


class WProjGpu(GpuWorkload):
    def _prepare(self):
        E, w = self.E, self.w
        self.wstep, npff = w.params["wstep"], w.params["NpixFF"]
        _, self.kmin, kmax = E.w_bins(self.uvw, self.wstep, self.st)
        self.nk = kmax - self.kmin + 1
        self.wlist = self.wstep * numpy.arange(self.kmin, kmax + 1).astype(float)
        self.kt = E.KernelTable(E.w_kernels(w.theta, self.wlist, npff, self.S, self.Q,
                                            dtype=E.CF).reshape(-1), False, self.Q, self.S)
        self._alloc_ws()
        self.groups_desc = "one launch per w-plane (%d)" % self.nk

    def tune_kidx(self):
        return self.E.w_bins(self.uvw, self.wstep, self.st)[0]

    def create_plan(self, h, uvw):
        P = self.P
        self.L.call("cg_plan_create_wbins", ctypes.byref(h), self.L.CG_PLAN_TILED,
                    ctypes.byref(self.kd), self.N, self.N, P(uvw), 3, self.w.lam, self.wstep,
                    self.kmin, self.n, P(self.ws), self.ws_bytes, P(self.st.t), self.sp)

    def plain(self, steps):
        """(ms per plain FP64 step, FP32-vs-FP64 errors)."""
        E, torch = self.E, self.torch
        kt64 = E.KernelTable(E.w_kernels(self.w.theta, self.wlist, self.w.params["NpixFF"],
                                         self.S, self.Q, dtype=E.CD).reshape(-1), False, self.Q,
                             self.S)
        vis64 = torch.from_numpy(self.w.vis).to(self.dev)
        g64 = torch.zeros((self.N, self.N), dtype=torch.complex128, device=self.dev)
        kidx = self.tune_kidx()
        ms = []
        for i in range(steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            plan = E.Plan(self.uvw, self.w.lam, (self.N, self.N), kt64, kidx,
                          self.L.CG_PLAN_GROUPS, status=self.st)
            g64.zero_()
            plan.grid_fp64(kt64, vis64, g64)
            o64 = plan.degrid_fp64(kt64, g64)
            torch.cuda.synchronize()
            if i:
                ms.append(1e3 * (time.perf_counter() - t0))
        self.step(self.uvw, self.vis)
        o32 = E.Plan(self.uvw, self.w.lam, (self.N, self.N), self.kt, kidx,
                     status=self.st).degrid(self.kt, g64.to(torch.complex64))
        torch.cuda.synchronize()
        return statistics.mean(ms), _rel(self.grid, g64), _rel(o32, o64)


class AWGpu(GpuWorkload):
    def _prepare(self):
        from crocodile_gb300 import awproj
        w = self.w
        self.op = awproj.AWProjection(w.theta, w.lam, self.uvw, w.params["a1"], w.params["a2"],
                                      w.params["beams"], w.params["wstep"], w.params["NpixFF"],
                                      phase_ms=getattr(self, "phase_ms", None))
        self.kt, self.rows = self.op.ktab, self.op.rows
        self._alloc_ws()
        self.groups_desc = "one launch per w-plane (%d)" % self.op.nbins

    def tune_kidx(self):
        return self.rows

    def create_plan(self, h, uvw):
        P = self.P
        self.L.call("cg_plan_create", ctypes.byref(h), self.L.CG_PLAN_TILED, ctypes.byref(self.kd),
                    self.N, self.N, P(uvw), 3, self.w.lam, P(self.rows), self.n, P(self.ws),
                    self.ws_bytes, P(self.st.t), self.sp)

    def kernel_bytes_per_vis(self):
        return self.S * self.S * 8  # each visibility's AW kernel slice

    def kernel_input_bytes(self):
        """The A-kernels and the w sub-kernels the AW kernels are made from, as
        complex64 (the AW table itself is derived data)."""
        return (self.op.A.numel() + self.op.Wk.numel()) * 8

    def plain(self, steps):
        """(ms per plain FP64 step, FP32-vs-FP64 errors): the same AW kernels held as
        complex128, FP64 atomics, one launch per w-plane."""
        E, torch, op, w = self.E, self.torch, self.op, self.w
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op.enable_fp64()  # complex128 AW kernels, FP64 throughout, and the groups plan
        torch.cuda.synchronize()
        self.kgen64_ms = 1e3 * (time.perf_counter() - t0)
        vis64 = torch.from_numpy(w.vis).to(self.dev)
        g64 = torch.zeros((self.N, self.N), dtype=torch.complex128, device=self.dev)
        ms = []
        for i in range(steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            plan = E.Plan(self.uvw, w.lam, (self.N, self.N), op.ktab64, op.rows,
                          mode=self.L.CG_PLAN_GROUPS, status=self.st, groups=(op.nbins, op.wbin))
            g64.zero_()
            plan.grid_fp64(op.ktab64, vis64, g64)
            o64 = plan.degrid_fp64(op.ktab64, g64)
            torch.cuda.synchronize()
            if i:
                ms.append(1e3 * (time.perf_counter() - t0))
        self.step(self.uvw, self.vis)
        o32 = op.degrid(g64.to(torch.complex64))
        torch.cuda.synchronize()
        errs = (_rel(self.grid, g64), _rel(o32, o64))
        del g64, vis64, plan
        op.disable_fp64()
        torch.cuda.empty_cache()
        return (statistics.mean(ms),) + errs


def reference_api_imaging(G):
    """Seconds of do_imaging through the drop-in's reference API on the whole AW
    set: host numpy uvw, src = [a1, a2] and vis in, host dirty image and PSF out,
    kernel_cache = aw_kernel_fn(host A kernels, w_kernel) keyed on the device and
    generated in one batched pass; cold (kernel generation included) and warm
    (the AW table cached on the callable, as the reference's kernel cache)."""
    import torch
    from crocodile_gb300 import synthesis as S
    w = G.w
    beams, npff = w.params["beams"], w.params["NpixFF"]
    akern = {}

    def a_fn(theta, a):
        if a not in akern:
            akern[a] = S.kernel_oversample(beams[int(a)], 1, 16)[0, 0]
        return akern[a]

    fn = S.aw_kernel_fn(a_fn, lambda theta, ww: S.w_kernel(theta, ww, npff, 16, 16))
    src = numpy.column_stack([w.params["a1"], w.params["a2"]])
    out = {}
    for leg in ("cold", "warm"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d, p, pm = S.do_imaging(w.theta, w.lam, w.uvw, src, w.vis, S.w_cache_imaging,
                                wstep=w.params["wstep"], kernel_cache=fn)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[leg] = {"s": dt, "mvis_s": len(w.uvw) / dt / 1e6}
    del d, p, fn
    torch.cuda.empty_cache()
    out["form"] = ("synthesis.do_imaging(theta, lam, uvw, src=[a1, a2], vis, w_cache_imaging, "
                   "wstep, kernel_cache=aw_kernel_fn(a_kernel_fn, w_kernel_fn)) on all %d "
                   "visibilities, host numpy in and out (mirror, weights, image and PSF "
                   "gridding, hermitian FFTs, two 8192^2 float64 images back); host clock"
                   % len(w.uvw))
    return out


def update_peaks(G):
    """Measured grid-point update peaks (updates/s): shared-memory float2
    read-modify-write in the lane gridder's form, and float2 atomics into L2."""
    torch, L = G.torch, G.L
    buf = torch.empty(32 << 20, dtype=torch.uint8, device=G.dev)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {}
    for name, kind, work in (("smem", 0, 4096), ("red", 1, 4096)):
        u = ctypes.c_double()
        L.call("cg_update_peak", kind, work, G.P(buf), buf.numel(), ctypes.byref(u), sp)
        best = float("inf")
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            L.call("cg_update_peak", kind, work, G.P(buf), buf.numel(), ctypes.byref(u), sp)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[name] = u.value / (best * 1e-3)
    del buf
    return out


def _rel(a, b):
    import torch
    a, b = a.to(torch.complex128), b.to(torch.complex128)
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


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
    from crocodile_gb300 import autotune

    w = make_workload(args.workload, rank)
    G = (AWGpu if args.workload == "aw" else WProjGpu)(args.workload, w)
    G.tune()
    n, N, S, Q = G.n, G.N, G.S, G.Q
    stream = G.stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=G.dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    info_plan = G.E.Plan(G.uvw, w.lam, (N, N), G.kt, G.tune_kidx(), status=G.st).info()
    G.st.reset()
    for _ in range(max(args.warmup, 3)):
        G.step(G.uvw, G.vis)
    torch.cuda.synchronize()
    G.st.check()

    # ---- timed region (device-resident inputs): the step (plan + grid + degrid,
    # every kernel group in one persistent launch each) captured once in a CUDA
    # graph and replayed; eager launches if the capture is refused
    graph, launch = None, "CUDA graph"
    try:
        graph = G.E.CapturedStep(lambda: G.step(G.uvw, G.vis))
    except RuntimeError as e:
        launch = "eager (graph capture failed: %s)" % str(e).splitlines()[0][:120]
    run_step = graph.replay if graph else (lambda: G.step(G.uvw, G.vis))
    for _ in range(3):
        run_step()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = ev(), ev()
        e0.record(stream)
        run_step()
        e1.record(stream)
        times.append((e0, e1))
    torch.cuda.synchronize()
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
    ms = statistics.mean(a.elapsed_time(b) for a, b in times)
    G.st.check()
    # per-kernel split from eager launches of the same step
    te, tg, td = [], [], []
    for _ in range(min(args.steps, 20)):
        flush.zero_()
        e0, e1 = ev(), ev()
        kev = [ev(), ev(), ev()]
        e0.record(stream)
        G.step(G.uvw, G.vis, kev)
        e1.record(stream)
        te.append((e0, e1))
        tg.append((kev[0], kev[1]))
        td.append((kev[1], kev[2]))
    torch.cuda.synchronize()
    G.st.check()
    ms_eager = statistics.mean(a.elapsed_time(b) for a, b in te)
    del run_step, graph
    ms_grid = statistics.mean(a.elapsed_time(b) for a, b in tg)
    ms_degrid = statistics.mean(a.elapsed_time(b) for a, b in td)
    ms = max_over_ranks(ms, world, G.dev)
    value = world * n / (ms * 1e-3) / 1e6

    # ---- end to end through the C ABI with host buffers (pinned), copies timed
    h_uvw = torch.from_numpy(w.uvw).pin_memory()
    h_vis = torch.from_numpy(w.vis.astype(numpy.complex64)).pin_memory()
    h_grid = [torch.empty((N, N), dtype=torch.complex64).pin_memory() for _ in range(2)]
    h_out = [torch.empty(n, dtype=torch.complex64).pin_memory() for _ in range(2)]
    # Pipelined over steps: step i's inputs are copied in on one copy stream and
    # its grid and predicted visibilities copied out on another, each step into
    # and out of its own (double-buffered) device buffers, so that copies of
    # neighbouring steps overlap step i's kernels.  Every step still moves its
    # own inputs and results; the time is first copy-in to last copy-out.
    d_uvw = [G.uvw, torch.empty_like(G.uvw)]
    d_vis = [G.vis, torch.empty_like(G.vis)]
    d_grid = [G.grid, torch.empty_like(G.grid)]
    d_out = [G.out, torch.empty_like(G.out)]
    s_in, s_outs = torch.cuda.Stream(), torch.cuda.Stream()
    k_steps = min(args.steps, 20)

    kernel_spans = []

    def pipeline(k):
        in_ready = [ev(), ev()]
        done = [None, None]
        copied = [None, None]
        kernel_spans.clear()
        t0, t1 = ev(), ev()
        t0.record(s_in)
        for i in range(k):
            b = i % 2
            if done[b] is not None:
                s_in.wait_event(done[b])  # step i - 2 finished reading buffer b
            with torch.cuda.stream(s_in):
                d_uvw[b].copy_(h_uvw, non_blocking=True)
                d_vis[b].copy_(h_vis, non_blocking=True)
            in_ready[b] = ev()
            in_ready[b].record(s_in)
            stream.wait_event(in_ready[b])
            if copied[b] is not None:
                stream.wait_event(copied[b])  # step i - 2's results are out
            k0 = ev()
            k0.record(stream)
            G.step(d_uvw[b], d_vis[b], grid=d_grid[b], out=d_out[b])
            done[b] = ev()
            done[b].record(stream)
            kernel_spans.append((k0, done[b]))
            s_outs.wait_event(done[b])
            with torch.cuda.stream(s_outs):
                h_grid[b].copy_(d_grid[b], non_blocking=True)
                h_out[b].copy_(d_out[b], non_blocking=True)
            copied[b] = ev()
            copied[b].record(s_outs)
        t1.record(s_outs)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / k

    pipeline(2)  # warm-up
    ms_e2e = pipeline(k_steps)
    # each step's kernels as they ran inside the pipeline (copies alongside)
    ms_kernels_in_pipeline = statistics.mean(a.elapsed_time(b) for a, b in kernel_spans)

    def copies_alone():
        # one step's copy-in and copy-out, each alone on its stream (no kernels)
        c = [ev() for _ in range(4)]
        torch.cuda.synchronize()
        c[0].record(s_in)
        with torch.cuda.stream(s_in):
            d_uvw[1].copy_(h_uvw, non_blocking=True)
            d_vis[1].copy_(h_vis, non_blocking=True)
        c[1].record(s_in)
        torch.cuda.synchronize()
        c[2].record(s_outs)
        with torch.cuda.stream(s_outs):
            h_grid[1].copy_(d_grid[1], non_blocking=True)
            h_out[1].copy_(d_out[1], non_blocking=True)
        c[3].record(s_outs)
        torch.cuda.synchronize()
        return c[0].elapsed_time(c[1]), c[2].elapsed_time(c[3])

    ms_in, ms_out = copies_alone()
    h2d = h_uvw.numel() * 8 + h_vis.numel() * 8
    d2h = h_grid[0].numel() * 8 + h_out[0].numel() * 8
    e2e = {"value": world * n / (ms_e2e * 1e-3) / 1e6, "unit": "Mvis/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "ms_per_step": ms_e2e,
           "kernels_ms_in_pipeline": ms_kernels_in_pipeline,
           "copy_in_alone_ms": ms_in, "copy_in_gb_s": h2d / ms_in / 1e6,
           "copy_out_alone_ms": ms_out, "copy_out_gb_s": d2h / ms_out / 1e6,
           "form": "pipelined over %d steps: copy-in, kernels and copy-out on three streams, "
                   "double-buffered device inputs and results" % k_steps}
    G.st.check()
    del d_uvw, d_vis, d_grid, d_out

    # ---- fused form: plan + one pass that degrids the grid and grids the visibilities
    for _ in range(3):
        G.fused_step()
    fused_times = []
    for _ in range(min(args.steps, 50)):
        flush.zero_()
        e0, e1 = ev(), ev()
        e0.record(stream)
        G.fused_step()
        e1.record(stream)
        fused_times.append((e0, e1))
    torch.cuda.synchronize()
    G.st.check()
    ms_fused = statistics.mean(a.elapsed_time(b) for a, b in fused_times)

    # ---- plain FP64 form and accuracy of FP32 vs FP64 (full size)
    del flush
    torch.cuda.empty_cache()
    ms_plain, err_grid, err_degrid = G.plain(args.plain_steps)
    plain_value = n / (ms_plain * 1e-3) / 1e6

    # ---- the reference's own AW call through the drop-in: do_imaging(theta, lam,
    # uvw, src=[a1, a2], vis, w_cache_imaging, wstep, kernel_cache=aw_kernel_fn(...))
    # from host numpy arrays to host images (scripts/image_dataset.py:162-187)
    ref_api = None
    if args.workload == "aw" and world == 1:
        ref_api = reference_api_imaging(G)

    # ---- kernel generation again in the running process (libraries loaded,
    # FFT plans cached): what a new data set's kernel table costs after the first
    def allocator_counts():
        m = torch.cuda.memory_stats(G.dev)
        return {k: int(m.get(k, 0)) for k in ("num_device_alloc", "num_device_free",
                                               "num_alloc_retries")}

    def allocator_delta(a, b):
        return {k: b[k] - a[k] for k in a}

    torch.cuda.synchronize()
    c0 = allocator_counts()
    t0 = time.perf_counter()
    G._prepare()
    torch.cuda.synchronize()
    kgen_warm_ms = 1e3 * (time.perf_counter() - t0)
    kgen_warm_alloc = allocator_delta(c0, allocator_counts())
    # once more with the device synchronised at each phase boundary: host time
    # per phase (key binning and compaction with its readbacks, A-kernels,
    # w-kernels, the AW table, the plan)
    G.phase_ms = {}
    G._prepare()
    kgen_phases = {k: round(v, 3) for k, v in G.phase_ms.items()}
    G.phase_ms = None
    # the same again with the caching allocator holding the blocks of the last
    # table (no fresh device allocation), and a bare allocation of the table's
    # size after the cache is released: what separates the two warm figures
    torch.cuda.synchronize()
    c0 = allocator_counts()
    t0 = time.perf_counter()
    G._prepare()
    torch.cuda.synchronize()
    kgen_cached_ms = 1e3 * (time.perf_counter() - t0)
    kgen_cached_alloc = allocator_delta(c0, allocator_counts())
    tbytes = G.kt.table.numel() * 8
    torch.cuda.empty_cache()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    probe = torch.empty(tbytes, dtype=torch.uint8, device=G.dev)
    torch.cuda.synchronize()
    alloc_ms = 1e3 * (time.perf_counter() - t0)
    # writing the fresh allocation once, then again: what its first use costs
    fills = []
    for _ in range(2):
        t0 = time.perf_counter()
        probe.fill_(0)
        torch.cuda.synchronize()
        fills.append(1e3 * (time.perf_counter() - t0))
    del probe

    # ---- roofline of the dominant kernel: the step's algorithmic bytes (inputs
    # and outputs of grid + degrid from the configuration's parameters), half of
    # them per direction; the bytes this implementation streams per launch (the
    # kernel slice of every visibility) and the DRAM traffic ncu measured are
    # reported beside them
    alg_step = G.algorithmic_bytes_step()
    alg = alg_step / 2
    kbytes = G.kernel_bytes_per_vis()
    stream_bytes = n * (16 + 4 + 8 + kbytes) + N * N * 8 + (0 if kbytes
                                                            else G.kt.table.numel() * 8)
    dom = "grid" if ms_grid >= ms_degrid else "degrid"
    dom_ms = max(ms_grid, ms_degrid)
    tuned = G.tuned
    if dom == "grid":
        lay = autotune.effective_layout(G.kt)
        kname = {L.CG_LAYOUT_LANE: "k_lane", L.CG_LAYOUT_OWNER: "k_grid_tiled"}.get(lay,
                                                                                   "k_grid_warp")
    else:
        kname = "k_degrid_ring" if tuned.get("dvis") == 3 else "k_degrid_tiled"
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg / (dom_ms * 1e-3) / 1e9
    traffic = traffic_src = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tf):
        # captures are keyed by kernel and work-item size (the plan's chunk)
        chunk = info_plan["chunk"]
        recs = json.load(open(tf)).get(args.workload, {})
        entry = recs.get("%s/chunk%d" % (kname, chunk)) or next(
            (v for k, v in recs.items() if k.split("/")[0] == kname), None)
        if entry:
            traffic = entry["bytes_per_launch"]
            traffic_src = entry["source"]

    # ---- update rate: 2 n S^2 grid-point updates per step against the measured
    # shared-memory update and L2 atomic peaks (microbenchmarks of cg_update_peak)
    upeaks = update_peaks(G)
    urate = 2 * n * S * S / (ms * 1e-3)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        arm = CpuArm(args.workload, w, 200_000, 1)
        arm.measure()
        # repeated passes over the sample until about 10 s of host time
        rates, total = [], 0.0
        while total < 10.0 and len(rates) < 50:
            r, dt = arm.measure()
            rates.append(r)
            total += dt
        arm.close()
        cpu = {"value": statistics.mean(rates), "unit": "Mvis/s", "cores": 1, "kind": "port",
               "sample": "%d of %d visibilities (%s), grid+degrid, numpy oracle, 1 process, "
                         "%d passes in %.1f s; kernels generated once before timing"
                         % (arm.sample, n, "all visibilities of the first baselines"
                            if args.workload == "aw" else "first visibilities", len(rates),
                            total)}

    # the other configurations (each its own workload, timed the same way)
    cfg_results = None
    if rank == 0 and world == 1 and not args.no_configs:
        from crocodile_gb300 import bench_configs
        del G.ws
        torch.cuda.empty_cache()
        skip = {"aw"} if args.workload == "aw" else {"wproj"}
        cfg_results = bench_configs.run([k for k in bench_configs.MEASURES if k not in skip])
        autotune.set_tuning(**tuned)
        if not args.no_cpu_baseline:
            r = cfg_results.get("recombine")
            if r:
                sec, how = recombine_cpu_facet_s()
                r["cpu_oracle"] = {"s_per_facet": sec, "s_whole_image": sec * r["facets"],
                                   "cores": 1, "kind": "port", "sample": how}
                r["speedup_vs_cpu_oracle"] = sec * r["facets"] / (r["ms"] * 1e-3)
            g = cfg_results.get("ingest")
            if g:
                from oracle import crocodile_oracle as O
                blocks = bench_configs.ingest_blocks()[:200]
                t0 = time.perf_counter()
                O.collect_blocks(blocks)
                dt = time.perf_counter() - t0
                nb = sum(b.nrow * b.nchan for b in blocks)
                g["cpu_oracle"] = {"mvis_s": nb / dt / 1e6, "cores": 1, "kind": "port",
                                   "sample": "the first 200 of 2016 blocks (%d visibilities), "
                                             "numpy collect_blocks, %.2f s" % (nb, dt)}
            a = cfg_results.get("awtowers")
            if a:
                from oracle import crocodile_oracle as O
                wt, src, aimage = bench_configs.awtowers_workload()
                sel = numpy.isin(src[:, 0] * 16 + src[:, 1], [1, 2, 17])[:len(wt.uvw)]
                t0 = time.perf_counter()
                O.aw_towers_imaging(wt.theta, wt.lam, wt.uvw[sel], src[sel], wt.vis[sel], 64, 16,
                                    wt.params["wstep"], aimage)
                dt = time.perf_counter() - t0
                a["cpu_oracle"] = {"mvis_s": int(sel.sum()) / dt / 1e6, "cores": 1, "kind": "port",
                                   "sample": "3 of 120 baselines (%d visibilities), %.2f s"
                                             % (int(sel.sum()), dt)}
            z = cfg_results.get("szetan")
            if z:
                sec, how = szetan_cpu_correction_s(z["h"])
                z["cpu_oracle_correction_s"] = sec
                z["cpu_oracle_sample"] = how
                z["speedup_vs_cpu_oracle"] = sec / (z["ms_correction"] * 1e-3)

    # kernels of ours per step: coords, bucket scan (1 or 3), scatter, items per tile,
    # their scan (1 or 3), work items, (slice padding,) grid, degrid
    ntiles = (N // info_plan["tile"] + 1) ** 2 if info_plan["tile"] else 1
    per_step = 1 + (3 if info_plan["buckets"] > 4096 else 1) + 1 + 1 + \
        (3 if ntiles > 4096 else 1) + 1 + (1 if S * S % 2 and
                                           tuned.get("layout") == L.CG_LAYOUT_LANE else 0) + 2
    line = {
        "metric": METRIC, "value": value, "unit": "Mvis/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded numpy point-source visibilities)",
        "config": {"workload": w.name, "n_vis": n, "N": N, "S": S, "Q": Q,
                   "kernels": G.kt.G, "kernel_table_gb": round(G.kt.table.numel() * 8 / 1e9, 3),
                   "coordinates": "fp64 bit-exact",
                   "l2": "256 MiB written between timed steps (outside the step events)",
                   "tile": info_plan["tile"], "chunk": info_plan["chunk"],
                   "tuning": tuned, "tuning_seconds": round(G.tune_s, 2)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": kname,
                     "algorithmic_bytes": alg, "ms": dom_ms,
                     "algorithmic_bytes_def": "half of one grid+degrid step's n*(24 uvw + 8 vis "
                                              "+ 4 kernel index + 8 vis out) + 2*N^2*8 grid + "
                                              "kernel inputs (complex64)",
                     "step": {"algorithmic_bytes": alg_step, "ms": ms,
                              "achieved": alg_step / (ms * 1e-3) / 1e9,
                              "frac": alg_step / (ms * 1e-3) / 1e9 / peak},
                     "streamed_bytes_per_launch": stream_bytes,
                     "streamed_bytes_def": "n*(16 record + 4 index + 8 value + %d kernel slice) + "
                                           "N^2*8: what this gridder reads per launch" % kbytes,
                     "traffic_over_algorithmic": traffic / alg if traffic else None,
                     "traffic_source": traffic_src,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks
                     else "fallback 6800 GB/s"},
        "update_roofline": {"updates_per_s": urate, "updates_per_step": 2 * n * S * S,
                            "peak_smem_updates_per_s": upeaks["smem"],
                            "frac_of_smem_peak": urate / upeaks["smem"],
                            "peak_l2_atomic_updates_per_s": upeaks["red"],
                            "frac_of_l2_atomic_peak": urate / upeaks["red"],
                            "peak_source": "cg_update_peak microbenchmarks run in this process "
                                           "(shared-memory float2 read-modify-write in the lane "
                                           "gridder's form; float2 red.global.add into a 32 MiB "
                                           "L2-resident buffer), best of 5 CUDA-event timings"},
        "launch": launch, "ms_per_step_eager": ms_eager,
        "kernel_ms": {"grid": ms_grid, "degrid": ms_degrid,
                      "plan_and_grid_zeroing": ms_eager - ms_grid - ms_degrid,
                      "kernel_generation_once": G.kgen_ms,
                      "kernel_generation_warm": kgen_warm_ms,
                      "kernel_generation_warm_cached_blocks": kgen_cached_ms,
                      "kernel_generation_warm_allocator": kgen_warm_alloc,
                      "kernel_generation_warm_cached_blocks_allocator": kgen_cached_alloc,
                      "kernel_generation_warm_phases": kgen_phases,
                      "fresh_allocation_of_table_size": alloc_ms,
                      "fresh_allocation_first_fill_ms": fills[0],
                      "fresh_allocation_second_fill_ms": fills[1],
                      "kernel_generation_fp64": getattr(G, "kgen64_ms", None)},
        "plain_fp64": {"value": plain_value, "unit": "Mvis/s", "ms_per_step": ms_plain,
                       "form": "complex128, FP64 atomics, " + G.groups_desc},
        "speedup_vs_plain": value / plain_value,
        "rel_err_vs_fp64": {"grid": err_grid, "degrid": err_degrid,
                            "against": "the plain FP64 form with complex128 kernels generated "
                                       "in FP64 throughout (kernel generation error included)"},
        "fused": {"value": n / (ms_fused * 1e-3) / 1e6, "unit": "Mvis/s", "ms_per_step": ms_fused,
                  "form": "plan + one degrid+grid pass (cg_degrid_grid), each kernel tap read "
                          "once", "speedup_vs_plain": ms_plain / ms_fused},
        "e2e": e2e,
        "reference_api": ref_api,
        "cold_start": {"value": n / ((ms_e2e + G.kgen_ms) * 1e-3) / 1e6, "unit": "Mvis/s",
                       "ms": ms_e2e + G.kgen_ms,
                       "form": "one end-to-end step plus the one-off generation of the step's "
                               "kernel table (host clock around generation and upload)"},
        "gpu_launches": args.steps * per_step,
        "clocks": clk,
        "cpu_baseline": cpu,
        "configs": cfg_results,
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
