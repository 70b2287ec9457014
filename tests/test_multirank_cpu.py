"""The N > 1 path of bench.py on CPU with two gloo ranks: every rank gets its
own shard of work (independent seeded workloads), the reported time is the
slowest rank's (max over ranks), only rank 0 prints, and the reference arm
runs on rank 0 alone while the other ranks exit without work."""

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, %(root)r)
import torch, torch.distributed as dist
import bench
dist.init_process_group("gloo")
world, rank, local = bench.dist_env()
ms = [10.0, 12.5][rank]
agg = bench.max_over_ranks(ms, world, torch.device("cpu"))
w = bench.make_workload("wproj", rank)
print(json.dumps({"rank": rank, "world": world, "agg": agg, "n": len(w.uvw),
                  "first": [float(x) for x in w.uvw[0]]}), flush=True)
dist.barrier()
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(code, nproc=2, extra_args=()):
    port = _free_port()
    procs = []
    for r in range(nproc):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(nproc),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", code, *extra_args], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=300)
        assert p.returncode == 0, e[-2000:]
        outs.append(o)
    return outs


def test_max_over_ranks_two_gloo_ranks():
    pytest.importorskip("torch")
    outs = _launch(WORKER % {"root": ROOT})
    lines = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(l["rank"] for l in lines) == [0, 1]
    assert all(l["world"] == 2 and l["agg"] == 12.5 for l in lines)
    # each rank works on its own shard of the same size (weak scaling)
    assert lines[0]["n"] == lines[1]["n"] and lines[0]["first"] != lines[1]["first"]


def test_reference_arm_non_zero_rank_exits_without_work():
    pytest.importorskip("torch")
    code = ("import sys; sys.path.insert(0, %r); sys.argv = ['bench.py', '--impl', 'reference'];"
            "import bench, types; bench.run_reference(types.SimpleNamespace("
            "workload='aw', gpus=2, steps=1, warmup=1))" % ROOT)
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", CUDA_VISIBLE_DEVICES="")
    p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
