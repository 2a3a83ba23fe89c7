"""The multi-GPU path is replicas only (independent value sets or patterns per
GPU, no exchange): what bench.py adds for N ranks is the barrier, the max of
the per-rank step times and rank 0 alone printing.  Covered here with gloo
ranks on CPU (world size 2)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, value, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    q.put((rank, bench.max_over_ranks(world, value)))
    dist.destroy_process_group()


def test_step_time_is_max_over_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, [0.25, 0.5][r], q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 0.5, 1: 0.5}


def test_reference_arm_under_torchrun_prints_once():
    """`bench.py --impl reference` launched with torchrun over N ranks:
    rank 0 alone measures and prints one JSON line; every rank exits 0."""
    pytest.importorskip("torch.distributed.run")
    port = 30500 + os.getpid() % 1000
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--workload", "cotan", "--size", "12", "--steps", "3", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
