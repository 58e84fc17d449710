"""The multi-GPU form on CPU: world_size 2 over gloo.

bench.py under torchrun runs independent replicas (one volume per rank per
step, no data-path collective): the slowest rank's time sets the whole-job
time (max over ranks), the whole-job rate counts every rank's volumes, and
the reference arm runs on rank 0 alone while the other ranks exit 0 without
work.  No GPU is used.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (r + 1) seconds for 10 steps and [2 + r, 1 - r / 2] in two other trials
        t = bench.max_over_ranks([rank + 1.0, 2.0 + rank, 1.0 - rank / 2], world, "cpu")
        out[rank] = (t, bench.whole_job_rate(world, 10, t[0]))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    for r in range(world):
        t, rate = out[r]
        assert t == [2.0, 3.0, 1.0]       # every rank sees the slowest rank's times
        assert rate == pytest.approx(10.0)  # 2 ranks x 10 volumes in 2 s


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun with 2 processes, rank 0 prints the reference arm's line
    and rank 1 prints nothing; both exit 0."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "plain_512_born", "--steps", "1", "--warmup", "0",
           "--ref-sample", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
