"""The multi-process (replicas) bench path on CPU: gloo, world size 2, 127.0.0.1.

The flow step does not shard (one instance needs halo exchanges and FFT
transposes), so ``bench.py`` under torchrun runs one independent replica per
rank: the job time is the slowest rank's, and rank 0 alone prints the line.
"""

from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _max_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, str(ROOT))
        import bench
        out[rank] = bench.max_over_ranks(1.5 + rank)
    finally:
        torch.distributed.destroy_process_group()


def test_max_over_ranks_gloo():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_max_worker, args=(2, port, out), nprocs=2, join=True)
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_max_over_ranks_without_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.25) == 3.25


@pytest.mark.timeout(300)
def test_reference_arm_under_torchrun_prints_one_line():
    """``--impl reference`` launched by torchrun with two ranks: rank 0 times the CPU path and prints
    the only JSON line; the other rank exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--workload", "cylinder2d", "--gpus", "2", "--steps", "3", "--warmup", "3", "--cpu-seconds", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=280, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
