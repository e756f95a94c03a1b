"""bench.py with more than one rank, on the CPU: two gloo ranks on 127.0.0.1.

With N GPUs the bench runs N replicas of the step, one a rank, with no collective in the data
path. Only the timing crosses ranks: each rank times its own step, the job's time is the
slowest rank's, and the whole-job throughput counts every rank's points. The reference arm
runs on rank 0 alone, and the other ranks exit without work.
"""
from __future__ import annotations

import importlib.util
import multiprocessing as mp
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _load_bench():
    spec = importlib.util.spec_from_file_location("oeb_bench_dist", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    argv = sys.argv
    sys.argv = ["bench.py"]
    try:
        spec.loader.exec_module(mod)
    finally:
        sys.argv = argv
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = _load_bench()
        assert bench._dist_env() == (rank, world, rank)
        ms = 10.0 + 5.0 * rank  # rank 1 is the slower one
        got = bench._max_over_ranks(torch, ms, "cpu")
        dist.barrier()
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    codes = [p.exitcode for p in procs]
    for p in procs:
        if p.is_alive():
            p.kill()
    assert codes == [0, 0], codes
    got = dict(out.get(timeout=10) for _ in range(2))
    assert got == {0: 15.0, 1: 15.0}


def test_max_over_ranks_without_process_group():
    import torch
    bench = _load_bench()
    assert bench._max_over_ranks(torch, 3.25, "cpu") == 3.25


def test_replica_throughput_counts_every_rank():
    bench = _load_bench()
    pts = 10 * 128 * 128 * 80
    one = bench._replica_gpts(1, pts, 20, 13.0)
    assert one == pytest.approx(pts * 20 / 13.0e-3 / 1e9)
    # two replicas, each as fast: twice the job's points in the same (slowest-rank) time
    assert bench._replica_gpts(2, pts, 20, 13.0) == pytest.approx(2 * one)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    proc = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "3",
                           "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert proc.returncode == 0, proc.stderr
    assert proc.stdout.strip() == ""
