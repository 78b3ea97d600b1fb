"""CPU tests of the multi-GPU replica path of bench.py: with world size 2 over
gloo, every rank gets the slowest rank's time and the whole-job throughput sums
the replicas; the reference arm runs on rank 0 only."""
import os
import subprocess
import sys

import pytest

import bench


def _rank(rank, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, 2, "cpu")
        q.put((rank, slowest, bench.replica_throughput(2, 1000, slowest)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_replica_throughput_gloo():
    import multiprocessing as mp
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert all(abs(r[2] - 2 * 1000 / 15.0) < 1e-9 for r in res)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, str(bench.REPO / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
