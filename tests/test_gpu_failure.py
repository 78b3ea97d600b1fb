"""Failure detection without a GPU fault: every spin-wait of the step kernels
(tile look-back, grid barrier, union retries, colouring passes) is bounded by a
runtime limit.  With the limit at one iteration the waits run out, the kernel
that waited returns at once, and the step fails with "a bounded wait timed
out" while the world keeps its state from before the step; with the default
limit restored the world steps on and matches the oracle bit for bit."""
import numpy as np
import pytest

from oracle import cpu
from test_gpu_parity import compare_worlds, island_mix_scene

pytestmark = pytest.mark.gpu

DT = 1 / 120


def test_bounded_wait_timeout_fails_the_step_and_the_world_recovers(gpu):
    # More than 4,096 manifolds: the multi-kernel solver (grid barriers in the
    # colouring and the sweeps) and multi-tile look-backs in the sort, the
    # scans and the narrowphase compaction.
    sc = island_mix_scene(10, 12)
    g = gpu.GpuWorld(algo=0, iterations=8)
    o = cpu.OracleWorld(algo=0, iterations=8, order_mode=1)
    g.load_scene(sc)
    o.load_scene(sc)
    for _ in range(3):
        g.step(DT)
        o.step(DT)
    compare_worlds(g, o, "before the forced timeouts")
    before = {k: v.copy() for k, v in g.bodies().items()}
    lib = gpu.lib()
    failures = 0
    try:
        gpu.check(lib.pe_debug_set_spin_limit(0, 1))
        for _ in range(4):
            try:
                g.step(DT)
            except Exception as e:  # noqa: BLE001 - the status and message are checked
                assert "a bounded wait timed out" in str(e), str(e)
                failures += 1
                continue
            o.step(DT)  # a step whose waits happened to finish in time
    finally:
        gpu.check(lib.pe_debug_set_spin_limit(0, 0))
    assert failures > 0
    if failures == 4:
        # every attempt failed: the bodies are exactly as before
        for k, v in g.bodies().items():
            assert np.array_equal(v.view(np.uint32), before[k].view(np.uint32)), k
    for s in range(4):
        g.step(DT)
        o.step(DT)
        compare_worlds(g, o, f"step {s} after the limit was restored")
    assert g.stats()["contact_count"] > 4096
