"""GPU tests of batched worlds: every world of a batch must equal the single-world
engine on the same bodies, step by step and bit for bit (bodies, candidate pairs,
contacts with impulses and feature ids, counters), and the CPU oracle in
graph-colour order."""
import numpy as np
import pytest

from helpers import assert_bit_equal, assert_manifolds_equal
from oracle import cpu
from phys_gb300 import scenes

pytestmark = pytest.mark.gpu

DT = 1 / 60
ITERATIONS = 10


def batch_scenes():
    # One world per size bucket and kind: a sparse field, resting boxes with
    # mixed friction/restitution, a sphere pile, a box pyramid (dense stacking:
    # its manifold count outgrows the initial per-world capacity), and a large
    # pile in the top bucket.
    return [
        scenes.generate(scenes.MIXED_VOLUME, 16, 43),
        scenes.generate(scenes.SPHERES_ON_FLOOR, 40, 3),
        scenes.generate(scenes.BOXES_ON_PLANE, 64, 5),
        scenes.generate(scenes.MIXED_VOLUME, 300, 44),
        scenes.generate(scenes.PYRAMIDS_BOXES_ONLY, 1, 7),
        scenes.generate(scenes.SPHERES_ON_FLOOR, 1200, 9),
    ]


def world_state(batch, w):
    pos, rot, lin, ang = batch.world_bodies(w)
    return {"pos": pos, "quat": rot, "lin": lin, "ang": ang}


def compare(batch, w, ref, what):
    gb, rb = world_state(batch, w), ref.bodies()
    for k in ("pos", "quat", "lin", "ang"):
        assert_bit_equal(gb[k], rb[k], f"{what} {k}")
    assert_bit_equal(batch.pairs(w), ref.pairs(), f"{what} pairs")
    assert_manifolds_equal(batch.contacts(w), ref.contacts(), what=what)


def test_batch_matches_single_world_engine_every_step(gpu):
    sc = batch_scenes()
    batch = gpu.GpuBatch(sc, iterations=ITERATIONS)
    worlds = []
    for s in sc:
        gw = gpu.GpuWorld(algo=gpu.SAP, iterations=ITERATIONS, order=gpu.ORDER_COLOR)
        gw.load_scene(s)
        worlds.append(gw)
    for step in range(40):
        batch.step(DT)
        for gw in worlds:
            gw.step(DT)
        for w, gw in enumerate(worlds):
            compare(batch, w, gw, f"step {step} world {w}")
            st, rst = batch.stats(w), gw.stats()
            for f in ("candidate_pairs", "contact_count", "solved_contact_count", "prepared_points",
                      "warm_start_matches", "warm_start_comparisons", "np_candidates", "np_contacts",
                      "color_count", "contact_points", "x_window_comparisons", "possible_pairs"):
                assert np.array_equal(st[f], rst[f]), f"step {step} world {w} {f}: {st[f]} != {rst[f]}"
    # resting boxes, the pyramid and the large sphere pile are in contact by now
    assert all(batch.stats(w)["contact_count"] > 0 for w in (2, 4, 5))


def test_batch_matches_oracle(gpu):
    sc = batch_scenes()[:5]
    batch = gpu.GpuBatch(sc, iterations=ITERATIONS)
    oracles = []
    for s in sc:
        ow = cpu.OracleWorld(algo=0, iterations=ITERATIONS, order_mode=1)
        ow.load_scene(s)
        oracles.append(ow)
    for step in range(30):
        batch.step(DT)
        for ow in oracles:
            ow.step(DT)
    for w, ow in enumerate(oracles):
        compare(batch, w, ow, f"world {w}")


def test_batch_graphs_autotune_and_direct_launches_agree(gpu):
    sc = batch_scenes()[1:4]
    a = gpu.GpuBatch(sc, iterations=ITERATIONS)
    b = gpu.GpuBatch(sc, iterations=ITERATIONS)
    b.set_graphs(False)
    a.step(DT, 5)
    a.autotune(DT, 2)
    tuned = a.buckets()
    assert np.all(tuned["tuned_ms"] > 0)
    assert np.all(tuned["threads"] > 0)
    b.step(DT, 5)
    a.step(DT, 20)
    b.step(DT, 20)
    for k in range(4):
        assert_bit_equal(a.bodies()[k], b.bodies()[k], f"bodies {k}")


def test_batch_forces_and_body_writes(gpu):
    sc = [scenes.generate(scenes.BOXES_ON_PLANE, 20, 1), scenes.generate(scenes.SPHERES_ON_FLOOR, 30, 2)]
    batch = gpu.GpuBatch(sc, iterations=ITERATIONS)
    worlds = []
    for s in sc:
        gw = gpu.GpuWorld(algo=gpu.SAP, iterations=ITERATIONS, order=gpu.ORDER_COLOR)
        gw.load_scene(s)
        worlds.append(gw)
    rng = np.random.default_rng(3)
    forces = rng.normal(0, 5, (batch.n, 3)).astype(np.float32)
    forces[batch.starts[:-1]] = 0  # floors are static; their force is ignored anyway
    batch.write_forces(forces)
    for w, gw in enumerate(worlds):
        gw.write_forces(forces[batch.starts[w]:batch.starts[w + 1]])
    for step in range(15):
        batch.step(DT)
        for gw in worlds:
            gw.step(DT)
    for w, gw in enumerate(worlds):
        compare(batch, w, gw, f"forces world {w}")
    pos = np.zeros((batch.n, 3), np.float32)
    rot = np.zeros((batch.n, 4), np.float32)
    batch.read_poses(pos, rot)
    assert_bit_equal(pos, batch.bodies()[0], "read_poses positions")
    assert_bit_equal(rot, batch.bodies()[1], "read_poses rotations")
    # pinned host arrays are read and written in place by the repacking kernels
    torch = pytest.importorskip("torch")
    pin = lambda count: torch.zeros(count, dtype=torch.float32).pin_memory().numpy()
    pf = pin(3 * batch.n).reshape(batch.n, 3)
    pf[:] = forces
    batch.write_forces(pf)
    for w, gw in enumerate(worlds):
        gw.write_forces(forces[batch.starts[w]:batch.starts[w + 1]])
    batch.step(DT)
    for gw in worlds:
        gw.step(DT)
    for w, gw in enumerate(worlds):
        compare(batch, w, gw, f"pinned forces world {w}")
    pp = pin(3 * batch.n).reshape(batch.n, 3)
    pq = pin(4 * batch.n + 1)[1:].reshape(batch.n, 4)  # not 16-byte aligned: written per float
    batch.read_poses(pp, pq)
    assert_bit_equal(np.array(pp), batch.bodies()[0], "pinned read_poses positions")
    assert_bit_equal(np.array(pq), batch.bodies()[1], "pinned read_poses rotations")
    # writing the state back unchanged leaves the next step identical
    p, q, l, a = batch.bodies()
    batch.write_bodies(p, q, l, a)
    batch.step(DT)
    for gw in worlds:
        gw.step(DT)
    for w, gw in enumerate(worlds):
        compare(batch, w, gw, f"rewritten world {w}")


def test_batch_rejects_invalid_input(gpu):
    with pytest.raises(ValueError):
        gpu.GpuBatch([scenes.generate(scenes.PYRAMIDS, 1, 1)])  # hulls are not batched
    big = scenes.generate(scenes.MIXED_VOLUME, 9000, 1)
    with pytest.raises(ValueError):
        gpu.GpuBatch([big])
