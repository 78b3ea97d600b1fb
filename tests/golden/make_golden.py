"""Generates the golden fixtures in tests/golden/ from the UNMODIFIED reference.

Run where the reference sources are present (it builds oracle/_ref with
`make -C oracle ref`):

    python tests/golden/make_golden.py

Each fixture stores its inputs together with the reference's outputs, so the
parity tests replay them anywhere (the GPU host has no reference sources).

Known-answer inputs restate the cases of the reference's own tests:
  broadphase  tests/collision/broadphase_tests.cpp:89-182
  narrowphase tests/collision/narrowphase_tests.cpp:35-182
  solver      tests/solver/sequential_impulse_solver_tests.cpp:24-291, 380-459
plus seeded random AABB sets / contact pairs, short seeded world runs and the
sleeping scenarios of tests/sleep_scenarios.py (tests/world/sleeping_tests.cpp).
`python tests/golden/make_golden.py sleeping` regenerates one fixture only.
"""
from __future__ import annotations

import math
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "phys-engine_gb300"))

from oracle import cpu  # noqa: E402
from phys_gb300 import scenes  # noqa: E402

F32MAX = np.float32(np.finfo(np.float32).max)


def aabb_cases():
    """Boundary / overflow AABB sets of broadphase_tests.cpp:89-182, then seeded
    random sets (30 scenes x 192 boxes, centres U[-20,20], half extents
    U[0.01,3], every third scene compressed, every third x-flattened)."""
    cases = []
    cases.append(np.zeros((0, 2, 3), np.float32))
    cases.append(np.array([[[0, 0, 0], [0, 0, 0]]], np.float32))
    cases.append(np.repeat(np.array([[[-1, -1, -1], [1, 1, 1]]], np.float32), 16, axis=0))
    cases.append(np.array([
        [[4, 0, 0], [5, 1, 1]], [[-2, -2, -2], [0, 0, 0]], [[0, 0, 0], [1, 1, 1]], [[1, 0, 0], [2, 1, 1]],
        [[1, 1, 0], [2, 2, 1]], [[1, 1, 1], [2, 2, 2]], [[0, 4, 0], [1, 5, 1]], [[0, 0, 4], [1, 1, 5]],
        [[1, 1, 1], [1, 1, 1]], [[-100, -0.5, -100], [100, 0, 100]]], np.float32))
    cases.append(np.repeat(np.array([[[-0.5, -0.5, -0.5], [0.5, 0.5, 0.5]]], np.float32), 2, axis=0))
    at = np.repeat(np.array([[[-0.5, -0.5, -0.5], [0.5, 0.5, 0.5]]], np.float32), 3, axis=0)
    cases.append(np.concatenate([at, np.array([[[0, 0, 0], [3, 3, 3]], [[0, 0, 0], [4, 3, 3]]], np.float32)]))
    cases.append(np.array([
        [[-0.5, -0.5, -0.5], [0.5, 0.5, 0.5]], [[0.5, -0.5, -0.5], [1.5, 0.5, 0.5]],
        [[-1.5, -0.5, -0.5], [-0.5, 0.5, 0.5]], [[-100000, -0.5, -100000], [100000, 0, 100000]],
        [[F32MAX, 0, 0], [F32MAX, 0, 0]], [[F32MAX, 0, 0], [F32MAX, 0, 0]],
        [[-2147483648.0, 0, 0], [-2147483648.0, 0, 0]], [[-2147483648.0, 0, 0], [-2147483648.0, 0, 0]]],
        np.float32))
    cases.append(np.array([[[-1, -1, -1], [1, 1, 1]], [[-F32MAX, -F32MAX, -F32MAX], [F32MAX, F32MAX, F32MAX]]],
                          np.float32))
    rng = np.random.default_rng(42)
    for scene in range(30):
        c = rng.uniform(-20, 20, (192, 3)).astype(np.float32)
        if scene % 3 == 0:
            c = c * np.float32(0.1)
        h = rng.uniform(0.01, 3.0, (192, 3)).astype(np.float32)
        lo, hi = c - h, c + h
        if scene % 3 == 1:
            lo[:, 0], hi[:, 0] = -1.0, 1.0
        cases.append(np.stack([lo, hi], axis=1).astype(np.float32))
    # -0 / +0 ties in the SAP sort key and touching-only overlaps
    cases.append(np.array([[[-0.0, 0, 0], [1, 1, 1]], [[0.0, 0, 0], [1, 1, 1]], [[1, 1, 1], [2, 2, 2]],
                           [[-0.0, -0.0, -0.0], [0.0, 0.0, 0.0]]], np.float32))
    return cases


def make_broadphase():
    cases = aabb_cases()
    out = {"count": np.array(len(cases))}
    for k, c in enumerate(cases):
        out[f"aabb_{k}"] = c
        for algo in (0, 1):
            pairs, st = cpu.broadphase("ref", c[:, 0], c[:, 1], algo)
            out[f"pairs_{k}_{algo}"] = pairs
            out[f"stats_{k}_{algo}"] = np.array([st["x_window_comparisons"], st["aabb_pairs"],
                                                 st["grid_comparisons"], st["grid_entries"],
                                                 st["grid_overflow_aabbs"]], np.uint64)
            out[f"cell_{k}_{algo}"] = np.array(st["grid_cell_size"], np.float64)
    np.savez_compressed(HERE / "broadphase.npz", **out)
    return len(cases)


def quat_axis_angle(axis, angle):
    """Quaternion::fromAxisAngle (include/phys/math/quaternion.hpp:18-22) in float."""
    half = np.float32(angle) * np.float32(0.5)
    s, c = np.float32(math.sin(half)), np.float32(math.cos(half))
    return np.array([axis[0] * s, axis[1] * s, axis[2] * s, c], np.float32)


def contact_cases():
    """(shape_a, dims_a, pos_a, quat_a, shape_b, dims_b, pos_b, quat_b) with
    dims = radius or half extents (narrowphase_tests.cpp:35-182) + seeded pairs."""
    ident = np.array([0, 0, 0, 1], np.float32)
    cases = [
        (0, [1, 0, 0], [0, 0, 0], ident, 0, [1, 0, 0], [1.5, 0, 0], ident),
        (1, [1, 1, 1], [0, 0, 0], quat_axis_angle([0, 0, 1], 1.57079632679), 0, [1, 0, 0], [0, 1.5, 0], ident),
        (1, [1, 1, 1], [0, 0, 0], quat_axis_angle([0, 1, 0], 0.4), 1, [1, 1, 1], [1.2, 0.8, 0.6],
         quat_axis_angle([1, 0, 0], 0.7)),
    ]
    for angle, height in ((0.3, 0.5 * (math.sin(0.3) + math.cos(0.3)) - 0.02), (0.1, 0.3)):
        floor = (1, [9, 0.5, 4], [0, -0.5, 0], quat_axis_angle([0, 0, 1], 0.0))
        box = (1, [0.5, 0.5, 0.5], [0, np.float32(height), 0], quat_axis_angle([0, 0, 1], angle))
        cases.append(floor + box)
        cases.append(box + floor)
    rng = np.random.default_rng(7)
    for _ in range(400):
        sa, sb = int(rng.integers(0, 2)), int(rng.integers(0, 2))
        dims = []
        for s in (sa, sb):
            dims.append([rng.uniform(0.2, 0.8), 0, 0] if s == 0 else list(rng.uniform(0.2, 0.8, 3)))
        qa = rng.normal(size=4)
        qa /= np.linalg.norm(qa)
        qb = rng.normal(size=4)
        qb /= np.linalg.norm(qb)
        pa = rng.uniform(-0.2, 0.2, 3)
        pb = pa + rng.uniform(-1.2, 1.2, 3)
        cases.append((sa, dims[0], pa, qa, sb, dims[1], pb, qb))
    # sphere centre inside a box (nearest-face branch) and coincident spheres
    cases.append((0, [0.3, 0, 0], [0.05, 0.01, -0.02], ident, 1, [0.5, 0.4, 0.6], [0, 0, 0], ident))
    cases.append((1, [0.5, 0.4, 0.6], [0, 0, 0], ident, 0, [0.3, 0, 0], [0, 0, 0], ident))
    cases.append((0, [0.5, 0, 0], [1, 2, 3], ident, 0, [0.25, 0, 0], [1, 2, 3], ident))
    return cases


def make_narrowphase():
    cases = contact_cases()
    n = len(cases)
    shapes = np.zeros((n, 2), np.int32)
    dims = np.zeros((n, 2, 3), np.float32)
    pos = np.zeros((n, 2, 3), np.float32)
    quat = np.zeros((n, 2, 4), np.float32)
    hits = np.zeros(n, np.uint8)
    manifolds = np.zeros(n, cpu.MANIFOLD_DTYPE)
    for k, (sa, da, pa, qa, sb, db, pb, qb) in enumerate(cases):
        shapes[k] = (sa, sb)
        dims[k, 0], dims[k, 1] = da, db
        pos[k, 0], pos[k, 1] = pa, pb
        quat[k, 0], quat[k, 1] = qa, qb
        hit, m = cpu.generate_contact("ref", sa, dims[k, 0], pos[k, 0], quat[k, 0], sb, dims[k, 1], pos[k, 1],
                                      quat[k, 1])
        hits[k] = hit
        manifolds[k] = m
    np.savez_compressed(HERE / "narrowphase.npz", shapes=shapes, dims=dims, pos=pos, quat=quat, hits=hits,
                        manifolds=manifolds)
    return n


def make_worlds():
    """Seeded scenes stepped through the reference PhysicsWorld (8 iterations,
    manifold order): final body state, contacts, candidate pairs and counters."""
    runs = [
        ("spheres_floor_sap", scenes.SPHERES_ON_FLOOR, 200, 0, 120),
        ("spheres_floor_grid", scenes.SPHERES_ON_FLOOR, 200, 1, 60),
        ("mixed_volume_sap", scenes.MIXED_VOLUME, 1500, 0, 40),
        ("mixed_volume_grid", scenes.MIXED_VOLUME, 1500, 1, 40),
        ("pyramid_sap", scenes.PYRAMIDS_BOXES_ONLY, 1, 0, 60),
        ("boxes_plane_sap", scenes.BOXES_ON_PLANE, 64, 0, 60),
        ("mixed_volume_tree", scenes.MIXED_VOLUME, 1500, 2, 40),
    ]
    for name, kind, n, algo, steps in runs:
        sc = scenes.generate(kind, n, 42)
        ref = cpu.RefWorld(algo=algo)
        ref.load_scene(sc)
        dt = np.float32(1.0 / 60.0)
        contacts_per_step = []
        for _ in range(steps):
            ref.step(dt)
            contacts_per_step.append(len(ref.contacts()))
        b = ref.bodies()
        st = ref.stats()
        mins, maxs = ref.bounds()
        # the standalone call rejects the tree; the tree reports the same
        # sorted pair set (dynamic_aabb_tree.cpp:306-327)
        pairs, _ = cpu.broadphase("ref", mins, maxs, 0 if algo == 2 else algo)
        np.savez_compressed(
            HERE / f"world_{name}.npz", algo=np.array(algo), steps=np.array(steps), dt=np.array(dt),
            shape=sc.shape, is_static=sc.is_static, dims=sc.dims, pos=sc.pos, density=sc.density,
            restitution=sc.restitution, friction=sc.friction, linvel=sc.linvel, spin=sc.spin,
            final_pos=b["pos"], final_quat=b["quat"], final_lin=b["lin"], final_ang=b["ang"],
            contacts=ref.contacts(), stats=np.array([st]), last_pairs=pairs,
            contacts_per_step=np.array(contacts_per_step, np.uint32))


def make_solver():
    """SequentialImpulseSolver::solve known answers (sequential_impulse_solver_tests.cpp)."""
    out = {}
    dt = np.float32(1.0 / 60.0)
    # off-centre contact (:24-73), restitution (:75-115)
    for name, rest, vel, anchor in (("offcenter", 0.0, -1.0, [1, 0, 0]), ("restitution", 0.5, -2.0, [0, 0, 0])):
        w = cpu.RefWorld()
        w.create_body(1, [2, 2, 2], [0, 0, 0], 1.0, 1, 0.0, 0.0)
        w.create_body(1, [2, 2, 2], [0, 0, 0], 1.0, 0, rest, 0.0)
        w.set_velocity(1, [0, vel, 0], None)
        m = np.zeros(1, cpu.MANIFOLD_DTYPE)
        m["body_a_index"], m["body_b_index"] = 0, 1
        m["normal"] = [0, 1, 0]
        m["point_count"] = 1
        m["restitution"] = rest
        m["anchor_a"][0, 0] = anchor
        m["anchor_b"][0, 0] = anchor
        solved, _ = w.solve(m, dt)
        b = w.bodies()
        out[f"{name}_in"] = m
        out[f"{name}_out"] = solved
        out[f"{name}_lin"] = b["lin"]
        out[f"{name}_ang"] = b["ang"]
        out[f"{name}_rest"] = np.array(rest, np.float32)
        out[f"{name}_vel"] = np.array(vel, np.float32)
    np.savez_compressed(HERE / "solver.npz", **out)


def make_sleeping():
    """Sleeping scenarios (tests/sleep_scenarios.py, after
    tests/world/sleeping_tests.cpp and benchmarks/cpu_profile.cpp): every
    observation of the reference world, scenario by scenario."""
    sys.path.insert(0, str(REPO / "tests"))
    import sleep_scenarios as ss

    out = {}
    for name, (ops, dt) in ss.all_scenarios().items():
        obs = ss.run(cpu.RefWorld(), ops, dt)
        out[f"{name}__checks"] = np.array(len(obs), np.uint32)
        for k, o in enumerate(obs):
            for f, v in o.items():
                out[f"{name}__{k}__{f}"] = v
    np.savez_compressed(HERE / "sleeping.npz", **out)


def main():
    cpu.build_reference()
    only = set(sys.argv[1:])
    if not only or "broadphase" in only:
        print("broadphase cases:", make_broadphase())
    if not only or "narrowphase" in only:
        print("narrowphase cases:", make_narrowphase())
    if not only or "solver" in only:
        make_solver()
    if not only or "worlds" in only:
        make_worlds()
    if not only or "sleeping" in only:
        make_sleeping()
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
