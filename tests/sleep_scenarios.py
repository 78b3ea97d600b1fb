"""World scenarios driven through any world with the test interface (the
oracle, the reference harness, the GPU engine).

``scenarios()``: sleeping, after the reference's tests/world/sleeping_tests.cpp —
a settled stack on a static floor, wake-ups by every mutator, collisions and
support changes, property and gravity edits, quiet-time thresholds, and larger
settled scenes.  ``compound_scenarios()``: bodies with several colliders at
local transforms (PhysicsWorld::addCollider, physics_world.cpp:276-298, :658-667,
:679-686), the same-body pair filter (:629-633) and collider removal.

A scenario is a list of operations; ``run`` returns the observations taken at
each ("check",) operation: body state, sleep flags, step counters and contacts.
"""
from __future__ import annotations

import numpy as np

from phys_gb300 import scenes

DT = np.float32(1.0 / 120.0)
STAT_FIELDS = ("contact_count", "solved_contact_count", "awake_body_count", "sleeping_body_count",
               "prepared_points", "warm_start_comparisons", "warm_start_matches")


def _box(pos, static=False, size=(1.0, 1.0, 1.0)):
    return ("body", 1, list(size), list(pos), 1.0, 1 if static else 0, 0.0, 0.6)


# tests/world/sleeping_tests.cpp:53-68: floor, lower, upper, other
STACK = [_box((0, -0.5, 0), True, (10, 1, 10)), _box((0, 0.5, 0)), _box((0, 1.52, 0)), _box((3, 0.5, 0))]
FLOOR, LOWER, UPPER, OTHER = 0, 1, 2, 3


def _settled(sleeping=True):
    return [("sleep", sleeping)] + STACK + [("steps", 360), ("check",)]


def scenarios():
    out = {}
    out["opt_in"] = ([("sleep", False)] + STACK + [("steps", 360), ("check",), ("sleep", True), ("steps", 120),
                      ("check",), ("force", UPPER, (0, 0, 0)), ("steps", 600), ("check",), ("sleep", False),
                      ("check",), ("steps", 1), ("check",)], DT)
    for k, op in enumerate([("force", UPPER, (0.1, 0, 0)), ("vel", UPPER, (0.001, 0, 0), None),
                            ("vel", UPPER, None, (0, 0.001, 0)), ("wake", UPPER), ("force", UPPER, (1e-30, 0, 0))]):
        out[f"mutator_{k}"] = (_settled() + [op, ("check",), ("steps", 1), ("check",), ("steps", 20), ("check",)],
                               DT)
    out["collision_wake"] = (_settled() + [_box((0, 2.45, 0)), ("vel", 4, (0, -2, 0), None), ("steps", 1),
                                           ("check",), ("steps", 60), ("check",)], DT)
    out["retain_warm_start"] = (_settled() + [("steps", 600), ("force", UPPER, (1, 0, 0)), ("steps", 1),
                                              ("check",)], DT)
    out["remove_floor_body"] = (_settled() + [("remove_body", FLOOR), ("steps", 1), ("check",), ("steps", 30),
                                              ("check",)], DT)
    out["remove_floor_collider"] = (_settled() + [("remove_collider", FLOOR), ("steps", 1), ("check",),
                                                  ("steps", 30), ("check",)], DT)
    out["replace_lower"] = (_settled() + [("remove_body", LOWER), _box((20, 5, 0)), ("steps", 1), ("check",),
                                          ("steps", 30), ("check",)], DT)
    out["new_static"] = (_settled() + [_box((0, 2.45, 0), True), ("steps", 1), ("check",), ("steps", 30),
                                       ("check",)], DT)
    out["driven"] = ([("sleep", False)] + STACK + [("steps", 360), ("sleep", True)] +
                     [("force", UPPER, (0.001, 0, 0)), ("steps", 1)] * 180 + [("check",)], DT)
    for k, op in enumerate([("material", LOWER, 2.0, 0.6, 0.0), ("material", LOWER, 1.0, 0.0, 0.0),
                            ("material", LOWER, 1.0, 0.6, 1.0), ("gravity", (0, 0, 0))]):
        out[f"property_{k}"] = (_settled() + [op, ("steps", 1), ("check",), ("steps", 10), ("check",)], DT)
    # quiet time in simulated seconds and the inclusive speed thresholds
    # (sleeping_tests.cpp:114-170)
    for name, dt in (("quiet_60", np.float32(1.0 / 60.0)), ("quiet_120", DT)):
        half = int(round(0.5 / float(dt)))
        out[name] = ([("gravity", (0, 0, 0)), ("sleep", True), _box((0, 0, 0)), ("steps", half), ("check",),
                      ("steps", 2), ("check",), ("vel", 0, (0.1, 0, 0), None), ("steps", 120), ("check",),
                      ("vel", 0, (0, 0, 0), (0, 0.1, 0)), ("steps", 120), ("check",),
                      ("vel", 0, None, (0, 0, 0))] + [("force", 0, (0.001, 0, 0)), ("steps", 1)] * 120 +
                     [("check",), ("vel", 0, (0.0501, 0, 0), None), ("steps", 120), ("check",),
                      ("vel", 0, (0.05, 0, 0), (0, 0.05, 0)), ("steps", 120), ("check",)], dt)
    # the reference's settled-box profile scene (benchmarks/cpu_profile.cpp:20-41):
    # 512 unit boxes in 256 two-high stacks on one static floor
    stacks = [("sleep", True), _box((0, -0.5, 0), True, (30, 1, 20))]
    for row in range(16):
        for column in range(16):
            for level in range(2):
                stacks.append(_box((np.float32(-12.0) + np.float32(1.6) * np.float32(column),
                                    np.float32(0.5) + np.float32(1.02) * np.float32(level),
                                    np.float32(-9.0) + np.float32(1.2) * np.float32(row))))
    out["stacks_512"] = (stacks + [("steps", 120), ("check",), ("steps", 120), ("check",),
                                   ("force", 100, (2, 0, 0)), ("steps", 1), ("check",), ("steps", 60), ("check",)],
                         DT)
    # larger settled scenes: boxes resting on a plane, and a pyramid
    plane = scenes.generate(scenes.BOXES_ON_PLANE, 64, 3)
    out["boxes_on_plane"] = ([("sleep", True), ("scene", plane)] + [("steps", 40), ("check",)] * 4 +
                             [("force", 5, (3, 0, 0)), ("remove_body", 9), ("steps", 1), ("check",), ("steps", 40),
                              ("check",)], np.float32(1.0 / 60.0))
    pyramid = scenes.generate(scenes.PYRAMIDS_BOXES_ONLY, 1, 42)
    out["pyramid"] = ([("sleep", True), ("scene", pyramid)] + [("steps", 60), ("check",)] * 3 +
                      [_box((0.2, 25.0, 0.1)), ("vel", pyramid.count, (0, -5, 0), None)] +
                      [("steps", 30), ("check",)] * 3, np.float32(1.0 / 60.0))
    return out


def _quat(axis, angle):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    s = np.sin(angle / 2)
    return [float(axis[0] * s), float(axis[1] * s), float(axis[2] * s), float(np.cos(angle / 2))]


def _compound_bodies():
    """Dumbbells (a box with two spheres), L shapes (two boxes, one tilted) and
    crosses (a sphere with a long box at a tilted local rotation), dropped in a
    grid over a static floor; creation body index k is op index k."""
    ops = [_box((0, -0.5, 0), True, (40, 1, 40))]
    body = 1
    rng = np.random.default_rng(7)
    for i in range(4):
        for j in range(3):
            x, z = -6.0 + 4.0 * i, -4.0 + 4.0 * j
            y = 1.5 + 1.3 * ((i + j) % 3)
            kind = (i + j) % 3
            spin = [float(v) for v in rng.uniform(-0.4, 0.4, 3)]
            if kind == 0:
                ops += [("body", 1, [1.2, 0.3, 0.3], [x, y, z], 1.0, 0, 0.1, 0.5),
                        ("collider", body, 0, [0.35, 0, 0], [0.75, 0, 0], [0, 0, 0, 1]),
                        ("collider", body, 0, [0.3, 0, 0], [-0.75, 0.05, 0], _quat([0, 1, 0], 0.3))]
            elif kind == 1:
                ops += [("body", 1, [1.0, 0.4, 0.4], [x, y, z], 2.0, 0, 0.0, 0.6),
                        ("collider", body, 1, [0.2, 0.5, 0.2], [0.4, 0.5, 0], _quat([0, 0, 1], 0.5))]
            else:
                ops += [("body", 0, [0.3, 0, 0], [x, y, z], 1.5, 0, 0.2, 0.4),
                        ("collider", body, 1, [0.9, 0.08, 0.12], [0, 0.1, 0], _quat([1, 1, 0], 0.7))]
            ops.append(("spin", body, spin))
            body += 1
    return ops


def compound_scenarios():
    out = {}
    base = _compound_bodies()
    out["compound_drop"] = (base + [("steps", 40), ("check",)] * 5, np.float32(1.0 / 60.0))
    out["compound_remove_collider"] = (base + [("steps", 60), ("check",), ("remove_extra", 2), ("remove_extra", 4),
                                               ("steps", 1), ("check",), ("steps", 60), ("check",)],
                                       np.float32(1.0 / 60.0))
    out["compound_sleep"] = ([("sleep", True)] + base + [("steps", 100), ("check",)] * 4 +
                             [("force", 3, (5, 0, 0)), ("steps", 1), ("check",), ("steps", 60), ("check",)],
                             np.float32(1.0 / 60.0))
    return out


def all_scenarios():
    return {**scenarios(), **compound_scenarios()}


def _is_gpu(world):
    return type(world).__name__ == "GpuWorld"


def _handle(world, h):
    if _is_gpu(world):
        from phys_gb300.engine import Handle

        return Handle(int(h[0]), int(h[1]))
    return int(h[0])


def observe(world, removed=()):
    st = world.stats()
    b = world.bodies()
    for k in b:  # slots of removed bodies hold no state
        b[k][list(removed)] = 0
    sleeping = world.sleeping().astype(np.uint8)
    sleeping[list(removed)] = 0
    return {"pos": b["pos"], "quat": b["quat"], "lin": b["lin"], "ang": b["ang"], "sleeping": sleeping,
            "stats": np.array([int(st[f]) for f in STAT_FIELDS], np.uint64), "contacts": world.contacts()}


def run(world, ops, dt):
    handles = []
    extra = []  # (collider idx, gen) of added colliders, in order
    obs = []
    removed = set()
    gpu = _is_gpu(world)
    for op in ops:
        kind = op[0]
        if kind == "sleep":
            world.set_sleeping_enabled(op[1])
        elif kind == "gravity":
            world.set_gravity(op[1])
        elif kind == "body":
            handles.append(world.create_body(*op[1:]))
            removed.discard(int(handles[-1][0]))
        elif kind == "scene":
            handles.extend(list(world.load_scene(op[1])))
        elif kind == "steps":
            for _ in range(op[1]):
                world.step(dt)
        elif kind == "check":
            obs.append(observe(world, sorted(removed)))
        elif kind == "force":
            world.apply_force(_handle(world, handles[op[1]]), np.asarray(op[2], np.float32))
        elif kind == "vel":
            lin = None if op[2] is None else np.asarray(op[2], np.float32)
            ang = None if op[3] is None else np.asarray(op[3], np.float32)
            world.set_velocity(_handle(world, handles[op[1]]), lin, ang)
        elif kind == "wake":
            (world.wake_up if gpu else world.wake_body)(_handle(world, handles[op[1]]))
        elif kind == "material":
            world.set_material(_handle(world, handles[op[1]]), *op[2:])
        elif kind == "remove_body":
            h = handles[op[1]]
            world.remove_body(int(h[0]), int(h[1]))
            removed.add(int(h[0]))
        elif kind == "collider":
            h = handles[op[1]]
            extra.append(world.add_collider(int(h[0]), int(h[1]), op[2], np.asarray(op[3], np.float32),
                                            np.asarray(op[4], np.float32), np.asarray(op[5], np.float32)))
        elif kind == "remove_extra":
            c = extra[op[1]]
            world.remove_collider(int(c[0]), int(c[1]))
        elif kind == "spin":
            world.apply_spin(_handle(world, handles[op[1]]), np.asarray(op[2], np.float32))
        elif kind == "remove_collider":
            h = handles[op[1]]
            world.remove_collider(int(h[2]), int(h[3]))
        else:
            raise ValueError(kind)
    return obs
