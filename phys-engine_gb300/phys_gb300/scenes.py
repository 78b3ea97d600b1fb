"""Seeded synthetic scenes (host-side workload generator).

Thin ctypes wrapper over ``pe_scene_generate`` (include/phys_gb300_scenes.h):
returns a :class:`Scene` of numpy arrays holding body-creation records in the
vocabulary of the reference's factories (``PhysicsWorld::createSphere`` /
``createBox``, include/phys/world/physics_world.hpp:43-50 of bkuangs/phys-engine).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _native

SPHERES_ON_FLOOR = 1
MIXED_VOLUME = 2
PYRAMIDS = 3
PYRAMIDS_BOXES_ONLY = 4
BOXES_ON_PLANE = 5


class _CScene(ctypes.Structure):
    _fields_ = [
        ("count", ctypes.c_uint32),
        ("shape", ctypes.POINTER(ctypes.c_uint8)),
        ("is_static", ctypes.POINTER(ctypes.c_uint8)),
        ("dims", ctypes.POINTER(ctypes.c_float)),
        ("pos", ctypes.POINTER(ctypes.c_float)),
        ("density", ctypes.POINTER(ctypes.c_float)),
        ("restitution", ctypes.POINTER(ctypes.c_float)),
        ("friction", ctypes.POINTER(ctypes.c_float)),
        ("linvel", ctypes.POINTER(ctypes.c_float)),
        ("spin", ctypes.POINTER(ctypes.c_float)),
        ("hull_id", ctypes.POINTER(ctypes.c_int32)),
        ("mass", ctypes.POINTER(ctypes.c_float)),
        ("inv_inertia", ctypes.POINTER(ctypes.c_float)),
        ("hull_count", ctypes.c_uint32),
        ("hull_offsets", ctypes.POINTER(ctypes.c_uint32)),
        ("hull_vertices", ctypes.POINTER(ctypes.c_float)),
    ]


@dataclass
class Scene:
    """Body-creation records, one row per body, in creation order."""

    shape: np.ndarray          # uint8 [n]: 0 sphere, 1 box, 2 hull
    is_static: np.ndarray      # uint8 [n]
    dims: np.ndarray           # float32 [n,3]: radius / full box size / hull semi-axes
    pos: np.ndarray            # float32 [n,3]
    density: np.ndarray        # float32 [n] (g/cm^3)
    restitution: np.ndarray    # float32 [n]
    friction: np.ndarray       # float32 [n]
    linvel: np.ndarray         # float32 [n,3]
    spin: np.ndarray           # float32 [n,3]
    hull_id: np.ndarray        # int32 [n]
    mass: np.ndarray           # float32 [n] (hulls)
    inv_inertia: np.ndarray    # float32 [n,3] (hulls)
    hull_offsets: np.ndarray = field(default_factory=lambda: np.zeros(1, np.uint32))
    hull_vertices: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))

    @property
    def count(self) -> int:
        return int(self.shape.shape[0])

    def hull(self, h: int) -> np.ndarray:
        return self.hull_vertices[self.hull_offsets[h]:self.hull_offsets[h + 1]]

    def subset(self, rows) -> "Scene":
        rows = np.asarray(rows)
        return Scene(self.shape[rows], self.is_static[rows], self.dims[rows], self.pos[rows],
                     self.density[rows], self.restitution[rows], self.friction[rows],
                     self.linvel[rows], self.spin[rows], self.hull_id[rows], self.mass[rows],
                     self.inv_inertia[rows], self.hull_offsets, self.hull_vertices)


def _arr(ptr, n, dtype, shape):
    if n == 0:
        return np.zeros(shape, dtype)
    a = np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)
    return a.reshape(shape)


def generate(kind: int, n: int, seed: int = 42) -> Scene:
    lib = _native.scenes_lib()
    cs = _CScene()
    rc = lib.pe_scene_generate(int(kind), int(n), int(seed), ctypes.byref(cs))
    if rc != 0:
        raise ValueError(f"pe_scene_generate({kind}, {n}, {seed}) failed with {rc}")
    try:
        c = cs.count
        hv = int(cs.hull_offsets[cs.hull_count]) if cs.hull_count else 0
        return Scene(
            shape=_arr(cs.shape, c, np.uint8, (c,)),
            is_static=_arr(cs.is_static, c, np.uint8, (c,)),
            dims=_arr(cs.dims, 3 * c, np.float32, (c, 3)),
            pos=_arr(cs.pos, 3 * c, np.float32, (c, 3)),
            density=_arr(cs.density, c, np.float32, (c,)),
            restitution=_arr(cs.restitution, c, np.float32, (c,)),
            friction=_arr(cs.friction, c, np.float32, (c,)),
            linvel=_arr(cs.linvel, 3 * c, np.float32, (c, 3)),
            spin=_arr(cs.spin, 3 * c, np.float32, (c, 3)),
            hull_id=_arr(cs.hull_id, c, np.int32, (c,)),
            mass=_arr(cs.mass, c, np.float32, (c,)),
            inv_inertia=_arr(cs.inv_inertia, 3 * c, np.float32, (c, 3)),
            hull_offsets=_arr(cs.hull_offsets, cs.hull_count + 1, np.uint32, (cs.hull_count + 1,)),
            hull_vertices=_arr(cs.hull_vertices, 3 * hv, np.float32, (hv, 3)),
        )
    finally:
        lib.pe_scene_free(ctypes.byref(cs))


def box_stacks(tiles_x: int = 1, tiles_z: int = 1) -> Scene:
    """The reference's settled-box profile scene (benchmarks/cpu_profile.cpp:20-41):
    a static 30 x 1 x 20 floor box and 512 unit boxes (density 1, restitution 0,
    friction 0.6) in 16 x 16 two-high stacks, 1.6 m apart along x and 1.2 m
    along z.  tiles_x x tiles_z copies of it lie side by side with 0.5 m gaps
    between the floors (floor, then its boxes, tile after tile)."""
    f = np.float32
    rows, cols, levels = np.meshgrid(np.arange(16), np.arange(16), np.arange(2), indexing="ij")
    rows, cols, levels = rows.reshape(-1), cols.reshape(-1), levels.reshape(-1)  # row, column, level order
    local = np.stack([f(-12.0) + f(1.6) * cols.astype(f), f(0.5) + f(1.02) * levels.astype(f),
                      f(-9.0) + f(1.2) * rows.astype(f)], axis=1).astype(f)
    pos, static, dims = [], [], []
    for tz in range(tiles_z):
        for tx in range(tiles_x):
            off = np.array([f(30.5) * f(tx), f(0.0), f(20.5) * f(tz)], f)
            pos.append(np.array([[0.0, -0.5, 0.0]], f) + off)
            pos.append(local + off)
            static.append(np.concatenate([[1], np.zeros(len(local), np.uint8)]).astype(np.uint8))
            dims.append(np.concatenate([np.array([[30, 1, 20]], f), np.ones((len(local), 3), f)]))
    pos, static, dims = np.concatenate(pos).astype(f), np.concatenate(static), np.concatenate(dims)
    n = len(pos)
    return Scene(shape=np.ones(n, np.uint8), is_static=static, dims=dims, pos=pos, density=np.ones(n, f),
                 restitution=np.zeros(n, f), friction=np.full(n, f(0.6)), linvel=np.zeros((n, 3), f),
                 spin=np.zeros((n, 3), f), hull_id=np.full(n, -1, np.int32), mass=np.zeros(n, f),
                 inv_inertia=np.zeros((n, 3), f))


def mixed_field(n: int, seed: int = 42) -> Scene:
    """The reference's own benchmark scene (benchmarks/bench_scenes.cpp:11-63,
    `phys_collision_bench ... mixed`): n dynamic bodies, half spheres (r 0.5) and
    half unit boxes in random order, two layers on a 1.5 m grid with +-5 cm
    jitter, restitution 0.1, friction 0.6, over one static floor slab 32 m wider
    than the grid on every side (its height capped so its volume stays within
    the body-size limit).  The reference draws the order and jitter from
    std::mt19937 through library distributions; this restatement draws them
    from numpy's generator with the same distributions."""
    f = np.float32
    cols_needed = (n + 1) // 2
    columns = int(np.ceil(np.sqrt(float(cols_needed))))
    rows = (cols_needed + columns - 1) // columns
    spacing, margin = f(1.5), f(32.0)
    fx = f(columns) * spacing + f(2.0) * margin
    fz = f(rows) * spacing + f(2.0) * margin
    fy = f(min(1.0, (4096.0 * 0.5) / (float(fx) * float(fz))))
    rng = np.random.default_rng(seed)
    sphere = np.zeros(n, bool)
    sphere[: (n + 1) // 2] = True
    rng.shuffle(sphere)
    jitter = rng.uniform(-0.05, 0.05, size=(n, 3)).astype(f)
    idx = np.arange(n)
    column = (idx // 2) % columns
    row = (idx // 2) // columns
    pos = np.stack([(column.astype(f) - f(columns - 1) * f(0.5)) * spacing + jitter[:, 0],
                    f(1.0) + (idx % 2).astype(f) * f(1.75) + jitter[:, 1],
                    (row.astype(f) - f(rows - 1) * f(0.5)) * spacing + jitter[:, 2]], axis=1).astype(f)
    m = n + 1
    shape = np.concatenate([[1], np.where(sphere, 0, 1)]).astype(np.uint8)
    dims = np.concatenate([np.array([[fx, fy, fz]], f),
                           np.where(sphere[:, None], np.array([[0.5, 0, 0]], f), np.ones((n, 3), f))]).astype(f)
    return Scene(shape=shape, is_static=np.concatenate([[1], np.zeros(n, np.uint8)]).astype(np.uint8), dims=dims,
                 pos=np.concatenate([np.array([[0.0, -fy * f(0.5), 0.0]], f), pos]).astype(f),
                 density=np.ones(m, f), restitution=np.concatenate([[0.0], np.full(n, 0.1)]).astype(f),
                 friction=np.full(m, f(0.6)), linvel=np.zeros((m, 3), f), spin=np.zeros((m, 3), f),
                 hull_id=np.full(m, -1, np.int32), mass=np.zeros(m, f), inv_inertia=np.zeros((m, 3), f))

