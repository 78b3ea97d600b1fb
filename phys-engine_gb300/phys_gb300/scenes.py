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
