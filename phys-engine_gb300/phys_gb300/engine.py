"""ctypes binding of the GPU engine's C ABI (include/phys_gb300.h).

:class:`GpuWorld` mirrors ``phys::PhysicsWorld`` (include/phys/world/physics_world.hpp
of bkuangs/phys-engine): bodies are created through the same factories with the
same validation, ``step(dt)`` runs the whole collision-and-contact path on the
GPU, and contacts / stats / candidate pairs can be read back.  Every call goes
through ``libphys_gb300.so``; there is no host fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native

_P = ctypes.c_void_p
_u32 = ctypes.c_uint32


class Handle(ctypes.Structure):
    _fields_ = [("index", ctypes.c_uint32), ("generation", ctypes.c_uint32)]


class BodyState(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 3), ("rotation", ctypes.c_float * 4),
                ("linear_velocity", ctypes.c_float * 3), ("angular_velocity", ctypes.c_float * 3),
                ("force", ctypes.c_float * 3), ("mass", ctypes.c_float), ("restitution", ctypes.c_float),
                ("friction", ctypes.c_float), ("is_static", ctypes.c_int32)]


MANIFOLD_DTYPE = np.dtype([
    ("body_a_index", "<u4"), ("body_a_generation", "<u4"),
    ("body_b_index", "<u4"), ("body_b_generation", "<u4"),
    ("normal", "<f4", (3,)), ("point_count", "<u4"),
    ("friction", "<f4"), ("restitution", "<f4"),
    ("anchor_a", "<f4", (4, 3)), ("anchor_b", "<f4", (4, 3)),
    ("penetration", "<f4", (4,)), ("normal_impulse", "<f4", (4,)),
    ("tangent_impulse1", "<f4", (4,)), ("tangent_impulse2", "<f4", (4,)),
    ("feature", "<u4", (4,)),
])
assert MANIFOLD_DTYPE.itemsize == 216

STATS_DTYPE = np.dtype([
    ("possible_pairs", "<u8"), ("candidate_pairs", "<u8"), ("contact_count", "<u8"),
    ("solved_contact_count", "<u8"), ("awake_body_count", "<u8"), ("sleeping_body_count", "<u8"),
    ("x_window_comparisons", "<u8"), ("aabb_pairs", "<u8"), ("grid_comparisons", "<u8"),
    ("grid_entries", "<u8"), ("grid_overflow_aabbs", "<u8"), ("grid_cell_size", "<f8"),
    ("np_candidates", "<u8", (4,)), ("np_contacts", "<u8", (4,)),
    ("prepared_points", "<u8"), ("warm_start_comparisons", "<u8"), ("warm_start_matches", "<u8"),
    ("velocity_point_visits", "<u8"), ("color_count", "<u8"), ("color_rounds", "<u8"),
    ("epa_failures", "<u8"), ("contact_points", "<u8"), ("total_ms", "<f8"),
    ("integrate_ms", "<f8"), ("broadphase_ms", "<f8"), ("narrowphase_ms", "<f8"), ("solver_ms", "<f8"),
    ("pose_ms", "<f8"), ("kernel_launches", "<u8"), ("graph_replayed", "<u8"),
])

SAP, GRID, TREE = 0, 1, 2
ORDER_MANIFOLD, ORDER_COLOR = 0, 1

PE_OK = 0
_STATUS = {1: ValueError, 2: ValueError, 3: LookupError, 4: OverflowError, 5: NotImplementedError,
           6: RuntimeError, 7: RuntimeError}

# Every entry point declared in include/phys_gb300.h: name -> (restype, argtypes).
SIGNATURES = {
    "pe_last_error": (ctypes.c_char_p, []),
    "pe_device_count": (ctypes.c_int, []),
    "pe_world_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
    "pe_world_destroy": (None, [_P]),
    "pe_world_clone": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "pe_world_set_gravity": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "pe_world_get_gravity": (ctypes.c_int, [_P, _P]),
    "pe_world_set_broadphase": (ctypes.c_int, [_P, ctypes.c_int]),
    "pe_world_get_broadphase": (ctypes.c_int, [_P, _P]),
    "pe_world_set_grid_cell_size": (ctypes.c_int, [_P, ctypes.c_double]),
    "pe_world_set_solver": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "pe_world_set_worker_counts": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]),
    "pe_world_set_sleeping_enabled": (ctypes.c_int, [_P, ctypes.c_int]),
    "pe_world_get_sleeping_enabled": (ctypes.c_int, [_P, _P]),
    "pe_world_create_sphere": (ctypes.c_int, [_P, ctypes.c_float, _P, ctypes.c_float, ctypes.c_int,
                                              ctypes.c_float, ctypes.c_float, _P, _P]),
    "pe_world_create_box": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, _P,
                                           ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_float, _P, _P]),
    "pe_world_create_bodies": (ctypes.c_int, [_P, _u32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "pe_world_create_hull": (ctypes.c_int, [_P, _P, _u32, _P, ctypes.c_float, _P, ctypes.c_int, ctypes.c_float,
                                            ctypes.c_float, _P, _P]),
    "pe_world_add_collider": (ctypes.c_int, [_P, Handle, ctypes.c_int, _P, _P, _P, _P]),
    "pe_world_remove_body": (ctypes.c_int, [_P, Handle]),
    "pe_world_remove_collider": (ctypes.c_int, [_P, Handle]),
    "pe_world_get_body": (ctypes.c_int, [_P, Handle, _P]),
    "pe_debug_set_spin_limit": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint32]),
    "pe_rollout_device_bytes": (ctypes.c_int, [_P, _P]),
    "pe_world_get_solver_phases": (ctypes.c_int, [_P, _P]),
    "pe_rollout_set_manifold_capacity": (ctypes.c_int, [_P, ctypes.c_float]),
    "pe_body_make_sphere": (ctypes.c_int, [ctypes.c_float, _P, ctypes.c_float, ctypes.c_int, ctypes.c_float,
                                           ctypes.c_float, _P]),
    "pe_body_make_box": (ctypes.c_int, [ctypes.c_float, ctypes.c_float, ctypes.c_float, _P, ctypes.c_float,
                                        ctypes.c_int, ctypes.c_float, ctypes.c_float, _P]),
    "pe_body_integrate": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_float]),
    "pe_world_add_body": (ctypes.c_int, [_P, _P, _P]),
    "pe_world_get_body_record": (ctypes.c_int, [_P, Handle, _P]),
    "pe_world_get_collider": (ctypes.c_int, [_P, Handle, _P, _P, _P, _P, _P]),
    "pe_world_set_collider": (ctypes.c_int, [_P, Handle, Handle, ctypes.c_int, _P, _P, _P]),
    "pe_world_set_body": (ctypes.c_int, [_P, Handle, _P]),
    "pe_world_body_integrate_rotation": (ctypes.c_int, [_P, Handle, ctypes.c_float]),
    "pe_world_body_is_sleeping": (ctypes.c_int, [_P, Handle, _P]),
    "pe_world_body_wake_up": (ctypes.c_int, [_P, Handle]),
    "pe_world_body_apply_force": (ctypes.c_int, [_P, Handle, _P]),
    "pe_world_body_set_velocity": (ctypes.c_int, [_P, Handle, _P, _P]),
    "pe_world_read_sleeping": (ctypes.c_int, [_P, _P]),
    "pe_world_body_slot_count": (_u32, [_P]),
    "pe_world_read_bodies": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "pe_world_write_forces": (ctypes.c_int, [_P, _P, _u32]),
    "pe_world_read_poses": (ctypes.c_int, [_P, _P, _P]),
    "pe_world_step_io": (ctypes.c_int, [_P, _P, _u32, ctypes.c_float, _P, _P]),
    "pe_world_get_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "pe_world_set_graphs": (ctypes.c_int, [_P, ctypes.c_int]),
    "pe_world_graph_error": (ctypes.c_char_p, [_P]),
    "pe_world_step": (ctypes.c_int, [_P, ctypes.c_float]),
    "pe_world_get_step_stats": (ctypes.c_int, [_P, _P]),
    "pe_world_get_contacts": (ctypes.c_int, [_P, _P, _u32, _P]),
    "pe_world_get_candidate_pairs": (ctypes.c_int, [_P, _P, _u32, _P]),
    "pe_world_get_solve_order": (ctypes.c_int, [_P, _P, _P, _u32, _P]),
    "pe_world_solve": (ctypes.c_int, [_P, _P, _u32, ctypes.c_float]),
    "pe_broadphase_find_pairs": (ctypes.c_int, [ctypes.c_int, _P, _P, _u32, ctypes.c_int, ctypes.c_double, _P,
                                                ctypes.c_uint64, _P, _P]),
    "pe_generate_contact": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P, _P, _P,
                                           _P]),
    "pe_broadphase_find_pairs_noalloc": (ctypes.c_int, [ctypes.c_int, _P, _P, _u32, _P, _u32, _P, _P]),
    "pe_batch_create": (ctypes.c_int, [ctypes.c_int, _u32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                       ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_uint64)]),
    "pe_batch_destroy": (None, [_P]),
    "pe_batch_set_gravity": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "pe_batch_set_iterations": (ctypes.c_int, [_P, ctypes.c_int]),
    "pe_batch_step": (ctypes.c_int, [_P, ctypes.c_float, _u32]),
    "pe_batch_autotune": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_int]),
    "pe_batch_bucket_count": (ctypes.c_int, [_P, _P]),
    "pe_batch_get_bucket": (ctypes.c_int, [_P, _u32, _P]),
    "pe_batch_body_count": (ctypes.c_int, [_P, _P]),
    "pe_batch_read_bodies": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "pe_batch_write_bodies": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "pe_batch_write_forces": (ctypes.c_int, [_P, _P]),
    "pe_batch_read_poses": (ctypes.c_int, [_P, _P, _P]),
    "pe_batch_get_world_stats": (ctypes.c_int, [_P, _u32, _P]),
    "pe_batch_get_world_pairs": (ctypes.c_int, [_P, _u32, _P, _u32, _P]),
    "pe_batch_get_world_contacts": (ctypes.c_int, [_P, _u32, _P, _u32, _P]),
    "pe_batch_get_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "pe_batch_set_graphs": (ctypes.c_int, [_P, ctypes.c_int]),
    "pe_rollout_create": (ctypes.c_int, [ctypes.c_int, _u32, _P, _P, _P, _P, _P, _u32, ctypes.c_float, ctypes.c_int,
                                         _u32, ctypes.POINTER(_P), _P]),
    "pe_rollout_destroy": (None, [_P]),
    "pe_rollout_set_gravity": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "pe_rollout_forward": (ctypes.c_int, [_P] + [_P] * 12),
    "pe_rollout_backward": (ctypes.c_int, [_P] + [_P] * 12),
    "pe_rollout_timings": (ctypes.c_int, [_P, _P, _P]),
}

BUCKET_DTYPE = np.dtype([
    ("min_bodies", "<u4"), ("max_bodies", "<u4"), ("world_count", "<u4"), ("threads", "<u4"),
    ("min_blocks_per_sm", "<u4"), ("blocks", "<u4"), ("tuned_ms", "<f8"), ("candidate_ms", "<f8", (8,)),
])
assert BUCKET_DTYPE.itemsize == 96

_lib = None


def lib():
    global _lib
    if _lib is None:
        l = _native.engine_lib()
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def _ptr(a):
    # a ctypes pointer object: it keeps the array alive for the call, so a
    # temporary array may be passed
    return None if a is None else a.ctypes.data_as(_P)


def _addr(a):
    # the buffer address as an int (cheaper per call than _ptr); only for
    # arrays that a name holds for the whole call
    return None if a is None else a.ctypes.data


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


PE_ERR_CAPACITY = 4


def check_size(rc: int):
    """Size query with a NULL / too-small buffer: PE_ERR_CAPACITY just reports the count."""
    if rc not in (PE_OK, PE_ERR_CAPACITY):
        check(rc)


def check(rc: int):
    if rc != PE_OK:
        msg = lib().pe_last_error().decode()
        raise _STATUS.get(rc, RuntimeError)(f"phys_gb300 status {rc}: {msg}")


class GpuWorld:
    """GPU-resident world with the reference PhysicsWorld's creation API."""

    def __init__(self, device=0, algo=SAP, cell_size=0.0, iterations=8, order=ORDER_COLOR):
        self.lib = lib()
        h = _P()
        check(self.lib.pe_world_create(int(device), ctypes.byref(h)))
        self.h = h
        self.device = device
        self.set_broadphase(algo, cell_size)
        self.set_solver(iterations, order)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pe_world_destroy(self.h)
            self.h = None

    def clone(self):
        """An independent copy (the PhysicsWorld copy constructor)."""
        h = _P()
        check(self.lib.pe_world_clone(self.h, ctypes.byref(h)))
        c = GpuWorld.__new__(GpuWorld)
        c.lib, c.h, c.device = self.lib, h, self.device
        return c

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # configuration -------------------------------------------------------
    def set_gravity(self, g):
        check(self.lib.pe_world_set_gravity(self.h, float(g[0]), float(g[1]), float(g[2])))

    def set_broadphase(self, algo, cell_size=0.0):
        check(self.lib.pe_world_set_broadphase(self.h, int(algo)))
        check(self.lib.pe_world_set_grid_cell_size(self.h, float(cell_size)))

    def set_solver(self, iterations, order):
        check(self.lib.pe_world_set_solver(self.h, int(iterations), int(order)))

    # bodies --------------------------------------------------------------
    def create_body(self, shape, dims, pos, density, is_static, restitution, friction):
        b, c = Handle(), Handle()
        p = _f32(pos)
        if int(shape) == 0:
            rc = self.lib.pe_world_create_sphere(self.h, float(dims[0]), _ptr(p), float(density), int(is_static),
                                                 float(restitution), float(friction), ctypes.byref(b), ctypes.byref(c))
        else:
            rc = self.lib.pe_world_create_box(self.h, float(dims[0]), float(dims[1]), float(dims[2]), _ptr(p),
                                              float(density), int(is_static), float(restitution), float(friction),
                                              ctypes.byref(b), ctypes.byref(c))
        check(rc)
        return np.array([b.index, b.generation, c.index, c.generation], np.uint32)

    def create_hull(self, vertices, pos, mass, inv_inertia, is_static, restitution, friction):
        b, c = Handle(), Handle()
        v = _f32(vertices)
        check(self.lib.pe_world_create_hull(self.h, _ptr(v), len(v), _ptr(_f32(pos)), float(mass),
                                            _ptr(_f32(inv_inertia)), int(is_static), float(restitution),
                                            float(friction), ctypes.byref(b), ctypes.byref(c)))
        return np.array([b.index, b.generation, c.index, c.generation], np.uint32)

    def load_scene(self, scene):
        """Creates the scene's bodies in order (spheres/boxes in one bulk call per
        run, hulls one by one) and returns [n, 4] handles (body idx, gen,
        collider idx, gen)."""
        n = scene.count
        handles = np.zeros((n, 4), np.uint32)
        i = 0
        while i < n:
            if scene.shape[i] == 2:
                handles[i] = self.create_hull(scene.hull(scene.hull_id[i]), scene.pos[i], scene.mass[i],
                                              scene.inv_inertia[i], scene.is_static[i], scene.restitution[i],
                                              scene.friction[i])
                h = Handle(int(handles[i, 0]), int(handles[i, 1]))
                if np.any(scene.spin[i] != 0) and not scene.is_static[i]:
                    self.apply_spin(h, scene.spin[i])
                if np.any(scene.linvel[i] != 0):
                    st = self.get_body(h)
                    st.linear_velocity[:] = [float(x) for x in scene.linvel[i]]
                    self.set_body(h, st)
                i += 1
                continue
            j = i
            while j < n and scene.shape[j] != 2:
                j += 1
            sl = slice(i, j)
            m = j - i
            bh = (Handle * m)()
            ch = (Handle * m)()
            failed = _u32()
            rc = self.lib.pe_world_create_bodies(
                self.h, m, _ptr(np.ascontiguousarray(scene.shape[sl], np.uint8)), _ptr(_f32(scene.dims[sl])),
                _ptr(_f32(scene.pos[sl])), _ptr(_f32(scene.density[sl])),
                _ptr(np.ascontiguousarray(scene.is_static[sl], np.uint8)), _ptr(_f32(scene.restitution[sl])),
                _ptr(_f32(scene.friction[sl])), _ptr(_f32(scene.linvel[sl])), _ptr(_f32(scene.spin[sl])),
                ctypes.cast(bh, _P), ctypes.cast(ch, _P), ctypes.byref(failed))
            check(rc)
            raw_b = np.ctypeslib.as_array(ctypes.cast(bh, ctypes.POINTER(ctypes.c_uint32)), shape=(2 * m,))
            raw_c = np.ctypeslib.as_array(ctypes.cast(ch, ctypes.POINTER(ctypes.c_uint32)), shape=(2 * m,))
            handles[sl, 0:2] = raw_b.reshape(m, 2)
            handles[sl, 2:4] = raw_c.reshape(m, 2)
            i = j
        return handles

    def get_body(self, h) -> BodyState:
        st = BodyState()
        check(self.lib.pe_world_get_body(self.h, h, ctypes.byref(st)))
        return st

    def set_body(self, h, st: BodyState):
        check(self.lib.pe_world_set_body(self.h, h, ctypes.byref(st)))

    def apply_spin(self, h, spin):
        """setAngularVelocity(spin); integrateRotation(1); setAngularVelocity(0)."""
        st = self.get_body(h)
        st.angular_velocity[:] = [float(x) for x in spin]
        self.set_body(h, st)
        check(self.lib.pe_world_body_integrate_rotation(self.h, h, 1.0))
        st = self.get_body(h)
        st.angular_velocity[:] = [0.0, 0.0, 0.0]
        self.set_body(h, st)

    def remove_body(self, idx, gen):
        check(self.lib.pe_world_remove_body(self.h, Handle(int(idx), int(gen))))

    def add_collider(self, body_idx, body_gen, shape, dims, local_pos=(0, 0, 0), local_rot=(0, 0, 0, 1)):
        """PhysicsWorld::addCollider on an existing body (dims: sphere radius /
        box half extents); returns (collider idx, gen)."""
        c = Handle()
        check(self.lib.pe_world_add_collider(self.h, Handle(int(body_idx), int(body_gen)), int(shape),
                                             _ptr(_f32(dims)), _ptr(_f32(local_pos)), _ptr(_f32(local_rot)),
                                             ctypes.byref(c)))
        return np.array([c.index, c.generation], np.uint32)

    def remove_collider(self, idx, gen):
        check(self.lib.pe_world_remove_collider(self.h, Handle(int(idx), int(gen))))

    # sleeping ------------------------------------------------------------
    def set_sleeping_enabled(self, enabled):
        check(self.lib.pe_world_set_sleeping_enabled(self.h, int(bool(enabled))))

    def sleeping_enabled(self):
        v = ctypes.c_int()
        check(self.lib.pe_world_get_sleeping_enabled(self.h, ctypes.byref(v)))
        return bool(v.value)

    def sleeping(self):
        """isSleeping() of every body slot."""
        out = np.zeros(self.body_count(), np.uint8)
        check(self.lib.pe_world_read_sleeping(self.h, _ptr(out)))
        return out.astype(bool)

    def is_sleeping(self, h):
        v = ctypes.c_int()
        check(self.lib.pe_world_body_is_sleeping(self.h, h, ctypes.byref(v)))
        return bool(v.value)

    def wake_up(self, h):
        check(self.lib.pe_world_body_wake_up(self.h, h))

    def apply_force(self, h, force):
        check(self.lib.pe_world_body_apply_force(self.h, h, _ptr(_f32(force))))

    def set_velocity(self, h, lin=None, ang=None):
        check(self.lib.pe_world_body_set_velocity(self.h, h, _ptr(None if lin is None else _f32(lin)),
                                                  _ptr(None if ang is None else _f32(ang))))

    def set_material(self, h, mass, friction, restitution):
        st = self.get_body(h)
        st.mass, st.friction, st.restitution = float(mass), float(friction), float(restitution)
        self.set_body(h, st)

    def body_count(self):
        return int(self.lib.pe_world_body_slot_count(self.h))

    def bodies(self):
        n = self.body_count()
        pos = np.zeros((n, 3), np.float32)
        quat = np.zeros((n, 4), np.float32)
        lin = np.zeros((n, 3), np.float32)
        ang = np.zeros((n, 3), np.float32)
        check(self.lib.pe_world_read_bodies(self.h, _ptr(pos), _ptr(quat), _ptr(lin), _ptr(ang)))
        return {"pos": pos, "quat": quat, "lin": lin, "ang": ang}

    # stepping ------------------------------------------------------------
    def step(self, dt):
        check(self.lib.pe_world_step(self.h, float(dt)))

    def set_graphs(self, enabled: bool):
        check(self.lib.pe_world_set_graphs(self.h, 1 if enabled else 0))

    def graph_error(self) -> str:
        return self.lib.pe_world_graph_error(self.h).decode()

    def write_forces(self, forces):
        f = _f32(forces)
        check(self.lib.pe_world_write_forces(self.h, _ptr(f), len(f)))

    def read_poses(self, positions=None, rotations=None):
        check(self.lib.pe_world_read_poses(self.h, _ptr(positions), _ptr(rotations)))

    def step_io(self, dt, forces=None, positions=None, rotations=None):
        """write_forces + step + read_poses with one synchronisation."""
        f = None if forces is None else _f32(forces)
        check(self.lib.pe_world_step_io(self.h, _addr(f), 0 if f is None else len(f), float(dt), _addr(positions),
                                        _addr(rotations)))

    def stream(self) -> int:
        s = _P()
        check(self.lib.pe_world_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def solver_phases(self):
        """Device ms of the one-cluster solver's phases in the last step:
        gap after the narrowphase, prepare kernel (prepare + flags + unions),
        gap, island lists, plan + staging, sweeps (island path: with the
        results and the cache), write-back + cache (colour-phase path), gap to
        the pose kernel."""
        ms = np.zeros(8, np.float64)
        check(self.lib.pe_world_get_solver_phases(self.h, _ptr(ms)))
        return ms

    def stats(self):
        s = np.zeros(1, STATS_DTYPE)
        check(self.lib.pe_world_get_step_stats(self.h, _ptr(s)))
        return s[0]

    def contacts(self):
        n = _u32()
        check_size(self.lib.pe_world_get_contacts(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, MANIFOLD_DTYPE)
        if n.value:
            check(self.lib.pe_world_get_contacts(self.h, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def pairs(self):
        n = _u32()
        check_size(self.lib.pe_world_get_candidate_pairs(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros((n.value, 2), np.uint32)
        if n.value:
            check(self.lib.pe_world_get_candidate_pairs(self.h, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def solve_order(self):
        n = _u32()
        check_size(self.lib.pe_world_get_solve_order(self.h, None, None, 0, ctypes.byref(n)))
        order = np.zeros(n.value, np.uint32)
        colors = np.zeros(n.value, np.uint32)
        if n.value:
            check(self.lib.pe_world_get_solve_order(self.h, _ptr(order), _ptr(colors), n.value, ctypes.byref(n)))
        return order, colors

    def solve(self, manifolds, dt):
        m = np.ascontiguousarray(manifolds.copy())
        check(self.lib.pe_world_solve(self.h, _ptr(m), len(m), float(dt)))
        return m


def broadphase(mins, maxs, algo=SAP, cell_size=0.0, device=0):
    """BroadPhase::findCandidatePairs on the GPU; returns (pairs[n,2], stats)."""
    l = lib()
    mins, maxs = _f32(mins).reshape(-1, 3), _f32(maxs).reshape(-1, 3)
    n = len(mins)
    cnt = ctypes.c_uint64()
    st = np.zeros(1, STATS_DTYPE)
    check_size(l.pe_broadphase_find_pairs(int(device), _ptr(mins), _ptr(maxs), n, int(algo), float(cell_size), None,
                                          0, ctypes.byref(cnt), _ptr(st)))
    pairs = np.zeros((cnt.value, 2), np.uint32)
    if cnt.value:
        check(l.pe_broadphase_find_pairs(int(device), _ptr(mins), _ptr(maxs), n, int(algo), float(cell_size),
                                         _ptr(pairs), cnt.value, ctypes.byref(cnt), _ptr(st)))
    return pairs, st[0]


def generate_contact(shape_a, dims_a, pos_a, quat_a, shape_b, dims_b, pos_b, quat_b, device=0):
    """NarrowPhase::generateContact on the GPU for one sphere/box pair (dims =
    radius or half extents)."""
    out = np.zeros(1, MANIFOLD_DTYPE)
    hit = ctypes.c_int()
    check(lib().pe_generate_contact(int(device), int(shape_a), _ptr(_f32(dims_a)), _ptr(_f32(pos_a)),
                                    _ptr(_f32(quat_a)), int(shape_b), _ptr(_f32(dims_b)), _ptr(_f32(pos_b)),
                                    _ptr(_f32(quat_b)), _ptr(out), ctypes.byref(hit)))
    return bool(hit.value), out[0]


class GpuBatch:
    """Many independent worlds stepped together (sphere/box bodies, one collider
    each, SAP broadphase, graph-colour solve order).  ``scenes`` is a list of
    :class:`phys_gb300.scenes.Scene` without hulls; world ``w`` holds the bodies
    of ``scenes[w]`` in order."""

    def __init__(self, scenes, device=0, iterations=8, gravity=(0.0, -9.81, 0.0)):
        self.lib = lib()
        counts = np.array([s.count for s in scenes], np.uint32)
        cat = lambda f, dt: np.ascontiguousarray(np.concatenate([getattr(s, f) for s in scenes]), dt)
        shape = cat("shape", np.uint8)
        if np.any(shape > 1):
            raise ValueError("batched worlds hold spheres and boxes only")
        h = _P()
        failed = ctypes.c_uint64()
        self.counts = counts
        self.starts = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)])
        check(self.lib.pe_batch_create(
            int(device), len(counts), _ptr(counts), _ptr(shape), _ptr(cat("dims", np.float32)),
            _ptr(cat("pos", np.float32)), _ptr(cat("density", np.float32)), _ptr(cat("is_static", np.uint8)),
            _ptr(cat("restitution", np.float32)), _ptr(cat("friction", np.float32)),
            _ptr(cat("linvel", np.float32)), _ptr(cat("spin", np.float32)), ctypes.byref(h), ctypes.byref(failed)))
        self.h = h
        self.n = int(self.starts[-1])
        check(self.lib.pe_batch_set_iterations(self.h, int(iterations)))
        check(self.lib.pe_batch_set_gravity(self.h, *[float(x) for x in gravity]))

    def close(self):
        if getattr(self, "h", None):
            self.lib.pe_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def world_count(self):
        return len(self.counts)

    def step(self, dt, steps=1):
        check(self.lib.pe_batch_step(self.h, float(dt), int(steps)))

    def autotune(self, dt, repetitions=3):
        check(self.lib.pe_batch_autotune(self.h, float(dt), int(repetitions)))

    def buckets(self):
        n = _u32()
        check(self.lib.pe_batch_bucket_count(self.h, ctypes.byref(n)))
        out = np.zeros(n.value, BUCKET_DTYPE)
        for i in range(n.value):
            check(self.lib.pe_batch_get_bucket(self.h, i, _ptr(out[i:i + 1])))
        return out

    def set_graphs(self, on):
        check(self.lib.pe_batch_set_graphs(self.h, int(bool(on))))

    def stream(self):
        s = _P()
        check(self.lib.pe_batch_get_stream(self.h, ctypes.byref(s)))
        return s.value

    def bodies(self):
        """(pos[n,3], rot[n,4], lin[n,3], ang[n,3]) of all worlds, world by world."""
        pos = np.zeros((self.n, 3), np.float32)
        rot = np.zeros((self.n, 4), np.float32)
        lin = np.zeros((self.n, 3), np.float32)
        ang = np.zeros((self.n, 3), np.float32)
        check(self.lib.pe_batch_read_bodies(self.h, _ptr(pos), _ptr(rot), _ptr(lin), _ptr(ang)))
        return pos, rot, lin, ang

    def world_bodies(self, w):
        s, e = self.starts[w], self.starts[w + 1]
        return tuple(a[s:e] for a in self.bodies())

    def write_bodies(self, pos=None, rot=None, lin=None, ang=None):
        f = lambda a: None if a is None else _ptr(_f32(a))
        check(self.lib.pe_batch_write_bodies(self.h, f(pos), f(rot), f(lin), f(ang)))

    def write_forces(self, forces):
        check(self.lib.pe_batch_write_forces(self.h, _ptr(_f32(forces))))

    def read_poses(self, pos, rot):
        check(self.lib.pe_batch_read_poses(self.h, _ptr(pos), _ptr(rot)))

    def stats(self, w):
        st = np.zeros(1, STATS_DTYPE)
        check(self.lib.pe_batch_get_world_stats(self.h, int(w), _ptr(st)))
        return st[0]

    def pairs(self, w):
        cnt = _u32()
        check_size(self.lib.pe_batch_get_world_pairs(self.h, int(w), None, 0, ctypes.byref(cnt)))
        out = np.zeros((cnt.value, 2), np.uint32)
        if cnt.value:
            check(self.lib.pe_batch_get_world_pairs(self.h, int(w), _ptr(out), cnt.value, ctypes.byref(cnt)))
        return out

    def contacts(self, w):
        cnt = _u32()
        check_size(self.lib.pe_batch_get_world_contacts(self.h, int(w), None, 0, ctypes.byref(cnt)))
        out = np.zeros(cnt.value, MANIFOLD_DTYPE)
        if cnt.value:
            check(self.lib.pe_batch_get_world_contacts(self.h, int(w), _ptr(out), cnt.value, ctypes.byref(cnt)))
        return out
