"""ctypes bindings for the CPU checkers (test infrastructure only).

* :class:`OracleWorld` — the restatement in oracle/pe_oracle.cpp (builds anywhere).
* :class:`RefWorld`    — the unmodified reference, compiled from its sources by
  ``make -C oracle ref``; available only where those sources are.

Both load a scene through their own public body-creation calls, so the tests
can drive every engine from the same records.
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "libpe_oracle.so"
REF_SO = HERE / "_ref" / "libref_harness.so"


def _reference_src() -> pathlib.Path:
    """The reference checkout the `ref` target compiles: PE_REFERENCE_SRC, else
    the location oracle/Makefile names (the build recipe owns that default)."""
    env = os.environ.get("PE_REFERENCE_SRC")
    if env:
        return pathlib.Path(env)
    try:
        out = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref"], check=True, capture_output=True,
                             text=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        out = ""
    return pathlib.Path(out) if out else HERE / "_no_reference"


REFERENCE_SRC = _reference_src()

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
    ("velocity_point_visits", "<u8"), ("color_count", "<u8"),
])

_P = ctypes.c_void_p
_libs: dict = {}


def build_oracle() -> pathlib.Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True, capture_output=True)
    return ORACLE_SO


def reference_available() -> bool:
    return REF_SO.exists() or (REFERENCE_SRC / "src").is_dir()


def build_reference() -> pathlib.Path:
    subprocess.run(["make", "-s", "-j8", "-C", str(HERE), "ref"], check=True, capture_output=True)
    return REF_SO


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def oracle_lib():
    if "oracle" not in _libs:
        if not ORACLE_SO.exists():
            build_oracle()
        lib = ctypes.CDLL(str(ORACLE_SO))
        lib.ow_create.restype = _P
        lib.ow_clone.restype = _P
        lib.ow_clone.argtypes = [_P]
        lib.ow_destroy.argtypes = [_P]
        lib.ow_set_gravity.argtypes = [_P, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.ow_set_broadphase.argtypes = [_P, ctypes.c_int, ctypes.c_double]
        lib.ow_set_solver.argtypes = [_P, ctypes.c_int, ctypes.c_int]
        lib.ow_set_threads.argtypes = [_P, ctypes.c_int]
        lib.ow_create_body.argtypes = [_P, ctypes.c_int, _P, _P, ctypes.c_float, ctypes.c_int,
                                       ctypes.c_float, ctypes.c_float, _P, ctypes.c_char_p, ctypes.c_int]
        lib.ow_add_hull_shape.argtypes = [_P, ctypes.c_uint32, _P]
        lib.ow_create_hull_body.argtypes = [_P, ctypes.c_int, _P, ctypes.c_float, _P, ctypes.c_int,
                                            ctypes.c_float, ctypes.c_float, _P]
        lib.ow_remove_body.argtypes = [_P, ctypes.c_uint32, ctypes.c_uint32]
        lib.ow_remove_collider.argtypes = [_P, ctypes.c_uint32, ctypes.c_uint32]
        lib.ow_add_collider.argtypes = [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, _P, _P, _P, _P]
        lib.ow_set_sleeping_enabled.argtypes = [_P, ctypes.c_int]
        lib.ow_get_sleeping.argtypes = [_P, _P]
        lib.ow_wake_body.argtypes = [_P, ctypes.c_uint32]
        lib.ow_apply_force.argtypes = [_P, ctypes.c_uint32, _P]
        lib.ow_body_slot_count.argtypes = [_P]
        lib.ow_body_slot_count.restype = ctypes.c_uint32
        lib.ow_get_bodies.argtypes = [_P, _P, _P, _P, _P]
        lib.ow_get_bodies_f64.argtypes = [_P, _P, _P, _P, _P]
        lib.ow_set_velocity.argtypes = [_P, ctypes.c_uint32, _P, _P]
        lib.ow_set_velocity_f64.argtypes = [_P, ctypes.c_uint32, _P, _P]
        lib.ow_set_position_f64.argtypes = [_P, ctypes.c_uint32, _P]
        lib.ow_apply_spin.argtypes = [_P, ctypes.c_uint32, _P]
        lib.ow_set_material.argtypes = [_P, ctypes.c_uint32, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.ow_get_material.argtypes = [_P, ctypes.c_uint32, _P, _P, _P]
        lib.ow_step.argtypes = [_P, ctypes.c_float]
        lib.ow_get_stats.argtypes = [_P, _P]
        lib.ow_pair_count.argtypes = [_P]
        lib.ow_pair_count.restype = ctypes.c_uint32
        lib.ow_get_pairs.argtypes = [_P, _P]
        lib.ow_contact_count.argtypes = [_P]
        lib.ow_contact_count.restype = ctypes.c_uint32
        lib.ow_get_contacts.argtypes = [_P, _P]
        lib.ow_get_solve_order.argtypes = [_P, _P, _P]
        lib.ow_broadphase.argtypes = [_P, _P, ctypes.c_uint32, ctypes.c_int, ctypes.c_double, _P,
                                      ctypes.c_uint64, _P]
        lib.ow_broadphase.restype = ctypes.c_uint64
        lib.ow_generate_contact.argtypes = [ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P, _P, _P]
        lib.ow_solve.argtypes = [_P, _P, ctypes.c_uint32, ctypes.c_float, ctypes.c_int, _P, _P]
        lib.ow_color_manifolds.argtypes = [_P, _P, ctypes.c_uint32, _P, _P]
        lib.ow_color_manifolds.restype = ctypes.c_uint32
        lib.ow_gjk_epa.argtypes = [_P, ctypes.c_uint32, _P, ctypes.c_uint32, _P, _P, _P]
        _libs["oracle"] = lib
    return _libs["oracle"]


def ref_lib():
    if "ref" not in _libs:
        if not REF_SO.exists():
            build_reference()
        lib = ctypes.CDLL(str(REF_SO))
        lib.rw_create.restype = _P
        lib.rw_clone.restype = _P
        lib.rw_clone.argtypes = [_P]
        lib.rw_destroy.argtypes = [_P]
        lib.rw_set_gravity.argtypes = [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        lib.rw_set_broadphase.argtypes = [_P, ctypes.c_int]
        lib.rw_set_workers.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.rw_create_body.argtypes = [_P, ctypes.c_int, _P, _P, ctypes.c_float, ctypes.c_int,
                                       ctypes.c_float, ctypes.c_float, _P, ctypes.c_char_p, ctypes.c_int]
        lib.rw_remove_body.argtypes = [_P, ctypes.c_uint32, ctypes.c_uint32]
        lib.rw_remove_collider.argtypes = [_P, ctypes.c_uint32, ctypes.c_uint32]
        lib.rw_add_collider.argtypes = [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, _P, _P, _P, _P]
        lib.rw_set_sleeping_enabled.argtypes = [_P, ctypes.c_int]
        lib.rw_get_sleeping.argtypes = [_P, _P]
        lib.rw_wake_body.argtypes = [_P, ctypes.c_uint32]
        lib.rw_apply_force.argtypes = [_P, ctypes.c_uint32, _P]
        lib.rw_set_material.argtypes = [_P, ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        lib.rw_body_slot_count.argtypes = [_P]
        lib.rw_body_slot_count.restype = ctypes.c_uint32
        lib.rw_apply_spin.argtypes = [_P, ctypes.c_uint32, _P]
        lib.rw_set_velocity.argtypes = [_P, ctypes.c_uint32, _P, _P]
        lib.rw_get_bodies.argtypes = [_P, _P, _P, _P, _P]
        lib.rw_get_bounds.argtypes = [_P, _P, _P]
        lib.rw_step.argtypes = [_P, ctypes.c_float]
        lib.rw_get_stats.argtypes = [_P, _P]
        lib.rw_contact_count.argtypes = [_P]
        lib.rw_contact_count.restype = ctypes.c_uint32
        lib.rw_get_contacts.argtypes = [_P, _P]
        lib.rw_broadphase.argtypes = [_P, _P, ctypes.c_uint32, ctypes.c_int, _P, ctypes.c_uint64, _P]
        lib.rw_broadphase.restype = ctypes.c_uint64
        lib.rw_generate_contact.argtypes = [ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P, _P, _P]
        lib.rw_solve.argtypes = [_P, _P, ctypes.c_uint32, ctypes.c_float, _P, _P]
        lib.rw_gjk_epa.argtypes = [_P, ctypes.c_uint32, _P, ctypes.c_uint32, _P, _P, _P]
        _libs["ref"] = lib
    return _libs["ref"]


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(shape) if shape else a


class _CpuWorld:
    _prefix = ""

    def _lib(self):
        raise NotImplementedError

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            getattr(self.lib, self._prefix + "destroy")(h)
            self.h = None

    def create_body(self, shape, dims, pos, density, is_static, restitution, friction):
        handles = np.zeros(4, np.uint32)
        err = ctypes.create_string_buffer(128)
        rc = getattr(self.lib, self._prefix + "create_body")(
            self.h, int(shape), _ptr(_f32(dims)), _ptr(_f32(pos)), float(density), int(is_static),
            float(restitution), float(friction), _ptr(handles), err, 128)
        if rc != 0:
            raise ValueError(err.value.decode())
        return handles

    def load_scene(self, scene):
        handles = np.zeros((scene.count, 4), np.uint32)
        for i in range(scene.count):
            if scene.shape[i] == 2:
                handles[i] = self._create_hull(scene, i)
            else:
                handles[i] = self.create_body(scene.shape[i], scene.dims[i], scene.pos[i], scene.density[i],
                                              scene.is_static[i], scene.restitution[i], scene.friction[i])
            idx = int(handles[i, 0])
            if np.any(scene.spin[i] != 0):
                self.apply_spin(idx, scene.spin[i])
            if np.any(scene.linvel[i] != 0):
                self.set_velocity(idx, scene.linvel[i], None)
        return handles

    def _create_hull(self, scene, i):
        raise NotImplementedError("the reference has no convex-hull collider")

    def apply_spin(self, idx, spin):
        getattr(self.lib, self._prefix + "apply_spin")(self.h, int(idx), _ptr(_f32(spin)))

    def set_velocity(self, idx, lin, ang):
        getattr(self.lib, self._prefix + "set_velocity")(
            self.h, int(idx), _ptr(None if lin is None else _f32(lin)), _ptr(None if ang is None else _f32(ang)))

    def remove_body(self, idx, gen):
        getattr(self.lib, self._prefix + "remove_body")(self.h, int(idx), int(gen))

    def add_collider(self, body_idx, body_gen, shape, dims, local_pos=(0, 0, 0), local_rot=(0, 0, 0, 1)):
        """Collider on an existing body (dims: sphere radius / box half extents);
        returns (collider idx, gen)."""
        h = np.zeros(2, np.uint32)
        rc = getattr(self.lib, self._prefix + "add_collider")(
            self.h, int(body_idx), int(body_gen), int(shape), _ptr(_f32(dims)), _ptr(_f32(local_pos)),
            _ptr(_f32(local_rot)), _ptr(h))
        if rc != 0:
            raise LookupError("stale body handle")
        return h

    def remove_collider(self, idx, gen):
        getattr(self.lib, self._prefix + "remove_collider")(self.h, int(idx), int(gen))

    def set_sleeping_enabled(self, enabled):
        getattr(self.lib, self._prefix + "set_sleeping_enabled")(self.h, int(bool(enabled)))

    def sleeping(self):
        out = np.zeros(self.body_count(), np.uint8)
        getattr(self.lib, self._prefix + "get_sleeping")(self.h, _ptr(out))
        return out.astype(bool)

    def wake_body(self, idx):
        getattr(self.lib, self._prefix + "wake_body")(self.h, int(idx))

    def apply_force(self, idx, force):
        getattr(self.lib, self._prefix + "apply_force")(self.h, int(idx), _ptr(_f32(force)))

    def step(self, dt):
        getattr(self.lib, self._prefix + "step")(self.h, float(dt))

    def body_count(self):
        return int(getattr(self.lib, self._prefix + "body_slot_count")(self.h))

    def bodies(self):
        n = self.body_count()
        pos = np.zeros((n, 3), np.float32)
        quat = np.zeros((n, 4), np.float32)
        lin = np.zeros((n, 3), np.float32)
        ang = np.zeros((n, 3), np.float32)
        getattr(self.lib, self._prefix + "get_bodies")(self.h, _ptr(pos), _ptr(quat), _ptr(lin), _ptr(ang))
        return {"pos": pos, "quat": quat, "lin": lin, "ang": ang}

    def stats(self):
        s = np.zeros(1, STATS_DTYPE)
        getattr(self.lib, self._prefix + "get_stats")(self.h, _ptr(s))
        return s[0]

    def contacts(self):
        n = int(getattr(self.lib, self._prefix + "contact_count")(self.h))
        out = np.zeros(n, MANIFOLD_DTYPE)
        if n:
            getattr(self.lib, self._prefix + "get_contacts")(self.h, _ptr(out))
        return out


class OracleWorld(_CpuWorld):
    """The restated step (float by default; ``fp64=True`` for finite differences)."""

    _prefix = "ow_"

    def __init__(self, fp64=False, algo=0, cell_size=0.0, iterations=8, order_mode=0, threads=1):
        self.lib = oracle_lib()
        self.h = self.lib.ow_create(1 if fp64 else 0)
        self.fp64 = fp64
        self.set_broadphase(algo, cell_size)
        self.set_solver(iterations, order_mode)
        self.lib.ow_set_threads(self.h, int(threads))

    def clone(self):
        w = OracleWorld.__new__(OracleWorld)
        w.lib = self.lib
        w.fp64 = self.fp64
        w.h = self.lib.ow_clone(self.h)
        return w

    def set_gravity(self, g):
        self.lib.ow_set_gravity(self.h, float(g[0]), float(g[1]), float(g[2]))

    def set_broadphase(self, algo, cell_size=0.0):
        self.lib.ow_set_broadphase(self.h, int(algo), float(cell_size))

    def set_solver(self, iterations, order_mode):
        self.lib.ow_set_solver(self.h, int(iterations), int(order_mode))

    def set_threads(self, threads):
        self.lib.ow_set_threads(self.h, int(threads))

    def _create_hull(self, scene, i):
        hid = self.lib.ow_add_hull_shape(self.h, len(scene.hull(scene.hull_id[i])),
                                         _ptr(_f32(scene.hull(scene.hull_id[i]))))
        handles = np.zeros(4, np.uint32)
        self.lib.ow_create_hull_body(self.h, hid, _ptr(_f32(scene.pos[i])), float(scene.mass[i]),
                                     _ptr(_f32(scene.inv_inertia[i])), int(scene.is_static[i]),
                                     float(scene.restitution[i]), float(scene.friction[i]), _ptr(handles))
        return handles

    def bodies_f64(self):
        n = self.body_count()
        out = {k: np.zeros((n, d), np.float64) for k, d in (("pos", 3), ("quat", 4), ("lin", 3), ("ang", 3))}
        self.lib.ow_get_bodies_f64(self.h, *(_ptr(out[k]) for k in ("pos", "quat", "lin", "ang")))
        return out

    def set_velocity_f64(self, idx, lin, ang):
        lin = None if lin is None else np.ascontiguousarray(lin, np.float64)
        ang = None if ang is None else np.ascontiguousarray(ang, np.float64)
        self.lib.ow_set_velocity_f64(self.h, int(idx), _ptr(lin), _ptr(ang))

    def set_position_f64(self, idx, pos):
        self.lib.ow_set_position_f64(self.h, int(idx), _ptr(np.ascontiguousarray(pos, np.float64)))

    def set_material(self, idx, mass, friction, restitution):
        self.lib.ow_set_material(self.h, int(idx), float(mass), float(friction), float(restitution))

    def material(self, idx):
        m, f, r = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self.lib.ow_get_material(self.h, int(idx), ctypes.byref(m), ctypes.byref(f), ctypes.byref(r))
        return m.value, f.value, r.value

    def pairs(self):
        n = int(self.lib.ow_pair_count(self.h))
        out = np.zeros((n, 2), np.uint32)
        if n:
            self.lib.ow_get_pairs(self.h, _ptr(out))
        return out

    def solve_order(self):
        n = int(self.lib.ow_contact_count(self.h))
        order = np.zeros(n, np.uint32)
        colors = np.zeros(n, np.uint32)
        if n:
            self.lib.ow_get_solve_order(self.h, _ptr(order), _ptr(colors))
        return order, colors

    def solve(self, manifolds, dt, iterations=8, order=None):
        m = np.ascontiguousarray(manifolds.copy())
        st = np.zeros(1, STATS_DTYPE)
        o = None if order is None else np.ascontiguousarray(order, np.uint32)
        self.lib.ow_solve(self.h, _ptr(m), len(m), float(dt), int(iterations), _ptr(o), _ptr(st))
        return m, st[0]

    def color(self, manifolds):
        m = np.ascontiguousarray(manifolds)
        order = np.zeros(len(m), np.uint32)
        colors = np.zeros(len(m), np.uint32)
        n = self.lib.ow_color_manifolds(self.h, _ptr(m), len(m), _ptr(order), _ptr(colors))
        return order, colors, int(n)


class RefWorld(_CpuWorld):
    """The unmodified reference PhysicsWorld (available where its sources are)."""

    _prefix = "rw_"

    def __init__(self, algo=0, workers=1):
        self.lib = ref_lib()
        self.h = self.lib.rw_create()
        self.lib.rw_set_broadphase(self.h, int(algo))
        self.lib.rw_set_workers(self.h, int(workers), int(workers), int(workers))

    def clone(self):
        w = RefWorld.__new__(RefWorld)
        w.lib = self.lib
        w.h = self.lib.rw_clone(self.h)
        return w

    def set_gravity(self, g):
        self.lib.rw_set_gravity(self.h, float(g[0]), float(g[1]), float(g[2]))

    def set_material(self, idx, mass, friction, restitution):
        self.lib.rw_set_material(self.h, int(idx), float(mass), float(friction), float(restitution))

    def bounds(self):
        n = self.body_count()
        mins = np.zeros((n, 3), np.float32)
        maxs = np.zeros((n, 3), np.float32)
        self.lib.rw_get_bounds(self.h, _ptr(mins), _ptr(maxs))
        return mins, maxs

    def solve(self, manifolds, dt, order=None):
        m = np.ascontiguousarray(manifolds.copy())
        st = np.zeros(1, STATS_DTYPE)
        o = None if order is None else np.ascontiguousarray(order, np.uint32)
        self.lib.rw_solve(self.h, _ptr(m), len(m), float(dt), _ptr(o), _ptr(st))
        return m, st[0]


def broadphase(lib_name, mins, maxs, algo, cell_size=0.0):
    """Stateless broadphase through the oracle ('oracle') or reference ('ref')."""
    mins = _f32(mins)
    maxs = _f32(maxs)
    n = len(mins)
    st = np.zeros(1, STATS_DTYPE)
    if lib_name == "oracle":
        lib = oracle_lib()
        count = lib.ow_broadphase(_ptr(mins), _ptr(maxs), n, int(algo), float(cell_size), None, 0, _ptr(st))
        pairs = np.zeros((count, 2), np.uint32)
        lib.ow_broadphase(_ptr(mins), _ptr(maxs), n, int(algo), float(cell_size), _ptr(pairs), count, _ptr(st))
    else:
        lib = ref_lib()
        count = lib.rw_broadphase(_ptr(mins), _ptr(maxs), n, int(algo), None, 0, _ptr(st))
        pairs = np.zeros((count, 2), np.uint32)
        lib.rw_broadphase(_ptr(mins), _ptr(maxs), n, int(algo), _ptr(pairs), count, _ptr(st))
    return pairs, st[0]


def generate_contact(lib_name, shape_a, dims_a, pos_a, quat_a, shape_b, dims_b, pos_b, quat_b):
    out = np.zeros(1, MANIFOLD_DTYPE)
    args = (int(shape_a), _ptr(_f32(dims_a)), _ptr(_f32(pos_a)), _ptr(_f32(quat_a)),
            int(shape_b), _ptr(_f32(dims_b)), _ptr(_f32(pos_b)), _ptr(_f32(quat_b)), _ptr(out))
    hit = (oracle_lib().ow_generate_contact if lib_name == "oracle" else ref_lib().rw_generate_contact)(*args)
    return bool(hit), out[0]


def gjk_epa(lib_name, points_a, points_b):
    a, b = _f32(points_a), _f32(points_b)
    normal = np.zeros(3, np.float32)
    depth = np.zeros(1, np.float32)
    size = np.zeros(1, np.uint32)
    fn = oracle_lib().ow_gjk_epa if lib_name == "oracle" else ref_lib().rw_gjk_epa
    rc = fn(_ptr(a), len(a), _ptr(b), len(b), _ptr(normal), _ptr(depth), _ptr(size))
    return int(rc), normal, float(depth[0]), int(size[0])
