"""Differentiable rollouts: batched worlds stepped forward on the GPU with a
hand-written adjoint (contact set frozen from the forward pass), a
``torch.autograd.Function`` around it, and the FP64 CPU evaluation of the same
step and adjoint used to check the GPU gradients.

State per body: position (3), rotation quaternion x, y, z, w (4), linear
velocity (3), angular velocity (3).  Parameters per body: mass (the RigidBody
``mass`` field; the local inverse inertia stays as created), friction and
restitution (the RigidBody fields).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native

_P = ctypes.c_void_p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _f64(a):
    return np.ascontiguousarray(a, np.float64)


_fp64 = None


def fp64_lib():
    global _fp64
    if _fp64 is None:
        lib = _native.fp64_lib()
        lib.pe_fp64_body_properties.argtypes = [ctypes.c_int, _P, ctypes.c_float, ctypes.c_int, _P, _P,
                                                ctypes.c_char_p, ctypes.c_int]
        lib.pe_fp64_body_properties.restype = ctypes.c_int
        lib.pe_fp64_rollout.argtypes = ([ctypes.c_uint32, _P, _P, _P, _P, _P, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_uint32] + [_P] * 22 + [ctypes.c_char_p, ctypes.c_int])
        lib.pe_fp64_rollout.restype = ctypes.c_int
        _fp64 = lib
    return _fp64


def body_properties(scene):
    """(mass[n], inverse inertia[n,3], half extents[n,3]) in float32, exactly as
    RigidBody::createSphere / createBox compute them; half extents hold the
    radius in column 0 for spheres."""
    lib = fp64_lib()
    n = scene.count
    mass = np.zeros(n, np.float32)
    iinv = np.zeros((n, 3), np.float32)
    err = ctypes.create_string_buffer(128)
    for i in range(n):
        m = ctypes.c_float()
        ii = np.zeros(3, np.float32)
        d = np.ascontiguousarray(scene.dims[i], np.float32)
        if lib.pe_fp64_body_properties(int(scene.shape[i]), _ptr(d), ctypes.c_float(float(scene.density[i])),
                                       int(scene.is_static[i]), ctypes.byref(m), _ptr(ii), err, 128) != 0:
            raise ValueError(f"body {i}: {err.value.decode()}")
        mass[i] = m.value
        iinv[i] = ii
    dims = scene.dims.astype(np.float32)
    he = np.where(scene.shape[:, None] == 0, dims, dims * np.float32(0.5)).astype(np.float32)
    return mass, iinv, he


def fp64_rollout(shape, is_static, half_extents, inv_inertia, state, mass, friction, restitution, steps, dt,
                 iterations, gravity=(0.0, -9.81, 0.0), d_final=None):
    """One world in double precision.  ``state`` = (x[n,3], q[n,4], v[n,3],
    w[n,3]); returns the final state, and with ``d_final`` (same shapes) also
    the gradients (dx0, dq0, dv0, dw0, dmass, dfriction, drestitution) of
    sum(d_final . final state).  Gravity and dt are rounded to float first, as
    the world stores them."""
    lib = fp64_lib()
    n = len(shape)
    x0, q0, v0, w0 = (_f64(a) for a in state)
    out = [np.zeros((n, 3)), np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 3))]
    grads = [np.zeros((n, 3)), np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n), np.zeros(n),
             np.zeros(n)]
    g = np.array([float(np.float32(c)) for c in gravity], np.float64)
    df = [None] * 4 if d_final is None else [_f64(a) for a in d_final]
    err = ctypes.create_string_buffer(256)
    rc = lib.pe_fp64_rollout(
        n, _ptr(np.ascontiguousarray(shape, np.uint8)), _ptr(np.ascontiguousarray(is_static, np.uint8)),
        _ptr(_f64(half_extents)), _ptr(_f64(inv_inertia)), _ptr(g), float(np.float32(dt)), int(iterations),
        int(steps), _ptr(x0), _ptr(q0), _ptr(v0), _ptr(w0), _ptr(_f64(mass)), _ptr(_f64(friction)),
        _ptr(_f64(restitution)), *[_ptr(o) for o in out], *[_ptr(a) for a in df],
        *[_ptr(a) if d_final is not None else None for a in grads], err, 256)
    if rc != 0:
        raise RuntimeError(f"fp64 rollout failed: {err.value.decode()}")
    return (out, grads) if d_final is not None else (out, None)


def initial_rotations(spin, is_static):
    """Rotations the body factories leave after the reference's orientation
    idiom setAngularVelocity(spin); integrateRotation(1); setAngularVelocity(0)
    (rigid_body.cpp:110-125), evaluated in float32 with the same operations."""
    spin = np.asarray(spin, np.float32)
    n = len(spin)
    q = np.zeros((n, 4), np.float32)
    q[:, 3] = 1
    h = np.float32(0.5) * np.float32(1.0)
    for i in range(n):
        wx, wy, wz = spin[i]
        if is_static[i] or (wx == 0 and wy == 0 and wz == 0):
            continue
        x, y, z, w = np.float32(0), np.float32(0), np.float32(0), np.float32(1)
        sw = np.float32(0)
        dx = sw * x + wx * w + wy * z - wz * y
        dy = sw * y - wx * z + wy * w + wz * x
        dz = sw * z + wx * y - wy * x + wz * w
        dw = sw * w - wx * x - wy * y - wz * z
        u = np.array([x + h * dx, y + h * dy, z + h * dz, w + h * dw], np.float32)
        ln = np.sqrt(np.float32(u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + u[3] * u[3]), dtype=np.float32)
        q[i] = u / ln if ln != 0 else np.array([0, 0, 0, 1], np.float32)
    return q


class GpuRollout:
    """Differentiable rollout of many worlds on the GPU (pe_rollout_*).  World w
    holds the bodies of ``scenes[w]``.  ``initial_state()`` gives the state the
    scene describes and ``mass``, ``friction``, ``restitution`` the created
    parameters, as numpy arrays; ``forward`` / ``backward`` take torch CUDA
    tensors."""

    def __init__(self, scenes, steps, dt, iterations=10, checkpoint_every=10, device=0, gravity=(0.0, -9.81, 0.0),
                 manifolds_per_body=None):
        from . import engine

        self.lib = engine.lib()
        self.device = device
        counts = np.array([s.count for s in scenes], np.uint32)
        cat = lambda f, dt_: np.ascontiguousarray(np.concatenate([getattr(s, f) for s in scenes]), dt_)
        self.shape = cat("shape", np.uint8)
        if np.any(self.shape > 1):
            raise ValueError("differentiable worlds hold spheres and boxes only")
        self.is_static = cat("is_static", np.uint8)
        self.counts = counts
        self.starts = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)])
        self.n = int(self.starts[-1])
        self.steps, self.dt, self.iterations = int(steps), float(dt), int(iterations)
        mass = np.zeros(self.n, np.float32)
        h = _P()
        engine.check(self.lib.pe_rollout_create(
            int(device), len(counts), _ptr(counts), _ptr(self.shape), _ptr(cat("dims", np.float32)),
            _ptr(cat("density", np.float32)), _ptr(self.is_static), int(steps), ctypes.c_float(dt), int(iterations),
            int(checkpoint_every), ctypes.byref(h), _ptr(mass)))
        self.h = h
        engine.check(self.lib.pe_rollout_set_gravity(self.h, *[float(g) for g in gravity]))
        if manifolds_per_body is not None:
            engine.check(self.lib.pe_rollout_set_manifold_capacity(self.h, float(manifolds_per_body)))
        self.mass = mass
        self.friction = np.maximum(cat("friction", np.float32), 0).astype(np.float32)
        self.restitution = np.clip(cat("restitution", np.float32), 0, 1).astype(np.float32)
        self._x0 = cat("pos", np.float32).reshape(-1, 3)
        self._q0 = initial_rotations(cat("spin", np.float32).reshape(-1, 3), self.is_static)
        self._v0 = cat("linvel", np.float32).reshape(-1, 3)
        self._w0 = np.zeros((self.n, 3), np.float32)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pe_rollout_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initial_state(self):
        return self._x0.copy(), self._q0.copy(), self._v0.copy(), self._w0.copy()

    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    @staticmethod
    def _p(t):
        return None if t is None else ctypes.c_void_p(t.data_ptr())

    def forward(self, x0, q0, v0, w0, mass, friction, restitution):
        import torch

        from . import engine

        args = [a.contiguous().float() for a in (x0, q0, v0, w0, mass, friction, restitution)]
        outs = [torch.empty_like(args[0]), torch.empty_like(args[1]), torch.empty_like(args[2]),
                torch.empty_like(args[3])]
        engine.check(self.lib.pe_rollout_forward(self.h, *[self._p(a) for a in args], *[self._p(o) for o in outs],
                                                 self._stream()))
        return outs

    def backward(self, dx, dq, dv, dw):
        import torch

        from . import engine

        dev = torch.device("cuda", self.device)
        g = [None if a is None else a.contiguous().float() for a in (dx, dq, dv, dw)]
        outs = [torch.empty((self.n, 3), device=dev), torch.empty((self.n, 4), device=dev),
                torch.empty((self.n, 3), device=dev), torch.empty((self.n, 3), device=dev),
                torch.empty(self.n, device=dev), torch.empty(self.n, device=dev), torch.empty(self.n, device=dev)]
        engine.check(self.lib.pe_rollout_backward(self.h, *[self._p(a) for a in g], *[self._p(o) for o in outs],
                                                  self._stream()))
        return outs

    def device_bytes(self) -> int:
        b = ctypes.c_uint64()
        self.lib.pe_rollout_device_bytes(self.h, ctypes.byref(b))
        return int(b.value)

    def timings(self):
        f, b = ctypes.c_double(), ctypes.c_double()
        self.lib.pe_rollout_timings(self.h, ctypes.byref(f), ctypes.byref(b))
        return f.value, b.value


def rollout_function():
    """torch.autograd.Function: (x0, q0, v0, w0, mass, friction, restitution)
    -> final (x, q, v, w), with the GPU adjoint as its backward."""
    import torch

    class RolloutFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, roll, x0, q0, v0, w0, mass, friction, restitution):
            ctx.roll = roll
            return tuple(roll.forward(x0, q0, v0, w0, mass, friction, restitution))

        @staticmethod
        def backward(ctx, dx, dq, dv, dw):
            return (None, *ctx.roll.backward(dx, dq, dv, dw))

    return RolloutFunction
