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
