"""Shared comparison helpers for the parity tests."""
import numpy as np


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def assert_bit_equal(actual, expected, what=""):
    a, e = np.asarray(actual), np.asarray(expected)
    assert a.shape == e.shape, f"{what}: shape {a.shape} != {e.shape}"
    if a.dtype == np.float32:
        diff = np.argwhere(bits(a) != bits(e))
        assert diff.size == 0, f"{what}: {len(diff)} values differ, first at {diff[0]}: {a[tuple(diff[0])]} vs {e[tuple(diff[0])]}"
    else:
        assert np.array_equal(a, e), f"{what}: arrays differ"


MANIFOLD_FIELDS = ("body_a_index", "body_a_generation", "body_b_index", "body_b_generation", "normal",
                   "point_count", "friction", "restitution", "anchor_a", "anchor_b", "penetration",
                   "normal_impulse", "tangent_impulse1", "tangent_impulse2")


def assert_manifolds_equal(actual, expected, features=True, what="manifolds"):
    assert len(actual) == len(expected), f"{what}: count {len(actual)} != {len(expected)}"
    for f in MANIFOLD_FIELDS + (("feature",) if features else ()):
        assert_bit_equal(actual[f], expected[f], f"{what}.{f}")


def colors_valid(manifolds, colors, static_mask):
    """No two manifolds of one colour share a non-static body."""
    seen = {}
    for m, c in enumerate(colors):
        for b in (int(manifolds["body_a_index"][m]), int(manifolds["body_b_index"][m])):
            if static_mask[b]:
                continue
            key = (int(c), b)
            if key in seen:
                return False
            seen[key] = m
    return True
