"""CPU checks of the native libraries: they build, load, and export every
entry point the public headers declare (no GPU work is done here)."""
import ctypes
import re

import numpy as np

from phys_gb300 import _native, engine, scenes


def declared(header):
    text = (_native.INCLUDE / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pe_[a-z0-9_]+)\s*\(", text)))


def test_engine_exports_every_declared_symbol():
    so = _native.build_engine()
    lib = ctypes.CDLL(str(so))
    names = declared("phys_gb300.h")
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(engine.SIGNATURES), set(names) ^ set(engine.SIGNATURES)


def test_scene_library_exports():
    lib = ctypes.CDLL(str(_native.build_scenes()))
    for n in declared("phys_gb300_scenes.h"):
        assert hasattr(lib, n), n


def test_fp64_library_exports():
    lib = ctypes.CDLL(str(_native.build_fp64()))
    names = declared("phys_gb300_fp64.h")
    assert names == ["pe_fp64_body_properties", "pe_fp64_rollout"]
    for n in names:
        assert hasattr(lib, n), n


def test_scenes_are_deterministic_and_valid():
    a = scenes.generate(scenes.MIXED_VOLUME, 2000, 42)
    b = scenes.generate(scenes.MIXED_VOLUME, 2000, 42)
    assert a.count == 2000
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.spin, b.spin)
    assert int((a.shape == 0).sum()) == 1000
    assert np.all(a.density == 1.0)
    # bounding spheres do not overlap
    r = np.where(a.shape == 0, a.dims[:, 0], np.linalg.norm(a.dims / 2, axis=1))
    d = np.linalg.norm(a.pos[:, None] - a.pos[None], axis=2)
    np.fill_diagonal(d, np.inf)
    assert np.all(d >= (r[:, None] + r[None]) - 1e-4)
    p = scenes.generate(scenes.PYRAMIDS, 2, 42)
    assert int((p.shape == 2).sum()) == 20000 * 4 // 256
    assert int((p.shape == 1).sum() - p.is_static.sum()) == 4 * 210


def test_last_error_without_device():
    lib = engine.lib()
    assert isinstance(lib.pe_last_error(), bytes)
    assert lib.pe_device_count() >= 0
