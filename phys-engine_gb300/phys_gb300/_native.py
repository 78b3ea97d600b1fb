"""Locating, building and loading the native libraries of phys-engine-gb300.

* ``libphys_gb300.so`` — the CUDA engine (sm_103a kernels + the C ABI declared in
  include/phys_gb300.h).  There is no CPU fallback: if it cannot be loaded the
  engine raises.
* ``libpe_scenes.so`` — the host-only scene generator (include/phys_gb300_scenes.h).
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = pathlib.Path(__file__).resolve().parent.parent      # phys-engine_gb300/
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD = PKG_DIR / "_build"
INCLUDE = REPO_DIR / "include"
ENGINE_SO = BUILD / "libphys_gb300.so"
SCENES_SO = BUILD / "libpe_scenes.so"
FP64_SO = BUILD / "libphys_gb300_fp64.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    "-std=c++17", "-O3", "-lineinfo", ARCH,
    # Bit-exact parity with the reference needs every float expression rounded
    # as written: no fused multiply-add contraction; IEEE division and sqrt.
    "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-O3",
]
CXX_FLAGS = ["-std=c++20", "-O3", "-fPIC", "-ffp-contract=off", "-Wall"]

_lock = threading.Lock()
_libs: dict[str, ctypes.CDLL] = {}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (cand == "nvcc" or os.path.exists(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(map(str, cmd))}\n{res.stdout}\n{res.stderr}")
    return res


def _stale(target: pathlib.Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(pathlib.Path(s).stat().st_mtime > t for s in sources)


def build_scenes(force: bool = False) -> pathlib.Path:
    src = CSRC / "scenes.cpp"
    deps = [src, INCLUDE / "phys_gb300_scenes.h"]
    BUILD.mkdir(parents=True, exist_ok=True)
    if force or _stale(SCENES_SO, deps):
        _run(["g++", *CXX_FLAGS, f"-I{INCLUDE}", "-shared", "-o", str(SCENES_SO), str(src)])
    return SCENES_SO


def build_fp64(force: bool = False) -> pathlib.Path:
    """The FP64 CPU evaluation of the differentiable rollout (a checking
    library for the GPU adjoint; plain C++ built from the same headers)."""
    src = CSRC / "rollout_fp64.cpp"
    deps = [src, CSRC / "ad_math.cuh", CSRC / "ad_geom.cuh", CSRC / "ad_world.cuh", INCLUDE / "phys_gb300_fp64.h"]
    BUILD.mkdir(parents=True, exist_ok=True)
    if force or _stale(FP64_SO, deps):
        _run(["g++", *CXX_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-shared", "-o", str(FP64_SO), str(src)])
    return FP64_SO


def build_engine(force: bool = False) -> pathlib.Path:
    """Compile every .cu / .cpp under csrc/ (except scenes.cpp) for sm_103a and
    link libphys_gb300.so.  Translation units compile in parallel."""
    BUILD.mkdir(parents=True, exist_ok=True)
    cu = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    objs = []
    jobs = []
    for src in cu:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append(([_nvcc(), *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", "-o", str(obj), str(src)]))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(ENGINE_SO, objs):
        _run([_nvcc(), ARCH, "-shared", "-o", str(ENGINE_SO), *map(str, objs), "-lcudart"])
    return ENGINE_SO


def _load(path: pathlib.Path, builder) -> ctypes.CDLL:
    key = str(path)
    with _lock:
        if key not in _libs:
            if not path.exists():
                builder()
            _libs[key] = ctypes.CDLL(key)
        return _libs[key]


def scenes_lib() -> ctypes.CDLL:
    return _load(SCENES_SO, build_scenes)


def fp64_lib() -> ctypes.CDLL:
    return _load(FP64_SO, build_fp64)


def engine_lib() -> ctypes.CDLL:
    """The CUDA engine.  Raises if it is missing or fails to load: the engine
    has no host fallback."""
    if not ENGINE_SO.exists():
        raise RuntimeError(
            f"{ENGINE_SO} is not built; run __graft_entry__.build() (the GPU path has no CPU fallback)")
    return _load(ENGINE_SO, build_engine)
