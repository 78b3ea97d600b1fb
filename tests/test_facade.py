"""The header-only C++ facade (include/phys_gb300_world.hpp): it compiles
against the C ABI, a program written with the reference's public API runs on
the GPU, and the reference's own test programs compile against it with only
their include paths and namespace redirected."""
import os
import pathlib
import subprocess

import pytest

from phys_gb300 import _native

SRC = pathlib.Path(__file__).resolve().parent / "cpp" / "facade_scenarios.cpp"

# The reference's own test programs that use only the API the facade mirrors
# (the broadphase tests also drive the incremental DynamicAabbTree class, which
# is not part of the GPU path).
REFERENCE_PROGRAMS = ["solver/sequential_impulse_solver_tests.cpp", "world/sleeping_tests.cpp",
                      "collision/narrowphase_tests.cpp", "dynamics/rigid_body_tests.cpp"]
# The reference headers those programs include; each becomes a one-line shim
# that includes the facade and names it `phys`.
SHIM_HEADERS = ["world/physics_world", "solver/sequential_impulse_solver", "collision/narrowphase",
                "collision/broadphase", "dynamics/rigid_body", "math/math_utils", "core/constants"]


def link_args(so):
    return [f"-L{so.parent}", "-lphys_gb300", f"-Wl,-rpath,{so.parent}"]


def compile_program(out: pathlib.Path):
    so = _native.build_engine()
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", f"-I{_native.INCLUDE}", str(SRC), "-o", str(out),
           *link_args(so)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_facade_compiles(tmp_path):
    compile_program(tmp_path / "facade")
    assert (tmp_path / "facade").exists()


def test_reference_test_programs_compile_against_facade(tmp_path):
    """The reference's own test programs, read in place from its checkout,
    build against the facade: a shim directory maps each `phys/...` include to
    the facade and `namespace phys = phys_gb300;`.  The rigid-body program
    needs no device (bodies as values, host integration) and also runs here."""
    from oracle import cpu

    tests = cpu.REFERENCE_SRC / "tests"
    if not tests.is_dir():
        pytest.skip("the reference's sources are not present on this host")
    shim = tmp_path / "shim"
    for h in SHIM_HEADERS:
        f = shim / "phys" / f"{h}.hpp"
        f.parent.mkdir(parents=True, exist_ok=True)
        f.write_text('#pragma once\n#include "phys_gb300_world.hpp"\nnamespace phys = phys_gb300;\n')
    so = _native.build_engine()
    for prog in REFERENCE_PROGRAMS:
        exe = tmp_path / pathlib.Path(prog).stem
        res = subprocess.run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", f"-I{shim}", f"-I{_native.INCLUDE}",
                              str(tests / prog), "-o", str(exe), *link_args(so)], capture_output=True, text=True)
        assert res.returncode == 0, f"{prog}:\n{res.stderr[-3000:]}"
    res = subprocess.run([str(tmp_path / "rigid_body_tests")], capture_output=True, text=True, timeout=120,
                         env={**os.environ, "CUDA_VISIBLE_DEVICES": ""})
    assert res.returncode == 0, res.stdout + res.stderr


@pytest.mark.gpu
def test_facade_scenarios_run_on_gpu(tmp_path, gpu):
    exe = tmp_path / "facade"
    compile_program(exe)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "facade scenarios ok" in res.stdout
