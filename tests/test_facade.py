"""The header-only C++ facade (include/phys_gb300_world.hpp) compiles against
the C ABI, and a program written like the reference's own tests runs on the GPU."""
import pathlib
import subprocess

import pytest

from phys_gb300 import _native

SRC = pathlib.Path(__file__).resolve().parent / "cpp" / "facade_scenarios.cpp"


def compile_program(out: pathlib.Path):
    so = _native.build_engine()
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{_native.INCLUDE}", str(SRC), "-o", str(out),
           f"-L{so.parent}", "-lphys_gb300", f"-Wl,-rpath,{so.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_facade_compiles(tmp_path):
    compile_program(tmp_path / "facade")
    assert (tmp_path / "facade").exists()


@pytest.mark.gpu
def test_facade_scenarios_run_on_gpu(tmp_path, gpu):
    exe = tmp_path / "facade"
    compile_program(exe)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "facade scenarios ok" in res.stdout
