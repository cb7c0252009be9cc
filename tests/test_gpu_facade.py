"""The C++ façade (include/tagpu/tiledarray.hpp) compiles TiledArray-style
expressions unchanged and runs them through libtagpu.so."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_facade(tmp_path):
    from tiledarray_gb300 import build as tb
    lib = tb.build()
    exe = str(tmp_path / "test_facade")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_facade.cpp"), "-o", exe,
                    lib, "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def test_facade_compiles(tmp_path):
    assert os.path.exists(build_facade(tmp_path))


def test_facade_services_compile(tmp_path):
    """truncate, is_zero, find, save and load compile as a TiledArray user
    would call them (compile only)."""
    obj = str(tmp_path / "facade_api.o")
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-c",
                    "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_api.cpp"), "-o", obj], check=True)
    assert os.path.exists(obj)


@pytest.mark.gpu
def test_facade_runs(tmp_path):
    exe = build_facade(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 4
