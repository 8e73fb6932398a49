"""Builds tests/cpp/test_wrappers.cpp against include/fluidloom_gb300.hpp and the
in-tree library with g++, then runs it on the GPU (the C++ host layer)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build():
    from fluidloom_gb300 import build
    lib = build.build()
    out = os.path.join(ROOT, "fluidloom_gb300", "_lib", "test_wrappers")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_wrappers.cpp"), "-L", os.path.dirname(lib),
                    "-lfluidloom_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", out], check=True)
    return out


def test_cpp_wrappers_compile():
    _build()


@pytest.mark.gpu
def test_cpp_wrappers_run():
    r = subprocess.run([_build()], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ALL PASSED" in r.stdout, r.stdout + r.stderr
