"""The C++ host facade (include/mcig/MCIntegrator.hpp) compiles against the C ABI
(CPU) and passes its integration checks on the GPU (tests/cpp/facade_test.cpp)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_facade_test():
    from mcintegratorplusplus_gb300 import _lib, build
    _lib.load()
    out = os.path.join(build.BUILD, "facade_test")
    subprocess.check_call(["g++", "-std=c++14", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "facade_test.cpp"), "-L", build.BUILD, "-lmcigpu",
                           "-Wl,-rpath," + build.BUILD, "-o", out])
    return out


def test_facade_compiles_and_links():
    assert os.path.exists(_build_facade_test())


@pytest.mark.gpu
def test_facade_integrates_on_gpu():
    exe = _build_facade_test()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "facade ok" in r.stdout
