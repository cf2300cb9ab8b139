"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports every entry point include/mcig.h declares (no device calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in ("mcig.h",):
        src = open(os.path.join(ROOT, "include", hdr)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_\s\*]*?\b(mcig_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "mcig_integrate" in names and "mcig_create" in names and len(names) > 40


def test_library_exports_every_declared_symbol():
    from mcintegratorplusplus_gb300 import _lib
    L = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # and the binding declares a signature for each of them
    assert not [n for n in declared_functions() if n not in _lib.SIGNATURES]


def test_library_is_built_for_sm_103a():
    from mcintegratorplusplus_gb300 import build
    log = open(os.path.join(build.BUILD, "sample_generic_f64.log")).read()
    assert "arch=compute_103a,code=sm_103a" in log
    assert "-fmad=false" in log


def test_version_and_error_string():
    from mcintegratorplusplus_gb300 import _lib
    L = _lib.load()
    assert b"sm_103a" in L.mcig_version()
    assert isinstance(L.mcig_last_error(), bytes)


def test_create_rejects_bad_arguments_before_touching_a_device():
    from mcintegratorplusplus_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.mcig_create(0, 1, 0, 0, ctypes.byref(h)) == 1  # ndim < 1: invalid_argument
    assert b"dimensions" in L.mcig_last_error()
    assert L.mcig_create(65, 1, 0, 0, ctypes.byref(h)) == 5  # beyond the device maximum
    assert L.mcig_create(3, 0, 0, 0, ctypes.byref(h)) == 1


def test_python_mirror_names_follow_reference():
    from mcintegratorplusplus_gb300 import MCI
    for name in ("setSeed", "setX", "getX", "centerX", "setMRT2Step", "getMRT2Step", "setTargetAcceptanceRate",
                 "setNfindMRT2Iterations", "setNdecorrelationSteps", "setTrialMove", "addSamplingFunction",
                 "popSamplingFunction", "clearSamplingFunctions", "addObservable", "popObservable",
                 "clearObservables", "setIRange", "resetDomain", "integrate", "getAcceptanceRate", "getNObsDim"):
        assert hasattr(MCI, name), name
