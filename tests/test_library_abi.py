"""CPU checks of the C ABI library: it builds for sm_103a, loads, exports every
entry point include/hdg_gb300.h declares, and refuses to run without a GPU
(no CPU fallback).  No compute calls are made here."""
import ctypes
import os
import re
import subprocess

import pytest

from gridaphybrid_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hdg_gb300.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(hdg_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def libpath():
    return _build.build()


def test_library_is_in_tree(libpath):
    assert os.path.commonpath([libpath, ROOT]) == ROOT
    assert os.path.basename(libpath) == "libgridaphybrid_gb300.so"


def test_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(hdg_\w+)", out))
    decl = declared_functions()
    assert len(decl) >= 25
    missing = [f for f in decl if f not in exported]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_loads_with_ctypes(libpath):
    lib = ctypes.CDLL(libpath)
    for name in declared_functions():
        assert hasattr(lib, name)
    lib.hdg_version.restype = ctypes.c_int
    assert lib.hdg_version() >= 100


def test_build_targets_sm103a_only():
    assert _build.ARCH_FLAGS == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_device_means_error_not_fallback():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.hdg_context_create(0, ctypes.byref(h))
    assert rc == _lib.HDG_ERR_NODEVICE
    with pytest.raises(_lib.HdgError):
        _lib.Context(0)


def test_julia_shim_binds_only_declared_exported_entry_points(libpath):
    """The Julia binding is shipped as source (no Julia here): every entry point
    it ccalls must exist in the header and in the library."""
    shim = os.path.join(ROOT, "gridaphybrid.jl_gb300", "julia", "GridapHybridGB300.jl")
    called = set(re.findall(r"ccall\(\(:(hdg_[a-z0-9_]+),", open(shim).read()))
    assert len(called) >= 10
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(hdg_\w+)", out))
    decl = set(declared_functions())
    assert not (called - decl), sorted(called - decl)
    assert not (called - exported), sorted(called - exported)
