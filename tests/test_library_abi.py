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


def _c_kind(decl):
    """'int' / 'double' / 'longlong' / 'ptr' of a C parameter or return type."""
    decl = decl.strip()
    if "*" in decl:
        return "ptr"
    words = [w for w in decl.replace("const ", " ").split() if w not in ("unsigned",)]
    if words[:2] == ["long", "long"]:
        return "longlong"
    if decl.split()[0] == "unsigned" and words in ([], ["int"]):
        return "uint"
    return words[0]


def c_prototypes():
    """name -> (return kind, [parameter kinds]) of every function the header declares."""
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = {}
    for ret, name, params in re.findall(r"([A-Za-z_][A-Za-z0-9_ \*]*?)\b(hdg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", txt):
        params = params.strip()
        # each parameter without its name
        kinds = [] if params in ("", "void") else [
            _c_kind(re.sub(r"\b[A-Za-z_][A-Za-z0-9_]*\s*$", "", p)) for p in params.split(",")]
        protos[name] = (_c_kind(ret), kinds)
    return protos


_JULIA_KIND = {"Cint": "int", "Int32": "int", "Cuint": "uint", "UInt32": "uint", "Cdouble": "double", "Float64": "double", "Clonglong": "longlong",
               "Int64": "longlong", "Cstring": "ptr"}


def _julia_kind(t):
    t = t.strip()
    if t.startswith(("Ptr{", "Ref{")) or t == "Cstring":
        return "ptr"
    return _JULIA_KIND[t]


def _split_top(s):
    """Split a comma-separated list at depth 0 (braces and parentheses nest)."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [x.strip() for x in out if x.strip()]


def julia_ccalls(src):
    """(name, return type, [argument types], [arguments]) of every ccall in the Julia source."""
    calls = []
    for m in re.finditer(r"ccall\(\(:(hdg_[a-z0-9_]+),\s*LIB\)", src):
        i, depth = m.start() + len("ccall("), 1
        j = i
        while depth:
            depth += {"(": 1, ")": -1}.get(src[j], 0)
            j += 1
        parts = _split_top(src[i:j - 1])
        ret, types = parts[1], parts[2]
        assert types.startswith("(") and types.endswith(")"), (m.group(1), types)
        calls.append((m.group(1), ret, _split_top(types[1:-1]), parts[3:]))
    return calls


def test_c_prototype_parser_reads_every_declaration():
    protos = c_prototypes()
    assert set(protos) == set(declared_functions())
    assert protos["hdg_static_condensation"] == ("int", ["ptr", "int", "int", "int", "int", "ptr", "ptr", "ptr",
                                                         "ptr", "ptr"])
    assert protos["hdg_launch_count"] == ("longlong", ["ptr"])
    assert protos["hdg_last_error"] == ("ptr", ["ptr"])
    assert protos["hdg_version"] == ("int", [])
    assert protos["hdg_check_bounded_waits"] == ("int", ["ptr", "uint", "ptr", "ptr"])


def test_python_binding_matches_c_prototypes():
    """Every ctypes signature has the C prototype's return kind, argument count and kinds."""
    def kind(t):
        if t is None:
            return "void"
        if t in (ctypes.c_int,):
            return "int"
        if t in (ctypes.c_uint,):
            return "uint"
        if t in (ctypes.c_double,):
            return "double"
        if t in (ctypes.c_longlong,):
            return "longlong"
        return "ptr"
    protos = c_prototypes()
    for name, (res, args) in _lib.SIGNATURES.items():
        ret, params = protos[name]
        assert kind(res) == ret, name
        assert [kind(a) for a in args] == params, name


def test_julia_ccalls_match_c_prototypes():
    """Every ccall of the Julia shim passes as many arguments as the C
    prototype has parameters, each of the prototype's kind (a transposed
    Cint / Cdouble, a missing argument or a wrong return type fails here)."""
    shim = os.path.join(ROOT, "gridaphybrid.jl_gb300", "julia", "GridapHybridGB300.jl")
    calls = julia_ccalls(open(shim).read())
    assert len(calls) >= 15
    protos = c_prototypes()
    for name, ret, types, args in calls:
        cret, params = protos[name]
        assert _julia_kind(ret) == cret, (name, ret)
        assert [_julia_kind(t) for t in types] == params, (name, types)
        assert len(args) == len(types), (name, args)


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


def test_pointer_placement_rule():
    """The rule the entry points apply to caller pointers (cudaMemoryType
    values: 0 unregistered, 1 host, 2 device, 3 managed): device memory of
    another GPU is refused with HDG_ERR_INVALID instead of being handed to a
    kernel that would fault on it."""
    lib = _lib.load()
    place = ctypes.c_int(-1)
    cases = [((0, -2, 0), _lib.HDG_OK, 0), ((1, 0, 0), _lib.HDG_OK, 0), ((2, 0, 0), _lib.HDG_OK, 1),
             ((2, 3, 3), _lib.HDG_OK, 1), ((3, 1, 0), _lib.HDG_OK, 1), ((2, 1, 0), _lib.HDG_ERR_INVALID, 2),
             ((2, 0, 5), _lib.HDG_ERR_INVALID, 2)]
    for args, rc, where in cases:
        assert lib.hdg_pointer_placement(*args, ctypes.byref(place)) == rc, args
        assert place.value == where, args
    assert lib.hdg_pointer_placement(2, 0, 0, None) == _lib.HDG_ERR_INVALID


def test_device_allocation_counter_without_gpu():
    lib = _lib.load()
    n = ctypes.c_longlong(-1)
    assert lib.hdg_device_allocations(ctypes.byref(n)) == _lib.HDG_OK
    assert n.value >= 0
