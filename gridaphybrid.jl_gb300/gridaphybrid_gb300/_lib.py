"""ctypes binding of libgridaphybrid_gb300.so (the C ABI in include/hdg_gb300.h).

There is no CPU fallback: if the library is missing or no sm_103a device is
present, every call raises.
"""
import ctypes
import os
import re
import weakref

import numpy as np

from . import _build

HDG_OK = 0
HDG_ERR_INVALID = 1
HDG_ERR_CUDA = 2
HDG_ERR_NOMEM = 3
HDG_ERR_SINGULAR = 4
HDG_ERR_NOT_CONVERGED = 5
HDG_ERR_STATE = 6
HDG_ERR_NODEVICE = 7

HDG_PREC_FP64 = 0
HDG_PREC_FP32_REFINED = 1
HDG_PREC_FF_BLOCK = 2
HDG_STAB_TEXTBOOK = 0
HDG_STAB_OWNER_SIGN = 1
HDG_PROBLEM_REF_LINEAR = 0
HDG_PROBLEM_LINEAR = 1
HDG_PROBLEM_SIN = 2
HDG_PHYSICS_DARCY = 0
HDG_PHYSICS_ELASTICITY = 1
HDG_EPROBLEM_LINEAR = 0
HDG_EPROBLEM_SMOOTH = 1
HDG_SOLVER_PCG = 0
HDG_SOLVER_DIRECT = 1
HDG_SPACE_Q = 0
HDG_SPACE_P = 1
HDG_SPACE_RT = 2

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                      "include", "hdg_gb300.h")


def _header_bytes_constant(name):
    """A byte-size macro of the C header, e.g. `#define NAME (32u * 1024u * 1024u)`."""
    with open(HEADER) as f:
        m = re.search(r"#define\s+%s\s+\(([^)]*)\)" % name, f.read())
    val = 1
    for factor in m.group(1).split("*"):
        val *= int(factor.strip().rstrip("uU"))
    return val


# Size of the fixed scratch array of hdg_static_condensation_noalloc.
HDG_NOALLOC_SCRATCH_BYTES = _header_bytes_constant("HDG_NOALLOC_SCRATCH_BYTES")

_ERR_NAMES = {
    1: "HDG_ERR_INVALID", 2: "HDG_ERR_CUDA", 3: "HDG_ERR_NOMEM", 4: "HDG_ERR_SINGULAR",
    5: "HDG_ERR_NOT_CONVERGED", 6: "HDG_ERR_STATE", 7: "HDG_ERR_NODEVICE",
}

# Every exported entry point with its C signature (restype, argtypes).
_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_ll = ctypes.c_longlong
SIGNATURES = {
    "hdg_version": (_i, []),
    "hdg_device_allocations": (_i, [ctypes.POINTER(_ll)]),
    "hdg_pointer_placement": (_i, [_i, _i, _i, ctypes.POINTER(_i)]),
    "hdg_context_create": (_i, [_i, ctypes.POINTER(_vp)]),
    "hdg_context_destroy": (_i, [_vp]),
    "hdg_last_error": (ctypes.c_char_p, [_vp]),
    "hdg_context_synchronize": (_i, [_vp]),
    "hdg_launch_count": (_ll, [_vp]),
    "hdg_context_record": (_i, [_vp, _i]),
    "hdg_context_elapsed_ms": (_i, [_vp, _i, _i, _vp]),
    "hdg_static_condensation": (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "hdg_backward_static_condensation": (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "hdg_sum_facets": (_i, [_vp, _i, _i, _i, _vp, _vp]),
    "hdg_static_condensation_noalloc": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "hdg_problem_create_cartesian": (_i, [_vp, _i, _vp, _vp, _i, ctypes.POINTER(_vp)]),
    "hdg_problem_create": (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "hdg_problem_create_cartesian_physics": (_i, [_vp, _i, _vp, _vp, _i, _i, ctypes.POINTER(_vp)]),
    "hdg_problem_create_cartesian_spaces": (_i, [_vp, _i, _vp, _vp, _i, _vp, _i, ctypes.POINTER(_vp)]),
    "hdg_problem_create_simplex_spaces": (_i, [_vp, _i, _vp, _vp, _i, _vp, _i, ctypes.POINTER(_vp)]),
    "hdg_set_elasticity": (_i, [_vp, _d, _d, _i]),
    "hdg_problem_destroy": (_i, [_vp]),
    "hdg_problem_info": (_i, [_vp, _vp]),
    "hdg_get_topology": (_i, [_vp, _vp, _vp, _vp]),
    "hdg_set_darcy": (_i, [_vp, _i, _d, _i]),
    "hdg_set_permeability": (_i, [_vp, _vp]),
    "hdg_set_dirichlet_values": (_i, [_vp, _vp]),
    "hdg_assemble": (_i, [_vp, _i, _vp]),
    "hdg_get_skeleton_system": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "hdg_solve_skeleton": (_i, [_vp, _i, _d, _i, _vp, _vp]),
    "hdg_recover": (_i, [_vp]),
    "hdg_get_free_dof_values": (_i, [_vp, _vp]),
    "hdg_get_cell_interior_values": (_i, [_vp, _vp]),
    "hdg_get_skeleton_values": (_i, [_vp, _vp]),
    "hdg_l2_errors": (_i, [_vp, _vp, _vp]),
    "hdg_solve": (_i, [_vp, _i, _i, _d, _i, _vp, _vp, _vp]),
    "hdg_get_timings": (_i, [_vp, _vp]),
    "hdg_get_solve_stats": (_i, [_vp, _vp]),
    "hdg_context_set_persistent_pcg": (_i, [_vp, ctypes.c_int]),
    "hdg_time_kernel": (_i, [_vp, _i, _i, _vp]),
    "hdg_measure_pipe_peaks": (_i, [_vp, _vp, _vp]),
    "hdg_check_bounded_waits": (_i, [_vp, ctypes.c_uint, _vp, _vp]),
    "hdg_problem_device_bytes": (_i, [_vp, _vp]),
    "hdg_set_refinement": (_i, [_vp, _d, _i]),
    "hdg_newton_solve": (_i, [_vp, _i, _d, _i, _d, _i, _vp, _vp, _vp]),
    "hdg_footprint": (_i, [_i, _i, _i, _i, _i, _vp]),
    "hdg_batch_create": (_i, [_vp, _i, _vp, ctypes.POINTER(_vp)]),
    "hdg_batch_destroy": (_i, [_vp]),
    "hdg_batch_assemble": (_i, [_vp, _i, _vp]),
    "hdg_batch_solve": (_i, [_vp, _i, _d, _i, _vp, _vp]),
    "hdg_batch_timings": (_i, [_vp, _vp]),
    "hdg_batch_tuning": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "hdg_server_create": (_i, [_i, _i, _d, ctypes.POINTER(_vp)]),
    "hdg_server_destroy": (_i, [_vp]),
    "hdg_server_submit": (_i, [_vp, _vp, _vp]),
    "hdg_server_poll": (_i, [_vp, _vp, _i, _d, _vp]),
    "hdg_server_drain": (_i, [_vp, _d]),
    "hdg_server_stats": (_i, [_vp, _vp]),
    "hdg_server_last_error": (ctypes.c_char_p, [_vp]),
}


class Request(ctypes.Structure):
    """struct hdg_request."""
    _fields_ = [("D", _i), ("n", _i), ("k", _i), ("problem", _i), ("stab_mode", _i), ("precision", _i),
                ("solver", _i), ("maxit", _i), ("tau", _d), ("rtol", _d), ("kappa", _vp), ("solution", _vp)]


class Response(ctypes.Structure):
    """struct hdg_response."""
    _fields_ = [("ticket", _ll), ("status", _i), ("iters", _i), ("relres", _d), ("err_flux", _d),
                ("err_pressure", _d), ("queue_ms", _d), ("run_ms", _d), ("latency_ms", _d),
                ("footprint_bytes", _d), ("reused_mesh", _i), ("slot", _i), ("message", ctypes.c_char * 160)]


class HdgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_ERR_NAMES.get(code, "HDG_ERR"), code, msg))
        self.code = code


_LIB = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=False):
    """Load the shared library (raises if it is absent and not built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(
                "libgridaphybrid_gb300.so is not built (run __graft_entry__.build()); "
                "there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def ptr(a):
    """Pointer of a C-contiguous numpy array (or None); torch tensors by data_ptr()."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("arrays passed to the C ABI must be C-contiguous")
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """One GPU + stream (hdg_context).  Objects that live on the context
    (problems, batches) register themselves and are released before it, so
    the context is never destroyed under them (e.g. when the interpreter
    tears down its objects in arbitrary order)."""

    def __init__(self, device=0):
        self.lib = load()
        self._children = weakref.WeakSet()
        h = ctypes.c_void_p()
        rc = self.lib.hdg_context_create(device, ctypes.byref(h))
        if rc != HDG_OK:
            raise HdgError(rc, "hdg_context_create(device=%d) failed: no usable sm_103a GPU" % device)
        self.handle = h

    def register(self, obj):
        self._children.add(obj)

    @property
    def alive(self):
        return getattr(self, "handle", None) is not None

    def check(self, rc):
        if rc != HDG_OK:
            raise HdgError(rc, self.lib.hdg_last_error(self.handle).decode())
        return rc

    @property
    def launches(self):
        return int(self.lib.hdg_launch_count(self.handle))

    def synchronize(self):
        self.check(self.lib.hdg_context_synchronize(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            for child in list(getattr(self, "_children", ())):
                try:
                    child.close()
                except Exception:
                    pass
            self.lib.hdg_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_DEFAULT = None


def default_context():
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Context(0)
    return _DEFAULT


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)
