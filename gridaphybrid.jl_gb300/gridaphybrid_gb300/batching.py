"""Size-class batching of many Darcy HDG problems (hdg_batch_* in
include/hdg_gb300.h): the problems are grouped by (D, k) and each class is
integrated and condensed by one persistent fused launch over all its cells,
with the tile (threads per cell) picked by the library's autotuner and the
launch sequence replayed as a CUDA graph.  No reference counterpart: the
reference assembles one problem per HybridAffineFEOperator.
"""
import ctypes

import numpy as np

from . import _lib
from .operators import CartesianDiscreteModel, _Problem


class Batch:
    """problems: iterable of dicts with keys D, n, k and optionally kappa,
    problem (HDG_PROBLEM_*), stab (HDG_STAB_*), tau."""

    def __init__(self, problems, context=None):
        self.ctx = context or _lib.default_context()
        c = self.ctx
        self.specs = [dict(p) for p in problems]
        self.pbs = []
        for p in self.specs:
            D, n, k = p["D"], p["n"], p["k"]
            pb = _Problem(c, CartesianDiscreteModel((0, 1) * D, (n,) * D), k)
            c.check(c.lib.hdg_set_darcy(pb.h, p.get("stab", _lib.HDG_STAB_TEXTBOOK), p.get("tau", 1.0),
                                        p.get("problem", _lib.HDG_PROBLEM_SIN)))
            kap = p.get("kappa")
            if kap is not None:
                c.check(c.lib.hdg_set_permeability(pb.h, _lib.ptr(np.ascontiguousarray(kap, dtype=np.float64))))
            self.pbs.append(pb)
        handles = (ctypes.c_void_p * len(self.pbs))(*[pb.h.value for pb in self.pbs])
        h = ctypes.c_void_p()
        c.check(c.lib.hdg_batch_create(c.handle, len(self.pbs), handles, ctypes.byref(h)))
        self.h = h
        c.register(self)

    @property
    def cells(self):
        return sum(pb.ncells for pb in self.pbs)

    def assemble(self, precision=_lib.HDG_PREC_FF_BLOCK):
        bad = np.zeros(len(self.pbs), dtype=np.int32)
        self.ctx.check(self.ctx.lib.hdg_batch_assemble(self.h, precision, _lib.ptr(bad)))
        return bad

    def solve(self, rtol=1e-10, maxit=20000, solver=_lib.HDG_SOLVER_PCG):
        it = np.zeros(len(self.pbs), dtype=np.int32)
        rel = np.zeros(len(self.pbs))
        self.ctx.check(self.ctx.lib.hdg_batch_solve(self.h, solver, rtol, maxit, _lib.ptr(it), _lib.ptr(rel)))
        return it, rel

    def timings(self):
        ms = np.zeros(3)
        self.ctx.check(self.ctx.lib.hdg_batch_timings(self.h, _lib.ptr(ms)))
        return {"fused_integrate_condense_ms": float(ms[0]), "skeleton_assembly_ms": float(ms[1]),
                "solve_recover_ms": float(ms[2])}

    def tuning(self, precision):
        m = 16
        D, k, tpc = (np.zeros(m, dtype=np.int32) for _ in range(3))
        ms = np.zeros(m)
        cells = np.zeros(m, dtype=np.int64)
        nc = ctypes.c_int()
        self.ctx.check(self.ctx.lib.hdg_batch_tuning(self.h, precision, m, _lib.ptr(D), _lib.ptr(k), _lib.ptr(tpc),
                                                     _lib.ptr(ms), _lib.ptr(cells), ctypes.byref(nc)))
        return [{"D": int(D[i]), "k": int(k[i]), "threads_per_cell": int(tpc[i]),
                 "cells_per_cta": 256 // int(tpc[i]) if tpc[i] else 0, "fused_ms": float(ms[i]),
                 "cells": int(cells[i])} for i in range(nc.value)]

    def free_dof_values(self, i):
        pb = self.pbs[i]
        out = np.empty(pb.ncells * pb.ni + pb.nfree)
        self.ctx.check(self.ctx.lib.hdg_get_free_dof_values(pb.h, _lib.ptr(out)))
        return out

    def skeleton_values(self, i):
        pb = self.pbs[i]
        rhs = np.empty(pb.nfree)
        val = np.empty(pb.nnz)
        self.ctx.check(self.ctx.lib.hdg_get_skeleton_system(pb.h, None, None, _lib.ptr(val), _lib.ptr(rhs)))
        return val, rhs

    def close(self):
        if getattr(self, "h", None):
            if self.ctx.alive:
                self.ctx.lib.hdg_batch_destroy(self.h)
            self.h = None
        for pb in getattr(self, "pbs", []):
            pb.close()
        self.pbs = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batching_workload(nproblems=64, seed=0, sigma=1.5):
    """The batching workload: 2D Darcy HDG problems with n ~ U{16..128} cells
    per side, k ~ U{1,2,3}, per-cell permeability exp(N(0, sigma^2))."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nproblems):
        n = int(rng.integers(16, 129))
        k = int(rng.integers(1, 4))
        out.append({"D": 2, "n": n, "k": k, "kappa": np.exp(sigma * rng.normal(size=n * n))})
    return out
