"""Affine meshes whose cell Jacobians are not diagonal.

The Cartesian meshes of the other tests have diagonal Jacobians. On those the
float-float integration skips the terms whose coefficients are structurally
zero, which leaves the general-Jacobian code paths unexercised. Here a
Cartesian mesh's topology is re-created through hdg_problem_create, with every
cell mapped by one global skew x -> B x. Three checks:
  * the assembled skeleton matrix against the oracle's affine-cell integration
    (orc_integrate_darcy_affine), condensation and assembly;
  * the fast precisions agree with the plain FP64 path, whose integration is
    independent code (test/DarcyHDGTests.jl:137-142 solves the same form);
  * with a linear pressure and kappa = 1 every path is exact on an affine mesh
    (the reference's exactness check, test/DarcyHDGTests.jl:142).
"""
import ctypes

import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from gridaphybrid_gb300.operators import _Problem
from oracle import oracle

pytestmark = pytest.mark.gpu

SKEW = {2: np.array([[1.0, 0.3], [0.2, 1.0]]),
        3: np.array([[1.0, 0.3, 0.1], [0.1, 1.0, 0.2], [0.05, 0.1, 1.0]])}


def relmax(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def skewed_problem(ctx, D, k, n):
    """The Cartesian [0,1]^D mesh with n cells per direction, every cell mapped by SKEW[D]."""
    base = _Problem(ctx, gh.CartesianDiscreteModel((0, 1) * D, n), k)
    cf, _, fd = base.topology()
    ncells, nfacets = base.ncells, base.nfacets
    base.close()
    B = SKEW[D]
    h = np.array([1.0 / m for m in n])
    origin = np.empty((ncells, D))
    jac = np.empty((ncells, D, D))  # [cell][col][row]: column-major per cell
    for c in range(ncells):
        idx, r = [], c
        for d in range(D):  # Gridap numbering: first direction fastest
            idx.append(r % n[d])
            r //= n[d]
        origin[c] = B @ (np.array(idx) * h)
        jac[c] = (B @ np.diag(h)).T
    ph = ctypes.c_void_p()
    ctx.check(ctx.lib.hdg_problem_create(ctx.handle, D, k, ncells, nfacets, _lib.ptr(np.ascontiguousarray(origin)),
                                         _lib.ptr(np.ascontiguousarray(jac)), _lib.ptr(np.ascontiguousarray(cf)),
                                         _lib.ptr(np.ascontiguousarray(fd)), ctypes.byref(ph)))
    info = np.zeros(8, dtype=np.int64)
    ctx.check(ctx.lib.hdg_problem_info(ph, _lib.ptr(info)))
    return ph, ncells, int(info[2]), int(info[4]), int(info[6]), origin, jac


def solve(ctx, ph, ncells, ni, nfree, precision, problem, kappa):
    ctx.check(ctx.lib.hdg_set_darcy(ph, _lib.HDG_STAB_TEXTBOOK, 1.0, problem))
    out = np.empty(ncells * ni + nfree)
    stats = np.zeros(8)
    kap = None if kappa is None else _lib.ptr(np.ascontiguousarray(kappa))
    ctx.check(ctx.lib.hdg_solve(ph, precision, _lib.HDG_SOLVER_PCG, 1e-12, 20000, kap, _lib.ptr(out),
                                _lib.ptr(stats)))
    ef, ep = ctypes.c_double(), ctypes.c_double()
    ctx.check(ctx.lib.hdg_l2_errors(ph, ctypes.byref(ef), ctypes.byref(ep)))
    return out, ef.value, ep.value


CASES = [(2, 1, (5, 4)), (2, 3, (4, 5)), (3, 1, (3, 2, 3)), (3, 2, (3, 3, 2))]
FAST = [_lib.HDG_PREC_FP32_REFINED, _lib.HDG_PREC_FF_BLOCK]


@pytest.mark.parametrize("D,k,n", CASES)
def test_skewed_mesh_fast_paths_match_fp64(D, k, n):
    ctx = gh.Context(0)
    ph, ncells, ni, nfree, _, _, _ = skewed_problem(ctx, D, k, n)
    kappa = np.exp(np.random.default_rng(5).normal(size=ncells))
    try:
        ref, ef64, _ = solve(ctx, ph, ncells, ni, nfree, _lib.HDG_PREC_FP64, _lib.HDG_PROBLEM_SIN, kappa)
        for prec in FAST:
            x, ef, _ = solve(ctx, ph, ncells, ni, nfree, prec, _lib.HDG_PROBLEM_SIN, kappa)
            assert relmax(x, ref) < 1e-8, prec
            assert abs(ef - ef64) <= 1e-6 * ef64
    finally:
        ctx.lib.hdg_problem_destroy(ph)
        ctx.close()


@pytest.mark.parametrize("D,k,n", CASES)
def test_skewed_mesh_linear_pressure_is_exact(D, k, n):
    ctx = gh.Context(0)
    ph, ncells, ni, nfree, _, _, _ = skewed_problem(ctx, D, k, n)
    try:
        for prec in [_lib.HDG_PREC_FP64] + FAST:
            _, ef, ep = solve(ctx, ph, ncells, ni, nfree, prec, _lib.HDG_PROBLEM_LINEAR, None)
            assert ef < 1e-8 and ep < 1e-8, prec
    finally:
        ctx.lib.hdg_problem_destroy(ph)
        ctx.close()


@pytest.mark.parametrize("D,k,n", CASES)
@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FP64, _lib.HDG_PREC_FF_BLOCK])
def test_skewed_mesh_assembled_matrix_vs_oracle(D, k, n, precision):
    ctx = gh.Context(0)
    ph, ncells, ni, nfree, nnz, origin, jac = skewed_problem(ctx, D, k, n)
    kappa = np.exp(np.random.default_rng(9).normal(size=ncells))
    try:
        ctx.check(ctx.lib.hdg_set_darcy(ph, _lib.HDG_STAB_TEXTBOOK, 1.0, _lib.HDG_PROBLEM_SIN))
        ctx.check(ctx.lib.hdg_set_permeability(ph, _lib.ptr(kappa)))
        info = np.zeros(ncells, dtype=np.int32)
        ctx.check(ctx.lib.hdg_assemble(ph, precision, _lib.ptr(info)))
        rowptr = np.empty(nfree + 1, dtype=np.int64)
        colind = np.empty(nnz, dtype=np.int32)
        val = np.empty(nnz)
        rhs = np.empty(nfree)
        ctx.check(ctx.lib.hdg_get_skeleton_system(ph, _lib.ptr(rowptr), _lib.ptr(colind), _lib.ptr(val),
                                                  _lib.ptr(rhs)))
    finally:
        ctx.lib.hdg_problem_destroy(ph)
        ctx.close()
    m = oracle.Mesh(D, n, k)
    A, b = m.integrate_affine(origin, jac, stab=oracle.STAB_TEXTBOOK, problem=oracle.PROBLEM_SIN, kappa=kappa)
    S, g, _ = oracle.static_condensation(A, b, m.ni)
    r0, c0, v0, _ = m.assemble(S, g, np.zeros(m.ndir))
    assert np.array_equal(rowptr, r0) and np.array_equal(colind, c0)
    assert relmax(val, v0) < 1e-12
