"""GPU tests of the linear elasticity HDG path
(test/LinearElasticityHDGTests.jl) against the C oracle: condensed blocks and
assembled systems in FP64 to 1e-12, solutions in FP64 and in FP32 LU + float-
float refinement against the FP64 oracle, the linear-displacement exactness
and the precision error report of the elasticity workload."""
import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def _op(D, k, n, nu, precision, problem="smooth", tau=None):
    model = gh.CartesianDiscreteModel((0, 1) * D, n)
    X, Y = gh.elasticity_spaces(model, k)
    return gh.HybridAffineFEOperator(gh.ElasticityHDG(tau=tau, nu=nu, problem=problem), X, Y, [1, 2], [3],
                                     precision=precision)


CASES = [(2, 1, (4, 3)), (2, 2, (3, 3)), (2, 3, (3, 2)), (3, 1, (3, 2, 2))]
# 3D k=2 (cell block n = 405): FP64 by block elimination, beyond the shared-memory LU
CASES_K2 = [(3, 2, (2, 2, 2))]


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FP64, _lib.HDG_PREC_FF_BLOCK])
@pytest.mark.parametrize("D,k,n", CASES + CASES_K2)
def test_elasticity_assembled_system_matches_oracle(D, k, n, precision):
    """FP64: to 1e-12.  Float-float block elimination: the condensed operator
    to 1e-12 as well (~48-bit arithmetic, no refinement involved)."""
    nu = np.random.default_rng(2).uniform(0.2, 0.45, size=int(np.prod(n)))
    op = _op(D, k, n, nu, precision)
    rowptr, colind, val, rhs = op.skeleton_system()
    m = oracle.ElasticityMesh(D, n, k)
    A, b = m.integrate(tau=float(n[0]), nu=nu, problem=oracle.EPROBLEM_SMOOTH)
    S, g, info = oracle.static_condensation(A, b, m.ni)
    r0, c0, v0, rhs0 = m.assemble(S, g, m.dirichlet_values(oracle.EPROBLEM_SMOOTH))
    assert np.array_equal(rowptr, r0) and np.array_equal(colind, c0)
    assert relmax(val, v0) < 1e-12 and relmax(rhs, rhs0) < 1e-12


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FP64, _lib.HDG_PREC_FP32_REFINED, _lib.HDG_PREC_FF_BLOCK])
@pytest.mark.parametrize("D,k,n", CASES + CASES_K2)
def test_elasticity_solution_matches_oracle(D, k, n, precision):
    if precision == _lib.HDG_PREC_FP32_REFINED and k == 2 and D == 3:
        pytest.skip("the FP32 shared-memory LU holds cell blocks up to n = 144 in 3D")
    nu = np.random.default_rng(3).uniform(0.2, 0.45, size=int(np.prod(n)))
    op = _op(D, k, n, nu, precision)
    xh = gh.solve(op, solver="pcg", rtol=1e-13)
    ref = oracle.solve_elasticity(D, k, n, nu=nu, problem=oracle.EPROBLEM_SMOOTH, solver=0)
    tol = 1e-10 if precision == _lib.HDG_PREC_FP64 else 1e-8
    assert relmax(xh.skeleton, ref["lam"]) < tol
    assert relmax(xh.cell_interior, ref["uint"]) < tol
    es, eu = xh.l2_errors()
    assert abs(es - ref["err_sigma"]) <= 1e-6 * ref["err_sigma"]
    assert abs(eu - ref["err_u"]) <= 1e-6 * ref["err_u"]


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FP64, _lib.HDG_PREC_FF_BLOCK])
@pytest.mark.parametrize("D,k,n", [(2, 1, (2, 2)), (2, 2, (3, 2)), (3, 1, (2, 2, 2)), (3, 2, (2, 2, 2))])
def test_elasticity_linear_displacement_exact_on_gpu(D, k, n, precision):
    op = _op(D, k, n, np.full(int(np.prod(n)), 0.31), precision, problem="linear")
    xh = gh.solve(op, solver="direct" if precision == _lib.HDG_PREC_FP64 else "pcg", rtol=1e-13)
    es, eu = xh.l2_errors()
    assert es < 1e-10 and eu < 1e-10


def test_elasticity_precision_report_3d():
    """3D, k=1, E=1, nu ~ U(0.2, 0.45) per cell, u = (sin pi x, cos pi y, xyz):
    the FP32 LU + float-float refinement path against the FP64 path."""
    n = (6, 6, 6)
    nu = np.random.default_rng(7).uniform(0.2, 0.45, size=216)
    x64 = gh.solve(_op(3, 1, n, nu, _lib.HDG_PREC_FP64), rtol=1e-13)
    x32 = gh.solve(_op(3, 1, n, nu, _lib.HDG_PREC_FP32_REFINED), rtol=1e-13)
    assert relmax(x32.free_dof_values, x64.free_dof_values) < 1e-8
    ref = oracle.solve_elasticity(3, 1, n, nu=nu, problem=oracle.EPROBLEM_SMOOTH, solver=1, sign=1.0, rtol=1e-13)
    assert relmax(x64.skeleton, ref["lam"]) < 1e-9


def test_elasticity_block_elimination_3d_k2_matches_fp64():
    """3D, k=2 (the order of the elasticity precision workload): the float-float
    block elimination + FP32 skeleton iterations with FP64 residual refinement
    against the FP64 block elimination, to 1e-8 (relative, max norm)."""
    n = (4, 4, 3)
    nu = np.random.default_rng(11).uniform(0.2, 0.45, size=int(np.prod(n)))
    x64 = gh.solve(_op(3, 2, n, nu, _lib.HDG_PREC_FP64), rtol=1e-13)
    xff = gh.solve(_op(3, 2, n, nu, _lib.HDG_PREC_FF_BLOCK), rtol=1e-13)
    assert relmax(xff.free_dof_values, x64.free_dof_values) < 1e-8
    ref = oracle.solve_elasticity(3, 2, n, nu=nu, problem=oracle.EPROBLEM_SMOOTH, solver=1, sign=1.0, rtol=1e-13)
    assert relmax(x64.skeleton, ref["lam"]) < 1e-9


def test_elasticity_block_elimination_deterministic():
    nu = np.random.default_rng(5).uniform(0.2, 0.45, size=27)
    a = gh.solve(_op(3, 2, (3, 3, 3), nu, _lib.HDG_PREC_FF_BLOCK), rtol=1e-12).free_dof_values
    b = gh.solve(_op(3, 2, (3, 3, 3), nu, _lib.HDG_PREC_FF_BLOCK), rtol=1e-12).free_dof_values
    assert np.array_equal(a, b)
