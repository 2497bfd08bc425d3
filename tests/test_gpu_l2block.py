"""GPU tests of the two-field block elimination with L2 panels
(k_condense_l2block.cu) on Darcy HDG cells beyond the shared-memory kernels:
3D, k=3 (256 interior + 96 facet DOFs, n = 352), in FP64 and in float-float,
against the C oracle (test/DarcyHDGTests.jl form, lognormal permeability)."""
import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def _op(n, kappa, precision, k=3, problem="sin", stabilization="textbook"):
    model = gh.CartesianDiscreteModel((0, 1) * 3, n)
    X, Y = gh.darcy_spaces(model, k)
    return gh.HybridAffineFEOperator(gh.DarcyHDG(tau=1.0, stabilization=stabilization, problem=problem,
                                                 kappa=kappa), X, Y, [1, 2], [3], precision=precision)


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FP64, _lib.HDG_PREC_FF_BLOCK])
def test_darcy_3d_k3_assembled_system_matches_oracle(precision):
    n = (3, 2, 2)
    kappa = np.exp(np.random.default_rng(4).normal(size=int(np.prod(n))))
    rowptr, colind, val, rhs = _op(n, kappa, precision).skeleton_system()
    m = oracle.Mesh(3, n, 3)
    A, b = m.integrate(problem=oracle.PROBLEM_SIN, kappa=kappa)
    S, g, _ = oracle.static_condensation(A, b, m.ni)
    r0, c0, v0, rhs0 = m.assemble(S, g, m.dirichlet_values(oracle.PROBLEM_SIN))
    assert np.array_equal(rowptr, r0) and np.array_equal(colind, c0)
    assert relmax(val, v0) < 1e-12 and relmax(rhs, rhs0) < 1e-12


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FP64, _lib.HDG_PREC_FF_BLOCK])
def test_darcy_3d_k3_solution_matches_oracle(precision):
    n = (3, 3, 2)
    kappa = np.exp(np.random.default_rng(6).normal(size=int(np.prod(n))))
    xh = gh.solve(_op(n, kappa, precision), solver="pcg", rtol=1e-13)
    ref = oracle.solve_darcy(3, 3, n, problem=oracle.PROBLEM_SIN, kappa=kappa, solver=0)
    tol = 1e-10 if precision == _lib.HDG_PREC_FP64 else 1e-8
    assert relmax(xh.skeleton, ref["lam"]) < tol
    assert relmax(xh.cell_interior, ref["uint"]) < tol
    ef, ep = xh.l2_errors()
    assert abs(ef - ref["err_flux"]) <= 1e-6 * ref["err_flux"]
    assert abs(ep - ref["err_pres"]) <= 1e-6 * ref["err_pres"]


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FP64, _lib.HDG_PREC_FF_BLOCK])
def test_darcy_3d_k3_reference_exactness(precision):
    """The reference's KAT (n.n_o stabilisation, linear flux, constant
    pressure) is reproduced exactly at k=3 as well."""
    xh = gh.solve(_op((2, 2, 2), None, precision, problem="ref_linear", stabilization="owner_sign"),
                  solver="direct")
    ef, ep = xh.l2_errors()
    assert ef < 1e-9 and ep < 1e-9


def test_darcy_3d_k3_deterministic():
    kappa = np.exp(np.random.default_rng(9).normal(size=27))
    a = gh.solve(_op((3, 3, 3), kappa, _lib.HDG_PREC_FF_BLOCK), rtol=1e-12).free_dof_values
    b = gh.solve(_op((3, 3, 3), kappa, _lib.HDG_PREC_FF_BLOCK), rtol=1e-12).free_dof_values
    assert np.array_equal(a, b)
