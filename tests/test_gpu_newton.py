"""GPU tests of the Newton path: HybridFEOperator + solve!(xh0,
FESolver(NLSolver(method=:newton)), op) (src/HybridFEOperators.jl,
src/HybridLinearSolvers.jl), pinned by the reference's own test
(test/DarcyHDGTests.jl:157-165) and against the affine path."""
import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def test_reference_newton_exactness():
    """test/DarcyHDGTests.jl:157-165: the n.n_o form, linear u, 2x2 quads,
    k = 1, Newton from zero: ||u - u_h|| < 1e-12."""
    model = gh.CartesianDiscreteModel((0, 1, 0, 1), (2, 2))
    X, Y = gh.darcy_spaces(model, 1)
    op = gh.HybridFEOperator(gh.DarcyHDG(tau=1.0, stabilization="owner_sign", problem="ref_linear"), X, Y, [1, 2], [3])
    solver = gh.FESolver(gh.NLSolver(method="newton", linear_solver="direct"))
    xh0 = gh.FEFunction(X, np.zeros(op.num_free_dofs()))
    xh, cache = gh.solve_(xh0, solver, op)
    ef, ep = xh.l2_errors()
    assert ef < 1e-12
    assert cache["iterations"] == 1  # a linear residual: one Newton step
    assert cache["residual_norms"][0] > 1e-3 and cache["residual_norms"][-1] <= 1e-8


# (3, 3): the Newton path keeps the cell blocks in HBM and condenses them with
# the FP64 L2-panel kernel; the affine path integrates inside that kernel
@pytest.mark.parametrize("D,k,n", [(2, 2, (6, 5)), (3, 2, (4, 4, 3)), (3, 1, (5, 4, 4)), (3, 3, (3, 2, 2))])
def test_newton_equals_affine_solve(D, k, n):
    kappa = np.exp(np.random.default_rng(5).normal(size=int(np.prod(n))))
    model = gh.CartesianDiscreteModel((0, 1) * D, n)
    X, Y = gh.darcy_spaces(model, k)
    form = gh.DarcyHDG(tau=1.0, problem="sin", kappa=kappa)
    aff = gh.solve(gh.HybridAffineFEOperator(form, X, Y, [1, 2], [3]), solver="pcg", rtol=1e-13)
    op = gh.HybridFEOperator(form, X, Y, [1, 2], [3])
    xh, cache = gh.solve_(None, gh.FESolver(gh.NLSolver(linear_solver="pcg", rtol=1e-13)), op)
    assert cache["iterations"] == 1
    assert relmax(xh.free_dof_values, aff.free_dof_values) < 1e-9
    assert abs(xh.l2_errors()[0] - aff.l2_errors()[0]) <= 1e-6 * aff.l2_errors()[0]


def test_newton_from_the_solution_takes_no_step_and_any_guess_one():
    model = gh.CartesianDiscreteModel((0, 1, 0, 1), (7, 6))
    X, Y = gh.darcy_spaces(model, 2)
    form = gh.DarcyHDG(tau=1.0, problem="sin")
    op = gh.HybridFEOperator(form, X, Y, [1, 2], [3])
    nls = gh.NLSolver(linear_solver="direct")
    xs, c0 = gh.solve_(None, gh.FESolver(nls), op)
    xh, c1 = gh.solve_(gh.FEFunction(X, xs.free_dof_values), gh.FESolver(nls), op)
    assert c1["iterations"] == 0 and relmax(xh.free_dof_values, xs.free_dof_values) == 0.0
    guess = np.random.default_rng(1).normal(size=op.num_free_dofs())
    xg, c2 = gh.solve_(gh.FEFunction(X, guess), gh.FESolver(nls), op)
    assert c2["iterations"] == 1 and relmax(xg.free_dof_values, xs.free_dof_values) < 1e-10


def test_newton_reports_non_convergence():
    model = gh.CartesianDiscreteModel((0, 1, 0, 1), (4, 4))
    X, Y = gh.darcy_spaces(model, 1)
    op = gh.HybridFEOperator(gh.DarcyHDG(tau=1.0, problem="sin"), X, Y, [1, 2], [3])
    with pytest.raises(_lib.HdgError) as e:
        gh.solve_(None, gh.FESolver(gh.NLSolver(iterations=0, linear_solver="direct")), op)
    assert e.value.code == _lib.HDG_ERR_NOT_CONVERGED
