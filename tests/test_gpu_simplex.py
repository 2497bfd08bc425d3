"""The Darcy HDG form on simplexified Cartesian meshes on the GPU.

  - the reference's simplex KAT (test/DarcyHDGTests.jl:174-177: simplexify of
    the 2x2 quads, flux P_1, pressure P_0, multiplier P_1, tau (n.n_o)
    stabilisation, u = (1+x, 1+y), p = -3.14): ||u - u_h|| < 1e-12, in 2D
    and on the 3D analogue;
  - the assembled skeleton systems of P_k forms on triangles and tetrahedra
    against the oracle's (oracle.solve_simplex: the same mesh, numbering and
    form restated on the CPU): 1e-12 relative to the largest entry; the
    solutions: FP64 PCG 1e-10, FP32 LU + refinement 1e-8; L2 errors within
    1e-6 of the oracle's.
"""
import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu

P = oracle.SPACE_P
STABS = {"textbook": oracle.STAB_TEXTBOOK, "owner_sign": oracle.STAB_OWNER_SIGN}


def relmax(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def dense(rowptr, colind, val, n):
    A = np.zeros((n, n))
    for i in range(n):
        A[i, colind[rowptr[i]:rowptr[i + 1]]] += val[rowptr[i]:rowptr[i + 1]]
    return A


def _simplex_op(D, n, ks, tau, stab, problem, kappa, precision=_lib.HDG_PREC_FP64):
    model = gh.simplexify(gh.CartesianDiscreteModel((0, 1) * D, n))
    Omega = gh.Triangulation(model)
    Gamma = gh.Triangulation(model, D - 1)
    V = gh.TestFESpace(Omega, gh.ReferenceFE(gh.lagrangian, "VectorValue", ks[0], space="P"))
    Q = gh.TestFESpace(Omega, gh.ReferenceFE(gh.lagrangian, "Float64", ks[1], space="P"))
    M = gh.TestFESpace(Gamma, gh.ReferenceFE(gh.lagrangian, "Float64", ks[2], space="P"), dirichlet_tags="boundary")
    Y = gh.MultiFieldFESpace([V, Q, M])
    X = gh.MultiFieldFESpace([gh.TrialFESpace(V), gh.TrialFESpace(Q), gh.TrialFESpace(M, "exact")])
    wf = gh.DarcyHDG(tau=tau, stabilization=stab, problem=problem, kappa=kappa)
    return gh.HybridAffineFEOperator(wf, X, Y, [1, 2], [3], precision=precision)


@pytest.mark.parametrize("D,n", [(2, (2, 2)), (3, (2, 2, 2))])
def test_reference_simplex_kat(D, n):
    op = _simplex_op(D, n, (1, 0, 1), 1.0, "owner_sign", "ref_linear", None)
    assert op.pb.ncells == np.prod(n) * (2 if D == 2 else 6)
    xh = gh.solve(op, solver="direct")
    ef, ep = xh.l2_errors()
    assert ef < 1e-12 and ep < 1e-12
    op.pb.close()


CASES = [(2, (4, 3), (1, 0, 1)), (2, (3, 3), (2, 1, 2)), (2, (3, 2), (1, 1, 1)), (2, (2, 3), (3, 2, 3)),
         (3, (2, 2, 2), (1, 0, 1)), (3, (2, 1, 2), (2, 2, 2))]


@pytest.mark.parametrize("D,n,ks", CASES)
@pytest.mark.parametrize("stab", ["textbook", "owner_sign"])
def test_simplex_system_and_solution_match_oracle(D, n, ks, stab):
    ncells = int(np.prod(n)) * (2 if D == 2 else 6)
    kappa = np.exp(np.random.default_rng(sum(ks)).normal(size=ncells))
    ref = oracle.solve_simplex(D, n, oracle.gs_spaces(P, ks[0], P, ks[1], P, ks[2]), tau=1.0, stab=STABS[stab],
                               problem=oracle.PROBLEM_SIN, coef=kappa)
    for precision, tol in ((_lib.HDG_PREC_FP64, 1e-10), (_lib.HDG_PREC_FP32_REFINED, 1e-8)):
        op = _simplex_op(D, n, ks, 1.0, stab, "sin", kappa, precision)
        if precision == _lib.HDG_PREC_FP64:
            rowptr, colind, val, rhs = op.skeleton_system()
            nfree = len(rhs)
            assert nfree == ref["mesh"].nfree
            Ag = dense(rowptr, colind, val, nfree)
            Ao = dense(ref["rowptr"], ref["colind"], ref["val"], nfree)
            assert relmax(Ag, Ao) < 1e-12
            assert relmax(rhs, ref["rhs"]) < 1e-12
        xh = gh.solve(op, solver="pcg", rtol=1e-13, maxit=20000)
        assert relmax(xh.skeleton, ref["lam"]) < tol
        assert relmax(xh.cell_interior, ref["uint"]) < tol
        e1, e2 = xh.l2_errors()
        assert abs(e1 - ref["err1"]) <= 1e-6 * ref["err1"]
        assert abs(e2 - ref["err2"]) <= 1e-6 * ref["err2"]
        op.pb.close()


def test_simplex_rejects_other_spaces_and_the_block_elimination():
    with pytest.raises(gh.HdgError):  # Q_k is not a simplex space
        model = gh.simplexify(gh.CartesianDiscreteModel((0, 1, 0, 1), (2, 2)))
        X, Y = gh.darcy_spaces(model, 1, space="Q")
        gh.HybridAffineFEOperator(gh.DarcyHDG(), X, Y, [1, 2], [3])
    with pytest.raises(gh.HdgError):
        _simplex_op(2, (2, 2), (1, 0, 1), 1.0, "textbook", "sin", None, _lib.HDG_PREC_FF_BLOCK)
