"""General-space forms on the GPU against the oracle and the reference's KATs.

  - the reference's Darcy HDG KAT on its own spaces (test/DarcyHDGTests.jl:
    34-36,137-142: flux P_1, pressure P_0, multiplier P_1, tau (n.n_o)
    stabilisation, 2x2 quads, u = (1+x, 1+y), p = -3.14): ||u - u_h|| < 1e-12;
  - its RT-H KAT (test/DarcyRTHTests.jl:26-91: flux RT_0, pressure and
    multiplier Q_0, tau = 0): ||u - u_h|| < 1e-12;
  - its multi-field KAT (test/MultiFieldLagrangeMultipliersTests.jl:24-88:
    two RT_0-H copies, bulk fields [1..4], skeleton fields [5, 6]): both
    copies exact;
  - assembled skeleton systems of P, RT and multi-field Darcy forms and of the
    elasticity forms of test/LinearElasticityHDGTests.jl:88-150 (stress P_k,
    displacement P_{k+1}, trace P_k, with and without P_m) against the
    oracle's: 1e-12 relative to the largest entry; solutions: FP64 1e-10,
    HDG_PREC_FP32_REFINED 1e-8;
  - with P_m the elasticity stress converges at k+1 and the displacement at
    k+2 (:133-150);
  - HDG_PREC_FF_BLOCK, whose kernels take equal-order Q_k blocks only, is
    refused for these forms.
"""
import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu

P, Q, RT = oracle.SPACE_P, oracle.SPACE_Q, oracle.SPACE_RT
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


def _darcy_op(D, n, k, space, tau, stab, problem, kappa, precision=_lib.HDG_PREC_FP64, copies=1):
    model = gh.CartesianDiscreteModel((0, 1) * D, n)
    X, Y = gh.darcy_spaces(model, k, space=space, copies=copies)
    wf = gh.DarcyHDG(tau=tau, stabilization=stab, problem=problem, kappa=kappa)
    c = len(X) // 3
    return gh.HybridAffineFEOperator(wf, X, Y, list(range(1, 2 * c + 1)), list(range(2 * c + 1, 3 * c + 1)),
                                     precision=precision)


def _oracle_spaces(space, k):
    if space == "RT":
        return oracle.gs_spaces(RT, k, Q, k, Q, k)
    return oracle.gs_spaces(P, k, P, k - 1, P, k)


def _check_system(op, ref):
    m = ref["mesh"]
    rowptr, colind, val, rhs = op.skeleton_system()
    nfree = len(rhs)
    assert nfree == m.nfree
    Ag = dense(rowptr, colind, val, nfree)
    Ao = dense(ref["rowptr"], ref["colind"], ref["val"], nfree)
    ro = ref["rhs"]
    if isinstance(m, oracle.GsCopiesMesh):
        idx = m.multi_field_order(np.arange(nfree))
        Ao, ro = Ao[np.ix_(idx, idx)], ro[idx]
    assert relmax(Ag, Ao) < 1e-12
    assert relmax(rhs, ro) < 1e-12


def _check_solution(xh, ref, tol):
    m = ref["mesh"]
    lam = m.multi_field_order(ref["lam"]) if isinstance(m, oracle.GsCopiesMesh) else ref["lam"]
    assert relmax(xh.skeleton, lam) < tol
    assert relmax(xh.cell_interior, ref["uint"]) < tol
    e1, e2 = xh.l2_errors()
    assert abs(e1 - ref["err1"]) <= 1e-6 * max(ref["err1"], 1e-12)
    assert abs(e2 - ref["err2"]) <= 1e-6 * max(ref["err2"], 1e-12)


@pytest.mark.parametrize("D,n", [(2, (2, 2)), (3, (2, 2, 2))])
def test_reference_darcy_kat_on_reference_spaces(D, n):
    op = _darcy_op(D, n, 1, "P", 1.0, "owner_sign", "ref_linear", None)
    xh = gh.solve(op, solver="direct")
    ef, ep = xh.l2_errors()
    assert ef < 1e-12 and ep < 1e-12
    op.pb.close()


@pytest.mark.parametrize("D,n,copies", [(2, (2, 2), 1), (3, (2, 2, 2), 1), (2, (2, 2), 2)])
def test_reference_rth_and_multifield_kats(D, n, copies):
    op = _darcy_op(D, n, 0, "RT", 0.0, "textbook", "ref_linear", None, copies=copies)
    nA = 2 * D  # RT_0: one flux DOF per cell face
    assert (op.pb.ni, op.pb.nfd) == ((nA + 1) * copies, copies)
    xh = gh.solve(op, solver="direct")
    ef, ep = xh.l2_errors()
    assert ef < 1e-12 and ep < 1e-12
    # Gridap's free DOF layout: each bulk field of all cells, then each skeleton field
    fd = xh.free_dof_values
    ncells = int(np.prod(n))
    for cp in range(copies):
        flux = fd[cp * ncells * nA:(cp + 1) * ncells * nA].reshape(ncells, nA)
        assert np.array_equal(flux, xh.cell_interior[:, cp * nA:(cp + 1) * nA])
    op.pb.close()


DARCY_CASES = [(2, (4, 3), 1, "P"), (2, (3, 3), 2, "P"), (3, (2, 3, 2), 1, "P"), (2, (2, 3), 3, "P"),
               (2, (3, 4), 0, "RT"), (2, (3, 2), 1, "RT"), (2, (2, 2), 2, "RT"), (3, (2, 2, 2), 1, "RT")]


@pytest.mark.parametrize("D,n,k,space", DARCY_CASES)
@pytest.mark.parametrize("stab", ["textbook", "owner_sign"])
def test_darcy_system_and_solution_match_oracle(D, n, k, space, stab):
    tau = 0.0 if space == "RT" else 1.0
    kappa = np.exp(np.random.default_rng(k).normal(size=int(np.prod(n))))
    ref = oracle.solve_gs(D, n, oracle.PHYS_DARCY, _oracle_spaces(space, k), tau=tau, stab=STABS[stab],
                          problem=oracle.PROBLEM_SIN, coef=kappa, solver=0)
    for precision, tol in ((_lib.HDG_PREC_FP64, 1e-10), (_lib.HDG_PREC_FP32_REFINED, 1e-8)):
        op = _darcy_op(D, n, k, space, tau, stab, "sin", kappa, precision)
        if precision == _lib.HDG_PREC_FP64:
            _check_system(op, ref)
        xh = gh.solve(op, solver="pcg", rtol=1e-13, maxit=20000)
        _check_solution(xh, ref, tol)
        op.pb.close()


@pytest.mark.parametrize("space,k", [("P", 1), ("RT", 1)])
def test_multifield_copies_match_oracle(space, k):
    D, n = 2, (3, 3)
    tau = 0.0 if space == "RT" else 1.0
    kappa = np.exp(np.random.default_rng(5).normal(size=9))
    ref = oracle.solve_gs(D, n, oracle.PHYS_DARCY, _oracle_spaces(space, k), tau=tau, problem=oracle.PROBLEM_SIN,
                          coef=kappa, solver=0, copies=2)
    op = _darcy_op(D, n, k, space, tau, "textbook", "sin", kappa, copies=2)
    _check_system(op, ref)
    xh = gh.solve(op, solver="pcg", rtol=1e-13, maxit=20000)
    _check_solution(xh, ref, 1e-10)
    op.pb.close()


ELAST_CASES = [(2, (3, 3), 1), (2, (2, 3), 2), (3, (2, 2, 2), 1)]


@pytest.mark.parametrize("D,n,k", ELAST_CASES)
@pytest.mark.parametrize("pm", [False, True])
def test_elasticity_system_and_solution_match_oracle(D, n, k, pm):
    nu = np.random.default_rng(k).uniform(0.2, 0.45, size=int(np.prod(n)))
    ref = oracle.solve_gs(D, n, oracle.PHYS_ELASTICITY, oracle.gs_spaces(P, k, P, k + 1, P, k, pm=pm),
                          tau=float(n[0]), problem=oracle.EPROBLEM_SMOOTH, coef=nu, solver=0)
    model = gh.CartesianDiscreteModel((0, 1) * D, n)
    X, Y = gh.elasticity_spaces(model, k, space="P")
    for precision, tol in ((_lib.HDG_PREC_FP64, 1e-10), (_lib.HDG_PREC_FP32_REFINED, 1e-8)):
        wf = gh.ElasticityHDG(nu=nu, problem="smooth", bulk_to_skeleton_projection=pm)
        op = gh.HybridAffineFEOperator(wf, X, Y, [1, 2], [3], precision=precision)
        if precision == _lib.HDG_PREC_FP64:
            _check_system(op, ref)
        xh = gh.solve(op, solver="pcg", rtol=1e-13, maxit=20000)
        _check_solution(xh, ref, tol)
        op.pb.close()


def test_elasticity_with_pm_converges_at_k_plus_one_and_k_plus_two():
    errs = []
    for n in (8, 16):
        model = gh.CartesianDiscreteModel((0, 1, 0, 1), (n, n))
        X, Y = gh.elasticity_spaces(model, 1, space="P")
        wf = gh.ElasticityHDG(nu=np.full(n * n, 0.3), problem="smooth", bulk_to_skeleton_projection=True)
        op = gh.HybridAffineFEOperator(wf, X, Y, [1, 2], [3])
        errs.append(gh.solve(op, solver="pcg", rtol=1e-13, maxit=20000).l2_errors())
        op.pb.close()
    rs = np.log2(errs[0][0] / errs[1][0])
    ru = np.log2(errs[0][1] / errs[1][1])
    assert rs > 1.9 and ru > 2.9, (rs, ru)


def test_ff_block_is_refused_for_general_spaces():
    with pytest.raises(gh.HdgError):
        _darcy_op(2, (2, 2), 1, "P", 1.0, "textbook", "sin", None, _lib.HDG_PREC_FF_BLOCK)
