"""CPU known-answer tests of the oracle's general-space forms (fields with
their own polynomial space and order, as the reference's tests choose them
with ReferenceFE(lagrangian, T, order; space=:P)).

  - the reference's own Darcy HDG KAT on its own spaces
    (test/DarcyHDGTests.jl:34-36,137-142: flux P_1, pressure P_0, facet
    multiplier P_1, tau (n.n_o) stabilisation, 2x2 quads, u = (1+x, 1+y),
    p = -3.14): ||u - u_h|| < 1e-12;
  - Q spaces everywhere reproduce the oracle's equal-order Q_k forms;
  - the P_k bases are Lagrange bases on their nodes;
  - the reference's RT-H KAT (test/DarcyRTHTests.jl:26-91: flux RT_0,
    pressure Q_0, multiplier Q_0, no stabilisation, 2x2 quads, the same
    u and p): ||u - u_h|| < 1e-12, and RT_k-H converging at k+1 in both
    fields;
  - the reference's multi-field KAT (test/MultiFieldLagrangeMultipliersTests.jl:
    24-88: two RT_0-H copies with skeleton fields [5, 6]): both copies exact,
    and copies of a form solve as the form does, copy by copy;
  - P_m (test/P_m.jl:4-22) leaves the displacement's trace residual
    mu-orthogonal to < 1e-14 (test/LinearElasticityHDGTests.jl:133-137), and
    with it the reference's elasticity configuration (stress P_k,
    displacement P_{k+1}, trace P_k) converges at k+1 in the stress and k+2
    in the displacement.
"""
import numpy as np
import pytest

from oracle import oracle

P, Q, RT = oracle.SPACE_P, oracle.SPACE_Q, oracle.SPACE_RT


@pytest.mark.parametrize("D,n", [(2, (2, 2)), (3, (2, 2, 2))])
def test_reference_darcy_kat_on_reference_spaces(D, n):
    sp = oracle.gs_spaces(P, 1, P, 0, P, 1)
    r = oracle.solve_gs(D, n, oracle.PHYS_DARCY, sp, tau=1.0, stab=oracle.STAB_OWNER_SIGN,
                        problem=oracle.PROBLEM_REF_LINEAR, solver=0)
    m = r["mesh"]
    # 2D: 7 interior (flux P1 2x3, pressure P0 1) + 8 facet DOFs, as the reference's spaces
    if D == 2:
        assert (m.ni, m.nf) == (7, 8)
    assert r["err1"] < 1e-12 and r["err2"] < 1e-12


@pytest.mark.parametrize("D,k,n", [(2, 2, (3, 2)), (3, 1, (2, 2, 2)), (2, 3, (2, 2))])
def test_q_spaces_reproduce_equal_order_forms(D, k, n):
    sp = oracle.gs_spaces(Q, k, Q, k, Q, k)
    g = oracle.GsMesh(D, n, oracle.PHYS_DARCY, sp)
    kap = np.exp(np.random.default_rng(1).normal(size=g.ncells))
    for stab in (oracle.STAB_TEXTBOOK, oracle.STAB_OWNER_SIGN):
        A, b = g.integrate(problem=oracle.PROBLEM_SIN, coef=kap, stab=stab)
        A0, b0 = oracle.Mesh(D, n, k).integrate(problem=oracle.PROBLEM_SIN, kappa=kap, stab=stab)
        assert np.abs(A - A0).max() <= 1e-14 * np.abs(A0).max()
        assert np.abs(b - b0).max() <= 1e-14 * np.abs(b0).max()
    ge = oracle.GsMesh(D, n, oracle.PHYS_ELASTICITY, sp)
    nu = np.random.default_rng(2).uniform(0.2, 0.45, size=ge.ncells)
    A, b = ge.integrate(tau=float(n[0]), problem=oracle.EPROBLEM_SMOOTH, coef=nu)
    A1, b1 = oracle.ElasticityMesh(D, n, k).integrate(tau=float(n[0]), nu=nu, problem=oracle.EPROBLEM_SMOOTH)
    assert np.abs(A - A1).max() <= 1e-14 * np.abs(A1).max()
    assert np.abs(b - b1).max() <= 1e-14 * np.abs(b1).max()


@pytest.mark.parametrize("d,k", [(1, 0), (1, 2), (2, 0), (2, 1), (2, 3), (3, 1), (3, 2)])
def test_p_basis_is_lagrange_on_its_nodes(d, k):
    if k == 0:
        val = oracle.gs_basis_eval(d, P, 0, np.random.default_rng(0).random((5, d)))
        assert np.allclose(val, 1.0)
        return
    idx = [e for e in np.ndindex(*(k + 1,) * d) if sum(e) <= k]
    # nodes in the basis' order: first dimension fastest
    idx.sort(key=lambda e: sum(e[j] * (k + 1) ** j for j in range(d)))
    nodes = np.array(idx, dtype=float)[:, ::1] / k
    val = oracle.gs_basis_eval(d, P, k, nodes)
    assert val.shape == (len(idx), len(idx))
    assert np.abs(val - np.eye(len(idx))).max() < 1e-12


def _pm_residual(D, k, kb):
    """max |int_F mu (phi - P_m phi)| over the local facets of the reference
    cube, trace basis P_k on the facet, bulk basis P_kb in the cell."""
    x1, w1 = np.polynomial.legendre.leggauss(max(k, kb) + 2)
    x1, w1 = 0.5 * (x1 + 1.0), 0.5 * w1
    pts = np.array(list(np.ndindex(*(len(x1),) * (D - 1))))
    s = x1[pts]
    w = np.prod(w1[pts], axis=1)
    worst = 0.0
    for lf in range(2 * D):
        dn, side = D - 1 - lf // 2, lf % 2
        xi = np.zeros((len(s), D))
        j = 0
        for d in range(D):
            if d == dn:
                xi[:, d] = side
            else:
                xi[:, d] = s[:, j]
                j += 1
        mu = oracle.gs_basis_eval(D - 1, P, k, s)
        ph = oracle.gs_basis_eval(D, P, kb, xi)
        L = (mu * w[:, None]).T @ mu
        B = (mu * w[:, None]).T @ ph
        Pm = np.linalg.solve(L, B)
        worst = max(worst, np.abs(B - L @ Pm).max())
    return worst


@pytest.mark.parametrize("D,k", [(2, 1), (2, 2), (3, 1)])
def test_pm_projection_residual_is_mu_orthogonal(D, k):
    assert _pm_residual(D, k, k + 1) < 1e-14


def test_elasticity_with_pm_converges_at_k_plus_one_and_k_plus_two():
    """The reference's elasticity configuration (stress P_1, displacement P_2,
    trace P_1, tau = 1/h, P_m on; test/LinearElasticityHDGTests.jl:88-150)
    on 8^2 and 16^2 cells: the stress converges at rate 2 = k+1, the
    displacement at rate 3 = k+2."""
    sp = oracle.gs_spaces(P, 1, P, 2, P, 1, pm=True)
    errs = []
    for n in (8, 16):
        r = oracle.solve_gs(2, (n, n), oracle.PHYS_ELASTICITY, sp, tau=float(n), problem=oracle.EPROBLEM_SMOOTH,
                            coef=np.full(n * n, 0.3), solver=0)
        errs.append((r["err1"], r["err2"]))
    rs = np.log2(errs[0][0] / errs[1][0])
    ru = np.log2(errs[0][1] / errs[1][1])
    assert rs > 1.9 and ru > 2.9, (rs, ru)


@pytest.mark.parametrize("D,n,copies", [(2, (2, 2), 1), (3, (2, 2, 2), 1), (2, (2, 2), 2)])
def test_reference_rth_and_multifield_kats(D, n, copies):
    sp = oracle.gs_spaces(RT, 0, Q, 0, Q, 0)
    r = oracle.solve_gs(D, n, oracle.PHYS_DARCY, sp, tau=0.0, problem=oracle.PROBLEM_REF_LINEAR, solver=0,
                        copies=copies)
    m = r["mesh"]
    if D == 2:  # RT_0: 4 flux + 1 pressure DOFs per copy, 1 DOF per facet per copy
        assert (m.ni, m.nfd) == (5 * copies, copies)
    assert r["err1"] < 1e-12 and r["err2"] < 1e-12


@pytest.mark.parametrize("k", [0, 1, 2])
def test_rth_converges_at_k_plus_one(k):
    sp = oracle.gs_spaces(RT, k, Q, k, Q, k)
    errs = [oracle.solve_gs(2, (n, n), oracle.PHYS_DARCY, sp, tau=0.0, problem=oracle.PROBLEM_SIN, solver=0)
            for n in (4, 8)]
    for key in ("err1", "err2"):
        assert np.log2(errs[0][key] / errs[1][key]) > k + 0.9


def test_copies_solve_copy_by_copy():
    sp = oracle.gs_spaces(P, 1, P, 0, P, 1)
    kw = dict(tau=1.0, problem=oracle.PROBLEM_SIN, solver=0)
    r1 = oracle.solve_gs(2, (3, 2), oracle.PHYS_DARCY, sp, **kw)
    r2 = oracle.solve_gs(2, (3, 2), oracle.PHYS_DARCY, sp, copies=2, **kw)
    lam = r2["mesh"].multi_field_order(r2["lam"]).reshape(2, -1)
    for cp in range(2):
        assert np.abs(lam[cp] - r1["lam"]).max() < 1e-13
        assert np.abs(r2["uint"][:, r2["mesh"].maps[cp][:r1["mesh"].ni]] - r1["uint"]).max() < 1e-13


@pytest.mark.parametrize("D,n", [(2, (2, 2)), (3, (2, 2, 2))])
def test_reference_darcy_kat_on_simplexified_mesh(D, n):
    """test/DarcyHDGTests.jl:174-177: simplexify of the 2x2 quads with the
    reference's P_1 / P_0 / P_1 spaces and the n.n_o form."""
    sp = oracle.gs_spaces(P, 1, P, 0, P, 1)
    r = oracle.solve_simplex(D, n, sp, tau=1.0, stab=oracle.STAB_OWNER_SIGN, problem=oracle.PROBLEM_REF_LINEAR)
    m = r["mesh"]
    assert m.ncells == np.prod(n) * (2 if D == 2 else 6)
    if D == 2:  # 8 triangles, 12 edges of the quads + 4 diagonals
        assert (m.ncells, m.nfacets, m.ni, m.nf) == (8, 16, 7, 6)
    assert r["err1"] < 1e-12 and r["err2"] < 1e-12


@pytest.mark.parametrize("D,k", [(2, 1), (2, 2), (3, 1)])
def test_simplex_hdg_converges_at_k_plus_one(D, k):
    sp = oracle.gs_spaces(P, k, P, k, P, k)
    ns = (3, 6) if D == 3 else (4, 8)
    errs = [oracle.solve_simplex(D, (n,) * D, sp, tau=1.0, problem=oracle.PROBLEM_SIN) for n in ns]
    for key in ("err1", "err2"):
        assert np.log2(errs[0][key] / errs[1][key]) > k + 0.8, key


def test_simplex_mesh_is_conforming_and_owner_signs_pair_up():
    m = oracle.SimplexMesh(3, (2, 3, 2), oracle.gs_spaces(P, 1, P, 0, P, 1))
    # every interior facet has exactly two cells, with opposite owner signs
    interior = m.facet_is_boundary == 0
    assert (m.facet_cells[interior, 1] >= 0).all() and (m.facet_cells[~interior, 1] < 0).all()
    c0, c1 = m.facet_cells[interior, 0], m.facet_cells[interior, 1]
    assert (c0 < c1).all()
    # boundary facets lie on the domain's boundary: all their vertices share a coordinate at 0 or 1
    X = m.coords
    for f in np.flatnonzero(~interior)[:50]:
        c, lf = m.facet_cell_lf[f]
        vs = [v for j, v in enumerate(m.cells[c]) if j != 3 - lf]
        pts = X[vs]
        assert any(np.allclose(pts[:, d], 0.0) or np.allclose(pts[:, d], 1.0) for d in range(3))
    # volumes add up to the domain's
    J = m.jac.reshape(-1, 3, 3)
    assert abs(np.abs(np.linalg.det(J)).sum() / 6.0 - 1.0) < 1e-12
