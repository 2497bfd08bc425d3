"""CPU tests that pin the oracle to the reference.

The reference (Julia + Gridap) cannot run here; these tests pin the oracle to
the reference's own known-answer tests and to golden vectors produced by an
independent LAPACK executing the reference's call sequence.
"""
import os

import numpy as np
import pytest

from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "static_condensation_lapack.npz")


def test_lagrange_node_order_quad():
    # Gridap QUAD: vertices (0,0),(1,0),(0,1),(1,1); edges [y=0, y=1, x=0, x=1]; interior
    assert oracle.lattice(2, 1).tolist() == [[0, 0], [1, 0], [0, 1], [1, 1]]
    assert oracle.lattice(2, 2).tolist() == [[0, 0], [2, 0], [0, 2], [2, 2], [1, 0], [1, 2], [0, 1], [2, 1], [1, 1]]
    # SEGMENT order 3: vertices then interior nodes from the first vertex on
    assert oracle.lattice(1, 3)[:, 0].tolist() == [0, 3, 1, 2]


def test_lagrange_node_order_hex():
    lat = oracle.lattice(3, 2).tolist()
    vertices = [[0, 0, 0], [2, 0, 0], [0, 2, 0], [2, 2, 0], [0, 0, 2], [2, 0, 2], [0, 2, 2], [2, 2, 2]]
    # HEX edges (1,2),(3,4),(1,3),(2,4),(5,6),(7,8),(5,7),(6,8),(1,5),(2,6),(3,7),(4,8)
    edges = [[1, 0, 0], [1, 2, 0], [0, 1, 0], [2, 1, 0], [1, 0, 2], [1, 2, 2], [0, 1, 2], [2, 1, 2],
             [0, 0, 1], [2, 0, 1], [0, 2, 1], [2, 2, 1]]
    # HEX facets [z=0, z=1, y=0, y=1, x=0, x=1]
    faces = [[1, 1, 0], [1, 1, 2], [1, 0, 1], [1, 2, 1], [0, 1, 1], [2, 1, 1]]
    assert lat == vertices + edges + faces + [[1, 1, 1]]
    assert len(oracle.lattice(3, 3)) == 64


@pytest.mark.parametrize("npts", [1, 2, 3, 4, 5, 6])
def test_gauss_legendre_exactness(npts):
    import ctypes
    x = np.zeros(npts)
    w = np.zeros(npts)
    oracle.lib().orc_gauss_legendre01(npts, oracle.P(x), oracle.P(w))
    for j in range(2 * npts):
        assert abs(np.sum(w * x ** j) - 1.0 / (j + 1)) < 1e-14


def test_cartesian_topology_gridap_numbering():
    m = oracle.Mesh(2, (2, 2), 1)
    # local facets [y0, y1, x0, x1]; facets numbered in first-encounter order
    assert m.cell_facets.tolist() == [[0, 1, 2, 3], [4, 5, 3, 6], [1, 7, 8, 9], [5, 10, 9, 11]]
    assert m.facet_cells[3].tolist() == [0, 1] and m.facet_cells[1].tolist() == [0, 2]
    assert m.nfacets == 12 and m.nfree == 4 * 2 and m.ndir == 8 * 2
    m3 = oracle.Mesh(3, (32, 32, 32), 2)
    assert m3.ncells == 32768 and m3.nfree == 857088
    r, c = oracle.Mesh(3, (4, 4, 4), 2).csr_pattern()
    assert np.all(np.diff(r) > 0) and all(np.all(np.diff(c[r[i]:r[i + 1]]) > 0) for i in range(len(r) - 1))


def test_csr_sizes_match_configs():
    m = oracle.Mesh(2, (8, 8), 1)
    r, c = m.csr_pattern()
    assert m.nfree == 224 and len(c) == 2784  # config 1: 224 free DOFs, 2,784 nnz


def test_sum_facets_kat():
    """test/SumFacetMapTests.jl:29: four equal facet blocks sum to 4a."""
    a = np.random.default_rng(0).random((2, 4))
    assert np.allclose(oracle.sum_facets(np.stack([a, a, a, a])) - 4 * a, 0.0)


def test_golden_lapack_vectors():
    """The oracle's restatement of getrf/getrs/gemm/gemv reproduces scipy LAPACK
    executing the reference's sequence."""
    z = np.load(GOLDEN)
    for i in range(int(z["ncases"])):
        A, b, ni = z["A%d" % i], z["b%d" % i], int(z["ni%d" % i])
        Acm = np.ascontiguousarray(A.T)[None]  # column-major per cell
        S, g, info = oracle.static_condensation(Acm, b[None], ni)
        assert info[0] == 0
        S = S[0].T
        assert np.abs(S - z["S%d" % i]).max() <= 1e-13 * np.abs(z["S%d" % i]).max()
        assert np.abs(g[0] - z["g%d" % i]).max() <= 1e-13 * np.abs(z["g%d" % i]).max()
        u, info = oracle.backward_static_condensation(Acm, b[None], z["x%d" % i][None], ni)
        assert np.abs(u[0] - z["u%d" % i]).max() <= 1e-13 * np.abs(z["u%d" % i]).max()


def test_static_condensation_identities():
    """Forward then backward solves the full block system (the property the
    reference's StaticCondensationMapTests exercises without asserting)."""
    rng = np.random.default_rng(1)
    ni, nf = 27, 12
    n = ni + nf
    A = rng.normal(size=(n, n)) + 3 * np.sqrt(n) * np.eye(n)
    b = rng.normal(size=n)
    S, g, _ = oracle.static_condensation(np.ascontiguousarray(A.T)[None], b[None], ni)
    xf = np.linalg.solve(S[0].T, g[0])
    u, _ = oracle.backward_static_condensation(np.ascontiguousarray(A.T)[None], b[None], xf[None], ni)
    full = np.linalg.solve(A, b)
    assert np.abs(full[:ni] - u[0]).max() < 1e-12 * np.abs(full).max()
    assert np.abs(full[ni:] - xf).max() < 1e-12 * np.abs(full).max()


def test_zero_pivot_info():
    ni, nf = 3, 2
    A = np.eye(5)
    A[1, 1] = 0.0
    A[2, 2] = 0.0
    S, g, info = oracle.static_condensation(np.ascontiguousarray(A.T)[None], np.ones((1, 5)), ni)
    assert info[0] == 2  # LAPACK info: first zero pivot (1-based)


@pytest.mark.parametrize("D,n", [(2, (2, 2)), (3, (2, 2, 2))])
def test_darcy_hdg_reference_exactness(D, n):
    """test/DarcyHDGTests.jl:137-142: u=(1+x,1+y), p=-3.14, the reference's
    n.n_o stabilisation, 2x2 mesh: L2 flux error < 1e-12."""
    r = oracle.solve_darcy(D, 1, n, stab=oracle.STAB_OWNER_SIGN, problem=oracle.PROBLEM_REF_LINEAR, solver=0)
    assert r["rc"] == 0
    assert r["err_flux"] < 1e-12 and r["err_pres"] < 1e-12


def test_cfg1_linear_pressure_exact():
    r = oracle.solve_darcy(2, 1, (8, 8), problem=oracle.PROBLEM_LINEAR, solver=0)
    assert r["err_flux"] < 1e-12 and r["err_pres"] < 1e-12


@pytest.mark.parametrize("k", [1, 2, 3])
def test_textbook_hdg_convergence_rates(k):
    errs = [oracle.solve_darcy(2, k, (n, n), problem=oracle.PROBLEM_SIN, solver=0) for n in (4, 8, 16)]
    ef = [e["err_flux"] for e in errs]
    ep = [e["err_pres"] for e in errs]
    rate_f = np.log2(ef[1] / ef[2])
    rate_p = np.log2(ep[1] / ep[2])
    assert rate_f > k + 1 - 0.25 and rate_p > k + 1 - 0.25


def test_skeleton_operator_negative_definite():
    """The textbook form's condensed skeleton operator is symmetric negative
    definite (why PCG runs on -S)."""
    m = oracle.Mesh(2, (4, 4), 2)
    A, b = m.integrate(problem=oracle.PROBLEM_SIN)
    S, g, _ = oracle.static_condensation(A, b, m.ni)
    r, c, v, rhs = m.assemble(S, g, m.dirichlet_values(oracle.PROBLEM_SIN))
    Md = np.zeros((m.nfree, m.nfree))
    for i in range(m.nfree):
        Md[i, c[r[i]:r[i + 1]]] = v[r[i]:r[i + 1]]
    assert np.abs(Md - Md.T).max() < 1e-12 * np.abs(Md).max()
    assert np.linalg.eigvalsh(Md).max() < 0


def test_pcg_matches_dense():
    kappa = np.exp(np.random.default_rng(2).normal(size=27))
    r0 = oracle.solve_darcy(3, 1, (3, 3, 3), problem=oracle.PROBLEM_SIN, kappa=kappa, solver=0)
    r1 = oracle.solve_darcy(3, 1, (3, 3, 3), problem=oracle.PROBLEM_SIN, kappa=kappa, solver=1, rtol=1e-14)
    assert np.abs(r0["lam"] - r1["lam"]).max() < 1e-11 * np.abs(r0["lam"]).max()
    assert np.abs(r0["uint"] - r1["uint"]).max() < 1e-11 * np.abs(r0["uint"]).max()


# ---------------------------------------------------------------------------
# Linear elasticity HDG (test/LinearElasticityHDGTests.jl)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("D,n,k", [(2, (2, 2), 1), (2, (3, 2), 2), (3, (2, 2, 2), 1)])
def test_elasticity_linear_displacement_is_exact(D, n, k):
    """A linear displacement (constant stress, f = 0) is in the discrete
    spaces: the HDG solution reproduces it (the reference's linear u_exact,
    test/LinearElasticityHDGTests.jl:48-50).  The Poisson ratio is uniform:
    with a per-cell ratio the constant-strain field is not an equilibrium
    (the traction jumps across cells)."""
    r = oracle.solve_elasticity(D, k, n, problem=oracle.EPROBLEM_LINEAR, nu=np.full(int(np.prod(n)), 0.37))
    assert r["rc"] == 0
    assert r["err_sigma"] < 1e-12 and r["err_u"] < 1e-12


def test_elasticity_convergence_rates():
    """Smooth 2D displacement of the reference test (:52-57), k = 1: stress
    error ~ h^k, displacement error ~ h^(k+1)."""
    es, eu = [], []
    for nn in (4, 8, 16):
        r = oracle.solve_elasticity(2, 1, (nn, nn), problem=oracle.EPROBLEM_SMOOTH)
        es.append(r["err_sigma"])
        eu.append(r["err_u"])
    rs = np.log2(es[1] / es[2])
    ru = np.log2(eu[1] / eu[2])
    assert 0.9 < rs < 1.6 and 1.8 < ru < 2.4


def test_elasticity_skeleton_operator_is_spd():
    m = oracle.ElasticityMesh(2, (3, 3), 1)
    nu = np.random.default_rng(0).uniform(0.2, 0.45, size=m.ncells)
    A, b = m.integrate(tau=3.0, nu=nu)
    S, g, info = oracle.static_condensation(A, b, m.ni)
    assert (info == 0).all()
    rowptr, colind, val, rhs = m.assemble(S, g, m.dirichlet_values(oracle.EPROBLEM_SMOOTH))
    K = np.zeros((m.nfree, m.nfree))
    for r in range(m.nfree):
        K[r, colind[rowptr[r]:rowptr[r + 1]]] = val[rowptr[r]:rowptr[r + 1]]
    assert np.abs(K - K.T).max() < 1e-12 * np.abs(K).max()
    assert np.linalg.eigvalsh(K).min() > 0.0
    # PCG on +S agrees with the dense solve
    d = oracle.solve_elasticity(2, 1, (3, 3), nu=nu, solver=0)
    p = oracle.solve_elasticity(2, 1, (3, 3), nu=nu, solver=1, sign=1.0, rtol=1e-13)
    assert np.abs(d["lam"] - p["lam"]).max() < 1e-9 * np.abs(d["lam"]).max()


def test_elasticity_sym_tensor_layout_sizes():
    for D, k, ni, nf in [(2, 1, (3 + 2) * 4, 4 * 2 * 2), (3, 1, (6 + 3) * 8, 6 * 3 * 4), (3, 2, (6 + 3) * 27, 6 * 3 * 9)]:
        m = oracle.ElasticityMesh(D, (2,) * D, k)
        assert (m.ni, m.nf) == (ni, nf)
        assert m.nfd == D * (k + 1) ** (D - 1)


@pytest.mark.parametrize("D,n,k", [(2, (4, 3), 1), (2, (3, 3), 3), (3, (2, 3, 2), 2)])
@pytest.mark.parametrize("stab", [oracle.STAB_TEXTBOOK, oracle.STAB_OWNER_SIGN])
def test_affine_cell_integration_equals_the_box_cells(D, n, k, stab):
    """orc_integrate_darcy_affine with the box cells' own diagonal Jacobians
    reproduces orc_integrate_darcy (which the reference's KATs pin)."""
    m = oracle.Mesh(D, n, k)
    kappa = np.exp(np.random.default_rng(1).normal(size=m.ncells))
    A, b = m.integrate(problem=oracle.PROBLEM_SIN, stab=stab, kappa=kappa)
    origin, jac = m.geometry()
    A2, b2 = m.integrate_affine(origin, jac, problem=oracle.PROBLEM_SIN, stab=stab, kappa=kappa)
    assert np.abs(A2 - A).max() <= 1e-14 * np.abs(A).max()
    assert np.abs(b2 - b).max() <= 1e-14 * np.abs(b).max()


@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("k", [1, 2, 3])
def test_pm_projection_kats(D, k):
    """P_m (test/P_m.jl; src/GridapAPIExtensions.jl:453-500) on every local facet:
    * bulk order k: the projected trace equals the trace (P_m is the identity on
      traces when the orders match), so P is a 0/1 selection;
    * bulk order k + 1: the residual is orthogonal to the facet space, the
      reference's own check (test/LinearElasticityHDGTests.jl:136-139, < 1e-14)."""
    for lf in range(2 * D):
        xi, w, mu = oracle.facet_quadrature(D, k, lf)
        Pk = oracle.pm_projection(D, k, k, lf)
        assert np.abs(oracle.cell_basis(D, k, xi) - mu @ Pk).max() < 1e-13
        assert np.abs(Pk - np.round(Pk)).max() < 1e-12
        assert set((np.round(Pk) == 1).sum(axis=1).tolist()) == {1}
        Pb = oracle.pm_projection(D, k, k + 1, lf)
        res = oracle.cell_basis(D, k + 1, xi) - mu @ Pb
        assert np.abs(mu.T @ (w[:, None] * res)).max() < 1e-14


SKEW = {2: np.array([[1.0, 0.3], [0.2, 1.0]]),
        3: np.array([[1.0, 0.3, 0.1], [0.1, 1.0, 0.2], [0.05, 0.1, 1.0]])}


@pytest.mark.parametrize("D,n,k", [(2, (4, 3), 1), (2, (3, 3), 2), (2, (3, 2), 3), (3, (2, 2, 2), 1),
                                   (3, (2, 2, 2), 2)])
def test_affine_cells_reproduce_a_linear_pressure(D, n, k):
    """The reference's exactness check (test/DarcyHDGTests.jl:142) on a mesh whose
    cells are all mapped by one skew: the oracle's affine-cell integration,
    condensation, assembly and dense solve give the skeleton values of the
    linear pressure at the free facet nodes."""
    m = oracle.Mesh(D, n, k)
    origin, jac = m.geometry()
    B = SKEW[D]
    origin = origin @ B.T
    jac = np.einsum("rd,cjd->cjr", B, jac)  # J' = B J, stored [cell][col][row]
    A, b = m.integrate_affine(origin, jac, stab=oracle.STAB_TEXTBOOK, problem=oracle.PROBLEM_LINEAR)
    S, g, info = oracle.static_condensation(A, b, m.ni)
    free, dirv = m.facet_node_values_affine(origin, jac, oracle.PROBLEM_LINEAR)
    rowptr, colind, val, rhs = m.assemble(S, g, dirv)
    lam = oracle.dense_solve(rowptr, colind, val, rhs)
    assert np.abs(lam - free).max() < 1e-10 * max(1.0, np.abs(free).max())
