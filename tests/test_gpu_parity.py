"""GPU parity tests: the sm_103a library (through its C ABI) against the CPU
oracle on the same seeded inputs.

Tolerances: FP64 cell-level results (S, g, recovered interiors) <= 1e-12
relative to the largest entry (the reference's StaticCondensationMap /
BackwardStaticCondensationMap run in FP64); skeleton patterns bit-exact;
whole solves <= 1e-10 relative (both solved to a residual of 1e-14 or by
dense LU).
"""
import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu

RTOL_CELL = 1e-12
RTOL_SOLVE = 1e-10


def relmax(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def ctx():
    return gh.default_context()


def _gpu_condense(ctx, A, b, ni, precision=_lib.HDG_PREC_FP64):
    """A: (ncells, n, n) column-major per cell (oracle layout)."""
    ncells, n, _ = A.shape
    nf = n - ni
    S = np.empty((ncells, nf, nf))
    g = np.empty((ncells, nf))
    info = np.zeros(ncells, dtype=np.int32)
    rc = ctx.lib.hdg_static_condensation(ctx.handle, precision, ncells, ni, nf, _lib.ptr(np.ascontiguousarray(A)),
                                         _lib.ptr(np.ascontiguousarray(b)), _lib.ptr(S), _lib.ptr(g),
                                         _lib.ptr(info))
    return rc, S, g, info


def _gpu_backward(ctx, A, b, x, ni):
    ncells, n, _ = A.shape
    u = np.empty((ncells, ni))
    info = np.zeros(ncells, dtype=np.int32)
    rc = ctx.lib.hdg_backward_static_condensation(ctx.handle, _lib.HDG_PREC_FP64, ncells, ni, n - ni,
                                                  _lib.ptr(np.ascontiguousarray(A)),
                                                  _lib.ptr(np.ascontiguousarray(b)),
                                                  _lib.ptr(np.ascontiguousarray(x)), _lib.ptr(u), _lib.ptr(info))
    return rc, u, info


@pytest.mark.parametrize("ni,nf,ncells", [(3, 2, 7), (12, 8, 64), (27, 12, 33), (48, 16, 20), (108, 54, 6)])
def test_condensation_random_blocks(ctx, ni, nf, ncells):
    rng = np.random.default_rng(ni * 100 + nf)
    n = ni + nf
    A = rng.normal(size=(ncells, n, n))
    A[:, np.arange(ni), np.arange(ni)] += 2.0 * np.sqrt(n)  # keep A_ii well conditioned
    b = rng.normal(size=(ncells, n))
    S0, g0, info0 = oracle.static_condensation(A, b, ni)
    rc, S, g, info = _gpu_condense(ctx, A, b, ni)
    assert rc == 0 and (info == 0).all() and (info0 == 0).all()
    for c in range(ncells):
        assert relmax(S[c], S0[c]) < RTOL_CELL
        assert relmax(g[c], g0[c]) < RTOL_CELL


@pytest.mark.parametrize("D,k,n", [(2, 1, (3, 2)), (2, 2, (3, 3)), (2, 3, (2, 3)), (3, 1, (2, 2, 2)), (3, 2, (2, 2, 2))])
@pytest.mark.parametrize("stab", [oracle.STAB_TEXTBOOK, oracle.STAB_OWNER_SIGN])
def test_condensation_hdg_blocks(ctx, D, k, n, stab):
    m = oracle.Mesh(D, n, k)
    kappa = np.exp(np.random.default_rng(1).normal(size=m.ncells))
    A, b = m.integrate(tau=1.0, stab=stab, problem=oracle.PROBLEM_SIN, kappa=kappa)
    S0, g0, _ = oracle.static_condensation(A, b, m.ni)
    rc, S, g, info = _gpu_condense(ctx, A, b, m.ni)
    assert rc == 0 and (info == 0).all()
    assert relmax(S, S0) < RTOL_CELL
    assert relmax(g, g0) < RTOL_CELL
    # backward map with an arbitrary skeleton vector
    x = np.random.default_rng(2).normal(size=(m.ncells, m.nf))
    u0, _ = oracle.backward_static_condensation(A, b, x, m.ni)
    rc, u, info = _gpu_backward(ctx, A, b, x, m.ni)
    assert rc == 0
    assert relmax(u, u0) < RTOL_CELL


def test_singular_interior_block_reports_info(ctx):
    ni, nf = 4, 2
    A = np.zeros((3, 6, 6))
    rng = np.random.default_rng(3)
    A[:] = rng.normal(size=(3, 6, 6))
    A[1, 0:2, 0:ni] = 0.0  # columns 0 and 1 of A_ii are zero in cell 1 (column-major: A[c, j, i])
    b = rng.normal(size=(3, 6))
    rc, S, g, info = _gpu_condense(ctx, A, b, ni)
    assert rc == _lib.HDG_ERR_SINGULAR
    assert info[0] == 0 and info[2] == 0 and info[1] == 1


def test_static_condensation_map_reference_test(ctx):
    """test/StaticCondensationMapTests.jl: 3x3 MatrixBlock with blocks [2:3,2:3]
    untouched, StaticCondensationMap([1,2],[3]) then the backward map; the
    reference has no assertion, here the results must solve the block system."""
    rng = np.random.default_rng(4)
    x = rng.random((3, 3))
    blocks = [[x, x + 3, x + 5], [x + 1, None, None], [x + 2, None, None]]
    touched = np.ones((3, 3), dtype=bool)
    touched[1:, 1:] = False
    A = gh.MatrixBlock(blocks, touched)
    xv = rng.random(3)
    bv = gh.VectorBlock([xv, xv + 1, xv + 2], [True] * 3)
    k = gh.StaticCondensationMap([1, 2], [3])
    cache = gh.return_cache(k, A, bv)
    S, g = gh.evaluate(cache, k, A, bv)
    Ad = np.zeros((9, 9))
    for i in range(3):
        for j in range(3):
            if touched[i, j]:
                Ad[3 * i:3 * i + 3, 3 * j:3 * j + 3] = blocks[i][j]
    bd = np.concatenate([xv, xv + 1, xv + 2])
    Aii, Aif, Afi, Aff = Ad[:6, :6], Ad[:6, 6:], Ad[6:, :6], Ad[6:, 6:]
    S_np = Aff - Afi @ np.linalg.solve(Aii, Aif)
    g_np = bd[6:] - Afi @ np.linalg.solve(Aii, bd[:6])
    # the reference's block pattern makes S vanish identically (A_fi A_ii^{-1} A_if
    # has no support on A_ff's rows), so compare against the input scale
    scale = np.abs(Ad).max() * np.abs(np.linalg.inv(Aii)).max() * np.abs(Ad).max()
    assert np.abs(S - S_np).max() < 1e-12 * scale and relmax(g, g_np) < 1e-10
    kb = gh.BackwardStaticCondensationMap([1, 2], [3])
    cb = gh.return_cache(kb, A, bv, g)
    out = gh.evaluate(cb, kb, A, bv, g)
    assert out.shape == (3,) and out.touched.all()
    ui = np.concatenate([out.array[0], out.array[1]])
    assert relmax(ui, np.linalg.solve(Aii, bd[:6] - Aif @ g)) < 1e-10
    assert np.array_equal(out.array[2], g)


def test_sum_facets_map_reference_kats(ctx):
    """test/SumFacetMapTests.jl:29 (four equal facet blocks sum to 4a) and :109
    (one-hot [1,f] facet blocks densify to hcat(a,a,a,a))."""
    rng = np.random.default_rng(5)
    a = rng.random((2, 4))
    ab = gh.VectorBlock([a, None, None], [True, False, False])
    abf = gh.VectorBlock([ab, ab, ab, ab], [True] * 4)
    m = gh.SumFacetsMap()
    res = gh.evaluate(gh.return_cache(m, abf), m, abf)
    assert np.allclose(res.array[0] - 4 * a, 0.0)
    a = rng.random((2, 1))
    facets = []
    for f in range(4):
        inner = np.empty((1, 4), dtype=object)
        t = np.zeros((1, 4), dtype=bool)
        inner[0, f] = a
        t[0, f] = True
        fb = gh.ArrayBlock(inner, t)
        outer = np.empty((1, 3), dtype=object)
        to = np.zeros((1, 3), dtype=bool)
        outer[0, 0] = fb
        to[0, 0] = True
        facets.append(gh.ArrayBlock(outer, to))
    abf = gh.VectorBlock(facets, [True] * 4)
    res = gh.densify(gh.evaluate(gh.return_cache(m, abf), m, abf))
    assert np.allclose(res.array[0, 0] - np.hstack([a, a, a, a]), 0.0)


def _problem(D, k, n, stab=oracle.STAB_TEXTBOOK, problem=oracle.PROBLEM_SIN, kappa=None, tau=1.0):
    model = gh.CartesianDiscreteModel((0, 1) * D, n)
    X, Y = gh.darcy_spaces(model, k)
    names = {0: "ref_linear", 1: "linear", 2: "sin"}
    stabs = {0: "textbook", 1: "owner_sign"}
    wf = gh.DarcyHDG(tau=tau, stabilization=stabs[stab], problem=names[problem], kappa=kappa)
    return gh.HybridAffineFEOperator(wf, X, Y, [1, 2], [3])


@pytest.mark.parametrize("D,n", [(2, (2, 2)), (3, (2, 2, 2))])
def test_darcy_reference_exactness(ctx, D, n):
    """test/DarcyHDGTests.jl:137-142 on the GPU: u=(1+x,1+y), p=-3.14 with the
    reference's n.n_o stabilisation; ||u - u_h|| < 1e-12."""
    op = _problem(D, 1, n, stab=oracle.STAB_OWNER_SIGN, problem=oracle.PROBLEM_REF_LINEAR)
    xh = gh.solve(op, solver="direct")
    ef, ep = xh.l2_errors()
    assert ef < 1e-12 and ep < 1e-12


def test_topology_and_pattern_bit_exact(ctx):
    for D, k, n in [(2, 1, (8, 8)), (2, 3, (3, 5)), (3, 2, (4, 3, 2))]:
        op = _problem(D, k, n)
        cf, fc, fd = op.pb.topology()
        m = oracle.Mesh(D, n, k)
        assert np.array_equal(cf, m.cell_facets)
        assert np.array_equal(fc[:, 0], m.facet_cells[:, 0])
        assert np.array_equal(fd, m.facet_dofs)
        rowptr, colind, val, rhs = op.skeleton_system()
        r0, c0 = m.csr_pattern()
        assert np.array_equal(rowptr, r0) and np.array_equal(colind, c0)


@pytest.mark.parametrize("D,k,n", [(2, 1, (8, 8)), (2, 2, (5, 4)), (2, 3, (4, 4)), (3, 1, (3, 3, 3)), (3, 2, (3, 2, 3))])
@pytest.mark.parametrize("stab", [oracle.STAB_TEXTBOOK, oracle.STAB_OWNER_SIGN])
def test_assembled_system_parity(ctx, D, k, n, stab):
    kappa = np.exp(np.random.default_rng(7).normal(size=int(np.prod(n))))
    op = _problem(D, k, n, stab=stab, kappa=kappa)
    rowptr, colind, val, rhs = op.skeleton_system()
    m = oracle.Mesh(D, n, k)
    A, b = m.integrate(stab=stab, problem=oracle.PROBLEM_SIN, kappa=kappa)
    S, g, _ = oracle.static_condensation(A, b, m.ni)
    dv = m.dirichlet_values(oracle.PROBLEM_SIN)
    r0, c0, v0, rhs0 = m.assemble(S, g, dv)
    assert relmax(val, v0) < RTOL_CELL
    assert relmax(rhs, rhs0) < RTOL_CELL


@pytest.mark.parametrize("D,k,n", [(2, 1, (8, 8)), (2, 2, (6, 6)), (2, 3, (4, 5)), (3, 1, (4, 4, 4)), (3, 2, (3, 3, 3))])
def test_solution_parity(ctx, D, k, n):
    kappa = np.exp(np.random.default_rng(11).normal(size=int(np.prod(n))))
    op = _problem(D, k, n, kappa=kappa)
    xh = gh.solve(op, solver="pcg", rtol=1e-14, maxit=5000)
    ref = oracle.solve_darcy(D, k, n, problem=oracle.PROBLEM_SIN, kappa=kappa, solver=0)
    assert ref["rc"] == 0
    assert relmax(xh.skeleton, ref["lam"]) < RTOL_SOLVE
    assert relmax(xh.cell_interior, ref["uint"]) < RTOL_SOLVE
    ef, ep = xh.l2_errors()
    assert abs(ef - ref["err_flux"]) <= 0.01 * ref["err_flux"]
    assert abs(ep - ref["err_pres"]) <= 0.01 * ref["err_pres"]
    # Gridap's free-DOF layout [flux | pressure | skeleton]
    pb = op.pb
    nk = (k + 1) ** D
    fd = xh.free_dof_values
    assert np.array_equal(fd[:pb.ncells * D * nk].reshape(pb.ncells, D * nk), xh.cell_interior[:, :D * nk])
    assert np.array_equal(fd[pb.ncells * D * nk:pb.ncells * pb.ni].reshape(pb.ncells, nk),
                          xh.cell_interior[:, D * nk:])


def test_cfg1_linear_pressure_exact(ctx):
    """2D Darcy HDG 8x8, k=1, tau=1, K=I, p=x+y: the discrete solution is exact."""
    op = _problem(2, 1, (8, 8), problem=oracle.PROBLEM_LINEAR)
    xh = gh.solve(op, solver="pcg", rtol=1e-14)
    ef, ep = xh.l2_errors()
    assert ef < 1e-11 and ep < 1e-11
    ref = oracle.solve_darcy(2, 1, (8, 8), problem=oracle.PROBLEM_LINEAR, solver=0)
    assert relmax(xh.cell_interior, ref["uint"]) < RTOL_SOLVE


def test_state_errors(ctx):
    op = _problem(2, 1, (2, 2))
    lib = ctx.lib
    # recover before solve -> HDG_ERR_STATE
    assert lib.hdg_recover(op.pb.h) == _lib.HDG_ERR_STATE
    # PCG with a non-positive tolerance -> HDG_ERR_INVALID
    assert lib.hdg_solve_skeleton(op.pb.h, 0, -1.0, 10, None, None) == _lib.HDG_ERR_INVALID
    # oversized Map-level block is rejected, not attempted
    A = np.zeros((1, 400, 400))
    b = np.zeros((1, 400))
    rc, S, g, info = _gpu_condense(ctx, A, b, 300)
    assert rc == _lib.HDG_ERR_INVALID


def test_full_size_3d_properties(ctx):
    """3D Darcy 32^3, k=2, lognormal K (the benchmark workload): the GPU
    solution satisfies the assembled skeleton system to the PCG tolerance and
    every sampled cell's interior equals the oracle's BackwardStaticCondensationMap
    applied to the GPU skeleton values."""
    import scipy.sparse as sp

    n = (32, 32, 32)
    kappa = np.exp(np.random.default_rng(0).normal(size=32 ** 3))
    op = _problem(3, 2, n, kappa=kappa)
    xh = gh.solve(op, solver="pcg", rtol=1e-10, maxit=5000)
    rowptr, colind, val, rhs = op.skeleton_system()
    A = sp.csr_matrix((val, colind, rowptr), shape=(len(rhs), len(rhs)))
    res = np.linalg.norm(rhs - A @ xh.skeleton) / np.linalg.norm(rhs)
    assert res < 1.2e-10
    # symmetry of the assembled operator (textbook form)
    d = (A - A.T).tocsr()
    assert (np.abs(d.data).max() if d.nnz else 0.0) <= 1e-12 * np.abs(val).max()
    m = oracle.Mesh(3, n, 2)
    sample = np.sort(np.random.default_rng(1).choice(m.ncells, size=64, replace=False))
    A_s, b_s = m.integrate_cells(sample, problem=oracle.PROBLEM_SIN, kappa=kappa)
    dv = m.dirichlet_values(oracle.PROBLEM_SIN)
    xc = m.cell_skeleton_values(xh.skeleton, dv)
    u0, _ = oracle.backward_static_condensation(A_s, b_s, xc[sample], m.ni)
    assert relmax(xh.cell_interior[sample], u0) < 1e-11
