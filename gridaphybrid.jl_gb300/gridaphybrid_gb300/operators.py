"""HybridAffineFEOperator / solve on the GPU (the operator level of GridapHybrid.jl).

Mirrors the reference's user API (test/DarcyHDGTests.jl:27-142):

    model = CartesianDiscreteModel((0,1,0,1), (2,2))
    dK    = Skeleton(model)
    reffe_u = ReferenceFE(lagrangian, VectorValue, order)  ...
    V = TestFESpace(Omega, reffe_u, conformity="L2") ...
    X = MultiFieldFESpace([U, P, L]);  Y = MultiFieldFESpace([V, Q, M])
    op = HybridAffineFEOperator(DarcyHDG(tau=1.0), X, Y, [1, 2], [3])
    xh = solve(op)

Python cannot evaluate Gridap weak-form closures, so the weak form is a
descriptor of the Darcy HDG form the reference's tests write out
(test/DarcyHDGTests.jl:125-135), with the textbook stabilisation as an option
and a per-cell permeability, or of the elasticity HDG form
(test/LinearElasticityHDGTests.jl:140-150).  Each field takes its own space
(ReferenceFE(lagrangian, T, k; space=:Q or :P), or raviart_thomas for the
Darcy flux: the RT-H form of test/DarcyRTHTests.jl is DarcyHDG(tau=0)), and
a multi-field space of c copies [A_1..A_c, B_1..B_c, T_1..T_c] with
bulk_fields [1..2c] and skeleton_fields [2c+1..3c] sums the form once per
copy (test/MultiFieldLagrangeMultipliersTests.jl).  Integration,
condensation, assembly, the skeleton solve and the recovery all run in
libgridaphybrid_gb300.
"""
import ctypes

import numpy as np

from . import _lib

lagrangian = "lagrangian"
raviart_thomas = "raviart_thomas"
VectorValue = "VectorValue"
SymTensorValue = "SymTensorValue"
Float64 = "Float64"


class CartesianDiscreteModel:
    """CartesianDiscreteModel(domain, partition): uniform quads/hexes, cells
    numbered lexicographically (x fastest), Gridap's facet numbering."""

    def __init__(self, domain, partition):
        self.partition = tuple(int(n) for n in partition)
        self.D = len(self.partition)
        if self.D not in (2, 3) or len(domain) != 2 * self.D:
            raise ValueError("domain must be (x0,x1,y0,y1[,z0,z1]) for 2 or 3 dimensions")
        self.domain = tuple(float(x) for x in domain)

    def num_cell_dims(self):
        return self.D

    def num_cells(self):
        return int(np.prod(self.partition))

    def cell_jacobians(self):
        h = [(self.domain[2 * d + 1] - self.domain[2 * d]) / self.partition[d] for d in range(self.D)]
        return np.broadcast_to(np.diag(h), (self.num_cells(), self.D, self.D))


class SimplexifiedModel(CartesianDiscreteModel):
    """simplexify(CartesianDiscreteModel(domain, partition)): every box split
    into D! simplices around its diagonal from the lowest to the highest vertex
    (2 triangles per square, 6 tetrahedra per cube), as the reference's
    simplex test builds its mesh (test/DarcyHDGTests.jl:174-177)."""

    simplex = True

    def num_cells(self):
        return int(np.prod(self.partition)) * (2 if self.D == 2 else 6)


def simplexify(model):
    return SimplexifiedModel(model.domain, model.partition)


CartesianDiscreteModel.simplex = False


class Triangulation:
    def __init__(self, model, dim=None):
        self.model = model
        self.dim = model.D if dim is None else dim


class SkeletonTriangulation(Triangulation):
    """Skeleton(model): each cell seen as the set of its facets (src/Skeleton.jl:113-147)."""

    def __init__(self, model):
        super().__init__(model, model.D - 1)


def Skeleton(model):
    return SkeletonTriangulation(model)


def _reference_normals(D):
    """Outward reference normals in Gridap local facet order [.., y0, y1, x0, x1]."""
    out = np.zeros((2 * D, D))
    for lf in range(2 * D):
        out[lf, D - 1 - lf // 2] = 1.0 if lf % 2 else -1.0
    return out


def get_cell_normal_vector(skel):
    """Unit outward normal per (cell, local facet): push_normal(J^{-T}, n_ref)
    (src/Skeleton.jl:524-527, 564-585).  Shape (ncells, 2D, D)."""
    m = skel.model
    Jinv_t = np.linalg.inv(np.asarray(m.cell_jacobians())).transpose(0, 2, 1)
    v = np.einsum("cij,fj->cfi", Jinv_t, _reference_normals(m.D))
    return v / np.linalg.norm(v, axis=2, keepdims=True)


def get_cell_owner_normal_vector(skel, facet_cells=None, cell_facets=None):
    """The owner cell's outward normal seen from each (cell, local facet): n on the
    facet's first cell, -n on the other (src/Skeleton.jl:549-556,
    src/SkeletonArrays.jl:219-229).  The glue comes from the library's topology."""
    n = get_cell_normal_vector(skel)
    if facet_cells is None or cell_facets is None:
        ctx = _lib.default_context()
        pb = _Problem(ctx, skel.model, 1)
        cell_facets, facet_cells, _ = pb.topology()
        pb.close()
    owner = facet_cells[cell_facets, 0]
    sign = np.where(owner == np.arange(n.shape[0])[:, None], 1.0, -1.0)
    return n * sign[:, :, None]


class ReferenceFE:
    """ReferenceFE(lagrangian, T, order; space=:Q|:P) or
    ReferenceFE(raviart_thomas, Float64, order) on the Cartesian cells."""

    KINDS = {"Q": _lib.HDG_SPACE_Q, "P": _lib.HDG_SPACE_P}

    def __init__(self, kind, value_type, order, space="Q"):
        space = str(space).lstrip(":")
        if kind == raviart_thomas:
            self.kind = _lib.HDG_SPACE_RT
        elif kind == lagrangian:
            if space not in self.KINDS:
                raise ValueError("lagrangian spaces are space='Q' (tensor product) or space='P' (total degree)")
            self.kind = self.KINDS[space]
        else:
            raise ValueError("reference FEs: lagrangian or raviart_thomas")
        self.value_type = value_type
        self.order = int(order)


class FESpace:
    def __init__(self, trian, reffe, conformity="L2", dirichlet_tags=None, dirichlet_value=None):
        if conformity != "L2":
            raise ValueError("hybridizable spaces are L2-conforming")
        self.trian = trian
        self.reffe = reffe
        self.dirichlet_tags = dirichlet_tags
        self.dirichlet_value = dirichlet_value


def TestFESpace(trian, reffe, conformity="L2", dirichlet_tags=None):
    return FESpace(trian, reffe, conformity, dirichlet_tags)


def TrialFESpace(space, dirichlet_value=None):
    return FESpace(space.trian, space.reffe, "L2", space.dirichlet_tags, dirichlet_value)


class MultiFieldFESpace:
    def __init__(self, spaces):
        self.spaces = list(spaces)

    def __getitem__(self, i):
        return self.spaces[i]

    def __len__(self):
        return len(self.spaces)


class DarcyHDG:
    """The Darcy HDG weak form of test/DarcyHDGTests.jl:125-135 with a per-cell
    permeability kappa:
      (v.u/kappa) - (div v) p - grad(q).u  on Omega,
      (v.n) l + q(u.n) + tau s q (p - l) + m(u.n) + tau s m (p - l)  on dK,
    s = n.n_o (stabilization="owner_sign", as the reference test) or 1
    ("textbook" LDG-H).  tau = 0 with a raviart_thomas flux is the RT-H form
    of test/DarcyRTHTests.jl:69-72 (q div u = -grad(q).u + q(u.n) per cell).  `problem` selects the built-in manufactured source,
    Dirichlet data and exact solution."""

    STABS = {"textbook": _lib.HDG_STAB_TEXTBOOK, "owner_sign": _lib.HDG_STAB_OWNER_SIGN}
    PROBLEMS = {"ref_linear": _lib.HDG_PROBLEM_REF_LINEAR, "linear": _lib.HDG_PROBLEM_LINEAR,
                "sin": _lib.HDG_PROBLEM_SIN}

    pm = False

    def __init__(self, tau=1.0, stabilization="textbook", problem="linear", kappa=None):
        self.tau = float(tau)
        self.stab = self.STABS[stabilization]
        self.problem = self.PROBLEMS[problem]
        self.kappa = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)


class ElasticityHDG:
    """The linear elasticity HDG form of test/LinearElasticityHDGTests.jl:140-150:
      v (.) A(sigma) + (div v).u - w.(div sigma) on Omega,
      -(v.n).uhat + tau w.(P_m(u) - uhat) + mu.(sigma.n) - tau mu.(P_m(u) - uhat) on dK,
    P_m the L2 projection of the displacement onto the trace space
    (bulk_to_skeleton_projection=True, :134-137) or the identity (False),
    compliance A(s) = (1+nu)/E s - nu/E tr(s) I (:15-38) with a per-cell
    Poisson ratio nu; `problem` selects the manufactured displacement
    ("linear" :48-50 or "smooth" :52-57) giving f = div sigma_exact and the
    Dirichlet data.  tau defaults to the reference's 1/h (cells per side)."""

    PROBLEMS = {"linear": _lib.HDG_EPROBLEM_LINEAR, "smooth": _lib.HDG_EPROBLEM_SMOOTH}
    physics = _lib.HDG_PHYSICS_ELASTICITY

    def __init__(self, tau=None, E=1.0, nu=None, problem="smooth", bulk_to_skeleton_projection=False):
        self.tau = None if tau is None else float(tau)
        self.pm = bool(bulk_to_skeleton_projection)
        self.E = float(E)
        self.problem = self.PROBLEMS[problem]
        self.nu = None if nu is None else np.ascontiguousarray(nu, dtype=np.float64)

    def apply(self, c, pb, model):
        tau = float(model.partition[0]) if self.tau is None else self.tau
        c.check(c.lib.hdg_set_elasticity(pb.h, tau, self.E, self.problem))
        c.check(c.lib.hdg_set_permeability(pb.h, _lib.ptr(self.nu)))


DarcyHDG.physics = _lib.HDG_PHYSICS_DARCY


def _darcy_apply(self, c, pb, model):
    c.check(c.lib.hdg_set_darcy(pb.h, self.stab, self.tau, self.problem))
    c.check(c.lib.hdg_set_permeability(pb.h, _lib.ptr(self.kappa)))


DarcyHDG.apply = _darcy_apply


class _Problem:
    """Owns an hdg_problem handle: the equal-order Q_k forms, or (spaces =
    int32[7] {kindA, kA, kindB, kB, kindT, kT, pm}) the general-space forms
    with `copies` copies."""

    def __init__(self, ctx, model, k, physics=_lib.HDG_PHYSICS_DARCY, spaces=None, copies=1):
        self.ctx = ctx
        h = ctypes.c_void_p()
        cells = np.array(model.partition, dtype=np.int32)
        dom = np.array(model.domain, dtype=np.float64)
        if model.simplex:
            sp = np.ascontiguousarray(spaces, dtype=np.int32)
            ctx.check(ctx.lib.hdg_problem_create_simplex_spaces(ctx.handle, model.D, _lib.ptr(cells), _lib.ptr(dom),
                                                                physics, _lib.ptr(sp), copies, ctypes.byref(h)))
        elif spaces is None:
            ctx.check(ctx.lib.hdg_problem_create_cartesian_physics(ctx.handle, model.D, _lib.ptr(cells),
                                                                   _lib.ptr(dom), k, physics, ctypes.byref(h)))
        else:
            sp = np.ascontiguousarray(spaces, dtype=np.int32)
            ctx.check(ctx.lib.hdg_problem_create_cartesian_spaces(ctx.handle, model.D, _lib.ptr(cells),
                                                                  _lib.ptr(dom), physics, _lib.ptr(sp), copies,
                                                                  ctypes.byref(h)))
        self.copies = copies
        self.h = h
        ctx.register(self)
        info = np.zeros(8, dtype=np.int64)
        ctx.check(ctx.lib.hdg_problem_info(h, _lib.ptr(info)))
        (self.ncells, self.nfacets, self.ni, self.nf, self.nfree, self.ndir, self.nnz,
         self.nfd) = (int(v) for v in info)
        self.D = model.D

    def topology(self):
        cf = np.empty((self.ncells, 2 * self.D), dtype=np.int32)
        fc = np.empty((self.nfacets, 2), dtype=np.int32)
        fd = np.empty((self.nfacets, self.nfd), dtype=np.int32)
        self.ctx.check(self.ctx.lib.hdg_get_topology(self.h, _lib.ptr(cf), _lib.ptr(fc), _lib.ptr(fd)))
        return cf, fc, fd

    def close(self):
        if self.h:
            if self.ctx.alive:  # a destroyed context took its device memory with it
                self.ctx.lib.hdg_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _general_spaces(trial, bulk_fields, skeleton_fields, weakform):
    """(spaces, copies) of a multi-field trial space [A_1..A_c, B_1..B_c,
    T_1..T_c] with bulk_fields [1..2c] and skeleton_fields [2c+1..3c]
    (src/HybridAffineFEOperators.jl:10-36 takes any such split); spaces is
    None for one copy of equal-order Q_k fields without P_m, the forms with
    the float-float fast path."""
    nf = len(trial)
    c = nf // 3
    if nf % 3 or c < 1 or bulk_fields != list(range(1, 2 * c + 1)) or \
            skeleton_fields != list(range(2 * c + 1, 3 * c + 1)):
        raise ValueError("the HDG operators expect fields [A_1..A_c, B_1..B_c, T_1..T_c] (flux/stress, "
                         "pressure/displacement, trace) with bulk_fields=[1..2c] and skeleton_fields=[2c+1..3c]")
    per_copy = []
    for cp in range(c):
        fe = [trial[cp].reffe, trial[c + cp].reffe, trial[2 * c + cp].reffe]
        per_copy.append(tuple(v for r in fe for v in (r.kind, r.order)))
    if len(set(per_copy)) != 1:
        raise ValueError("the copies of a multi-field HDG space must use the same spaces")
    sp = per_copy[0]
    q = _lib.HDG_SPACE_Q
    simplex = getattr(trial[0].trian.model, "simplex", False)
    if not simplex and c == 1 and not weakform.pm and sp[0::2] == (q, q, q) and len(set(sp[1::2])) == 1:
        return None, 1
    return np.array(list(sp) + [1 if weakform.pm else 0], dtype=np.int32), c


class HybridAffineFEOperator:
    """HybridAffineFEOperator(weakform, trial, test, bulk_fields, skeleton_fields)
    (src/HybridAffineFEOperators.jl:10-50): integrates, condenses every cell
    (keeping the factors on the GPU) and assembles the skeleton system."""

    def __init__(self, weakform, trial, test, bulk_fields, skeleton_fields,
                 precision=_lib.HDG_PREC_FP64, context=None):
        self.weakform, self.trial, self.test = weakform, trial, test
        self.bulk_fields, self.skeleton_fields = list(bulk_fields), list(skeleton_fields)
        self.precision = precision
        model = trial[0].trian.model
        spaces, copies = _general_spaces(trial, self.bulk_fields, self.skeleton_fields, weakform)
        self.k = trial[0].reffe.order
        self.model = model
        self.ctx = context or _lib.default_context()
        self.pb = _Problem(self.ctx, model, self.k, weakform.physics, spaces, copies)
        c = self.ctx
        weakform.apply(c, self.pb, model)
        self.info = np.zeros(self.pb.ncells, dtype=np.int32)
        c.check(c.lib.hdg_assemble(self.pb.h, precision, _lib.ptr(self.info)))

    def skeleton_system(self):
        """(rowptr, colind, val, rhs) of op.skeleton_op, CSR with sorted columns."""
        pb, c = self.pb, self.ctx
        rowptr = np.empty(pb.nfree + 1, dtype=np.int64)
        colind = np.empty(pb.nnz, dtype=np.int32)
        val = np.empty(pb.nnz)
        rhs = np.empty(pb.nfree)
        c.check(c.lib.hdg_get_skeleton_system(pb.h, _lib.ptr(rowptr), _lib.ptr(colind), _lib.ptr(val),
                                              _lib.ptr(rhs)))
        return rowptr, colind, val, rhs


class HybridFEFunction:
    """The multi-field solution: free DOF values in Gridap's layout
    [flux | pressure | skeleton] plus per-cell views."""

    def __init__(self, op, iters, relres):
        pb, c = op.pb, op.ctx
        self.op = op
        self.iterations = iters
        self.relres = relres
        self.free_dof_values = np.empty(pb.ncells * pb.ni + pb.nfree)
        c.check(c.lib.hdg_get_free_dof_values(pb.h, _lib.ptr(self.free_dof_values)))
        self.cell_interior = np.empty((pb.ncells, pb.ni))
        c.check(c.lib.hdg_get_cell_interior_values(pb.h, _lib.ptr(self.cell_interior)))
        self.skeleton = self.free_dof_values[pb.ncells * pb.ni:]

    def l2_errors(self):
        """(||q - q_h||, ||p - p_h||) against the problem's exact solution."""
        ef, ep = ctypes.c_double(), ctypes.c_double()
        c = self.op.ctx
        c.check(c.lib.hdg_l2_errors(self.op.pb.h, ctypes.byref(ef), ctypes.byref(ep)))
        return ef.value, ep.value


def solve(op, solver="pcg", rtol=1e-10, maxit=20000):
    """solve(op::HybridAffineFEOperator) (src/HybridAffineFEOperators.jl:67-100):
    skeleton solve, then recovery of the interior fields from the stored factors."""
    s = {"pcg": _lib.HDG_SOLVER_PCG, "direct": _lib.HDG_SOLVER_DIRECT}[solver]
    it, rel = ctypes.c_int(), ctypes.c_double()
    c = op.ctx
    c.check(c.lib.hdg_solve_skeleton(op.pb.h, s, rtol, maxit, ctypes.byref(it), ctypes.byref(rel)))
    c.check(c.lib.hdg_recover(op.pb.h))
    return HybridFEFunction(op, it.value, rel.value)


class HybridFEOperator:
    """HybridFEOperator(residual, X, Y, bulk_fields, skeleton_fields)
    (src/HybridFEOperators.jl:68-145): the nonlinear-operator form, solved by
    Newton's method; its Jacobian is the hybridizable cell matrix, so every
    Newton step runs the whole hybridization path (integrate, condense,
    assemble, skeleton solve, recover) on the residual."""

    def __init__(self, weakform, trial, test, bulk_fields, skeleton_fields, context=None):
        if list(bulk_fields) != [1, 2] or list(skeleton_fields) != [3]:
            raise ValueError("the Darcy HDG operator expects bulk_fields=[1,2] (flux, pressure) "
                             "and skeleton_fields=[3] (trace)")
        self.weakform, self.trial, self.test = weakform, trial, test
        orders = {s.reffe.order for s in trial.spaces}
        if len(orders) != 1:
            raise ValueError("flux, pressure and trace must share the order k (Q_k / Q_k / Q_k)")
        self.k = orders.pop()
        self.model = trial[0].trian.model
        self.ctx = context or _lib.default_context()
        self.pb = _Problem(self.ctx, self.model, self.k, weakform.physics)
        weakform.apply(self.ctx, self.pb, self.model)

    def num_free_dofs(self):
        return self.pb.ncells * self.pb.ni + self.pb.nfree


class NLSolver:
    """NLSolver(method=:newton, ftol=1e-8, iterations=1000) (NLsolve.jl's Newton
    without line search, as used by test/DarcyHDGTests.jl:151,160); the linear
    solve of each step is the hybridized one (src/HybridLinearSolvers.jl)."""

    def __init__(self, method="newton", ftol=1e-8, iterations=1000, linear_solver="direct", rtol=1e-12,
                 maxit=20000, show_trace=False):
        if method != "newton":
            raise ValueError("only method='newton' is provided")
        self.ftol, self.iterations = float(ftol), int(iterations)
        self.linear_solver = {"pcg": _lib.HDG_SOLVER_PCG, "direct": _lib.HDG_SOLVER_DIRECT}[linear_solver]
        self.rtol, self.maxit = float(rtol), int(maxit)
        self.show_trace = show_trace


class FESolver:
    def __init__(self, nls):
        self.nls = nls


class FEFunction:
    """FEFunction(X, free_values): an initial guess for solve_."""

    def __init__(self, space, free_values):
        self.space = space
        self.free_dof_values = np.ascontiguousarray(free_values, dtype=np.float64)


def solve_(xh0, solver, op):
    """solve!(xh0, solver, op) for a HybridFEOperator
    (src/HybridLinearSolvers.jl:15-59 inside NLsolve's Newton loop): returns
    (xh, cache) with the converged HybridFEFunction and the Newton history."""
    nls = solver.nls
    x0 = None
    if xh0 is not None:
        if xh0.free_dof_values.size != op.num_free_dofs():
            raise ValueError("the initial guess has %d values, the space %d" % (xh0.free_dof_values.size,
                                                                               op.num_free_dofs()))
        x0 = xh0.free_dof_values
    norms = np.zeros(nls.iterations + 1)
    it = ctypes.c_int()
    c = op.ctx
    c.check(c.lib.hdg_newton_solve(op.pb.h, nls.linear_solver, nls.rtol, nls.maxit, nls.ftol, nls.iterations,
                                   _lib.ptr(x0), _lib.ptr(norms), ctypes.byref(it)))
    hist = norms[:it.value + 1].copy()
    if nls.show_trace:
        for i, r in enumerate(hist):
            print("Newton %3d  residual %.3e" % (i, r))
    return HybridFEFunction(op, it.value, float(hist[-1])), {"iterations": it.value, "residual_norms": hist}


def _copies(V, Q, M, dirichlet, copies):
    Y = MultiFieldFESpace([V] * copies + [Q] * copies + [M] * copies)
    X = MultiFieldFESpace([TrialFESpace(V)] * copies + [TrialFESpace(Q)] * copies +
                          [TrialFESpace(M, dirichlet)] * copies)
    return X, Y


def elasticity_spaces(model, k, space="Q", displacement_order=None, copies=1):
    """The spaces of the elasticity HDG test: symmetric stress, displacement
    and displacement trace with Dirichlet facets on the whole boundary
    (test/LinearElasticityHDGTests.jl:79-110).  space="Q": all Q_k (the
    equal-order forms); space="P": stress P_k, displacement P_{k+1}, trace P_k
    as the reference's test; displacement_order overrides the displacement's."""
    Omega = Triangulation(model)
    Gamma = Triangulation(model, model.D - 1)
    ku = displacement_order if displacement_order is not None else (k + 1 if space == "P" else k)
    V = TestFESpace(Omega, ReferenceFE(lagrangian, SymTensorValue, k, space=space), conformity="L2")
    W = TestFESpace(Omega, ReferenceFE(lagrangian, VectorValue, ku, space=space), conformity="L2")
    M = TestFESpace(Gamma, ReferenceFE(lagrangian, VectorValue, k, space=space), conformity="L2",
                    dirichlet_tags="boundary")
    return _copies(V, W, M, "u_exact", copies)


def darcy_spaces(model, k, space="Q", copies=1):
    """The spaces of the Darcy tests with Dirichlet facets on the whole
    boundary: space="Q": Q_k flux, pressure and trace (the equal-order forms);
    "P": flux P_k, pressure P_{k-1}, trace P_k (test/DarcyHDGTests.jl:32-52);
    "RT": flux RT_k, pressure Q_k, trace Q_k (test/DarcyRTHTests.jl:32-54).
    copies > 1 repeats each field (test/MultiFieldLagrangeMultipliersTests.jl:
    37-62)."""
    Omega = Triangulation(model)
    Gamma = Triangulation(model, model.D - 1)
    if space == "RT":
        rv = ReferenceFE(raviart_thomas, Float64, k)
        rq = ReferenceFE(lagrangian, Float64, k)
        rm = ReferenceFE(lagrangian, Float64, k)
    else:
        rv = ReferenceFE(lagrangian, VectorValue, k, space=space)
        rq = ReferenceFE(lagrangian, Float64, k - 1 if space == "P" else k, space=space)
        rm = ReferenceFE(lagrangian, Float64, k, space=space)
    V = TestFESpace(Omega, rv, conformity="L2")
    Q = TestFESpace(Omega, rq, conformity="L2")
    M = TestFESpace(Gamma, rm, conformity="L2", dirichlet_tags="boundary")
    return _copies(V, Q, M, "exact", copies)
