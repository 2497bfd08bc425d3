"""Python access to the CPU FP64 oracle (oracle/hdg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; the GPU product never uses it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "hdg_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

PROBLEM_REF_LINEAR, PROBLEM_LINEAR, PROBLEM_SIN = 0, 1, 2
STAB_TEXTBOOK, STAB_OWNER_SIGN = 0, 1


def build(force=False):
    """gcc -O2 -fopenmp -shared oracle/hdg_oracle.c -> oracle/liboracle.so"""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "hdg_oracle.h"))):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", tmp, SRC, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stderr)
    os.replace(tmp, LIB)
    return LIB


_L = None


def lib():
    global _L
    if _L is None:
        build()
        _L = ctypes.CDLL(LIB)
        _L.orc_solve_darcy.restype = ctypes.c_int
    return _L


def P(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def lattice(D, k):
    out = np.zeros(((k + 1) ** D, max(D, 1)), dtype=np.int32)
    n = lib().orc_lagrange_lattice(D, k, P(out))
    return out[:n]


def cell_sizes(D, k):
    ni, nf = ctypes.c_int(), ctypes.c_int()
    lib().orc_cell_sizes(D, k, ctypes.byref(ni), ctypes.byref(nf))
    return ni.value, nf.value


class Mesh:
    """Cartesian mesh in Gridap numbering, as the oracle builds it."""

    def __init__(self, D, n, k, domain=None):
        L = lib()
        self.D, self.k = D, k
        self.n = np.array(n, dtype=np.int32)
        self.domain = np.array(domain if domain is not None else [0.0, 1.0] * D, dtype=np.float64)
        nc, nfc = ctypes.c_int(), ctypes.c_int()
        L.orc_cart_counts(D, P(self.n), ctypes.byref(nc), ctypes.byref(nfc))
        self.ncells, self.nfacets = nc.value, nfc.value
        self.cell_facets = np.zeros((self.ncells, 2 * D), dtype=np.int32)
        self.facet_cells = np.zeros((self.nfacets, 2), dtype=np.int32)
        self.facet_is_boundary = np.zeros(self.nfacets, dtype=np.int32)
        L.orc_cart_topology(D, P(self.n), P(self.cell_facets), P(self.facet_cells), P(self.facet_is_boundary))
        self.nfd = (k + 1) ** (D - 1)
        self.facet_dofs = np.zeros((self.nfacets, self.nfd), dtype=np.int32)
        nfree, ndir = ctypes.c_int(), ctypes.c_int()
        L.orc_facet_dofs(D, k, self.nfacets, P(self.facet_is_boundary), P(self.facet_dofs),
                         ctypes.byref(nfree), ctypes.byref(ndir))
        self.nfree, self.ndir = nfree.value, ndir.value
        self.ni, self.nf = cell_sizes(D, k)

    def integrate(self, tau=1.0, stab=STAB_TEXTBOOK, problem=PROBLEM_LINEAR, kappa=None):
        n = self.ni + self.nf
        A = np.zeros((self.ncells, n, n))  # A[c, j, i] = A_c(i, j): column-major per cell
        b = np.zeros((self.ncells, n))
        kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        rc = lib().orc_integrate_darcy(self.D, self.k, P(self.n), P(self.domain), ctypes.c_double(tau), stab,
                                       problem, P(kap), P(self.facet_cells), P(self.cell_facets), P(A), P(b))
        assert rc == 0
        return A, b

    def geometry(self):
        """Per-cell origin (ncells x D) and Jacobian (ncells x D x D, [cell][col][row]) of the box cells."""
        D = self.D
        h = (self.domain[1::2] - self.domain[0::2]) / self.n
        origin = np.zeros((self.ncells, D))
        jac = np.zeros((self.ncells, D, D))
        for c in range(self.ncells):
            r = c
            for d in range(D):  # first direction fastest
                origin[c, d] = self.domain[2 * d] + (r % self.n[d]) * h[d]
                r //= self.n[d]
            jac[c] = np.diag(h)
        return origin, jac

    def integrate_affine(self, origin, jac, tau=1.0, stab=STAB_TEXTBOOK, problem=PROBLEM_LINEAR, kappa=None):
        """The cell blocks of this topology with every cell an affine map x = origin_c + J_c xi
        (jac[c] column-major, [cell][col][row]) (orc_integrate_darcy_affine)."""
        n = self.ni + self.nf
        A = np.zeros((self.ncells, n, n))
        b = np.zeros((self.ncells, n))
        kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        rc = lib().orc_integrate_darcy_affine(self.D, self.k, self.ncells, P(np.ascontiguousarray(origin)),
                                              P(np.ascontiguousarray(jac)), ctypes.c_double(tau), stab, problem,
                                              P(kap), P(self.facet_cells), P(self.cell_facets), P(A), P(b))
        assert rc == 0
        return A, b

    def facet_node_values_affine(self, origin, jac, problem):
        """(free, dirichlet) nodal values of the manufactured pressure at the facet DOFs
        of this topology with affine cells (orc_facet_node_values_affine)."""
        free = np.zeros(max(self.nfree, 1))
        dirv = np.zeros(max(self.ndir, 1))
        rc = lib().orc_facet_node_values_affine(self.D, self.k, self.ncells, P(np.ascontiguousarray(origin)),
                                                P(np.ascontiguousarray(jac)), P(self.cell_facets),
                                                P(self.facet_cells), problem, self.nfacets, P(self.facet_dofs),
                                                P(free), P(dirv))
        assert rc == 0
        return free[:self.nfree], dirv[:self.ndir]

    def integrate_cells(self, cells, tau=1.0, stab=STAB_TEXTBOOK, problem=PROBLEM_LINEAR, kappa=None):
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        n = self.ni + self.nf
        A = np.zeros((len(cells), n, n))
        b = np.zeros((len(cells), n))
        kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        rc = lib().orc_integrate_darcy_cells(self.D, self.k, P(self.n), P(self.domain), ctypes.c_double(tau),
                                             stab, problem, P(kap), P(self.facet_cells), P(self.cell_facets),
                                             len(cells), P(cells), P(A), P(b))
        assert rc == 0
        return A, b

    def dirichlet_values(self, problem):
        vals = np.zeros(max(self.ndir, 1))
        lib().orc_dirichlet_values(self.D, self.k, P(self.n), P(self.domain), problem, self.nfacets,
                                   P(self.facet_is_boundary), P(self.facet_dofs), self.ndir, P(vals))
        return vals[:self.ndir] if self.ndir else vals[:0]

    def csr_pattern(self):
        nnz = ctypes.c_int64()
        L = lib()
        L.orc_csr_pattern(self.D, self.k, self.ncells, self.nfacets, P(self.cell_facets), P(self.facet_dofs),
                          self.nfree, None, None, ctypes.byref(nnz))
        rowptr = np.zeros(self.nfree + 1, dtype=np.int64)
        colind = np.zeros(nnz.value, dtype=np.int32)
        L.orc_csr_pattern(self.D, self.k, self.ncells, self.nfacets, P(self.cell_facets), P(self.facet_dofs),
                          self.nfree, P(rowptr), P(colind), ctypes.byref(nnz))
        return rowptr, colind

    def assemble(self, S, g, dirvals):
        rowptr, colind = self.csr_pattern()
        val = np.zeros(len(colind))
        rhs = np.zeros(self.nfree)
        dv = np.ascontiguousarray(dirvals if len(dirvals) else np.zeros(1))
        rc = lib().orc_assemble(self.D, self.k, self.ncells, P(self.cell_facets), P(self.facet_dofs), self.nfree,
                                P(dv), P(np.ascontiguousarray(S)), P(np.ascontiguousarray(g)), P(rowptr),
                                P(colind), P(val), P(rhs))
        assert rc == 0
        return rowptr, colind, val, rhs

    def cell_skeleton_values(self, lam, dirvals):
        x = np.zeros((self.ncells, self.nf))
        dv = np.ascontiguousarray(dirvals if len(dirvals) else np.zeros(1))
        lib().orc_cell_skeleton_values(self.D, self.k, self.ncells, P(self.cell_facets), P(self.facet_dofs),
                                       P(np.ascontiguousarray(lam)), P(dv), P(x))
        return x

    def l2_errors(self, problem, uint, kappa=None):
        ef, ep = ctypes.c_double(), ctypes.c_double()
        kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        lib().orc_l2_errors(self.D, self.k, P(self.n), P(self.domain), problem, P(kap),
                            P(np.ascontiguousarray(uint)), ctypes.byref(ef), ctypes.byref(ep))
        return ef.value, ep.value


def pm_projection(D, k, kb, lf):
    """P_m on local facet lf: (nfd x (kb+1)^D) coefficients in the order-k facet
    basis of the projected trace of each order-kb cell basis function."""
    nfd, nkb = (k + 1) ** (D - 1), (kb + 1) ** D
    pm = np.zeros((nkb, nfd))  # column-major nfd x nkb
    rc = lib().orc_pm_projection(D, k, kb, lf, P(pm))
    assert rc == 0
    return pm.T.copy()


def facet_quadrature(D, k, lf):
    """(xi (nqf x D), w (nqf), mu (nqf x nfd)) of the order-k tables on local facet lf."""
    n1 = k + 2
    nq = n1 ** (D - 1)
    xi, w, mu = np.zeros((nq, D)), np.zeros(nq), np.zeros((nq, (k + 1) ** (D - 1)))
    assert lib().orc_facet_quadrature(D, k, lf, P(xi), P(w), P(mu)) == nq
    return xi, w, mu


def cell_basis(D, k, xi):
    xi = np.ascontiguousarray(xi, dtype=np.float64)
    val = np.zeros((xi.shape[0], (k + 1) ** D))
    assert lib().orc_cell_basis(D, k, xi.shape[0], P(xi), P(val)) == 0
    return val


def static_condensation(A, b, ni):
    """A: (ncells, n, n) column-major per cell (A[c, j, i]); returns S (column-major), g, info."""
    ncells, n, _ = A.shape
    nf = n - ni
    S = np.zeros((ncells, nf, nf))
    g = np.zeros((ncells, nf))
    info = np.zeros(ncells, dtype=np.int32)
    lib().orc_static_condensation(ncells, ni, nf, P(np.ascontiguousarray(A)), P(np.ascontiguousarray(b)),
                                  P(S), P(g), P(info))
    return S, g, info


def backward_static_condensation(A, b, x, ni):
    ncells, n, _ = A.shape
    u = np.zeros((ncells, ni))
    info = np.zeros(ncells, dtype=np.int32)
    lib().orc_backward_static_condensation(ncells, ni, n - ni, P(np.ascontiguousarray(A)),
                                           P(np.ascontiguousarray(b)), P(np.ascontiguousarray(x)), P(u),
                                           P(info))
    return u, info


def sum_facets(blocks):
    blocks = np.ascontiguousarray(blocks, dtype=np.float64)
    out = np.zeros(blocks[0].size)
    rc = lib().orc_sum_facets(blocks.shape[0], blocks[0].size, P(blocks), P(out))
    assert rc == 0
    return out.reshape(blocks[0].shape)


def dense_solve(rowptr, colind, val, rhs):
    x = np.zeros(len(rhs))
    rc = lib().orc_dense_solve(len(rhs), P(rowptr), P(colind), P(val), P(rhs), P(x))
    assert rc == 0, "singular skeleton system"
    return x


def pcg(rowptr, colind, val, rhs, bs, rtol=1e-12, maxit=100000):
    x = np.zeros(len(rhs))
    it, rel = ctypes.c_int(), ctypes.c_double()
    rc = lib().orc_pcg(len(rhs), bs, P(rowptr), P(colind), P(val), P(rhs), P(x), ctypes.c_double(-1.0),
                       ctypes.c_double(rtol), maxit, ctypes.byref(it), ctypes.byref(rel))
    return x, it.value, rel.value, rc


def solve_darcy(D, k, n, tau=1.0, stab=STAB_TEXTBOOK, problem=PROBLEM_LINEAR, kappa=None, solver=0,
                rtol=1e-12, maxit=100000, want_solution=True, domain=None):
    """The whole path on the CPU; returns a dict with the interior values per cell
    (ncells x ni), the free skeleton values, timings and errors."""
    L = lib()
    n = np.array(n, dtype=np.int32)
    dom = np.array(domain if domain is not None else [0.0, 1.0] * D, dtype=np.float64)
    m = Mesh(D, n, k, dom)
    uint = np.zeros((m.ncells, m.ni)) if want_solution else None
    lam = np.zeros(max(m.nfree, 1)) if want_solution else None
    times = np.zeros(5)
    it, rel, ef, ep = ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
    rc = L.orc_solve_darcy(D, k, P(n), P(dom), ctypes.c_double(tau), stab, problem, P(kap), solver,
                           ctypes.c_double(rtol), maxit, P(uint), P(lam), P(times), ctypes.byref(it),
                           ctypes.byref(rel), ctypes.byref(ef), ctypes.byref(ep))
    return dict(rc=rc, uint=uint, lam=None if lam is None else lam[:m.nfree], times=times, iters=it.value,
                relres=rel.value, err_flux=ef.value, err_pres=ep.value, mesh=m)


class DarcySetup:
    """A Cartesian Darcy mesh set up once (topology, facet DOFs, Dirichlet
    values, CSR pattern: orc_darcy_setup), then solved any number of times
    (orc_darcy_step).  The split lets a timing compare the per-solve work alone."""

    def __init__(self, D, k, n, problem=PROBLEM_LINEAR, domain=None):
        L = lib()
        self.D, self.k = D, k
        self.n = np.array(n, dtype=np.int32)
        self.domain = np.array(domain if domain is not None else [0.0, 1.0] * D, dtype=np.float64)
        self.ni, self.nf = cell_sizes(D, k)
        self.ncells = int(np.prod(self.n))
        self.h = ctypes.c_void_p()
        nnz, nfree = ctypes.c_int64(), ctypes.c_int()
        rc = L.orc_darcy_setup(D, k, P(self.n), P(self.domain), problem, ctypes.byref(self.h), ctypes.byref(nnz),
                               ctypes.byref(nfree))
        assert rc == 0
        self.nnz, self.nfree = nnz.value, nfree.value

    def step(self, tau=1.0, stab=STAB_TEXTBOOK, kappa=None, solver=1, rtol=1e-12, maxit=100000,
             want_solution=True, want_system=False):
        uint = np.zeros((self.ncells, self.ni)) if want_solution else None
        lam = np.zeros(max(self.nfree, 1)) if want_solution else None
        val = np.zeros(max(self.nnz, 1)) if want_system else None
        rhs = np.zeros(max(self.nfree, 1)) if want_system else None
        times = np.zeros(5)
        it, rel, ef, ep = ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        rc = lib().orc_darcy_step(self.h, ctypes.c_double(tau), stab, P(kap), solver, ctypes.c_double(rtol), maxit,
                                  P(uint), P(lam), P(val), P(rhs), P(times), ctypes.byref(it), ctypes.byref(rel),
                                  ctypes.byref(ef), ctypes.byref(ep))
        return dict(rc=rc, uint=uint, lam=None if lam is None else lam[:self.nfree],
                    val=None if val is None else val[:self.nnz], rhs=None if rhs is None else rhs[:self.nfree],
                    times=times, iters=it.value, relres=rel.value, err_flux=ef.value, err_pres=ep.value)

    def close(self):
        if self.h:
            lib().orc_darcy_free(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


EPROBLEM_LINEAR = 0
EPROBLEM_SMOOTH = 1

# General spaces: a polynomial space per field (Q_k tensor product or P_k
# total degree), as ReferenceFE(lagrangian, T, order; space=...) chooses them,
# or RT_k (raviart_thomas on a box: flux component c of order k+1 along x_c and
# k across) for the Darcy flux; Q_0 is the constant.
SPACE_Q, SPACE_P, SPACE_RT = 0, 1, 2
PHYS_DARCY, PHYS_ELASTICITY = 0, 1


def gs_spaces(kindA, kA, kindB, kB, kindT, kT, pm=False):
    """spaces[7] of the general-space functions: first bulk field (Darcy flux /
    stress), second (pressure / displacement), trace; pm projects the
    displacement onto the trace space in the tau terms (P_m)."""
    return np.array([kindA, kA, kindB, kB, kindT, kT, 1 if pm else 0], dtype=np.int32)


def gs_basis_eval(d, kind, k, xi, grad=False):
    xi = np.ascontiguousarray(np.atleast_2d(xi), dtype=np.float64)
    npts = xi.shape[0]
    nb = lib().orc_gs_basis_eval(d, kind, k, 0, P(xi), None, None)
    assert nb > 0
    val = np.zeros((npts, nb))
    gr = np.zeros((npts, nb, d)) if grad else None
    lib().orc_gs_basis_eval(d, kind, k, npts, P(xi), P(val), P(gr))
    return (val, gr) if grad else val


class GsMesh(Mesh):
    """A Cartesian mesh with general-space Darcy or elasticity HDG forms: its
    facet space has nfd = (trace components) x (trace basis size) DOFs per
    facet, numbered as Gridap numbers an L2 facet space with Dirichlet
    boundary."""

    def __init__(self, D, n, phys, spaces, domain=None):
        super().__init__(D, n, 1, domain)
        L = lib()
        self.phys = phys
        self.spaces = np.ascontiguousarray(spaces, dtype=np.int32)
        sz = np.zeros(7, dtype=np.int32)
        rc = L.orc_gs_sizes(D, phys, P(self.spaces), P(sz))
        assert rc == 0, "unsupported spaces"
        self.ni, self.nf, self.nfd, self.nA, self.nB, self.nT, self.nqv = (int(v) for v in sz)
        self.facet_dofs = np.zeros((self.nfacets, self.nfd), dtype=np.int32)
        nfree, ndir = ctypes.c_int(), ctypes.c_int()
        L.orc_facet_dofs_n(self.nfd, self.nfacets, P(self.facet_is_boundary), P(self.facet_dofs),
                           ctypes.byref(nfree), ctypes.byref(ndir))
        self.nfree, self.ndir = nfree.value, ndir.value

    def integrate(self, tau=1.0, stab=STAB_TEXTBOOK, problem=PROBLEM_LINEAR, coef=None, E=1.0):
        n = self.ni + self.nf
        A = np.zeros((self.ncells, n, n))
        b = np.zeros((self.ncells, n))
        cf = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
        rc = lib().orc_gs_integrate(self.D, self.phys, P(self.spaces), P(self.n), P(self.domain),
                                    ctypes.c_double(tau), stab, problem, P(cf), ctypes.c_double(E), P(A), P(b))
        assert rc == 0
        return A, b

    def dirichlet_values(self, problem):
        vals = np.zeros(max(self.ndir, 1))
        lib().orc_gs_dirichlet_values(self.D, self.phys, P(self.spaces), P(self.n), P(self.domain), problem,
                                      P(self.facet_dofs), self.ndir, P(vals))
        return vals[:self.ndir] if self.ndir else vals[:0]

    def l2_errors(self, problem, uint, coef=None, E=1.0):
        e1, e2 = ctypes.c_double(), ctypes.c_double()
        cf = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
        lib().orc_gs_l2_errors(self.D, self.phys, P(self.spaces), P(self.n), P(self.domain), problem, P(cf),
                               ctypes.c_double(E), P(np.ascontiguousarray(uint)), ctypes.byref(e1),
                               ctypes.byref(e2))
        return e1.value, e2.value


class GsCopiesMesh(GsMesh):
    """`copies` independent copies of one general-space form on one mesh, as a
    multi-field space [A_1..A_c, B_1..B_c, T_1..T_c] sums the same block form
    once per copy (test/MultiFieldLagrangeMultipliersTests.jl:40-88).  The
    cell matrix holds the copies' first fields, then their second fields, then
    per local facet the copies' trace DOFs one copy after the other
    (facet-major); `multi_field_order` maps facet-major skeleton values to
    Gridap's numbering, all DOFs of the first trace field before the second."""

    def __init__(self, D, n, phys, spaces, copies, domain=None):
        self.one = GsMesh(D, n, phys, spaces, domain)
        Mesh.__init__(self, D, n, 1, domain)
        o = self.one
        self.phys, self.spaces, self.copies = phys, o.spaces, copies
        self.nA, self.nB, self.nT, self.nqv = o.nA, o.nB, o.nT, o.nqv
        self.ni, self.nfd = copies * o.ni, copies * o.nfd
        self.nf = 2 * D * self.nfd
        self.facet_dofs = np.zeros((self.nfacets, self.nfd), dtype=np.int32)
        nfree, ndir = ctypes.c_int(), ctypes.c_int()
        lib().orc_facet_dofs_n(self.nfd, self.nfacets, P(self.facet_is_boundary), P(self.facet_dofs),
                               ctypes.byref(nfree), ctypes.byref(ndir))
        self.nfree, self.ndir = nfree.value, ndir.value
        ncA = D if phys == PHYS_DARCY else D * (D + 1) // 2
        na = ncA * o.nA  # first-field DOFs of one copy
        self.maps = []
        for cp in range(copies):
            i1 = np.arange(o.ni + o.nf)
            lf, a = np.divmod(i1 - o.ni, o.nfd)
            m = np.where(i1 < na, cp * na + i1,
                         np.where(i1 < o.ni, copies * na + cp * (o.ni - na) + i1 - na,
                                  self.ni + lf * self.nfd + cp * o.nfd + a))
            self.maps.append(m)

    def integrate(self, **kw):
        A1, b1 = self.one.integrate(**kw)
        n = self.ni + self.nf
        A = np.zeros((self.ncells, n, n))
        b = np.zeros((self.ncells, n))
        for m in self.maps:
            A[:, m[:, None], m[None, :]] = A1
            b[:, m] = b1
        return A, b

    def dirichlet_values(self, problem):
        dv1 = self.one.dirichlet_values(problem)
        dv = np.zeros(self.ndir)
        nfd1 = self.one.nfd
        for cp in range(self.copies):
            fd = self.facet_dofs[:, cp * nfd1:(cp + 1) * nfd1]
            on = fd < 0
            dv[-1 - fd[on]] = dv1[-1 - self.one.facet_dofs[on]]
        return dv

    def multi_field_order(self, lam):
        nfd1 = self.one.nfd
        per = self.nfree // self.copies
        return np.asarray(lam).reshape(-1, self.copies, nfd1).transpose(1, 0, 2).reshape(self.copies * per)

    def l2_errors(self, problem, uint, coef=None, E=1.0):
        s1 = s2 = 0.0
        for m in self.maps:
            e1, e2 = self.one.l2_errors(problem, uint[:, m[:self.one.ni]], coef=coef, E=E)
            s1, s2 = s1 + e1 * e1, s2 + e2 * e2
        return np.sqrt(s1), np.sqrt(s2)


class ElasticityMesh(Mesh):
    """The linear elasticity HDG spaces on the same Cartesian mesh: symmetric
    stress Q_k, displacement Q_k, displacement trace Q_k (D components per
    facet node, component-major) with Dirichlet data on the boundary."""

    def __init__(self, D, n, k, domain=None):
        super().__init__(D, n, k, domain)
        L = lib()
        ni, nf, nfd = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.orc_elasticity_sizes(D, k, ctypes.byref(ni), ctypes.byref(nf), ctypes.byref(nfd))
        self.ni, self.nf, self.nfd = ni.value, nf.value, nfd.value
        self.facet_dofs = np.zeros((self.nfacets, self.nfd), dtype=np.int32)
        nfree, ndir = ctypes.c_int(), ctypes.c_int()
        L.orc_facet_dofs_n(self.nfd, self.nfacets, P(self.facet_is_boundary), P(self.facet_dofs),
                           ctypes.byref(nfree), ctypes.byref(ndir))
        self.nfree, self.ndir = nfree.value, ndir.value

    def integrate(self, tau=1.0, E=1.0, nu=None, problem=EPROBLEM_SMOOTH):
        n = self.ni + self.nf
        A = np.zeros((self.ncells, n, n))  # A[c, j, i] = A_c(i, j)
        b = np.zeros((self.ncells, n))
        v = None if nu is None else np.ascontiguousarray(nu, dtype=np.float64)
        rc = lib().orc_integrate_elasticity(self.D, self.k, P(self.n), P(self.domain), ctypes.c_double(tau),
                                            ctypes.c_double(E), P(v), problem, P(A), P(b))
        assert rc == 0
        return A, b

    def dirichlet_values(self, problem):
        vals = np.zeros(max(self.ndir, 1))
        lib().orc_dirichlet_values_elasticity(self.D, self.k, P(self.n), P(self.domain), problem, self.nfacets,
                                              P(self.facet_is_boundary), P(self.facet_dofs), self.ndir, P(vals))
        return vals[:self.ndir] if self.ndir else vals[:0]

    def csr_pattern(self):
        nnz = ctypes.c_int64()
        L = lib()
        L.orc_csr_pattern_n(self.D, self.nfd, self.ncells, self.nfacets, P(self.cell_facets), P(self.facet_dofs),
                            self.nfree, None, None, ctypes.byref(nnz))
        rowptr = np.zeros(self.nfree + 1, dtype=np.int64)
        colind = np.zeros(nnz.value, dtype=np.int32)
        L.orc_csr_pattern_n(self.D, self.nfd, self.ncells, self.nfacets, P(self.cell_facets), P(self.facet_dofs),
                            self.nfree, P(rowptr), P(colind), ctypes.byref(nnz))
        return rowptr, colind

    def assemble(self, S, g, dirvals):
        rowptr, colind = self.csr_pattern()
        val = np.zeros(len(colind))
        rhs = np.zeros(self.nfree)
        dv = np.ascontiguousarray(dirvals if len(dirvals) else np.zeros(1))
        rc = lib().orc_assemble_n(self.D, self.nfd, self.ncells, P(self.cell_facets), P(self.facet_dofs),
                                  self.nfree, P(dv), P(np.ascontiguousarray(S)), P(np.ascontiguousarray(g)),
                                  P(rowptr), P(colind), P(val), P(rhs))
        assert rc == 0
        return rowptr, colind, val, rhs

    def cell_skeleton_values(self, lam, dirvals):
        x = np.zeros((self.ncells, self.nf))
        dv = np.ascontiguousarray(dirvals if len(dirvals) else np.zeros(1))
        lib().orc_cell_skeleton_values_n(self.D, self.nfd, self.ncells, P(self.cell_facets), P(self.facet_dofs),
                                         P(np.ascontiguousarray(lam)), P(dv), P(x))
        return x

    def l2_errors(self, problem, uint, E=1.0, nu=None):
        es, eu = ctypes.c_double(), ctypes.c_double()
        v = None if nu is None else np.ascontiguousarray(nu, dtype=np.float64)
        lib().orc_l2_errors_elasticity(self.D, self.k, P(self.n), P(self.domain), ctypes.c_double(E), P(v), problem,
                                       P(np.ascontiguousarray(uint)), ctypes.byref(es), ctypes.byref(eu))
        return es.value, eu.value


def solve_elasticity(D, k, n, tau=None, E=1.0, nu=None, problem=EPROBLEM_SMOOTH, solver=0, sign=1.0,
                     rtol=1e-12, maxit=100000, domain=None):
    """The elasticity path on the CPU (solver 0: dense LU, 1: block-Jacobi PCG on
    sign * S); tau defaults to the reference's 1/h (cells per side)."""
    L = lib()
    n = np.array(n, dtype=np.int32)
    dom = np.array(domain if domain is not None else [0.0, 1.0] * D, dtype=np.float64)
    m = ElasticityMesh(D, n, k, dom)
    tau = float(n[0]) if tau is None else float(tau)
    uint = np.zeros((m.ncells, m.ni))
    lam = np.zeros(max(m.nfree, 1))
    it, rel, es, eu = ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    v = None if nu is None else np.ascontiguousarray(nu, dtype=np.float64)
    rc = L.orc_solve_elasticity(D, k, P(n), P(dom), ctypes.c_double(tau), ctypes.c_double(E), P(v), problem, solver,
                                ctypes.c_double(sign), ctypes.c_double(rtol), maxit, P(uint), P(lam),
                                ctypes.byref(it), ctypes.byref(rel), ctypes.byref(es), ctypes.byref(eu))
    return dict(rc=rc, uint=uint, lam=lam[:m.nfree], iters=it.value, relres=rel.value, err_sigma=es.value,
                err_u=eu.value, mesh=m, tau=tau)


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return int(lib().orc_max_threads())


GsMesh.csr_pattern = ElasticityMesh.csr_pattern
GsMesh.assemble = ElasticityMesh.assemble
GsMesh.cell_skeleton_values = ElasticityMesh.cell_skeleton_values


class SimplexMesh:
    """simplexify(CartesianDiscreteModel(domain, n)): every box cell split into
    D! simplices around its diagonal from the lowest to the highest vertex
    (Kuhn: one simplex per order in which the path from that vertex steps along
    the axes; 2 triangles per square, 6 tetrahedra per cube), in box order then
    in lexicographic order of the axis permutation.  Vertices are the lattice
    points numbered with x fastest; a cell lists its vertices in increasing
    global order; local facet lf is the face opposite local vertex D - lf;
    facets are numbered in first-met order over (cell, local facet); the owner
    of a facet is its first cell; facet DOFs are numbered facet by facet, the
    boundary facets' DOFs Dirichlet (negative ids)."""

    def __init__(self, D, n, spaces, domain=None):
        import itertools
        self.D, self.n = D, tuple(int(v) for v in n)
        self.domain = np.array(domain if domain is not None else [0.0, 1.0] * D, dtype=np.float64)
        self.spaces = np.ascontiguousarray(spaces, dtype=np.int32)
        sz = np.zeros(7, dtype=np.int32)
        assert lib().orc_sx_sizes(D, P(self.spaces), P(sz)) == 0, "unsupported simplex spaces"
        self.ni, self.nf, self.nfd, self.nA, self.nB, self.nT, self.nqv = (int(v) for v in sz)
        nv = [v + 1 for v in self.n]
        h = [(self.domain[2 * d + 1] - self.domain[2 * d]) / self.n[d] for d in range(D)]

        def vid(idx):
            r, m = 0, 1
            for d in range(D):
                r += idx[d] * m
                m *= nv[d]
            return r

        cells = []
        for box in itertools.product(*[range(v) for v in reversed(self.n)]):
            box = tuple(reversed(box))  # x fastest
            for perm in itertools.permutations(range(D)):
                cur = list(box)
                verts = [vid(cur)]
                for ax in perm:
                    cur[ax] += 1
                    verts.append(vid(cur))
                cells.append(sorted(verts))
        self.cells = np.array(cells, dtype=np.int64)
        self.ncells = len(cells)
        coords = np.zeros((int(np.prod(nv)), D))
        for idx in itertools.product(*[range(v) for v in nv]):
            coords[vid(idx)] = [self.domain[2 * d] + idx[d] * h[d] for d in range(D)]
        self.coords = coords
        nl = D + 1
        self.nl = nl
        fid = {}
        cell_facets = np.zeros((self.ncells, nl), dtype=np.int32)
        fcells = []
        for c, vs in enumerate(cells):
            for lf in range(nl):
                opp = D - lf
                key = tuple(v for j, v in enumerate(vs) if j != opp)
                if key not in fid:
                    fid[key] = len(fcells)
                    fcells.append([c, lf, -1, -1])
                else:
                    fcells[fid[key]][2:] = [c, lf]
                cell_facets[c, lf] = fid[key]
        self.cell_facets = cell_facets
        self.nfacets = len(fcells)
        fc = np.array(fcells, dtype=np.int32)
        self.facet_cells = np.ascontiguousarray(fc[:, [0, 2]])
        self.facet_cell_lf = np.ascontiguousarray(fc[:, [0, 1]])
        self.facet_is_boundary = (fc[:, 2] < 0).astype(np.int32)
        self.facet_dofs = np.zeros((self.nfacets, self.nfd), dtype=np.int32)
        nfree, ndir = ctypes.c_int(), ctypes.c_int()
        lib().orc_facet_dofs_n(self.nfd, self.nfacets, P(self.facet_is_boundary), P(self.facet_dofs),
                               ctypes.byref(nfree), ctypes.byref(ndir))
        self.nfree, self.ndir = nfree.value, ndir.value
        X = coords[self.cells]  # ncells x (D+1) x D
        self.origin = np.ascontiguousarray(X[:, 0, :])
        # column-major J per cell: column j = x_{j+1} - x_0
        self.jac = np.ascontiguousarray((X[:, 1:, :] - X[:, :1, :]).reshape(self.ncells, D * D))
        self.sgn = np.where(self.facet_cells[cell_facets, 0] == np.arange(self.ncells)[:, None], 1.0, -1.0)

    def integrate(self, tau=1.0, stab=STAB_TEXTBOOK, problem=PROBLEM_LINEAR, coef=None):
        n = self.ni + self.nf
        A = np.zeros((self.ncells, n, n))
        b = np.zeros((self.ncells, n))
        cf = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
        rc = lib().orc_sx_integrate(self.D, P(self.spaces), self.ncells, P(self.origin), P(self.jac),
                                    P(np.ascontiguousarray(self.sgn)), ctypes.c_double(tau), stab, problem, P(cf),
                                    P(A), P(b))
        assert rc == 0
        return A, b

    def dirichlet_values(self, problem):
        vals = np.zeros(max(self.ndir, 1))
        lib().orc_sx_dirichlet_values(self.D, P(self.spaces), self.nfacets, P(self.facet_cell_lf), P(self.origin),
                                      P(self.jac), problem, P(self.facet_dofs), self.ndir, P(vals))
        return vals[:self.ndir]

    def csr_pattern(self):
        nnz = ctypes.c_int64()
        L = lib()
        L.orc_csr_pattern_nl(self.nl, self.nfd, self.ncells, self.nfacets, P(self.cell_facets), P(self.facet_dofs),
                             self.nfree, None, None, ctypes.byref(nnz))
        rowptr = np.zeros(self.nfree + 1, dtype=np.int64)
        colind = np.zeros(nnz.value, dtype=np.int32)
        L.orc_csr_pattern_nl(self.nl, self.nfd, self.ncells, self.nfacets, P(self.cell_facets), P(self.facet_dofs),
                             self.nfree, P(rowptr), P(colind), ctypes.byref(nnz))
        return rowptr, colind

    def assemble(self, S, g, dirvals):
        rowptr, colind = self.csr_pattern()
        val = np.zeros(len(colind))
        rhs = np.zeros(self.nfree)
        dv = np.ascontiguousarray(dirvals if len(dirvals) else np.zeros(1))
        rc = lib().orc_assemble_nl(self.nl, self.nfd, self.ncells, P(self.cell_facets), P(self.facet_dofs),
                                   self.nfree, P(dv), P(np.ascontiguousarray(S)), P(np.ascontiguousarray(g)),
                                   P(rowptr), P(colind), P(val), P(rhs))
        assert rc == 0
        return rowptr, colind, val, rhs

    def cell_skeleton_values(self, lam, dirvals):
        x = np.zeros((self.ncells, self.nf))
        dv = np.ascontiguousarray(dirvals if len(dirvals) else np.zeros(1))
        lib().orc_cell_skeleton_values_nl(self.nl, self.nfd, self.ncells, P(self.cell_facets), P(self.facet_dofs),
                                          P(np.ascontiguousarray(lam)), P(dv), P(x))
        return x

    def l2_errors(self, problem, uint, coef=None):
        e1, e2 = ctypes.c_double(), ctypes.c_double()
        cf = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
        lib().orc_sx_l2_errors(self.D, P(self.spaces), self.ncells, P(self.origin), P(self.jac), problem, P(cf),
                               P(np.ascontiguousarray(uint)), ctypes.byref(e1), ctypes.byref(e2))
        return e1.value, e2.value


def solve_simplex(D, n, spaces, tau=1.0, stab=STAB_TEXTBOOK, problem=PROBLEM_LINEAR, coef=None, domain=None):
    """The Darcy HDG path on a simplexified Cartesian mesh, on the CPU:
    integrate, StaticCondensationMap, assemble, dense LU on the skeleton,
    BackwardStaticCondensationMap, L2 errors of the flux and the pressure."""
    m = SimplexMesh(D, n, spaces, domain)
    A, b = m.integrate(tau=tau, stab=stab, problem=problem, coef=coef)
    S, g, info = static_condensation(A, b, m.ni)
    assert (info == 0).all()
    dv = m.dirichlet_values(problem)
    rowptr, colind, val, rhs = m.assemble(S, g, dv)
    lam = dense_solve(rowptr, colind, val, rhs)
    xc = m.cell_skeleton_values(lam, dv)
    uint, _ = backward_static_condensation(A, b, xc, m.ni)
    e1, e2 = m.l2_errors(problem, uint, coef=coef)
    return dict(uint=uint, lam=lam, err1=e1, err2=e2, mesh=m, A=A, b=b, S=S, g=g, val=val, rhs=rhs,
                rowptr=rowptr, colind=colind)


def solve_gs(D, n, phys, spaces, tau=1.0, stab=STAB_TEXTBOOK, problem=PROBLEM_LINEAR, coef=None, E=1.0, solver=0,
             sign=None, rtol=1e-13, maxit=100000, domain=None, copies=1):
    """The general-space path on the CPU: integrate, StaticCondensationMap,
    assemble, skeleton solve (0: dense LU, 1: block-Jacobi PCG on sign*S; sign
    defaults to -1 for Darcy, +1 for elasticity), BackwardStaticCondensationMap,
    L2 errors of the two bulk fields (root sum of squares over copies)."""
    m = GsMesh(D, n, phys, spaces, domain) if copies == 1 else GsCopiesMesh(D, n, phys, spaces, copies, domain)
    A, b = m.integrate(tau=tau, stab=stab, problem=problem, coef=coef, E=E)
    S, g, info = static_condensation(A, b, m.ni)
    assert (info == 0).all()
    dv = m.dirichlet_values(problem)
    rowptr, colind, val, rhs = m.assemble(S, g, dv)
    if solver == 0:
        lam = dense_solve(rowptr, colind, val, rhs)
        it, rel = 0, 0.0
    else:
        if sign is None:
            sign = -1.0 if phys == PHYS_DARCY else 1.0
        lam = np.zeros(len(rhs))
        itc, relc = ctypes.c_int(), ctypes.c_double()
        rc = lib().orc_pcg(len(rhs), m.nfd, P(rowptr), P(colind), P(val), P(rhs), P(lam), ctypes.c_double(sign),
                           ctypes.c_double(rtol), maxit, ctypes.byref(itc), ctypes.byref(relc))
        assert rc == 0
        it, rel = itc.value, relc.value
    xc = m.cell_skeleton_values(lam, dv)
    uint, _ = backward_static_condensation(A, b, xc, m.ni)
    e1, e2 = m.l2_errors(problem, uint, coef=coef, E=E)
    return dict(uint=uint, lam=lam, err1=e1, err2=e2, mesh=m, A=A, b=b, S=S, g=g, val=val, rhs=rhs,
                rowptr=rowptr, colind=colind, iters=it, relres=rel)

