/*
 * hdg_oracle.c -- CPU FP64 restatement of GridapHybrid.jl's hybridization path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Loaded by tests/, smoke() and the
 * CPU-baseline leg of bench.py; never by the GPU product path.
 *
 * Reference files are cited as path:line inside the GridapHybrid.jl repository.
 * Gridap.jl (0.18.2, branch exploring_hybridization, tree d7c0d281) is a
 * dependency that is not vendored with the reference; where its behaviour is
 * restated (node ordering, face numbering, quadrature, assembly) the comment
 * says so.
 */
#include "hdg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXD 3
#define MAXK 6

static double wtime(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.0;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* ------------------------------------------------------------------------ */
/* Reference element: Gridap's Lagrangian node order on n-cubes.             */
/* ------------------------------------------------------------------------ */

static int ipow(int b, int e) {
  int r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

int orc_num_nodes(int D, int k) { return ipow(k + 1, D); }

typedef struct {
  int free_mask; /* bit d set: dimension d is a parameter of the face */
  int fixed;     /* bit d: coordinate value (0/1) of a fixed dimension */
} cube_face;

static int popc(int x) {
  int c = 0;
  while (x) {
    c += x & 1;
    x >>= 1;
  }
  return c;
}

/* Faces of the D-cube in Gridap's ExtrusionPolytope order: the (d+1)-cube's
 * faces are the d-cube's faces at x_d = 0, then at x_d = 1, then extruded
 * along x_d, stably sorted by dimension.  For QUAD this gives vertices
 * (0,0),(1,0),(0,1),(1,1), edges [y=0, y=1, x=0, x=1]; for HEX the facets
 * [z=0, z=1, y=0, y=1, x=0, x=1] (Gridap.ReferenceFEs polytope conventions,
 * used by test/DarcyHDGTests.jl through CartesianDiscreteModel). */
static int cube_faces(int D, cube_face *out) {
  cube_face cur[27], tmp[81];
  int n = 1;
  cur[0].free_mask = 0;
  cur[0].fixed = 0;
  for (int d = 0; d < D; ++d) {
    int m = 0;
    for (int i = 0; i < n; ++i) tmp[m++] = cur[i];
    for (int i = 0; i < n; ++i) {
      tmp[m] = cur[i];
      tmp[m].fixed |= (1 << d);
      ++m;
    }
    for (int i = 0; i < n; ++i) {
      tmp[m] = cur[i];
      tmp[m].free_mask |= (1 << d);
      ++m;
    }
    n = 0;
    for (int dim = 0; dim <= d + 1; ++dim)
      for (int i = 0; i < m; ++i)
        if (popc(tmp[i].free_mask) == dim) cur[n++] = tmp[i];
  }
  memcpy(out, cur, sizeof(cube_face) * n);
  return n;
}

/* Node lattice indices (i_0..i_{D-1}, each in 0..k) in Gridap's node order:
 * nodes are owned by faces in face order; a face's own nodes are the interior
 * lattice points of that face, first face parameter fastest. */
int orc_lagrange_lattice(int D, int k, int *lattice) {
  if (D < 1 || D > MAXD || k < 1 || k > MAXK) return -1;
  cube_face faces[27];
  int nfaces = cube_faces(D, faces);
  int cnt = 0;
  for (int fi = 0; fi < nfaces; ++fi) {
    int fm = faces[fi].free_mask;
    int nfree = popc(fm);
    int free_dims[MAXD];
    int t = 0;
    for (int d = 0; d < D; ++d)
      if (fm & (1 << d)) free_dims[t++] = d;
    int nint = ipow(k - 1, nfree);
    for (int s = 0; s < nint; ++s) {
      int r = s;
      int idx[MAXD];
      for (int d = 0; d < D; ++d) idx[d] = (faces[fi].fixed & (1 << d)) ? k : 0;
      for (int j = 0; j < nfree; ++j) {
        idx[free_dims[j]] = 1 + r % (k - 1);
        r /= (k - 1);
      }
      for (int d = 0; d < D; ++d) lattice[cnt * D + d] = idx[d];
      ++cnt;
    }
  }
  return cnt;
}

/* 1D Lagrange polynomial on equispaced nodes t_j = j/k, and its derivative. */
static void lag1d(int k, int i, double x, double *val, double *der) {
  double v = 1.0, dv = 0.0;
  double ti = (double)i / k;
  for (int j = 0; j <= k; ++j) {
    if (j == i) continue;
    double tj = (double)j / k;
    double f = (x - tj) / (ti - tj);
    double df = 1.0 / (ti - tj);
    dv = dv * f + v * df;
    v = v * f;
  }
  *val = v;
  *der = dv;
}

/* Gauss-Legendre rule on [0,1] (Gridap's tensor-product quadrature uses
 * ceil((degree+1)/2) Gauss-Legendre points per direction). */
void orc_gauss_legendre01(int npts, double *x, double *w) {
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < npts; ++i) {
    double z = cos(pi * (i + 0.75) / (npts + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int j = 2; j <= npts; ++j) {
        double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (npts == 1) {
        p1 = z;
        p0 = 1.0;
      }
      dp = npts * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    {
      double p0 = 1.0, p1 = z;
      for (int j = 2; j <= npts; ++j) {
        double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (npts == 1) {
        p1 = z;
        p0 = 1.0;
      }
      dp = npts * (z * p1 - p0) / (z * z - 1.0);
    }
    x[npts - 1 - i] = 0.5 * (1.0 + z);
    w[npts - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

/* ------------------------------------------------------------------------ */
/* Cartesian mesh in Gridap numbering.                                       */
/* ------------------------------------------------------------------------ */

int orc_cart_counts(int D, const int *n, int *ncells, int *nfacets) {
  if (D < 1 || D > MAXD) return -1;
  long nc = 1, nfc = 0;
  for (int d = 0; d < D; ++d) nc *= n[d];
  for (int d = 0; d < D; ++d) nfc += nc / n[d] * (n[d] + 1);
  *ncells = (int)nc;
  *nfacets = (int)nfc;
  return 0;
}

/* local facet index of (normal dimension d, side s) in Gridap order */
static int lface_of(int D, int d, int s) { return 2 * (D - 1 - d) + s; }

/* Facet numbering of Gridap's grid topology (faces are numbered in the order
 * they are first met when looping cells and their local faces); cells around
 * a facet are listed in increasing cell id, so facet_cells[2f] is the owner
 * used by get_cell_owner_normal_vector (src/Skeleton.jl:549-556,
 * src/SkeletonArrays.jl:219-229) and by the recovery glue
 * (src/HybridAffineFEOperators.jl:210-224). */
int orc_cart_topology(int D, const int *n, int *cell_facets, int *facet_cells,
                      int *facet_is_boundary) {
  int ncells, nfacets;
  if (orc_cart_counts(D, n, &ncells, &nfacets)) return -1;
  int stride[MAXD];
  stride[0] = 1;
  for (int d = 1; d < D; ++d) stride[d] = stride[d - 1] * n[d - 1];
  int next = 0;
  for (int c = 0; c < ncells; ++c) {
    int idx[MAXD], r = c;
    for (int d = 0; d < D; ++d) {
      idx[d] = r % n[d];
      r /= n[d];
    }
    for (int lf = 0; lf < 2 * D; ++lf) {
      int d = D - 1 - lf / 2, s = lf % 2;
      int f;
      if (s == 0 && idx[d] > 0) {
        f = cell_facets[(c - stride[d]) * 2 * D + lface_of(D, d, 1)];
        facet_cells[2 * f + 1] = c;
        facet_is_boundary[f] = 0;
      } else {
        f = next++;
        facet_cells[2 * f] = c;
        facet_cells[2 * f + 1] = -1;
        facet_is_boundary[f] = 1;
        if (s == 1 && idx[d] < n[d] - 1) facet_is_boundary[f] = 0;
      }
      cell_facets[c * 2 * D + lf] = f;
    }
  }
  return next == nfacets ? 0 : -2;
}

/* DOF numbering of the L2-conforming facet space with Dirichlet tags on the
 * boundary (test/DarcyHDGTests.jl:44-47): facets in order, each facet's DOFs
 * consecutive, free and Dirichlet DOFs numbered separately. */
int orc_facet_dofs(int D, int k, int nfacets, const int *facet_is_boundary,
                   int *facet_dofs, int *nfree, int *ndir) {
  return orc_facet_dofs_n(ipow(k + 1, D - 1), nfacets, facet_is_boundary, facet_dofs, nfree, ndir);
}

/* The same with nfd DOFs per facet (a vector-valued facet space has
 * D * (k+1)^(D-1), component-major within the facet). */
int orc_facet_dofs_n(int nfd, int nfacets, const int *facet_is_boundary, int *facet_dofs, int *nfree,
                     int *ndir) {
  int fr = 0, di = 0;
  for (int f = 0; f < nfacets; ++f)
    for (int a = 0; a < nfd; ++a)
      facet_dofs[f * nfd + a] = facet_is_boundary[f] ? -1 - (di++) : fr++;
  *nfree = fr;
  *ndir = di;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Reference tables and manufactured problems.                               */
/* ------------------------------------------------------------------------ */

typedef struct {
  int D, k, nk, nfd, ni, nf, n, n1, nqv, nqf;
  int lat[216 * 3];  /* cell lattice (nk x D) */
  int flat[36 * 2];  /* facet lattice (nfd x (D-1)) */
  double *qv_xi;     /* nqv x D */
  double *qv_w;      /* nqv */
  double *phi;       /* nqv x nk */
  double *dphi;      /* nqv x nk x D (reference gradient) */
  double *qf_w;      /* nqf */
  double *fphi;      /* 2D x nqf x nk : cell basis on facet points */
  double *fxi;       /* 2D x nqf x D : cell-local coordinates of facet points */
  double *mu;        /* nqf x nfd : facet basis */
} reftab;

static void basis_eval(const reftab *t, const double *xi, double *val,
                       double *grad) {
  int D = t->D, k = t->k;
  for (int a = 0; a < t->nk; ++a) {
    double l[MAXD], dl[MAXD];
    for (int d = 0; d < D; ++d) lag1d(k, t->lat[a * D + d], xi[d], &l[d], &dl[d]);
    double v = 1.0;
    for (int d = 0; d < D; ++d) v *= l[d];
    val[a] = v;
    if (grad)
      for (int e = 0; e < D; ++e) {
        double g = dl[e];
        for (int d = 0; d < D; ++d)
          if (d != e) g *= l[d];
        grad[a * D + e] = g;
      }
  }
}

static void reftab_free(reftab *t) {
  free(t->qv_xi);
  free(t->qv_w);
  free(t->phi);
  free(t->dphi);
  free(t->qf_w);
  free(t->fphi);
  free(t->fxi);
  free(t->mu);
}

static int reftab_init(reftab *t, int D, int k) {
  memset(t, 0, sizeof(*t));
  if (D < 2 || D > 3 || k < 1 || k > MAXK) return -1;
  t->D = D;
  t->k = k;
  t->nk = ipow(k + 1, D);
  t->nfd = ipow(k + 1, D - 1);
  t->ni = (D + 1) * t->nk;
  t->nf = 2 * D * t->nfd;
  t->n = t->ni + t->nf;
  /* test/DarcyHDGTests.jl:54-55: degree = 2*(order+1) */
  int degree = 2 * (k + 1);
  t->n1 = (degree + 2) / 2; /* ceil((degree+1)/2) */
  t->nqv = ipow(t->n1, D);
  t->nqf = ipow(t->n1, D - 1);
  orc_lagrange_lattice(D, k, t->lat);
  orc_lagrange_lattice(D - 1, k, t->flat);
  double x1[16], w1[16];
  orc_gauss_legendre01(t->n1, x1, w1);
  t->qv_xi = malloc(sizeof(double) * t->nqv * D);
  t->qv_w = malloc(sizeof(double) * t->nqv);
  t->phi = malloc(sizeof(double) * t->nqv * t->nk);
  t->dphi = malloc(sizeof(double) * t->nqv * t->nk * D);
  t->qf_w = malloc(sizeof(double) * t->nqf);
  t->fphi = malloc(sizeof(double) * 2 * D * t->nqf * t->nk);
  t->fxi = malloc(sizeof(double) * 2 * D * t->nqf * D);
  t->mu = malloc(sizeof(double) * t->nqf * t->nfd);
  for (int q = 0; q < t->nqv; ++q) {
    int r = q;
    double w = 1.0;
    for (int d = 0; d < D; ++d) {
      t->qv_xi[q * D + d] = x1[r % t->n1];
      w *= w1[r % t->n1];
      r /= t->n1;
    }
    t->qv_w[q] = w;
    basis_eval(t, &t->qv_xi[q * D], &t->phi[q * t->nk], &t->dphi[q * t->nk * D]);
  }
  for (int q = 0; q < t->nqf; ++q) {
    int r = q;
    double w = 1.0, s[MAXD];
    for (int d = 0; d < D - 1; ++d) {
      s[d] = x1[r % t->n1];
      w *= w1[r % t->n1];
      r /= t->n1;
    }
    t->qf_w[q] = w;
    for (int b = 0; b < t->nfd; ++b) {
      double v = 1.0, dl;
      for (int d = 0; d < D - 1; ++d) {
        double l;
        lag1d(k, t->flat[b * (D - 1) + d], s[d], &l, &dl);
        v *= l;
      }
      t->mu[q * t->nfd + b] = v;
    }
    /* facet parameters are the non-normal dimensions in increasing order */
    for (int lf = 0; lf < 2 * D; ++lf) {
      int dn = D - 1 - lf / 2, side = lf % 2, j = 0;
      double *xi = &t->fxi[(lf * t->nqf + q) * D];
      for (int d = 0; d < D; ++d) xi[d] = (d == dn) ? (double)side : s[j++];
      basis_eval(t, xi, &t->fphi[(lf * t->nqf + q) * t->nk], NULL);
    }
  }
  return 0;
}

enum { PROB_REF_LINEAR = 0, PROB_LINEAR = 1, PROB_SIN = 2 };

/* Exact pressure, flux, flux-equation source f_u and mass source g for
 * kappa^{-1} q + grad p = f_u, div q = g.  PROB_REF_LINEAR is the manufactured
 * solution of test/DarcyHDGTests.jl:8-13 (u = (1+x,1+y), p = -3.14, f = u + grad p,
 * g = div u). */
static void exact(int problem, int D, const double *x, double kappa, double *p,
                  double *q, double *fu, double *g) {
  const double pi = 3.14159265358979323846;
  if (problem == PROB_REF_LINEAR) {
    *p = -3.14;
    for (int d = 0; d < D; ++d) {
      q[d] = 1.0 + x[d];
      fu[d] = q[d] / kappa;
    }
    *g = (double)D;
  } else if (problem == PROB_LINEAR) {
    double s = 0.0;
    for (int d = 0; d < D; ++d) s += x[d];
    *p = s;
    for (int d = 0; d < D; ++d) {
      q[d] = -kappa;
      fu[d] = 0.0;
    }
    *g = 0.0;
  } else {
    double sv[MAXD], cv[MAXD], prod = 1.0;
    for (int d = 0; d < D; ++d) {
      sv[d] = sin(pi * x[d]);
      cv[d] = cos(pi * x[d]);
      prod *= sv[d];
    }
    *p = prod;
    for (int d = 0; d < D; ++d) {
      double gd = pi * cv[d];
      for (int e = 0; e < D; ++e)
        if (e != d) gd *= sv[e];
      q[d] = -kappa * gd;
      fu[d] = 0.0;
    }
    *g = kappa * D * pi * pi * prod;
  }
}

int orc_cell_sizes(int D, int k, int *ni, int *nf) {
  if (D < 2 || D > 3 || k < 1 || k > MAXK) return -1;
  *ni = (D + 1) * ipow(k + 1, D);
  *nf = 2 * D * ipow(k + 1, D - 1);
  return 0;
}

static void cell_geom(int D, const int *n, const double *domain, int c,
                      double *x0, double *h) {
  int r = c;
  for (int d = 0; d < D; ++d) {
    int i = r % n[d];
    r /= n[d];
    h[d] = (domain[2 * d + 1] - domain[2 * d]) / n[d];
    x0[d] = domain[2 * d] + i * h[d];
  }
}

/* Per-cell matrix and vector of the Darcy HDG weak form of
 * test/DarcyHDGTests.jl:125-135 (stab_mode 1: tau*(n.n_o) terms exactly as
 * written there; stab_mode 0: the textbook LDG-H stabilisation tau*(p-l)),
 * with a per-cell permeability kappa in the flux mass term.  Volume and facet
 * contributions are integrated point by point (Gridap IntegrationMap over
 * the facet blocks, src/GridapAPIExtensions.jl:418-451), summed over facets
 * (src/SumFacetsMap.jl:19-30) and merged with the volume part into one cell
 * block (src/HybridAffineFEOperators.jl:254-286).  A is column-major n x n. */
static void integrate_cell(const reftab *t, int c, const int *n,
                           const double *domain, double tau, int stab_mode,
                           int problem, double kappa, const int *facet_cells,
                           const int *cell_facets, double *A, double *b) {
  int D = t->D, nk = t->nk, nfd = t->nfd, ni = t->ni, N = t->n;
  double x0[MAXD], h[MAXD];
  cell_geom(D, n, domain, c, x0, h);
  double detJ = 1.0;
  for (int d = 0; d < D; ++d) detJ *= h[d];
  memset(A, 0, sizeof(double) * N * N);
  memset(b, 0, sizeof(double) * N);
#define AIJ(i, j) A[(size_t)(i) + (size_t)N * (j)]
  /* volume: vh.uh/kappa - (div vh) ph - grad(qh).uh ; vh.f_u + qh g */
  for (int q = 0; q < t->nqv; ++q) {
    const double *ph = &t->phi[q * nk];
    const double *dph = &t->dphi[q * nk * D];
    double wq = t->qv_w[q] * detJ;
    double x[MAXD], pe, qe[MAXD], fu[MAXD], g;
    for (int d = 0; d < D; ++d) x[d] = x0[d] + h[d] * t->qv_xi[q * D + d];
    exact(problem, D, x, kappa, &pe, qe, fu, &g);
    for (int a = 0; a < nk; ++a) {
      for (int bb = 0; bb < nk; ++bb) {
        double m = wq * ph[a] * ph[bb] / kappa;
        for (int d = 0; d < D; ++d) AIJ(d * nk + a, d * nk + bb) += m;
        for (int d = 0; d < D; ++d) {
          /* physical derivative of an affine box map: d/dx_d = (1/h_d) d/dxi_d */
          AIJ(d * nk + a, D * nk + bb) -= wq * (dph[a * D + d] / h[d]) * ph[bb];
          AIJ(D * nk + a, d * nk + bb) -= wq * (dph[a * D + d] / h[d]) * ph[bb];
        }
      }
      for (int d = 0; d < D; ++d) b[d * nk + a] += wq * ph[a] * fu[d];
      b[D * nk + a] += wq * ph[a] * g;
    }
  }
  /* facets of the cell boundary dK */
  for (int lf = 0; lf < 2 * D; ++lf) {
    int dn = D - 1 - lf / 2, side = lf % 2;
    double nrm[MAXD] = {0, 0, 0};
    nrm[dn] = side ? 1.0 : -1.0;
    double detF = 1.0;
    for (int d = 0; d < D; ++d)
      if (d != dn) detF *= h[d];
    int f = cell_facets[c * 2 * D + lf];
    /* n.n_o = +1 on the facet owner (first cell around the facet), -1 otherwise */
    double s = 1.0;
    if (stab_mode == 1) s = (facet_cells[2 * f] == c) ? 1.0 : -1.0;
    int off = ni + lf * nfd;
    for (int q = 0; q < t->nqf; ++q) {
      const double *ph = &t->fphi[(lf * t->nqf + q) * nk];
      const double *mu = &t->mu[q * nfd];
      double wq = t->qf_w[q] * detF;
      for (int a = 0; a < nk; ++a) {
        /* (vh.n) lh and mh (uh.n) */
        for (int bb = 0; bb < nfd; ++bb) {
          for (int d = 0; d < D; ++d) {
            double v = wq * ph[a] * nrm[d] * mu[bb];
            AIJ(d * nk + a, off + bb) += v;
            AIJ(off + bb, d * nk + a) += v;
          }
          /* -tau qh lh (n.no) and +tau mh ph (n.no) */
          AIJ(D * nk + a, off + bb) -= wq * tau * s * ph[a] * mu[bb];
          AIJ(off + bb, D * nk + a) += wq * tau * s * mu[bb] * ph[a];
        }
        for (int bb = 0; bb < nk; ++bb) {
          /* qh (uh.n) and tau qh ph (n.no) */
          for (int d = 0; d < D; ++d)
            AIJ(D * nk + a, d * nk + bb) += wq * ph[a] * ph[bb] * nrm[d];
          AIJ(D * nk + a, D * nk + bb) += wq * tau * s * ph[a] * ph[bb];
        }
      }
      /* -tau mh lh (n.no) */
      for (int a = 0; a < nfd; ++a)
        for (int bb = 0; bb < nfd; ++bb)
          AIJ(off + a, off + bb) -= wq * tau * s * mu[a] * mu[bb];
    }
  }
#undef AIJ
}

/* The same cell block for a general affine cell x = x0 + J xi (J[row][col],
 * from cell_jacobian column-major per cell), as Gridap integrates on any
 * affine map: physical gradients through J^{-T}, the outward unit normal of
 * facet lf as J^{-T} n_ref / |J^{-T} n_ref| (src/Skeleton.jl:524-585,
 * push_normal), the facet measure |det J| |J^{-T} n_ref|.  For a diagonal J
 * it computes what integrate_cell computes (checked by a KAT). */
static void integrate_cell_affine(const reftab *t, int c, const double *x0, const double *jac, double tau,
                                  int stab_mode, int problem, double kappa, const int *facet_cells,
                                  const int *cell_facets, double *A, double *b) {
  int D = t->D, nk = t->nk, nfd = t->nfd, ni = t->ni, N = t->n;
  double J[MAXD][MAXD] = {{0}}, Ji[MAXD][MAXD] = {{0}}, det;
  for (int col = 0; col < D; ++col)
    for (int row = 0; row < D; ++row) J[row][col] = jac[col * D + row];
  if (D == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Ji[0][0] = J[1][1] / det;
    Ji[0][1] = -J[0][1] / det;
    Ji[1][0] = -J[1][0] / det;
    Ji[1][1] = J[0][0] / det;
  } else {
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) {  /* cofactor of J[q][r] -> Ji[r][q] */
        const int r1 = (q + 1) % 3, r2 = (q + 2) % 3, c1 = (r + 1) % 3, c2 = (r + 2) % 3;
        Ji[r][q] = J[r1][c1] * J[r2][c2] - J[r1][c2] * J[r2][c1];
      }
    det = J[0][0] * Ji[0][0] + J[0][1] * Ji[1][0] + J[0][2] * Ji[2][0];
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) Ji[r][q] /= det;
  }
  const double detJ = fabs(det);
  memset(A, 0, sizeof(double) * N * N);
  memset(b, 0, sizeof(double) * N);
#define AIJ(i, j) A[(size_t)(i) + (size_t)N * (j)]
  for (int q = 0; q < t->nqv; ++q) {
    const double *ph = &t->phi[q * nk];
    const double *dph = &t->dphi[q * nk * D];
    double wq = t->qv_w[q] * detJ;
    double x[MAXD], pe, qe[MAXD], fu[MAXD], g;
    for (int d = 0; d < D; ++d) {
      x[d] = x0[d];
      for (int e = 0; e < D; ++e) x[d] += J[d][e] * t->qv_xi[q * D + e];
    }
    exact(problem, D, x, kappa, &pe, qe, fu, &g);
    for (int a = 0; a < nk; ++a) {
      double gx[MAXD];  /* physical gradient of basis a: d/dx_d = sum_e Ji[e][d] d/dxi_e */
      for (int d = 0; d < D; ++d) {
        gx[d] = 0.0;
        for (int e = 0; e < D; ++e) gx[d] += Ji[e][d] * dph[a * D + e];
      }
      for (int bb = 0; bb < nk; ++bb) {
        double m = wq * ph[a] * ph[bb] / kappa;
        for (int d = 0; d < D; ++d) AIJ(d * nk + a, d * nk + bb) += m;
        for (int d = 0; d < D; ++d) {
          AIJ(d * nk + a, D * nk + bb) -= wq * gx[d] * ph[bb];
          AIJ(D * nk + a, d * nk + bb) -= wq * gx[d] * ph[bb];
        }
      }
      for (int d = 0; d < D; ++d) b[d * nk + a] += wq * ph[a] * fu[d];
      b[D * nk + a] += wq * ph[a] * g;
    }
  }
  for (int lf = 0; lf < 2 * D; ++lf) {
    int dn = D - 1 - lf / 2, side = lf % 2;
    double v[MAXD] = {0, 0, 0}, nv = 0.0;
    for (int d = 0; d < D; ++d) {
      v[d] = (side ? 1.0 : -1.0) * Ji[dn][d];
      nv += v[d] * v[d];
    }
    nv = sqrt(nv);
    double nrm[MAXD] = {0, 0, 0};
    for (int d = 0; d < D; ++d) nrm[d] = v[d] / nv;
    const double detF = detJ * nv;
    int f = cell_facets[c * 2 * D + lf];
    double s = 1.0;
    if (stab_mode == 1) s = (facet_cells[2 * f] == c) ? 1.0 : -1.0;
    int off = ni + lf * nfd;
    for (int q = 0; q < t->nqf; ++q) {
      const double *ph = &t->fphi[(lf * t->nqf + q) * nk];
      const double *mu = &t->mu[q * nfd];
      double wq = t->qf_w[q] * detF;
      for (int a = 0; a < nk; ++a) {
        for (int bb = 0; bb < nfd; ++bb) {
          for (int d = 0; d < D; ++d) {
            double w = wq * ph[a] * nrm[d] * mu[bb];
            AIJ(d * nk + a, off + bb) += w;
            AIJ(off + bb, d * nk + a) += w;
          }
          AIJ(D * nk + a, off + bb) -= wq * tau * s * ph[a] * mu[bb];
          AIJ(off + bb, D * nk + a) += wq * tau * s * mu[bb] * ph[a];
        }
        for (int bb = 0; bb < nk; ++bb) {
          for (int d = 0; d < D; ++d)
            AIJ(D * nk + a, d * nk + bb) += wq * ph[a] * ph[bb] * nrm[d];
          AIJ(D * nk + a, D * nk + bb) += wq * tau * s * ph[a] * ph[bb];
        }
      }
      for (int a = 0; a < nfd; ++a)
        for (int bb = 0; bb < nfd; ++bb)
          AIJ(off + a, off + bb) -= wq * tau * s * mu[a] * mu[bb];
    }
  }
#undef AIJ
}

int orc_integrate_darcy_affine(int D, int k, int ncells, const double *origin, const double *jacobian,
                               double tau, int stab_mode, int problem, const double *kappa,
                               const int *facet_cells, const int *cell_facets, double *A, double *b) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  size_t N = t.n;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncells; ++c)
    integrate_cell_affine(&t, c, origin + (size_t)c * D, jacobian + (size_t)c * D * D, tau, stab_mode, problem,
                          kappa ? kappa[c] : 1.0, facet_cells, cell_facets, A + (size_t)c * N * N,
                          b + (size_t)c * N);
  reftab_free(&t);
  return 0;
}

/* Bulk-to-skeleton L2 projection P_m on local facet lf of the reference cell
 * (test/P_m.jl:4-22; compute_bulk_to_skeleton_l2_projection_dofs,
 * src/GridapAPIExtensions.jl:453-500): with the order-k facet basis mu and
 * the order-kb cell basis phi,
 *   A = int_F mu mu^T (nfd x nfd),  B = int_F mu phi^T (nfd x nkb),  P = A \ B,
 * the coefficients in the facet basis of the projected trace of every cell
 * basis function (P column-major, nfd x nkb).  On an affine cell the facet
 * measure scales A and B alike, so P is the same on every cell.  The facet
 * quadrature is the order-k table's (k + 2 points per direction: exact for
 * the degree 2k + 1 of mu phi when kb = k + 1). */
static int getrf(int n, double *A, int lda, int *ipiv);
static void getrs(int n, int nrhs, const double *LU, int lda, const int *ipiv, double *B, int ldb);

int orc_pm_projection(int D, int k, int kb, int lf, double *P) {
  if (kb < 1 || kb > MAXK || lf < 0 || lf >= 2 * D) return -1;
  reftab t, tb;
  if (reftab_init(&t, D, k)) return -1;
  if (reftab_init(&tb, D, kb)) {
    reftab_free(&t);
    return -1;
  }
  const int nfd = t.nfd, nkb = tb.nk;
  double *A = (double *)calloc((size_t)nfd * nfd, sizeof(double));
  double *phi = (double *)malloc(sizeof(double) * nkb);
  int *ipiv = (int *)malloc(sizeof(int) * nfd);
  memset(P, 0, sizeof(double) * (size_t)nfd * nkb);
  for (int q = 0; q < t.nqf; ++q) {
    const double *mu = &t.mu[q * nfd];
    const double w = t.qf_w[q];
    basis_eval(&tb, &t.fxi[(lf * t.nqf + q) * D], phi, NULL);
    for (int a = 0; a < nfd; ++a) {
      for (int b = 0; b < nfd; ++b) A[a + (size_t)nfd * b] += w * mu[a] * mu[b];
      for (int j = 0; j < nkb; ++j) P[a + (size_t)nfd * j] += w * mu[a] * phi[j];
    }
  }
  int rc = getrf(nfd, A, nfd, ipiv);
  if (rc == 0) getrs(nfd, nkb, A, nfd, ipiv, P, nfd);
  free(A);
  free(phi);
  free(ipiv);
  reftab_free(&t);
  reftab_free(&tb);
  return rc;
}

/* The facet quadrature of the order-k table on local facet lf (for checks of
 * P_m): cell-local points xi (nqf x D), weights w (nqf), facet basis mu
 * (nqf x nfd); returns nqf. */
int orc_facet_quadrature(int D, int k, int lf, double *xi, double *w, double *mu) {
  reftab t;
  if (lf < 0 || lf >= 2 * D || reftab_init(&t, D, k)) return -1;
  const int nq = t.nqf;
  if (xi) memcpy(xi, &t.fxi[(size_t)lf * nq * D], sizeof(double) * nq * D);
  if (w) memcpy(w, t.qf_w, sizeof(double) * nq);
  if (mu) memcpy(mu, t.mu, sizeof(double) * nq * t.nfd);
  reftab_free(&t);
  return nq;
}

/* Cell basis of order k at cell-local points xi (npts x D) -> val (npts x nk). */
int orc_cell_basis(int D, int k, int npts, const double *xi, double *val) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  for (int p = 0; p < npts; ++p) basis_eval(&t, &xi[(size_t)p * D], &val[(size_t)p * t.nk], NULL);
  reftab_free(&t);
  return 0;
}

int orc_integrate_darcy(int D, int k, const int *n, const double *domain,
                        double tau, int stab_mode, int problem,
                        const double *kappa, const int *facet_cells,
                        const int *cell_facets, double *A, double *b) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  int ncells, nfacets;
  orc_cart_counts(D, n, &ncells, &nfacets);
  size_t N = t.n;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncells; ++c)
    integrate_cell(&t, c, n, domain, tau, stab_mode, problem,
                   kappa ? kappa[c] : 1.0, facet_cells, cell_facets,
                   A + (size_t)c * N * N, b + (size_t)c * N);
  reftab_free(&t);
  return 0;
}

/* Same for a subset of cells (cells[0..nsel)), output packed in that order. */
int orc_integrate_darcy_cells(int D, int k, const int *n, const double *domain,
                              double tau, int stab_mode, int problem,
                              const double *kappa, const int *facet_cells,
                              const int *cell_facets, int nsel, const int *cells,
                              double *A, double *b) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  size_t N = t.n;
#pragma omp parallel for schedule(static)
  for (int s = 0; s < nsel; ++s) {
    int c = cells[s];
    integrate_cell(&t, c, n, domain, tau, stab_mode, problem,
                   kappa ? kappa[c] : 1.0, facet_cells, cell_facets,
                   A + (size_t)s * N * N, b + (size_t)s * N);
  }
  reftab_free(&t);
  return 0;
}

/* Dirichlet values of the trial skeleton space TrialFESpace(M, p)
 * (test/DarcyHDGTests.jl:52): nodal interpolation of p at the facet
 * Lagrange nodes. */
int orc_dirichlet_values(int D, int k, const int *n, const double *domain,
                         int problem, int nfacets, const int *facet_is_boundary,
                         const int *facet_dofs, int ndir, double *vals) {
  int ncells, nf2;
  orc_cart_counts(D, n, &ncells, &nf2);
  int *cell_facets = malloc(sizeof(int) * ncells * 2 * D);
  int *facet_cells = malloc(sizeof(int) * nfacets * 2);
  int *isb = malloc(sizeof(int) * nfacets);
  orc_cart_topology(D, n, cell_facets, facet_cells, isb);
  int flat[36 * 2];
  orc_lagrange_lattice(D - 1, k, flat);
  int nfd = ipow(k + 1, D - 1);
  for (int c = 0; c < ncells; ++c) {
    double x0[MAXD], h[MAXD];
    cell_geom(D, n, domain, c, x0, h);
    for (int lf = 0; lf < 2 * D; ++lf) {
      int f = cell_facets[c * 2 * D + lf];
      if (!facet_is_boundary[f]) continue;
      int dn = D - 1 - lf / 2, side = lf % 2;
      for (int a = 0; a < nfd; ++a) {
        int id = facet_dofs[f * nfd + a];
        if (id >= 0) continue;
        double x[MAXD];
        int j = 0;
        for (int d = 0; d < D; ++d) {
          double xi = (d == dn) ? (double)side : (double)flat[a * (D - 1) + j++] / k;
          x[d] = x0[d] + h[d] * xi;
        }
        double p, q[MAXD], fu[MAXD], g;
        exact(problem, D, x, 1.0, &p, q, fu, &g);
        if (-1 - id < ndir) vals[-1 - id] = p;
      }
    }
  }
  free(cell_facets);
  free(facet_cells);
  free(isb);
  return 0;
}

/* Nodal values of the manufactured pressure at every facet DOF of a mesh of
 * affine cells (x = origin_c + J_c xi; jacobian column-major per cell), at
 * the facet Lagrange nodes seen from the facet's first cell: free DOF id >= 0
 * -> free_vals[id], Dirichlet DOF id < 0 -> dir_vals[-1 - id] (the values of
 * TrialFESpace(M, p), test/DarcyHDGTests.jl:52, on any affine mesh). */
int orc_facet_node_values_affine(int D, int k, int ncells, const double *origin, const double *jacobian,
                                 const int *cell_facets, const int *facet_cells, int problem, int nfacets,
                                 const int *facet_dofs, double *free_vals, double *dir_vals) {
  int flat[36 * 2];
  orc_lagrange_lattice(D - 1, k, flat);
  int nfd = ipow(k + 1, D - 1);
  for (int c = 0; c < ncells; ++c) {
    const double *x0 = origin + (size_t)c * D, *J = jacobian + (size_t)c * D * D;
    for (int lf = 0; lf < 2 * D; ++lf) {
      int f = cell_facets[c * 2 * D + lf];
      if (f < 0 || f >= nfacets || facet_cells[2 * f] != c) continue;  /* the facet's first cell */
      int dn = D - 1 - lf / 2, side = lf % 2;
      for (int a = 0; a < nfd; ++a) {
        double xi[MAXD], x[MAXD];
        int j = 0;
        for (int d = 0; d < D; ++d) xi[d] = (d == dn) ? (double)side : (double)flat[a * (D - 1) + j++] / k;
        for (int d = 0; d < D; ++d) {
          x[d] = x0[d];
          for (int e = 0; e < D; ++e) x[d] += J[e * D + d] * xi[e];
        }
        double p, q[MAXD], fu[MAXD], g;
        exact(problem, D, x, 1.0, &p, q, fu, &g);
        int id = facet_dofs[f * nfd + a];
        if (id >= 0) {
          if (free_vals) free_vals[id] = p;
        } else if (dir_vals) {
          dir_vals[-1 - id] = p;
        }
      }
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* LAPACK/BLAS restatements used by the maps.                                */
/* ------------------------------------------------------------------------ */

/* dgetrf (unblocked dgetf2 form): partial pivoting on the first maximal
 * |a_ij| (idamax), row swaps over the full row, scaling by the reciprocal
 * pivot, rank-1 update.  Returns LAPACK's info (0 or first zero pivot). */
static int getrf(int n, double *A, int lda, int *ipiv) {
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int p = j;
    double amax = fabs(A[j + (size_t)lda * j]);
    for (int i = j + 1; i < n; ++i) {
      double v = fabs(A[i + (size_t)lda * j]);
      if (v > amax) {
        amax = v;
        p = i;
      }
    }
    ipiv[j] = p;
    if (A[p + (size_t)lda * j] != 0.0) {
      if (p != j)
        for (int c = 0; c < n; ++c) {
          double tmp = A[j + (size_t)lda * c];
          A[j + (size_t)lda * c] = A[p + (size_t)lda * c];
          A[p + (size_t)lda * c] = tmp;
        }
      double r = 1.0 / A[j + (size_t)lda * j];
      for (int i = j + 1; i < n; ++i) A[i + (size_t)lda * j] *= r;
    } else if (info == 0) {
      info = j + 1;
    }
    for (int c = j + 1; c < n; ++c) {
      double u = A[j + (size_t)lda * c];
      if (u != 0.0)
        for (int i = j + 1; i < n; ++i)
          A[i + (size_t)lda * c] -= A[i + (size_t)lda * j] * u;
    }
  }
  return info;
}

/* dgetrs('N'): row interchanges, unit-lower forward solve, upper back solve. */
static void getrs(int n, int nrhs, const double *LU, int lda, const int *ipiv,
                  double *B, int ldb) {
  for (int c = 0; c < nrhs; ++c) {
    double *x = B + (size_t)ldb * c;
    for (int i = 0; i < n; ++i)
      if (ipiv[i] != i) {
        double tmp = x[i];
        x[i] = x[ipiv[i]];
        x[ipiv[i]] = tmp;
      }
    for (int j = 0; j < n; ++j) {
      double xj = x[j];
      if (xj != 0.0)
        for (int i = j + 1; i < n; ++i) x[i] -= xj * LU[i + (size_t)lda * j];
    }
    for (int j = n - 1; j >= 0; --j) {
      if (x[j] != 0.0) {
        x[j] /= LU[j + (size_t)lda * j];
        double xj = x[j];
        for (int i = 0; i < j; ++i) x[i] -= xj * LU[i + (size_t)lda * j];
      }
    }
  }
}

/* C = C - A*B (dgemm 'N','N', alpha = -1, beta = 1; reference loop order) */
static void gemm_sub(int m, int nn, int kk, const double *A, int lda,
                     const double *B, int ldb, double *C, int ldc) {
  for (int j = 0; j < nn; ++j)
    for (int l = 0; l < kk; ++l) {
      double tmp = -B[l + (size_t)ldb * j];
      if (tmp != 0.0)
        for (int i = 0; i < m; ++i) C[i + (size_t)ldc * j] += tmp * A[i + (size_t)lda * l];
    }
}

/* y = y - A*x (dgemv 'N', alpha = -1, beta = 1) */
static void gemv_sub(int m, int nn, const double *A, int lda, const double *x,
                     double *y) {
  for (int j = 0; j < nn; ++j) {
    double tmp = -x[j];
    if (tmp != 0.0)
      for (int i = 0; i < m; ++i) y[i] += tmp * A[i + (size_t)lda * j];
  }
}

static void copy_block(const double *A, int lda, int r0, int c0, int m, int nn,
                       double *out) {
  for (int j = 0; j < nn; ++j)
    for (int i = 0; i < m; ++i) out[i + (size_t)m * j] = A[(r0 + i) + (size_t)lda * (c0 + j)];
}

/* StaticCondensationMap evaluate! (src/StaticCondensationMap.jl:146-196),
 * op for op: A11 = L11 U11 (getrf, :179), A12 = A11^{-1} A12 (getrs, :183),
 * A22 -= A21 A12 (gemm, :186), b1 = A11^{-1} b1 (getrs, :189),
 * b2 -= A21 b1 (gemv, :192); returns (A22, b2) = (S, g). */
static int static_condensation_cell(int ni, int nf, const double *A,
                                    const double *b, double *S, double *g,
                                    double *work, int *ipiv) {
  int n = ni + nf;
  double *A11 = work, *A12 = A11 + (size_t)ni * ni, *A21 = A12 + (size_t)ni * nf,
         *b1 = A21 + (size_t)nf * ni;
  copy_block(A, n, 0, 0, ni, ni, A11);
  copy_block(A, n, 0, ni, ni, nf, A12);
  copy_block(A, n, ni, 0, nf, ni, A21);
  copy_block(A, n, ni, ni, nf, nf, S);
  memcpy(b1, b, sizeof(double) * ni);
  memcpy(g, b + ni, sizeof(double) * nf);
  int info = getrf(ni, A11, ni, ipiv);
  getrs(ni, nf, A11, ni, ipiv, A12, ni);
  gemm_sub(nf, nf, ni, A21, nf, A12, ni, S, nf);
  getrs(ni, 1, A11, ni, ipiv, b1, ni);
  gemv_sub(nf, ni, A21, nf, b1, g);
  return info;
}

int orc_static_condensation(int ncells, int ni, int nf, const double *A,
                            const double *b, double *S, double *g, int *info) {
  int n = ni + nf, bad = 0;
#pragma omp parallel reduction(+ : bad)
  {
    double *work = malloc(sizeof(double) * ((size_t)ni * ni + 2 * (size_t)ni * nf + ni));
    int *ipiv = malloc(sizeof(int) * ni);
#pragma omp for schedule(static)
    for (int c = 0; c < ncells; ++c) {
      int inf = static_condensation_cell(ni, nf, A + (size_t)c * n * n, b + (size_t)c * n,
                                         S + (size_t)c * nf * nf, g + (size_t)c * nf, work, ipiv);
      if (info) info[c] = inf;
      if (inf) ++bad;
    }
    free(work);
    free(ipiv);
  }
  return bad ? 1 : 0;
}

/* BackwardStaticCondensationMap evaluate! (src/BackwardStaticCondensationMap.jl:61-102):
 * b2 = x (:88); b1 -= A12 b2 (gemv, :91); A11 = L11 U11 (getrf, :95, the map
 * refactorises); b1 = A11^{-1} b1 (getrs, :99).  Output u = b1 (the interior
 * block of the re-blocked [b1; x] vector, :133-151). */
static int backward_cell(int ni, int nf, const double *A, const double *b,
                         const double *x, double *u, double *work, int *ipiv) {
  int n = ni + nf;
  double *A11 = work, *A12 = A11 + (size_t)ni * ni;
  copy_block(A, n, 0, 0, ni, ni, A11);
  copy_block(A, n, 0, ni, ni, nf, A12);
  memcpy(u, b, sizeof(double) * ni);
  gemv_sub(ni, nf, A12, ni, x, u);
  int info = getrf(ni, A11, ni, ipiv);
  getrs(ni, 1, A11, ni, ipiv, u, ni);
  return info;
}

int orc_backward_static_condensation(int ncells, int ni, int nf,
                                     const double *A, const double *b,
                                     const double *x, double *u, int *info) {
  int n = ni + nf, bad = 0;
#pragma omp parallel reduction(+ : bad)
  {
    double *work = malloc(sizeof(double) * ((size_t)ni * ni + (size_t)ni * nf));
    int *ipiv = malloc(sizeof(int) * ni);
#pragma omp for schedule(static)
    for (int c = 0; c < ncells; ++c) {
      int inf = backward_cell(ni, nf, A + (size_t)c * n * n, b + (size_t)c * n,
                              x + (size_t)c * nf, u + (size_t)c * ni, work, ipiv);
      if (info) info[c] = inf;
      if (inf) ++bad;
    }
    free(work);
    free(ipiv);
  }
  return bad ? 1 : 0;
}

/* SumFacetsMap (src/SumFacetsMap.jl:19-30): fold the facet blocks with (+). */
int orc_sum_facets(int nfacets, int len, const double *blocks, double *out) {
  if (nfacets < 2) return -1; /* the reference map needs at least two blocks */
  for (int i = 0; i < len; ++i) out[i] = blocks[i] + blocks[len + i];
  for (int f = 2; f < nfacets; ++f)
    for (int i = 0; i < len; ++i) out[i] += blocks[(size_t)f * len + i];
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Assembly and skeleton solve.                                              */
/* ------------------------------------------------------------------------ */

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* Sparsity pattern of Gridap's SparseMatrixAssembler on the skeleton space
 * (src/HybridAffineFEOperators.jl:38-46): every pair of free skeleton DOFs
 * that share a cell, rows = free DOFs, sorted columns.  The cell DOF ids
 * are the cell's facets' DOFs in local facet order
 * (src/HybridAffineFEOperators.jl:424-434).  rowptr==NULL: count only. */
int orc_csr_pattern(int D, int k, int ncells, int nfacets,
                    const int *cell_facets, const int *facet_dofs, int nfree,
                    int64_t *rowptr, int32_t *colind, int64_t *nnz) {
  return orc_csr_pattern_n(D, ipow(k + 1, D - 1), ncells, nfacets, cell_facets, facet_dofs, nfree, rowptr, colind,
                           nnz);
}

int orc_csr_pattern_nl(int nl, int nfd, int ncells, int nfacets, const int *cell_facets, const int *facet_dofs,
                       int nfree, int64_t *rowptr, int32_t *colind, int64_t *nnz);

/* box cells: 2D facets per cell */
int orc_csr_pattern_n(int D, int nfd, int ncells, int nfacets, const int *cell_facets, const int *facet_dofs,
                      int nfree, int64_t *rowptr, int32_t *colind, int64_t *nnz) {
  return orc_csr_pattern_nl(2 * D, nfd, ncells, nfacets, cell_facets, facet_dofs, nfree, rowptr, colind, nnz);
}

/* nl facets per cell (2D for boxes, D + 1 for simplices) */
int orc_csr_pattern_nl(int nl, int nfd, int ncells, int nfacets, const int *cell_facets, const int *facet_dofs,
                       int nfree, int64_t *rowptr, int32_t *colind, int64_t *nnz) {
  /* facet -> cells */
  int *fc = malloc(sizeof(int) * 2 * nfacets);
  for (int f = 0; f < 2 * nfacets; ++f) fc[f] = -1;
  for (int c = 0; c < ncells; ++c)
    for (int lf = 0; lf < nl; ++lf) {
      int f = cell_facets[c * nl + lf];
      if (fc[2 * f] < 0) fc[2 * f] = c;
      else fc[2 * f + 1] = c;
    }
  int *cols = malloc(sizeof(int) * 2 * nl * nfd);
  int64_t total = 0;
  if (rowptr) rowptr[0] = 0;
  /* rows are numbered by free DOF id; gather per row via its facet */
  int *dof_facet = malloc(sizeof(int) * (nfree > 0 ? nfree : 1));
  int *dof_local = malloc(sizeof(int) * (nfree > 0 ? nfree : 1));
  for (int f = 0; f < nfacets; ++f)
    for (int a = 0; a < nfd; ++a) {
      int id = facet_dofs[f * nfd + a];
      if (id >= 0) {
        dof_facet[id] = f;
        dof_local[id] = a;
      }
    }
  for (int r = 0; r < nfree; ++r) {
    int f = dof_facet[r], nc = 0;
    for (int s = 0; s < 2; ++s) {
      int c = fc[2 * f + s];
      if (c < 0) continue;
      for (int lf = 0; lf < nl; ++lf) {
        int g = cell_facets[c * nl + lf];
        for (int bb = 0; bb < nfd; ++bb) {
          int id = facet_dofs[g * nfd + bb];
          if (id >= 0) cols[nc++] = id;
        }
      }
    }
    qsort(cols, nc, sizeof(int), cmp_int);
    int m = 0;
    for (int i = 0; i < nc; ++i)
      if (m == 0 || cols[i] != cols[m - 1]) cols[m++] = cols[i];
    if (colind)
      for (int i = 0; i < m; ++i) colind[total + i] = cols[i];
    total += m;
    if (rowptr) rowptr[r + 1] = total;
  }
  *nnz = total;
  free(fc);
  free(cols);
  free(dof_facet);
  free(dof_local);
  return 0;
}

static int64_t find_col(const int64_t *rowptr, const int32_t *colind, int r, int c) {
  int64_t lo = rowptr[r], hi = rowptr[r + 1] - 1;
  while (lo <= hi) {
    int64_t mid = (lo + hi) / 2;
    if (colind[mid] == c) return mid;
    if (colind[mid] < c) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

/* assemble_matrix_and_vector with the Dirichlet lift of _attach_dirichlet
 * (src/HybridAffineFEOperators.jl:41-46): g_c -= S_c x_D with the Dirichlet
 * values on Dirichlet DOFs and 0 elsewhere, then add free rows/cols, serially
 * in cell order. */
int orc_assemble(int D, int k, int ncells, const int *cell_facets,
                 const int *facet_dofs, int nfree, const double *dir_vals,
                 const double *S, const double *g, const int64_t *rowptr,
                 const int32_t *colind, double *val, double *rhs) {
  return orc_assemble_n(D, ipow(k + 1, D - 1), ncells, cell_facets, facet_dofs, nfree, dir_vals, S, g, rowptr,
                        colind, val, rhs);
}

int orc_assemble_nl(int nl, int nfd, int ncells, const int *cell_facets, const int *facet_dofs, int nfree,
                    const double *dir_vals, const double *S, const double *g, const int64_t *rowptr,
                    const int32_t *colind, double *val, double *rhs);

int orc_assemble_n(int D, int nfd, int ncells, const int *cell_facets, const int *facet_dofs, int nfree,
                   const double *dir_vals, const double *S, const double *g, const int64_t *rowptr,
                   const int32_t *colind, double *val, double *rhs) {
  return orc_assemble_nl(2 * D, nfd, ncells, cell_facets, facet_dofs, nfree, dir_vals, S, g, rowptr, colind, val,
                         rhs);
}

int orc_assemble_nl(int nl, int nfd, int ncells, const int *cell_facets, const int *facet_dofs, int nfree,
                    const double *dir_vals, const double *S, const double *g, const int64_t *rowptr,
                    const int32_t *colind, double *val, double *rhs) {
  int nf = nl * nfd;
  if (nf > 512) return -1;
  memset(val, 0, sizeof(double) * rowptr[nfree]);
  memset(rhs, 0, sizeof(double) * nfree);
  int ids[512];
  double gl[512];
  for (int c = 0; c < ncells; ++c) {
    const double *Sc = S + (size_t)c * nf * nf;
    for (int lf = 0; lf < nl; ++lf)
      for (int a = 0; a < nfd; ++a) ids[lf * nfd + a] = facet_dofs[cell_facets[c * nl + lf] * nfd + a];
    for (int i = 0; i < nf; ++i) gl[i] = g[(size_t)c * nf + i];
    for (int j = 0; j < nf; ++j)
      if (ids[j] < 0) {
        double xd = dir_vals[-1 - ids[j]];
        for (int i = 0; i < nf; ++i) gl[i] -= Sc[i + (size_t)nf * j] * xd;
      }
    for (int i = 0; i < nf; ++i) {
      if (ids[i] < 0) continue;
      rhs[ids[i]] += gl[i];
      for (int j = 0; j < nf; ++j) {
        if (ids[j] < 0) continue;
        int64_t p = find_col(rowptr, colind, ids[i], ids[j]);
        if (p < 0) return -1;
        val[p] += Sc[i + (size_t)nf * j];
      }
    }
  }
  return 0;
}

/* Dense LU solve of the assembled system (stands in for Gridap's sparse
 * direct A\b, src/HybridAffineFEOperators.jl:74, at small sizes). */
int orc_dense_solve(int n, const int64_t *rowptr, const int32_t *colind,
                    const double *val, const double *rhs, double *x) {
  double *M = calloc((size_t)n * n, sizeof(double));
  int *ipiv = malloc(sizeof(int) * (n > 0 ? n : 1));
  if (!M || !ipiv) return -1;
  for (int r = 0; r < n; ++r)
    for (int64_t p = rowptr[r]; p < rowptr[r + 1]; ++p) M[r + (size_t)n * colind[p]] = val[p];
  int info = getrf(n, M, n, ipiv);
  memcpy(x, rhs, sizeof(double) * n);
  if (!info) getrs(n, 1, M, n, ipiv, x, n);
  free(M);
  free(ipiv);
  return info;
}

static void spmv(int n, const int64_t *rowptr, const int32_t *colind,
                 const double *val, const double *x, double *y, double sign) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < n; ++r) {
    double s = 0.0;
    for (int64_t p = rowptr[r]; p < rowptr[r + 1]; ++p) s += val[p] * x[colind[p]];
    y[r] = sign * s;
  }
}

static double dot(int n, const double *a, const double *b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* Block-Jacobi preconditioned CG on (sign*A) x = sign*rhs with bs x bs
 * diagonal blocks (one block per facet).  A stand-in for the reference's
 * sparse direct solve at sizes where a direct factorisation is impractical. */
int orc_pcg(int n, int bs, const int64_t *rowptr, const int32_t *colind,
            const double *val, const double *rhs, double *x, double sign,
            double rtol, int maxit, int *iters, double *relres) {
  if (n % bs) return -1;
  int nb = n / bs;
  double *Binv = malloc(sizeof(double) * (size_t)nb * bs * bs);
  double *r = malloc(sizeof(double) * n), *z = malloc(sizeof(double) * n);
  double *p = malloc(sizeof(double) * n), *Ap = malloc(sizeof(double) * n);
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int blk = 0; blk < nb; ++blk) {
    double M[36 * 36], I[36 * 36];
    for (int i = 0; i < bs; ++i)
      for (int j = 0; j < bs; ++j) {
        int r0 = blk * bs + i, c0 = blk * bs + j;
        double v = 0.0;
        for (int64_t q = rowptr[r0]; q < rowptr[r0 + 1]; ++q)
          if (colind[q] == c0) v = val[q];
        M[i * bs + j] = sign * v;
        I[i * bs + j] = (i == j);
      }
    for (int c = 0; c < bs; ++c) { /* Gauss-Jordan with partial pivoting */
      int pr = c;
      for (int i = c + 1; i < bs; ++i)
        if (fabs(M[i * bs + c]) > fabs(M[pr * bs + c])) pr = i;
      if (M[pr * bs + c] == 0.0) {
        ++bad;
        break;
      }
      for (int j = 0; j < bs; ++j) {
        double t = M[c * bs + j]; M[c * bs + j] = M[pr * bs + j]; M[pr * bs + j] = t;
        t = I[c * bs + j]; I[c * bs + j] = I[pr * bs + j]; I[pr * bs + j] = t;
      }
      double piv = 1.0 / M[c * bs + c];
      for (int j = 0; j < bs; ++j) { M[c * bs + j] *= piv; I[c * bs + j] *= piv; }
      for (int i = 0; i < bs; ++i) {
        if (i == c) continue;
        double f = M[i * bs + c];
        if (f != 0.0)
          for (int j = 0; j < bs; ++j) { M[i * bs + j] -= f * M[c * bs + j]; I[i * bs + j] -= f * I[c * bs + j]; }
      }
    }
    memcpy(&Binv[(size_t)blk * bs * bs], I, sizeof(double) * bs * bs);
  }
  int it = 0;
  double bnorm = sqrt(dot(n, rhs, rhs)), rr = 0.0;
  for (int i = 0; i < n; ++i) { x[i] = 0.0; r[i] = sign * rhs[i]; }
  if (bad || bnorm == 0.0) {
    *iters = 0;
    *relres = 0.0;
    free(Binv); free(r); free(z); free(p); free(Ap);
    return bad ? -2 : 0;
  }
#define PRECOND(dst, src)                                                         \
  _Pragma("omp parallel for schedule(static)") for (int blk = 0; blk < nb; ++blk) \
    for (int i = 0; i < bs; ++i) {                                                \
      double s_ = 0.0;                                                            \
      for (int j = 0; j < bs; ++j) s_ += Binv[((size_t)blk * bs + i) * bs + j] * src[blk * bs + j]; \
      dst[blk * bs + i] = s_;                                                     \
    }
  PRECOND(z, r);
  memcpy(p, z, sizeof(double) * n);
  double rz = dot(n, r, z);
  rr = sqrt(dot(n, r, r));
  while (rr > rtol * bnorm && it < maxit) {
    spmv(n, rowptr, colind, val, p, Ap, sign);
    double alpha = rz / dot(n, p, Ap);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
    PRECOND(z, r);
    double rz1 = dot(n, r, z);
    double beta = rz1 / rz;
    rz = rz1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    rr = sqrt(dot(n, r, r));
    ++it;
  }
#undef PRECOND
  *iters = it;
  *relres = rr / bnorm;
  free(Binv); free(r); free(z); free(p); free(Ap);
  return rr <= rtol * bnorm ? 0 : 1;
}

/* Cell-wise skeleton values lh_K = get_cell_dof_values(lh, dK)
 * (src/HybridAffineFEOperators.jl:113): free values from the solution,
 * Dirichlet values from the trial space. */
int orc_cell_skeleton_values(int D, int k, int ncells, const int *cell_facets,
                             const int *facet_dofs, const double *xfree,
                             const double *dir_vals, double *xcell) {
  return orc_cell_skeleton_values_n(D, ipow(k + 1, D - 1), ncells, cell_facets, facet_dofs, xfree, dir_vals, xcell);
}

int orc_cell_skeleton_values_nl(int nl, int nfd, int ncells, const int *cell_facets, const int *facet_dofs,
                                const double *xfree, const double *dir_vals, double *xcell);

int orc_cell_skeleton_values_n(int D, int nfd, int ncells, const int *cell_facets, const int *facet_dofs,
                               const double *xfree, const double *dir_vals, double *xcell) {
  return orc_cell_skeleton_values_nl(2 * D, nfd, ncells, cell_facets, facet_dofs, xfree, dir_vals, xcell);
}

int orc_cell_skeleton_values_nl(int nl, int nfd, int ncells, const int *cell_facets, const int *facet_dofs,
                                const double *xfree, const double *dir_vals, double *xcell) {
  int nf = nl * nfd;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncells; ++c)
    for (int lf = 0; lf < nl; ++lf)
      for (int a = 0; a < nfd; ++a) {
        int id = facet_dofs[cell_facets[c * nl + lf] * nfd + a];
        xcell[(size_t)c * nf + lf * nfd + a] = id >= 0 ? xfree[id] : dir_vals[-1 - id];
      }
  return 0;
}

/* L2 errors sqrt(sum(int((u-uh).(u-uh))dOmega)) (test/DarcyHDGTests.jl:141-142)
 * for the flux and the pressure; uint holds ni interior values per cell. */
int orc_l2_errors(int D, int k, const int *n, const double *domain,
                  int problem, const double *kappa, const double *uint,
                  double *err_flux, double *err_pres) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  int ncells, nfacets;
  orc_cart_counts(D, n, &ncells, &nfacets);
  double ef = 0.0, ep = 0.0;
#pragma omp parallel for reduction(+ : ef, ep) schedule(static)
  for (int c = 0; c < ncells; ++c) {
    double x0[MAXD], h[MAXD], detJ = 1.0;
    cell_geom(D, n, domain, c, x0, h);
    for (int d = 0; d < D; ++d) detJ *= h[d];
    const double *u = uint + (size_t)c * t.ni;
    double kap = kappa ? kappa[c] : 1.0;
    for (int q = 0; q < t.nqv; ++q) {
      double x[MAXD], p, qe[MAXD], fu[MAXD], g;
      for (int d = 0; d < D; ++d) x[d] = x0[d] + h[d] * t.qv_xi[q * D + d];
      exact(problem, D, x, kap, &p, qe, fu, &g);
      double qh[MAXD] = {0, 0, 0}, ph = 0.0;
      for (int a = 0; a < t.nk; ++a) {
        double v = t.phi[q * t.nk + a];
        for (int d = 0; d < D; ++d) qh[d] += u[d * t.nk + a] * v;
        ph += u[D * t.nk + a] * v;
      }
      double w = t.qv_w[q] * detJ, e2 = 0.0;
      for (int d = 0; d < D; ++d) e2 += (qe[d] - qh[d]) * (qe[d] - qh[d]);
      ef += w * e2;
      ep += w * (p - ph) * (p - ph);
    }
  }
  *err_flux = sqrt(ef);
  *err_pres = sqrt(ep);
  reftab_free(&t);
  return 0;
}

/* What the reference builds once per mesh and space (Skeleton(model), the
 * facet space M with its Dirichlet values, and the sparsity pattern of the
 * skeleton system: src/Skeleton.jl:113-147, src/HybridAffineFEOperators.jl:
 * 152-162,358-439, Gridap's assembler's symbolic pass).  A step
 * (orc_darcy_step) then integrates, condenses, assembles the values, solves
 * and recovers on it. */
struct orc_darcy {
  int D, k, n[MAXD];
  double domain[2 * MAXD];
  int problem;
  int ncells, nfacets, nfree, ndir;
  int *cell_facets, *facet_cells, *isb, *fdofs;
  double *dvals;
  int64_t nnz;
  int64_t *rowptr;
  int32_t *colind;
};

void orc_darcy_free(orc_darcy *h) {
  if (!h) return;
  free(h->cell_facets); free(h->facet_cells); free(h->isb); free(h->fdofs); free(h->dvals);
  free(h->rowptr); free(h->colind);
  free(h);
}

int orc_darcy_setup(int D, int k, const int *n, const double *domain, int problem, orc_darcy **out,
                    int64_t *nnz_out, int *nfree_out) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  orc_darcy *h = calloc(1, sizeof(orc_darcy));
  h->D = D;
  h->k = k;
  h->problem = problem;
  for (int d = 0; d < D; ++d) {
    h->n[d] = n[d];
    h->domain[2 * d] = domain[2 * d];
    h->domain[2 * d + 1] = domain[2 * d + 1];
  }
  orc_cart_counts(D, n, &h->ncells, &h->nfacets);
  int nl = 2 * D, nfd = t.nfd;
  h->cell_facets = malloc(sizeof(int) * h->ncells * nl);
  h->facet_cells = malloc(sizeof(int) * h->nfacets * 2);
  h->isb = malloc(sizeof(int) * h->nfacets);
  h->fdofs = malloc(sizeof(int) * h->nfacets * nfd);
  orc_cart_topology(D, n, h->cell_facets, h->facet_cells, h->isb);
  orc_facet_dofs(D, k, h->nfacets, h->isb, h->fdofs, &h->nfree, &h->ndir);
  h->dvals = malloc(sizeof(double) * (h->ndir > 0 ? h->ndir : 1));
  orc_dirichlet_values(D, k, n, domain, problem, h->nfacets, h->isb, h->fdofs, h->ndir, h->dvals);
  h->rowptr = malloc(sizeof(int64_t) * (h->nfree + 1));
  orc_csr_pattern(D, k, h->ncells, h->nfacets, h->cell_facets, h->fdofs, h->nfree, NULL, NULL, &h->nnz);
  h->colind = malloc(sizeof(int32_t) * (h->nnz > 0 ? h->nnz : 1));
  orc_csr_pattern(D, k, h->ncells, h->nfacets, h->cell_facets, h->fdofs, h->nfree, h->rowptr, h->colind, &h->nnz);
  reftab_free(&t);
  if (nnz_out) *nnz_out = h->nnz;
  if (nfree_out) *nfree_out = h->nfree;
  *out = h;
  return 0;
}

/* One solve on a set-up mesh (src/HybridAffineFEOperators.jl:10-50 and
 * :72-150): integrate + condense per cell, assemble the values into the
 * pattern, solve the skeleton system (solver 0: dense LU, 1: block-Jacobi PCG
 * on -S), then re-integrate and run BackwardStaticCondensationMap per cell
 * (the reference re-evaluates the weak form and refactorises A_ii in
 * solve!).  Cell matrices are never stored for the whole mesh (one per
 * thread).  uint_out: ncells x ni or NULL; lambda_out: nfree or NULL;
 * val_out (nnz), rhs_out (nfree): the assembled skeleton system or NULL;
 * times_out[5]: integrate+condense, assemble, solve, recover, total (s). */
int orc_darcy_step(orc_darcy *h, double tau, int stab_mode, const double *kappa, int solver, double rtol,
                   int maxit, double *uint_out, double *lambda_out, double *val_out, double *rhs_out,
                   double *times_out, int *iters, double *relres, double *err_flux, double *err_pres) {
  reftab t;
  const int D = h->D, k = h->k, problem = h->problem;
  const int *n = h->n;
  const double *domain = h->domain;
  if (reftab_init(&t, D, k)) return -1;
  double t0 = wtime();
  const int ncells = h->ncells, nfree = h->nfree;
  const int nl = 2 * D, nfd = t.nfd, ni = t.ni, nf = t.nf, N = t.n;
  const int *cell_facets = h->cell_facets, *facet_cells = h->facet_cells, *fdofs = h->fdofs;
  const double *dvals = h->dvals;
  double *S = malloc(sizeof(double) * (size_t)ncells * nf * nf);
  double *g = malloc(sizeof(double) * (size_t)ncells * nf);
  int bad = 0;
  double t1 = wtime();
#pragma omp parallel reduction(+ : bad)
  {
    double *A = malloc(sizeof(double) * (size_t)N * N), *b = malloc(sizeof(double) * N);
    double *work = malloc(sizeof(double) * ((size_t)ni * ni + 2 * (size_t)ni * nf + ni));
    int *ipiv = malloc(sizeof(int) * ni);
#pragma omp for schedule(static)
    for (int c = 0; c < ncells; ++c) {
      integrate_cell(&t, c, n, domain, tau, stab_mode, problem, kappa ? kappa[c] : 1.0,
                     facet_cells, cell_facets, A, b);
      if (static_condensation_cell(ni, nf, A, b, S + (size_t)c * nf * nf, g + (size_t)c * nf, work, ipiv))
        ++bad;
    }
    free(A); free(b); free(work); free(ipiv);
  }
  double t2 = wtime();
  const int64_t nnz = h->nnz;
  double *val = val_out ? val_out : malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
  double *rhs = rhs_out ? rhs_out : malloc(sizeof(double) * (nfree > 0 ? nfree : 1));
  double *lam = malloc(sizeof(double) * (nfree > 0 ? nfree : 1));
  int rc = orc_assemble(D, k, ncells, cell_facets, fdofs, nfree, dvals, S, g, h->rowptr, h->colind, val, rhs);
  double t3 = wtime();
  int it = 0;
  double rel = 0.0;
  if (!rc) {
    if (solver == 0) rc = orc_dense_solve(nfree, h->rowptr, h->colind, val, rhs, lam);
    else rc = orc_pcg(nfree, nfd, h->rowptr, h->colind, val, rhs, lam, -1.0, rtol, maxit, &it, &rel);
  }
  double t4 = wtime();
  double *ucells = uint_out ? uint_out : malloc(sizeof(double) * (size_t)ncells * ni);
#pragma omp parallel reduction(+ : bad)
  {
    double *A = malloc(sizeof(double) * (size_t)N * N), *b = malloc(sizeof(double) * N);
    double *work = malloc(sizeof(double) * ((size_t)ni * ni + (size_t)ni * nf));
    double *xc = malloc(sizeof(double) * nf);
    int *ipiv = malloc(sizeof(int) * ni);
#pragma omp for schedule(static)
    for (int c = 0; c < ncells; ++c) {
      for (int lf = 0; lf < nl; ++lf)
        for (int a = 0; a < nfd; ++a) {
          int id = fdofs[cell_facets[c * nl + lf] * nfd + a];
          xc[lf * nfd + a] = id >= 0 ? lam[id] : dvals[-1 - id];
        }
      integrate_cell(&t, c, n, domain, tau, stab_mode, problem, kappa ? kappa[c] : 1.0,
                     facet_cells, cell_facets, A, b);
      if (backward_cell(ni, nf, A, b, xc, ucells + (size_t)c * ni, work, ipiv)) ++bad;
    }
    free(A); free(b); free(work); free(xc); free(ipiv);
  }
  double t5 = wtime();
  if (times_out) {
    times_out[0] = t2 - t1;
    times_out[1] = t3 - t2;
    times_out[2] = t4 - t3;
    times_out[3] = t5 - t4;
    times_out[4] = t5 - t0;
  }
  if (iters) *iters = it;
  if (relres) *relres = rel;
  if (err_flux && err_pres) orc_l2_errors(D, k, n, domain, problem, kappa, ucells, err_flux, err_pres);
  if (lambda_out) memcpy(lambda_out, lam, sizeof(double) * nfree);
  if (!uint_out) free(ucells);
  if (!val_out) free(val);
  if (!rhs_out) free(rhs);
  free(S); free(g); free(lam);
  reftab_free(&t);
  if (bad) return 2;
  return rc;
}

/* Whole path as the reference runs it: orc_darcy_setup + orc_darcy_step;
 * times_out[4] (total) includes the set-up. */
int orc_solve_darcy(int D, int k, const int *n, const double *domain,
                    double tau, int stab_mode, int problem, const double *kappa,
                    int solver, double rtol, int maxit, double *uint_out,
                    double *lambda_out, double *times_out, int *iters,
                    double *relres, double *err_flux, double *err_pres) {
  double t0 = wtime();
  orc_darcy *h = NULL;
  if (orc_darcy_setup(D, k, n, domain, problem, &h, NULL, NULL)) return -1;
  int rc = orc_darcy_step(h, tau, stab_mode, kappa, solver, rtol, maxit, uint_out, lambda_out, NULL, NULL,
                          times_out, iters, relres, err_flux, err_pres);
  if (times_out) times_out[4] = wtime() - t0;
  orc_darcy_free(h);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Linear elasticity HDG (test/LinearElasticityHDGTests.jl:140-150 with the  */
/* compliance of :15-38), without the P_m bulk-to-skeleton projection (the    */
/* reference's bulk_to_skeleton_projection=false).  Spaces: symmetric stress */
/* Q_k (D(D+1)/2 components), displacement Q_k (D components), displacement  */
/* trace Q_k on facets (D components, Dirichlet on the boundary); per-cell   */
/* Poisson ratio nu, Young's modulus E.  Vector/tensor DOFs are component-   */
/* major, tensor components in upper-triangle order                          */
/* (src/tmp_fixes_symmetric_valued_lagrangian_reffes.jl:104-125).            */
/* ------------------------------------------------------------------------ */

enum { EPROB_LINEAR = 0, EPROB_SMOOTH = 1 };

static int sym_ncomp(int D) { return D * (D + 1) / 2; }

static void sym_pair(int D, int c, int *i, int *j) {
  static const int p2[3][2] = {{0, 0}, {0, 1}, {1, 1}};
  static const int p3[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
  *i = D == 2 ? p2[c][0] : p3[c][0];
  *j = D == 2 ? p2[c][1] : p3[c][1];
}

/* entry (r, s) of the symmetric unit tensor of component c */
static double sym_unit(int D, int c, int r, int s) {
  int i, j;
  sym_pair(D, c, &i, &j);
  return ((r == i && s == j) || (r == j && s == i)) ? 1.0 : 0.0;
}

/* Displacement u, gradient gu[i][j] = du_i/dx_j and Hessian hu[i][j][k].
 * EPROB_LINEAR: u = (x+2y, 2x+y) (test/LinearElasticityHDGTests.jl:48-50) and
 * (x+2y, 2x+y+z, y+3z) in 3D; EPROB_SMOOTH: u = (10 sin(pi x)(1-x)(y-y^2)(1-y/2), 0)
 * (:52-57) in 2D and (sin pi x, cos pi y, xyz) in 3D. */
static void elast_exact(int problem, int D, const double *x, double *u, double gu[3][3], double hu[3][3][3]) {
  const double pi = 3.14159265358979323846;
  memset(u, 0, sizeof(double) * 3);
  memset(gu, 0, sizeof(double) * 9);
  memset(hu, 0, sizeof(double) * 27);
  if (problem == EPROB_LINEAR) {
    if (D == 2) {
      u[0] = x[0] + 2 * x[1];
      u[1] = 2 * x[0] + x[1];
      gu[0][0] = 1; gu[0][1] = 2; gu[1][0] = 2; gu[1][1] = 1;
    } else {
      u[0] = x[0] + 2 * x[1];
      u[1] = 2 * x[0] + x[1] + x[2];
      u[2] = x[1] + 3 * x[2];
      gu[0][0] = 1; gu[0][1] = 2; gu[1][0] = 2; gu[1][1] = 1; gu[1][2] = 1; gu[2][1] = 1; gu[2][2] = 3;
    }
  } else if (D == 2) {
    const double X = x[0], Y = x[1];
    const double A = sin(pi * X) * (1 - X), dA = pi * cos(pi * X) * (1 - X) - sin(pi * X),
                 ddA = -pi * pi * sin(pi * X) * (1 - X) - 2 * pi * cos(pi * X);
    const double B = Y - 1.5 * Y * Y + 0.5 * Y * Y * Y, dB = 1 - 3 * Y + 1.5 * Y * Y, ddB = -3 + 3 * Y;
    u[0] = 10 * A * B;
    gu[0][0] = 10 * dA * B;
    gu[0][1] = 10 * A * dB;
    hu[0][0][0] = 10 * ddA * B;
    hu[0][0][1] = hu[0][1][0] = 10 * dA * dB;
    hu[0][1][1] = 10 * A * ddB;
  } else {
    const double X = x[0], Y = x[1], Z = x[2];
    u[0] = sin(pi * X);
    u[1] = cos(pi * Y);
    u[2] = X * Y * Z;
    gu[0][0] = pi * cos(pi * X);
    gu[1][1] = -pi * sin(pi * Y);
    gu[2][0] = Y * Z; gu[2][1] = X * Z; gu[2][2] = X * Y;
    hu[0][0][0] = -pi * pi * sin(pi * X);
    hu[1][1][1] = -pi * pi * cos(pi * Y);
    hu[2][0][1] = hu[2][1][0] = Z;
    hu[2][0][2] = hu[2][2][0] = Y;
    hu[2][1][2] = hu[2][2][1] = X;
  }
}

/* sigma = A^{-1} eps for A(s) = (1+nu)/E s - nu/E tr(s) I (:15-38):
 * sigma = 2 mu eps + lam tr(eps) I, mu = E/(2(1+nu)), lam = nu E/((1+nu)(1+nu-D nu)) */
static void elast_lame(int D, double E, double nu, double *mu, double *lam) {
  *mu = E / (2.0 * (1.0 + nu));
  *lam = nu * E / ((1.0 + nu) * (1.0 + nu - D * nu));
}

static void elast_sigma(int D, double E, double nu, double gu[3][3], double sig[3][3]) {
  double mu, lam, tr = 0.0;
  elast_lame(D, E, nu, &mu, &lam);
  for (int d = 0; d < D; ++d) tr += gu[d][d];
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) sig[i][j] = mu * (gu[i][j] + gu[j][i]) + (i == j ? lam * tr : 0.0);
}

/* f = div sigma_exact */
static void elast_force(int D, double E, double nu, double hu[3][3][3], double *f) {
  double mu, lam;
  elast_lame(D, E, nu, &mu, &lam);
  for (int i = 0; i < D; ++i) {
    double v = 0.0;
    for (int j = 0; j < D; ++j) v += mu * (hu[i][j][j] + hu[j][i][j]);
    for (int k2 = 0; k2 < D; ++k2) v += lam * hu[k2][i][k2];
    f[i] = v;
  }
}

int orc_elasticity_sizes(int D, int k, int *ni, int *nf, int *nfd) {
  if (D < 2 || D > 3 || k < 1 || k > MAXK) return -1;
  int nk = ipow(k + 1, D);
  *nfd = D * ipow(k + 1, D - 1);
  *ni = (sym_ncomp(D) + D) * nk;
  *nf = 2 * D * *nfd;
  return 0;
}

/* Cell block of
 *   int( v (.) A(sigma) + (div v).u - w.(div sigma) )dOmega - int((v.n).uhat)d(dK)
 *   + int(tau w.u) - int(tau w.uhat) + int(mu.(sigma.n)) - int(tau mu.u) + int(tau mu.uhat) on dK,
 *   l = int(-w.f)dOmega,
 * DOFs [sigma (nsym x nk) | u (D x nk) | uhat per local facet (D x nfs)],
 * integrated point by point; A column-major. */
static void integrate_cell_elast(const reftab *t, int c, const int *n, const double *domain, double tau, double E,
                                 double nu, int problem, double *A, double *b) {
  const int D = t->D, nk = t->nk, nfs = t->nfd, ns = sym_ncomp(D);
  const int ni = (ns + D) * nk, nfd = D * nfs, N = ni + 2 * D * nfd;
  const int ou = ns * nk;  /* first displacement DOF */
  double x0[MAXD], h[MAXD];
  cell_geom(D, n, domain, c, x0, h);
  double detJ = 1.0;
  for (int d = 0; d < D; ++d) detJ *= h[d];
  memset(A, 0, sizeof(double) * (size_t)N * N);
  memset(b, 0, sizeof(double) * N);
#define AIJ(i, j) A[(size_t)(i) + (size_t)N * (j)]
  double Cm[6][6];  /* E_c (.) A(E_d) */
  for (int ca = 0; ca < ns; ++ca)
    for (int cb = 0; cb < ns; ++cb) {
      double dd = 0.0, trc = 0.0, trd = 0.0;
      for (int r = 0; r < D; ++r) {
        trc += sym_unit(D, ca, r, r);
        trd += sym_unit(D, cb, r, r);
        for (int s2 = 0; s2 < D; ++s2) dd += sym_unit(D, ca, r, s2) * sym_unit(D, cb, r, s2);
      }
      Cm[ca][cb] = (1.0 + nu) / E * dd - nu / E * trc * trd;
    }
  for (int q = 0; q < t->nqv; ++q) {
    const double *ph = &t->phi[q * nk];
    const double *dph = &t->dphi[q * nk * D];
    const double wq = t->qv_w[q] * detJ;
    double x[MAXD], u[3], gu[3][3], hu[3][3][3], f[3];
    for (int d = 0; d < D; ++d) x[d] = x0[d] + h[d] * t->qv_xi[q * D + d];
    elast_exact(problem, D, x, u, gu, hu);
    elast_force(D, E, nu, hu, f);
    for (int a = 0; a < nk; ++a) {
      for (int bb = 0; bb < nk; ++bb) {
        const double mm = wq * ph[a] * ph[bb];
        for (int ca = 0; ca < ns; ++ca)
          for (int cb = 0; cb < ns; ++cb) AIJ(ca * nk + a, cb * nk + bb) += Cm[ca][cb] * mm;
        for (int ca = 0; ca < ns; ++ca)
          for (int kk = 0; kk < D; ++kk) {
            double dv = 0.0;  /* ((div (phi_a E_ca)) . e_kk) */
            for (int j = 0; j < D; ++j) dv += sym_unit(D, ca, kk, j) * dph[a * D + j] / h[j];
            /* (div v).u */
            AIJ(ca * nk + a, ou + kk * nk + bb) += wq * dv * ph[bb];
            /* -w.(div sigma): test (kk, bb), trial (ca, a) */
            AIJ(ou + kk * nk + bb, ca * nk + a) -= wq * ph[bb] * dv;
          }
      }
      for (int kk = 0; kk < D; ++kk) b[ou + kk * nk + a] -= wq * ph[a] * f[kk];
    }
  }
  for (int lf = 0; lf < 2 * D; ++lf) {
    const int dn = D - 1 - lf / 2, side = lf % 2;
    double nrm[MAXD] = {0, 0, 0};
    nrm[dn] = side ? 1.0 : -1.0;
    double detF = 1.0;
    for (int d = 0; d < D; ++d)
      if (d != dn) detF *= h[d];
    const int off = ni + lf * nfd;
    for (int q = 0; q < t->nqf; ++q) {
      const double *ph = &t->fphi[(lf * t->nqf + q) * nk];
      const double *mu = &t->mu[q * nfs];
      const double wq = t->qf_w[q] * detF;
      for (int a = 0; a < nk; ++a) {
        for (int m = 0; m < nfs; ++m)
          for (int kk = 0; kk < D; ++kk) {
            const int hu_i = off + kk * nfs + m;
            for (int ca = 0; ca < ns; ++ca) {
              double en = 0.0;  /* ((E_ca) n) . e_kk */
              for (int j = 0; j < D; ++j) en += sym_unit(D, ca, kk, j) * nrm[j];
              if (en == 0.0) continue;
              AIJ(ca * nk + a, hu_i) -= wq * en * ph[a] * mu[m];  /* -(v.n).uhat */
              AIJ(hu_i, ca * nk + a) += wq * en * mu[m] * ph[a];  /* mu.(sigma.n) */
            }
            AIJ(ou + kk * nk + a, hu_i) -= wq * tau * ph[a] * mu[m];  /* -tau w.uhat */
            AIJ(hu_i, ou + kk * nk + a) -= wq * tau * mu[m] * ph[a];  /* -tau mu.u */
          }
        for (int bb = 0; bb < nk; ++bb)
          for (int kk = 0; kk < D; ++kk) AIJ(ou + kk * nk + a, ou + kk * nk + bb) += wq * tau * ph[a] * ph[bb];
      }
      for (int m = 0; m < nfs; ++m)
        for (int m2 = 0; m2 < nfs; ++m2)
          for (int kk = 0; kk < D; ++kk) AIJ(off + kk * nfs + m, off + kk * nfs + m2) += wq * tau * mu[m] * mu[m2];
    }
  }
#undef AIJ
}

int orc_integrate_elasticity(int D, int k, const int *n, const double *domain, double tau, double E,
                             const double *nu, int problem, double *A, double *b) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  int ncells, nfacets, ni, nf, nfd;
  orc_cart_counts(D, n, &ncells, &nfacets);
  orc_elasticity_sizes(D, k, &ni, &nf, &nfd);
  const size_t N = (size_t)ni + nf;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncells; ++c)
    integrate_cell_elast(&t, c, n, domain, tau, E, nu ? nu[c] : 0.3, problem, A + (size_t)c * N * N, b + (size_t)c * N);
  reftab_free(&t);
  return 0;
}

/* TrialFESpace(M, u_exact) (:96-98): nodal interpolation of u at the facet
 * nodes, component-major per facet. */
int orc_dirichlet_values_elasticity(int D, int k, const int *n, const double *domain, int problem, int nfacets,
                                    const int *facet_is_boundary, const int *facet_dofs, int ndir, double *vals) {
  int ncells, nf2;
  orc_cart_counts(D, n, &ncells, &nf2);
  int *cell_facets = malloc(sizeof(int) * ncells * 2 * D);
  int *facet_cells = malloc(sizeof(int) * nfacets * 2);
  int *isb = malloc(sizeof(int) * nfacets);
  orc_cart_topology(D, n, cell_facets, facet_cells, isb);
  int flat[36 * 2];
  orc_lagrange_lattice(D - 1, k, flat);
  const int nfs = ipow(k + 1, D - 1), nfd = D * nfs;
  for (int c = 0; c < ncells; ++c) {
    double x0[MAXD], h[MAXD];
    cell_geom(D, n, domain, c, x0, h);
    for (int lf = 0; lf < 2 * D; ++lf) {
      int f = cell_facets[c * 2 * D + lf];
      if (!facet_is_boundary[f]) continue;
      int dn = D - 1 - lf / 2, side = lf % 2;
      for (int a = 0; a < nfs; ++a) {
        double x[MAXD];
        int j = 0;
        for (int d = 0; d < D; ++d) {
          double xi = (d == dn) ? (double)side : (double)flat[a * (D - 1) + j++] / k;
          x[d] = x0[d] + h[d] * xi;
        }
        double u[3], gu[3][3], hu[3][3][3];
        elast_exact(problem, D, x, u, gu, hu);
        for (int kk = 0; kk < D; ++kk) {
          int id = facet_dofs[f * nfd + kk * nfs + a];
          if (id < 0 && -1 - id < ndir) vals[-1 - id] = u[kk];
        }
      }
    }
  }
  free(cell_facets);
  free(facet_cells);
  free(isb);
  return 0;
}

/* sqrt(sum(int(e_sigma (.) e_sigma))) and sqrt(sum(int(e_u . e_u))) (:153-157) */
int orc_l2_errors_elasticity(int D, int k, const int *n, const double *domain, double E, const double *nu,
                             int problem, const double *uint, double *err_sigma, double *err_u) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  int ncells, nfacets, ni, nf, nfd;
  orc_cart_counts(D, n, &ncells, &nfacets);
  orc_elasticity_sizes(D, k, &ni, &nf, &nfd);
  const int nk = t.nk, ns = sym_ncomp(D), ou = ns * nk;
  double es = 0.0, eu = 0.0;
#pragma omp parallel for reduction(+ : es, eu) schedule(static)
  for (int c = 0; c < ncells; ++c) {
    double x0[MAXD], h[MAXD], detJ = 1.0;
    cell_geom(D, n, domain, c, x0, h);
    for (int d = 0; d < D; ++d) detJ *= h[d];
    const double *v = uint + (size_t)c * ni;
    const double nuc = nu ? nu[c] : 0.3;
    for (int q = 0; q < t.nqv; ++q) {
      double x[MAXD], u[3], gu[3][3], hu[3][3][3], sig[3][3];
      for (int d = 0; d < D; ++d) x[d] = x0[d] + h[d] * t.qv_xi[q * D + d];
      elast_exact(problem, D, x, u, gu, hu);
      elast_sigma(D, E, nuc, gu, sig);
      double sh[6] = {0, 0, 0, 0, 0, 0}, uh[3] = {0, 0, 0};
      for (int a = 0; a < nk; ++a) {
        const double ph = t.phi[q * nk + a];
        for (int cc = 0; cc < ns; ++cc) sh[cc] += v[cc * nk + a] * ph;
        for (int kk = 0; kk < D; ++kk) uh[kk] += v[ou + kk * nk + a] * ph;
      }
      double e2 = 0.0, u2 = 0.0;
      for (int cc = 0; cc < ns; ++cc) {
        int i, j;
        sym_pair(D, cc, &i, &j);
        const double d = sig[i][j] - sh[cc];
        e2 += (i == j ? 1.0 : 2.0) * d * d;
      }
      for (int kk = 0; kk < D; ++kk) u2 += (u[kk] - uh[kk]) * (u[kk] - uh[kk]);
      const double w = t.qv_w[q] * detJ;
      es += w * e2;
      eu += w * u2;
    }
  }
  *err_sigma = sqrt(es);
  *err_u = sqrt(eu);
  reftab_free(&t);
  return 0;
}

/* Whole path as for Darcy (integrate + condense per cell, assemble, skeleton
 * solve: 0 dense LU, 1 block-Jacobi PCG on sign*S; re-integrate + backward map
 * per cell).  sign: the sign that makes the skeleton operator SPD for PCG. */
int orc_solve_elasticity(int D, int k, const int *n, const double *domain, double tau, double E, const double *nu,
                         int problem, int solver, double sign, double rtol, int maxit, double *uint_out,
                         double *lambda_out, int *iters, double *relres, double *err_sigma, double *err_u) {
  reftab t;
  if (reftab_init(&t, D, k)) return -1;
  int ncells, nfacets, nfree, ndir, ni, nf, nfd;
  orc_cart_counts(D, n, &ncells, &nfacets);
  orc_elasticity_sizes(D, k, &ni, &nf, &nfd);
  const int nl = 2 * D, N = ni + nf;
  int *cell_facets = malloc(sizeof(int) * ncells * nl);
  int *facet_cells = malloc(sizeof(int) * nfacets * 2);
  int *isb = malloc(sizeof(int) * nfacets);
  int *fdofs = malloc(sizeof(int) * nfacets * nfd);
  orc_cart_topology(D, n, cell_facets, facet_cells, isb);
  orc_facet_dofs_n(nfd, nfacets, isb, fdofs, &nfree, &ndir);
  double *dvals = malloc(sizeof(double) * (ndir > 0 ? ndir : 1));
  orc_dirichlet_values_elasticity(D, k, n, domain, problem, nfacets, isb, fdofs, ndir, dvals);
  double *S = malloc(sizeof(double) * (size_t)ncells * nf * nf);
  double *g = malloc(sizeof(double) * (size_t)ncells * nf);
  int bad = 0;
#pragma omp parallel reduction(+ : bad)
  {
    double *A = malloc(sizeof(double) * (size_t)N * N), *b = malloc(sizeof(double) * N);
    double *work = malloc(sizeof(double) * ((size_t)ni * ni + 2 * (size_t)ni * nf + ni));
    int *ipiv = malloc(sizeof(int) * ni);
#pragma omp for schedule(static)
    for (int c = 0; c < ncells; ++c) {
      integrate_cell_elast(&t, c, n, domain, tau, E, nu ? nu[c] : 0.3, problem, A, b);
      if (static_condensation_cell(ni, nf, A, b, S + (size_t)c * nf * nf, g + (size_t)c * nf, work, ipiv)) ++bad;
    }
    free(A); free(b); free(work); free(ipiv);
  }
  int64_t nnz;
  int64_t *rowptr = malloc(sizeof(int64_t) * (nfree + 1));
  orc_csr_pattern_n(D, nfd, ncells, nfacets, cell_facets, fdofs, nfree, NULL, NULL, &nnz);
  int32_t *colind = malloc(sizeof(int32_t) * (nnz > 0 ? nnz : 1));
  double *val = malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
  double *rhs = malloc(sizeof(double) * (nfree > 0 ? nfree : 1));
  double *lam = malloc(sizeof(double) * (nfree > 0 ? nfree : 1));
  orc_csr_pattern_n(D, nfd, ncells, nfacets, cell_facets, fdofs, nfree, rowptr, colind, &nnz);
  int rc = orc_assemble_n(D, nfd, ncells, cell_facets, fdofs, nfree, dvals, S, g, rowptr, colind, val, rhs);
  int it = 0;
  double rel = 0.0;
  if (!rc) {
    if (solver == 0) rc = orc_dense_solve(nfree, rowptr, colind, val, rhs, lam);
    else rc = orc_pcg(nfree, nfd, rowptr, colind, val, rhs, lam, sign, rtol, maxit, &it, &rel);
  }
  double *ucells = uint_out ? uint_out : malloc(sizeof(double) * (size_t)ncells * ni);
#pragma omp parallel reduction(+ : bad)
  {
    double *A = malloc(sizeof(double) * (size_t)N * N), *b = malloc(sizeof(double) * N);
    double *work = malloc(sizeof(double) * ((size_t)ni * ni + (size_t)ni * nf));
    double *xc = malloc(sizeof(double) * nf);
    int *ipiv = malloc(sizeof(int) * ni);
#pragma omp for schedule(static)
    for (int c = 0; c < ncells; ++c) {
      for (int lf = 0; lf < nl; ++lf)
        for (int a = 0; a < nfd; ++a) {
          int id = fdofs[cell_facets[c * nl + lf] * nfd + a];
          xc[lf * nfd + a] = id >= 0 ? lam[id] : dvals[-1 - id];
        }
      integrate_cell_elast(&t, c, n, domain, tau, E, nu ? nu[c] : 0.3, problem, A, b);
      if (backward_cell(ni, nf, A, b, xc, ucells + (size_t)c * ni, work, ipiv)) ++bad;
    }
    free(A); free(b); free(work); free(xc); free(ipiv);
  }
  if (iters) *iters = it;
  if (relres) *relres = rel;
  if (err_sigma && err_u) orc_l2_errors_elasticity(D, k, n, domain, E, nu, problem, ucells, err_sigma, err_u);
  if (lambda_out) memcpy(lambda_out, lam, sizeof(double) * nfree);
  if (!uint_out) free(ucells);
  free(cell_facets); free(facet_cells); free(isb); free(fdofs); free(dvals);
  free(S); free(g); free(rowptr); free(colind); free(val); free(rhs); free(lam);
  reftab_free(&t);
  if (bad) return 2;
  return rc;
}


/* ------------------------------------------------------------------------ */
/* General spaces.  Each field has its own polynomial space and order, as    */
/* the reference's tests choose them with ReferenceFE(lagrangian, T, order;  */
/* space=:P) (test/DarcyHDGTests.jl:34-36 flux P_k, pressure P_{k-1}, trace   */
/* P_k; test/LinearElasticityHDGTests.jl:88-93 stress P_k, displacement      */
/* P_{k+1}, trace P_k).  space Q: tensor Lagrange of order k in Gridap's node */
/* order; space P: total degree <= k, Lagrange at the simplex lattice points */
/* x = i/k (the constant for k = 0).  The interior bases only change the     */
/* interior DOF values, not the skeleton system (a Schur complement does not */
/* depend on the interior basis) nor the L2 errors the reference's tests     */
/* check.  Box cells of a Cartesian mesh; everything integrated point by     */
/* point.  spaces[7] = {kindA, kA, kindB, kB, kindT, kT, pm}: A the first    */
/* bulk field (Darcy flux / elasticity stress), B the second (pressure /     */
/* displacement), T the trace; pm = 1 projects the displacement onto the     */
/* trace space in the tau terms (P_m, src/GridapAPIExtensions.jl:453-500,    */
/* test/P_m.jl:4-22, used at test/LinearElasticityHDGTests.jl:134-150).      */
/* ------------------------------------------------------------------------ */

enum { GS_PHYS_DARCY = 0, GS_PHYS_ELAST = 1, GS_Q = 0, GS_P = 1, GS_RT = 2 };

typedef struct {
  int d, kind, k, nb;
  int aniso, ko[3]; /* tensor Lagrange with order ko[e] along dimension e */
  int *lat;      /* Q: nb x d lattice indices */
  int *mono;     /* P: nb x d exponents */
  double *coef;  /* P: nb x nb, phi_a = sum_m coef[a nb + m] x^mono_m */
  double *nodes; /* nb x d */
} obasis;

static void obasis_free(obasis *b) {
  free(b->lat);
  free(b->mono);
  free(b->coef);
  free(b->nodes);
  memset(b, 0, sizeof(*b));
}

/* dense inverse (row-major, in place) by Gauss-Jordan with partial pivoting */
static int dense_inverse(int n, double *A) {
  double *I = calloc((size_t)n * n, sizeof(double));
  for (int i = 0; i < n; ++i) I[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int pr = c;
    for (int i = c + 1; i < n; ++i)
      if (fabs(A[i * n + c]) > fabs(A[pr * n + c])) pr = i;
    if (!(fabs(A[pr * n + c]) > 0.0)) {
      free(I);
      return -1;
    }
    for (int j = 0; j < n; ++j) {
      double t = A[c * n + j]; A[c * n + j] = A[pr * n + j]; A[pr * n + j] = t;
      t = I[c * n + j]; I[c * n + j] = I[pr * n + j]; I[pr * n + j] = t;
    }
    const double piv = A[c * n + c];
    for (int j = 0; j < n; ++j) {
      A[c * n + j] /= piv;
      I[c * n + j] /= piv;
    }
    for (int i = 0; i < n; ++i) {
      if (i == c) continue;
      const double f = A[i * n + c];
      if (f != 0.0)
        for (int j = 0; j < n; ++j) {
          A[i * n + j] -= f * A[c * n + j];
          I[i * n + j] -= f * I[c * n + j];
        }
    }
  }
  memcpy(A, I, sizeof(double) * n * n);
  free(I);
  return 0;
}

/* tensor Lagrange of order orders[e] along dimension e (nodes i/m, the
 * midpoint for order 0), first dimension fastest */
static int obasis_init_aniso(obasis *b, int d, const int *orders) {
  memset(b, 0, sizeof(*b));
  b->d = d;
  b->kind = GS_Q;
  b->aniso = 1;
  if (d < 1 || d > 3) return -1;
  b->nb = 1;
  for (int e = 0; e < d; ++e) {
    if (orders[e] < 0 || orders[e] > 4) return -1;
    b->ko[e] = orders[e];
    if (orders[e] > b->k) b->k = orders[e];
    b->nb *= orders[e] + 1;
  }
  b->lat = malloc(sizeof(int) * b->nb * d);
  b->nodes = malloc(sizeof(double) * b->nb * d);
  for (int a = 0; a < b->nb; ++a) {
    int r = a;
    for (int e = 0; e < d; ++e) {
      const int i = r % (b->ko[e] + 1);
      r /= b->ko[e] + 1;
      b->lat[a * d + e] = i;
      b->nodes[a * d + e] = b->ko[e] == 0 ? 0.5 : (double)i / b->ko[e];
    }
  }
  return 0;
}

static int obasis_init(obasis *b, int d, int kind, int k) {
  memset(b, 0, sizeof(*b));
  b->d = d;
  b->kind = kind;
  b->k = k;
  if (d < 1 || d > 3 || k < 0 || k > 4) return -1;
  if (kind == GS_Q && k == 0) {
    const int zero[3] = {0, 0, 0};
    return obasis_init_aniso(b, d, zero);
  }
  if (kind == GS_Q) {
    b->nb = ipow(k + 1, d);
    b->lat = malloc(sizeof(int) * b->nb * d);
    orc_lagrange_lattice(d, k, b->lat);
    b->nodes = malloc(sizeof(double) * b->nb * d);
    for (int i = 0; i < b->nb * d; ++i) b->nodes[i] = (double)b->lat[i] / k;
    return 0;
  }
  if (kind != GS_P) return -1;
  int cnt = 0, tot = ipow(k + 1, d);
  b->mono = malloc(sizeof(int) * tot * d);
  for (int a = 0; a < tot; ++a) {
    int e[3], s = 0, r = a;
    for (int j = 0; j < d; ++j) {
      e[j] = r % (k + 1);
      r /= (k + 1);
      s += e[j];
    }
    if (s <= k) {
      for (int j = 0; j < d; ++j) b->mono[cnt * d + j] = e[j];
      ++cnt;
    }
  }
  b->nb = cnt;
  b->nodes = malloc(sizeof(double) * cnt * d);
  for (int a = 0; a < cnt; ++a)
    for (int j = 0; j < d; ++j) b->nodes[a * d + j] = k == 0 ? 0.5 : (double)b->mono[a * d + j] / k;
  double *V = malloc(sizeof(double) * cnt * cnt);
  for (int r = 0; r < cnt; ++r)
    for (int m = 0; m < cnt; ++m) {
      double v = 1.0;
      for (int j = 0; j < d; ++j) v *= pow(b->nodes[r * d + j], b->mono[m * d + j]);
      V[r * cnt + m] = v;
    }
  if (dense_inverse(cnt, V)) {
    free(V);
    return -1;
  }
  b->coef = malloc(sizeof(double) * cnt * cnt);
  for (int a = 0; a < cnt; ++a)
    for (int m = 0; m < cnt; ++m) b->coef[a * cnt + m] = V[m * cnt + a]; /* V^{-T} */
  free(V);
  return 0;
}

static void obasis_eval(const obasis *b, const double *xi, double *val, double *grad) {
  const int d = b->d, nb = b->nb;
  if (b->aniso) {
    for (int a = 0; a < nb; ++a) {
      double l[3], dl[3];
      for (int e = 0; e < d; ++e) {
        if (b->ko[e] == 0) {
          l[e] = 1.0;
          dl[e] = 0.0;
        } else {
          lag1d(b->ko[e], b->lat[a * d + e], xi[e], &l[e], &dl[e]);
        }
      }
      double v = 1.0;
      for (int e = 0; e < d; ++e) v *= l[e];
      val[a] = v;
      if (grad)
        for (int e = 0; e < d; ++e) {
          double g = dl[e];
          for (int j = 0; j < d; ++j)
            if (j != e) g *= l[j];
          grad[a * d + e] = g;
        }
    }
    return;
  }
  if (b->kind == GS_Q) {
    for (int a = 0; a < nb; ++a) {
      double l[3], dl[3];
      for (int e = 0; e < d; ++e) lag1d(b->k, b->lat[a * d + e], xi[e], &l[e], &dl[e]);
      double v = 1.0;
      for (int e = 0; e < d; ++e) v *= l[e];
      val[a] = v;
      if (grad)
        for (int e = 0; e < d; ++e) {
          double g = dl[e];
          for (int j = 0; j < d; ++j)
            if (j != e) g *= l[j];
          grad[a * d + e] = g;
        }
    }
    return;
  }
  for (int a = 0; a < nb; ++a) {
    val[a] = 0.0;
    if (grad)
      for (int e = 0; e < d; ++e) grad[a * d + e] = 0.0;
  }
  for (int m = 0; m < nb; ++m) {
    double mv = 1.0, md[3];
    for (int j = 0; j < d; ++j) mv *= pow(xi[j], b->mono[m * d + j]);
    for (int e = 0; e < d; ++e) {
      const int pe = b->mono[m * d + e];
      double g = pe == 0 ? 0.0 : pe * pow(xi[e], pe - 1);
      for (int j = 0; j < d; ++j)
        if (j != e) g *= pow(xi[j], b->mono[m * d + j]);
      md[e] = g;
    }
    for (int a = 0; a < nb; ++a) {
      const double c = b->coef[a * nb + m];
      val[a] += c * mv;
      if (grad)
        for (int e = 0; e < d; ++e) grad[a * d + e] += c * md[e];
    }
  }
}

int orc_gs_basis_eval(int d, int kind, int k, int npts, const double *xi, double *val, double *grad) {
  obasis b;
  if (obasis_init(&b, d, kind, k)) return -1;
  for (int p = 0; p < npts; ++p)
    obasis_eval(&b, xi + p * d, val + (size_t)p * b.nb, grad ? grad + (size_t)p * b.nb * d : NULL);
  const int nb = b.nb;
  obasis_free(&b);
  return nb;
}

typedef struct {
  int D, phys, pm;
  obasis A[6], B, T; /* A: one basis per component of the first field (RT_k: different ones) */
  int ncA, ncB, ncT, nA, nB, nT, ni, nf, nfd, n;
  int n1, nqv, nqf;
  double *qv_xi, *qv_w, *qf_w, *qf_s; /* volume points, facet points (nqf x (D-1) parameters) */
} gstab;

static void gstab_free(gstab *g) {
  for (int c = 0; c < 6; ++c) obasis_free(&g->A[c]);
  obasis_free(&g->B);
  obasis_free(&g->T);
  free(g->qv_xi);
  free(g->qv_w);
  free(g->qf_w);
  free(g->qf_s);
}

static int gstab_init(gstab *g, int D, int phys, const int *sp) {
  memset(g, 0, sizeof(*g));
  if (D < 2 || D > 3 || (phys != GS_PHYS_DARCY && phys != GS_PHYS_ELAST)) return -1;
  g->D = D;
  g->phys = phys;
  g->pm = sp[6];
  const int ns = D * (D + 1) / 2;
  g->ncA = phys == GS_PHYS_DARCY ? D : ns;
  int bad = 0;
  for (int c = 0; c < g->ncA; ++c) {
    if (sp[0] == GS_RT) { /* RT_k: component c of order k+1 along c and k across */
      int ord[3];
      for (int e = 0; e < D; ++e) ord[e] = sp[1] + (e == c ? 1 : 0);
      bad |= phys != GS_PHYS_DARCY || obasis_init_aniso(&g->A[c], D, ord);
    } else {
      bad |= obasis_init(&g->A[c], D, sp[0], sp[1]);
    }
  }
  if (bad || obasis_init(&g->B, D, sp[2], sp[3]) || obasis_init(&g->T, D - 1, sp[4], sp[5])) {
    gstab_free(g);
    return -1;
  }
  g->ncB = phys == GS_PHYS_DARCY ? 1 : D;
  g->ncT = phys == GS_PHYS_DARCY ? 1 : D;
  g->nA = g->A[0].nb;
  g->nB = g->B.nb;
  g->nT = g->T.nb;
  g->ni = g->ncA * g->nA + g->ncB * g->nB;
  g->nfd = g->ncT * g->nT;
  g->nf = 2 * D * g->nfd;
  g->n = g->ni + g->nf;
  int kmax = sp[3] > sp[5] ? sp[3] : sp[5];
  for (int c = 0; c < g->ncA; ++c)
    if (g->A[c].k > kmax) kmax = g->A[c].k;
  g->n1 = kmax + 2;
  g->nqv = ipow(g->n1, D);
  g->nqf = ipow(g->n1, D - 1);
  double x1[16], w1[16];
  orc_gauss_legendre01(g->n1, x1, w1);
  g->qv_xi = malloc(sizeof(double) * g->nqv * D);
  g->qv_w = malloc(sizeof(double) * g->nqv);
  for (int q = 0; q < g->nqv; ++q) {
    double w = 1.0;
    for (int d = 0, r = q; d < D; ++d, r /= g->n1) {
      g->qv_xi[q * D + d] = x1[r % g->n1];
      w *= w1[r % g->n1];
    }
    g->qv_w[q] = w;
  }
  g->qf_w = malloc(sizeof(double) * g->nqf);
  g->qf_s = malloc(sizeof(double) * g->nqf * (D - 1));
  for (int q = 0; q < g->nqf; ++q) {
    double w = 1.0;
    for (int d = 0, r = q; d < D - 1; ++d, r /= g->n1) {
      g->qf_s[q * (D - 1) + d] = x1[r % g->n1];
      w *= w1[r % g->n1];
    }
    g->qf_w[q] = w;
  }
  return 0;
}

int orc_gs_sizes(int D, int phys, const int *spaces, int *sizes /* ni, nf, nfd, nA, nB, nT, nqv */) {
  gstab g;
  if (gstab_init(&g, D, phys, spaces)) return -1;
  sizes[0] = g.ni;
  sizes[1] = g.nf;
  sizes[2] = g.nfd;
  sizes[3] = g.nA;
  sizes[4] = g.nB;
  sizes[5] = g.nT;
  sizes[6] = g.nqv;
  gstab_free(&g);
  return 0;
}

/* cell-local coordinates of facet lf's point with parameters s (the
 * non-normal dimensions in increasing order) */
static void facet_point(int D, int lf, const double *s, double *xi) {
  const int dn = D - 1 - lf / 2, side = lf % 2;
  for (int d = 0, j = 0; d < D; ++d) xi[d] = (d == dn) ? (double)side : s[j++];
}

/* P_m on local facet lf: P = (int mu mu^T) \ (int mu phiB^T), nT x nB row-major */
static int gs_pm_matrix(const gstab *g, int lf, double *P) {
  const int D = g->D, nT = g->nT, nB = g->nB;
  double *L = calloc((size_t)nT * nT, sizeof(double)), *mu = malloc(sizeof(double) * nT),
         *ph = malloc(sizeof(double) * nB);
  memset(P, 0, sizeof(double) * nT * nB);
  for (int q = 0; q < g->nqf; ++q) {
    double xi[3];
    facet_point(D, lf, &g->qf_s[q * (D - 1)], xi);
    obasis_eval(&g->T, &g->qf_s[q * (D - 1)], mu, NULL);
    obasis_eval(&g->B, xi, ph, NULL);
    for (int m = 0; m < nT; ++m) {
      for (int m2 = 0; m2 < nT; ++m2) L[m * nT + m2] += g->qf_w[q] * mu[m] * mu[m2];
      for (int b = 0; b < nB; ++b) P[m * nB + b] += g->qf_w[q] * mu[m] * ph[b];
    }
  }
  int rc = dense_inverse(nT, L);
  if (!rc) {
    double *tmp = malloc(sizeof(double) * nT * nB);
    for (int m = 0; m < nT; ++m)
      for (int b = 0; b < nB; ++b) {
        double v = 0.0;
        for (int m2 = 0; m2 < nT; ++m2) v += L[m * nT + m2] * P[m2 * nB + b];
        tmp[m * nB + b] = v;
      }
    memcpy(P, tmp, sizeof(double) * nT * nB);
    free(tmp);
  }
  free(L);
  free(mu);
  free(ph);
  return rc;
}

/* The Darcy HDG form of test/DarcyHDGTests.jl:125-135 (stab 1: tau (n.n_o)
 * terms as written there, 0: tau (p - l)) with flux in A, pressure in B,
 * trace in T; DOFs [flux (D x nA, component-major) | pressure (nB) | trace
 * per local facet (nT)].  The elasticity form of
 * test/LinearElasticityHDGTests.jl:140-150 (compliance :15-38) with stress in
 * A (upper-triangle components), displacement in B, trace in T (D comps),
 * and, when pm, P_m(u) in the tau w.u and tau mu.u terms.  A column-major. */
static void gs_integrate_cell(const gstab *g, int c, const int *n, const double *domain, double tau, int stab,
                              int problem, double coef, double E, const int *facet_cells, const int *cell_facets,
                              double *A, double *b) {
  const int D = g->D, nA = g->nA, nB = g->nB, nT = g->nT, ncA = g->ncA, N = g->n, ni = g->ni;
  const int oB = ncA * nA;
  double x0[MAXD], h[MAXD];
  cell_geom(D, n, domain, c, x0, h);
  double detJ = 1.0;
  for (int d = 0; d < D; ++d) detJ *= h[d];
  memset(A, 0, sizeof(double) * (size_t)N * N);
  memset(b, 0, sizeof(double) * N);
  /* first-field basis values / gradients per component (RT_k: one basis per
   * component); pA, dA: component 0, which every elasticity stress component uses */
  double *pAc = malloc(sizeof(double) * 6 * nA), *dAc = malloc(sizeof(double) * 6 * nA * D);
  double *pA = pAc, *dA = dAc, *pB = malloc(sizeof(double) * nB),
         *dB = malloc(sizeof(double) * nB * D), *mu = malloc(sizeof(double) * nT), *pm = malloc(sizeof(double) * nB),
         *P = malloc(sizeof(double) * nT * nB);
#define AIJ(i, j) A[(size_t)(i) + (size_t)N * (j)]
  const int ns = D * (D + 1) / 2;
  double Cm[6][6];
  if (g->phys == GS_PHYS_ELAST)
    for (int ca = 0; ca < ns; ++ca)
      for (int cb = 0; cb < ns; ++cb) {
        double dd = 0.0, trc = 0.0, trd = 0.0;
        for (int r = 0; r < D; ++r) {
          trc += sym_unit(D, ca, r, r);
          trd += sym_unit(D, cb, r, r);
          for (int s2 = 0; s2 < D; ++s2) dd += sym_unit(D, ca, r, s2) * sym_unit(D, cb, r, s2);
        }
        Cm[ca][cb] = (1.0 + coef) / E * dd - coef / E * trc * trd;
      }
  for (int q = 0; q < g->nqv; ++q) {
    const double *xi = &g->qv_xi[q * D];
    for (int c2 = 0; c2 < g->ncA; ++c2) obasis_eval(&g->A[c2], xi, pAc + c2 * nA, dAc + c2 * nA * D);
    obasis_eval(&g->B, xi, pB, dB);
    const double wq = g->qv_w[q] * detJ;
    double x[MAXD];
    for (int d = 0; d < D; ++d) x[d] = x0[d] + h[d] * xi[d];
    if (g->phys == GS_PHYS_DARCY) {
      double pe, qe[MAXD], fu[MAXD], gg;
      exact(problem, D, x, coef, &pe, qe, fu, &gg);
      for (int a = 0; a < nA; ++a) {
        for (int a2 = 0; a2 < nA; ++a2)
          for (int d = 0; d < D; ++d) AIJ(d * nA + a, d * nA + a2) += wq * pAc[d * nA + a] * pAc[d * nA + a2] / coef;
        for (int bb = 0; bb < nB; ++bb)
          for (int d = 0; d < D; ++d) {
            AIJ(d * nA + a, oB + bb) -= wq * (dAc[(d * nA + a) * D + d] / h[d]) * pB[bb]; /* -(div v) p */
            AIJ(oB + bb, d * nA + a) -= wq * (dB[bb * D + d] / h[d]) * pAc[d * nA + a];   /* -grad(q).u */
          }
        for (int d = 0; d < D; ++d) b[d * nA + a] += wq * pAc[d * nA + a] * fu[d];
      }
      for (int bb = 0; bb < nB; ++bb) b[oB + bb] += wq * pB[bb] * gg;
    } else {
      double u[3], gu[3][3], hu[3][3][3], f[3];
      elast_exact(problem, D, x, u, gu, hu);
      elast_force(D, E, coef, hu, f);
      for (int a = 0; a < nA; ++a) {
        for (int a2 = 0; a2 < nA; ++a2)
          for (int ca = 0; ca < ns; ++ca)
            for (int cb = 0; cb < ns; ++cb) AIJ(ca * nA + a, cb * nA + a2) += Cm[ca][cb] * wq * pA[a] * pA[a2];
        for (int bb = 0; bb < nB; ++bb)
          for (int ca = 0; ca < ns; ++ca)
            for (int kk = 0; kk < D; ++kk) {
              double dv = 0.0; /* (div (phiA_a E_ca)) . e_kk */
              for (int j = 0; j < D; ++j) dv += sym_unit(D, ca, kk, j) * dA[a * D + j] / h[j];
              AIJ(ca * nA + a, oB + kk * nB + bb) += wq * dv * pB[bb]; /* (div v).u */
              AIJ(oB + kk * nB + bb, ca * nA + a) -= wq * pB[bb] * dv; /* -w.(div sigma) */
            }
      }
      for (int bb = 0; bb < nB; ++bb)
        for (int kk = 0; kk < D; ++kk) b[oB + kk * nB + bb] -= wq * pB[bb] * f[kk];
    }
  }
  for (int lf = 0; lf < 2 * D; ++lf) {
    const int dn = D - 1 - lf / 2, side = lf % 2;
    double nrm[MAXD] = {0, 0, 0};
    nrm[dn] = side ? 1.0 : -1.0;
    double detF = 1.0;
    for (int d = 0; d < D; ++d)
      if (d != dn) detF *= h[d];
    const int f = cell_facets[c * 2 * D + lf];
    double s = 1.0;
    if (g->phys == GS_PHYS_DARCY && stab == 1) s = (facet_cells[2 * f] == c) ? 1.0 : -1.0;
    const int off = ni + lf * g->nfd;
    if (g->phys == GS_PHYS_ELAST && g->pm) gs_pm_matrix(g, lf, P);
    for (int q = 0; q < g->nqf; ++q) {
      double xi[3];
      facet_point(D, lf, &g->qf_s[q * (D - 1)], xi);
      for (int c2 = 0; c2 < g->ncA; ++c2) obasis_eval(&g->A[c2], xi, pAc + c2 * nA, NULL);
      obasis_eval(&g->B, xi, pB, NULL);
      obasis_eval(&g->T, &g->qf_s[q * (D - 1)], mu, NULL);
      const double wq = g->qf_w[q] * detF;
      if (g->phys == GS_PHYS_DARCY) {
        for (int a = 0; a < nA; ++a)
          for (int m = 0; m < nT; ++m)
            for (int d = 0; d < D; ++d) {
              const double v = wq * pAc[d * nA + a] * nrm[d] * mu[m];
              AIJ(d * nA + a, off + m) += v; /* (v.n) l */
              AIJ(off + m, d * nA + a) += v; /* m (u.n) */
            }
        for (int bb = 0; bb < nB; ++bb) {
          for (int m = 0; m < nT; ++m) {
            AIJ(oB + bb, off + m) -= wq * tau * s * pB[bb] * mu[m]; /* -tau q l (n.no) */
            AIJ(off + m, oB + bb) += wq * tau * s * mu[m] * pB[bb]; /* tau m p (n.no) */
          }
          for (int a = 0; a < nA; ++a)
            for (int d = 0; d < D; ++d) AIJ(oB + bb, d * nA + a) += wq * pB[bb] * pAc[d * nA + a] * nrm[d]; /* q (u.n) */
          for (int b2 = 0; b2 < nB; ++b2) AIJ(oB + bb, oB + b2) += wq * tau * s * pB[bb] * pB[b2];
        }
        for (int m = 0; m < nT; ++m)
          for (int m2 = 0; m2 < nT; ++m2) AIJ(off + m, off + m2) -= wq * tau * s * mu[m] * mu[m2];
      } else {
        /* the trial displacement on the facet: u, or P_m(u) = sum_m P[m][b] mu_m */
        for (int bb = 0; bb < nB; ++bb) {
          if (g->pm) {
            double v = 0.0;
            for (int m = 0; m < nT; ++m) v += P[m * nB + bb] * mu[m];
            pm[bb] = v;
          } else {
            pm[bb] = pB[bb];
          }
        }
        for (int m = 0; m < nT; ++m)
          for (int kk = 0; kk < D; ++kk) {
            const int hu_i = off + kk * nT + m;
            for (int a = 0; a < nA; ++a)
              for (int ca = 0; ca < ns; ++ca) {
                double en = 0.0; /* ((E_ca) n) . e_kk */
                for (int j = 0; j < D; ++j) en += sym_unit(D, ca, kk, j) * nrm[j];
                if (en == 0.0) continue;
                AIJ(ca * nA + a, hu_i) -= wq * en * pA[a] * mu[m]; /* -(v.n).uhat */
                AIJ(hu_i, ca * nA + a) += wq * en * mu[m] * pA[a]; /* mu.(sigma.n) */
              }
            for (int bb = 0; bb < nB; ++bb) {
              AIJ(oB + kk * nB + bb, hu_i) -= wq * tau * pB[bb] * mu[m]; /* -tau w.uhat */
              AIJ(hu_i, oB + kk * nB + bb) -= wq * tau * mu[m] * pm[bb]; /* -tau mu.P(u) */
            }
            for (int m2 = 0; m2 < nT; ++m2) AIJ(hu_i, off + kk * nT + m2) += wq * tau * mu[m] * mu[m2]; /* tau mu.uhat */
          }
        for (int bb = 0; bb < nB; ++bb)
          for (int b2 = 0; b2 < nB; ++b2)
            for (int kk = 0; kk < D; ++kk) AIJ(oB + kk * nB + bb, oB + kk * nB + b2) += wq * tau * pB[bb] * pm[b2]; /* tau w.P(u) */
      }
    }
  }
#undef AIJ
  free(pAc); free(dAc); free(pB); free(dB); free(mu); free(pm); free(P);
}

int orc_gs_integrate(int D, int phys, const int *spaces, const int *n, const double *domain, double tau, int stab,
                     int problem, const double *coef, double E, double *A, double *b) {
  gstab g;
  if (gstab_init(&g, D, phys, spaces)) return -1;
  int ncells, nfacets;
  orc_cart_counts(D, n, &ncells, &nfacets);
  int *cell_facets = malloc(sizeof(int) * ncells * 2 * D), *facet_cells = malloc(sizeof(int) * nfacets * 2),
      *isb = malloc(sizeof(int) * nfacets);
  orc_cart_topology(D, n, cell_facets, facet_cells, isb);
  const size_t N = (size_t)g.n;
  const double dflt = phys == GS_PHYS_DARCY ? 1.0 : 0.3;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncells; ++c)
    gs_integrate_cell(&g, c, n, domain, tau, stab, problem, coef ? coef[c] : dflt, E, facet_cells, cell_facets,
                      A + (size_t)c * N * N, b + (size_t)c * N);
  free(cell_facets); free(facet_cells); free(isb);
  gstab_free(&g);
  return 0;
}

/* TrialFESpace(M, p) / TrialFESpace(M, u_exact): the exact trace at the
 * trace basis' nodes on every Dirichlet facet, component-major per facet. */
int orc_gs_dirichlet_values(int D, int phys, const int *spaces, const int *n, const double *domain, int problem,
                            const int *facet_dofs, int ndir, double *vals) {
  gstab g;
  if (gstab_init(&g, D, phys, spaces)) return -1;
  int ncells, nfacets;
  orc_cart_counts(D, n, &ncells, &nfacets);
  int *cell_facets = malloc(sizeof(int) * ncells * 2 * D), *facet_cells = malloc(sizeof(int) * nfacets * 2),
      *isb = malloc(sizeof(int) * nfacets);
  orc_cart_topology(D, n, cell_facets, facet_cells, isb);
  for (int c = 0; c < ncells; ++c) {
    double x0[MAXD], h[MAXD];
    cell_geom(D, n, domain, c, x0, h);
    for (int lf = 0; lf < 2 * D; ++lf) {
      const int f = cell_facets[c * 2 * D + lf];
      if (!isb[f]) continue;
      for (int m = 0; m < g.nT; ++m) {
        double xi[3], x[3];
        facet_point(D, lf, &g.T.nodes[m * (D - 1)], xi);
        for (int d = 0; d < D; ++d) x[d] = x0[d] + h[d] * xi[d];
        for (int kk = 0; kk < g.ncT; ++kk) {
          double v;
          if (phys == GS_PHYS_DARCY) {
            double p, qv[3], fu[3], gg;
            exact(problem, D, x, 1.0, &p, qv, fu, &gg);
            v = p;
          } else {
            double u[3], gu[3][3], hu[3][3][3];
            elast_exact(problem, D, x, u, gu, hu);
            v = u[kk];
          }
          const int id = facet_dofs[f * g.nfd + kk * g.nT + m];
          if (id < 0 && -1 - id < ndir) vals[-1 - id] = v;
        }
      }
    }
  }
  free(cell_facets); free(facet_cells); free(isb);
  gstab_free(&g);
  return 0;
}

/* L2 errors of the two bulk fields against the exact solution:
 * Darcy (flux, pressure), elasticity (stress, displacement). */
int orc_gs_l2_errors(int D, int phys, const int *spaces, const int *n, const double *domain, int problem,
                     const double *coef, double E, const double *uint, double *err1, double *err2) {
  gstab g;
  if (gstab_init(&g, D, phys, spaces)) return -1;
  int ncells, nfacets;
  orc_cart_counts(D, n, &ncells, &nfacets);
  const int nA = g.nA, nB = g.nB, ns = D * (D + 1) / 2, oB = g.ncA * nA;
  double e1 = 0.0, e2 = 0.0;
#pragma omp parallel for reduction(+ : e1, e2) schedule(static)
  for (int c = 0; c < ncells; ++c) {
    double x0[MAXD], h[MAXD], detJ = 1.0;
    cell_geom(D, n, domain, c, x0, h);
    for (int d = 0; d < D; ++d) detJ *= h[d];
    const double *u = uint + (size_t)c * g.ni;
    const double cf = coef ? coef[c] : (phys == GS_PHYS_DARCY ? 1.0 : 0.3);
    double pAc[6 * 216], pB[216];
    const double *pA = pAc;
    for (int q = 0; q < g.nqv; ++q) {
      const double *xi = &g.qv_xi[q * D];
      for (int c2 = 0; c2 < g.ncA; ++c2) obasis_eval(&g.A[c2], xi, pAc + c2 * nA, NULL);
      obasis_eval(&g.B, xi, pB, NULL);
      double x[MAXD];
      for (int d = 0; d < D; ++d) x[d] = x0[d] + h[d] * xi[d];
      const double w = g.qv_w[q] * detJ;
      if (phys == GS_PHYS_DARCY) {
        double p, qe[MAXD], fu[MAXD], gg;
        exact(problem, D, x, cf, &p, qe, fu, &gg);
        double s1 = 0.0, ph = 0.0;
        for (int d = 0; d < D; ++d) {
          double qh = 0.0;
          for (int a = 0; a < nA; ++a) qh += u[d * nA + a] * pAc[d * nA + a];
          s1 += (qe[d] - qh) * (qe[d] - qh);
        }
        for (int bb = 0; bb < nB; ++bb) ph += u[oB + bb] * pB[bb];
        e1 += w * s1;
        e2 += w * (p - ph) * (p - ph);
      } else {
        double ue[3], gu[3][3], hu[3][3][3], sig[3][3];
        elast_exact(problem, D, x, ue, gu, hu);
        elast_sigma(D, E, cf, gu, sig);
        double s1 = 0.0, s2 = 0.0;
        for (int ca = 0; ca < ns; ++ca) {
          int i, j;
          sym_pair(D, ca, &i, &j);
          double sh = 0.0;
          for (int a = 0; a < nA; ++a) sh += u[ca * nA + a] * pA[a];
          const double e = sig[i][j] - sh;
          s1 += (i == j ? 1.0 : 2.0) * e * e;
        }
        for (int kk = 0; kk < D; ++kk) {
          double uh = 0.0;
          for (int bb = 0; bb < nB; ++bb) uh += u[oB + kk * nB + bb] * pB[bb];
          s2 += (ue[kk] - uh) * (ue[kk] - uh);
        }
        e1 += w * s1;
        e2 += w * s2;
      }
    }
  }
  *err1 = sqrt(e1);
  *err2 = sqrt(e2);
  gstab_free(&g);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Simplex meshes: the Darcy HDG form on triangles and tetrahedra with P_k   */
/* fields, as test/DarcyHDGTests.jl:174-177 runs it on simplexify(...) of    */
/* the Cartesian model.  The reference simplex has vertices v_0 = 0 and      */
/* v_j = e_{j-1}; local facet lf is the face opposite vertex D - lf, its     */
/* vertices in increasing local order (the lexicographic face order of a     */
/* simplex polytope).  A cell's vertices are listed in increasing global     */
/* order, so a facet's parametrisation (its vertices in increasing global    */
/* order) is the same from both of its cells and the trace basis needs no    */
/* permutation (the reference handles general vertex orders through the     */
/* face vertex permutations of src/Skeleton.jl:282-342).  Cell geometry is   */
/* given as x = x0 + J xi; gradients go through J^{-T}, normals are          */
/* J^{-T} n_ref / |J^{-T} n_ref|, and the facet measure is |det J|           */
/* |J^{-T} n_ref| times the reference face's measure over the unit           */
/* (D-1)-simplex (sqrt(D) for the face opposite v_0, 1 for the others).      */
/* ------------------------------------------------------------------------ */

typedef struct {
  int D, kA, kB, kT, nA, nB, nT, ni, nfd, nf, n, n1, nqv, nqf;
  obasis A, B, T;
  double *qv_xi, *qv_w, *qf_s, *qf_w;
} sxtab;

static void sxtab_free(sxtab *t) {
  obasis_free(&t->A);
  obasis_free(&t->B);
  obasis_free(&t->T);
  free(t->qv_xi); free(t->qv_w); free(t->qf_s); free(t->qf_w);
}

/* collapsed (Duffy) Gauss rule on the unit d-simplex, n1 points per direction:
 * xi_1 = u_1, xi_2 = u_2 (1 - u_1), xi_3 = u_3 (1 - u_1)(1 - u_2) */
static int simplex_rule(int d, int n1, double **xi, double **w) {
  double x1[16], w1[16];
  orc_gauss_legendre01(n1, x1, w1);
  const int nq = d == 0 ? 1 : ipow(n1, d);
  *xi = malloc(sizeof(double) * nq * (d > 0 ? d : 1));
  *w = malloc(sizeof(double) * nq);
  for (int q = 0; q < nq; ++q) {
    double u[3] = {0, 0, 0}, wt = 1.0, scale = 1.0;
    for (int j = 0, r = q; j < d; ++j, r /= n1) {
      u[j] = x1[r % n1];
      wt *= w1[r % n1];
    }
    for (int j = 0; j < d; ++j) {
      (*xi)[q * d + j] = u[j] * scale;
      if (j + 1 < d) {
        wt *= pow(1.0 - u[j], d - 1 - j);
        scale *= 1.0 - u[j];
      }
    }
    (*w)[q] = wt;
  }
  return nq;
}

static int sxtab_init(sxtab *t, int D, const int *sp) {
  memset(t, 0, sizeof(*t));
  if (D < 2 || D > 3 || sp[0] != GS_P || sp[2] != GS_P || sp[4] != GS_P) return -1;
  t->D = D;
  t->kA = sp[1];
  t->kB = sp[3];
  t->kT = sp[5];
  if (obasis_init(&t->A, D, GS_P, sp[1]) || obasis_init(&t->B, D, GS_P, sp[3]) ||
      obasis_init(&t->T, D - 1, GS_P, sp[5])) {
    sxtab_free(t);
    return -1;
  }
  t->nA = t->A.nb;
  t->nB = t->B.nb;
  t->nT = t->T.nb;
  t->ni = D * t->nA + t->nB;
  t->nfd = t->nT;
  t->nf = (D + 1) * t->nfd;
  t->n = t->ni + t->nf;
  int kmax = t->kA > t->kB ? t->kA : t->kB;
  if (t->kT > kmax) kmax = t->kT;
  t->n1 = kmax + 2;
  t->nqv = simplex_rule(D, t->n1, &t->qv_xi, &t->qv_w);
  t->nqf = simplex_rule(D - 1, t->n1, &t->qf_s, &t->qf_w);
  return 0;
}

static void simplex_face_point(int D, int lf, const double *s, double *xi) {
  int fv[3], k = 0;
  const int opp = D - lf;
  for (int v = 0; v <= D; ++v)
    if (v != opp) fv[k++] = v;
  double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int d = 0; d < D; ++d) {
    xi[d] = V[fv[0]][d];
    for (int j = 0; j + 1 < D; ++j) xi[d] += s[j] * (V[fv[j + 1]][d] - V[fv[0]][d]);
  }
}

static void simplex_ref_normal(int D, int lf, double *nh, double *ratio) {
  const int opp = D - lf;
  for (int d = 0; d < D; ++d) nh[d] = 0.0;
  if (opp == 0) {
    for (int d = 0; d < D; ++d) nh[d] = 1.0 / sqrt((double)D);
    *ratio = sqrt((double)D);
  } else {
    nh[opp - 1] = -1.0;
    *ratio = 1.0;
  }
}

/* inverse (row-major Ji[r][c]) and determinant of the D x D column-major J */
static double sx_inverse(int D, const double *Jc, double Ji[3][3]) {
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int c = 0; c < D; ++c)
    for (int r = 0; r < D; ++r) J[r][c] = Jc[c * D + r];
  double det;
  if (D == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
    Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
  } else {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1], c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2],
                 c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    Ji[0][0] = c00 / det; Ji[1][0] = c01 / det; Ji[2][0] = c02 / det;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  }
  return det;
}

int orc_sx_sizes(int D, const int *spaces, int *sizes /* ni, nf, nfd, nA, nB, nT, nqv */) {
  sxtab t;
  if (sxtab_init(&t, D, spaces)) return -1;
  sizes[0] = t.ni; sizes[1] = t.nf; sizes[2] = t.nfd; sizes[3] = t.nA; sizes[4] = t.nB; sizes[5] = t.nT;
  sizes[6] = t.nqv;
  sxtab_free(&t);
  return 0;
}

/* The Darcy HDG cell blocks (the form of test/DarcyHDGTests.jl:125-135 with a
 * per-cell permeability in the flux mass term and the box form's term
 * layout) on simplex cells: origin (ncells x D), jac (ncells x D x D,
 * column-major), sgn (ncells x (D+1): n . n_owner of each local facet),
 * coef (ncells, NULL = 1).  A column-major n x n per cell, b n per cell. */
int orc_sx_integrate(int D, const int *spaces, int ncells, const double *origin, const double *jac,
                     const double *sgn, double tau, int stab, int problem, const double *coef, double *A,
                     double *b) {
  sxtab t;
  if (sxtab_init(&t, D, spaces)) return -1;
  const int nA = t.nA, nB = t.nB, nT = t.nT, N = t.n, ni = t.ni, oB = D * nA;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(| : bad)
  for (int c = 0; c < ncells; ++c) {
    double Ji[3][3];
    const double *Jc = jac + (size_t)c * D * D, *x0 = origin + (size_t)c * D;
    const double det = sx_inverse(D, Jc, Ji), adet = fabs(det);
    const double kap = coef ? coef[c] : 1.0;
    double *Ac = A + (size_t)c * N * N, *bc = b + (size_t)c * N;
    memset(Ac, 0, sizeof(double) * (size_t)N * N);
    memset(bc, 0, sizeof(double) * N);
#define AIJ(i, j) Ac[(size_t)(i) + (size_t)N * (j)]
    double pA[64], dA[64 * 3], gA[64 * 3], pB[64], dB[64 * 3], gB[64 * 3], mu[64];
    if (nA > 64 || nB > 64 || nT > 64) {
      bad |= 1;
      continue;
    }
    for (int q = 0; q < t.nqv; ++q) {
      const double *xi = &t.qv_xi[q * D];
      obasis_eval(&t.A, xi, pA, dA);
      obasis_eval(&t.B, xi, pB, dB);
      for (int a = 0; a < nA; ++a)
        for (int d = 0; d < D; ++d) {
          gA[a * D + d] = 0.0;
          for (int e = 0; e < D; ++e) gA[a * D + d] += Ji[e][d] * dA[a * D + e];
        }
      for (int a = 0; a < nB; ++a)
        for (int d = 0; d < D; ++d) {
          gB[a * D + d] = 0.0;
          for (int e = 0; e < D; ++e) gB[a * D + d] += Ji[e][d] * dB[a * D + e];
        }
      const double wq = t.qv_w[q] * adet;
      double x[3];
      for (int d = 0; d < D; ++d) {
        x[d] = x0[d];
        for (int e = 0; e < D; ++e) x[d] += Jc[e * D + d] * xi[e];
      }
      double pe, qe[3], fu[3], gg;
      exact(problem, D, x, kap, &pe, qe, fu, &gg);
      for (int a = 0; a < nA; ++a) {
        for (int a2 = 0; a2 < nA; ++a2)
          for (int d = 0; d < D; ++d) AIJ(d * nA + a, d * nA + a2) += wq * pA[a] * pA[a2] / kap;
        for (int bb = 0; bb < nB; ++bb)
          for (int d = 0; d < D; ++d) {
            AIJ(d * nA + a, oB + bb) -= wq * gA[a * D + d] * pB[bb]; /* -(div v) p */
            AIJ(oB + bb, d * nA + a) -= wq * gB[bb * D + d] * pA[a]; /* -grad(q).u */
          }
        for (int d = 0; d < D; ++d) bc[d * nA + a] += wq * pA[a] * fu[d];
      }
      for (int bb = 0; bb < nB; ++bb) bc[oB + bb] += wq * pB[bb] * gg;
    }
    for (int lf = 0; lf <= D; ++lf) {
      double nh[3], ratio, v[3] = {0, 0, 0}, nv = 0.0, nrm[3];
      simplex_ref_normal(D, lf, nh, &ratio);
      for (int d = 0; d < D; ++d) {
        for (int e = 0; e < D; ++e) v[d] += Ji[e][d] * nh[e];
        nv += v[d] * v[d];
      }
      nv = sqrt(nv);
      for (int d = 0; d < D; ++d) nrm[d] = v[d] / nv;
      const double area = adet * nv * ratio;
      const double s = stab == 1 ? sgn[(size_t)c * (D + 1) + lf] : 1.0;
      const int off = ni + lf * t.nfd;
      for (int q = 0; q < t.nqf; ++q) {
        double xi[3];
        simplex_face_point(D, lf, &t.qf_s[q * (D - 1)], xi);
        obasis_eval(&t.A, xi, pA, NULL);
        obasis_eval(&t.B, xi, pB, NULL);
        obasis_eval(&t.T, &t.qf_s[q * (D - 1)], mu, NULL);
        const double wq = t.qf_w[q] * area;
        for (int a = 0; a < nA; ++a)
          for (int m = 0; m < nT; ++m)
            for (int d = 0; d < D; ++d) {
              const double vv = wq * pA[a] * nrm[d] * mu[m];
              AIJ(d * nA + a, off + m) += vv; /* (v.n) l */
              AIJ(off + m, d * nA + a) += vv; /* m (u.n) */
            }
        for (int bb = 0; bb < nB; ++bb) {
          for (int m = 0; m < nT; ++m) {
            AIJ(oB + bb, off + m) -= wq * tau * s * pB[bb] * mu[m]; /* -tau q l (n.no) */
            AIJ(off + m, oB + bb) += wq * tau * s * mu[m] * pB[bb]; /* tau m p (n.no) */
          }
          for (int a = 0; a < nA; ++a)
            for (int d = 0; d < D; ++d) AIJ(oB + bb, d * nA + a) += wq * pB[bb] * pA[a] * nrm[d]; /* q (u.n) */
          for (int b2 = 0; b2 < nB; ++b2) AIJ(oB + bb, oB + b2) += wq * tau * s * pB[bb] * pB[b2];
        }
        for (int m = 0; m < nT; ++m)
          for (int m2 = 0; m2 < nT; ++m2) AIJ(off + m, off + m2) -= wq * tau * s * mu[m] * mu[m2];
      }
    }
#undef AIJ
  }
  sxtab_free(&t);
  return bad ? -1 : 0;
}

/* Dirichlet values: the exact pressure at the trace basis' nodes of each
 * boundary facet (its own parametrisation), through the facet's cell
 * (cell_lf[f] = (c, lf) of a cell around facet f). */
int orc_sx_dirichlet_values(int D, const int *spaces, int nfacets, const int *facet_cell_lf, const double *origin,
                            const double *jac, int problem, const int *facet_dofs, int ndir, double *vals) {
  sxtab t;
  if (sxtab_init(&t, D, spaces)) return -1;
  for (int f = 0; f < nfacets; ++f) {
    const int c = facet_cell_lf[2 * f], lf = facet_cell_lf[2 * f + 1];
    for (int m = 0; m < t.nT; ++m) {
      const int id = facet_dofs[f * t.nfd + m];
      if (id >= 0) continue;
      double xi[3], x[3];
      simplex_face_point(D, lf, &t.T.nodes[m * (D - 1)], xi);
      const double *x0 = origin + (size_t)c * D, *Jc = jac + (size_t)c * D * D;
      for (int d = 0; d < D; ++d) {
        x[d] = x0[d];
        for (int e = 0; e < D; ++e) x[d] += Jc[e * D + d] * xi[e];
      }
      double p, qv[3], fu[3], gg;
      exact(problem, D, x, 1.0, &p, qv, fu, &gg);
      if (-1 - id < ndir) vals[-1 - id] = p;
    }
  }
  sxtab_free(&t);
  return 0;
}

int orc_sx_l2_errors(int D, const int *spaces, int ncells, const double *origin, const double *jac, int problem,
                     const double *coef, const double *uint, double *e1, double *e2) {
  sxtab t;
  if (sxtab_init(&t, D, spaces)) return -1;
  const int nA = t.nA, nB = t.nB, ni = t.ni;
  double ef = 0.0, ep = 0.0;
#pragma omp parallel for reduction(+ : ef, ep) schedule(static)
  for (int c = 0; c < ncells; ++c) {
    double Ji[3][3], pA[64], pB[64];
    const double *Jc = jac + (size_t)c * D * D, *x0 = origin + (size_t)c * D;
    const double adet = fabs(sx_inverse(D, Jc, Ji)), kap = coef ? coef[c] : 1.0;
    const double *u = uint + (size_t)c * ni;
    for (int q = 0; q < t.nqv; ++q) {
      const double *xi = &t.qv_xi[q * D];
      obasis_eval(&t.A, xi, pA, NULL);
      obasis_eval(&t.B, xi, pB, NULL);
      double x[3];
      for (int d = 0; d < D; ++d) {
        x[d] = x0[d];
        for (int e = 0; e < D; ++e) x[d] += Jc[e * D + d] * xi[e];
      }
      double p, qe[3], fu[3], gg;
      exact(problem, D, x, kap, &p, qe, fu, &gg);
      const double w = t.qv_w[q] * adet;
      for (int d = 0; d < D; ++d) {
        double qh = 0.0;
        for (int a = 0; a < nA; ++a) qh += u[d * nA + a] * pA[a];
        ef += w * (qe[d] - qh) * (qe[d] - qh);
      }
      double ph = 0.0;
      for (int a = 0; a < nB; ++a) ph += u[D * nA + a] * pB[a];
      ep += w * (p - ph) * (p - ph);
    }
  }
  *e1 = sqrt(ef);
  *e2 = sqrt(ep);
  sxtab_free(&t);
  return 0;
}
