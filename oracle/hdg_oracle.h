/*
 * hdg_oracle.h -- CPU FP64 oracle for the cellwise hybridization hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke()
 * entry point and bench.py's CPU-baseline leg load it.  The GPU product path
 * never links, loads or calls it.
 *
 * It restates, in plain C, what GridapHybrid.jl (Julia, on top of Gridap.jl
 * 0.18.2 "exploring_hybridization" and OpenBLAS/LAPACK) computes on the path
 * integrate -> StaticCondensationMap -> assemble -> skeleton solve ->
 * BackwardStaticCondensationMap.  Each function names the reference file:line
 * it follows (paths relative to the GridapHybrid.jl repository).
 *
 * Parity status: the reference cannot run here (no Julia toolchain, Gridap is
 * not vendored).  The oracle is pinned against the reference's own known-answer
 * tests (test/DarcyHDGTests.jl:137-142 exactness < 1e-12,
 * test/SumFacetMapTests.jl:29,109, test/StaticCondensationMapTests.jl) and
 * against golden vectors produced by an independent LAPACK (scipy) executing
 * the reference's getrf/getrs/gemm/gemv call sequence; numeric golden vectors
 * from the reference itself are not available ("parity partially pinned").
 *
 * Conventions
 *  - Cell matrices are column-major (Julia layout), n = ni + nf, DOF order
 *    [flux (component-major) | pressure | skeleton (cell-local facet order)].
 *  - Facet DOF ids: >= 0 free (0-based), < 0 Dirichlet: id = -1 - dirichlet_index.
 *  - Return value 0 = ok, non-zero = error / singular pivot.
 */
#ifndef HDG_ORACLE_H
#define HDG_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Reference element ------------------------------------------------------ */
int orc_num_nodes(int D, int k);
int orc_lagrange_lattice(int D, int k, int *lattice /* nnodes x D */);
void orc_gauss_legendre01(int npts, double *x, double *w);

/* Cartesian mesh in Gridap numbering ------------------------------------- */
int orc_cart_counts(int D, const int *n, int *ncells, int *nfacets);
int orc_cart_topology(int D, const int *n, int *cell_facets, int *facet_cells,
                      int *facet_is_boundary);
int orc_facet_dofs(int D, int k, int nfacets, const int *facet_is_boundary,
                   int *facet_dofs, int *nfree, int *ndir);
int orc_facet_dofs_n(int nfd, int nfacets, const int *facet_is_boundary, int *facet_dofs, int *nfree,
                     int *ndir);

/* Integration of the Darcy HDG forms -------------------------------------- */
int orc_cell_sizes(int D, int k, int *ni, int *nf);
int orc_integrate_darcy(int D, int k, const int *n, const double *domain,
                        double tau, int stab_mode, int problem,
                        const double *kappa, const int *facet_cells,
                        const int *cell_facets, double *A, double *b);
/* Manufactured pressure at every facet DOF of a mesh of affine cells (free
 * ids -> free_vals, Dirichlet ids -> dir_vals; either may be NULL). */
int orc_facet_node_values_affine(int D, int k, int ncells, const double *origin, const double *jacobian,
                                 const int *cell_facets, const int *facet_cells, int problem, int nfacets,
                                 const int *facet_dofs, double *free_vals, double *dir_vals);
/* Bulk-to-skeleton L2 projection P_m (facet order k, cell order kb) on local
 * facet lf of the reference cell: P = (int mu mu^T) \ (int mu phi^T), column-major
 * nfd x (kb+1)^D.  Returns getrf's info. */
int orc_pm_projection(int D, int k, int kb, int lf, double *P);
/* facet quadrature of the order-k tables on local facet lf; returns nqf */
int orc_facet_quadrature(int D, int k, int lf, double *xi, double *w, double *mu);
/* order-k cell basis at cell-local points (npts x D) -> (npts x (k+1)^D) */
int orc_cell_basis(int D, int k, int npts, const double *xi, double *val);
/* General affine cells: origin (ncells x D), jacobian (ncells x D x D,
 * column-major per cell), topology as above. */
int orc_integrate_darcy_affine(int D, int k, int ncells, const double *origin, const double *jacobian,
                               double tau, int stab_mode, int problem, const double *kappa,
                               const int *facet_cells, const int *cell_facets, double *A, double *b);
int orc_integrate_darcy_cells(int D, int k, const int *n, const double *domain,
                              double tau, int stab_mode, int problem,
                              const double *kappa, const int *facet_cells,
                              const int *cell_facets, int nsel, const int *cells,
                              double *A, double *b);
int orc_dirichlet_values(int D, int k, const int *n, const double *domain,
                         int problem, int nfacets, const int *facet_is_boundary,
                         const int *facet_dofs, int ndir, double *vals);

/* Maps -------------------------------------------------------------------- */
int orc_static_condensation(int ncells, int ni, int nf, const double *A,
                            const double *b, double *S, double *g, int *info);
int orc_backward_static_condensation(int ncells, int ni, int nf,
                                     const double *A, const double *b,
                                     const double *x, double *u, int *info);
int orc_sum_facets(int nfacets, int len, const double *blocks, double *out);

/* Assembly and skeleton solve --------------------------------------------- */
int orc_csr_pattern(int D, int k, int ncells, int nfacets,
                    const int *cell_facets, const int *facet_dofs, int nfree,
                    int64_t *rowptr, int32_t *colind, int64_t *nnz);
int orc_assemble(int D, int k, int ncells, const int *cell_facets,
                 const int *facet_dofs, int nfree, const double *dir_vals,
                 const double *S, const double *g, const int64_t *rowptr,
                 const int32_t *colind, double *val, double *rhs);
/* the same with nfd DOFs per facet */
int orc_csr_pattern_n(int D, int nfd, int ncells, int nfacets, const int *cell_facets, const int *facet_dofs,
                      int nfree, int64_t *rowptr, int32_t *colind, int64_t *nnz);
int orc_assemble_n(int D, int nfd, int ncells, const int *cell_facets, const int *facet_dofs, int nfree,
                   const double *dir_vals, const double *S, const double *g, const int64_t *rowptr,
                   const int32_t *colind, double *val, double *rhs);
int orc_cell_skeleton_values_n(int D, int nfd, int ncells, const int *cell_facets, const int *facet_dofs,
                               const double *xfree, const double *dir_vals, double *xcell);
int orc_dense_solve(int n, const int64_t *rowptr, const int32_t *colind,
                    const double *val, const double *rhs, double *x);
int orc_pcg(int n, int bs, const int64_t *rowptr, const int32_t *colind,
            const double *val, const double *rhs, double *x, double sign,
            double rtol, int maxit, int *iters, double *relres);

/* Recovery helpers, errors, full pipeline ---------------------------------- */
int orc_cell_skeleton_values(int D, int k, int ncells, const int *cell_facets,
                             const int *facet_dofs, const double *xfree,
                             const double *dir_vals, double *xcell);
int orc_l2_errors(int D, int k, const int *n, const double *domain,
                  int problem, const double *kappa, const double *uint,
                  double *err_flux, double *err_pres);
/* Set-up of a Cartesian Darcy mesh once (topology, facet DOFs, Dirichlet
 * values, CSR pattern), then solves on it; orc_solve_darcy = both. */
typedef struct orc_darcy orc_darcy;
int orc_darcy_setup(int D, int k, const int *n, const double *domain, int problem, orc_darcy **out,
                    int64_t *nnz, int *nfree);
int orc_darcy_step(orc_darcy *h, double tau, int stab_mode, const double *kappa, int solver, double rtol,
                   int maxit, double *uint_out, double *lambda_out, double *val_out, double *rhs_out,
                   double *times_out, int *iters, double *relres, double *err_flux, double *err_pres);
void orc_darcy_free(orc_darcy *h);
int orc_solve_darcy(int D, int k, const int *n, const double *domain,
                    double tau, int stab_mode, int problem, const double *kappa,
                    int solver, double rtol, int maxit, double *uint_out,
                    double *lambda_out, double *times_out, int *iters,
                    double *relres, double *err_flux, double *err_pres);
/* Linear elasticity HDG (test/LinearElasticityHDGTests.jl) --------------- */
int orc_elasticity_sizes(int D, int k, int *ni, int *nf, int *nfd);
int orc_integrate_elasticity(int D, int k, const int *n, const double *domain, double tau, double E,
                             const double *nu, int problem, double *A, double *b);
int orc_dirichlet_values_elasticity(int D, int k, const int *n, const double *domain, int problem, int nfacets,
                                    const int *facet_is_boundary, const int *facet_dofs, int ndir, double *vals);
int orc_l2_errors_elasticity(int D, int k, const int *n, const double *domain, double E, const double *nu,
                             int problem, const double *uint, double *err_sigma, double *err_u);
int orc_solve_elasticity(int D, int k, const int *n, const double *domain, double tau, double E, const double *nu,
                         int problem, int solver, double sign, double rtol, int maxit, double *uint_out,
                         double *lambda_out, int *iters, double *relres, double *err_sigma, double *err_u);
int orc_max_threads(void);
void orc_set_threads(int nthreads);

#ifdef __cplusplus
}
#endif
#endif
