/*
 * hdg_gb300.h -- C ABI of the GB300 (sm_103a) cellwise hybridization library
 * (libgridaphybrid_gb300.so).
 *
 * The library replaces, on one GPU, the hot path of GridapHybrid.jl:
 * per-cell integration of the cell + facet bilinear forms (SumFacetsMap path),
 * StaticCondensationMap, assembly of the skeleton system, the skeleton solve,
 * and BackwardStaticCondensationMap.  Each entry point names the reference
 * interface it stands in for (paths relative to the GridapHybrid.jl repo).
 *
 * Conventions
 *  - Every function returns an int status (HDG_OK == 0).  A failing call
 *    leaves a message in hdg_last_error(ctx).
 *  - Pointer arguments may point to host memory (pageable or pinned) or to
 *    device memory of the context's GPU; the library detects which.  Outputs
 *    are written when the call returns (calls are synchronous unless noted).
 *  - Dense cell blocks are column-major (Julia layout).  Per cell the DOF
 *    order is [interior fields | skeleton fields], the interior fields in
 *    the order of `bulk_fields` and each field's DOFs in its reference-FE
 *    order, the skeleton DOFs in cell-local facet order
 *    (src/HybridAffineFEOperators.jl:424-434).
 *  - Facet DOF ids follow Gridap's sign convention shifted to 0-based:
 *    id >= 0 is a free DOF, id < 0 is Dirichlet DOF number (-1 - id).
 *  - No entry point falls back to the CPU: without a usable sm_103a device
 *    hdg_context_create fails with HDG_ERR_NODEVICE.
 */
#ifndef HDG_GB300_H
#define HDG_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define HDG_OK 0
#define HDG_ERR_INVALID 1       /* bad argument or size */
#define HDG_ERR_CUDA 2          /* CUDA runtime error */
#define HDG_ERR_NOMEM 3         /* device allocation failed */
#define HDG_ERR_SINGULAR 4      /* zero pivot in a cell's interior block (info > 0) */
#define HDG_ERR_NOT_CONVERGED 5 /* skeleton solver did not reach the tolerance */
#define HDG_ERR_STATE 6         /* call out of order (e.g. solve before assemble) */
#define HDG_ERR_NODEVICE 7      /* no usable CUDA device */

/* Arithmetic of the cell-local work. */
#define HDG_PREC_FP64 0          /* FP64 integration, LU and Schur complement */
#define HDG_PREC_FP32_REFINED 1  /* FP32 LU, refined with high-precision residuals */
/* Operator path only (hdg_assemble): the first bulk block of the cell matrix
 * is a reference mass matrix times a per-cell factor -- Darcy flux:
 * (|J|/kappa)(I (x) M_ref); elasticity stress: |J| (C_nu (x) M_ref) -- so the
 * condensation is done by block elimination (an LU of the second field's Schur
 * complement and dense products) entirely in float-float on the FP32 pipes;
 * skeleton solve and recovery as for HDG_PREC_FP32_REFINED.  D=2, k<=3 and
 * D=3, k<=2.  FP64 elasticity cell blocks too large for the shared-memory LU
 * (D=3, k=2) are condensed by the same block elimination in FP64. */
#define HDG_PREC_FF_BLOCK 2

/* Stabilisation of the Darcy HDG form. */
#define HDG_STAB_TEXTBOOK 0     /* tau*(p - l) on every facet side (LDG-H) */
#define HDG_STAB_OWNER_SIGN 1   /* tau*(p - l)*(n.n_o), test/DarcyHDGTests.jl:125-135 */

/* Built-in manufactured problems (sources, Dirichlet data, exact solution). */
#define HDG_PROBLEM_REF_LINEAR 0 /* u=(1+x,1+y[,1+z]), p=-3.14 (test/DarcyHDGTests.jl:8-13) */
#define HDG_PROBLEM_LINEAR 1     /* p = x+y[+z], q = -kappa grad p, f = 0 */
#define HDG_PROBLEM_SIN 2        /* p = prod sin(pi x_d), q = -kappa grad p, f = div q */

/* Physics of a problem (fixes the field layout at creation). */
#define HDG_PHYSICS_DARCY 0      /* flux (D comps) + pressure inside, scalar trace (test/DarcyHDGTests.jl) */
#define HDG_PHYSICS_ELASTICITY 1 /* symmetric stress + displacement inside, displacement trace
                                    (test/LinearElasticityHDGTests.jl) */

/* Built-in manufactured elasticity problems. */
#define HDG_EPROBLEM_LINEAR 0 /* u = (x+2y, 2x+y) (:48-50); 3D (x+2y, 2x+y+z, y+3z) */
#define HDG_EPROBLEM_SMOOTH 1 /* u = (10 sin(pi x)(1-x)(y-y^2)(1-y/2), 0) (:52-57); 3D (sin pi x, cos pi y, xyz) */

/* Skeleton solvers. */
#define HDG_SOLVER_PCG 0        /* facet-block-Jacobi PCG on -S (SPD forms) */
#define HDG_SOLVER_DIRECT 1     /* dense LU with partial pivoting (small systems, any form) */

typedef struct hdg_context hdg_context;
typedef struct hdg_problem hdg_problem;

/* Library version (major*10000 + minor*100 + patch). */
int hdg_version(void);

/* Number of device allocations the library has made since it was loaded (all
 * contexts and problems; every device buffer is allocated through one routine
 * that counts).  No reference counterpart. */
int hdg_device_allocations(long long *count);

/* The rule every entry point applies to a caller's pointer, from the
 * (memory_type, device) that cudaPointerGetAttributes reports for it and the
 * context's GPU: *place = 0 host memory (staged through the context's
 * buffers), 1 usable in place (device memory of the context's GPU, or managed
 * memory), 2 refused: device memory of another GPU, which the kernels could
 * not read without peer access; the entry points then return HDG_ERR_INVALID
 * and so does this query.  No reference counterpart. */
int hdg_pointer_placement(int memory_type, int pointer_device, int context_device, int *place);

/* Context: one GPU, one stream, a device memory pool.  One context per host
 * thread.  No reference counterpart (the reference is single-threaded Julia). */
int hdg_context_create(int device, hdg_context **out);
int hdg_context_destroy(hdg_context *ctx);
const char *hdg_last_error(const hdg_context *ctx);
int hdg_context_synchronize(hdg_context *ctx);
/* Number of this library's kernels launched on ctx so far. */
long long hdg_launch_count(const hdg_context *ctx);
/* CUDA events on the context's stream for timing a sequence of calls:
 * record into slot 0..3, then the device time between two recorded slots. */
int hdg_context_record(hdg_context *ctx, int slot);
int hdg_context_elapsed_ms(hdg_context *ctx, int slot_from, int slot_to, double *ms);

/* ---------------------------------------------------------------------- */
/* Map level (batched over cells).                                          */
/* ---------------------------------------------------------------------- */

/* StaticCondensationMap: Gridap.Arrays.evaluate!(cache, k, A, b)
 * (src/StaticCondensationMap.jl:146-196; cache :41-70).  For each of ncells
 * cells, A is (ni+nf)^2 column-major and b is (ni+nf); outputs
 * S = A_ff - A_fi A_ii^{-1} A_if (nf x nf, column-major) and
 * g = b_f - A_fi A_ii^{-1} b_i (nf).  info[c] is LAPACK's getrf info of the
 * cell's A_ii (0 = ok), which the reference checks with @check info==0
 * (:180); a non-zero info makes the call return HDG_ERR_SINGULAR.
 * info may be NULL. */
int hdg_static_condensation(hdg_context *ctx, int precision, int ncells, int ni,
                            int nf, const double *A, const double *b, double *S,
                            double *g, int *info);

/* BackwardStaticCondensationMap: evaluate!(cache, k, A, b, x)
 * (src/BackwardStaticCondensationMap.jl:61-102): u_i = A_ii^{-1}(b_i - A_if x)
 * for each cell; x is nf per cell, u is ni per cell (the interior blocks of the
 * re-blocked vector, :133-151). */
int hdg_backward_static_condensation(hdg_context *ctx, int precision,
                                     int ncells, int ni, int nf,
                                     const double *A, const double *b,
                                     const double *x, double *u, int *info);

/* SumFacetsMap: evaluate!(cache, k, a) (src/SumFacetsMap.jl:19-30).  For each
 * of nitems items, sums nfacets blocks of len values each:
 * out[i] = sum_f blocks[(i*nfacets + f)*len + :].  nfacets >= 2. */
int hdg_sum_facets(hdg_context *ctx, int nitems, int nfacets, int len,
                   const double *blocks, double *out);

/* hdg_static_condensation with HDG_PREC_FP32_REFINED, for callers that cannot
 * allocate device memory (a host framework whose caching allocator already
 * holds the device's free memory, or a pipeline step where an allocation would
 * synchronise the device).  No counterpart in the reference.
 *  - Allocates nothing: A, b, S, g (and info, if not NULL) must be device
 *    pointers; the temporaries (the FP32 hi/lo staging of every cell block)
 *    live in one fixed device array of HDG_NOALLOC_SCRATCH_BYTES bytes that
 *    every GPU loading this library keeps until the process exits.
 *  - A batch needs 8*ncells*((ni+nf)^2 + ni+nf) bytes plus a little, and
 *    4*ncells more when info is NULL; a larger batch is rejected with
 *    HDG_ERR_INVALID (split it).
 *  - The first call on a device looks the array's address up
 *    (cudaGetSymbolAddress).
 *  - Each call waits for its own work (it synchronises the context's stream
 *    to read the pivot flag) and gives the caller's current device back, so
 *    no call can be captured into a CUDA graph: a call made while the
 *    context's stream is capturing fails and ends that capture.
 *  - Pointers must be device memory of the context's GPU (or managed);
 *    host memory and other GPUs' memory are refused with HDG_ERR_INVALID.
 *  - Every call uses the same array: calls that overlap on the GPU race, so
 *    issue them on one stream (the context's) or order them with events.
 * Results equal hdg_static_condensation(ctx, HDG_PREC_FP32_REFINED, ...). */
#define HDG_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int hdg_static_condensation_noalloc(hdg_context *ctx, int ncells, int ni, int nf,
                                    const double *A, const double *b, double *S,
                                    double *g, int *info);

/* ---------------------------------------------------------------------- */
/* Operator level: HybridAffineFEOperator / solve.                          */
/* ---------------------------------------------------------------------- */

/* Skeleton(model) + the L2 facet space of order k with Dirichlet facets on the
 * boundary, for CartesianDiscreteModel(domain, cells) (src/Skeleton.jl:113-147;
 * test/DarcyHDGTests.jl:27-52).  Cells, facets and DOFs are numbered as
 * Gridap numbers them; domain is (x0,x1,y0,y1[,z0,z1]). */
int hdg_problem_create_cartesian(hdg_context *ctx, int D, const int *cells,
                                 const double *domain, int k,
                                 hdg_problem **out);

/* Same from an explicit affine mesh: cell_origin (ncells x D), cell_jacobian
 * (ncells x D x D, column-major per cell), cell_facets (ncells x 2D, 0-based,
 * Gridap local facet order), facet_dofs (nfacets x (k+1)^(D-1), sign convention
 * above; each free facet's DOFs consecutive and increasing).  These are the
 * arrays the reference obtains from get_faces(topo, D, D-1) and
 * get_cell_dof_ids(L) (src/HybridAffineFEOperators.jl:152-162, :436-439).
 * Facets must be seen with the same vertex order from both sides. */
int hdg_problem_create(hdg_context *ctx, int D, int k, int ncells, int nfacets,
                       const double *cell_origin, const double *cell_jacobian,
                       const int *cell_facets, const int *facet_dofs,
                       hdg_problem **out);
/* The same Cartesian mesh for a given physics (HDG_PHYSICS_*): the facet
 * space has one (Darcy) or D (elasticity) components per facet node,
 * component-major within a facet as Gridap's vector-valued Lagrangian spaces
 * (src/tmp_fixes_symmetric_valued_lagrangian_reffes.jl:104-125). */
int hdg_problem_create_cartesian_physics(hdg_context *ctx, int D, const int *cells,
                                         const double *domain, int k, int physics,
                                         hdg_problem **out);
/* The same Cartesian mesh with a polynomial space of its own for each field,
 * as the reference's tests choose them: ReferenceFE(lagrangian, T, order;
 * space=:P) (test/DarcyHDGTests.jl:34-36: flux P_k, pressure P_{k-1},
 * multiplier P_k; test/LinearElasticityHDGTests.jl:88-93: stress P_k,
 * displacement P_{k+1}, displacement trace P_k) and raviart_thomas
 * (test/DarcyRTHTests.jl:28-30: flux RT_k, pressure Q_k, multiplier Q_k,
 * no stabilisation: hdg_set_darcy with tau = 0).  spaces[7] = {kindA, kA,
 * kindB, kB, kindT, kT, pm}: A the first bulk field (Darcy flux /
 * elasticity stress), B the second (pressure / displacement), T the trace;
 * kind HDG_SPACE_Q (tensor Lagrange, order 0..4), HDG_SPACE_P (total degree,
 * order 0..4; Lagrange at the simplex lattice points i/k, the constant for
 * order 0) or, for the Darcy flux, HDG_SPACE_RT (order 0..3); pm = 1 applies
 * the bulk-to-skeleton projection P_m to the displacement in the tau terms
 * (src/GridapAPIExtensions.jl:453-500, test/LinearElasticityHDGTests.jl:
 * 134-150).  copies > 1 builds that many decoupled copies of the form, each
 * with its own fields and its own skeleton field: the skeleton system of
 * several fields of test/MultiFieldLagrangeMultipliersTests.jl (bulk fields
 * [A_1 .. A_c, B_1 .. B_c], skeleton fields [T_1 .. T_c]); the skeleton
 * values, free DOF values and hdg_get_skeleton_system use that multi-field
 * numbering (each copy's skeleton field numbered on its own, one after the
 * other), hdg_l2_errors sums the copies' squared errors.  The cell blocks are
 * integrated in FP64 and condensed with HDG_PREC_FP64 or
 * HDG_PREC_FP32_REFINED; the other calls (hdg_set_darcy /
 * hdg_set_elasticity, hdg_assemble, hdg_solve_skeleton, hdg_recover,
 * hdg_get_*, hdg_l2_errors, hdg_solve) work as for the equal-order problems.
 * Free DOF values keep Gridap's layout [each bulk field of all cells |
 * skeleton]. */
#define HDG_SPACE_Q 0
#define HDG_SPACE_P 1
#define HDG_SPACE_RT 2
int hdg_problem_create_cartesian_spaces(hdg_context *ctx, int D, const int *cells, const double *domain,
                                        int physics, const int *spaces, int copies, hdg_problem **out);

/* The same on simplexify(CartesianDiscreteModel(domain, cells))
 * (test/DarcyHDGTests.jl:174-177): every box split into D! simplices around
 * its diagonal from the lowest to the highest vertex (2 triangles per square,
 * 6 tetrahedra per cube; boxes x fastest, then the axis orders of the path
 * lexicographically); a cell lists its vertices in increasing global order
 * (lattice points, x fastest), local facet lf is the face opposite local
 * vertex D - lf, facets are numbered in first-met order over (cell, local
 * facet) and the first cell of a facet is its owner.  The Darcy form
 * (physics HDG_PHYSICS_DARCY) with P_k fields only (HDG_SPACE_P, pm = 0);
 * everything else as hdg_problem_create_cartesian_spaces. */
int hdg_problem_create_simplex_spaces(hdg_context *ctx, int D, const int *cells, const double *domain,
                                      int physics, const int *spaces, int copies, hdg_problem **out);
int hdg_problem_destroy(hdg_problem *pb);

/* info[0..7] = ncells, nfacets, ni, nf, nfree, ndirichlet, nnz, nfacet_dofs */
int hdg_problem_info(const hdg_problem *pb, long long *info);

/* The skeleton glue of the problem: cell_facets (ncells x 2D, Gridap local facet
 * order), facet_cells (nfacets x 2, cells around each facet in increasing order,
 * -1 if none; the first is the owner of get_cell_owner_normal_vector), facet_dofs
 * (nfacets x nfacet_dofs).  get_faces(topo, D, D-1) / get_faces(topo, D-1, D) /
 * get_cell_dof_ids(L) (src/HybridAffineFEOperators.jl:152-162; src/Skeleton.jl:549-556).
 * Any pointer may be NULL. */
int hdg_get_topology(const hdg_problem *pb, int *cell_facets, int *facet_cells,
                     int *facet_dofs);

/* The weak form (test/DarcyHDGTests.jl:125-135 with a per-cell permeability
 * in the flux mass term): stab_mode HDG_STAB_*, tau > 0, problem HDG_PROBLEM_*
 * (sources + Dirichlet data).  kappa: ncells values (NULL = 1). */
int hdg_set_darcy(hdg_problem *pb, int stab_mode, double tau, int problem);
/* The per-cell coefficient (ncells values): the permeability kappa of the
 * Darcy form (NULL = 1), or the Poisson ratio nu of the elasticity form
 * (NULL = 0.3). */
int hdg_set_permeability(hdg_problem *pb, const double *kappa);
/* Dirichlet values of the trial skeleton space, ndirichlet values
 * (TrialFESpace(M, p), test/DarcyHDGTests.jl:52).  hdg_set_darcy interpolates
 * the problem's exact pressure; this call overrides it. */
int hdg_set_dirichlet_values(hdg_problem *pb, const double *vals);

/* HybridAffineFEOperator(weakform, X, Y, bulk, skel)
 * (src/HybridAffineFEOperators.jl:10-50): integrate, condense (keeping the
 * factors of every A_ii on the device) and assemble the skeleton system with
 * the Dirichlet lift.  info: ncells values or NULL. */
int hdg_assemble(hdg_problem *pb, int precision, int *info);

/* The assembled skeleton system of op.skeleton_op (:46-48) as CSR with sorted
 * columns: rowptr (nfree+1), colind (nnz), val (nnz), rhs (nfree).  Any
 * pointer may be NULL.  Gridap stores the same matrix as SparseMatrixCSC;
 * for the symmetric forms here the arrays coincide. */
int hdg_get_skeleton_system(hdg_problem *pb, long long *rowptr, int *colind,
                            double *val, double *rhs);

/* solve(op.skeleton_op) (src/HybridAffineFEOperators.jl:74).  rtol is the
 * relative residual of PCG; iters/relres may be NULL. */
int hdg_solve_skeleton(hdg_problem *pb, int solver, double rtol, int maxit,
                       int *iters, double *relres);

/* HybridFEOperator(res, X, Y, bulk, skel) + solve!(xh0, FESolver(NLSolver(
 * method=:newton)), op) (src/HybridFEOperators.jl:68-239,
 * src/HybridLinearSolvers.jl:15-59, test/DarcyHDGTests.jl:157-165).  Newton
 * iterations x <- x - dx: each step integrates the Jacobian (the cell
 * matrices A_c) and the residual r_c = A_c x_c - b_c of the iterate,
 * condenses [A_c | r_c], solves the skeleton system for dx with zero
 * Dirichlet data (the correction vanishes there, :49-50) and recovers the
 * interior corrections.  Stops when the max norm of the assembled residual
 * is <= ftol (NLsolve's default 1e-8) or returns HDG_ERR_NOT_CONVERGED after
 * max_iters steps.  x0: the initial free DOF values (hdg_get_free_dof_values
 * layout), or NULL for zeros (FEFunction(X, zeros(num_free_dofs(X))));
 * res_norms (max_iters + 1 values, may be NULL) receives the residual norm
 * before each step; iters the number of steps.  FP64 arithmetic.  The
 * result is the problem's solution (hdg_get_free_dof_values, hdg_l2_errors). */
int hdg_newton_solve(hdg_problem *pb, int solver, double lin_rtol, int lin_maxit, double ftol,
                     int max_iters, const double *x0, double *res_norms, int *iters);

/* The linear elasticity HDG form of test/LinearElasticityHDGTests.jl:140-150
 * without the P_m projection (bulk_to_skeleton_projection=false):
 *   v (.) A(sigma) + (div v).u - w.(div sigma) on Omega,
 *   -(v.n).uhat + tau w.(u - uhat) + mu.(sigma.n) - tau mu.(u - uhat) on dK,
 * compliance A(s) = (1+nu)/E s - nu/E tr(s) I (:15-38) with the per-cell
 * Poisson ratio given by hdg_set_permeability (the per-cell coefficient),
 * f = div sigma_exact and Dirichlet data u_exact (problem: HDG_EPROBLEM_*).
 * The problem must have been created with HDG_PHYSICS_ELASTICITY.
 * hdg_l2_errors then returns the stress and displacement errors. */
int hdg_set_elasticity(hdg_problem *pb, double tau, double young, int problem);

/* Options of the fast precisions' skeleton solve (an FP32 PCG inside FP64
 * residual refinement; no reference counterpart).  delta: the relative
 * residual reduction the FP32 iterations make between two FP64 residuals
 * (default 1e-2 for D = 3, 3e-2 for D = 2); keep_direction: 1 (default) replaces the FP32 residual by
 * the FP64 one and keeps the search direction (reliable updates), 0 restarts
 * the FP32 PCG at every FP64 residual. */
int hdg_set_refinement(hdg_problem *pb, double delta, int keep_direction);

/* Interior recovery _compute_hybridizable_from_skeleton_free_dof_values
 * (src/HybridAffineFEOperators.jl:102-150) with the stored factors. */
int hdg_recover(hdg_problem *pb);

/* Free DOF values of the multi-field trial space in Gridap's consecutive
 * layout [first bulk field of all cells | second bulk field of all cells |
 * free skeleton DOFs] (FEFunction(op.trial, free_dof_values), :99): Darcy
 * [flux | pressure | trace], elasticity [stress | displacement | trace].
 * Length ncells*ni + nfree. */
int hdg_get_free_dof_values(hdg_problem *pb, double *out);
/* Interior values per cell (ncells x ni) and free skeleton values (nfree). */
int hdg_get_cell_interior_values(hdg_problem *pb, double *out);
int hdg_get_skeleton_values(hdg_problem *pb, double *out);

/* sqrt(sum(int((u-uh).(u-uh))dOmega)) (test/DarcyHDGTests.jl:141-142) for the
 * flux and the pressure against the problem's exact solution. */
int hdg_l2_errors(hdg_problem *pb, double *err_flux, double *err_pres);

/* solve(op) in one call (src/HybridAffineFEOperators.jl:67-100):
 * set kappa (may be NULL), assemble, solve the skeleton, recover, and copy the
 * free DOF values (may be NULL) out.  stats (may be NULL) receives
 * [pcg iterations, relative residual, ms integrate+condense, ms assemble,
 *  ms skeleton solve, ms recover, ms total]. */
int hdg_solve(hdg_problem *pb, int precision, int solver, double rtol,
              int maxit, const double *kappa, double *free_dof_values,
              double *stats);

/* Inner FP32 skeleton iterations of the fast paths as one cooperative launch
 * per chunk (on = 1: every iteration's SpMV and update phases inside one
 * kernel, separated by bounded grid barriers) instead of replays of a CUDA
 * graph of two-kernel iterations (on = 0, the default).  Same arithmetic; the
 * sums run over a different number of CTAs, so the last bits may differ. */
int hdg_context_set_persistent_pcg(hdg_context *ctx, int on);

/* Device-event timings of the last hdg_assemble/solve_skeleton/recover calls
 * in ms: [integrate, condense, assemble, skeleton solve, recover]. */
int hdg_get_timings(const hdg_problem *pb, double *ms);

/* The last skeleton solve: [iterations, relative residual, FP64 residual
 * refinements (fast precisions; 0 for FP64), iterations of the FP64
 * correction solve that finishes a refined solve whose FP32 cycles stalled
 * (0 when none was needed)].  No reference counterpart. */
int hdg_get_solve_stats(const hdg_problem *pb, double *stats);

/* Benchmark support (no reference counterpart): relaunches one kernel of the
 * path `reps` times between CUDA events on the library's stream and returns
 * the mean device time per launch in ms.  which: 0 integrate, 1 condense,
 * 2 assemble (gather + rhs), 3 skeleton SpMV, 4 recover.  The problem must
 * have been assembled (and solved for 3, 4); state is recomputed, not
 * changed. */
int hdg_time_kernel(hdg_problem *pb, int which, int reps, double *ms_per_launch);

/* Benchmark support (no reference counterpart): the device's measured FMA
 * pipe peaks in TFLOP/s (an FMA counts 2 flops), from a few-ms kernel of
 * independent FMA chains at full occupancy timed by CUDA events: FP32 (the
 * pipes of the float-float paths) and FP64 (the plain FP64 path). */
int hdg_measure_pipe_peaks(hdg_context *ctx, double *fp32_tflops, double *fp64_tflops);

/* Diagnostic (no reference counterpart): runs the two bounded wait
 * primitives the kernels use -- the mbarrier wait of the bulk-copy rings and
 * the generation wait of the cooperative grid barrier -- against a barrier
 * phase and a word that nothing completes or writes, each for `polls` polls
 * (1 .. 2^20), with nothing in flight.  expired[0..1] = 1 when the mbarrier /
 * generation wait gave up (the expected result); ns_per_poll[0..1] = the
 * time of one poll at the device's rated clock.  The kernels' own limits are
 * 2^18 polls (mbarrier) and 2^22 polls (grid barrier), about one second each
 * on a GB300; on expiry they set an
 * error flag, wait (bounded) for their own copies in flight and return, and
 * the call fails with HDG_ERR_CUDA while the context stays usable. */
int hdg_check_bounded_waits(hdg_context *ctx, unsigned polls, int *expired, double *ns_per_poll);

/* Device bytes currently reserved by the problem (all its buffers). */
int hdg_problem_device_bytes(const hdg_problem *pb, double *bytes);

/* ------------------------------------------------------------------------
 * Size-class batching (no reference counterpart: the reference assembles one
 * problem per HybridAffineFEOperator).  The problems of a batch share one
 * context and are grouped by (D, k); each class is integrated and condensed
 * by ONE persistent fused launch over the cells of all its problems, the cell
 * blocks staying on chip (FP64: in shared memory) or in L2 (float-float block
 * elimination), and the condensed blocks are then assembled into each
 * problem's skeleton system.  The first assemble of a class times the tile
 * choices (threads per cell = 32, 64, 128, 256, i.e. 8..1 cells per CTA) and
 * keeps the fastest; the whole launch sequence is captured in a CUDA graph
 * and replayed while the problems' buffers stay put.  After
 * hdg_batch_assemble every problem is assembled exactly as hdg_assemble would
 * leave it (same state, same values), so hdg_solve_skeleton / hdg_recover /
 * hdg_get_* work per problem.
 * ------------------------------------------------------------------------ */
typedef struct hdg_batch hdg_batch;
int hdg_batch_create(hdg_context *ctx, int nproblems, hdg_problem *const *problems,
                     hdg_batch **out);
int hdg_batch_destroy(hdg_batch *b);
/* precision: HDG_PREC_FP64 or HDG_PREC_FF_BLOCK.  bad (may be NULL, nproblems
 * values, batch order) receives each problem's first zero pivot (0 = ok). */
int hdg_batch_assemble(hdg_batch *b, int precision, int *bad);
/* Skeleton solve + recovery of every problem; iters/relres may be NULL. */
int hdg_batch_solve(hdg_batch *b, int solver, double rtol, int maxit, int *iters,
                    double *relres);
/* ms of the last calls: [fused integrate+condense (all classes),
 * skeleton assembly (all problems), solve + recover (all problems)]. */
int hdg_batch_timings(const hdg_batch *b, double *ms);
/* The tuned tile per class for a precision: D, k, threads per cell, the
 * fused launch's ms at tuning time and the class's cells (arrays of
 * max_classes); nclasses receives the number of classes. */
int hdg_batch_tuning(const hdg_batch *b, int precision, int max_classes, int *D, int *k,
                     int *tpc, double *ms, long long *cells, int *nclasses);

/* ------------------------------------------------------------------------
 * Serving (no reference counterpart: the reference solves one problem per
 * `solve(op)` call).  A server owns `slots` worker threads; each runs one
 * request at a time on its own stream, so admitted requests overlap on the
 * device.  Requests are admitted in arrival order (a smaller one may pass a
 * larger one that does not fit yet, a bounded number of times) as slots and
 * the HBM budget free up; a request's footprint is hdg_footprint().  Meshes
 * stay resident after a solve (connectivity, CSR pattern, buffers) and are
 * reused by the next request with the same (D, n, k); idle resident meshes
 * are evicted least-recently-used when the budget is needed or when they hold
 * more than half of it.  A result does
 * not depend on what else was running (deterministic kernels).
 * ------------------------------------------------------------------------ */
typedef struct hdg_server hdg_server;

typedef struct hdg_request {
  int D, n, k;         /* unit square/cube, n cells per side, order k */
  int problem;         /* HDG_PROBLEM_* manufactured solution */
  int stab_mode;       /* HDG_STAB_* */
  int precision;       /* HDG_PREC_* */
  int solver;          /* HDG_SOLVER_* */
  int maxit;
  double tau, rtol;
  const double *kappa; /* n^D per-cell permeabilities (copied at submit) or NULL (all 1) */
  double *solution;    /* NULL, or host buffer of ncells*ni + nfree free DOF values,
                          written before the response is posted */
} hdg_request;

typedef struct hdg_response {
  long long ticket;
  int status;            /* HDG_OK or the failing call's code */
  int iters;
  double relres;
  double err_flux, err_pressure; /* L2 errors against the manufactured solution */
  double queue_ms;       /* submit -> admitted */
  double run_ms;         /* admitted -> done */
  double latency_ms;     /* submit -> done */
  double footprint_bytes;/* reserved at admission */
  int reused_mesh;       /* 1 if the mesh was already resident */
  int slot;              /* worker that ran it */
  char message[160];     /* the failing call's hdg_last_error text ("" on success) */
} hdg_response;

/* Upper bound of the device bytes one request of this shape needs. */
int hdg_footprint(int D, int n, int k, int precision, int solver, double *bytes);

/* hbm_budget_bytes <= 0 selects 85% of the device's free memory. */
int hdg_server_create(int device, int slots, double hbm_budget_bytes, hdg_server **out);
/* Stops the workers after the running requests finish; queued requests are
 * answered with HDG_ERR_STATE. */
int hdg_server_destroy(hdg_server *s);
/* Non-blocking.  Rejects (HDG_ERR_INVALID) shapes the library cannot solve
 * and requests larger than the whole budget. */
int hdg_server_submit(hdg_server *s, const hdg_request *req, long long *ticket);
/* Moves up to `max` finished responses into out; waits up to timeout_ms for
 * the first one when none is ready. */
int hdg_server_poll(hdg_server *s, hdg_response *out, int max, double timeout_ms, int *count);
/* Waits until no request is queued or running (HDG_ERR_NOT_CONVERGED on timeout). */
int hdg_server_drain(hdg_server *s, double timeout_ms);
/* [submitted, completed, failed, running, queued, bytes in use, budget,
 *  peak bytes in use, mesh hits, mesh misses, evictions, max concurrent,
 *  summed run ms of finished requests, requests run a second time after a
 *  device allocation failed] (14 values).  A request whose allocation fails
 *  below the admission budget (memory the pool keeps, or another user of the
 *  GPU) is run once more after every idle mesh is evicted and the pool's
 *  unused memory is returned to the device. */
int hdg_server_stats(hdg_server *s, double *stats);
const char *hdg_server_last_error(hdg_server *s);

#ifdef __cplusplus
}
#endif
#endif
