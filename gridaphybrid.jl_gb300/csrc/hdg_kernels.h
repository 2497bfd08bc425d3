// hdg_kernels.h -- launch wrappers of the sm_103a kernels (host-callable).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hdg {

// Exact solutions / sources of the built-in manufactured problems, shared by
// the kernels and the host-side Dirichlet interpolation.
//   kappa^{-1} q + grad p = f_u,  div q = g.
#if defined(__CUDACC__)
#define HDG_HD __host__ __device__ __forceinline__
#else
#define HDG_HD inline
#endif
HDG_HD void exact_solution(int problem, int D, const double *x, double kappa,
                           double &p, double *q, double *fu, double &g) {
  const double pi = 3.14159265358979323846;
  if (problem == 0) {  // test/DarcyHDGTests.jl:8-13
    p = -3.14;
    for (int d = 0; d < D; ++d) {
      q[d] = 1.0 + x[d];
      fu[d] = q[d] / kappa;
    }
    g = (double)D;
  } else if (problem == 1) {
    p = 0.0;
    for (int d = 0; d < D; ++d) {
      p += x[d];
      q[d] = -kappa;
      fu[d] = 0.0;
    }
    g = 0.0;
  } else {
    double s[3], c[3], prod = 1.0;
    for (int d = 0; d < D; ++d) {
#ifdef __CUDA_ARCH__
      sincospi(x[d], &s[d], &c[d]);  // sin(pi x), cos(pi x) without rounding pi x first
#else
      s[d] = sin(pi * x[d]);
      c[d] = cos(pi * x[d]);
#endif
      prod *= s[d];
    }
    p = prod;
    for (int d = 0; d < D; ++d) {
      double gd = pi * c[d];
      for (int e = 0; e < D; ++e)
        if (e != d) gd *= s[e];
      q[d] = -kappa * gd;
      fu[d] = 0.0;
    }
    g = kappa * D * pi * pi * prod;
  }
}

// Linear elasticity manufactured solutions (test/LinearElasticityHDGTests.jl):
// displacement u, gradient gu[i][j] = du_i/dx_j, Hessian hu[i][j][k].
HDG_HD void elasticity_exact(int problem, int D, const double *x, double *u, double (*gu)[3],
                             double (*hu)[3][3]) {
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < 3; ++i) {
    u[i] = 0.0;
    for (int j = 0; j < 3; ++j) {
      gu[i][j] = 0.0;
      for (int k = 0; k < 3; ++k) hu[i][j][k] = 0.0;
    }
  }
  if (problem == 0) {  // linear: u = (x+2y, 2x+y) (:48-50); 3D (x+2y, 2x+y+z, y+3z)
    u[0] = x[0] + 2 * x[1];
    u[1] = 2 * x[0] + x[1];
    gu[0][0] = 1; gu[0][1] = 2; gu[1][0] = 2; gu[1][1] = 1;
    if (D == 3) {
      u[1] += x[2];
      u[2] = x[1] + 3 * x[2];
      gu[1][2] = 1; gu[2][1] = 1; gu[2][2] = 3;
    }
  } else if (D == 2) {  // (:52-57)
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
  } else {  // (sin pi x, cos pi y, xyz)
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

// sigma = A^{-1}(eps) for A(s) = (1+nu)/E s - nu/E tr(s) I (:15-38):
// 2 mu eps + lam tr(eps) I with mu = E/(2(1+nu)), lam = nu E/((1+nu)(1+nu-D nu))
HDG_HD void elasticity_lame(int D, double E, double nu, double &mu, double &lam) {
  mu = E / (2.0 * (1.0 + nu));
  lam = nu * E / ((1.0 + nu) * (1.0 + nu - D * nu));
}

// f = div sigma_exact
HDG_HD void elasticity_force(int D, double E, double nu, const double (*hu)[3][3], double *f) {
  double mu, lam;
  elasticity_lame(D, E, nu, mu, lam);
  for (int i = 0; i < D; ++i) {
    double v = 0.0;
    for (int j = 0; j < D; ++j) v += mu * (hu[i][j][j] + hu[j][i][j]);
    for (int k = 0; k < D; ++k) v += lam * hu[k][i][k];
    f[i] = v;
  }
}

// the (i, j) pair of symmetric-tensor component c (upper triangle, row by row)
HDG_HD void sym_pair(int D, int c, int &i, int &j) {
  if (D == 2) {
    i = c == 2 ? 1 : 0;
    j = c == 0 ? 0 : 1;
  } else {
    const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
    i = ii[c];
    j = jj[c];
  }
}

// entry (r, s) of the symmetric unit tensor of component c
HDG_HD double sym_unit(int D, int c, int r, int s) {
  int i, j;
  sym_pair(D, c, i, j);
  return ((r == i && s == j) || (r == j && s == i)) ? 1.0 : 0.0;
}

// Everything the cell kernels read, as plain device pointers.
struct CellArgs {
  int D, k, nk, nfd, ni, nf, n, nqv, ncells;
  int phys, nsym, nfs;  // physics, symmetric-tensor components, scalar facet nodes
  double young;         // elasticity: Young's modulus (kappa holds the Poisson ratio)
  const double *M, *G, *F, *H, *L, *qxi, *qw, *qphi;  // reference tables
  const double *origin, *jac, *kappa;                // per cell
  const int *cell_facets, *facet_cell;               // topology
  const int *facet_dofs;
  double tau;
  int stab_mode, problem;
  int axis;  // every cell Jacobian is diagonal (axis-aligned cells)
};

// FP64 integration of the cell matrices/vectors (column-major n x n, n).
cudaError_t launch_integrate_fp64(const CellArgs &a, double *A, double *b,
                                  cudaStream_t s, int num_sms, long long *launches);

// General-space forms (fields with their own spaces; the tables of GsTables on
// the device).  cell: geometry, coefficients and form parameters, with qxi /
// qw / nqv the general-space quadrature.  DOFs per cell [A field of each copy
// (ncA x nA) | B field of each copy (ncB x nB) | per local facet the trace of
// each copy (ncT x nT)], component-major.
struct GsArgs {
  CellArgs cell;
  int phys, nA, nB, nT, ncA, ncB, copies, ni1, nfd1, ni, nf, nfd, n, nqv;
  int nl, simplex;  // facets per cell; simplex cells (cell_factors_simplex)
  const double *MAA, *GAB, *GBA, *FBA, *FBB, *HA, *HB, *L, *qphiA, *qphiB;
};
cudaError_t launch_integrate_gs(const GsArgs &g, double *A, double *b, cudaStream_t s, int num_sms,
                                long long *launches);
// per-cell squared L2 errors of the two bulk fields, summed over the copies (errs: ncells x 2)
cudaError_t launch_l2_errors_gs(const GsArgs &g, const double *uint, double *errs, cudaStream_t s, int num_sms,
                                long long *launches);
// FP64 condensation of caller-provided cells.  fact (ncells x ni x (n+1)) may
// be null; it receives [U11 | U12 | y] for the recovery.
cudaError_t launch_condense_fp64(int ncells, int ni, int nf, const double *A,
                                 const double *b, double *S, double *g,
                                 double *fact, int *info, cudaStream_t s,
                                 int num_sms, long long *launches);
// Map-level backward condensation (refactorises A_ii, as the reference map).
cudaError_t launch_backward_fp64(int ncells, int ni, int nf, const double *A,
                                 const double *b, const double *x, double *u,
                                 int *info, cudaStream_t s, int num_sms,
                                 long long *launches);
// Recovery from stored factors and the global skeleton solution.
cudaError_t launch_recover_fp64(const CellArgs &a, const double *fact,
                                const double *lambda, const double *dirvals,
                                double *uint, cudaStream_t s, int num_sms,
                                long long *launches);
cudaError_t launch_sum_facets(int nitems, int nfacets, int len,
                              const double *blocks, double *out, cudaStream_t s,
                              long long *launches);
// Per-cell squared L2 errors -> errs[2*ncells]
cudaError_t launch_l2_errors(const CellArgs &a, const double *uint, double *errs,
                             cudaStream_t s, int num_sms, long long *launches);

// Reference tables split into float-float pairs (hi, lo) for the mixed path.
struct MixedTables {
  const float *Mh, *Ml, *Gh, *Gl, *Fh, *Fl, *Hh, *Hl, *Lh, *Ll;
};
// Mixed precision: float-float integration -> (A_hi, A_lo), (b_hi, b_lo)
// skip_uu: leave the flux-flux block unwritten (block elimination does not
// read it); with coef (34 float2 + 1 double per cell of scratch) and D <= 3, k <= 2 (3D)
// or k <= 3 (2D) the flux rows' pressure columns are left unwritten as well
// and the entries are formed by the per-entry kernels
cudaError_t launch_integrate_mixed(const CellArgs &a, const MixedTables &T, float *Ahi, float *Alo,
                                   float *bhi, float *blo, cudaStream_t s, int num_sms,
                                   long long *launches, bool skip_uu = false, float2 *coef = nullptr);
cudaError_t launch_split_fp64(size_t count, const double *x, float *hi, float *lo, cudaStream_t s,
                              int num_sms, long long *launches);
// FP32 LU + one float-float refinement step; Xhi/Xlo (ncells x ni x (nf+1)) may be null
size_t condense_mixed_smem(int ni, int nf);
cudaError_t launch_condense_mixed(int ncells, int ni, int nf, const float *Ahi, const float *Alo,
                                  const float *bhi, const float *blo, double *S, double *g,
                                  float *Xhi, float *Xlo, int *info, cudaStream_t s, int num_sms,
                                  long long *launches);
// Darcy block elimination in float-float (HDG_PREC_FF_BLOCK)
bool ffblock_supported(int D, int k);
// the per-facet coupled interior rows the elimination runs over (lat: the
// Q_k node lattice, nk x D; axis: every cell axis-aligned)
size_t ffblock_pattern_ints(int D, int k);
void ffblock_pattern(int D, int k, const int *lat, bool axis, int *out);
// per cell 10 doubles: 1/m and the panel coefficients cg[e][d]/m (cell_y_coef)
cudaError_t launch_inv_mass_scale(const CellArgs &a, double *coef, cudaStream_t s, long long *launches);
// MG_h, MG_l: M^{-1} G_e (D x nk x nk, float-float)
cudaError_t launch_condense_ffblock(int D, int k, int ncells, const float *Ahi, const float *Alo,
                                    const float *bhi, const float *blo, const float *Minv_h,
                                    const float *Minv_l, const float *MG_h, const float *MG_l, const int *pat,
                                    const double *coef, double *S, double *g, float *Xhi, float *Xlo, int *info,
                                    cudaStream_t s, int num_sms, long long *launches);
// Two-field block elimination with L2 panels (k_condense_l2block.cu):
// elasticity (all built orders) and Darcy cells beyond the shared-memory
// block elimination; float-float or FP64
struct L2BlockArgs {
  int ncells;
  const void *A0, *A1, *b0, *b1;  // cell blocks: FP64 in A0/b0, or (hi, lo) float arrays
  const void *Minv0, *Minv1;      // reference mass inverse, the same way
  CellArgs cell;
  double *S, *g;
  void *X0, *X1;  // recovery X = A_ii^{-1} [A_if | b_i] (ni x (nf+1)), the same way; may be null
  int *info;
  void *scratch;   // per-CTA panels (and the fused kernel's cell block), then the per-cell factors
  const void *prep;  // set by the launcher: the per-cell factors in the scratch
  MixedTables Tb;  // float-float reference tables (fused float-float integration)
  // sparse reference products M^{-1} G_e, M^{-1} H_F: index lists (ref_idx)
  // and values (ref_v0/ref_v1: FP64, or (hi, lo) float arrays)
  const int *ref_idx;
  const void *ref_v0, *ref_v1;
  int off_cidx, off_rptr, off_ridx, off_hptr, off_hidx;  // in ref_idx
  int voff_c, voff_r, voff_h, voff_hd;                   // in the values
};
struct L2BlockLaunch {
  bool elasticity;
  int D, k;
  bool fp64;
  bool fused;  // integrate each cell into its CTA's slot instead of reading A, b from HBM
  int nqv;     // quadrature points (the fused kernel's shared memory)
  size_t smem_optin;
  int num_sms;
  size_t scratch_bytes;        // bytes at args.scratch
  size_t *scratch_bytes_out;   // receives the bytes the launch needs (may be null)
  bool dry_run;                // only size the scratch
};
bool l2block_supported(bool elasticity, int D, int k);
cudaError_t launch_condense_l2block(const L2BlockArgs &args, const L2BlockLaunch &L, cudaStream_t s,
                                    long long *launches);
// u = y - X_f x_f from an FP64 X of the block elimination
cudaError_t launch_recover_x64(const CellArgs &a, const double *X, const double *lambda, const double *dirvals,
                               double *uint, cudaStream_t s, int num_sms, long long *launches);
cudaError_t launch_recover_mixed(const CellArgs &a, const float *Xhi, const float *Xlo,
                                 const double *lambda, const double *dirvals, double *uint,
                                 cudaStream_t s, int num_sms, long long *launches);

// Skeleton side --------------------------------------------------------------
struct AssembleArgs {
  int nf, nfd, nl, nblockrows, ncells;
  int64_t nblocks;
  const int64_t *blk_off;
  const int *blk_rowlen, *blk_src, *br_row0, *br_src;
  const int *dir_cells;
  int ndir_cells;
  const int *cell_facets, *facet_dofs;
  const double *dirvals;
};
cudaError_t launch_assemble(const AssembleArgs &a, const double *S,
                            const double *g, double *glift, double *val,
                            double *rhs, cudaStream_t s, int num_sms,
                            long long *launches);

struct PcgArgs {
  int n, nfd, nblockrows;
  const int64_t *rowptr;
  const int *colind;
  const double *val;   // FP64 skeleton matrix values
  const float *val32;  // FP32 copy used by the SpMV when non-null
  const double *rhs;
  double *Binv, *x, *r, *z, *p, *p2, *q, *partials, *scal;
  unsigned int *counter;  // last-CTA arrival counter (0 between launches)
  int nparts;
  const int *diag_blk;
  const int64_t *blk_off;
  const int *blk_rowlen;
  double sign;
  int max_rowlen;  // longest skeleton row (at most 11 blocks: the SpMV's staged tile)
  int tile_ctas;   // CTAs of the SpMV (tiles of whole block rows; at most 8 per SM)
};
cudaError_t launch_pcg_setup(const PcgArgs &a, double rtol, cudaStream_t s,
                             int num_sms, long long *launches);
// two PCG iterations (the double-buffered p returns to its starting buffer)
cudaError_t launch_pcg_iteration_pair(const PcgArgs &a, cudaStream_t s, int num_sms,
                                      long long *launches);
// one skeleton SpMV q = sign*A p (+ its dot product), as launched inside PCG
cudaError_t launch_spmv(const PcgArgs &a, cudaStream_t s, long long *launches);
// facet block sizes the PCG kernels are instantiated for
bool pcg_supports_nfd(int nfd);
// (facets per cell, DOFs per facet) the skeleton assembly is instantiated for
bool assemble_supports(int nl, int nfd);

// Inner FP32 PCG of the mixed-precision skeleton solve (solves M e = rhs,
// M = sign*A, with FP32 values and vectors; dot products in float-float).
// The facet-block-Jacobi preconditioner is applied by symmetric scaling: with
// D_f = L_f L_f^T the Cholesky factor of each free facet's diagonal block and
// W = blockdiag(L_f^{-1}), CG runs on M^ = W M W^T (unit diagonal blocks) for
// y = W^{-T} e with right-hand side W rhs -- the same iterates as PCG with
// the preconditioner D^{-1}, without reading D^{-1} every iteration (z = r).
// M^ is applied unassembled: per cell the facet blocks above the diagonal of
// W_a sign*(S_c + S_c^T)/2 W_b^T in FP32, streamed with bulk async copies;
// the two cells of a facet are summed in the update kernel, which adds p for
// the diagonal blocks (their sum over a facet's cells is the identity).
struct Pcg32Args {
  int n, nfd, nblockrows;
  const double *W;    // nblockrows x nfd x nfd, row-major lower-triangular L_f^{-1}
  const double *rhs;  // inner right-hand side (the outer residual, M frame, unscaled)
  float *x, *r, *z, *p, *p2;  // z aliases r (identity preconditioner in the scaled frame)
  double *partials, *scal;
  unsigned int *counter;
  int nparts;             // grid of the vector kernels
  int ncells, nl, rec;    // rec: floats per cell record
  const float *blocks;    // ncells x rec
  const int *cell_blk;    // ncells x nl: 2*block row + (cell owns the facet), -1 on Dirichlet facets
  float *qc;              // nblockrows x 2 x nfd: the owner cell's product M^_c p_c on the block
                          // row, then the other cell's (zero where the facet has one cell)
  int nstage, ctas;       // pipeline depth and grid of the streaming kernel
  unsigned int *error;    // set to 1 when a bulk copy never completed
  int uctas;              // grid of the update kernel (partials: 2 x uctas)
};
// The inner FP32 PCG as one cooperative launch (k_pcg32_persistent.cu):
// grid, ring depth and dynamic shared memory for this shape (grid 0: not
// available), then the launch of up to iter_cap iterations (stops at
// SC_DONE; a.nstage must be the configured depth).  Uses counter[2],
// counter[3] (zeroed before the first launch) for its grid barriers and
// partials[0 .. 3 grid).
int pcg32_persistent_config(int nl, int nfd, size_t smem_optin, int num_sms, int want, int *nstage, size_t *smem);
cudaError_t launch_pcg32_persistent(const Pcg32Args &a, int grid, size_t smem, int iter_cap, cudaStream_t s,
                                    long long *launches);
// threads per CTA of the PCG vector kernels (kPcgThreads on the device side)
// and the longest skeleton row their FP64 SpMV stages (kMaxRowLen)
constexpr int kPcgThreadsHost = 256;
constexpr int kMaxSkeletonRowLen = 304;
// blocks in a skeleton row (a facet, the other facets of its two cells)
constexpr int kSkeletonRowBlocks = 11;
// CTAs for the FP64 CSR kernels that take tiles of kPcgThreadsHost / nfd
// whole block rows: at most 8 per SM (their partials fit 8 per SM), with
// the tiles spread evenly (every CTA the same count, up to one)
inline int csr_tile_ctas(int nblockrows, int nfd, int num_sms) {
  const long long br = kPcgThreadsHost / nfd;
  const long long tiles = (nblockrows + br - 1) / br;
  const long long cap = 8LL * num_sms;
  const long long per = (tiles + cap - 1) / cap;
  const long long g = per > 0 ? (tiles + per - 1) / per : 1;
  return g < 1 ? 1 : (int)g;
}
// Cell-operator layout: threads per cell, cells per CTA stage, floats per record.
HDG_HD constexpr int cellop_tpc(int nf) { return nf <= 8 ? 8 : nf <= 16 ? 16 : ((nf + 31) / 32) * 32; }
HDG_HD constexpr int cellop_cps(int nf) { return cellop_tpc(nf) >= 256 ? 1 : 256 / cellop_tpc(nf); }
// A cell record holds the nl (nl - 1) / 2 blocks (a, b), a < b, of the scaled
// cell operator: the assembled diagonal blocks of the scaled operator are the
// identity, so no cell stores its diagonal blocks.
HDG_HD constexpr int cellop_blocks(int nl) { return nl * (nl - 1) / 2; }
// Floats from one block of a record to the next: nfd^2, padded where that
// spreads the SpMV's shared-memory reads over more banks (3D k = 2 Darcy
// blocks: 85 instead of 81, about 1.5 instead of 2.1 wavefronts per load in a
// model of the kernel's access pattern; 27-DOF elasticity blocks: 731).
HDG_HD constexpr int cellop_bstride(int nfd) { return nfd == 9 ? 85 : nfd == 27 ? 731 : nfd * nfd; }
HDG_HD constexpr int cellop_rec(int nl, int nfd) { return (cellop_blocks(nl) * cellop_bstride(nfd) + 3) / 4 * 4; }
bool cellop_supported(int nl, int nfd);
// pipeline depth and grid for the streaming kernel (sets its shared-memory limit)
cudaError_t cellop_configure(int nl, int nfd, size_t smem_optin, int num_sms, int *nstage, int *ctas);
// packs sign*(S_c + S_c^T)/2 (column-major FP64 cell blocks) into cell records
// W = blockdiag(L_f^{-1}) from the assembled FP64 diagonal blocks sign*D_f = L_f L_f^T (a block
// that is not positive definite gets the identity)
cudaError_t launch_block_chol_inv(const PcgArgs &a, double *W, cudaStream_t s, int num_sms, long long *launches);
// the scaled FP32 cell records: per cell the upper facet blocks of W_a sign*(S_c + S_c^T)/2 W_b^T
cudaError_t launch_pack_cell_blocks(int ncells, int nl, int nfd, double sign, const double *S, const int *cell_blk,
                                    const double *W, float *out, size_t smem_optin, cudaStream_t s, int num_sms,
                                    long long *launches);
// Outer FP64 refinement: x, r = sign*rhs - M x with the FP64 matrix.
struct OuterArgs {
  int n, nfd, nblockrows;
  const int64_t *rowptr;
  const int *colind;
  const double *val;
  const double *rhs;
  double *x, *r;
  double *partials, *scal;  // scal[0] = |c|^2, scal[1] = |r|^2
  unsigned int *counter;
  int nparts;
  double sign;
  const double *W;  // the inner frame's scaling (x += W^T y), or null (x += y)
  int max_rowlen;   // longest skeleton row (at most 11 blocks: the residual's staged tile)
  int tile_ctas;    // CTAs of the residual (tiles of whole block rows; at most 8 per SM)
};
cudaError_t launch_pcg32_init(const Pcg32Args &a, double eta, cudaStream_t s, long long *launches);
cudaError_t launch_pcg32_iteration_pair(const Pcg32Args &a, cudaStream_t s, long long *launches);
// residual replacement keeping the search direction (reliable update)
cudaError_t launch_pcg32_replace(const Pcg32Args &a, double eta, cudaStream_t s, long long *launches);
// one unassembled SpMV (+ its dot product) as launched inside the inner PCG
cudaError_t launch_pcg32_spmv(const Pcg32Args &a, cudaStream_t s, long long *launches);
cudaError_t launch_outer_init(const OuterArgs &a, cudaStream_t s, long long *launches);
// x += W^T e (x += e without W), then r = c - M x and |r|^2
cudaError_t launch_outer_update(const OuterArgs &a, const float *e, cudaStream_t s, long long *launches);
// x = xsaved + sign * x (x holds an FP64 correction e with A e = sign (c - A xsaved))
cudaError_t launch_outer_combine(const OuterArgs &a, const double *xsaved, cudaStream_t s, long long *launches);
// Size-class batching: one persistent fused integrate -> condense launch over
// the cells of several problems of one (D, k) class.
struct BatchProblem {
  CellArgs a;
  MixedTables T;
  const float *Mh, *Ml;    // M_ref^{-1} (hi, lo), block elimination
  const float *MGh, *MGl;  // M_ref^{-1} G_e (hi, lo)
  const int *ffpat;        // coupling pattern of the block elimination (ffblock_pattern)
  double *S, *g;         // condensed blocks and vectors
  float *Xh, *Xl;        // float-float recovery pairs, block elimination
  double *fact;          // FP64 recovery factors [U11 | U12 | y]
  int *info;             // per cell
  long long first;       // first item (cell) of this problem in the class
};
struct FusedLaunch {
  int precision, D, k, n, ni, nf, nqv;
  int tpc;                     // threads per cell: 32, 64, 128 or 256 (256/tpc cells per CTA)
  const BatchProblem *probs;   // device array, ordered by `first`
  int nprob;
  long long total;             // cells in the class
  float *scratch;              // block elimination: per-group cell slots
  size_t scratch_bytes;
  size_t *scratch_bytes_out;   // receives the slots' size for this configuration (may be null)
  bool dry_run;                // size the launch only
  int *bad;                    // per problem: largest zero-pivot index (0 = ok)
  int num_sms;
  size_t smem_optin;
};
bool fused_batch_supported(int D, int k, int precision);
cudaError_t launch_fused_batch(const FusedLaunch &L, cudaStream_t s, long long *launches);

// Newton path: b_c <- A_c x_c - b_c for the iterate (interior values cell-major,
// free skeleton values), rmax[0] / rmax[1] = max |r| over interior rows / the
// assembled free skeleton rows; and x <- x - dx.
cudaError_t launch_newton_residual(const CellArgs &a, const AssembleArgs &as, const double *A, double *b,
                                   const double *xint, const double *xskel, const double *dirvals, double *rmax,
                                   cudaStream_t s, int num_sms, long long *launches);
cudaError_t launch_newton_update(size_t count, double *x, const double *dx, cudaStream_t s, int num_sms,
                                 long long *launches);

// Linear elasticity HDG cells: blocks in FP64 (A, b) or as float-float pairs
// (with Tb: every entry computed in float-float from the float-float tables;
// without: computed in FP64 and split), and the stress / displacement L2 error
// contributions per cell (errs: 2 per cell).  skip_ss: the stress-stress block
// is not written (the block elimination never reads it).
cudaError_t launch_integrate_elasticity(const CellArgs &a, double *A, double *b, float *Ahi, float *Alo, float *bhi,
                                        float *blo, cudaStream_t s, int num_sms, long long *launches,
                                        bool skip_ss = false, const MixedTables *Tb = nullptr);
cudaError_t launch_l2_errors_elasticity(const CellArgs &a, const double *uint, double *errs, cudaStream_t s,
                                        int num_sms, long long *launches);

// dense LU solve of a CSR system (small n), one CTA
cudaError_t launch_dense_solve(int n, const int64_t *rowptr, const int *colind,
                               const double *val, const double *rhs, double *work,
                               double *x, int *info, cudaStream_t s,
                               long long *launches);

}  // namespace hdg
