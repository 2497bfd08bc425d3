// hdg_internal.h -- internal types of libgridaphybrid_gb300 (not installed).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/hdg_gb300.h"

namespace hdg {

constexpr int kMaxD = 3;
constexpr int kMaxK = 4;

// Device allocations made through DBuf::reserve since the library was loaded
// (all contexts), reported by hdg_device_allocations.
extern std::atomic<long long> g_device_allocs;

// ---------------------------------------------------------------------------
// Where a caller's pointer lives, seen from a context on `ctx_device`.
// ---------------------------------------------------------------------------
enum class PtrPlace { Host, Device, OtherDevice };
// The placement rule on cudaPointerAttributes' (type, device): device memory
// of the context's GPU and managed memory are used in place, host memory is
// staged, device memory of another GPU is refused (the kernels would fault on
// it without peer access).
inline PtrPlace ptr_place_rule(int memory_type, int ptr_device, int ctx_device) {
  if (memory_type == cudaMemoryTypeManaged) return PtrPlace::Device;
  if (memory_type == cudaMemoryTypeDevice)
    return ptr_device == ctx_device ? PtrPlace::Device : PtrPlace::OtherDevice;
  return PtrPlace::Host;
}
inline PtrPlace ptr_place(const void *p, int ctx_device, int *ptr_device = nullptr) {
  if (!p) return PtrPlace::Host;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return PtrPlace::Host;
  }
  if (ptr_device) *ptr_device = at.device;
  return ptr_place_rule((int)at.type, at.device, ctx_device);
}

// Makes `device` current for the scope and gives the caller's current device
// back on exit (host frameworks track their own current device).
struct DeviceGuard {
  int prev = -1;
  cudaError_t status = cudaSuccess;
  explicit DeviceGuard(int device) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
    }
    if (prev != device) status = cudaSetDevice(device);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard &) = delete;
  DeviceGuard &operator=(const DeviceGuard &) = delete;
};

// ---------------------------------------------------------------------------
// Device buffer owned by a context or problem.
// ---------------------------------------------------------------------------
// With `stream` set, allocation and release are stream-ordered
// (cudaMallocAsync / cudaFreeAsync from the device's pool), so growing or
// freeing one problem's buffers does not synchronise the device while other
// streams run; every use of the buffer must then be ordered after the
// allocation on that stream (the library uses one stream per context).
struct DBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void release() {
    if (ptr) {
      if (stream)
        cudaFreeAsync(ptr, stream);
      else
        cudaFree(ptr);
    }
    ptr = nullptr;
    bytes = 0;
  }
  // grows (never shrinks); returns cudaSuccess or the allocation error
  cudaError_t reserve(size_t nbytes) {
    if (nbytes <= bytes && ptr) return cudaSuccess;
    release();
    if (nbytes == 0) nbytes = 16;
    cudaError_t e = stream ? cudaMallocAsync(&ptr, nbytes, stream) : cudaMalloc(&ptr, nbytes);
    if (e != cudaSuccess) {
      ptr = nullptr;
      return e;
    }
    g_device_allocs.fetch_add(1, std::memory_order_relaxed);
    bytes = nbytes;
    return cudaSuccess;
  }
  template <typename T>
  T *as() const {
    return static_cast<T *>(ptr);
  }
};

// ---------------------------------------------------------------------------
// Reference-element tables (host FP64).  The quadrature sums over reference
// points are contracted once; on an affine cell with cell-constant
// coefficients the cell integrals are these tables times per-cell scalars.
// ---------------------------------------------------------------------------
struct RefTables {
  int D = 0, k = 0, nk = 0, nfd = 0, ni = 0, nf = 0, n = 0, n1 = 0, nqv = 0;
  // physics (HDG_PHYSICS_*), symmetric-tensor components (elasticity), scalar
  // facet nodes; nfd = DOFs per facet = (facet components) x nfs
  int phys = 0, nsym = 0, nfs = 0;
  std::vector<int> lat;    // nk x D cell node lattice (Gridap node order)
  std::vector<int> flat;   // nfd x (D-1) facet node lattice
  std::vector<double> M;   // nk x nk      int phi_a phi_b
  std::vector<double> G;   // D x nk x nk  int d_e phi_a phi_b
  std::vector<double> F;   // 2D x nk x nk int_F phi_a phi_b (unit facet measure)
  std::vector<double> H;   // 2D x nk x nfs int_F phi_a mu_b
  std::vector<double> L;   // nfs x nfs    int_F mu_a mu_b
  std::vector<double> qxi; // nqv x D volume points
  std::vector<double> qw;  // nqv
  std::vector<double> qphi;// nqv x nk
  std::vector<double> Minv;// nk x nk inverse of M (block elimination path)
  // M^{-1} G_e (D x nk x nk) and M^{-1} H_lf (2D x nk x nfs), entries below
  // 1e-12 of the matrix's largest set to zero: on the tensor-product cell they
  // vanish exactly (a node couples only along one lattice line / to its facet line)
  std::vector<double> MG, MH;
};
// The sparse reference operators of the L2-panel block elimination as
// column lists (MG by column b, MG by row a, MH by column): int data
// [cptr (D nk + 1) | cidx | rptr (D nk + 1) | ridx | hptr (2D nfs + 1) | hidx]
// and the values in the same order, followed by MH dense (2D x nk x nfs).
struct L2RefHost {
  std::vector<int> idx;
  std::vector<double> val;
  int off_cidx = 0, off_rptr = 0, off_ridx = 0, off_hptr = 0, off_hidx = 0;   // in idx
  int voff_c = 0, voff_r = 0, voff_h = 0, voff_hd = 0;                         // in val
};
void build_l2_ref(const RefTables &t, L2RefHost &r);
int build_ref_tables(int D, int k, RefTables &t, int phys = 0);

// Lagrange lattice of Q_k on [0,1]^D in Gridap's node order (lattice index i
// is the coordinate i/k), the 1D Lagrange polynomial of node i, and
// Gauss-Legendre points on [0,1].
std::vector<int> node_lattice(int D, int k);
void lagrange1d(int k, int i, double x, double &v, double &dv);
void gauss01(int np, std::vector<double> &x, std::vector<double> &w);

// A scalar polynomial basis on the reference cube [0,1]^d: Q_k (tensor
// Lagrange in Gridap's node order; the constant for k = 0) or P_k (total
// degree <= k, Lagrange at the simplex lattice points i/k; the constant for
// k = 0), or a tensor Lagrange basis with an order per dimension.
constexpr int kBasisQ = 0;
constexpr int kBasisP = 1;
// first bulk field of the Darcy form only: Raviart-Thomas RT_k on the box,
// component d in the tensor space of order k+1 along d and k across
constexpr int kBasisRT = 2;
struct ScalarBasis {
  int d = 0, kind = kBasisQ, k = 0, nb = 0;
  bool aniso = false;         // tensor Lagrange with an order per dimension (ko)
  int ko[kMaxD] = {0, 0, 0};
  std::vector<int> lat;       // Q: nb x d lattice indices
  std::vector<int> mono;      // P: nb x d monomial exponents
  std::vector<double> coef;   // P: nb x nb, phi_a = sum_m coef[a nb + m] x^mono_m
  std::vector<double> nodes;  // nb x d nodal points
  int init(int dim, int basis_kind, int order);
  // tensor Lagrange of order orders[e] along dimension e (equispaced nodes i/m,
  // the midpoint for order 0), first dimension fastest
  int init_aniso(int dim, const int *orders);
  // values (nb) and reference gradients (nb x d, may be null) at xi
  void eval(const double *xi, double *val, double *grad) const;
};

// Reference tables of a general-space form (fields with their own spaces):
// A the first bulk field (Darcy flux / elasticity stress), B the second
// (pressure / displacement), T the trace on facets.  spaces[7] = {kindA, kA,
// kindB, kB, kindT, kT, pm}; pm: P_m of the displacement in the tau terms.
// All tables FP64, packed in `packed` at the offsets below (in doubles); the
// A tables hold one slab per component c of the first field (nA functions
// each; the slabs are equal unless the field is RT_k):
//   MAA  ncA x nA x nA          int phiA_a phiA_b
//   GAB  ncA x D x nA x nB      int d_e phiA_a phiB_b
//   GBA  ncA x D x nB x nA      int d_e phiB_b phiA_a
//   FBA  ncA x 2D x nB x nA     int_F phiB_b phiA_a       (unit facet measure)
//   FBB  2D x nB x nB           int_F phiB_b phiB_c, or with pm H_B L^{-1} H_B^T
//   HA   ncA x 2D x nA x nT     int_F phiA_a mu_m
//   HB   2D x nB x nT           int_F phiB_b mu_m
//   L    nT x nT                int_F mu_m mu_n
//   qxi (nqv x D), qw (nqv), qphiA (ncA x nqv x nA), qphiB (nqv x nB)
// copies > 1: that many decoupled copies of the form, each with its own
// fields and its own skeleton field (a skeleton system of several fields).
// Cell DOFs [A of copy 0 .. A of copy c-1 | B of copy 0 .. | per local facet:
// the trace DOFs of copy 0, copy 1, ..].
struct GsTables {
  int D = 0, phys = 0, pm = 0, copies = 1;
  bool simplex = false;  // cells are simplices (D + 1 facets): the reference simplex's tables and rules
  int nl = 0;            // facets per cell
  int spaces[7] = {0, 0, 0, 0, 0, 0, 0};
  ScalarBasis A[kMaxD > 6 ? kMaxD : 6], B, T;  // A: one basis per component
  int ncA = 0, ncB = 0, ncT = 0, nA = 0, nB = 0, nT = 0, ni = 0, nf = 0, nfd = 0, n = 0, n1 = 0, nqv = 0;
  int ni1 = 0, nfd1 = 0;  // one copy: interior DOFs, DOFs per facet
  std::vector<double> packed;
  int oMAA = 0, oGAB = 0, oGBA = 0, oFBA = 0, oFBB = 0, oHA = 0, oHB = 0, oL = 0, oqxi = 0, oqw = 0, oqphiA = 0,
      oqphiB = 0;
};
int build_gs_tables(int D, int phys, const int *spaces, int copies, GsTables &t, std::string &err,
                    bool simplex = false);

// Offsets (in doubles) of each table inside the packed device table buffer.
struct TableOffsets {
  int M, G, F, H, L, qxi, qw, qphi, total;
};
TableOffsets pack_tables(const RefTables &t, std::vector<double> &packed);
// The same tables as float-float pairs: for each table its hi then lo floats,
// at the offsets returned (in floats).
struct TableOffsetsF {
  int Mh, Ml, Gh, Gl, Fh, Fl, Hh, Hl, Lh, Ll, total;
};
TableOffsetsF pack_tables_ff(const RefTables &t, std::vector<float> &packed);

// ---------------------------------------------------------------------------
// Mesh + skeleton space + assembly pattern (host side, built once).
// ---------------------------------------------------------------------------
struct HostMesh {
  int D = 0, k = 0, ncells = 0, nfacets = 0, nfd = 0, nfree = 0, ndir = 0;
  int nl = 0;            // facets per cell: 2 D (boxes) or D + 1 (simplices)
  bool simplex = false;
  bool cartesian = false;
  int cells[kMaxD] = {0, 0, 0};
  double domain[2 * kMaxD] = {0, 0, 0, 0, 0, 0};
  std::vector<double> origin;     // ncells x D
  std::vector<double> jac;        // ncells x D x D (column-major per cell)
  bool axis = false;              // every jac is diagonal
  std::vector<int> cell_facets;   // ncells x nl
  std::vector<int> facet_dofs;    // nfacets x nfd
  std::vector<int> facet_cell;    // nfacets x 2 : cells around (first = owner), -1
  std::vector<int> facet_lface;   // nfacets x 2 : local facet index in that cell
  std::vector<int> facet_first_dof; // nfacets: first free DOF or -1
};
// ncomp: components of the facet field (1 scalar trace, D displacement trace);
// nfd > 0 sets the DOFs per facet directly (general-space trace bases)
int build_cartesian_mesh(int D, const int *cells, const double *domain, int k,
                         HostMesh &m, std::string &err, int ncomp = 1, int nfd = 0);
int finish_mesh(HostMesh &m, std::string &err);  // derives facet_cell etc.
// simplexify of the Cartesian mesh: every box split into D! simplices around
// its diagonal from the lowest to the highest vertex (Kuhn), nfd DOFs per facet
int build_simplex_mesh(int D, const int *cells, const double *domain, int nfd, HostMesh &m, std::string &err);

// Skeleton CSR pattern and the block maps used by the deterministic gather.
struct HostPattern {
  int nrows = 0;
  int64_t nnz = 0;
  int nblockrows = 0;                // free facets
  int64_t nblocks = 0;
  std::vector<int64_t> rowptr;       // nrows+1
  std::vector<int32_t> colind;       // nnz
  std::vector<int> br_facet;         // block row -> facet
  std::vector<int> br_row0;          // block row -> first row (free DOF)
  std::vector<int> br_src;           // block row -> 2 x (cell*2D + lf) or -1 (rhs)
  std::vector<int64_t> blk_off;      // block -> val offset of entry (0,0)
  std::vector<int> blk_rowlen;       // block -> row length of its block row
  std::vector<int> blk_src;          // block -> 2 x (cell*(2D)^2 + lf_row*2D + lf_col) or -1
  std::vector<int> diag_blk;         // block row -> index of its diagonal block
  std::vector<int> dir_cells;        // cells touching a Dirichlet DOF
  std::vector<int> cell_blk;         // cell x lf -> 2*block row + owns, -1 (Dirichlet)
  int max_rowlen = 0;                // longest skeleton row
};
int build_pattern(const HostMesh &m, HostPattern &p, std::string &err);

// Whether the library has kernels for this (D, k, precision, solver) on a
// device with `smem_optin` bytes of shared memory per CTA; `why` says what is missing.
bool shape_supported(int D, int k, int precision, int solver, size_t smem_optin, std::string &why);
// Upper bound of the device bytes of a Cartesian problem n^D, order k, solved
// with (precision, solver).
double footprint_bound(int D, int n, int k, int precision, int solver);

}  // namespace hdg

// ---------------------------------------------------------------------------
// Public opaque types.
// ---------------------------------------------------------------------------
struct hdg_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  long long launches = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  bool coop = false;       // cooperative launches (the persistent inner PCG)
  int persistent_pcg = 0;  // use them when the grid can be co-resident (opt-in)
  hdg::DBuf scratch[6];  // Map-level staging buffers
  cudaEvent_t ev[8] = {nullptr};
  cudaEvent_t user_ev[4] = {nullptr};
  int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
};

struct hdg_problem {
  hdg_context *ctx = nullptr;
  hdg::HostMesh mesh;
  hdg::RefTables tab;
  hdg::TableOffsets toff{};
  hdg::TableOffsetsF toff_f{};
  hdg::DBuf d_tabf;
  hdg::HostPattern pat;
  int stab_mode = HDG_STAB_TEXTBOOK;
  int problem = HDG_PROBLEM_LINEAR;
  double tau = 1.0;
  int physics = HDG_PHYSICS_DARCY;
  double young = 1.0;  // elasticity: Young's modulus (the per-cell coefficient is the Poisson ratio)
  bool form_set = false, assembled = false, solved = false, recovered = false;
  int precision = HDG_PREC_FP64;
  double timings[5] = {0, 0, 0, 0, 0};
  int last_iters = 0;
  double last_relres = 0.0;
  // device state
  hdg::DBuf d_tab, d_origin, d_jac, d_cell_facets, d_facet_dofs, d_facet_cell;
  hdg::DBuf d_kappa, d_dirvals;
  hdg::DBuf d_A, d_b, d_S, d_g, d_fact, d_info, d_aux;
  hdg::DBuf d_rowptr, d_colind, d_val, d_rhs;
  hdg::DBuf d_br_row0, d_br_src, d_blk_off, d_blk_rowlen, d_blk_src, d_diag_blk,
      d_dir_cells;
  hdg::DBuf d_Binv, d_x, d_r, d_z, d_p, d_p2, d_q, d_partials, d_scal, d_counter;
  // mixed-precision skeleton solve: the scaled FP32 operator as symmetric
  // cell blocks, its cell map, the products by block row, the scaling
  // W = blockdiag(L_f^{-1}) (FP64), inner vectors (x, r, p, p2), outer scalars
  hdg::DBuf d_cellop, d_cell_blk, d_qc, d_W, d_v32, d_scal2;
  // block-elimination path: M_ref^{-1} as (hi, lo) floats then FP64, 1/m per
  // cell, the elasticity kernel's per-CTA scratch panels
  hdg::DBuf d_minv, d_invm, d_escratch, d_ffpat;
  // the L2-panel kernel's sparse reference products: index lists, values
  // ((hi, lo) floats then FP64) and their offsets
  hdg::DBuf d_l2ref_idx, d_l2ref_val;
  hdg::L2RefHost l2ref;
  // the elasticity cell blocks of this assembly are condensed by block
  // elimination (float-float, or FP64 when the dense block exceeds shared memory)
  bool eblock = false;
  // ... integrating each cell into the kernel's L2 slot (no cell blocks in HBM)
  bool l2_fused = false;
  cudaGraphExec_t pcg32_graph = nullptr;
  int cellop_nstage = 0, cellop_ctas = 0;  // streaming-kernel pipeline depth and grid
  // FP64 residual refinement of the FP32 skeleton solve: the inner reduction
  // between FP64 residuals, and whether the search direction survives them
  double refine_delta = 3e-2;
  int refine_keep = 1;
  int last_outer = 0;
  int last_fp64_iters = 0;  // FP64 correction iterations of the last refined solve (0: none needed)
  hdg::DBuf d_uint, d_errs;
  // Newton path: the iterate [interior cell-major | free skeleton], the
  // residual norms, and zero Dirichlet data for the corrections
  hdg::DBuf d_newton, d_rmax, d_dirzero;
  bool zero_dirichlet = false;
  // general-space form (fields with their own spaces, hdg_problem_create_cartesian_spaces)
  bool gs = false;
  hdg::GsTables gst;
  hdg::DBuf d_gstab;
  hdg::DBuf h_pinned;  // host staging
  cudaGraphExec_t pcg_graph = nullptr;
  int pcg_graph_chunk = 0;
  // every device buffer of the problem (not the pinned host staging)
  std::vector<hdg::DBuf *> device_buffers() {
    return {&d_tabf, &d_tab, &d_origin, &d_jac, &d_cell_facets, &d_facet_dofs, &d_facet_cell, &d_kappa,
            &d_dirvals, &d_A, &d_b, &d_S, &d_g, &d_fact, &d_info, &d_aux, &d_rowptr, &d_colind, &d_val,
            &d_rhs, &d_br_row0, &d_br_src, &d_blk_off, &d_blk_rowlen, &d_blk_src, &d_diag_blk, &d_dir_cells,
            &d_Binv, &d_x, &d_r, &d_z, &d_p, &d_p2, &d_q, &d_partials, &d_scal, &d_counter, &d_cellop,
            &d_cell_blk, &d_qc, &d_W, &d_v32, &d_scal2, &d_minv, &d_invm, &d_escratch, &d_ffpat, &d_l2ref_idx, &d_l2ref_val, &d_uint, &d_errs,
            &d_newton, &d_rmax, &d_dirzero, &d_gstab};
  }
  ~hdg_problem();
};
