// hdg_capi.cu -- the extern "C" entry points of libgridaphybrid_gb300.
// Everything numeric runs on the GPU; the host side validates arguments,
// stages host buffers, builds the mesh/pattern once per problem and drives
// the kernels on the context's stream.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <thread>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "hdg_internal.h"
#include "hdg_kernels.h"

using namespace hdg;

std::atomic<long long> hdg::g_device_allocs(0);

#define CUDA_TRY(ctx, call)                                                          \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return (ctx)->fail(e_ == cudaErrorMemoryAllocation ? HDG_ERR_NOMEM : HDG_ERR_CUDA, \
                         "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

namespace {

bool is_device_ptr(const hdg_context *ctx, const void *p) {
  return p && ptr_place(p, ctx->device) == PtrPlace::Device;
}

// HDG_ERR_INVALID when p is device memory of another GPU than the context's.
int check_ptr_device(hdg_context *ctx, const void *p) {
  int dev = -1;
  if (p && ptr_place(p, ctx->device, &dev) == PtrPlace::OtherDevice)
    return ctx->fail(HDG_ERR_INVALID, "a pointer argument is device memory of GPU %d; the context is on GPU %d",
                     dev, ctx->device);
  return HDG_OK;
}

// Device view of a caller buffer: the pointer itself when it is device memory,
// else a staging buffer (filled from host when `in`).
template <typename T>
int stage_in(hdg_context *ctx, DBuf &buf, const T *src, size_t count, const T **out) {
  if (int rc = check_ptr_device(ctx, src)) return rc;
  if (is_device_ptr(ctx, src)) {
    *out = src;
    return HDG_OK;
  }
  CUDA_TRY(ctx, buf.reserve(sizeof(T) * count));
  if (count) CUDA_TRY(ctx, cudaMemcpyAsync(buf.ptr, src, sizeof(T) * count, cudaMemcpyHostToDevice, ctx->stream));
  *out = buf.as<T>();
  return HDG_OK;
}

template <typename T>
int stage_out(hdg_context *ctx, DBuf &buf, T *dst, size_t count, T **out) {
  if (int rc = check_ptr_device(ctx, dst)) return rc;
  if (is_device_ptr(ctx, dst)) {
    *out = dst;
    return HDG_OK;
  }
  CUDA_TRY(ctx, buf.reserve(sizeof(T) * (count ? count : 1)));
  *out = buf.as<T>();
  return HDG_OK;
}

template <typename T>
int finish_out(hdg_context *ctx, const T *dev, T *dst, size_t count) {
  if (!dst || dev == dst || count == 0) return HDG_OK;
  CUDA_TRY(ctx, cudaMemcpyAsync(dst, dev, sizeof(T) * count, cudaMemcpyDeviceToHost, ctx->stream));
  return HDG_OK;
}

template <typename T>
int upload(hdg_context *ctx, DBuf &buf, const std::vector<T> &v) {
  CUDA_TRY(ctx, buf.reserve(sizeof(T) * (v.empty() ? 1 : v.size())));
  if (!v.empty())
    CUDA_TRY(ctx, cudaMemcpyAsync(buf.ptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, ctx->stream));
  return HDG_OK;
}

CellArgs cell_args(hdg_problem *pb) {
  const RefTables &t = pb->tab;
  const double *tb = pb->d_tab.as<double>();
  CellArgs a{};
  a.D = t.D;
  a.k = t.k;
  a.nk = t.nk;
  a.nfd = t.nfd;
  a.ni = t.ni;
  a.nf = t.nf;
  a.n = t.n;
  a.nqv = t.nqv;
  a.ncells = pb->mesh.ncells;
  a.M = tb + pb->toff.M;
  a.G = tb + pb->toff.G;
  a.F = tb + pb->toff.F;
  a.H = tb + pb->toff.H;
  a.L = tb + pb->toff.L;
  a.qxi = tb + pb->toff.qxi;
  a.qw = tb + pb->toff.qw;
  a.qphi = tb + pb->toff.qphi;
  a.origin = pb->d_origin.as<double>();
  a.jac = pb->d_jac.as<double>();
  a.axis = pb->mesh.axis ? 1 : 0;
  a.kappa = pb->d_kappa.ptr ? pb->d_kappa.as<double>() : nullptr;
  a.cell_facets = pb->d_cell_facets.as<int>();
  a.facet_cell = pb->d_facet_cell.as<int>();
  a.facet_dofs = pb->d_facet_dofs.as<int>();
  a.tau = pb->tau;
  a.stab_mode = pb->stab_mode;
  a.problem = pb->problem;
  a.phys = t.phys;
  a.nsym = t.nsym;
  a.nfs = t.nfs;
  a.young = pb->young;
  return a;
}

// The general-space form's tables and sizes; the cell part carries the
// geometry, coefficients and form parameters with the form's own quadrature.
GsArgs gs_args(hdg_problem *pb) {
  const GsTables &t = pb->gst;
  const double *T = pb->d_gstab.as<double>();
  GsArgs g{};
  g.cell = cell_args(pb);
  g.cell.qxi = T + t.oqxi;
  g.cell.qw = T + t.oqw;
  g.cell.nqv = t.nqv;
  g.phys = t.phys;
  g.nA = t.nA;
  g.nB = t.nB;
  g.nT = t.nT;
  g.ncA = t.ncA;
  g.ncB = t.ncB;
  g.copies = t.copies;
  g.ni1 = t.ni1;
  g.nfd1 = t.nfd1;
  g.ni = t.ni;
  g.nf = t.nf;
  g.nfd = t.nfd;
  g.n = t.n;
  g.nqv = t.nqv;
  g.nl = t.nl;
  g.simplex = t.simplex ? 1 : 0;
  g.MAA = T + t.oMAA;
  g.GAB = T + t.oGAB;
  g.GBA = T + t.oGBA;
  g.FBA = T + t.oFBA;
  g.FBB = T + t.oFBB;
  g.HA = T + t.oHA;
  g.HB = T + t.oHB;
  g.L = T + t.oL;
  g.qphiA = T + t.oqphiA;
  g.qphiB = T + t.oqphiB;
  return g;
}

MixedTables mixed_tables(hdg_problem *pb) {
  const float *t = pb->d_tabf.as<float>();
  const TableOffsetsF &o = pb->toff_f;
  MixedTables T{};
  T.Mh = t + o.Mh;
  T.Ml = t + o.Ml;
  T.Gh = t + o.Gh;
  T.Gl = t + o.Gl;
  T.Fh = t + o.Fh;
  T.Fl = t + o.Fl;
  T.Hh = t + o.Hh;
  T.Hl = t + o.Hl;
  T.Lh = t + o.Lh;
  T.Ll = t + o.Ll;
  return T;
}

// Phase launches on the problem's buffers, for the precision of the last assemble.
// General-space forms: FP64 cell blocks; for the FP32 LU + refinement they
// are integrated into the scratch and split into the (hi, lo) float pairs.
cudaError_t run_integrate_gs(hdg_problem *pb) {
  hdg_context *ctx = pb->ctx;
  const GsArgs g = gs_args(pb);
  const size_t nc = pb->mesh.ncells, n = pb->gst.n;
  if (pb->precision == HDG_PREC_FP64)
    return launch_integrate_gs(g, pb->d_A.as<double>(), pb->d_b.as<double>(), ctx->stream, ctx->num_sms,
                               &ctx->launches);
  double *A64 = pb->d_escratch.as<double>(), *b64 = A64 + nc * n * n;
  float *Ahi = pb->d_A.as<float>(), *bhi = pb->d_b.as<float>();
  cudaError_t e = launch_integrate_gs(g, A64, b64, ctx->stream, ctx->num_sms, &ctx->launches);
  if (e == cudaSuccess)
    e = launch_split_fp64(nc * n * n, A64, Ahi, Ahi + nc * n * n, ctx->stream, ctx->num_sms, &ctx->launches);
  if (e == cudaSuccess)
    e = launch_split_fp64(nc * n, b64, bhi, bhi + nc * n, ctx->stream, ctx->num_sms, &ctx->launches);
  return e;
}

cudaError_t run_integrate(hdg_problem *pb) {
  hdg_context *ctx = pb->ctx;
  if (pb->gs) return run_integrate_gs(pb);
  if (pb->eblock && pb->l2_fused) return cudaSuccess;  // integrated inside the condensation kernel
  CellArgs a = cell_args(pb);
  const size_t nc = pb->mesh.ncells, n = pb->tab.n;
  if (pb->physics == HDG_PHYSICS_ELASTICITY) {
    if (pb->precision == HDG_PREC_FP64)
      return launch_integrate_elasticity(a, pb->d_A.as<double>(), pb->d_b.as<double>(), nullptr, nullptr, nullptr,
                                         nullptr, ctx->stream, ctx->num_sms, &ctx->launches);
    float *Ahi = pb->d_A.as<float>(), *bhi = pb->d_b.as<float>();
    // float-float entries for the block elimination; FP64 entries split for the FP32 LU + refinement
    const MixedTables T = mixed_tables(pb);
    const bool ffb = pb->precision == HDG_PREC_FF_BLOCK;
    return launch_integrate_elasticity(a, nullptr, nullptr, Ahi, Ahi + nc * n * n, bhi, bhi + nc * n, ctx->stream,
                                       ctx->num_sms, &ctx->launches, ffb, ffb ? &T : nullptr);
  }
  if (pb->precision == HDG_PREC_FP64)
    return launch_integrate_fp64(a, pb->d_A.as<double>(), pb->d_b.as<double>(), ctx->stream, ctx->num_sms,
                                 &ctx->launches);
  float *Ahi = pb->d_A.as<float>(), *bhi = pb->d_b.as<float>();
  // FF_BLOCK on the shared-memory elimination: the float-float cell
  // coefficients go after the panel coefficients (10 doubles per cell)
  const bool ffb = pb->precision == HDG_PREC_FF_BLOCK;
  const bool have = ffb && !pb->eblock && pb->d_invm.bytes >= sizeof(double) * 11 * nc + sizeof(float) * 2 * 34 * nc;
  float2 *coef = have ? reinterpret_cast<float2 *>(pb->d_invm.as<double>() + 10 * nc) : nullptr;
  return launch_integrate_mixed(a, mixed_tables(pb), Ahi, Ahi + nc * n * n, bhi, bhi + nc * n, ctx->stream,
                                ctx->num_sms, &ctx->launches, ffb, coef);
}

// The L2-panel block elimination's launch description (dry_run: size only).
L2BlockLaunch l2block_launch(const hdg_problem *pb, size_t *need, bool dry_run) {
  L2BlockLaunch L{};
  L.elasticity = pb->physics == HDG_PHYSICS_ELASTICITY;
  L.fused = pb->l2_fused;
  L.nqv = pb->tab.nqv;
  L.D = pb->tab.D;
  L.k = pb->tab.k;
  L.fp64 = pb->precision == HDG_PREC_FP64;
  L.smem_optin = pb->ctx->smem_optin;
  L.num_sms = pb->ctx->num_sms;
  L.scratch_bytes = pb->d_escratch.bytes;
  L.scratch_bytes_out = need;
  L.dry_run = dry_run;
  return L;
}

cudaError_t run_condense_l2block(hdg_problem *pb) {
  hdg_context *ctx = pb->ctx;
  const size_t nc = pb->mesh.ncells, n = pb->tab.n, ni = pb->tab.ni, nf = pb->tab.nf, nk = pb->tab.nk;
  L2BlockArgs A{};
  A.ncells = (int)nc;
  A.cell = cell_args(pb);
  A.S = pb->d_S.as<double>();
  A.g = pb->d_g.as<double>();
  A.info = pb->d_info.as<int>();
  A.scratch = pb->d_escratch.ptr;
  A.Tb = mixed_tables(pb);
  {
    const L2RefHost &r = pb->l2ref;
    const size_t nv = r.val.size();
    const float *vf = pb->d_l2ref_val.as<float>();
    A.ref_idx = pb->d_l2ref_idx.as<int>();
    A.ref_v0 = pb->precision == HDG_PREC_FP64 ? (const void *)(vf + 2 * nv) : (const void *)vf;
    A.ref_v1 = pb->precision == HDG_PREC_FP64 ? nullptr : (const void *)(vf + nv);
    A.off_cidx = r.off_cidx;
    A.off_rptr = r.off_rptr;
    A.off_ridx = r.off_ridx;
    A.off_hptr = r.off_hptr;
    A.off_hidx = r.off_hidx;
    A.voff_c = r.voff_c;
    A.voff_r = r.voff_r;
    A.voff_h = r.voff_h;
    A.voff_hd = r.voff_hd;
  }
  const float *Mf = pb->d_minv.as<float>();
  if (pb->precision == HDG_PREC_FP64) {
    A.A0 = pb->d_A.ptr;
    A.b0 = pb->d_b.ptr;
    A.Minv0 = Mf + 2 * nk * nk;
    A.X0 = pb->d_fact.ptr;
  } else {
    const float *Ahi = pb->d_A.as<float>(), *bhi = pb->d_b.as<float>();
    float *Xhi = pb->d_fact.as<float>();
    A.A0 = Ahi;
    A.A1 = Ahi + nc * n * n;
    A.b0 = bhi;
    A.b1 = bhi + nc * n;
    A.Minv0 = Mf;
    A.Minv1 = Mf + nk * nk;
    A.X0 = Xhi;
    A.X1 = Xhi + nc * ni * (nf + 1);
  }
  return launch_condense_l2block(A, l2block_launch(pb, nullptr, false), ctx->stream, &ctx->launches);
}

cudaError_t run_condense(hdg_problem *pb) {
  hdg_context *ctx = pb->ctx;
  const size_t nc = pb->mesh.ncells, n = pb->tab.n, ni = pb->tab.ni, nf = pb->tab.nf;
  if (pb->eblock) return run_condense_l2block(pb);
  if (pb->precision == HDG_PREC_FP64)
    return launch_condense_fp64((int)nc, (int)ni, (int)nf, pb->d_A.as<double>(), pb->d_b.as<double>(),
                                pb->d_S.as<double>(), pb->d_g.as<double>(), pb->d_fact.as<double>(),
                                pb->d_info.as<int>(), ctx->stream, ctx->num_sms, &ctx->launches);
  float *Ahi = pb->d_A.as<float>(), *bhi = pb->d_b.as<float>(), *Xhi = pb->d_fact.as<float>();
  if (pb->precision == HDG_PREC_FF_BLOCK) {
    CellArgs a = cell_args(pb);
    cudaError_t e = launch_inv_mass_scale(a, pb->d_invm.as<double>(), ctx->stream, &ctx->launches);
    if (e != cudaSuccess) return e;
    const size_t nk2 = (size_t)pb->tab.nk * pb->tab.nk;
    const float *Mh = pb->d_minv.as<float>(), *Ml = Mh + nk2;
    const float *MGh = Mh + 4 * nk2, *MGl = MGh + pb->tab.D * nk2;
    return launch_condense_ffblock(pb->tab.D, pb->tab.k, (int)nc, Ahi, Ahi + nc * n * n, bhi, bhi + nc * n, Mh, Ml,
                                   MGh, MGl, pb->d_ffpat.as<int>(), pb->d_invm.as<double>(), pb->d_S.as<double>(),
                                   pb->d_g.as<double>(), Xhi,
                                   Xhi + nc * ni * (nf + 1), pb->d_info.as<int>(), ctx->stream, ctx->num_sms,
                                   &ctx->launches);
  }
  return launch_condense_mixed((int)nc, (int)ni, (int)nf, Ahi, Ahi + nc * n * n, bhi, bhi + nc * n,
                               pb->d_S.as<double>(), pb->d_g.as<double>(), Xhi, Xhi + nc * ni * (nf + 1),
                               pb->d_info.as<int>(), ctx->stream, ctx->num_sms, &ctx->launches);
}

// The Dirichlet data the lift and the recovery use: the problem's values, or
// zeros while the Newton path solves for a correction.
// The sign that makes the condensed skeleton operator SPD: the Darcy forms'
// is negative definite, the elasticity form's positive definite.
// DOFs per cell of the first bulk field (Darcy flux: D nk; elasticity stress: nsym nk)
// Free skeleton DOF r of a problem with several copies of its form: the
// library numbers the DOFs of a facet together ([copy 0 | copy 1 | ..] inside
// each facet block row); the multi-field space numbers each copy's skeleton
// field on its own, one after the other (MultiFieldFESpace([M1, M2, ..])).
int gs_skeleton_copy(const hdg_problem *pb, size_t r) {
  const GsTables &g = pb->gst;
  return (int)((r % (size_t)g.nfd) / (size_t)g.nfd1);
}
size_t gs_skeleton_id(const hdg_problem *pb, size_t r) {
  const GsTables &g = pb->gst;
  const size_t nfd = g.nfd, nfd1 = g.nfd1;
  const size_t br = r / nfd, j = r % nfd, cp = j / nfd1, a = j % nfd1;
  const size_t per_copy = pb->mesh.nfree / (size_t)g.copies;
  return cp * per_copy + br * nfd1 + a;
}

size_t first_field_width(const hdg_problem *pb) {
  if (pb->gs) return (size_t)pb->gst.ncA * pb->gst.nA;
  const RefTables &t = pb->tab;
  return (size_t)(pb->physics == HDG_PHYSICS_ELASTICITY ? t.nsym : t.D) * t.nk;
}

double skeleton_sign(const hdg_problem *pb) { return pb->physics == HDG_PHYSICS_ELASTICITY ? 1.0 : -1.0; }

const double *dirichlet_values(const hdg_problem *pb) {
  return pb->zero_dirichlet ? pb->d_dirzero.as<double>() : pb->d_dirvals.as<double>();
}

cudaError_t run_recover(hdg_problem *pb) {
  hdg_context *ctx = pb->ctx;
  CellArgs a = cell_args(pb);
  const size_t nc = pb->mesh.ncells, ni = pb->tab.ni, nf = pb->tab.nf;
  if (pb->precision == HDG_PREC_FP64 && pb->eblock)
    return launch_recover_x64(a, pb->d_fact.as<double>(), pb->d_x.as<double>(), dirichlet_values(pb),
                              pb->d_uint.as<double>(), ctx->stream, ctx->num_sms, &ctx->launches);
  if (pb->precision == HDG_PREC_FP64)
    return launch_recover_fp64(a, pb->d_fact.as<double>(), pb->d_x.as<double>(), dirichlet_values(pb),
                               pb->d_uint.as<double>(), ctx->stream, ctx->num_sms, &ctx->launches);
  const float *Xhi = pb->d_fact.as<float>();
  return launch_recover_mixed(a, Xhi, Xhi + nc * ni * (nf + 1), pb->d_x.as<double>(), dirichlet_values(pb),
                              pb->d_uint.as<double>(), ctx->stream, ctx->num_sms, &ctx->launches);
}

AssembleArgs assemble_args(hdg_problem *pb) {
  const RefTables &t = pb->tab;
  AssembleArgs as{};
  as.nf = t.nf;
  as.nfd = t.nfd;
  as.nl = pb->mesh.nl;
  as.nblockrows = pb->pat.nblockrows;
  as.ncells = pb->mesh.ncells;
  as.nblocks = pb->pat.nblocks;
  as.blk_off = pb->d_blk_off.as<int64_t>();
  as.blk_rowlen = pb->d_blk_rowlen.as<int>();
  as.blk_src = pb->d_blk_src.as<int>();
  as.br_row0 = pb->d_br_row0.as<int>();
  as.br_src = pb->d_br_src.as<int>();
  as.dir_cells = pb->d_dir_cells.as<int>();
  as.ndir_cells = (int)pb->pat.dir_cells.size();
  as.cell_facets = pb->d_cell_facets.as<int>();
  as.facet_dofs = pb->d_facet_dofs.as<int>();
  as.dirvals = dirichlet_values(pb);
  return as;
}

// Nodal interpolation of the exact pressure at the Dirichlet facet nodes
// (TrialFESpace(M, p), test/DarcyHDGTests.jl:52).
void interpolate_dirichlet(const hdg_problem *pb, std::vector<double> &vals) {
  const HostMesh &m = pb->mesh;
  const RefTables &t = pb->tab;
  const int D = m.D, nfd = m.nfd, k = m.k;
  vals.assign(m.ndir > 0 ? m.ndir : 1, 0.0);
  if (pb->gs) {
    // the exact trace at the nodes of the trace basis, component-major per
    // facet, the same data for every copy of the form
    const GsTables &g = pb->gst;
    for (int f = 0; f < m.nfacets; ++f) {
      if (m.facet_first_dof[f] >= 0) continue;
      const int c = m.facet_cell[2 * (size_t)f], lf = m.facet_lface[2 * (size_t)f];
      const int dn = D - 1 - lf / 2, side = lf % 2;
      for (int b = 0; b < nfd; ++b) {
        const int id = m.facet_dofs[(size_t)f * nfd + b];
        const int bb = b % g.nfd1, comp = bb / g.nT, node = bb - comp * g.nT;
        double xi[3], x[3];
        if (g.simplex) {
          // the face opposite vertex D - lf of the reference simplex, through
          // its vertices in increasing order
          static const double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
          int fv[3], q = 0;
          for (int v = 0; v <= D; ++v)
            if (v != D - lf) fv[q++] = v;
          for (int d = 0; d < D; ++d) {
            xi[d] = V[fv[0]][d];
            for (int j = 0; j + 1 < D; ++j) xi[d] += g.T.nodes[(size_t)node * (D - 1) + j] * (V[fv[j + 1]][d] - V[fv[0]][d]);
          }
        } else {
          for (int d = 0, j = 0; d < D; ++d)
            xi[d] = (d == dn) ? double(side) : g.T.nodes[(size_t)node * (D - 1) + j++];
        }
        for (int d = 0; d < D; ++d) {
          x[d] = m.origin[(size_t)c * D + d];
          for (int e = 0; e < D; ++e) x[d] += m.jac[(size_t)c * D * D + e * D + d] * xi[e];
        }
        if (pb->physics == HDG_PHYSICS_ELASTICITY) {
          double u[3], gu[3][3], hu[3][3][3];
          elasticity_exact(pb->problem, D, x, u, gu, hu);
          vals[-1 - id] = u[comp];
        } else {
          double p, q[3], fu[3], gg;
          exact_solution(pb->problem, D, x, 1.0, p, q, fu, gg);
          vals[-1 - id] = p;
        }
      }
    }
    return;
  }
  for (int f = 0; f < m.nfacets; ++f) {
    if (m.facet_first_dof[f] >= 0) continue;
    const int c = m.facet_cell[2 * (size_t)f], lf = m.facet_lface[2 * (size_t)f];
    const int dn = D - 1 - lf / 2, side = lf % 2;
    for (int b = 0; b < nfd; ++b) {
      const int id = m.facet_dofs[(size_t)f * nfd + b];
      double xi[3], x[3];
      for (int d = 0, j = 0; d < D; ++d)
        xi[d] = (d == dn) ? double(side) : double(t.flat[(b % t.nfs) * (D - 1) + j++]) / k;
      for (int d = 0; d < D; ++d) {
        x[d] = m.origin[(size_t)c * D + d];
        for (int e = 0; e < D; ++e) x[d] += m.jac[(size_t)c * D * D + e * D + d] * xi[e];
      }
      if (pb->physics == HDG_PHYSICS_ELASTICITY) {
        double u[3], gu[3][3], hu[3][3][3];
        elasticity_exact(pb->problem, D, x, u, gu, hu);
        vals[-1 - id] = u[b / t.nfs];  // component-major within the facet
      } else {
        double p, q[3], fu[3], g;
        exact_solution(pb->problem, D, x, 1.0, p, q, fu, g);
        vals[-1 - id] = p;
      }
    }
  }
}

int upload_dirichlet(hdg_problem *pb) {
  std::vector<double> vals;
  interpolate_dirichlet(pb, vals);
  return upload(pb->ctx, pb->d_dirvals, vals);
}

int setup_problem(hdg_problem *pb) {
  hdg_context *ctx = pb->ctx;
  std::string err;
  // residual reduction between two FP64 residuals of the fast skeleton solve:
  // 1e-2 in 3D (fewer iterations than 3e-2 on Darcy k = 2, 3 and elasticity
  // k = 2), 3e-2 in 2D (where 1e-2 lets the FP32 recurrence drift)
  pb->refine_delta = pb->mesh.D == 3 ? 1e-2 : 3e-2;
  if (build_ref_tables(pb->mesh.D, pb->mesh.k, pb->tab, pb->physics))
    return ctx->fail(HDG_ERR_INVALID, "unsupported D/k");
  int rc = build_pattern(pb->mesh, pb->pat, err);
  if (rc) return ctx->fail(rc, "%s", err.c_str());
  std::vector<double> packed;
  pb->toff = pack_tables(pb->tab, packed);
  if ((rc = upload(ctx, pb->d_tab, packed))) return rc;
  std::vector<float> packed_f;
  pb->toff_f = pack_tables_ff(pb->tab, packed_f);
  if ((rc = upload(ctx, pb->d_tabf, packed_f))) return rc;
  {  // M_ref^{-1} for the block-elimination paths: (hi, lo) floats, then FP64
    const std::vector<double> &Mi = pb->tab.Minv;
    // [M^{-1} hi | lo | FP64 | M^{-1} G_e hi | lo]
    const std::vector<double> &MG = pb->tab.MG;
    std::vector<float> mf(4 * Mi.size() + 2 * MG.size());
    for (size_t i = 0; i < Mi.size(); ++i) {
      mf[i] = (float)Mi[i];
      mf[Mi.size() + i] = (float)(Mi[i] - (double)mf[i]);
    }
    memcpy(mf.data() + 2 * Mi.size(), Mi.data(), sizeof(double) * Mi.size());
    for (size_t i = 0; i < MG.size(); ++i) {
      mf[4 * Mi.size() + i] = (float)MG[i];
      mf[4 * Mi.size() + MG.size() + i] = (float)(MG[i] - (double)(float)MG[i]);
    }
    if ((rc = upload(ctx, pb->d_minv, mf))) return rc;
  }
  if (l2block_supported(pb->physics == HDG_PHYSICS_ELASTICITY, pb->mesh.D, pb->mesh.k)) {
    // sparse M^{-1} G_e, M^{-1} H_F for the L2-panel block elimination
    build_l2_ref(pb->tab, pb->l2ref);
    if ((rc = upload(ctx, pb->d_l2ref_idx, pb->l2ref.idx))) return rc;
    const std::vector<double> &v = pb->l2ref.val;
    std::vector<float> vf(4 * v.size());
    for (size_t i = 0; i < v.size(); ++i) {
      vf[i] = (float)v[i];
      vf[v.size() + i] = (float)(v[i] - (double)vf[i]);
    }
    memcpy(vf.data() + 2 * v.size(), v.data(), sizeof(double) * v.size());
    if ((rc = upload(ctx, pb->d_l2ref_val, vf))) return rc;
  }
  if ((rc = upload(ctx, pb->d_origin, pb->mesh.origin))) return rc;
  {
    HostMesh &m = pb->mesh;
    m.axis = true;
    for (size_t c = 0; c < (size_t)m.ncells && m.axis; ++c)
      for (int col = 0; col < m.D; ++col)
        for (int row = 0; row < m.D; ++row)
          if (row != col && m.jac[c * m.D * m.D + col * m.D + row] != 0.0) m.axis = false;
  }
  if ((rc = upload(ctx, pb->d_jac, pb->mesh.jac))) return rc;
  if (pb->physics == HDG_PHYSICS_DARCY && ffblock_supported(pb->mesh.D, pb->mesh.k)) {
    std::vector<int> pat(ffblock_pattern_ints(pb->mesh.D, pb->mesh.k));
    ffblock_pattern(pb->mesh.D, pb->mesh.k, pb->tab.lat.data(), pb->mesh.axis, pat.data());
    if ((rc = upload(ctx, pb->d_ffpat, pat))) return rc;
  }
  if ((rc = upload(ctx, pb->d_cell_facets, pb->mesh.cell_facets))) return rc;
  if ((rc = upload(ctx, pb->d_facet_dofs, pb->mesh.facet_dofs))) return rc;
  if ((rc = upload(ctx, pb->d_facet_cell, pb->mesh.facet_cell))) return rc;
  const HostPattern &p = pb->pat;
  if ((rc = upload(ctx, pb->d_rowptr, p.rowptr))) return rc;
  if ((rc = upload(ctx, pb->d_colind, p.colind))) return rc;
  if ((rc = upload(ctx, pb->d_br_row0, p.br_row0))) return rc;
  if ((rc = upload(ctx, pb->d_br_src, p.br_src))) return rc;
  if ((rc = upload(ctx, pb->d_blk_off, p.blk_off))) return rc;
  if ((rc = upload(ctx, pb->d_blk_rowlen, p.blk_rowlen))) return rc;
  if ((rc = upload(ctx, pb->d_blk_src, p.blk_src))) return rc;
  if ((rc = upload(ctx, pb->d_diag_blk, p.diag_blk))) return rc;
  if ((rc = upload(ctx, pb->d_dir_cells, p.dir_cells))) return rc;
  if ((rc = upload(ctx, pb->d_cell_blk, p.cell_blk))) return rc;
  if ((rc = upload_dirichlet(pb))) return rc;
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return HDG_OK;
}

}  // namespace

hdg_problem::~hdg_problem() {
  if (pcg_graph) cudaGraphExecDestroy(pcg_graph);
  if (pcg32_graph) cudaGraphExecDestroy(pcg32_graph);
  if (h_pinned.ptr) {
    cudaFreeHost(h_pinned.ptr);
    h_pinned.ptr = nullptr;
    h_pinned.bytes = 0;
  }
}

extern "C" {

int hdg_version(void) { return 100; }

int hdg_device_allocations(long long *count) {
  if (!count) return HDG_ERR_INVALID;
  *count = g_device_allocs.load(std::memory_order_relaxed);
  return HDG_OK;
}

int hdg_pointer_placement(int memory_type, int pointer_device, int context_device, int *place) {
  if (!place) return HDG_ERR_INVALID;
  switch (ptr_place_rule(memory_type, pointer_device, context_device)) {
    case PtrPlace::Host: *place = 0; return HDG_OK;
    case PtrPlace::Device: *place = 1; return HDG_OK;
    default: *place = 2; return HDG_ERR_INVALID;
  }
}

int hdg_context_create(int device, hdg_context **out) {
  if (!out) return HDG_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return HDG_ERR_NODEVICE;
  }
  if (device < 0 || device >= ndev) return HDG_ERR_NODEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return HDG_ERR_NODEVICE;
  // the library carries sm_103a code only
  if (prop.major != 10 || prop.minor != 3) return HDG_ERR_NODEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return HDG_ERR_NODEVICE;
  hdg_context *ctx = new (std::nothrow) hdg_context();
  if (!ctx) return HDG_ERR_NOMEM;
  ctx->device = device;
  ctx->num_sms = prop.multiProcessorCount;
  ctx->smem_optin = prop.sharedMemPerBlockOptin;
  ctx->coop = prop.cooperativeLaunch != 0;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return HDG_ERR_CUDA;
  }
  for (auto &e : ctx->ev) cudaEventCreate(&e);
  for (auto &e : ctx->user_ev) cudaEventCreate(&e);
  for (auto &b : ctx->scratch) b.stream = ctx->stream;
  {
    // freed pool memory stays with this process for reuse instead of being
    // returned at every synchronisation (a property of the process's pool,
    // gone when the process ends)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  *out = ctx;
  return HDG_OK;
}

int hdg_context_destroy(hdg_context *ctx) {
  if (!ctx) return HDG_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto &b : ctx->scratch) b.release();
  cudaStreamSynchronize(ctx->stream);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto &e : ctx->user_ev)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return HDG_OK;
}

const char *hdg_last_error(const hdg_context *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int hdg_context_synchronize(hdg_context *ctx) {
  if (!ctx) return HDG_ERR_INVALID;
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return HDG_OK;
}

long long hdg_launch_count(const hdg_context *ctx) { return ctx ? ctx->launches : -1; }

int hdg_context_record(hdg_context *ctx, int slot) {
  if (!ctx) return HDG_ERR_INVALID;
  if (slot < 0 || slot > 3) return ctx->fail(HDG_ERR_INVALID, "event slot must be 0..3");
  cudaSetDevice(ctx->device);
  CUDA_TRY(ctx, cudaEventRecord(ctx->user_ev[slot], ctx->stream));
  return HDG_OK;
}

int hdg_context_elapsed_ms(hdg_context *ctx, int slot_from, int slot_to, double *ms) {
  if (!ctx || !ms) return HDG_ERR_INVALID;
  if (slot_from < 0 || slot_from > 3 || slot_to < 0 || slot_to > 3)
    return ctx->fail(HDG_ERR_INVALID, "event slot must be 0..3");
  cudaSetDevice(ctx->device);
  CUDA_TRY(ctx, cudaEventSynchronize(ctx->user_ev[slot_to]));
  float f = 0.f;
  CUDA_TRY(ctx, cudaEventElapsedTime(&f, ctx->user_ev[slot_from], ctx->user_ev[slot_to]));
  *ms = f;
  return HDG_OK;
}

// ---------------------------------------------------------------------------
// Map level
// ---------------------------------------------------------------------------
int hdg_static_condensation(hdg_context *ctx, int precision, int ncells, int ni, int nf,
                            const double *A, const double *b, double *S, double *g,
                            int *info) {
  if (!ctx) return HDG_ERR_INVALID;
  if (ncells < 0 || ni < 1 || nf < 0 || !A || !b || !S || !g)
    return ctx->fail(HDG_ERR_INVALID, "hdg_static_condensation: bad arguments");
  if (precision != HDG_PREC_FP64 && precision != HDG_PREC_FP32_REFINED)
    return ctx->fail(HDG_ERR_INVALID, "unknown precision %d", precision);
  if (ncells == 0) return HDG_OK;
  const int n = ni + nf;
  const size_t need = precision == HDG_PREC_FP64 ? (size_t)n * (n + 1) * sizeof(double)
                                                 : condense_mixed_smem(ni, nf);
  if (need > ctx->smem_optin - 1024)
    return ctx->fail(HDG_ERR_INVALID, "cell block %d x %d exceeds the shared-memory condensation kernel", n, n);
  cudaSetDevice(ctx->device);
  const double *dA, *db;
  double *dS, *dg;
  int *dinfo;
  int rc;
  if ((rc = stage_in(ctx, ctx->scratch[0], A, (size_t)ncells * n * n, &dA))) return rc;
  if ((rc = stage_in(ctx, ctx->scratch[1], b, (size_t)ncells * n, &db))) return rc;
  if ((rc = stage_out(ctx, ctx->scratch[2], S, (size_t)ncells * nf * nf, &dS))) return rc;
  if ((rc = stage_out(ctx, ctx->scratch[3], g, (size_t)ncells * nf, &dg))) return rc;
  CUDA_TRY(ctx, ctx->scratch[4].reserve(sizeof(int) * ncells));
  dinfo = ctx->scratch[4].as<int>();
  if (precision == HDG_PREC_FP64) {
    CUDA_TRY(ctx, launch_condense_fp64(ncells, ni, nf, dA, db, dS, dg, nullptr, dinfo, ctx->stream,
                                       ctx->num_sms, &ctx->launches));
  } else {
    // split the caller's FP64 blocks into float-float pairs, then FP32 LU + refinement
    const size_t na = (size_t)ncells * n * n, nb = (size_t)ncells * n;
    CUDA_TRY(ctx, ctx->scratch[5].reserve(sizeof(float) * 2 * (na + nb)));
    float *Ahi = ctx->scratch[5].as<float>(), *Alo = Ahi + na, *bhi = Alo + na, *blo = bhi + nb;
    CUDA_TRY(ctx, launch_split_fp64(na, dA, Ahi, Alo, ctx->stream, ctx->num_sms, &ctx->launches));
    CUDA_TRY(ctx, launch_split_fp64(nb, db, bhi, blo, ctx->stream, ctx->num_sms, &ctx->launches));
    CUDA_TRY(ctx, launch_condense_mixed(ncells, ni, nf, Ahi, Alo, bhi, blo, dS, dg, nullptr, nullptr, dinfo,
                                        ctx->stream, ctx->num_sms, &ctx->launches));
  }
  if ((rc = finish_out(ctx, dS, S, (size_t)ncells * nf * nf))) return rc;
  if ((rc = finish_out(ctx, dg, g, (size_t)ncells * nf))) return rc;
  std::vector<int> hinfo(ncells);
  CUDA_TRY(ctx, cudaMemcpyAsync(hinfo.data(), dinfo, sizeof(int) * ncells, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  bool bad = false;
  for (int c = 0; c < ncells; ++c) bad |= hinfo[c] != 0;
  if (info) {
    if ((rc = check_ptr_device(ctx, info))) return rc;
    if (is_device_ptr(ctx, info))
    {
      CUDA_TRY(ctx, cudaMemcpyAsync(info, dinfo, sizeof(int) * ncells, cudaMemcpyDeviceToDevice, ctx->stream));
      CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    else
      memcpy(info, hinfo.data(), sizeof(int) * ncells);
  }
  if (bad) return ctx->fail(HDG_ERR_SINGULAR, "zero pivot in an interior block (see info)");
  return HDG_OK;
}

int hdg_backward_static_condensation(hdg_context *ctx, int precision, int ncells, int ni,
                                     int nf, const double *A, const double *b,
                                     const double *x, double *u, int *info) {
  if (!ctx) return HDG_ERR_INVALID;
  if (ncells < 0 || ni < 1 || nf < 0 || !A || !b || !u || (nf > 0 && !x))
    return ctx->fail(HDG_ERR_INVALID, "hdg_backward_static_condensation: bad arguments");
  if (precision != HDG_PREC_FP64 && precision != HDG_PREC_FP32_REFINED)
    return ctx->fail(HDG_ERR_INVALID, "unknown precision %d", precision);
  if (ncells == 0) return HDG_OK;
  const int n = ni + nf;
  if ((size_t)ni * (ni + 1) * sizeof(double) > ctx->smem_optin - 1024)
    return ctx->fail(HDG_ERR_INVALID, "interior block %d exceeds the shared-memory kernel", ni);
  cudaSetDevice(ctx->device);
  const double *dA, *db, *dx = nullptr;
  double *du;
  int rc;
  if ((rc = stage_in(ctx, ctx->scratch[0], A, (size_t)ncells * n * n, &dA))) return rc;
  if ((rc = stage_in(ctx, ctx->scratch[1], b, (size_t)ncells * n, &db))) return rc;
  if (nf > 0 && (rc = stage_in(ctx, ctx->scratch[5], x, (size_t)ncells * nf, &dx))) return rc;
  if ((rc = stage_out(ctx, ctx->scratch[2], u, (size_t)ncells * ni, &du))) return rc;
  CUDA_TRY(ctx, ctx->scratch[4].reserve(sizeof(int) * ncells));
  int *dinfo = ctx->scratch[4].as<int>();
  CUDA_TRY(ctx, launch_backward_fp64(ncells, ni, nf, dA, db, dx, du, dinfo, ctx->stream, ctx->num_sms,
                                     &ctx->launches));
  if ((rc = finish_out(ctx, du, u, (size_t)ncells * ni))) return rc;
  std::vector<int> hinfo(ncells);
  CUDA_TRY(ctx, cudaMemcpyAsync(hinfo.data(), dinfo, sizeof(int) * ncells, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  bool bad = false;
  for (int c = 0; c < ncells; ++c) bad |= hinfo[c] != 0;
  if (info) memcpy(info, hinfo.data(), sizeof(int) * ncells);
  if (bad) return ctx->fail(HDG_ERR_SINGULAR, "zero pivot in an interior block (see info)");
  return HDG_OK;
}

int hdg_sum_facets(hdg_context *ctx, int nitems, int nfacets, int len, const double *blocks,
                   double *out) {
  if (!ctx) return HDG_ERR_INVALID;
  if (nitems < 0 || nfacets < 2 || len < 0 || !blocks || !out)
    return ctx->fail(HDG_ERR_INVALID, "hdg_sum_facets: bad arguments (nfacets must be >= 2)");
  if (nitems == 0 || len == 0) return HDG_OK;
  cudaSetDevice(ctx->device);
  const double *db;
  double *dout;
  int rc;
  if ((rc = stage_in(ctx, ctx->scratch[0], blocks, (size_t)nitems * nfacets * len, &db))) return rc;
  if ((rc = stage_out(ctx, ctx->scratch[2], out, (size_t)nitems * len, &dout))) return rc;
  CUDA_TRY(ctx, launch_sum_facets(nitems, nfacets, len, db, dout, ctx->stream, &ctx->launches));
  if ((rc = finish_out(ctx, dout, out, (size_t)nitems * len))) return rc;
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return HDG_OK;
}

// ---------------------------------------------------------------------------
// Problems
// ---------------------------------------------------------------------------
int hdg_problem_create_cartesian(hdg_context *ctx, int D, const int *cells, const double *domain,
                                 int k, hdg_problem **out) {
  return hdg_problem_create_cartesian_physics(ctx, D, cells, domain, k, HDG_PHYSICS_DARCY, out);
}

int hdg_problem_create_cartesian_physics(hdg_context *ctx, int D, const int *cells, const double *domain, int k,
                                         int physics, hdg_problem **out) {
  if (!ctx) return HDG_ERR_INVALID;
  if (!cells || !domain || !out) return ctx->fail(HDG_ERR_INVALID, "null argument");
  if (physics != HDG_PHYSICS_DARCY && physics != HDG_PHYSICS_ELASTICITY)
    return ctx->fail(HDG_ERR_INVALID, "unknown physics %d", physics);
  *out = nullptr;
  cudaSetDevice(ctx->device);
  hdg_problem *pb = new (std::nothrow) hdg_problem();
  if (!pb) return ctx->fail(HDG_ERR_NOMEM, "host allocation failed");
  pb->ctx = ctx;
  pb->physics = physics;
  for (DBuf *b : pb->device_buffers()) b->stream = ctx->stream;
  std::string err;
  int rc = build_cartesian_mesh(D, cells, domain, k, pb->mesh, err, physics == HDG_PHYSICS_ELASTICITY ? D : 1);
  if (rc) {
    delete pb;
    return ctx->fail(rc, "%s", err.c_str());
  }
  if ((rc = setup_problem(pb))) {
    delete pb;
    return rc;
  }
  *out = pb;
  return HDG_OK;
}

static int create_spaces_problem(hdg_context *ctx, int D, const int *cells, const double *domain, int physics,
                                 const int *spaces, int copies, bool simplex, hdg_problem **out) {
  if (!ctx) return HDG_ERR_INVALID;
  if (!cells || !domain || !spaces || !out) return ctx->fail(HDG_ERR_INVALID, "null argument");
  if (physics != HDG_PHYSICS_DARCY && physics != HDG_PHYSICS_ELASTICITY)
    return ctx->fail(HDG_ERR_INVALID, "unknown physics %d", physics);
  *out = nullptr;
  DeviceGuard guard(ctx->device);
  hdg_problem *pb = new (std::nothrow) hdg_problem();
  if (!pb) return ctx->fail(HDG_ERR_NOMEM, "host allocation failed");
  pb->ctx = ctx;
  pb->physics = physics;
  pb->gs = true;
  for (DBuf *b : pb->device_buffers()) b->stream = ctx->stream;
  std::string err;
  int rc = build_gs_tables(D, physics, spaces, copies, pb->gst, err, simplex);
  if (!rc) {
    const GsTables &g = pb->gst;
    if (g.n * (g.n + 1) * sizeof(double) > ctx->smem_optin - 1024) {
      err = "the cell block exceeds the shared-memory condensation kernel";
      rc = HDG_ERR_INVALID;
    } else if (!assemble_supports(g.nl, g.nfd)) {
      err = "no skeleton assembly kernel for this many DOFs per facet";
      rc = HDG_ERR_INVALID;
    }
  }
  // the mesh's facet space: every copy's trace DOFs on every facet
  if (!rc)
    rc = simplex ? build_simplex_mesh(D, cells, domain, pb->gst.nfd, pb->mesh, err)
                 : build_cartesian_mesh(D, cells, domain, std::max(1, spaces[5]), pb->mesh, err, 1, pb->gst.nfd);
  if (rc) {
    delete pb;
    return ctx->fail(rc, "%s", err.c_str());
  }
  if ((rc = setup_problem(pb))) {
    delete pb;
    return rc;
  }
  // the sizes every later stage reads
  RefTables &t = pb->tab;
  t.ni = pb->gst.ni;
  t.nf = pb->gst.nf;
  t.n = pb->gst.n;
  t.nfd = pb->gst.nfd;
  t.nfs = pb->gst.nT;
  if ((rc = upload(ctx, pb->d_gstab, pb->gst.packed))) {
    delete pb;
    return rc;
  }
  *out = pb;
  return HDG_OK;
}

int hdg_problem_create_cartesian_spaces(hdg_context *ctx, int D, const int *cells, const double *domain,
                                        int physics, const int *spaces, int copies, hdg_problem **out) {
  return create_spaces_problem(ctx, D, cells, domain, physics, spaces, copies, false, out);
}

int hdg_problem_create_simplex_spaces(hdg_context *ctx, int D, const int *cells, const double *domain, int physics,
                                      const int *spaces, int copies, hdg_problem **out) {
  return create_spaces_problem(ctx, D, cells, domain, physics, spaces, copies, true, out);
}

int hdg_problem_create(hdg_context *ctx, int D, int k, int ncells, int nfacets,
                       const double *cell_origin, const double *cell_jacobian,
                       const int *cell_facets, const int *facet_dofs, hdg_problem **out) {
  if (!ctx) return HDG_ERR_INVALID;
  if (!out || !cell_origin || !cell_jacobian || !cell_facets || !facet_dofs)
    return ctx->fail(HDG_ERR_INVALID, "null argument");
  if (D < 2 || D > 3 || k < 1 || k > kMaxK || ncells < 1 || nfacets < 1)
    return ctx->fail(HDG_ERR_INVALID, "bad sizes");
  *out = nullptr;
  cudaSetDevice(ctx->device);
  hdg_problem *pb = new (std::nothrow) hdg_problem();
  if (!pb) return ctx->fail(HDG_ERR_NOMEM, "host allocation failed");
  pb->ctx = ctx;
  for (DBuf *b : pb->device_buffers()) b->stream = ctx->stream;
  HostMesh &m = pb->mesh;
  m.D = D;
  m.k = k;
  m.ncells = ncells;
  m.nfacets = nfacets;
  m.nfd = 1;
  for (int d = 0; d < D - 1; ++d) m.nfd *= (k + 1);
  m.origin.assign(cell_origin, cell_origin + (size_t)ncells * D);
  m.jac.assign(cell_jacobian, cell_jacobian + (size_t)ncells * D * D);
  m.cell_facets.assign(cell_facets, cell_facets + (size_t)ncells * 2 * D);
  m.facet_dofs.assign(facet_dofs, facet_dofs + (size_t)nfacets * m.nfd);
  std::string err;
  int rc = finish_mesh(m, err);
  if (rc) {
    delete pb;
    return ctx->fail(rc, "%s", err.c_str());
  }
  if ((rc = setup_problem(pb))) {
    delete pb;
    return rc;
  }
  *out = pb;
  return HDG_OK;
}

int hdg_problem_destroy(hdg_problem *pb) {
  if (!pb) return HDG_OK;
  cudaSetDevice(pb->ctx->device);
  cudaStream_t st = pb->ctx->stream;
  cudaStreamSynchronize(st);
  delete pb;  // stream-ordered frees
  cudaStreamSynchronize(st);
  return HDG_OK;
}

int hdg_problem_info(const hdg_problem *pb, long long *info) {
  if (!pb || !info) return HDG_ERR_INVALID;
  info[0] = pb->mesh.ncells;
  info[1] = pb->mesh.nfacets;
  info[2] = pb->tab.ni;
  info[3] = pb->tab.nf;
  info[4] = pb->mesh.nfree;
  info[5] = pb->mesh.ndir;
  info[6] = pb->pat.nnz;
  info[7] = pb->mesh.nfd;
  return HDG_OK;
}

int hdg_get_topology(const hdg_problem *pb, int *cell_facets, int *facet_cells, int *facet_dofs) {
  if (!pb) return HDG_ERR_INVALID;
  const HostMesh &m = pb->mesh;
  if (cell_facets) memcpy(cell_facets, m.cell_facets.data(), sizeof(int) * m.cell_facets.size());
  if (facet_cells) memcpy(facet_cells, m.facet_cell.data(), sizeof(int) * m.facet_cell.size());
  if (facet_dofs) memcpy(facet_dofs, m.facet_dofs.data(), sizeof(int) * m.facet_dofs.size());
  return HDG_OK;
}

int hdg_set_elasticity(hdg_problem *pb, double tau, double young, int problem) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (pb->physics != HDG_PHYSICS_ELASTICITY)
    return ctx->fail(HDG_ERR_INVALID, "the problem was not created for elasticity");
  if (!(tau > 0.0) || !std::isfinite(tau)) return ctx->fail(HDG_ERR_INVALID, "tau must be > 0");
  if (!(young > 0.0) || !std::isfinite(young)) return ctx->fail(HDG_ERR_INVALID, "Young's modulus must be > 0");
  if (problem != HDG_EPROBLEM_LINEAR && problem != HDG_EPROBLEM_SMOOTH)
    return ctx->fail(HDG_ERR_INVALID, "unknown problem %d", problem);
  cudaSetDevice(ctx->device);
  pb->stab_mode = HDG_STAB_TEXTBOOK;
  pb->tau = tau;
  pb->young = young;
  pb->problem = problem;
  pb->form_set = true;
  pb->assembled = pb->solved = pb->recovered = false;
  int rc = upload_dirichlet(pb);
  if (rc) return rc;
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return HDG_OK;
}

int hdg_set_darcy(hdg_problem *pb, int stab_mode, double tau, int problem) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (pb->physics != HDG_PHYSICS_DARCY) return ctx->fail(HDG_ERR_INVALID, "the problem was not created for Darcy");
  if (stab_mode != HDG_STAB_TEXTBOOK && stab_mode != HDG_STAB_OWNER_SIGN)
    return ctx->fail(HDG_ERR_INVALID, "unknown stabilisation %d", stab_mode);
  // tau = 0: the hybridized mixed form without stabilisation (general-space problems, e.g. an RT_k flux)
  if (!(tau > 0.0 || (pb->gs && tau == 0.0)) || !std::isfinite(tau))
    return ctx->fail(HDG_ERR_INVALID, pb->gs ? "tau must be >= 0" : "tau must be > 0");
  if (problem < 0 || problem > 2) return ctx->fail(HDG_ERR_INVALID, "unknown problem %d", problem);
  cudaSetDevice(ctx->device);
  pb->stab_mode = stab_mode;
  pb->tau = tau;
  pb->problem = problem;
  pb->form_set = true;
  pb->assembled = pb->solved = pb->recovered = false;
  int rc = upload_dirichlet(pb);
  if (rc) return rc;
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return HDG_OK;
}

int hdg_set_permeability(hdg_problem *pb, const double *kappa) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  cudaSetDevice(ctx->device);
  const size_t nc = pb->mesh.ncells;
  if (!kappa) {
    pb->d_kappa.release();
  } else {
    CUDA_TRY(ctx, pb->d_kappa.reserve(sizeof(double) * nc));
    CUDA_TRY(ctx, cudaMemcpyAsync(pb->d_kappa.ptr, kappa, sizeof(double) * nc, cudaMemcpyDefault, ctx->stream));
  }
  pb->assembled = pb->solved = pb->recovered = false;
  return HDG_OK;
}

int hdg_set_dirichlet_values(hdg_problem *pb, const double *vals) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!vals) return ctx->fail(HDG_ERR_INVALID, "null values");
  cudaSetDevice(ctx->device);
  const size_t nd = pb->mesh.ndir;
  CUDA_TRY(ctx, pb->d_dirvals.reserve(sizeof(double) * (nd ? nd : 1)));
  if (nd) CUDA_TRY(ctx, cudaMemcpyAsync(pb->d_dirvals.ptr, vals, sizeof(double) * nd, cudaMemcpyDefault, ctx->stream));
  pb->assembled = pb->solved = pb->recovered = false;
  return HDG_OK;
}

static float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();  // not a failure of the computation: leave no error behind
    ms = 0.f;
  }
  return ms;
}

}  // extern "C"

// Validates the precision for this problem and reserves the buffers of an
// assembly.  cell_blocks: the separate integrate / condense kernels keep the
// cell blocks A, b in HBM (the batched fused kernels do not).
static int assemble_prepare(hdg_problem *pb, int precision, bool cell_blocks, bool allow_fused) {
  hdg_context *ctx = pb->ctx;
  if (precision != HDG_PREC_FP64 && precision != HDG_PREC_FP32_REFINED && precision != HDG_PREC_FF_BLOCK)
    return ctx->fail(HDG_ERR_INVALID, "unknown precision %d", precision);
  const RefTables &t = pb->tab;
  const size_t nc = pb->mesh.ncells, n = t.n, ni = t.ni, nf = t.nf;
  const bool mixed = precision != HDG_PREC_FP64;
  const bool elast = pb->physics == HDG_PHYSICS_ELASTICITY;
  if (pb->gs && precision == HDG_PREC_FF_BLOCK)
    return ctx->fail(HDG_ERR_INVALID, "general-space forms are condensed in FP64 or FP32 + refinement");
  const bool l2ok = !pb->gs && l2block_supported(elast, t.D, t.k);
  if (precision == HDG_PREC_FF_BLOCK && !(l2ok || (!elast && ffblock_supported(t.D, t.k))))
    return ctx->fail(HDG_ERR_INVALID, "block elimination is built for D=2, k<=3 and D=3, k<=2 (Darcy: k<=3)");
  // the L2-panel block elimination: every elasticity FF_BLOCK assembly, Darcy
  // beyond the shared-memory one, and FP64 cell blocks beyond the shared-memory LU
  const bool dense64_fits = n * (n + 1) * sizeof(double) <= ctx->smem_optin - 1024;
  const bool eblock = l2ok && ((precision == HDG_PREC_FF_BLOCK && (elast || !ffblock_supported(t.D, t.k))) ||
                               (precision == HDG_PREC_FP64 && !dense64_fits));
  const size_t need = precision == HDG_PREC_FP32_REFINED          ? condense_mixed_smem((int)ni, (int)nf)
                      : (precision == HDG_PREC_FP64 && !eblock)  ? n * (n + 1) * sizeof(double)
                                                                 : 0;
  if (need > ctx->smem_optin - 1024)
    return ctx->fail(HDG_ERR_INVALID, "cell block %zu exceeds the shared-memory condensation kernel", n);
  const int nl = pb->mesh.nl;
  if (mixed && !cellop_supported(nl, (int)t.nfd))
    return ctx->fail(HDG_ERR_INVALID, "no unassembled FP32 operator for %d facets of %zu DOFs", nl, t.nfd);
  if (precision == HDG_PREC_FF_BLOCK && cell_blocks && !eblock)
    CUDA_TRY(ctx, pb->d_invm.reserve(sizeof(double) * 11 * nc + sizeof(float) * 2 * 34 * nc));
  pb->precision = precision;
  pb->eblock = eblock;
  // the L2-panel kernel integrates its cells itself unless the caller needs
  // the cell blocks (the Newton path's residuals)
  pb->l2_fused = eblock && allow_fused;
  if (pb->l2_fused) cell_blocks = false;
  if (eblock) {
    size_t scratch = 0;
    L2BlockArgs sizing{};
    sizing.ncells = (int)nc;
    CUDA_TRY(ctx, launch_condense_l2block(sizing, l2block_launch(pb, &scratch, true), ctx->stream,
                                          &ctx->launches));
    CUDA_TRY(ctx, pb->d_escratch.reserve(scratch));
  }
  if (cell_blocks) {
    // cell blocks: FP64, or (hi, lo) float pairs in the same bytes
    CUDA_TRY(ctx, pb->d_A.reserve(sizeof(double) * nc * n * n));
    CUDA_TRY(ctx, pb->d_b.reserve(sizeof(double) * nc * n));
  }
  if (pb->gs && mixed)  // the FP64 cell blocks before their float-float split
    CUDA_TRY(ctx, pb->d_escratch.reserve(sizeof(double) * nc * (n * n + n)));
  CUDA_TRY(ctx, pb->d_S.reserve(sizeof(double) * nc * nf * nf));
  CUDA_TRY(ctx, pb->d_g.reserve(sizeof(double) * nc * nf));
  CUDA_TRY(ctx, pb->d_aux.reserve(sizeof(double) * nc * nf));
  // recovery factors: FP64 [U11 | U12 | y], or the float-float pair X1 = (X0, delta)
  CUDA_TRY(ctx, pb->d_fact.reserve(mixed || eblock ? sizeof(float) * 2 * nc * ni * (nf + 1)
                                                   : sizeof(double) * nc * ni * (n + 1)));
  CUDA_TRY(ctx, pb->d_info.reserve(sizeof(int) * nc));
  CUDA_TRY(ctx, pb->d_val.reserve(sizeof(double) * (pb->pat.nnz ? pb->pat.nnz : 1)));
  CUDA_TRY(ctx, pb->d_rhs.reserve(sizeof(double) * (pb->mesh.nfree ? pb->mesh.nfree : 1)));
  if (mixed) {
    CUDA_TRY(ctx, pb->d_cellop.reserve(sizeof(float) * nc * cellop_rec(nl, (int)t.nfd)));
    // W, then one double: set when a facet block is not positive definite
    CUDA_TRY(ctx, pb->d_W.reserve(sizeof(double) * (std::max<size_t>(pb->pat.nblockrows, 1) * t.nfd * t.nfd + 1)));
  }
  pb->precision = precision;
  pb->assembled = pb->solved = pb->recovered = false;
  return HDG_OK;
}

// Skeleton side of an assembly: the CSR gather + Dirichlet lift, and on the
// fast paths the FP32 cell operator of the inner skeleton iterations.
static cudaError_t assemble_skeleton(hdg_problem *pb) {
  hdg_context *ctx = pb->ctx;
  const RefTables &t = pb->tab;
  AssembleArgs as = assemble_args(pb);
  cudaError_t e = launch_assemble(as, pb->d_S.as<double>(), pb->d_g.as<double>(), pb->d_aux.as<double>(),
                                  pb->d_val.as<double>(), pb->d_rhs.as<double>(), ctx->stream, ctx->num_sms,
                                  &ctx->launches);
  if (e != cudaSuccess || pb->precision == HDG_PREC_FP64) return e;
  // the scaling of the inner frame, W = blockdiag(L_f^{-1}) with sign*D_f = L_f L_f^T
  // from the assembled diagonal blocks, then the scaled operator in the SPD frame
  PcgArgs da{};
  da.n = pb->mesh.nfree;
  da.nfd = t.nfd;
  da.nblockrows = pb->pat.nblockrows;
  da.val = pb->d_val.as<double>();
  da.diag_blk = pb->d_diag_blk.as<int>();
  da.blk_off = pb->d_blk_off.as<int64_t>();
  da.blk_rowlen = pb->d_blk_rowlen.as<int>();
  da.sign = skeleton_sign(pb);
  e = launch_block_chol_inv(da, pb->d_W.as<double>(), ctx->stream, ctx->num_sms, &ctx->launches);
  if (e != cudaSuccess) return e;
  return launch_pack_cell_blocks(pb->mesh.ncells, pb->mesh.nl, t.nfd, skeleton_sign(pb), pb->d_S.as<double>(),
                                 pb->d_cell_blk.as<int>(), pb->d_W.as<double>(), pb->d_cellop.as<float>(),
                                 ctx->smem_optin, ctx->stream, ctx->num_sms, &ctx->launches);
}

extern "C" {

int hdg_assemble(hdg_problem *pb, int precision, int *info) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  cudaSetDevice(ctx->device);
  int rc = assemble_prepare(pb, precision, true, true);
  if (rc) return rc;
  const size_t nc = pb->mesh.ncells;
  cudaEvent_t *ev = ctx->ev;
  CUDA_TRY(ctx, cudaEventRecord(ev[0], ctx->stream));
  CUDA_TRY(ctx, run_integrate(pb));
  CUDA_TRY(ctx, cudaEventRecord(ev[1], ctx->stream));
  CUDA_TRY(ctx, run_condense(pb));
  CUDA_TRY(ctx, cudaEventRecord(ev[2], ctx->stream));
  CUDA_TRY(ctx, assemble_skeleton(pb));
  CUDA_TRY(ctx, cudaEventRecord(ev[3], ctx->stream));
  std::vector<int> hinfo(nc);
  CUDA_TRY(ctx, cudaMemcpyAsync(hinfo.data(), pb->d_info.ptr, sizeof(int) * nc, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  pb->timings[0] = elapsed(ev[0], ev[1]);
  pb->timings[1] = elapsed(ev[1], ev[2]);
  pb->timings[2] = elapsed(ev[2], ev[3]);
  bool bad = false;
  for (size_t c = 0; c < nc; ++c) bad |= hinfo[c] != 0;
  if (info) memcpy(info, hinfo.data(), sizeof(int) * nc);
  if (bad) return ctx->fail(HDG_ERR_SINGULAR, "zero pivot in an interior block (see info)");
  pb->assembled = true;
  pb->solved = pb->recovered = false;
  return HDG_OK;
}

int hdg_get_skeleton_system(hdg_problem *pb, long long *rowptr, int *colind, double *val,
                            double *rhs) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!pb->assembled) return ctx->fail(HDG_ERR_STATE, "assemble first");
  cudaSetDevice(ctx->device);
  const HostPattern &p = pb->pat;
  if (pb->gs && pb->gst.copies > 1) {
    // the multi-field numbering [skeleton field of copy 0 | copy 1 | ..], and
    // only the blocks of each field with itself (the copies do not couple)
    const size_t n = pb->mesh.nfree;
    std::vector<double> v(p.nnz), b(n);
    if (p.nnz)
      CUDA_TRY(ctx, cudaMemcpyAsync(v.data(), pb->d_val.ptr, sizeof(double) * p.nnz, cudaMemcpyDeviceToHost,
                                    ctx->stream));
    if (n) CUDA_TRY(ctx, cudaMemcpyAsync(b.data(), pb->d_rhs.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<size_t> inv(n);
    for (size_t r = 0; r < n; ++r) inv[gs_skeleton_id(pb, r)] = r;
    std::vector<long long> rp(n + 1, 0);
    std::vector<std::pair<int, double>> row;
    std::vector<int> ci;
    std::vector<double> cv;
    for (size_t r2 = 0; r2 < n; ++r2) {
      const size_t r = inv[r2];
      const int cr = gs_skeleton_copy(pb, r);
      row.clear();
      for (int64_t e = p.rowptr[r]; e < p.rowptr[r + 1]; ++e)
        if (gs_skeleton_copy(pb, p.colind[e]) == cr) row.emplace_back((int)gs_skeleton_id(pb, p.colind[e]), v[e]);
      std::sort(row.begin(), row.end());
      for (auto &x : row) {
        ci.push_back(x.first);
        cv.push_back(x.second);
      }
      rp[r2 + 1] = (long long)ci.size();
    }
    if (rowptr) memcpy(rowptr, rp.data(), sizeof(long long) * (n + 1));
    if (colind && !ci.empty()) memcpy(colind, ci.data(), sizeof(int) * ci.size());
    if (val && !cv.empty()) memcpy(val, cv.data(), sizeof(double) * cv.size());
    if (rhs)
      for (size_t r = 0; r < n; ++r) rhs[gs_skeleton_id(pb, r)] = b[r];
    return HDG_OK;
  }
  if (rowptr)
    CUDA_TRY(ctx, cudaMemcpyAsync(rowptr, p.rowptr.data(), sizeof(long long) * p.rowptr.size(), cudaMemcpyDefault, ctx->stream));
  if (colind && p.nnz)
    CUDA_TRY(ctx, cudaMemcpyAsync(colind, p.colind.data(), sizeof(int) * p.nnz, cudaMemcpyDefault, ctx->stream));
  if (val && p.nnz)
    CUDA_TRY(ctx, cudaMemcpyAsync(val, pb->d_val.ptr, sizeof(double) * p.nnz, cudaMemcpyDefault, ctx->stream));
  if (rhs && pb->mesh.nfree)
    CUDA_TRY(ctx, cudaMemcpyAsync(rhs, pb->d_rhs.ptr, sizeof(double) * pb->mesh.nfree, cudaMemcpyDefault, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return HDG_OK;
}

// Grid of the PCG vector and SpMV kernels: four CTAs per SM for large
// skeletons, fewer for small ones (about two 256-row tiles per CTA) so that
// the kernels of concurrent small problems share the GPU.
static int pcg_grid(const hdg_problem *pb) {
  const long long rows = pb->mesh.nfree;
  long long g = (rows + 511) / 512;
  const long long cap = (long long)pb->ctx->num_sms * 4;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

static PcgArgs pcg_args(hdg_problem *pb) {
  PcgArgs a{};
  a.n = pb->mesh.nfree;
  a.nfd = pb->mesh.nfd;
  a.nblockrows = pb->pat.nblockrows;
  a.rowptr = pb->d_rowptr.as<int64_t>();
  a.colind = pb->d_colind.as<int>();
  a.val = pb->d_val.as<double>();
  a.rhs = pb->d_rhs.as<double>();
  a.Binv = pb->d_Binv.as<double>();
  a.x = pb->d_x.as<double>();
  a.r = pb->d_r.as<double>();
  a.z = pb->d_z.as<double>();
  a.p = pb->d_p.as<double>();
  a.p2 = pb->d_p2.as<double>();
  a.q = pb->d_q.as<double>();
  a.partials = pb->d_partials.as<double>();
  a.scal = pb->d_scal.as<double>();
  a.counter = pb->d_counter.as<unsigned int>();
  a.val32 = nullptr;
  a.nparts = pcg_grid(pb);
  a.diag_blk = pb->d_diag_blk.as<int>();
  a.blk_off = pb->d_blk_off.as<int64_t>();
  a.blk_rowlen = pb->d_blk_rowlen.as<int>();
  a.sign = skeleton_sign(pb);
  a.max_rowlen = pb->pat.max_rowlen;
  a.tile_ctas = csr_tile_ctas(pb->pat.nblockrows, pb->mesh.nfd, pb->ctx->num_sms);
  return a;
}

static Pcg32Args pcg32_args(hdg_problem *pb) {
  const size_t n = pb->mesh.nfree;
  float *v = pb->d_v32.as<float>();
  Pcg32Args ia{};
  ia.n = (int)n;
  ia.nfd = pb->mesh.nfd;
  ia.nblockrows = pb->pat.nblockrows;
  ia.W = pb->d_W.as<double>();
  ia.rhs = pb->d_r.as<double>();  // the outer residual
  ia.x = v;
  ia.r = v + n;
  ia.z = ia.r;  // identity preconditioner in the scaled frame
  ia.p = v + 3 * n;
  ia.p2 = v + 4 * n;
  ia.partials = pb->d_partials.as<double>();
  ia.scal = pb->d_scal.as<double>();
  ia.counter = pb->d_counter.as<unsigned int>();
  ia.nparts = pcg_grid(pb);
  ia.ncells = pb->mesh.ncells;
  ia.nl = pb->mesh.nl;
  ia.rec = cellop_rec(ia.nl, ia.nfd);
  ia.blocks = pb->d_cellop.as<float>();
  ia.cell_blk = pb->d_cell_blk.as<int>();
  ia.qc = pb->d_qc.as<float>();
  ia.nstage = pb->cellop_nstage;
  ia.ctas = pb->cellop_ctas;
  ia.error = pb->d_counter.as<unsigned int>() + 1;
  {  // update kernel: about eight rows per thread (four loads in flight), at most eight CTAs per SM;
     // PCG at 32^3 k = 2 with 4 / 8 / 16 / 32 rows per thread: 22.2 / 21.2 / 21.4 / 22.3 ms
    long long g = ((long long)n + 8 * kPcgThreadsHost - 1) / (8 * kPcgThreadsHost);
    const long long cap = (long long)pb->ctx->num_sms * 8;
    ia.uctas = g > cap ? (int)cap : g < 1 ? 1 : (int)g;
  }
  return ia;
}

// FP64 PCG iterations from the state launch_pcg_setup left (x = 0, r = the
// right-hand side), as replays of a CUDA graph of 16 iterations, until the
// device-side done flag or maxit.
static int run_pcg64(hdg_problem *pb, const PcgArgs &a, int maxit, int *it_out, double *rel_out) {
  hdg_context *ctx = pb->ctx;
  const int pairs = 8;  // 16 iterations per graph replay
  if (!pb->pcg_graph) {
    cudaGraph_t g;
    long long dummy = 0;
    CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int i = 0; i < pairs && le == cudaSuccess; ++i) le = launch_pcg_iteration_pair(a, ctx->stream, ctx->num_sms, &dummy);
    CUDA_TRY(ctx, cudaStreamEndCapture(ctx->stream, &g));
    if (le != cudaSuccess) {
      cudaGraphDestroy(g);
      return ctx->fail(HDG_ERR_CUDA, "PCG iteration capture: %s", cudaGetErrorString(le));
    }
    cudaError_t e = cudaGraphInstantiate(&pb->pcg_graph, g, 0);
    cudaGraphDestroy(g);
    CUDA_TRY(ctx, e);
    pb->pcg_graph_chunk = 2 * pairs;
  }
  double *h = static_cast<double *>(pb->h_pinned.ptr);
  int it = 0;
  double rel = 0.0;
  int status = HDG_OK;
  for (;;) {
    CUDA_TRY(ctx, cudaGraphLaunch(pb->pcg_graph, ctx->stream));
    ctx->launches += 2LL * pb->pcg_graph_chunk;
    CUDA_TRY(ctx, cudaMemcpyAsync(h, pb->d_scal.ptr, sizeof(double) * 16, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    it = (int)h[8];
    rel = h[5] > 0 ? std::sqrt(h[4] / h[5]) : 0.0;
    if (h[7] != 0.0) break;
    if (it >= maxit) {
      status = ctx->fail(HDG_ERR_NOT_CONVERGED, "PCG: relative residual %.3e after %d iterations", rel, it);
      break;
    }
    if (!std::isfinite(rel)) {
      status = ctx->fail(HDG_ERR_NOT_CONVERGED, "PCG breakdown (non-finite residual)");
      break;
    }
  }
  *it_out = it;
  *rel_out = rel;
  return status;
}

// Correction solve in FP64 for a refined solve whose FP32 cycles stall (the
// FP32 operator's rounding, about 6e-8 of each entry, times the system's
// condition number approaches one): with the outer residual r = sign (c - A x)
// as right-hand side, FP64 PCG solves A e = r from zero, and x <- x + sign e.
// The outer residual is then recomputed in FP64.  Uses the FP32 inner
// vectors (no longer needed) to hold the saved iterate.
static int refine_fp64_correction(hdg_problem *pb, const OuterArgs &oa, double rtol_corr, int maxit, int *its) {
  hdg_context *ctx = pb->ctx;
  const size_t n = pb->mesh.nfree;
  double *xsaved = pb->d_v32.as<double>();             // 5n floats hold n doubles ...
  float *zero = pb->d_v32.as<float>() + 2 * n;          // ... and n zero floats after them
  CUDA_TRY(ctx, cudaMemcpyAsync(xsaved, oa.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  CUDA_TRY(ctx, cudaMemsetAsync(zero, 0, sizeof(float) * n, ctx->stream));
  PcgArgs a = pcg_args(pb);
  a.rhs = oa.r;  // read once by the init kernel, row by row, before r is overwritten
  CUDA_TRY(ctx, launch_pcg_setup(a, rtol_corr, ctx->stream, ctx->num_sms, &ctx->launches));
  double rel = 0.0;
  int status = run_pcg64(pb, a, maxit, its, &rel);
  if (status == HDG_ERR_CUDA) return status;
  // x = xsaved + sign * e (e is in a.x == oa.x), then the FP64 residual
  CUDA_TRY(ctx, launch_outer_combine(oa, xsaved, ctx->stream, &ctx->launches));
  CUDA_TRY(ctx, launch_outer_update(oa, zero, ctx->stream, &ctx->launches));
  return status;
}

// Mixed-precision skeleton solve: FP32 inner PCG inside an FP64 residual loop.
static int solve_pcg_refined(hdg_problem *pb, double rtol, int maxit, int *it_out, double *rel_out) {
  hdg_context *ctx = pb->ctx;
  const size_t n = pb->mesh.nfree, nfd = pb->mesh.nfd, nbr = pb->pat.nblockrows;
  if (!pb->d_cellop.ptr) return ctx->fail(HDG_ERR_STATE, "the FP32 cell operator is missing (assemble in a fast precision)");
  if (pb->pat.max_rowlen > kSkeletonRowBlocks * (int)nfd)
    return ctx->fail(HDG_ERR_INVALID, "skeleton rows of %d entries exceed the residual kernel's %d", pb->pat.max_rowlen,
                     kSkeletonRowBlocks * (int)nfd);
  const int nl = pb->mesh.nl;
  CUDA_TRY(ctx, cellop_configure(nl, (int)nfd, ctx->smem_optin, ctx->num_sms, &pb->cellop_nstage, &pb->cellop_ctas));
  {  // at least two stages of cells per CTA on small problems
    const int cps = cellop_cps(nl * (int)nfd);
    const long long units = (pb->mesh.ncells + cps - 1) / cps;
    const long long want = (units + 1) / 2;
    if (want < pb->cellop_ctas) pb->cellop_ctas = want < 1 ? 1 : (int)want;
  }
  if (pb->cellop_ctas > ctx->num_sms * 4)
    return ctx->fail(HDG_ERR_INVALID, "cell operator grid exceeds the partials buffer");
  if (!pb->d_W.ptr) return ctx->fail(HDG_ERR_STATE, "the inner frame's scaling is missing (assemble in a fast precision)");
  CUDA_TRY(ctx, pb->d_v32.reserve(sizeof(float) * 5 * n));
  CUDA_TRY(ctx, pb->d_qc.reserve(sizeof(float) * nbr * 2 * nfd));
  // the other-cell half of a facet with one cell is never written: zero
  CUDA_TRY(ctx, cudaMemsetAsync(pb->d_qc.ptr, 0, sizeof(float) * nbr * 2 * nfd, ctx->stream));
  // last-CTA counter, bulk-copy error flag and the grid-barrier count and generation start at zero
  CUDA_TRY(ctx, cudaMemsetAsync(pb->d_counter.ptr, 0, sizeof(unsigned int) * 4, ctx->stream));
  CUDA_TRY(ctx, pb->d_scal2.reserve(sizeof(double) * 16));
  Pcg32Args ia = pcg32_args(pb);
  OuterArgs oa{};
  oa.n = (int)n;
  oa.nfd = (int)nfd;
  oa.nblockrows = (int)nbr;
  oa.rowptr = pb->d_rowptr.as<int64_t>();
  oa.colind = pb->d_colind.as<int>();
  oa.val = pb->d_val.as<double>();
  oa.rhs = pb->d_rhs.as<double>();
  oa.x = pb->d_x.as<double>();
  oa.r = pb->d_r.as<double>();
  oa.partials = ia.partials;
  oa.scal = pb->d_scal2.as<double>();
  oa.counter = ia.counter;
  oa.nparts = ia.nparts;
  oa.sign = skeleton_sign(pb);
  oa.W = pb->d_W.as<double>();
  oa.max_rowlen = pb->pat.max_rowlen;
  oa.tile_ctas = csr_tile_ctas((int)nbr, (int)nfd, ctx->num_sms);
  const int pairs = 8;
  // the inner iterations as one cooperative launch per chunk where its grid
  // can be co-resident (about two cell units per CTA on small problems), else
  // replays of a graph of 8 two-kernel iteration pairs
  int pgrid = 0, pstage = 0;
  size_t psmem = 0;
  if (ctx->coop && ctx->persistent_pcg) {
    const int cps = cellop_cps(nl * (int)nfd);
    const long long units = (pb->mesh.ncells + cps - 1) / cps;
    const long long want = std::min<long long>(std::max<long long>((units + 1) / 2, 1), (long long)ctx->num_sms * 8);
    pgrid = pcg32_persistent_config(nl, (int)nfd, ctx->smem_optin, ctx->num_sms, (int)want, &pstage, &psmem);
  }
  if (!pgrid && !pb->pcg32_graph) {
    cudaGraph_t g;
    long long dummy = 0;
    CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int i = 0; i < pairs && le == cudaSuccess; ++i) le = launch_pcg32_iteration_pair(ia, ctx->stream, &dummy);
    CUDA_TRY(ctx, cudaStreamEndCapture(ctx->stream, &g));
    if (le != cudaSuccess) {
      cudaGraphDestroy(g);
      return ctx->fail(HDG_ERR_CUDA, "inner PCG iteration capture: %s", cudaGetErrorString(le));
    }
    cudaError_t e = cudaGraphInstantiate(&pb->pcg32_graph, g, 0);
    cudaGraphDestroy(g);
    CUDA_TRY(ctx, e);
  }
  double *h = static_cast<double *>(pb->h_pinned.ptr);
  double *ho = h + 16;
  CUDA_TRY(ctx, launch_outer_init(oa, ctx->stream, &ctx->launches));
  CUDA_TRY(ctx, cudaMemcpyAsync(ho, oa.scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(ctx, cudaMemcpyAsync(ho + 2, pb->d_W.as<double>() + nbr * nfd * nfd, sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const double cc = ho[0];
  double rr = ho[1];
  // a facet block that is not positive definite kept W_f = I, so the records
  // (which leave out the diagonal blocks as the identity) do not hold for it:
  // the FP64 solve below takes the whole system
  const bool not_pd = ho[2] != 0.0;
  int total = 0, outer = 0;
  int status = HDG_OK;
  int base = 0;         // iterations counted before the last init (SC_ITERS restarts there)
  int cycle_start = 0;  // iterations counted when the graph last started from ia.p
  pb->last_fp64_iters = 0;
  bool restart = true;  // next cycle starts a fresh Krylov space
  int slow = 0;         // consecutive cycles that cut the FP64 residual less than 2x
  bool stalled = false;
  while (cc > 0.0 && rr > rtol * rtol * cc) {
    if (total < maxit && (not_pd || slow >= 3 || outer >= 60)) {
      stalled = true;  // finished below by an FP64 correction solve
      break;
    }
    if (total >= maxit) {
      status = ctx->fail(HDG_ERR_NOT_CONVERGED, "refined PCG: relative residual %.3e after %d iterations",
                         std::sqrt(rr / cc), total);
      break;
    }
    // the reduction the inner solve is asked for before the next FP64
    // residual: refine_delta, or just what is still missing at the end
    const double eta = std::max(pb->refine_delta, 0.3 * rtol * std::sqrt(cc / rr));
    const double rr_before = rr;
    if (restart || !pb->refine_keep) {
      CUDA_TRY(ctx, launch_pcg32_init(ia, eta, ctx->stream, &ctx->launches));
      base = total;
    } else {
      // the graph's first SpMV reads p_old from ia.p; after an odd number of
      // iterations since it last started, the current p is in ia.p2
      if ((total - cycle_start) & 1)
        CUDA_TRY(ctx, cudaMemcpyAsync(ia.p, ia.p2, sizeof(float) * n, cudaMemcpyDeviceToDevice, ctx->stream));
      CUDA_TRY(ctx, launch_pcg32_replace(ia, eta, ctx->stream, &ctx->launches));
    }
    cycle_start = total;
    for (;;) {
      if (pgrid) {
        Pcg32Args pa = ia;
        pa.nstage = pstage;
        int cap = std::min(maxit - total, 4096) & ~1;  // even: the next launch starts from ia.p
        if (cap < 2) cap = 2;
        CUDA_TRY(ctx, launch_pcg32_persistent(pa, pgrid, psmem, cap, ctx->stream, &ctx->launches));
      } else {
        CUDA_TRY(ctx, cudaGraphLaunch(pb->pcg32_graph, ctx->stream));
        ctx->launches += 4LL * pairs;
      }
      CUDA_TRY(ctx, cudaMemcpyAsync(h, ia.scal, sizeof(double) * 16, cudaMemcpyDeviceToHost, ctx->stream));
      CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      total = base + (int)h[8];
      if (h[7] != 0.0 || total >= maxit || !std::isfinite(h[4])) break;
    }
    ++outer;
    CUDA_TRY(ctx, launch_outer_update(oa, ia.x, ctx->stream, &ctx->launches));
    CUDA_TRY(ctx, cudaMemcpyAsync(ho, oa.scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    rr = ho[1];
    if (!std::isfinite(rr)) {
      status = ctx->fail(HDG_ERR_NOT_CONVERGED, "refined PCG breakdown (non-finite residual)");
      break;
    }
    // a kept direction that no longer cuts the true residual (the FP32
    // recurrence drifted) is dropped: the next cycle restarts
    restart = rr > 0.0625 * rr_before;
    slow = rr > 0.25 * rr_before ? slow + 1 : 0;
  }
  if (stalled && status == HDG_OK) {
    int extra = 0;
    const double rtol_corr = 0.5 * rtol * std::sqrt(cc / rr);
    status = refine_fp64_correction(pb, oa, rtol_corr, maxit - total, &extra);
    if (status == HDG_ERR_CUDA) return status;
    total += extra;
    ++outer;
    pb->last_fp64_iters = extra;
    CUDA_TRY(ctx, cudaMemcpyAsync(ho, oa.scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    rr = ho[1];
    if (status == HDG_OK && !(rr <= rtol * rtol * cc))
      status = ctx->fail(HDG_ERR_NOT_CONVERGED, "refined PCG with FP64 correction: relative residual %.3e after %d "
                         "iterations", std::sqrt(rr / cc), total);
  }
  {
    unsigned int herr = 0;
    CUDA_TRY(ctx, cudaMemcpyAsync(&herr, pb->d_counter.as<unsigned int>() + 1, sizeof(herr), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (herr) status = ctx->fail(HDG_ERR_CUDA, "a bulk copy of cell blocks did not complete");
  }
  pb->last_outer = outer;
  *it_out = total;
  *rel_out = cc > 0.0 ? std::sqrt(rr / cc) : 0.0;
  return status;
}

// Every buffer a PCG solve and the recovery use, reserved up front (so that a
// solve run on another stream allocates nothing).
static int solve_reserve(hdg_problem *pb) {
  hdg_context *ctx = pb->ctx;
  const size_t n = pb->mesh.nfree ? pb->mesh.nfree : 1, nfd = pb->mesh.nfd, nbr = pb->pat.nblockrows;
  CUDA_TRY(ctx, pb->d_x.reserve(sizeof(double) * n));
  CUDA_TRY(ctx, pb->d_Binv.reserve(sizeof(double) * nbr * nfd * nfd));
  for (DBuf *b : {&pb->d_r, &pb->d_z, &pb->d_p, &pb->d_p2, &pb->d_q}) CUDA_TRY(ctx, b->reserve(sizeof(double) * n));
  CUDA_TRY(ctx, pb->d_partials.reserve(sizeof(double) * 3 * ctx->num_sms * 8));
  CUDA_TRY(ctx, pb->d_scal.reserve(sizeof(double) * 16));
  CUDA_TRY(ctx, pb->d_counter.reserve(sizeof(unsigned int) * 4));
  if (!pb->h_pinned.ptr) {
    CUDA_TRY(ctx, cudaMallocHost(&pb->h_pinned.ptr, 4096));
    pb->h_pinned.bytes = 4096;
  }
  if (pb->precision != HDG_PREC_FP64) {
    CUDA_TRY(ctx, pb->d_v32.reserve(sizeof(float) * 5 * n));
    CUDA_TRY(ctx, pb->d_qc.reserve(sizeof(float) * std::max<size_t>(nbr, 1) * 2 * nfd));
    CUDA_TRY(ctx, pb->d_scal2.reserve(sizeof(double) * 16));
  }
  CUDA_TRY(ctx, pb->d_uint.reserve(sizeof(double) * pb->mesh.ncells * pb->tab.ni));
  return HDG_OK;
}

int hdg_solve_skeleton(hdg_problem *pb, int solver, double rtol, int maxit, int *iters,
                       double *relres) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!pb->assembled) return ctx->fail(HDG_ERR_STATE, "assemble first");
  if (solver != HDG_SOLVER_PCG && solver != HDG_SOLVER_DIRECT)
    return ctx->fail(HDG_ERR_INVALID, "unknown solver %d", solver);
  if (solver == HDG_SOLVER_PCG && (!(rtol > 0.0) || maxit < 1))
    return ctx->fail(HDG_ERR_INVALID, "PCG needs rtol > 0 and maxit >= 1");
  cudaSetDevice(ctx->device);
  const size_t n = pb->mesh.nfree, nfd = pb->mesh.nfd;
  CUDA_TRY(ctx, pb->d_x.reserve(sizeof(double) * (n ? n : 1)));
  cudaEvent_t *ev = ctx->ev;
  CUDA_TRY(ctx, cudaEventRecord(ev[4], ctx->stream));
  int it = 0;
  double rel = 0.0;
  int status = HDG_OK;
  pb->last_outer = 0;
  pb->last_fp64_iters = 0;
  if (n == 0) {
    // nothing to solve
  } else if (solver == HDG_SOLVER_DIRECT) {
    if (n > 16384) return ctx->fail(HDG_ERR_INVALID, "direct solver limited to 16384 unknowns");
    CUDA_TRY(ctx, pb->d_z.reserve(sizeof(double) * n * (n + 1)));
    CUDA_TRY(ctx, pb->d_info.reserve(sizeof(int) * std::max<size_t>(pb->mesh.ncells, 1)));
    CUDA_TRY(ctx, launch_dense_solve((int)n, pb->d_rowptr.as<int64_t>(), pb->d_colind.as<int>(),
                                     pb->d_val.as<double>(), pb->d_rhs.as<double>(), pb->d_z.as<double>(),
                                     pb->d_x.as<double>(), pb->d_info.as<int>(), ctx->stream, &ctx->launches));
    int hinfo = 0;
    CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, pb->d_info.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (hinfo) status = ctx->fail(HDG_ERR_SINGULAR, "singular skeleton system (pivot %d)", hinfo);
    pb->d_z.release();
  } else {
    if (pb->pat.max_rowlen > kMaxSkeletonRowLen || pb->pat.max_rowlen > kSkeletonRowBlocks * (int)nfd)
      return ctx->fail(HDG_ERR_INVALID, "skeleton rows of %d entries exceed the SpMV kernel's %d", pb->pat.max_rowlen,
                       std::min(kMaxSkeletonRowLen, kSkeletonRowBlocks * (int)nfd));
    if (!pcg_supports_nfd((int)nfd))
      return ctx->fail(HDG_ERR_INVALID, "PCG has no kernel for %zu DOFs per facet", nfd);
    CUDA_TRY(ctx, pb->d_Binv.reserve(sizeof(double) * pb->pat.nblockrows * nfd * nfd));
    CUDA_TRY(ctx, pb->d_r.reserve(sizeof(double) * n));
    CUDA_TRY(ctx, pb->d_z.reserve(sizeof(double) * n));
    CUDA_TRY(ctx, pb->d_p.reserve(sizeof(double) * n));
    CUDA_TRY(ctx, pb->d_p2.reserve(sizeof(double) * n));
    CUDA_TRY(ctx, pb->d_q.reserve(sizeof(double) * n));
    CUDA_TRY(ctx, pb->d_partials.reserve(sizeof(double) * 3 * ctx->num_sms * 8));
    CUDA_TRY(ctx, pb->d_scal.reserve(sizeof(double) * 16));
    CUDA_TRY(ctx, pb->d_counter.reserve(sizeof(unsigned int) * 4));
    if (!pb->h_pinned.ptr) {
      CUDA_TRY(ctx, cudaMallocHost(&pb->h_pinned.ptr, 4096));
      pb->h_pinned.bytes = 4096;
    }
    PcgArgs a = pcg_args(pb);
    if (pb->precision != HDG_PREC_FP64) {
      // the FP64 block inverses are needed only if an FP64 correction solve runs
      status = solve_pcg_refined(pb, rtol, maxit, &it, &rel);
      if (status == HDG_ERR_CUDA) return status;
    } else {
      CUDA_TRY(ctx, launch_pcg_setup(a, rtol, ctx->stream, ctx->num_sms, &ctx->launches));
      status = run_pcg64(pb, a, maxit, &it, &rel);
      if (status == HDG_ERR_CUDA) return status;
    }
  }
  CUDA_TRY(ctx, cudaEventRecord(ev[5], ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  pb->timings[3] = elapsed(ev[4], ev[5]);
  pb->last_iters = it;
  pb->last_relres = rel;
  if (iters) *iters = it;
  if (relres) *relres = rel;
  pb->solved = (status == HDG_OK);
  pb->recovered = false;
  return status;
}

int hdg_recover(hdg_problem *pb) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!pb->solved) return ctx->fail(HDG_ERR_STATE, "solve the skeleton system first");
  cudaSetDevice(ctx->device);
  const size_t nc = pb->mesh.ncells, ni = pb->tab.ni;
  CUDA_TRY(ctx, pb->d_uint.reserve(sizeof(double) * nc * ni));
  cudaEvent_t *ev = ctx->ev;
  CUDA_TRY(ctx, cudaEventRecord(ev[6], ctx->stream));
  CUDA_TRY(ctx, run_recover(pb));
  CUDA_TRY(ctx, cudaEventRecord(ev[7], ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  pb->timings[4] = elapsed(ev[6], ev[7]);
  pb->recovered = true;
  return HDG_OK;
}

int hdg_get_cell_interior_values(hdg_problem *pb, double *out) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!pb->recovered) return ctx->fail(HDG_ERR_STATE, "recover first");
  if (!out) return ctx->fail(HDG_ERR_INVALID, "null output");
  cudaSetDevice(ctx->device);
  CUDA_TRY(ctx, cudaMemcpyAsync(out, pb->d_uint.ptr, sizeof(double) * pb->mesh.ncells * pb->tab.ni,
                                cudaMemcpyDefault, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return HDG_OK;
}

int hdg_get_skeleton_values(hdg_problem *pb, double *out) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!pb->solved) return ctx->fail(HDG_ERR_STATE, "solve first");
  if (!out) return ctx->fail(HDG_ERR_INVALID, "null output");
  cudaSetDevice(ctx->device);
  const size_t nfree = pb->mesh.nfree;
  if (nfree && pb->gs && pb->gst.copies > 1) {
    std::vector<double> x(nfree), y(nfree);
    CUDA_TRY(ctx, cudaMemcpyAsync(x.data(), pb->d_x.ptr, sizeof(double) * nfree, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (size_t r = 0; r < nfree; ++r) y[gs_skeleton_id(pb, r)] = x[r];
    CUDA_TRY(ctx, cudaMemcpyAsync(out, y.data(), sizeof(double) * nfree, cudaMemcpyDefault, ctx->stream));
  } else if (nfree) {
    CUDA_TRY(ctx, cudaMemcpyAsync(out, pb->d_x.ptr, sizeof(double) * nfree, cudaMemcpyDefault, ctx->stream));
  }
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return HDG_OK;
}

int hdg_get_free_dof_values(hdg_problem *pb, double *out) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!pb->recovered) return ctx->fail(HDG_ERR_STATE, "recover first");
  if (!out) return ctx->fail(HDG_ERR_INVALID, "null output");
  cudaSetDevice(ctx->device);
  const size_t nc = pb->mesh.ncells, ni = pb->tab.ni;
  const double *u = pb->d_uint.as<double>();
  // [each bulk field of all cells, in the multi-field order | free skeleton values]
  std::vector<size_t> widths;
  if (pb->gs) {
    for (int c = 0; c < pb->gst.copies; ++c) widths.push_back((size_t)pb->gst.ncA * pb->gst.nA);
    for (int c = 0; c < pb->gst.copies; ++c) widths.push_back((size_t)pb->gst.ncB * pb->gst.nB);
  } else {
    widths.push_back(first_field_width(pb));
    widths.push_back(ni - widths[0]);
  }
  size_t col = 0, off = 0;
  for (size_t w : widths) {
    CUDA_TRY(ctx, cudaMemcpy2DAsync(out + off, w * sizeof(double), u + col, ni * sizeof(double), w * sizeof(double),
                                    nc, cudaMemcpyDefault, ctx->stream));
    col += w;
    off += nc * w;
  }
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (pb->mesh.nfree) {
    int rc = hdg_get_skeleton_values(pb, out + nc * ni);
    if (rc) return rc;
  }
  return HDG_OK;
}

int hdg_l2_errors(hdg_problem *pb, double *err_flux, double *err_pres) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!pb->recovered) return ctx->fail(HDG_ERR_STATE, "recover first");
  cudaSetDevice(ctx->device);
  const size_t nc = pb->mesh.ncells;
  CUDA_TRY(ctx, pb->d_errs.reserve(sizeof(double) * 2 * nc));
  CellArgs a = cell_args(pb);
  if (pb->gs)
    CUDA_TRY(ctx, launch_l2_errors_gs(gs_args(pb), pb->d_uint.as<double>(), pb->d_errs.as<double>(), ctx->stream,
                                      ctx->num_sms, &ctx->launches));
  else if (pb->physics == HDG_PHYSICS_ELASTICITY)
    CUDA_TRY(ctx, launch_l2_errors_elasticity(a, pb->d_uint.as<double>(), pb->d_errs.as<double>(), ctx->stream,
                                              ctx->num_sms, &ctx->launches));
  else
    CUDA_TRY(ctx, launch_l2_errors(a, pb->d_uint.as<double>(), pb->d_errs.as<double>(), ctx->stream, ctx->num_sms,
                                   &ctx->launches));
  std::vector<double> h(2 * nc);
  CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), pb->d_errs.ptr, sizeof(double) * 2 * nc, cudaMemcpyDeviceToHost,
                                ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  double ef = 0.0, ep = 0.0;
  for (size_t c = 0; c < nc; ++c) {
    ef += h[2 * c];
    ep += h[2 * c + 1];
  }
  if (err_flux) *err_flux = std::sqrt(ef);
  if (err_pres) *err_pres = std::sqrt(ep);
  return HDG_OK;
}

int hdg_solve(hdg_problem *pb, int precision, int solver, double rtol, int maxit,
              const double *kappa, double *free_dof_values, double *stats) {
  if (!pb) return HDG_ERR_INVALID;
  int rc;
  if (kappa && (rc = hdg_set_permeability(pb, kappa))) return rc;
  if ((rc = hdg_assemble(pb, precision, nullptr))) return rc;
  int it = 0;
  double rel = 0.0;
  if ((rc = hdg_solve_skeleton(pb, solver, rtol, maxit, &it, &rel))) return rc;
  if ((rc = hdg_recover(pb))) return rc;
  if (free_dof_values && (rc = hdg_get_free_dof_values(pb, free_dof_values))) return rc;
  if (stats) {
    stats[0] = it;
    stats[1] = rel;
    stats[2] = pb->timings[0] + pb->timings[1];
    stats[3] = pb->timings[2];
    stats[4] = pb->timings[3];
    stats[5] = pb->timings[4];
    stats[6] = pb->timings[0] + pb->timings[1] + pb->timings[2] + pb->timings[3] + pb->timings[4];
  }
  return HDG_OK;
}

int hdg_newton_solve(hdg_problem *pb, int solver, double lin_rtol, int lin_maxit, double ftol, int max_iters,
                     const double *x0, double *res_norms, int *iters) {
  if (!pb) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (!pb->form_set) return ctx->fail(HDG_ERR_STATE, "set the weak form first (hdg_set_darcy)");
  if (pb->mesh.simplex) return ctx->fail(HDG_ERR_INVALID, "the Newton path takes box cells");
  if (!(ftol > 0.0) || max_iters < 0) return ctx->fail(HDG_ERR_INVALID, "ftol must be > 0 and max_iters >= 0");
  cudaSetDevice(ctx->device);
  int rc = assemble_prepare(pb, HDG_PREC_FP64, true, false);
  if (rc) return rc;
  const size_t nc = pb->mesh.ncells, ni = pb->tab.ni;
  const size_t w1 = first_field_width(pb), w2 = ni - w1;
  const size_t nfree = pb->mesh.nfree, nint = nc * ni, ndir = pb->mesh.ndir;
  CUDA_TRY(ctx, pb->d_newton.reserve(sizeof(double) * (nint + nfree + 1)));
  CUDA_TRY(ctx, pb->d_rmax.reserve(sizeof(double) * 2));
  CUDA_TRY(ctx, pb->d_dirzero.reserve(sizeof(double) * (ndir ? ndir : 1)));
  CUDA_TRY(ctx, cudaMemsetAsync(pb->d_dirzero.ptr, 0, sizeof(double) * (ndir ? ndir : 1), ctx->stream));
  CUDA_TRY(ctx, pb->d_uint.reserve(sizeof(double) * nint));
  CUDA_TRY(ctx, pb->d_x.reserve(sizeof(double) * (nfree ? nfree : 1)));
  double *xint = pb->d_newton.as<double>(), *xskel = xint + nint;
  if (x0) {
    // Gridap layout [first bulk field of all cells | second | free skeleton] -> cell-major
    CUDA_TRY(ctx, cudaMemcpy2DAsync(xint, ni * sizeof(double), x0, w1 * sizeof(double), w1 * sizeof(double), nc,
                                    cudaMemcpyDefault, ctx->stream));
    CUDA_TRY(ctx, cudaMemcpy2DAsync(xint + w1, ni * sizeof(double), x0 + nc * w1, w2 * sizeof(double),
                                    w2 * sizeof(double), nc, cudaMemcpyDefault, ctx->stream));
    if (nfree)
      CUDA_TRY(ctx, cudaMemcpyAsync(xskel, x0 + nint, sizeof(double) * nfree, cudaMemcpyDefault, ctx->stream));
  } else {
    CUDA_TRY(ctx, cudaMemsetAsync(xint, 0, sizeof(double) * (nint + nfree), ctx->stream));
  }
  CellArgs a = cell_args(pb);
  int it = 0;
  int status = HDG_OK;
  double hr[2];
  for (;; ++it) {
    // Jacobian (the cell matrices) and residual r_c = A_c x_c - b_c
    CUDA_TRY(ctx, run_integrate(pb));
    AssembleArgs as = assemble_args(pb);
    CUDA_TRY(ctx, launch_newton_residual(a, as, pb->d_A.as<double>(), pb->d_b.as<double>(), xint, xskel,
                                         pb->d_dirvals.as<double>(), pb->d_rmax.as<double>(), ctx->stream,
                                         ctx->num_sms, &ctx->launches));
    CUDA_TRY(ctx, cudaMemcpyAsync(hr, pb->d_rmax.ptr, sizeof(hr), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    const double norm = std::max(hr[0], hr[1]);
    if (res_norms) res_norms[it] = norm;
    if (!std::isfinite(norm)) {
      status = ctx->fail(HDG_ERR_NOT_CONVERGED, "Newton: non-finite residual");
      break;
    }
    if (norm <= ftol) break;
    if (it == max_iters) {
      status = ctx->fail(HDG_ERR_NOT_CONVERGED, "Newton: residual %.3e after %d iterations", norm, it);
      break;
    }
    // the hybridized linear solve of J dx = r with zero Dirichlet data
    // (src/HybridLinearSolvers.jl:22-59)
    CUDA_TRY(ctx, run_condense(pb));
    pb->zero_dirichlet = true;
    cudaError_t e = assemble_skeleton(pb);
    pb->zero_dirichlet = false;
    CUDA_TRY(ctx, e);
    pb->assembled = true;
    int lit = 0;
    double lrel = 0.0;
    pb->zero_dirichlet = true;
    rc = hdg_solve_skeleton(pb, solver, lin_rtol, lin_maxit, &lit, &lrel);
    if (rc == HDG_OK) rc = run_recover(pb) == cudaSuccess ? HDG_OK : HDG_ERR_CUDA;
    pb->zero_dirichlet = false;
    if (rc) {
      status = rc == HDG_ERR_CUDA ? ctx->fail(HDG_ERR_CUDA, "Newton: correction recovery failed") : rc;
      break;
    }
    // x <- x - dx
    CUDA_TRY(ctx, launch_newton_update(nint, xint, pb->d_uint.as<double>(), ctx->stream, ctx->num_sms,
                                       &ctx->launches));
    CUDA_TRY(ctx, launch_newton_update(nfree, xskel, pb->d_x.as<double>(), ctx->stream, ctx->num_sms,
                                       &ctx->launches));
  }
  if (iters) *iters = it;
  // the iterate becomes the problem's solution (free DOF values, L2 errors)
  CUDA_TRY(ctx, cudaMemcpyAsync(pb->d_uint.ptr, xint, sizeof(double) * nint, cudaMemcpyDeviceToDevice, ctx->stream));
  if (nfree)
    CUDA_TRY(ctx, cudaMemcpyAsync(pb->d_x.ptr, xskel, sizeof(double) * nfree, cudaMemcpyDeviceToDevice, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  pb->solved = pb->recovered = status == HDG_OK;
  return status;
}

int hdg_problem_device_bytes(const hdg_problem *pb, double *bytes) {
  if (!pb || !bytes) return HDG_ERR_INVALID;
  double s = 0.0;
  for (const DBuf *b : const_cast<hdg_problem *>(pb)->device_buffers()) s += (double)b->bytes;
  *bytes = s;
  return HDG_OK;
}

int hdg_set_refinement(hdg_problem *pb, double delta, int keep_direction) {
  if (!pb) return HDG_ERR_INVALID;
  if (!(delta >= 1e-8 && delta < 1.0)) return pb->ctx->fail(HDG_ERR_INVALID, "delta must lie in [1e-8, 1)");
  pb->refine_delta = delta;
  pb->refine_keep = keep_direction ? 1 : 0;
  return HDG_OK;
}

int hdg_footprint(int D, int n, int k, int precision, int solver, double *bytes) {
  if (!bytes || D < 2 || D > 3 || n < 1 || k < 1 || k > kMaxK) return HDG_ERR_INVALID;
  *bytes = footprint_bound(D, n, k, precision, solver);
  return HDG_OK;
}

int hdg_context_set_persistent_pcg(hdg_context *ctx, int on) {
  if (!ctx) return HDG_ERR_INVALID;
  if (on && !ctx->coop) return ctx->fail(HDG_ERR_INVALID, "the device has no cooperative launches");
  ctx->persistent_pcg = on ? 1 : 0;
  return HDG_OK;
}

int hdg_get_timings(const hdg_problem *pb, double *ms) {
  if (!pb || !ms) return HDG_ERR_INVALID;
  for (int i = 0; i < 5; ++i) ms[i] = pb->timings[i];
  return HDG_OK;
}

int hdg_get_solve_stats(const hdg_problem *pb, double *stats) {
  if (!pb || !stats) return HDG_ERR_INVALID;
  stats[0] = pb->last_iters;
  stats[1] = pb->last_relres;
  stats[2] = pb->last_outer;
  stats[3] = pb->last_fp64_iters;
  return HDG_OK;
}

int hdg_time_kernel(hdg_problem *pb, int which, int reps, double *ms_per_launch) {
  if (!pb || !ms_per_launch) return HDG_ERR_INVALID;
  hdg_context *ctx = pb->ctx;
  if (reps < 1 || which < 0 || which > 4) return ctx->fail(HDG_ERR_INVALID, "bad kernel id or reps");
  if (!pb->assembled) return ctx->fail(HDG_ERR_STATE, "assemble first");
  if ((which == 3 || which == 4) && !pb->solved) return ctx->fail(HDG_ERR_STATE, "solve first");
  if (which == 3 && !pb->d_q.ptr) return ctx->fail(HDG_ERR_STATE, "SpMV timing needs a PCG solve first");
  if (which == 4 && !pb->recovered) return ctx->fail(HDG_ERR_STATE, "recover first");
  cudaSetDevice(ctx->device);
  AssembleArgs as = assemble_args(pb);
  PcgArgs pa{};
  Pcg32Args pa32{};
  DBuf zero_scal;
  const bool mixed_spmv = which == 3 && pb->precision != HDG_PREC_FP64;
  if (mixed_spmv && (!pb->d_v32.ptr || !pb->d_qc.ptr || !pb->cellop_ctas))
    return ctx->fail(HDG_ERR_STATE, "SpMV timing needs a refined PCG solve first");
  if (which == 3) {
    pa = pcg_args(pb);
    pa32 = pcg32_args(pb);
    CUDA_TRY(ctx, zero_scal.reserve(sizeof(double) * 16));
    CUDA_TRY(ctx, cudaMemsetAsync(zero_scal.ptr, 0, sizeof(double) * 16, ctx->stream));
    pa.scal = zero_scal.as<double>();  // an SC_DONE of 0 keeps the kernel active
    pa32.scal = zero_scal.as<double>();
  }
  auto launch = [&]() -> cudaError_t {
    switch (which) {
      case 0:
        return run_integrate(pb);
      case 1:
        return run_condense(pb);
      case 2:
        return launch_assemble(as, pb->d_S.as<double>(), pb->d_g.as<double>(), pb->d_aux.as<double>(),
                               pb->d_val.as<double>(), pb->d_rhs.as<double>(), ctx->stream, ctx->num_sms,
                               &ctx->launches);
      case 3:
        // the SpMV the solve iterates: the FP32 cell-operator SpMV on the fast paths
        return mixed_spmv ? launch_pcg32_spmv(pa32, ctx->stream, &ctx->launches)
                          : launch_spmv(pa, ctx->stream, &ctx->launches);
      default:
        return run_recover(pb);
    }
  };
  CUDA_TRY(ctx, launch());  // warm-up
  CUDA_TRY(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
  for (int r = 0; r < reps; ++r) CUDA_TRY(ctx, launch());
  CUDA_TRY(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  *ms_per_launch = elapsed(ctx->ev[0], ctx->ev[1]) / reps;
  return HDG_OK;
}

// ---------------------------------------------------------------------------
// Size-class batching.
// ---------------------------------------------------------------------------
}  // extern "C"

struct hdg_batch {
  hdg_context *ctx = nullptr;
  std::vector<hdg_problem *> probs;
  struct Class {
    int D = 0, k = 0;
    std::vector<int> members;  // indices into probs, in batch order
    long long total = 0;       // cells
    int tpc[3] = {0, 0, 0};    // tuned threads per cell, by precision
    double tuned_ms[3] = {0, 0, 0};
  };
  std::vector<Class> classes;
  DBuf d_probs, d_bad, d_scratch;
  std::vector<BatchProblem> h_probs;
  // the launch sequence as two CUDA graphs (fused cell work; skeleton
  // assembly), timed by events recorded between the replays
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int graph_precision = -1;
  std::vector<const void *> graph_key;  // buffer addresses the graphs were captured with
  long long graph_launches[2] = {0, 0}; // kernels one replay launches
  std::vector<hdg_context *> workers;   // streams of the concurrent skeleton solves
  double timings[3] = {0, 0, 0};        // fused integrate+condense, skeleton assembly, solve+recover (ms)
  ~hdg_batch() {
    for (auto &g : graph)
      if (g) cudaGraphExecDestroy(g);
    for (hdg_context *w : workers) hdg_context_destroy(w);
  }
};

namespace {

const int kTpcCandidates[4] = {256, 128, 64, 32};
constexpr size_t kBatchSolveStreams = 8;

int prec_slot(int precision) { return precision == HDG_PREC_FP64 ? 0 : precision == HDG_PREC_FF_BLOCK ? 1 : 2; }

FusedLaunch fused_launch(hdg_batch *b, size_t ci, int precision, int tpc, size_t prob_off) {
  hdg_context *ctx = b->ctx;
  const hdg_batch::Class &cl = b->classes[ci];
  const RefTables &t = b->probs[(size_t)cl.members[0]]->tab;
  FusedLaunch L{};
  L.precision = precision;
  L.D = cl.D;
  L.k = cl.k;
  L.n = t.n;
  L.ni = t.ni;
  L.nf = t.nf;
  L.nqv = t.nqv;
  L.tpc = tpc;
  L.probs = b->d_probs.as<BatchProblem>() + prob_off;
  L.nprob = (int)cl.members.size();
  L.total = cl.total;
  L.scratch = b->d_scratch.as<float>();
  L.scratch_bytes = b->d_scratch.bytes;
  L.bad = b->d_bad.as<int>() + prob_off;
  L.num_sms = ctx->num_sms;
  L.smem_optin = ctx->smem_optin;
  return L;
}

}  // namespace

extern "C" {

int hdg_batch_create(hdg_context *ctx, int nproblems, hdg_problem *const *problems, hdg_batch **out) {
  if (!ctx || !out || nproblems < 1 || !problems) return ctx ? ctx->fail(HDG_ERR_INVALID, "bad arguments") : 1;
  *out = nullptr;
  hdg_batch *b = new (std::nothrow) hdg_batch();
  if (!b) return ctx->fail(HDG_ERR_NOMEM, "host allocation failed");
  b->ctx = ctx;
  for (int i = 0; i < nproblems; ++i) {
    hdg_problem *pb = problems[i];
    if (!pb || pb->ctx != ctx) {
      delete b;
      return ctx->fail(HDG_ERR_INVALID, "problem %d is null or belongs to another context", i);
    }
    b->probs.push_back(pb);
    size_t ci = 0;
    for (; ci < b->classes.size(); ++ci)
      if (b->classes[ci].D == pb->mesh.D && b->classes[ci].k == pb->mesh.k) break;
    if (ci == b->classes.size()) {
      b->classes.emplace_back();
      b->classes.back().D = pb->mesh.D;
      b->classes.back().k = pb->mesh.k;
    }
    b->classes[ci].members.push_back(i);
    b->classes[ci].total += pb->mesh.ncells;
  }
  *out = b;
  return HDG_OK;
}

int hdg_batch_destroy(hdg_batch *b) {
  if (!b) return HDG_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  for (DBuf *d : {&b->d_probs, &b->d_bad, &b->d_scratch}) d->stream = b->ctx->stream;
  delete b;
  return HDG_OK;
}

int hdg_batch_assemble(hdg_batch *b, int precision, int *bad) {
  if (!b) return HDG_ERR_INVALID;
  hdg_context *ctx = b->ctx;
  if (precision != HDG_PREC_FP64 && precision != HDG_PREC_FF_BLOCK)
    return ctx->fail(HDG_ERR_INVALID, "batched kernels exist for HDG_PREC_FP64 and HDG_PREC_FF_BLOCK");
  cudaSetDevice(ctx->device);
  for (const auto &cl : b->classes)
    if (!fused_batch_supported(cl.D, cl.k, precision))
      return ctx->fail(HDG_ERR_INVALID, "no fused batch kernel for D=%d k=%d at this precision", cl.D, cl.k);
  int rc;
  for (hdg_problem *pb : b->probs)
    if ((rc = assemble_prepare(pb, precision, false, false))) return rc;
  for (DBuf *d : {&b->d_probs, &b->d_bad, &b->d_scratch}) d->stream = ctx->stream;
  // per-problem descriptors, class by class
  const size_t np = b->probs.size();
  b->h_probs.assign(np, BatchProblem{});
  std::vector<size_t> class_off(b->classes.size());
  {
    size_t k = 0;
    for (size_t ci = 0; ci < b->classes.size(); ++ci) {
      class_off[ci] = k;
      long long first = 0;
      for (int m : b->classes[ci].members) {
        hdg_problem *pb = b->probs[(size_t)m];
        BatchProblem &P = b->h_probs[k++];
        const size_t nc = pb->mesh.ncells, ni = pb->tab.ni, nf = pb->tab.nf;
        P.a = cell_args(pb);
        P.T = mixed_tables(pb);
        P.Mh = pb->d_minv.as<float>();
        P.Ml = P.Mh + (size_t)pb->tab.nk * pb->tab.nk;
        P.MGh = P.Mh + 4 * (size_t)pb->tab.nk * pb->tab.nk;
        P.MGl = P.MGh + (size_t)pb->tab.D * pb->tab.nk * pb->tab.nk;
        P.ffpat = pb->d_ffpat.as<int>();
        P.S = pb->d_S.as<double>();
        P.g = pb->d_g.as<double>();
        P.Xh = pb->d_fact.as<float>();
        P.Xl = P.Xh + nc * ni * (nf + 1);
        P.fact = pb->d_fact.as<double>();
        P.info = pb->d_info.as<int>();
        P.first = first;
        first += (long long)nc;
      }
    }
  }
  CUDA_TRY(ctx, b->d_probs.reserve(sizeof(BatchProblem) * np));
  CUDA_TRY(ctx, b->d_bad.reserve(sizeof(int) * np));
  CUDA_TRY(ctx, cudaMemcpyAsync(b->d_probs.ptr, b->h_probs.data(), sizeof(BatchProblem) * np, cudaMemcpyHostToDevice,
                                ctx->stream));
  const int slot = prec_slot(precision);
  // scratch for every candidate tile (block elimination keeps cells in L2 slots)
  size_t scratch = 16;
  for (size_t ci = 0; ci < b->classes.size(); ++ci)
    for (int tpc : kTpcCandidates) {
      FusedLaunch L = fused_launch(b, ci, precision, tpc, class_off[ci]);
      size_t need = 0;
      L.dry_run = true;
      L.scratch_bytes_out = &need;
      if (launch_fused_batch(L, ctx->stream, &ctx->launches) == cudaSuccess) scratch = std::max(scratch, need);
      cudaGetLastError();
    }
  CUDA_TRY(ctx, b->d_scratch.reserve(scratch));
  // autotune: threads per cell (cells per CTA) for each class, timed on this batch
  cudaEvent_t *ev = ctx->ev;
  for (size_t ci = 0; ci < b->classes.size(); ++ci) {
    hdg_batch::Class &cl = b->classes[ci];
    if (cl.tpc[slot]) continue;
    double best = 1e300;
    for (int tpc : kTpcCandidates) {
      FusedLaunch L = fused_launch(b, ci, precision, tpc, class_off[ci]);
      if (launch_fused_batch(L, ctx->stream, &ctx->launches) != cudaSuccess) {  // infeasible tile
        cudaGetLastError();
        continue;
      }
      CUDA_TRY(ctx, cudaEventRecord(ev[0], ctx->stream));
      CUDA_TRY(ctx, launch_fused_batch(L, ctx->stream, &ctx->launches));
      CUDA_TRY(ctx, cudaEventRecord(ev[1], ctx->stream));
      CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      const double ms = elapsed(ev[0], ev[1]);
      if (ms < best) {
        best = ms;
        cl.tpc[slot] = tpc;
      }
    }
    if (!cl.tpc[slot]) return ctx->fail(HDG_ERR_INVALID, "no feasible tile for class D=%d k=%d", cl.D, cl.k);
    cl.tuned_ms[slot] = best;
  }
  // the batch's launch sequence as one CUDA graph (re-captured when buffers move)
  std::vector<const void *> key{b->d_probs.ptr, b->d_bad.ptr, b->d_scratch.ptr};
  for (hdg_problem *pb : b->probs)
    for (const DBuf *d : pb->device_buffers()) key.push_back(d->ptr);
  auto enqueue_cells = [&]() -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(b->d_bad.ptr, 0, sizeof(int) * np, ctx->stream);
    for (size_t ci = 0; ci < b->classes.size() && e == cudaSuccess; ++ci)
      e = launch_fused_batch(fused_launch(b, ci, precision, b->classes[ci].tpc[slot], class_off[ci]), ctx->stream,
                             &ctx->launches);
    return e;
  };
  auto enqueue_skeleton = [&]() -> cudaError_t {
    cudaError_t e = cudaSuccess;
    for (hdg_problem *pb : b->probs)
      if (e == cudaSuccess) e = assemble_skeleton(pb);
    return e;
  };
  if (!b->graph[0] || b->graph_precision != precision || b->graph_key != key) {
    for (int gi = 0; gi < 2; ++gi) {
      if (b->graph[gi]) cudaGraphExecDestroy(b->graph[gi]);
      b->graph[gi] = nullptr;
      cudaGraph_t g;
      const long long l0 = ctx->launches;
      CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = gi == 0 ? enqueue_cells() : enqueue_skeleton();
      cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
      b->graph_launches[gi] = ctx->launches - l0;
      ctx->launches = l0;
      CUDA_TRY(ctx, e);
      CUDA_TRY(ctx, e2);
      e = cudaGraphInstantiate(&b->graph[gi], g, 0);
      cudaGraphDestroy(g);
      CUDA_TRY(ctx, e);
    }
    b->graph_precision = precision;
    b->graph_key = key;
  }
  CUDA_TRY(ctx, cudaEventRecord(ev[4], ctx->stream));
  CUDA_TRY(ctx, cudaGraphLaunch(b->graph[0], ctx->stream));
  CUDA_TRY(ctx, cudaEventRecord(ev[5], ctx->stream));
  CUDA_TRY(ctx, cudaGraphLaunch(b->graph[1], ctx->stream));
  CUDA_TRY(ctx, cudaEventRecord(ev[6], ctx->stream));
  ctx->launches += b->graph_launches[0] + b->graph_launches[1];
  std::vector<int> hbad(np);
  CUDA_TRY(ctx, cudaMemcpyAsync(hbad.data(), b->d_bad.ptr, sizeof(int) * np, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  b->timings[0] = elapsed(ev[4], ev[5]);
  b->timings[1] = elapsed(ev[5], ev[6]);
  // descriptors are in class order; report per problem in batch order
  std::vector<int> bad_by_problem(np, 0);
  {
    size_t k = 0;
    for (const auto &cl : b->classes)
      for (int m : cl.members) bad_by_problem[(size_t)m] = hbad[k++];
  }
  bool any = false;
  for (size_t i = 0; i < np; ++i) {
    any |= bad_by_problem[i] != 0;
    hdg_problem *pb = b->probs[i];
    pb->timings[0] = 0.0;
    pb->timings[1] = b->timings[0];
    pb->timings[2] = b->timings[1];
    pb->assembled = bad_by_problem[i] == 0;
  }
  if (bad) memcpy(bad, bad_by_problem.data(), sizeof(int) * np);
  if (any) return ctx->fail(HDG_ERR_SINGULAR, "zero pivot in an interior block of a batched problem (see bad)");
  return HDG_OK;
}

int hdg_batch_solve(hdg_batch *b, int solver, double rtol, int maxit, int *iters, double *relres) {
  if (!b) return HDG_ERR_INVALID;
  hdg_context *ctx = b->ctx;
  cudaSetDevice(ctx->device);
  const auto h0 = std::chrono::steady_clock::now();
  const size_t np = b->probs.size();
  for (hdg_problem *pb : b->probs)
    if (!pb->assembled) return ctx->fail(HDG_ERR_STATE, "assemble the batch first");
  const int nworkers = solver == HDG_SOLVER_PCG ? (int)std::min<size_t>(np, kBatchSolveStreams) : 1;
  if (nworkers <= 1) {
    for (size_t i = 0; i < np; ++i) {
      int it = 0;
      double rel = 0.0;
      int rc = hdg_solve_skeleton(b->probs[i], solver, rtol, maxit, &it, &rel);
      if (iters) iters[i] = it;
      if (relres) relres[i] = rel;
      if (rc) return rc;
      if ((rc = hdg_recover(b->probs[i]))) return rc;
    }
  } else {
    // The problems' skeleton solves are independent: worker threads run them
    // concurrently, each on its own stream.  Everything a solve touches is
    // reserved first on the batch stream, so the workers allocate nothing.
    int rc;
    for (hdg_problem *pb : b->probs)
      if ((rc = solve_reserve(pb))) return rc;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    while ((int)b->workers.size() < nworkers) {
      hdg_context *w = nullptr;
      if ((rc = hdg_context_create(ctx->device, &w))) return ctx->fail(rc, "worker stream creation failed");
      b->workers.push_back(w);
    }
    std::atomic<size_t> next(0);
    std::vector<int> rcs(np, HDG_OK);
    std::vector<std::string> msgs(np);
    std::vector<std::thread> threads;
    for (int t = 0; t < nworkers; ++t)
      threads.emplace_back([&, t] {
        hdg_context *w = b->workers[(size_t)t];
        cudaSetDevice(w->device);
        for (size_t i = next++; i < np; i = next++) {
          hdg_problem *pb = b->probs[i];
          hdg_context *own = pb->ctx;
          pb->ctx = w;  // this solve runs on the worker's stream
          int it = 0;
          double rel = 0.0;
          int r = hdg_solve_skeleton(pb, solver, rtol, maxit, &it, &rel);
          if (r == HDG_OK) r = hdg_recover(pb);
          cudaStreamSynchronize(w->stream);
          if (r != HDG_OK) msgs[i] = w->err;
          pb->ctx = own;
          rcs[i] = r;
          if (iters) iters[i] = it;
          if (relres) relres[i] = rel;
        }
      });
    for (auto &th : threads) th.join();
    for (hdg_context *w : b->workers) {
      ctx->launches += w->launches;
      w->launches = 0;
    }
    for (size_t i = 0; i < np; ++i)
      if (rcs[i] != HDG_OK) return ctx->fail(rcs[i], "problem %zu: %s", i, msgs[i].c_str());
  }
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  b->timings[2] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0).count();
  return HDG_OK;
}

int hdg_batch_timings(const hdg_batch *b, double *ms) {
  if (!b || !ms) return HDG_ERR_INVALID;
  for (int i = 0; i < 3; ++i) ms[i] = b->timings[i];
  return HDG_OK;
}

int hdg_batch_tuning(const hdg_batch *b, int precision, int max_classes, int *D, int *k, int *tpc, double *ms,
                     long long *cells, int *nclasses) {
  if (!b || !nclasses) return HDG_ERR_INVALID;
  const int slot = prec_slot(precision);
  const int nc = (int)b->classes.size();
  *nclasses = nc;
  for (int i = 0; i < nc && i < max_classes; ++i) {
    const auto &cl = b->classes[(size_t)i];
    if (D) D[i] = cl.D;
    if (k) k[i] = cl.k;
    if (tpc) tpc[i] = cl.tpc[slot];
    if (ms) ms[i] = cl.tuned_ms[slot];
    if (cells) cells[i] = cl.total;
  }
  return HDG_OK;
}

}  // extern "C"
