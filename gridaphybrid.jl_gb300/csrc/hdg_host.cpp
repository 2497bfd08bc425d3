// hdg_host.cpp -- host-side set-up of libgridaphybrid_gb300: reference-element
// tables, Cartesian meshes in Gridap numbering, the skeleton CSR pattern and
// the block maps of the deterministic assembly gather.  Runs once per problem.
#include <algorithm>
#include <unordered_map>
#include <cmath>
#include <cstring>

#include "hdg_internal.h"

namespace hdg {

static int ipow(int b, int e) {
  int r = 1;
  while (e-- > 0) r *= b;
  return r;
}

// ---------------------------------------------------------------------------
// Gridap's Lagrangian node order on the D-cube.  Faces are enumerated the way
// an extrusion polytope builds them (faces of the lower cube at x_d = 0, at
// x_d = 1, then extruded along x_d; grouped by dimension, stable), and every
// face owns its interior lattice points, first face parameter fastest.  This
// yields vertices lexicographically, QUAD edges [y0,y1,x0,x1] and HEX facets
// [z0,z1,y0,y1,x0,x1] as in Gridap.ReferenceFEs.
// ---------------------------------------------------------------------------
struct CubeFace {
  int free_mask, fixed;
};

static std::vector<CubeFace> cube_face_list(int D) {
  std::vector<CubeFace> cur{{0, 0}};
  for (int d = 0; d < D; ++d) {
    std::vector<CubeFace> ext;
    for (auto f : cur) ext.push_back({f.free_mask, f.fixed});
    for (auto f : cur) ext.push_back({f.free_mask, f.fixed | (1 << d)});
    for (auto f : cur) ext.push_back({f.free_mask | (1 << d), f.fixed});
    std::stable_sort(ext.begin(), ext.end(), [](const CubeFace &a, const CubeFace &b) {
      return __builtin_popcount(a.free_mask) < __builtin_popcount(b.free_mask);
    });
    cur.swap(ext);
  }
  return cur;
}

std::vector<int> node_lattice(int D, int k) {
  std::vector<int> lat;
  if (D == 0) {
    return lat;
  }
  for (const CubeFace &f : cube_face_list(D)) {
    std::vector<int> dims;
    for (int d = 0; d < D; ++d)
      if (f.free_mask >> d & 1) dims.push_back(d);
    int cnt = ipow(k - 1, (int)dims.size());
    for (int s = 0; s < cnt; ++s) {
      int idx[kMaxD];
      for (int d = 0; d < D; ++d) idx[d] = (f.fixed >> d & 1) ? k : 0;
      int r = s;
      for (int d : dims) {
        idx[d] = 1 + r % (k - 1);
        r /= (k - 1);
      }
      for (int d = 0; d < D; ++d) lat.push_back(idx[d]);
    }
  }
  return lat;
}

// 1D Lagrange polynomial through the equispaced nodes j/k, value + derivative.
void lagrange1d(int k, int i, double x, double &v, double &dv) {
  v = 1.0;
  dv = 0.0;
  const double xi = double(i) / k;
  for (int j = 0; j <= k; ++j) {
    if (j == i) continue;
    const double xj = double(j) / k, den = xi - xj;
    dv = dv * (x - xj) / den + v / den;
    v *= (x - xj) / den;
  }
}

// Gauss-Legendre points/weights on [0,1] by Newton iteration on P_n.
void gauss01(int np, std::vector<double> &x, std::vector<double> &w) {
  x.assign(np, 0.0);
  w.assign(np, 0.0);
  for (int i = 0; i < np; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (np + 0.5)), dp = 1.0;
    for (int it = 0; it < 60; ++it) {
      double p_prev = 1.0, p = z;
      for (int j = 2; j <= np; ++j) {
        double pn = ((2 * j - 1) * z * p - (j - 1) * p_prev) / j;
        p_prev = p;
        p = pn;
      }
      dp = np * (z * p - p_prev) / (z * z - 1.0);
      double step = p / dp;
      z -= step;
      if (std::fabs(step) < 1e-16) break;
    }
    double p_prev = 1.0, p = z;
    for (int j = 2; j <= np; ++j) {
      double pn = ((2 * j - 1) * z * p - (j - 1) * p_prev) / j;
      p_prev = p;
      p = pn;
    }
    dp = np * (z * p - p_prev) / (z * z - 1.0);
    x[np - 1 - i] = 0.5 * (1.0 + z);
    w[np - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

int build_ref_tables(int D, int k, RefTables &t, int phys) {
  if (D < 2 || D > kMaxD || k < 1 || k > kMaxK) return -1;
  t.D = D;
  t.k = k;
  t.phys = phys;
  t.nk = ipow(k + 1, D);
  t.nfs = ipow(k + 1, D - 1);
  if (phys == HDG_PHYSICS_ELASTICITY) {
    // [symmetric stress | displacement] inside, displacement trace on facets
    t.nsym = D * (D + 1) / 2;
    t.ni = (t.nsym + D) * t.nk;
    t.nfd = D * t.nfs;
  } else {
    // [flux | pressure] inside, scalar trace on facets
    t.nsym = 0;
    t.ni = (D + 1) * t.nk;
    t.nfd = t.nfs;
  }
  t.nf = 2 * D * t.nfd;
  t.n = t.ni + t.nf;
  // quadrature degree 2(k+1) as the reference's Measure(., 2*(order+1))
  t.n1 = k + 2;
  t.nqv = ipow(t.n1, D);
  t.lat = node_lattice(D, k);
  t.flat = node_lattice(D - 1, k);
  if (D - 1 == 0) t.flat.clear();
  std::vector<double> x1, w1;
  gauss01(t.n1, x1, w1);
  const int nk = t.nk, nfd = t.nfs;  // scalar facet basis for the tables

  auto eval_cell = [&](const double *xi, double *val, double *grad) {
    for (int a = 0; a < nk; ++a) {
      double l[kMaxD], dl[kMaxD];
      for (int d = 0; d < D; ++d) lagrange1d(k, t.lat[a * D + d], xi[d], l[d], dl[d]);
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
  };

  // volume tables
  t.M.assign(nk * nk, 0.0);
  t.G.assign(D * nk * nk, 0.0);
  t.qxi.assign(t.nqv * D, 0.0);
  t.qw.assign(t.nqv, 0.0);
  t.qphi.assign(t.nqv * nk, 0.0);
  std::vector<double> val(nk), grad(nk * D);
  for (int q = 0; q < t.nqv; ++q) {
    double xi[kMaxD], wq = 1.0;
    for (int d = 0, r = q; d < D; ++d, r /= t.n1) {
      xi[d] = x1[r % t.n1];
      wq *= w1[r % t.n1];
    }
    eval_cell(xi, val.data(), grad.data());
    for (int d = 0; d < D; ++d) t.qxi[q * D + d] = xi[d];
    t.qw[q] = wq;
    for (int a = 0; a < nk; ++a) t.qphi[q * nk + a] = val[a];
    for (int a = 0; a < nk; ++a)
      for (int b = 0; b < nk; ++b) {
        t.M[a * nk + b] += wq * val[a] * val[b];
        for (int e = 0; e < D; ++e) t.G[(e * nk + a) * nk + b] += wq * grad[a * D + e] * val[b];
      }
  }
  // M^{-1} (Gauss-Jordan with partial pivoting, FP64) for the block-elimination path
  {
    std::vector<double> Mw(t.M), Iv(nk * nk, 0.0);
    for (int i = 0; i < nk; ++i) Iv[i * nk + i] = 1.0;
    for (int c = 0; c < nk; ++c) {
      int pr = c;
      for (int i = c + 1; i < nk; ++i)
        if (std::fabs(Mw[i * nk + c]) > std::fabs(Mw[pr * nk + c])) pr = i;
      if (pr != c)
        for (int j = 0; j < nk; ++j) {
          std::swap(Mw[c * nk + j], Mw[pr * nk + j]);
          std::swap(Iv[c * nk + j], Iv[pr * nk + j]);
        }
      const double piv = Mw[c * nk + c];
      for (int j = 0; j < nk; ++j) {
        Mw[c * nk + j] /= piv;
        Iv[c * nk + j] /= piv;
      }
      for (int i = 0; i < nk; ++i) {
        if (i == c) continue;
        const double f = Mw[i * nk + c];
        if (f != 0.0)
          for (int j = 0; j < nk; ++j) {
            Mw[i * nk + j] -= f * Mw[c * nk + j];
            Iv[i * nk + j] -= f * Iv[c * nk + j];
          }
      }
    }
    t.Minv = Iv;
  }
  // M^{-1} G_e, cleaned of rounding noise
  t.MG.assign(D * nk * nk, 0.0);
  for (int e = 0; e < D; ++e) {
    double mx = 0.0;
    for (int a = 0; a < nk; ++a)
      for (int b = 0; b < nk; ++b) {
        double v = 0.0;
        for (int j = 0; j < nk; ++j) v += t.Minv[a * nk + j] * t.G[(e * nk + j) * nk + b];
        t.MG[(e * nk + a) * nk + b] = v;
        mx = std::max(mx, std::fabs(v));
      }
    for (int i = 0; i < nk * nk; ++i)
      if (std::fabs(t.MG[e * nk * nk + i]) < 1e-12 * mx) t.MG[e * nk * nk + i] = 0.0;
  }
  // facet tables: facet parameters are the non-normal directions, increasing
  const int nqf = ipow(t.n1, D - 1);
  t.F.assign(2 * D * nk * nk, 0.0);
  t.H.assign(2 * D * nk * nfd, 0.0);
  t.L.assign(nfd * nfd, 0.0);
  std::vector<double> mu(nfd);
  for (int q = 0; q < nqf; ++q) {
    double s[kMaxD], wq = 1.0;
    for (int d = 0, r = q; d < D - 1; ++d, r /= t.n1) {
      s[d] = x1[r % t.n1];
      wq *= w1[r % t.n1];
    }
    for (int b = 0; b < nfd; ++b) {
      double v = 1.0;
      for (int d = 0; d < D - 1; ++d) {
        double l, dl;
        lagrange1d(k, t.flat[b * (D - 1) + d], s[d], l, dl);
        v *= l;
      }
      mu[b] = v;
    }
    for (int a = 0; a < nfd; ++a)
      for (int b = 0; b < nfd; ++b) t.L[a * nfd + b] += wq * mu[a] * mu[b];
    for (int lf = 0; lf < 2 * D; ++lf) {
      const int dn = D - 1 - lf / 2, side = lf % 2;
      double xi[kMaxD];
      for (int d = 0, j = 0; d < D; ++d) xi[d] = (d == dn) ? double(side) : s[j++];
      eval_cell(xi, val.data(), nullptr);
      for (int a = 0; a < nk; ++a) {
        for (int b = 0; b < nk; ++b) t.F[(lf * nk + a) * nk + b] += wq * val[a] * val[b];
        for (int b = 0; b < nfd; ++b) t.H[(lf * nk + a) * nfd + b] += wq * val[a] * mu[b];
      }
    }
  }
  // M^{-1} H_lf, cleaned of rounding noise
  t.MH.assign(2 * D * nk * nfd, 0.0);
  for (int lf = 0; lf < 2 * D; ++lf) {
    double mx = 0.0;
    for (int a = 0; a < nk; ++a)
      for (int b = 0; b < nfd; ++b) {
        double v = 0.0;
        for (int j = 0; j < nk; ++j) v += t.Minv[a * nk + j] * t.H[(lf * nk + j) * nfd + b];
        t.MH[(lf * nk + a) * nfd + b] = v;
        mx = std::max(mx, std::fabs(v));
      }
    for (int i = 0; i < nk * nfd; ++i)
      if (std::fabs(t.MH[lf * nk * nfd + i]) < 1e-12 * mx) t.MH[lf * nk * nfd + i] = 0.0;
  }
  return 0;
}

void build_l2_ref(const RefTables &t, L2RefHost &r) {
  const int D = t.D, nk = t.nk, nfs = t.nfs, nl = 2 * D;
  r.idx.clear();
  r.val.clear();
  // MG by column: for (e, b) the rows a
  for (int e = 0, cnt = 0; e < D; ++e)
    for (int b = 0; b < nk; ++b) {
      r.idx.push_back(cnt);
      for (int a = 0; a < nk; ++a)
        if (t.MG[(e * nk + a) * nk + b] != 0.0) ++cnt;
      if (e == D - 1 && b == nk - 1) r.idx.push_back(cnt);
    }
  r.off_cidx = (int)r.idx.size();
  r.voff_c = 0;
  for (int e = 0; e < D; ++e)
    for (int b = 0; b < nk; ++b)
      for (int a = 0; a < nk; ++a)
        if (t.MG[(e * nk + a) * nk + b] != 0.0) {
          r.idx.push_back(a);
          r.val.push_back(t.MG[(e * nk + a) * nk + b]);
        }
  // MG by row: for (e, a) the columns b
  r.off_rptr = (int)r.idx.size();
  r.voff_r = (int)r.val.size();
  for (int e = 0, cnt = 0; e < D; ++e)
    for (int a = 0; a < nk; ++a) {
      r.idx.push_back(cnt);
      for (int b = 0; b < nk; ++b)
        if (t.MG[(e * nk + a) * nk + b] != 0.0) ++cnt;
      if (e == D - 1 && a == nk - 1) r.idx.push_back(cnt);
    }
  r.off_ridx = (int)r.idx.size();
  for (int e = 0; e < D; ++e)
    for (int a = 0; a < nk; ++a)
      for (int b = 0; b < nk; ++b)
        if (t.MG[(e * nk + a) * nk + b] != 0.0) {
          r.idx.push_back(b);
          r.val.push_back(t.MG[(e * nk + a) * nk + b]);
        }
  // MH by column: for (lf, fb) the rows a
  r.off_hptr = (int)r.idx.size();
  r.voff_h = (int)r.val.size();
  for (int lf = 0, cnt = 0; lf < nl; ++lf)
    for (int fb = 0; fb < nfs; ++fb) {
      r.idx.push_back(cnt);
      for (int a = 0; a < nk; ++a)
        if (t.MH[(lf * nk + a) * nfs + fb] != 0.0) ++cnt;
      if (lf == nl - 1 && fb == nfs - 1) r.idx.push_back(cnt);
    }
  r.off_hidx = (int)r.idx.size();
  for (int lf = 0; lf < nl; ++lf)
    for (int fb = 0; fb < nfs; ++fb)
      for (int a = 0; a < nk; ++a)
        if (t.MH[(lf * nk + a) * nfs + fb] != 0.0) {
          r.idx.push_back(a);
          r.val.push_back(t.MH[(lf * nk + a) * nfs + fb]);
        }
  // MH dense
  r.voff_hd = (int)r.val.size();
  r.val.insert(r.val.end(), t.MH.begin(), t.MH.end());
}

TableOffsets pack_tables(const RefTables &t, std::vector<double> &packed) {
  TableOffsets o{};
  packed.clear();
  auto put = [&](const std::vector<double> &v) {
    int off = (int)packed.size();
    packed.insert(packed.end(), v.begin(), v.end());
    while (packed.size() % 4) packed.push_back(0.0);  // 32-byte alignment
    return off;
  };
  o.M = put(t.M);
  o.G = put(t.G);
  o.F = put(t.F);
  o.H = put(t.H);
  o.L = put(t.L);
  o.qxi = put(t.qxi);
  o.qw = put(t.qw);
  o.qphi = put(t.qphi);
  o.total = (int)packed.size();
  return o;
}

TableOffsetsF pack_tables_ff(const RefTables &t, std::vector<float> &packed) {
  TableOffsetsF o{};
  packed.clear();
  auto put = [&](const std::vector<double> &v, int &hi_off, int &lo_off) {
    hi_off = (int)packed.size();
    for (double x : v) packed.push_back((float)x);
    while (packed.size() % 8) packed.push_back(0.0f);
    lo_off = (int)packed.size();
    for (double x : v) packed.push_back((float)(x - (double)(float)x));
    while (packed.size() % 8) packed.push_back(0.0f);
  };
  put(t.M, o.Mh, o.Ml);
  put(t.G, o.Gh, o.Gl);
  put(t.F, o.Fh, o.Fl);
  put(t.H, o.Hh, o.Hl);
  put(t.L, o.Lh, o.Ll);
  o.total = (int)packed.size();
  return o;
}

// ---------------------------------------------------------------------------
// Cartesian mesh with Gridap's numbering: cells lexicographic (x fastest);
// facets numbered in the order they are first met looping cells and their
// local facets [.., y0, y1, x0, x1]; facet DOFs facet by facet, boundary
// facets Dirichlet.
// ---------------------------------------------------------------------------
int build_cartesian_mesh(int D, const int *cells, const double *domain, int k,
                         HostMesh &m, std::string &err, int ncomp, int nfd) {
  if (D < 2 || D > kMaxD) {
    err = "D must be 2 or 3";
    return HDG_ERR_INVALID;
  }
  if (k < 1 || k > kMaxK) {
    err = "order k must be in 1..4";
    return HDG_ERR_INVALID;
  }
  long long nc = 1;
  for (int d = 0; d < D; ++d) {
    if (cells[d] < 1) {
      err = "cells per direction must be >= 1";
      return HDG_ERR_INVALID;
    }
    nc *= cells[d];
  }
  if (nc > (1LL << 28)) {
    err = "too many cells";
    return HDG_ERR_INVALID;
  }
  m = HostMesh();
  m.D = D;
  m.k = k;
  m.cartesian = true;
  m.ncells = (int)nc;
  m.nfd = nfd > 0 ? nfd : ncomp * ipow(k + 1, D - 1);
  for (int d = 0; d < D; ++d) {
    m.cells[d] = cells[d];
    m.domain[2 * d] = domain[2 * d];
    m.domain[2 * d + 1] = domain[2 * d + 1];
  }
  const int nl = 2 * D;
  m.nl = nl;
  int stride[kMaxD];
  stride[0] = 1;
  for (int d = 1; d < D; ++d) stride[d] = stride[d - 1] * cells[d - 1];
  m.origin.resize((size_t)m.ncells * D);
  m.jac.assign((size_t)m.ncells * D * D, 0.0);
  m.cell_facets.resize((size_t)m.ncells * nl);
  std::vector<char> boundary;
  boundary.reserve((size_t)m.ncells * 4);
  int next = 0;
  for (int c = 0; c < m.ncells; ++c) {
    int idx[kMaxD];
    int r = c;
    for (int d = 0; d < D; ++d) {
      idx[d] = r % cells[d];
      r /= cells[d];
    }
    for (int d = 0; d < D; ++d) {
      double h = (domain[2 * d + 1] - domain[2 * d]) / cells[d];
      m.origin[(size_t)c * D + d] = domain[2 * d] + idx[d] * h;
      m.jac[(size_t)c * D * D + d * D + d] = h;
    }
    for (int lf = 0; lf < nl; ++lf) {
      const int d = D - 1 - lf / 2, s = lf % 2;
      int f;
      if (s == 0 && idx[d] > 0) {
        f = m.cell_facets[(size_t)(c - stride[d]) * nl + 2 * (D - 1 - d) + 1];
      } else {
        f = next++;
        boundary.push_back(!(s == 1 && idx[d] < cells[d] - 1));
      }
      m.cell_facets[(size_t)c * nl + lf] = f;
    }
  }
  m.nfacets = next;
  m.facet_dofs.resize((size_t)m.nfacets * m.nfd);
  int fr = 0, di = 0;
  for (int f = 0; f < m.nfacets; ++f)
    for (int a = 0; a < m.nfd; ++a)
      m.facet_dofs[(size_t)f * m.nfd + a] = boundary[f] ? -1 - (di++) : fr++;
  return finish_mesh(m, err);
}

// simplexify(CartesianDiscreteModel(domain, cells)): each box (x fastest) is
// split into D! simplices, one per order (lexicographic over the axis
// permutations) in which the path from the box's lowest vertex to its highest
// steps along the axes (Kuhn's triangulation, conforming across boxes).  A
// cell lists its vertices in increasing global order (lattice points, x
// fastest); local facet lf is the face opposite local vertex D - lf; facets
// are numbered in first-met order over (cell, local facet), the first cell is
// the facet's owner, and the facets' DOFs are numbered facet by facet, the
// boundary facets' DOFs Dirichlet.  Cell maps x = x_0 + J xi with column j of
// J the edge from vertex 0 to vertex j+1.
int build_simplex_mesh(int D, const int *cells, const double *domain, int nfd, HostMesh &m, std::string &err) {
  if (D < 2 || D > 3) {
    err = "D must be 2 or 3";
    return HDG_ERR_INVALID;
  }
  long long nbox = 1, nvert = 1;
  int nv[kMaxD];
  for (int d = 0; d < D; ++d) {
    if (cells[d] < 1) {
      err = "cells must be >= 1";
      return HDG_ERR_INVALID;
    }
    nbox *= cells[d];
    nv[d] = cells[d] + 1;
    nvert *= nv[d];
  }
  const int nperm = D == 2 ? 2 : 6;
  if (nbox * nperm > (1LL << 30) || nvert >= (1LL << 21)) {
    err = "mesh too large";
    return HDG_ERR_INVALID;
  }
  m = HostMesh();
  m.D = D;
  m.k = 1;
  m.nl = D + 1;
  m.simplex = true;
  m.cartesian = false;
  m.nfd = nfd;
  m.ncells = (int)(nbox * nperm);
  for (int d = 0; d < D; ++d) {
    m.cells[d] = cells[d];
    m.domain[2 * d] = domain[2 * d];
    m.domain[2 * d + 1] = domain[2 * d + 1];
  }
  static const int perms3[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  static const int perms2[2][3] = {{0, 1, 0}, {1, 0, 0}};
  const int nl = m.nl;
  m.origin.resize((size_t)m.ncells * D);
  m.jac.resize((size_t)m.ncells * D * D);
  m.cell_facets.resize((size_t)m.ncells * nl);
  std::unordered_map<unsigned long long, int> fid;
  fid.reserve((size_t)m.ncells * 3);
  std::vector<char> boundary;
  std::vector<int> first_cell;
  auto vid = [&](const int *idx) {
    long long r = 0, mul = 1;
    for (int d = 0; d < D; ++d) {
      r += idx[d] * mul;
      mul *= nv[d];
    }
    return (int)r;
  };
  auto coord = [&](int v, int d) {
    int r = v;
    for (int e = 0; e < d; ++e) r /= nv[e];
    const int i = r % nv[d];
    return domain[2 * d] + i * (domain[2 * d + 1] - domain[2 * d]) / cells[d];
  };
  int c = 0;
  for (long long b = 0; b < nbox; ++b) {
    int box[kMaxD];
    long long r = b;
    for (int d = 0; d < D; ++d) {
      box[d] = (int)(r % cells[d]);
      r /= cells[d];
    }
    for (int pi = 0; pi < nperm; ++pi, ++c) {
      const int *perm = D == 2 ? perms2[pi] : perms3[pi];
      int cur[kMaxD], verts[kMaxD + 1];
      for (int d = 0; d < D; ++d) cur[d] = box[d];
      verts[0] = vid(cur);
      for (int j = 0; j < D; ++j) {
        ++cur[perm[j]];
        verts[j + 1] = vid(cur);
      }
      std::sort(verts, verts + D + 1);
      for (int d = 0; d < D; ++d) {
        m.origin[(size_t)c * D + d] = coord(verts[0], d);
        for (int j = 0; j < D; ++j)
          m.jac[(size_t)c * D * D + j * D + d] = coord(verts[j + 1], d) - coord(verts[0], d);
      }
      for (int lf = 0; lf < nl; ++lf) {
        const int opp = D - lf;
        unsigned long long key = 0;
        for (int j = 0, sh = 0; j <= D; ++j)
          if (j != opp) {
            key |= (unsigned long long)verts[j] << sh;
            sh += 21;
          }
        auto it = fid.find(key);
        int f;
        if (it == fid.end()) {
          f = (int)first_cell.size();
          fid.emplace(key, f);
          first_cell.push_back(c);
          boundary.push_back(1);
        } else {
          f = it->second;
          boundary[f] = 0;  // a second cell: interior
        }
        m.cell_facets[(size_t)c * nl + lf] = f;
      }
    }
  }
  m.nfacets = (int)first_cell.size();
  m.facet_dofs.resize((size_t)m.nfacets * m.nfd);
  int fr = 0, di = 0;
  for (int f = 0; f < m.nfacets; ++f)
    for (int a = 0; a < m.nfd; ++a) m.facet_dofs[(size_t)f * m.nfd + a] = boundary[f] ? -1 - (di++) : fr++;
  return finish_mesh(m, err);
}

int finish_mesh(HostMesh &m, std::string &err) {
  if (m.nl == 0) m.nl = 2 * m.D;
  const int nl = m.nl, nfd = m.nfd;
  m.facet_cell.assign((size_t)m.nfacets * 2, -1);
  m.facet_lface.assign((size_t)m.nfacets * 2, -1);
  for (int c = 0; c < m.ncells; ++c)
    for (int lf = 0; lf < nl; ++lf) {
      int f = m.cell_facets[(size_t)c * nl + lf];
      if (f < 0 || f >= m.nfacets) {
        err = "cell_facets entry out of range";
        return HDG_ERR_INVALID;
      }
      int slot = m.facet_cell[2 * (size_t)f] < 0 ? 0 : 1;
      if (slot == 1 && m.facet_cell[2 * (size_t)f + 1] >= 0) {
        err = "a facet is shared by more than two cells";
        return HDG_ERR_INVALID;
      }
      m.facet_cell[2 * (size_t)f + slot] = c;
      m.facet_lface[2 * (size_t)f + slot] = lf;
    }
  m.facet_first_dof.assign(m.nfacets, -1);
  int maxfree = -1, nd = 0;
  for (int f = 0; f < m.nfacets; ++f) {
    const int *ids = &m.facet_dofs[(size_t)f * nfd];
    if (ids[0] >= 0) {
      for (int a = 0; a < nfd; ++a)
        if (ids[a] != ids[0] + a) {
          err = "free DOFs of a facet must be consecutive and increasing";
          return HDG_ERR_INVALID;
        }
      m.facet_first_dof[f] = ids[0];
      maxfree = std::max(maxfree, ids[nfd - 1]);
    } else {
      for (int a = 0; a < nfd; ++a) {
        if (ids[a] >= 0) {
          err = "a facet mixes free and Dirichlet DOFs";
          return HDG_ERR_INVALID;
        }
        nd = std::max(nd, -ids[a]);
      }
    }
    if (m.facet_cell[2 * (size_t)f] < 0) {
      err = "a facet belongs to no cell";
      return HDG_ERR_INVALID;
    }
  }
  m.nfree = maxfree + 1;
  m.ndir = nd;
  return HDG_OK;
}

// ---------------------------------------------------------------------------
// Skeleton CSR pattern: every pair of free skeleton DOFs that share a cell,
// sorted columns (the pattern Gridap's SparseMatrixAssembler builds from the
// cell DOF ids).  Each free facet is a block row of nfd rows with identical
// column structure; a block (f,g) gets its values from the cells that contain
// both f and g (two cells on the diagonal block of an interior facet, one
// otherwise), in increasing cell order.
// ---------------------------------------------------------------------------
int build_pattern(const HostMesh &m, HostPattern &p, std::string &err) {
  const int nl = m.nl, nfd = m.nfd;
  p = HostPattern();
  p.nrows = m.nfree;
  std::vector<int> free_facets;
  for (int f = 0; f < m.nfacets; ++f)
    if (m.facet_first_dof[f] >= 0) free_facets.push_back(f);
  std::sort(free_facets.begin(), free_facets.end(),
            [&](int a, int b) { return m.facet_first_dof[a] < m.facet_first_dof[b]; });
  for (size_t i = 0; i < free_facets.size(); ++i)
    if (m.facet_first_dof[free_facets[i]] != (int)i * nfd) {
      err = "free skeleton DOFs must be numbered facet by facet without gaps";
      return HDG_ERR_INVALID;
    }
  p.nblockrows = (int)free_facets.size();
  p.br_facet = free_facets;
  p.br_row0.resize(p.nblockrows);
  p.br_src.assign((size_t)p.nblockrows * 2, -1);
  p.rowptr.assign((size_t)p.nrows + 1, 0);
  p.diag_blk.assign(p.nblockrows, -1);
  // first pass: neighbour lists
  std::vector<int64_t> br_nbr_ptr(p.nblockrows + 1, 0);
  std::vector<int> nbrs;
  nbrs.reserve((size_t)p.nblockrows * (2 * nl - 1));
  for (int br = 0; br < p.nblockrows; ++br) {
    const int f = free_facets[br];
    int tmp[2 * 2 * kMaxD];
    int cnt = 0;
    for (int s = 0; s < 2; ++s) {
      const int c = m.facet_cell[2 * (size_t)f + s];
      if (c < 0) continue;
      p.br_src[2 * (size_t)br + s] = c * nl + m.facet_lface[2 * (size_t)f + s];
      for (int lf = 0; lf < nl; ++lf) {
        int g = m.cell_facets[(size_t)c * nl + lf];
        if (m.facet_first_dof[g] >= 0) tmp[cnt++] = g;
      }
    }
    std::sort(tmp, tmp + cnt, [&](int a, int b) { return m.facet_first_dof[a] < m.facet_first_dof[b]; });
    cnt = (int)(std::unique(tmp, tmp + cnt) - tmp);
    nbrs.insert(nbrs.end(), tmp, tmp + cnt);
    br_nbr_ptr[br + 1] = br_nbr_ptr[br] + cnt;
  }
  p.nblocks = br_nbr_ptr[p.nblockrows];
  p.nnz = p.nblocks * nfd * nfd;
  if (p.nnz > (int64_t)1 << 40) {
    err = "pattern too large";
    return HDG_ERR_INVALID;
  }
  p.colind.resize((size_t)p.nnz);
  p.blk_off.resize((size_t)p.nblocks);
  p.blk_rowlen.resize((size_t)p.nblocks);
  p.blk_src.assign((size_t)p.nblocks * 2, -1);
  int64_t pos = 0;
  for (int br = 0; br < p.nblockrows; ++br) {
    const int f = free_facets[br];
    const int row0 = br * nfd;
    p.br_row0[br] = row0;
    const int64_t b0 = br_nbr_ptr[br], b1 = br_nbr_ptr[br + 1];
    const int rowlen = (int)(b1 - b0) * nfd;
    p.max_rowlen = std::max(p.max_rowlen, rowlen);
    for (int a = 0; a < nfd; ++a) {
      p.rowptr[row0 + a] = pos + (int64_t)a * rowlen;
      for (int64_t b = b0; b < b1; ++b)
        for (int j = 0; j < nfd; ++j)
          p.colind[pos + (int64_t)a * rowlen + (b - b0) * nfd + j] = m.facet_first_dof[nbrs[b]] + j;
    }
    for (int64_t b = b0; b < b1; ++b) {
      const int g = nbrs[b];
      p.blk_off[b] = pos + (b - b0) * nfd;
      p.blk_rowlen[b] = rowlen;
      if (g == f) p.diag_blk[br] = (int)b;
      int ns = 0;
      for (int s = 0; s < 2; ++s) {
        const int c = m.facet_cell[2 * (size_t)f + s];
        if (c < 0) continue;
        const int lf_f = m.facet_lface[2 * (size_t)f + s];
        for (int lg = 0; lg < nl; ++lg)
          if (m.cell_facets[(size_t)c * nl + lg] == g) {
            if (ns >= 2) {
              err = "more than two cells contribute to a skeleton block";
              return HDG_ERR_INVALID;
            }
            p.blk_src[2 * b + ns++] = (c * nl + lf_f) * nl + lg;
          }
      }
    }
    pos += (int64_t)nfd * rowlen;
  }
  p.rowptr[p.nrows] = pos;
  // cells with Dirichlet DOFs (their condensed vector needs the lift)
  for (int c = 0; c < m.ncells; ++c) {
    bool has = false;
    for (int lf = 0; lf < nl && !has; ++lf)
      has = m.facet_first_dof[m.cell_facets[(size_t)c * nl + lf]] < 0;
    if (has) p.dir_cells.push_back(c);
  }
  // per (cell, local facet): the facet's block row (free facets are numbered
  // in block-row order, first DOF = block row * nfd) and whether the cell owns it
  p.cell_blk.assign((size_t)m.ncells * nl, -1);
  for (int c = 0; c < m.ncells; ++c)
    for (int lf = 0; lf < nl; ++lf) {
      const int f = m.cell_facets[(size_t)c * nl + lf];
      const int first = m.facet_first_dof[f];
      if (first < 0) continue;
      p.cell_blk[(size_t)c * nl + lf] = 2 * (first / nfd) + (m.facet_cell[2 * (size_t)f] == c ? 1 : 0);
    }
  return HDG_OK;
}

}  // namespace hdg
