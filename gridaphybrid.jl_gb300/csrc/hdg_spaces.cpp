// hdg_spaces.cpp -- reference bases and tables of the general-space cell
// forms: fields with their own polynomial spaces and orders, Q_k (tensor
// product) or P_k (total degree), as the reference's tests choose them with
// ReferenceFE(lagrangian, T, order; space=:P) (test/DarcyHDGTests.jl:34-36,
// test/LinearElasticityHDGTests.jl:88-93).
//
// On an affine cell with cell-constant coefficients every entry of these
// forms is a reference integral times per-cell geometric factors, so the
// tables below are contracted once on the host (FP64) and the GPU kernels
// combine them per cell.
#include <algorithm>
#include <cmath>

#include "hdg_internal.h"

namespace hdg {

namespace {

int ipow_i(int b, int e) {
  int r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

// Gauss-Jordan inverse with partial pivoting (n x n, row-major, in place); false if singular.
bool invert(std::vector<double> &A, int n) {
  std::vector<double> I(n * n, 0.0);
  for (int i = 0; i < n; ++i) I[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int pr = c;
    for (int i = c + 1; i < n; ++i)
      if (std::fabs(A[i * n + c]) > std::fabs(A[pr * n + c])) pr = i;
    if (!(std::fabs(A[pr * n + c]) > 0.0)) return false;
    if (pr != c)
      for (int j = 0; j < n; ++j) {
        std::swap(A[c * n + j], A[pr * n + j]);
        std::swap(I[c * n + j], I[pr * n + j]);
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
  A = I;
  return true;
}

}  // namespace

int ScalarBasis::init(int dim, int basis_kind, int order) {
  d = dim;
  kind = basis_kind;
  k = order;
  lat.clear();
  mono.clear();
  coef.clear();
  nodes.clear();
  aniso = false;
  if (d < 0 || d > kMaxD || k < 0 || k > kMaxK) return -1;
  if (kind == kBasisQ && k == 0) {  // Q_0: the constant
    const int zero[kMaxD] = {0, 0, 0};
    return init_aniso(dim, zero);
  }
  if (kind == kBasisQ) {
    // Gridap's Lagrangian node order (vertices, then edges, faces, interior)
    nb = ipow_i(k + 1, d);
    lat = node_lattice(d, k);
    nodes.resize((size_t)nb * std::max(d, 1));
    for (int a = 0; a < nb; ++a)
      for (int e = 0; e < d; ++e) nodes[(size_t)a * d + e] = double(lat[(size_t)a * d + e]) / k;
    return 0;
  }
  if (kind != kBasisP) return -1;
  // exponents with total degree <= k, first dimension fastest
  std::vector<int> e(std::max(d, 1), 0);
  for (int a = 0; a < ipow_i(k + 1, d); ++a) {
    int s = 0;
    for (int j = 0, r = a; j < d; ++j, r /= (k + 1)) {
      e[j] = r % (k + 1);
      s += e[j];
    }
    if (s <= k)
      for (int j = 0; j < d; ++j) mono.push_back(e[j]);
  }
  if (d == 0) mono.clear();
  nb = d == 0 ? 1 : (int)mono.size() / d;
  // Lagrange at the simplex lattice points x = i / k (the centroid for k = 0)
  nodes.resize((size_t)nb * std::max(d, 1));
  for (int a = 0; a < nb; ++a)
    for (int j = 0; j < d; ++j) nodes[(size_t)a * d + j] = k == 0 ? 0.5 : double(mono[(size_t)a * d + j]) / k;
  // basis a = sum_m coef[a][m] x^mono_m with phi_a(node_b) = delta_ab:
  // coef = V^{-T}, V[b][m] = node_b^mono_m
  std::vector<double> V((size_t)nb * nb);
  for (int b = 0; b < nb; ++b)
    for (int m = 0; m < nb; ++m) {
      double v = 1.0;
      for (int j = 0; j < d; ++j) v *= std::pow(nodes[(size_t)b * d + j], mono[(size_t)m * d + j]);
      V[(size_t)b * nb + m] = v;
    }
  if (!invert(V, nb)) return -1;
  coef.resize((size_t)nb * nb);
  for (int a = 0; a < nb; ++a)
    for (int m = 0; m < nb; ++m) coef[(size_t)a * nb + m] = V[(size_t)m * nb + a];
  return 0;
}

int ScalarBasis::init_aniso(int dim, const int *orders) {
  d = dim;
  kind = kBasisQ;
  aniso = true;
  k = 0;
  lat.clear();
  mono.clear();
  coef.clear();
  nodes.clear();
  if (d < 0 || d > kMaxD) return -1;
  nb = 1;
  for (int e = 0; e < d; ++e) {
    if (orders[e] < 0 || orders[e] > kMaxK) return -1;
    ko[e] = orders[e];
    k = std::max(k, orders[e]);
    nb *= orders[e] + 1;
  }
  lat.resize((size_t)nb * std::max(d, 1));
  nodes.resize((size_t)nb * std::max(d, 1));
  for (int a = 0; a < nb; ++a)
    for (int e = 0, r = a; e < d; r /= (ko[e] + 1), ++e) {
      const int i = r % (ko[e] + 1);
      lat[(size_t)a * d + e] = i;
      nodes[(size_t)a * d + e] = ko[e] == 0 ? 0.5 : double(i) / ko[e];
    }
  return 0;
}

void ScalarBasis::eval(const double *xi, double *val, double *grad) const {
  if (aniso) {
    for (int a = 0; a < nb; ++a) {
      double l[kMaxD], dl[kMaxD];
      for (int e = 0; e < d; ++e) {
        if (ko[e] == 0) {
          l[e] = 1.0;
          dl[e] = 0.0;
        } else {
          lagrange1d(ko[e], lat[(size_t)a * d + e], xi[e], l[e], dl[e]);
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
          grad[(size_t)a * d + e] = g;
        }
    }
    return;
  }
  if (kind == kBasisQ) {
    for (int a = 0; a < nb; ++a) {
      double l[kMaxD], dl[kMaxD];
      for (int e = 0; e < d; ++e) lagrange1d(k, lat[(size_t)a * d + e], xi[e], l[e], dl[e]);
      double v = 1.0;
      for (int e = 0; e < d; ++e) v *= l[e];
      val[a] = v;
      if (grad)
        for (int e = 0; e < d; ++e) {
          double g = dl[e];
          for (int j = 0; j < d; ++j)
            if (j != e) g *= l[j];
          grad[(size_t)a * d + e] = g;
        }
    }
    return;
  }
  // monomials and their derivatives at xi
  std::vector<double> mv(nb), md((size_t)nb * std::max(d, 1));
  for (int m = 0; m < nb; ++m) {
    double v = 1.0;
    for (int j = 0; j < d; ++j) v *= std::pow(xi[j], mono[(size_t)m * d + j]);
    mv[m] = v;
    for (int e = 0; e < d; ++e) {
      const int pe = mono[(size_t)m * d + e];
      double g = pe == 0 ? 0.0 : pe * std::pow(xi[e], pe - 1);
      for (int j = 0; j < d; ++j)
        if (j != e) g *= std::pow(xi[j], mono[(size_t)m * d + j]);
      md[(size_t)m * d + e] = g;
    }
  }
  for (int a = 0; a < nb; ++a) {
    double v = 0.0;
    for (int m = 0; m < nb; ++m) v += coef[(size_t)a * nb + m] * mv[m];
    val[a] = v;
    if (grad)
      for (int e = 0; e < d; ++e) {
        double g = 0.0;
        for (int m = 0; m < nb; ++m) g += coef[(size_t)a * nb + m] * md[(size_t)m * d + e];
        grad[(size_t)a * d + e] = g;
      }
  }
}

// Cell-local coordinates of local facet lf's point with facet parameters s
// (the non-normal dimensions in increasing order; Gridap's face numbering
// through lf = 2 (D - 1 - normal dimension) + side).
static void facet_point(int D, int lf, const double *sp, double *xi) {
  const int dn = D - 1 - lf / 2, side = lf % 2;
  for (int d = 0, j = 0; d < D; ++d) xi[d] = (d == dn) ? double(side) : sp[j++];
}

// Reference simplex: vertices v_0 = 0, v_j = e_{j-1}; local facet lf is the
// face opposite vertex D - lf, parametrised over the unit (D-1)-simplex by its
// vertices in increasing order.
static void simplex_facet_point(int D, int lf, const double *sp, double *xi) {
  static const double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  int fv[kMaxD], k = 0;
  for (int v = 0; v <= D; ++v)
    if (v != D - lf) fv[k++] = v;
  for (int d = 0; d < D; ++d) {
    xi[d] = V[fv[0]][d];
    for (int j = 0; j + 1 < D; ++j) xi[d] += sp[j] * (V[fv[j + 1]][d] - V[fv[0]][d]);
  }
}

// Collapsed (Duffy) Gauss rule on the unit d-simplex from n1 Gauss points per
// direction: xi_1 = u_1, xi_2 = u_2 (1 - u_1), xi_3 = u_3 (1 - u_1)(1 - u_2);
// exact for degree 2 n1 - d (the collapse adds d - 1 to the degree in u_1).
static void simplex_rule(int d, int n1, const std::vector<double> &x1, const std::vector<double> &w1,
                         std::vector<double> &xi, std::vector<double> &w) {
  const int nq = d == 0 ? 1 : ipow_i(n1, d);
  xi.assign((size_t)nq * (d > 0 ? d : 1), 0.0);
  w.assign(nq, 0.0);
  for (int q = 0; q < nq; ++q) {
    double u[kMaxD] = {0, 0, 0}, wt = 1.0, scale = 1.0;
    for (int j = 0, r = q; j < d; ++j, r /= n1) {
      u[j] = x1[r % n1];
      wt *= w1[r % n1];
    }
    for (int j = 0; j < d; ++j) {
      xi[(size_t)q * d + j] = u[j] * scale;
      if (j + 1 < d) {
        wt *= std::pow(1.0 - u[j], d - 1 - j);
        scale *= 1.0 - u[j];
      }
    }
    w[q] = wt;
  }
}

int build_gs_tables(int D, int phys, const int *spaces, int copies, GsTables &t, std::string &err, bool simplex) {
  t = GsTables();
  if (D < 2 || D > kMaxD) {
    err = "D must be 2 or 3";
    return HDG_ERR_INVALID;
  }
  if (phys != HDG_PHYSICS_DARCY && phys != HDG_PHYSICS_ELASTICITY) {
    err = "unknown physics";
    return HDG_ERR_INVALID;
  }
  if (copies < 1 || copies > 4) {
    err = "copies must be 1..4";
    return HDG_ERR_INVALID;
  }
  for (int i = 0; i < 7; ++i) t.spaces[i] = spaces[i];
  const int nsym = D * (D + 1) / 2;
  t.ncA = phys == HDG_PHYSICS_DARCY ? D : nsym;
  t.ncB = phys == HDG_PHYSICS_DARCY ? 1 : D;
  t.ncT = phys == HDG_PHYSICS_DARCY ? 1 : D;
  bool ok = true;
  if (spaces[0] == kBasisRT) {
    if (phys != HDG_PHYSICS_DARCY || spaces[1] < 0 || spaces[1] > 3) {
      err = "RT_k (k = 0..3) is a flux space of the Darcy form";
      return HDG_ERR_INVALID;
    }
    for (int c = 0; c < D; ++c) {
      int ord[kMaxD];
      for (int e = 0; e < D; ++e) ord[e] = spaces[1] + (e == c ? 1 : 0);
      ok = ok && t.A[c].init_aniso(D, ord) == 0;
    }
  } else {
    ok = t.A[0].init(D, spaces[0], spaces[1]) == 0;
    for (int c = 1; c < t.ncA && ok; ++c) t.A[c] = t.A[0];
  }
  ok = ok && t.B.init(D, spaces[2], spaces[3]) == 0 && t.T.init(D - 1, spaces[4], spaces[5]) == 0;
  if (!ok) {
    err = "unsupported space (kind Q or P of order 0..4; RT_k, k = 0..3, for the Darcy flux)";
    return HDG_ERR_INVALID;
  }
  if (simplex && (phys != HDG_PHYSICS_DARCY || spaces[0] != kBasisP || spaces[2] != kBasisP ||
                  spaces[4] != kBasisP || spaces[6] != 0)) {
    err = "simplex cells take the Darcy form with P_k fields";
    return HDG_ERR_INVALID;
  }
  t.D = D;
  t.phys = phys;
  t.copies = copies;
  t.simplex = simplex;
  t.nl = simplex ? D + 1 : 2 * D;
  t.pm = spaces[6] != 0 && phys == HDG_PHYSICS_ELASTICITY;
  t.nA = t.A[0].nb;
  t.nB = t.B.nb;
  t.nT = t.T.nb;
  t.ni1 = t.ncA * t.nA + t.ncB * t.nB;
  t.nfd1 = t.ncT * t.nT;
  t.ni = copies * t.ni1;
  t.nfd = copies * t.nfd1;
  t.nf = t.nl * t.nfd;
  t.n = t.ni + t.nf;
  int kmax = std::max(spaces[3], spaces[5]);
  for (int c = 0; c < t.ncA; ++c) kmax = std::max(kmax, t.A[c].k);
  t.n1 = kmax + 2;  // Gauss points per direction: exact for degree 2 kmax + 3 (box), 2 kmax + 4 - D (simplex)
  const int nl = t.nl, ncA = t.ncA;
  const int nA = t.nA, nB = t.nB, nT = t.nT;
  std::vector<double> x1, w1;
  gauss01(t.n1, x1, w1);
  // volume and facet rules: tensor Gauss on the unit box / cube, or the
  // collapsed rules on the unit simplices
  std::vector<double> vxi, vw, fs, fw;
  if (simplex) {
    simplex_rule(D, t.n1, x1, w1, vxi, vw);
    simplex_rule(D - 1, t.n1, x1, w1, fs, fw);
  } else {
    const int nv = ipow_i(t.n1, D), nfq = ipow_i(t.n1, D - 1);
    vxi.assign((size_t)nv * D, 0.0);
    vw.assign(nv, 1.0);
    for (int q = 0; q < nv; ++q)
      for (int d = 0, r = q; d < D; ++d, r /= t.n1) {
        vxi[(size_t)q * D + d] = x1[r % t.n1];
        vw[q] *= w1[r % t.n1];
      }
    fs.assign((size_t)nfq * (D - 1), 0.0);
    fw.assign(nfq, 1.0);
    for (int q = 0; q < nfq; ++q)
      for (int d = 0, r = q; d < D - 1; ++d, r /= t.n1) {
        fs[(size_t)q * (D - 1) + d] = x1[r % t.n1];
        fw[q] *= w1[r % t.n1];
      }
  }
  t.nqv = (int)vw.size();
  const int nqf = (int)fw.size();
  size_t o = 0;
  auto take = [&](int &off, size_t count) {
    off = (int)o;
    o += count;
  };
  take(t.oMAA, (size_t)ncA * nA * nA);
  take(t.oGAB, (size_t)ncA * D * nA * nB);
  take(t.oGBA, (size_t)ncA * D * nB * nA);
  take(t.oFBA, (size_t)ncA * nl * nB * nA);
  take(t.oFBB, (size_t)nl * nB * nB);
  take(t.oHA, (size_t)ncA * nl * nA * nT);
  take(t.oHB, (size_t)nl * nB * nT);
  take(t.oL, (size_t)nT * nT);
  take(t.oqxi, (size_t)t.nqv * D);
  take(t.oqw, (size_t)t.nqv);
  take(t.oqphiA, (size_t)ncA * t.nqv * nA);
  take(t.oqphiB, (size_t)t.nqv * nB);
  t.packed.assign(o, 0.0);
  double *P = t.packed.data();
  std::vector<double> pA(nA), dA((size_t)nA * D), pB(nB), dB((size_t)nB * D), mu(nT);
  // volume
  for (int q = 0; q < t.nqv; ++q) {
    double xi[kMaxD];
    for (int d = 0; d < D; ++d) xi[d] = vxi[(size_t)q * D + d];
    const double wq = vw[q];
    t.B.eval(xi, pB.data(), dB.data());
    for (int d = 0; d < D; ++d) P[t.oqxi + q * D + d] = xi[d];
    P[t.oqw + q] = wq;
    for (int b = 0; b < nB; ++b) P[t.oqphiB + (size_t)q * nB + b] = pB[b];
    for (int c = 0; c < ncA; ++c) {
      t.A[c].eval(xi, pA.data(), dA.data());
      for (int a = 0; a < nA; ++a) P[t.oqphiA + ((size_t)c * t.nqv + q) * nA + a] = pA[a];
      for (int a = 0; a < nA; ++a) {
        for (int a2 = 0; a2 < nA; ++a2) P[t.oMAA + ((size_t)c * nA + a) * nA + a2] += wq * pA[a] * pA[a2];
        for (int b = 0; b < nB; ++b)
          for (int e = 0; e < D; ++e) {
            P[t.oGAB + (((size_t)c * D + e) * nA + a) * nB + b] += wq * dA[(size_t)a * D + e] * pB[b];
            P[t.oGBA + (((size_t)c * D + e) * nB + b) * nA + a] += wq * dB[(size_t)b * D + e] * pA[a];
          }
      }
    }
  }
  // facets, over the facet's parameter domain (unit box or unit simplex)
  for (int q = 0; q < nqf; ++q) {
    double sp[kMaxD] = {0, 0, 0};
    for (int d = 0; d < D - 1; ++d) sp[d] = fs[(size_t)q * (D - 1) + d];
    const double wq = fw[q];
    t.T.eval(sp, mu.data(), nullptr);
    for (int m = 0; m < nT; ++m)
      for (int m2 = 0; m2 < nT; ++m2) P[t.oL + (size_t)m * nT + m2] += wq * mu[m] * mu[m2];
    for (int lf = 0; lf < nl; ++lf) {
      double xi[kMaxD];
      if (simplex)
        simplex_facet_point(D, lf, sp, xi);
      else
        facet_point(D, lf, sp, xi);
      t.B.eval(xi, pB.data(), nullptr);
      for (int b = 0; b < nB; ++b) {
        for (int b2 = 0; b2 < nB; ++b2) P[t.oFBB + ((size_t)lf * nB + b) * nB + b2] += wq * pB[b] * pB[b2];
        for (int m = 0; m < nT; ++m) P[t.oHB + ((size_t)lf * nB + b) * nT + m] += wq * pB[b] * mu[m];
      }
      for (int c = 0; c < ncA; ++c) {
        t.A[c].eval(xi, pA.data(), nullptr);
        for (int b = 0; b < nB; ++b)
          for (int a = 0; a < nA; ++a) P[t.oFBA + (((size_t)c * nl + lf) * nB + b) * nA + a] += wq * pB[b] * pA[a];
        for (int a = 0; a < nA; ++a)
          for (int m = 0; m < nT; ++m) P[t.oHA + (((size_t)c * nl + lf) * nA + a) * nT + m] += wq * pA[a] * mu[m];
      }
    }
  }
  if (t.pm) {
    // P_m(phiB_c) on facet lf = sum_m (L^{-1} H_B^T)[m][c] mu_m, so the tau w.P_m(u)
    // block is H_B L^{-1} H_B^T (src/GridapAPIExtensions.jl:453-500; the tau mu.P_m(u)
    // block equals tau mu.u because L L^{-1} H_B^T = H_B^T)
    std::vector<double> Li(P + t.oL, P + t.oL + (size_t)nT * nT);
    if (!invert(Li, nT)) {
      err = "singular trace mass matrix";
      return HDG_ERR_INVALID;
    }
    for (int lf = 0; lf < nl; ++lf) {
      const double *H = P + t.oHB + (size_t)lf * nB * nT;
      std::vector<double> X((size_t)nT * nB, 0.0);  // L^{-1} H^T
      for (int m = 0; m < nT; ++m)
        for (int c = 0; c < nB; ++c) {
          double v = 0.0;
          for (int m2 = 0; m2 < nT; ++m2) v += Li[(size_t)m * nT + m2] * H[(size_t)c * nT + m2];
          X[(size_t)m * nB + c] = v;
        }
      for (int b = 0; b < nB; ++b)
        for (int c = 0; c < nB; ++c) {
          double v = 0.0;
          for (int m = 0; m < nT; ++m) v += H[(size_t)b * nT + m] * X[(size_t)m * nB + c];
          P[t.oFBB + ((size_t)lf * nB + b) * nB + c] = v;
        }
    }
  }
  return HDG_OK;
}

}  // namespace hdg
