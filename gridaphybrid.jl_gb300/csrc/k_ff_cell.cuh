// k_ff_cell.cuh -- float-float cell integration shared by the single-problem
// and the batched kernels (sm_103a).  A value is the unevaluated sum hi + lo
// of two FP32 numbers (~48 significant bits), computed on the FP32 pipes.
#pragma once
#include <cuda_runtime.h>

#include "hdg_kernels.h"

namespace hdg {

// ---------------------------------------------------------------------------
// float-float helpers (Knuth two-sum, fma two-product)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (acc_hi, acc_lo) += (a_hi + a_lo) * x
__device__ __forceinline__ void ff_mac(float &acc_hi, float &acc_lo, float a_hi, float a_lo, float x) {
  const float p = a_hi * x;
  float pe = fmaf(a_hi, x, -p);
  pe = fmaf(a_lo, x, pe);
  float s, e;
  two_sum(acc_hi, p, s, e);
  acc_hi = s;
  acc_lo += e + pe;
}

// (acc_hi, acc_lo) += (a_hi + a_lo) * (x_hi + x_lo)
__device__ __forceinline__ void ff_mac2(float &acc_hi, float &acc_lo, float a_hi, float a_lo, float x_hi,
                                        float x_lo) {
  const float p = a_hi * x_hi;
  float pe = fmaf(a_hi, x_hi, -p);
  pe = fmaf(a_lo, x_hi, pe);
  pe = fmaf(a_hi, x_lo, pe);
  float s, e;
  two_sum(acc_hi, p, s, e);
  acc_hi = s;
  acc_lo += e + pe;
}

__device__ __forceinline__ void split_double(double v, float &hi, float &lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// ---------------------------------------------------------------------------
// Integration in float-float: entry (i, j) = sum over terms of
// coefficient (cell scalar, float-float) x reference table (float-float).
// ---------------------------------------------------------------------------
struct CellFactorsFF {
  float cm[2];
  float cg[3][3][2];
  float cn[6][3][2];
  float ct[6][2];
  double detJ, x0[3], J[3][3];
};

__device__ __forceinline__ void cell_factors_ff(const CellArgs &a, int c, CellFactorsFF &f) {
  const int D = a.D;
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, Ji[3][3];
  for (int col = 0; col < D; ++col)
    for (int row = 0; row < D; ++row) J[row][col] = a.jac[(size_t)c * D * D + col * D + row];
  double det;
  if (D == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Ji[0][0] = J[1][1] / det;
    Ji[0][1] = -J[0][1] / det;
    Ji[1][0] = -J[1][0] / det;
    Ji[1][1] = J[0][0] / det;
  } else {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    Ji[0][0] = c00 / det;
    Ji[1][0] = c01 / det;
    Ji[2][0] = c02 / det;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  }
  const double adet = fabs(det);
  const double kap = a.kappa ? a.kappa[c] : 1.0;
  f.detJ = adet;
  split_double(adet / kap, f.cm[0], f.cm[1]);
  for (int e = 0; e < 3; ++e)
    for (int d = 0; d < 3; ++d) {
      const double v = (e < D && d < D) ? -adet * Ji[e][d] : 0.0;
      split_double(v, f.cg[e][d][0], f.cg[e][d][1]);
    }
  for (int d = 0; d < D; ++d) {
    f.x0[d] = a.origin[(size_t)c * D + d];
    for (int e = 0; e < D; ++e) f.J[d][e] = J[d][e];
  }
  for (int lf = 0; lf < 2 * D; ++lf) {
    const int dn = D - 1 - lf / 2;
    const double sg = (lf % 2) ? 1.0 : -1.0;
    double v[3], nv = 0.0;
    for (int d = 0; d < D; ++d) {
      v[d] = sg * Ji[dn][d];
      nv += v[d] * v[d];
    }
    nv = sqrt(nv);
    const double area = adet * nv;
    for (int d = 0; d < 3; ++d) {
      const double cnv = d < D ? area * (v[d] / nv) : 0.0;
      split_double(cnv, f.cn[lf][d][0], f.cn[lf][d][1]);
    }
    double s = 1.0;
    if (a.stab_mode == 1) {
      const int fct = a.cell_facets[(size_t)c * 2 * D + lf];
      s = (a.facet_cell[2 * (size_t)fct] == c) ? 1.0 : -1.0;
    }
    split_double(a.tau * s * area, f.ct[lf][0], f.ct[lf][1]);
  }
}

__device__ __forceinline__ void decode_row(int i, int D, int nk, int ni, int nfd, int &type, int &sub,
                                           int &idx) {
  if (i < D * nk) {
    type = 0;
    sub = i / nk;
    idx = i - sub * nk;
  } else if (i < ni) {
    type = 1;
    sub = 0;
    idx = i - D * nk;
  } else {
    type = 2;
    sub = (i - ni) / nfd;
    idx = i - ni - sub * nfd;
  }
}

// acc += coef * table[k]   (coef, table entries float-float)
__device__ __forceinline__ void ff_term(float &h, float &l, const float *coef, const float *Th, const float *Tl,
                                        int k) {
  if (coef[0] == 0.0f) return;
  ff_mac2(h, l, Th[k], Tl[k], coef[0], coef[1]);
}

__device__ __forceinline__ void cell_entry_ff(const CellArgs &a, const MixedTables &T, const CellFactorsFF &f, int ti, int si,
                              int ii, int tj, int sj, int jj, float &h, float &l) {
  const int D = a.D, nk = a.nk, nfd = a.nfd, nl = 2 * D;
  h = 0.0f;
  l = 0.0f;
  float neg[2];
  if (ti == 0) {
    if (tj == 0) {
      if (si == sj) ff_term(h, l, f.cm, T.Mh, T.Ml, ii * nk + jj);
    } else if (tj == 1) {
      for (int e = 0; e < D; ++e) ff_term(h, l, f.cg[e][si], T.Gh, T.Gl, (e * nk + ii) * nk + jj);
    } else {
      ff_term(h, l, f.cn[sj][si], T.Hh, T.Hl, (sj * nk + ii) * nfd + jj);
    }
  } else if (ti == 1) {
    if (tj == 0) {
      for (int e = 0; e < D; ++e) ff_term(h, l, f.cg[e][sj], T.Gh, T.Gl, (e * nk + ii) * nk + jj);
      for (int lf = 0; lf < nl; ++lf) ff_term(h, l, f.cn[lf][sj], T.Fh, T.Fl, (lf * nk + ii) * nk + jj);
    } else if (tj == 1) {
      for (int lf = 0; lf < nl; ++lf) ff_term(h, l, f.ct[lf], T.Fh, T.Fl, (lf * nk + ii) * nk + jj);
    } else {
      neg[0] = -f.ct[sj][0];
      neg[1] = -f.ct[sj][1];
      ff_term(h, l, neg, T.Hh, T.Hl, (sj * nk + ii) * nfd + jj);
    }
  } else {
    if (tj == 0) {
      ff_term(h, l, f.cn[si][sj], T.Hh, T.Hl, (si * nk + jj) * nfd + ii);
    } else if (tj == 1) {
      ff_term(h, l, f.ct[si], T.Hh, T.Hl, (si * nk + jj) * nfd + ii);
    } else if (si == sj) {
      neg[0] = -f.ct[si][0];
      neg[1] = -f.ct[si][1];
      ff_term(h, l, neg, T.Lh, T.Ll, ii * nfd + jj);
    }
  }
  // renormalise so that |lo| <= ulp(hi)/2
  float s, e;
  two_sum(h, l, s, e);
  h = s;
  l = e;
}

// Integrates cell c into (Ah, Al) (column-major n x n) and (bh, bl) (n) with
// threads t = 0..nt-1 of the caller's group; f and fq (nqv*(D+1) doubles) are
// the group's shared scratch.  Every thread of the CTA must call it (it
// contains CTA barriers); threads of groups without a cell pass active=false
// and still reach the barriers.
// skip_uu: the flux-flux block (rows and columns < D*nk) is not written (the
// block elimination uses (|J|/kappa) M_ref^{-1} instead of reading it).
__device__ __forceinline__ void integrate_cell_ff(const CellArgs &a, const MixedTables &T, int c, bool active,
                                                  CellFactorsFF &f, double *fq, float *Ah, float *Al, float *bh,
                                                  float *bl, int t, int nt, bool skip_uu = false) {
  const int n = a.n, D = a.D;
  if (t == 0 && active) cell_factors_ff(a, c, f);
  __syncthreads();
  // the manufactured source is not polynomial: evaluated point by point in FP64
  if (active) {
    const double kap = a.kappa ? a.kappa[c] : 1.0;
    for (int q = t; q < a.nqv; q += nt) {
      double x[3], p, qe[3], fu[3], g;
      for (int d = 0; d < D; ++d) {
        x[d] = f.x0[d];
        for (int e = 0; e < D; ++e) x[d] += f.J[d][e] * a.qxi[q * D + e];
      }
      exact_solution(a.problem, D, x, kap, p, qe, fu, g);
      const double w = a.qw[q] * f.detJ;
      for (int d = 0; d < D; ++d) fq[q * (D + 1) + d] = w * fu[d];
      fq[q * (D + 1) + D] = w * g;
    }
  }
  __syncthreads();
  if (active) {
    const int nu = skip_uu ? D * a.nk : 0;
    for (int e = t; e < n * n; e += nt) {
      const int j = e / n, i = e - j * n;
      if (i < nu && j < nu) continue;
      int ti, si, ii, tj, sj, jj;
      decode_row(i, D, a.nk, a.ni, a.nfd, ti, si, ii);
      decode_row(j, D, a.nk, a.ni, a.nfd, tj, sj, jj);
      float h, l;
      cell_entry_ff(a, T, f, ti, si, ii, tj, sj, jj, h, l);
      Ah[e] = h;
      Al[e] = l;
    }
    for (int i = t; i < n; i += nt) {
      int ti, si, ii;
      decode_row(i, D, a.nk, a.ni, a.nfd, ti, si, ii);
      double v = 0.0;
      if (ti < 2) {
        const int comp = ti == 0 ? si : D;
        for (int q = 0; q < a.nqv; ++q) v += fq[q * (D + 1) + comp] * a.qphi[q * a.nk + ii];
      }
      float h, l;
      split_double(v, h, l);
      bh[i] = h;
      bl[i] = l;
    }
  }
  __syncthreads();
}

// 1/m = kappa / |det J| of cell c in FP64 (the flux mass block is m (I (x) M_ref))
__device__ __forceinline__ double cell_inv_mass(const CellArgs &a, int c) {
  const int D = a.D;
  const double *J = a.jac + (size_t)c * D * D;
  double det;
  if (D == 2) {
    det = J[0] * J[3] - J[2] * J[1];
  } else {
    det = J[0] * (J[4] * J[8] - J[7] * J[5]) - J[3] * (J[1] * J[8] - J[7] * J[2]) + J[6] * (J[1] * J[5] - J[4] * J[2]);
  }
  const double kap = a.kappa ? a.kappa[c] : 1.0;
  return kap / fabs(det);
}

}  // namespace hdg
