// k_fp64_cell.cuh -- FP64 cell integration and partial elimination, shared by
// the single-problem and the batched kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>

#include "hdg_kernels.h"

namespace hdg {

// ---------------------------------------------------------------------------
// Per-cell geometric factors of the hoisted integrals on an affine cell.
// ---------------------------------------------------------------------------
struct CellFactors {
  double cm;                   // |det J| / kappa
  double cg[3][3];             // -|det J| Jinv[e][d]
  double cn[6][3];             // |J_F| n_d  per local facet
  double ct[6];                // tau s |J_F|
  double detJ;                 // |det J|
  double x0[3], J[3][3];       // affine map x = x0 + J xi
};

// The affine map of cell c (x = x0 + J xi, J column-major in a.jac) and its
// inverse Ji; returns det J.
__device__ __forceinline__ double cell_affine(const CellArgs &a, int c, double J[3][3], double Ji[3][3]) {
  const int D = a.D;
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) J[r][q] = 0.0;
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
    double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
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
  return det;
}

// The volume factors shared by box and simplex cells.
__device__ __forceinline__ double cell_volume_factors(const CellArgs &a, int c, CellFactors &f, double Ji[3][3]) {
  const int D = a.D;
  double J[3][3];
  const double adet = fabs(cell_affine(a, c, J, Ji));
  const double kap = a.kappa ? a.kappa[c] : 1.0;
  f.detJ = adet;
  f.cm = adet / kap;
  for (int e = 0; e < D; ++e)
    for (int d = 0; d < D; ++d) f.cg[e][d] = -adet * Ji[e][d];
  for (int d = 0; d < D; ++d) {
    f.x0[d] = a.origin[(size_t)c * D + d];
    for (int e = 0; e < D; ++e) f.J[d][e] = J[d][e];
  }
  return adet;
}

// Facet factors from the reference normal nh of local facet lf (outward on
// the reference cell) and the ratio of the reference face's measure to its
// parameter domain's: n = J^{-T} nh / |J^{-T} nh|, the facet Jacobian |J_F| =
// |det J| |J^{-T} nh| ratio (Nanson), and tau (n . n_owner) |J_F|.
__device__ __forceinline__ void facet_factors(const CellArgs &a, int c, int nl, int lf, const double *nh,
                                              double ratio, double adet, const double Ji[3][3], CellFactors &f) {
  const int D = a.D;
  double v[3], nv = 0.0;
  for (int d = 0; d < D; ++d) {
    v[d] = 0.0;
    for (int e = 0; e < D; ++e) v[d] += Ji[e][d] * nh[e];  // J^{-T} n_ref
    nv += v[d] * v[d];
  }
  nv = sqrt(nv);
  const double area = adet * nv * ratio;
  for (int d = 0; d < D; ++d) f.cn[lf][d] = area * (v[d] / nv);
  double s = 1.0;
  if (a.stab_mode == 1) {
    const int fct = a.cell_facets[(size_t)c * nl + lf];
    s = (a.facet_cell[2 * (size_t)fct] == c) ? 1.0 : -1.0;  // n . n_owner
  }
  f.ct[lf] = a.tau * s * area;
}

// Box cells: local facet lf has the reference normal +-e_dn, dn = D-1-lf/2
// (Gridap's face numbering), and a unit parameter square.
__device__ __forceinline__ void cell_factors(const CellArgs &a, int c, CellFactors &f) {
  const int D = a.D;
  double Ji[3][3];
  const double adet = cell_volume_factors(a, c, f, Ji);
  for (int lf = 0; lf < 2 * D; ++lf) {
    double nh[3] = {0.0, 0.0, 0.0};
    nh[D - 1 - lf / 2] = (lf % 2) ? 1.0 : -1.0;
    facet_factors(a, c, 2 * D, lf, nh, 1.0, adet, Ji, f);
  }
}

// Simplex cells (vertices v_0 = 0, v_j = e_{j-1} on the reference cell):
// local facet lf is the face opposite vertex D - lf, with reference normal
// (1, .., 1)/sqrt(D) opposite v_0 and -e_{m-1} opposite v_m, parametrised over
// the unit (D-1)-simplex (measure ratio sqrt(D) opposite v_0, 1 otherwise).
__device__ __forceinline__ void cell_factors_simplex(const CellArgs &a, int c, CellFactors &f) {
  const int D = a.D;
  double Ji[3][3];
  const double adet = cell_volume_factors(a, c, f, Ji);
  for (int lf = 0; lf <= D; ++lf) {
    const int opp = D - lf;
    double nh[3] = {0.0, 0.0, 0.0}, ratio = 1.0;
    if (opp == 0) {
      for (int d = 0; d < D; ++d) nh[d] = 1.0 / sqrt((double)D);
      ratio = sqrt((double)D);
    } else {
      nh[opp - 1] = -1.0;
    }
    facet_factors(a, c, D + 1, lf, nh, ratio, adet, Ji, f);
  }
}

// The Darcy block elimination's per-cell coefficients: w[0] = 1/m =
// kappa/|det J| and w[1 + 3e + d] = cg[e][d] / m, so that the flux panel
// Y_d = (1/m) M^{-1} A_{u_d p} = sum_e w[1 + 3e + d] M^{-1} G_e.
__device__ __forceinline__ void cell_y_coef(const CellArgs &a, int c, double *w) {
  CellFactors f;
  cell_factors(a, c, f);
  const double im = (a.kappa ? a.kappa[c] : 1.0) / f.detJ;
  w[0] = im;
  for (int e = 0; e < 3; ++e)
    for (int d = 0; d < 3; ++d) w[1 + 3 * e + d] = (e < a.D && d < a.D) ? f.cg[e][d] * im : 0.0;
}

// Row decode: type 0 = flux (sub = component), 1 = pressure, 2 = skeleton (sub = lf)
__device__ __forceinline__ void decode(int i, int D, int nk, int ni, int nfd,
                                       int &type, int &sub, int &idx) {
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

// Entry (i, j) of the Darcy HDG cell matrix (test/DarcyHDGTests.jl:125-135
// with kappa): volume  v.u/kappa - (div v) p - grad(q).u ;  facets
// (v.n) l + q (u.n) + tau s q p - tau s q l + m (u.n) + tau s m p - tau s m l.
template <typename R>
__device__ __forceinline__ R cell_entry(const CellArgs &a, const CellFactors &f,
                                        int ti, int si, int ii, int tj, int sj,
                                        int jj) {
  const int D = a.D, nk = a.nk, nfd = a.nfd, nl = 2 * D;
  R v = 0;
  if (ti == 0) {
    if (tj == 0) {
      if (si == sj) v = f.cm * a.M[ii * nk + jj];
    } else if (tj == 1) {
      for (int e = 0; e < D; ++e)
        if (f.cg[e][si] != 0.0) v += f.cg[e][si] * a.G[(e * nk + ii) * nk + jj];
    } else {
      v = f.cn[sj][si] * a.H[(sj * nk + ii) * nfd + jj];
    }
  } else if (ti == 1) {
    if (tj == 0) {
      for (int e = 0; e < D; ++e)
        if (f.cg[e][sj] != 0.0) v += f.cg[e][sj] * a.G[(e * nk + ii) * nk + jj];
      for (int lf = 0; lf < nl; ++lf)
        if (f.cn[lf][sj] != 0.0) v += f.cn[lf][sj] * a.F[(lf * nk + ii) * nk + jj];
    } else if (tj == 1) {
      for (int lf = 0; lf < nl; ++lf) v += f.ct[lf] * a.F[(lf * nk + ii) * nk + jj];
    } else {
      v = -f.ct[sj] * a.H[(sj * nk + ii) * nfd + jj];
    }
  } else {
    if (tj == 0) {
      v = f.cn[si][sj] * a.H[(si * nk + jj) * nfd + ii];
    } else if (tj == 1) {
      v = f.ct[si] * a.H[(si * nk + jj) * nfd + ii];
    } else if (si == sj) {
      v = -f.ct[si] * a.L[ii * nfd + jj];
    }
  }
  return v;
}

// Source vector b_i = int f . v over the volume (per-point quadrature, the
// source is not polynomial).  Requires fq[nqv*(D+1)] computed by the caller.
__device__ __forceinline__ void source_values(const CellArgs &a, const CellFactors &f, int c, double *fq,
                                              int t, int nt) {
  const int D = a.D;
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

// ---------------------------------------------------------------------------
// Partial elimination in shared memory (the FP64 StaticCondensationMap).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void warp_argmax(double &v, int &i) {
  for (int off = 16; off > 0; off >>= 1) {
    double ov = __shfl_down_sync(0xffffffffu, v, off);
    int oi = __shfl_down_sync(0xffffffffu, i, off);
    if (ov > v || (ov == v && oi < i)) {
      v = ov;
      i = oi;
    }
  }
}

// Eliminates columns [0, ne) of the n x (ncols) shared block W (ld = n),
// pivot rows searched in [j, npiv).  Returns LAPACK-style info.
// Threads t = 0..nt-1 (nt a multiple of 32) of the caller's group; every
// thread of the CTA must call it (CTA barriers).
__device__ __forceinline__ int eliminate_fp64(double *W, int n, int ncols, int ne, int npiv, int *s_piv, int t,
                                              int nt) {
  const int lane = t & 31, warp = t >> 5, nw = nt >> 5;
  int info = 0;
  for (int j = 0; j < ne; ++j) {
    if (warp == 0) {
      double best = -1.0;
      int bi = j;
      for (int i = j + lane; i < npiv; i += 32) {
        double v = fabs(W[i + (size_t)n * j]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      warp_argmax(best, bi);
      if (lane == 0) *s_piv = (best > 0.0) ? bi : -1;
    }
    __syncthreads();
    // the same barriers on every path: several cells may share a CTA
    const int p = *s_piv;
    const bool ok = p >= 0;
    if (!ok && info == 0) info = j + 1;
    if (ok && p != j)
      for (int c = j + t; c < ncols; c += nt) {
        double tmp = W[j + (size_t)n * c];
        W[j + (size_t)n * c] = W[p + (size_t)n * c];
        W[p + (size_t)n * c] = tmp;
      }
    __syncthreads();
    if (ok) {
      const double r = 1.0 / W[j + (size_t)n * j];
      for (int i = j + 1 + t; i < n; i += nt) W[i + (size_t)n * j] *= r;
    }
    __syncthreads();
    if (ok)
      for (int c = j + 1 + warp; c < ncols; c += nw) {
        const double u = W[j + (size_t)n * c];
        if (u != 0.0)
          for (int i = j + 1 + lane; i < n; i += 32) W[i + (size_t)n * c] -= W[i + (size_t)n * j] * u;
      }
    __syncthreads();
  }
  return info;
}

}  // namespace hdg
