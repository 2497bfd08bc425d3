// k_elast_cell.cuh -- one linear elasticity HDG cell (test/LinearElasticityHDGTests.jl:140-150
// without the P_m projection, compliance :15-38), shared by the integration
// kernel and the fused block elimination.  DOFs per cell: [symmetric stress
// (nsym comps x nk) | displacement (D x nk) | displacement trace per local
// facet (D x nfs)], component-major.  Every entry is a short sum of reference
// tables (M, G, F, H, L) times the affine cell's factors.
#pragma once
#include <cuda_runtime.h>

#include "hdg_kernels.h"
#include "k_ff_cell.cuh"
#include "k_fp64_cell.cuh"

namespace hdg {

struct ElastRow {
  int type, comp, node, lf;  // type 0 stress, 1 displacement, 2 trace (local facet lf)
};

__device__ __forceinline__ ElastRow elast_decode(const CellArgs &a, int i) {
  ElastRow r;
  const int nk = a.nk, ns = a.nsym;
  if (i < ns * nk) {
    r.type = 0;
    r.comp = i / nk;
    r.node = i - r.comp * nk;
    r.lf = -1;
  } else if (i < a.ni) {
    const int j = i - ns * nk;
    r.type = 1;
    r.comp = j / nk;
    r.node = j - r.comp * nk;
    r.lf = -1;
  } else {
    const int j = i - a.ni;
    r.lf = j / a.nfd;
    const int m = j - r.lf * a.nfd;
    r.type = 2;
    r.comp = m / a.nfs;
    r.node = m - r.comp * a.nfs;
  }
  return r;
}

// Per-cell factors of the entries, from the affine map and the compliance:
//   dterm[c][k][e] = sum_jj E_c(k, jj) cg[e][jj]   (the divergence coupling)
//   nterm[c][k][lf] = sum_jj E_c(k, jj) cn[lf][jj]  (the normal coupling)
//   cmj[c][d] = C_nu[c][d] |J|
struct ElastCellTerms {
  double dterm[6][3][3], nterm[6][3][6], cmj[6][6];
};

// DOF i of the cell packed as type | comp << 2 | lf << 5 | node << 8
__device__ __forceinline__ int elast_pack(const CellArgs &a, int i) {
  const ElastRow r = elast_decode(a, i);
  return r.type | r.comp << 2 | (r.lf < 0 ? 0 : r.lf) << 5 | r.node << 8;
}

__device__ __forceinline__ double elast_entry_t(const CellArgs &a, const CellFactors &f, const ElastCellTerms &T,
                                                int ri, int si) {
  const int nk = a.nk, nfs = a.nfs;
  const int rt = ri & 3, rc = (ri >> 2) & 7, rl = (ri >> 5) & 7, rn = ri >> 8;
  const int st = si & 3, sc = (si >> 2) & 7, sl = (si >> 5) & 7, sn = si >> 8;
  const double *G = a.G, *H = a.H;
  if (rt == 0) {
    if (st == 0) return T.cmj[rc][sc] * a.M[rn * nk + sn];
    if (st == 1) {  // (div v).u
      double v = 0.0;
      for (int e = 0; e < a.D; ++e) v -= T.dterm[rc][sc][e] * G[(e * nk + rn) * nk + sn];
      return v;
    }
    return -T.nterm[rc][sc][sl] * H[(sl * nk + rn) * nfs + sn];  // -(v.n).uhat
  }
  if (rt == 1) {
    if (st == 0) {  // -w.(div sigma)
      double v = 0.0;
      for (int e = 0; e < a.D; ++e) v += T.dterm[sc][rc][e] * G[(e * nk + sn) * nk + rn];
      return v;
    }
    if (rc != sc) return 0.0;
    if (st == 1) {  // tau w.u
      double v = 0.0;
      for (int lf = 0; lf < 2 * a.D; ++lf) v += f.ct[lf] * a.F[(lf * nk + rn) * nk + sn];
      return v;
    }
    return -f.ct[sl] * H[(sl * nk + rn) * nfs + sn];  // -tau w.uhat
  }
  if (st == 0) return T.nterm[sc][rc][rl] * H[(rl * nk + sn) * nfs + rn];  // mu.(sigma.n)
  if (rc != sc) return 0.0;
  if (st == 1) return -f.ct[rl] * H[(rl * nk + sn) * nfs + rn];  // -tau mu.u
  return rl == sl ? f.ct[rl] * a.L[rn * nfs + sn] : 0.0;         // tau mu.uhat
}

// The same entry in float-float from the float-float reference tables and
// the cell terms split into (hi, lo) pairs (TF: dterm, nterm, cmj, ct in the
// order of ElastCellTerms followed by ct[6]) -- FP32 pipes only.
struct ElastCellTermsFF {
  float dterm[6][3][3][2], nterm[6][3][6][2], cmj[6][6][2], ct[6][2];
};

__device__ __forceinline__ void ffc(float &h, float &l, const float *Th, const float *Tl, int k, const float *cf,
                                    bool neg) {
  if (cf[0] == 0.0f) return;
  ff_mac2(h, l, Th[k], Tl[k], neg ? -cf[0] : cf[0], neg ? -cf[1] : cf[1]);
}

__device__ __forceinline__ void elast_entry_ff(const CellArgs &a, const MixedTables &Tb, const ElastCellTermsFF &T,
                                               int ri, int si, float &h, float &l) {
  const int nk = a.nk, nfs = a.nfs;
  const int rt = ri & 3, rc = (ri >> 2) & 7, rl = (ri >> 5) & 7, rn = ri >> 8;
  const int st = si & 3, sc = (si >> 2) & 7, sl = (si >> 5) & 7, sn = si >> 8;
  h = 0.0f;
  l = 0.0f;
  if (rt == 0) {
    if (st == 0) {
      ffc(h, l, Tb.Mh, Tb.Ml, rn * nk + sn, T.cmj[rc][sc], false);
    } else if (st == 1) {
      for (int e = 0; e < a.D; ++e) ffc(h, l, Tb.Gh, Tb.Gl, (e * nk + rn) * nk + sn, T.dterm[rc][sc][e], true);
    } else {
      ffc(h, l, Tb.Hh, Tb.Hl, (sl * nk + rn) * nfs + sn, T.nterm[rc][sc][sl], true);
    }
  } else if (rt == 1) {
    if (st == 0) {
      for (int e = 0; e < a.D; ++e) ffc(h, l, Tb.Gh, Tb.Gl, (e * nk + sn) * nk + rn, T.dterm[sc][rc][e], false);
    } else if (rc == sc) {
      if (st == 1)
        for (int lf = 0; lf < 2 * a.D; ++lf) ffc(h, l, Tb.Fh, Tb.Fl, (lf * nk + rn) * nk + sn, T.ct[lf], false);
      else
        ffc(h, l, Tb.Hh, Tb.Hl, (sl * nk + rn) * nfs + sn, T.ct[sl], true);
    }
  } else {
    if (st == 0)
      ffc(h, l, Tb.Hh, Tb.Hl, (rl * nk + sn) * nfs + rn, T.nterm[sc][rc][rl], false);
    else if (rc == sc && st == 1)
      ffc(h, l, Tb.Hh, Tb.Hl, (rl * nk + sn) * nfs + rn, T.ct[rl], true);
    else if (rc == sc && rl == sl)
      ffc(h, l, Tb.Lh, Tb.Ll, rn * nfs + sn, T.ct[rl], false);
  }
  float s, e;
  two_sum(h, l, s, e);
  h = s;
  l = e;
}

// Everything an entry needs, per cell (shared memory of the caller).
struct ElastScratch {
  CellFactors f;
  ElastCellTerms T;
  ElastCellTermsFF TF;
};

// Cell c's factors and terms (and their float-float split when ff) and the
// body-force values -w.f per quadrature point (fq: nqv x D).  Every thread of
// the CTA calls it (CTA barriers); t / nt: this thread and the thread count.
__device__ __forceinline__ void elast_cell_prepare(const CellArgs &a, int c, ElastScratch &S, double *fq, bool ff,
                                                   int t, int nt, const CellFactors *pre = nullptr) {
  const int D = a.D;
  const double nu = a.kappa ? a.kappa[c] : 0.3;
  if (pre) {  // the factors computed beforehand (one thread per cell): copied by the whole CTA
    static_assert(sizeof(CellFactors) % sizeof(double) == 0, "CellFactors holds doubles only");
    for (int e = t; e < (int)(sizeof(CellFactors) / sizeof(double)); e += nt)
      reinterpret_cast<double *>(&S.f)[e] = reinterpret_cast<const double *>(pre)[e];
  } else if (t == 0) {
    cell_factors(a, c, S.f);
  }
  __syncthreads();
  for (int e = t; e < 6 * 3 * 3 + 6 * 3 * 6 + 36; e += nt) {
    if (e < 54) {
      const int cc = e / 9, k = (e / 3) % 3, ee = e % 3;
      double v = 0.0;
      if (cc < a.nsym && k < D && ee < D)
        for (int jj = 0; jj < D; ++jj) v += sym_unit(D, cc, k, jj) * S.f.cg[ee][jj];
      S.T.dterm[cc][k][ee] = v;
    } else if (e < 54 + 108) {
      const int o = e - 54, cc = o / 18, k = (o / 6) % 3, lf = o % 6;
      double v = 0.0;
      if (cc < a.nsym && k < D && lf < 2 * D)
        for (int jj = 0; jj < D; ++jj) v += sym_unit(D, cc, k, jj) * S.f.cn[lf][jj];
      S.T.nterm[cc][k][lf] = v;
    } else {
      const int o = e - 162, cc = o / 6, d = o % 6;
      double v = 0.0;
      if (cc < a.nsym && d < a.nsym) {
        double dd = 0.0, trc = 0.0, trd = 0.0;
        for (int r = 0; r < D; ++r) {
          trc += sym_unit(D, cc, r, r);
          trd += sym_unit(D, d, r, r);
          for (int s2 = 0; s2 < D; ++s2) dd += sym_unit(D, cc, r, s2) * sym_unit(D, d, r, s2);
        }
        v = ((1.0 + nu) / a.young * dd - nu / a.young * trc * trd) * S.f.detJ;
      }
      S.T.cmj[cc][d] = v;
    }
  }
  if (ff) {
    __syncthreads();
    const double *src = &S.T.dterm[0][0][0];
    float *dst = &S.TF.dterm[0][0][0][0];
    for (int e = t; e < 54 + 108 + 36; e += nt) split_double(src[e], dst[2 * e], dst[2 * e + 1]);
    for (int e = t; e < 6; e += nt) split_double(S.f.ct[e], S.TF.ct[e][0], S.TF.ct[e][1]);
  }
  // -w.f per quadrature point (f = div sigma_exact, evaluated in FP64)
  for (int q = t; q < a.nqv; q += nt) {
    double x[3], u[3], gu[3][3], hu[3][3][3], fv[3];
    for (int d = 0; d < D; ++d) {
      x[d] = S.f.x0[d];
      for (int e = 0; e < D; ++e) x[d] += S.f.J[d][e] * a.qxi[q * D + e];
    }
    elasticity_exact(a.problem, D, x, u, gu, hu);
    elasticity_force(D, a.young, nu, hu, fv);
    const double w = a.qw[q] * S.f.detJ;
    for (int d = 0; d < D; ++d) fq[q * D + d] = -w * fv[d];
  }
  __syncthreads();
}

// b entry i of the cell: -int w.f on the displacement rows
__device__ __forceinline__ double elast_source_entry(const CellArgs &a, const double *fq, int i) {
  const ElastRow r = elast_decode(a, i);
  double v = 0.0;
  if (r.type == 1)
    for (int q = 0; q < a.nqv; ++q) v += fq[q * a.D + r.comp] * a.qphi[q * a.nk + r.node];
  return v;
}

}  // namespace hdg
