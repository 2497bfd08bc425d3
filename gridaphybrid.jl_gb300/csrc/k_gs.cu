// k_gs.cu -- FP64 integration and L2 errors of the general-space cell forms
// (sm_103a): fields with their own polynomial spaces and orders, as the
// reference's tests choose them -- the Darcy HDG form with flux P_k,
// pressure P_{k-1}, multiplier P_k (test/DarcyHDGTests.jl:34-36,125-135); the
// hybridized Raviart-Thomas form (flux RT_k, no stabilisation,
// test/DarcyRTHTests.jl:24-68); the elasticity HDG form with stress P_k,
// displacement P_{k+1}, trace P_k and the P_m projection in the tau terms
// (test/LinearElasticityHDGTests.jl:88-150, src/GridapAPIExtensions.jl:453-500);
// and several decoupled copies of a form, each with its own skeleton field
// (test/MultiFieldLagrangeMultipliersTests.jl).
//
// On an affine cell every entry is a short sum of reference tables (contracted
// once on the host) times the cell's factors: one CTA per cell, threads over
// the n^2 entries.  Box cells (2D facets) and, for the Darcy form with P_k
// fields, simplex cells (D + 1 facets: simplexify of the Cartesian model,
// test/DarcyHDGTests.jl:174-177) share the kernels; only the reference tables
// and the facet factors differ.  The cell blocks then go through the same condensation,
// assembly, skeleton solve and recovery as every other form.
#include <cuda_runtime.h>

#include "../../include/hdg_gb300.h"
#include "hdg_kernels.h"
#include "k_elast_cell.cuh"
#include "k_fp64_cell.cuh"

namespace hdg {

namespace {

struct GsDof {
  int t, copy, comp, idx, lf;  // t: 0 field A, 1 field B, 2 trace (local facet lf)
};

__device__ __forceinline__ GsDof gs_decode(const GsArgs &g, int i) {
  GsDof r;
  r.lf = 0;
  const int wA = g.ncA * g.nA, wB = g.ncB * g.nB;
  if (i < g.copies * wA) {
    r.t = 0;
    r.copy = i / wA;
    const int j = i - r.copy * wA;
    r.comp = j / g.nA;
    r.idx = j - r.comp * g.nA;
  } else if (i < g.ni) {
    const int j0 = i - g.copies * wA;
    r.t = 1;
    r.copy = j0 / wB;
    const int j = j0 - r.copy * wB;
    r.comp = j / g.nB;
    r.idx = j - r.comp * g.nB;
  } else {
    const int j = i - g.ni;
    r.lf = j / g.nfd;
    const int m0 = j - r.lf * g.nfd;
    r.t = 2;
    r.copy = m0 / g.nfd1;
    const int m = m0 - r.copy * g.nfd1;
    r.comp = m / g.nT;
    r.idx = m - r.comp * g.nT;
  }
  return r;
}

// Darcy entry (row test function r, column trial function s): volume
// v.u/kappa - (div v) p - grad(q).u, facets (v.n) l + q (u.n) + tau s q p -
// tau s q l + m (u.n) + tau s m p - tau s m l (s = n.n_o or 1).  With tau = 0
// and the flux in RT_k it is the hybridized Raviart-Thomas form of
// test/DarcyRTHTests.jl:60-62 (-grad(q).u + q (u.n) = q div u on each cell).
__device__ __forceinline__ double gs_darcy_entry(const GsArgs &g, const CellFactors &f, const GsDof &r,
                                                 const GsDof &s) {
  const int D = g.cell.D, nA = g.nA, nB = g.nB, nT = g.nT, nl = g.nl;
  double v = 0.0;
  if (r.t == 0) {
    const int c = r.comp;
    if (s.t == 0) {
      if (c == s.comp) v = f.cm * g.MAA[(c * nA + r.idx) * nA + s.idx];
    } else if (s.t == 1) {
      for (int e = 0; e < D; ++e) v += f.cg[e][c] * g.GAB[((c * D + e) * nA + r.idx) * nB + s.idx];
    } else {
      v = f.cn[s.lf][c] * g.HA[((c * nl + s.lf) * nA + r.idx) * nT + s.idx];
    }
  } else if (r.t == 1) {
    if (s.t == 0) {
      const int c = s.comp;
      for (int e = 0; e < D; ++e) v += f.cg[e][c] * g.GBA[((c * D + e) * nB + r.idx) * nA + s.idx];
      for (int lf = 0; lf < nl; ++lf) v += f.cn[lf][c] * g.FBA[((c * nl + lf) * nB + r.idx) * nA + s.idx];
    } else if (s.t == 1) {
      for (int lf = 0; lf < nl; ++lf) v += f.ct[lf] * g.FBB[(lf * nB + r.idx) * nB + s.idx];
    } else {
      v = -f.ct[s.lf] * g.HB[(s.lf * nB + r.idx) * nT + s.idx];
    }
  } else {
    if (s.t == 0) {
      const int c = s.comp;
      v = f.cn[r.lf][c] * g.HA[((c * nl + r.lf) * nA + s.idx) * nT + r.idx];
    } else if (s.t == 1) {
      v = f.ct[r.lf] * g.HB[(r.lf * nB + s.idx) * nT + r.idx];
    } else if (r.lf == s.lf) {
      v = -f.ct[r.lf] * g.L[r.idx * nT + s.idx];
    }
  }
  return v;
}

// Elasticity HDG entry: v (.) A(sigma) + (div v).u - w.(div sigma) on the
// cell; -(v.n).uhat + tau w.P(u) - tau w.uhat + mu.(sigma.n) - tau mu.P(u) +
// tau mu.uhat on its facets (P = P_m or the identity; FBB holds the tau w.P(u)
// table, and tau mu.P_m(u) = tau mu.u).  The stress components share one basis.
__device__ __forceinline__ double gs_elast_entry(const GsArgs &g, const CellFactors &f, const ElastCellTerms &T,
                                                 const GsDof &r, const GsDof &s) {
  const int D = g.cell.D, nA = g.nA, nB = g.nB, nT = g.nT, nl = g.nl;
  if (r.t == 0) {
    if (s.t == 0) return T.cmj[r.comp][s.comp] * g.MAA[r.idx * nA + s.idx];
    if (s.t == 1) {
      double v = 0.0;
      for (int e = 0; e < D; ++e) v -= T.dterm[r.comp][s.comp][e] * g.GAB[(e * nA + r.idx) * nB + s.idx];
      return v;
    }
    return -T.nterm[r.comp][s.comp][s.lf] * g.HA[(s.lf * nA + r.idx) * nT + s.idx];
  }
  if (r.t == 1) {
    if (s.t == 0) {
      double v = 0.0;
      for (int e = 0; e < D; ++e) v += T.dterm[s.comp][r.comp][e] * g.GAB[(e * nA + s.idx) * nB + r.idx];
      return v;
    }
    if (r.comp != s.comp) return 0.0;
    if (s.t == 1) {
      double v = 0.0;
      for (int lf = 0; lf < nl; ++lf) v += f.ct[lf] * g.FBB[(lf * nB + r.idx) * nB + s.idx];
      return v;
    }
    return -f.ct[s.lf] * g.HB[(s.lf * nB + r.idx) * nT + s.idx];
  }
  if (s.t == 0) return T.nterm[s.comp][r.comp][r.lf] * g.HA[(r.lf * nA + s.idx) * nT + r.idx];
  if (r.comp != s.comp) return 0.0;
  if (s.t == 1) return -f.ct[r.lf] * g.HB[(r.lf * nB + s.idx) * nT + r.idx];
  return r.lf == s.lf ? f.ct[r.lf] * g.L[r.idx * nT + s.idx] : 0.0;
}

constexpr int kGsMaxQv = 216;  // 6^3 volume points

__global__ void __launch_bounds__(256) integrate_gs_kernel(GsArgs g, double *A, double *b) {
  __shared__ ElastScratch S;
  __shared__ double fq[kGsMaxQv * 4];
  const CellArgs &a = g.cell;
  const int n = g.n, D = a.D;
  const bool elast = g.phys == HDG_PHYSICS_ELASTICITY;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    if (elast) {
      elast_cell_prepare(a, c, S, fq, false, threadIdx.x, blockDim.x);  // fq: -w f per point (nqv x D)
    } else {
      if (threadIdx.x == 0) {
        if (g.simplex)
          cell_factors_simplex(a, c, S.f);
        else
          cell_factors(a, c, S.f);
      }
      __syncthreads();
      source_values(a, S.f, c, fq, threadIdx.x, blockDim.x);  // fq: w (f_u, g) per point (nqv x (D+1))
      __syncthreads();
    }
    double *Ac = A + (size_t)c * n * n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int j = e / n, i = e - j * n;
      const GsDof r = gs_decode(g, i), s = gs_decode(g, j);
      double v = 0.0;
      if (r.copy == s.copy) v = elast ? gs_elast_entry(g, S.f, S.T, r, s) : gs_darcy_entry(g, S.f, r, s);
      Ac[e] = v;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const GsDof r = gs_decode(g, i);
      double v = 0.0;
      if (elast) {
        if (r.t == 1)
          for (int q = 0; q < g.nqv; ++q) v += fq[q * D + r.comp] * g.qphiB[q * g.nB + r.idx];
      } else if (r.t == 0) {
        const double *pA = g.qphiA + (size_t)r.comp * g.nqv * g.nA;
        for (int q = 0; q < g.nqv; ++q) v += fq[q * (D + 1) + r.comp] * pA[q * g.nA + r.idx];
      } else if (r.t == 1) {
        for (int q = 0; q < g.nqv; ++q) v += fq[q * (D + 1) + D] * g.qphiB[q * g.nB + r.idx];
      }
      b[(size_t)c * n + i] = v;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(128) l2_errors_gs_kernel(GsArgs g, const double *__restrict__ uint,
                                                           double *errs) {
  __shared__ CellFactors f;
  __shared__ double red[2][4];
  const CellArgs &a = g.cell;
  const int D = a.D, nA = g.nA, nB = g.nB, wA = g.ncA * nA, wB = g.ncB * nB;
  const bool elast = g.phys == HDG_PHYSICS_ELASTICITY;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    if (threadIdx.x == 0) {
      if (g.simplex)
        cell_factors_simplex(a, c, f);
      else
        cell_factors(a, c, f);
    }
    __syncthreads();
    const double coef = a.kappa ? a.kappa[c] : (elast ? 0.3 : 1.0);
    double e1 = 0.0, e2 = 0.0;
    for (int q = threadIdx.x; q < g.nqv; q += blockDim.x) {
      double x[3];
      for (int d = 0; d < D; ++d) {
        x[d] = f.x0[d];
        for (int e = 0; e < D; ++e) x[d] += f.J[d][e] * a.qxi[q * D + e];
      }
      const double *pB = g.qphiB + (size_t)q * nB;
      const double w = a.qw[q] * f.detJ;
      for (int cp = 0; cp < g.copies; ++cp) {
        const double *vA = uint + (size_t)c * g.ni + cp * wA;
        const double *vB = uint + (size_t)c * g.ni + g.copies * wA + cp * wB;
        if (elast) {
          const double *pA = g.qphiA + (size_t)q * nA;
          double u[3], gu[3][3], hu[3][3][3], mu, lam, tr = 0.0;
          elasticity_exact(a.problem, D, x, u, gu, hu);
          elasticity_lame(D, a.young, coef, mu, lam);
          for (int d = 0; d < D; ++d) tr += gu[d][d];
          double s1 = 0.0, s2 = 0.0;
          for (int cc = 0; cc < a.nsym; ++cc) {
            int i, j;
            sym_pair(D, cc, i, j);
            double sh = 0.0;
            for (int na = 0; na < nA; ++na) sh += vA[cc * nA + na] * pA[na];
            const double d = mu * (gu[i][j] + gu[j][i]) + (i == j ? lam * tr : 0.0) - sh;
            s1 += (i == j ? 1.0 : 2.0) * d * d;
          }
          for (int k = 0; k < D; ++k) {
            double uh = 0.0;
            for (int nb = 0; nb < nB; ++nb) uh += vB[k * nB + nb] * pB[nb];
            s2 += (u[k] - uh) * (u[k] - uh);
          }
          e1 += w * s1;
          e2 += w * s2;
        } else {
          double p, qe[3], fu[3], gg;
          exact_solution(a.problem, D, x, coef, p, qe, fu, gg);
          double s1 = 0.0, ph = 0.0;
          for (int d = 0; d < D; ++d) {
            const double *pA = g.qphiA + ((size_t)d * g.nqv + q) * nA;
            double qh = 0.0;
            for (int na = 0; na < nA; ++na) qh += vA[d * nA + na] * pA[na];
            s1 += (qe[d] - qh) * (qe[d] - qh);
          }
          for (int nb = 0; nb < nB; ++nb) ph += vB[nb] * pB[nb];
          e1 += w * s1;
          e2 += w * (p - ph) * (p - ph);
        }
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      e1 += __shfl_down_sync(0xffffffffu, e1, off);
      e2 += __shfl_down_sync(0xffffffffu, e2, off);
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = e1;
      red[1][threadIdx.x >> 5] = e2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      errs[2 * (size_t)c] = red[0][0] + red[0][1] + red[0][2] + red[0][3];
      errs[2 * (size_t)c + 1] = red[1][0] + red[1][1] + red[1][2] + red[1][3];
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_integrate_gs(const GsArgs &g, double *A, double *b, cudaStream_t s, int num_sms,
                                long long *launches) {
  if (g.nqv > kGsMaxQv || g.cell.nsym > 6 || g.cell.D > 3) return cudaErrorInvalidValue;
  int grid = g.cell.ncells < num_sms * 8 ? g.cell.ncells : num_sms * 8;
  if (grid < 1) grid = 1;
  integrate_gs_kernel<<<grid, 256, 0, s>>>(g, A, b);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_l2_errors_gs(const GsArgs &g, const double *uint, double *errs, cudaStream_t s, int num_sms,
                                long long *launches) {
  int grid = g.cell.ncells < num_sms * 8 ? g.cell.ncells : num_sms * 8;
  if (grid < 1) grid = 1;
  l2_errors_gs_kernel<<<grid, 128, 0, s>>>(g, uint, errs);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace hdg
