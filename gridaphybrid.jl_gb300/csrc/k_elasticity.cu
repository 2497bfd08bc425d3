// k_elasticity.cu -- linear elasticity HDG cell blocks for sm_103a
// (test/LinearElasticityHDGTests.jl:140-150 without the P_m projection,
// compliance :15-38).  DOFs per cell: [symmetric stress (nsym comps x nk) |
// displacement (D x nk) | displacement trace per local facet (D x nfs)],
// component-major.  Every entry is a short sum of reference tables (M, G, F,
// H, L) times the affine cell's factors, as for the Darcy form; the
// compliance couples the stress components through a per-cell 6x6 matrix.
// The condensation, assembly, skeleton solve and recovery are the
// field-agnostic kernels the Darcy path uses.
#include <cuda_runtime.h>

#include "hdg_kernels.h"
#include "k_ff_cell.cuh"
#include "k_fp64_cell.cuh"

namespace hdg {

namespace {

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

// -sum_jj E_c(k, jj) sum_e cg[e][jj] G[e][a][b]  (= sum_jj E_c(k, jj) d_jj phi_a, integrated with phi_b)
__device__ __forceinline__ double div_term(const CellArgs &a, const CellFactors &f, int c, int k, int na, int nb) {
  const int nk = a.nk, D = a.D;
  double v = 0.0;
  for (int jj = 0; jj < D; ++jj) {
    const double e = sym_unit(D, c, k, jj);
    if (e == 0.0) continue;
    for (int ee = 0; ee < D; ++ee) v -= e * f.cg[ee][jj] * a.G[(ee * nk + na) * nk + nb];
  }
  return v;
}

// sum_jj E_c(k, jj) n_jj |F| (the facet factor of (v.n).uhat and mu.(sigma.n))
__device__ __forceinline__ double normal_term(const CellArgs &a, const CellFactors &f, int c, int k, int lf) {
  double v = 0.0;
  for (int jj = 0; jj < a.D; ++jj) v += sym_unit(a.D, c, k, jj) * f.cn[lf][jj];
  return v;
}

__device__ double elast_entry(const CellArgs &a, const CellFactors &f, const double (*Cm)[6], double detJ, int i,
                              int j) {
  const ElastRow r = elast_decode(a, i), s = elast_decode(a, j);
  const int nk = a.nk, nfs = a.nfs, nl = 2 * a.D;
  if (r.type == 0) {
    if (s.type == 0) return Cm[r.comp][s.comp] * detJ * a.M[r.node * nk + s.node];
    if (s.type == 1) return div_term(a, f, r.comp, s.comp, r.node, s.node);  // (div v).u
    return -normal_term(a, f, r.comp, s.comp, s.lf) * a.H[(s.lf * nk + r.node) * nfs + s.node];  // -(v.n).uhat
  }
  if (r.type == 1) {
    if (s.type == 0) return -div_term(a, f, s.comp, r.comp, s.node, r.node);  // -w.(div sigma)
    if (s.type == 1) {
      if (r.comp != s.comp) return 0.0;
      double v = 0.0;  // tau w.u
      for (int lf = 0; lf < nl; ++lf) v += f.ct[lf] * a.F[(lf * nk + r.node) * nk + s.node];
      return v;
    }
    return r.comp == s.comp ? -f.ct[s.lf] * a.H[(s.lf * nk + r.node) * nfs + s.node] : 0.0;  // -tau w.uhat
  }
  if (s.type == 0)  // mu.(sigma.n)
    return normal_term(a, f, s.comp, r.comp, r.lf) * a.H[(r.lf * nk + s.node) * nfs + r.node];
  if (s.type == 1)  // -tau mu.u
    return r.comp == s.comp ? -f.ct[r.lf] * a.H[(r.lf * nk + s.node) * nfs + r.node] : 0.0;
  // tau mu.uhat
  return (r.lf == s.lf && r.comp == s.comp) ? f.ct[r.lf] * a.L[r.node * nfs + s.node] : 0.0;
}

// E_c (.) A(E_d) = (1+nu)/E (E_c (.) E_d) - nu/E tr(E_c) tr(E_d)
__device__ void compliance(int D, int nsym, double E, double nu, double (*Cm)[6]) {
  for (int c = 0; c < nsym; ++c)
    for (int d = 0; d < nsym; ++d) {
      double dd = 0.0, trc = 0.0, trd = 0.0;
      for (int r = 0; r < D; ++r) {
        trc += sym_unit(D, c, r, r);
        trd += sym_unit(D, d, r, r);
        for (int s = 0; s < D; ++s) dd += sym_unit(D, c, r, s) * sym_unit(D, d, r, s);
      }
      Cm[c][d] = (1.0 + nu) / E * dd - nu / E * trc * trd;
    }
}

__global__ void __launch_bounds__(256) integrate_elasticity_kernel(CellArgs a, double *A, double *b, float *Ahi,
                                                                   float *Alo, float *bhi, float *blo, bool skip_ss) {
  __shared__ CellFactors f;
  __shared__ double Cm[6][6];
  __shared__ double fq[512 * 3];
  const int n = a.n, D = a.D;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    const double nu = a.kappa ? a.kappa[c] : 0.3;
    if (threadIdx.x == 0) {
      cell_factors(a, c, f);
      compliance(D, a.nsym, a.young, nu, Cm);
    }
    __syncthreads();
    // -w.f per quadrature point (f = div sigma_exact, evaluated in FP64)
    for (int q = threadIdx.x; q < a.nqv; q += blockDim.x) {
      double x[3], u[3], gu[3][3], hu[3][3][3], fv[3];
      for (int d = 0; d < D; ++d) {
        x[d] = f.x0[d];
        for (int e = 0; e < D; ++e) x[d] += f.J[d][e] * a.qxi[q * D + e];
      }
      elasticity_exact(a.problem, D, x, u, gu, hu);
      elasticity_force(D, a.young, nu, hu, fv);
      const double w = a.qw[q] * f.detJ;
      for (int d = 0; d < D; ++d) fq[q * D + d] = -w * fv[d];
    }
    __syncthreads();
    const size_t base = (size_t)c * n * n;
    const int ns = a.nsym * a.nk;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int j = e / n, i = e - j * n;
      if (skip_ss && i < ns && j < ns) continue;
      const double v = elast_entry(a, f, Cm, f.detJ, i, j);
      if (A) {
        A[base + e] = v;
      } else {
        float h, l;
        split_double(v, h, l);
        Ahi[base + e] = h;
        Alo[base + e] = l;
      }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const ElastRow r = elast_decode(a, i);
      double v = 0.0;
      if (r.type == 1)
        for (int q = 0; q < a.nqv; ++q) v += fq[q * D + r.comp] * a.qphi[q * a.nk + r.node];
      if (b) {
        b[(size_t)c * n + i] = v;
      } else {
        float h, l;
        split_double(v, h, l);
        bhi[(size_t)c * n + i] = h;
        blo[(size_t)c * n + i] = l;
      }
    }
    __syncthreads();
  }
}

// stress and displacement L2 error contributions of each cell
__global__ void __launch_bounds__(128) l2_errors_elasticity_kernel(CellArgs a, const double *__restrict__ uint,
                                                                   double *errs) {
  __shared__ CellFactors f;
  __shared__ double red[2][4];
  const int D = a.D, nk = a.nk, ns = a.nsym, ou = ns * nk;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    if (threadIdx.x == 0) cell_factors(a, c, f);
    __syncthreads();
    const double nu = a.kappa ? a.kappa[c] : 0.3;
    const double *v = uint + (size_t)c * a.ni;
    double es = 0.0, eu = 0.0;
    for (int q = threadIdx.x; q < a.nqv; q += blockDim.x) {
      double x[3], u[3], gu[3][3], hu[3][3][3];
      for (int d = 0; d < D; ++d) {
        x[d] = f.x0[d];
        for (int e = 0; e < D; ++e) x[d] += f.J[d][e] * a.qxi[q * D + e];
      }
      elasticity_exact(a.problem, D, x, u, gu, hu);
      double mu, lam, tr = 0.0;
      elasticity_lame(D, a.young, nu, mu, lam);
      for (int d = 0; d < D; ++d) tr += gu[d][d];
      double sh[6] = {0, 0, 0, 0, 0, 0}, uh[3] = {0, 0, 0};
      for (int na = 0; na < nk; ++na) {
        const double ph = a.qphi[q * nk + na];
        for (int cc = 0; cc < ns; ++cc) sh[cc] += v[cc * nk + na] * ph;
        for (int k = 0; k < D; ++k) uh[k] += v[ou + k * nk + na] * ph;
      }
      double e2 = 0.0, u2 = 0.0;
      for (int cc = 0; cc < ns; ++cc) {
        int i, j;
        sym_pair(D, cc, i, j);
        const double sig = mu * (gu[i][j] + gu[j][i]) + (i == j ? lam * tr : 0.0);
        const double d = sig - sh[cc];
        e2 += (i == j ? 1.0 : 2.0) * d * d;
      }
      for (int k = 0; k < D; ++k) u2 += (u[k] - uh[k]) * (u[k] - uh[k]);
      const double w = a.qw[q] * f.detJ;
      es += w * e2;
      eu += w * u2;
    }
    for (int off = 16; off > 0; off >>= 1) {
      es += __shfl_down_sync(0xffffffffu, es, off);
      eu += __shfl_down_sync(0xffffffffu, eu, off);
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = es;
      red[1][threadIdx.x >> 5] = eu;
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

cudaError_t launch_integrate_elasticity(const CellArgs &a, double *A, double *b, float *Ahi, float *Alo, float *bhi,
                                        float *blo, cudaStream_t s, int num_sms, long long *launches, bool skip_ss) {
  if (a.nqv > 512 || a.nsym > 6) return cudaErrorInvalidValue;
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  if (grid < 1) grid = 1;
  integrate_elasticity_kernel<<<grid, 256, 0, s>>>(a, A, b, Ahi, Alo, bhi, blo, skip_ss);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_l2_errors_elasticity(const CellArgs &a, const double *uint, double *errs, cudaStream_t s,
                                        int num_sms, long long *launches) {
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  if (grid < 1) grid = 1;
  l2_errors_elasticity_kernel<<<grid, 128, 0, s>>>(a, uint, errs);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace hdg
