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
#include "k_elast_cell.cuh"

namespace hdg {

namespace {

__global__ void __launch_bounds__(256) integrate_elasticity_kernel(CellArgs a, double *A, double *b, float *Ahi,
                                                                   float *Alo, float *bhi, float *blo, bool skip_ss,
                                                                   MixedTables Tb, bool ff) {
  __shared__ ElastScratch S;
  __shared__ double fq[512 * 3];
  __shared__ int dec[512];
  const int n = a.n, ns = a.nsym * a.nk;
  for (int i = threadIdx.x; i < n; i += blockDim.x) dec[i] = elast_pack(a, i);
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    elast_cell_prepare(a, c, S, fq, ff, threadIdx.x, blockDim.x);
    const size_t base = (size_t)c * n * n;
    // entries e = i + n j, threads over consecutive e (i, j stepped without division)
    int i = threadIdx.x % n, j = threadIdx.x / n;
    const int di = blockDim.x % n, dj = blockDim.x / n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      if (!(skip_ss && i < ns && j < ns)) {
        if (ff) {
          float h, l;
          elast_entry_ff(a, Tb, S.TF, dec[i], dec[j], h, l);
          Ahi[base + e] = h;
          Alo[base + e] = l;
        } else {
          const double v = elast_entry_t(a, S.f, S.T, dec[i], dec[j]);
          if (A) {
            A[base + e] = v;
          } else {
            float h, l;
            split_double(v, h, l);
            Ahi[base + e] = h;
            Alo[base + e] = l;
          }
        }
      }
      i += di;
      j += dj;
      if (i >= n) {
        i -= n;
        ++j;
      }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double v = elast_source_entry(a, fq, i);
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
                                        float *blo, cudaStream_t s, int num_sms, long long *launches, bool skip_ss,
                                        const MixedTables *Tb) {
  if (a.nqv > 512 || a.nsym > 6) return cudaErrorInvalidValue;
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  if (grid < 1) grid = 1;
  const bool ff = Tb != nullptr && A == nullptr;
  integrate_elasticity_kernel<<<grid, 256, 0, s>>>(a, A, b, Ahi, Alo, bhi, blo, skip_ss, ff ? *Tb : MixedTables{},
                                                   ff);
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
