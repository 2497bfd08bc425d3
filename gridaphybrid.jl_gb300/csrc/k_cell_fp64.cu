// k_cell_fp64.cu -- FP64 cell kernels for sm_103a: integration of the Darcy
// HDG cell blocks, static condensation (StaticCondensationMap), backward
// condensation (BackwardStaticCondensationMap), recovery from stored factors,
// SumFacetsMap and per-cell L2 errors.
//
// GB300 executes FP64 at ~1/74 of its FP32 rate (1.05 vs 78 TFLOP/s measured),
// so this path is DFMA-bound: a CTA per cell, the cell block resident in
// shared memory, no effort spent on memory-side tiling.
#include <cuda_runtime.h>

#include "hdg_kernels.h"
#include "k_fp64_cell.cuh"

namespace hdg {

__global__ void __launch_bounds__(256) integrate_fp64_kernel(CellArgs a, double *A, double *b) {
  __shared__ CellFactors f;
  __shared__ double fq[512 * 4];
  const int n = a.n;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    if (threadIdx.x == 0) cell_factors(a, c, f);
    __syncthreads();
    source_values(a, f, c, fq, threadIdx.x, blockDim.x);
    __syncthreads();
    double *Ac = A + (size_t)c * n * n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int j = e / n, i = e - j * n;
      int ti, si, ii, tj, sj, jj;
      decode(i, a.D, a.nk, a.ni, a.nfd, ti, si, ii);
      decode(j, a.D, a.nk, a.ni, a.nfd, tj, sj, jj);
      Ac[e] = cell_entry<double>(a, f, ti, si, ii, tj, sj, jj);
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      int ti, si, ii;
      decode(i, a.D, a.nk, a.ni, a.nfd, ti, si, ii);
      double v = 0.0;
      if (ti < 2) {
        const int comp = ti == 0 ? si : a.D;
        for (int q = 0; q < a.nqv; ++q) v += fq[q * (a.D + 1) + comp] * a.qphi[q * a.nk + ii];
      }
      b[(size_t)c * n + i] = v;
    }
    __syncthreads();
  }
}

cudaError_t launch_integrate_fp64(const CellArgs &a, double *A, double *b,
                                  cudaStream_t s, int num_sms, long long *launches) {
  if (a.nqv > 512) return cudaErrorInvalidValue;
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  integrate_fp64_kernel<<<grid, 256, 0, s>>>(a, A, b);
  ++*launches;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Static condensation, FP64.  The augmented block W = [A | b] (n x (n+1),
// column-major) sits in shared memory; the first ni columns are eliminated
// with partial pivoting restricted to the interior rows (the pivots getrf
// picks on A_ii), every row of W updated.  The trailing block is then
// S = A_ff - A_fi A_ii^{-1} A_if and the trailing column g
// (src/StaticCondensationMap.jl:179-192 computed as one partial elimination).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) condense_fp64_kernel(int ncells, int ni, int nf,
                                                            const double *__restrict__ A,
                                                            const double *__restrict__ b,
                                                            double *S, double *g,
                                                            double *fact, int *info) {
  extern __shared__ double W[];
  __shared__ int s_piv;
  const int n = ni + nf;
  for (int c = blockIdx.x; c < ncells; c += gridDim.x) {
    const double *Ac = A + (size_t)c * n * n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) W[e] = Ac[e];
    for (int i = threadIdx.x; i < n; i += blockDim.x) W[(size_t)n * n + i] = b[(size_t)c * n + i];
    __syncthreads();
    int inf = eliminate_fp64(W, n, n + 1, ni, ni, &s_piv, threadIdx.x, blockDim.x);
    double *Sc = S + (size_t)c * nf * nf;
    for (int e = threadIdx.x; e < nf * nf; e += blockDim.x) {
      const int jj = e / nf, ii = e - jj * nf;
      Sc[e] = W[(ni + ii) + (size_t)n * (ni + jj)];
    }
    for (int i = threadIdx.x; i < nf; i += blockDim.x) g[(size_t)c * nf + i] = W[(ni + i) + (size_t)n * n];
    if (fact) {
      double *Fc = fact + (size_t)c * ni * (n + 1);
      for (int e = threadIdx.x; e < ni * (n + 1); e += blockDim.x) {
        const int jj = e / ni, ii = e - jj * ni;
        Fc[e] = W[ii + (size_t)n * jj];
      }
    }
    if (info && threadIdx.x == 0) info[c] = inf;
    __syncthreads();
  }
}

cudaError_t launch_condense_fp64(int ncells, int ni, int nf, const double *A,
                                 const double *b, double *S, double *g,
                                 double *fact, int *info, cudaStream_t s,
                                 int num_sms, long long *launches) {
  const int n = ni + nf;
  const size_t smem = sizeof(double) * (size_t)n * (n + 1);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(condense_fp64_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int threads = n > 64 ? 256 : 128;
  const int per_sm = (int)((228 * 1024) / (smem + 1024));
  int grid = num_sms * (per_sm > 0 ? per_sm : 1);
  if (grid > ncells) grid = ncells;
  if (grid < 1) grid = 1;
  condense_fp64_kernel<<<grid, threads, smem, s>>>(ncells, ni, nf, A, b, S, g, fact, info);
  ++*launches;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Map-level backward condensation: u = A_ii^{-1}(b_i - A_if x), with A_ii
// refactorised (src/BackwardStaticCondensationMap.jl:88-99).
// ---------------------------------------------------------------------------
__device__ void back_substitute(const double *W, int n, int ld, double *rhs, double *out) {
  // W: upper triangle of n x n (ld), rhs in shared memory (overwritten)
  for (int j = n - 1; j >= 0; --j) {
    __syncthreads();
    const double uj = rhs[j] / W[j + (size_t)ld * j];
    __syncthreads();
    if (threadIdx.x == 0) rhs[j] = uj;
    for (int i = threadIdx.x; i < j; i += blockDim.x) rhs[i] -= W[i + (size_t)ld * j] * uj;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = rhs[i];
  __syncthreads();
}

__global__ void __launch_bounds__(256) backward_fp64_kernel(int ncells, int ni, int nf,
                                                            const double *__restrict__ A,
                                                            const double *__restrict__ b,
                                                            const double *__restrict__ x,
                                                            double *u, int *info) {
  extern __shared__ double W[];  // ni x (ni+1)
  __shared__ int s_piv;
  const int n = ni + nf;
  double *rhs = W + (size_t)ni * ni;
  for (int c = blockIdx.x; c < ncells; c += gridDim.x) {
    const double *Ac = A + (size_t)c * n * n;
    for (int e = threadIdx.x; e < ni * ni; e += blockDim.x) {
      const int jj = e / ni, ii = e - jj * ni;
      W[e] = Ac[ii + (size_t)n * jj];
    }
    for (int i = threadIdx.x; i < ni; i += blockDim.x) {
      double v = b[(size_t)c * n + i];
      for (int j = 0; j < nf; ++j) v -= Ac[i + (size_t)n * (ni + j)] * x[(size_t)c * nf + j];
      rhs[i] = v;
    }
    __syncthreads();
    int inf = eliminate_fp64(W, ni, ni + 1, ni, ni, &s_piv, threadIdx.x, blockDim.x);
    back_substitute(W, ni, ni, rhs, u + (size_t)c * ni);
    if (info && threadIdx.x == 0) info[c] = inf;
    __syncthreads();
  }
}

cudaError_t launch_backward_fp64(int ncells, int ni, int nf, const double *A,
                                 const double *b, const double *x, double *u,
                                 int *info, cudaStream_t s, int num_sms,
                                 long long *launches) {
  const size_t smem = sizeof(double) * (size_t)ni * (ni + 1);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(backward_fp64_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int grid = ncells < num_sms * 4 ? ncells : num_sms * 4;
  if (grid < 1) grid = 1;
  backward_fp64_kernel<<<grid, 128, smem, s>>>(ncells, ni, nf, A, b, x, u, info);
  ++*launches;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Recovery from the stored factors [U11 | U12 | y] (rows already permuted):
// u = U11^{-1} (y - U12 x_f), x_f gathered from the skeleton solution and
// the Dirichlet values (src/HybridAffineFEOperators.jl:110-118).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) recover_fp64_kernel(CellArgs a, const double *__restrict__ fact,
                                                           const double *__restrict__ lambda,
                                                           const double *__restrict__ dirvals,
                                                           double *uint) {
  __shared__ double xf[6 * 64];
  __shared__ double rhs[4 * 512];
  const int ni = a.ni, nf = a.nf, n = a.n, nfd = a.nfd, nl = a.nf / a.nfd;  // facets per cell (box or simplex)
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    for (int e = threadIdx.x; e < nf; e += blockDim.x) {
      const int lf = e / nfd, j = e - lf * nfd;
      const int id = a.facet_dofs[(size_t)a.cell_facets[(size_t)c * nl + lf] * nfd + j];
      xf[e] = id >= 0 ? lambda[id] : dirvals[-1 - id];
    }
    __syncthreads();
    const double *Fc = fact + (size_t)c * ni * (n + 1);
    for (int i = threadIdx.x; i < ni; i += blockDim.x) {
      double v = Fc[i + (size_t)ni * n];
      for (int j = 0; j < nf; ++j) v -= Fc[i + (size_t)ni * (ni + j)] * xf[j];
      rhs[i] = v;
    }
    back_substitute(Fc, ni, ni, rhs, uint + (size_t)c * ni);
  }
}

cudaError_t launch_recover_fp64(const CellArgs &a, const double *fact,
                                const double *lambda, const double *dirvals,
                                double *uint, cudaStream_t s, int num_sms,
                                long long *launches) {
  if (a.nf > 6 * 64 || a.ni > 4 * 512) return cudaErrorInvalidValue;
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  recover_fp64_kernel<<<grid, 128, 0, s>>>(a, fact, lambda, dirvals, uint);
  ++*launches;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// SumFacetsMap (src/SumFacetsMap.jl:19-30): out = a_1 + a_2 + ... + a_nfacets
// folded left to right as the reference's chain of BroadcastingFieldOpMap(+).
// ---------------------------------------------------------------------------
__global__ void sum_facets_kernel(int nitems, int nfacets, int len, const double *blocks,
                                  double *out) {
  const size_t total = (size_t)nitems * len;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t it = e / len, i = e - it * len;
    const double *bp = blocks + it * nfacets * len + i;
    double v = bp[0] + bp[len];
    for (int f = 2; f < nfacets; ++f) v += bp[(size_t)f * len];
    out[e] = v;
  }
}

cudaError_t launch_sum_facets(int nitems, int nfacets, int len, const double *blocks,
                              double *out, cudaStream_t s, long long *launches) {
  size_t total = (size_t)nitems * len;
  int grid = (int)((total + 255) / 256);
  if (grid > 65535) grid = 65535;
  if (grid < 1) grid = 1;
  sum_facets_kernel<<<grid, 256, 0, s>>>(nitems, nfacets, len, blocks, out);
  ++*launches;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-cell squared L2 errors of flux and pressure against the exact solution
// (test/DarcyHDGTests.jl:141-142), quadrature of degree 2(k+1).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) l2_errors_kernel(CellArgs a, const double *__restrict__ uint,
                                                        double *errs) {
  __shared__ CellFactors f;
  __shared__ double red[2][4];
  const int D = a.D, nk = a.nk;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    if (threadIdx.x == 0) cell_factors(a, c, f);
    __syncthreads();
    const double *u = uint + (size_t)c * a.ni;
    const double kap = a.kappa ? a.kappa[c] : 1.0;
    double ef = 0.0, ep = 0.0;
    for (int q = threadIdx.x; q < a.nqv; q += blockDim.x) {
      double x[3], p, qe[3], fu[3], g;
      for (int d = 0; d < D; ++d) {
        x[d] = f.x0[d];
        for (int e = 0; e < D; ++e) x[d] += f.J[d][e] * a.qxi[q * D + e];
      }
      exact_solution(a.problem, D, x, kap, p, qe, fu, g);
      double qh[3] = {0, 0, 0}, ph = 0.0;
      for (int b = 0; b < nk; ++b) {
        const double v = a.qphi[q * nk + b];
        for (int d = 0; d < D; ++d) qh[d] += u[d * nk + b] * v;
        ph += u[D * nk + b] * v;
      }
      const double w = a.qw[q] * f.detJ;
      double e2 = 0.0;
      for (int d = 0; d < D; ++d) e2 += (qe[d] - qh[d]) * (qe[d] - qh[d]);
      ef += w * e2;
      ep += w * (p - ph) * (p - ph);
    }
    for (int off = 16; off > 0; off >>= 1) {
      ef += __shfl_down_sync(0xffffffffu, ef, off);
      ep += __shfl_down_sync(0xffffffffu, ep, off);
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = ef;
      red[1][threadIdx.x >> 5] = ep;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double s0 = 0.0, s1 = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        s0 += red[0][w];
        s1 += red[1][w];
      }
      errs[2 * (size_t)c] = s0;
      errs[2 * (size_t)c + 1] = s1;
    }
    __syncthreads();
  }
}

cudaError_t launch_l2_errors(const CellArgs &a, const double *uint, double *errs,
                             cudaStream_t s, int num_sms, long long *launches) {
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  l2_errors_kernel<<<grid, 128, 0, s>>>(a, uint, errs);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace hdg
