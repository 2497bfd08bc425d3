// k_newton.cu -- the residual side of the Newton path (HybridFEOperator +
// NLSolver(method=:newton), src/HybridFEOperators.jl:68-239 and
// src/HybridLinearSolvers.jl:15-59) for sm_103a: per-cell residuals
// r_c = A_c x_c - b_c of the current iterate, the max norm of the assembled
// residual, and the update x <- x - dx.
#include <cuda_runtime.h>

#include "hdg_kernels.h"

namespace hdg {

// max of non-negative doubles through their bit patterns (order-independent)
__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
  atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double block_max(double v, double *red) {
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double m = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = fmax(m, red[i]);
  return m;  // valid in thread 0
}

// b_c <- A_c x_c - b_c with x_c = [interior values of the iterate | facet
// values: free ones from the iterate, Dirichlet ones from dirvals];
// rmax[0] = max over cells of |r| on interior rows
__global__ void __launch_bounds__(256) newton_residual_kernel(CellArgs a, const double *__restrict__ A, double *b,
                                                              const double *__restrict__ xint,
                                                              const double *__restrict__ xskel,
                                                              const double *__restrict__ dirvals, double *rmax) {
  extern __shared__ double xs[];  // n
  __shared__ double red[32];
  const int n = a.n, ni = a.ni, nfd = a.nfd, nl = 2 * a.D;
  double m = 0.0;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double v;
      if (i < ni) {
        v = xint[(size_t)c * ni + i];
      } else {
        const int lf = (i - ni) / nfd, k = (i - ni) - lf * nfd;
        const int id = a.facet_dofs[(size_t)a.cell_facets[(size_t)c * nl + lf] * nfd + k];
        v = id >= 0 ? xskel[id] : dirvals[-1 - id];
      }
      xs[i] = v;
    }
    __syncthreads();
    const double *Ac = A + (size_t)c * n * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double r = -b[(size_t)c * n + i];
      for (int j = 0; j < n; ++j) r += Ac[i + (size_t)n * j] * xs[j];
      b[(size_t)c * n + i] = r;
      if (i < ni) m = fmax(m, fabs(r));
    }
    __syncthreads();
  }
  const double bm = block_max(m, red);
  if (threadIdx.x == 0) atomic_max_nonneg(rmax, bm);
}

// rmax[1] = max over free skeleton DOFs of |sum over the facet's cells of r_f|
__global__ void __launch_bounds__(256) newton_skeleton_norm_kernel(AssembleArgs a, int n, int ni,
                                                                   const double *__restrict__ r, double *rmax) {
  __shared__ double red[32];
  const int nfd = a.nfd, nl = a.nl;
  const int nrows = a.nblockrows * nfd;
  double m = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < nrows; row += gridDim.x * blockDim.x) {
    const int br = row / nfd, i = row - br * nfd;
    double v = 0.0;
    for (int s = 0; s < 2; ++s) {
      const int src = a.br_src[2 * br + s];
      if (src < 0) continue;
      const int c = src / nl, lf = src - c * nl;
      v += r[(size_t)c * n + ni + lf * nfd + i];
    }
    m = fmax(m, fabs(v));
  }
  const double bm = block_max(m, red);
  if (threadIdx.x == 0) atomic_max_nonneg(rmax + 1, bm);
}

__global__ void newton_update_kernel(size_t count, double *x, const double *__restrict__ dx) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    x[i] -= dx[i];
}

cudaError_t launch_newton_residual(const CellArgs &a, const AssembleArgs &as, const double *A, double *b,
                                   const double *xint, const double *xskel, const double *dirvals, double *rmax,
                                   cudaStream_t s, int num_sms, long long *launches) {
  cudaError_t e = cudaMemsetAsync(rmax, 0, 2 * sizeof(double), s);
  if (e != cudaSuccess) return e;
  int g = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  if (g < 1) g = 1;
  const size_t smem = sizeof(double) * a.n;
  if (smem > 48 * 1024) return cudaErrorInvalidValue;
  newton_residual_kernel<<<g, 256, smem, s>>>(a, A, b, xint, xskel, dirvals, rmax);
  const int nrows = as.nblockrows * as.nfd;
  int g2 = (nrows + 255) / 256;
  if (g2 > num_sms * 8) g2 = num_sms * 8;
  if (g2 < 1) g2 = 1;
  newton_skeleton_norm_kernel<<<g2, 256, 0, s>>>(as, a.n, a.ni, b, rmax);
  *launches += 2;
  return cudaGetLastError();
}

cudaError_t launch_newton_update(size_t count, double *x, const double *dx, cudaStream_t s, int num_sms,
                                 long long *launches) {
  if (count == 0) return cudaSuccess;
  size_t g = (count + 255) / 256;
  if (g > (size_t)num_sms * 8) g = (size_t)num_sms * 8;
  newton_update_kernel<<<(int)g, 256, 0, s>>>(count, x, dx);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace hdg
