// k_pcg32.cu -- skeleton solve for the FP32 + refinement path (sm_103a).
//
// Mixed-precision iterative refinement around an FP32 PCG:
//   outer (FP64):  x = 0, r = c  (c = sign*rhs, the SPD frame M = sign*A)
//                  repeat: solve M e ~= r with the inner PCG; x += e;
//                          r = c - M x with the FP64 matrix; until |r| <= rtol |c|
//   inner (FP32):  facet-block-Jacobi PCG on the FP32 copy of the matrix with
//                  FP32 vectors; its dot products accumulate in FP64.
// GB300 executes FP64 at 1/62 of its FP32 rate, which makes even an FP64
// SpMV arithmetic-bound; the inner iterations stay on the FP32 pipes and
// stream half the bytes, the FP64 residual runs once per outer step.
#include <cuda_runtime.h>

#include "hdg_kernels.h"
#include "k_pcg_common.cuh"

namespace hdg {

// Binv32 = (float) Binv
__global__ void binv_to_f32_kernel(size_t count, const double *__restrict__ Binv, float *Binv32) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    Binv32[i] = (float)Binv[i];
}

// z = Binv32 r for the rows of this CTA's tile (whole facet blocks, rows in smem)
__device__ __forceinline__ float apply_binv32(const Pcg32Args &a, int row, float rval, float *rs) {
  const int nfd = a.nfd;
  rs[threadIdx.x] = rval;
  __syncthreads();
  float z = 0.0f;
  if (row < a.n) {
    const int br = row / nfd, i = row - br * nfd;
    const int first = (int)threadIdx.x - i;
    const float *B = a.Binv32 + (size_t)br * nfd * nfd + (size_t)i * nfd;
    for (int j = 0; j < nfd; ++j) z = fmaf(B[j], rs[first + j], z);
  }
  __syncthreads();
  return z;
}

// inner start: x = 0, r = (float) rhs, z = Binv r, p = 0; scalars by the last CTA
__global__ void __launch_bounds__(kPcgThreads) pcg32_init_kernel(Pcg32Args a, double eta) {
  __shared__ float rs[kPcgThreads];
  __shared__ double red[32];
  const int tile = (kPcgThreads / a.nfd) * a.nfd;
  double rz = 0.0, rr = 0.0;
  for (int base = blockIdx.x * tile; base < a.n; base += gridDim.x * tile) {
    const int row = base + (int)threadIdx.x;
    const bool act = threadIdx.x < (unsigned)tile && row < a.n;
    float r = 0.0f;
    if (act) {
      r = (float)a.rhs[row];
      a.x[row] = 0.0f;
      a.r[row] = r;
      a.p[row] = 0.0f;
      a.p2[row] = 0.0f;
      rr += (double)r * r;
    }
    const float z = apply_binv32(a, act ? row : a.n, r, rs);
    if (act) {
      a.z[row] = z;
      rz += (double)r * z;
    }
  }
  double s = block_sum(rz, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
  s = block_sum(rr, red);
  if (threadIdx.x == 0) a.partials[a.nparts + blockIdx.x] = s;
  if (last_cta(a.counter)) {
    const double vrz = sum_partials(a.partials, a.nparts, 0, red);
    const double vrr = sum_partials(a.partials, a.nparts, 1, red);
    if (threadIdx.x == 0) {
      a.scal[SC_RZ] = vrz;
      a.scal[SC_RR] = vrr;
      a.scal[SC_BB] = vrr;
      a.scal[SC_TOL2] = eta * eta * vrr;
      a.scal[SC_BETA] = 0.0;
      a.scal[SC_ITERS] = 0.0;
      a.scal[SC_DONE] = (vrr == 0.0) ? 1.0 : 0.0;
      *a.counter = 0u;
    }
  }
}

// p_new = z + beta p_old ; q = M32 p_new ; alpha = (r,z)/(p_new,q)
template <int NFD>
__global__ void __launch_bounds__(kPcgThreads) pcg32_spmv_kernel(Pcg32Args a, const float *__restrict__ p_old,
                                                                 float *__restrict__ p_new) {
  __shared__ double red[32];
  __shared__ float xs[kPcgThreads / 32][kMaxRowLen];
  if (a.scal[SC_DONE] != 0.0) return;
  const float beta = (float)a.scal[SC_BETA];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (int br = wid; br < a.nblockrows; br += nw) {
    const int row0 = br * NFD;
    const int64_t base = a.rowptr[row0];
    const int rowlen = (int)(a.rowptr[row0 + 1] - base);
    for (int j = lane; j < rowlen; j += 32) {
      const int col = a.colind[base + j];
      xs[w][j] = fmaf(beta, p_old[col], a.z[col]);
    }
    float pown = 0.0f;
    if (lane < NFD) {
      pown = fmaf(beta, p_old[row0 + lane], a.z[row0 + lane]);
      p_new[row0 + lane] = pown;
    }
    __syncwarp();
    constexpr int P = Pow2Ceil<NFD>::v;
    float v[P];
#pragma unroll
    for (int r = 0; r < P; ++r) v[r] = 0.0f;
    for (int j = lane; j < rowlen; j += 32) {
      const float xv = xs[w][j];
      const float *vj = a.val32 + base + j;
#pragma unroll
      for (int r = 0; r < NFD; ++r) v[r] = fmaf(__ldcs(vj + (int64_t)r * rowlen), xv, v[r]);
    }
    const float tot = warp_reduce_scatter<float, P>(v, lane);
    const int myrow = reduce_scatter_row<P>(lane);
    const float pmine = __shfl_sync(0xffffffffu, pown, myrow < NFD ? myrow : 0);
    if (myrow < NFD && reduce_scatter_writer<P>(lane)) {
      const float q = (float)a.sign * tot;
      a.q[row0 + myrow] = q;
      acc += (double)q * pmine;
    }
    __syncwarp();
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
  if (last_cta(a.counter)) {
    const double pq = sum_partials(a.partials, a.nparts, 0, red);
    if (threadIdx.x == 0) {
      a.scal[SC_PAP] = pq;
      a.scal[SC_ALPHA] = a.scal[SC_RZ] / pq;
      *a.counter = 0u;
    }
  }
}

// x += alpha p; r -= alpha q; z = Binv r; beta; convergence against eta |rhs|
__global__ void __launch_bounds__(kPcgThreads) pcg32_update_kernel(Pcg32Args a, const float *__restrict__ p) {
  __shared__ float rs[kPcgThreads];
  __shared__ double red[32];
  if (a.scal[SC_DONE] != 0.0) return;
  const float alpha = (float)a.scal[SC_ALPHA];
  const int tile = (kPcgThreads / a.nfd) * a.nfd;
  double rz = 0.0, rr = 0.0;
  for (int base = blockIdx.x * tile; base < a.n; base += gridDim.x * tile) {
    const int row = base + (int)threadIdx.x;
    const bool act = threadIdx.x < (unsigned)tile && row < a.n;
    float r = 0.0f;
    if (act) {
      a.x[row] = fmaf(alpha, p[row], a.x[row]);
      r = fmaf(-alpha, a.q[row], a.r[row]);
      a.r[row] = r;
      rr += (double)r * r;
    }
    const float z = apply_binv32(a, act ? row : a.n, r, rs);
    if (act) {
      a.z[row] = z;
      rz += (double)r * z;
    }
  }
  double s = block_sum(rz, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
  s = block_sum(rr, red);
  if (threadIdx.x == 0) a.partials[a.nparts + blockIdx.x] = s;
  if (last_cta(a.counter)) {
    const double vrz = sum_partials(a.partials, a.nparts, 0, red);
    const double vrr = sum_partials(a.partials, a.nparts, 1, red);
    if (threadIdx.x == 0) {
      a.scal[SC_BETA] = vrz / a.scal[SC_RZ];
      a.scal[SC_RZ] = vrz;
      a.scal[SC_RR] = vrr;
      a.scal[SC_ITERS] += 1.0;
      if (vrr <= a.scal[SC_TOL2] || !(vrr == vrr)) a.scal[SC_DONE] = 1.0;
      *a.counter = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// Outer FP64 refinement.
// ---------------------------------------------------------------------------

// x = 0, r = c = sign*rhs, |c|^2
__global__ void __launch_bounds__(kPcgThreads) outer_init_kernel(OuterArgs a) {
  __shared__ double red[32];
  double cc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    const double c = a.sign * a.rhs[i];
    a.x[i] = 0.0;
    a.r[i] = c;
    cc += c * c;
  }
  const double s = block_sum(cc, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
  if (last_cta(a.counter)) {
    const double v = sum_partials(a.partials, a.nparts, 0, red);
    if (threadIdx.x == 0) {
      a.scal[0] = v;  // |c|^2
      a.scal[1] = v;  // |r|^2
      *a.counter = 0u;
    }
  }
}

// x += e (the inner correction)
__global__ void outer_axpy_kernel(int n, const float *__restrict__ e, double *x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += (double)e[i];
}

// r = c - M x with the FP64 matrix (block-row gather of x), |r|^2
template <int NFD>
__global__ void __launch_bounds__(kPcgThreads) outer_residual_kernel(OuterArgs a) {
  __shared__ double red[32];
  __shared__ double xs[kPcgThreads / 32][kMaxRowLen];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (int br = wid; br < a.nblockrows; br += nw) {
    const int row0 = br * NFD;
    const int64_t base = a.rowptr[row0];
    const int rowlen = (int)(a.rowptr[row0 + 1] - base);
    for (int j = lane; j < rowlen; j += 32) xs[w][j] = a.x[a.colind[base + j]];
    __syncwarp();
    constexpr int P = Pow2Ceil<NFD>::v;
    double v[P];
#pragma unroll
    for (int r = 0; r < P; ++r) v[r] = 0.0;
    for (int j = lane; j < rowlen; j += 32) {
      const double xv = xs[w][j];
      const double *vj = a.val + base + j;
#pragma unroll
      for (int r = 0; r < NFD; ++r) v[r] += __ldcs(vj + (int64_t)r * rowlen) * xv;
    }
    const double tot = warp_reduce_scatter<double, P>(v, lane);
    const int myrow = reduce_scatter_row<P>(lane);
    if (myrow < NFD && reduce_scatter_writer<P>(lane)) {
      const double r = a.sign * a.rhs[row0 + myrow] - a.sign * tot;
      a.r[row0 + myrow] = r;
      acc += r * r;
    }
    __syncwarp();
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
  if (last_cta(a.counter)) {
    const double v = sum_partials(a.partials, a.nparts, 0, red);
    if (threadIdx.x == 0) {
      a.scal[1] = v;
      *a.counter = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
cudaError_t launch_binv_to_f32(size_t count, const double *Binv, float *Binv32, cudaStream_t s,
                               long long *launches) {
  size_t g = (count + 255) / 256;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  binv_to_f32_kernel<<<(int)g, 256, 0, s>>>(count, Binv, Binv32);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_pcg32_init(const Pcg32Args &a, double eta, cudaStream_t s, long long *launches) {
  pcg32_init_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a, eta);
  ++*launches;
  return cudaGetLastError();
}

template <int NFD>
static void pcg32_pair(const Pcg32Args &a, cudaStream_t s) {
  pcg32_spmv_kernel<NFD><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p, a.p2);
  pcg32_update_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a, a.p2);
  pcg32_spmv_kernel<NFD><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p2, a.p);
  pcg32_update_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a, a.p);
}

cudaError_t launch_pcg32_iteration_pair(const Pcg32Args &a, cudaStream_t s, long long *launches) {
  switch (a.nfd) {
    case 2: pcg32_pair<2>(a, s); break;
    case 3: pcg32_pair<3>(a, s); break;
    case 4: pcg32_pair<4>(a, s); break;
    case 5: pcg32_pair<5>(a, s); break;
    case 9: pcg32_pair<9>(a, s); break;
    case 16: pcg32_pair<16>(a, s); break;
    case 25: pcg32_pair<25>(a, s); break;
    default: return cudaErrorInvalidValue;
  }
  *launches += 4;
  return cudaGetLastError();
}

cudaError_t launch_pcg32_spmv(const Pcg32Args &a, cudaStream_t s, long long *launches) {
  switch (a.nfd) {
    case 2: pcg32_spmv_kernel<2><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p, a.p2); break;
    case 3: pcg32_spmv_kernel<3><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p, a.p2); break;
    case 4: pcg32_spmv_kernel<4><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p, a.p2); break;
    case 5: pcg32_spmv_kernel<5><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p, a.p2); break;
    case 9: pcg32_spmv_kernel<9><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p, a.p2); break;
    case 16: pcg32_spmv_kernel<16><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p, a.p2); break;
    case 25: pcg32_spmv_kernel<25><<<a.nparts, kPcgThreads, 0, s>>>(a, a.p, a.p2); break;
    default: return cudaErrorInvalidValue;
  }
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_outer_init(const OuterArgs &a, cudaStream_t s, long long *launches) {
  outer_init_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_outer_update(const OuterArgs &a, const float *e, cudaStream_t s, long long *launches) {
  int g = (a.n + 255) / 256;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  outer_axpy_kernel<<<g, 256, 0, s>>>(a.n, e, a.x);
  switch (a.nfd) {
    case 2: outer_residual_kernel<2><<<a.nparts, kPcgThreads, 0, s>>>(a); break;
    case 3: outer_residual_kernel<3><<<a.nparts, kPcgThreads, 0, s>>>(a); break;
    case 4: outer_residual_kernel<4><<<a.nparts, kPcgThreads, 0, s>>>(a); break;
    case 5: outer_residual_kernel<5><<<a.nparts, kPcgThreads, 0, s>>>(a); break;
    case 9: outer_residual_kernel<9><<<a.nparts, kPcgThreads, 0, s>>>(a); break;
    case 16: outer_residual_kernel<16><<<a.nparts, kPcgThreads, 0, s>>>(a); break;
    case 25: outer_residual_kernel<25><<<a.nparts, kPcgThreads, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  *launches += 2;
  return cudaGetLastError();
}

}  // namespace hdg
