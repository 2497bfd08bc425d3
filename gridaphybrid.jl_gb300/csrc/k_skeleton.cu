// k_skeleton.cu -- skeleton-side kernels for sm_103a: deterministic assembly
// of the condensed cell blocks into the skeleton CSR matrix (gather through
// precomputed per-block source maps, no atomics), the Dirichlet lift, a
// facet-block-Jacobi PCG whose scalars never leave the device, and a dense LU
// solve for small (possibly indefinite) skeleton systems.
#include <cuda_runtime.h>

#include "hdg_kernels.h"
#include "k_pcg_common.cuh"

namespace hdg {

// ---------------------------------------------------------------------------
// Assembly.
// ---------------------------------------------------------------------------

// glift_c -= S_c x_D for every cell touching a Dirichlet facet (the lift of
// Gridap's _attach_dirichlet, src/HybridAffineFEOperators.jl:41-42).
__global__ void dirichlet_lift_kernel(AssembleArgs a, const double *__restrict__ S,
                                      double *glift) {
  const int nf = a.nf, nfd = a.nfd, nl = a.nl;
  __shared__ double xd[6 * 64];
  for (int t = blockIdx.x; t < a.ndir_cells; t += gridDim.x) {
    const int c = a.dir_cells[t];
    for (int j = threadIdx.x; j < nf; j += blockDim.x) {
      const int lf = j / nfd, b = j - lf * nfd;
      const int id = a.facet_dofs[(size_t)a.cell_facets[(size_t)c * nl + lf] * nfd + b];
      xd[j] = id < 0 ? a.dirvals[-1 - id] : 0.0;
    }
    __syncthreads();
    const double *Sc = S + (size_t)c * nf * nf;
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
      double v = glift[(size_t)c * nf + i];
      for (int j = 0; j < nf; ++j) v -= Sc[i + (size_t)nf * j] * xd[j];
      glift[(size_t)c * nf + i] = v;
    }
    __syncthreads();
  }
}

// One warp per skeleton block (f,g): val = sum over the (one or two)
// contributing cells of their condensed sub-block, cells in increasing order.
// Block shapes are compile-time so the index arithmetic is shifts and
// multiplies and every lane issues all of its loads before its stores.
template <int NL, int NFD>
__global__ void __launch_bounds__(256) assemble_blocks_kernel(AssembleArgs a, const double *__restrict__ S,
                                                              double *__restrict__ val) {
  constexpr int NB = NFD * NFD, NF = NL * NFD, PER = (NB + 31) / 32;
  const int lane = threadIdx.x & 31;
  const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t blk = wid; blk < a.nblocks; blk += nw) {
    const int64_t off = a.blk_off[blk];
    const int rowlen = a.blk_rowlen[blk];
    const int s0 = a.blk_src[2 * blk], s1 = a.blk_src[2 * blk + 1];
    const double *S0 = S + (size_t)(s0 / (NL * NL)) * NF * NF + ((s0 / NL) % NL) * NFD + (size_t)NF * ((s0 % NL) * NFD);
    const double *S1 =
        s1 >= 0 ? S + (size_t)(s1 / (NL * NL)) * NF * NF + ((s1 / NL) % NL) * NFD + (size_t)NF * ((s1 % NL) * NFD)
                : nullptr;
    double v[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int e = lane + 32 * k;
      if (e < NB) {
        const int ra = e / NFD, cb = e - ra * NFD;
        v[k] = S0[ra + NF * cb];
      }
    }
    if (S1) {
#pragma unroll
      for (int k = 0; k < PER; ++k) {
        const int e = lane + 32 * k;
        if (e < NB) {
          const int ra = e / NFD, cb = e - ra * NFD;
          v[k] += S1[ra + NF * cb];
        }
      }
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int e = lane + 32 * k;
      if (e < NB) {
        const int ra = e / NFD, cb = e - ra * NFD;
        val[off + (int64_t)ra * rowlen + cb] = v[k];
      }
    }
  }
}

__global__ void assemble_rhs_kernel(AssembleArgs a, const double *__restrict__ glift,
                                    double *rhs) {
  const int nfd = a.nfd, nf = a.nf, nl = a.nl;
  const int nrows = a.nblockrows * nfd;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    const int br = r / nfd, i = r - br * nfd;
    double v = 0.0;
    for (int s = 0; s < 2; ++s) {
      const int src = a.br_src[2 * br + s];
      if (src < 0) continue;
      const int c = src / nl, lf = src - c * nl;
      v += glift[(size_t)c * nf + lf * nfd + i];
    }
    rhs[a.br_row0[br] + i] = v;
  }
}

cudaError_t launch_assemble(const AssembleArgs &a, const double *S, const double *g,
                            double *glift, double *val, double *rhs, cudaStream_t s,
                            int num_sms, long long *launches) {
  if (a.nf > 6 * 64) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemcpyAsync(glift, g, sizeof(double) * (size_t)a.ncells * a.nf,
                                  cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  if (a.ndir_cells > 0) {
    int grid = a.ndir_cells < num_sms * 8 ? a.ndir_cells : num_sms * 8;
    dirichlet_lift_kernel<<<grid, 64, 0, s>>>(a, S, glift);
    ++*launches;
  }
  {
    int64_t warps = a.nblocks;
    int64_t grid = (warps * 32 + 255) / 256;
    if (grid > (int64_t)num_sms * 16) grid = (int64_t)num_sms * 16;
    if (grid < 1) grid = 1;
#define HDG_ASM(L, F) \
  else if (a.nl == L && a.nfd == F) assemble_blocks_kernel<L, F><<<(int)grid, 256, 0, s>>>(a, S, val);
    if (false) {
    }
    HDG_ASM(4, 2) HDG_ASM(4, 3) HDG_ASM(4, 4) HDG_ASM(4, 5) HDG_ASM(6, 1) HDG_ASM(6, 4) HDG_ASM(6, 9)
    HDG_ASM(6, 16) HDG_ASM(6, 25) HDG_ASM(4, 1) HDG_ASM(4, 6) HDG_ASM(4, 8) HDG_ASM(6, 12) HDG_ASM(6, 27)
    HDG_ASM(6, 3) HDG_ASM(6, 6) HDG_ASM(4, 10)
    HDG_ASM(3, 1) HDG_ASM(3, 2) HDG_ASM(3, 3) HDG_ASM(3, 4) HDG_ASM(3, 5) HDG_ASM(3, 6) HDG_ASM(3, 8)
    else return cudaErrorInvalidValue;
#undef HDG_ASM
    ++*launches;
  }
  {
    int nrows = a.nblockrows * a.nfd;
    int grid = (nrows + 255) / 256;
    if (grid > num_sms * 8) grid = num_sms * 8;
    if (grid < 1) grid = 1;
    assemble_rhs_kernel<<<grid, 256, 0, s>>>(a, glift, rhs);
    ++*launches;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// PCG on (sign*A) x = sign*rhs with facet-block-Jacobi preconditioning, two
// kernels per iteration:
//   spmv:   p_new = z + beta p_old (formed while gathering), q = sign*A p_new,
//           alpha = (r,z) / (p_new,q)
//   update: x += alpha p_new, r -= alpha q, z = Binv r, beta, convergence
// Each kernel's dot products are finished by its last CTA, which sums the
// per-CTA partials in index order (deterministic for a fixed grid).  p is
// double-buffered, so a CUDA graph of an even number of iterations can be
// replayed; once SC_DONE is set every kernel returns immediately.
// ---------------------------------------------------------------------------
// Inverse of each facet's diagonal block of sign*A (Gauss-Jordan, partial pivoting).
// Facet-block inverses for small blocks (nfd <= NMAX): one thread per skeleton
// block row, Gauss-Jordan with partial pivoting on [sign*D | I] in registers
// and local memory; a singular block gets the identity.
template <int NMAX>
__global__ void __launch_bounds__(128) binv_thread_kernel(PcgArgs a) {
  const int nfd = a.nfd;
  double M[NMAX * NMAX], I[NMAX * NMAX];
  for (int br = blockIdx.x * blockDim.x + threadIdx.x; br < a.nblockrows; br += gridDim.x * blockDim.x) {
    const int blk = a.diag_blk[br];
    const int64_t off = a.blk_off[blk];
    const int rl = a.blk_rowlen[blk];
    for (int i = 0; i < nfd; ++i)
      for (int j = 0; j < nfd; ++j) {
        M[i * nfd + j] = a.sign * a.val[off + (int64_t)i * rl + j];
        I[i * nfd + j] = (i == j) ? 1.0 : 0.0;
      }
    bool singular = false;
    for (int c = 0; c < nfd && !singular; ++c) {
      int pr = c;
      for (int i = c + 1; i < nfd; ++i)
        if (fabs(M[i * nfd + c]) > fabs(M[pr * nfd + c])) pr = i;
      if (!(fabs(M[pr * nfd + c]) > 0.0)) {
        singular = true;
        break;
      }
      if (pr != c)
        for (int j = 0; j < nfd; ++j) {
          double t = M[c * nfd + j];
          M[c * nfd + j] = M[pr * nfd + j];
          M[pr * nfd + j] = t;
          t = I[c * nfd + j];
          I[c * nfd + j] = I[pr * nfd + j];
          I[pr * nfd + j] = t;
        }
      const double piv = 1.0 / M[c * nfd + c];
      for (int j = 0; j < nfd; ++j) {
        M[c * nfd + j] *= piv;
        I[c * nfd + j] *= piv;
      }
      for (int i = 0; i < nfd; ++i) {
        if (i == c) continue;
        const double f = M[i * nfd + c];
        if (f != 0.0)
          for (int j = 0; j < nfd; ++j) {
            M[i * nfd + j] -= f * M[c * nfd + j];
            I[i * nfd + j] -= f * I[c * nfd + j];
          }
      }
    }
    double *out = a.Binv + (size_t)br * nfd * nfd;
    for (int i = 0; i < nfd; ++i)
      for (int j = 0; j < nfd; ++j) out[i * nfd + j] = singular ? (i == j ? 1.0 : 0.0) : I[i * nfd + j];
  }
}

// Facet-block inverses of the block-Jacobi preconditioner: one warp per
// skeleton block row, Gauss-Jordan with partial pivoting on [sign*D | I] in
// shared memory (lanes over the 2 nfd columns); a singular block gets the
// identity.
constexpr int kBinvWarps = 4;
__global__ void __launch_bounds__(32 * kBinvWarps) binv_kernel(PcgArgs a) {
  extern __shared__ double Wsm[];  // kBinvWarps x nfd x 2 nfd
  const int nfd = a.nfd, w2 = 2 * nfd;
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  double *W = Wsm + (size_t)wl * nfd * w2;
  const int nw = gridDim.x * kBinvWarps;
  for (int br = blockIdx.x * kBinvWarps + wl; br < a.nblockrows; br += nw) {
    const int blk = a.diag_blk[br];
    const int64_t off = a.blk_off[blk];
    const int rl = a.blk_rowlen[blk];
    for (int e = lane; e < nfd * w2; e += 32) {
      const int i = e / w2, j = e - i * w2;
      W[e] = j < nfd ? a.sign * a.val[off + (int64_t)i * rl + j] : (j - nfd == i ? 1.0 : 0.0);
    }
    __syncwarp();
    bool singular = false;
    for (int c = 0; c < nfd; ++c) {
      double best = -1.0;
      int bi = c;
      for (int i = c + lane; i < nfd; i += 32) {
        const double v = fabs(W[i * w2 + c]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (!(best > 0.0)) {
        singular = true;
        break;
      }
      if (bi != c)
        for (int j = lane; j < w2; j += 32) {
          const double t = W[c * w2 + j];
          W[c * w2 + j] = W[bi * w2 + j];
          W[bi * w2 + j] = t;
        }
      __syncwarp();
      const double piv = 1.0 / W[c * w2 + c];
      __syncwarp();
      for (int j = lane; j < w2; j += 32) W[c * w2 + j] *= piv;
      // column c of every row, held by lane i (nfd <= 32)
      const double fl = lane < nfd ? W[lane * w2 + c] : 0.0;
      __syncwarp();
      for (int i = 0; i < nfd; ++i) {
        const double f = __shfl_sync(0xffffffffu, fl, i);
        if (i == c || f == 0.0) continue;
        for (int j = lane; j < w2; j += 32) W[i * w2 + j] -= f * W[c * w2 + j];
      }
      __syncwarp();
    }
    double *out = a.Binv + (size_t)br * nfd * nfd;
    for (int e = lane; e < nfd * nfd; e += 32) {
      const int i = e / nfd, j = e - i * nfd;
      out[e] = singular ? (i == j ? 1.0 : 0.0) : W[i * w2 + nfd + j];
    }
    __syncwarp();
  }
}

// z = Binv r for the block rows of this CTA's tile (rows staged in smem).
__device__ __forceinline__ double apply_binv(const PcgArgs &a, int row, int nrows, double rval, double *rs) {
  const int nfd = a.nfd;
  rs[threadIdx.x] = rval;
  __syncthreads();
  double z = 0.0;
  if (row < nrows) {
    const int br = row / nfd, i = row - br * nfd;
    const int first = (int)threadIdx.x - i;
    const double *B = a.Binv + (size_t)br * nfd * nfd + (size_t)i * nfd;
    for (int j = 0; j < nfd; ++j) z += B[j] * rs[first + j];
  }
  __syncthreads();
  return z;
}

// x = 0, r = sign*rhs, z = Binv r, p buffers = 0; scalars by the last CTA
__global__ void __launch_bounds__(kPcgThreads) pcg_init_kernel(PcgArgs a, double rtol) {
  __shared__ double rs[kPcgThreads];
  __shared__ double red[32];
  const int tile = (kPcgThreads / a.nfd) * a.nfd;
  double rz = 0.0, rr = 0.0, bb = 0.0;
  for (int base = blockIdx.x * tile; base < a.n; base += gridDim.x * tile) {
    const int row = base + (int)threadIdx.x;
    const bool act = threadIdx.x < (unsigned)tile && row < a.n;
    double r = 0.0;
    if (act) {
      const double b = a.rhs[row];
      r = a.sign * b;
      a.x[row] = 0.0;
      a.r[row] = r;
      a.p[row] = 0.0;
      a.p2[row] = 0.0;
      bb += b * b;
      rr += r * r;
    }
    const double z = apply_binv(a, act ? row : a.n, a.n, r, rs);
    if (act) {
      a.z[row] = z;
      rz += r * z;
    }
  }
  double s = block_sum(rz, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
  s = block_sum(rr, red);
  if (threadIdx.x == 0) a.partials[a.nparts + blockIdx.x] = s;
  s = block_sum(bb, red);
  if (threadIdx.x == 0) a.partials[2 * a.nparts + blockIdx.x] = s;
  if (last_cta(a.counter)) {
    const double vrz = sum_partials(a.partials, a.nparts, 0, red);
    const double vrr = sum_partials(a.partials, a.nparts, 1, red);
    const double vbb = sum_partials(a.partials, a.nparts, 2, red);
    if (threadIdx.x == 0) {
      a.scal[SC_RZ] = vrz;
      a.scal[SC_RR] = vrr;
      a.scal[SC_BB] = vbb;
      a.scal[SC_TOL2] = rtol * rtol * vbb;
      a.scal[SC_BETA] = 0.0;
      a.scal[SC_ITERS] = 0.0;
      a.scal[SC_DONE] = (vrr <= rtol * rtol * vbb) ? 1.0 : 0.0;
      *a.counter = 0u;
    }
  }
}

// p_new = z + beta p_old ; q = sign*A p_new ; alpha = rz / (p_new, q).
// One warp per facet block row: its nfd rows share one column list, read
// once; p_new on those columns is formed in shared memory, then the block
// row's nfd*rowlen contiguous values are streamed.
// q = sign A p with p = z + beta p_old formed at the staged columns (the
// owner rows write p_new), a lane pair per row over tiles of whole block
// rows; alpha = (r,z) / (p,q) by the last CTA
template <typename V, int NFD>
__global__ void __launch_bounds__(kPcgThreads) pcg_spmv_kernel(PcgArgs a, const V *__restrict__ val,
                                                               const double *__restrict__ p_old,
                                                               double *__restrict__ p_new) {
  using T = RowTile<NFD>;
  __shared__ double red[32];
  __shared__ double xs[T::BR * T::LMAX];
  if (a.scal[SC_DONE] != 0.0) return;
  const double beta = a.scal[SC_BETA];
  const double *__restrict__ z = a.z;
  double acc = 0.0;
  for (int br0 = blockIdx.x * T::BR; br0 < a.nblockrows; br0 += gridDim.x * T::BR) {
    const int nbr = min(T::BR, a.nblockrows - br0);
    stage_tile_columns<NFD>(a.rowptr, a.colind, br0, nbr, xs, [&](int col) { return z[col] + beta * p_old[col]; });
    __syncthreads();
    tile_row_products<NFD>(a.rowptr, val, br0, nbr, xs, [&](int row, int, double t) {
      const double pown = z[row] + beta * p_old[row];
      p_new[row] = pown;
      const double q = a.sign * t;
      a.q[row] = q;
      acc += q * pown;
    });
    __syncthreads();  // xs is restaged for the next tile
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
  if (last_cta(a.counter)) {
    const double pq = sum_partials(a.partials, (int)gridDim.x, 0, red);
    if (threadIdx.x == 0) {
      a.scal[SC_PAP] = pq;
      a.scal[SC_ALPHA] = a.scal[SC_RZ] / pq;
      *a.counter = 0u;
    }
  }
}

// x += alpha p; r -= alpha q; z = Binv r; beta = (r,z)_new / (r,z); convergence
__global__ void __launch_bounds__(kPcgThreads) pcg_update_kernel(PcgArgs a, const double *__restrict__ p) {
  __shared__ double rs[kPcgThreads];
  __shared__ double red[32];
  if (a.scal[SC_DONE] != 0.0) return;
  const double alpha = a.scal[SC_ALPHA];
  const int tile = (kPcgThreads / a.nfd) * a.nfd;
  double rz = 0.0, rr = 0.0;
  for (int base = blockIdx.x * tile; base < a.n; base += gridDim.x * tile) {
    const int row = base + (int)threadIdx.x;
    const bool act = threadIdx.x < (unsigned)tile && row < a.n;
    double r = 0.0;
    if (act) {
      a.x[row] += alpha * p[row];
      r = a.r[row] - alpha * a.q[row];
      a.r[row] = r;
      rr += r * r;
    }
    const double z = apply_binv(a, act ? row : a.n, a.n, r, rs);
    if (act) {
      a.z[row] = z;
      rz += r * z;
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

cudaError_t launch_pcg_setup(const PcgArgs &a, double rtol, cudaStream_t s, int num_sms,
                             long long *launches) {
  if (a.nfd > 27) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  if (a.nfd <= 12) {  // small blocks: one thread per block row
    int g = (a.nblockrows + 127) / 128;
    if (g < 1) g = 1;
    binv_thread_kernel<12><<<g, 128, 0, s>>>(a);
  } else {
    int g = (a.nblockrows + kBinvWarps - 1) / kBinvWarps;
    if (g > num_sms * 16) g = num_sms * 16;
    if (g < 1) g = 1;
    binv_kernel<<<g, 32 * kBinvWarps, sizeof(double) * kBinvWarps * a.nfd * 2 * a.nfd, s>>>(a);
  }
  pcg_init_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a, rtol);
  *launches += 2;
  return cudaGetLastError();
}

template <typename V>
static cudaError_t spmv_dispatch(const PcgArgs &a, const V *val, const double *po, double *pn, cudaStream_t s) {
  if (a.max_rowlen > kRowBlocks * a.nfd) return cudaErrorInvalidValue;  // the staged tile holds 11 blocks a row
  switch (a.nfd) {
#define HDG_SPMV_CASE(N) \
  case N:                \
    pcg_spmv_kernel<V, N><<<a.tile_ctas, kPcgThreads, 0, s>>>(a, val, po, pn); break;
    HDG_SPMV_CASE(1)
    HDG_SPMV_CASE(2)
    HDG_SPMV_CASE(3)
    HDG_SPMV_CASE(4)
    HDG_SPMV_CASE(5)
    HDG_SPMV_CASE(6)
    HDG_SPMV_CASE(8)
    HDG_SPMV_CASE(9)
    HDG_SPMV_CASE(10)
    HDG_SPMV_CASE(12)
    HDG_SPMV_CASE(16)
    HDG_SPMV_CASE(25)
    HDG_SPMV_CASE(27)
#undef HDG_SPMV_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

static cudaError_t spmv_any(const PcgArgs &a, const double *po, double *pn, cudaStream_t s) {
  return a.val32 ? spmv_dispatch<float>(a, a.val32, po, pn, s) : spmv_dispatch<double>(a, a.val, po, pn, s);
}

bool assemble_supports(int nl, int nfd) {
  // triangles (P_k traces and their copies), quads / tetrahedra, hexahedra
  if (nl == 3) return nfd == 1 || nfd == 2 || nfd == 3 || nfd == 4 || nfd == 5 || nfd == 6 || nfd == 8;
  if (nl == 4)
    return nfd == 1 || nfd == 2 || nfd == 3 || nfd == 4 || nfd == 5 || nfd == 6 || nfd == 8 || nfd == 10;
  return nl == 6 && (nfd == 1 || nfd == 3 || nfd == 4 || nfd == 6 || nfd == 9 || nfd == 12 || nfd == 16 ||
                     nfd == 25 || nfd == 27);
}

bool pcg_supports_nfd(int nfd) {
  // scalar traces (k+1)^(D-1) (1: RT_0 / Q_0 multipliers); displacement traces D (k+1)^(D-1): 4, 6, 8
  // (2D), 12, 27 (3D k=1, 2)
  return nfd == 1 || nfd == 2 || nfd == 3 || nfd == 4 || nfd == 5 || nfd == 6 || nfd == 8 || nfd == 9 || nfd == 10 ||
         nfd == 12 || nfd == 16 || nfd == 25 || nfd == 27;
}

cudaError_t launch_spmv(const PcgArgs &a, cudaStream_t s, long long *launches) {
  ++*launches;
  return spmv_any(a, a.p, a.p2, s);
}

// Two PCG iterations (p buffers swap back to where they started).
cudaError_t launch_pcg_iteration_pair(const PcgArgs &a, cudaStream_t s, int num_sms,
                                      long long *launches) {
  for (int half = 0; half < 2; ++half) {
    const double *po = half ? a.p2 : a.p;
    double *pn = half ? a.p : a.p2;
    cudaError_t e = spmv_any(a, po, pn, s);
    if (e != cudaSuccess) return e;
    pcg_update_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a, pn);
  }
  *launches += 4;
  (void)num_sms;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Dense LU solve (small systems; any sign/definiteness): one CTA, the
// augmented matrix [A | b] in global scratch (column-major, ld = n).
// ---------------------------------------------------------------------------
__global__ void dense_fill_kernel(int n, const int64_t *rowptr, const int *colind,
                                  const double *val, const double *rhs, double *W) {
  const size_t total = (size_t)n * (n + 1);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x)
    W[e] = 0.0;
}

__global__ void dense_scatter_kernel(int n, const int64_t *rowptr, const int *colind,
                                     const double *val, const double *rhs, double *W) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    for (int64_t p = rowptr[r]; p < rowptr[r + 1]; ++p) W[r + (size_t)n * colind[p]] = val[p];
    W[r + (size_t)n * n] = rhs[r];
  }
}

__global__ void __launch_bounds__(1024) dense_lu_kernel(int n, double *W, double *x, int *info) {
  __shared__ int s_piv;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int inf = 0;
  for (int j = 0; j < n; ++j) {
    if (warp == 0) {
      double best = -1.0;
      int bi = j;
      for (int i = j + lane; i < n; i += 32) {
        double v = fabs(W[i + (size_t)n * j]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        double ov = __shfl_down_sync(0xffffffffu, best, off);
        int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) s_piv = best > 0.0 ? bi : -1;
    }
    __syncthreads();
    const int p = s_piv;
    if (p < 0) {
      if (!inf) inf = j + 1;
      __syncthreads();
      continue;
    }
    if (p != j)
      for (int c = j + threadIdx.x; c <= n; c += blockDim.x) {
        double t = W[j + (size_t)n * c];
        W[j + (size_t)n * c] = W[p + (size_t)n * c];
        W[p + (size_t)n * c] = t;
      }
    __syncthreads();
    const double r = 1.0 / W[j + (size_t)n * j];
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) W[i + (size_t)n * j] *= r;
    __syncthreads();
    for (int c = j + 1 + warp; c <= n; c += nw) {
      const double u = W[j + (size_t)n * c];
      if (u != 0.0)
        for (int i = j + 1 + lane; i < n; i += 32) W[i + (size_t)n * c] -= W[i + (size_t)n * j] * u;
    }
    __syncthreads();
  }
  double *rhs = W + (size_t)n * n;
  for (int j = n - 1; j >= 0; --j) {
    __syncthreads();
    const double diag = W[j + (size_t)n * j];
    const double uj = diag != 0.0 ? rhs[j] / diag : 0.0;
    __syncthreads();
    if (threadIdx.x == 0) rhs[j] = uj;
    for (int i = threadIdx.x; i < j; i += blockDim.x) rhs[i] -= W[i + (size_t)n * j] * uj;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = rhs[i];
  if (threadIdx.x == 0) *info = inf;
}

cudaError_t launch_dense_solve(int n, const int64_t *rowptr, const int *colind,
                               const double *val, const double *rhs, double *work,
                               double *x, int *info, cudaStream_t s, long long *launches) {
  int g = (int)(((size_t)n * (n + 1) + 255) / 256);
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  dense_fill_kernel<<<g, 256, 0, s>>>(n, rowptr, colind, val, rhs, work);
  dense_scatter_kernel<<<(n + 255) / 256 > 0 ? (n + 255) / 256 : 1, 256, 0, s>>>(n, rowptr, colind, val, rhs, work);
  dense_lu_kernel<<<1, 1024, 0, s>>>(n, work, x, info);
  *launches += 3;
  return cudaGetLastError();
}

}  // namespace hdg
