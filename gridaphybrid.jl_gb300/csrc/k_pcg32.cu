// k_pcg32.cu -- skeleton solve for the FP32 + refinement path (sm_103a).
//
// Mixed-precision iterative refinement around an FP32 PCG:
//   outer (FP64):  x = 0, r = c  (c = sign*rhs, the SPD frame M = sign*A)
//                  repeat: solve M e ~= r with the inner PCG; x += e;
//                          r = c - M x with the FP64 matrix; until |r| <= rtol |c|
//   inner (FP32):  facet-block-Jacobi PCG with FP32 vectors on the FP32
//                  operator held as unassembled symmetric cell blocks, the
//                  preconditioner applied as a symmetric scaling of the
//                  records (CG on W M W^T, W = blockdiag(L_f^{-1}) with
//                  D_f = L_f L_f^T), so an iteration reads no block inverse;
//                  its dot products accumulate in float-float.
// GB300 executes FP64 at about 1/74 of its FP32 rate, which makes even an
// FP64 SpMV arithmetic-bound; the inner iterations stay on the FP32 pipes and
// stream about a sixth of the FP64 CSR bytes (FP32, the facet blocks above the
// diagonal only), the FP64 CSR residual runs once per outer step.
#include <cuda_runtime.h>

#include "hdg_kernels.h"
#include "k_bulk.cuh"
#include "k_pcg_common.cuh"

namespace hdg {

// W rhs for the rows of this CTA's tile (whole facet blocks; the tile's rhs
// values staged in shared memory); W is lower triangular.
__device__ __forceinline__ double apply_w64(const Pcg32Args &a, int row, double v, double *rs) {
  const int nfd = a.nfd;
  rs[threadIdx.x] = v;
  __syncthreads();
  double y = 0.0;
  if (row < a.n) {
    const int br = row / nfd, i = row - br * nfd;
    const int first = (int)threadIdx.x - i;
    const double *Wr = a.W + (size_t)br * nfd * nfd + (size_t)i * nfd;
    for (int j = 0; j <= i; ++j) y = fma(Wr[j], rs[first + j], y);
  }
  __syncthreads();
  return y;
}

// inner start: x = 0, r = z = (float) W rhs, p = 0; scalars by the last CTA
__global__ void __launch_bounds__(kPcgThreads) pcg32_init_kernel(Pcg32Args a, double eta) {
  __shared__ double rs[kPcgThreads];
  __shared__ double red[32];
  const int tile = (kPcgThreads / a.nfd) * a.nfd;
  double rr = 0.0;
  for (int base = blockIdx.x * tile; base < a.n; base += gridDim.x * tile) {
    const int row = base + (int)threadIdx.x;
    const bool act = threadIdx.x < (unsigned)tile && row < a.n;
    const double y = apply_w64(a, act ? row : a.n, act ? a.rhs[row] : 0.0, rs);
    if (act) {
      const float r = (float)y;
      a.x[row] = 0.0f;
      a.r[row] = r;
      a.p[row] = 0.0f;
      a.p2[row] = 0.0f;
      rr += (double)r * r;
    }
  }
  const double s = block_sum(rr, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
  if (last_cta(a.counter)) {
    const double vrr = sum_partials(a.partials, a.nparts, 0, red);
    if (threadIdx.x == 0) {
      a.scal[SC_RZ] = vrr;
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

// reliable update: the inner residual is replaced by the (scaled) FP64 outer
// residual (x = 0 again: the correction so far went into the FP64 iterate)
// and the search direction p is kept, so the Krylov space is not thrown
// away: beta = (r,r)_new / (r,r) of the iteration before, and the next SpMV
// forms p = r + beta p as in any other iteration.
__global__ void __launch_bounds__(kPcgThreads) pcg32_replace_kernel(Pcg32Args a, double eta) {
  __shared__ double rs[kPcgThreads];
  __shared__ double red[32];
  const int tile = (kPcgThreads / a.nfd) * a.nfd;
  double rr = 0.0;
  for (int base = blockIdx.x * tile; base < a.n; base += gridDim.x * tile) {
    const int row = base + (int)threadIdx.x;
    const bool act = threadIdx.x < (unsigned)tile && row < a.n;
    const double y = apply_w64(a, act ? row : a.n, act ? a.rhs[row] : 0.0, rs);
    if (act) {
      const float r = (float)y;
      a.x[row] = 0.0f;
      a.r[row] = r;
      rr += (double)r * r;
    }
  }
  const double s = block_sum(rr, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
  if (last_cta(a.counter)) {
    const double vrr = sum_partials(a.partials, a.nparts, 0, red);
    if (threadIdx.x == 0) {
      // the update that ended the cycle stored beta = (r,r)_N / (r,r)_{N-1}
      // and (r,r)_N; with r_N replaced, beta = (r,r)_new / (r,r)_{N-1}
      const double old = a.scal[SC_RZ];
      a.scal[SC_BETA] = old != 0.0 ? a.scal[SC_BETA] * (vrr / old) : 0.0;
      a.scal[SC_RZ] = vrr;
      a.scal[SC_RR] = vrr;
      a.scal[SC_TOL2] = eta * eta * vrr;
      a.scal[SC_DONE] = (vrr == 0.0) ? 1.0 : 0.0;
      *a.counter = 0u;
    }
  }
}

// W = blockdiag(L_f^{-1}) in FP64, with the Cholesky factor of sign*D_f and
// its inverse held in registers: a group of nfd lanes per free facet (32/nfd
// facets per warp), lane i holding row i of L while it is factored and then
// column i of L^{-1} (forward substitution of every column at once), the
// other lanes' entries passed by shuffles.  In FP64: the scaled operator
// W sign*A W^T then has the identity as its assembled diagonal blocks to FP64
// rounding, and the cell records leave those blocks out (the inner iteration
// adds p for them), so W's own rounding must not show there.  A block that is
// not positive definite gets W = I and raises the flag after the last block
// (W[nblockrows * nfd^2] = 1.0): the records do not hold for it, and the host
// finishes such a solve in FP64.
template <int NFD>
__global__ void __launch_bounds__(128) block_chol_inv_kernel(PcgArgs a, double *W) {
  constexpr int G = 32 / NFD;  // facets per warp
  const int lane = threadIdx.x & 31;
  const int sub = lane / NFD, i = lane - sub * NFD;
  const int base = sub * NFD;  // the group's first lane (past 31 for the idle lanes: shuffles wrap, values unused)
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  const int wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  for (int br0 = wid * G; br0 < a.nblockrows; br0 += nwarps * G) {
    const int br = br0 + sub;
    const bool act = sub < G && br < a.nblockrows;
    double Lr[NFD];  // row i of sign*D_f, then of L (entries j <= i used)
    if (act) {
      const int blk = a.diag_blk[br];
      const int64_t off = a.blk_off[blk] + (int64_t)i * a.blk_rowlen[blk];
#pragma unroll
      for (int j = 0; j < NFD; ++j) Lr[j] = a.sign * a.val[off + j];
    } else {
#pragma unroll
      for (int j = 0; j < NFD; ++j) Lr[j] = j == i ? 1.0 : 0.0;
    }
    bool ok = true;
    double dinv[NFD];  // 1 / L[c][c], the same in the whole group
    // fixed trip counts (fully unrolled: the rows stay in registers); one
    // reciprocal square root per pivot and no division (FP64 runs at a small
    // fraction of the FP32 rate here)
#pragma unroll NFD
    for (int c = 0; c < NFD; ++c) {
      double d = __shfl_sync(0xffffffffu, Lr[c], base + c);  // the pivot, the same in the whole group
      if (!(d > 0.0) || !isfinite(d)) {
        ok = false;
        d = 1.0;  // keep the arithmetic finite; the block gets W = I
      }
      const double inv = rsqrt(d);
      dinv[c] = inv;
      Lr[c] = i == c ? d * inv : (i > c ? Lr[c] * inv : Lr[c]);
#pragma unroll NFD
      for (int j = 1; j < NFD; ++j) {
        if (j <= c) continue;
        const double ljc = __shfl_sync(0xffffffffu, Lr[c], base + j);  // L[j][c], scaled above
        Lr[j] = j <= i ? fma(-Lr[c], ljc, Lr[j]) : Lr[j];
      }
    }
    // column i of L^{-1}: X[r] = (delta_ri - sum_{k<r} L[r][k] X[k]) / L[r][r]
    double X[NFD];
#pragma unroll
    for (int r = 0; r < NFD; ++r) {
      double v = r == i ? 1.0 : 0.0;
#pragma unroll
      for (int k = 0; k < r; ++k) v = fma(-__shfl_sync(0xffffffffu, Lr[k], base + r), X[k], v);
      X[r] = v * dinv[r];
    }
    if (act) {
      double *out = W + (size_t)br * NFD * NFD + i;
#pragma unroll
      for (int r = 0; r < NFD; ++r) out[r * NFD] = ok ? X[r] : (r == i ? 1.0 : 0.0);
      if (!ok && i == 0) W[(size_t)a.nblockrows * NFD * NFD] = 1.0;
    }
  }
}

// ---------------------------------------------------------------------------
// The unassembled FP32 operator.
//
// Cell record: the facet blocks above the diagonal (a < b, row-major order of
// (a, b)) of the scaled cell operator W_a sign*(S_c + S_c^T)/2 W_b^T (W_f the
// facet's L_f^{-1}, the identity on Dirichlet facets, whose rows the SpMV
// skips), each block nfd x nfd row-major at a stride of cellop_bstride(nfd)
// floats, the record padded to a multiple of four floats (16 bytes) so it can
// be bulk-copied.  The diagonal blocks are left out:
// summed over a facet's cells they give W_f sign*D_f W_f^T = I, which the
// inner iteration applies as p itself.  The storage streams 15/36 of the full
// 3D cell matrix (21/36 with the diagonal blocks); the lower blocks are read
// transposed from shared memory.  The two triangular products run in FP32
// from the FP64 symmetric part.
__device__ __forceinline__ void upper_block(int nl, int blk, int &lo, int &hi) {
  int l = 0, rem = blk;
  while (rem >= nl - 1 - l) {
    rem -= nl - 1 - l;
    ++l;
  }
  lo = l;
  hi = l + 1 + rem;
}

__global__ void pack_cell_blocks_kernel(int ncells, int nl, int nfd, int rec, double sign,
                                        const double *__restrict__ S, const int *__restrict__ cell_blk,
                                        const double *__restrict__ W, float *__restrict__ out) {
  extern __shared__ double Ss[];  // nf^2 doubles, then nl nb + 2 nblk nb floats
  const int nf = nl * nfd, nb = nfd * nfd, nblk = cellop_blocks(nl);
  float *Ws = reinterpret_cast<float *>(Ss + (size_t)nf * nf);
  float *Ts = Ws + nl * nb;    // the FP32 symmetric part sign (S + S^T)/2 of every upper block
  float *Us = Ts + nblk * nb;  // T W_hi^T
  for (int c = blockIdx.x; c < ncells; c += gridDim.x) {
    const double *Sc = S + (size_t)c * nf * nf;
    for (int e = threadIdx.x; e < nf * nf; e += blockDim.x) Ss[e] = Sc[e];
    for (int e = threadIdx.x; e < nl * nb; e += blockDim.x) {
      const int lf = e / nb, w = e - lf * nb, r = w / nfd, q = w - r * nfd;
      const int ent = cell_blk[(size_t)c * nl + lf];
      Ws[e] = ent >= 0 ? (float)W[(size_t)(ent >> 1) * nb + w] : (r == q ? 1.0f : 0.0f);
    }
    __syncthreads();
    // T[blk][p][q] = sign (S(lo p, hi q) + S(hi q, lo p)) / 2
    for (int e = threadIdx.x; e < nblk * nb; e += blockDim.x) {
      const int blk = e / nb, w = e - blk * nb, p = w / nfd, q = w - p * nfd;
      int lo, hi;
      upper_block(nl, blk, lo, hi);
      const int i = lo * nfd + p, j = hi * nfd + q;
      Ts[e] = (float)(0.5 * sign * (Ss[i + (size_t)nf * j] + Ss[j + (size_t)nf * i]));
    }
    __syncthreads();
    // U[blk][p][s] = sum_{q <= s} T[blk][p][q] W_hi[s][q]
    for (int e = threadIdx.x; e < nblk * nb; e += blockDim.x) {
      const int blk = e / nb, w = e - blk * nb, p = w / nfd, sc = w - p * nfd;
      int lo, hi;
      upper_block(nl, blk, lo, hi);
      const float *Wh = Ws + hi * nb + sc * nfd;
      const float *T = Ts + blk * nb + p * nfd;
      float u = 0.0f;
      for (int q = 0; q <= sc; ++q) u = fmaf(T[q], Wh[q], u);
      Us[e] = u;
    }
    __syncthreads();
    // record[blk][r][s] = sum_{p <= r} W_lo[r][p] U[blk][p][s]
    float *o = out + (size_t)c * rec;
    const int bs = cellop_bstride(nfd);
    for (int e = threadIdx.x; e < rec; e += blockDim.x) {
      float v = 0.0f;
      const int blk = e / bs, w = e - blk * bs;
      if (blk < nblk && w < nb) {  // else: padding
        const int r = w / nfd, sc = w - r * nfd;
        int lo, hi;
        upper_block(nl, blk, lo, hi);
        const float *Wl = Ws + lo * nb + r * nfd;
        const float *U = Us + blk * nb + sc;
        for (int p = 0; p <= r; ++p) v = fmaf(Wl[p], U[p * nfd], v);
      }
      o[e] = v;
    }
    __syncthreads();
  }
}

// The same kernel with the block shape at compile time (constant divisors,
// the upper-block decode from a table).
template <int NL, int NFD>
__global__ void __launch_bounds__(256) pack_cell_blocks_t(int ncells, int rec, double sign,
                                                          const double *__restrict__ S, const int *__restrict__ cell_blk,
                                                          const double *__restrict__ W, float *__restrict__ out) {
  constexpr int NF = NL * NFD, NB = NFD * NFD, NBLK = cellop_blocks(NL);
  extern __shared__ double Ss[];
  float *Ws = reinterpret_cast<float *>(Ss + NF * NF);
  float *Ts = Ws + NL * NB;
  float *Us = Ts + NBLK * NB;
  __shared__ unsigned char blo[NBLK], bhi[NBLK];
  if (threadIdx.x < NBLK) {
    int lo, hi;
    upper_block(NL, threadIdx.x, lo, hi);
    blo[threadIdx.x] = (unsigned char)lo;
    bhi[threadIdx.x] = (unsigned char)hi;
  }
  for (int c = blockIdx.x; c < ncells; c += gridDim.x) {
    const double *Sc = S + (size_t)c * NF * NF;
    for (int e = threadIdx.x; e < NF * NF; e += blockDim.x) Ss[e] = Sc[e];
    for (int e = threadIdx.x; e < NL * NB; e += blockDim.x) {
      const int lf = e / NB, w = e - lf * NB, r = w / NFD, q = w - r * NFD;
      const int ent = cell_blk[(size_t)c * NL + lf];
      Ws[e] = ent >= 0 ? (float)W[(size_t)(ent >> 1) * NB + w] : (r == q ? 1.0f : 0.0f);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NBLK * NB; e += blockDim.x) {
      const int blk = e / NB, w = e - blk * NB, p = w / NFD, q = w - p * NFD;
      const int i = blo[blk] * NFD + p, j = bhi[blk] * NFD + q;
      Ts[e] = (float)(0.5 * sign * (Ss[i + NF * j] + Ss[j + NF * i]));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NBLK * NB; e += blockDim.x) {
      const int blk = e / NB, w = e - blk * NB, p = w / NFD, sc = w - p * NFD;
      const float *Wh = Ws + bhi[blk] * NB + sc * NFD;
      const float *T = Ts + blk * NB + p * NFD;
      float u = 0.0f;
      for (int q = 0; q <= sc; ++q) u = fmaf(T[q], Wh[q], u);
      Us[e] = u;
    }
    __syncthreads();
    float *o = out + (size_t)c * rec;
    constexpr int BS = cellop_bstride(NFD);
    for (int e = threadIdx.x; e < rec; e += blockDim.x) {
      float v = 0.0f;
      const int blk = e / BS, w = e - blk * BS;
      if (blk < NBLK && w < NB) {  // else: padding
        const int r = w / NFD, sc = w - r * NFD;
        const float *Wl = Ws + blo[blk] * NB + r * NFD;
        const float *U = Us + blk * NB + sc;
        for (int p = 0; p <= r; ++p) v = fmaf(Wl[p], U[p * NFD], v);
      }
      o[e] = v;
    }
    __syncthreads();
  }
}

// The same records for large cells (the whole S_c does not fit a CTA's
// shared memory): one CTA per cell, the cell's nl facet factors W staged once
// in FP32, then its upper blocks one after the other, each block and its
// transposed partner staged as two nfd x nfd FP64 tiles.
__global__ void pack_cell_blocks_tiled_kernel(int ncells, int nl, int nfd, int rec, double sign,
                                              const double *__restrict__ S, const int *__restrict__ cell_blk,
                                              const double *__restrict__ W, float *__restrict__ out) {
  extern __shared__ double T[];  // 2 nb doubles, then (nl + 2) nb floats
  const int nf = nl * nfd, nb = nfd * nfd, nblk = cellop_blocks(nl);
  double *T1 = T, *T2 = T + nb;
  float *Ws = reinterpret_cast<float *>(T + 2 * nb), *U = Ws + (size_t)nl * nb, *Ts = U + nb;
  for (int c = blockIdx.x; c < ncells; c += gridDim.x) {
    const double *Sc = S + (size_t)c * nf * nf;
    for (int e = threadIdx.x; e < nl * nb; e += blockDim.x) {
      const int lf = e / nb, w = e - lf * nb, wr = w / nfd, wc = w - wr * nfd;  // row-major W index
      const int ent = cell_blk[(size_t)c * nl + lf];
      Ws[e] = ent >= 0 ? (float)W[(size_t)(ent >> 1) * nb + w] : (wr == wc ? 1.0f : 0.0f);
    }
    for (int blk = 0; blk < nblk; ++blk) {
      int lo, hi;
      upper_block(nl, blk, lo, hi);
      // T1[r + nfd s] = S(lo nfd + r, hi nfd + s), T2[r + nfd s] = S(hi nfd + r, lo nfd + s)
      for (int e = threadIdx.x; e < nb; e += blockDim.x) {
        const int sc = e / nfd, r = e - sc * nfd;
        T1[e] = Sc[(size_t)(lo * nfd + r) + (size_t)nf * (hi * nfd + sc)];
        T2[e] = Sc[(size_t)(hi * nfd + r) + (size_t)nf * (lo * nfd + sc)];
      }
      __syncthreads();
      // Ts[p][q] = sign (S(lo p, hi q) + S(hi q, lo p))/2, one FP64 sum per entry
      for (int e = threadIdx.x; e < nb; e += blockDim.x) {
        const int p = e / nfd, q = e - p * nfd;
        Ts[e] = (float)(0.5 * sign * (T1[p + nfd * q] + T2[q + nfd * p]));
      }
      __syncthreads();
      // U[p][s] = sum_{q <= s} Ts[p][q] W_hi[s][q]
      const float *Wh = Ws + (size_t)hi * nb, *Wl = Ws + (size_t)lo * nb;
      for (int e = threadIdx.x; e < nb; e += blockDim.x) {
        const int p = e / nfd, sc = e - p * nfd;
        float u = 0.0f;
        for (int q = 0; q <= sc; ++q) u = fmaf(Ts[p * nfd + q], Wh[sc * nfd + q], u);
        U[e] = u;
      }
      __syncthreads();
      float *o = out + (size_t)c * rec + (size_t)blk * cellop_bstride(nfd);
      for (int w = nb + threadIdx.x; w < cellop_bstride(nfd); w += blockDim.x) o[w] = 0.0f;  // padding
      for (int w = threadIdx.x; w < nb; w += blockDim.x) {
        const int r = w / nfd, sc = w - r * nfd;
        float v = 0.0f;
        for (int p = 0; p <= r; ++p) v = fmaf(Wl[r * nfd + p], U[p * nfd + sc], v);
        o[w] = v;
      }
    }
    for (int e = nblk * cellop_bstride(nfd) + threadIdx.x; e < rec; e += blockDim.x)
      out[(size_t)c * rec + e] = 0.0f;  // padding
    __syncthreads();
  }
}

// Large cells with the block size at compile time: one CTA per cell, the
// symmetric part of every upper block staged in FP32 (21 blocks of 27 x 27
// for 3D elasticity k = 2: 61 KB) with the cell's facet factors W, then
// U = T W_hi^T in place row by row (a thread keeps its row of T in registers)
// and the record W_lo U column by column, all blocks at once: two barriers
// per cell.
template <int NL, int NFD>
__global__ void __launch_bounds__(256) pack_cell_blocks_large_t(int ncells, int rec, double sign,
                                                                const double *__restrict__ S,
                                                                const int *__restrict__ cell_blk,
                                                                const double *__restrict__ W, float *__restrict__ out) {
  constexpr int NF = NL * NFD, NB = NFD * NFD, NBLK = cellop_blocks(NL), BS = cellop_bstride(NFD);
  extern __shared__ float smx[];
  float *Ts = smx, *Ws = smx + NBLK * NB;
  __shared__ unsigned char blo[NBLK], bhi[NBLK];
  if (threadIdx.x < NBLK) {
    int lo, hi;
    upper_block(NL, threadIdx.x, lo, hi);
    blo[threadIdx.x] = (unsigned char)lo;
    bhi[threadIdx.x] = (unsigned char)hi;
  }
  for (int c = blockIdx.x; c < ncells; c += gridDim.x) {
    const double *Sc = S + (size_t)c * NF * NF;
    for (int e = threadIdx.x; e < NL * NB; e += blockDim.x) {
      const int lf = e / NB, w = e - lf * NB, wr = w / NFD, wc = w - wr * NFD;  // row-major W index
      const int ent = cell_blk[(size_t)c * NL + lf];
      Ws[e] = ent >= 0 ? (float)W[(size_t)(ent >> 1) * NB + w] : (wr == wc ? 1.0f : 0.0f);
    }
    __syncthreads();  // blo / bhi on the first cell
    // T[blk][p][q] = sign (S(lo p, hi q) + S(hi q, lo p)) / 2, p fastest (the
    // first read coalesced); eight entries per thread in flight at a time
    constexpr int UNR = 8;
    for (int e0 = threadIdx.x; e0 < NBLK * NB; e0 += UNR * blockDim.x) {
      double a[UNR], b[UNR];
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        const int e = e0 + u * blockDim.x;
        a[u] = b[u] = 0.0;
        if (e < NBLK * NB) {
          const int blk = e / NB, w = e - blk * NB, q = w / NFD, p = w - q * NFD;
          const int i = blo[blk] * NFD + p, j = bhi[blk] * NFD + q;
          a[u] = __ldcs(Sc + i + (size_t)NF * j);
          b[u] = __ldcs(Sc + j + (size_t)NF * i);
        }
      }
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        const int e = e0 + u * blockDim.x;
        if (e < NBLK * NB) {
          const int blk = e / NB, w = e - blk * NB, q = w / NFD, p = w - q * NFD;
          Ts[blk * NB + p * NFD + q] = (float)(0.5 * sign * (a[u] + b[u]));
        }
      }
    }
    __syncthreads();
    // U[blk][p][s] = sum_{q <= s} T[blk][p][q] W_hi[s][q], in place
    for (int it = threadIdx.x; it < NBLK * NFD; it += blockDim.x) {
      const int blk = it / NFD, p = it - blk * NFD;
      float *row = Ts + blk * NB + p * NFD;
      const float *Wh = Ws + bhi[blk] * NB;
      float t[NFD];
#pragma unroll
      for (int q = 0; q < NFD; ++q) t[q] = row[q];
#pragma unroll
      for (int sc = 0; sc < NFD; ++sc) {
        float u = 0.0f;
#pragma unroll
        for (int q = 0; q <= sc; ++q) u = fmaf(t[q], Wh[sc * NFD + q], u);
        row[sc] = u;
      }
    }
    __syncthreads();
    // record[blk][r][s] = sum_{p <= r} W_lo[r][p] U[blk][p][s]
    float *o = out + (size_t)c * rec;
    for (int it = threadIdx.x; it < NBLK * NFD; it += blockDim.x) {
      const int blk = it / NFD, sc = it - blk * NFD;
      const float *col = Ts + blk * NB + sc;
      const float *Wl = Ws + blo[blk] * NB;
      float u[NFD];
#pragma unroll
      for (int p = 0; p < NFD; ++p) u[p] = col[p * NFD];
#pragma unroll
      for (int r = 0; r < NFD; ++r) {
        float v = 0.0f;
#pragma unroll
        for (int p = 0; p <= r; ++p) v = fmaf(Wl[r * NFD + p], u[p], v);
        o[blk * BS + r * NFD + sc] = v;
      }
    }
    for (int e = threadIdx.x; e < rec; e += blockDim.x) {  // padding between and after the blocks
      const int blk = e / BS, w = e - blk * BS;
      if (blk >= NBLK || w >= NB) o[e] = 0.0f;
    }
    __syncthreads();  // Ts and Ws are read above until here
  }
}

constexpr int kMaxBulkStages = 8;

template <int NL, int NFD>
struct CellOp {
  static constexpr int NF = NL * NFD;
  static constexpr int TPC = cellop_tpc(NF);
  static constexpr int CPS = cellop_cps(NF);
  static constexpr int THREADS = CPS * TPC;
  static constexpr int REC = cellop_rec(NL, NFD);
};

// p_new = z + beta p_old (formed while gathering, stored by the owning cell);
// qc_c = M_c p_c for every cell without the diagonal blocks (whose sum over a
// facet's cells is the identity); alpha = (r,z) / ((p, p) + sum_c (p_c, qc_c)).
// Persistent CTAs take stages of CPS consecutive cells round-robin; thread 0
// keeps `nstage` stages of cell records in flight with bulk copies (L2
// evict-first: the records are read once per iteration, the vectors stay).
// One CTA barrier per stage: the gathered p alternates between two buffers by
// stage parity, and the ring slot of stage t-1 is refilled once every thread
// has passed stage t's barrier (a second barrier at the end of each stage
// cost 40.7 against 39.1 us per launch at 32^3).
template <int NL, int NFD>
__global__ void __launch_bounds__(CellOp<NL, NFD>::THREADS, 2)
    cell_spmv32_kernel(Pcg32Args a, const float *__restrict__ p_old, float *__restrict__ p_new) {
  using C = CellOp<NL, NFD>;
  extern __shared__ __align__(128) float ring[];
  __shared__ __align__(8) uint64_t bars[kMaxBulkStages];
  __shared__ __align__(16) float ps2[2][C::CPS][C::TPC];  // by stage parity: one CTA barrier per stage
  __shared__ float2 redf[32];
  __shared__ int abort_flag;
  if (a.scal[SC_DONE] != 0.0) return;
  const float beta = (float)a.scal[SC_BETA];
  const int g = threadIdx.x / C::TPC, i = threadIdx.x - g * C::TPC;
  const int lf = i / NFD, r = i - lf * NFD;
  const int nunits = (a.ncells + C::CPS - 1) / C::CPS;
  const int mine = (int)blockIdx.x < nunits ? (nunits - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const int nstage = a.nstage;
  uint64_t pol = 0;
  int issued = 0;  // meaningful in thread 0
  auto issue = [&](int t) {
    const int c0 = ((int)blockIdx.x + t * (int)gridDim.x) * C::CPS;
    const int nc = min(C::CPS, a.ncells - c0);
    const uint32_t bytes = (uint32_t)nc * C::REC * 4u;
    const int slot = t % nstage;
    mbar_arrive_expect_tx(&bars[slot], bytes);
    bulk_copy_g2s(ring + (size_t)slot * C::CPS * C::REC, a.blocks + (size_t)c0 * C::REC, bytes, &bars[slot], pol);
  };
  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < nstage; ++s) mbar_init(&bars[s], 1);
    mbar_init_fence();
    pol = l2_evict_first_policy();
    for (; issued < min(nstage, mine); ++issued) issue(issued);
  }
  __syncthreads();
  FFSum acc;  // (p, qc) over this thread's rows, float-float
  // The gather of p = z + beta p_old is pipelined across stages: the block-row
  // entry of stage t+2 and the p_old / z values of stage t+1 are loaded while
  // stage t is computed (two dependent loads, each hidden behind one stage).
  auto load_ent = [&](int tt) -> int {
    const int cc = ((int)blockIdx.x + tt * (int)gridDim.x) * C::CPS + g;
    return (tt < mine && i < C::NF && cc < a.ncells) ? a.cell_blk[(size_t)cc * NL + lf] : -1;
  };
  int ent_a = load_ent(0), ent_b = load_ent(1);
  float po_a = 0.0f, z_a = 0.0f;
  if (ent_a >= 0) {
    const int row = (ent_a >> 1) * NFD + r;
    po_a = p_old[row];
    z_a = a.z[row];
  }
  for (int t = 0; t < mine; ++t) {
    const int slot = t % nstage;
    const int c = ((int)blockIdx.x + t * (int)gridDim.x) * C::CPS + g;
    const bool act = i < C::NF && c < a.ncells;
    const int ent = ent_a;  // this stage's block-row entry (ent_a moves on below)
    float pv = 0.0f;
    if (ent_a >= 0) {
      pv = fmaf(beta, po_a, z_a);
      if (ent_a & 1) {
        p_new[(ent_a >> 1) * NFD + r] = pv;
        acc.add_prod(pv, pv);  // (p, I p) over the facet's diagonal block, once per row
      }
    }
    // stage t+1's values, stage t+2's entry
    ent_a = ent_b;
    if (ent_a >= 0) {
      const int row = (ent_a >> 1) * NFD + r;
      po_a = p_old[row];
      z_a = a.z[row];
    }
    ent_b = load_ent(t + 2);
    float (*ps)[C::TPC] = ps2[t & 1];
    ps[g][i] = pv;
    if (!mbar_wait_bounded(&bars[slot], (uint32_t)(t / nstage) & 1u)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) {
      // a copy never landed: record it, give the copies in flight a bounded
      // chance to finish (they target this CTA's shared memory) and stop
      if (threadIdx.x == 0) {
        atomicExch(a.error, 1u);
        for (int u = t; u < issued; ++u) mbar_wait_bounded(&bars[u % nstage], (uint32_t)(u / nstage) & 1u);
      }
      return;
    }
    // every thread is past stage t-1: its ring slot can be refilled
    if (threadIdx.x == 0 && t >= 1 && issued < mine) {
      async_proxy_fence();
      issue(issued);
      ++issued;
    }
    if (act) {
      const float *B = ring + (size_t)slot * C::CPS * C::REC + (size_t)g * C::REC;
      float q = 0.0f;
      if constexpr (C::NF <= 64) {
        // the cell's p in registers (vector loads), so the inner loop only reads B
        constexpr int NV = (C::NF + 3) / 4;
        float pr[4 * NV];
        const float4 *p4 = reinterpret_cast<const float4 *>(&ps[g][0]);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const float4 t4 = p4[v];
          pr[4 * v] = t4.x;
          pr[4 * v + 1] = t4.y;
          pr[4 * v + 2] = t4.z;
          pr[4 * v + 3] = t4.w;
        }
        // one partial sum per facet block (independent FMA chains), added in block order
        float qb[NL];
#pragma unroll
        for (int b = 0; b < NL; ++b) {
          // block (lf, b) is stored for b > lf; below the diagonal read (b, lf)
          // transposed; the diagonal block's part is p itself (the update adds it)
          qb[b] = 0.0f;
          if (b == lf) continue;
          const bool up = b > lf;
          const int lo = up ? lf : b, hi = up ? b : lf;
          const float *Bb = B + offdiag_block<NL>(lo, hi) * cellop_bstride(NFD) + (up ? r * NFD : r);
          const int st = up ? 1 : NFD;
#pragma unroll
          for (int s = 0; s < NFD; ++s) qb[b] = fmaf(Bb[s * st], pr[b * NFD + s], qb[b]);
        }
#pragma unroll
        for (int b = 0; b < NL; ++b) q += qb[b];
      } else {
#pragma unroll
        for (int b = 0; b < NL; ++b) {
          if (b == lf) continue;
          const bool up = b > lf;
          const int lo = up ? lf : b, hi = up ? b : lf;
          const float *Bb = B + offdiag_block<NL>(lo, hi) * cellop_bstride(NFD) + (up ? r * NFD : r);
          const int st = up ? 1 : NFD;
#pragma unroll
          for (int s = 0; s < NFD; ++s) q = fmaf(Bb[s * st], ps[g][b * NFD + s], q);
        }
      }
      // by block row: the owner's product first, then the other cell's
      if (ent >= 0) a.qc[(size_t)(ent >> 1) * (2 * NFD) + ((ent & 1) ? 0 : NFD) + r] = q;
      acc.add_prod(pv, q);
    }
  }
  // this CTA's part of (p, A p); the update kernel's CTAs sum the parts
  // themselves (no last-CTA step at the end of this launch)
  const float2 tsum = block_sum_ff(acc.hi, acc.lo, redf);
  if (threadIdx.x == 0) store_partial_ff(a.partials, (int)gridDim.x, 0, tsum);
}

// alpha = (r, z) / (p, A p), every CTA summing the SpMV's per-CTA parts in
// index order (the same value in all of them) while its first rows load;
// q = qc(owner) + qc(other) + p per free row (p: the identity diagonal
// block); x += alpha p; r -= alpha q; z = r (the preconditioner is in the
// scaled records); beta; convergence against eta |rhs|.  Every load of a row
// is independent of the others (the products sit by block row), so a row
// costs one memory round trip; rows are spread over the grid (a.uctas CTAs:
// about eight rows per thread) with a grid-stride loop.  This kernel's own
// parts go after the SpMV's (a.ctas of them), which other CTAs may still be
// reading.
static_assert(kPcgThreads == kPcgThreadsHost, "host and device PCG block sizes differ");
static_assert(kMaxRowLen == kMaxSkeletonRowLen, "host and device skeleton row limits differ");
static_assert(kRowBlocks == kSkeletonRowBlocks, "host and device skeleton row limits differ");

template <int NFD>
__global__ void __launch_bounds__(kPcgThreads) pcg32_update_rows_kernel(Pcg32Args a, const float *__restrict__ p) {
  __shared__ float2 redf[32];
  __shared__ float s_alpha;
  if (a.scal[SC_DONE] != 0.0) return;
  const float *__restrict__ qc = a.qc;
  float *__restrict__ xg = a.x;
  float *__restrict__ rg = a.r;
  FFSum rr;  // float-float: no FP64 in the per-row or per-CTA sums
  const int stride = gridDim.x * blockDim.x;
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  // four rows at a time, every load issued before the first product: each
  // row is one L2 round trip, so a thread keeps four in flight
  float q0[4], q1[4], pv[4], xv[4], r0[4];
  auto load4 = [&](int rb) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int rw = rb + u * stride;
      if (rw < a.n) {
        const int br = rw / NFD, i = rw - br * NFD;
        const float *qb = qc + (size_t)br * (2 * NFD) + i;
        q0[u] = qb[0];
        q1[u] = qb[NFD];
        pv[u] = p[rw];
        xv[u] = xg[rw];
        r0[u] = rg[rw];
      }
    }
  };
  auto update4 = [&](int rb, float alpha) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int rw = rb + u * stride;
      if (rw < a.n) {
        xg[rw] = fmaf(alpha, pv[u], xv[u]);
        const float rv = fmaf(-alpha, (q0[u] + q1[u]) + pv[u], r0[u]);
        rg[rw] = rv;
        rr.add_prod(rv, rv);
      }
    }
  };
  load4(row);
  const double pap = sum_partials_ff(a.partials, a.ctas, 0, redf);  // valid in thread 0
  if (threadIdx.x == 0) s_alpha = (float)(a.scal[SC_RZ] / pap);
  __syncthreads();
  const float alpha = s_alpha;
  update4(row, alpha);
  for (row += 4 * stride; row + 3 * stride < a.n; row += 4 * stride) {
    load4(row);
    update4(row, alpha);
  }
  for (; row < a.n; row += stride) {
    const int br = row / NFD, i = row - br * NFD;
    const float *qb = qc + (size_t)br * (2 * NFD) + i;
    const float q0s = qb[0], q1s = qb[NFD];
    const float pvs = p[row], xvs = xg[row], r0s = rg[row];
    xg[row] = fmaf(alpha, pvs, xvs);
    const float rv = fmaf(-alpha, (q0s + q1s) + pvs, r0s);
    rg[row] = rv;
    rr.add_prod(rv, rv);
  }
  const int np = (int)gridDim.x;
  const float2 s = block_sum_ff(rr.hi, rr.lo, redf);
  if (threadIdx.x == 0) store_partial_ff(a.partials + a.ctas, np, 0, s);
  if (last_cta(a.counter)) {
    const double vrr = sum_partials_ff(a.partials + a.ctas, np, 0, redf);
    if (threadIdx.x == 0) {
      a.scal[SC_PAP] = pap;
      a.scal[SC_ALPHA] = a.scal[SC_RZ] / pap;
      a.scal[SC_BETA] = vrr / a.scal[SC_RZ];
      a.scal[SC_RZ] = vrr;
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

// x += W^T y: the inner correction y back from the scaled frame (W lower
// triangular per facet block: row i of W^T is column i of W, entries j >= i)
__global__ void outer_axpy_scaled_kernel(int n, int nfd, const double *__restrict__ W, const float *__restrict__ y,
                                         double *x) {
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
    const int br = row / nfd, i = row - br * nfd;
    const double *Wb = W + (size_t)br * nfd * nfd;
    const float *yb = y + (size_t)br * nfd;
    double e = 0.0;
    for (int j = i; j < nfd; ++j) e = fma(Wb[j * nfd + i], (double)yb[j], e);
    x[row] += e;
  }
}

__global__ void outer_combine_kernel(int n, const double *__restrict__ xs, double sign, double *x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = xs[i] + sign * x[i];
}

// r = c - M x with the FP64 matrix, a lane pair per row over tiles of whole
// block rows (x staged per block row), |r|^2
template <int NFD>
__global__ void __launch_bounds__(kPcgThreads) outer_residual_kernel(OuterArgs a) {
  using T = RowTile<NFD>;
  __shared__ double red[32];
  __shared__ double xs[T::BR * T::LMAX];
  const double *__restrict__ x = a.x;
  double acc = 0.0;
  for (int br0 = blockIdx.x * T::BR; br0 < a.nblockrows; br0 += gridDim.x * T::BR) {
    const int nbr = min(T::BR, a.nblockrows - br0);
    stage_tile_columns<NFD>(a.rowptr, a.colind, br0, nbr, xs, [&](int col) { return x[col]; });
    __syncthreads();
    tile_row_products<NFD>(a.rowptr, a.val, br0, nbr, xs, [&](int row, int, double t) {
      const double r = a.sign * a.rhs[row] - a.sign * t;
      a.r[row] = r;
      acc += r * r;
    });
    __syncthreads();  // xs is restaged for the next tile
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
  if (last_cta(a.counter)) {
    const double v = sum_partials(a.partials, (int)gridDim.x, 0, red);
    if (threadIdx.x == 0) {
      a.scal[1] = v;
      *a.counter = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
cudaError_t launch_block_chol_inv(const PcgArgs &a, double *W, cudaStream_t s, int num_sms, long long *launches) {
  // the not-positive-definite flag after the last block starts at zero
  cudaError_t e = cudaMemsetAsync(W + (size_t)a.nblockrows * a.nfd * a.nfd, 0, sizeof(double), s);
  if (e != cudaSuccess || a.nblockrows < 1) return e;
  switch (a.nfd) {
#define HDG_CHOL_CASE(N)                                    \
  case N: {                                                 \
    constexpr int G = 32 / N;                               \
    const long long warps = (a.nblockrows + G - 1) / G;     \
    long long g = (warps + 3) / 4;                          \
    if (g > num_sms * 16) g = num_sms * 16;                 \
    block_chol_inv_kernel<N><<<(int)g, 128, 0, s>>>(a, W);  \
    break;                                                  \
  }
    HDG_CHOL_CASE(1)
    HDG_CHOL_CASE(2)
    HDG_CHOL_CASE(3)
    HDG_CHOL_CASE(4)
    HDG_CHOL_CASE(5)
    HDG_CHOL_CASE(6)
    HDG_CHOL_CASE(8)
    HDG_CHOL_CASE(9)
    HDG_CHOL_CASE(10)
    HDG_CHOL_CASE(12)
    HDG_CHOL_CASE(16)
    HDG_CHOL_CASE(25)
    HDG_CHOL_CASE(27)
#undef HDG_CHOL_CASE
    default:
      return cudaErrorInvalidValue;
  }
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_pcg32_init(const Pcg32Args &a, double eta, cudaStream_t s, long long *launches) {
  pcg32_init_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a, eta);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_pcg32_replace(const Pcg32Args &a, double eta, cudaStream_t s, long long *launches) {
  pcg32_replace_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a, eta);
  ++*launches;
  return cudaGetLastError();
}

template <int NL, int NFD>
static size_t cellop_dyn_smem(int nstage) {
  using C = CellOp<NL, NFD>;
  return (size_t)nstage * C::CPS * C::REC * sizeof(float);
}

#define HDG_CELLOP_CASES(X) \
  X(3, 1) X(3, 2) X(3, 3) X(3, 4) X(4, 10) X(4, 1) X(6, 1) X(4, 2) X(4, 3) X(4, 4) X(4, 5) X(4, 6) X(4, 8) X(6, 3) X(6, 4) X(6, 6) X(6, 9) X(6, 12) X(6, 16) X(6, 25) X(6, 27)

bool cellop_supported(int nl, int nfd) {
#define X(L, F) \
  if (nl == L && nfd == F) return true;
  HDG_CELLOP_CASES(X)
#undef X
  return false;
}

template <int NL, int NFD>
static cudaError_t cellop_configure_t(size_t smem_optin, int num_sms, int *nstage, int *ctas) {
  using C = CellOp<NL, NFD>;
  const size_t stage = (size_t)C::CPS * C::REC * sizeof(float);
  // Stages up to 32 KB (3D Darcy k=2: 4 cells, 20 KB): up to 64 KB of records
  // in flight per CTA, so three CTAs fit an SM -- more warps to hide the
  // per-stage barriers and gathers (4.90 vs 4.56 TB/s against two CTAs with
  // four stages each, measured with 27 KB stages).  Larger stages: about
  // 108 KB per CTA, two CTAs per SM where two stages each fit; otherwise (one
  // cell of 3D elasticity k=2: 43 KB) one CTA with as many stages as fit.
  int ns = (int)((stage <= 32 * 1024 ? 64 * 1024 : 110 * 1024) / stage);
  ns = ns > kMaxBulkStages ? kMaxBulkStages : ns;
  if (2 * (2 * stage + 4096) > smem_optin) ns = (int)((smem_optin - 4096) / stage);
  ns = ns > kMaxBulkStages ? kMaxBulkStages : ns;
  if (ns < 2) ns = 2;
  while (ns > 2 && (size_t)ns * stage + 4096 > smem_optin) --ns;
  if ((size_t)ns * stage + 4096 > smem_optin) return cudaErrorInvalidValue;
  const size_t dyn = cellop_dyn_smem<NL, NFD>(ns);
  cudaError_t e = cudaFuncSetAttribute(cell_spmv32_kernel<NL, NFD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cell_spmv32_kernel<NL, NFD>, C::THREADS, dyn);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidValue;
  if (per_sm > 4) per_sm = 4;
  *nstage = ns;
  *ctas = per_sm * num_sms;
  return cudaSuccess;
}

cudaError_t cellop_configure(int nl, int nfd, size_t smem_optin, int num_sms, int *nstage, int *ctas) {
#define X(L, F) \
  if (nl == L && nfd == F) return cellop_configure_t<L, F>(smem_optin, num_sms, nstage, ctas);
  HDG_CELLOP_CASES(X)
#undef X
  return cudaErrorInvalidValue;
}

cudaError_t launch_pack_cell_blocks(int ncells, int nl, int nfd, double sign, const double *S, const int *cell_blk,
                                    const double *W, float *out, size_t smem_optin, cudaStream_t s, int num_sms,
                                    long long *launches) {
  const int nf = nl * nfd, nb = nfd * nfd, nblk = cellop_blocks(nl);
  const size_t smem = sizeof(double) * nf * nf + sizeof(float) * (size_t)(nl + 2 * nblk) * nb;
  if (smem > 64 * 1024) {  // large cells
#define HDG_PACK_LARGE(L, F)                                                                                  \
  if (nl == L && nfd == F) {                                                                                  \
    const size_t lsmem = sizeof(float) * (size_t)(cellop_blocks(L) + L) * F * F;                                  \
    cudaError_t e = cudaFuncSetAttribute(pack_cell_blocks_large_t<L, F>,                                      \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsmem);             \
    if (e != cudaSuccess) return e;                                                                           \
    int per_sm = 0;                                                                                           \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pack_cell_blocks_large_t<L, F>, 256, lsmem);   \
    if (e != cudaSuccess) return e;                                                                           \
    int grid = num_sms * (per_sm > 0 ? per_sm : 1);                                                           \
    if (grid > ncells) grid = ncells;                                                                         \
    if (grid < 1) grid = 1;                                                                                   \
    pack_cell_blocks_large_t<L, F><<<grid, 256, lsmem, s>>>(ncells, cellop_rec(L, F), sign, S, cell_blk, W,  \
                                                            out);                                             \
    ++*launches;                                                                                              \
    return cudaGetLastError();                                                                                \
  }
    HDG_PACK_LARGE(6, 27)
    HDG_PACK_LARGE(6, 16)
#undef HDG_PACK_LARGE
    // other shapes: one cell per CTA, block by block
    const size_t tsmem = 2 * sizeof(double) * nb + (size_t)(nl + 2) * sizeof(float) * nb;
    if (tsmem > 48 * 1024) return cudaErrorInvalidValue;
    int grid = ncells < num_sms * 8 ? ncells : num_sms * 8;
    if (grid < 1) grid = 1;
    pack_cell_blocks_tiled_kernel<<<grid, 256, tsmem, s>>>(ncells, nl, nfd, cellop_rec(nl, nfd), sign, S,
                                                           cell_blk, W, out);
    ++*launches;
    return cudaGetLastError();
  }
  int grid = ncells < num_sms * 16 ? ncells : num_sms * 16;
  if (grid < 1) grid = 1;
  cudaError_t e = cudaErrorInvalidValue;
#define X(L, F)                                                                                              \
  if (nl == L && nfd == F) {                                                                                 \
    e = cudaFuncSetAttribute(pack_cell_blocks_t<L, F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e == cudaSuccess)                                                                                    \
      pack_cell_blocks_t<L, F><<<grid, 256, smem, s>>>(ncells, cellop_rec(L, F), sign, S, cell_blk, W, out);  \
  }
  HDG_CELLOP_CASES(X)
#undef X
  if (e == cudaErrorInvalidValue) {  // a shape without an instance: the runtime-sized kernel
    e = cudaFuncSetAttribute(pack_cell_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    pack_cell_blocks_kernel<<<grid, 256, smem, s>>>(ncells, nl, nfd, cellop_rec(nl, nfd), sign, S, cell_blk, W, out);
  } else if (e != cudaSuccess) {
    return e;
  }
  ++*launches;
  return cudaGetLastError();
}

template <int NL, int NFD>
static void cell_spmv(const Pcg32Args &a, const float *po, float *pn, cudaStream_t s) {
  cell_spmv32_kernel<NL, NFD><<<a.ctas, CellOp<NL, NFD>::THREADS, cellop_dyn_smem<NL, NFD>(a.nstage), s>>>(a, po, pn);
}

template <int NL, int NFD>
static void pcg32_pair(const Pcg32Args &a, cudaStream_t s) {
  cell_spmv<NL, NFD>(a, a.p, a.p2, s);
  pcg32_update_rows_kernel<NFD><<<a.uctas, kPcgThreads, 0, s>>>(a, a.p2);
  cell_spmv<NL, NFD>(a, a.p2, a.p, s);
  pcg32_update_rows_kernel<NFD><<<a.uctas, kPcgThreads, 0, s>>>(a, a.p);
}

cudaError_t launch_pcg32_iteration_pair(const Pcg32Args &a, cudaStream_t s, long long *launches) {
#define X(L, F)                    \
  if (a.nl == L && a.nfd == F) {   \
    pcg32_pair<L, F>(a, s);        \
    *launches += 4;                \
    return cudaGetLastError();     \
  }
  HDG_CELLOP_CASES(X)
#undef X
  return cudaErrorInvalidValue;
}

cudaError_t launch_pcg32_spmv(const Pcg32Args &a, cudaStream_t s, long long *launches) {
#define X(L, F)                    \
  if (a.nl == L && a.nfd == F) {   \
    cell_spmv<L, F>(a, a.p, a.p2, s); \
    ++*launches;                   \
    return cudaGetLastError();     \
  }
  HDG_CELLOP_CASES(X)
#undef X
  return cudaErrorInvalidValue;
}

cudaError_t launch_outer_init(const OuterArgs &a, cudaStream_t s, long long *launches) {
  outer_init_kernel<<<a.nparts, kPcgThreads, 0, s>>>(a);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_outer_combine(const OuterArgs &a, const double *xsaved, cudaStream_t s, long long *launches) {
  int g = (a.n + 255) / 256;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  outer_combine_kernel<<<g, 256, 0, s>>>(a.n, xsaved, a.sign, a.x);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_outer_update(const OuterArgs &a, const float *e, cudaStream_t s, long long *launches) {
  if (a.max_rowlen > kRowBlocks * a.nfd) return cudaErrorInvalidValue;  // the staged tile holds 11 blocks a row
  if (a.tile_ctas < 1 || a.tile_ctas > 8 * 1024) return cudaErrorInvalidValue;
  int g = (a.n + 255) / 256;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  if (a.W)
    outer_axpy_scaled_kernel<<<g, 256, 0, s>>>(a.n, a.nfd, a.W, e, a.x);
  else
    outer_axpy_kernel<<<g, 256, 0, s>>>(a.n, e, a.x);
  switch (a.nfd) {
    case 1: outer_residual_kernel<1><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 2: outer_residual_kernel<2><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 3: outer_residual_kernel<3><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 4: outer_residual_kernel<4><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 5: outer_residual_kernel<5><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 6: outer_residual_kernel<6><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 8: outer_residual_kernel<8><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 9: outer_residual_kernel<9><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 10: outer_residual_kernel<10><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 12: outer_residual_kernel<12><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 16: outer_residual_kernel<16><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 25: outer_residual_kernel<25><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    case 27: outer_residual_kernel<27><<<a.tile_ctas, kPcgThreads, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  *launches += 2;
  return cudaGetLastError();
}

}  // namespace hdg
