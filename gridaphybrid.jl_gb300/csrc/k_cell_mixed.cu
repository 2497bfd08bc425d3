// k_cell_mixed.cu -- FP32 local factorisation with high-precision refinement,
// for sm_103a.
//
// GB300 runs FP64 at ~1/74 of its FP32 rate, so "high precision" here is
// float-float arithmetic (a value is an unevaluated sum hi + lo of two FP32
// numbers, ~48 significant bits) executed on the FP32 pipes:
//  * integration produces every cell block as (A_hi, A_lo) FP32 pairs;
//  * the LU of A_ii and the solves run in plain FP32 on A_hi;
//  * one refinement step: X0 = A_ii^{-1}[A_if | b_i] (FP32), residual
//    R = [A_if | b_i] - A_ii X0 in float-float, X1 = X0 + A_ii^{-1} R (FP32
//    correction), then S = A_ff - A_fi X1 and g = b_f - A_fi y1 in
//    float-float, returned in FP64.  On 32^3 k=2 cells this brings S from
//    ~3e-7 (FP32 alone) to ~5e-13 relative;
//  * X1 (as the pair X0, delta) is kept for the recovery u = y1 - X1_f x_f.
#include <cuda_runtime.h>

#include "hdg_kernels.h"
#include "k_condense_mixed_rt.cuh"
#include "k_ff_cell.cuh"

namespace hdg {

__global__ void __launch_bounds__(256) integrate_mixed_kernel(CellArgs a, MixedTables T, float *Ahi, float *Alo,
                                                              float *bhi, float *blo, bool skip_uu) {
  __shared__ CellFactorsFF f;
  __shared__ double fq[512 * 4];
  const int n = a.n;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x)
    integrate_cell_ff(a, T, c, true, f, fq, Ahi + (size_t)c * n * n, Alo + (size_t)c * n * n, bhi + (size_t)c * n,
                      blo + (size_t)c * n, threadIdx.x, blockDim.x, skip_uu);
}

// ---------------------------------------------------------------------------
// Darcy integration for the block elimination (HDG_PREC_FF_BLOCK), sizes
// fixed at compile time.  Every entry of a cell block is a sum of at most
// D + 2D terms (cell coefficient) x (reference table value), so the entry's
// decode and its table values are the same for every cell: one thread owns an
// entry and sweeps a group of cells, reading the cells' coefficients from
// shared memory.  The flux rows' flux and pressure columns (A_uu, A_up) are
// not written: the elimination takes A_uu from (|J|/kappa) M_ref and the flux
// panel from M^{-1} G_e, and reads neither.
// ---------------------------------------------------------------------------
constexpr int kFFCoef = 34;  // float-float pairs per cell: m, cg[3][3], cn[6][3], ct[6]
constexpr int kFFCells = 64;  // cells per entry-kernel CTA

template <int D, int K>
struct DarcyShape {
  static constexpr int K1 = K + 1, NK = D == 2 ? K1 * K1 : K1 * K1 * K1, NFD = D == 2 ? K1 : K1 * K1;
  static constexpr int NL = 2 * D, NU = D * NK, NI = (D + 1) * NK, NF = NL * NFD, N = NI + NF;
  static constexpr int R0 = N - NU;              // rows written in a column j < NI
  static constexpr int NE = NI * R0 + NF * N;    // entries written per cell
};

// per cell: the coefficients of cell_entry_ff as float-float pairs, slots
// [0] m = |det J|/kappa, [1 + 3e + d] cg[e][d], [10 + 3lf + d] cn[lf][d], [28 + lf] ct[lf]
__global__ void ff_cell_coef_kernel(CellArgs a, float2 *coef, double *detj) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.ncells; c += gridDim.x * blockDim.x) {
    CellFactorsFF f{};
    cell_factors_ff(a, c, f);
    float2 *o = coef + (size_t)c * kFFCoef;
    detj[c] = f.detJ;
    o[0] = make_float2(f.cm[0], f.cm[1]);
    for (int e = 0; e < 3; ++e)
      for (int d = 0; d < 3; ++d) o[1 + 3 * e + d] = make_float2(f.cg[e][d][0], f.cg[e][d][1]);
    for (int lf = 0; lf < 6; ++lf) {
      for (int d = 0; d < 3; ++d) o[10 + 3 * lf + d] = make_float2(f.cn[lf][d][0], f.cn[lf][d][1]);
      o[28 + lf] = make_float2(f.ct[lf][0], f.ct[lf][1]);
    }
  }
}

// entry = sum over the kept terms t (bit t of keep) of coef[slot_t] *
// (th_t + tl_t) over the group's cells, in the term order of cell_entry_ff;
// wkeep (the warp's union of keep) skips the terms no lane keeps
template <int NT, size_t CS>
__device__ __forceinline__ void ff_entry_cells(const float2 *cs, int ncg, unsigned keep, unsigned wkeep,
                                               const int *sl, const float *th, const float *tl, float *ah,
                                               float *al) {
#pragma unroll 4
  for (int cl = 0; cl < ncg; ++cl) {
    const float2 *cf = cs + cl * kFFCoef;
    float h = 0.0f, l = 0.0f;
#pragma unroll
    for (int t = 0; t < NT; ++t)
      if ((wkeep >> t) & 1u)
        if ((keep >> t) & 1u) {
          const float2 v = cf[sl[t]];
          ff_mac2(h, l, th[t], tl[t], v.x, v.y);
        }
    float s, e;
    two_sum(h, l, s, e);
    ah[(size_t)cl * CS] = s;
    al[(size_t)cl * CS] = e;
  }
}

// axis: every cell's Jacobian is diagonal, so cg[e][d] = 0 for e != d and
// cn[lf][d] = 0 unless d is the axis normal to facet lf; those terms (and
// terms whose table value is zero) are skipped -- they add exact zeros, as
// cell_entry_ff's zero-coefficient test does.  Four CTAs per SM (64
// registers): the kernel is issue-bound, and the extra warps took the 32^3
// integrate phase from 2.51 to 2.44 ms.
template <int D, int K>
__global__ void __launch_bounds__(256, 4) integrate_ffentries_kernel(int ncells, MixedTables T, bool axis,
                                                                  const float2 *__restrict__ coef, float *Ahi,
                                                                  float *Alo) {
  using S = DarcyShape<D, K>;
  constexpr int N = S::N, NK = S::NK, NFD = S::NFD, NU = S::NU, NI = S::NI, NL = S::NL, R0 = S::R0;
  constexpr size_t CS = (size_t)N * N;
  __shared__ float2 cs[kFFCells * kFFCoef];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = e < S::NE;
  int i = 0, j = 0;
  if (active) {
    if (e < NI * R0) {
      j = e / R0;
      i = NU + (e - j * R0);
    } else {
      const int r = e - NI * R0, jf = r / N;
      j = NI + jf;
      i = r - jf * N;
    }
  }
  // row / column types: 0 flux (component s, node x), 1 pressure (node x), 2 facet (s, node x)
  const int ti = i < NU ? 0 : (i < NI ? 1 : 2), tj = j < NU ? 0 : (j < NI ? 1 : 2);
  const int si = ti == 0 ? i / NK : (ti == 2 ? (i - NI) / NFD : 0);
  const int ii = ti == 0 ? i - si * NK : (ti == 1 ? i - NU : i - NI - si * NFD);
  const int sj = tj == 0 ? j / NK : (tj == 2 ? (j - NI) / NFD : 0);
  const int jj = tj == 0 ? j - sj * NK : (tj == 1 ? j - NU : j - NI - sj * NFD);
  auto normal_axis = [](int lf) { return D - 1 - lf / 2; };
  constexpr int NTM = D + NL;
  int sl[NTM];
  float th[NTM], tl[NTM];
  bool keep[NTM];
#pragma unroll
  for (int t = 0; t < NTM; ++t) {
    sl[t] = 0;
    th[t] = 0.0f;
    tl[t] = 0.0f;
    keep[t] = false;
  }
  if (active) {
    int k = -1, slot = 0;
    const float *Th = nullptr, *Tl = nullptr;
    bool neg = false, zc = false;
    if (ti == 1 && tj == 0) {  // G terms, then F terms
#pragma unroll
      for (int t = 0; t < D; ++t) {
        sl[t] = 1 + 3 * t + sj;
        th[t] = __ldg(T.Gh + (t * NK + ii) * NK + jj);
        tl[t] = __ldg(T.Gl + (t * NK + ii) * NK + jj);
        keep[t] = !(axis && t != sj);
      }
#pragma unroll
      for (int lf = 0; lf < NL; ++lf) {
        sl[D + lf] = 10 + 3 * lf + sj;
        th[D + lf] = __ldg(T.Fh + (lf * NK + ii) * NK + jj);
        tl[D + lf] = __ldg(T.Fl + (lf * NK + ii) * NK + jj);
        keep[D + lf] = !(axis && normal_axis(lf) != sj);
      }
    } else if (ti == 1 && tj == 1) {
#pragma unroll
      for (int lf = 0; lf < NL; ++lf) {
        sl[lf] = 28 + lf;
        th[lf] = __ldg(T.Fh + (lf * NK + ii) * NK + jj);
        tl[lf] = __ldg(T.Fl + (lf * NK + ii) * NK + jj);
        keep[lf] = true;
      }
    } else if (ti == 0) {  // tj == 2
      slot = 10 + 3 * sj + si, Th = T.Hh, Tl = T.Hl, k = (sj * NK + ii) * NFD + jj;
      zc = axis && normal_axis(sj) != si;
    } else if (ti == 1) {  // tj == 2
      slot = 28 + sj, Th = T.Hh, Tl = T.Hl, k = (sj * NK + ii) * NFD + jj, neg = true;
    } else if (tj == 0) {
      slot = 10 + 3 * si + sj, Th = T.Hh, Tl = T.Hl, k = (si * NK + jj) * NFD + ii;
      zc = axis && normal_axis(si) != sj;
    } else if (tj == 1) {
      slot = 28 + si, Th = T.Hh, Tl = T.Hl, k = (si * NK + jj) * NFD + ii;
    } else if (si == sj) {
      slot = 28 + si, Th = T.Lh, Tl = T.Ll, k = ii * NFD + jj, neg = true;
    }
    if (k >= 0 && !zc) {
      const float h = __ldg(Th + k), l = __ldg(Tl + k);
      sl[0] = slot;
      th[0] = neg ? -h : h;
      tl[0] = neg ? -l : l;
      keep[0] = true;
    }
  }
  unsigned km = 0;
#pragma unroll
  for (int t = 0; t < NTM; ++t)
    if (keep[t] && (th[t] != 0.0f || tl[t] != 0.0f)) km |= 1u << t;
  const unsigned wkm = __reduce_or_sync(0xffffffffu, km);
  const int ngroups = (ncells + kFFCells - 1) / kFFCells;
  for (int grp = blockIdx.y; grp < ngroups; grp += gridDim.y) {
    const int c0 = grp * kFFCells, ncg = min(kFFCells, ncells - c0);
    __syncthreads();
    for (int o = threadIdx.x; o < ncg * kFFCoef; o += blockDim.x) cs[o] = coef[(size_t)c0 * kFFCoef + o];
    __syncthreads();
    if (!active) continue;
    float *ah = Ahi + (size_t)c0 * CS + (size_t)j * N + i, *al = Alo + (size_t)c0 * CS + (size_t)j * N + i;
    if (wkm == 0)
      for (int cl = 0; cl < ncg; ++cl) {
        ah[(size_t)cl * CS] = 0.0f;
        al[(size_t)cl * CS] = 0.0f;
      }
    else if (wkm == 1u)  // single-term entries (the facet couplings): no per-term tests
      ff_entry_cells<1, CS>(cs, ncg, km, wkm, sl, th, tl, ah, al);
    else
      ff_entry_cells<NTM, CS>(cs, ncg, km, wkm, sl, th, tl, ah, al);
  }
}

// b = [int f_u . v ; int g w ; 0] per cell: one warp per cell, in FP64 and
// in the operation order of integrate_cell_ff (the batched assembly gives
// the same bits).  |det J| comes from ff_cell_coef_kernel.
template <int D, int K>
__global__ void __launch_bounds__(256) ff_cell_rhs_kernel(CellArgs a, const double *__restrict__ detj, float *bhi,
                                                          float *blo) {
  using S = DarcyShape<D, K>;
  constexpr int NK = S::NK, NU = S::NU, NI = S::NI, N = S::N, NW = 8;
  extern __shared__ double rs[];
  const int nq = a.nqv, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *phi = rs, *fq = phi + nq * NK + warp * nq * (D + 1);
  for (int o = threadIdx.x; o < nq * NK; o += blockDim.x) phi[o] = a.qphi[o];
  __syncthreads();
  for (int c = blockIdx.x * NW + warp; c < a.ncells; c += gridDim.x * NW) {
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, x0[3] = {0, 0, 0};
    for (int col = 0; col < D; ++col) {
      x0[col] = a.origin[(size_t)c * D + col];
      for (int row = 0; row < D; ++row) J[row][col] = a.jac[(size_t)c * D * D + col * D + row];
    }
    const double adet = detj[c], kap = a.kappa ? a.kappa[c] : 1.0;
    for (int q = lane; q < nq; q += 32) {
      double x[3], p, qe[3], fu[3], g;
      for (int d = 0; d < D; ++d) {
        x[d] = x0[d];
        for (int e = 0; e < D; ++e) x[d] += J[d][e] * a.qxi[q * D + e];
      }
      exact_solution(a.problem, D, x, kap, p, qe, fu, g);
      const double w = a.qw[q] * adet;
      for (int d = 0; d < D; ++d) fq[q * (D + 1) + d] = w * fu[d];
      fq[q * (D + 1) + D] = w * g;
    }
    __syncwarp();
    // the source components that vanish at every quadrature point (the flux
    // source of the manufactured problems): their rows are +0 without the
    // DFMA loop, the same bits the loop gives (a sum of zero products from +0)
    unsigned live = 0u;
    for (int q = lane; q < nq; q += 32)
      for (int d = 0; d <= D; ++d)
        if (fq[q * (D + 1) + d] != 0.0) live |= 1u << d;
    live = __reduce_or_sync(0xffffffffu, live);
    for (int i = lane; i < N; i += 32) {
      double v = 0.0;
      if (i < NI) {
        const int comp = i < NU ? i / NK : D, ii = i < NU ? i - comp * NK : i - NU;
        if (live >> comp & 1u)
          for (int q = 0; q < nq; ++q) v += fq[q * (D + 1) + comp] * phi[q * NK + ii];
      }
      float h, l;
      split_double(v, h, l);
      bhi[(size_t)c * N + i] = h;
      blo[(size_t)c * N + i] = l;
    }
    __syncwarp();
  }
}

template <int D, int K>
static cudaError_t launch_integrate_ffblock(const CellArgs &a, const MixedTables &T, float *Ahi, float *Alo,
                                            float *bhi, float *blo, float2 *coef, cudaStream_t s, int num_sms,
                                            long long *launches) {
  using S = DarcyShape<D, K>;
  double *detj = reinterpret_cast<double *>(coef + (size_t)kFFCoef * a.ncells);
  int g0 = (a.ncells + 255) / 256;
  if (g0 > 8 * num_sms) g0 = 8 * num_sms;
  if (g0 < 1) g0 = 1;
  ff_cell_coef_kernel<<<g0, 256, 0, s>>>(a, coef, detj);
  ++*launches;
  const size_t rsmem = sizeof(double) * ((size_t)a.nqv * S::NK + 8 * (size_t)a.nqv * (D + 1));
  if (rsmem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(ff_cell_rhs_kernel<D, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)rsmem);
    if (e != cudaSuccess) return e;
  }
  int g1 = (a.ncells + 7) / 8;
  if (g1 > 4 * num_sms) g1 = 4 * num_sms;
  if (g1 < 1) g1 = 1;
  ff_cell_rhs_kernel<D, K><<<g1, 256, rsmem, s>>>(a, detj, bhi, blo);
  ++*launches;
  const int ngroups = (a.ncells + kFFCells - 1) / kFFCells;
  dim3 grid((S::NE + 255) / 256, ngroups < 65535 ? ngroups : 65535);
  integrate_ffentries_kernel<D, K><<<grid, 256, 0, s>>>(a.ncells, T, a.axis != 0, coef, Ahi, Alo);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_integrate_mixed(const CellArgs &a, const MixedTables &T, float *Ahi, float *Alo, float *bhi,
                                   float *blo, cudaStream_t s, int num_sms, long long *launches, bool skip_uu,
                                   float2 *coef) {
  if (a.nqv > 512) return cudaErrorInvalidValue;
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
#define HDG_IFB(DD, KK)                                                                                     \
  if (skip_uu && coef && a.D == DD && a.k == KK)                                                            \
    return launch_integrate_ffblock<DD, KK>(a, T, Ahi, Alo, bhi, blo, coef, s, num_sms, launches);
  HDG_IFB(2, 1)
  HDG_IFB(2, 2)
  HDG_IFB(2, 3)
  HDG_IFB(3, 1)
  HDG_IFB(3, 2)
#undef HDG_IFB
  integrate_mixed_kernel<<<grid, 256, 0, s>>>(a, T, Ahi, Alo, bhi, blo, skip_uu);
  ++*launches;
  return cudaGetLastError();
}

// FP64 cell blocks (Map-level callers) -> float-float pairs
__global__ void split_fp64_kernel(size_t count, const double *__restrict__ x, float *hi, float *lo) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    float h, l;
    split_double(x[i], h, l);
    hi[i] = h;
    lo[i] = l;
  }
}

cudaError_t launch_split_fp64(size_t count, const double *x, float *hi, float *lo, cudaStream_t s, int num_sms,
                              long long *launches) {
  size_t g = (count + 255) / 256;
  if (g > (size_t)num_sms * 32) g = (size_t)num_sms * 32;
  if (g < 1) g = 1;
  split_fp64_kernel<<<(int)g, 256, 0, s>>>(count, x, hi, lo);
  ++*launches;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Condensation: FP32 LU of A_ii with one float-float refinement step.
// Shared memory: W = [A_ii | A_if | b_i] (ni x (n+1), FP32, column-major,
// ld = ni) factorised in place, R (ni x (nf+1)) for the residual/correction.
// ---------------------------------------------------------------------------
constexpr int kMixedThreads = 256;
constexpr int kColChunk = 28;  // right-hand-side columns per thread in the float-float products

__device__ int lu_fp32_interior(float *W, int ni, int ncols, int *ipiv, int *s_piv) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int info = 0;
  for (int j = 0; j < ni; ++j) {
    if (warp == 0) {
      float best = -1.0f;
      int bi = j;
      for (int i = j + lane; i < ni; i += 32) {
        const float v = fabsf(W[i + ni * j]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const float ov = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) {
        *s_piv = best > 0.0f ? bi : -1;
        ipiv[j] = best > 0.0f ? bi : j;
      }
    }
    __syncthreads();
    const int p = *s_piv;
    if (p < 0) {
      if (!info) info = j + 1;
      __syncthreads();
      continue;
    }
    if (p != j)
      for (int c = threadIdx.x; c < ncols; c += blockDim.x) {  // whole rows: L stays consistent
        const float t = W[j + ni * c];
        W[j + ni * c] = W[p + ni * c];
        W[p + ni * c] = t;
      }
    __syncthreads();
    const float r = 1.0f / W[j + ni * j];
    for (int i = j + 1 + threadIdx.x; i < ni; i += blockDim.x) W[i + ni * j] *= r;
    __syncthreads();
    for (int c = j + 1 + warp; c < ncols; c += nw) {
      const float u = W[j + ni * c];
      if (u != 0.0f)
        for (int i = j + 1 + lane; i < ni; i += 32) W[i + ni * c] = fmaf(-W[i + ni * j], u, W[i + ni * c]);
    }
    __syncthreads();
  }
  return info;
}

// B (ni x nb, ld ldb) <- U^{-1} B with U the upper triangle of W (ld ni)
__device__ void upper_solve(const float *W, int ni, float *B, int ldb, int nb) {
  for (int j = ni - 1; j >= 0; --j) {
    const float d = 1.0f / W[j + ni * j];
    for (int c = threadIdx.x; c < nb; c += blockDim.x) B[j + ldb * c] *= d;
    __syncthreads();
    const int work = j * nb;
    for (int e = threadIdx.x; e < work; e += blockDim.x) {
      const int c = e / j, i = e - c * j;
      B[i + ldb * c] = fmaf(-W[i + ni * j], B[j + ldb * c], B[i + ldb * c]);
    }
    __syncthreads();
  }
}

// B <- L^{-1} P B (unit lower L in W's strict lower triangle, LAPACK ipiv)
__device__ void lower_solve_perm(const float *W, int ni, const int *ipiv, float *B, int ldb, int nb) {
  for (int c = threadIdx.x; c < nb; c += blockDim.x)
    for (int j = 0; j < ni; ++j) {
      const int p = ipiv[j];
      if (p != j) {
        const float t = B[j + ldb * c];
        B[j + ldb * c] = B[p + ldb * c];
        B[p + ldb * c] = t;
      }
    }
  __syncthreads();
  for (int j = 0; j < ni; ++j) {
    const int rows = ni - j - 1;
    const int work = rows * nb;
    for (int e = threadIdx.x; e < work; e += blockDim.x) {
      const int c = e / rows, i = j + 1 + (e - c * rows);
      B[i + ldb * c] = fmaf(-W[i + ni * j], B[j + ldb * c], B[i + ldb * c]);
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kMixedThreads) condense_mixed_kernel(
    int ncells, int ni, int nf, const float *__restrict__ Ahi, const float *__restrict__ Alo,
    const float *__restrict__ bhi, const float *__restrict__ blo, double *S, double *g, float *Xhi, float *Xlo,
    int *info) {
  extern __shared__ float smem[];
  __shared__ int s_piv;
  const int n = ni + nf, nc = nf + 1;
  float *W = smem;                                         // ni x (n+1)
  float *R = W + (size_t)ni * (n + 1);                     // ni x nc
  int *ipiv = reinterpret_cast<int *>(R + (size_t)ni * nc);  // ni
  float *X0 = W + (size_t)ni * ni;                         // columns ni..n of W after the solve
  const int half = blockDim.x / 2, grp = threadIdx.x / half, lt = threadIdx.x - grp * half;
  const int nchunks = (nc + kColChunk - 1) / kColChunk;
  for (int c = blockIdx.x; c < ncells; c += gridDim.x) {
    const float *Ah = Ahi + (size_t)c * n * n, *Al = Alo + (size_t)c * n * n;
    const float *bh = bhi + (size_t)c * n, *bl = blo + (size_t)c * n;
    // 1. W = [A_ii | A_if | b_i] (hi parts)
    for (int e = threadIdx.x; e < ni * n; e += blockDim.x) {
      const int j = e / ni, i = e - j * ni;
      W[e] = Ah[i + (size_t)n * j];
    }
    for (int i = threadIdx.x; i < ni; i += blockDim.x) W[(size_t)ni * n + i] = bh[i];
    __syncthreads();
    // 2. FP32 LU with partial pivoting; U12 and y become L^{-1} P [A_if | b_i]
    const int inf = lu_fp32_interior(W, ni, n + 1, ipiv, &s_piv);
    // 3. X0 = U^{-1} [U12 | y]
    upper_solve(W, ni, X0, ni, nc);
    // 4. R = [A_if | b_i] - A_ii X0 in float-float (A in original row order)
    for (int chunk = grp; chunk < nchunks; chunk += 2) {
      const int c0 = chunk * kColChunk;
      const int ncol = min(kColChunk, nc - c0);
      for (int i = lt; i < ni; i += half) {
        float hs[kColChunk], ls[kColChunk];
#pragma unroll
        for (int q = 0; q < kColChunk; ++q) {
          hs[q] = 0.0f;
          ls[q] = 0.0f;
        }
        for (int k = 0; k < ni; ++k) {
          const float ah = Ah[i + (size_t)n * k], al = Al[i + (size_t)n * k];
#pragma unroll
          for (int q = 0; q < kColChunk; ++q)
            if (q < ncol) ff_mac(hs[q], ls[q], ah, al, X0[k + ni * (c0 + q)]);
        }
#pragma unroll
        for (int q = 0; q < kColChunk; ++q)
          if (q < ncol) {
            const int col = c0 + q;
            const float rh = col < nf ? Ah[i + (size_t)n * (ni + col)] : bh[i];
            const float rl = col < nf ? Al[i + (size_t)n * (ni + col)] : bl[i];
            // r = (rh + rl) - (hs + ls), hi part only is kept
            R[i + ni * col] = ((rh - hs[q]) + rl) - ls[q];
          }
      }
    }
    __syncthreads();
    // 5. delta = A_ii^{-1} R with the FP32 factors
    lower_solve_perm(W, ni, ipiv, R, ni, nc);
    upper_solve(W, ni, R, ni, nc);
    // 6. S = A_ff - A_fi (X0 + delta), g = b_f - A_fi (y0 + delta_y), float-float
    for (int chunk = grp; chunk < nchunks; chunk += 2) {
      const int c0 = chunk * kColChunk;
      const int ncol = min(kColChunk, nc - c0);
      for (int a = lt; a < nf; a += half) {
        float hs[kColChunk], ls[kColChunk];
#pragma unroll
        for (int q = 0; q < kColChunk; ++q) {
          hs[q] = 0.0f;
          ls[q] = 0.0f;
        }
        for (int k = 0; k < ni; ++k) {
          const float ah = Ah[(ni + a) + (size_t)n * k], al = Al[(ni + a) + (size_t)n * k];
#pragma unroll
          for (int q = 0; q < kColChunk; ++q)
            if (q < ncol) ff_mac2(hs[q], ls[q], ah, al, X0[k + ni * (c0 + q)], R[k + ni * (c0 + q)]);
        }
#pragma unroll
        for (int q = 0; q < kColChunk; ++q)
          if (q < ncol) {
            const int col = c0 + q;
            const double rhs = col < nf ? (double)Ah[(ni + a) + (size_t)n * (ni + col)] +
                                              (double)Al[(ni + a) + (size_t)n * (ni + col)]
                                        : (double)bh[ni + a] + (double)bl[ni + a];
            const double v = rhs - ((double)hs[q] + (double)ls[q]);
            if (col < nf)
              S[(size_t)c * nf * nf + a + (size_t)nf * col] = v;
            else
              g[(size_t)c * nf + a] = v;
          }
      }
    }
    // 7. keep X1 = (X0, delta) for the recovery
    if (Xhi) {
      float *xh = Xhi + (size_t)c * ni * nc, *xl = Xlo + (size_t)c * ni * nc;
      for (int e = threadIdx.x; e < ni * nc; e += blockDim.x) {
        xh[e] = X0[e];
        xl[e] = R[e];
      }
    }
    if (info && threadIdx.x == 0) info[c] = inf;
    __syncthreads();
  }
}

size_t condense_mixed_smem(int ni, int nf) {
  const int n = ni + nf;
  return sizeof(float) * ((size_t)ni * (n + 1) + (size_t)ni * (nf + 1)) + sizeof(int) * ni;
}

template <class C>
static cudaError_t launch_rt(int ncells, const float *Ahi, const float *Alo, const float *bhi, const float *blo,
                             double *S, double *g, float *Xhi, float *Xlo, int *info, cudaStream_t s, int num_sms) {
  const size_t smem = C::smem_bytes;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(rt::condense_mixed_rt_kernel<C>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = (int)((228 * 1024) / (smem + 1024));
  const int by_threads = 2048 / C::NT;
  if (per_sm > by_threads) per_sm = by_threads;
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  if (grid > ncells) grid = ncells;
  if (grid < 1) grid = 1;
  rt::condense_mixed_rt_kernel<C><<<grid, C::NT, smem, s>>>(ncells, Ahi, Alo, bhi, blo, S, g, Xhi, Xlo, info);
  return cudaGetLastError();
}

cudaError_t launch_condense_mixed(int ncells, int ni, int nf, const float *Ahi, const float *Alo,
                                  const float *bhi, const float *blo, double *S, double *g, float *Xhi,
                                  float *Xlo, int *info, cudaStream_t s, int num_sms, long long *launches) {
  // register-tiled kernel for the cell sizes of the Darcy HDG spaces
  // (2D k = 1, 2, 3; 3D k = 1, 2); the shared-memory kernel below otherwise
#define HDG_RT_CASE(NI, NF, TR, TC)                                                                      \
  if (ni == NI && nf == NF) {                                                                            \
    ++*launches;                                                                                         \
    return launch_rt<rt::Cfg<NI, NF, TR, TC>>(ncells, Ahi, Alo, bhi, blo, S, g, Xhi, Xlo, info, s, num_sms); \
  }
  HDG_RT_CASE(108, 54, 16, 16)
  HDG_RT_CASE(48, 16, 16, 8)
  HDG_RT_CASE(32, 24, 16, 8)
  HDG_RT_CASE(27, 12, 8, 8)
  HDG_RT_CASE(12, 8, 4, 8)
  // linear elasticity cells: 3D k=1, 2D k=1..3
  HDG_RT_CASE(72, 72, 16, 16)
  HDG_RT_CASE(20, 16, 8, 8)
  HDG_RT_CASE(45, 24, 16, 8)
  HDG_RT_CASE(80, 32, 16, 16)
#undef HDG_RT_CASE
  const size_t smem = condense_mixed_smem(ni, nf);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(condense_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int per_sm = (int)((228 * 1024) / (smem + 1024));
  int grid = num_sms * (per_sm > 0 ? per_sm : 1);
  if (grid > ncells) grid = ncells;
  if (grid < 1) grid = 1;
  condense_mixed_kernel<<<grid, kMixedThreads, smem, s>>>(ncells, ni, nf, Ahi, Alo, bhi, blo, S, g, Xhi, Xlo,
                                                          info);
  ++*launches;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Recovery: u = y1 - X1_f x_f in float-float, X1 = (X0 + delta) from the
// condensation, x_f the cell's skeleton values (FP64, split).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) recover_mixed_kernel(CellArgs a, const float *__restrict__ Xhi,
                                                            const float *__restrict__ Xlo,
                                                            const double *__restrict__ lambda,
                                                            const double *__restrict__ dirvals, double *uint) {
  __shared__ float xf[2][6 * 64];
  const int ni = a.ni, nf = a.nf, nfd = a.nfd, nl = a.nf / a.nfd, nc = nf + 1;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    for (int e = threadIdx.x; e < nf; e += blockDim.x) {
      const int lf = e / nfd, j = e - lf * nfd;
      const int id = a.facet_dofs[(size_t)a.cell_facets[(size_t)c * nl + lf] * nfd + j];
      const double v = id >= 0 ? lambda[id] : dirvals[-1 - id];
      split_double(v, xf[0][e], xf[1][e]);
    }
    __syncthreads();
    const float *xh = Xhi + (size_t)c * ni * nc, *xl = Xlo + (size_t)c * ni * nc;
    for (int i = threadIdx.x; i < ni; i += blockDim.x) {
      float h = 0.0f, l = 0.0f;
      for (int j = 0; j < nf; ++j) ff_mac2(h, l, xh[i + ni * j], xl[i + ni * j], xf[0][j], xf[1][j]);
      const double y = (double)xh[i + ni * nf] + (double)xl[i + ni * nf];
      uint[(size_t)c * ni + i] = y - ((double)h + (double)l);
    }
    __syncthreads();
  }
}

cudaError_t launch_recover_mixed(const CellArgs &a, const float *Xhi, const float *Xlo, const double *lambda,
                                 const double *dirvals, double *uint, cudaStream_t s, int num_sms,
                                 long long *launches) {
  if (a.nf > 6 * 64) return cudaErrorInvalidValue;
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  recover_mixed_kernel<<<grid, 128, 0, s>>>(a, Xhi, Xlo, lambda, dirvals, uint);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace hdg
