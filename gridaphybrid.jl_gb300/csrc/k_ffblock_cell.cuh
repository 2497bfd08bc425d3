// k_ffblock_cell.cuh -- one cell of the Darcy block elimination in
// float-float (see k_condense_ffblock.cu), shared by the single-problem and
// the batched kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>

namespace hdg {
namespace ffb {

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  e = b - (s - a);
}

// (h, l) += (ah + al) * (bh + bl)
__device__ __forceinline__ void mac(float &h, float &l, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  float pe = fmaf(ah, bh, -p);
  pe = fmaf(al, bh, pe);
  pe = fmaf(ah, bl, pe);
  float s, e;
  two_sum(h, p, s, e);
  h = s;
  l += e + pe;
}

// normalised product (ah + al) * (bh + bl)
__device__ __forceinline__ void mul(float ah, float al, float bh, float bl, float &h, float &l) {
  const float p = ah * bh;
  float pe = fmaf(ah, bh, -p);
  pe = fmaf(al, bh, pe);
  pe = fmaf(ah, bl, pe);
  fast_two_sum(p, pe, h, l);
}

// normalised (ah + al) - (bh + bl)
__device__ __forceinline__ void sub(float ah, float al, float bh, float bl, float &h, float &l) {
  float s, e;
  two_sum(ah, -bh, s, e);
  e += al - bl;
  fast_two_sum(s, e, h, l);
}

// normalised (ah + al) / (bh + bl)
__device__ __forceinline__ void div(float ah, float al, float bh, float bl, float &h, float &l) {
  const float q1 = ah / bh;
  float ph, pl;
  mul(q1, 0.0f, bh, bl, ph, pl);
  float rh, rl;
  sub(ah, al, ph, pl, rh, rl);
  const float q2 = rh / bh;
  fast_two_sum(q1, q2, h, l);
}


// normalised (ah + al) - (bh + bl) * (ch + cl) without normalising the
// product first (three FP32 operations fewer than mul then sub)
__device__ __forceinline__ void fms(float ah, float al, float bh, float bl, float ch, float cl, float &h, float &l) {
  const float p = bh * ch;
  float pe = fmaf(bh, ch, -p);
  pe = fmaf(bl, ch, pe);
  pe = fmaf(bh, cl, pe);
  float s, e;
  two_sum(ah, -p, s, e);
  e += al - pe;
  fast_two_sum(s, e, h, l);
}

__device__ __forceinline__ void normalise(float &h, float &l) {
  float s, e;
  fast_two_sum(h, l, s, e);
  h = s;
  l = e;
}

template <int D_, int NK_, int NFD_>
struct Cfg {
  static constexpr int D = D_, NK = NK_, NFD = NFD_;
  static constexpr int NU = D * NK, NI = (D + 1) * NK, NF = 2 * D * NFD, N = NI + NF, NC = NF + 1;
  static constexpr int NT = 256;
  static constexpr int NL = 2 * D;
  // interior rows the trace of one facet can couple to: the facet's nodes of
  // each flux component and of the pressure
  static constexpr int CMAX = (D + 1) * NFD;
  // the Y region holds Y (D NK NK) until X_u is formed, then the staged
  // coupled entries of A_fi (CMAX x NF)
  static constexpr int YREG = D * NK * NK > NF * CMAX ? D * NK * NK : NF * CMAX;
  // shared memory (floats): Y region, P (NK NK; holds M^{-1} until P is
  // formed), Z (D NK NC), Q (NK NC), each hi + lo -- 71 KB for 3D k=2, three
  // CTAs per SM
  static constexpr size_t smem_floats = 2 * ((size_t)YREG + NK * NK + (size_t)D * NK * NC + NK * NC);
  // the coupling pattern: per local facet its coupled interior rows (CMAX
  // slots each), the counts (8 slots), the start of each field's rows (4
  // slots per facet)
  static constexpr int PAT_INTS = NL * CMAX + 8 + NL * 4;
  // + flags (64 ints) + pattern + Y's zero masks (2 D NK) + the pivot rows (32)
  static constexpr size_t smem_bytes = smem_floats * 4 + 64 * 4 + ((size_t)PAT_INTS + 2 * D * NK + 32) * 4;
};

// A entry (row r, column c) of the column-major N x N cell matrix (hi, lo) and
// b entries; RO: A and b are not written during the kernel, so the read-only
// data path may be used.
template <bool RO>
__device__ __forceinline__ float ld_cell(const float *p) {
  if constexpr (RO)
    return __ldg(p);
  else
    return *p;
}
#define AH(r, c) ld_cell<RO>(Ah + (size_t)(r) + (size_t)N * (c))
#define AL(r, c) ld_cell<RO>(Al + (size_t)(r) + (size_t)N * (c))
#define LDB(v, i) ld_cell<RO>((v) + (i))

// LU with partial pivoting of the NK x NK pressure Schur complement P (NK <=
// 32) by one warp, lane i working on row i.  Rows stay in place: perm[j] is
// the row chosen as pivot of step j; each other free row keeps its multiplier
// in column j.  So U's row j is row perm[j] from column j on, and L's row j
// is row perm[j] left of column j.  The pivot is the largest |P[.][j]| among
// the free rows, ties going to the row that a row-swapping LU would hold at
// the lowest position (pos tracks each row's position under those swaps), so
// the pivots, multipliers and updates are those of lu_solve_group, bit for
// bit.  Writes the first zero pivot step + 1 (or 0) to *info.
template <int NK>
__device__ __forceinline__ void lu_pivot_warp(float *Ph, float *Pl, int *perm, int *info, int lane) {
  bool free_row = lane < NK;
  int pos = lane;
  int first_zero = 0;
  for (int j = 0; j < NK; ++j) {
    float v = -1.0f;
    if (free_row) {
      v = fabsf(Ph[lane * NK + j]);
      if (v != v) v = INFINITY;  // a NaN pivot candidate: every lane must pick the same row
    }
    int bpos = free_row ? pos : 1 << 20, bi = lane;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, v, off);
      const int op = __shfl_xor_sync(0xffffffffu, bpos, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (ov > v || (ov == v && op < bpos)) {
        v = ov;
        bpos = op;
        bi = oi;
      }
    }
    const int p = bi;  // the same in every lane
    if (v == 0.0f && first_zero == 0) first_zero = j + 1;
    if (lane == 0) perm[j] = p;
    // a row-swapping LU exchanges the rows at positions j and bpos
    if (free_row && pos == j && lane != p) pos = bpos;
    if (lane == p) {
      free_row = false;
      pos = j;
    }
    const float pvh = Ph[p * NK + j], pvl = Pl[p * NK + j];
    if (free_row && pvh != 0.0f) {
      float lh, ll;
      div(Ph[lane * NK + j], Pl[lane * NK + j], pvh, pvl, lh, ll);
      Ph[lane * NK + j] = lh;
      Pl[lane * NK + j] = ll;
      for (int c = j + 1; c < NK; ++c) {
        float rh, rl;
        fms(Ph[lane * NK + c], Pl[lane * NK + c], lh, ll, Ph[p * NK + c], Pl[p * NK + c], rh, rl);
        Ph[lane * NK + c] = rh;
        Pl[lane * NK + c] = rl;
      }
    }
    __syncwarp();
  }
  if (lane == 0) *info = first_zero;
}

// Q = R_p - sum_d G'_d Z_d with the NQ threads tq = 0..NQ-1: thread (a, g)
// forms row a of a run of consecutive columns, so each A_pu entry it loads
// serves every column of the run that takes its field (a column of a facet
// that field d does not couple to skips d; b takes every field).  The sums run
// over d, then k, in increasing order.
template <class C, int NQ, bool RO>
__device__ __forceinline__ void form_q(const float *__restrict__ Ah, const float *__restrict__ Al,
                                       const float *__restrict__ bh, const float *__restrict__ bl, const float *Zh,
                                       const float *Zl, float *Qh, float *Ql, const int *fseg, int tq) {
  constexpr int D = C::D, NK = C::NK, NU = C::NU, NI = C::NI, NF = C::NF, N = C::N, NC = C::NC, NFDc = C::NFD;
  constexpr int G = NQ / NK;           // row groups (NK <= 27 < 32 <= NQ)
  constexpr int R = (NC + G - 1) / G;  // columns per group
  constexpr int RC = NQ >= 128 ? 8 : 4;  // columns per pass (fewer registers in small groups)
  if (tq >= G * NK) return;
  const int a = tq % NK, g = tq / NK;
  const int c_end = (g + 1) * R < NC ? (g + 1) * R : NC;
  for (int c0 = g * R; c0 < c_end; c0 += RC) {
    float h[RC], l[RC];
    unsigned need[D];
#pragma unroll
    for (int d = 0; d < D; ++d) need[d] = 0u;
#pragma unroll
    for (int j = 0; j < RC; ++j) {
      h[j] = 0.0f;
      l[j] = 0.0f;
      const int cc = c0 + j;
      if (cc < c_end) {
        const int lf = cc < NF ? cc / NFDc : 0;
#pragma unroll
        for (int d = 0; d < D; ++d)
          if (cc == NF || fseg[lf * 4 + d] != fseg[lf * 4 + d + 1]) need[d] |= 1u << j;
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      if (!need[d]) continue;
      for (int k = 0; k < NK; ++k) {
        const float ah = AH(NU + a, d * NK + k), al = AL(NU + a, d * NK + k);
        const float *zh = Zh + (d * NK + k) * NC + c0, *zl = Zl + (d * NK + k) * NC + c0;
#pragma unroll
        for (int j = 0; j < RC; ++j)
          if (need[d] >> j & 1u) mac(h[j], l[j], ah, al, zh[j], zl[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < RC; ++j) {
      const int cc = c0 + j;
      if (cc < c_end) {
        const float rh0 = cc < NF ? AH(NU + a, NI + cc) : LDB(bh, NU + a);
        const float rl0 = cc < NF ? AL(NU + a, NI + cc) : LDB(bl, NU + a);
        float rh, rl;
        sub(rh0, rl0, h[j], l[j], rh, rl);
        Qh[a * NC + cc] = rh;
        Ql[a * NC + cc] = rl;
      }
    }
  }
}

// X_p = P^{-1} Q in place in Q, from lu_pivot_warp's factors: every column
// by four lanes of one warp (eight columns per warp), lane sl keeping the
// entries j = sl, sl + 4, ... in registers.  Forward substitution with L,
// then back substitution with U, each step's value passed among the four
// lanes by shuffles: no CTA barrier.
template <class C, int NT>
__device__ __forceinline__ void solve_columns(const float *Ph, const float *Pl, float *Qh, float *Ql,
                                              const int *perm, int t) {
  constexpr int NK = C::NK, NC = C::NC, RPL = (NK + 3) / 4;
  const int lane = t & 31, warp = t >> 5, nwarps = NT >> 5;
  const int sl = lane & 3, base = lane & ~3;
  int pr[RPL];
#pragma unroll
  for (int s = 0; s < RPL; ++s) pr[s] = 4 * s + sl < NK ? perm[4 * s + sl] : 0;
  for (int cg = warp; cg * 8 < NC; cg += nwarps) {
    const int c = cg * 8 + (lane >> 2);
    const bool ok = c < NC;
    const int cc = ok ? c : 0;
    float yh[RPL], yl[RPL];
#pragma unroll
    for (int s = 0; s < RPL; ++s) {
      const bool in = 4 * s + sl < NK;
      yh[s] = in ? Qh[pr[s] * NC + cc] : 0.0f;
      yl[s] = in ? Ql[pr[s] * NC + cc] : 0.0f;
    }
    __syncwarp();
    // forward: y_j -= L[j][i] y_i for j > i, L[j][i] = P[perm[j]][i]
#pragma unroll
    for (int i = 0; i < NK - 1; ++i) {
      const float vh = __shfl_sync(0xffffffffu, yh[i >> 2], base | (i & 3));
      const float vl = __shfl_sync(0xffffffffu, yl[i >> 2], base | (i & 3));
#pragma unroll
      for (int s = 0; s < RPL; ++s) {
        if (4 * s + 3 <= i) continue;  // no entry of slot s lies below row i
        const int j = 4 * s + sl;
        if (j > i && j < NK) {
          float rh, rl;
          fms(yh[s], yl[s], Ph[pr[s] * NK + i], Pl[pr[s] * NK + i], vh, vl, rh, rl);
          yh[s] = rh;
          yl[s] = rl;
        }
      }
    }
    // back: x_i = y_i / U[i][i], then y_j -= U[j][i] x_i for j < i,
    // U[j][i] = P[perm[j]][i] (a zero pivot gives x_i = 0)
#pragma unroll
    for (int i = NK - 1; i >= 0; --i) {
      float xh = 0.0f, xl = 0.0f;
      if (sl == (i & 3)) {
        const float uh = Ph[pr[i >> 2] * NK + i], ul = Pl[pr[i >> 2] * NK + i];
        if (uh != 0.0f) div(yh[i >> 2], yl[i >> 2], uh, ul, xh, xl);
        yh[i >> 2] = xh;
        yl[i >> 2] = xl;
      }
      xh = __shfl_sync(0xffffffffu, xh, base | (i & 3));
      xl = __shfl_sync(0xffffffffu, xl, base | (i & 3));
#pragma unroll
      for (int s = 0; s < RPL; ++s) {
        if (4 * s >= i) continue;  // no entry of slot s lies above row i
        const int j = 4 * s + sl;
        if (j < i) {
          float rh, rl;
          fms(yh[s], yl[s], Ph[pr[s] * NK + i], Pl[pr[s] * NK + i], xh, xl, rh, rl);
          yh[s] = rh;
          yl[s] = rl;
        }
      }
    }
    __syncwarp();
    if (ok) {
#pragma unroll
      for (int s = 0; s < RPL; ++s) {
        const int j = 4 * s + sl;
        if (j < NK) {
          Qh[j * NC + c] = yh[s];
          Ql[j * NC + c] = yl[s];
        }
      }
    }
    __syncwarp();
  }
}

// [P | Q] -> [U | X_p] by the whole group: LU with partial pivoting (pivot
// search by warp 0, rows swapped in place), then back substitution on the NC
// columns of Q.  For groups of one or two warps (the batched kernels' small
// cells), where the warp-factorisation path would leave the group's only warp
// serial.
template <class C, int NT>
__device__ __forceinline__ void lu_solve_group(float *Ph, float *Pl, float *Qh, float *Ql, int *sflag, int t) {
  constexpr int NK = C::NK, NC = C::NC;
  for (int j = 0; j < NK; ++j) {
    if (t < 32) {
      float best = -1.0f;
      int bi = j;
      for (int i = j + t; i < NK; i += 32) {
        const float v = fabsf(Ph[i * NK + j]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const float ob = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (t == 0) {
        sflag[0] = bi;
        if (best == 0.0f && sflag[1] == 0) sflag[1] = j + 1;
      }
    }
    __syncthreads();
    const int p = sflag[0];
    if (p != j) {
      for (int c = t; c < NK + NC; c += NT) {
        float *rh = c < NK ? Ph : Qh, *rl = c < NK ? Pl : Ql;
        const int ld = c < NK ? NK : NC, cc = c < NK ? c : c - NK;
        const float th = rh[j * ld + cc], tl = rl[j * ld + cc];
        rh[j * ld + cc] = rh[p * ld + cc];
        rl[j * ld + cc] = rl[p * ld + cc];
        rh[p * ld + cc] = th;
        rl[p * ld + cc] = tl;
      }
    }
    __syncthreads();
    const float pvh = Ph[j * NK + j], pvl = Pl[j * NK + j];
    const int rows = NK - j - 1, cols = NK - j - 1 + NC;
    for (int i = j + 1 + t; i < NK; i += NT) {
      if (pvh != 0.0f) {
        float qh, ql;
        div(Ph[i * NK + j], Pl[i * NK + j], pvh, pvl, qh, ql);
        Ph[i * NK + j] = qh;
        Pl[i * NK + j] = ql;
      }
    }
    __syncthreads();
    for (int e = t; e < rows * cols; e += NT) {
      const int i = j + 1 + e / cols, c = e % cols;
      const float lh = Ph[i * NK + j], ll = Pl[i * NK + j];
      float uh, ul, *th, *tl;
      if (c < NK - j - 1) {
        const int cc = j + 1 + c;
        uh = Ph[j * NK + cc];
        ul = Pl[j * NK + cc];
        th = Ph + i * NK + cc;
        tl = Pl + i * NK + cc;
      } else {
        const int cc = c - (NK - j - 1);
        uh = Qh[j * NC + cc];
        ul = Ql[j * NC + cc];
        th = Qh + i * NC + cc;
        tl = Ql + i * NC + cc;
      }
      float rh, rl;
      fms(*th, *tl, lh, ll, uh, ul, rh, rl);
      *th = rh;
      *tl = rl;
    }
    __syncthreads();
  }
  for (int j = NK - 1; j >= 0; --j) {
    const float pvh = Ph[j * NK + j], pvl = Pl[j * NK + j];
    for (int c = t; c < NC; c += NT) {
      float qh = 0.0f, ql = 0.0f;
      if (pvh != 0.0f) div(Qh[j * NC + c], Ql[j * NC + c], pvh, pvl, qh, ql);
      Qh[j * NC + c] = qh;
      Ql[j * NC + c] = ql;
    }
    __syncthreads();
    for (int e = t; e < j * NC; e += NT) {
      const int i = e / NC, c = e % NC;
      float rh, rl;
      fms(Qh[i * NC + c], Ql[i * NC + c], Ph[i * NK + j], Pl[i * NK + j], Qh[j * NC + c], Ql[j * NC + c], rh, rl);
      Qh[i * NC + c] = rh;
      Ql[i * NC + c] = rl;
    }
    __syncthreads();
  }
}

// One cell of the block elimination with the NT threads t = 0..NT-1 of the
// caller's group.  smem: the group's C::smem_bytes of shared memory.  Every
// thread of the CTA must call it (it contains CTA barriers); a group without a
// cell passes active = false (it then computes on its own scratch and writes
// nothing).  pat: the coupling pattern (ffblock_pattern, C::PAT_INTS ints).
// Outputs: Sc (NF x NF column-major), gc (NF), the recovery pair xh/xl
// (NI x NC column-major, may be null) and infoc (may be null).
template <class C, int NT, bool RO>
__device__ __forceinline__ void ffblock_cell(bool active, const float *__restrict__ Ah, const float *__restrict__ Al,
                                             const float *__restrict__ bh, const float *__restrict__ bl,
                                             const float *__restrict__ Minv_h, const float *__restrict__ Minv_l,
                                             const float *__restrict__ MG_h, const float *__restrict__ MG_l,
                                             const int *__restrict__ pat, const double *coef, float *smem, double *Sc,
                                             double *gc, float *xh, float *xl, int *infoc, int t) {
  constexpr int D = C::D, NK = C::NK, NU = C::NU, NI = C::NI, NF = C::NF, N = C::N, NC = C::NC;
  constexpr int YREG = C::YREG, CMAX = C::CMAX;
  float *Yh = smem, *Yl = Yh + YREG;                 // [d][a][b]
  float *Ph = Yl + YREG, *Pl = Ph + NK * NK;         // [a][b]
  float *Zh = Pl + NK * NK, *Zl = Zh + D * NK * NC;  // [d][a][c]
  float *Qh = Zl + D * NK * NC, *Ql = Qh + NK * NC;  // [a][c]
  const float *Mh = Ph, *Ml = Pl;                      // M^{-1} [a][k], until P is formed
  int *sflag = reinterpret_cast<int *>(Ql + NK * NC);  // [1] info
  // [32..49]: the panel coefficients coef[1 + 3e + d] as float-float pairs,
  // split once per cell (FP64 is a narrow pipe on GB300)
  float *wsp = reinterpret_cast<float *>(sflag + 32);
  int *flist = sflag + 64;                             // [lf][q]: interior rows / columns coupled to facet lf
  int *fcnt = flist + C::NL * CMAX;                    // [lf]: their count
  int *fseg = fcnt + 8;                                // [lf][d]: start of field d's entries (d <= D)
  unsigned *ycol = reinterpret_cast<unsigned *>(flist + C::PAT_INTS);  // [d][c]: rows a with Y_d[a][c] != 0
  unsigned *yrow = ycol + D * NK;                                       // [d][a]: columns c with Y_d[a][c] != 0
  int *perm = reinterpret_cast<int *>(yrow + D * NK);                   // pivot row of each LU step
  constexpr int NFDc = C::NFD;
  const int lane = t & 31, warp = t >> 5, nwarps = NT >> 5;
  // The coupling pattern: the interior rows each local facet's trace columns
  // couple to (A_if), which are also the interior columns its trace rows
  // couple to (A_fi): the facet's nodes of the flux components that have a
  // normal component there and of the pressure.  The other entries are
  // exactly zero and add nothing to Z, Q and S.
  for (int e = t; e < C::PAT_INTS; e += NT) flist[e] = __ldg(pat + e);
  // Threads run fastest over the row index of each output, so the
  // column-major A entries they read are broadcast (one column entry per
  // warp) or contiguous (consecutive rows of one column).
  float imh, iml;  // 1/m as float-float
  {
    const double v = coef[0];
    imh = (float)v;
    iml = (float)(v - (double)imh);
  }
  // Y_d = (1/m) M^{-1} G_d = sum_e w_ed MG_e from the reference products
  // (MG_e = M^{-1} G_e, exactly sparse on the tensor-product cell), and
  // Z_d = (1/m) M^{-1} R_{u_d}
  for (int e = t; e < NK * NK; e += NT) {
    Ph[e] = __ldg(Minv_h + e);
    Pl[e] = __ldg(Minv_l + e);
  }
  if (t < 9) {
    const double w = coef[1 + t];
    const float wh = (float)w;
    wsp[2 * t] = wh;
    wsp[2 * t + 1] = (float)(w - (double)wh);
  }
  __syncthreads();
  for (int o = t; o < D * NK * (NK + NC); o += NT) {
    const int a = o % NK, rest = o / NK;
    const int c = rest % (NK + NC), d = rest / (NK + NC);
    float h = 0.0f, l = 0.0f;
    if (c < NK) {  // Y_d column c (pressure DOF c)
      for (int e = 0; e < D; ++e) {
        const float wh = wsp[2 * (3 * e + d)], wl = wsp[2 * (3 * e + d) + 1];
        if (wh == 0.0f && wl == 0.0f) continue;
        mac(h, l, __ldg(MG_h + (e * NK + a) * NK + c), __ldg(MG_l + (e * NK + a) * NK + c), wh, wl);
      }
      normalise(h, l);
      Yh[(d * NK + a) * NK + c] = h;
      Yl[(d * NK + a) * NK + c] = l;
      continue;
    } else if (c - NK < NF) {  // skeleton column: only field d's rows coupled to its facet
      const int cc = c - NK, lf = cc / NFDc;
      const int q1 = fseg[lf * 4 + d + 1];
      for (int q = fseg[lf * 4 + d]; q < q1; ++q) {
        const int k = flist[lf * CMAX + q] - d * NK;
        mac(h, l, Mh[a * NK + k], Ml[a * NK + k], AH(d * NK + k, NI + cc), AL(d * NK + k, NI + cc));
      }
    } else {  // b
      for (int k = 0; k < NK; ++k) mac(h, l, Mh[a * NK + k], Ml[a * NK + k], LDB(bh, d * NK + k), LDB(bl, d * NK + k));
    }
    float ph, pl;
    normalise(h, l);
    mul(h, l, imh, iml, ph, pl);
    Zh[(d * NK + a) * NC + (c - NK)] = ph;
    Zl[(d * NK + a) * NC + (c - NK)] = pl;
  }
  __syncthreads();
  // Y's zero pattern by columns and by rows (NK <= 32: one ballot each)
  for (int idx = warp; idx < 2 * D * NK; idx += nwarps) {
    const bool bycol = idx < D * NK;
    const int dx = bycol ? idx : idx - D * NK, dd = dx / NK, x = dx - dd * NK;
    const bool nz = lane < NK && (bycol ? Yh[(dd * NK + lane) * NK + x] : Yh[(dd * NK + x) * NK + lane]) != 0.0f;
    const unsigned bal = __ballot_sync(0xffffffffu, nz);
    if (lane == 0) (bycol ? ycol : yrow)[dx] = bal;
  }
  __syncthreads();
  // P = T - sum_d G'_d Y_d
  for (int o = t; o < NK * NK; o += NT) {
    const int a = o % NK, c = o / NK;
    float h = 0.0f, l = 0.0f;
    for (int d = 0; d < D; ++d)
      for (unsigned m = ycol[d * NK + c]; m; m &= m - 1) {
        const int k = __ffs(m) - 1;
        mac(h, l, AH(NU + a, d * NK + k), AL(NU + a, d * NK + k), Yh[(d * NK + k) * NK + c],
            Yl[(d * NK + k) * NK + c]);
      }
    float rh, rl;
    sub(AH(NU + a, NU + c), AL(NU + a, NU + c), h, l, rh, rl);
    Ph[a * NK + c] = rh;
    Pl[a * NK + c] = rl;
  }
  // the warp factorisation pays off where the group has warps to spare (the
  // whole-group LU measured slower at 256 threads for every cell size)
  if constexpr (NT >= 128) {
    __syncthreads();
    // warp 0 factors P while the other warps form Q
    if (warp == 0) lu_pivot_warp<NK>(Ph, Pl, perm, sflag + 1, lane);
    if (warp > 0) form_q<C, NT - 32, RO>(Ah, Al, bh, bl, Zh, Zl, Qh, Ql, fseg, t - 32);
    __syncthreads();
    // X_p = P^{-1} Q (in place in Q)
    solve_columns<C, NT>(Ph, Pl, Qh, Ql, perm, t);
  } else {
    form_q<C, NT, RO>(Ah, Al, bh, bl, Zh, Zl, Qh, Ql, fseg, t);
    if (t == 0) sflag[1] = 0;
    __syncthreads();
    lu_solve_group<C, NT>(Ph, Pl, Qh, Ql, sflag, t);
  }
  __syncthreads();
  // X_{u_d} = Z_d - Y_d X_p (in place in Z)
  for (int o = t; o < D * NK * NC; o += NT) {
    const int d = o / (NK * NC), rem = o - d * NK * NC, a = rem / NC, c = rem - a * NC;
    float h = 0.0f, l = 0.0f;
    for (unsigned m = yrow[d * NK + a]; m; m &= m - 1) {
      const int k = __ffs(m) - 1;
      mac(h, l, Yh[(d * NK + a) * NK + k], Yl[(d * NK + a) * NK + k], Qh[k * NC + c], Ql[k * NC + c]);
    }
    float rh, rl;
    sub(Zh[(d * NK + a) * NC + c], Zl[(d * NK + a) * NC + c], h, l, rh, rl);
    Zh[(d * NK + a) * NC + c] = rh;
    Zl[(d * NK + a) * NC + c] = rl;
  }
  __syncthreads();
  // the coupled entries of A_fi, staged in the Y region: As[q][f] = A(NI + f,
  // flist[lf(f)][q]) (consecutive threads read consecutive rows of a column)
  float *Ash = Yh, *Asl = Yl;
  for (int e = t; e < NF * CMAX; e += NT) {
    const int q = e / NF, f = e - q * NF, lf = f / NFDc;
    if (q < fcnt[lf]) {
      const int k = flist[lf * CMAX + q];
      Ash[e] = AH(NI + f, k);
      Asl[e] = AL(NI + f, k);
    }
  }
  __syncthreads();
  // S = A_ff - A_fi X, g = b_f - A_fi y, by tiles of SR trace rows of one
  // facet x SC columns: per coupled interior row q a thread loads SR staged
  // A_fi entries and SC entries of X and makes SR x SC products
  {
    // tiles only where they still give every thread work (small cells keep
    // one output per thread: the phase is latency-bound there)
    constexpr int SR0 = NFDc % 3 == 0 ? 3 : (NFDc % 2 == 0 ? 2 : 1);
    constexpr bool TILE = NF * NC / (SR0 * 2) >= NT;
    constexpr int SR = TILE ? SR0 : 1, SC = TILE ? 2 : 1;
    constexpr int RT = NFDc / SR, CT = (NC + SC - 1) / SC, TILES = C::NL * RT * CT;
    for (int tile = t; tile < TILES; tile += NT) {
      const int ct = tile % CT, rest = tile / CT, rt = rest % RT, lf = rest / RT;
      const int f0 = lf * NFDc + rt * SR, cb = ct * SC;
      float h[SR][SC], l[SR][SC];
#pragma unroll
      for (int r = 0; r < SR; ++r)
#pragma unroll
        for (int j = 0; j < SC; ++j) {
          h[r][j] = 0.0f;
          l[r][j] = 0.0f;
        }
      const int cnt = fcnt[lf];
      for (int q = 0; q < cnt; ++q) {
        const int k = flist[lf * CMAX + q];
        const float *xhr = k < NU ? Zh + k * NC : Qh + (k - NU) * NC;
        const float *xlr = k < NU ? Zl + k * NC : Ql + (k - NU) * NC;
        float vh[SC], vl[SC];
#pragma unroll
        for (int j = 0; j < SC; ++j) {
          const int c = cb + j < NC ? cb + j : cb;  // a duplicate column at the ragged end
          vh[j] = xhr[c];
          vl[j] = xlr[c];
        }
#pragma unroll
        for (int r = 0; r < SR; ++r) {
          const float ah = Ash[q * NF + f0 + r], al = Asl[q * NF + f0 + r];
#pragma unroll
          for (int j = 0; j < SC; ++j) mac(h[r][j], l[r][j], ah, al, vh[j], vl[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < SC; ++j) {
        const int c = cb + j;
        if (c >= NC) continue;
#pragma unroll
        for (int r = 0; r < SR; ++r) {
          const int f = f0 + r;
          // the difference in float-float, one conversion to FP64
          const float rh = c < NF ? AH(NI + f, NI + c) : LDB(bh, NI + f);
          const float rl = c < NF ? AL(NI + f, NI + c) : LDB(bl, NI + f);
          float vh, vl;
          sub(rh, rl, h[r][j], l[r][j], vh, vl);
          const double v = (double)vh + (double)vl;
          if (active) {
            if (c < NF)
              Sc[f + (size_t)NF * c] = v;
            else
              gc[f] = v;
          }
        }
      }
    }
  }
  // X = [X_u; X_p] (ni x nc, column-major) as float-float pairs for the recovery
  if (xh && active) {
    for (int e = t; e < NI * NC; e += NT) {
      const int c = e / NI, m = e - c * NI;
      const bool u = m < NU;
      xh[e] = u ? Zh[m * NC + c] : Qh[(m - NU) * NC + c];
      xl[e] = u ? Zl[m * NC + c] : Ql[(m - NU) * NC + c];
    }
  }
  if (t == 0 && infoc && active) *infoc = sflag[1];
  __syncthreads();
}

#undef AH
#undef AL
#undef LDB

}  // namespace ffb
}  // namespace hdg
