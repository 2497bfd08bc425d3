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
  // shared memory (floats): Y (D NK NK), P (NK NK; holds M^{-1} until P is
  // formed), Z (D NK NC), Q (NK NC), each hi + lo -- 71 KB for 3D k=2, three
  // CTAs per SM
  static constexpr size_t smem_floats = 2 * ((size_t)D * NK * NK + NK * NK + (size_t)D * NK * NC + NK * NC);
  // + flags (64 ints) + per local facet the interior columns its trace rows couple to (2D x NI ints, counts)
  static constexpr int NL = 2 * D;
  static constexpr size_t smem_bytes = smem_floats * 4 + 64 * 4 + ((size_t)NL * NI + 8 + NL * 4 + 2 * D * NK) * 4;
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

// One cell of the block elimination with the NT threads t = 0..NT-1 of the
// caller's group.  smem: the group's C::smem_bytes of shared memory.  Every
// thread of the CTA must call it (it contains CTA barriers); a group without a
// cell passes active = false (it then computes on its own scratch and writes
// nothing).  Outputs: Sc (NF x NF column-major), gc (NF), the recovery pair
// xh/xl (NI x NC column-major, may be null) and infoc (may be null).
template <class C, int NT, bool RO>
__device__ __forceinline__ void ffblock_cell(bool active, const float *__restrict__ Ah, const float *__restrict__ Al,
                                             const float *__restrict__ bh, const float *__restrict__ bl,
                                             const float *__restrict__ Minv_h, const float *__restrict__ Minv_l,
                                             const float *__restrict__ MG_h, const float *__restrict__ MG_l,
                                             const double *coef, float *smem, double *Sc, double *gc, float *xh,
                                             float *xl, int *infoc, int t) {
  constexpr int D = C::D, NK = C::NK, NU = C::NU, NI = C::NI, NF = C::NF, N = C::N, NC = C::NC;
  float *Yh = smem, *Yl = Yh + D * NK * NK;          // [d][a][b]
  float *Ph = Yl + D * NK * NK, *Pl = Ph + NK * NK;  // [a][b]
  float *Zh = Pl + NK * NK, *Zl = Zh + D * NK * NC;  // [d][a][c]
  float *Qh = Zl + D * NK * NC, *Ql = Qh + NK * NC;  // [a][c]
  const float *Mh = Ph, *Ml = Pl;                      // M^{-1} [a][k], until P is formed
  int *sflag = reinterpret_cast<int *>(Ql + NK * NC);  // [0] pivot row, [1] info
  // [32..49]: the panel coefficients coef[1 + 3e + d] as float-float pairs,
  // split once per cell (FP64 is a narrow pipe on GB300)
  float *wsp = reinterpret_cast<float *>(sflag + 32);
  int *flist = sflag + 64;                             // [lf][q]: interior rows / columns coupled to facet lf
  int *fcnt = flist + C::NL * NI;                      // [lf]: their count
  int *fseg = fcnt + 8;                                // [lf][d]: start of field d's entries (d <= D)
  unsigned *ycol = reinterpret_cast<unsigned *>(fseg + C::NL * 4);  // [d][c]: rows a with Y_d[a][c] != 0
  unsigned *yrow = ycol + D * NK;                                    // [d][a]: columns c with Y_d[a][c] != 0
  constexpr int NFACE = C::NL, NFDc = C::NFD;
  const int lane = t & 31, warp = t >> 5, nwarps = NT >> 5;
  // The interior rows each local facet's trace columns couple to (A_if: its
  // exactly-zero entries add nothing to Z and Q), in increasing order, with
  // the start of each field's rows: one warp per facet, ballot compaction.
  for (int lf = warp; lf < NFACE; lf += nwarps) {
    int base = 0;
    for (int r0 = 0; r0 < NI; r0 += 32) {
      const int row = r0 + lane;
      bool nz = false;
      if (row < NI)
        for (int j = 0; j < NFDc; ++j) nz |= AH(row, NI + lf * NFDc + j) != 0.0f;
      const unsigned bal = __ballot_sync(0xffffffffu, nz);
      if (nz) flist[lf * NI + base + __popc(bal & ((1u << lane) - 1u))] = row;
      base += __popc(bal);
    }
    __syncwarp();
    if (lane == 0) {
      fcnt[lf] = base;
      int q = 0;
      for (int d = 0; d <= D; ++d) {  // fields: D flux components, then the pressure
        while (q < base && flist[lf * NI + q] < d * NK) ++q;
        fseg[lf * 4 + d] = q;
      }
    }
  }
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
        const int k = flist[lf * NI + q] - d * NK;
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
  // P = T - sum_d G'_d Y_d ;  Q = R_p - sum_d G'_d Z_d
  for (int o = t; o < NK * (NK + NC); o += NT) {
    const int a = o % NK, c = o / NK;
    float h = 0.0f, l = 0.0f;
    if (c < NK) {
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
    } else {
      const int cc = c - NK, lf = cc / NFDc;
      for (int d = 0; d < D; ++d) {
        // a skeleton column of Z_d is exactly zero when no row of field d couples to its facet
        if (cc < NF && fseg[lf * 4 + d] == fseg[lf * 4 + d + 1]) continue;
        for (int k = 0; k < NK; ++k)
          mac(h, l, AH(NU + a, d * NK + k), AL(NU + a, d * NK + k), Zh[(d * NK + k) * NC + cc],
              Zl[(d * NK + k) * NC + cc]);
      }
      const float rh0 = cc < NF ? AH(NU + a, NI + cc) : LDB(bh, NU + a);
      const float rl0 = cc < NF ? AL(NU + a, NI + cc) : LDB(bl, NU + a);
      float rh, rl;
      sub(rh0, rl0, h, l, rh, rl);
      Qh[a * NC + cc] = rh;
      Ql[a * NC + cc] = rl;
    }
  }
  if (t == 0) sflag[1] = 0;
  __syncthreads();
  // LU with partial pivoting of [P | Q] (pivot search by warp 0), then X_p = U^{-1} Q
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
        float th = rh[j * ld + cc], tl = rl[j * ld + cc];
        rh[j * ld + cc] = rh[p * ld + cc];
        rl[j * ld + cc] = rl[p * ld + cc];
        rh[p * ld + cc] = th;
        rl[p * ld + cc] = tl;
      }
    }
    __syncthreads();
    const float pvh = Ph[j * NK + j], pvl = Pl[j * NK + j];
    const int rows = NK - j - 1, cols = NK - j - 1 + NC;
    // multipliers (column j below the diagonal)
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
      float ph, pl, rh, rl;
      mul(lh, ll, uh, ul, ph, pl);
      sub(*th, *tl, ph, pl, rh, rl);
      *th = rh;
      *tl = rl;
    }
    __syncthreads();
  }
  for (int j = NK - 1; j >= 0; --j) {  // back substitution on Q (NC columns)
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
      float ph, pl, rh, rl;
      mul(Ph[i * NK + j], Pl[i * NK + j], Qh[j * NC + c], Ql[j * NC + c], ph, pl);
      sub(Qh[i * NC + c], Ql[i * NC + c], ph, pl, rh, rl);
      Qh[i * NC + c] = rh;
      Ql[i * NC + c] = rl;
    }
    __syncthreads();
  }
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
  // the interior columns each local facet's trace rows couple to (entries of
  // A_fi that are exactly zero add nothing to S: skipping them leaves the bits
  // unchanged), in increasing order: one warp per facet, ballot compaction
  {
    for (int lf = warp; lf < NFACE; lf += nwarps) {
      int base = 0;
      for (int c0 = 0; c0 < NI; c0 += 32) {
        const int col = c0 + lane;
        bool nz = false;
        if (col < NI)
          for (int j = 0; j < NFDc; ++j) nz |= AH(NI + lf * NFDc + j, col) != 0.0f;
        const unsigned bal = __ballot_sync(0xffffffffu, nz);
        if (nz) flist[lf * NI + base + __popc(bal & ((1u << lane) - 1u))] = col;
        base += __popc(bal);
      }
      if (lane == 0) fcnt[lf] = base;
    }
  }
  __syncthreads();
  // S = A_ff - A_fi X, g = b_f - A_fi y
  for (int o = t; o < NF * NC; o += NT) {
    const int f = o % NF, c = o / NF, lf = f / C::NFD;
    float h = 0.0f, l = 0.0f;
    const int cnt = fcnt[lf];
    for (int q = 0; q < cnt; ++q) {
      const int k = flist[lf * NI + q];
      if (k < NU)
        mac(h, l, AH(NI + f, k), AL(NI + f, k), Zh[k * NC + c], Zl[k * NC + c]);
      else
        mac(h, l, AH(NI + f, k), AL(NI + f, k), Qh[(k - NU) * NC + c], Ql[(k - NU) * NC + c]);
    }
    // the difference in float-float, one conversion to FP64
    const float rh = c < NF ? AH(NI + f, NI + c) : LDB(bh, NI + f);
    const float rl = c < NF ? AL(NI + f, NI + c) : LDB(bl, NI + f);
    float vh, vl;
    sub(rh, rl, h, l, vh, vl);
    const double v = (double)vh + (double)vl;
    if (!active) continue;
    if (c < NF)
      Sc[f + (size_t)NF * c] = v;
    else
      gc[f] = v;
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
