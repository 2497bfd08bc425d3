// k_condense_mixed_rt.cuh -- register-tiled FP32 LU + float-float refinement
// (the fast form of condense_mixed for the cell sizes it is instantiated for).
//
// One CTA per cell.  The interior rows of [A_ii | A_if | b_i] (NI x (N+1))
// live in registers for the whole kernel: thread (tr, tc) of a TR x TC grid
// owns rows i = tr + TR*a and columns c = tc + TC*b.  Partial pivoting is
// implicit: the pivot row of step j is "retired" (its rank is j) instead of
// being swapped, so no data moves; each step publishes the pivot row and the
// multipliers through shared memory and updates the owned tile in registers.
// After the factorisation the L\U part of the tile stays put and only the
// right-hand-side columns are rewritten by the solves:
//   X0 = A_ii^{-1} [A_if | b_i]                       (FP32)
//   repeat NSTEP times:  R = [A_if | b_i] - A_ii X     (float-float)
//                        X += A_ii^{-1} R              (FP32 correction)
//   S = A_ff - A_fi X,  g = b_f - A_fi y               (float-float)
// X is held as the unevaluated pair (X0, sum of corrections).
#pragma once
#include <cuda_runtime.h>

#include <climits>

namespace hdg {
namespace rt {

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (h, l) += (ah + al) * x
__device__ __forceinline__ void ff_mac(float &h, float &l, float ah, float al, float x) {
  const float p = ah * x;
  float pe = fmaf(ah, x, -p);
  pe = fmaf(al, x, pe);
  float s, e;
  two_sum(h, p, s, e);
  h = s;
  l += e + pe;
}

// (h, l) += (ah + al) * (xh + xl)
__device__ __forceinline__ void ff_mac2(float &h, float &l, float ah, float al, float xh, float xl) {
  const float p = ah * xh;
  float pe = fmaf(ah, xh, -p);
  pe = fmaf(al, xh, pe);
  pe = fmaf(ah, xl, pe);
  float s, e;
  two_sum(h, p, s, e);
  h = s;
  l += e + pe;
}

template <int NI_, int NF_, int TR_, int TC_>
struct Cfg {
  static constexpr int NI = NI_, NF = NF_, TR = TR_, TC = TC_;
  static constexpr int N = NI + NF, NC = NF + 1, NCOL = N + 1;
  static constexpr int RPT = (NI + TR - 1) / TR;
  static constexpr int CPT = (NCOL + TC - 1) / TC;
  static constexpr int NT = TR * TC;
  static constexpr int CC = 7;  // right-hand-side columns per task in the float-float products
  static constexpr int NCHUNK = (NC + CC - 1) / CC;
  static constexpr int NSTEP = 2;  // refinement steps
  static constexpr size_t smem_floats = 3 * (size_t)NI * NC + 2 * NI + 2 * NCOL + NI;
  static constexpr size_t smem_bytes = smem_floats * 4 + (NI + 2) * 4;
};

constexpr int kRetiredNot = INT_MAX;

template <int RPT, int CPT>
__device__ __forceinline__ float pick(const float (&W)[RPT][CPT], int a, int b) {
  float v = 0.0f;
#pragma unroll
  for (int x = 0; x < RPT; ++x)
    if (x == a) v = W[x][b];
  return v;
}

template <int RPT, int CPT>
__device__ __forceinline__ void put(float (&W)[RPT][CPT], int a, int b, float v) {
#pragma unroll
  for (int x = 0; x < RPT; ++x)
    if (x == a) W[x][b] = v;
}

// element b (a runtime index) of a register row, without dynamic indexing
template <int CPT>
__device__ __forceinline__ float colget(const float (&row)[CPT], int b) {
  float v = 0.0f;
#pragma unroll
  for (int y = 0; y < CPT; ++y)
    if (y == b) v = row[y];
  return v;
}

template <int CPT>
__device__ __forceinline__ void colset(float (&row)[CPT], int b, float v) {
#pragma unroll
  for (int y = 0; y < CPT; ++y)
    if (y == b) row[y] = v;
}

// Back substitution on the RHS columns (c >= NI): U x = y in rank order; x_m
// ends up in the row of rank m.  lbuf/ubuf double-buffered by step parity.
template <class C>
__device__ __forceinline__ void back_substitute(float (&W)[C::RPT][C::CPT], const int (&rk)[C::RPT],
                                                const int *perm, const float *rdiag, float *lbuf,
                                                float *ubuf, int tr, int tc) {
  for (int m = C::NI - 1; m >= 0; --m) {
    const int buf = m & 1;
    const int pm = perm[m];
    const int trp = pm % C::TR, ap = pm / C::TR;
    if (tr == trp) {
      const float rd = rdiag[m];
#pragma unroll
      for (int b = 0; b < C::CPT; ++b) {
        const int c = tc + C::TC * b;
        if (c >= C::NI && c < C::NCOL) {
          const float v = pick(W, ap, b) * rd;
          put(W, ap, b, v);
          ubuf[buf * C::NCOL + c] = v;
        }
      }
    }
    const int tcm = m % C::TC, bm = m / C::TC;
    if (tc == tcm) {
#pragma unroll
      for (int a = 0; a < C::RPT; ++a) {
        const int i = tr + C::TR * a;
        if (i < C::NI && rk[a] < m) lbuf[buf * C::NI + i] = colget(W[a], bm);
      }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < C::RPT; ++a) {
      const int i = tr + C::TR * a;
      if (i < C::NI && rk[a] < m) {
        const float l = lbuf[buf * C::NI + i];
#pragma unroll
        for (int b = 0; b < C::CPT; ++b) {
          const int c = tc + C::TC * b;
          if (c >= C::NI && c < C::NCOL) W[a][b] = fmaf(-l, ubuf[buf * C::NCOL + c], W[a][b]);
        }
      }
    }
  }
  __syncthreads();
}

// Forward elimination L^{-1} P on the RHS columns (rows in rank order).
template <class C>
__device__ __forceinline__ void forward_eliminate(float (&W)[C::RPT][C::CPT], const int (&rk)[C::RPT],
                                                  const int *perm, float *lbuf, float *ubuf, int tr, int tc) {
  for (int j = 0; j < C::NI; ++j) {
    const int buf = j & 1;
    const int p = perm[j];
    const int trp = p % C::TR, ap = p / C::TR;
    if (tr == trp) {
#pragma unroll
      for (int b = 0; b < C::CPT; ++b) {
        const int c = tc + C::TC * b;
        if (c >= C::NI && c < C::NCOL) ubuf[buf * C::NCOL + c] = pick(W, ap, b);
      }
    }
    const int tcj = j % C::TC, bj = j / C::TC;
    if (tc == tcj) {
#pragma unroll
      for (int a = 0; a < C::RPT; ++a) {
        const int i = tr + C::TR * a;
        if (i < C::NI && rk[a] > j) lbuf[buf * C::NI + i] = colget(W[a], bj);
      }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < C::RPT; ++a) {
      const int i = tr + C::TR * a;
      if (i < C::NI && rk[a] > j) {
        const float l = lbuf[buf * C::NI + i];
#pragma unroll
        for (int b = 0; b < C::CPT; ++b) {
          const int c = tc + C::TC * b;
          if (c >= C::NI && c < C::NCOL) W[a][b] = fmaf(-l, ubuf[buf * C::NCOL + c], W[a][b]);
        }
      }
    }
  }
  __syncthreads();
}

// Rs (natural row order) = [A_if | b_i] - A_ii (X0s + Ds) in float-float;
// with_d = false ignores Ds (first step).
template <class C>
__device__ __forceinline__ void residual(const float *__restrict__ Ah, const float *__restrict__ Al,
                                         const float *__restrict__ bh, const float *__restrict__ bl,
                                         const float *X0s, const float *Ds, float *Rs, bool with_d) {
  constexpr int NI = C::NI, NF = C::NF, N = C::N, NC = C::NC, CC = C::CC;
  for (int task = threadIdx.x; task < NI * C::NCHUNK; task += C::NT) {
    const int i = task % NI, c0 = (task / NI) * CC;
    float hs[CC], ls[CC];
#pragma unroll
    for (int q = 0; q < CC; ++q) hs[q] = ls[q] = 0.0f;
    for (int k = 0; k < NI; ++k) {
      const float ah = __ldg(Ah + i + (size_t)N * k), al = __ldg(Al + i + (size_t)N * k);
      if (with_d) {
#pragma unroll
        for (int q = 0; q < CC; ++q)
          if (c0 + q < NC) ff_mac2(hs[q], ls[q], ah, al, X0s[k + NI * (c0 + q)], Ds[k + NI * (c0 + q)]);
      } else {
#pragma unroll
        for (int q = 0; q < CC; ++q)
          if (c0 + q < NC) ff_mac(hs[q], ls[q], ah, al, X0s[k + NI * (c0 + q)]);
      }
    }
#pragma unroll
    for (int q = 0; q < CC; ++q) {
      const int col = c0 + q;
      if (col < NC) {
        const float rh = col < NF ? __ldg(Ah + i + (size_t)N * (NI + col)) : bh[i];
        const float rl = col < NF ? __ldg(Al + i + (size_t)N * (NI + col)) : bl[i];
        Rs[i + NI * col] = ((rh - hs[q]) + rl) - ls[q];
      }
    }
  }
  __syncthreads();
}

template <class C>
__global__ void __launch_bounds__(C::NT, (C::NT <= 128 ? 4 : 2))
    condense_mixed_rt_kernel(int ncells, const float *__restrict__ Ahi, const float *__restrict__ Alo,
                             const float *__restrict__ bhi, const float *__restrict__ blo, double *S, double *g,
                             float *Xhi, float *Xlo, int *info) {
  constexpr int NI = C::NI, NF = C::NF, N = C::N, NC = C::NC, NCOL = C::NCOL, RPT = C::RPT, CPT = C::CPT;
  constexpr int TR = C::TR, TC = C::TC, CC = C::CC, NCHUNK = C::NCHUNK;
  extern __shared__ float smem[];
  float *X0s = smem;                 // NI x NC column-major, unknown order
  float *Ds = X0s + NI * NC;         // NI x NC, sum of the corrections, unknown order
  float *Rs = Ds + NI * NC;          // NI x NC, residual, natural row order
  float *lbuf = Rs + NI * NC;        // 2 x NI
  float *ubuf = lbuf + 2 * NI;       // 2 x NCOL
  float *rdiag = ubuf + 2 * NCOL;    // NI
  int *perm = reinterpret_cast<int *>(rdiag + NI);  // NI: pivot row of step j
  int *spiv = perm + NI;             // 2 (double-buffered pivot row)
  const int t = threadIdx.x, tr = t % TR, tc = t / TR;
  for (int cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    const float *Ah = Ahi + (size_t)cell * N * N, *Al = Alo + (size_t)cell * N * N;
    const float *bh = bhi + (size_t)cell * N, *bl = blo + (size_t)cell * N;
    float W[RPT][CPT];
    int rk[RPT];
#pragma unroll
    for (int a = 0; a < RPT; ++a) {
      const int i = tr + TR * a;
      rk[a] = kRetiredNot;
#pragma unroll
      for (int b = 0; b < CPT; ++b) {
        const int c = tc + TC * b;
        float v = 0.0f;
        if (i < NI && c < N) v = Ah[i + (size_t)N * c];
        else if (i < NI && c == N) v = bh[i];
        W[a][b] = v;
      }
    }
    int cell_info = 0;
    // ---------------- LU with implicit partial pivoting ----------------
    for (int j = 0; j < NI; ++j) {
      const int buf = j & 1;
      const int tcj = j % TC, bj = j / TC;
      float best = -1.0f, bval = 0.0f;
      int bi = INT_MAX;
      if (tc == tcj) {
#pragma unroll
        for (int a = 0; a < RPT; ++a) {
          const int i = tr + TR * a;
          if (i < NI && rk[a] == kRetiredNot) {
            const float v = colget(W[a], bj), av = fabsf(v);
            if (av > best || (av == best && i < bi)) {
              best = av;
              bi = i;
              bval = v;
            }
          }
        }
      }
#pragma unroll
      for (int off = TR / 2; off >= 1; off >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        const float ov = __shfl_xor_sync(0xffffffffu, bval, off);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
          bval = ov;
        }
      }
      if (tc == tcj && tr == 0) {
        spiv[buf] = bi;
        rdiag[j] = bval != 0.0f ? 1.0f / bval : 0.0f;
        perm[j] = bi;
      }
      __syncthreads();
      const int p = spiv[buf];
      const float rp = rdiag[j];
      if (rp == 0.0f && !cell_info) cell_info = j + 1;
      const int trp = p % TR, ap = p / TR;
      if (tr == trp) {
#pragma unroll
        for (int b = 0; b < CPT; ++b) {
          const int c = tc + TC * b;
          if (c > j && c < NCOL) ubuf[buf * NCOL + c] = pick(W, ap, b);
        }
#pragma unroll
        for (int a = 0; a < RPT; ++a)
          if (a == ap) rk[a] = j;
      }
      if (tc == tcj) {
#pragma unroll
        for (int a = 0; a < RPT; ++a) {
          const int i = tr + TR * a;
          if (i < NI && rk[a] == kRetiredNot) {
            const float l = colget(W[a], bj) * rp;
            colset(W[a], bj, l);
            lbuf[buf * NI + i] = l;
          }
        }
      }
      __syncthreads();
#pragma unroll
      for (int a = 0; a < RPT; ++a) {
        const int i = tr + TR * a;
        if (i < NI && rk[a] == kRetiredNot) {
          const float l = lbuf[buf * NI + i];
#pragma unroll
          for (int b = 0; b < CPT; ++b) {
            const int c = tc + TC * b;
            if (c > j && c < NCOL) W[a][b] = fmaf(-l, ubuf[buf * NCOL + c], W[a][b]);
          }
        }
      }
    }
    __syncthreads();
    // ---------------- X0 = U^{-1} (L^{-1} P [A_if | b_i]) ----------------
    back_substitute<C>(W, rk, perm, rdiag, lbuf, ubuf, tr, tc);
#pragma unroll
    for (int a = 0; a < RPT; ++a) {
      const int i = tr + TR * a;
      if (i >= NI) continue;
#pragma unroll
      for (int b = 0; b < CPT; ++b) {
        const int c = tc + TC * b;
        if (c >= NI && c < NCOL) X0s[rk[a] + NI * (c - NI)] = W[a][b];
      }
    }
    __syncthreads();
    // ---------------- refinement: X += A_ii^{-1} ([A_if | b_i] - A_ii X) ----------------
    for (int step = 0; step < C::NSTEP; ++step) {
      residual<C>(Ah, Al, bh, bl, X0s, Ds, Rs, step > 0);
      // the L\U part of the tile is untouched; reload only the RHS columns
#pragma unroll
      for (int a = 0; a < RPT; ++a) {
        const int i = tr + TR * a;
#pragma unroll
        for (int b = 0; b < CPT; ++b) {
          const int c = tc + TC * b;
          if (i < NI && c >= NI && c < NCOL) W[a][b] = Rs[i + NI * (c - NI)];
        }
      }
      forward_eliminate<C>(W, rk, perm, lbuf, ubuf, tr, tc);
      back_substitute<C>(W, rk, perm, rdiag, lbuf, ubuf, tr, tc);
#pragma unroll
      for (int a = 0; a < RPT; ++a) {
        const int i = tr + TR * a;
        if (i >= NI) continue;
#pragma unroll
        for (int b = 0; b < CPT; ++b) {
          const int c = tc + TC * b;
          if (c >= NI && c < NCOL) {
            const int e = rk[a] + NI * (c - NI);
            Ds[e] = step == 0 ? W[a][b] : Ds[e] + W[a][b];
          }
        }
      }
      __syncthreads();
    }
    // ---------------- S = A_ff - A_fi X, g = b_f - A_fi y (float-float) ----------------
    for (int task = t; task < NF * NCHUNK; task += C::NT) {
      const int ar = task % NF, c0 = (task / NF) * CC;
      float hs[CC], ls[CC];
#pragma unroll
      for (int q = 0; q < CC; ++q) hs[q] = ls[q] = 0.0f;
      for (int k = 0; k < NI; ++k) {
        const float ah = __ldg(Ah + (NI + ar) + (size_t)N * k), al = __ldg(Al + (NI + ar) + (size_t)N * k);
#pragma unroll
        for (int q = 0; q < CC; ++q)
          if (c0 + q < NC) ff_mac2(hs[q], ls[q], ah, al, X0s[k + NI * (c0 + q)], Ds[k + NI * (c0 + q)]);
      }
#pragma unroll
      for (int q = 0; q < CC; ++q) {
        const int col = c0 + q;
        if (col < NC) {
          const double rhs = col < NF ? (double)__ldg(Ah + (NI + ar) + (size_t)N * (NI + col)) +
                                            (double)__ldg(Al + (NI + ar) + (size_t)N * (NI + col))
                                      : (double)bh[NI + ar] + (double)bl[NI + ar];
          const double v = rhs - ((double)hs[q] + (double)ls[q]);
          if (col < NF)
            S[(size_t)cell * NF * NF + ar + (size_t)NF * col] = v;
          else
            g[(size_t)cell * NF + ar] = v;
        }
      }
    }
    if (Xhi) {
      float *xh = Xhi + (size_t)cell * NI * NC, *xl = Xlo + (size_t)cell * NI * NC;
      for (int e = t; e < NI * NC; e += C::NT) {
        xh[e] = X0s[e];
        xl[e] = Ds[e];
      }
    }
    if (t == 0 && info) info[cell] = cell_info;
    __syncthreads();
  }
}

}  // namespace rt
}  // namespace hdg
