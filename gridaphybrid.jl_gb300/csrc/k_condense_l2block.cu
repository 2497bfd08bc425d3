// k_condense_l2block.cu -- static condensation by two-field block
// elimination with the panels in L2 (sm_103a), in float-float on the FP32
// pipes or in plain FP64 (the same algorithm: the FP64 path for cell blocks
// too large for the shared-memory LU).
//
// Cell DOFs: [field 1 s (NC1 comps x NK) | field 2 u (NC2 x NK) | trace f
// (2D facets x NC2 x NFS)], component-major.  Field 1's block is a reference
// mass matrix times a per-cell factor:
//   elasticity (s = symmetric stress, u = displacement, NC1 = D(D+1)/2,
//     NC2 = D): A_ss = |J| (C_nu (x) M_ref), C_nu[c][d] = E_c : A(E_d);
//   Darcy (s = flux, u = pressure, NC1 = D, NC2 = 1):
//     A_ss = (|J|/kappa) (I_D (x) M_ref);
// so A_ss^{-1} = (C^{-1} (x) M_ref^{-1}) with a small per-cell C^{-1} (6x6 at
// most) and the reference mass inverse; A_ss itself is never read.  With
// R = [A_sf | b_s] and R_u = [A_uf | b_u]:
//   Y = A_ss^{-1} A_su,  Z = A_ss^{-1} R      (never formed for A_su, A_sf: below)
//   P = A_uu - A_us Y,   Q = R_u - A_us Z    NU x NU, NU x NC (shared memory)
//   X_u = P^{-1} Q   (LU with partial pivoting of field 2's Schur complement)
//   X_s = Z - Y X_u                           NS x NC (per-CTA scratch, L2)
//   S = A_ff - A_fs X_s - A_fu X_u,   g = b_f - A_fs y_s - A_fu y_u
// The coupling blocks are per-cell coefficients times reference tables,
//   A_su[(c,a),(k,b)] = sum_e alpha[c][k][e] G_e[a][b],
//   A_sf[(c,a),(F,j,b)] = delta[c][j][F] H_F[a][b],
// so with the reference products MG_e = M^{-1} G_e and MH_F = M^{-1} H_F
//   Y[(c,a),(k,b)] = sum_e W_e[c][k] MG_e[a][b],   W_e = C^{-1} alpha_e,
//   Z[(c,a),(F,j,b)] = Dh[c][j][F] MH_F[a][b],     Dh = C^{-1} delta.
// On the tensor-product reference cell MG_e and MH_F have k+1 entries per
// column (a node couples along one lattice line); the products with Y and Z
// run over those entries only.
// Zeros are skipped (only exact zeros, so the results do not change):
//   - elasticity: A_us / A_su couple displacement component k only to the
//     stress components whose index pair contains k (every affine cell);
//   - A_fs / A_fu / A_sf couple a trace row of facet F only to the volume
//     nodes on F (Lagrange nodes off F vanish on F), found from the H table;
//   - per cell, the components a trace row/column of (F, trace component j)
//     couples to on those nodes, found by scanning the cell's entries (on
//     an axis-aligned cell: one stress or flux component, one displacement
//     component).
#include <cuda_runtime.h>

#include <type_traits>

#include "hdg_kernels.h"
#include "k_elast_cell.cuh"
#include "k_ff_cell.cuh"
#include "k_ffblock_cell.cuh"
#include "k_fp64_cell.cuh"

// threads per CTA for the largest cells (3D elasticity k=2, 3D Darcy k=3)
#ifndef HDG_L2BLOCK_BIG_NT
#define HDG_L2BLOCK_BIG_NT 512
#endif

namespace hdg {
namespace be {

// float-float values (hi, lo) on the FP32 pipes
struct ArFF {
  struct __align__(8) V {
    float h, l;
  };
  static __device__ __forceinline__ V zero() { return V{0.0f, 0.0f}; }
  static __device__ __forceinline__ void mac(V &c, V a, V b) { ffb::mac(c.h, c.l, a.h, a.l, b.h, b.l); }
  static __device__ __forceinline__ V fin(V a) {
    ffb::normalise(a.h, a.l);
    return a;
  }
  static __device__ __forceinline__ V sub(V a, V b) {
    V r;
    ffb::sub(a.h, a.l, b.h, b.l, r.h, r.l);
    return r;
  }
  static __device__ __forceinline__ V mul(V a, V b) {
    V r;
    ffb::mul(a.h, a.l, b.h, b.l, r.h, r.l);
    return r;
  }
  static __device__ __forceinline__ V div(V a, V b) {
    V r;
    ffb::div(a.h, a.l, b.h, b.l, r.h, r.l);
    return r;
  }
  static __device__ __forceinline__ float mag(V a) { return fabsf(a.h); }
  static __device__ __forceinline__ bool nonzero(V a) { return a.h != 0.0f; }
  static __device__ __forceinline__ double dbl(V a) { return (double)a.h + (double)a.l; }
  static __device__ __forceinline__ V of(double x) {
    V r;
    r.h = (float)x;
    r.l = (float)(x - (double)r.h);
    return r;
  }
  // element i of a (hi array, lo array) pair
  static __device__ __forceinline__ V ld(const void *p0, const void *p1, size_t i) {
    return V{__ldg(static_cast<const float *>(p0) + i), __ldg(static_cast<const float *>(p1) + i)};
  }
  static __device__ __forceinline__ void st(void *p0, void *p1, size_t i, V v) {
    static_cast<float *>(p0)[i] = v.h;
    static_cast<float *>(p1)[i] = v.l;
  }
  // the same through the coherent path (data written earlier in this kernel)
  static __device__ __forceinline__ V ldc(const void *p0, const void *p1, size_t i) {
    return V{static_cast<const float *>(p0)[i], static_cast<const float *>(p1)[i]};
  }
};

// plain FP64
struct Ar64 {
  using V = double;
  static __device__ __forceinline__ V zero() { return 0.0; }
  static __device__ __forceinline__ void mac(V &c, V a, V b) { c = fma(a, b, c); }
  static __device__ __forceinline__ V fin(V a) { return a; }
  static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
  static __device__ __forceinline__ V mul(V a, V b) { return a * b; }
  static __device__ __forceinline__ V div(V a, V b) { return a / b; }
  static __device__ __forceinline__ double mag(V a) { return fabs(a); }
  static __device__ __forceinline__ bool nonzero(V a) { return a != 0.0; }
  static __device__ __forceinline__ double dbl(V a) { return a; }
  static __device__ __forceinline__ V of(double x) { return x; }
  static __device__ __forceinline__ V ld(const void *p0, const void *, size_t i) {
    return __ldg(static_cast<const double *>(p0) + i);
  }
  static __device__ __forceinline__ void st(void *p0, void *, size_t i, V v) { static_cast<double *>(p0)[i] = v; }
  static __device__ __forceinline__ V ldc(const void *p0, const void *, size_t i) {
    return static_cast<const double *>(p0)[i];
  }
};

__host__ __device__ constexpr int ipow_c(int b, int e) { return e == 0 ? 1 : b * ipow_c(b, e - 1); }

template <int D_, int K_, bool ELAST_>
struct ECfg {
  static constexpr int D = D_, K = K_;
  static constexpr bool ELAST = ELAST_;
  static constexpr int NK = ipow_c(K + 1, D), NC1 = ELAST ? D * (D + 1) / 2 : D, NC2 = ELAST ? D : 1;
  static constexpr int NS = NC1 * NK, NU = NC2 * NK;
  static constexpr int NI = NS + NU, NFS = ipow_c(K + 1, D - 1), NFD = NC2 * NFS, NL = 2 * D, NF = NL * NFD;
  static constexpr int N = NI + NF, NC = NF + 1;
  // register-tile heights: rows of one field-2 component (phase 2), rows of
  // one facet and trace component (phase 6)
  static constexpr int TR = NK % 4 == 0 ? 4 : NK % 3 == 0 ? 3 : NK % 2 == 0 ? 2 : 1;
  static constexpr int TF = NFS % 4 == 0 ? 4 : NFS % 3 == 0 ? 3 : NFS % 2 == 0 ? 2 : 1;
  static constexpr int NT = ELAST && NU * NC >= 4096 ? HDG_L2BLOCK_BIG_NT : 256;
  // M^{-1} in shared memory, except where leaving it in L1 lets two CTAs share an SM
  static constexpr bool MI_SHARED = ELAST || NK < 64;
  // shared: P (NU x NU), Q (NU x NC), M^{-1} (NK x NK), C^{-1}/|J| (6 x 6),
  // the panel coefficients W (D x NC1 x NC2) and Dh (NC1 x NC2 x NL), as values
  // P's row stride
  static constexpr int LDP = NU;
  static constexpr size_t smem_values =
      (size_t)NU * LDP + (size_t)NU * NC + (MI_SHARED ? (size_t)NK * NK : 0) + 36 + 54 + 108;
  // per-CTA scratch, column-major, as values: Z / X_s (NS x NC), the products
  // T (D NU x NC); the fused kernel adds the cell block A (N x N) and b (N)
  static constexpr size_t slot_values = (size_t)NS * NC + (size_t)D * NU * NC;
  // the fused kernel stores only rows NS.. of the cell block (the field-1 rows
  // are never read: A_ss, A_su, A_sf enter through their factors)
  static constexpr int NR = N - NS;
  static constexpr size_t slot_values_fused = slot_values + (size_t)NR * N + N;
};

// shared-memory bookkeeping beside the value arrays
template <class C>
struct Lists {
  int fn_cnt[C::NL];          // volume nodes on local facet lf ...
  int fn_node[C::NL][C::NK];  // ... and their indices
  int fn_max;                 // max over facets of fn_cnt
  int kmask[3];               // bit c: field-1 component c couples to field-2 component k
  int kc_cnt[3], kc_comp[3][6];
  // this cell: bit c (field-1 component c) / bit NC1 + k (field-2 component k)
  // is set when a trace row or column of (facet lf, trace component j) has a
  // nonzero coupling to that component on the facet's nodes
  int fmask[C::NL][3];
  // the same couplings as a list per (facet, trace component): the cell-block
  // columns m (volume node on the facet x coupled component), node-major
  short slist[C::NL][3][C::NK * (C::NC1 + C::NC2)];
  int slen[C::NL][3];
  int piv, info;
  int pivs[8];        // the pivot rows of the current LU panel
  double cinv[6][6];  // C^{-1} / |J| of the cell (FP64)
  CellFactors cf;     // the cell's geometric factors (FP64)
};

template <class C, class Ar>
constexpr size_t smem_bytes() {
  return C::smem_values * sizeof(typename Ar::V) + sizeof(Lists<C>) + 16;
}

// Per-cell factors computed before the elimination, one thread per cell: the
// geometric factors and C^{-1}/|J| (elasticity: the inverse compliance;
// Darcy: kappa/|J| on the diagonal).  Computed inside the elimination they
// were FP64 divisions and square roots on one thread while the CTA waited.
struct CellPrep {
  CellFactors cf;
  double cinv[6][6];
  CellFactorsFF cff;  // Darcy: the float-float integration's factors
};

// the fused kernel's integration scratch: cell factors / terms, per-point
// source values (nqv x (D+1)), the row decode table (elasticity)
template <class C>
size_t integ_bytes(int nqv) {
  size_t fac = sizeof(ElastScratch);
  if (sizeof(CellFactors) > fac) fac = sizeof(CellFactors);
  if (sizeof(CellFactorsFF) > fac) fac = sizeof(CellFactorsFF);
  fac = (fac + 15) / 16 * 16;
  return fac + (size_t)nqv * (C::D + 1) * sizeof(double) + (size_t)C::N * sizeof(int) + 16;
}

// Cell `cell` integrated into the CTA's slot: rows NS..N-1 of A (column-major,
// leading dimension NR = N - NS) and the whole b, as (hi, lo) float arrays or
// FP64.  Row and column decoding divide by compile-time sizes.
template <class C, class Ar>
__device__ void integrate_into_slot(const L2BlockArgs &a, int cell, void *A0, void *A1, void *b0, void *b1,
                                    unsigned char *integ, int t) {
  constexpr int N = C::N, NT = C::NT, NS = C::NS, NR = C::NR, D = C::D, NK = C::NK, NI = C::NI, NFD = C::NFD;
  constexpr bool FF = !std::is_same<Ar, Ar64>::value;
  const CellArgs &ca = a.cell;
  size_t fac = sizeof(ElastScratch);
  if (sizeof(CellFactors) > fac) fac = sizeof(CellFactors);
  if (sizeof(CellFactorsFF) > fac) fac = sizeof(CellFactorsFF);
  fac = (fac + 15) / 16 * 16;
  double *fq = reinterpret_cast<double *>(integ + fac);
  int *dec = reinterpret_cast<int *>(fq + (size_t)ca.nqv * (C::D + 1));
  if constexpr (C::ELAST) {
    ElastScratch &S = *reinterpret_cast<ElastScratch *>(integ);
    for (int i = t; i < N; i += NT) dec[i] = elast_pack(ca, i);
    elast_cell_prepare(ca, cell, S, fq, FF, t, NT, &static_cast<const CellPrep *>(a.prep)[cell].cf);  // barriers inside
    for (int e = t; e < NR * N; e += NT) {
      const int j = e / NR, i = NS + (e - j * NR);
      if constexpr (FF) {
        float h, l;
        elast_entry_ff(ca, a.Tb, S.TF, dec[i], dec[j], h, l);
        static_cast<float *>(A0)[e] = h;
        static_cast<float *>(A1)[e] = l;
      } else {
        static_cast<double *>(A0)[e] = elast_entry_t(ca, S.f, S.T, dec[i], dec[j]);
      }
    }
    for (int r = t; r < N; r += NT) {
      const double v = elast_source_entry(ca, fq, r);
      if constexpr (FF) {
        split_double(v, static_cast<float *>(b0)[r], static_cast<float *>(b1)[r]);
      } else {
        static_cast<double *>(b0)[r] = v;
      }
    }
    __syncthreads();
  } else {
    // Darcy: the cell factors (float-float or FP64) and the source per point
    CellFactorsFF &fF = *reinterpret_cast<CellFactorsFF *>(integ);
    CellFactors &f6 = *reinterpret_cast<CellFactors *>(integ);
    {  // computed beforehand (l2block_prep_kernel), copied by the whole CTA
      const CellPrep &pp = static_cast<const CellPrep *>(a.prep)[cell];
      static_assert(sizeof(CellFactorsFF) % 4 == 0 && sizeof(CellFactors) % 4 == 0, "word copies");
      const unsigned *src = FF ? reinterpret_cast<const unsigned *>(&pp.cff) : reinterpret_cast<const unsigned *>(&pp.cf);
      unsigned *dst = reinterpret_cast<unsigned *>(integ);
      const int words = (int)((FF ? sizeof(CellFactorsFF) : sizeof(CellFactors)) / 4);
      for (int e = t; e < words; e += NT) dst[e] = src[e];
    }
    __syncthreads();
    {
      const double kap = ca.kappa ? ca.kappa[cell] : 1.0;
      for (int q = t; q < ca.nqv; q += NT) {
        double x[3], p, qe[3], fu[3], g;
        for (int d = 0; d < D; ++d) {
          x[d] = FF ? fF.x0[d] : f6.x0[d];
          for (int e = 0; e < D; ++e) x[d] += (FF ? fF.J[d][e] : f6.J[d][e]) * ca.qxi[q * D + e];
        }
        exact_solution(ca.problem, D, x, kap, p, qe, fu, g);
        const double w = ca.qw[q] * (FF ? fF.detJ : f6.detJ);
        for (int d = 0; d < D; ++d) fq[q * (D + 1) + d] = w * fu[d];
        fq[q * (D + 1) + D] = w * g;
      }
    }
    __syncthreads();
    for (int e = t; e < NR * N; e += NT) {
      const int j = e / NR, i = NS + (e - j * NR);
      int ti, si, ii, tj, sj, jj;
      decode_row(i, D, NK, NI, NFD, ti, si, ii);
      decode_row(j, D, NK, NI, NFD, tj, sj, jj);
      if constexpr (FF) {
        float h, l;
        cell_entry_ff(ca, a.Tb, fF, ti, si, ii, tj, sj, jj, h, l);
        static_cast<float *>(A0)[e] = h;
        static_cast<float *>(A1)[e] = l;
      } else {
        static_cast<double *>(A0)[e] = cell_entry<double>(ca, f6, ti, si, ii, tj, sj, jj);
      }
    }
    for (int r = t; r < N; r += NT) {
      int ti, si, ii;
      decode_row(r, D, NK, NI, NFD, ti, si, ii);
      double v = 0.0;
      if (ti < 2) {
        const int comp = ti == 0 ? si : D;
        for (int q = 0; q < ca.nqv; ++q) v += fq[q * (D + 1) + comp] * ca.qphi[q * NK + ii];
      }
      if constexpr (FF) {
        split_double(v, static_cast<float *>(b0)[r], static_cast<float *>(b1)[r]);
      } else {
        static_cast<double *>(b0)[r] = v;
      }
    }
    __syncthreads();
  }
}

// C_nu^{-1} / |J| in FP64: Gauss-Jordan with partial pivoting on the compliance
__device__ void compliance_inverse(int D, int nsym, double E, double nu, double detJ, double (*Ci)[6]) {
  double Cm[6][6], I[6][6];
  for (int c = 0; c < nsym; ++c)
    for (int d = 0; d < nsym; ++d) {
      double dd = 0.0, trc = 0.0, trd = 0.0;
      for (int r = 0; r < D; ++r) {
        trc += sym_unit(D, c, r, r);
        trd += sym_unit(D, d, r, r);
        for (int s = 0; s < D; ++s) dd += sym_unit(D, c, r, s) * sym_unit(D, d, r, s);
      }
      Cm[c][d] = (1.0 + nu) / E * dd - nu / E * trc * trd;
      I[c][d] = c == d ? 1.0 : 0.0;
    }
  for (int col = 0; col < nsym; ++col) {
    int pr = col;
    for (int i = col + 1; i < nsym; ++i)
      if (fabs(Cm[i][col]) > fabs(Cm[pr][col])) pr = i;
    for (int j = 0; j < nsym; ++j) {
      double t = Cm[col][j];
      Cm[col][j] = Cm[pr][j];
      Cm[pr][j] = t;
      t = I[col][j];
      I[col][j] = I[pr][j];
      I[pr][j] = t;
    }
    const double piv = 1.0 / Cm[col][col];
    for (int j = 0; j < nsym; ++j) {
      Cm[col][j] *= piv;
      I[col][j] *= piv;
    }
    for (int i = 0; i < nsym; ++i) {
      if (i == col) continue;
      const double f = Cm[i][col];
      for (int j = 0; j < nsym; ++j) {
        Cm[i][j] -= f * Cm[col][j];
        I[i][j] -= f * I[col][j];
      }
    }
  }
  for (int c = 0; c < nsym; ++c)
    for (int d = 0; d < nsym; ++d) Ci[c][d] = I[c][d] / detJ;
}

// One thread per cell (see CellPrep).
__global__ void __launch_bounds__(128) l2block_prep_kernel(CellArgs ca, int ncells, int elast, int nsym,
                                                           CellPrep *out) {
  const int D = ca.D;
  for (int cell = blockIdx.x * blockDim.x + threadIdx.x; cell < ncells; cell += gridDim.x * blockDim.x) {
    CellPrep p;
    cell_factors(ca, cell, p.cf);
    if (!elast) cell_factors_ff(ca, cell, p.cff);
    const double *J = ca.jac + (size_t)cell * D * D;
    const double det = D == 2 ? J[0] * J[3] - J[2] * J[1]
                              : J[0] * (J[4] * J[8] - J[7] * J[5]) - J[3] * (J[1] * J[8] - J[7] * J[2]) +
                                    J[6] * (J[1] * J[5] - J[4] * J[2]);
    if (elast) {
      compliance_inverse(D, nsym, ca.young, ca.kappa ? ca.kappa[cell] : 0.3, fabs(det), p.cinv);
    } else {  // kappa / |J| on the diagonal
      const double sc = (ca.kappa ? ca.kappa[cell] : 1.0) / fabs(det);
      for (int c = 0; c < 6; ++c)
        for (int d = 0; d < 6; ++d) p.cinv[c][d] = c == d ? sc : 0.0;
    }
    out[cell] = p;
  }
}

template <class C, class Ar, bool FUSED>
__global__ void __launch_bounds__(C::NT, C::MI_SHARED ? 1 : 2) condense_l2block_kernel(L2BlockArgs a) {
  using V = typename Ar::V;
  constexpr int D = C::D, NK = C::NK, NSYM = C::NC1, NC2 = C::NC2, NS = C::NS, NU = C::NU, NI = C::NI, NF = C::NF, N = C::N,
                NC = C::NC, NT = C::NT, NFD = C::NFD, NL = C::NL, NFS = C::NFS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *P = reinterpret_cast<V *>(smem_raw);  // [r][j]
  constexpr int LDP = C::LDP;
  V *Q = P + NU * LDP;                     // [r][c]
  V *Mi = Q + (size_t)NU * NC;             // [a][k]
  V *Ci = Mi + (C::MI_SHARED ? NK * NK : 0);  // [c][d]
  V *Wc = Ci + 36;                         // [(e NC1 + c) NC2 + k]
  V *Dh = Wc + 54;                         // [(c NC2 + j) NL + F]
  Lists<C> &L = *reinterpret_cast<Lists<C> *>(Dh + 108);
  unsigned char *integ = reinterpret_cast<unsigned char *>(&L + 1);
  integ += (16 - reinterpret_cast<uintptr_t>(integ) % 16) % 16;
  constexpr size_t slot = FUSED ? C::slot_values_fused : C::slot_values;
  V *Z = static_cast<V *>(a.scratch) + (size_t)blockIdx.x * slot;  // [m + NS c]
  V *Tp = Z + (size_t)NS * NC;                                     // [(e NU + u) + D NU c]
  // the fused kernel's cell block in the slot: (hi, lo) float arrays or FP64
  V *slotA = Tp + (size_t)D * NU * NC;
  // sparse reference products
  const int *rcp = a.ref_idx, *rci = a.ref_idx + a.off_cidx;  // MG by column
  const int *rrp = a.ref_idx + a.off_rptr, *rri = a.ref_idx + a.off_ridx;  // MG by row
  const int *rhp = a.ref_idx + a.off_hptr, *rhi = a.ref_idx + a.off_hidx;  // MH by column
  auto RV = [&](int i) { return Ar::ld(a.ref_v0, a.ref_v1, (size_t)i); };
  void *sA0 = slotA, *sA1 = nullptr, *sb0 = nullptr, *sb1 = nullptr;
  constexpr int NR = C::NR;
  if constexpr (sizeof(V) == 8 && !std::is_same<Ar, Ar64>::value) {
    sA1 = reinterpret_cast<float *>(slotA) + (size_t)NR * N;
    sb0 = reinterpret_cast<float *>(slotA) + 2 * (size_t)NR * N;
    sb1 = reinterpret_cast<float *>(slotA) + 2 * (size_t)NR * N + N;
  } else {
    sb0 = reinterpret_cast<double *>(slotA) + (size_t)NR * N;
  }
  const CellArgs &ca = a.cell;
  const int t = threadIdx.x;
  if constexpr (C::MI_SHARED)
    for (int e = t; e < NK * NK; e += NT) Mi[e] = Ar::ld(a.Minv0, a.Minv1, e);
  auto MI = [&](int i) {
    if constexpr (C::MI_SHARED)
      return Mi[i];
    else
      return Ar::ld(a.Minv0, a.Minv1, (size_t)i);
  };
  if (t < NL) {  // volume nodes with a nonzero trace coupling on facet t
    int cnt = 0;
    for (int node = 0; node < NK; ++node) {
      bool nz = false;
      for (int b = 0; b < NFS; ++b) nz |= ca.H[((size_t)t * NK + node) * NFS + b] != 0.0;
      if (nz) L.fn_node[t][cnt++] = node;
    }
    L.fn_cnt[t] = cnt;
  }
  __syncthreads();
  if (t == 0) {
    int mx = 0;
    for (int lf = 0; lf < NL; ++lf) mx = max(mx, L.fn_cnt[lf]);
    L.fn_max = mx;
  }
  if (t == 0) {
    for (int k = 0; k < NC2; ++k) {
      int m = 0, cnt = 0;
      for (int c = 0; c < NSYM; ++c) {
        bool couples = true;  // Darcy: the pressure couples to every flux component
        if (C::ELAST) {
          int i, j;
          sym_pair(D, c, i, j);
          couples = i == k || j == k;
        }
        if (couples) {
          m |= 1 << c;
          L.kc_comp[k][cnt++] = c;
        }
      }
      L.kmask[k] = m;
      L.kc_cnt[k] = cnt;
    }
  }
  for (int cell = blockIdx.x; cell < a.ncells; cell += gridDim.x) {
    const size_t A0 = FUSED ? 0 : (size_t)cell * N * N, b0 = FUSED ? 0 : (size_t)cell * N;
    auto A = [&](int r, int c) {  // rows r >= NS only
      if constexpr (FUSED)
        return Ar::ldc(sA0, sA1, (size_t)(r - NS) + (size_t)NR * c);
      else
        return Ar::ld(a.A0, a.A1, A0 + (size_t)r + (size_t)N * c);
    };
    auto B = [&](int r) {
      if constexpr (FUSED)
        return Ar::ldc(sb0, sb1, (size_t)r);
      else
        return Ar::ld(a.b0, a.b1, b0 + r);
    };
    __syncthreads();  // the previous cell's readers of the lists / Ci / slot are done
    if constexpr (FUSED) integrate_into_slot<C, Ar>(a, cell, sA0, sA1, sb0, sb1, integ, t);
    {  // the cell's factors and C^{-1}/|J|, computed beforehand (l2block_prep_kernel)
      const CellPrep &pp = static_cast<const CellPrep *>(a.prep)[cell];
      for (int e = t; e < NSYM * NSYM; e += NT) {
        const int c = e / NSYM, d = e - c * NSYM;
        const double v = pp.cinv[c][d];
        Ci[c * 6 + d] = Ar::of(v);
        L.cinv[c][d] = v;
      }
      for (int e = t; e < (int)(sizeof(CellFactors) / sizeof(double)); e += NT)
        reinterpret_cast<double *>(&L.cf)[e] = reinterpret_cast<const double *>(&pp.cf)[e];
      if (t == 0) L.info = 0;
    }
    if (t < NL * 3) L.fmask[t / 3][t % 3] = 0;
    __syncthreads();
    // panel coefficients W_e = C^{-1} alpha_e and Dh = C^{-1} delta (FP64,
    // the integration's own factors: alpha, delta are its coefficients of G, H)
    for (int o = t; o < D * NSYM * NC2 + NSYM * NC2 * NL; o += NT) {
      double v = 0.0;
      if (o < D * NSYM * NC2) {
        const int e = o / (NSYM * NC2), c = (o / NC2) % NSYM, k = o % NC2;
        for (int cp = 0; cp < NSYM; ++cp) {
          double al;
          if (C::ELAST) {  // -sum_jj E_cp(k, jj) cg[e][jj]  (the (div v).u term)
            al = 0.0;
            for (int jj = 0; jj < D; ++jj) al += sym_unit(D, cp, k, jj) * L.cf.cg[e][jj];
            al = -al;
          } else {  // cg[e][d] (the -(div v) p term)
            al = L.cf.cg[e][cp];
          }
          v += L.cinv[c][cp] * al;
        }
        Wc[o] = Ar::of(v);
      } else {
        const int r = o - D * NSYM * NC2, c = r / (NC2 * NL), j = (r / NL) % NC2, F = r % NL;
        for (int cp = 0; cp < NSYM; ++cp) {
          double de;
          if (C::ELAST) {  // -sum_jj E_cp(j, jj) cn[F][jj]  (the -(v.n).uhat term)
            de = 0.0;
            for (int jj = 0; jj < D; ++jj) de += sym_unit(D, cp, j, jj) * L.cf.cn[F][jj];
            de = -de;
          } else {  // cn[F][d]  (the (v.n) l term)
            de = L.cf.cn[F][cp];
          }
          v += L.cinv[c][cp] * de;
        }
        Dh[r] = Ar::of(v);
      }
    }
    // the cell's trace couplings: entries of A_fi on the facet's nodes that
    // are exactly zero are skipped below (they contribute nothing)
    {
      const int fm = L.fn_max;
      for (int e = t; e < NF * (NSYM + NC2) * fm; e += NT) {
        const int f = e % NF, rest = e / NF, cc = rest % (NSYM + NC2), q = rest / (NSYM + NC2);
        const int lf = f / NFD, kf = (f - lf * NFD) / NFS;
        if (q >= L.fn_cnt[lf]) continue;
        const int node = L.fn_node[lf][q];
        const int m = cc < NSYM ? cc * NK + node : NS + (cc - NSYM) * NK + node;
        if (Ar::nonzero(A(NI + f, m))) atomicOr(&L.fmask[lf][kf], 1 << cc);
      }
    }
    __syncthreads();
    // the coupling lists of the S phase, from the masks
    for (int pr = t; pr < NL * (NFD / NFS); pr += NT) {
      const int lf = pr / (NFD / NFS), kf = pr - lf * (NFD / NFS), msk = L.fmask[lf][kf];
      int len = 0;
      for (int q = 0; q < L.fn_cnt[lf]; ++q) {
        const int node = L.fn_node[lf][q];
        for (int cc = 0; cc < NSYM + NC2; ++cc)
          if (msk >> cc & 1) L.slist[lf][kf][len++] = (short)(cc < NSYM ? cc * NK + node : NS + (cc - NSYM) * NK + node);
      }
      L.slen[lf][kf] = len;
    }
    __syncthreads();
    // 1. the b column of Z: A_ss^{-1} b_s (M^{-1} on each field-1 component,
    //    then the components mixed by C^{-1})
    for (int an = t; an < NK; an += NT) {
      V T[NSYM];
#pragma unroll
      for (int cp = 0; cp < NSYM; ++cp) {
        T[cp] = Ar::zero();
        for (int k = 0; k < NK; ++k) Ar::mac(T[cp], MI(an * NK + k), B(cp * NK + k));
        T[cp] = Ar::fin(T[cp]);
      }
#pragma unroll
      for (int c = 0; c < NSYM; ++c) {
        V v = Ar::zero();
#pragma unroll
        for (int cp = 0; cp < NSYM; ++cp) Ar::mac(v, Ci[c * 6 + cp], T[cp]);
        Z[c * NK + an + (size_t)NS * NF] = Ar::fin(v);
      }
    }
    __syncthreads();
    // 2. P = A_uu - A_us Y,  Q = [A_uf | b_u] - A_us Z, register tiles of TR
    //    rows (one field-2 component) x one column; Y, Z through their factors
    {
      constexpr int TR = C::TR, RT = NU / TR;
      for (int o = t; o < RT * (NU + NC); o += NT) {
        const int r0 = (o % RT) * TR, col = o / RT, kr = r0 / NK;
        V acc[TR];
#pragma unroll
        for (int i = 0; i < TR; ++i) acc[i] = Ar::zero();
        const int cnt = L.kc_cnt[kr];  // A_us: only these field-1 components couple to row component kr
        if (col < NU) {  // Y column (k, b): sum_c sum_e W_e[c][k] sum_a A_us[r][(c,a)] MG_e[a][b]
          const int k = col / NK, b = col - k * NK;
          for (int q = 0; q < cnt; ++q) {
            const int c = L.kc_comp[kr][q];
            for (int e = 0; e < D; ++e) {
              const V w = Wc[(e * NSYM + c) * NC2 + k];
              if (!Ar::nonzero(w)) continue;
              V sm[TR];
#pragma unroll
              for (int i = 0; i < TR; ++i) sm[i] = Ar::zero();
              for (int p = rcp[e * NK + b]; p < rcp[e * NK + b + 1]; ++p) {
                const int am = c * NK + rci[p];
                const V rv = RV(a.voff_c + p);
#pragma unroll
                for (int i = 0; i < TR; ++i) Ar::mac(sm[i], A(NS + r0 + i, am), rv);
              }
#pragma unroll
              for (int i = 0; i < TR; ++i) Ar::mac(acc[i], Ar::fin(sm[i]), w);
            }
          }
        } else if (col < NU + NF) {  // Z facet column (F, j, b): sum_c Dh[c][j][F] sum_a A_us[r][(c,a)] MH_F[a][b]
          const int f = col - NU, F = f / NFD, j = (f - F * NFD) / NFS, b = f % NFS;
          for (int q = 0; q < cnt; ++q) {
            const int c = L.kc_comp[kr][q];
            const V w = Dh[(c * NC2 + j) * NL + F];
            if (!Ar::nonzero(w)) continue;
            V sm[TR];
#pragma unroll
            for (int i = 0; i < TR; ++i) sm[i] = Ar::zero();
            for (int p = rhp[F * NFS + b]; p < rhp[F * NFS + b + 1]; ++p) {
              const int am = c * NK + rhi[p];
              const V rv = RV(a.voff_h + p);
#pragma unroll
              for (int i = 0; i < TR; ++i) Ar::mac(sm[i], A(NS + r0 + i, am), rv);
            }
#pragma unroll
            for (int i = 0; i < TR; ++i) Ar::mac(acc[i], Ar::fin(sm[i]), w);
          }
        } else {  // the b column of Z (dense)
          for (int q = 0; q < cnt; ++q) {
            const int m0 = L.kc_comp[kr][q] * NK;
            for (int k = 0; k < NK; ++k) {
              const V zv = Z[m0 + k + (size_t)NS * NF];
#pragma unroll
              for (int i = 0; i < TR; ++i) Ar::mac(acc[i], A(NS + r0 + i, m0 + k), zv);
            }
          }
        }
#pragma unroll
        for (int i = 0; i < TR; ++i) {
          const int r = r0 + i;
          const V rv = col < NU ? A(NS + r, NS + col) : col - NU < NF ? A(NS + r, NI + col - NU) : B(NS + r);
          const V v = Ar::sub(rv, Ar::fin(acc[i]));
          if (col < NU)
            P[r * LDP + col] = v;
          else
            Q[r * NC + col - NU] = v;
        }
      }
    }
    __syncthreads();
    // 3. blocked LU with partial pivoting of [P | Q], panels of NB columns:
    //    warp 0 factors the panel (pivot search, row swaps and updates inside
    //    the panel, __syncwarp only); then the CTA applies the panel's swaps to
    //    the trailing columns, solves the panel's block row and updates the
    //    trailing matrix with register tiles (rank-NB).  The multipliers of L
    //    are not swapped (only U and the transformed Q are used later).
    {
      constexpr int NB = 8, TCW = NU + NC;  // columns of [P | Q]
      auto W = [&](int r, int c) -> V & { return c < NU ? P[r * LDP + c] : Q[r * NC + (c - NU)]; };
      for (int j0 = 0; j0 < NU; j0 += NB) {
        const int nb = min(NB, NU - j0);
        if (t < 32) {
          for (int jj = j0; jj < j0 + nb; ++jj) {
            auto best = Ar::mag(Ar::zero()) - 1;
            int bi = jj;
            for (int i = jj + t; i < NU; i += 32) {
              const auto v = Ar::mag(P[i * LDP + jj]);
              if (v > best) {
                best = v;
                bi = i;
              }
            }
            for (int off = 16; off > 0; off >>= 1) {
              const auto ob = __shfl_xor_sync(0xffffffffu, best, off);
              const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
              if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
              }
            }
            if (t == 0) {
              L.pivs[jj - j0] = bi;
              if (!(best > 0) && L.info == 0) L.info = jj + 1;
            }
            if (bi != jj && t < nb) {  // swap rows jj and bi inside the panel
              const V tmp = P[jj * LDP + j0 + t];
              P[jj * LDP + j0 + t] = P[bi * LDP + j0 + t];
              P[bi * LDP + j0 + t] = tmp;
            }
            __syncwarp();
            const V pv = P[jj * LDP + jj];
            for (int i = jj + 1 + t; i < NU; i += 32) {
              const V l = Ar::nonzero(pv) ? Ar::div(P[i * LDP + jj], pv) : Ar::zero();
              P[i * LDP + jj] = l;
              for (int c = jj + 1; c < j0 + nb; ++c) P[i * LDP + c] = Ar::sub(P[i * LDP + c], Ar::mul(l, P[jj * LDP + c]));
            }
            __syncwarp();
          }
        }
        __syncthreads();
        // the panel's swaps on the trailing columns, then its block row U12 = L11^{-1} A12
        for (int c = j0 + nb + t; c < TCW; c += NT) {
          for (int q = 0; q < nb; ++q) {
            const int pr = L.pivs[q];
            if (pr != j0 + q) {
              const V tmp = W(j0 + q, c);
              W(j0 + q, c) = W(pr, c);
              W(pr, c) = tmp;
            }
          }
          for (int i = 1; i < nb; ++i) {
            V acc = Ar::zero();
            for (int m = 0; m < i; ++m) Ar::mac(acc, P[(j0 + i) * LDP + j0 + m], W(j0 + m, c));
            W(j0 + i, c) = Ar::sub(W(j0 + i, c), Ar::fin(acc));
          }
        }
        __syncthreads();
        // trailing update: W[i][c] -= L21[i][.] U12[.][c], tiles of 4 rows x 4 columns
        {
          const int r0 = j0 + nb, rows = NU - r0, c0s = j0 + nb, cols = TCW - c0s;
          const int RTt = (rows + 3) / 4, CTt = (cols + 3) / 4;
          for (int o = t; o < RTt * CTt; o += NT) {  // columns fastest: L broadcast, U rows contiguous
            const int cb = c0s + (o % CTt), ib = r0 + (o / CTt) * 4;  // columns cb + j CTt
            V acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[i][j] = Ar::zero();
            for (int m = 0; m < nb; ++m) {
              V lv[4], uv[4];
#pragma unroll
              for (int i = 0; i < 4; ++i) lv[i] = P[min(ib + i, NU - 1) * LDP + j0 + m];
#pragma unroll
              for (int j = 0; j < 4; ++j) uv[j] = W(j0 + m, min(cb + j * CTt, TCW - 1));
#pragma unroll
              for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) Ar::mac(acc[i][j], lv[i], uv[j]);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j)
                if (ib + i < NU && cb + j * CTt < TCW)
                  W(ib + i, cb + j * CTt) = Ar::sub(W(ib + i, cb + j * CTt), Ar::fin(acc[i][j]));
          }
        }
        __syncthreads();
      }
    }
    // 4. blocked back substitution X_u = U^{-1} Q, in Q: the diagonal block of
    //    NB rows column by column, then the rows above by register tiles
    {
      constexpr int NB = 8;
      for (int i1 = NU; i1 > 0; i1 -= NB) {
        const int i0 = max(0, i1 - NB);
        for (int c = t; c < NC; c += NT)
          for (int i = i1 - 1; i >= i0; --i) {
            V acc = Ar::zero();
            for (int m = i + 1; m < i1; ++m) Ar::mac(acc, P[i * LDP + m], Q[m * NC + c]);
            const V pv = P[i * LDP + i];
            const V r = Ar::sub(Q[i * NC + c], Ar::fin(acc));
            Q[i * NC + c] = Ar::nonzero(pv) ? Ar::div(r, pv) : Ar::zero();
          }
        __syncthreads();
        const int RTt = (i0 + 3) / 4, CTt = (NC + 3) / 4;
        for (int o = t; o < RTt * CTt; o += NT) {  // columns fastest
          const int cb = o % CTt, ib = (o / CTt) * 4;  // columns cb + j CTt
          V acc[4][4];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = Ar::zero();
          for (int m = i0; m < i1; ++m) {
            V lv[4], xv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) lv[i] = P[min(ib + i, i0 - 1) * LDP + m];
#pragma unroll
            for (int j = 0; j < 4; ++j) xv[j] = Q[m * NC + min(cb + j * CTt, NC - 1)];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j) Ar::mac(acc[i][j], lv[i], xv[j]);
          }
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
              if (ib + i < i0 && cb + j * CTt < NC)
                Q[(ib + i) * NC + cb + j * CTt] = Ar::sub(Q[(ib + i) * NC + cb + j * CTt], Ar::fin(acc[i][j]));
        }
        __syncthreads();
      }
    }
    // 5. X_s = Z - Y X_u = Z - sum_e sum_k W_e[:][k] (MG_e X_u[(k, .)]):
    //    first T_e[(k,a)][c] = sum_b MG_e[a][b] X_u[(k,b)][c] (4 columns per thread)
    {
      constexpr int CT = (NC + 3) / 4;
      for (int o = t; o < D * NU * CT; o += NT) {
        const int c0 = o % CT, row = o / CT, e = row / NU, u = row - e * NU, k = u / NK, an = u - k * NK;  // columns c0 + j CT
        V acc[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = Ar::zero();
        for (int p = rrp[e * NK + an]; p < rrp[e * NK + an + 1]; ++p) {
          const V rv = RV(a.voff_r + p);
          const V *xq = Q + (k * NK + rri[p]) * NC;
#pragma unroll
          for (int j = 0; j < 4; ++j) Ar::mac(acc[j], rv, xq[min(c0 + j * CT, NC - 1)]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (c0 + j * CT < NC) Tp[(size_t)(e * NU + u) + (size_t)D * NU * (c0 + j * CT)] = Ar::fin(acc[j]);
      }
    }
    __syncthreads();
    //    then X_s[(c,a)][col] = Z[(c,a)][col] - sum_e sum_k W_e[c][k] T_e[(k,a)][col],
    //    Z's facet columns from their factors, its b column in place
    {
      constexpr int CT = (NC + 3) / 4;
      for (int o = t; o < NS * CT; o += NT) {
        const int c0 = o % CT, m = o / CT, c = m / NK, an = m - c * NK;  // columns c0 + j CT
        V acc[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = Ar::zero();
        for (int e = 0; e < D; ++e)
          for (int k = 0; k < NC2; ++k) {
            const V w = Wc[(e * NSYM + c) * NC2 + k];
            if (!Ar::nonzero(w)) continue;
            const V *tp = Tp + (size_t)(e * NU + k * NK + an);
#pragma unroll
            for (int j = 0; j < 4; ++j) Ar::mac(acc[j], w, tp[(size_t)D * NU * min(c0 + j * CT, NC - 1)]);
          }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int col = c0 + j * CT;
          if (col >= NC) continue;
          V z;
          if (col < NF) {
            const int F = col / NFD, jj = (col - F * NFD) / NFS, b = col % NFS;
            z = Ar::mul(Dh[(c * NC2 + jj) * NL + F], RV(a.voff_hd + (F * NK + an) * NFS + b));
          } else {
            z = Z[m + (size_t)NS * NF];
          }
          Z[m + (size_t)NS * col] = Ar::sub(z, Ar::fin(acc[j]));
        }
      }
    }
    __syncthreads();
    // 6. S = A_ff - A_fs X_s - A_fu X_u and g, over the volume nodes on the
    //    rows' facet: register tiles of TF rows (one facet) x 4 columns
    {
      constexpr int TF = C::TF, FT = NF / TF, CT = (NC + 3) / 4;
      for (int o = t; o < FT * CT; o += NT) {
        const int f0 = (o % FT) * TF, c0 = (o / FT) * 4, lf = f0 / NFD, kf = (f0 - lf * NFD) / NFS;
        const short *lst = L.slist[lf][kf];  // the tile's rows share (lf, trace component)
        const int len = L.slen[lf][kf];
        int cj[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) cj[j] = min(c0 + j, NC - 1);
        V acc[TF][4];
#pragma unroll
        for (int i = 0; i < TF; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = Ar::zero();
        auto load = [&](int m, V *av, V *xv) {
#pragma unroll
          for (int i = 0; i < TF; ++i) av[i] = A(NI + f0 + i, m);
#pragma unroll
          for (int j = 0; j < 4; ++j) xv[j] = m < NS ? Z[m + (size_t)NS * cj[j]] : Q[(m - NS) * NC + cj[j]];
        };
        auto macs = [&](const V *av, const V *xv) {
#pragma unroll
          for (int i = 0; i < TF; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) Ar::mac(acc[i][j], av[i], xv[j]);
        };
        // two list entries per step, their loads issued together (the sums
        // keep the list order: the same bits as one entry at a time)
        int q = 0;
        for (; q + 1 < len; q += 2) {
          V av0[TF], xv0[4], av1[TF], xv1[4];
          load(lst[q], av0, xv0);
          load(lst[q + 1], av1, xv1);
          macs(av0, xv0);
          macs(av1, xv1);
        }
        if (q < len) {
          V av0[TF], xv0[4];
          load(lst[q], av0, xv0);
          macs(av0, xv0);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int c = c0 + j;
          if (c >= NC) continue;
#pragma unroll
          for (int i = 0; i < TF; ++i) {
            const int f = f0 + i;
            const V rhs = c < NF ? A(NI + f, NI + c) : B(NI + f);
            const double v = Ar::dbl(rhs) - Ar::dbl(Ar::fin(acc[i][j]));
            if (c < NF)
              a.S[(size_t)cell * NF * NF + f + (size_t)NF * c] = v;
            else
              a.g[(size_t)cell * NF + f] = v;
          }
        }
      }
    }
    // 7. X = [X_s; X_u] (NI x NC, column-major) for the recovery
    if (a.X0) {
      const size_t x0 = (size_t)cell * NI * NC;
      for (int e = t; e < NI * NC; e += NT) {
        const int c = e / NI, m = e - c * NI;
        Ar::st(a.X0, a.X1, x0 + e, m < NS ? Z[m + (size_t)NS * c] : Q[(m - NS) * NC + c]);
      }
    }
    if (t == 0 && a.info) a.info[cell] = L.info;
  }
}

template <class C, class Ar, bool FUSED>
cudaError_t launch_cfg(const L2BlockArgs &args, const L2BlockLaunch &L, cudaStream_t s, long long *launches) {
  auto kern = condense_l2block_kernel<C, Ar, FUSED>;
  const size_t smem = smem_bytes<C, Ar>() + (FUSED ? integ_bytes<C>(L.nqv) + 16 : 0);
  if (smem > L.smem_optin) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  long long grid = (long long)per_sm * L.num_sms;
  if (grid > args.ncells) grid = args.ncells;
  if (grid < 1) grid = 1;
  const size_t slots = ((size_t)grid * (FUSED ? C::slot_values_fused : C::slot_values) * sizeof(typename Ar::V) + 255) /
                       256 * 256;
  const size_t need = slots + (size_t)args.ncells * sizeof(CellPrep);
  if (L.scratch_bytes_out) *L.scratch_bytes_out = need;
  if (L.dry_run) return cudaSuccess;
  if (need > L.scratch_bytes || !args.scratch) return cudaErrorMemoryAllocation;
  L2BlockArgs a2 = args;
  CellPrep *prep = reinterpret_cast<CellPrep *>(static_cast<char *>(args.scratch) + slots);
  a2.prep = prep;
  int pg = (args.ncells + 127) / 128;
  if (pg > L.num_sms * 16) pg = L.num_sms * 16;
  if (pg < 1) pg = 1;
  l2block_prep_kernel<<<pg, 128, 0, s>>>(args.cell, args.ncells, C::ELAST ? 1 : 0, C::NC1, prep);
  kern<<<(int)grid, C::NT, smem, s>>>(a2);
  *launches += 2;
  return cudaGetLastError();
}

}  // namespace be

bool l2block_supported(bool elasticity, int D, int k) {
  if (elasticity) return (D == 2 && k >= 1 && k <= 3) || (D == 3 && k >= 1 && k <= 2);
  return D == 3 && k == 3;  // Darcy: the shared-memory block elimination covers D=2, k<=3 and D=3, k<=2
}

cudaError_t launch_condense_l2block(const L2BlockArgs &args, const L2BlockLaunch &L, cudaStream_t s,
                                    long long *launches) {
  // fused (integration in the slot): float-float and FP64; cell blocks from
  // HBM: FP64 only (the Newton path keeps them for its residuals)
  if (!L.fused && !L.fp64) return cudaErrorInvalidValue;
#define HDG_L2B(EL, DD, KK)                                                                        \
  if (L.elasticity == EL && L.D == DD && L.k == KK) {                                              \
    using CF = be::ECfg<DD, KK, EL>;                                                               \
    if (!L.fused) return be::launch_cfg<CF, be::Ar64, false>(args, L, s, launches);                \
    return L.fp64 ? be::launch_cfg<CF, be::Ar64, true>(args, L, s, launches)                       \
                  : be::launch_cfg<CF, be::ArFF, true>(args, L, s, launches);                      \
  }
  HDG_L2B(true, 2, 1)
  HDG_L2B(true, 2, 2)
  HDG_L2B(true, 2, 3)
  HDG_L2B(true, 3, 1)
  HDG_L2B(true, 3, 2)
  HDG_L2B(false, 3, 3)
#undef HDG_L2B
  return cudaErrorInvalidValue;
}

// u = y - X_f x_f per cell, X = [X_f | y] (ni x (nf+1), column-major, FP64)
__global__ void __launch_bounds__(128) recover_x64_kernel(CellArgs a, const double *__restrict__ X,
                                                          const double *__restrict__ lambda,
                                                          const double *__restrict__ dirvals, double *uint) {
  __shared__ double xf[6 * 64];
  const int ni = a.ni, nf = a.nf, nfd = a.nfd, nl = 2 * a.D, nc = nf + 1;
  for (int c = blockIdx.x; c < a.ncells; c += gridDim.x) {
    for (int e = threadIdx.x; e < nf; e += blockDim.x) {
      const int lf = e / nfd, j = e - lf * nfd;
      const int id = a.facet_dofs[(size_t)a.cell_facets[(size_t)c * nl + lf] * nfd + j];
      xf[e] = id >= 0 ? lambda[id] : dirvals[-1 - id];
    }
    __syncthreads();
    const double *x = X + (size_t)c * ni * nc;
    for (int i = threadIdx.x; i < ni; i += blockDim.x) {
      double v = x[i + (size_t)ni * nf];
      for (int j = 0; j < nf; ++j) v -= x[i + (size_t)ni * j] * xf[j];
      uint[(size_t)c * ni + i] = v;
    }
    __syncthreads();
  }
}

cudaError_t launch_recover_x64(const CellArgs &a, const double *X, const double *lambda, const double *dirvals,
                               double *uint, cudaStream_t s, int num_sms, long long *launches) {
  if (a.nf > 6 * 64) return cudaErrorInvalidValue;
  int grid = a.ncells < num_sms * 8 ? a.ncells : num_sms * 8;
  if (grid < 1) grid = 1;
  recover_x64_kernel<<<grid, 128, 0, s>>>(a, X, lambda, dirvals, uint);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace hdg
