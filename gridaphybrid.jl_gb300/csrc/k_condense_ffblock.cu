// k_condense_ffblock.cu -- static condensation of the Darcy HDG cell blocks by
// block elimination, entirely in float-float on the FP32 pipes (sm_103a).
//
// With a per-cell scalar permeability the flux block of the cell matrix is
//   A_uu = m (I_D (x) M_ref),   m = |det J| / kappa,
// (D identical reference mass matrices), so A_uu^{-1} = (1/m) (I_D (x) M_ref^{-1})
// with M_ref^{-1} inverted once on the host.  With G_d = A_{u_d p},
// G'_d = A_{p u_d}, T = A_pp and the right-hand sides R = [A_if | b_i]:
//   Y_d = (1/m) M^{-1} G_d                 P = T - sum_d G'_d Y_d   (NK x NK)
//   Z_d = (1/m) M^{-1} R_{u_d}             Q = R_p - sum_d G'_d Z_d
//   X_p = P^{-1} Q (LU with partial pivoting of the NK x NK pressure Schur)
//   X_{u_d} = Z_d - Y_d X_p
//   S = A_ff - A_fi X,   g = b_f - A_fi y
// Y_d comes from the reference products M^{-1} G_e (exactly sparse on the
// tensor-product cell) and per-cell coefficients; P, X_u, Z, Q and S skip the
// exactly-zero entries.  The only sequential part is the NK-step LU of P.  Every value is a float-float pair (~48 significant bits),
// so no refinement is needed (S agrees with the FP64 elimination to ~1e-14).
#include <cuda_runtime.h>

#include <algorithm>

#include "hdg_kernels.h"
#include "k_ff_cell.cuh"
#include "k_ffblock_cell.cuh"
#include "k_fp64_cell.cuh"

namespace hdg {
namespace ffb {

template <class C>
__global__ void __launch_bounds__(C::NT, 3)
    condense_ffblock_kernel(int ncells, const float *__restrict__ Ahi, const float *__restrict__ Alo,
                            const float *__restrict__ bhi, const float *__restrict__ blo,
                            const float *__restrict__ Minv_h, const float *__restrict__ Minv_l,
                            const float *__restrict__ MG_h, const float *__restrict__ MG_l,
                            const int *__restrict__ pat, const double *__restrict__ coef, double *S, double *g,
                            float *Xhi, float *Xlo, int *info) {
  constexpr int N = C::N, NF = C::NF, NI = C::NI, NC = C::NC;
  extern __shared__ float smem[];
  for (int cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    ffblock_cell<C, C::NT, true>(true, Ahi + (size_t)cell * N * N, Alo + (size_t)cell * N * N, bhi + (size_t)cell * N,
                                 blo + (size_t)cell * N, Minv_h, Minv_l, MG_h, MG_l, pat, coef + 10 * (size_t)cell, smem,
                                 S + (size_t)cell * NF * NF,
                                 g + (size_t)cell * NF, Xhi ? Xhi + (size_t)cell * NI * NC : nullptr,
                                 Xlo ? Xlo + (size_t)cell * NI * NC : nullptr, info ? info + cell : nullptr,
                                 threadIdx.x);
  }
}


template <class C>
static cudaError_t launch_cfg(int ncells, const float *Ahi, const float *Alo, const float *bhi, const float *blo,
                              const float *Mh, const float *Ml, const float *MGh, const float *MGl,
                              const int *pat, const double *coef, double *S, double *g, float *Xhi, float *Xlo,
                              int *info, cudaStream_t s, int num_sms) {
  const size_t smem = C::smem_bytes;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(condense_ffblock_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  cudaError_t oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, condense_ffblock_kernel<C>, C::NT, smem);
  if (oe != cudaSuccess) return oe;
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  if (grid > ncells) grid = ncells;
  if (grid < 1) grid = 1;
  condense_ffblock_kernel<C><<<grid, C::NT, smem, s>>>(ncells, Ahi, Alo, bhi, blo, Mh, Ml, MGh, MGl, pat, coef, S,
                                                       g, Xhi, Xlo, info);
  return cudaGetLastError();
}

}  // namespace ffb

bool ffblock_supported(int D, int k) {
  return (D == 2 && k >= 1 && k <= 3) || (D == 3 && k >= 1 && k <= 2);
}

// coupled interior rows of one facet at most: the facet's (k+1)^(D-1) nodes
// of each of the D flux components and of the pressure
static int ffblock_pattern_stride(int D, int k) {
  int nfd = 1;
  for (int d = 0; d < D - 1; ++d) nfd *= k + 1;
  return (D + 1) * nfd;
}

size_t ffblock_pattern_ints(int D, int k) {
  return (size_t)2 * D * ffblock_pattern_stride(D, k) + 8 + (size_t)2 * D * 4;
}

// The interior rows of the Darcy cell block that the trace of local facet lf
// couples to: the cell nodes on the facet (lattice index along the facet's
// normal dimension dn = D-1-lf/2 equal to k for the upper side lf%2 = 1, 0 for
// the lower), for the flux components (only the normal one when every cell
// is axis-aligned: the normal has no other component) and for the pressure;
// Q_k Lagrange functions of the other nodes vanish on the facet, so the other
// entries of A_if and A_fi are exactly zero.  Layout (ffblock_pattern_ints):
// [lf][(D+1) (k+1)^(D-1)] rows in increasing order, then 8 counts, then
// [lf][4] the index of each field's first row (flux components 0..D-1,
// pressure D).
void ffblock_pattern(int D, int k, const int *lat, bool axis, int *out) {
  int nk = 1;
  for (int d = 0; d < D; ++d) nk *= k + 1;
  const int nl = 2 * D, stride = ffblock_pattern_stride(D, k);
  std::fill(out, out + ffblock_pattern_ints(D, k), 0);
  int *cnt = out + (size_t)nl * stride, *seg = cnt + 8;
  for (int lf = 0; lf < nl; ++lf) {
    const int dn = D - 1 - lf / 2, side = (lf % 2) * k;
    int q = 0;
    for (int fld = 0; fld <= D; ++fld) {
      seg[lf * 4 + fld] = q;
      if (fld < D && axis && fld != dn) continue;
      for (int a = 0; a < nk; ++a)
        if (lat[a * D + dn] == side) out[lf * stride + q++] = fld * nk + a;
    }
    cnt[lf] = q;
  }
}

cudaError_t launch_condense_ffblock(int D, int k, int ncells, const float *Ahi, const float *Alo, const float *bhi,
                                    const float *blo, const float *Minv_h, const float *Minv_l, const float *MG_h,
                                    const float *MG_l, const int *pat, const double *coef, double *S, double *g,
                                    float *Xhi, float *Xlo, int *info, cudaStream_t s, int num_sms,
                                    long long *launches) {
  ++*launches;
#define HDG_FFB(DD, KK)                                                                                   \
  if (D == DD && k == KK)                                                                                 \
    return ffb::launch_cfg<ffb::Cfg<DD, (KK + 1) * (KK + 1) * (DD == 3 ? (KK + 1) : 1),                    \
                                    (DD == 3 ? (KK + 1) * (KK + 1) : (KK + 1))>>(                          \
        ncells, Ahi, Alo, bhi, blo, Minv_h, Minv_l, MG_h, MG_l, pat, coef, S, g, Xhi, Xlo, info, s, num_sms);
  HDG_FFB(2, 1)
  HDG_FFB(2, 2)
  HDG_FFB(2, 3)
  HDG_FFB(3, 1)
  HDG_FFB(3, 2)
#undef HDG_FFB
  --*launches;
  return cudaErrorInvalidValue;
}

// per cell: 1/m = kappa / |det J| and the panel coefficients cg[e][d] / m
// (10 doubles, cell_y_coef), in FP64
__global__ void inv_mass_scale_kernel(CellArgs a, double *coef) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.ncells; c += gridDim.x * blockDim.x)
    cell_y_coef(a, c, coef + 10 * (size_t)c);
}

cudaError_t launch_inv_mass_scale(const CellArgs &a, double *inv_m, cudaStream_t s, long long *launches) {
  int g = (a.ncells + 255) / 256;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  inv_mass_scale_kernel<<<g, 256, 0, s>>>(a, inv_m);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace hdg
