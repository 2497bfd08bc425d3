// k_batch.cu -- size-class batching (sm_103a): one persistent fused
// integrate -> condense launch over the cells of every problem of one
// (D, k) class.  The cell block never reaches HBM:
//  * FP64: the cell is integrated straight into the shared-memory block
//    W = [A | b] that the partial elimination works on;
//  * float-float block elimination: the cell's (A_hi, A_lo, b_hi, b_lo) go to
//    a per-group scratch slot that stays in L2 and is read back by the same
//    CTA right away.
// A CTA runs CPC = 256 / TPC cells side by side, TPC threads per cell; TPC is
// the tile parameter the autotuner picks per class.  All groups of a CTA run
// the same barrier sequence; a group without a cell in the last wave computes
// on its own scratch and writes nothing.
#include <cuda_runtime.h>

#include "../../include/hdg_gb300.h"
#include "hdg_kernels.h"
#include "k_ff_cell.cuh"
#include "k_ffblock_cell.cuh"
#include "k_fp64_cell.cuh"

namespace hdg {

namespace {

constexpr int kBatchThreads = 256;

__device__ __forceinline__ int find_problem(const BatchProblem *probs, int nprob, long long item) {
  int lo = 0, hi = nprob - 1;  // last problem with first <= item
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].first <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__host__ __device__ constexpr size_t align16(size_t b) { return (b + 15) / 16 * 16; }

// integrate_cell_ff with the class's sizes fixed at compile time (constant
// divisors in the row decode) and only the entries the block elimination
// reads: the flux rows' flux and pressure columns are skipped.  Each entry
// and b come from the same cell_entry_ff / source loop, so the values equal
// the single-problem kernels' bit for bit.
template <class C>
__device__ __forceinline__ void integrate_cell_ffc(const CellArgs &a, const MixedTables &T, int c, bool active,
                                                   CellFactorsFF &f, double *fq, float *Ah, float *Al, float *bh,
                                                   float *bl, int t, int nt) {
  constexpr int D = C::D, NK = C::NK, NFD = C::NFD, NU = C::NU, NI = C::NI, N = C::N;
  constexpr int R0 = N - NU, NE = NI * R0 + (N - NI) * N;  // written entries
  if (t == 0 && active) cell_factors_ff(a, c, f);
  __syncthreads();
  if (active) {
    const double kap = a.kappa ? a.kappa[c] : 1.0;
    for (int q = t; q < a.nqv; q += nt) {
      double x[3], p, qe[3], fu[3], g;
      for (int d = 0; d < D; ++d) {
        x[d] = f.x0[d];
        for (int e = 0; e < D; ++e) x[d] += f.J[d][e] * a.qxi[q * D + e];
      }
      exact_solution(a.problem, D, x, kap, p, qe, fu, g);
      const double w = a.qw[q] * f.detJ;
      for (int d = 0; d < D; ++d) fq[q * (D + 1) + d] = w * fu[d];
      fq[q * (D + 1) + D] = w * g;
    }
  }
  __syncthreads();
  if (active) {
    for (int e = t; e < NE; e += nt) {
      int i, j;
      if (e < NI * R0) {
        j = e / R0;
        i = NU + (e - j * R0);
      } else {
        const int r = e - NI * R0, jf = r / N;
        j = NI + jf;
        i = r - jf * N;
      }
      int ti, si, ii, tj, sj, jj;
      decode_row(i, D, NK, NI, NFD, ti, si, ii);
      decode_row(j, D, NK, NI, NFD, tj, sj, jj);
      float h, l;
      cell_entry_ff(a, T, f, ti, si, ii, tj, sj, jj, h, l);
      Ah[j * N + i] = h;
      Al[j * N + i] = l;
    }
    for (int i = t; i < N; i += nt) {
      int ti, si, ii;
      decode_row(i, D, NK, NI, NFD, ti, si, ii);
      double v = 0.0;
      if (ti < 2) {
        const int comp = ti == 0 ? si : D;
        for (int q = 0; q < a.nqv; ++q) v += fq[q * (D + 1) + comp] * a.qphi[q * NK + ii];
      }
      float h, l;
      split_double(v, h, l);
      bh[i] = h;
      bl[i] = l;
    }
  }
  __syncthreads();
}

template <class C>
struct FfbLayout {
  static constexpr size_t ffb = align16(C::smem_bytes);
  static constexpr size_t fac = align16(sizeof(CellFactorsFF));
  static constexpr size_t fqb(int nqv) { return align16((size_t)nqv * (C::D + 1) * sizeof(double)); }
  // + the cell's 10 panel coefficients (cell_y_coef)
  static constexpr size_t group(int nqv) { return ffb + fac + fqb(nqv) + align16(10 * sizeof(double)); }
  static constexpr size_t slot_floats = 2 * ((size_t)C::N * C::N + C::N);
};

template <class C, int TPC>
__global__ void __launch_bounds__(kBatchThreads, 4) fused_ffblock_kernel(const BatchProblem *__restrict__ probs, int nprob,
                                                                      long long total, size_t group_bytes,
                                                                      float *scratch, int *bad) {
  constexpr int CPC = kBatchThreads / TPC, N = C::N, NF = C::NF, NI = C::NI, NC = C::NC;
  using L = FfbLayout<C>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int grp = threadIdx.x / TPC, t = threadIdx.x - grp * TPC;
  unsigned char *base = smem_raw + (size_t)grp * group_bytes;
  float *fsm = reinterpret_cast<float *>(base);
  CellFactorsFF &f = *reinterpret_cast<CellFactorsFF *>(base + L::ffb);
  double *fq = reinterpret_cast<double *>(base + L::ffb + L::fac);
  double *coef = reinterpret_cast<double *>(base + group_bytes - align16(10 * sizeof(double)));
  float *Ah = scratch + ((size_t)blockIdx.x * CPC + grp) * L::slot_floats;
  float *Al = Ah + (size_t)N * N, *bh = Al + (size_t)N * N, *bl = bh + N;
  const long long per_wave = (long long)gridDim.x * CPC;
  const long long waves = (total + per_wave - 1) / per_wave;
  for (long long w = 0; w < waves; ++w) {
    const long long item = (w * gridDim.x + blockIdx.x) * CPC + grp;
    const bool active = item < total;
    const int p = active ? find_problem(probs, nprob, item) : 0;
    const BatchProblem &P = probs[p];
    const int c = active ? (int)(item - P.first) : 0;
    // the cell's panel coefficients, once per cell (FP64 divisions: one
    // thread, not the whole group); integrate_cell_ffc's first barrier
    // publishes them, the barrier here retires the previous cell's readers
    __syncthreads();
    if (t == 0) {
      if (active) {
        cell_y_coef(P.a, c, coef);
      } else {
        coef[0] = 1.0;
        for (int q = 1; q < 10; ++q) coef[q] = 0.0;
      }
    }
    integrate_cell_ffc<C>(P.a, P.T, c, active, f, fq, Ah, Al, bh, bl, t, TPC);
    int *infoc = active ? P.info + c : nullptr;
    ffb::ffblock_cell<C, TPC, false>(active, Ah, Al, bh, bl, P.Mh, P.Ml, P.MGh, P.MGl, P.ffpat, coef, fsm,
                                     P.S + (size_t)c * NF * NF,
                                     P.g + (size_t)c * NF, P.Xh + (size_t)c * NI * NC, P.Xl + (size_t)c * NI * NC,
                                     infoc, t);
    if (active && t == 0 && *infoc) atomicMax(bad + p, *infoc);
  }
}

template <int TPC>
__global__ void __launch_bounds__(kBatchThreads) fused_fp64_kernel(const BatchProblem *__restrict__ probs, int nprob,
                                                                   long long total, int n, int ni, int nf,
                                                                   size_t group_bytes, int *bad) {
  constexpr int CPC = kBatchThreads / TPC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int grp = threadIdx.x / TPC, t = threadIdx.x - grp * TPC;
  unsigned char *base = smem_raw + (size_t)grp * group_bytes;
  double *W = reinterpret_cast<double *>(base);  // n x (n+1), column-major
  const size_t wbytes = align16(sizeof(double) * (size_t)n * (n + 1));
  CellFactors &f = *reinterpret_cast<CellFactors *>(base + wbytes);
  double *fq = reinterpret_cast<double *>(base + wbytes + align16(sizeof(CellFactors)));
  int *s_piv = reinterpret_cast<int *>(base + group_bytes - 16);
  const long long per_wave = (long long)gridDim.x * CPC;
  const long long waves = (total + per_wave - 1) / per_wave;
  for (long long w = 0; w < waves; ++w) {
    const long long item = (w * gridDim.x + blockIdx.x) * CPC + grp;
    const bool active = item < total;
    const int p = active ? find_problem(probs, nprob, item) : 0;
    const BatchProblem &P = probs[p];
    const CellArgs &a = P.a;
    const int c = active ? (int)(item - P.first) : 0;
    if (t == 0 && active) cell_factors(a, c, f);
    __syncthreads();
    if (active) source_values(a, f, c, fq, t, TPC);
    __syncthreads();
    if (active) {
      for (int e = t; e < n * n; e += TPC) {
        const int j = e / n, i = e - j * n;
        int ti, si, ii, tj, sj, jj;
        decode(i, a.D, a.nk, a.ni, a.nfd, ti, si, ii);
        decode(j, a.D, a.nk, a.ni, a.nfd, tj, sj, jj);
        W[e] = cell_entry<double>(a, f, ti, si, ii, tj, sj, jj);
      }
      for (int i = t; i < n; i += TPC) {
        int ti, si, ii;
        decode(i, a.D, a.nk, a.ni, a.nfd, ti, si, ii);
        double v = 0.0;
        if (ti < 2) {
          const int comp = ti == 0 ? si : a.D;
          for (int q = 0; q < a.nqv; ++q) v += fq[q * (a.D + 1) + comp] * a.qphi[q * a.nk + ii];
        }
        W[(size_t)n * n + i] = v;
      }
    }
    __syncthreads();
    const int inf = eliminate_fp64(W, n, n + 1, ni, ni, s_piv, t, TPC);
    if (active) {
      double *Sc = P.S + (size_t)c * nf * nf;
      for (int e = t; e < nf * nf; e += TPC) {
        const int jj = e / nf, ii = e - jj * nf;
        Sc[e] = W[(ni + ii) + (size_t)n * (ni + jj)];
      }
      for (int i = t; i < nf; i += TPC) P.g[(size_t)c * nf + i] = W[(ni + i) + (size_t)n * n];
      double *Fc = P.fact + (size_t)c * ni * (n + 1);
      for (int e = t; e < ni * (n + 1); e += TPC) {
        const int jj = e / ni, ii = e - jj * ni;
        Fc[e] = W[ii + (size_t)n * jj];
      }
      if (t == 0) {
        P.info[c] = inf;
        if (inf) atomicMax(bad + p, inf);
      }
    }
    __syncthreads();
  }
}

// The kernel's shared-memory limit is raised to the device maximum (not to
// this launch's size): one instantiation serves classes of different sizes,
// and a captured graph replays all of them without re-setting the attribute.
template <class K>
cudaError_t occupancy_grid(K kernel, size_t smem, size_t smem_optin, int num_sms, long long total, int cpc,
                           int *grid) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_optin);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBatchThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  long long g = (long long)per_sm * num_sms;
  const long long need = (total + cpc - 1) / cpc;
  if (g > need) g = need;
  *grid = g < 1 ? 1 : (int)g;
  return cudaSuccess;
}

template <class C, int TPC>
cudaError_t ffb_fused(const FusedLaunch &L, cudaStream_t s) {
  using Lay = FfbLayout<C>;
  constexpr int CPC = kBatchThreads / TPC;
  const size_t gb = Lay::group(L.nqv);
  const size_t smem = gb * CPC;
  if (smem > L.smem_optin) return cudaErrorInvalidConfiguration;
  int grid = 0;
  cudaError_t e = occupancy_grid(fused_ffblock_kernel<C, TPC>, smem, L.smem_optin, L.num_sms, L.total, CPC, &grid);
  if (e != cudaSuccess) return e;
  const size_t need = (size_t)grid * CPC * Lay::slot_floats * sizeof(float);
  if (L.scratch_bytes_out) *L.scratch_bytes_out = need;
  if (L.dry_run) return cudaSuccess;
  if (need > L.scratch_bytes) return cudaErrorMemoryAllocation;
  fused_ffblock_kernel<C, TPC><<<grid, kBatchThreads, smem, s>>>(L.probs, L.nprob, L.total, gb, L.scratch, L.bad);
  return cudaGetLastError();
}

template <int TPC>
cudaError_t fp64_fused(const FusedLaunch &L, cudaStream_t s) {
  constexpr int CPC = kBatchThreads / TPC;
  const size_t gb = align16(sizeof(double) * (size_t)L.n * (L.n + 1)) + align16(sizeof(CellFactors)) +
                    align16((size_t)L.nqv * (L.D + 1) * sizeof(double)) + 16;
  const size_t smem = gb * CPC;
  if (smem > L.smem_optin) return cudaErrorInvalidConfiguration;
  int grid = 0;
  cudaError_t e = occupancy_grid(fused_fp64_kernel<TPC>, smem, L.smem_optin, L.num_sms, L.total, CPC, &grid);
  if (e != cudaSuccess) return e;
  if (L.scratch_bytes_out) *L.scratch_bytes_out = 0;
  if (L.dry_run) return cudaSuccess;
  fused_fp64_kernel<TPC><<<grid, kBatchThreads, smem, s>>>(L.probs, L.nprob, L.total, L.n, L.ni, L.nf, gb, L.bad);
  return cudaGetLastError();
}

template <class C>
cudaError_t ffb_by_tpc(const FusedLaunch &L, cudaStream_t s) {
  switch (L.tpc) {
    case 32: return ffb_fused<C, 32>(L, s);
    case 64: return ffb_fused<C, 64>(L, s);
    case 128: return ffb_fused<C, 128>(L, s);
    case 256: return ffb_fused<C, 256>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

bool fused_batch_supported(int D, int k, int precision) {
  if (precision == HDG_PREC_FF_BLOCK) return ffblock_supported(D, k);
  if (precision == HDG_PREC_FP64) return true;  // the shared-memory bound is checked at launch
  return false;
}

cudaError_t launch_fused_batch(const FusedLaunch &L, cudaStream_t s, long long *launches) {
  cudaError_t e = cudaErrorInvalidValue;
  if (L.precision == HDG_PREC_FP64) {
    switch (L.tpc) {
      case 32: e = fp64_fused<32>(L, s); break;
      case 64: e = fp64_fused<64>(L, s); break;
      case 128: e = fp64_fused<128>(L, s); break;
      case 256: e = fp64_fused<256>(L, s); break;
      default: break;
    }
  } else if (L.precision == HDG_PREC_FF_BLOCK) {
#define HDG_FFB(DD, KK)                                                                                          \
  if (L.D == DD && L.k == KK)                                                                                    \
    e = ffb_by_tpc<ffb::Cfg<DD, (KK + 1) * (KK + 1) * (DD == 3 ? (KK + 1) : 1),                                   \
                            (DD == 3 ? (KK + 1) * (KK + 1) : (KK + 1))>>(L, s);
    HDG_FFB(2, 1)
    HDG_FFB(2, 2)
    HDG_FFB(2, 3)
    HDG_FFB(3, 1)
    HDG_FFB(3, 2)
#undef HDG_FFB
  }
  if (e == cudaSuccess && !L.dry_run) ++*launches;
  return e;
}

}  // namespace hdg
