// k_pcg32_persistent.cu -- the inner FP32 skeleton PCG as ONE cooperative
// launch (sm_103a): every iteration is the cell-operator SpMV phase, a grid
// barrier, the update phase, a grid barrier -- no kernel boundaries, no
// pipeline refills.  The same arithmetic as the two-kernel iteration
// (cell_spmv32_kernel + pcg32_update_cells_kernel):
//   SpMV:   p = r + beta p_old (owner writes), qc = M^_c p_c by block row,
//           partial (p, Ap)
//   update: q = qc(owner) + qc(other), x += alpha p, r -= alpha q (z = r: the
//           preconditioner is a scaling of the records), partial (r, r)
// Every CTA sums the per-CTA partials itself in one fixed order after each
// barrier (so all CTAs hold the same alpha, beta and convergence decision,
// and the result does not depend on timing).  The cell records of a CTA are
// the same every iteration, so its bulk-copy ring keeps prefetching the next
// iteration's first records across the barriers.
//
// The grid is co-resident (cudaLaunchCooperativeKernel).  Every wait is
// bounded: a grid barrier that times out or a bulk copy that never lands sets
// the error flag and SC_DONE; the CTA waits (bounded) for its own copies in
// flight and returns.
#include <cuda_runtime.h>

#include "hdg_kernels.h"
#include "k_bulk.cuh"
#include "k_pcg_common.cuh"

namespace hdg {

namespace {

constexpr int kPersistStagesMax = 8;

// Grid-wide barrier of a co-resident grid: arrive on count; the last arriver
// resets it and opens the next generation.  Returns false (in every thread of
// the CTA) when the wait gave up.
__device__ bool grid_barrier(unsigned *count, unsigned *gen, unsigned &my_gen, int *flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g = my_gen;
    __threadfence();
    if (atomicAdd(count, 1u) == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      ok = wait_word_change(gen, g) ? 1 : 0;
    }
    __threadfence();
    my_gen = g + 1;
    *flag = ok;
  }
  __syncthreads();
  return *flag != 0;
}

// sum of the n float-float per-CTA partials k*n .. k*n+n-1 in one fixed order,
// returned in every thread (every CTA gets the same bits)
__device__ __forceinline__ double sum_all_ff(const double *partials, int n, int k, float2 *redf) {
  __shared__ double bc;
  const double v0 = sum_partials_ff(partials, n, k, redf);  // valid in thread 0
  if (threadIdx.x == 0) bc = v0;
  __syncthreads();
  const double v = bc;
  __syncthreads();
  return v;
}

}  // namespace

template <int NL, int NFD>
__global__ void __launch_bounds__(kPcgThreads) pcg32_persistent_kernel(Pcg32Args a, int iter_cap) {
  constexpr int NF = NL * NFD;
  constexpr int TPC = cellop_tpc(NF), CPS = cellop_cps(NF), REC = cellop_rec(NL, NFD);
  extern __shared__ __align__(128) float ring[];
  __shared__ __align__(8) uint64_t bars[kPersistStagesMax];
  __shared__ __align__(16) float ps[CPS][TPC];
  __shared__ float2 redf[32];
  __shared__ int flag, abort_flag;
  if (a.scal[SC_DONE] != 0.0) return;
  unsigned *bar_count = a.counter + 2, *bar_gen = a.counter + 3;
  unsigned my_gen = ld_acquire_u32(bar_gen);
  const int G = (int)gridDim.x;
  const int nstage = a.nstage;
  // SpMV work: units of CPS consecutive cells, round-robin over the CTAs
  const int g = threadIdx.x / TPC, i = threadIdx.x - g * TPC;
  const int lf = i / NFD, r = i - lf * NFD;
  const bool spmv_thread = threadIdx.x < CPS * TPC;
  const int nunits = (a.ncells + CPS - 1) / CPS;
  const int mine = (int)blockIdx.x < nunits ? (nunits - 1 - (int)blockIdx.x) / G + 1 : 0;
  uint64_t pol = 0;
  long long issued = 0;  // stages issued (thread 0); stage s holds the records of unit s % mine
  auto issue = [&](long long s) {
    const int u = (int)(s % mine);
    const int c0 = ((int)blockIdx.x + u * G) * CPS;
    const int nc = min(CPS, a.ncells - c0);
    const uint32_t bytes = (uint32_t)nc * REC * 4u;
    const int slot = (int)(s % nstage);
    mbar_arrive_expect_tx(&bars[slot], bytes);
    bulk_copy_g2s(ring + (size_t)slot * CPS * REC, a.blocks + (size_t)c0 * REC, bytes, &bars[slot], pol);
  };
  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < nstage; ++s) mbar_init(&bars[s], 1);
    mbar_init_fence();
    pol = l2_evict_first_policy();
    if (mine > 0)
      for (; issued < nstage; ++issued) issue(issued);
  }
  __syncthreads();
  // before returning: this CTA's copies in flight (they target its shared memory)
  auto drain = [&](long long consumed) {
    if (threadIdx.x == 0)
      for (long long s = consumed; s < issued; ++s)
        mbar_wait_bounded(&bars[s % nstage], (uint32_t)((s / nstage) & 1));
    __syncthreads();
  };
  auto fail = [&](long long consumed) {
    if (threadIdx.x == 0) {
      atomicExch(a.error, 1u);
      if (blockIdx.x == 0) a.scal[SC_DONE] = 1.0;
    }
    drain(consumed);
  };
  double rz = a.scal[SC_RZ], beta = a.scal[SC_BETA], tol2 = a.scal[SC_TOL2];
  double iters = a.scal[SC_ITERS];
  const float *p_old = a.p;
  float *p_new = a.p2;
  long long stage = 0;  // stages consumed
  for (int it = 0; it < iter_cap; ++it) {
    // ---- SpMV phase (dot products in float-float: GB300's FP64 pipe is narrow)
    FFSum acc;
    const float fbeta = (float)beta;
    for (int s = 0; s < mine; ++s, ++stage) {
      const int slot = (int)(stage % nstage);
      const int c = ((int)blockIdx.x + s * G) * CPS + g;
      const bool act = spmv_thread && i < NF && c < a.ncells;
      float pv = 0.0f;
      int ent = -1;
      if (act) {
        ent = a.cell_blk[(size_t)c * NL + lf];
        if (ent >= 0) {  // p_old and z were written by other CTAs: read through L2
          const int row = (ent >> 1) * NFD + r;
          pv = fmaf(fbeta, __ldcg(p_old + row), __ldcg(a.z + row));
          if (ent & 1) p_new[row] = pv;
        }
      }
      if (spmv_thread) ps[g][i] = pv;
      if (!mbar_wait_bounded(&bars[slot], (uint32_t)((stage / nstage) & 1))) abort_flag = 1;
      __syncthreads();
      if (abort_flag) {
        fail(stage);
        return;
      }
      if (act) {
        const float *B = ring + (size_t)slot * CPS * REC + (size_t)g * REC;
        float q = 0.0f;
        if constexpr (NF <= 64) {  // the cell's p in registers: the inner loop only reads B
          constexpr int NV = (NF + 3) / 4;
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
#pragma unroll
          for (int b = 0; b < NL; ++b) {
            if (b == lf) continue;  // the identity diagonal block: added in the update phase
            const bool up = b > lf;
            const int lo = up ? lf : b, hi = up ? b : lf;
            const float *Bb = B + offdiag_block<NL>(lo, hi) * cellop_bstride(NFD) + (up ? r * NFD : r);
            const int st = up ? 1 : NFD;
#pragma unroll
            for (int k = 0; k < NFD; ++k) q = fmaf(Bb[k * st], pr[b * NFD + k], q);
          }
        } else {
#pragma unroll
          for (int b = 0; b < NL; ++b) {
            if (b == lf) continue;
            const bool up = b > lf;
            const int lo = up ? lf : b, hi = up ? b : lf;
            const float *Bb = B + offdiag_block<NL>(lo, hi) * cellop_bstride(NFD) + (up ? r * NFD : r);
            const int st = up ? 1 : NFD;
#pragma unroll
            for (int k = 0; k < NFD; ++k) q = fmaf(Bb[k * st], ps[g][b * NFD + k], q);
          }
        }
        if (ent >= 0) a.qc[(size_t)(ent >> 1) * (2 * NFD) + ((ent & 1) ? 0 : NFD) + r] = q;
        acc.add_prod(pv, q);
        if (ent >= 0 && (ent & 1)) acc.add_prod(pv, pv);  // the identity diagonal block, once per row
      }
      __syncthreads();  // the slot and ps are free again: refill with a later stage's records
      if (threadIdx.x == 0) {
        async_proxy_fence();
        issue(issued);
        ++issued;
      }
    }
    const float2 sp = block_sum_ff(acc.hi, acc.lo, redf);
    if (threadIdx.x == 0) store_partial_ff(a.partials, G, 0, sp);
    if (!grid_barrier(bar_count, bar_gen, my_gen, &flag)) {
      fail(stage);
      return;
    }
    const double pq = sum_all_ff(a.partials, G, 0, redf);
    const double alpha_d = rz / pq;
    const float alpha = (float)alpha_d;
    // ---- update phase: rows round-robin over the grid (the same rows every
    // iteration, so x and r are only ever touched by this CTA)
    FFSum rr;
    for (int row = blockIdx.x * kPcgThreads + threadIdx.x; row < a.n; row += G * kPcgThreads) {
      const int br = row / NFD, ri = row - br * NFD;
      const float *qb = a.qc + (size_t)br * (2 * NFD) + ri;
      const float q = __ldcg(qb) + __ldcg(qb + NFD);  // written by other CTAs: read through L2
      const float pv = __ldcg(p_new + row);
      a.x[row] = fmaf(alpha, pv, a.x[row]);
      const float rv = fmaf(-alpha, q + pv, a.r[row]);  // + p: the identity diagonal block
      a.r[row] = rv;
      rr.add_prod(rv, rv);
    }
    const float2 s1 = block_sum_ff(rr.hi, rr.lo, redf);
    if (threadIdx.x == 0) store_partial_ff(a.partials, G, 1, s1);
    if (!grid_barrier(bar_count, bar_gen, my_gen, &flag)) {
      fail(stage);
      return;
    }
    const double vrr = sum_all_ff(a.partials, G, 1, redf);
    const double vrz = vrr;  // z = r
    beta = vrz / rz;
    rz = vrz;
    iters += 1.0;
    const bool done = vrr <= tol2 || !(vrr == vrr);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.scal[SC_PAP] = pq;
      a.scal[SC_ALPHA] = alpha_d;
      a.scal[SC_BETA] = beta;
      a.scal[SC_RZ] = rz;
      a.scal[SC_RR] = vrr;
      a.scal[SC_ITERS] = iters;
      if (done) a.scal[SC_DONE] = 1.0;
    }
    // the next iteration's p_old is this iteration's p_new
    const float *t = p_old;
    p_old = p_new;
    p_new = const_cast<float *>(t);
    if (done) break;
  }
  drain(stage);
}

// Grid and ring depth for the cooperative launch (grid 0 when the kernel
// cannot be co-resident).  Two CTAs per SM with at least three stages each
// where that fits, else one CTA with as many stages as fit.  want: the CTAs
// asked for (about two cell units each on small problems).
template <int NL, int NFD>
static int persistent_grid(size_t smem_optin, int num_sms, int want, int *nstage_out, size_t *smem_out) {
  constexpr int NF = NL * NFD;
  const size_t stage = (size_t)cellop_cps(NF) * cellop_rec(NL, NFD) * sizeof(float);
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, pcg32_persistent_kernel<NL, NFD>) != cudaSuccess) return 0;
  const size_t avail = smem_optin > fa.sharedSizeBytes + 1024 ? smem_optin - fa.sharedSizeBytes - 1024 : 0;
  int ns = (int)((avail / 2 - fa.sharedSizeBytes - 1024) / stage);  // two CTAs per SM
  if (avail / 2 < fa.sharedSizeBytes + 1024 || ns < 3) ns = (int)(avail / stage);
  if (ns > kPersistStagesMax) ns = kPersistStagesMax;
  if (ns < 2) return 0;
  const size_t smem = (size_t)ns * stage;
  if (cudaFuncSetAttribute(pcg32_persistent_kernel<NL, NFD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg32_persistent_kernel<NL, NFD>, kPcgThreads, smem) !=
          cudaSuccess ||
      per_sm < 1)
    return 0;
  int grid = per_sm * num_sms;
  if (want < grid) grid = want;
  if (grid < 1) grid = 1;
  *nstage_out = ns;
  *smem_out = smem;
  return grid;
}

#define HDG_PERSIST_CASES(X) \
  X(3, 1) X(3, 2) X(3, 3) X(3, 4) X(4, 10) X(4, 1) X(6, 1) X(4, 2) X(4, 3) X(4, 4) X(4, 5) X(4, 6) X(4, 8) X(6, 3) X(6, 4) X(6, 6) X(6, 9) X(6, 12) X(6, 16) X(6, 25) X(6, 27)

int pcg32_persistent_config(int nl, int nfd, size_t smem_optin, int num_sms, int want, int *nstage, size_t *smem) {
#define X(L, F) \
  if (nl == L && nfd == F) return persistent_grid<L, F>(smem_optin, num_sms, want, nstage, smem);
  HDG_PERSIST_CASES(X)
#undef X
  return 0;
}

cudaError_t launch_pcg32_persistent(const Pcg32Args &a, int grid, size_t smem, int iter_cap, cudaStream_t s,
                                    long long *launches) {
  Pcg32Args args = a;
  void *params[] = {&args, &iter_cap};
  cudaError_t e = cudaErrorInvalidValue;
#define X(L, F)                                                                                           \
  if (a.nl == L && a.nfd == F)                                                                            \
    e = cudaLaunchCooperativeKernel((const void *)pcg32_persistent_kernel<L, F>, dim3(grid), dim3(kPcgThreads), \
                                    params, smem, s);
  HDG_PERSIST_CASES(X)
#undef X
  if (e == cudaSuccess) ++*launches;
  return e;
}

}  // namespace hdg
