// k_pcg_common.cuh -- device helpers shared by the skeleton PCG kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hdg {

// Device scalars of a PCG solve (double array).
enum {
  SC_RZ = 0,     // (r, z)
  SC_PAP = 1,    // (p, A p)
  SC_ALPHA = 2,
  SC_BETA = 3,
  SC_RR = 4,     // (r, r)
  SC_BB = 5,     // (b, b)
  SC_TOL2 = 6,   // rtol^2 (b, b)
  SC_DONE = 7,   // 1 once converged
  SC_ITERS = 8,  // completed iterations
  SC_NSCAL = 16
};

constexpr int kPcgThreads = 256;
constexpr int kMaxRowLen = 304;  // 11 neighbour facets x 27 DOFs (3D elasticity, k=2) fits

__device__ __forceinline__ double block_sum(double v, double *red) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  return s;  // valid in thread 0
}

// After every CTA has stored its partials: true in the CTA that arrives last.
// Thread 0 stores a CTA's partials, so its fence before the arrival is the
// one the last CTA's reads (through L2) need; a fence in every thread only
// stalled them.
__device__ __forceinline__ bool last_cta(unsigned int *counter) {
  __shared__ bool is_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    is_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  return is_last;
}

// sum of partials[k*nparts + 0..nparts) in index order (called by the last CTA)
__device__ __forceinline__ double sum_partials(const double *partials, int nparts, int k, double *red) {
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += __ldcg(partials + (size_t)k * nparts + i);
  return block_sum(s, red);
}

// ---------------------------------------------------------------------------
// Dot products on the FP32 pipes.  GB300 issues FP64 at a small fraction of
// its FP32 rate, and reductions that every CTA runs at the same moment (the
// end of a one-wave launch) serialise on that pipe; float-float pairs
// (unevaluated hi + lo, ~48 significant bits) carry the same sums on the
// FP32 pipes.  FP64 remains for the final scalars only.
// ---------------------------------------------------------------------------
// (ah, al) += (bh, bl): Knuth two-sum of the high parts, then renormalised
__device__ __forceinline__ void ff_add(float &ah, float &al, float bh, float bl) {
  const float s = ah + bh;
  const float bb = s - ah;
  float e = (ah - (s - bb)) + (bh - bb);
  e += al + bl;
  ah = s + e;
  al = e - (ah - s);
}

// running sum of FP32 products: fma gives each product's rounding error exactly
struct FFSum {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);
    const float s = hi + p;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (p - bb);
    hi = s;
    lo += e + pe;
  }
};

// block sum of float-float pairs, in a fixed order; valid in thread 0
__device__ __forceinline__ float2 block_sum_ff(float hi, float lo, float2 *redf) {
  for (int off = 16; off > 0; off >>= 1) {
    const float bh = __shfl_down_sync(0xffffffffu, hi, off), bl = __shfl_down_sync(0xffffffffu, lo, off);
    ff_add(hi, lo, bh, bl);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) redf[w] = make_float2(hi, lo);
  __syncthreads();
  float2 s = make_float2(0.0f, 0.0f);
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) ff_add(s.x, s.y, redf[i].x, redf[i].y);
  return s;
}

// A CTA's float-float partial k, stored as a float2 in the double-sized slot
// k*nparts + blockIdx.x of the partials array.
__device__ __forceinline__ void store_partial_ff(double *partials, int nparts, int k, float2 v) {
  reinterpret_cast<float2 *>(partials)[(size_t)k * nparts + blockIdx.x] = v;
}

// sum of the float-float partials k*nparts + 0..nparts in a fixed order (the
// last CTA), returned in FP64; valid in thread 0
__device__ __forceinline__ double sum_partials_ff(const double *partials, int nparts, int k, float2 *redf) {
  const float2 *p = reinterpret_cast<const float2 *>(partials) + (size_t)k * nparts;
  float hi = 0.0f, lo = 0.0f;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    const float2 v = __ldcg(p + i);
    ff_add(hi, lo, v.x, v.y);
  }
  const float2 s = block_sum_ff(hi, lo, redf);
  return (double)s.x + (double)s.y;
}

// ---------------------------------------------------------------------------
// FP64 CSR products, two lanes per row.  GB300's FP64 pipe is the bound of an
// FP64 CSR SpMV (one DFMA per stored entry against 12 bytes of traffic), so
// every FP64 instruction counts: a row per lane pair needs one DFMA per entry
// and a single shuffle-add (a warp per block row with a reduce-scatter issued
// about 1.9x that on 3D k = 2 rows), while each pair still reads its row in
// 32-byte pieces (one row per lane left most of every sector to a later load
// and ran at half the bandwidth).  A CTA takes a tile of whole block rows; the
// vector at the tile's columns is staged once per block row in shared memory
// and shared by the block row's NFD rows.
// ---------------------------------------------------------------------------
// A facet's row couples to its own block and to the other facets of its at
// most two cells (at most six facets each): at most 11 blocks.  The host
// checks every problem's longest row against kRowBlocks * nfd.
constexpr int kRowBlocks = 11;

template <int NFD>
struct RowTile {
  static constexpr int BR = kPcgThreads / NFD;   // block rows per tile
  static constexpr int LMAX = kRowBlocks * NFD;  // staged entries per block row
  static constexpr int ROWS = BR * NFD;          // rows per tile
  static constexpr int RPP = kPcgThreads / 2;    // rows per pass of the CTA
  static constexpr int PASSES = (ROWS + RPP - 1) / RPP;
};

// This lane's half of sum_j v[j] xk[j] (half = 0, 1 of the lane pair): the
// row in 16-byte loads, the pair's two loads 32 contiguous bytes, after an
// 8-byte one (half 0) where the row starts unaligned; the two halves summed
// by the caller.  Four loads per lane are issued before their products: the
// rows stream from HBM, and one load in flight per lane held the kernel to
// about 2.7 TB/s.
__device__ __forceinline__ double row_dot_half(const double *__restrict__ v, const double *xk, int len, int half) {
  double t = 0.0;
  int j = 0;
  if (len > 0 && (reinterpret_cast<uintptr_t>(v) & 15u) != 0) {
    if (half == 0) t = fma(__ldg(v), xk[0], t);
    j = 1;
  }
  for (; j + 15 < len; j += 16) {
    double2 w[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) w[u] = __ldg(reinterpret_cast<const double2 *>(v + j + 4 * u + 2 * half));
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int q = j + 4 * u + 2 * half;
      t = fma(w[u].x, xk[q], t);
      t = fma(w[u].y, xk[q + 1], t);
    }
  }
  for (; j + 3 < len; j += 4) {
    const int q = j + 2 * half;
    const double2 w = __ldg(reinterpret_cast<const double2 *>(v + q));
    t = fma(w.x, xk[q], t);
    t = fma(w.y, xk[q + 1], t);
  }
  for (int q = j + half; q < len; q += 2) t = fma(__ldg(v + q), xk[q], t);
  return t;
}
__device__ __forceinline__ double row_dot_half(const float *__restrict__ v, const double *xk, int len, int half) {
  double t = 0.0;
  for (int q = half; q < len; q += 2) t = fma((double)__ldg(v + q), xk[q], t);
  return t;
}

// For every row of the tile (block rows br0 .. br0+nbr-1, staged columns in
// xs): emit(row, k, sum_j val[row, j] x[col_j]) in the pair's even lane (k =
// block row in the tile).  Called by the whole CTA.
template <int NFD, typename V, typename E>
__device__ __forceinline__ void tile_row_products(const int64_t *__restrict__ rowptr, const V *__restrict__ val,
                                                  int br0, int nbr, const double *xs, E emit) {
  using T = RowTile<NFD>;
  const int half = threadIdx.x & 1;
#pragma unroll 1
  for (int pass = 0; pass < T::PASSES; ++pass) {
    const int tr = pass * T::RPP + ((int)threadIdx.x >> 1);
    const bool act = tr < nbr * NFD;
    const int k = tr / NFD;
    const int row = br0 * NFD + tr;
    double t = 0.0;
    if (act) {
      const int64_t b = rowptr[row];
      t = row_dot_half(val + b, xs + k * T::LMAX, (int)(rowptr[row + 1] - b), half);
    }
    t += __shfl_xor_sync(0xffffffffu, t, 1);  // the same bits in both lanes
    if (act && half == 0) emit(row, k, t);
  }
}

// Stages f(col) for the columns of block rows br0 .. br0+nbr-1 into
// xs[k * LMAX + j] (k = block row in the tile, j = entry), warp by warp;
// the caller synchronises before reading.
template <int NFD, typename F>
__device__ __forceinline__ void stage_tile_columns(const int64_t *__restrict__ rowptr, const int *__restrict__ colind,
                                                   int br0, int nbr, double *xs, F f) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = w; k < nbr; k += nw) {
    const int64_t base = rowptr[(int64_t)(br0 + k) * NFD];
    const int len = (int)(rowptr[(int64_t)(br0 + k) * NFD + 1] - base);
    for (int j = lane; j < len; j += 32) xs[k * RowTile<NFD>::LMAX + j] = f(colind[base + j]);
  }
}

// index of the facet block (lo, hi), lo < hi, in a cell record of the
// unassembled FP32 operator (the blocks above the diagonal, row-major order)
template <int NL>
__device__ __forceinline__ int offdiag_block(int lo, int hi) {
  return lo * (NL - 1) - (lo * (lo - 1)) / 2 + (hi - lo - 1);
}

template <int N>
struct Pow2Ceil {
  static constexpr int v = N <= 1 ? 1 : N <= 2 ? 2 : N <= 4 ? 4 : N <= 8 ? 8 : N <= 16 ? 16 : 32;
};

// Warp reduce-scatter of P per-lane partial sums (P a power of two <= 32):
// each butterfly step keeps half of the remaining entries, so a lane does
// P/2 + P/4 + ... + 1 (+ the remaining plain steps) additions instead of
// 5 per entry.  Afterwards lane l holds the warp-wide total of entry
// reduce_scatter_row<P>(l); the 32/P lanes with equal high bits share it.
template <typename T, int P>
__device__ __forceinline__ T warp_reduce_scatter(T (&v)[P], int lane) {
  int cnt = P;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    if (cnt > 1) {
      const int half = cnt / 2;
      const bool upper = (lane & off) != 0;
#pragma unroll
      for (int i = 0; i < half; ++i) {
        const T send = upper ? v[i] : v[i + half];
        const T keep = upper ? v[i + half] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
      }
      cnt = half;
    } else {
      v[0] += __shfl_xor_sync(0xffffffffu, v[0], off);
    }
  }
  return v[0];
}

template <int P>
__device__ __forceinline__ int reduce_scatter_row(int lane) {
  int r = 0, cnt = P;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    if (cnt > 1) {
      const int half = cnt / 2;
      if (lane & off) r += half;
      cnt = half;
    }
  }
  return r;
}

// the lowest lane holding each entry after warp_reduce_scatter<P>
template <int P>
__device__ __forceinline__ bool reduce_scatter_writer(int lane) {
  return (lane & (32 / P - 1)) == 0;
}

}  // namespace hdg
