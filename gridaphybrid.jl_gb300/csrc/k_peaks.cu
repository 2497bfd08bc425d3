// k_peaks.cu -- measured FP32 and FP64 FMA pipe peaks of the device, the
// denominators of the compute rooflines of the cell-local kernels
// (integration and condensation run on the FP32 pipes in float-float, or on
// the FP64 pipe in the plain FP64 path).
//
// Each thread runs kChains independent FMA recurrences x <- x*a + b for
// `iters` steps (enough independent work per warp to keep the pipe issuing
// every cycle at full occupancy), one CTA of 256 threads per resident slot
// (num_sms x 8 CTAs), timed by CUDA events.  The recurrences stay finite
// (|a| < 1) and the final values are summed into one output so that no step
// can be removed by the compiler.
#include <cuda_runtime.h>

#include "hdg_internal.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kThreads) fma_peak_kernel(int iters, T a, T b, T *out) {
  T x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = T(threadIdx.x + c) * T(1e-3);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == T(-12345.0)) out[blockIdx.x] = s;  // never true; keeps the chains live
}

template <typename T>
cudaError_t time_peak(hdg_context *ctx, int iters, double *tflops) {
  const int grid = ctx->num_sms * 8;
  hdg::DBuf out;
  out.stream = ctx->stream;
  cudaError_t e = out.reserve(sizeof(T) * grid);
  if (e != cudaSuccess) return e;
  const T a = T(0.999), b = T(1e-4);
  fma_peak_kernel<T><<<grid, kThreads, 0, ctx->stream>>>(iters / 8, a, b, out.as<T>());  // warm-up
  ++ctx->launches;
  if ((e = cudaEventRecord(ctx->ev[0], ctx->stream)) != cudaSuccess) return e;
  fma_peak_kernel<T><<<grid, kThreads, 0, ctx->stream>>>(iters, a, b, out.as<T>());
  ++ctx->launches;
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(ctx->ev[1], ctx->stream)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return e;
  float ms = 0.f;
  if ((e = cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1])) != cudaSuccess) return e;
  const double fmas = (double)grid * kThreads * kChains * iters;
  *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
  return cudaSuccess;
}

}  // namespace

extern "C" int hdg_measure_pipe_peaks(hdg_context *ctx, double *fp32_tflops, double *fp64_tflops) {
  if (!ctx || !fp32_tflops || !fp64_tflops) return ctx ? ctx->fail(HDG_ERR_INVALID, "null output") : HDG_ERR_INVALID;
  hdg::DeviceGuard guard(ctx->device);
  cudaError_t e = guard.status;
  // about 3 ms each on a GB300 at full clock
  if (e == cudaSuccess) e = time_peak<float>(ctx, 1 << 15, fp32_tflops);
  if (e == cudaSuccess) e = time_peak<double>(ctx, 1 << 10, fp64_tflops);
  if (e != cudaSuccess) return ctx->fail(HDG_ERR_CUDA, "hdg_measure_pipe_peaks: %s", cudaGetErrorString(e));
  return HDG_OK;
}
