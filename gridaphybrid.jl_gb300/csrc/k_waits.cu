// k_waits.cu -- a check of the library's bounded device waits.
//
// The kernels wait in two places: the mbarrier waits of the bulk-copy rings
// (skeleton SpMV, persistent PCG) and the generation wait of the cooperative
// grid barrier (persistent PCG).  Both give up after a fixed number of polls,
// record an error and return, so that a copy or a CTA that never arrives
// cannot hang the GPU.  This check runs the same two wait primitives, with a
// short poll limit, against a barrier phase and a word that nothing completes
// or writes, and reports that each gave up and how long one poll took (so
// the production limits, 2^18 and 2^22 polls, can be stated in seconds).
// Nothing is in flight while they wait: no copy is issued and no other CTA
// exists, so giving up leaves the context as it was.
#include <cuda_runtime.h>

#include "hdg_internal.h"
#include "k_bulk.cuh"

namespace {

__global__ void bounded_wait_check_kernel(uint32_t polls, const unsigned *word, int *expired,
                                          long long *cycles) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  hdg::mbar_init(&bar, 1);
  hdg::mbar_init_fence();
  const long long t0 = clock64();
  // phase 0 of bar completes only after one arrival, and none is made
  const bool m = hdg::mbar_wait_bounded(&bar, 0u, polls);
  const long long t1 = clock64();
  // nothing writes word
  const bool g = hdg::wait_word_change(word, hdg::ld_acquire_u32(word), polls);
  const long long t2 = clock64();
  expired[0] = m ? 0 : 1;
  expired[1] = g ? 0 : 1;
  cycles[0] = t1 - t0;
  cycles[1] = t2 - t1;
}

}  // namespace

extern "C" int hdg_check_bounded_waits(hdg_context *ctx, unsigned polls, int *expired, double *ns_per_poll) {
  if (!ctx || !expired || !ns_per_poll) return ctx ? ctx->fail(HDG_ERR_INVALID, "null output") : HDG_ERR_INVALID;
  if (polls == 0 || polls > (1u << 20))
    return ctx->fail(HDG_ERR_INVALID, "hdg_check_bounded_waits: polls must be in [1, 2^20]");
  hdg::DeviceGuard guard(ctx->device);
  cudaError_t e = guard.status;
  hdg::DBuf buf;
  buf.stream = ctx->stream;
  // [word (4 B) | expired (2 x 4 B) | pad | cycles (2 x 8 B)]
  if (e == cudaSuccess) e = buf.reserve(32);
  if (e == cudaSuccess) e = cudaMemsetAsync(buf.ptr, 0, 32, ctx->stream);
  if (e == cudaSuccess) {
    unsigned *word = buf.as<unsigned>();
    int *dexp = reinterpret_cast<int *>(word + 1);
    long long *dcyc = reinterpret_cast<long long *>(buf.as<char>() + 16);
    bounded_wait_check_kernel<<<1, 32, 0, ctx->stream>>>(polls, word, dexp, dcyc);
    ++ctx->launches;
    e = cudaGetLastError();
  }
  unsigned char host[32];
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, buf.ptr, 32, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  int khz = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, ctx->device);
  if (e != cudaSuccess) return ctx->fail(HDG_ERR_CUDA, "hdg_check_bounded_waits: %s", cudaGetErrorString(e));
  const int *hexp = reinterpret_cast<const int *>(host + 4);
  const long long *hcyc = reinterpret_cast<const long long *>(host + 16);
  for (int i = 0; i < 2; ++i) {
    expired[i] = hexp[i];
    ns_per_poll[i] = khz > 0 ? (double)hcyc[i] / polls / (khz * 1e-6) : 0.0;
  }
  return HDG_OK;
}
