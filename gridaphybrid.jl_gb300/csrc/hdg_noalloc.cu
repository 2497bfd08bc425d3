// hdg_noalloc.cu -- an allocation-free variant of the FP32 + float-float
// refined static condensation (hdg_static_condensation_noalloc).
//
// Some callers cannot allocate device memory: a host framework whose caching
// allocator already holds the device's free memory, or a step that runs inside
// a larger pipeline where an allocation would synchronise the device or take
// allocator locks.  This entry point gives them the FP32+refined condensation
// with every temporary in a fixed, file-scope device array instead of
// allocator memory.
//
// The refined condensation stages each FP64 cell block as a pair of FP32
// arrays (hi, lo) before the FP32 LU; those staging arrays are the scratch.
// It lives in `noalloc_scratch` below: HDG_NOALLOC_SCRATCH_BYTES bytes that
// every GPU which loads this library holds until the process exits.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in).  The device address is looked up once per
// device with cudaGetSymbolAddress, with that device current, on the first
// call made on that device.
// Every call waits for its own work to finish (it synchronises the context's
// stream to read the pivot flag) before it returns, and leaves the caller's
// current device as it found it.  Because of that synchronisation no call can
// be captured into a CUDA graph.
// All calls share the one array: calls whose work overlaps on the GPU race
// with each other and must be serialised by the caller (one stream, or
// events).  The array keeps the contents of the last call; everything that
// must start at zero is cleared by each call.
#include <cuda_runtime.h>

#include <mutex>

#include "hdg_internal.h"
#include "hdg_kernels.h"

namespace {

constexpr size_t kNoallocBytes = HDG_NOALLOC_SCRATCH_BYTES;

// The scratch: [ A_hi | A_lo | b_hi | b_lo ] as floats, then one int flag,
// then ncells ints of LAPACK info when the caller passes info == NULL.
static __device__ __align__(256) unsigned char noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of noalloc_scratch on `device` (which must be current).
cudaError_t scratch_address(int device, void **out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return cudaSuccess;
}

__global__ void noalloc_any_nonzero(int n, const int *__restrict__ info, int *flag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (info[i] != 0) atomicOr(flag, 1);
}

// Device memory of the context's GPU (or managed memory): the only pointers
// this entry point takes.  Device memory of another GPU is refused too.
bool on_ctx_device(const hdg_context *ctx, const void *p) {
  return hdg::ptr_place(p, ctx->device) == hdg::PtrPlace::Device;
}

}  // namespace

extern "C" int hdg_static_condensation_noalloc(hdg_context *ctx, int ncells, int ni, int nf,
                                               const double *A, const double *b, double *S,
                                               double *g, int *info) {
  if (!ctx) return HDG_ERR_INVALID;
  if (ncells < 0 || ni < 1 || nf < 0 || !A || !b || !S || !g)
    return ctx->fail(HDG_ERR_INVALID, "hdg_static_condensation_noalloc: bad arguments");
  if (ncells == 0) return HDG_OK;
  const size_t n = (size_t)ni + nf;
  const size_t nA = (size_t)ncells * n * n, nb = (size_t)ncells * n;
  const size_t floats = 2 * (nA + nb);
  const size_t flag_off = (floats * sizeof(float) + 255) / 256 * 256;
  const size_t need = flag_off + 256 + (info ? 0 : sizeof(int) * (size_t)ncells);
  if (need > kNoallocBytes)
    return ctx->fail(HDG_ERR_INVALID,
                     "hdg_static_condensation_noalloc: %d cells of %zu x %zu need %zu bytes of scratch, "
                     "the fixed maximum is %zu bytes; split the batch",
                     ncells, n, n, need, kNoallocBytes);
  if (hdg::condense_mixed_smem(ni, nf) > ctx->smem_optin - 1024)
    return ctx->fail(HDG_ERR_INVALID, "cell block %zu x %zu exceeds the shared-memory condensation kernel", n, n);
  if (!on_ctx_device(ctx, A) || !on_ctx_device(ctx, b) || !on_ctx_device(ctx, S) || !on_ctx_device(ctx, g) ||
      (info && !on_ctx_device(ctx, info)))
    return ctx->fail(HDG_ERR_INVALID,
                     "hdg_static_condensation_noalloc takes device pointers of the context's GPU (%d) only",
                     ctx->device);
  // the caller's current device is given back on every return below
  hdg::DeviceGuard guard(ctx->device);
  cudaError_t e = guard.status;
  void *base = nullptr;
  if (e == cudaSuccess) e = scratch_address(ctx->device, &base);
  if (e != cudaSuccess)
    return ctx->fail(HDG_ERR_CUDA, "noalloc scratch set-up: %s", cudaGetErrorString(e));
  float *Ahi = static_cast<float *>(base), *Alo = Ahi + nA, *bhi = Alo + nA, *blo = bhi + nb;
  int *flag = reinterpret_cast<int *>(static_cast<unsigned char *>(base) + flag_off);
  int *dinfo = info ? info : flag + 64;
  e = cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream);
  if (e == cudaSuccess)
    e = hdg::launch_split_fp64(nA, A, Ahi, Alo, ctx->stream, ctx->num_sms, &ctx->launches);
  if (e == cudaSuccess)
    e = hdg::launch_split_fp64(nb, b, bhi, blo, ctx->stream, ctx->num_sms, &ctx->launches);
  if (e == cudaSuccess)
    e = hdg::launch_condense_mixed(ncells, ni, nf, Ahi, Alo, bhi, blo, S, g, nullptr, nullptr, dinfo,
                                   ctx->stream, ctx->num_sms, &ctx->launches);
  if (e == cudaSuccess) {
    const int grid = (ncells + 255) / 256 < 1024 ? (ncells + 255) / 256 : 1024;
    noalloc_any_nonzero<<<grid, 256, 0, ctx->stream>>>(ncells, dinfo, flag);
    ++ctx->launches;
    e = cudaGetLastError();
  }
  int bad = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return ctx->fail(HDG_ERR_CUDA, "hdg_static_condensation_noalloc: %s", cudaGetErrorString(e));
  if (bad) return ctx->fail(HDG_ERR_SINGULAR, "zero pivot in an interior block (see info)");
  return HDG_OK;
}
