// dmsc_noalloc.cu -- an exclusive prefix scan that allocates no device memory.
//
// dmsc_prefix_scan takes its scratch (the per-block partial sums) from the
// stream-ordered allocator.  Some callers cannot let a library allocate:
//  - a host runtime that reserves all of the GPU's memory for its own pool
//    up front.  A cudaMalloc or cudaMallocAsync from inside the library then
//    fails, or takes memory the pool has promised elsewhere.
//  - a latency-bound serving loop.  cudaMalloc synchronises the device and
//    cudaFree can stall behind queued work, so neither may appear on that path.
// For them this file keeps the scratch in a fixed device array compiled into
// the library.  Every GPU that loads libdmsc.so holds the array until the
// process exits.
#include <cuda.h>

#include <mutex>
#include <string>

#include "dmsc.h"
#include "dmsc_internal.h"
#include "grid_types.h"

namespace {
// Largest scan the fixed scratch can serve: 2^26 (67,108,864) elements.
constexpr long long kNoAllocScanMax = 1ll << 26;
// Partial sums of every level for kNoAllocScanMax elements (4096 per block):
// 2 * 16384 + 2 * 4 words, rounded up.  About 128 KiB.
constexpr long long kNoAllocScratchWords = 2 * (kNoAllocScanMax / 4096) + 64;
constexpr int kMaxDevices = 64;

std::mutex g_setup_mu;
// Per device: the array's device address and the context it was looked up
// in.  A device reset (cudaDeviceReset, or the primary context torn down and
// created again) gives the device a new context in which the array may sit
// elsewhere, so the address is looked up again when the context changes.
uint32_t *g_scratch_addr[kMaxDevices] = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};

// cuCtxGetCurrent through the runtime's driver entry point: the library does
// not link the driver library itself.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return (CtxGetCurrentFn)p;
  }();
  return fn;
}
}  // namespace

// The scratch itself.  In host code its name is only a stand-in for the
// symbol, so kernels are always given the address from cudaGetSymbolAddress.
static __device__ __align__(256) uint32_t g_noalloc_scan_scratch[kNoAllocScratchWords];

extern "C" int dmsc_prefix_scan_noalloc(dmsc_ctx *ctx, uint32_t *d_out, const uint32_t *d_in, int64_t n,
                                        uint32_t *d_total, void *stream) {
  if (!ctx || n < 0 || (n > 0 && (!d_out || !d_in))) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "bad argument");
  if (n > kNoAllocScanMax)
    return dmsc::set_last_error(DMSC_ERR_BAD_ARG,
                                ("dmsc_prefix_scan_noalloc: n = " + std::to_string(n) + " exceeds the fixed scratch limit of " +
                                 std::to_string(kNoAllocScanMax) + " elements; use dmsc_prefix_scan").c_str());
  if (ctx->device < 0 || ctx->device >= kMaxDevices) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "device id out of range");
  if (dmsc::scan_scratch_words(n) > kNoAllocScratchWords)
    return dmsc::set_last_error(DMSC_ERR_INVARIANT, "scan scratch sizing");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return dmsc::set_last_error(DMSC_ERR_CUDA, cudaGetErrorString(e));
  uint32_t *scratch = nullptr;
  {
    // First call on a device (or on its new context after a reset): look up
    // the array's device address with that device current.  (This is why the
    // first call should come before any stream capture.)
    std::lock_guard<std::mutex> lk(g_setup_mu);
    CUcontext cur = nullptr;
    const CtxGetCurrentFn get = ctx_get_current();
    if (get && get(&cur) != CUDA_SUCCESS) cur = nullptr;
    if (!g_scratch_addr[ctx->device] || cur != g_scratch_ctx[ctx->device]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
      if (e != cudaSuccess) return dmsc::set_last_error(DMSC_ERR_CUDA, cudaGetErrorString(e));
      g_scratch_addr[ctx->device] = (uint32_t *)p;
      if (get && get(&cur) != CUDA_SUCCESS) cur = nullptr;  // the lookup makes the context current
      g_scratch_ctx[ctx->device] = cur;
    }
    scratch = g_scratch_addr[ctx->device];
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  // No scratch word is read before it is written, so leftovers of an earlier
  // call need no clearing.
  e = dmsc::scan_exclusive_u32_scratch(d_in, n, d_out, d_total, scratch, st);
  if (e != cudaSuccess) return dmsc::set_last_error(DMSC_ERR_CUDA, cudaGetErrorString(e));
  return DMSC_OK;
}
