// dsgl_noalloc.cu -- sgns_minibatch_update_noalloc: the explicit-row minibatch update
// for callers that must not have the library allocate device memory.
//
// Such callers exist: a process whose device memory is owned by its own allocator (a
// framework's caching allocator, or a serving process that reserves the GPU's memory
// up front) cannot have a library call cudaMalloc behind its back -- the call can fail
// for lack of memory the caller has already claimed, fragments a pool the caller
// manages, and cudaMalloc/cudaFree may synchronise the device in the middle of the
// caller's pipeline.  This entry point keeps its scratch (the per-minibatch row offsets
// and a status word) and the sigmoid table in statically allocated device memory
// instead: g_noalloc_scratch below, sized for kNoAllocMaxBatches minibatches.  Every GPU
// that loads the library holds these arrays (about 1 MiB) until the process exits.
//
// The kernel and the arithmetic are those of sgns_minibatch_update; only where the
// scratch lives differs.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "sgns.h"
#include "sgns_internal.h"

namespace sgns {
namespace {

constexpr int kNoAllocMaxBatches = 65536;
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
  int64_t offsets[2 * kNoAllocMaxBatches];  // per-minibatch row offsets (inputs, outputs)
  int32_t status;                           // set by the kernel for an over-limit minibatch
  int32_t pad[63];
  float exp_table[kExpTableSize + 1 + 3];   // sigmoid table of dsgl.hpp:1557-1562
};

// Device-side scratch.  In host code this name is only a stand-in for the symbol; the
// device address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_setup_mx;
NoAllocScratch* g_scratch_addr[kMaxDevices] = {nullptr};

// Once per device, with that device current: resolve the scratch address and fill the
// sigmoid table (a copy to an existing symbol; nothing is allocated).
int setup_device(int dev, NoAllocScratch** out) {
  std::lock_guard<std::mutex> g(g_setup_mx);
  if (!g_scratch_addr[dev]) {
    NoAllocScratch* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&ptr), g_noalloc_scratch);
    if (e != cudaSuccess)
      return report_error(SGNS_ECUDA, "minibatch (no-alloc): cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    float et[kExpTableSize + 1];
    host_exp_table(et);
    e = cudaMemcpyToSymbol(g_noalloc_scratch, et, sizeof et, offsetof(NoAllocScratch, exp_table),
                           cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
      return report_error(SGNS_ECUDA, "minibatch (no-alloc): sigmoid table upload failed: %s", cudaGetErrorString(e));
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return SGNS_OK;
}

}  // namespace
}  // namespace sgns

using namespace sgns;

extern "C" sgns_status sgns_minibatch_update_noalloc(int32_t d, int32_t n, const int32_t* in_count,
                                                     const int32_t* in_first, const int32_t* out_count,
                                                     const int32_t* out_meta, const float* alpha,
                                                     const float* in_rows, const float* out_rows, float* d_in,
                                                     float* d_out, void* stream) {
  if (d < 4 || d > kDMax || d % 4 || n < 0)
    return (sgns_status)report_error(SGNS_EINVAL, "minibatch (no-alloc): bad arguments (d=%d, n=%d)", d, n);
  if (n > kNoAllocMaxBatches)
    return (sgns_status)report_error(SGNS_EINVAL,
                                     "minibatch (no-alloc): %d minibatches exceed the static scratch limit of %d; "
                                     "split the call or use sgns_minibatch_update",
                                     n, kNoAllocMaxBatches);
  if (n == 0) return SGNS_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return (sgns_status)report_error(SGNS_ECUDA, "minibatch (no-alloc): no usable current device");
  NoAllocScratch* sc = nullptr;
  int st = setup_device(dev, &sc);
  if (st != SGNS_OK) return (sgns_status)st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the status word keeps the previous call's value: clear it
  cudaError_t e = cudaMemsetAsync(&sc->status, 0, sizeof(int32_t), s);
  if (e == cudaSuccess)
    e = launch_minibatch(d, n, kIMax, kOMax, in_count, in_first, out_count, out_meta, alpha, in_rows, out_rows, d_in,
                         d_out, sc->exp_table, sc->offsets, &sc->status, s);
  int32_t hs = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, &sc->status, sizeof hs, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return (sgns_status)report_error(SGNS_ECUDA, "minibatch (no-alloc): %s", cudaGetErrorString(e));
  if (hs)
    return (sgns_status)report_error(SGNS_EINVAL, "minibatch (no-alloc): a minibatch exceeds %d inputs / %d outputs "
                                     "or has first > inputs", kIMax, kOMax);
  return SGNS_OK;
}
