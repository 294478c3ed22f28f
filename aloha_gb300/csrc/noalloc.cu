// noalloc.cu -- aloha_composite_over_noalloc: the ordered "over" composite
// without any device allocation.
//
// aloha_composite_over stages the composite order in a device buffer it
// allocates per call (cudaMalloc / cudaFree).  Some callers cannot allocate
// device memory at that point: a compositing stage called from inside
// another library's frame loop whose memory pool forbids extra allocations,
// or a real-time host that bans allocation after start-up.  This entry point
// stages the order in a fixed device array that lives in the library instead:
//
//   * the array is a file-scope __device__ array of kNoAllocMaxRanks ints
//     (16 KB); every GPU that loads the library holds it until exit;
//   * its device address is looked up with cudaGetSymbolAddress once per
//     device, on the first call made with that device current;
//   * the call cannot be recorded into a CUDA graph (its order copy is from
//     pageable memory): on a capturing stream it returns
//     ALOHA_ERR_UNSUPPORTED without touching the stream;
//   * every call on a device shares the one array and overwrites the first
//     n_ranks entries, so calls whose copies or kernels overlap on the GPU
//     race; issue them on one stream or wait in between;
//   * more than kNoAllocMaxRanks ranks is rejected with
//     ALOHA_ERR_OUT_OF_RANGE.
//
// Images and the frame buffer must be device memory of the current device
// (the caller owns them); the order is read from host memory.  The call
// takes a private snapshot of the order, checks the snapshot and copies the
// snapshot into the array, so the caller may change or free its order buffer
// as soon as the call returns.  The snapshot lives in pageable memory: the
// runtime stages it before the copy call returns, after waiting for the
// stream's earlier work, so the call is not fully asynchronous.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "batch_internal.h"
#include "internal.h"

namespace aloha {

constexpr int kNoAllocMaxRanks = 4096;
constexpr int kNoAllocMaxDevices = 64;

namespace {

__device__ __align__(256) int g_noalloc_order[kNoAllocMaxRanks];

std::mutex g_setup_mutex;
int* g_order_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_order for the current device (set up once).
cudaError_t order_scratch(int** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_order_ptr[dev]) {
    int* p = nullptr;
    e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_order);
    if (e != cudaSuccess) return e;
    g_order_ptr[dev] = p;
  }
  *out = g_order_ptr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace aloha

extern "C" int aloha_composite_over_noalloc(const float* rank_images, const int* order, int n_ranks, int width,
                                            int height, int mode, uint32_t* fb, void* stream) {
  using namespace aloha;
  if (!rank_images || !order || !fb) return ALOHA_ERR_NULL_POINTER;
  if (n_ranks < 1 || width < 1 || height < 1 || (long long)width * height > (1ll << 30))
    return ALOHA_ERR_INVALID_ARGUMENT;
  if (n_ranks > kNoAllocMaxRanks) return ALOHA_ERR_OUT_OF_RANGE;
  if (mode != ALOHA_COMPOSITE_FP32 && mode != ALOHA_COMPOSITE_UBYTE) return ALOHA_ERR_INVALID_ARGUMENT;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return ALOHA_ERR_CUDA;
  if (!device_pointer_on(rank_images, dev) || !device_pointer_on(fb, dev) || ctx_is_device_pointer(order))
    return ALOHA_ERR_INVALID_ARGUMENT;
  // Snapshot first, then check and copy the snapshot: the caller's buffer is
  // read once, here, so later changes to it cannot reach the kernel.
  int snapshot[kNoAllocMaxRanks];
  std::memcpy(snapshot, order, sizeof(int) * (size_t)n_ranks);
  for (int k = 0; k < n_ranks; ++k)
    if (snapshot[k] < 0 || snapshot[k] >= n_ranks) return ALOHA_ERR_OUT_OF_RANGE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  {
    // The snapshot copy is from pageable memory, which a stream capture
    // cannot record; refuse before touching the stream, so that the caller's
    // capture stays valid.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
      cudaGetLastError();
      return ALOHA_ERR_UNSUPPORTED;
    }
    if (cs != cudaStreamCaptureStatusNone) return ALOHA_ERR_UNSUPPORTED;
  }
  int* d_order = nullptr;
  if (order_scratch(&d_order) != cudaSuccess) return ALOHA_ERR_CUDA;
  // pageable source: staged by the runtime before the call returns
  if (cudaMemcpyAsync(d_order, snapshot, sizeof(int) * (size_t)n_ranks, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return ALOHA_ERR_CUDA;
  if (launch_composite_f32(reinterpret_cast<const float4*>(rank_images), d_order, n_ranks, width * height, mode, fb,
                           s) != cudaSuccess)
    return ALOHA_ERR_CUDA;
  return ALOHA_OK;
}
