// sl_sort_keys16_noalloc: the stable 16-bit key sort of sl_sort_keys16 for callers that are not allowed to allocate
// device memory.  Typical such callers are a host engine that owns every byte of device memory through its own pool
// and runs this library under a hard memory cap, or a frame loop with a fixed latency budget in which an allocator
// call (which may take a lock or wait on the device) is not acceptable.  Instead of cudaMallocAsync this variant uses
// one fixed scratch area: a file-scope __device__ array sized for at most kNoAllocMaxKeys keys, which every GPU that
// loads this library keeps for the life of the process.
//
// Host code cannot pass the array's name to a kernel: on the host that name is only a stand-in for the device
// symbol, not a device address.  Every call therefore looks the address up with cudaGetSymbolAddress while the
// caller's device is current.  No address is cached: after cudaDeviceReset, or in another context on the same
// device, the library's module is loaded again (possibly at another address), and a cached pointer would be stale.
// The first call in a context loads the module; make it before any stream capture is in progress.
#include <string>

#include "sl_runtime.h"

namespace sl {

// defined in sort_api.cu
cudaError_t sort16_in_scratch(const uint16_t* keys, uint32_t n, uint32_t* order, char* base, cudaStream_t s);

namespace {

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;  // 1,048,576 keys
// exactly the layout one sort of kNoAllocMaxKeys keys needs: digit histograms, counters and tile tickets, the
// look-back words of both passes over its tiles, the ping-pong keys (2 B) and values (4 B)
constexpr size_t kScratchBytes = sort16_layout(kNoAllocMaxKeys).total;
static_assert(kScratchBytes < (8u << 20), "the no-allocation scratch array should stay modest");

}  // namespace

static __device__ __align__(256) unsigned char g_sort16_scratch[kScratchBytes];

}  // namespace sl

using namespace sl;

extern "C" int sl_sort_keys16_noalloc(const uint16_t* keys_dev, uint32_t n, uint32_t* order_dev, void* stream) {
  if (n == 0) return SL_OK;
  if (!keys_dev || !order_dev) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n > kNoAllocMaxKeys)
    return fail(SL_ERR_INVALID_ARG, "sl_sort_keys16_noalloc sorts at most " + std::to_string(kNoAllocMaxKeys) +
                                        " keys (its fixed scratch size); got " + std::to_string(n) +
                                        ": use sl_sort_keys16");
  if (sort16_layout(n).total > kScratchBytes) return fail(SL_ERR_INVALID_ARG, "scratch layout exceeds the array");
  void* sym = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&sym, g_sort16_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(sort scratch)");
  char* base = static_cast<char*>(sym);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // every call shares the array and it keeps the previous call's contents: sort16_in_scratch clears the histograms,
  // counters and look-back status before use; keys/values scratch is fully rewritten by the passes
  e = sort16_in_scratch(keys_dev, n, order_dev, base, s);
  FrameCounters hc{};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&hc, base + sort16_layout(n).counters, sizeof(hc), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "sl_sort_keys16_noalloc");
  if (hc.timeout) return fail(SL_ERR_TIMEOUT, "sort look-back wait gave up");
  return SL_OK;
}
