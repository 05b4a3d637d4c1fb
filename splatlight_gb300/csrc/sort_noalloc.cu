// sl_sort_keys16_noalloc: the stable 16-bit key sort of sl_sort_keys16 for callers that are not allowed to allocate
// device memory.  Typical such callers are a host engine that owns every byte of device memory through its own pool
// and runs this library under a hard memory cap, or a frame loop with a fixed latency budget in which an allocator
// call (which may take a lock or wait on the device) is not acceptable.  Instead of cudaMallocAsync this variant uses
// one fixed scratch area: a file-scope __device__ array sized for at most kNoAllocMaxKeys keys, which every GPU that
// loads this library keeps for the life of the process.
//
// Host code cannot pass the array's name to a kernel: on the host that name is only a stand-in for the device
// symbol, not a device address.  The first call on each device therefore looks the address up with
// cudaGetSymbolAddress while that device is current and caches it; later calls on that device reuse it.  Make the
// first call on a device before any stream capture is in progress.
#include <mutex>
#include <string>

#include "sl_runtime.h"

namespace sl {

// defined in sort_api.cu
struct Sort16Layout {
  size_t hist, counters, tile_ctr, status, keys_alt, vals_alt, total;
  uint32_t tiles;
};
Sort16Layout sort16_layout(uint32_t n);
cudaError_t sort16_in_scratch(const uint16_t* keys, uint32_t n, uint32_t* order, char* base, cudaStream_t s);

namespace {

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;  // 1,048,576 keys
// sort16_layout(kNoAllocMaxKeys): histograms 2 KiB, counters and tile counters 256 B each (256-byte aligned),
// look-back status 2 passes x 256 tiles x 256 digits x 4 B, keys 2 B and values 4 B per key
constexpr size_t kScratchBytes = 2048 + 256 + 256 + 2ull * 256 * 256 * 4 + 2ull * kNoAllocMaxKeys +
                                 4ull * kNoAllocMaxKeys;  // 6,818,304 B (6.5 MiB)

std::mutex g_mu;
char* g_scratch_addr[128] = {};  // device address of the array, per device ordinal

}  // namespace

static __device__ __align__(256) unsigned char g_sort16_scratch[kScratchBytes];

// Device address of g_sort16_scratch on the current device (looked up once per device).
static cudaError_t scratch_address(char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 128) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort16_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = static_cast<char*>(p);
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

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
  char* base = nullptr;
  cudaError_t e = scratch_address(&base);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(sort scratch)");
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
