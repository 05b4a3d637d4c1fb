// Standalone stable sort of 16-bit keys (the depth-key sort of shaders/radix.wgsl:1-139, outside a frame): the
// digit histograms, then the two onesweep passes of sort.cu.  Scratch is allocated stream-ordered
// (cudaMallocAsync/cudaFreeAsync) per call.
#include <string>

#include "sl_runtime.h"

namespace sl {

// Scratch layout of one 16-bit sort of up to n keys (all offsets 256-byte aligned).
struct Sort16Layout {
  size_t hist, counters, tile_ctr, status, keys_alt, vals_alt, total;
  uint32_t tiles;
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

Sort16Layout sort16_layout(uint32_t n) {
  Sort16Layout L;
  L.tiles = (uint32_t)sort_tiles_for(n ? n : 1);
  size_t off = 0;
  L.hist = off;
  off = align256(off + 2 * 256 * 4);
  L.counters = off;
  off = align256(off + sizeof(FrameCounters));
  L.tile_ctr = off;
  off = align256(off + 16);
  L.status = off;
  off = align256(off + 2ull * 256 * 4 * L.tiles);
  L.keys_alt = off;
  off = align256(off + 2ull * n);
  L.vals_alt = off;
  off = align256(off + 4ull * n);
  L.total = off;
  return L;
}

// Runs the sort in `base` (a scratch block laid out by sort16_layout(n)); clears what must start at zero.
cudaError_t sort16_in_scratch(const uint16_t* keys, uint32_t n, uint32_t* order, char* base, cudaStream_t s) {
  Sort16Layout L = sort16_layout(n);
  cudaError_t e = cudaMemsetAsync(base, 0, L.status, s);  // histograms, counters, tile counters
  if (e != cudaSuccess) return e;
  uint32_t* hist = reinterpret_cast<uint32_t*>(base + L.hist);
  FrameCounters* ctr = reinterpret_cast<FrameCounters*>(base + L.counters);
  if ((e = launch_digit_hist16(keys, n, 2, hist, s)) != cudaSuccess) return e;
  SortScratch sc{reinterpret_cast<uint16_t*>(base + L.keys_alt), reinterpret_cast<uint32_t*>(base + L.vals_alt),
                 reinterpret_cast<uint32_t*>(base + L.status), reinterpret_cast<uint32_t*>(base + L.tile_ctr),
                 L.tiles};
  return sort16_pairs(const_cast<uint16_t*>(keys), nullptr, order, n, nullptr, 16, hist, sc, ctr, s);
}

}  // namespace sl

using namespace sl;

extern "C" int sl_sort_keys16(const uint16_t* keys_dev, uint32_t n, uint32_t* order_dev, void* stream) {
  if (n == 0) return SL_OK;
  if (!keys_dev || !order_dev) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n > (1u << 30) - 1) return fail(SL_ERR_INVALID_ARG, "n must be below 2^30");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Sort16Layout L = sort16_layout(n);
  char* base = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&base), L.total, s);
  if (e != cudaSuccess) return cuda_fail(e, "sl_sort_keys16 scratch");
  e = sort16_in_scratch(keys_dev, n, order_dev, base, s);
  FrameCounters hc{};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&hc, base + L.counters, sizeof(hc), cudaMemcpyDeviceToHost, s);
  cudaError_t e2 = cudaFreeAsync(base, s);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "sl_sort_keys16");
  if (hc.timeout) return fail(SL_ERR_TIMEOUT, "sort look-back wait gave up");
  return SL_OK;
}
