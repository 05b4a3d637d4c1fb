// Standalone stable sorts of 16- and 32-bit keys (the depth-key sort of shaders/radix.wgsl:1-139, outside a frame):
// the digit histograms, then the onesweep passes of sort.cu.  Scratch is allocated stream-ordered per call from a
// memory pool private to the library whose memory is kept between calls (a release threshold of "never"), so a
// repeated sort maps no new memory; the pool holds at most the largest scratch ever requested per device.
#include <mutex>
#include <string>

#include "sl_runtime.h"

namespace sl {

// The per-device scratch pool (created on first use).
static cudaError_t scratch_pool(cudaMemPool_t* out) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    if ((e = cudaMemPoolCreate(&pools[dev], &props)) != cudaSuccess) return e;
    uint64_t keep = ~0ull;
    if ((e = cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) return e;
  }
  *out = pools[dev];
  return cudaSuccess;
}

static cudaError_t scratch_alloc(char** base, size_t bytes, cudaStream_t s) {
  cudaMemPool_t pool;
  cudaError_t e = scratch_pool(&pool);
  if (e != cudaSuccess) return e;
  return cudaMallocFromPoolAsync(reinterpret_cast<void**>(base), bytes, pool, s);
}

static size_t align256(size_t x) { return align256c(x); }

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

namespace {

// scatter.wgsl's histogram side (shaders/project.wgsl:369 atomicAdd(histogram[key])): one count per valid key
__global__ void __launch_bounds__(256) key_hist_kernel(const uint16_t* __restrict__ key16, uint32_t n,
                                                       uint32_t* __restrict__ hist) {
  const uint32_t i = blockIdx.x * 256u + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = key16[i];
  if (k != kInvalidKey16) atomicAdd(&hist[k], 1u);
}

// shaders/scatter.wgsl:9-18: each valid slot takes the next position of its key's range
__global__ void __launch_bounds__(256) key_scatter_kernel(const uint16_t* __restrict__ key16, uint32_t n,
                                                          uint32_t* __restrict__ offsets, uint32_t* __restrict__ order) {
  const uint32_t i = blockIdx.x * 256u + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = key16[i];
  if (k != kInvalidKey16) order[atomicAdd(&offsets[k], 1u)] = i;
}

}  // namespace

cudaError_t launch_key_hist(const uint16_t* key16, uint32_t n, uint32_t* hist, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  key_hist_kernel<<<(n + 255u) / 256u, 256, 0, s>>>(key16, n, hist);
  return cudaGetLastError();
}

cudaError_t launch_key_scatter(const uint16_t* key16, uint32_t n, uint32_t* offsets, uint32_t* order, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  key_scatter_kernel<<<(n + 255u) / 256u, 256, 0, s>>>(key16, n, offsets, order);
  return cudaGetLastError();
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
  cudaError_t e = scratch_alloc(&base, L.total, s);
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

extern "C" int sl_sort_keys32(const uint32_t* keys_dev, uint32_t n, uint32_t bits, uint32_t* order_dev, void* stream) {
  if (n == 0) return SL_OK;
  if (!keys_dev || !order_dev) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n > (1u << 30) - 1) return fail(SL_ERR_INVALID_ARG, "n must be below 2^30");
  if (bits < 1 || bits > 32) return fail(SL_ERR_INVALID_ARG, "bits must be 1..32");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int passes = bits <= 8 ? 1 : (int)((bits + 7) / 8);
  const uint32_t tiles = (uint32_t)sort_tiles_for(n);
  size_t off = 0;
  const size_t o_hist = off;
  off = align256(off + 4 * 256 * 4);
  const size_t o_ctr = off;
  off = align256(off + sizeof(FrameCounters));
  const size_t o_tctr = off;
  off = align256(off + 16);
  const size_t o_status = off;
  off = align256(off + 4ull * 256 * 4 * tiles);
  const size_t o_ka = off;
  off = align256(off + 4ull * n);
  const size_t o_kb = off;
  off = align256(off + 4ull * n);
  const size_t o_va = off;
  off = align256(off + 4ull * n);
  char* base = nullptr;
  cudaError_t e = scratch_alloc(&base, off, s);
  if (e != cudaSuccess) return cuda_fail(e, "sl_sort_keys32 scratch");
  e = cudaMemsetAsync(base, 0, o_status, s);
  uint32_t* hist = reinterpret_cast<uint32_t*>(base + o_hist);
  FrameCounters* ctr = reinterpret_cast<FrameCounters*>(base + o_ctr);
  if (e == cudaSuccess) e = launch_digit_hist32(keys_dev, n, passes, hist, s);
  if (e == cudaSuccess)
    e = sort32_pairs(reinterpret_cast<uint32_t*>(base + o_ka), reinterpret_cast<uint32_t*>(base + o_kb), nullptr,
                     order_dev, reinterpret_cast<uint32_t*>(base + o_va), n, nullptr, (int)bits, hist,
                     reinterpret_cast<uint32_t*>(base + o_status), reinterpret_cast<uint32_t*>(base + o_tctr), tiles,
                     ctr, s, nullptr, keys_dev);
  FrameCounters hc{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, s);
  cudaError_t e2 = cudaFreeAsync(base, s);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "sl_sort_keys32");
  if (hc.timeout) return fail(SL_ERR_TIMEOUT, "sort look-back wait gave up");
  return SL_OK;
}
