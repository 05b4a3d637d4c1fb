// Host-side runtime objects behind the C ABI (renderer, device buffers, error reporting).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "sl_internal.h"

namespace sl {

// thread-local last error text (sl_last_error)
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// A device buffer that grows on demand (contents are not preserved across growth).
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t b = want + want / 4 + 256;
    cudaError_t e = cudaMalloc(&ptr, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(ptr);
  }
};

// Per-view working buffers of the project -> sort -> bin -> composite chain.
struct ViewBuffers {
  DevBuf key16, recs, rects, order, slot_counts, slot_offsets;  // per slot
  DevBuf keys_alt, vals_alt, status, tile_ctr;                 // sort scratch (max of slots, entries)
  DevBuf tile_keys, tile_vals;                                 // per entry
  DevBuf tile_counts, tile_starts, ranges, run_start, run_end; // per tile
  DevBuf digit_hist;                                           // [4][256]: depth-key passes, tile-key passes
  DevBuf scan_scratch;
  DevBuf counters;                                             // FrameCounters
  DevBuf out, counts;                                          // composite targets when the caller's are on the host
  void release_all();
};

struct RenderTimings {
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};

}  // namespace sl

struct sl_renderer {
  int device = 0;
  uint32_t count = 0, part_count = 0, max_emitters = 0, n_emitters = 0;
  sl::DevBuf gaussians, emitters;
  std::vector<sl_part> parts;
  const float4* colour = nullptr;  // bound radiance (float4 per Gaussian)
  const float4* lo_b = nullptr;
  sl_lighting* lighting = nullptr;
  uint32_t tile_w = 16, tile_h = 16;
  float t_stop_scale = 1e-4f;
  uint64_t entry_capacity = 0;
  bool timing = false;
  sl::RenderTimings tm;
  sl::ViewBuffers vb;
  sl::FrameCounters* host_ctr = nullptr;  // pinned
  // last frame (debug read-back)
  uint32_t last_slots = 0, last_w = 0, last_h = 0, last_tiles = 0, last_entries = 0, last_mode = 0;
  bool have_frame = false;
};
