// Per-tile splat lists.  After the depth sort, every visible splat (in back-to-front order) is expanded into one
// (tile, slot) entry per screen tile its candidate rectangle overlaps; a stable radix sort by tile id then leaves each
// tile's splats contiguous and still in depth order, and the runs of equal ids in the sorted keys give the ranges
// (no per-entry global atomics: only the sort's digit histograms are counted, in shared memory).  This replaces the
// reference's fixed-function path (one instanced quad per sorted splat, shaders/splat.wgsl:51-55, src/renderer.js:
// 474-485): the ranges are the rasteriser's coverage made explicit per tile.
#include "sl_internal.h"
#include "sl_tilespan.h"
#include "sl_emit.cuh"

namespace sl {
namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) tile_count_kernel(const uint32_t* __restrict__ order,
                                                              const ushort4* __restrict__ rects,
                                                              const SplatRec* __restrict__ recs, uint32_t n,
                                                              uint32_t tw, uint32_t th, const FrameCounters* ctr,
                                                              uint32_t* __restrict__ counts) {
  const uint32_t p = blockIdx.x * kThreads + threadIdx.x;
  const uint32_t visible = ctr->visible;
  const bool mine = p < n && p < visible;
  ushort4 r = make_ushort4(1, 1, 0, 0);
  SplatRec rec{};
  if (mine) {
    const uint32_t slot = order[p];
    r = rects[slot];
    rec = recs[slot];
  }
  const uint32_t c = count_warp(mine, r, rec, tw, th);
  if (p < n) counts[p] = c;
}

__global__ void __launch_bounds__(kThreads) tile_emit_kernel(const uint32_t* __restrict__ order,
                                                             const ushort4* __restrict__ rects,
                                                             const SplatRec* __restrict__ recs,
                                                             const uint32_t* __restrict__ offsets,
                                                             const uint32_t* __restrict__ counts, uint32_t n,
                                                             uint32_t tiles_x, uint32_t tw, uint32_t th,
                                                             uint32_t capacity, FrameCounters* ctr,
                                                             uint16_t* __restrict__ tile_keys,
                                                             uint32_t* __restrict__ tile_vals,
                                                             uint32_t* __restrict__ digit_hist) {
  __shared__ uint32_t h_lo[256], h_hi[256], warp_tot[kThreads / 32];
  const int t = threadIdx.x;
  RunHist16 h{h_lo, h_hi};
  h.clear();
  const uint32_t p = blockIdx.x * kThreads + t;
  const uint32_t visible = ctr->visible;
  __syncthreads();
  bool mine = false;
  uint32_t slot = 0, e0 = 0, cnt = 0;
  ushort4 r = make_ushort4(1, 1, 0, 0);
  SplatRec rec{};
  if (p < n && p < visible) {
    cnt = counts[p];
    if (cnt) {
      slot = order[p];
      r = rects[slot];
      rec = recs[slot];
      e0 = offsets[p];
      if (e0 + cnt > capacity) atomicExch(&ctr->overflow, 1u);
      else mine = true;
    }
  }
  emit_warp<uint16_t>(mine, slot, r, rec, e0, cnt, tw, th, 0u, tiles_x, tile_keys, tile_vals, h);
  __syncthreads();
  h.flush(digit_hist, warp_tot);
}

// runs of equal ids in the sorted tile keys: start and end of each tile's run
__global__ void __launch_bounds__(kThreads) tile_runs_kernel(const uint16_t* __restrict__ keys,
                                                             const uint32_t* __restrict__ n_dev, uint32_t n_max,
                                                             uint32_t* __restrict__ run_start,
                                                             uint32_t* __restrict__ run_end) {
  const uint32_t nd = *n_dev;
  const uint32_t n = nd <= n_max ? nd : 0u;  // overflowed frames are re-run by the host
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const uint32_t k = keys[i];
    if (i == 0 || keys[i - 1] != k) run_start[k] = i;
    if (i + 1 == n || keys[i + 1] != k) run_end[k] = i + 1;
  }
}

__global__ void tile_run_counts_kernel(const uint32_t* __restrict__ run_start, const uint32_t* __restrict__ run_end,
                                       uint32_t tiles, uint32_t* __restrict__ counts) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < tiles) counts[t] = run_end[t] - run_start[t];
}

__global__ void tile_ranges_kernel(const uint32_t* __restrict__ starts, const uint32_t* __restrict__ counts,
                                   uint32_t tiles, uint2* __restrict__ ranges) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < tiles) ranges[t] = make_uint2(starts[t], starts[t] + counts[t]);
}

}  // namespace

cudaError_t launch_tile_counts(const uint32_t* order, const ushort4* rects, const SplatRec* recs, uint32_t n,
                               uint32_t tw, uint32_t th, const FrameCounters* ctr, uint32_t* counts, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  tile_count_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(order, rects, recs, n, tw, th, ctr, counts);
  return cudaGetLastError();
}

cudaError_t launch_tile_emit(const uint32_t* order, const ushort4* rects, const SplatRec* recs,
                             const uint32_t* offsets, const uint32_t* counts, uint32_t n, uint32_t tiles_x,
                             uint32_t tw, uint32_t th, uint32_t capacity, FrameCounters* ctr, uint16_t* tile_keys,
                             uint32_t* tile_vals, uint32_t* digit_hist, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  tile_emit_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(order, rects, recs, offsets, counts, n, tiles_x,
                                                                       tw, th, capacity, ctr, tile_keys, tile_vals,
                                                                       digit_hist);
  return cudaGetLastError();
}

cudaError_t launch_tile_runs(const uint16_t* sorted_keys, const uint32_t* n_dev, uint32_t n_max, uint32_t* run_start,
                             uint32_t* run_end, cudaStream_t s) {
  if (n_max == 0) return cudaSuccess;
  uint32_t blocks = (n_max + kThreads * 8 - 1) / (kThreads * 8);
  if (blocks > 152 * 8) blocks = 152 * 8;
  tile_runs_kernel<<<blocks, kThreads, 0, s>>>(sorted_keys, n_dev, n_max, run_start, run_end);
  return cudaGetLastError();
}

cudaError_t launch_tile_run_counts(const uint32_t* run_start, const uint32_t* run_end, uint32_t tiles,
                                   uint32_t* counts, cudaStream_t s) {
  if (tiles == 0) return cudaSuccess;
  tile_run_counts_kernel<<<(tiles + 255) / 256, 256, 0, s>>>(run_start, run_end, tiles, counts);
  return cudaGetLastError();
}

cudaError_t launch_tile_ranges(const uint32_t* tile_starts, const uint32_t* tile_counts, uint32_t tiles,
                               uint2* ranges, cudaStream_t s) {
  if (tiles == 0) return cudaSuccess;
  tile_ranges_kernel<<<(tiles + 255) / 256, 256, 0, s>>>(tile_starts, tile_counts, tiles, ranges);
  return cudaGetLastError();
}

}  // namespace sl
