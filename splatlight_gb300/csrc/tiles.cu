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

// Tile counts, their offsets and the entries in one pass over the depth-sorted visible splats (positions below
// ctr->visible): each block of 256 positions counts its splats' tile entries (the per-row spans), learns the entries
// of every earlier block by a decoupled look-back (blocks take their positions from a ticket counter), and writes its
// entries -- key the tile id ty * tiles_x + tx, value the slot -- at the running offset, so entries stay in depth
// order.
// The digit counts of the tile id go to digit_hist for the tile sort; the last block writes the entry total to
// ctr->entries (which may exceed capacity: the entries past it are not written and the overflow flag is set).
__global__ void __launch_bounds__(kThreads) tile_bin_kernel(const uint32_t* __restrict__ order,
                                                            const ushort4* __restrict__ rects,
                                                            const SplatRec* __restrict__ recs, uint32_t n,
                                                            uint32_t tiles_x, uint32_t tw, uint32_t th,
                                                            uint32_t capacity, FrameCounters* ctr,
                                                            uint16_t* __restrict__ tile_keys,
                                                            uint32_t* __restrict__ tile_vals,
                                                            uint32_t* __restrict__ digit_hist, uint32_t* ticket,
                                                            uint64_t* status) {
  __shared__ uint32_t h_lo[256], h_hi[256], warp_tot[kThreads / 32];
  __shared__ uint32_t s_blk, s_excl;
  const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
  const uint32_t visible = ctr->visible;
  const uint32_t nv = visible < n ? visible : n;
  if (t == 0) s_blk = atomicAdd(ticket, 1u);
  RunHist16 h{h_lo, h_hi};
  h.clear();
  __syncthreads();
  const uint32_t blk = s_blk;
  if (blk * kThreads >= nv) return;  // past the visible positions (the whole block)
  const uint32_t p = blk * kThreads + t;
  const bool in = p < nv;
  uint32_t slot = 0;
  ushort4 r = make_ushort4(1, 1, 0, 0);
  SplatRec rec{};
  if (in) {
    slot = order[p];
    r = rects[slot];
    if (r.x <= r.z && r.y <= r.w) rec = recs[slot];  // culled slots (empty rectangle) need no record
  }
  const uint32_t cnt = count_warp(in, r, rec, tw, th);
  uint32_t x = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31u) warp_tot[w] = x;
  __syncthreads();
  uint32_t wbase = 0, agg = 0;
#pragma unroll
  for (uint32_t k = 0; k < kThreads / 32; k++) {
    const uint32_t tt = warp_tot[k];
    wbase += k < w ? tt : 0u;
    agg += tt;
  }
  if (w == 0) {  // warp 0: the block's offset from the look-back
    const uint32_t excl = lookback_warp(status, blk, 0u, agg, &ctr->timeout);
    if (lane == 0) {
      s_excl = excl;
      if ((blk + 1u) * kThreads >= nv) ctr->entries = excl + agg;  // the last block
    }
  }
  __syncthreads();
  const uint32_t e0 = s_excl + wbase + x - cnt;
  bool mine = false;
  if (cnt) {
    if (e0 + cnt > capacity) atomicExch(&ctr->overflow, 1u);
    else mine = true;
  }
  emit_warp<uint16_t>(mine, slot, r, rec, e0, cnt, tw, th, 0u, tiles_x, tile_keys, tile_vals, h);
  __syncthreads();
  h.flush(digit_hist, warp_tot);
}

// After the stable sort by tile id each tile's entries are one contiguous, depth-ordered run: its bounds go straight
// to ranges[tile] (ranges zeroed beforehand: empty tiles keep [0, 0)).
__global__ void __launch_bounds__(kThreads) tile_ranges_kernel(const uint16_t* __restrict__ keys,
                                                               const uint32_t* __restrict__ n_dev, uint32_t n_max,
                                                               uint2* __restrict__ ranges) {
  const uint32_t nd = *n_dev;
  const uint32_t n = nd <= n_max ? nd : 0u;  // overflowed frames are re-run by the host
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const uint32_t k = keys[i];
    const bool first = i == 0 || keys[i - 1] != k, last = i + 1 == n || keys[i + 1] != k;
    if (first) ranges[k].x = i;
    if (last) ranges[k].y = i + 1;
  }
}

}  // namespace

size_t tile_bin_scratch_bytes(uint32_t n) { return 16 + 8ull * ((n + kThreads - 1) / kThreads + 1); }

cudaError_t launch_tile_bin(const uint32_t* order, const ushort4* rects, const SplatRec* recs, uint32_t n,
                            uint32_t tiles_x, uint32_t tw, uint32_t th, uint32_t capacity, FrameCounters* ctr,
                            uint16_t* tile_keys, uint32_t* tile_vals, uint32_t* digit_hist, void* scratch,
                            cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(scratch, 0, tile_bin_scratch_bytes(n), s);
  if (e != cudaSuccess) return e;
  uint32_t* ticket = reinterpret_cast<uint32_t*>(scratch);
  uint64_t* status = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(scratch) + 16);
  tile_bin_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(order, rects, recs, n, tiles_x, tw, th, capacity,
                                                                      ctr, tile_keys, tile_vals, digit_hist, ticket,
                                                                      status);
  return cudaGetLastError();
}

cudaError_t launch_tile_ranges(const uint16_t* sorted_keys, const uint32_t* n_dev, uint32_t n_max, uint2* ranges,
                               cudaStream_t s) {
  if (n_max == 0) return cudaSuccess;
  uint32_t blocks = (n_max + kThreads * 8 - 1) / (kThreads * 8);
  if (blocks > 152 * 8) blocks = 152 * 8;
  tile_ranges_kernel<<<blocks, kThreads, 0, s>>>(sorted_keys, n_dev, n_max, ranges);
  return cudaGetLastError();
}

}  // namespace sl
