// Batched tile binning: the per-view binning of tiles.cu over all views of a batch at once.  The depth-sorted
// permutation covers every view's slots in view order (keys carry the view above the depth bits), so each visible
// splat emits (global tile id, slot) entries with global tile id = the view's first tile + its local tile id; one
// stable sort by that id leaves every tile's list contiguous and in back-to-front order.  Element counts are read
// on the device (grids are sized for the batch's capacity, so a CUDA graph of the chain can be replayed for any
// batch that fits).
#include "sl_internal.h"
#include "sl_tilespan.h"
#include "sl_emit.cuh"
#include "sl_lighting.h"

namespace sl {
namespace {

constexpr int kThreads = 256;

// The binning of the batch in one pass over the depth-sorted visible splats: each block of 256 sorted positions
// counts its splats' tile entries (the per-row spans), learns the entries of every earlier block by a decoupled
// look-back over per-block status words (blocks take their positions from a ticket counter, so every earlier block is
// already running and the wait ends), and writes its entries: key (view << 16) | view-local tile id, value the slot,
// at the running offset, so entries stay in sorted (view, depth) order.  The digit counts of the local id go to
// digit_hist for the tile sort; the last block writes the batch's entry total (which may exceed capacity: the entries
// past it are not written and the overflow flag is set).
template <int MinB>
__global__ void __launch_bounds__(kThreads, MinB) btile_bin_kernel(const uint32_t* __restrict__ order,
                                                             const ushort4* __restrict__ rects,
                                                             const SplatRec* __restrict__ recs,
                                                             const BatchView* __restrict__ views,
                                                             const uint32_t* __restrict__ block_view,
                                                             const uint32_t* __restrict__ n_dev, uint32_t n_max,
                                                             uint32_t tw, uint32_t th, uint32_t capacity,
                                                             FrameCounters* ctr, uint32_t* __restrict__ tile_keys,
                                                             uint32_t* __restrict__ tile_vals,
                                                             uint32_t* __restrict__ digit_hist, uint32_t* ticket,
                                                             uint64_t* status) {
  __shared__ uint32_t h_lo[256], h_hi[256], warp_tot[kThreads / 32];
  __shared__ uint32_t s_blk, s_excl;
  const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
  const uint32_t nd = *n_dev;
  const uint32_t n = nd < n_max ? nd : n_max;
  if (t == 0) s_blk = atomicAdd(ticket, 1u);
  RunHist16 hh{h_lo, h_hi};  // the digits of the 16-bit view-local tile id
  hh.clear();
  __syncthreads();
  const uint32_t blk = s_blk;
  if (blk * kThreads >= n) return;  // past the visible positions (the whole block)
  const uint32_t p = blk * kThreads + t;
  const bool in = p < n;
  uint32_t slot = 0;
  ushort4 r = make_ushort4(1, 1, 0, 0);
  SplatRec rec{};
  if (in) {
    slot = order[p];
    r = rects[slot];
    if (r.x <= r.z && r.y <= r.w) rec = recs[slot];  // culled slots (empty rectangle) need no record
  }
  const uint32_t cnt = count_warp(in, r, rec, tw, th);
  uint32_t base = 0, stride = 0;
  if (cnt) {  // the view's tile-id base and row stride, fetched while the block waits for its offset
    const uint32_t v = block_view[slot >> 8];
    base = v << 16;
    stride = views[v].tiles_x;
  }

  // block-wide exclusive scan of the counts, then the offset of the block from the look-back
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
      if ((blk + 1u) * kThreads >= n) ctr->entries = excl + agg;  // the last block
    }
  }
  __syncthreads();
  const uint32_t e0 = s_excl + wbase + x - cnt;
  bool mine = false;
  if (cnt) {
    if (e0 + cnt > capacity) atomicExch(&ctr->overflow, 1u);
    else mine = true;
  }
  emit_warp<uint32_t>(mine, slot, r, rec, e0, cnt, tw, th, base, stride, tile_keys, tile_vals, hh);
  __syncthreads();
  hh.flush(digit_hist, warp_tot);
}

// shading-list candidates: position g of the padded slots <-> the view's Gaussian order[g - slot_base] (shading
// order); a Gaussian is shaded when the coverage pass marked it (it blends a fragment before its pixels terminate)
__device__ __forceinline__ bool shade_candidate(const BatchView* views, const BatchScene* scenes,
                                                const uint32_t* block_view, const uint8_t* marks, uint32_t g,
                                                uint32_t& view, uint32_t& gslot) {
  const uint32_t v = block_view[g >> 8];
  if (v == kNoView) return false;
  const BatchView& V = views[v];
  const BatchScene& S = scenes[V.scene];
  const uint32_t j = g - V.slot_base;
  if (V.P.view_mode != 3u || !S.lit || j >= V.P.count) return false;
  view = v;
  gslot = V.slot_base + S.order[j];
  return marks[gslot] != 0u;
}

// The shading list of the batch in one pass over the padded slots: each block of 256 slots (one view's) flags the
// Gaussians of its positions in shading order that the coverage pass marked, takes a range of the view's list for
// them with one atomic add on view_shade[view] (zeroed beforehand; it ends as the view's count) and writes their
// global slots there in shading order, adding its count to ctr->shade_n.  Blocks claim their ranges in any order:
// each Gaussian is shaded on its own and the view's radiance bound is a maximum, so the order of the list changes no
// result; within a block the entries keep the shading order, which keeps a warp's Gaussians close together.
__global__ void __launch_bounds__(kThreads) bshade_list_kernel(const BatchView* __restrict__ views,
                                                               const BatchScene* __restrict__ scenes,
                                                               const uint32_t* __restrict__ block_view,
                                                               const uint8_t* __restrict__ marks,
                                                               const uint32_t* __restrict__ totals,
                                                               FrameCounters* ctr, uint32_t* __restrict__ list,
                                                               uint32_t* __restrict__ view_shade) {
  __shared__ uint32_t warp_n[kThreads / 32];
  __shared__ uint32_t s_base;
  const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
  const uint32_t v = block_view[blockIdx.x];
  if (v == kNoView) return;  // padding past the batch (the whole block)
  const uint32_t g = blockIdx.x * kThreads + t;
  uint32_t vv = 0, gslot = 0;
  const bool f = g < totals[0] && shade_candidate(views, scenes, block_view, marks, g, vv, gslot);
  const uint32_t m = __ballot_sync(0xffffffffu, f);
  if (lane == 0) warp_n[w] = __popc(m);
  __syncthreads();
  uint32_t wbase = 0, agg = 0;
#pragma unroll
  for (uint32_t k = 0; k < kThreads / 32; k++) {
    const uint32_t c = warp_n[k];
    wbase += k < w ? c : 0u;
    agg += c;
  }
  if (agg == 0) return;  // the whole block
  if (t == 0) {
    s_base = atomicAdd(&view_shade[v], agg);
    atomicAdd(&ctr->shade_n, agg);
  }
  __syncthreads();
  if (f) list[views[v].slot_base + s_base + wbase + __popc(m & ((1u << lane) - 1u))] = gslot;
}

// After the stable sort on the local tile id the entries run in (local tile, view, depth) order: every (view, tile)
// pair is one contiguous run of its depth-ordered entries.  Its bounds go straight to ranges[tile_base[view] + local]
// (ranges zeroed beforehand: empty tiles keep [0, 0)).
__global__ void __launch_bounds__(kThreads) btile_runs_kernel(const uint32_t* __restrict__ keys,
                                                              const uint32_t* __restrict__ n_dev, uint32_t n_max,
                                                              const BatchViewOut* __restrict__ views,
                                                              uint2* __restrict__ ranges) {
  const uint32_t nd = *n_dev;
  const uint32_t n = nd <= n_max ? nd : 0u;
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const uint32_t k = keys[i];
    const bool first = i == 0 || keys[i - 1] != k, last = i + 1 == n || keys[i + 1] != k;
    if (!first && !last) continue;
    const uint32_t g = views[k >> 16].tile_base + (k & 0xffffu);
    if (first) ranges[g].x = i;
    if (last) ranges[g].y = i + 1;
  }
}

// One block of 256 slots: its valid keys (depth bits not 0xFFFF) and their slots, in slot order, from block_off[blk]
// (a ballot per warp, the warps' counts in shared memory).
__global__ void __launch_bounds__(kThreads) bcompact_kernel(const uint32_t* __restrict__ block_view,
                                                            const uint32_t* __restrict__ keys32,
                                                            const uint32_t* __restrict__ block_off,
                                                            uint32_t* __restrict__ keys_c,
                                                            uint32_t* __restrict__ slots_c) {
  __shared__ uint32_t warp_n[kThreads / 32];
  const uint32_t blk = blockIdx.x;
  if (block_view[blk] == kNoView) return;
  const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
  const uint32_t gslot = blk * kThreads + t;
  const uint32_t key = keys32[gslot];
  const bool valid = (key & 0xFFFFu) != 0xFFFFu;
  const uint32_t m = __ballot_sync(0xffffffffu, valid);
  if (lane == 0) warp_n[w] = __popc(m);
  __syncthreads();
  uint32_t pos = block_off[blk] + __popc(m & ((1u << lane) - 1u));
  for (uint32_t k = 0; k < w; k++) pos += warp_n[k];
  if (valid) {
    keys_c[pos] = key;
    slots_c[pos] = gslot;
  }
}

}  // namespace

cudaError_t launch_bcompact(const uint32_t* block_view, const uint32_t* keys32, const uint32_t* block_off,
                            uint32_t max_blocks, uint32_t* keys_c, uint32_t* slots_c, cudaStream_t s) {
  if (!max_blocks) return cudaSuccess;
  bcompact_kernel<<<max_blocks, kThreads, 0, s>>>(block_view, keys32, block_off, keys_c, slots_c);
  return cudaGetLastError();
}

size_t btile_bin_scratch_bytes(uint32_t n_max) { return 16 + 8ull * ((n_max + kThreads - 1) / kThreads + 1); }

cudaError_t launch_btile_bin(const uint32_t* order, const ushort4* rects, const SplatRec* recs, const BatchView* views,
                             const uint32_t* block_view, const uint32_t* n_dev, uint32_t n_max, uint32_t tw,
                             uint32_t th, uint32_t capacity, FrameCounters* ctr, uint32_t* tile_keys,
                             uint32_t* tile_vals, uint32_t* digit_hist, void* scratch, int variant, cudaStream_t s) {
  if (!n_max) return cudaSuccess;
  const uint32_t blocks = (n_max + kThreads - 1) / kThreads;
  cudaError_t e = cudaMemsetAsync(scratch, 0, btile_bin_scratch_bytes(n_max), s);
  if (e != cudaSuccess) return e;
  uint32_t* ticket = reinterpret_cast<uint32_t*>(scratch);
  uint64_t* status = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(scratch) + 16);
  switch (kTuneMinBlocks[1][variant]) {
    case 4:
      btile_bin_kernel<4><<<blocks, kThreads, 0, s>>>(order, rects, recs, views, block_view, n_dev, n_max, tw, th,
                                                      capacity, ctr, tile_keys, tile_vals, digit_hist, ticket, status);
      break;
    case 5:
      btile_bin_kernel<5><<<blocks, kThreads, 0, s>>>(order, rects, recs, views, block_view, n_dev, n_max, tw, th,
                                                      capacity, ctr, tile_keys, tile_vals, digit_hist, ticket, status);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_bshade_list(const BatchView* views, const BatchScene* scenes, const uint32_t* block_view,
                               const uint8_t* marks, const uint32_t* totals, uint32_t max_blocks, uint32_t n_views,
                               FrameCounters* ctr, uint32_t* list, uint32_t* view_shade, cudaStream_t s) {
  if (!max_blocks) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(view_shade, 0, 4ull * n_views, s);
  if (e != cudaSuccess) return e;
  bshade_list_kernel<<<max_blocks, kThreads, 0, s>>>(views, scenes, block_view, marks, totals, ctr, list, view_shade);
  return cudaGetLastError();
}

cudaError_t launch_btile_runs(const uint32_t* keys, const uint32_t* n_dev, uint32_t n_max, const BatchViewOut* views,
                              uint2* ranges, cudaStream_t s) {
  if (!n_max) return cudaSuccess;
  uint32_t blocks = (n_max + kThreads * 8 - 1) / (kThreads * 8);
  if (blocks > 152 * 8) blocks = 152 * 8;
  btile_runs_kernel<<<blocks, kThreads, 0, s>>>(keys, n_dev, n_max, views, ranges);
  return cudaGetLastError();
}

}  // namespace sl
