// Tile-entry emission shared by the per-view and the batched binning: every visible splat, at its sorted position p,
// writes one (tile id, slot) entry per tile of its row spans, starting at offsets[p].  Small splats (<= kSmallTiles
// tiles) are written by their own thread; the few large ones, which would leave the rest of a warp waiting, are
// written by the whole warp together, one row of tiles per lane (the rows' entry ranges from a warp prefix sum).
// The per-row spans come from the same function and record values as the counts, so both agree entry for entry.
#pragma once

#include "sl_internal.h"
#include "sl_tilespan.h"

namespace sl {

constexpr uint32_t kSmallTiles = 48;

// Digit counting for the tile sort that follows: Hist::add(tile, n) for n consecutive ids starting at tile.
template <typename KeyT, typename Hist>
__device__ __forceinline__ void emit_row(uint32_t row_base, uint32_t t0, uint32_t t1, uint32_t slot, uint32_t e,
                                         KeyT* __restrict__ tile_keys, uint32_t* __restrict__ tile_vals, Hist& h) {
  for (uint32_t tx = t0; tx <= t1; tx++) {
    tile_keys[e] = (KeyT)(row_base + tx);
    tile_vals[e] = slot;
    e++;
  }
  h.add(row_base + t0, t1 - t0 + 1u);
}

// One warp's 32 splats (lane = one sorted position; `mine` false for lanes without one).  Tile id of (tx, ty) in this
// lane's view = base + ty * stride + tx.
template <typename KeyT, typename Hist>
__device__ __forceinline__ void emit_warp(bool mine, uint32_t slot, ushort4 r, const SplatRec& rec, uint32_t e0,
                                          uint32_t cnt, uint32_t tw, uint32_t th, uint32_t base, uint32_t stride,
                                          KeyT* __restrict__ tile_keys, uint32_t* __restrict__ tile_vals, Hist& h) {
  const uint32_t lane = threadIdx.x & 31u;
  const bool small = mine && cnt <= kSmallTiles;
  if (small) {
    uint32_t e = e0;
    for (uint32_t ty = r.y; ty <= r.w; ty++) {
      uint32_t t0, t1;
      if (!sl_row_tiles(rec.a.x, rec.a.y, rec.a.z, rec.a.w, rec.b.x, rec.b.y, rec.b.w, r.x, r.z, ty, tw, th, &t0, &t1))
        continue;
      emit_row(base + ty * stride, t0, t1, slot, e, tile_keys, tile_vals, h);
      e += t1 - t0 + 1u;
    }
  }
  uint32_t big = __ballot_sync(0xffffffffu, mine && !small);
  while (big) {
    const int src = __ffs(big) - 1;
    big &= big - 1u;
    // the splat of lane src, for the whole warp
    const uint32_t s_slot = __shfl_sync(0xffffffffu, slot, src);
    const uint32_t s_xy = __shfl_sync(0xffffffffu, (uint32_t)r.x | ((uint32_t)r.y << 16), src);
    const uint32_t s_zw = __shfl_sync(0xffffffffu, (uint32_t)r.z | ((uint32_t)r.w << 16), src);
    const float ax = __shfl_sync(0xffffffffu, rec.a.x, src), ay = __shfl_sync(0xffffffffu, rec.a.y, src);
    const float az = __shfl_sync(0xffffffffu, rec.a.z, src), aw = __shfl_sync(0xffffffffu, rec.a.w, src);
    const float bx = __shfl_sync(0xffffffffu, rec.b.x, src), by = __shfl_sync(0xffffffffu, rec.b.y, src);
    const float bw = __shfl_sync(0xffffffffu, rec.b.w, src);
    uint32_t e_base = __shfl_sync(0xffffffffu, e0, src);
    const uint32_t rx = s_xy & 0xffffu, ry = s_xy >> 16, rz = s_zw & 0xffffu, rw = s_zw >> 16;
    const uint32_t s_base = __shfl_sync(0xffffffffu, base, src), s_stride = __shfl_sync(0xffffffffu, stride, src);
    for (uint32_t ty0 = ry; ty0 <= rw; ty0 += 32u) {
      const uint32_t ty = ty0 + lane;
      uint32_t t0 = 0, t1 = 0, len = 0;
      if (ty <= rw && sl_row_tiles(ax, ay, az, aw, bx, by, bw, rx, rz, ty, tw, th, &t0, &t1)) len = t1 - t0 + 1u;
      uint32_t incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
      }
      if (len) emit_row(s_base + ty * s_stride, t0, t1, s_slot, e_base + incl - len, tile_keys, tile_vals, h);
      e_base += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
}

// The tile count of this lane's splat (0 when !mine), the same per-row spans summed; splats whose candidate rectangle
// has more than kSmallTiles tiles are counted by the whole warp, a row per lane.
__device__ __forceinline__ uint32_t count_warp(bool mine, ushort4 r, const SplatRec& rec, uint32_t tw, uint32_t th) {
  const uint32_t lane = threadIdx.x & 31u;
  const bool valid = mine && r.x <= r.z && r.y <= r.w;
  const bool small = valid && (uint32_t)(r.z - r.x + 1) * (uint32_t)(r.w - r.y + 1) <= kSmallTiles;
  uint32_t n = 0;
  if (small)
    for (uint32_t ty = r.y; ty <= r.w; ty++) {
      uint32_t t0, t1;
      if (sl_row_tiles(rec.a.x, rec.a.y, rec.a.z, rec.a.w, rec.b.x, rec.b.y, rec.b.w, r.x, r.z, ty, tw, th, &t0, &t1))
        n += t1 - t0 + 1u;
    }
  uint32_t big = __ballot_sync(0xffffffffu, valid && !small);
  while (big) {
    const int src = __ffs(big) - 1;
    big &= big - 1u;
    const uint32_t s_xy = __shfl_sync(0xffffffffu, (uint32_t)r.x | ((uint32_t)r.y << 16), src);
    const uint32_t s_zw = __shfl_sync(0xffffffffu, (uint32_t)r.z | ((uint32_t)r.w << 16), src);
    const float ax = __shfl_sync(0xffffffffu, rec.a.x, src), ay = __shfl_sync(0xffffffffu, rec.a.y, src);
    const float az = __shfl_sync(0xffffffffu, rec.a.z, src), aw = __shfl_sync(0xffffffffu, rec.a.w, src);
    const float bx = __shfl_sync(0xffffffffu, rec.b.x, src), by = __shfl_sync(0xffffffffu, rec.b.y, src);
    const float bw = __shfl_sync(0xffffffffu, rec.b.w, src);
    const uint32_t rx = s_xy & 0xffffu, ry = s_xy >> 16, rz = s_zw & 0xffffu, rw = s_zw >> 16;
    uint32_t sum = 0;
    for (uint32_t ty = ry + lane; ty <= rw; ty += 32u) {
      uint32_t t0, t1;
      if (sl_row_tiles(ax, ay, az, aw, bx, by, bw, rx, rz, ty, tw, th, &t0, &t1)) sum += t1 - t0 + 1u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == (uint32_t)src) n = sum;
  }
  return n;
}

}  // namespace sl
