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

// Decoupled look-back over per-block status words (u64: flag << 32 | count; flag 1 the block's own count, 2 the
// count of every block up to it), for blocks that take their positions from a ticket counter, so every earlier block
// is already running and each wait ends (bounded all the same: past the limit the frame's timeout flag is set).
constexpr uint64_t kLookAgg = 1ull << 32;
constexpr uint64_t kLookPrefix = 2ull << 32;
constexpr uint32_t kLookSpinLimit = 1u << 22;

__device__ __forceinline__ uint64_t load_relaxed64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Publishes a status word (flag and count in one aligned 64-bit word: a relaxed store suffices, and unlike an atomic
// exchange it does not hold the thread for a round trip).
__device__ __forceinline__ void store_relaxed64(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Called by one whole warp for block blk with its count agg (blocks before `first` count as a prefix of 0): publishes
// agg, reads 32 earlier blocks' words per step (the nearest in lane 0) until a prefix, publishes this block's prefix
// and returns the count of the blocks in [first, blk) in every lane.
__device__ __forceinline__ uint32_t lookback_warp(uint64_t* status, uint32_t blk, uint32_t first, uint32_t agg,
                                                  uint32_t* timeout_flag) {
  const uint32_t lane = threadIdx.x & 31u;
  const bool head = blk == first;
  if (lane == 0) store_relaxed64(status + blk, (head ? kLookPrefix : kLookAgg) | agg);
  uint32_t excl = 0;
  const int32_t lo = (int32_t)first;
  int32_t top = (int32_t)blk - 1;
  uint32_t spins = 0;
  while (top >= lo) {
    const int32_t j = top - (int32_t)lane;
    const uint64_t st = j >= lo ? load_relaxed64(status + j) : kLookPrefix;  // before the first block: a prefix of 0
    const uint32_t flag = (uint32_t)(st >> 32);
    const uint32_t pm = __ballot_sync(0xffffffffu, flag == 2u), zm = __ballot_sync(0xffffffffu, flag == 0u);
    const uint32_t pfirst = pm ? (uint32_t)__ffs(pm) - 1u : 32u, zfirst = zm ? (uint32_t)__ffs(zm) - 1u : 32u;
    if (zfirst < pfirst) {  // a nearer block has not published yet: read the window again
      if (++spins > kLookSpinLimit) {
        if (lane == 0) atomicExch(timeout_flag, 1u);
        break;
      }
      __nanosleep(32);
      continue;
    }
    excl += __reduce_add_sync(0xffffffffu, lane <= pfirst ? (uint32_t)st : 0u);
    if (pm) break;
    top -= 32;
  }
  if (lane == 0 && !head) store_relaxed64(status + blk, kLookPrefix | (excl + agg));
  return excl;
}

// Digit counts of the low 16 bits of the emitted tile keys, for the two passes of the tile sort that follows, in a
// block's shared memory.  A row of the emission is n consecutive ids: its high-byte digits are one or two runs (an
// add per run), its low-byte digits n consecutive bins mod 256, kept as a difference array (a step up at the first
// bin, a step down after the last; n / 256 whole cycles raise every bin) so a row costs a few shared atomics rather
// than one per entry.  flush() turns the differences into counts (a block prefix sum) and adds both histograms to
// digit_hist[0..511].
struct RunHist16 {
  uint32_t* lo_diff;  // [256]
  uint32_t* hi;       // [256]
  __device__ __forceinline__ void clear() {
    lo_diff[threadIdx.x] = 0u;
    hi[threadIdx.x] = 0u;
  }
  __device__ __forceinline__ void add(uint32_t first, uint32_t n) {
    const uint32_t a = first & 0xffu, full = n >> 8, rem = n & 0xffu;
    if (full) atomicAdd(&lo_diff[0], full);
    if (rem) {
      atomicAdd(&lo_diff[a], 1u);
      const uint32_t end = a + rem;  // one past the last bin, unwrapped
      if (end > 256u) {
        atomicAdd(&lo_diff[0], 1u);
        atomicAdd(&lo_diff[end - 256u], 0xffffffffu);
      } else if (end < 256u) {
        atomicAdd(&lo_diff[end], 0xffffffffu);
      }
    }
    for (uint32_t x = first, stop_all = first + n; x < stop_all;) {
      const uint32_t stop = min(stop_all, (x | 0xffu) + 1u);
      atomicAdd(&hi[(x >> 8) & 0xffu], stop - x);
      x = stop;
    }
  }
  // after a __syncthreads that follows the block's last add; 256 threads; warp_tot: 8 words of shared scratch
  __device__ __forceinline__ void flush(uint32_t* digit_hist, uint32_t* warp_tot) {
    const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
    uint32_t x = lo_diff[t];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31u) warp_tot[w] = x;
    __syncthreads();
    for (uint32_t k = 0; k < w; k++) x += warp_tot[k];
    if (x) atomicAdd(&digit_hist[t], x);
    if (hi[t]) atomicAdd(&digit_hist[256 + t], hi[t]);
  }
};

// Writes one row of entries.
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

// The per-splat span preparation of lane src, for the whole warp.
__device__ __forceinline__ sl_span_prep shfl_prep(const sl_span_prep& p, int src) {
  sl_span_prep q;
  q.cx = __shfl_sync(0xffffffffu, p.cx, src);
  q.cy = __shfl_sync(0xffffffffu, p.cy, src);
  q.a = __shfl_sync(0xffffffffu, p.a, src);
  q.b = __shfl_sync(0xffffffffu, p.b, src);
  q.D = __shfl_sync(0xffffffffu, p.D, src);
  q.Q = __shfl_sync(0xffffffffu, p.Q, src);
  q.half_w = __shfl_sync(0xffffffffu, p.half_w, src);
  q.ylim = __shfl_sync(0xffffffffu, p.ylim, src);
  q.ys = __shfl_sync(0xffffffffu, p.ys, src);
  q.m = __shfl_sync(0xffffffffu, p.m, src);
  q.full = __shfl_sync(0xffffffffu, p.full, src);
  return q;
}

__device__ __forceinline__ sl_span_prep span_prep(const SplatRec& rec) {
  sl_span_prep p;
  sl_span_init(rec.a.x, rec.a.y, rec.a.z, rec.a.w, rec.b.x, rec.b.y, rec.b.w, &p);
  return p;
}

// One warp's 32 splats (lane = one sorted position; `mine` false for lanes without one).  Tile id of (tx, ty) in this
// lane's view = base + ty * stride + tx.  Tile widths are powers of two (tile_shift = log2 tw).
template <typename KeyT, typename Hist>
__device__ __forceinline__ void emit_warp(bool mine, uint32_t slot, ushort4 r, const SplatRec& rec, uint32_t e0,
                                          uint32_t cnt, uint32_t tw, uint32_t th, uint32_t base, uint32_t stride,
                                          KeyT* __restrict__ tile_keys, uint32_t* __restrict__ tile_vals, Hist& h) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t tsh = sl_tile_shift(tw);
  const bool small = mine && cnt <= kSmallTiles;
  sl_span_prep sp{};
  if (mine) sp = span_prep(rec);
  if (small) {
    uint32_t e = e0;
    for (uint32_t ty = r.y; ty <= r.w; ty++) {
      uint32_t t0, t1;
      if (!sl_span_row(&sp, r.x, r.z, ty, tw, tsh, th, &t0, &t1)) continue;
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
    const sl_span_prep q = shfl_prep(sp, src);
    uint32_t e_base = __shfl_sync(0xffffffffu, e0, src);
    const uint32_t rx = s_xy & 0xffffu, ry = s_xy >> 16, rz = s_zw & 0xffffu, rw = s_zw >> 16;
    const uint32_t s_base = __shfl_sync(0xffffffffu, base, src), s_stride = __shfl_sync(0xffffffffu, stride, src);
    for (uint32_t ty0 = ry; ty0 <= rw; ty0 += 32u) {
      const uint32_t ty = ty0 + lane;
      uint32_t t0 = 0, t1 = 0, len = 0;
      if (ty <= rw && sl_span_row(&q, rx, rz, ty, tw, tsh, th, &t0, &t1)) len = t1 - t0 + 1u;
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
  const uint32_t tsh = sl_tile_shift(tw);
  const bool valid = mine && r.x <= r.z && r.y <= r.w;
  const bool small = valid && (uint32_t)(r.z - r.x + 1) * (uint32_t)(r.w - r.y + 1) <= kSmallTiles;
  sl_span_prep sp{};
  if (valid) sp = span_prep(rec);
  uint32_t n = 0;
  if (small)
    for (uint32_t ty = r.y; ty <= r.w; ty++) {
      uint32_t t0, t1;
      if (sl_span_row(&sp, r.x, r.z, ty, tw, tsh, th, &t0, &t1)) n += t1 - t0 + 1u;
    }
  uint32_t big = __ballot_sync(0xffffffffu, valid && !small);
  while (big) {
    const int src = __ffs(big) - 1;
    big &= big - 1u;
    const uint32_t s_xy = __shfl_sync(0xffffffffu, (uint32_t)r.x | ((uint32_t)r.y << 16), src);
    const uint32_t s_zw = __shfl_sync(0xffffffffu, (uint32_t)r.z | ((uint32_t)r.w << 16), src);
    const sl_span_prep q = shfl_prep(sp, src);
    const uint32_t rx = s_xy & 0xffffu, ry = s_xy >> 16, rz = s_zw & 0xffffu, rw = s_zw >> 16;
    uint32_t sum = 0;
    for (uint32_t ty = ry + lane; ty <= rw; ty += 32u) {
      uint32_t t0, t1;
      if (sl_span_row(&q, rx, rz, ty, tw, tsh, th, &t0, &t1)) sum += t1 - t0 + 1u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == (uint32_t)src) n = sum;
  }
  return n;
}

}  // namespace sl
