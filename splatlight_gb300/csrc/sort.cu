// Stable LSD radix sort of 16- or 32-bit keys with 32-bit values, onesweep style (one read and one write of the keys and
// values per 8-bit digit pass, Adinets & Merrill 2022): the digit histograms of every pass are counted up front (by
// the producer kernel, or launch_digit_hist16), then each pass is a single kernel over tiles of kTile keys that
//   1. ranks its keys per warp in index order (stability): the lanes holding the same digit find each other through
//      a per-warp mask word per digit that each lane ORs its bit into (a shared-memory atomic), and a per-warp digit
//      counter carries the count from one item to the next -- a handful of instructions per key instead of one ballot
//      per digit bit;
//   2. publishes its per-digit counts and looks back over earlier tiles for the exclusive prefix (decoupled
//      look-back, one thread per digit): kLookWindow predecessors' words per round trip, because with hundreds of
//      tiles in flight a tile's walk back to the nearest published prefix is long; every spin is bounded and a give-up
//      sets FrameCounters::timeout;
//   3. reorders the tile in shared memory by digit (values read straight into place) and writes it out in digit runs
//      (coalesced), each key's destination one shared load (the digit's global start less its start within the
//      tile) plus its position.
// Tiles are taken in launch order from an atomic counter, so a tile only waits on tiles that already started.  (A
// wait-free variant -- a counting kernel, a scan of the per-tile counts, then this rank-and-scatter -- was measured:
// its scatter ran 25% faster than this whole pass, but the extra counting pass over the keys cost more than that.)
// Replaces the three-dispatch-per-pass radix sort of shaders/radix.wgsl:1-139 (the same order: by key, ties in index
// order); INVALID keys (0xFFFF) sort after every valid key, as there.
#include "sl_internal.h"

namespace sl {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
// Keys per thread: 16 (tiles of 4096, four blocks per SM) for 16-bit keys, 24 (tiles of 6144, three blocks per SM) for
// 32-bit keys -- the faster of the sizes measured for each (12, 16 and 24 keys per thread).  Scratch is sized for the
// smaller tile (the most tiles).
template <typename KeyT> struct SortCfg;
template <> struct SortCfg<uint16_t> {
  static constexpr int kItems = 16, kMinBlocks = 4;
};
template <> struct SortCfg<uint32_t> {
  static constexpr int kItems = 24, kMinBlocks = 3;
};
static_assert(kThreads * SortCfg<uint16_t>::kItems == kSortTileKeys, "sort tile size and the scratch layouts disagree");
static_assert(SortCfg<uint32_t>::kItems >= SortCfg<uint16_t>::kItems, "scratch is sized for the smaller tile");
// Predecessors' words read per look-back round trip (4 measured faster than 16: the walks are short enough).
constexpr int kLookWindow = 4;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t load_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Publishes a look-back word (value and flag in one aligned 32-bit word, so a plain relaxed store is enough and
// the thread does not wait for a round trip as it would for an atomic exchange).
__device__ __forceinline__ void store_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Exclusive scan of one value per thread over a 256-thread block; returns the exclusive prefix.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  uint32_t base = 0;
#pragma unroll
  for (int k = 0; k < kWarps; k++) base += (k < w) ? warp_tot[k] : 0u;
  __syncthreads();
  return base + x - v;
}

template <typename KeyT, uint32_t kTile>
struct PassSmem {
  uint32_t tile;
  uint32_t warp_tot[kWarps];
  uint32_t cnt[kWarps][256];      // per warp and digit: running count while ranking, then the warp's start
  uint32_t match[2][kWarps][256]; // per warp and digit: the lanes holding it in the current item (two, alternating)
  uint32_t local_start[256];      // the digit's first position in the reordered tile
  uint32_t gofs[256];             // the digit's global start less local_start
  KeyT keys[kTile];
  uint32_t vals[kTile];
};

template <typename KeyT>
__global__ void __launch_bounds__(kThreads, SortCfg<KeyT>::kMinBlocks) onesweep_pass(const KeyT* __restrict__ keys_in,
                                                          const uint32_t* __restrict__ vals_in,
                                                          KeyT* __restrict__ keys_out,
                                                          uint32_t* __restrict__ vals_out, uint32_t n_max,
                                                          const uint32_t* __restrict__ n_dev, int shift,
                                                          const uint32_t* __restrict__ digit_hist,
                                                          uint32_t* status, uint32_t* tile_ctr, FrameCounters* ctr) {
  constexpr int kItems = SortCfg<KeyT>::kItems;
  constexpr uint32_t kTile = kThreads * kItems;
  __shared__ PassSmem<KeyT, kTile> sm;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  // element count: a host bound, or the smaller device-side count (tile entries, known only on the device)
  // (a device count above the bound means the producer overflowed its buffer: sort nothing, the host re-runs)
  uint32_t n = n_max;
  if (n_dev) {
    const uint32_t nd = *n_dev;
    n = nd <= n_max ? nd : 0u;
  }
  if (t == 0) sm.tile = atomicAdd(tile_ctr, 1u);
  const uint32_t hist_t = digit_hist[t];  // this digit's pass count, read early (its latency overlaps the ranking)
#pragma unroll
  for (int k = 0; k < kWarps; k++) {
    sm.cnt[k][t] = 0u;
    sm.match[0][k][t] = 0u;
    sm.match[1][k][t] = 0u;
  }
  __syncthreads();
  const uint32_t tile = sm.tile;
  const uint32_t tile_base = tile * kTile;
  if (tile_base >= n) return;  // the grid covers n_max; tiles past n have nothing to do (no later tile waits on them)

  // warp w holds [tile_base + w 32 kItems, + 32 kItems), item it of lane l at + 32 it + l (coalesced loads)
  const uint32_t wbase = tile_base + (uint32_t)w * (32u * kItems) + (uint32_t)lane;
  const bool full = tile_base + kTile <= n;
  uint32_t keys[kItems];
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    const uint32_t idx = wbase + (uint32_t)it * 32u;
    keys[it] = (full || idx < n) ? (uint32_t)keys_in[idx] : 0u;
  }

  // ranks in index order: item by item, the lanes sharing a digit OR their bits into match[it & 1][w][d]; each lane's
  // rank is the warp's count of that digit so far plus its peers below it.  After every peer has read the mask and
  // the count (a warp barrier), the lowest peer advances the count and clears the mask word, which is ORed into
  // again only two items later, after two more warp barriers.
  const uint32_t lt = lanemask_lt();
  uint32_t ranks[kItems];
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    const uint32_t idx = wbase + (uint32_t)it * 32u;
    const bool valid = full || idx < n;
    const uint32_t d = (keys[it] >> shift) & 0xffu;
    uint32_t* mw = &sm.match[it & 1][w][d];
    if (valid) atomicOr(mw, 1u << lane);
    __syncwarp();
    const uint32_t peers = valid ? *mw : 0u;
    const uint32_t before = valid ? sm.cnt[w][d] : 0u;
    __syncwarp();
    const uint32_t below = peers & lt;
    if (valid && below == 0u) {
      sm.cnt[w][d] = before + __popc(peers);
      *mw = 0u;
    }
    ranks[it] = before + __popc(below);
  }
  __syncthreads();

  // per digit t: the warps' exclusive starts within the tile, and the tile's count
  uint32_t run = 0;
#pragma unroll
  for (int k = 0; k < kWarps; k++) {
    const uint32_t c = sm.cnt[k][t];
    sm.cnt[k][t] = run;
    run += c;
  }
  const uint32_t tile_count = run;

  // publish this tile's counts, then look back for the exclusive prefix of digit t: kLookWindow predecessors' words
  // per round trip, taken in order -- an aggregate adds and the walk goes on, a prefix adds and ends it, a word not
  // yet published is read again (after a short sleep; bounded)
  uint32_t* st = status + (size_t)tile * 256u;
  store_relaxed(&st[t], (tile == 0 ? kFlagPrefix : kFlagAgg) | tile_count);
  uint32_t excl = 0;
  if (tile > 0) {
    int32_t j = (int32_t)tile - 1;
    uint32_t spins = 0;
    bool done = false;
    while (!done) {
      uint32_t sv[kLookWindow];
#pragma unroll
      for (int k = 0; k < kLookWindow; k++)
        sv[k] = j - k >= 0 ? load_relaxed(status + (size_t)(j - k) * 256u + t) : 0u;
      bool stalled = false;
#pragma unroll
      for (int k = 0; k < kLookWindow; k++) {
        if (done || stalled) continue;
        const uint32_t flag = sv[k] & ~kValueMask;
        if (flag == 0u) {
          stalled = true;  // not yet published: read again from here
          continue;
        }
        excl += sv[k] & kValueMask;
        j--;
        if (flag == kFlagPrefix) done = true;
      }
      if (done) break;
      if (stalled) {
        if (++spins > kSpinLimit) {
          atomicExch(&ctr->timeout, 1u);
          break;
        }
        __nanosleep(32);
      }
      // j < 0 cannot happen: tile 0 publishes a prefix at once, so the walk ends there at the latest
    }
    store_relaxed(&st[t], kFlagPrefix | ((excl + tile_count) & kValueMask));
  }

  // global start of digit t: exclusive scan of the pass histogram, plus earlier tiles; its start within the tile
  const uint32_t gstart = block_exclusive_scan(hist_t, sm.warp_tot);
  const uint32_t lstart = block_exclusive_scan(tile_count, sm.warp_tot);
  sm.local_start[t] = lstart;
  sm.gofs[t] = gstart + excl - lstart;
  __syncthreads();

  // reorder the tile by digit in shared memory; values are read here, straight from global memory
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    const uint32_t idx = wbase + (uint32_t)it * 32u;
    if (full || idx < n) {
      const uint32_t d = (keys[it] >> shift) & 0xffu;
      const uint32_t pos = sm.local_start[d] + sm.cnt[w][d] + ranks[it];
      sm.keys[pos] = (KeyT)keys[it];
      sm.vals[pos] = vals_in ? vals_in[idx] : idx;
    }
  }
  __syncthreads();

  const uint32_t tile_n = (n - tile_base) < kTile ? (n - tile_base) : kTile;
#pragma unroll 4
  for (uint32_t j = t; j < tile_n; j += kThreads) {
    const uint32_t key = sm.keys[j];
    const uint32_t dst = sm.gofs[(key >> shift) & 0xffu] + j;
    if (dst >= n) continue;  // only after a look-back timeout (reported); never write out of range
    if (keys_out) keys_out[dst] = (KeyT)key;
    vals_out[dst] = sm.vals[j];
  }
}

__global__ void __launch_bounds__(kThreads) digit_hist16_kernel(const uint16_t* __restrict__ keys, uint32_t n,
                                                                int passes, uint32_t* hist) {
  __shared__ uint32_t h[2][256];
  const int t = threadIdx.x;
  h[0][t] = 0u;
  h[1][t] = 0u;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + t; i < n; i += gridDim.x * kThreads) {
    uint32_t k = keys[i];
    atomicAdd(&h[0][k & 0xffu], 1u);
    if (passes > 1) atomicAdd(&h[1][k >> 8], 1u);
  }
  __syncthreads();
  if (h[0][t]) atomicAdd(&hist[t], h[0][t]);
  if (passes > 1 && h[1][t]) atomicAdd(&hist[256 + t], h[1][t]);
}

__global__ void __launch_bounds__(kThreads) digit_hist32_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                                int passes, uint32_t* hist) {
  __shared__ uint32_t h[4][256];
  const int t = threadIdx.x;
  for (int p = 0; p < 4; p++) h[p][t] = 0u;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + t; i < n; i += gridDim.x * kThreads) {
    const uint32_t k = keys[i];
    for (int p = 0; p < passes; p++) atomicAdd(&h[p][(k >> (8 * p)) & 0xffu], 1u);
  }
  __syncthreads();
  for (int p = 0; p < passes; p++)
    if (h[p][t]) atomicAdd(&hist[256 * p + t], h[p][t]);
}

}  // namespace

size_t sort_tiles_for(uint32_t n) { return sort_tiles_const(n); }

cudaError_t launch_digit_hist32(const uint32_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  uint32_t blocks = (n + kThreads * 16 - 1) / (kThreads * 16);
  if (blocks > 1216) blocks = 1216;
  digit_hist32_kernel<<<blocks, kThreads, 0, s>>>(keys, n, passes, hist);
  return cudaGetLastError();
}

cudaError_t launch_digit_hist16(const uint16_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  uint32_t blocks = (n + kThreads * 16 - 1) / (kThreads * 16);
  if (blocks > 1216) blocks = 1216;  // 8 per SM on 152 SMs
  digit_hist16_kernel<<<blocks, kThreads, 0, s>>>(keys, n, passes, hist);
  return cudaGetLastError();
}

namespace {

// LSD passes over the low `bits` key bits, 8 per pass.  Keys ping-pong between `keys` (clobbered) and keys_alt;
// values land in vals_out after the last pass (through vals_alt when that is needed to avoid reading and writing one
// buffer in the same pass); keys_out, if given, receives the sorted keys.
template <typename KeyT>
cudaError_t sort_pairs(KeyT* keys, KeyT* keys_alt, const uint32_t* vals_in, uint32_t* vals_out, uint32_t* vals_alt,
                       uint32_t n, const uint32_t* n_dev, int bits, const uint32_t* digit_hist, uint32_t* status,
                       uint32_t* tile_ctr, uint32_t max_tiles, FrameCounters* ctr, cudaStream_t s, KeyT* keys_out,
                       const KeyT* keys_first = nullptr) {
  if (n == 0) return cudaSuccess;
  if (n > kValueMask) return cudaErrorInvalidValue;
  constexpr uint32_t kTile = kThreads * SortCfg<KeyT>::kItems;
  const uint32_t tiles = (n + kTile - 1) / kTile;
  if (tiles > max_tiles) return cudaErrorInvalidValue;
  const int passes = bits <= 8 ? 1 : (bits + 7) / 8;
  if (passes > 4) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(uint32_t) * 256u * tiles * (size_t)passes, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(tile_ctr, 0, sizeof(uint32_t) * 4, s);
  if (e != cudaSuccess) return e;
  // value buffers per pass: the last pass writes vals_out; earlier ones alternate so no pass reads what it writes
  uint32_t* vdst[4];
  for (int p = 0; p < passes; p++) vdst[p] = ((passes - 1 - p) % 2 == 0) ? vals_out : vals_alt;
  bool copy_back = false;
  if (vals_in && vals_in == vdst[0]) {  // the first pass would overwrite its own input: shift by one buffer
    for (int p = 0; p < passes; p++) vdst[p] = (vdst[p] == vals_out) ? vals_alt : vals_out;
    copy_back = true;  // the result then sits in vals_alt
  }
  const KeyT* kin = keys_first ? keys_first : keys;  // keys_first: read by the first pass only (left intact)
  const uint32_t* vin = vals_in;
  for (int p = 0; p < passes; p++) {
    const bool last = p == passes - 1;
    KeyT* kdst = last ? keys_out : ((p % 2 == 0) ? keys_alt : keys);
    if (last && keys_out && keys_out == kin) kdst = (kin == keys) ? keys_alt : keys;  // never write what is read
    onesweep_pass<KeyT><<<tiles, kThreads, 0, s>>>(kin, vin, kdst, vdst[p], n, n_dev, 8 * p, digit_hist + 256 * p,
                                                   status + (size_t)256u * tiles * p, tile_ctr + p, ctr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (last && keys_out && kdst != keys_out)
      if ((e = cudaMemcpyAsync(keys_out, kdst, sizeof(KeyT) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    kin = kdst ? kdst : kin;
    vin = vdst[p];
  }
  if (copy_back) e = cudaMemcpyAsync(vals_out, vals_alt, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
  return e;
}

}  // namespace

cudaError_t sort16_pairs(uint16_t* keys, const uint32_t* vals_in, uint32_t* vals_out, uint32_t n,
                         const uint32_t* n_dev, int bits, const uint32_t* digit_hist, SortScratch& sc,
                         FrameCounters* ctr, cudaStream_t s, uint16_t* keys_out) {
  return sort_pairs<uint16_t>(keys, sc.keys_alt, vals_in, vals_out, sc.vals_alt, n, n_dev, bits, digit_hist,
                              sc.status, sc.tile_ctr, sc.max_tiles, ctr, s, keys_out);
}

cudaError_t sort32_pairs(uint32_t* keys, uint32_t* keys_alt, const uint32_t* vals_in, uint32_t* vals_out,
                         uint32_t* vals_alt, uint32_t n, const uint32_t* n_dev, int bits, const uint32_t* digit_hist,
                         uint32_t* status, uint32_t* tile_ctr, uint32_t max_tiles, FrameCounters* ctr, cudaStream_t s,
                         uint32_t* keys_out, const uint32_t* keys_first) {
  return sort_pairs<uint32_t>(keys, keys_alt, vals_in, vals_out, vals_alt, n, n_dev, bits, digit_hist, status,
                              tile_ctr, max_tiles, ctr, s, keys_out, keys_first);
}

}  // namespace sl
