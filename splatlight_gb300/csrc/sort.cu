// Stable LSD radix sort of 16- or 32-bit keys with 32-bit values, onesweep style (one read and one write of the keys and
// values per 8-bit digit pass, Adinets & Merrill 2022): the digit histograms of every pass are counted up front (by
// the producer kernel, or launch_digit_hist16), then each pass is a single kernel over tiles of 6144 keys that
//   1. ranks its keys per warp -- the peers holding the same digit found by one ballot per digit bit, a per-warp
//      digit counter in shared memory -- so ranks follow index order within the tile (stability);
//   2. publishes its per-digit counts and looks back over earlier tiles (decoupled look-back, one thread per digit)
//      for the exclusive prefix; every spin is bounded and a give-up sets FrameCounters::timeout;
//   3. reorders the tile in shared memory by digit and writes it out in digit runs (coalesced).
// Tiles are taken in launch order from an atomic counter, so a tile only waits on tiles that already started.
// Replaces the three-dispatch-per-pass radix sort of shaders/radix.wgsl:1-139 (same stable order: by key, ties in
// index order); INVALID keys (0xFFFF) sort after every valid key, as there.
#include "sl_internal.h"

namespace sl {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 24;
constexpr uint32_t kTile = kThreads * kItems;  // 6144
static_assert(kTile == kSortTileKeys, "sort tile size and the scratch layouts disagree");
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

// Exclusive scan of one value per thread over a 256-thread block; returns the exclusive prefix, *total = sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  uint32_t base = 0, sum = 0;
#pragma unroll
  for (int k = 0; k < kWarps; k++) {
    uint32_t t = warp_tot[k];
    base += (k < w) ? t : 0u;
    sum += t;
  }
  __syncthreads();
  if (total) *total = sum;
  return base + x - v;
}

// Lanes of `mask` whose 8-bit digit equals this lane's: the intersection over the digit's bits of the ballot of
// lanes sharing that bit (eight ballots; measured faster than the match instruction in this kernel).
__device__ __forceinline__ uint32_t digit_peers(uint32_t mask, uint32_t d) {
  uint32_t peers = mask;
#pragma unroll
  for (int b = 0; b < 8; b++) {
    const uint32_t m = __ballot_sync(mask, (d >> b) & 1u);
    peers &= ((d >> b) & 1u) ? m : ~m;
  }
  return peers;
}

// Tiles of 6144 keys at three blocks per SM (the best of the tile sizes and register budgets measured).
template <typename KeyT>
__global__ void __launch_bounds__(kThreads, 3) onesweep_pass(const KeyT* __restrict__ keys_in,
                                                          const uint32_t* __restrict__ vals_in,
                                                          KeyT* __restrict__ keys_out,
                                                          uint32_t* __restrict__ vals_out, uint32_t n_max,
                                                          const uint32_t* __restrict__ n_dev, int shift,
                                                          const uint32_t* __restrict__ digit_hist,
                                                          uint32_t* status, uint32_t* tile_ctr, FrameCounters* ctr) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t warp_hist[kWarps][256];
  __shared__ uint32_t digit_base[256];
  __shared__ uint32_t local_start[256];
  __shared__ uint32_t warp_tot[kWarps];
  __shared__ KeyT s_keys[kTile];
  __shared__ uint32_t s_vals[kTile];

  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  // element count: a host bound, or the smaller device-side count (tile entries, known only on the device)
  // (a device count above the bound means the producer overflowed its buffer: sort nothing, the host re-runs)
  uint32_t n = n_max;
  if (n_dev) {
    uint32_t nd = *n_dev;
    n = nd <= n_max ? nd : 0u;
  }
  if (t == 0) s_tile = atomicAdd(tile_ctr, 1u);
#pragma unroll
  for (int k = 0; k < kWarps; k++) warp_hist[k][t] = 0u;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t tile_base = tile * kTile;
  if (tile_base >= n) return;  // the grid covers n_max; tiles past n have nothing to do (no later tile waits on them)

  uint32_t keys[kItems], vals[kItems], ranks[kItems];
  const uint32_t wbase = tile_base + (uint32_t)w * (32u * kItems) + (uint32_t)lane;
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    uint32_t idx = wbase + (uint32_t)it * 32u;
    bool valid = idx < n;
    keys[it] = valid ? (uint32_t)keys_in[idx] : 0xffffffffu;
    vals[it] = valid ? (vals_in ? vals_in[idx] : idx) : 0u;
  }
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    uint32_t idx = wbase + (uint32_t)it * 32u;
    bool valid = idx < n;
    uint32_t vmask = __ballot_sync(0xffffffffu, valid);
    uint32_t d = (keys[it] >> shift) & 0xffu;
    uint32_t rank = 0;
    if (valid) {
      uint32_t peers = digit_peers(vmask, d);
      uint32_t before = warp_hist[w][d];
      rank = before + __popc(peers & lt);
      __syncwarp(vmask);
      if ((peers & lt) == 0u) warp_hist[w][d] = before + __popc(peers);
      __syncwarp(vmask);
    }
    ranks[it] = rank;
  }
  __syncthreads();

  // per digit: exclusive prefix across warps, and the tile's count
  uint32_t run = 0;
#pragma unroll
  for (int k = 0; k < kWarps; k++) {
    uint32_t c = warp_hist[k][t];
    warp_hist[k][t] = run;
    run += c;
  }
  const uint32_t tile_count = run;

  // publish this tile's counts, then look back for the exclusive prefix of digit t
  uint32_t* st = status + (size_t)tile * 256u;
  if (tile == 0) {
    atomicExch(&st[t], kFlagPrefix | tile_count);
  } else {
    atomicExch(&st[t], kFlagAgg | tile_count);
  }
  uint32_t excl = 0;
  if (tile > 0) {
    int32_t j = (int32_t)tile - 1;
    uint32_t spins = 0;
    while (j >= 0) {
      uint32_t s = load_relaxed(status + (size_t)j * 256u + t);
      uint32_t flag = s & ~kValueMask;
      if (flag == 0u) {
        if (++spins > kSpinLimit) {
          atomicExch(&ctr->timeout, 1u);
          break;
        }
        __nanosleep(32);
        continue;
      }
      excl += s & kValueMask;
      if (flag == kFlagPrefix) break;
      j--;
    }
    atomicExch(&st[t], kFlagPrefix | ((excl + tile_count) & kValueMask));
  }

  // global start of digit t: exclusive scan of the pass histogram, plus earlier tiles
  uint32_t gstart = block_exclusive_scan(digit_hist[t], warp_tot, nullptr);
  digit_base[t] = gstart + excl;
  local_start[t] = block_exclusive_scan(tile_count, warp_tot, nullptr);
  __syncthreads();

#pragma unroll
  for (int it = 0; it < kItems; it++) {
    uint32_t idx = wbase + (uint32_t)it * 32u;
    if (idx < n) {
      uint32_t d = (keys[it] >> shift) & 0xffu;
      uint32_t pos = local_start[d] + warp_hist[w][d] + ranks[it];
      s_keys[pos] = (KeyT)keys[it];
      s_vals[pos] = vals[it];
    }
  }
  __syncthreads();

  const uint32_t tile_n = (n - tile_base) < kTile ? (n - tile_base) : kTile;
  for (uint32_t j = t; j < tile_n; j += kThreads) {
    uint32_t key = s_keys[j];
    uint32_t d = (key >> shift) & 0xffu;
    uint32_t dst = digit_base[d] + (j - local_start[d]);
    if (dst >= n) continue;  // only after a look-back timeout (reported); never write out of range
    if (keys_out) keys_out[dst] = (KeyT)key;
    vals_out[dst] = s_vals[j];
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
  const uint32_t tiles = (uint32_t)sort_tiles_for(n);
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
