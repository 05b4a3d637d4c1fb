// Device-wide exclusive scan of u32 in one pass (decoupled look-back over tiles of 4096 values).  Used for the
// per-splat tile counts (entry offsets) and the per-tile entry counts (tile ranges).  Replaces the one-workgroup
// serial scans of shaders/scan.wgsl:16-43 and shaders/radix.wgsl:71-91.
#include "sl_internal.h"

namespace sl {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr uint32_t kTile = kThreads * kItems;
constexpr uint64_t kAgg = 1ull << 32;
constexpr uint64_t kPrefix = 2ull << 32;
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint64_t load_relaxed64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// publishes a status word (flag and value in one aligned word) without waiting for a round trip
__device__ __forceinline__ void store_relaxed64(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__global__ void __launch_bounds__(kThreads) scan_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                        uint32_t n, uint32_t* total, uint32_t* tile_ctr,
                                                        uint64_t* status, FrameCounters* ctr) {
  __shared__ uint32_t s_tile, s_excl;
  __shared__ uint32_t warp_tot[kThreads / 32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) s_tile = atomicAdd(tile_ctr, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t base = tile * kTile + (uint32_t)t * kItems;

  uint32_t v[kItems];
  if (base + kItems <= n) {
    const uint4* p = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
    for (int k = 0; k < kItems / 4; k++) {
      uint4 q = p[k];
      v[4 * k] = q.x;
      v[4 * k + 1] = q.y;
      v[4 * k + 2] = q.z;
      v[4 * k + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kItems; k++) v[k] = (base + k < n) ? in[base + k] : 0u;
  }
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kItems; k++) sum += v[k];

  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  uint32_t wbase = 0, agg = 0;
#pragma unroll
  for (int k = 0; k < kThreads / 32; k++) {
    uint32_t tt = warp_tot[k];
    wbase += (k < w) ? tt : 0u;
    agg += tt;
  }
  if (t == 0) {
    uint64_t* st = status + tile;
    uint32_t excl = 0;
    if (tile == 0) {
      store_relaxed64(st, kPrefix | agg);
    } else {
      store_relaxed64(st, kAgg | agg);
      int32_t j = (int32_t)tile - 1;
      uint32_t spins = 0;
      while (j >= 0) {
        uint64_t s = load_relaxed64(status + j);
        uint64_t flag = s & 0xffffffff00000000ull;
        if (flag == 0) {
          if (++spins > kSpinLimit) {
            atomicExch(&ctr->timeout, 1u);
            break;
          }
          __nanosleep(32);
          continue;
        }
        excl += (uint32_t)s;
        if (flag == kPrefix) break;
        j--;
      }
      store_relaxed64(st, kPrefix | (uint32_t)(excl + agg));
    }
    s_excl = excl;
    if (total && tile * kTile + kTile >= n) *total = excl + agg;
  }
  __syncthreads();
  uint32_t run = s_excl + wbase + x - sum;
  if (base + kItems <= n) {
    uint4* p = reinterpret_cast<uint4*>(out + base);
#pragma unroll
    for (int k = 0; k < kItems / 4; k++) {
      uint4 q;
      q.x = run;
      run += v[4 * k];
      q.y = run;
      run += v[4 * k + 1];
      q.z = run;
      run += v[4 * k + 2];
      q.w = run;
      run += v[4 * k + 3];
      p[k] = q;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      if (base + k < n) out[base + k] = run;
      run += v[k];
    }
  }
}

}  // namespace

size_t scan_scratch_bytes(uint32_t n) {
  size_t tiles = (n + kTile - 1) / kTile;
  return 16 + 8 * (tiles + 1);
}

// scratch: [0, 16) tile counter, then one u64 status word per tile.  in/out must be 16-byte aligned.
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, void* scratch,
                               FrameCounters* ctr, cudaStream_t s) {
  if (n == 0) {
    if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
    return cudaSuccess;
  }
  uint32_t tiles = (n + kTile - 1) / kTile;
  cudaError_t e = cudaMemsetAsync(scratch, 0, 16 + 8 * (size_t)tiles, s);
  if (e != cudaSuccess) return e;
  uint32_t* tile_ctr = reinterpret_cast<uint32_t*>(scratch);
  uint64_t* status = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(scratch) + 16);
  scan_kernel<<<tiles, kThreads, 0, s>>>(in, out, n, total, tile_ctr, status, ctr);
  return cudaGetLastError();
}

}  // namespace sl
