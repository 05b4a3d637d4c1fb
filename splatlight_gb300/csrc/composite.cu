// Tile compositor: one CTA of 256 threads per screen tile, one pixel per thread, each warp an 8x4-pixel block.  The
// tile's sorted splat list is walked from its nearest entry to its farthest (front to back), in batches of 256
// records; each batch is gathered into shared memory by the TMA unit (cp.async.bulk, one 48-byte bulk copy per
// record, completion counted on an mbarrier) while the previous batch is composited (double buffering).  Once a batch
// lands, every thread tests its own record's candidate box against the 8 warp blocks and the warps ballot those
// bits into per-block masks, so each warp visits only the records that can reach its pixels.  Per pixel:
//   local = (d . g0, d . g1), q = |local|^2, keep if q <= qcut (alpha >= 1/255),
//   alpha = 1 - exp(-tau0 exp(-q/2)), C += T alpha rgb, T *= 1 - alpha
// which composites the same ordered splats as the reference's back-to-front premultiplied "over" blend
// (shaders/splat.wgsl:66-78, src/renderer.js:133-143), in fp32.  A pixel stops once T < t_stop / max radiance (the
// skipped tail is below 1e-4 in every channel); a warp whose pixels all stopped skips the batch (warp vote) and the CTA
// leaves when every pixel stopped.  The overdraw view (count_mode) never stops early and counts kept fragments.
// Every mbarrier wait is bounded; a give-up sets FrameCounters::timeout and the kernel still drains its copies.
#include <cuda_fp16.h>

#include "sl_internal.h"

namespace sl {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kRecBytes = sizeof(SplatRec);
constexpr uint32_t kWaitLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// true when the phase with the given parity completed; bounded
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (uint32_t k = 0; k < kWaitLimit; k++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// One tile: (x0, y0) its origin in a width x height image, [s, e) its range in tile_vals, out/counts the image.
// kMark: the coverage pass of the batched path -- the same walk, no colour, the transmittance kept as log2 T (one ex2
// per fragment; it follows the composite's T to within rounding, and the composite's own threshold is at least twice
// this one): marks[slot] = 1 for every splat that blends a fragment before the pixel's transmittance falls below
// t_stop (never, for t_stop <= 0), and no image is written.
template <int TW, bool kMark = false>
__device__ __forceinline__ void composite_tile(uint32_t x0, uint32_t y0, uint32_t width, uint32_t height, uint32_t s,
                                               uint32_t e, const uint32_t* __restrict__ tile_vals,
                                               const SplatRec* __restrict__ recs, uint32_t count_mode, float t_stop,
                                               FrameCounters* ctr, float4* __restrict__ out,
                                               uint32_t* __restrict__ counts, uint8_t* __restrict__ marks = nullptr,
                                               const uint8_t* __restrict__ keep = nullptr) {
  constexpr int TH = kThreads / TW;
  constexpr int BX = TW / 8;  // warp blocks of 8 x 4 pixels per tile row
  constexpr int BY = TH / 4;
  static_assert(BX * BY == kThreads / 32, "one 8x4 block per warp");
  __shared__ SplatRec buf[2][kThreads];
  __shared__ uint32_t sslot[kMark ? 2 : 1][kMark ? kThreads : 1];  // coverage pass: the slots of the batch
  __shared__ uint8_t smark[kMark ? 2 : 1][kMark ? kThreads : 1];    // coverage pass: the batch's blended records
  // coverage pass: per record of the batch, (g0, o0, -tau0 log2 e) and (g1, o1, qcut'), with o = -g . (centre - tile
  // origin), so a fragment's lx = g0 . (pixel - tile origin) + o0 is two FMAs (g, o and the cutoff scaled to give q
  // in units of the exponent of 2); written by the record's thread in the culling step, read after its barrier, and
  // rewritten by the next batch only after this batch's closing barrier
  __shared__ float4 mrec[kMark ? 2 * kThreads : 1];
  __shared__ uint32_t masks[kThreads / 32][kThreads / 32];  // [warp block][loader warp]: records touching the block
  __shared__ __align__(8) uint64_t bars[2];

  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const uint32_t px = x0 + (uint32_t)((w % BX) * 8 + (lane & 7));
  const uint32_t py = y0 + (uint32_t)((w / BX) * 4 + (lane >> 3));
  const bool inside = px < width && py < height;

  const uint32_t bar0 = smem_addr(&bars[0]), bar1 = smem_addr(&bars[1]);
  if constexpr (kMark) smark[0][t] = smark[1][t] = 0;
  if (t == 0) {
    mbar_init(bar0, kThreads);
    mbar_init(bar1, kThreads);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const uint32_t n_batches = (e - s + kThreads - 1) / kThreads;
  const float pxc = (float)px + 0.5f, pyc = (float)py + 0.5f;
  const float pxr = (float)(px - x0) + 0.5f, pyr = (float)(py - y0) + 0.5f;  // relative to the tile's origin
  const float fx0 = (float)x0, fy0 = (float)y0;
  const float kNegHalfLog2e = -0.72134752044448170f;
  const float kNegLog2e = -1.44269504088896341f;
  // coverage pass: its keep test evaluates q in tile-relative coordinates (a few ulps away from the composite's q,
  // whose rounding it need not match), so it keeps fragments up to a cutoff 1e-4 (relative) above the composite's:
  // every fragment the composite blends is marked
  const float kMarkCutScale = 1.0001f;

  float T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f;
  uint32_t kept = 0;
  // coverage pass: log2 T, which falls by tau0 exp(-q/2) log2(e) per blended fragment (the composite's factor
  // 1 - alpha = exp(-tau0 exp(-q/2))), against log2 of the threshold (never reached for t_stop <= 0)
  float l2T = 0.0f;
  const float l2stop = kMark && t_stop > 0.0f ? __log2f(t_stop) : -INFINITY;
  bool alive = inside;
  bool timed_out = false;

  // gather batch b (entries [max(s, e-256(b+1)), e-256b), nearest first) into buf[b & 1]; with keep (a lit view of the
  // batched path: the coverage pass's marks), a record whose splat blends no fragment anywhere is neither copied nor
  // culled (bit b & 1 of dropped, for the thread's own record)
  uint32_t dropped = 0;
  auto issue = [&](uint32_t b) {
    const uint32_t hi = e - kThreads * b;
    const uint32_t lo = (hi - s) > (uint32_t)kThreads ? hi - kThreads : s;
    const uint32_t bar = (b & 1u) ? bar1 : bar0;
    dropped &= ~(1u << (b & 1u));
    if ((uint32_t)t < hi - lo) {
      const uint32_t slot = tile_vals[hi - 1u - (uint32_t)t];
      if constexpr (kMark) sslot[b & 1u][t] = slot;
      if (keep && keep[slot] == 0u) {
        dropped |= 1u << (b & 1u);
        mbar_arrive(bar);
      } else {
        mbar_arrive_expect(bar, kRecBytes);
        bulk_copy_g2s(smem_addr(&buf[b & 1u][t]), recs + slot, kRecBytes, bar);
      }
    } else {
      mbar_arrive(bar);
    }
  };

  if (n_batches > 0) issue(0);
  for (uint32_t b = 0; b < n_batches; b++) {
    if (b + 1 < n_batches) issue(b + 1);
    const uint32_t bar = (b & 1u) ? bar1 : bar0;
    if (!mbar_wait(bar, (b >> 1) & 1u)) timed_out = true;
    const uint32_t hi = e - kThreads * b;
    const uint32_t nb = (hi - s) > (uint32_t)kThreads ? (uint32_t)kThreads : hi - s;
    const SplatRec* rb = buf[b & 1u];

    // culling, SIMD across records: which warp blocks can record t reach?  Its candidate box is centre +- (hx, hy)
    // (one pixel of margin included, rounded up); block (bx, by) holds pixel centres x0 + 8bx + [0.5, 7.5],
    // y0 + 4by + [0.5, 3.5].
    uint32_t bits = 0;
    if ((uint32_t)t < nb && !((dropped >> (b & 1u)) & 1u)) {
      const float4 A = rb[t].a;
      const float hb = rb[t].b.z;
      const __half2 hxy = *reinterpret_cast<const __half2*>(&hb);
      const float hx = __low2float(hxy), hy = __high2float(hxy);
      int bx0 = (int)ceilf((A.x - hx - 7.5f - fx0) * 0.125f), bx1 = (int)floorf((A.x + hx - 0.5f - fx0) * 0.125f);
      int by0 = (int)ceilf((A.y - hy - 3.5f - fy0) * 0.25f), by1 = (int)floorf((A.y + hy - 0.5f - fy0) * 0.25f);
      bx0 = max(bx0, 0);
      by0 = max(by0, 0);
      bx1 = min(bx1, BX - 1);
      by1 = min(by1, BY - 1);
      if (bx0 <= bx1 && by0 <= by1) {
        // of the blocks in the box, keep those the ellipse q <= qcut can reach: with local = G d, a pixel p of a
        // block centred at c has |G (p - mu)| >= |G (c - mu)| - R, R the largest |G h| over the block's half-extent
        // corners h = (+-3.5, +-1.5) (a norm is convex, so its maximum over the rectangle is at a corner); a block
        // with |G (c - mu)| > sqrt(qcut) + R holds no kept pixel.  The limit carries a relative margin of 1e-3 and
        // an absolute one of 1e-3, far above the rounding of the per-pixel q, so no kept fragment is ever culled.
        const float g00 = A.z, g01 = A.w, g10 = rb[t].b.x, g11 = rb[t].b.y;
        const float r1x = fmaf(3.5f, g00, 1.5f * g01), r1y = fmaf(3.5f, g10, 1.5f * g11);
        const float r2x = fmaf(3.5f, g00, -1.5f * g01), r2y = fmaf(3.5f, g10, -1.5f * g11);
        const float R = sqrtf(fmaxf(fmaf(r1x, r1x, r1y * r1y), fmaf(r2x, r2x, r2y * r2y)));
        const float lim = fmaf(sqrtf(fmaxf(rb[t].b.w, 0.0f)) + R, 1.001f, 1e-3f);
        const float lim2 = lim * lim;
        const float ox = fx0 + 4.0f - A.x, oy = fy0 + 2.0f - A.y;  // block (0, 0)'s centre less the splat's
        for (int by = by0; by <= by1; by++) {
          const float dy = fmaf(4.0f, (float)by, oy);
          for (int bx = bx0; bx <= bx1; bx++) {
            const float dx = fmaf(8.0f, (float)bx, ox);
            const float lx = fmaf(dx, g00, dy * g01), ly = fmaf(dx, g10, dy * g11);
            if (fmaf(lx, lx, ly * ly) <= lim2) bits |= 1u << (by * BX + bx);
          }
        }
      }
      if constexpr (kMark) {
        const float4 B = rb[t].b;
        const float cxr = A.x - fx0, cyr = A.y - fy0;
        // gradients and offsets scaled by sqrt(log2(e) / 2): q comes out as (q / 2) log2 e, the exponent of 2 the
        // fragment's exp(-q / 2) needs, and the cutoff is scaled alike
        const float ks = 0.84932180f;
        mrec[2 * t] = make_float4(A.z * ks, A.w * ks, -(A.z * cxr + A.w * cyr) * ks, rb[t].c.w * kNegLog2e);
        mrec[2 * t + 1] = make_float4(B.x * ks, B.y * ks, -(B.x * cxr + B.y * cyr) * ks,
                                      B.w * kMarkCutScale * -kNegHalfLog2e);
      }
    }
#pragma unroll
    for (int k = 0; k < kThreads / 32; k++) {
      const uint32_t m = __ballot_sync(0xffffffffu, (bits >> k) & 1u);
      if (lane == 0) masks[k][w] = m;
    }
    __syncthreads();

    if (__any_sync(0xffffffffu, alive)) {
      for (int lw = 0; lw < kThreads / 32; lw++) {
        uint32_t m = masks[w][lw];
        while (m) {
          const uint32_t j = (uint32_t)(lw * 32 + __ffs(m) - 1);
          m &= m - 1u;
          if constexpr (kMark) {
            const float4 P0 = mrec[2 * j], P1 = mrec[2 * j + 1];
            const float lx = fmaf(pxr, P0.x, fmaf(pyr, P0.y, P0.z));
            const float ly = fmaf(pxr, P1.x, fmaf(pyr, P1.y, P1.z));
            const float q = fmaf(lx, lx, ly * ly);
            if (alive && q <= P1.w) {
              l2T = fmaf(P0.w, ex2_approx(-q), l2T);
              smark[b & 1u][j] = 1u;
              if (l2T < l2stop) alive = false;
            }
            continue;
          }
          const float4 A = rb[j].a;
          const float4 B = rb[j].b;
          const float dx = pxc - A.x, dy = pyc - A.y;
          const float lx = fmaf(dx, A.z, dy * A.w);
          const float ly = fmaf(dx, B.x, dy * B.y);
          const float q = fmaf(lx, lx, ly * ly);
          if (alive && q <= B.w) {
            const float4 C = rb[j].c;
            const float ev = ex2_approx(q * kNegHalfLog2e);
            const float alpha = 1.0f - ex2_approx(C.w * kNegLog2e * ev);
            const float wgt = T * alpha;
            cr = fmaf(wgt, C.x, cr);
            cg = fmaf(wgt, C.y, cg);
            cb = fmaf(wgt, C.z, cb);
            T = T - wgt;
            kept++;
            if (T < t_stop) alive = false;
          }
        }
        if (!__any_sync(0xffffffffu, alive)) break;
      }
    }
    const bool any_alive = __syncthreads_count(alive) != 0;
    if constexpr (kMark) {  // one store per blended record of the batch
      if (smark[b & 1u][t]) {
        marks[sslot[b & 1u][t]] = 1u;
        smark[b & 1u][t] = 0;
      }
    }
    if (!any_alive) {
      // every pixel is done: drain the batch already in flight before leaving
      if (b + 1 < n_batches) {
        if (!mbar_wait((b & 1u) ? bar0 : bar1, ((b + 1) >> 1) & 1u)) timed_out = true;
      }
      break;
    }
  }
  if (timed_out) atomicExch(&ctr->timeout, 1u);
  if constexpr (kMark) return;
  const uint32_t wk = __reduce_add_sync(0xffffffffu, kept);
  if (lane == 0 && wk) atomicAdd(&ctr->fragments, wk);
  if (inside) {
    const size_t pix = (size_t)py * width + px;
    if (count_mode) {
      out[pix] = make_float4((float)kept, 0.0f, 0.0f, 0.0f);
      if (counts) counts[pix] = kept;
    } else {
      out[pix] = make_float4(cr, cg, cb, 1.0f - T);
    }
  }
}


template <int TW>
__global__ void __launch_bounds__(kThreads) composite_kernel(const CompositeParams P, const uint2* __restrict__ ranges,
                                                             const uint32_t* __restrict__ tile_vals,
                                                             const SplatRec* __restrict__ recs,
                                                             FrameCounters* ctr, float4* __restrict__ out,
                                                             uint32_t* __restrict__ counts) {
  constexpr int TH = kThreads / TW;
  const uint32_t tile = blockIdx.x;
  const uint32_t tx = tile % P.tiles_x, ty = tile / P.tiles_x;
  const uint2 rg = ranges[tile];
  const float maxrad = fmaxf(__uint_as_float(ctr->max_rad_bits), 1.0f);
  const float t_stop = P.count_mode ? -1.0f : P.t_stop_scale / maxrad;
  composite_tile<TW>(tx * TW, ty * TH, P.width, P.height, rg.x, rg.y, tile_vals, recs, P.count_mode, t_stop, ctr, out,
                     counts);
}

// Batched: one CTA per tile of any view; the view comes from a binary search of the tiles' prefix over views.
// MinB blocks per SM (the autotuner's variants: 6 = at most 40 registers, a few bytes spilled on a cold path; 5 =
// uncapped at 46 registers, which measured 4% slower on the 64-view mix).
template <int TW, int MinB>
__global__ void __launch_bounds__(kThreads, MinB) bcomposite_kernel(const BatchComposite B, const uint2* __restrict__ ranges,
                                                              const uint32_t* __restrict__ tile_vals,
                                                              const SplatRec* __restrict__ recs,
                                                              const BatchViewOut* __restrict__ views,
                                                              const uint32_t* __restrict__ view_maxrad,
                                                              const BatchDyn* __restrict__ dyn, FrameCounters* ctr,
                                                              const uint8_t* __restrict__ marks) {
  constexpr int TH = kThreads / TW;
  const uint32_t tile = blockIdx.x;
  if (tile >= dyn->total_tiles) return;  // grid sized for the capacity
  float4* out = dyn->out;
  uint32_t lo = 0, hi = dyn->n_views;  // the last view whose tile_base <= tile
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (views[mid].tile_base <= tile) lo = mid; else hi = mid;
  }
  const BatchViewOut v = views[lo];
  const uint32_t lt = tile - v.tile_base;
  const uint32_t tx = lt % v.tiles_x, ty = lt / v.tiles_x;
  const uint2 rg = ranges[tile];
  const float maxrad = fmaxf(__uint_as_float(view_maxrad[lo]), 1.0f);
  const float t_stop = v.count_mode ? -1.0f : B.t_stop_scale / maxrad;
  // a lit view blends only splats the coverage pass marked (its cut is conservative: an unmarked splat blends no
  // fragment before T < t_stop), so the rest of its list is skipped
  composite_tile<TW>(tx * TW, ty * TH, v.width, v.height, rg.x, rg.y, tile_vals, recs, v.count_mode, t_stop, ctr,
                     out + v.out_offset, nullptr, nullptr, v.lit ? marks : nullptr);
}

// The batched coverage pass over the tiles of lit views (see composite_tile): mode 1 stops each pixel at the view's
// t_mark, mode 2 never stops (every splat that blends any pixel is marked).
template <int TW>
__global__ void __launch_bounds__(kThreads) bmark_kernel(const BatchComposite B, const uint2* __restrict__ ranges,
                                                         const uint32_t* __restrict__ tile_vals,
                                                         const SplatRec* __restrict__ recs,
                                                         const BatchViewOut* __restrict__ views,
                                                         const uint32_t* __restrict__ view_maxrad,
                                                         const BatchDyn* __restrict__ dyn, FrameCounters* ctr,
                                                         uint8_t* __restrict__ marks, float* __restrict__ view_tmark) {
  constexpr int TH = kThreads / TW;
  const uint32_t tile = blockIdx.x;
  if (tile >= dyn->total_tiles) return;
  uint32_t lo = 0, hi = dyn->n_views;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (views[mid].tile_base <= tile) lo = mid; else hi = mid;
  }
  const BatchViewOut v = views[lo];
  if (v.lit == 0u) return;  // only lit views are shaded
  const float t_mark = B.t_stop_scale / fmaxf(2.0f * __uint_as_float(view_maxrad[lo]), v.rad_cap);
  const uint32_t lt = tile - v.tile_base;
  if (lt == 0 && threadIdx.x == 0) view_tmark[lo] = t_mark;
  const uint32_t tx = lt % v.tiles_x, ty = lt / v.tiles_x;
  const uint2 rg = ranges[tile];
  composite_tile<TW, true>(tx * TW, ty * TH, v.width, v.height, rg.x, rg.y, tile_vals, recs, 0u,
                           v.lit == 1u ? t_mark : -1.0f, ctr, nullptr, nullptr, marks);
}

}  // namespace

cudaError_t launch_bmark(const BatchComposite& B, const uint2* ranges, const uint32_t* tile_vals, const SplatRec* recs,
                         const BatchViewOut* views, const uint32_t* view_maxrad, const BatchDyn* dyn,
                         uint32_t max_tiles, FrameCounters* ctr, uint8_t* marks, float* view_tmark, cudaStream_t s) {
  if (max_tiles == 0) return cudaSuccess;
  switch (B.tile_w) {
    case 16:
      bmark_kernel<16><<<max_tiles, kThreads, 0, s>>>(B, ranges, tile_vals, recs, views, view_maxrad, dyn, ctr, marks,
                                                      view_tmark);
      break;
    case 8:
      bmark_kernel<8><<<max_tiles, kThreads, 0, s>>>(B, ranges, tile_vals, recs, views, view_maxrad, dyn, ctr, marks,
                                                     view_tmark);
      break;
    case 32:
      bmark_kernel<32><<<max_tiles, kThreads, 0, s>>>(B, ranges, tile_vals, recs, views, view_maxrad, dyn, ctr, marks,
                                                      view_tmark);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_composite(const CompositeParams& P, const uint2* ranges, const uint32_t* tile_vals,
                             const SplatRec* recs, FrameCounters* ctr, float4* out, uint32_t* counts,
                             cudaStream_t s) {
  const uint32_t tiles = P.tiles_x * P.tiles_y;
  if (tiles == 0) return cudaSuccess;
  if (P.tile_w * P.tile_h != (uint32_t)kThreads) return cudaErrorInvalidValue;
  switch (P.tile_w) {
    case 16:
      composite_kernel<16><<<tiles, kThreads, 0, s>>>(P, ranges, tile_vals, recs, ctr, out, counts);
      break;
    case 8:
      composite_kernel<8><<<tiles, kThreads, 0, s>>>(P, ranges, tile_vals, recs, ctr, out, counts);
      break;
    case 32:
      composite_kernel<32><<<tiles, kThreads, 0, s>>>(P, ranges, tile_vals, recs, ctr, out, counts);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace sl

namespace sl {
cudaError_t launch_bcomposite(const BatchComposite& B, const uint2* ranges, const uint32_t* tile_vals,
                              const SplatRec* recs, const BatchViewOut* views, const uint32_t* view_maxrad,
                              const BatchDyn* dyn, uint32_t max_tiles, FrameCounters* ctr, const uint8_t* marks,
                              int variant, cudaStream_t s) {
  if (max_tiles == 0) return cudaSuccess;
  const int mb = kTuneMinBlocks[3][variant];
  if (mb != 5 && mb != 6) return cudaErrorInvalidValue;
#define SL_BCOMP(TW, MB)                                                                                        \
  bcomposite_kernel<TW, MB><<<max_tiles, kThreads, 0, s>>>(B, ranges, tile_vals, recs, views, view_maxrad, dyn, \
                                                           ctr, marks)
  switch (B.tile_w) {
    case 16:
      if (mb == 6) SL_BCOMP(16, 6); else SL_BCOMP(16, 5);
      break;
    case 8:
      if (mb == 6) SL_BCOMP(8, 6); else SL_BCOMP(8, 5);
      break;
    case 32:
      if (mb == 6) SL_BCOMP(32, 6); else SL_BCOMP(32, 5);
      break;
    default:
      return cudaErrorInvalidValue;
  }
#undef SL_BCOMP
  return cudaGetLastError();
}
}  // namespace sl
