// Internal declarations shared by the CUDA translation units of libsplatlight.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "splatlight.h"

namespace sl {

constexpr uint32_t kInvalidKey16 = 0xffffu;   // 16-bit depth key of a culled slot (sorts after every valid key)
constexpr uint32_t kEmitterMaterial = 254u;   // shaders/common.wgsl:41
constexpr uint32_t kMaxParts = 32u;           // shaders/common.wgsl:39
constexpr uint32_t kPartHidden = 4u;          // shaders/common.wgsl:40

// One projected splat as the compositor reads it: 48 B, 16-byte aligned, one bulk copy per record.
//   a = (cx, cy, g0x, g0y)   centre in framebuffer pixels (y down) and the first grad row
//   b = (g1x, g1y, hxy, qcut) second grad row, half2 half extents of the candidate box (bits), keep bound q <= qcut
//   c = (r, g, b, tau0)      radiance and peak optical depth
struct __align__(16) SplatRec {
  float4 a, b, c;
};

// Per-part data the projection reads (shaders/common.wgsl:17-25 Part, RenderFrame.part_material/part_fade).
struct PartXf {
  float xf[12];
  float xf_prev[12];  // the pose at the start of the exposure (motion blur of a moving part, flags bit 1)
  uint32_t flags;
  uint32_t material;
  float keep;  // 1 - clamp(part_fade)
  uint32_t pad;
};

// Everything project() reads from the RenderFrame, packed once per frame by the host (kernel parameter).
struct ProjectParams {
  float view[16];
  float focal[2];
  float viewport[2];
  float near_plane, far_plane, lowpass_px2, albedo_scale;
  float bounce_gain;
  float shutter;         // palette[3].z: motion-blur shutter fraction (0 = off)
  uint32_t blur_cov;     // palette[3].w > 0.5: cap a smeared splat's peak coverage at the sharp one's
  uint32_t count, n_emit, n_slots, view_mode, part_count;
  uint32_t tile_w, tile_h, tiles_x, tiles_y;
  float palette[8][4];  // slots 0-7 (slot 3 = white, w 0)
  uint32_t lod_on, node_base, n_int, lod_pad;  // screen-space LOD (frame.lod): slots from node_base are tree nodes
  PartXf parts[kMaxParts];
};

// What the projection reads of a screen-space LOD cut (csrc/lod.cu): the flag of every tree node (2 = drawn), the
// internal nodes' Gaussian records and their lit colours.
struct LodDraw {
  const uint32_t* flags;
  const sl_gaussian* nodes;
  const float4* colour;
};

// Frame-wide device counters written by the pipeline (one per view).
struct FrameCounters {
  uint32_t visible;        // valid keys
  uint32_t max_rad_bits;   // max radiance component (float bits, >= 0)
  uint32_t entries;        // tile entries
  uint32_t overflow;       // entries beyond capacity
  uint32_t timeout;        // a bounded device wait gave up
  uint32_t fragments;      // fragments composited (kept and blended) by the compositor
  uint32_t shade_n;        // batched path: marked Gaussians of lit views (the shading list's length)
  uint32_t pad;
};

// ---- launchers (each returns cudaError_t of the launch) ----------------------------------------------------------

// project.cu
cudaError_t launch_project(const ProjectParams& P, const sl_gaussian* gaussians, const sl_gaussian* emitters,
                           const float4* colour, const float4* lo_b, uint16_t* key16, SplatRec* recs,
                           ushort4* rects, uint32_t* digit_hist /*[2][256]*/, FrameCounters* ctr, cudaStream_t s,
                           LodDraw lod = LodDraw{nullptr, nullptr, nullptr});

// sort_api.cu: the counting sort of 16-bit depth keys (shaders/scan.wgsl + scatter.wgsl): key counts (valid keys),
// then, after an exclusive scan of the 65536 counts into offsets, order[atomicAdd(&offsets[key], 1)] = i.
cudaError_t launch_key_hist(const uint16_t* key16, uint32_t n, uint32_t* hist, cudaStream_t s);
cudaError_t launch_key_scatter(const uint16_t* key16, uint32_t n, uint32_t* offsets, uint32_t* order, cudaStream_t s);

// lod.cu: one tree depth of lod_select (nodes level[off, off + n_all)) / lod_colour (the depth's internal nodes)
struct LodPart {
  float xf[12], xf_prev[12];
  uint32_t root, flags;
};
struct LodSelectParams {
  float view[16];
  float focal, near_plane, threshold, shutter, blur_lod;
  uint32_t G, emit_part, size_rule, part_count;
  LodPart parts[kMaxParts];
};
cudaError_t launch_lod_select(const LodSelectParams& P, const sl_node* nodes, const uint32_t* kids,
                              const uint32_t* level, uint32_t off, uint32_t n_all, uint32_t* flags, cudaStream_t s);
cudaError_t launch_lod_colour(uint32_t G, float gain, uint32_t colour_all, const sl_node* nodes, const uint32_t* kids,
                              const uint32_t* level, uint32_t off, uint32_t n_int, const uint32_t* flags,
                              const float4* colour, const float4* lo_b, float4* ncolour, cudaStream_t s);
// The depths [0, depths) in one CTA (lvl_off / lvl_all / lvl_int: device copies of the per-depth tables).
constexpr uint32_t kLodTopNodes = 1024;  // a depth with at most this many nodes joins the one-CTA top
cudaError_t launch_lod_select_top(const LodSelectParams& P, const sl_node* nodes, const uint32_t* kids,
                                  const uint32_t* level, const uint32_t* lvl_off, const uint32_t* lvl_all,
                                  uint32_t depths, uint32_t* flags, cudaStream_t s);
cudaError_t launch_lod_colour_top(uint32_t G, float gain, uint32_t colour_all, const sl_node* nodes,
                                  const uint32_t* kids, const uint32_t* level, const uint32_t* lvl_off,
                                  const uint32_t* lvl_int, uint32_t depths, const uint32_t* flags,
                                  const float4* colour, const float4* lo_b, float4* ncolour, cudaStream_t s);

// sort.cu: onesweep LSD radix sort of 16-bit keys with u32 values, over tiles of kSortTileKeys keys.
constexpr uint32_t kSortTileKeys = 4096;
constexpr size_t sort_tiles_const(uint32_t n) { return (n + kSortTileKeys - 1) / kSortTileKeys; }

// Scratch layout of one standalone 16-bit sort of n keys (sort_api.cu): every offset 256-byte aligned.
struct Sort16Layout {
  size_t hist, counters, tile_ctr, status, keys_alt, vals_alt, total;
  uint32_t tiles;
};
constexpr size_t align256c(size_t x) { return (x + 255) & ~size_t(255); }
constexpr Sort16Layout sort16_layout(uint32_t n) {
  Sort16Layout L{};
  L.tiles = (uint32_t)sort_tiles_const(n ? n : 1);
  L.hist = 0;                                                  // [2][256] digit counts
  L.counters = align256c(L.hist + 2 * 256 * 4);                // FrameCounters
  L.tile_ctr = align256c(L.counters + sizeof(FrameCounters));  // one tile ticket per pass
  L.status = align256c(L.tile_ctr + 16);                       // look-back words, [2][tiles][256]
  L.keys_alt = align256c(L.status + 2ull * 256 * 4 * L.tiles);
  L.vals_alt = align256c(L.keys_alt + 2ull * n);
  L.total = align256c(L.vals_alt + 4ull * n);
  return L;
}

struct SortScratch {
  uint16_t* keys_alt;
  uint32_t* vals_alt;
  uint32_t* status;      // [passes][max_tiles][256]
  uint32_t* tile_ctr;    // [passes]
  uint32_t max_tiles;
};
size_t sort_tiles_for(uint32_t n);
// Sorts keys[0, n) (16-bit, `bits` significant bits) stably; vals: input values (NULL = slot index);
// writes the permutation/values to vals_out.  digit_hist: [passes][256] counts of the digits of every key
// (pass p = bits 8p .. 8p+7), filled by the producer kernel.  Keys are ping-ponged through scratch.
// n is the element count, or with n_dev non-null an upper bound and *n_dev (read on the device) the count.
// keys_out: where the last pass writes the sorted keys (NULL: not written).
cudaError_t sort16_pairs(uint16_t* keys, const uint32_t* vals_in, uint32_t* vals_out, uint32_t n,
                         const uint32_t* n_dev, int bits, const uint32_t* digit_hist, SortScratch& sc,
                         FrameCounters* ctr, cudaStream_t s, uint16_t* keys_out = nullptr);
// The same for 32-bit keys (up to 4 passes); status holds 256 words per tile and pass, tile_ctr 4 counters.
cudaError_t sort32_pairs(uint32_t* keys, uint32_t* keys_alt, const uint32_t* vals_in, uint32_t* vals_out,
                         uint32_t* vals_alt, uint32_t n, const uint32_t* n_dev, int bits, const uint32_t* digit_hist,
                         uint32_t* status, uint32_t* tile_ctr, uint32_t max_tiles, FrameCounters* ctr, cudaStream_t s,
                         uint32_t* keys_out = nullptr, const uint32_t* keys_first = nullptr);
// keys_first (optional): the first pass reads the keys from there and leaves them intact (keys is then scratch).
// Counts the digit histograms of u32 keys ([passes][256]).
cudaError_t launch_digit_hist32(const uint32_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s);
// Counts the digit histograms of u16 keys (used when no producer kernel filled them).
cudaError_t launch_digit_hist16(const uint16_t* keys, uint32_t n, int passes, uint32_t* hist, cudaStream_t s);

// scan.cu: exclusive scan of u32 (single pass, decoupled look-back); total written to *total if not null.
size_t scan_scratch_bytes(uint32_t n);
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, void* scratch,
                               FrameCounters* ctr, cudaStream_t s);

// tiles.cu
// One pass: tile counts, their offsets (decoupled look-back) and the entries of the visible sorted splats; the
// entry total to ctr->entries.  scratch: tile_bin_scratch_bytes(n) bytes, cleared by the launcher.
size_t tile_bin_scratch_bytes(uint32_t n);
cudaError_t launch_tile_bin(const uint32_t* order, const ushort4* rects, const SplatRec* recs, uint32_t n,
                            uint32_t tiles_x, uint32_t tw, uint32_t th, uint32_t capacity, FrameCounters* ctr,
                            uint16_t* tile_keys, uint32_t* tile_vals, uint32_t* digit_hist /*[2][256]*/,
                            void* scratch, cudaStream_t s);
// ranges[tile] = the run of the tile's entries in the sorted keys (ranges zeroed beforehand: empty tiles [0, 0)).
cudaError_t launch_tile_ranges(const uint16_t* sorted_keys, const uint32_t* n_dev, uint32_t n_max, uint2* ranges,
                               cudaStream_t s);

// composite.cu
struct CompositeParams {
  uint32_t width, height, tile_w, tile_h, tiles_x, tiles_y;
  uint32_t count_mode;  // 1: overdraw view (contributor counts, no early termination)
  float t_stop_scale;   // early termination when T < t_stop_scale / max radiance
};
cudaError_t launch_composite(const CompositeParams& P, const uint2* ranges, const uint32_t* tile_vals,
                             const SplatRec* recs, FrameCounters* ctr, float4* out, uint32_t* counts,
                             cudaStream_t s);

// ---- batched path ---------------------------------------------------------------------------------------------

// One view of a batch as the projection and shading read it (device array).
struct BatchView {
  ProjectParams P;                       // the view's RenderFrame, packed as for the per-view path
  const float4* gaussians;               // its scene's records
  const float4* emitters;
  const float4* colour;                  // bound radiance of a scene without lighting (else null: the shading pass)
  const float4* lo_b;
  uint32_t scene;                        // index into the batch's scenes
  uint32_t slot_base;                    // first global slot (a multiple of 256)
  uint32_t block_first;                  // slot_base / 256
  uint32_t tile_base, tiles_x;           // first global tile, tiles per row
  float eye[3];                          // shading eye
  float light_scale;                     // the request's light-intensity scale (emitters and distant lights)
};
constexpr uint32_t kNoView = 0xFFFFFFFFu;
// block_valid[block]: the block's valid keys (0 for blocks past the batch); digit_hist counts valid keys only.
// The batched chain's block-size variants, picked per kernel by sl_batch_autotune: blocks per SM that each kernel's
// register budget is compiled for (variant 0 is the default).
constexpr int kTuneKernels = 4;                  // bproject, btile_bin, bshade, bcomposite
constexpr int kTuneVariants[kTuneKernels] = {2, 2, 3, 2};
constexpr int kTuneMinBlocks[kTuneKernels][3] = {{4, 3, 0}, {4, 5, 0}, {4, 3, 5}, {6, 5, 0}};
cudaError_t launch_bproject(const BatchView* views, const uint32_t* block_view, uint32_t max_blocks, uint32_t* keys32,
                            SplatRec* recs, ushort4* rects, uint32_t* digit_hist /*[3][256]*/,
                            uint32_t* view_maxrad, uint32_t* view_visible, uint32_t* block_valid, int variant,
                            cudaStream_t s);
// batch.cu: the valid keys of every block, in slot order, at block_off[block] (the exclusive scan of block_valid):
// keys_c / slots_c, for the depth sort over the visible slots only.
cudaError_t launch_bcompact(const uint32_t* block_view, const uint32_t* keys32, const uint32_t* block_off,
                            uint32_t max_blocks, uint32_t* keys_c, uint32_t* slots_c, cudaStream_t s);

// What the batched compositor needs of each view (device array, ascending tile_base).
struct BatchViewOut {
  uint32_t tile_base, tiles_x, width, height;
  uint32_t count_mode;
  uint32_t lit;         // 0: not shaded; shaded (view mode 3 of a lit scene) where the coverage pass marks a splat,
                        // 1: blended before T < t_mark (launch_bmark), 2: blended anywhere (never stops)
  uint64_t out_offset;  // first float4 of the view's image in the packed output
  float rad_cap;        // the coverage pass's radiance allowance: kRadianceCap x max(1, the view's light scale)
  uint32_t pad;
};
struct BatchComposite {
  uint32_t tile_w, tile_h;
  float t_stop_scale;
  uint32_t pad;
};
// Per-batch values the captured chain reads from device memory (uploaded before every launch).
struct BatchDyn {
  uint32_t total_slots;   // padded slots of all views
  uint32_t total_tiles;
  uint32_t n_views;
  uint32_t total_blocks;
  float4* out;            // the packed images
};
cudaError_t launch_bcomposite(const BatchComposite& B, const uint2* ranges, const uint32_t* tile_vals,
                              const SplatRec* recs, const BatchViewOut* views, const uint32_t* view_maxrad,
                              const BatchDyn* dyn, uint32_t max_tiles, FrameCounters* ctr, const uint8_t* marks,
                              int variant, cudaStream_t s);
// batch.cu (totals: the BatchDyn, read as u32 words: [0] total slots, [1] total tiles)
// batch.cu: the batch's tile entries in one pass (counts, their ordered offsets by a decoupled look-back, emission);
// the entry total goes to ctr->entries.  scratch: btile_bin_scratch_bytes(n_max) bytes, cleared by the launcher.
size_t btile_bin_scratch_bytes(uint32_t n_max);
cudaError_t launch_btile_bin(const uint32_t* order, const ushort4* rects, const SplatRec* recs, const BatchView* views,
                             const uint32_t* block_view, const uint32_t* n_dev, uint32_t n_max, uint32_t tw,
                             uint32_t th, uint32_t capacity, FrameCounters* ctr, uint32_t* tile_keys,
                             uint32_t* tile_vals, uint32_t* digit_hist, void* scratch, int variant, cudaStream_t s);
// The batched coverage pass over the tiles of lit views, run between binning and shading: marks[slot] = 1 for each
// splat that blends a fragment before the pixel's transmittance falls below t_mark (BatchViewOut::lit 1) or at all
// (lit 2).  t_mark = t_stop_scale / max(2 r, rad_cap), r the view's radiance bound so far (its unshaded splats,
// view_maxrad), rad_cap = allowance x max(1, light scale) (shaded radiance scales with the light intensities;
// the allowance is sl_batch_options.radiance_allowance, kRadianceCap by default), is
// written to view_tmark[view].  The composite, whose threshold is t_stop_scale / (the bound after
// shading), blends only marked splats as long as that threshold stays >= 2 t_mark.
constexpr float kRadianceCap = 64.0f;
cudaError_t launch_bmark(const BatchComposite& B, const uint2* ranges, const uint32_t* tile_vals, const SplatRec* recs,
                         const BatchViewOut* views, const uint32_t* view_maxrad, const BatchDyn* dyn,
                         uint32_t max_tiles, FrameCounters* ctr, uint8_t* marks, float* view_tmark, cudaStream_t s);
// The batched shading list: per view, the Gaussians of lit views the coverage pass marked, at list[slot_base, +n)
// (their global slots; each block's in shading order, the blocks in any order), n in view_shade[view] (n_views words,
// cleared by the launcher) and the batch's total added to ctr->shade_n.
struct BatchScene;
cudaError_t launch_bshade_list(const BatchView* views, const BatchScene* scenes, const uint32_t* block_view,
                               const uint8_t* marks, const uint32_t* totals, uint32_t max_blocks, uint32_t n_views,
                               FrameCounters* ctr, uint32_t* list, uint32_t* view_shade, cudaStream_t s);
// Tile keys are (view << 16) | view-local tile id; after the stable sort on the local id each (view, tile) run's
// bounds are written to ranges[tile_base[view] + local] (ranges zeroed first).
cudaError_t launch_btile_runs(const uint32_t* keys, const uint32_t* n_dev, uint32_t n_max, const BatchViewOut* views,
                              uint2* ranges, cudaStream_t s);

}  // namespace sl
