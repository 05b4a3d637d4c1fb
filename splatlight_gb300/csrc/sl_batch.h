// Host state of a batch renderer (capi_batch.cu) and the steps of one batch, shared with the request server.
#pragma once

#include <vector>

#include "sl_runtime.h"

struct sl_batch {
  int device = 0;
  std::vector<sl_renderer*> scenes;
  std::vector<sl_lighting*> lights;
  // capacity
  uint32_t max_views = 0, max_blocks = 0, max_tiles = 0;
  uint64_t max_slots = 0, entry_cap = 0;
  uint32_t tile_w = 16, tile_h = 16;
  int variant[sl::kTuneKernels] = {0, 0, 0, 0};  // block-size variant of bproject, btile_bin, bshade, bcomposite
  float t_stop_scale = 1e-4f;
  float rad_allow = sl::kRadianceCap;  // the coverage pass's radiance allowance (sl_batch_options)
  float entry_ratio = 0.0f;  // the most tile entries per slot a batch has had: the capacity class must hold the
                             // batch's slots times this (a class too small for the entries costs a second launch)
  bool use_graph = true;
  // device buffers
  sl::DevBuf views, views_out, block_view, scenes_dev, dyn, keys32, keys_alt, vals_alt, order, recs, rects,
      tile_keys, tile_keys_alt, tile_vals, tile_vals_alt, status, tile_ctr, hist,
      scan_scratch, bin_scratch, ranges, block_valid, block_off, counters, view_maxrad, view_visible, marks,
      view_tmark, view_shade;
  // pinned staging
  sl::BatchView* h_views = nullptr;
  sl::BatchViewOut* h_out = nullptr;
  uint32_t* h_block_view = nullptr;
  sl::BatchScene* h_scenes = nullptr;
  sl::BatchDyn* h_dyn = nullptr;
  sl::FrameCounters* h_ctr = nullptr;
  uint32_t* h_visible = nullptr;
  uint32_t* h_maxrad = nullptr;  // per view: its radiance bound (float bits) after shading
  float* h_tmark = nullptr;      // per view: its coverage pass's threshold
  // graph
  cudaStream_t cap_stream = nullptr;
  // per tile shape (16x16, 8x32, 32x8) and capacity class (grids and clears sized for 1/16, 1/4 or all of the
  // capacity: a small batch does not pay for the largest one)
  static constexpr int kClasses = 3;
  cudaGraphExec_t exec[3][kClasses] = {};
  int cls = 0;      // the class of the current launch
  int cls_min = 0;  // raised when a launch's tile entries outgrew its class (this batch only)
  bool timing = false;
  bool stage_timing = false;   // per-stage events: the chain runs directly (not from its graph)
  bool stage_events = false;   // set while enqueue() records them
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaEvent_t sev[7] = {};     // stage boundaries: start, projected, depth-sorted, binned, marked, shaded, composited
  // last batch
  uint32_t last_views = 0, last_slots = 0, last_tiles = 0, last_entries = 0;
  std::vector<uint64_t> offsets;
  std::vector<uint32_t> slot_base, tile_base, n_slots, tiles;
  std::vector<uint8_t> shade_blended;  // per view of this batch: shade every blended splat (coverage mode 2)
};

namespace sl {
// Validates a frame for a renderer; lod: the renderer's screen-space LOD (null: frames with LOD on are refused).
int check_frame(const sl_render_frame* f, uint32_t count, uint32_t n_emitters, const sl_lod* lod = nullptr);
void pack_project_params(const sl_render_frame* f, const std::vector<sl_part>& parts, uint32_t count,
                         uint32_t n_emit, uint32_t tile_w, uint32_t tile_h, ProjectParams& P);

// The per-view layout of a batch (validates every frame): slot ranges padded to 256, tile ranges, image offsets
// (floats) into b->slot_base / tile_base / n_slots / tiles / offsets; totals to *slots, *tiles, *pixels.
int batch_layout(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames, uint32_t n_views,
                 uint64_t* slots, uint64_t* tiles, uint64_t* pixels);
// Grows the capacities to hold the layout (buffers reallocated, graphs dropped).
int batch_fit(sl_batch* b, uint64_t slots, uint64_t tiles);
// Starts a new batch of n_views (per-view state that its re-launches keep: the coverage mode of each view).
void batch_begin(sl_batch* b, uint32_t n_views);
// Stages the batch and launches its chain on s (asynchronous).  light_scales may be null (1 for every view).
int batch_launch(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames, const float* eyes,
                 const float* light_scales, uint32_t n_views, float* out_dev, uint64_t slots, uint64_t tiles,
                 cudaStream_t s, bool* replayed);
// After the chain completed: *retry when the tile entries overflowed (capacity grown: launch again), else the
// batch's results are final (stats filled if not null).
int batch_finish(sl_batch* b, uint32_t n_views, uint64_t slots, uint64_t tiles, bool replayed, uint64_t* view_offsets,
                 sl_batch_stats* stats, bool* retry);
}  // namespace sl
