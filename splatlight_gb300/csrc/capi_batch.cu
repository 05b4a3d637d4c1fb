// Batched rendering over several resident scenes (C ABI): a ragged batch of views, each with its own scene, camera,
// resolution and view mode, goes through one chain of kernels -- batched projection, one segmented depth sort (view id
// above the 16 depth bits), batched tile binning, one two-pass tile sort on the view-local tile id, a coverage pass
// over the lit views' tiles, batched shading of the Gaussians it marked (deferred shading: each view at its own eye),
// one compositor launch over every tile of every view.  Grids are sized for the batch's capacity and every per-batch value
// the kernels read comes from device memory uploaded (from pinned staging) at the head of the chain, so the chain is
// captured once in a CUDA graph and replayed for every batch that fits.  An autotuner picks the tile shape, then the
// block-size variant (blocks per SM its registers are budgeted for) of each of bproject, btile_bin, bshade and
// bcomposite.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "sl_batch.h"


namespace sl {
namespace {

int bits_for(uint64_t v) {
  int b = 1;
  while (b < 32 && (1ull << b) <= v) b++;
  return b;
}

void free_pinned(sl_batch* b) {
  cudaFreeHost(b->h_views);
  cudaFreeHost(b->h_out);
  cudaFreeHost(b->h_block_view);
  cudaFreeHost(b->h_scenes);
  cudaFreeHost(b->h_dyn);
  cudaFreeHost(b->h_ctr);
  cudaFreeHost(b->h_visible);
  cudaFreeHost(b->h_maxrad);
  cudaFreeHost(b->h_tmark);
  b->h_views = nullptr;
  b->h_out = nullptr;
  b->h_block_view = nullptr;
  b->h_scenes = nullptr;
  b->h_dyn = nullptr;
  b->h_ctr = nullptr;
  b->h_visible = nullptr;
  b->h_maxrad = nullptr;
  b->h_tmark = nullptr;
}

void drop_graph(sl_batch* b) {
  for (auto& row : b->exec)
    for (auto& x : row) {
      if (x) cudaGraphExecDestroy(x);
      x = nullptr;
    }
}

// The sizes a launch of capacity class c works with: slots, blocks of 256 slots, tiles, tile entries.
struct ClassCaps {
  uint32_t S, B, T, E;
};
ClassCaps class_caps(const sl_batch* b, int c) {
  static const uint32_t kDiv[sl_batch::kClasses] = {16, 4, 1};
  ClassCaps k;
  k.S = (uint32_t)std::max<uint64_t>(256, ((b->max_slots / kDiv[c]) + 255) & ~255ull);
  k.B = k.S / 256;
  k.T = std::max<uint32_t>(64, b->max_tiles / kDiv[c]);
  k.E = (uint32_t)std::max<uint64_t>(6144, b->entry_cap / kDiv[c]);
  return k;
}

int shape_index(uint32_t tile_w, uint32_t tile_h) {
  if (tile_w == 16 && tile_h == 16) return 0;
  if (tile_w == 8 && tile_h == 32) return 1;
  if (tile_w == 32 && tile_h == 8) return 2;
  return -1;
}

constexpr uint32_t kMaxBatchViews = 256;  // view ids take at most 8 bits above the 16 depth bits (3 sort passes)
constexpr uint64_t kMaxCap = 0x3FFFFFFFull;

// Sizes every buffer for the current capacity (contents not kept); invalidates the graph.
cudaError_t allocate(sl_batch* b) {
  drop_graph(b);
  free_pinned(b);
  const uint64_t S = b->max_slots, E = b->entry_cap;
  const uint32_t T = b->max_tiles, V = b->max_views, B = b->max_blocks;
  cudaError_t e;
#define ENS(buf, bytes) \
  if ((e = (buf).ensure(bytes)) != cudaSuccess) return e
  ENS(b->views, sizeof(BatchView) * V);
  ENS(b->views_out, sizeof(BatchViewOut) * V);
  ENS(b->block_view, 4ull * B + 16);
  ENS(b->scenes_dev, sizeof(BatchScene) * b->scenes.size());
  ENS(b->dyn, sizeof(BatchDyn));
  ENS(b->keys32, 4 * S + 16);
  ENS(b->keys_alt, 4 * S + 16);
  ENS(b->vals_alt, 4 * std::max(S, E) + 16);
  ENS(b->order, 4 * S + 16);
  ENS(b->recs, sizeof(SplatRec) * S);
  ENS(b->rects, 8 * S);
  ENS(b->bin_scratch, btile_bin_scratch_bytes((uint32_t)S));
  ENS(b->tile_keys, 4 * E + 16);
  ENS(b->tile_keys_alt, 4 * E + 16);
  ENS(b->tile_vals, 4 * E + 16);
  ENS(b->tile_vals_alt, 4 * E + 16);
  ENS(b->status, 4ull * 256 * 4 * (sort_tiles_for((uint32_t)std::max(S, E)) + 1));
  ENS(b->tile_ctr, 16);
  ENS(b->hist, 4ull * 6 * 256);
  ENS(b->scan_scratch, std::max(scan_scratch_bytes((uint32_t)S), scan_scratch_bytes(T)));
  ENS(b->ranges, 8ull * T + 16);
  ENS(b->counters, sizeof(FrameCounters));
  ENS(b->view_maxrad, 4ull * V + 16);
  ENS(b->view_visible, 4ull * V + 16);
  ENS(b->block_valid, 4ull * B + 16);
  ENS(b->block_off, 4ull * B + 16);
  ENS(b->marks, S + 16);
  ENS(b->view_tmark, 4ull * V + 16);
  ENS(b->view_shade, 4ull * V + 16);
#undef ENS
  if ((e = cudaMallocHost((void**)&b->h_views, sizeof(BatchView) * V)) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&b->h_out, sizeof(BatchViewOut) * V)) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&b->h_block_view, 4ull * B + 16)) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&b->h_scenes, sizeof(BatchScene) * b->scenes.size())) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&b->h_dyn, sizeof(BatchDyn))) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&b->h_ctr, sizeof(FrameCounters))) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&b->h_visible, 4ull * V + 16)) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&b->h_maxrad, 4ull * V + 16)) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&b->h_tmark, 4ull * V + 16)) != cudaSuccess) return e;
  return cudaSuccess;
}

// The whole chain on stream s for capacity class b->cls, reading every per-batch value from device memory.
cudaError_t enqueue(sl_batch* b, cudaStream_t s) {
  cudaError_t e;
#define CK(x) \
  if ((e = (x)) != cudaSuccess) return e
  const ClassCaps k = class_caps(b, b->cls);
  const uint32_t V = b->max_views, B = k.B, T = k.T, S = k.S, E = k.E;
  CK(cudaMemcpyAsync(b->views.ptr, b->h_views, sizeof(BatchView) * V, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b->views_out.ptr, b->h_out, sizeof(BatchViewOut) * V, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b->block_view.ptr, b->h_block_view, 4ull * B, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b->scenes_dev.ptr, b->h_scenes, sizeof(BatchScene) * b->scenes.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b->dyn.ptr, b->h_dyn, sizeof(BatchDyn), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(b->counters.ptr, 0, sizeof(FrameCounters), s));
  CK(cudaMemsetAsync(b->hist.ptr, 0, 4ull * 6 * 256, s));
  CK(cudaMemsetAsync(b->view_maxrad.ptr, 0, 4ull * V, s));
  CK(cudaMemsetAsync(b->view_visible.ptr, 0, 4ull * V, s));
  CK(cudaMemsetAsync(b->ranges.ptr, 0, 8ull * T, s));
  CK(cudaMemsetAsync(b->marks.ptr, 0, S, s));
  FrameCounters* ctr = b->counters.as<FrameCounters>();
  const uint32_t* totals = b->dyn.as<uint32_t>();  // BatchDyn words: total slots, total tiles, ...
  uint32_t* hist = b->hist.as<uint32_t>();
  // stage boundaries for the per-stage timing (never while the chain is being captured)
  auto stage = [&](int k) { return b->stage_events ? cudaEventRecord(b->sev[k], s) : cudaSuccess; };
  CK(stage(0));
  CK(launch_bproject(b->views.as<BatchView>(), b->block_view.as<uint32_t>(), B, b->keys32.as<uint32_t>(),
                     b->recs.as<SplatRec>(), b->rects.as<ushort4>(), hist, b->view_maxrad.as<uint32_t>(),
                     b->view_visible.as<uint32_t>(), b->block_valid.as<uint32_t>(), b->variant[0], s));
  // the depth sort runs over the visible slots only: their keys compacted in slot order (stability kept), the count
  // in ctr->visible (read on the device by the sort and the binning)
  CK(exclusive_scan_u32(b->block_valid.as<uint32_t>(), b->block_off.as<uint32_t>(), B, &ctr->visible,
                        b->scan_scratch.ptr, ctr, s));
  CK(launch_bcompact(b->block_view.as<uint32_t>(), b->keys32.as<uint32_t>(), b->block_off.as<uint32_t>(), B,
                     b->tile_keys.as<uint32_t>(), b->tile_vals.as<uint32_t>(), s));
  CK(stage(1));
  const uint32_t* n_visible = &ctr->visible;
  const uint32_t max_tiles_sort = (uint32_t)(b->status.bytes / (4ull * 256 * 4));
  CK(sort32_pairs(b->tile_keys.as<uint32_t>(), b->keys_alt.as<uint32_t>(), b->tile_vals.as<uint32_t>(),
                  b->order.as<uint32_t>(), b->vals_alt.as<uint32_t>(), S, n_visible, 16 + bits_for(V - 1), hist,
                  b->status.as<uint32_t>(), b->tile_ctr.as<uint32_t>(), max_tiles_sort, ctr, s));
  CK(stage(2));
  CK(launch_btile_bin(b->order.as<uint32_t>(), b->rects.as<ushort4>(), b->recs.as<SplatRec>(), b->views.as<BatchView>(),
                      b->block_view.as<uint32_t>(), n_visible, S, b->tile_w, b->tile_h, E, ctr,
                      b->tile_keys.as<uint32_t>(), b->tile_vals.as<uint32_t>(), hist + 768, b->bin_scratch.ptr,
                      b->variant[1], s));
  // the tile sort: stable on the 16-bit view-local tile id (two passes); entries arrive in (view, depth) order, so
  // each (view, tile) run comes out contiguous and depth-ordered
  CK(sort32_pairs(b->tile_keys.as<uint32_t>(), b->tile_keys_alt.as<uint32_t>(), b->tile_vals.as<uint32_t>(),
                  b->tile_vals.as<uint32_t>(), b->tile_vals_alt.as<uint32_t>(), E, &ctr->entries, 16, hist + 768,
                  b->status.as<uint32_t>(), b->tile_ctr.as<uint32_t>(), max_tiles_sort, ctr, s,
                  b->tile_keys.as<uint32_t>()));
  CK(launch_btile_runs(b->tile_keys.as<uint32_t>(), &ctr->entries, E, b->views_out.as<BatchViewOut>(),
                       b->ranges.as<uint2>(), s));
  CK(stage(3));
  // deferred shading: the coverage pass marks the splats of lit views that blend a fragment, the shading list is
  // their Gaussians in shading order, and only those are shaded before the composite
  const BatchComposite C{b->tile_w, b->tile_h, b->t_stop_scale, 0};
  CK(launch_bmark(C, b->ranges.as<uint2>(), b->tile_vals.as<uint32_t>(), b->recs.as<SplatRec>(),
                  b->views_out.as<BatchViewOut>(), b->view_maxrad.as<uint32_t>(), b->dyn.as<BatchDyn>(), T, ctr,
                  b->marks.as<uint8_t>(), b->view_tmark.as<float>(), s));
  CK(stage(4));
  CK(launch_bshade_list(b->views.as<BatchView>(), b->scenes_dev.as<BatchScene>(), b->block_view.as<uint32_t>(),
                        b->marks.as<uint8_t>(), totals, B, V, ctr, b->vals_alt.as<uint32_t>(),
                        b->view_shade.as<uint32_t>(), s));
  CK(launch_bshade(b->views.as<BatchView>(), b->scenes_dev.as<BatchScene>(), b->block_view.as<uint32_t>(), B,
                   b->vals_alt.as<uint32_t>(), b->view_shade.as<uint32_t>(), b->recs.as<SplatRec>(),
                   b->view_maxrad.as<uint32_t>(), b->variant[2], s));
  CK(stage(5));
  CK(launch_bcomposite(C, b->ranges.as<uint2>(), b->tile_vals.as<uint32_t>(), b->recs.as<SplatRec>(),
                       b->views_out.as<BatchViewOut>(), b->view_maxrad.as<uint32_t>(), b->dyn.as<BatchDyn>(), T, ctr,
                       b->marks.as<uint8_t>(), b->variant[3], s));
  CK(stage(6));
  CK(cudaMemcpyAsync(b->h_ctr, ctr, sizeof(FrameCounters), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(b->h_visible, b->view_visible.ptr, 4ull * V, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(b->h_maxrad, b->view_maxrad.ptr, 4ull * V, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(b->h_tmark, b->view_tmark.ptr, 4ull * V, cudaMemcpyDeviceToHost, s));
#undef CK
  return cudaSuccess;
}

}  // namespace
}  // namespace sl

using namespace sl;

namespace {

bool valid_shape(uint32_t w, uint32_t h) { return shape_index(w, h) >= 0; }

int view_fail(uint32_t v, int rc) {
  char buf[512];
  sl_last_error(buf, sizeof buf);
  return fail(rc, "view " + std::to_string(v) + ": " + buf);
}

// Grows the capacities to hold `slots` padded slots and `tiles` tiles (25% headroom); reallocates when they grew.
int fit_capacity(sl_batch* b, uint64_t slots, uint64_t tiles) {
  if (slots <= b->max_slots && tiles <= b->max_tiles) return SL_OK;
  uint64_t ns = std::max<uint64_t>(b->max_slots, (slots + slots / 4 + 255) & ~255ull);
  uint64_t nt = std::max<uint64_t>(b->max_tiles, tiles + tiles / 4 + 64);
  if (ns > kMaxCap || nt > (1ull << 24)) return fail(SL_ERR_INVALID_ARG, "batch too large (2^30 slots or 2^24 tiles)");
  b->max_slots = ns;
  b->max_blocks = (uint32_t)(ns / 256);
  b->max_tiles = (uint32_t)nt;
  b->entry_cap = std::min<uint64_t>(std::max<uint64_t>(b->entry_cap, 2 * ns), kMaxCap);
  cudaError_t e = allocate(b);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? fail(SL_ERR_OOM, "batch buffers") : cuda_fail(e, "batch buffers");
  return SL_OK;
}

// Fills the pinned staging for this batch (views, outputs, block map, scenes, totals).
void stage(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames, const float* eyes,
           const float* light_scales, uint32_t n_views, float* out_dev, uint64_t slot, uint64_t tile) {
  for (uint32_t v = 0; v < n_views; v++) {
    sl_renderer* r = b->scenes[scene_of_view[v]];
    BatchView& V = b->h_views[v];
    memset(&V, 0, sizeof(V));
    pack_project_params(&frames[v], r->parts, r->count, (uint32_t)frames[v].palette[3][1], b->tile_w, b->tile_h, V.P);
    V.gaussians = r->gaussians.as<float4>();
    V.emitters = r->emitters.as<float4>();
    if (!b->lights[scene_of_view[v]]) {  // a scene without lighting draws its bound radiance, as sl_render does
      V.colour = r->colour;
      V.lo_b = r->lo_b;
    }
    V.scene = scene_of_view[v];
    V.slot_base = b->slot_base[v];
    V.block_first = b->slot_base[v] / 256;
    V.tile_base = b->tile_base[v];
    V.tiles_x = V.P.tiles_x;
    for (int c = 0; c < 3; c++) V.eye[c] = eyes[3 * v + c];
    V.light_scale = light_scales ? light_scales[v] : 1.0f;
    BatchViewOut& O = b->h_out[v];
    O.tile_base = b->tile_base[v];
    O.tiles_x = V.P.tiles_x;
    O.width = (uint32_t)frames[v].viewport[0];
    O.height = (uint32_t)frames[v].viewport[1];
    O.count_mode = frames[v].view_mode == 2u ? 1u : 0u;
    const sl_lighting* l = b->lights[scene_of_view[v]];
    O.lit = (frames[v].view_mode == 3u && l && l->iso_done) ? (b->shade_blended[v] ? 2u : 1u) : 0u;
    O.rad_cap = b->rad_allow * std::max(1.0f, V.light_scale);
    O.pad = 0;
    O.out_offset = b->offsets[v] / 4;
  }
  for (uint32_t v = n_views; v < b->max_views; v++) {  // unused view rows: past every tile
    memset(&b->h_views[v], 0, sizeof(BatchView));
    memset(&b->h_out[v], 0, sizeof(BatchViewOut));
    b->h_out[v].tile_base = 0xFFFFFFFFu;
  }
  const uint32_t used = (uint32_t)(slot / 256);
  for (uint32_t v = 0; v < n_views; v++) {
    const uint32_t first = b->slot_base[v] / 256, nb = (b->n_slots[v] + 255) / 256;
    for (uint32_t k = 0; k < nb; k++) b->h_block_view[first + k] = v;
  }
  const uint32_t nb = class_caps(b, b->cls).B;
  for (uint32_t blk = used; blk < nb; blk++) b->h_block_view[blk] = kNoView;
  for (size_t k = 0; k < b->scenes.size(); k++) {
    BatchScene& S = b->h_scenes[k];
    memset(&S, 0, sizeof(S));
    sl_lighting* l = b->lights[k];
    if (l) {
      S.nodes = l->nodes.as<sl_node>();
      S.vgrid = l->vgrid.as<sl_vgrid>();
      S.parts = l->parts.as<sl_part>();
      S.mats = l->materials.as<sl_material>();
      S.tree = l->tree.as<float>();
      S.lamp_T = l->lamp_T.as<float>();
      S.env_T = l->env_T.as<float4>();
      S.order = l->order.as<uint32_t>();
      shade_params(l, nullptr, S.SH);
      S.lit = l->iso_done ? 1u : 0u;  // maps exist after the lighting's first update
    }
  }
  b->h_dyn->total_slots = (uint32_t)slot;
  b->h_dyn->total_tiles = (uint32_t)tile;
  b->h_dyn->n_views = n_views;
  b->h_dyn->total_blocks = used;
  b->h_dyn->out = reinterpret_cast<float4*>(out_dev);
}

// Runs the chain once on s (replaying the tile shape's graph, capturing it first if needed).
int launch_chain(sl_batch* b, cudaStream_t s, bool* replayed) {
  cudaError_t e;
  *replayed = false;
  if (b->use_graph) {
    cudaGraphExec_t& exec = b->exec[shape_index(b->tile_w, b->tile_h)][b->cls];
    if (!exec) {
      cudaGraph_t g = nullptr;
      e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t e1 = enqueue(b, b->cap_stream);
        e = cudaStreamEndCapture(b->cap_stream, &g);
        if (e1 != cudaSuccess) e = e1;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        exec = nullptr;
        return cuda_fail(e, "capturing the batch graph");
      }
    } else {
      *replayed = true;
    }
    e = cudaGraphLaunch(exec, s);
  } else {
    e = enqueue(b, s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "batch launch");
  return SL_OK;
}

}  // namespace

namespace sl {

int batch_layout(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames, uint32_t n_views,
                 uint64_t* slots, uint64_t* tiles, uint64_t* pixels) {
  b->slot_base.assign(n_views, 0);
  b->tile_base.assign(n_views, 0);
  b->n_slots.assign(n_views, 0);
  b->tiles.assign(n_views, 0);
  b->offsets.assign(n_views, 0);
  if (b->shade_blended.size() != n_views) b->shade_blended.assign(n_views, 0);
  uint64_t slot = 0, tile = 0, pix = 0;
  for (uint32_t v = 0; v < n_views; v++) {
    const uint32_t k = scene_of_view[v];
    if (k >= b->scenes.size()) return fail(SL_ERR_INVALID_ARG, "view " + std::to_string(v) + ": bad scene index");
    sl_renderer* r = b->scenes[k];
    int rc = check_frame(&frames[v], r->count, r->n_emitters);
    if (rc) return view_fail(v, rc);
    const uint32_t W = (uint32_t)frames[v].viewport[0], H = (uint32_t)frames[v].viewport[1];
    const uint32_t n = r->count + 1u + (uint32_t)frames[v].palette[3][1];
    const uint32_t tx = (W + b->tile_w - 1) / b->tile_w, ty = (H + b->tile_h - 1) / b->tile_h;
    if ((uint64_t)tx * ty > 65536u)  // tile keys hold the view-local tile id in 16 bits
      return fail(SL_ERR_INVALID_ARG, "view " + std::to_string(v) + ": more than 65536 tiles");
    b->slot_base[v] = (uint32_t)slot;
    b->n_slots[v] = n;
    b->tile_base[v] = (uint32_t)tile;
    b->tiles[v] = tx * ty;
    b->offsets[v] = 4 * pix;
    slot += ((uint64_t)n + 255) & ~255ull;
    tile += (uint64_t)tx * ty;
    pix += (uint64_t)W * H;
    if (slot > kMaxCap) return fail(SL_ERR_INVALID_ARG, "batch too large (2^30 slots)");
  }
  *slots = slot;
  *tiles = tile;
  *pixels = pix;
  return SL_OK;
}

int batch_fit(sl_batch* b, uint64_t slots, uint64_t tiles) { return fit_capacity(b, slots, tiles); }

void batch_begin(sl_batch* b, uint32_t n_views) {
  b->shade_blended.assign(n_views, 0);
  b->cls_min = 0;
}

int batch_launch(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames, const float* eyes,
                 const float* light_scales, uint32_t n_views, float* out_dev, uint64_t slots, uint64_t tiles,
                 cudaStream_t s, bool* replayed) {
  // the smallest capacity class that holds the batch's slots and tiles and the entries it is expected to have (and,
  // after an overflow, its entries)
  b->cls = sl_batch::kClasses - 1;
  const double est_entries = (double)slots * (double)b->entry_ratio;
  for (int c = b->cls_min; c < sl_batch::kClasses; c++) {
    const ClassCaps k = class_caps(b, c);
    if (slots <= k.S && tiles <= k.T && est_entries <= (double)k.E) {
      b->cls = c;
      break;
    }
  }
  stage(b, scene_of_view, frames, eyes, light_scales, n_views, out_dev, slots, tiles);
  cudaError_t e;
  if (b->timing && (e = cudaEventRecord(b->ev[0], s)) != cudaSuccess) return cuda_fail(e, "timing");
  int rc = SL_OK;
  if (b->stage_timing) {  // per-stage events between the kernels: the same chain, launched directly
    b->stage_events = true;
    cudaError_t e2 = enqueue(b, s);
    b->stage_events = false;
    *replayed = false;
    if (e2 != cudaSuccess) return cuda_fail(e2, "batch launch");
  } else {
    rc = launch_chain(b, s, replayed);
  }
  if (rc) return rc;
  if (b->timing && (e = cudaEventRecord(b->ev[1], s)) != cudaSuccess) return cuda_fail(e, "timing");
  return SL_OK;
}

int batch_finish(sl_batch* b, uint32_t n_views, uint64_t slots, uint64_t tiles, bool replayed, uint64_t* view_offsets,
                 sl_batch_stats* stats, bool* retry) {
  *retry = false;
  const FrameCounters& hc = *b->h_ctr;
  if (slots) b->entry_ratio = std::max(b->entry_ratio, (float)((double)hc.entries / (double)slots));
  if (hc.overflow || hc.entries > class_caps(b, b->cls).E) {  // the caller launches again
    // a larger class whose entries hold them, else grow the tile-entry capacity
    for (int c = b->cls + 1; c < sl_batch::kClasses; c++)
      if (hc.entries <= class_caps(b, c).E) {
        b->cls_min = c;
        *retry = true;
        return SL_OK;
      }
    const uint64_t want = (uint64_t)hc.entries + hc.entries / 4 + 4096;
    if (b->entry_cap >= kMaxCap || hc.entries >= kMaxCap) return fail(SL_ERR_OVERFLOW, "tile entries beyond 2^30");
    b->entry_cap = std::min<uint64_t>(std::max<uint64_t>(want, 2 * b->entry_cap), kMaxCap);
    cudaError_t e = allocate(b);
    if (e != cudaSuccess) return cuda_fail(e, "growing the tile entries");
    b->cls_min = sl_batch::kClasses - 1;  // the grown capacity holds them
    *retry = true;
    return SL_OK;
  }
  // A lit view whose composite threshold (t_stop / its radiance bound after shading) fell below twice its coverage
  // threshold may have composited past the marked splats: it runs again with every blended splat shaded (mode 2).
  // The decision and its result depend on the view alone, not on the rest of the batch.
  bool again = false;
  for (uint32_t v = 0; v < n_views; v++) {
    if (b->h_out[v].lit != 1u) continue;
    const float t_stop = b->t_stop_scale / std::max(__builtin_bit_cast(float, b->h_maxrad[v]), 1.0f);
    if (t_stop < 2.0f * b->h_tmark[v]) {
      b->shade_blended[v] = 1;
      again = true;
    }
  }
  if (again) {
    *retry = true;
    return SL_OK;
  }
  b->last_views = n_views;
  b->last_slots = (uint32_t)slots;
  b->last_tiles = (uint32_t)tiles;
  b->last_entries = hc.entries;
  if (view_offsets)
    for (uint32_t v = 0; v < n_views; v++) view_offsets[v] = b->offsets[v];
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->views = n_views;
    stats->slots = (uint32_t)slots;
    stats->tiles = (uint32_t)tiles;
    stats->entries = hc.entries;
    stats->fragments = hc.fragments;
    uint64_t vis = 0;
    for (uint32_t v = 0; v < n_views; v++) vis += b->h_visible[v];
    stats->visible = vis;
    stats->graph_replayed = replayed ? 1u : 0u;
    stats->shaded = hc.shade_n;
    for (uint32_t v = 0; v < n_views; v++) {
      stats->reshaded_views += b->shade_blended[v];
      stats->max_radiance = std::max(stats->max_radiance, __builtin_bit_cast(float, b->h_maxrad[v]));
    }
    if (b->timing) cudaEventElapsedTime(&stats->ms_total, b->ev[0], b->ev[1]);
    if (b->stage_timing)
      for (int k = 0; k < 6; k++) cudaEventElapsedTime(&stats->ms_stage[k], b->sev[k], b->sev[k + 1]);
  }
  if (hc.timeout) return fail(SL_ERR_TIMEOUT, "a bounded device-side wait gave up");
  return SL_OK;
}

}  // namespace sl

extern "C" {

int sl_batch_create(sl_renderer* const* renderers, sl_lighting* const* lightings, uint32_t n_scenes,
                    const sl_batch_options* opt, sl_batch** out) {
  if (!out) return fail(SL_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  if (!renderers || n_scenes == 0 || n_scenes > 4096) return fail(SL_ERR_INVALID_ARG, "bad scene list");
  for (uint32_t k = 0; k < n_scenes; k++) {
    if (!renderers[k]) return fail(SL_ERR_INVALID_ARG, "null renderer");
    if (renderers[k]->device != renderers[0]->device) return fail(SL_ERR_INVALID_ARG, "renderers on different devices");
    if (lightings && lightings[k] && lightings[k]->r != renderers[k])
      return fail(SL_ERR_INVALID_ARG, "lighting " + std::to_string(k) + " belongs to another renderer");
  }
  const uint32_t mv = opt && opt->max_views ? opt->max_views : 64;
  if (mv > kMaxBatchViews) return fail(SL_ERR_INVALID_ARG, "at most 256 views per batch");
  uint32_t tw = 16, th = 16;
  if (opt && (opt->tile_w || opt->tile_h)) {
    if (!valid_shape(opt->tile_w, opt->tile_h)) return fail(SL_ERR_INVALID_ARG, "tile shape must be 16x16, 8x32 or 32x8");
    tw = opt->tile_w;
    th = opt->tile_h;
  }
  const uint64_t ms = opt && opt->max_slots ? ((opt->max_slots + 255) & ~255ull) : (1ull << 20);
  const uint64_t mt = opt && opt->max_tiles ? opt->max_tiles : 8192;
  const uint64_t me = opt && opt->max_entries ? opt->max_entries : 2 * ms;
  if (ms > kMaxCap || me > kMaxCap || mt > (1ull << 24))
    return fail(SL_ERR_INVALID_ARG, "capacities: slots and entries below 2^30, tiles at most 2^24");
  sl_batch* b = new sl_batch();
  b->device = renderers[0]->device;
  cudaSetDevice(b->device);
  b->scenes.assign(renderers, renderers + n_scenes);
  b->lights.assign(n_scenes, nullptr);
  if (lightings)
    for (uint32_t k = 0; k < n_scenes; k++) b->lights[k] = lightings[k];
  b->max_views = mv;
  b->max_slots = ms;
  b->max_blocks = (uint32_t)(ms / 256);
  b->max_tiles = (uint32_t)mt;
  b->entry_cap = me;
  b->tile_w = tw;
  b->tile_h = th;
  b->use_graph = !(opt && opt->no_graph);
  if (opt && opt->radiance_allowance > 0.0f) b->rad_allow = opt->radiance_allowance;
  cudaError_t e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev[1]);
  for (auto& ev : b->sev)
    if (e == cudaSuccess) e = cudaEventCreate(&ev);
  if (e == cudaSuccess) e = allocate(b);
  if (e != cudaSuccess) {
    sl_batch_destroy(b);
    return e == cudaErrorMemoryAllocation ? fail(SL_ERR_OOM, "batch buffers") : cuda_fail(e, "sl_batch_create");
  }
  *out = b;
  return SL_OK;
}

int sl_batch_destroy(sl_batch* b) {
  if (!b) return SL_OK;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  drop_graph(b);
  free_pinned(b);
  sl::DevBuf* all[] = {&b->views, &b->views_out, &b->block_view, &b->scenes_dev, &b->dyn, &b->keys32, &b->keys_alt,
                       &b->vals_alt, &b->order, &b->recs, &b->rects,
                       &b->tile_keys, &b->tile_keys_alt, &b->tile_vals, &b->tile_vals_alt, &b->status, &b->tile_ctr,
                       &b->hist, &b->scan_scratch, &b->bin_scratch, &b->block_valid, &b->block_off,
                       &b->ranges, &b->counters, &b->view_maxrad, &b->view_visible, &b->marks,
                       &b->view_tmark, &b->view_shade};
  for (sl::DevBuf* x : all) x->release();
  for (auto& ev : b->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : b->sev)
    if (ev) cudaEventDestroy(ev);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  delete b;
  return SL_OK;
}

int sl_batch_set_tile(sl_batch* b, uint32_t tile_w, uint32_t tile_h) {
  if (!b) return fail(SL_ERR_INVALID_ARG, "null batch");
  if (!valid_shape(tile_w, tile_h)) return fail(SL_ERR_INVALID_ARG, "tile shape must be 16x16, 8x32 or 32x8");
  b->tile_w = tile_w;
  b->tile_h = tile_h;
  return SL_OK;
}

int sl_batch_set_timing(sl_batch* b, int enabled) {
  if (!b) return fail(SL_ERR_INVALID_ARG, "null batch");
  if (enabled < 0 || enabled > 2) return fail(SL_ERR_INVALID_ARG, "timing: 0 off, 1 total, 2 per stage");
  b->timing = enabled != 0;
  b->stage_timing = enabled == 2;
  return SL_OK;
}

int sl_batch_render(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames, const float* eyes,
                    const float* light_scales, uint32_t n_views, float* out_dev, uint64_t out_floats,
                    uint64_t* view_offsets, sl_batch_stats* stats, void* stream) {
  if (!b || !scene_of_view || !frames || !eyes || !out_dev || n_views == 0) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n_views > b->max_views) return fail(SL_ERR_INVALID_ARG, "more views than the batch's max_views");
  if (reinterpret_cast<uintptr_t>(out_dev) % 16) return fail(SL_ERR_INVALID_ARG, "out_dev must be 16-byte aligned");
  cudaSetDevice(b->device);
  {
    // page-locked host memory: the compositor writes the images in place over the host link (no staging copy)
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, out_dev) == cudaSuccess && pa.type == cudaMemoryTypeHost) {
      if (!pa.devicePointer || reinterpret_cast<uintptr_t>(pa.devicePointer) % 16)
        return fail(SL_ERR_INVALID_ARG, "out_dev: host memory the device cannot write");
      out_dev = static_cast<float*>(pa.devicePointer);
    } else if (pa.type == cudaMemoryTypeUnregistered) {
      cudaGetLastError();
      return fail(SL_ERR_INVALID_ARG, "out_dev: pageable host memory (pass device or page-locked host memory)");
    }
    cudaGetLastError();
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  uint64_t slot = 0, tile = 0, pix = 0;
  int rc = batch_layout(b, scene_of_view, frames, n_views, &slot, &tile, &pix);
  if (rc) return rc;
  if (4 * pix > out_floats) return fail(SL_ERR_INVALID_ARG, "output buffer too small for the batch's images");
  rc = batch_fit(b, slot, tile);
  if (rc) return rc;
  batch_begin(b, n_views);
  for (int attempt = 0; attempt < 3; attempt++) {
    bool replayed = false, retry = false;
    rc = batch_launch(b, scene_of_view, frames, eyes, light_scales, n_views, out_dev, slot, tile, s, &replayed);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "batch");
    rc = batch_finish(b, n_views, slot, tile, replayed, view_offsets, stats, &retry);
    if (rc || !retry) return rc;
  }
  return fail(SL_ERR_OVERFLOW, "tile entry capacity kept overflowing");
}

int sl_batch_autotune(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames, const float* eyes,
                      const float* light_scales, uint32_t n_views, float* out_dev, uint64_t out_floats,
                      uint32_t reps, uint32_t* tile_w, uint32_t* tile_h, float* ms_out, void* stream) {
  if (!b) return fail(SL_ERR_INVALID_ARG, "null batch");
  static const uint32_t kShapes[3][2] = {{16, 16}, {8, 32}, {32, 8}};
  if (reps == 0) reps = 3;
  const bool timing = b->timing;
  const uint32_t tw0 = b->tile_w, th0 = b->tile_h;
  b->timing = true;
  float best = 0.0f;
  int best_k = -1;
  for (int k = 0; k < 3; k++) {
    b->tile_w = kShapes[k][0];
    b->tile_h = kShapes[k][1];
    sl_batch_stats st;
    int rc = sl_batch_render(b, scene_of_view, frames, eyes, light_scales, n_views, out_dev, out_floats, nullptr, &st,
                             stream);
    float sum = 0.0f;
    for (uint32_t r = 0; rc == SL_OK && r < reps; r++) {
      rc = sl_batch_render(b, scene_of_view, frames, eyes, light_scales, n_views, out_dev, out_floats, nullptr, &st,
                           stream);
      sum += st.ms_total;
    }
    if (rc) {
      b->timing = timing;
      b->tile_w = tw0;
      b->tile_h = th0;
      return rc;
    }
    const float ms = sum / (float)reps;
    if (ms_out) ms_out[k] = ms;
    if (best_k < 0 || ms < best) {
      best = ms;
      best_k = k;
    }
  }
  b->tile_w = kShapes[best_k][0];
  b->tile_h = kShapes[best_k][1];
  // then each tunable kernel's block-size variant, one kernel at a time, by the device time of its stage
  static const int kStageOf[kTuneKernels] = {0, 2, 4, 5};  // sl_batch_stats.ms_stage: project, bin, shade, composite
  const bool stage_timing = b->stage_timing;
  b->stage_timing = true;
  int rc = SL_OK;
  for (int k = 0; k < kTuneKernels && rc == SL_OK; k++) {
    int best_v = b->variant[k];
    float best_ms = 0.0f;
    for (int v = 0; v < kTuneVariants[k] && rc == SL_OK; v++) {
      b->variant[k] = v;
      drop_graph(b);
      sl_batch_stats st;
      rc = sl_batch_render(b, scene_of_view, frames, eyes, light_scales, n_views, out_dev, out_floats, nullptr, &st,
                           stream);
      float sum = 0.0f;
      for (uint32_t r = 0; rc == SL_OK && r < reps; r++) {
        rc = sl_batch_render(b, scene_of_view, frames, eyes, light_scales, n_views, out_dev, out_floats, nullptr,
                             &st, stream);
        sum += st.ms_stage[kStageOf[k]];
      }
      if (rc == SL_OK && (v == 0 || sum < best_ms)) {
        best_ms = sum;
        best_v = v;
      }
    }
    b->variant[k] = best_v;
  }
  drop_graph(b);
  b->stage_timing = stage_timing;
  b->timing = timing;
  if (rc) return rc;
  if (tile_w) *tile_w = b->tile_w;
  if (tile_h) *tile_h = b->tile_h;
  return SL_OK;
}

int sl_batch_set_tuning(sl_batch* b, const uint32_t* min_blocks) {
  if (!b || !min_blocks) return fail(SL_ERR_INVALID_ARG, "null argument");
  int v[kTuneKernels];
  for (int k = 0; k < kTuneKernels; k++) {
    v[k] = -1;
    for (int j = 0; j < kTuneVariants[k]; j++)
      if ((uint32_t)kTuneMinBlocks[k][j] == min_blocks[k]) v[k] = j;
    if (v[k] < 0) return fail(SL_ERR_INVALID_ARG, "no such block-size variant");
  }
  for (int k = 0; k < kTuneKernels; k++) b->variant[k] = v[k];
  drop_graph(b);
  return SL_OK;
}

int sl_batch_get_tuning(sl_batch* b, uint32_t* tile_w, uint32_t* tile_h, uint32_t* min_blocks) {
  if (!b) return fail(SL_ERR_INVALID_ARG, "null batch");
  if (tile_w) *tile_w = b->tile_w;
  if (tile_h) *tile_h = b->tile_h;
  if (min_blocks)
    for (int k = 0; k < kTuneKernels; k++) min_blocks[k] = (uint32_t)kTuneMinBlocks[k][b->variant[k]];
  return SL_OK;
}

int sl_batch_read_view(sl_batch* b, uint32_t view, uint32_t* order, uint32_t* ranges, uint32_t* entries,
                       uint64_t entries_cap, uint64_t* n_entries) {
  if (!b) return fail(SL_ERR_INVALID_ARG, "null batch");
  if (view >= b->last_views) return fail(SL_ERR_INVALID_ARG, "no such view in the last batch");
  cudaSetDevice(b->device);
  const uint32_t sb = b->slot_base[view], n = b->n_slots[view], tb = b->tile_base[view], nt = b->tiles[view];
  std::vector<uint2> rg(nt);
  cudaError_t e = cudaMemcpy(rg.data(), b->ranges.as<uint2>() + tb, 8ull * nt, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "ranges");
  // each tile's run is contiguous, the view's runs are spread over the batch's entries ((local tile, view) order):
  // gathered here in tile order, the ranges rebased to that list
  uint64_t total = 0;
  uint32_t lo = UINT32_MAX, hi = 0;
  for (uint32_t t = 0; t < nt; t++) {
    total += rg[t].y - rg[t].x;
    if (rg[t].y > rg[t].x) {
      lo = std::min(lo, rg[t].x);
      hi = std::max(hi, rg[t].y);
    }
  }
  if (order) {
    // the depth sort ran over the visible slots only (views in order): this view's are at the sum of the earlier
    // views' visible counts; its culled slots follow in index order, as the per-view stable sort places them
    uint64_t pos = 0;
    for (uint32_t v = 0; v < view; v++) pos += b->h_visible[v];
    const uint32_t vis = b->h_visible[view];
    if (vis > n) return fail(SL_ERR_INVALID_ARG, "inconsistent visible count");
    e = cudaMemcpy(order, b->order.as<uint32_t>() + pos, 4ull * vis, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "order");
    for (uint32_t i = 0; i < vis; i++) order[i] -= sb;
    std::vector<uint32_t> keys(n);
    e = cudaMemcpy(keys.data(), b->keys32.as<uint32_t>() + sb, 4ull * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "keys");
    uint32_t at = vis;
    for (uint32_t i = 0; i < n && at < n; i++)
      if ((keys[i] & 0xFFFFu) == 0xFFFFu) order[at++] = i;
  }
  if (ranges) {
    uint32_t at = 0;
    for (uint32_t t = 0; t < nt; t++) {
      ranges[2 * t] = at;
      at += rg[t].y - rg[t].x;
      ranges[2 * t + 1] = at;
    }
  }
  if (n_entries) *n_entries = total;
  if (entries && total) {
    if (entries_cap < total) return fail(SL_ERR_INVALID_ARG, "entries buffer too small");
    std::vector<uint32_t> span(hi - lo);
    e = cudaMemcpy(span.data(), b->tile_vals.as<uint32_t>() + lo, 4ull * (hi - lo), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "entries");
    uint64_t at = 0;
    for (uint32_t t = 0; t < nt; t++)
      for (uint32_t i = rg[t].x; i < rg[t].y; i++) entries[at++] = span[i - lo] - sb;
  }
  return SL_OK;
}

}  // extern "C"
