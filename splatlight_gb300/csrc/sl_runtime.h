// Host-side runtime objects behind the C ABI (renderer, device buffers, error reporting).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "sl_internal.h"
#include "sl_bounce.h"
#include "sl_lighting.h"

namespace sl {

// thread-local last error text (sl_last_error)
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// A device buffer that grows on demand (contents are not preserved across growth).
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t b = want + want / 4 + 256;
    cudaError_t e = cudaMalloc(&ptr, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(ptr);
  }
};

// Per-view working buffers of the project -> sort -> bin -> composite chain.
struct ViewBuffers {
  DevBuf key16, recs, rects, order;                            // per slot
  DevBuf bin_scratch;                                          // the one-pass binning's ticket and look-back words
  DevBuf keys_alt, vals_alt, status, tile_ctr;                 // sort scratch (max of slots, entries)
  DevBuf tile_keys, tile_vals;                                 // per entry
  DevBuf ranges;                                               // per tile
  DevBuf digit_hist;                                           // [4][256]: depth-key passes, tile-key passes
  DevBuf key_hist;                                             // counting sort: 65536 key counts, then offsets
  DevBuf scan_scratch;
  DevBuf counters;                                             // FrameCounters
  DevBuf out, counts;                                          // composite targets when the caller's are on the host
  void release_all();
};

struct RenderTimings {
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};

}  // namespace sl

struct sl_renderer {
  int device = 0;
  uint32_t count = 0, part_count = 0, max_emitters = 0, n_emitters = 0;
  sl::DevBuf gaussians, emitters;
  std::vector<sl_part> parts;
  const float4* colour = nullptr;  // bound radiance (float4 per Gaussian)
  const float4* lo_b = nullptr;
  sl_lighting* lighting = nullptr;
  sl_lod* lod = nullptr;  // screen-space LOD of this renderer's scene (capi_lod.cu)
  uint32_t tile_w = 16, tile_h = 16;
  uint32_t sort_mode = 1;  // 1 stable radix sort, 2 counting sort
  float t_stop_scale = 1e-4f;
  uint64_t entry_capacity = 0;
  bool timing = false;
  sl::RenderTimings tm;
  sl::ViewBuffers vb;
  sl::FrameCounters* host_ctr = nullptr;  // pinned
  // last frame (debug read-back)
  uint32_t last_slots = 0, last_w = 0, last_h = 0, last_tiles = 0, last_entries = 0, last_mode = 0;
  bool have_frame = false;
};

// Host state of a screen-space LOD (capi_lod.cu): the tree, its internal nodes as Gaussians, the flags of the cut,
// the nodes' lit colours, and the nodes by depth (each depth: its internal nodes, then its leaves).
struct sl_lod {
  sl_renderer* r = nullptr;
  int device = 0;
  uint32_t N = 0, G = 0, n_int = 0;
  sl::DevBuf nodes, kids, flags, records, colour, level;
  sl::DevBuf tables;                                 // device copy of lvl_off, lvl_all, lvl_int (depth-major rows)
  std::vector<uint32_t> lvl_off, lvl_int, lvl_all;  // per depth: offset into level, internal count, all count
  uint32_t top = 0;                                  // depths [0, top) run in one CTA (kLodTopNodes nodes at most)
};

// Host state of a Lighting object (capi_lighting.cu).
struct sl_lighting {
  sl_renderer* r = nullptr;
  int device = 0;
  uint32_t count = 0, material_count = 0;
  sl::DevBuf nodes, vgrid, materials, parts, tree, lamp_T, env_T, colour;
  sl::DevBuf order;  // shading order (Morton order of the means)
  bool iso_done = false;
  // emitters (src/lighting.js:612-721, EmitParams :657-673)
  std::vector<float> rec;
  uint32_t n_emit = 0, root = 0, one_sided = 0, skip_part = 0xFFFFFFFFu;
  float scale = 1.0f, normal[3] = {0.0f, 0.0f, 1.0f}, edge_soft = 0.2f;
  double root_cov[6] = {0, 0, 0, 0, 0, 0};
  // options
  uint32_t shadow_res = 512, sun_res = 512, mode = 1;
  float theta = 4.0f;
  uint32_t asg = 1;
  // environment (src/environment.js:111-153)
  std::vector<sl_env_light> lights;
  float sky_ambient = 0.0f;
  // light map A
  sl::DevBuf lm_acc, lm_mip;
  sl::LightMapParams LP{};
  bool lm_dirty = true;
  // sun maps
  sl::DevBuf sm_acc, sm_mip, sm_layers, sm_dirty;
  sl::SunParams SP{};
  std::vector<sl::SunLayer> layers;
  std::vector<int> have_center;
  bool sm_dirty_all = true;
  bool lamp_filled = false, env_filled = false;
  // motion blur for the lighting (motion_blur.wgsl, lighting.js:468-507): the opacity-map splats draw these copies
  float blur_shutter = 0.0f, cut_k = 1.0f;
  bool blur_init = false;
  uint32_t blur_prev = 0;  // the parts that moved in the previous update (their copies go back to rest)
  sl::DevBuf g_blur, n_blur;
  // the scene's tree for the motion-blur cut and the probe gather (leaves then internal nodes), every node's parent,
  // the children lists, and per node its depth and part (host)
  uint32_t n_tree = 0, n_kids = 0;
  sl::DevBuf tree_nodes, node_parent, kids;
  std::vector<uint32_t> tree_depth, tree_part;
  // probe bounce (bounce.cu; lighting.js initBounce / encodeBounce): the layout and frame state in BP, the internal
  // nodes by depth for node_up, the sky SH
  bool bounce_on = false, bn_first = true, bn_emit_dark = true;
  uint32_t bn_frame = 0;
  float bn_blend = 1.0f;
  sl::BounceParams BP{};
  std::vector<uint32_t> bn_level_off, bn_level_cnt;
  float sky[48] = {};
  bool has_sky = false;
  sl::DevBuf bn_tab, bn_ground, bn_up, probe_data, probe_sh, xfer, lo_dir, lo_b, node_acc, node_sh, bn_quarters,
      bn_leaf_w, probe_hist;
  uint32_t bn_quarter_off[5] = {};
  // the sender cut (bounce.wgsl sc_select): on/off, re-select on the next frame; every node by depth (sc_level);
  // the internal nodes as Gaussians and their V grids; per node its mark; per internal node the cut's transfer and
  // direct light, shadow T and distant-light T; the cut nodes' list and count
  bool bn_sc = false, bn_sc_stale = true;
  std::vector<uint32_t> sc_level_off, sc_level_cnt;
  sl::DevBuf sc_level, sc_gs, sc_vg, sc_flag, sc_X, sc_T, sc_E, sc_list;
};

namespace sl {
// ShadeParams of a lighting object seen from `eye` (capi_lighting.cu)
void shade_params(const sl_lighting* l, const float* eye, ShadeParams& SH);
// nodeGaussians (capi_lod.cu; src/lod.js:44-107): the internal nodes G..N-1 as Gaussian records, and (vg non-null)
// their V grids, the mass-weighted mean of their children's cells
int node_records(const sl_gaussian* gauss, uint32_t G, const sl_node* nodes, uint32_t N, const uint32_t* kids,
                 uint32_t n_kids, std::vector<sl_gaussian>& out, const sl_vgrid* leaf_vg = nullptr,
                 std::vector<sl_vgrid>* vg = nullptr);
}  // namespace sl
