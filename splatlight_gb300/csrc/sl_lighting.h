// Internal declarations of the lighting kernels and their parameter blocks.
#pragma once

#include <vector>

#include "sl_internal.h"

namespace sl {

// light map A frame and layout (light_shadow.wgsl:26-38 LSParams, the fields map A reads)
struct LightMapParams {
  float center[3], normal[3], t1[3], t2[3];
  float sigma_l;
  uint32_t hemi, res, levels, layer_texels, part_count, skip_part, dirty;
  uint32_t level_off[16];
};

// The motion-blur cut of the opacity-map splats (light_shadow.wgsl:158-210, sun_map.wgsl:119-153): a moving part
// splats the nodes of its tree about k x its smear across (radius <= k |d| < the parent's), each keeping its rest
// coverage; still parts splat their leaves.  k = 0 (or no tree): leaves only, as stretched by blur_records.
struct BlurCut {
  const sl_gaussian* g_rest;  // the rest records (receivers' shapes, the cut's coverage reference)
  const sl_node* n_rest;      // n_nodes rest nodes: the leaves, then the tree's internal nodes
  const uint32_t* parent;     // n_nodes parents (0xFFFFFFFF for roots)
  uint32_t n_nodes;
  float k, shutter;
};

struct EnvLightDev {
  float dir[3];
  float std;
  float irr[3];
  uint32_t shadows;
};

// sun_map.wgsl:24-35 SunParams (what the kernels read) + the layer ranges per part
struct SunParams {
  uint32_t n_layers, res, levels, layer_texels, n_parts;
  uint32_t level_off[16];
  uint32_t part_first[32], part_layers[32];
  EnvLightDev lights[4];
};

// one sun-map layer (sun_map.wgsl:32 SunLayer + the plan's kind and dirty flag)
struct SunLayer {
  float c[2];
  float half, zref;
  float t1[3], t2[3];
  uint32_t part, light, kind, dirty;
};

struct ShadeParams {
  float eye[3];
  uint32_t n_emit, root, mode, asg, one_sided, material_count, n_lights;
  float scale, theta, edge_soft, sky_ambient;
  float normal[3];
  EnvLightDev lights[4];
};

// One scene's lighting as the batched shading pass reads it.
struct BatchScene {
  const sl_node* nodes;
  const sl_vgrid* vgrid;
  const sl_part* parts;
  const sl_material* mats;
  const float* tree;
  const float* lamp_T;
  const float4* env_T;
  const uint32_t* order;  // shading order of the scene's Gaussians
  ShadeParams SH;   // eye replaced per view
  uint32_t lit;     // 0: no lighting bound (radiance 0, as an unbound colour buffer)
};
// Shades each lit view's marked Gaussians (the shading list; see launch_bshade_list) at the view's eye and light
// scale into their splat records' radiance, and raises the view's maximum radiance.
cudaError_t launch_bshade(const BatchView* views, const BatchScene* scenes, const uint32_t* block_view,
                          uint32_t max_blocks, const uint32_t* list, const uint32_t* view_shade, SplatRec* recs,
                          uint32_t* view_maxrad, int variant, cudaStream_t s);

cudaError_t upload_iso_dirs(const float* dirs128x4, cudaStream_t s);
// motion_blur.wgsl blur_records over the records (count leaves, then tree nodes up to n_nodes) of the parts in
// `mask`: g_dst / n_dst receive each stretched along its part's motion (flags bit 1, shutter > 0) or its rest record.
cudaError_t launch_blur_records(const sl_part* parts, uint32_t part_count, float shutter, uint32_t mask,
                                const sl_gaussian* g_src, const sl_node* n_src, sl_gaussian* g_dst, sl_node* n_dst,
                                uint32_t count, uint32_t n_nodes, cudaStream_t s);
cudaError_t launch_iso(const sl_gaussian* gs, sl_node* nodes, const sl_vgrid* vgrid, uint32_t count, cudaStream_t s);
cudaError_t launch_lsm_splat(const LightMapParams& L, const sl_gaussian* gs, const sl_node* nodes,
                             const sl_part* parts, uint32_t count, const BlurCut& bc, uint32_t* acc, cudaStream_t s);
cudaError_t launch_resolve(const uint32_t* acc, float fix, uint32_t texels, uint32_t layers, uint32_t layer_texels,
                           const uint32_t* dirty_layers, float4* mip, cudaStream_t s);
cudaError_t launch_mips(float4* mip, uint32_t res, uint32_t levels, const uint32_t* level_off, uint32_t layers,
                        uint32_t layer_texels, const uint32_t* dirty_layers, cudaStream_t s);
cudaError_t launch_lsm_lookup(const LightMapParams& L, const sl_gaussian* gs, const sl_part* parts, uint32_t count,
                              const float4* mip, float* lamp_T, cudaStream_t s);
cudaError_t launch_sm_splat(const SunParams& SP, const SunLayer* layers, const sl_gaussian* gs, const sl_node* nodes,
                            const sl_part* parts, uint32_t count, const BlurCut& bc, uint32_t* acc, cudaStream_t s);
cudaError_t launch_sm_lookup(const SunParams& SP, const SunLayer* layers, const sl_gaussian* gs, const sl_part* parts,
                             uint32_t count, const float4* mip, float4* env_T, cudaStream_t s);
cudaError_t launch_shade(const ShadeParams& SH, const sl_gaussian* gs, const sl_node* nodes, const sl_vgrid* vgrid,
                         const sl_part* parts, const sl_material* mats, const float* tree, const float* lamp_T,
                         const float4* env_T, const uint32_t* order, float4* colour, uint32_t count, cudaStream_t s);

// The emitter tree of n records (16 floats each, albedo = Le), each emitter's Le scaled by le_scale[k] (NULL: 1), as
// the shading pass walks it (24 floats per node); returns the root.  dtab (optional): per node and emitter the
// derivatives of the node's Le (3) and M (6) with respect to that emitter's scale, [node][emitter][9].
uint32_t build_emitter_tree(const float* rec, uint32_t n, const double* le_scale, std::vector<float>& out,
                            std::vector<float>* dtab);

}  // namespace sl
