// Internal declarations of the probe bounce (bounce.cu): its parameter block and device buffers.
#pragma once

#include <vector>

#include "sl_lighting.h"

struct sl_lighting;

namespace sl {

// the constant table (one device buffer): 128 cells x (direction, solid angle), D14, the 9 x 14 SH2 fit, and per cell
// its elevation and azimuth tangents and angular variances as a light (cell_asg_phase)
constexpr uint32_t kTabCells = 0;
constexpr uint32_t kTabD14 = 512;
constexpr uint32_t kTabPinv = 512 + 42;
constexpr uint32_t kTabCellAsg = 512 + 42 + 126;
constexpr uint32_t kTabFloats = 512 + 42 + 126 + 1024;

// bounce.wgsl ProbeParams (the fields this path reads) + the frame's inputs
struct BounceParams {
  uint32_t G, N, NP, NL, part_count, mat_count;  // NP: every probe; NL: the lattice's (then 8 per part, volumes)
  uint32_t vol_first[32], vol_dims[32][3];       // per part: its static volume's first probe after the lattice, grid
  uint32_t dims[3], terrain;
  float lo[3], step[3], levels[16];
  float tmax, brad, alpha;
  uint32_t frame, force, moved_mask, has_sky;
  uint32_t dark_part;  // the part whose Gaussians send nothing into the probes (0xFFFFFFFF: none)
  uint32_t asg_cells;  // near-mirror Gaussians see the cells near their mirror direction as lights with a size
  float eye[3];
  float sky[48];  // 16 SH coefficients (bands 0-3), rgb
  uint32_t sender_cut;   // the sender cut (bounce.wgsl sc_select .. node_sh2_sc) instead of every leaf
  uint32_t sc_reselect;  // the cut is selected again this frame (the first frame, or a part moved)
};

// a node's mark under the sender cut (bounce.wgsl:1463-1466)
constexpr uint32_t kScBelow = 0, kScOpen = 1, kScNode = 2, kScLeaf = 3;

struct BounceBuffers {
  const sl_gaussian* gs;
  const sl_node* nodes;   // the lighting's leaves (iso_norm)
  const sl_node* tnodes;  // the tree: the leaves, then the internal nodes
  const uint32_t* kids;
  const sl_vgrid* vgrid;
  const sl_part* parts;
  const sl_material* mats;
  const float* tree;      // emitter tree
  const float* lamp_T;
  const float4* env_T;
  const float* tab;
  const float* ground;    // dims[0] x dims[1] ground heights, or null
  const uint32_t* up_list;  // internal nodes grouped by depth
  const uint32_t* quarters; // the Gaussians g with g % 4 == q, for q = 0..3 in turn, each in the shading (Morton) order
  uint32_t quarter_off[5];  // quarter q is quarters[quarter_off[q] .. quarter_off[q + 1])
  float4 *xfer, *lo_dir, *lo_b, *node_acc, *probe_data, *probe_sh;
  float4* probe_hist;  // per ray the last two gathers, (rgb, m1), (m2): the FIR blend's history
  float* leaf_w;  // per Gaussian node_leaf's 14 weights (footprint x V toward D14), refreshed with the transfer
  uint32_t* node_sh;
  // the sender cut: every node by depth, parents, the internal nodes as Gaussians and their V grids (N - G each),
  // per node its mark, per internal node 8 vec4 (two faces' transfer and exposure, their direct light), the lamp T
  // and distant-light T, the cut nodes' list with its count at sc_list[0] (nodes from sc_list[1])
  const uint32_t* sc_level;
  const uint32_t* parent;
  const sl_gaussian* sc_gs;
  const sl_vgrid* sc_vg;
  uint32_t* sc_flag;
  float4* sc_X;
  float* sc_T;
  float4* sc_E;
  uint32_t* sc_list;
};

// The shading pass's parameters for an eye (capi_lighting.cu); iso_init's 128 cells, float64 then rounded.
void shade_params(const sl_lighting* l, const float* eye, ShadeParams& SH);
void iso_dirs(float* d);
// D14 and the 9 x 14 least-squares SH2 fit on it (lighting.js:188-209), float64 then rounded.
void bounce_tables(float* d14, float* pinv);
// cell_asg_phase's per-cell frame (bounce.wgsl:180-191): e_el, e_az, then s_el^2, s_az^2, 8 floats a cell, float64
void cell_asg_table(float* t);

// direct_dirs_emit + env_dirs for the Gaussians g % 4 == frame % 4 (bounce_direct.cu) into lo_dir; with the sender
// cut only the cut's leaves among them, then direct_dirs_nodes_sc + env_dirs_nodes_sc for the cut nodes that refresh
// this frame into sc_X
cudaError_t launch_bounce_direct(const BounceParams& B, const ShadeParams& SH, const BounceBuffers& D, cudaStream_t s);

// One frame of the bounce: level_off / level_cnt give each depth's internal nodes in up_list (depths 1 ..
// max_depth - 1 are summed, deepest first); sc_off / sc_cnt every node of each depth in sc_level (the sender cut).
cudaError_t launch_bounce_frame(const BounceParams& B, const ShadeParams& SH, const BounceBuffers& D,
                                const std::vector<uint32_t>& level_off, const std::vector<uint32_t>& level_cnt,
                                const std::vector<uint32_t>& sc_off, const std::vector<uint32_t>& sc_cnt,
                                cudaStream_t s);

}  // namespace sl
