/*
 * sl_oracle_light.h -- CPU restatement of the per-Gaussian lighting (TEST INFRASTRUCTURE; see sl_oracle_light.c).
 */
#ifndef SL_ORACLE_LIGHT_H
#define SL_ORACLE_LIGHT_H

#include <stdint.h>

#include "splatlight.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_env_light {
  float dir[3];   /* unit direction toward the light (world) */
  float std;      /* angular standard deviation, radians */
  float irr[3];   /* irradiance on a plane facing the light */
  int32_t shadows;
} orc_env_light;

typedef struct orc_light_setup {
  /* emissive Gaussian lights: 16 floats per record (a Gaussian in world space, albedo = Le) */
  const float* emit_rec;
  uint32_t n_emit;
  float scale;        /* EmitParams.scale (overlap correction) */
  float theta;        /* cut rule, EMIT_THETA = 4 */
  uint32_t mode;      /* 1: light cut, 0: every emitter */
  uint32_t asg;       /* EmitParams.n5 bit 3: lights as shapes in shiny highlights */
  uint32_t one_sided; /* emitters emit toward +normal only */
  float normal[3];
  float edge_soft;
  uint32_t skip_part; /* the emitters' own part (0xFFFFFFFF: none) */
  uint32_t shadow_res;/* light map A resolution per part layer (0: no emitter shadows) */
  /* distant lights */
  const orc_env_light* lights;
  uint32_t n_lights;
  uint32_t sun_res;   /* sun map resolution (0: no sun shadows) */
  float sky_ambient;  /* constant ambient (no reference counterpart) */
  float eye[3];
  float fwd[3];       /* camera forward, for the sun cascades */
  uint32_t shade_only;/* 1: nodes (iso_norm), lamp_T and env_T are inputs from an earlier call; only shade */
  float blur_shutter; /* > 0: the opacity-map splats draw moving parts' records stretched over the exposure
                         (motion_blur.wgsl blur_records; every part with flags bit 1 moves) */
  /* the motion-blur cut (light_shadow.wgsl:158-210): the scene's tree (the leaves, then the internal nodes), every
   * node's parent, and the cut factor k (0: every leaf stretched) */
  const sl_node* tree_nodes;
  const uint32_t* tree_parent;
  uint32_t n_tree;
  float cut_k;
} orc_light_setup;

/* motion_blur.wgsl blur_records (:80-127) for one leaf: its Gaussian and node stretched along its part's motion over
 * the exposure (shutter x (xf - xf_prev)), mass kept; unchanged for a part that does not move (flags bit 1). */
void orc_blur_record(const sl_part* parts, uint32_t part_count, float shutter, const sl_gaussian* g_in,
                     const sl_node* n_in, sl_gaussian* g_out, sl_node* n_out);

/* The 128 iso_init cell directions and solid angles (iso_init.wgsl:39-45), 4 floats each, computed in float64. */
void orc_iso_dirs(float* dirs);

/* buildEmitterTree (src/lighting.js:99-169): 2n-1 nodes of 24 floats (EmitNode + its ASG covariance, the packing
 * of packEmitNodes); returns the root index; root_cov: the root's widened covariance (xx yy zz xy xz yz). */
uint32_t orc_emitter_tree(const float* rec, uint32_t n, float* nodes_out, float* root_cov);

/* The whole lighting update: iso_init into nodes[].pad0, emitter tree, light map A -> lamp_T, sun maps -> env_T,
 * then shade_emit + env_direct + sky ambient -> colour (float4 per Gaussian). */
int orc_lighting(const sl_gaussian* gs, uint32_t count, const sl_part* parts, uint32_t part_count, sl_node* nodes,
                 const sl_vgrid* vgrid, const sl_material* mats, uint32_t mat_count, const orc_light_setup* S,
                 float* colour, float* lamp_T, float* env_T, int nthreads);


/* ---- probe bounce (bounce.wgsl; lighting.js probeLayout / initBounce / encodeBounce) -------------------------- */
typedef struct orc_probe_layout {
  uint32_t dims[3];
  uint32_t terrain;
  float lo[3];
  float step[3];
  float levels[16];
  const float* ground; /* dims[0] x dims[1], or NULL (0) */
  float tmax;
  uint32_t part_probes; /* 1: 8 probes per part after the lattice, gathering for the movable ones */
  uint32_t n_vols;      /* static probe volumes: (part, nx, ny, nz) each */
  uint32_t vols[32][4];
} orc_probe_layout;

typedef struct orc_bounce_in {
  const sl_gaussian* gs;
  uint32_t count;
  const sl_part* parts;
  uint32_t part_count;
  const sl_node* nodes; /* the leaves (iso_norm in pad0) then the internal nodes */
  uint32_t n_nodes;
  const uint32_t* kids;
  const sl_vgrid* vgrid;
  const sl_material* mats;
  uint32_t mat_count;
  const float* tree; /* emitter tree, 24 floats per node (orc_emitter_tree) */
  uint32_t tree_root, n_emit, emit_mode, one_sided;
  float emit_theta, emit_scale, edge_soft;
  float normal[3];
  const float* lamp_T; /* per Gaussian */
  const float* env_T;  /* 4 per Gaussian */
  const orc_env_light* lights;
  uint32_t n_lights;
  const float* sky_sh; /* 16 x 3, or NULL */
  orc_probe_layout lay;
  uint32_t max_depth;
  float eye[3];
  float alpha; /* this gather's history weight */
  uint32_t frame;
  uint32_t force;      /* iso_xfer refreshes every Gaussian */
  uint32_t moved_mask; /* parts that moved this frame (the reference's Part flags bit 1) */
  uint32_t dark_part;  /* the part whose Gaussians send nothing into the probes (PP.refl.w - 1; NONE: none) */
  uint32_t asg_cells;  /* U.iso bit 2 (asgSpec): near-mirror Gaussians see the cells near their mirror direction as
                          lights with an angular size (cell_asg_phase) */
  uint32_t sender_cut;  /* the sender cut (bounce.wgsl sc_select; the reference's default): only the senders some probe
                           resolves are lit, the rest of each part's tree as the nodes every probe uses whole */
  uint32_t sc_reselect; /* re-select the cut this frame (the first frame, or a part moved) */
  const sl_gaussian* node_gs; /* the internal nodes as Gaussians (orc_lod_records), N - G */
  const sl_vgrid* node_vg;    /* their V grids (orc_lod_vgrids), N - G */
} orc_bounce_in;

typedef struct orc_bounce_state {
  float* probe_data; /* NP x 128 x 8 */
  float* probe_sh;   /* NP x 9 x 4 */
  float* xfer;       /* G x 12 */
  float* lo_dir;     /* G x 4 */
  float* lo_b;       /* G x 12 */
  float* node_acc;   /* N x 14 x 4 */
  uint32_t* node_sh; /* N x 14 */
  float* probe_hist; /* NP x 128 x 16: the last two gathers per ray, (rgb, m1), (m2, 0, 0, 0) each */
  /* the sender cut's state (unused without it) */
  uint32_t* sc_flag; /* N: BELOW 0, OPEN 1, NODE 2, LEAF 3 */
  float* sc_X;       /* (N - G) x 32: per cut node the two faces' transfer and exposure (24), their direct light (8) */
  float* sc_T;       /* N - G: a cut node's lamp T */
  float* sc_envT;    /* (N - G) x 4: its distant lights' T */
} orc_bounce_state;


/* One frame of the probe bounce (the reference's encodeBounce): iso_xfer, direct_dirs_emit + env_dirs for the
 * Gaussians g % 4 == frame % 4, node_leaf, node_up, node_sh2, probe_gather, probe_valid, probe_sh2, bounce_sh; with
 * the sender cut (in->sender_cut) sc_select, sc_xfer, sc_shadow and the cut nodes' direct light, node_leaf on the cut's
 * leaves, node_cut, node_up on the open nodes.  The state persists between frames (zero it before the first). */
int orc_bounce_frame(const orc_bounce_in* in, orc_bounce_state* st, int nthreads);
/* D14 (14 x 3) and the 9 x 14 least-squares SH2 fit on it, float64 then rounded */
void orc_bounce_tables(float* d14, float* pinv);
/* f32 -> f16 bits, round to nearest even */
uint32_t orc_f32_to_f16(float f);

#ifdef __cplusplus
}
#endif

#endif
