/*
 * sl_oracle.h -- CPU restatement of the reference splat pipeline.  TEST INFRASTRUCTURE ONLY: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark link this; the product never does.
 *
 * Parity status: there are no golden vectors in the reference (it has no tests); this restatement is pinned by
 * reading the WGSL it cites, by the reference's own closed forms (e.g. the quad radius bound), and by the committed
 * fixtures it generates (tests/golden).  The WGSL itself cannot run here (WebGPU), so "parity unpinned" applies to
 * the reference-vs-restatement link; GPU-vs-restatement parity is bit-exact for keys, permutation, tile ranges and
 * contributor counts, and within 1e-3 for linear RGB.
 */
#ifndef SL_ORACLE_H
#define SL_ORACLE_H

#include <stdint.h>
#include "splatlight.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One projected splat as the restatement keeps it (pixel space, framebuffer y down). */
typedef struct orc_splat {
  float cx, cy;          /* centre, pixels */
  float g0x, g0y;        /* local.x = dx*g0x + dy*g0y (splat.wgsl grad varying, y flipped) */
  float g1x, g1y;        /* local.y = dx*g1x + dy*g1y */
  float r;               /* Mahalanobis cutoff radius */
  float qcut;            /* 2 ln(tau_cut / tau_min) = r^2 before the sqrt */
  float tau0;            /* peak optical depth */
  float rgb[3];
  int32_t ix0, iy0, ix1, iy1; /* candidate pixel rectangle (inclusive); ix0 > ix1 = none */
  uint32_t valid;
} orc_splat;

/* A screen-space LOD cut as the projection reads it (shaders/project.wgsl:90-109): node flags (2 = drawn; leaves
 * [0, count), internal nodes from count), the internal nodes' Gaussian records and lit colours (4 floats each), and
 * their slots [node_base, node_base + n_int). */
typedef struct orc_lod {
  const uint32_t* flags;
  const sl_gaussian* nodes;
  const float* colour;
  uint32_t node_base, n_int;
} orc_lod;

/* project.wgsl main (shaders/project.wgsl:84-370), plain path: writes per slot the key (INVALID 0xFFFFFFFF) and
 * the splat.  n = count + 1 + n_emit slots.  colour: float4 per Gaussian (lit view) or NULL; lo_b: 3 float4 per
 * Gaussian or NULL.  Returns the number of valid keys. */
uint32_t orc_project(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                     const sl_gaussian* emitters, const float* colour, const float* lo_b,
                     const sl_render_frame* frame, uint32_t n_slots, uint32_t* keys, orc_splat* splats, int nthreads);

/* orc_project with a screen-space LOD cut (lod may be NULL); n_slots = node_base + n_int with LOD on. */
uint32_t orc_project_lod(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                         const sl_gaussian* emitters, const float* colour, const float* lo_b,
                         const sl_render_frame* frame, uint32_t n_slots, uint32_t* keys, orc_splat* splats,
                         int nthreads, const orc_lod* lod);

/* radix.wgsl (shaders/radix.wgsl:1-139): stable LSD sort of the low 16 key bits, values = slot index. */
void orc_sort16(const uint32_t* keys, uint32_t n, uint32_t* order);

/* Tile binning of the sorted visible splats: per tile, the splats whose candidate rectangle overlaps it, in sort
 * order.  ranges: 2 per tile [start, end) into entries (slot indices).  Returns the entry count, or -1 if `cap`
 * is too small. */
int64_t orc_bin(const orc_splat* splats, const uint32_t* order, uint32_t visible, uint32_t width, uint32_t height,
                uint32_t tile_w, uint32_t tile_h, uint32_t* ranges, uint32_t* entries, uint64_t cap);
/* sl_row_tiles of one splat (tile row ty), for tests. */
int orc_row_tiles(const orc_splat* s, uint32_t ty, uint32_t tile_w, uint32_t tile_h, uint32_t* t0, uint32_t* t1);

/* splat.wgsl vs/fs + premultiplied "over" blend (shaders/splat.wgsl:22-78; src/renderer.js:133-143), back to front
 * in sort order, fp32.  rgba: W x H x 4 (row 0 at the top); counts: fragments kept (alpha >= 1/255). */
void orc_composite(const orc_splat* splats, const uint32_t* order, uint32_t visible, uint32_t width,
                   uint32_t height, float* rgba, uint32_t* counts, int nthreads);

/* Whole frame: project, sort, bin, composite.  Any output may be NULL.  Returns visible count or a negative code. */
int64_t orc_render(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                   const sl_gaussian* emitters, const float* colour, const float* lo_b,
                   const sl_render_frame* frame, uint32_t tile_w, uint32_t tile_h,
                   uint32_t* keys, uint32_t* order, uint32_t* ranges, uint32_t* entries, uint64_t entries_cap,
                   uint64_t* n_entries, float* rgba, uint32_t* counts, int nthreads);

/* orc_render with a screen-space LOD cut (lod may be NULL). */
int64_t orc_render_lod(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                       const sl_gaussian* emitters, const float* colour, const float* lo_b,
                       const sl_render_frame* frame, uint32_t tile_w, uint32_t tile_h,
                       uint32_t* keys, uint32_t* order, uint32_t* ranges, uint32_t* entries, uint64_t entries_cap,
                       uint64_t* n_entries, float* rgba, uint32_t* counts, int nthreads, const orc_lod* lod);

/* Screen-space LOD (sl_oracle_lod.c): src/lod.js nodeGaussians (internal nodes G..N-1 as Gaussian records, float64;
 * returns 0), lod.wgsl lod_select (flags updated in place, depth by depth) and lod_colour (ncolour: 4 floats per
 * internal node, deepest first; colour: 4 floats per leaf or NULL; lo_b: 12 floats per leaf or NULL). */
int orc_lod_records(const sl_gaussian* gauss, uint32_t G, const sl_node* nodes, uint32_t N, const uint32_t* kids,
                    sl_gaussian* out);
/* nodeGaussians' node V grids (src/lod.js): N - G records, the mass-weighted mean of the children's cells */
int orc_lod_vgrids(uint32_t G, const sl_node* nodes, uint32_t N, const uint32_t* kids, const sl_vgrid* leaf_vg,
                   sl_vgrid* out);
void orc_lod_select(const sl_node* nodes, uint32_t N, uint32_t G, const uint32_t* kids, const sl_part* parts,
                    uint32_t part_count, const sl_render_frame* f, uint32_t emit_part, uint32_t size_rule,
                    float blur_lod, uint32_t* flags);
void orc_lod_colour(const sl_node* nodes, uint32_t N, uint32_t G, const uint32_t* kids, const uint32_t* flags,
                    const float* colour, const float* lo_b, float gain, uint32_t colour_all, float* ncolour);

/* element-wise sl_logf / sl_expf of include/sl_detmath.h (accuracy tests) */
void orc_logf_n(const float* x, float* y, uint64_t n);
void orc_expf_n(const float* x, float* y, uint64_t n);
void orc_atan2f_n(const float* y, const float* x, float* out, uint64_t n);
void orc_asinf_n(const float* x, float* y, uint64_t n);
void orc_acosf_n(const float* x, float* y, uint64_t n);

#ifdef __cplusplus
}
#endif

#endif
