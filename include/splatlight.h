/*
 * splatlight.h -- C ABI of the GB300 splat pipeline (project -> stable depth sort -> per-tile ranges -> composite,
 * with the per-Gaussian lighting it composites).  Plain C: pointers, sizes and int status codes; no CUDA or torch
 * types.  Streams are passed as `void*` holding a cudaStream_t (NULL = the legacy default stream).
 *
 * Each entry point names the reference interface it replaces.  Paths are within the reference project.
 *
 * Memory: the caller owns host memory; the library owns every device buffer it allocates (opaque handles, *_destroy).
 * Output pointers may be host or device memory: the `*_on_device` flag says which.
 * Errors: every call returns SL_OK (0) or a negative SL_ERR_* code and never aborts; sl_last_error() gives the text
 * of the last failure on the calling thread.
 * Threading: a handle is thread-compatible (one caller at a time); distinct handles may be used concurrently.
 */
#ifndef SPLATLIGHT_H
#define SPLATLIGHT_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SL_API __attribute__((visibility("default")))
#else
#define SL_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------------------------- */
#define SL_OK 0
#define SL_ERR_INVALID_ARG (-1)   /* a null pointer, a bad size or a value out of range */
#define SL_ERR_LAYOUT (-2)        /* asset layout check failed (format, version, stride, field offset, count) */
#define SL_ERR_OOM (-3)           /* device allocation failed */
#define SL_ERR_CUDA (-4)          /* a CUDA runtime call failed */
#define SL_ERR_TIMEOUT (-5)       /* a bounded device-side wait gave up (the stream stays usable) */
#define SL_ERR_UNSUPPORTED (-6)   /* the frame enables a feature outside this pipeline (explode, lens warp ...) */
#define SL_ERR_ADMISSION (-7)     /* serving: the request does not fit the device-memory budget */
#define SL_ERR_OVERFLOW (-8)      /* a fixed-capacity buffer (tile entries) was too small; grow and retry */
#define SL_ERR_NO_DEVICE (-9)     /* no CUDA device, or the device is not an sm_103 part */
#define SL_ERR_CANCELLED (-10)    /* serving: the server shut down before the request was admitted */

/* ---- scene records (gs-runtime layout; shaders/common.wgsl:5-25, runtime/wgsl/common.wgsl:4-65) --------------- */

/* 64 B, uploaded unchanged from gaussians.bin (src/asset.js:9; shaders/common.wgsl:6-14) */
typedef struct sl_gaussian {
  float mu[3];           /* centre, part rest frame */
  float kappa;           /* peak extinction scale, 1/m */
  float quat[4];         /* x, y, z, w */
  float scale[3];        /* std devs, ascending: x = short axis */
  uint32_t part_surface; /* part | surface << 16 */
  float albedo[3];       /* linear albedo; emitter records: emitted radiance Le */
  uint32_t flags;        /* low 16 bits: material */
} sl_gaussian;

/* 128 B (src/asset.js:10; shaders/common.wgsl:17-25).  xf rows are [R row | t] (world_from_rest). */
typedef struct sl_part {
  float xf[12];
  float xf_prev[12];
  float bound[4];        /* rest-frame centre, radius */
  uint32_t root, g_lo, g_hi, flags; /* flags bit 1 moved this frame, bit 2 hidden */
} sl_part;

/* 96 B tree node; leaves are nodes [0, count) (runtime/wgsl/common.wgsl:12-19) */
typedef struct sl_node {
  float mean[3];
  float radius;
  float cinv_diag[3];
  float kappa;
  float cinv_off[3];     /* xy xz yz */
  float smax;
  float sn_diag[3];      /* SGGX S-hat (projected-area extinction) */
  uint32_t part;
  float sn_off[3];
  uint32_t child_lo;
  uint32_t child_hi, depth, pad0, pad1; /* leaves: pad0 = bits of iso_norm after sl_lighting_init_iso */
} sl_node;

/* 32 B (runtime/wgsl/common.wgsl:59-65; specular mix runtime/wgsl/material_ext.wgsl:10-42) */
typedef struct sl_material {
  float flake[3];          /* SGGX diagonal in the Gaussian's frame: (1, r^2, r^2) for roughness r */
  uint32_t phase_samples;
  float vfloor;
  uint32_t flags;          /* bit 0 emissive, bit 2 one-sided, bit 3 specular flakes */
  uint32_t pad0, pad1;     /* specular: pad0 low half = fp16 k; emissive: fp16 (r, g), (b, 0) */
} sl_material;

/* 128 B V grid: 8 x 16 bytes of own-part visibility (runtime/wgsl/common.wgsl:21) */
typedef struct sl_vgrid { uint32_t w[32]; } sl_vgrid;

/* The 1200-byte RenderFrame uniform exactly as the host writes it (shaders/common.wgsl:44-77; src/main.js:526-556;
 * FRAME_BYTES src/renderer.js:9).  Fields this pipeline reads are marked (*); the others must hold their "off"
 * values (zero), else sl_render returns SL_ERR_UNSUPPORTED. */
typedef struct sl_render_frame {
  float view[16];                /* (*) column-major world -> view (src/math.js:36-46) */
  float proj[16];                /* carried, unused (the path projects with focal lengths) */
  float palette[4][4];           /* (*) slots 0-2; palette[3] = (bounce gain*, emitter count*, blur shutter, blur cov) */
  uint32_t part_material[16];    /* (*) palette slot per part 0-15 */
  float lamp[4];                 /* lamp.w must be 0 (camera-only flakes are outside the pipeline) */
  float lamp_color[4];           /* lamp_color.w = reflection flags, must be 0 (no coverage split) */
  float viewport[2];             /* (*) pixels */
  float focal[2];                /* (*) pixels */
  float near_plane;              /* (*) */
  float far_plane;               /* (*) */
  uint32_t count;                /* (*) Gaussians in the asset */
  uint32_t view_mode;            /* (*) 0 flat albedo, 1 depth, 2 overdraw (contributor count), 3 lit */
  float albedo_scale;            /* (*) */
  float flake_roughness;
  float exposure;
  float lowpass_px2;             /* (*) screen-space dilation of the 2D covariance */
  float palette_ext[4][4];       /* (*) palette slots 4-7 */
  float mat_view[16][4];         /* (*) only .w bit 0 (glass) is read: glass flags the splat, nothing else */
  uint32_t part_material_ext[16];/* (*) palette slot per part 16-31 */
  uint32_t lod[4];               /* screen-space LOD: threshold px (float bits, 0 = off), node slot base, internal
                                    nodes (sl_lod_create on the renderer first; not in batches) */
  float explode[4];
  float explode_c[4];
  float explode_k[4];            /* explode_k.z must be <= 0.5 (explode off) */
  float mat_view_ext[16][4];
  uint32_t tone[4];
  float part_fade[32];           /* (*) per part draw-time fade */
  uint32_t particles[4];         /* particles.y must be 0 */
} sl_render_frame;

/* ---- errors -------------------------------------------------------------------------------------------------- */

/* Copies the calling thread's last error text (NUL-terminated, truncated to `cap`).  Returns its full length. */
SL_API size_t sl_last_error(char* buf, size_t cap);

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
SL_API int sl_version(void);

/* ---- asset layout (src/asset.js:18-38 checkHeader / checkBuffer) --------------------------------------------- */

/* checkHeader's format and version test (src/asset.js:19-20): `format` must be "gs-runtime" and the major part of
 * `version` (the text before the first '.') must be "0", the major version of the layout this library reads.
 * Returns SL_OK or SL_ERR_LAYOUT with the reference's message ("Unknown asset format X", "Unsupported asset version
 * V") in sl_last_error; a null argument is SL_ERR_LAYOUT as an absent field is there. */
SL_API int sl_asset_check_header(const char* format, const char* version);

/* Checks one buffer description of asset.json against the layout the kernels assume: the buffer name is one of
 * gaussians, parts, lamps, materials, nodes, kids, vgrid; stride and every listed field offset must match, and
 * 0 < count <= 2^24.  `field_names`/`field_offsets` hold `n_fields` pairs (offset UINT32_MAX = missing field).
 * Returns SL_OK or SL_ERR_LAYOUT (text in sl_last_error).  Replaces checkHeader's per-buffer loop, src/asset.js:21-29. */
SL_API int sl_asset_check_buffer(const char* name, uint32_t stride, uint32_t count, const char* const* field_names,
                          const uint32_t* field_offsets, uint32_t n_fields);

/* Checks a buffer's byte length against count x stride (src/asset.js:32-38 checkBuffer). */
SL_API int sl_asset_check_bytes(uint64_t byte_length, uint32_t count, uint32_t stride);

/* ---- renderer (src/renderer.js SplatRenderer) ---------------------------------------------------------------- */

typedef struct sl_renderer sl_renderer;
typedef struct sl_lighting sl_lighting;

/* Tile shape of the binned compositor: 16x16 (default), 8x32 or 32x8 pixels. */
typedef struct sl_render_options {
  uint32_t tile_w, tile_h;       /* 0 = keep */
  float t_stop;                  /* early-termination transmittance scale (0 = default 1e-4 / max radiance) */
  uint32_t entry_capacity;       /* tile entries pre-allocated (0 = grow on demand) */
  uint32_t sort_mode;            /* 0 keep; 1 the stable radix sort (default, radix.wgsl); 2 the counting sort
                                    (scan.wgsl + scatter.wgsl: 65536-bucket key histogram, exclusive offsets, atomic
                                    placement -- splats sharing a key land in arbitrary order) (src/renderer.js:122) */
} sl_render_options;

typedef struct sl_render_stats {
  uint32_t slots;                /* n = count + 1 + emitters: the slots projected and sorted */
  uint32_t visible;              /* valid keys (scan.wgsl's instance count) */
  uint32_t entries;              /* (tile, splat) pairs binned */
  uint32_t tiles;                /* tiles in the view */
  uint32_t fragments;            /* fragments the compositor blended (after early termination) */
  float ms_project, ms_sort, ms_bin, ms_composite, ms_total; /* device times when timing is on, else 0 */
} sl_render_stats;

/* new SplatRenderer(device, canvasFormat, shaders, asset) (src/renderer.js:38-233): uploads the asset's Gaussians
 * and parts and sizes every per-slot buffer for count + 1 + max_emitters slots (MAX_EMITTERS, src/renderer.js:17). */
SL_API int sl_renderer_create(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                       uint32_t max_emitters, sl_renderer** out);
SL_API int sl_renderer_destroy(sl_renderer* r);

/* writeParts(partBytes) (src/renderer.js:407-409): replaces the part records (xf, xf_prev, flags). */
SL_API int sl_renderer_set_parts(sl_renderer* r, const sl_part* parts, uint32_t part_count);

/* The emitters buffer project.wgsl draws in slots count+1 .. count+n (shaders/project.wgsl:121, 226-230; the
 * renderer's emitterBuf): world-space emissive Gaussians whose albedo holds Le.  n <= max_emitters. */
SL_API int sl_renderer_set_emitters(sl_renderer* r, const sl_gaussian* emitters, uint32_t n);

/* bindColour(colourBuf, bounceBuf, emitterBuf) (src/renderer.js:264-268) with caller-provided radiance: `colour`
 * holds one float4 per Gaussian (rgb used), `lo_b` three float4 per Gaussian (the eye bounce at [3i]) or NULL.
 * Device pointers; they must stay valid while bound.  Replaced by sl_renderer_bind_lighting. */
SL_API int sl_renderer_bind_colour(sl_renderer* r, const float* colour_dev, const float* lo_b_dev);

SL_API int sl_renderer_set_options(sl_renderer* r, const sl_render_options* opt);

/* Turns per-stage CUDA-event timing into the stats on (1) or off (0). */
SL_API int sl_renderer_set_timing(sl_renderer* r, int on);

/* encode(encoder, target, frameBytes, viewMode, timers) (src/renderer.js:411-524) without the display pass: project
 * -> stable radix sort of the 16-bit depth keys -> per-tile ranges -> front-to-back composite.  `frame` is the
 * 1200-byte RenderFrame (view_mode inside it).  Writes viewport W x H RGBA fp32 (row 0 at the top; premultiplied
 * linear rgb, alpha = coverage) to `out_rgba`.  View mode 2 writes the per-pixel contributor count to .r (and to
 * the counts debug buffer).  Stream-ordered on `stream`; with a host `out_rgba` the call returns once the image is
 * there (page-locked host memory is written in place by the compositor over the host link; pageable memory through
 * a device copy). */
SL_API int sl_render(sl_renderer* r, const sl_render_frame* frame, float* out_rgba, int out_on_device,
              sl_render_stats* stats, void* stream);

/* Debug read-back of the last sl_render on this renderer (host buffers; any may be NULL):
 *   keys   u32 per slot, INVALID 0xFFFFFFFF (project.wgsl's keys[])
 *   order  u32 per slot, the stable permutation (radix.wgsl's vals_out after the last pass)
 *   ranges u32 pairs [start, end) per tile, row-major tiles
 *   counts u32 per pixel: fragments with alpha >= 1/255 (the overdraw view; filled by view mode 2 only)
 * Sizes: slots, slots, 2 x tiles, W x H as returned in the stats. */
SL_API int sl_renderer_read_debug(sl_renderer* r, uint32_t* keys, uint32_t* order, uint32_t* ranges, uint32_t* counts);

/* The per-tile splat lists of the last sl_render: `entries` (slot indices, tile after tile, each tile's splats in
 * back-to-front order) holds stats.entries values; [ranges[2t], ranges[2t+1]) indexes tile t's list. */
SL_API int sl_renderer_read_entries(sl_renderer* r, uint32_t* entries, uint64_t cap);

/* ---- lighting (src/lighting.js Lighting, src/environment.js Environment) -------------------------------------- */

/* A distant light (the sun) as environment.wgsl's EnvLight (:20-23, written by src/environment.js:111-153). */
typedef struct sl_env_light {
  float dir[3];          /* unit direction toward the light, world */
  float std;             /* angular standard deviation, radians */
  float irradiance[3];   /* on a plane facing the light */
  int32_t casts_shadows;
} sl_env_light;

/* new Lighting(device, sources, asset, gaussBuf, partBuf) (src/lighting.js:318-525): the lighting of a renderer's
 * scene.  nodes: the asset's leaf nodes (count records, runtime/wgsl/common.wgsl:12-19; pad0 is overwritten by
 * iso_init); vgrid: one V grid per Gaussian; materials: material_count records (<= 256). */
SL_API int sl_lighting_create(sl_renderer* r, const sl_node* nodes, const sl_vgrid* vgrid, const sl_material* materials,
                              uint32_t material_count, sl_lighting** out);
SL_API int sl_lighting_destroy(sl_lighting* l);

/* setEmitters / setAssetEmitters + writeEmitParams (src/lighting.js:612-721, :657-673): the emissive Gaussians
 * (world space, albedo = Le) become the light set; the emitter tree is built on the host (buildEmitterTree,
 * src/lighting.js:99-169), EmitParams.scale = scale, one_sided / normal / skip_part as EmitParams.  The renderer
 * draws the same records in its emitter slots (its max_emitters permitting).  The light's shadow maps re-splat at
 * the next update. */
SL_API int sl_lighting_set_emitters(sl_lighting* l, const sl_gaussian* emitters, uint32_t n, float scale,
                                    int one_sided, const float* normal, uint32_t skip_part);

/* buildEmitterTree + packEmitNodes (src/lighting.js:99-169) on the host alone (no device is touched): the tree of n
 * emitter records, each emitter's Le scaled by le_scale[k] (NULL: 1), as the shading pass walks it -- 24 floats per
 * node into nodes_out (2n - 1 nodes: mean, radius, M diagonal, skip link, M off-diagonal, child_lo, Le, child_hi,
 * the ASG covariance; word 19 set where the walk's 48-entry stack would be full) -- and the root into *root.
 * dtab_out (optional, (2n - 1) x n x 9 floats): per node and emitter, d(Le rgb, M xx yy zz xy xz yz) / d le_scale[k]
 * (central differences of the float64 build). */
SL_API int sl_emitter_tree(const sl_gaussian* emitters, uint32_t n, const double* le_scale, float* nodes_out,
                           float* dtab_out, uint32_t* root);

/* Environment.set / write (src/environment.js:106-153): up to 4 distant lights; sky_ambient adds albedo * sky_ambient
 * to every non-emissive Gaussian (a constant stand-in for sky light where the probe bounce is not set; 0 with it). */
SL_API int sl_lighting_set_environment(sl_lighting* l, const sl_env_light* lights, uint32_t n, float sky_ambient);

/* Resolution of the emitter light's per-part opacity map (src/light_shadow.js:18, default 512) and of the sun's maps
 * (src/sun_map.js:54, default 512), 0 = no such shadows; light-cut mode (1 cut, 0 every emitter; emissive.wgsl:23),
 * cut angle theta (EMIT_THETA = 4) and ASG highlights (EmitParams.n5 bit 3, on by default). */
SL_API int sl_lighting_set_options(sl_lighting* l, uint32_t shadow_res, uint32_t sun_res, uint32_t mode, float theta,
                                   int asg);

/* Motion blur for the lighting (src/lighting.js:468-507, runtime/wgsl/motion_blur.wgsl): with shutter > 0 (the
 * reference's default is 0.5), every update rewrites copies of the records of the parts that moved this update or the
 * last (moved_mask), each record of a moving part (sl_part.flags bit 1) stretched along its motion over the exposure,
 * shutter x (xf - xf_prev): covariance C + d d^T / 12 centred mid-exposure, mass kept; the opacity-map splats (light
 * map A and the sun maps) draw the copies, so a moving part casts a smeared shadow, while every receiver keeps its
 * rest record.  With a tree (sl_lighting_set_tree) and cut_k > 0 (the reference's ?blurcut, default 1) a moving part
 * splats the cut of its tree whose nodes are about cut_k x its smear across (light_shadow.wgsl:158-210,
 * sun_map.wgsl:119-153), each keeping its rest coverage; cut_k 0 (or no tree) stretches every leaf.  shutter 0 (the
 * default here) turns it off.  The maps re-splat at the next update. */
SL_API int sl_lighting_set_blur(sl_lighting* l, float shutter, float cut_k);
/* The scene's tree for the motion-blur cut and the probe gather (src/lighting.js initNodeParents, :557-567): n_nodes
 * records, the leaves
 * (the renderer's Gaussians, in order) then the internal nodes, whose children are kids[child_lo .. child_hi); the
 * parts' roots come from the renderer's parts (sl_part.root).  Host arrays, copied. */
SL_API int sl_lighting_set_tree(sl_lighting* l, const sl_node* nodes, uint32_t n_nodes, const uint32_t* kids,
                                uint32_t n_kids);

/* The probe lattice of the bounce (src/lighting.js probeLayout :220-286; runtime/wgsl/bounce.wgsl ProbeParams :23-56):
 * dims[0] x dims[1] columns at lo.xy + step.xy (i, j), each with dims[2] probes at ground[i dims[1] + j] + levels[k].
 * The room layout (terrain 0): ground 0, levels lo.z + k step.z; the terrain layout (terrain 1): ground heights per
 * column, levels above them, step.z 0. */
typedef struct sl_probe_layout {
  uint32_t dims[3];     /* x, y columns (2 .. 1024 columns in all) and levels (2 .. 16) */
  uint32_t terrain;
  float lo[3];
  float step[3];
  float levels[16];     /* ascending */
  const float* ground;  /* dims[0] x dims[1] heights, or NULL (0); copied */
  float tmax;           /* probe ray length: TMAX 6 m, or the scene's diagonal with an environment (lighting.js:226) */
  uint32_t n_vols;      /* static probe volumes (probeVolumes, lighting.js:289-314): up to 32 */
  uint32_t vols[32][4]; /* (part 0-31, nx, ny, nz): a grid over the part's rest-frame box serving its Gaussians */
} sl_probe_layout;

/* Lighting.initBounce (src/lighting.js:723-816), with every leaf a sender (?sendercut=0; the reference's default sender
 * cut is sl_lighting_set_sender_cut): after each update's shading the
 * probe bounce runs one frame (encodeBounce :1018-1103; runtime/wgsl/bounce.wgsl, M39 stage 2): the Gaussians'
 * transfer SH2 (iso_xfer, on the first frame and near parts that moved), their light toward the probes for a quarter
 * of them (direct_dirs_emit + env_dirs), the tree's sums of it and their SH2 (node_leaf, node_up over depths
 * max_depth - 1 .. 1 (0: the tree's depth), node_sh2), the probes' gather through every part's tree with the sky
 * beyond (probe_gather), their validity and SH2 (probe_valid, probe_sh2), then each Gaussian's bounce from its 8
 * probes (bounce_sh, gloss_sh) into lo_b, which the projection adds to the lit colour times the frame's bounce gain
 * (palette[3].x).  After the lattice come 8 probes per part (part_probe_frame's cube, riding with the part; those of
 * movable parts gather, skipping their own part, and serve that part's Gaussians), then the static volumes' grids
 * (serving their part's Gaussians).  blend: the history weight of each gather after the first (1: taken as is, the
 * reference's default; 0.5: ?probeblend=ema; -1: ?probeblend=fir, the gather and the two before it tapered 0.5, 0.3,
 * 0.2).  Needs sl_lighting_set_tree and the renderer's parts (their count is fixed from here on).  emitters_dark (the
 * reference's emitBounceFix, on by default there): the Gaussians of the emitters' own part (sl_lighting_set_emitters'
 * skip_part) send nothing into the probes -- their light reaches the scene as direct light -- though they still
 * occlude.  Near-mirror materials (a flake lobe below 0.1 rad) take bounce_dirs' per-cell path, with the cells near
 * the eye's mirror direction as lights with a size when ASG highlights are on (sl_lighting_set_options).  Not built:
 * near-field visibility and reflection (off by default in the reference). */
SL_API int sl_lighting_set_probes(sl_lighting* l, const sl_probe_layout* layout, uint32_t max_depth, float blend,
                                  int emitters_dark);
/* The environment's sky for the probes (src/environment.js:116-124; bounce.wgsl sky_radiance :148-160): n_coef (<= 16)
 * real SH coefficients, rgb, bands 0-3, seen by probe rays that leave the scene.  0 coefficients: no sky. */
SL_API int sl_lighting_set_sky(sl_lighting* l, const float* sh_rgb, uint32_t n_coef);
/* The sender cut (src/lighting.js senderCut, :411-412, 1057-1095; runtime/wgsl/bounce.wgsl sc_select .. node_sh2_sc
 * :1448-1730; the reference's default): on (1), only the senders some probe's gather can resolve are lit.  Each frame
 * in which a part moved (and the first) marks every node of the parts' trees top down: BELOW (never read), OPEN (some
 * probe opens it), NODE (every probe uses it whole) or LEAF (a leaf under an open node).  The cut's leaves send as
 * before (a quarter of them a frame); each cut node is lit as one two-sided Gaussian (nodeGaussians' record and V
 * grid, src/lod.js:44-107; the shadow T of 8 leaves reached by mass-weighted descents, sc_shadow), its light plus the
 * probes' SH2 at its centre through its two faces' transfer (sc_xfer, node_cut); node_up sums the open nodes only.
 * A cut node refreshes its shadow and direct light in the frames node % 4 == frame % 4 (every cut node in a frame
 * that re-selected), and the cut is not capped (the reference opens nodes past 2^18 a frame, in the order its atomics
 * hand out slots).  Needs sl_lighting_set_probes, a tree at most 64 levels deep whose internal nodes all have
 * children, and the renderer bound; off (0) returns to every leaf.  Setting the tree again turns it off. */
SL_API int sl_lighting_set_sender_cut(sl_lighting* l, uint32_t on);
/* Debug read-back of the bounce (synchronous; bytes from the start): what = 0 lo_b (3 float4 per Gaussian: toward
 * the eye, toward the probes, lanes), 1 lo_dir (float4 per Gaussian), 2 the transfer (3 float4 per Gaussian), 3 the
 * probes' SH2 (9 float4 per probe), 4 probe_data (2 float4 per probe and cell), 5 node_sh (14 words per node),
 * 6 node_acc (14 float4 per node); with the sender cut on: 7 the marks (one word per node: 0 below, 1 open, 2 node,
 * 3 leaf), 8 the cut nodes' transfer and direct light (8 float4 per internal node: each face's transfer t0-3, t4-7,
 * (t8, exposure), then the faces' direct light), 9 their lamp T (float per internal node), 10 their distant-light T
 * (float4 per internal node); entries of nodes off the cut hold what an earlier cut left. */
SL_API int sl_lighting_read_bounce(sl_lighting* l, uint32_t what, void* dst, size_t bytes);

/* encode(encoder, eye, timers, changed, still) (src/lighting.js:1258-1274) + Environment.encodeDirect
 * (src/environment.js:181-189): iso_init on first use, the opacity maps of moved parts (moved_mask bit p) or of
 * every part after a light change, then shade_emit + env_direct into the radiance buffer the renderer reads.
 * forward (may be NULL) centres the sun cascades ahead of the camera.  Stream-ordered. */
SL_API int sl_lighting_update(sl_lighting* l, const float* eye, const float* forward, uint32_t moved_mask,
                              void* stream);

/* The shading pass alone at a new eye, with the opacity maps and cut as the last sl_lighting_update left them (the
 * per-frame shade_emit + env_direct dispatches of src/lighting.js when no layer is dirty).  Needs a prior update. */
SL_API int sl_lighting_shade(sl_lighting* l, const float* eye, void* stream);

/* Debug read-back (host buffers, any may be NULL): radiance float4 per Gaussian, the emitter shadow T per Gaussian
 * (lamp_state slot 0), the distant-light T float4 per Gaussian (env_T), the leaf nodes with iso_norm. */
SL_API int sl_lighting_read(sl_lighting* l, float* colour, float* lamp_T, float* env_T, sl_node* nodes);

/* bindColour with a Lighting object's radiance buffer (src/renderer.js:264-268). */
SL_API int sl_renderer_bind_lighting(sl_renderer* r, sl_lighting* l);

/* ---- screen-space LOD (src/lod.js nodeGaussians + Lod, runtime/wgsl/lod.wgsl) -------------------------------- */

/* The asset's tree drawn as a level of detail: every internal node is a moment-matched Gaussian of its subtree, drawn in
 * place of its leaves when it is small on screen.  A frame with LOD on has frame.lod = (threshold px as float bits,
 * node slot base, internal node count, 0): slots [count, base) hold the lamp marker and the emitters (the rest of
 * them unused), slots [base, base + N - count) the internal nodes; only the leaves and nodes of the cut are drawn. */
typedef struct sl_lod sl_lod;

/* nodeGaussians(asset) + new Lod(...) (src/lod.js:44-128): n_nodes records, leaves [0, count) of the renderer's scene
 * first, then the internal nodes; kids: the children lists ([child_lo, child_hi) of each internal node index it).  The
 * internal nodes' Gaussian records (mean, kappa, eigen-frame quaternion and scales of the covariance, the part, the
 * leaves' mass-weighted albedo, the first leaf's material) are made on the host in float64 and kept on the device
 * with the per-depth node lists.  Part roots come from the renderer's parts (sl_part.root).  One LOD per renderer:
 * sl_render reads it for frames with LOD on.  Needs at most 32 parts. */
SL_API int sl_lod_create(sl_renderer* r, const sl_node* nodes, uint32_t n_nodes, const uint32_t* kids,
                         uint32_t n_kids, sl_lod** out);
SL_API int sl_lod_destroy(sl_lod* l);
/* Lod.encodeSelect (src/lod.js:139-167), lod.wgsl lod_select: the cut for this frame, top-down, one launch per tree
 * depth (threshold = frame.lod[0] as float; the view, focal and near plane of the frame; the renderer's part poses).
 * emit_part: the emitters' part, always opened to its leaves (0xFFFFFFFF: none); size_rule: 1 projected area (the
 * reference's default), 0 bounding radius; blur_lod > 0 with the frame's shutter open: a moving part opens only nodes
 * larger than blur_lod x its smear (motion blur variant D). */
SL_API int sl_lod_select(sl_lod* l, const sl_render_frame* frame, uint32_t emit_part, uint32_t size_rule,
                         float blur_lod, void* stream);
/* Lod.encodeColour (src/lod.js:170-172), lod.wgsl lod_colour: the lit colour of the drawn nodes (colour_all: of every
 * node), bottom-up, one launch per depth: the mass-weighted mean of the children's shown colours (a leaf's: its
 * bound radiance + bounce gain x its bounce toward the eye, frame.palette[3].x).  Run after the lighting and
 * sl_lod_select, before sl_render of a lit view. */
SL_API int sl_lod_colour(sl_lod* l, const sl_render_frame* frame, uint32_t colour_all, void* stream);
/* Debug read-back (host; any may be NULL): flags (n_nodes u32: 0 none, 1 open, 2 drawn, 3 candidate, 4 under a drawn
 * node), node colours (4 floats per internal node), the internal nodes' Gaussian records. */
SL_API int sl_lod_read(sl_lod* l, uint32_t* flags, float* node_colour, sl_gaussian* records);

/* ---- display resolve (shaders/display.wgsl:120-189) -------------------------------------------------------------- */

/* The frame's linear RGBA image (device, W x H x 4 floats, as sl_render writes it) to 8-bit sRGB RGBA (device,
 * W x H x 4 bytes): exposure (frame->exposure), the tone curve frame->tone[0] (0 clamp, 1 AgX, 2 ACES filmic,
 * 3 Reinhard on luminance, 4 Khronos PBR Neutral, 5 Hable filmic), the sRGB transfer function; view mode 2 maps the
 * contributor count through the reference's heat ramp.  Bare pixels stay black here; sl_display_env adds the
 * environment's sky and light discs where the splats leave the sky showing.  Stream-ordered. */
SL_API int sl_display(const float* image_dev, uint32_t width, uint32_t height, const sl_render_frame* frame,
                      uint8_t* out_dev, void* stream);

/* The environment as the display draws it (src/environment.js write :111-150, shaders/display.wgsl Env / SkyBg
 * :7-20): the lighting sky's 16 SH coefficients, the distant lights (direction toward the light, angular std,
 * irradiance, the visible disc's std or 0), and the background sky: up to 81 SH coefficients (bands 0-8; 0 = the
 * lighting sky), the horizon ring's lobes with their widths (ring_par = 1 / (2 along^2), 1 / (2 across^2)), the ground
 * below the horizon (ground_blend = sin of the blend half-width) and the glow round the sun (std 0 = none). */
typedef struct sl_display_sky {
  uint32_t has_sky;          /* Env.info.y: a lighting sky is present */
  uint32_t n_lights;         /* up to 4 */
  float sky_sh[16][3];
  float light_dir[4][3];
  float light_std[4];
  float light_irr[4][3];
  float disc_std[4];
  uint32_t bg_count;         /* background coefficients, 0-81 (a square: (l + 1)^2) */
  uint32_t ring_count;       /* horizon lobes, 0-8 */
  float bg_sh[81][3];
  float ring[8][3];
  float ground[3];
  float ground_blend;
  float ring_par[2];
  float glow[3];
  float glow_std;
  float glow_dir[3];
} sl_display_sky;

/* sl_display with the environment (display.wgsl fs :120-133): in the lit view, where the splats leave the sky showing
 * (bare = 1 - alpha > 1/1024), the pixel adds bare x (the background sky toward its view direction, the glow, the
 * horizon ring and the ground, when a sky is present, plus the distant lights' discs), before exposure and the tone
 * curve.  sky NULL: as sl_display. */
SL_API int sl_display_env(const float* image_dev, uint32_t width, uint32_t height, const sl_render_frame* frame,
                          const sl_display_sky* sky, uint8_t* out_dev, void* stream);

/* ---- sort (shaders/radix.wgsl) --------------------------------------------------------------------------------- */

/* The stable sort of 16-bit depth keys on its own (shaders/radix.wgsl:1-139; encoded by src/renderer.js:425-434):
 * writes to order_dev the permutation that sorts keys_dev[0, n) ascending, ties in index order (radix.wgsl's vals_out
 * after its last pass, values = index).  Device pointers; n < 2^30.  Scratch is allocated stream-ordered on `stream`
 * from a memory pool private to the library (its memory kept between calls) and returned to it before return; the call returns after the sort completed (SL_ERR_TIMEOUT if a bounded device-side
 * wait gave up). */
SL_API int sl_sort_keys16(const uint16_t* keys_dev, uint32_t n, uint32_t* order_dev, void* stream);

/* The same stable sort for 32-bit keys of which the low `bits` are significant (1..32; one onesweep pass per 8 bits):
 * the segmented form the batched path sorts with (view id above the 16 depth bits; tile ids of many views).  keys_dev
 * is left intact.  No reference counterpart beyond radix.wgsl's 16-bit case. */
SL_API int sl_sort_keys32(const uint32_t* keys_dev, uint32_t n, uint32_t bits, uint32_t* order_dev, void* stream);

/* sl_sort_keys16 without any device allocation, for callers that may not allocate (a host engine that owns all
 * device memory through its own pool under a hard cap, or a frame loop whose latency budget rules out allocator
 * calls).  No counterpart in the reference.  Same inputs, output and status codes as sl_sort_keys16, for
 * n <= 1,048,576 keys (larger n: SL_ERR_INVALID_ARG).  Scratch is one fixed device array inside the library
 * (6,644,224 B: exactly one sort of 1,048,576 keys), held by every GPU that loads it until the process exits; the
 * caller still passes keys and order.  Every call looks up the array's device address in the current context (no
 * address is kept between calls, so a cudaDeviceReset or another context on the device is safe); the first call in
 * a context loads the library's module, so make it before any stream capture.  All calls share the array and it
 * keeps the last call's contents (each call clears what must start at zero): calls that overlap on the GPU (other
 * streams, other threads) race, so serialise them. */
SL_API int sl_sort_keys16_noalloc(const uint16_t* keys_dev, uint32_t n, uint32_t* order_dev, void* stream);

/* ---- batched frames (no counterpart in the reference, which draws one RenderFrame per call) ------------------- */

/* A ragged batch of views over several resident scenes (renderers), each view its own RenderFrame (camera,
 * resolution, view mode), rendered by one chain of kernels: one projection launch over every view's slots, one
 * shading launch (lit views, with their scene's lighting maps and the view's eye), one segmented depth sort (view id
 * above the 16 depth bits), one tile binning, one tile sort, one compositor launch.  Every view's image, permutation,
 * per-tile ranges and contributor counts equal what sl_render gives for that frame alone, with the same tile shape
 * (the lit radiance: with the lighting's maps as of its last sl_lighting_update).  The chain runs as one CUDA graph,
 * captured for the batch's capacity and replayed while batches fit. */
typedef struct sl_batch sl_batch;

typedef struct sl_batch_options {
  uint32_t max_views;            /* views per batch (0 = 64; at most 256) */
  uint32_t max_tiles;            /* tiles of all views (0 = grow on demand) */
  uint64_t max_slots;            /* slots of all views, each view padded to 256 (0 = grow on demand) */
  uint64_t max_entries;          /* tile entries of all views (0 = 2 per slot, grown on overflow) */
  uint32_t tile_w, tile_h;       /* 16x16 (default), 8x32 or 32x8 */
  uint32_t no_graph;             /* 1: launch the chain directly instead of replaying a graph */
  float radiance_allowance;      /* the coverage pass's allowance for shaded radiance (0 = 64): it marks the splats
                                    blending before T falls below t_stop / max(2 r, allowance x max(1, light
                                    scale)); a view whose shaded radiance exceeds half of that is re-run with every
                                    blended splat shaded, so any allowance gives a correct image */
} sl_batch_options;

typedef struct sl_batch_stats {
  uint32_t views, slots, tiles, entries; /* slots: padded total; entries: (tile, splat) pairs of all views */
  uint64_t visible, fragments;
  float ms_total;                /* device time of the chain when timing is on, else 0 */
  uint32_t graph_replayed;       /* 1 when the chain ran as a replay of the captured graph */
  uint32_t shaded;               /* Gaussians shaded, over the lit views (those the coverage pass marked) */
  uint32_t reshaded_views;       /* lit views run a second time with every blended splat shaded (radiance bound) */
  float max_radiance;            /* largest radiance bound of a view (the compositor's stop is t_stop / it) */
  float ms_stage[6];             /* with per-stage timing (sl_batch_set_timing 2), device ms of: projection (+ scan
                                    and compaction of the visible keys), depth sort, binning (+ tile sort, ranges),
                                    coverage pass, shading (list + shading pass), composite; else 0 */
} sl_batch_stats;

/* Creates a batch over n_scenes renderers (lightings[k]: the lighting bound to renderers[k], or NULL / a NULL array
 * for unlit scenes; lit views of an unlit scene get radiance 0).  Capacities grow on demand (buffers reallocated,
 * the graph re-captured). */
SL_API int sl_batch_create(sl_renderer* const* renderers, sl_lighting* const* lightings, uint32_t n_scenes,
                           const sl_batch_options* opt, sl_batch** out);
SL_API int sl_batch_destroy(sl_batch* b);
/* Tile shape for the following batches: 16x16, 8x32 or 32x8 (SL_ERR_INVALID_ARG otherwise). */
SL_API int sl_batch_set_tile(sl_batch* b, uint32_t tile_w, uint32_t tile_h);
/* Device timing of the following batches: 0 off, 1 the whole chain (stats.ms_total), 2 also each stage
 * (stats.ms_stage; the chain is then launched kernel by kernel instead of from its graph, with the same results). */
SL_API int sl_batch_set_timing(sl_batch* b, int enabled);
/* Renders n_views views: view v draws frames[v] of scene scene_of_view[v], eyes[3v..3v+2] its camera position (the
 * lit radiance's view direction), light_scales[v] (NULL = all 1) the intensity scale of every light of its scene
 * (emitters and distant lights; the sky ambient is unscaled) -- the same radiance as sl_lighting_set_emitters with
 * scale x light_scale and sl_lighting_set_environment with each irradiance x light_scale.  Images are packed in view order into out_dev (device memory, or page-locked host
 * memory that the compositor writes in place over the host link; float RGBA, out_floats floats at least 4 x the sum
 * of W x H); view_offsets[v] (optional, host) receives the first float of view v.  The
 * call returns after the batch completed; stats (optional) describe it. */
SL_API int sl_batch_render(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames,
                           const float* eyes, const float* light_scales, uint32_t n_views, float* out_dev,
                           uint64_t out_floats, uint64_t* view_offsets, sl_batch_stats* stats, void* stream);
/* Debug read-back of view `view` of the last batch, in that view's own indices (as sl_renderer_read_debug):
 * order (n slots), ranges (2 per tile), entries (the tile lists' slots, entries_cap at least *n_entries).  Any
 * pointer may be NULL. */
SL_API int sl_batch_read_view(sl_batch* b, uint32_t view, uint32_t* order, uint32_t* ranges, uint32_t* entries,
                              uint64_t entries_cap, uint64_t* n_entries);
/* Picks the fastest tile shape for this batch of views (renders it with each of 16x16, 8x32, 32x8, timed on the
 * device, `reps` times each) and keeps it; writes the per-shape times (ms) to ms_out[3] if not NULL.  Then, with that
 * shape, picks each of bproject's, btile_bin's, bshade's and bcomposite's block-size variant (the blocks per SM its
 * register budget is compiled for) by the device time of its stage, one kernel after the other. */
SL_API int sl_batch_autotune(sl_batch* b, const uint32_t* scene_of_view, const sl_render_frame* frames,
                             const float* eyes, const float* light_scales, uint32_t n_views, float* out_dev,
                             uint64_t out_floats, uint32_t reps, uint32_t* tile_w, uint32_t* tile_h, float* ms_out,
                             void* stream);

/* The batch's tuning: tile shape and, per kernel (bproject, btile_bin, bshade, bcomposite), the blocks per SM of
 * the variant in use (min_blocks[4]).  Any pointer may be NULL. */
SL_API int sl_batch_get_tuning(sl_batch* b, uint32_t* tile_w, uint32_t* tile_h, uint32_t* min_blocks);
/* Sets the block-size variants by their blocks per SM (min_blocks[4], as sl_batch_get_tuning reports them; bproject
 * 4 or 3, btile_bin 4 or 5, bshade 4, 3 or 5, bcomposite 6 or 5; SL_ERR_INVALID_ARG for any other).  Every variant
 * computes the same results. */
SL_API int sl_batch_set_tuning(sl_batch* b, const uint32_t* min_blocks);

/* ---- differentiable rendering (no counterpart in the reference) ------------------------------------------------- */

/* An inverse-rendering step over free per-Gaussian parameters: the forward projects them as the splat path does
 * (view-space covariance, 2D conic with the low-pass dilation, peak optical depth tau0 = softplus(opacity logit)
 * sqrt(det0/det) / (s0 sqrt(q_d)); shaders/project.wgsl:234-261 with kappa = softplus(logit) / (sqrt(2 pi) s0)),
 * lights each Gaussian as the product's shading pass does with emissive Gaussian lights (shade_leaf,
 * runtime/wgsl/emissive.wgsl:853-980: the light cut over the emitter tree built from the lights, intensity
 * Le scale sqrt(w^T M w), V grid, footprint transfer, SGGX specular lobe with its iso damping; the receiver's leaf
 * quantities follow from its parameters, the flake from its roughness), times the receiver's opacity-map
 * transmittance and iso_norm (per-scene lighting state: inputs, held constant), plus albedo x ambient, and composites
 * front to back with alpha = min(1 - exp(-tau0 e^{-q/2}), 0.99), fragments of optical depth below 1e-6 skipped and a
 * pixel stopping before its transmittance would fall below 1e-4 (16x16 tiles, the same depth keys and stable sort).
 * The backward of L = sum over pixels and rgb of (image - target)^2 walks each tile list back to front, recovering
 * transmittance from the final value (no per-pixel fragment lists), then the projection's chain rule (hand-written)
 * and the lighting's Jacobian (forward-mode dual numbers through the same lighting code, one parameter direction at
 * a time; the light intensities through the emitter tree's derivative tables).  The ASG light-shape highlight is
 * not part of this model.  Parameter and gradient arrays are device pointers. */
typedef struct sl_diff sl_diff;

typedef struct sl_diff_scene {
  const float* means;            /* n x 3, world */
  const float* log_scales;       /* n x 3 */
  const float* quats;            /* n x 4 (x, y, z, w), normalised in the forward */
  const float* opacity_logits;   /* n */
  const float* albedo;           /* n x 3 */
  const float* roughness;        /* n, > 0 */
  uint32_t n, n_lights;          /* n_lights <= 32 */
  const sl_gaussian* lights;     /* HOST, n_lights emissive Gaussians (world space; albedo = Le at intensity 1) */
  const float* light_scale;      /* n_lights: the intensities being optimised (each multiplies its light's Le) */
  float ambient, ks;             /* albedo x ambient added to every Gaussian; the specular weight of every material */
  const sl_vgrid* vgrid;         /* n V grids, or NULL (every direction visible) */
  const float* lamp_T;           /* n: the opacity-map transmittance toward the lights, or NULL (1) */
  const float* iso_norm;         /* n: iso_init's normalisation, or NULL (1) */
} sl_diff_scene;

typedef struct sl_diff_grads {   /* same shapes as the parameters; every array is overwritten */
  float *means, *log_scales, *quats, *opacity_logits, *albedo, *roughness, *light_scale;
} sl_diff_grads;

SL_API int sl_diff_create(uint32_t n, sl_diff** out);
SL_API int sl_diff_destroy(sl_diff* d);
/* The forward alone: W x H x 4 RGBA (alpha = 1 - T) into image_dev.  Camera, viewport, near/far and low-pass from
 * frame; eye = the camera position for the shading. */
SL_API int sl_diff_forward(sl_diff* d, const sl_diff_scene* scene, const sl_render_frame* frame, const float* eye,
                           float* image_dev, void* stream);
/* Forward + backward against target_dev (W x H x 4; rgb used): gradients into grads, the loss to *loss, the image to
 * image_dev if not NULL.  Returns after the step completed. */
SL_API int sl_diff_step(sl_diff* d, const sl_diff_scene* scene, const sl_render_frame* frame, const float* eye,
                        const float* target_dev, float* image_dev, const sl_diff_grads* grads, double* loss,
                        void* stream);
/* The depth order of the last forward (host; n_visible entries, far to near). */
SL_API int sl_diff_read_order(sl_diff* d, uint32_t* order, uint32_t* n_visible);

/* ---- serving (no counterpart in the reference) ----------------------------------------------------------------- */

/* A request server over resident scenes: requests (scene, RenderFrame, eye, light-intensity scale) arrive from any
 * thread and are rendered by continuous batching -- a worker thread admits pending requests, first come first
 * served, into the next batch of a free pipeline while the batch's slots, tiles and pixels fit its limits, launches
 * it (the batched chain of sl_batch_render, as a replayed graph) and copies each image into a pinned result slot.
 * With two or more pipelines a batch forms and launches while earlier ones run, so their work overlaps on the
 * device.  Each result equals sl_batch_render of that request alone (same tile shape), whatever else shares its
 * batch.  Device memory is fixed at creation (scenes + pipelines); a request whose footprint exceeds an empty batch
 * is refused at submit (SL_ERR_ADMISSION).  The renderers and lightings must stay unchanged while the server runs. */
typedef struct sl_server sl_server;

typedef struct sl_server_options {
  uint32_t max_views;            /* requests per batch (0 = 64, at most 256) */
  uint32_t pipelines;            /* batches in flight (0 = 2, at most 8) */
  uint64_t max_slots;            /* padded slots per batch (0 = 32 Mi) */
  uint64_t max_pixels;           /* image pixels per batch (0 = 32 Mi) */
  uint64_t max_view_pixels;      /* pixels of one request (0 = 1920 x 1080): the size of a result slot */
  uint64_t hbm_budget_bytes;     /* device memory the pipelines may take (0 = unchecked) */
  uint32_t max_tiles;            /* tiles per batch (0 = 512 Ki) */
  uint32_t result_slots;         /* pinned result slots (0 = 2 x max_views) */
  uint32_t tile_w, tile_h;       /* 16x16 (default), 8x32 or 32x8 */
  uint32_t max_pending;          /* requests waiting for admission (0 = unbounded); beyond it submit refuses
                                    (SL_ERR_ADMISSION), which bounds the latency of what is admitted under overload */
  uint32_t pad;
} sl_server_options;

typedef struct sl_server_request {
  uint32_t scene;                /* index into the server's scenes */
  float eye[3];                  /* camera position (lit radiance) */
  float light_scale;             /* intensity scale of the scene's lights (1 = as set) */
  uint32_t pad;
  sl_render_frame frame;
} sl_server_request;

typedef struct sl_server_result {
  uint64_t tag;                  /* the submit's tag */
  int32_t status;                /* SL_OK, or why the request failed (SL_ERR_CANCELLED: never admitted) */
  uint32_t batch_views;          /* requests in the batch it ran in */
  uint32_t width, height;
  uint32_t result_slot;          /* release with sl_server_release after reading the image */
  uint32_t pad;
  double t_submit, t_start, t_done; /* seconds since the server started: submitted, launched, results ready */
  const float* image;            /* height x width x 4 linear RGBA in pinned host memory (NULL on failure) */
} sl_server_result;

typedef struct sl_server_stats {
  uint64_t submitted, completed, rejected, failed, batches, batch_views, graph_replays, pending;
  uint64_t device_bytes;         /* scenes + pipeline buffers */
  uint64_t free_result_slots;
  uint64_t reshaded_views;       /* views re-run with every blended splat shaded (sl_batch_stats.reshaded_views) */
  uint64_t relaunches;           /* batches launched again (tile entries beyond the capacity class, or a re-shade) */
} sl_server_stats;

SL_API int sl_server_create(sl_renderer* const* renderers, sl_lighting* const* lightings, uint32_t n_scenes,
                            const sl_server_options* opt, sl_server** out);
/* Queues one request (validated here: SL_ERR_INVALID_ARG, or SL_ERR_ADMISSION when it can never fit a batch or the
 * pending queue is full). */
SL_API int sl_server_submit(sl_server* s, const sl_server_request* req, uint64_t tag);
/* Up to cap finished results (waits up to wait_us microseconds for the first); *n_out = how many. */
SL_API int sl_server_poll(sl_server* s, sl_server_result* out, uint32_t cap, uint32_t* n_out, uint32_t wait_us);
/* Returns a result slot to the pool (its image pointer is invalid afterwards). */
SL_API int sl_server_release(sl_server* s, uint32_t result_slot);
SL_API int sl_server_get_stats(sl_server* s, sl_server_stats* stats);
/* Stops accepting requests, finishes the admitted and pending ones while result slots last (the rest are cancelled),
 * and frees everything. */
SL_API int sl_server_destroy(sl_server* s);

#ifdef __cplusplus
}
#endif

#endif /* SPLATLIGHT_H */
