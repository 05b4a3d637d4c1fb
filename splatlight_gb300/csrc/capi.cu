// C ABI of the splat pipeline: renderer object, asset layout checks, per-frame orchestration.
// The per-frame chain (sl_render) is stream-ordered and launches, in order:
//   project  -> onesweep pass x2 (depth keys) -> tile counts -> scan -> tile emit -> onesweep pass x1-2 (tile ids)
//   -> scan (tile starts) -> ranges -> composite
// with one synchronisation at the end (frame counters: visible, entries, overflow, timeout); the tile sort reads the
// entry count on the device.  If the tile-entry capacity was too small the frame is re-run after growing it.
#include <cstdio>
#include <cstring>
#include <string>

#include "sl_runtime.h"

namespace sl {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  set_error(m);
  return e == cudaErrorMemoryAllocation ? SL_ERR_OOM : SL_ERR_CUDA;
}

void ViewBuffers::release_all() {
  DevBuf* all[] = {&key16,    &recs,       &rects,        &order,    &bin_scratch, &keys_alt, &vals_alt,
                   &status,   &tile_ctr,   &tile_keys,    &tile_vals, &ranges,      &digit_hist, &scan_scratch,
                   &counters, &out,        &counts,       &key_hist};
  for (DevBuf* b : all) b->release();
}

}  // namespace sl

using namespace sl;

#define SL_CHECK_CUDA(expr, what)                 \
  do {                                            \
    cudaError_t _e = (expr);                      \
    if (_e != cudaSuccess) return cuda_fail(_e, what); \
  } while (0)

extern "C" {

size_t sl_last_error(char* buf, size_t cap) {
  const std::string& s = g_last_error;
  if (buf && cap) {
    size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
    memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return s.size();
}

int sl_version(void) { return 100; }

// ---- asset layout (src/asset.js:8-38) ----------------------------------------------------------------------------

struct FieldSpec {
  const char* name;
  uint32_t offset;
};
struct BufferSpec {
  const char* name;
  uint32_t stride;
  FieldSpec fields[10];
  int n_fields;
};
static const BufferSpec kLayout[] = {
    {"gaussians", 64, {{"mu", 0}, {"kappa", 12}, {"quat", 16}, {"scale", 32}, {"part_surface", 44}, {"albedo", 48}}, 6},
    {"parts", 128, {{"xf", 0}, {"xf_prev", 48}, {"bound", 96}, {"root", 112}, {"g_lo", 116}, {"g_hi", 120}, {"flags", 124}}, 7},
    {"lamps", 96, {{"center", 0}, {"kind", 12}, {"e1", 16}, {"radius", 28}, {"e2", 32}, {"normal", 48}, {"radiance", 64}, {"center_prev", 80}}, 8},
    {"materials", 32, {{"flake", 0}, {"phase_samples", 12}, {"vfloor", 16}, {"flags", 20}}, 4},
    {"nodes", 96, {}, 0},
    {"kids", 4, {}, 0},
    {"vgrid", 128, {}, 0},
};

int sl_asset_check_header(const char* format, const char* version) {
  // src/asset.js:19: header.format !== 'gs-runtime'
  if (!format || strcmp(format, "gs-runtime") != 0)
    return fail(SL_ERR_LAYOUT, std::string("Unknown asset format ") + (format ? format : "undefined"));
  // src/asset.js:20: String(header.version).split('.')[0] !== MAJOR ('0')
  std::string v = version ? version : "undefined";
  if (v.substr(0, v.find('.')) != "0") return fail(SL_ERR_LAYOUT, "Unsupported asset version " + v);
  return SL_OK;
}

int sl_asset_check_buffer(const char* name, uint32_t stride, uint32_t count, const char* const* field_names,
                          const uint32_t* field_offsets, uint32_t n_fields) {
  if (!name) return fail(SL_ERR_INVALID_ARG, "buffer name is null");
  const BufferSpec* spec = nullptr;
  for (const BufferSpec& b : kLayout)
    if (strcmp(b.name, name) == 0) spec = &b;
  if (!spec) return fail(SL_ERR_LAYOUT, std::string("Asset has no ") + name + " buffer");
  if (stride != spec->stride)
    return fail(SL_ERR_LAYOUT, std::string(name) + " stride " + std::to_string(stride) + ", renderer expects " +
                                   std::to_string(spec->stride));
  for (int f = 0; f < spec->n_fields; f++) {
    uint32_t got = UINT32_MAX;
    for (uint32_t k = 0; k < n_fields; k++)
      if (field_names && field_names[k] && strcmp(field_names[k], spec->fields[f].name) == 0)
        got = field_offsets ? field_offsets[k] : UINT32_MAX;
    if (got != spec->fields[f].offset)
      return fail(SL_ERR_LAYOUT, std::string(name) + "." + spec->fields[f].name + " at " +
                                     (got == UINT32_MAX ? std::string("undefined") : std::to_string(got)) +
                                     ", renderer expects " + std::to_string(spec->fields[f].offset));
  }
  if (count == 0 || count > (1u << 24))
    return fail(SL_ERR_LAYOUT, std::string("Bad ") + name + " count " + std::to_string(count));
  return SL_OK;
}

int sl_asset_check_bytes(uint64_t byte_length, uint32_t count, uint32_t stride) {
  if (byte_length != (uint64_t)count * stride)
    return fail(SL_ERR_LAYOUT, "buffer is " + std::to_string(byte_length) + " B, expected " + std::to_string(count) +
                                   " x " + std::to_string(stride) + " B");
  return SL_OK;
}

// ---- renderer ------------------------------------------------------------------------------------------------------

static int check_device() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  cudaDeviceProp p;
  e = cudaGetDeviceProperties(&p, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
  if (p.major != 10 || p.minor != 3)
    return fail(SL_ERR_NO_DEVICE, "libsplatlight is built for sm_103a; device is sm_" + std::to_string(p.major) +
                                      std::to_string(p.minor));
  return SL_OK;
}

int sl_renderer_create(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                       uint32_t max_emitters, sl_renderer** out) {
  if (!out) return fail(SL_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  if (!gaussians || count == 0 || count > (1u << 24)) return fail(SL_ERR_INVALID_ARG, "bad Gaussian count");
  if (!parts || part_count == 0 || part_count > kMaxParts) return fail(SL_ERR_INVALID_ARG, "bad part count");
  if (max_emitters > 16384) return fail(SL_ERR_INVALID_ARG, "max_emitters > 16384 (MAX_EMITTERS)");
  for (uint32_t i = 0; i < count; i++) {
    uint32_t p = gaussians[i].part_surface & 0xffffu;
    if (p > kMaxParts - 1) p = kMaxParts - 1;
    if (p >= part_count)
      return fail(SL_ERR_INVALID_ARG, "Gaussian " + std::to_string(i) + " references part " + std::to_string(p) +
                                          " of " + std::to_string(part_count));
  }
  int rc = check_device();
  if (rc) return rc;
  sl_renderer* r = new sl_renderer();
  cudaGetDevice(&r->device);
  r->count = count;
  r->part_count = part_count;
  r->max_emitters = max_emitters;
  r->parts.assign(parts, parts + part_count);
  cudaError_t e = r->gaussians.ensure(sizeof(sl_gaussian) * (size_t)count);
  if (e == cudaSuccess) e = cudaMemcpy(r->gaussians.ptr, gaussians, sizeof(sl_gaussian) * (size_t)count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = r->emitters.ensure(sizeof(sl_gaussian) * (size_t)(max_emitters ? max_emitters : 1));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&r->host_ctr, sizeof(FrameCounters));
  if (e != cudaSuccess) {
    r->gaussians.release();
    r->emitters.release();
    delete r;
    return cuda_fail(e, "sl_renderer_create");
  }
  *out = r;
  return SL_OK;
}

int sl_renderer_destroy(sl_renderer* r) {
  if (!r) return SL_OK;
  cudaSetDevice(r->device);
  cudaDeviceSynchronize();
  if (r->lod) r->lod->r = nullptr;  // the LOD outlives its renderer only as an empty handle
  r->vb.release_all();
  r->gaussians.release();
  r->emitters.release();
  for (cudaEvent_t& ev : r->tm.ev)
    if (ev) cudaEventDestroy(ev);
  if (r->host_ctr) cudaFreeHost(r->host_ctr);
  delete r;
  return SL_OK;
}

int sl_renderer_set_parts(sl_renderer* r, const sl_part* parts, uint32_t part_count) {
  if (!r || !parts) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (part_count != r->part_count) return fail(SL_ERR_INVALID_ARG, "part count differs from the asset's");
  r->parts.assign(parts, parts + part_count);
  return SL_OK;
}

int sl_renderer_set_emitters(sl_renderer* r, const sl_gaussian* emitters, uint32_t n) {
  if (!r || (n && !emitters)) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n > r->max_emitters) return fail(SL_ERR_INVALID_ARG, "more emitters than max_emitters");
  cudaSetDevice(r->device);
  if (n) SL_CHECK_CUDA(cudaMemcpy(r->emitters.ptr, emitters, sizeof(sl_gaussian) * n, cudaMemcpyHostToDevice), "emitters");
  r->n_emitters = n;
  return SL_OK;
}

int sl_renderer_bind_colour(sl_renderer* r, const float* colour_dev, const float* lo_b_dev) {
  if (!r) return fail(SL_ERR_INVALID_ARG, "null renderer");
  r->colour = reinterpret_cast<const float4*>(colour_dev);
  r->lo_b = reinterpret_cast<const float4*>(lo_b_dev);
  return SL_OK;
}

int sl_renderer_set_options(sl_renderer* r, const sl_render_options* opt) {
  if (!r || !opt) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (opt->tile_w || opt->tile_h) {
    bool ok = (opt->tile_w == 16 && opt->tile_h == 16) || (opt->tile_w == 8 && opt->tile_h == 32) ||
              (opt->tile_w == 32 && opt->tile_h == 8);
    if (!ok) return fail(SL_ERR_INVALID_ARG, "tile shape must be 16x16, 8x32 or 32x8");
    r->tile_w = opt->tile_w;
    r->tile_h = opt->tile_h;
  }
  if (opt->t_stop > 0.0f) r->t_stop_scale = opt->t_stop;
  if (opt->entry_capacity) r->entry_capacity = opt->entry_capacity;
  if (opt->sort_mode > 2u) return fail(SL_ERR_INVALID_ARG, "sort_mode must be 0 (keep), 1 (stable) or 2 (counting)");
  if (opt->sort_mode) r->sort_mode = opt->sort_mode;
  return SL_OK;
}

int sl_renderer_set_timing(sl_renderer* r, int on) {
  if (!r) return fail(SL_ERR_INVALID_ARG, "null renderer");
  cudaSetDevice(r->device);
  if (on && !r->tm.ev[0])
    for (cudaEvent_t& ev : r->tm.ev) SL_CHECK_CUDA(cudaEventCreate(&ev), "cudaEventCreate");
  r->timing = on != 0;
  return SL_OK;
}

}  // extern "C"

// ---- frame validation and parameter packing -------------------------------------------------------------------------

namespace sl {

int check_frame(const sl_render_frame* f, uint32_t count, uint32_t n_emitters, const sl_lod* lod) {
  if (f->count != count) return fail(SL_ERR_INVALID_ARG, "frame.count differs from the renderer's Gaussian count");
  if (!(f->viewport[0] >= 1.0f && f->viewport[1] >= 1.0f && f->viewport[0] <= 16384.0f && f->viewport[1] <= 16384.0f) ||
      f->viewport[0] != (float)(uint32_t)f->viewport[0] || f->viewport[1] != (float)(uint32_t)f->viewport[1])
    return fail(SL_ERR_INVALID_ARG, "viewport must be whole pixels in [1, 16384]");
  if (!(f->near_plane > 0.0f) || !(f->far_plane > f->near_plane))
    return fail(SL_ERR_INVALID_ARG, "need 0 < near < far");
  if (!(f->focal[0] > 0.0f) || !(f->focal[1] > 0.0f)) return fail(SL_ERR_INVALID_ARG, "focal must be positive");
  if (f->view_mode > 3u) return fail(SL_ERR_INVALID_ARG, "view_mode must be 0..3");
  float ne = f->palette[3][1];
  if (!(ne >= 0.0f) || (uint32_t)ne > n_emitters)
    return fail(SL_ERR_INVALID_ARG, "frame emitter count (palette[3].y) exceeds the emitters set");
  if (f->lamp[3] > 0.5f) return fail(SL_ERR_UNSUPPORTED, "camera-only flakes (lamp.w = 1) are outside this pipeline");
  if ((uint32_t)(f->lamp_color[3] + 0.5f) != 0u)
    return fail(SL_ERR_UNSUPPORTED, "reflection coverage / Fresnel (lamp_color.w) are outside this pipeline");
  if (f->lod[0] != 0u) {
    if (!lod)
      return fail(SL_ERR_UNSUPPORTED, "screen-space LOD (frame.lod) needs sl_lod_create on this renderer (and is not "
                                      "batched)");
    if ((uint64_t)f->lod[1] < (uint64_t)count + 1u + (uint32_t)ne || f->lod[2] != lod->n_int ||
        (uint64_t)f->lod[1] + f->lod[2] > 0x7FFFFFFFull)
      return fail(SL_ERR_INVALID_ARG, "frame.lod: the node slot base must follow the frame's emitters and the node "
                                      "count must be the tree's internal node count");
  }
  if (f->explode_k[2] > 0.5f) return fail(SL_ERR_UNSUPPORTED, "explode is outside this pipeline");
  if (f->particles[1] != 0u) return fail(SL_ERR_UNSUPPORTED, "Gaussian particles are outside this pipeline");
  return SL_OK;
}

void pack_project_params(const sl_render_frame* f, const std::vector<sl_part>& parts, uint32_t count,
                         uint32_t n_emit, uint32_t tile_w, uint32_t tile_h, ProjectParams& P) {
  memset(&P, 0, sizeof(P));
  memcpy(P.view, f->view, sizeof(P.view));
  P.focal[0] = f->focal[0];
  P.focal[1] = f->focal[1];
  P.viewport[0] = f->viewport[0];
  P.viewport[1] = f->viewport[1];
  P.near_plane = f->near_plane;
  P.far_plane = f->far_plane;
  P.lowpass_px2 = f->lowpass_px2;
  P.albedo_scale = f->albedo_scale;
  P.bounce_gain = f->palette[3][0];
  P.shutter = f->palette[3][2];
  P.blur_cov = f->palette[3][3] > 0.5f ? 1u : 0u;
  P.count = count;
  P.n_emit = n_emit;
  P.n_slots = count + 1u + n_emit;
  P.view_mode = f->view_mode;
  P.part_count = (uint32_t)parts.size();
  P.tile_w = tile_w;
  P.tile_h = tile_h;
  uint32_t W = (uint32_t)f->viewport[0], H = (uint32_t)f->viewport[1];
  P.tiles_x = (W + tile_w - 1) / tile_w;
  P.tiles_y = (H + tile_h - 1) / tile_h;
  for (int m = 0; m < 8; m++) {
    const float* src = m < 3 ? f->palette[m] : (m >= 4 ? f->palette_ext[m - 4] : nullptr);
    float white[4] = {1.0f, 1.0f, 1.0f, 0.0f};
    memcpy(P.palette[m], src ? src : white, sizeof(float) * 4);
  }
  for (uint32_t p = 0; p < kMaxParts; p++) {
    PartXf& x = P.parts[p];
    if (p < parts.size()) {
      memcpy(x.xf, parts[p].xf, sizeof(x.xf));
      memcpy(x.xf_prev, parts[p].xf_prev, sizeof(x.xf_prev));
      x.flags = parts[p].flags;
    } else {
      x.flags = kPartHidden;
    }
    x.material = p < 16 ? f->part_material[p] : f->part_material_ext[p - 16];
    float fade = f->part_fade[p];
    fade = fade < 0.0f ? 0.0f : (fade > 1.0f ? 1.0f : fade);
    x.keep = 1.0f - fade;
  }
}

static int bits_for(uint32_t v) {
  int b = 0;
  while ((1u << b) <= v && b < 32) b++;
  return b < 1 ? 1 : b;
}

// Sizes every per-view buffer for n slots, `tiles` tiles and `cap` entries.
static cudaError_t ensure_view_buffers(ViewBuffers& vb, uint32_t n, uint32_t tiles, uint64_t cap, uint32_t pixels,
                                       bool need_out, bool need_counts) {
  cudaError_t e;
#define ENS(buf, bytes) \
  if ((e = (buf).ensure(bytes)) != cudaSuccess) return e
  ENS(vb.key16, 2ull * n + 16);
  ENS(vb.recs, sizeof(SplatRec) * (size_t)n);
  ENS(vb.rects, 8ull * n);
  ENS(vb.order, 4ull * n + 16);
  ENS(vb.bin_scratch, tile_bin_scratch_bytes(n));
  uint64_t big = cap > n ? cap : n;
  ENS(vb.keys_alt, 2 * big + 16);
  ENS(vb.vals_alt, 4 * big + 16);
  ENS(vb.status, 4ull * 256 * 2 * (sort_tiles_for((uint32_t)big) + 1));
  ENS(vb.tile_ctr, 16);
  ENS(vb.tile_keys, 2 * cap + 16);
  ENS(vb.tile_vals, 4 * cap + 16);
  ENS(vb.ranges, 8ull * tiles + 16);
  ENS(vb.digit_hist, 4ull * 4 * 256);
  ENS(vb.key_hist, 2 * 4ull * 65536);
  ENS(vb.scan_scratch, scan_scratch_bytes(65536u));  // the counting sort's 65536 key offsets
  ENS(vb.counters, sizeof(FrameCounters));
  if (need_out) ENS(vb.out, 16ull * pixels);
  if (need_counts) ENS(vb.counts, 4ull * pixels);
#undef ENS
  return cudaSuccess;
}

// One attempt at a frame; returns SL_OK, SL_ERR_OVERFLOW (grow and retry) or an error.
static int render_once(sl_renderer* r, const sl_render_frame* f, float4* out_dev, uint32_t* counts_dev,
                       cudaStream_t s, sl_render_stats* stats) {
  const uint32_t n_emit = (uint32_t)f->palette[3][1];
  ProjectParams P;
  pack_project_params(f, r->parts, r->count, n_emit, r->tile_w, r->tile_h, P);
  LodDraw lod{nullptr, nullptr, nullptr};
  if (f->lod[0] != 0u) {  // screen-space LOD: the tree's internal nodes take the slots from frame.lod[1]
    P.lod_on = 1u;
    P.node_base = f->lod[1];
    P.n_int = f->lod[2];
    P.n_slots = P.node_base + P.n_int;
    lod = LodDraw{r->lod->flags.as<uint32_t>(), r->lod->records.as<sl_gaussian>(), r->lod->colour.as<float4>()};
  }
  const uint32_t n = P.n_slots;
  const uint32_t tiles = P.tiles_x * P.tiles_y;
  const uint32_t W = (uint32_t)f->viewport[0], H = (uint32_t)f->viewport[1];
  if (tiles > 65535u) return fail(SL_ERR_INVALID_ARG, "too many tiles for 16-bit tile keys");
  if (r->entry_capacity == 0) r->entry_capacity = (uint64_t)n * 4 + 4096;
  const uint64_t cap = r->entry_capacity;
  ViewBuffers& vb = r->vb;
  FrameCounters* ctr = vb.counters.as<FrameCounters>();
  uint32_t* hist = vb.digit_hist.as<uint32_t>();
  SortScratch sc{vb.keys_alt.as<uint16_t>(), vb.vals_alt.as<uint32_t>(), vb.status.as<uint32_t>(),
                 vb.tile_ctr.as<uint32_t>(), (uint32_t)(vb.status.bytes / (4ull * 256 * 2))};
  const float4* colour = r->colour;
  const float4* lo_b = r->lo_b;
  cudaEvent_t* ev = r->timing ? r->tm.ev : nullptr;

  if (ev) SL_CHECK_CUDA(cudaEventRecord(ev[0], s), "event");
  SL_CHECK_CUDA(cudaMemsetAsync(ctr, 0, sizeof(FrameCounters), s), "memset counters");
  SL_CHECK_CUDA(cudaMemsetAsync(hist, 0, 4 * 4 * 256, s), "memset hist");
  SL_CHECK_CUDA(cudaMemsetAsync(vb.ranges.ptr, 0, 8ull * tiles, s), "memset ranges");
  SL_CHECK_CUDA(launch_project(P, r->gaussians.as<sl_gaussian>(), r->emitters.as<sl_gaussian>(), colour, lo_b,
                               vb.key16.as<uint16_t>(), vb.recs.as<SplatRec>(), vb.rects.as<ushort4>(), hist, ctr, s,
                               lod),
                "project");
  if (ev) SL_CHECK_CUDA(cudaEventRecord(ev[1], s), "event");
  if (r->sort_mode == 2u) {  // counting sort (scan.wgsl, scatter.wgsl): ties land in arbitrary order
    SL_CHECK_CUDA(cudaMemsetAsync(vb.key_hist.ptr, 0, 4ull * 65536, s), "memset key histogram");
    SL_CHECK_CUDA(launch_key_hist(vb.key16.as<uint16_t>(), n, vb.key_hist.as<uint32_t>(), s), "key histogram");
    uint32_t* offsets = vb.key_hist.as<uint32_t>() + 65536;
    SL_CHECK_CUDA(exclusive_scan_u32(vb.key_hist.as<uint32_t>(), offsets, 65536, nullptr, vb.scan_scratch.ptr, ctr, s),
                  "key offsets");
    SL_CHECK_CUDA(launch_key_scatter(vb.key16.as<uint16_t>(), n, offsets, vb.order.as<uint32_t>(), s), "key scatter");
  } else {
    SL_CHECK_CUDA(sort16_pairs(vb.key16.as<uint16_t>(), nullptr, vb.order.as<uint32_t>(), n, nullptr, 16, hist, sc,
                               ctr, s),
                  "depth sort");
  }
  if (ev) SL_CHECK_CUDA(cudaEventRecord(ev[2], s), "event");
  SL_CHECK_CUDA(launch_tile_bin(vb.order.as<uint32_t>(), vb.rects.as<ushort4>(), vb.recs.as<SplatRec>(), n,
                                P.tiles_x, P.tile_w, P.tile_h, (uint32_t)(cap > 0xffffffffull ? 0xffffffffu : cap), ctr,
                                vb.tile_keys.as<uint16_t>(), vb.tile_vals.as<uint32_t>(), hist + 512,
                                vb.bin_scratch.ptr, s),
                "tile binning");
  // the entry count is only known on the device: the tile sort reads it there (grid sized for the capacity)
  const uint32_t cap32 = (uint32_t)(cap > 0xffffffffull ? 0xffffffffu : cap);
  SL_CHECK_CUDA(sort16_pairs(vb.tile_keys.as<uint16_t>(), vb.tile_vals.as<uint32_t>(), vb.tile_vals.as<uint32_t>(),
                             cap32, &ctr->entries, bits_for(tiles - 1), hist + 512, sc, ctr, s,
                             vb.tile_keys.as<uint16_t>()),
                "tile sort");
  SL_CHECK_CUDA(launch_tile_ranges(vb.tile_keys.as<uint16_t>(), &ctr->entries, cap32, vb.ranges.as<uint2>(), s),
                "tile ranges");
  if (ev) SL_CHECK_CUDA(cudaEventRecord(ev[3], s), "event");
  CompositeParams C;
  C.width = W;
  C.height = H;
  C.tile_w = r->tile_w;
  C.tile_h = r->tile_h;
  C.tiles_x = P.tiles_x;
  C.tiles_y = P.tiles_y;
  C.count_mode = f->view_mode == 2u ? 1u : 0u;
  C.t_stop_scale = r->t_stop_scale;
  SL_CHECK_CUDA(launch_composite(C, vb.ranges.as<uint2>(), vb.tile_vals.as<uint32_t>(), vb.recs.as<SplatRec>(), ctr,
                                 out_dev, counts_dev, s),
                "composite");
  if (ev) SL_CHECK_CUDA(cudaEventRecord(ev[4], s), "event");
  SL_CHECK_CUDA(cudaMemcpyAsync(r->host_ctr, ctr, sizeof(FrameCounters), cudaMemcpyDeviceToHost, s), "counters");
  r->last_slots = n;
  r->last_w = W;
  r->last_h = H;
  r->last_tiles = tiles;
  r->last_mode = f->view_mode;
  if (stats) {
    stats->slots = n;
    stats->tiles = tiles;
  }
  return SL_OK;
}

}  // namespace sl

extern "C" {

int sl_render(sl_renderer* r, const sl_render_frame* f, float* out_rgba, int out_on_device, sl_render_stats* stats,
              void* stream) {
  if (!r || !f || !out_rgba) return fail(SL_ERR_INVALID_ARG, "null argument");
  int rc = check_frame(f, r->count, r->n_emitters, r->lod);
  if (rc) return rc;
  cudaSetDevice(r->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const uint32_t n_emit = (uint32_t)f->palette[3][1];
  // slots: the scene, the lamp marker, the frame's emitters; with LOD on, up to the end of the tree's node slots
  const uint32_t n = f->lod[0] != 0u ? f->lod[1] + f->lod[2] : r->count + 1u + n_emit;
  const uint32_t W = (uint32_t)f->viewport[0], H = (uint32_t)f->viewport[1];
  const uint32_t tiles = ((W + r->tile_w - 1) / r->tile_w) * ((H + r->tile_h - 1) / r->tile_h);
  const bool count_mode = f->view_mode == 2u;
  for (int attempt = 0; attempt < 3; attempt++) {
    if (r->entry_capacity == 0) r->entry_capacity = (uint64_t)n * 4 + 4096;
    cudaError_t e = ensure_view_buffers(r->vb, n, tiles, r->entry_capacity, W * H, !out_on_device, count_mode);
    if (e != cudaSuccess) return cuda_fail(e, "allocating view buffers");
    float4* out_dev = out_on_device ? reinterpret_cast<float4*>(out_rgba) : r->vb.out.as<float4>();
    // a pinned (page-locked, device-mapped) host image: the compositor writes it in place over the host link, the
    // device-to-host read fused into the kernel that produces the image (no staging copy)
    bool direct = false;
    if (!out_on_device) {
      cudaPointerAttributes pa{};
      if (cudaPointerGetAttributes(&pa, out_rgba) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
          pa.devicePointer != nullptr && reinterpret_cast<uintptr_t>(pa.devicePointer) % 16 == 0) {
        out_dev = reinterpret_cast<float4*>(pa.devicePointer);
        direct = true;
      } else {
        cudaGetLastError();  // a pageable pointer is not an error here
      }
    }
    uint32_t* counts_dev = count_mode ? r->vb.counts.as<uint32_t>() : nullptr;
    sl_render_stats local{};
    rc = render_once(r, f, out_dev, counts_dev, s, stats ? &local : nullptr);
    if (rc) return rc;
    if (!out_on_device && !direct)
      SL_CHECK_CUDA(cudaMemcpyAsync(out_rgba, out_dev, 16ull * W * H, cudaMemcpyDeviceToHost, s), "output copy");
    SL_CHECK_CUDA(cudaStreamSynchronize(s), "sync");
    const FrameCounters& hc = *r->host_ctr;
    if (hc.overflow || hc.entries > r->entry_capacity) {  // too many tile entries: grow and render again
      r->entry_capacity = (uint64_t)hc.entries + hc.entries / 4 + 4096;
      continue;
    }
    r->last_entries = hc.entries;
    local.entries = hc.entries;
    r->have_frame = true;
    if (stats) {
      *stats = local;
      stats->visible = hc.visible;
      stats->fragments = hc.fragments;
      if (r->timing) {
        float ms[4] = {0, 0, 0, 0};
        cudaEventElapsedTime(&ms[0], r->tm.ev[0], r->tm.ev[1]);
        cudaEventElapsedTime(&ms[1], r->tm.ev[1], r->tm.ev[2]);
        cudaEventElapsedTime(&ms[2], r->tm.ev[2], r->tm.ev[3]);
        cudaEventElapsedTime(&ms[3], r->tm.ev[3], r->tm.ev[4]);
        stats->ms_project = ms[0];
        stats->ms_sort = ms[1];
        stats->ms_bin = ms[2];
        stats->ms_composite = ms[3];
        cudaEventElapsedTime(&stats->ms_total, r->tm.ev[0], r->tm.ev[4]);
      }
    }
    if (hc.timeout) return fail(SL_ERR_TIMEOUT, "a bounded device-side wait gave up (look-back or mbarrier)");
    return SL_OK;
  }
  return fail(SL_ERR_OVERFLOW, "tile entry capacity kept overflowing");
}

int sl_renderer_read_debug(sl_renderer* r, uint32_t* keys, uint32_t* order, uint32_t* ranges, uint32_t* counts) {
  if (!r) return fail(SL_ERR_INVALID_ARG, "null renderer");
  if (!r->have_frame) return fail(SL_ERR_INVALID_ARG, "no frame rendered yet");
  cudaSetDevice(r->device);
  const uint32_t n = r->last_slots;
  if (keys) {
    std::vector<uint16_t> k16(n);
    SL_CHECK_CUDA(cudaMemcpy(k16.data(), r->vb.key16.ptr, 2ull * n, cudaMemcpyDeviceToHost), "keys");
    for (uint32_t i = 0; i < n; i++) keys[i] = k16[i] == kInvalidKey16 ? 0xffffffffu : k16[i];
  }
  if (order) SL_CHECK_CUDA(cudaMemcpy(order, r->vb.order.ptr, 4ull * n, cudaMemcpyDeviceToHost), "order");
  if (ranges) {
    SL_CHECK_CUDA(cudaMemcpy(ranges, r->vb.ranges.ptr, 8ull * r->last_tiles, cudaMemcpyDeviceToHost), "ranges");
    // the device keeps [0, 0) for empty tiles; read back as the cumulative bounds of the tiles' lists in tile order
    // (an empty tile at the end of the lists before it)
    uint32_t at = 0;
    for (uint32_t t = 0; t < r->last_tiles; t++) {
      if (ranges[2 * t + 1] > ranges[2 * t]) at = ranges[2 * t + 1];
      else ranges[2 * t] = ranges[2 * t + 1] = at;
    }
  }
  if (counts) {
    if (r->last_mode != 2u) return fail(SL_ERR_INVALID_ARG, "contributor counts come from view mode 2");
    SL_CHECK_CUDA(cudaMemcpy(counts, r->vb.counts.ptr, 4ull * r->last_w * r->last_h, cudaMemcpyDeviceToHost), "counts");
  }
  return SL_OK;
}

int sl_renderer_read_entries(sl_renderer* r, uint32_t* entries, uint64_t cap) {
  if (!r || !entries) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (!r->have_frame) return fail(SL_ERR_INVALID_ARG, "no frame rendered yet");
  if (cap < r->last_entries) return fail(SL_ERR_INVALID_ARG, "entries buffer too small");
  cudaSetDevice(r->device);
  if (r->last_entries)
    SL_CHECK_CUDA(cudaMemcpy(entries, r->vb.tile_vals.ptr, 4ull * r->last_entries, cudaMemcpyDeviceToHost), "entries");
  return SL_OK;
}

}  // extern "C"
