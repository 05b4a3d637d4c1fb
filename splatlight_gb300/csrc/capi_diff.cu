// Differentiable rendering through the C ABI (sl_diff_*): the forward of diff.cu over caller-owned device parameter
// arrays, the shared depth sort and tile binning, and the backward of an L2 image loss into caller-owned gradient
// arrays -- one inverse-rendering step per call.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "sl_diff.h"
#include "sl_lighting.h"
#include "sl_runtime.h"

struct sl_diff {
  int device = 0;
  uint32_t n = 0;
  uint64_t entry_cap = 0;
  sl::ViewBuffers vb;
  sl::DevBuf drec, img, tfinal, ncontrib, dimg, g2, loss, target, tree, dtab;
  std::vector<float> h_tree, h_dtab;
  std::vector<double> h_scale;
  sl::FrameCounters* host_ctr = nullptr;
  double* host_loss = nullptr;
  uint32_t last_visible = 0, last_entries = 0, last_w = 0, last_h = 0;
};

namespace sl {
namespace {

int bits16(uint32_t v) {
  int b = 1;
  while (b < 16 && (1u << b) <= v) b++;
  return b;
}

int check_scene(const sl_diff_scene* sc, uint32_t n) {
  if (!sc || !sc->means || !sc->log_scales || !sc->quats || !sc->opacity_logits || !sc->albedo || !sc->roughness)
    return fail(SL_ERR_INVALID_ARG, "null parameter array");
  if (sc->n != n) return fail(SL_ERR_INVALID_ARG, "scene size differs from the diff object's");
  if (sc->n_lights > kMaxDiffLights || (sc->n_lights && (!sc->lights || !sc->light_scale)))
    return fail(SL_ERR_INVALID_ARG, "bad lights (at most 32)");
  return SL_OK;
}

// The emitter tree of the lights at their current intensities (read back from the device), with its derivative
// table, uploaded for this step.
int build_lights(sl_diff* d, const sl_diff_scene* sc, DiffLights& L, cudaStream_t s) {
  const uint32_t n = sc->n_lights;
  L.tree = dsh::EmitTree{nullptr, 0xFFFFFFFFu, 0u, 1u, 4.0f, 1.0f};
  L.dtab = nullptr;
  L.n = n;
  if (!n) return SL_OK;
  std::vector<float> scale(n);
  cudaError_t e = cudaMemcpyAsync(scale.data(), sc->light_scale, 4ull * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "light intensities");
  d->h_scale.assign(scale.begin(), scale.end());
  const uint32_t root = build_emitter_tree(reinterpret_cast<const float*>(sc->lights), n, d->h_scale.data(), d->h_tree,
                                           &d->h_dtab);
  if ((e = d->tree.ensure(4 * d->h_tree.size())) != cudaSuccess ||
      (e = d->dtab.ensure(4 * d->h_dtab.size())) != cudaSuccess ||
      (e = cudaMemcpyAsync(d->tree.ptr, d->h_tree.data(), 4 * d->h_tree.size(), cudaMemcpyHostToDevice, s)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(d->dtab.ptr, d->h_dtab.data(), 4 * d->h_dtab.size(), cudaMemcpyHostToDevice, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)  // the host vectors are rewritten by the next step
    return cuda_fail(e, "emitter tree");
  L.tree = dsh::EmitTree{d->tree.as<float>(), root, n, 1u, 4.0f, 1.0f};
  L.dtab = d->dtab.as<float>();
  return SL_OK;
}

void pack(const sl_diff_scene* sc, const sl_render_frame* f, const float* eye, DiffCamera& K, DiffParams& P,
          DiffLights& L) {
  memcpy(K.view, f->view, sizeof(K.view));
  K.focal[0] = f->focal[0];
  K.focal[1] = f->focal[1];
  K.viewport[0] = f->viewport[0];
  K.viewport[1] = f->viewport[1];
  K.near_plane = f->near_plane;
  K.far_plane = f->far_plane;
  K.lowpass = f->lowpass_px2;
  for (int k = 0; k < 3; k++) K.eye[k] = eye[k];
  P = DiffParams{sc->means, sc->log_scales, sc->quats, sc->opacity_logits, sc->albedo, sc->roughness, sc->light_scale};
  L.ambient = sc->ambient;
  L.ks = sc->ks;
  L.vgrid = sc->vgrid;
  L.lamp_T = sc->lamp_T;
  L.iso_norm = sc->iso_norm;
}

cudaError_t ensure(sl_diff* d, uint32_t tiles, uint32_t pixels) {
  ViewBuffers& vb = d->vb;
  const uint32_t n = d->n;
  const uint64_t cap = d->entry_cap, big = std::max<uint64_t>(cap, n);
  cudaError_t e;
#define ENS(buf, bytes) \
  if ((e = (buf).ensure(bytes)) != cudaSuccess) return e
  ENS(vb.key16, 2ull * n + 16);
  ENS(vb.recs, sizeof(SplatRec) * (size_t)n + 16);
  ENS(vb.rects, 8ull * n + 16);
  ENS(vb.order, 4ull * n + 16);
  ENS(vb.keys_alt, 2 * big + 16);
  ENS(vb.vals_alt, 4 * big + 16);
  ENS(vb.status, 4ull * 256 * 2 * (sort_tiles_for((uint32_t)big) + 1));
  ENS(vb.tile_ctr, 16);
  ENS(vb.tile_keys, 2 * cap + 16);
  ENS(vb.tile_vals, 4 * cap + 16);
  ENS(vb.ranges, 8ull * tiles + 16);
  ENS(vb.digit_hist, 4ull * 4 * 256);
  ENS(vb.bin_scratch, tile_bin_scratch_bytes(n));
  ENS(vb.counters, sizeof(FrameCounters));
  ENS(d->drec, sizeof(DiffRec) * (size_t)n + 16);
  ENS(d->g2, sizeof(DiffGrad2D) * (size_t)n + 16);
  ENS(d->img, 16ull * pixels);
  ENS(d->tfinal, 4ull * pixels);
  ENS(d->ncontrib, 4ull * pixels);
  ENS(d->dimg, 16ull * pixels);
  ENS(d->loss, 8);
#undef ENS
  return cudaSuccess;
}

// Forward (and with grads, the backward) on stream s; the counters and the loss are copied to pinned host memory.
int run(sl_diff* d, const sl_diff_scene* sc, const sl_render_frame* f, const float* eye, const float* target,
        float* image_out, const sl_diff_grads* G, cudaStream_t s) {
  DiffCamera K;
  DiffParams P;
  DiffLights L{};
  pack(sc, f, eye, K, P, L);
  int lrc = build_lights(d, sc, L, s);
  if (lrc) return lrc;
  const uint32_t W = (uint32_t)f->viewport[0], H = (uint32_t)f->viewport[1];
  const uint32_t tx = (W + 15) / 16, ty = (H + 15) / 16, tiles = tx * ty, npix = W * H;
  if (tiles > 65535u) return fail(SL_ERR_INVALID_ARG, "too many tiles for 16-bit tile keys");
  if (d->entry_cap == 0) d->entry_cap = (uint64_t)d->n * 8 + 4096;
  cudaError_t e = ensure(d, tiles, npix);
  if (e != cudaSuccess) return cuda_fail(e, "diff buffers");
  ViewBuffers& vb = d->vb;
  FrameCounters* ctr = vb.counters.as<FrameCounters>();
  uint32_t* hist = vb.digit_hist.as<uint32_t>();
  SortScratch scr{vb.keys_alt.as<uint16_t>(), vb.vals_alt.as<uint32_t>(), vb.status.as<uint32_t>(),
                  vb.tile_ctr.as<uint32_t>(), (uint32_t)(vb.status.bytes / (4ull * 256 * 2))};
  const uint32_t n = d->n;
  const uint32_t cap32 = (uint32_t)std::min<uint64_t>(d->entry_cap, 0xffffffffull);
#define CK(x, what)                                  \
  if ((e = (x)) != cudaSuccess) return cuda_fail(e, what)
  CK(cudaMemsetAsync(ctr, 0, sizeof(FrameCounters), s), "memset");
  CK(cudaMemsetAsync(hist, 0, 4 * 4 * 256, s), "memset");
  CK(cudaMemsetAsync(vb.ranges.ptr, 0, 8ull * tiles, s), "memset");
  CK(launch_dproject(K, P, L, n, vb.key16.as<uint16_t>(), d->drec.as<DiffRec>(), vb.recs.as<SplatRec>(),
                     vb.rects.as<ushort4>(), hist, ctr, s),
     "diff project");
  CK(sort16_pairs(vb.key16.as<uint16_t>(), nullptr, vb.order.as<uint32_t>(), n, nullptr, 16, hist, scr, ctr, s),
     "depth sort");
  CK(launch_tile_bin(vb.order.as<uint32_t>(), vb.rects.as<ushort4>(), vb.recs.as<SplatRec>(), n, tx, 16, 16, cap32,
                     ctr, vb.tile_keys.as<uint16_t>(), vb.tile_vals.as<uint32_t>(), hist + 512, vb.bin_scratch.ptr, s),
     "tile binning");
  CK(sort16_pairs(vb.tile_keys.as<uint16_t>(), vb.tile_vals.as<uint32_t>(), vb.tile_vals.as<uint32_t>(), cap32,
                  &ctr->entries, bits16(tiles - 1), hist + 512, scr, ctr, s, vb.tile_keys.as<uint16_t>()),
     "tile sort");
  CK(launch_tile_ranges(vb.tile_keys.as<uint16_t>(), &ctr->entries, cap32, vb.ranges.as<uint2>(), s), "tile ranges");
  CK(launch_dcomposite_fwd(vb.ranges.as<uint2>(), vb.tile_vals.as<uint32_t>(), d->drec.as<DiffRec>(), W, H, tx, tiles,
                           d->img.as<float4>(), d->tfinal.as<float>(), d->ncontrib.as<uint32_t>(), s),
     "diff composite");
  if (G) {
    CK(cudaMemsetAsync(d->g2.ptr, 0, sizeof(DiffGrad2D) * (size_t)n, s), "memset");
    CK(cudaMemsetAsync(d->loss.ptr, 0, 8, s), "memset");
    if (sc->n_lights) CK(cudaMemsetAsync(G->light_scale, 0, 4ull * sc->n_lights, s), "memset");
    CK(launch_dloss(d->img.as<float4>(), reinterpret_cast<const float4*>(target), npix, d->dimg.as<float4>(),
                    d->loss.as<double>(), s),
       "loss");
    CK(launch_dcomposite_bwd(vb.ranges.as<uint2>(), vb.tile_vals.as<uint32_t>(), d->drec.as<DiffRec>(), W, H, tx,
                             tiles, d->dimg.as<float4>(), d->tfinal.as<float>(), d->ncontrib.as<uint32_t>(),
                             d->g2.as<DiffGrad2D>(), s),
       "diff composite backward");
    DiffGrads g{G->means, G->log_scales, G->quats, G->opacity_logits, G->albedo, G->roughness, G->light_scale};
    CK(launch_dproject_bwd(K, P, L, n, d->g2.as<DiffGrad2D>(), d->drec.as<DiffRec>(), g, s), "diff project backward");
    CK(cudaMemcpyAsync(d->host_loss, d->loss.ptr, 8, cudaMemcpyDeviceToHost, s), "loss");
  }
  if (image_out) CK(cudaMemcpyAsync(image_out, d->img.ptr, 16ull * npix, cudaMemcpyDeviceToDevice, s), "image");
  CK(cudaMemcpyAsync(d->host_ctr, ctr, sizeof(FrameCounters), cudaMemcpyDeviceToHost, s), "counters");
  CK(cudaStreamSynchronize(s), "diff step");
#undef CK
  d->last_w = W;
  d->last_h = H;
  return SL_OK;
}

int run_retry(sl_diff* d, const sl_diff_scene* sc, const sl_render_frame* f, const float* eye, const float* target,
              float* image_out, const sl_diff_grads* G, double* loss, void* stream) {
  if (!d || !f || !eye) return fail(SL_ERR_INVALID_ARG, "null argument");
  int rc = check_scene(sc, d->n);
  if (rc) return rc;
  if (!(f->viewport[0] >= 1.0f && f->viewport[1] >= 1.0f && f->viewport[0] <= 16384.0f && f->viewport[1] <= 16384.0f))
    return fail(SL_ERR_INVALID_ARG, "bad viewport");
  cudaSetDevice(d->device);
  for (int attempt = 0; attempt < 4; attempt++) {
    rc = run(d, sc, f, eye, target, image_out, G, reinterpret_cast<cudaStream_t>(stream));
    if (rc) return rc;
    const FrameCounters& hc = *d->host_ctr;
    if (hc.timeout) return fail(SL_ERR_TIMEOUT, "a bounded device-side wait gave up");
    if (hc.overflow || hc.entries > d->entry_cap) {
      d->entry_cap = std::max<uint64_t>((uint64_t)hc.entries + hc.entries / 4 + 4096, 2 * d->entry_cap);
      continue;
    }
    d->last_visible = hc.visible;
    d->last_entries = hc.entries;
    if (loss) *loss = G ? *d->host_loss : 0.0;
    return SL_OK;
  }
  return fail(SL_ERR_OVERFLOW, "tile entry capacity kept overflowing");
}

}  // namespace
}  // namespace sl

using namespace sl;

extern "C" {

int sl_diff_create(uint32_t n, sl_diff** out) {
  if (!out) return fail(SL_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  if (n == 0 || n > (1u << 26)) return fail(SL_ERR_INVALID_ARG, "Gaussian count out of range");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "no device");
  sl_diff* d = new sl_diff();
  d->device = dev;
  d->n = n;
  if ((e = cudaMallocHost((void**)&d->host_ctr, sizeof(FrameCounters))) != cudaSuccess ||
      (e = cudaMallocHost((void**)&d->host_loss, sizeof(double))) != cudaSuccess) {
    sl_diff_destroy(d);
    return cuda_fail(e, "pinned counters");
  }
  *out = d;
  return SL_OK;
}

int sl_diff_destroy(sl_diff* d) {
  if (!d) return SL_OK;
  cudaSetDevice(d->device);
  cudaDeviceSynchronize();
  d->vb.release_all();
  sl::DevBuf* all[] = {&d->drec, &d->img, &d->tfinal, &d->ncontrib, &d->dimg, &d->g2, &d->loss, &d->target,
                       &d->tree, &d->dtab};
  for (sl::DevBuf* b : all) b->release();
  if (d->host_ctr) cudaFreeHost(d->host_ctr);
  if (d->host_loss) cudaFreeHost(d->host_loss);
  delete d;
  return SL_OK;
}

int sl_diff_forward(sl_diff* d, const sl_diff_scene* scene, const sl_render_frame* frame, const float* eye,
                    float* image_dev, void* stream) {
  return run_retry(d, scene, frame, eye, nullptr, image_dev, nullptr, nullptr, stream);
}

int sl_diff_step(sl_diff* d, const sl_diff_scene* scene, const sl_render_frame* frame, const float* eye,
                 const float* target_dev, float* image_dev, const sl_diff_grads* grads, double* loss, void* stream) {
  if (!target_dev || !grads || !grads->means || !grads->log_scales || !grads->quats || !grads->opacity_logits ||
      !grads->albedo || !grads->roughness || (scene && scene->n_lights && !grads->light_scale))
    return fail(SL_ERR_INVALID_ARG, "null target or gradient array");
  return run_retry(d, scene, frame, eye, target_dev, image_dev, grads, loss, stream);
}

int sl_diff_read_order(sl_diff* d, uint32_t* order, uint32_t* n_visible) {
  if (!d) return fail(SL_ERR_INVALID_ARG, "null diff");
  cudaSetDevice(d->device);
  if (n_visible) *n_visible = d->last_visible;
  if (order) {
    cudaError_t e = cudaMemcpy(order, d->vb.order.ptr, 4ull * d->last_visible, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "order");
  }
  return SL_OK;
}

}  // extern "C"
