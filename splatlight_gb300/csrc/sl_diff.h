// Internal declarations of the differentiable splat path (diff.cu, capi_diff.cu).
#pragma once

#include "sl_dshade.cuh"
#include "sl_internal.h"

namespace sl {

constexpr float kDiffTauMin = 1e-6f;     // fragments of smaller optical depth are skipped
constexpr float kDiffAlphaMax = 0.99f;   // alpha clamp (keeps T_f = T_{f+1} / (1 - alpha_f) well conditioned)
constexpr float kDiffTStop = 1e-4f;      // a pixel stops before the fragment that would take T below this
constexpr uint32_t kMaxDiffLights = 32;

struct DiffCamera {
  float view[16];
  float focal[2], viewport[2];
  float near_plane, far_plane, lowpass;
  float eye[3];
};

struct DiffParams {
  const float* means;           // n x 3 (world)
  const float* log_scales;      // n x 3
  const float* quats;           // n x 4 (x, y, z, w), normalised in the forward
  const float* opacity_logits;  // n
  const float* albedo;          // n x 3
  const float* roughness;       // n
  const float* light_scale;     // lights
};

// The lighting of the differentiable path (sl_dshade.cuh): the emitter tree built on the host from the lights at
// their current intensities, its derivative table ([node][light][9]: d(Le rgb, M xx yy zz xy xz yz) / d intensity),
// and the per-Gaussian lighting state held constant (V grids, opacity-map T, iso_norm; null = visible / 1 / 1).
struct DiffLights {
  dsh::EmitTree tree;
  const float* dtab;
  uint32_t n;
  float ambient, ks;
  const sl_vgrid* vgrid;
  const float* lamp_T;
  const float* iso_norm;
};

struct DiffGrads {
  float *means, *log_scales, *quats, *opacity_logits, *albedo, *roughness, *light_scale;
};

// per splat: screen centre, pixel-space conic, tau0, radiance, candidate half extents (48 B)
struct DiffRec {
  float cx, cy, A, B, C, tau0, r, g, bl, hx, hy, pad;
};

// per splat: gradients of the loss with respect to the DiffRec quantities (accumulated by the backward compositor)
struct DiffGrad2D {
  float cx, cy, A, B, C, tau0, r, g, b, pad[3];
};

cudaError_t launch_dproject(const DiffCamera& K, const DiffParams& P, const DiffLights& L, uint32_t n, uint16_t* key16,
                            DiffRec* drec, SplatRec* recs, ushort4* rects, uint32_t* digit_hist, FrameCounters* ctr,
                            cudaStream_t s);
cudaError_t launch_dcomposite_fwd(const uint2* ranges, const uint32_t* tile_vals, const DiffRec* drec, uint32_t width,
                                  uint32_t height, uint32_t tiles_x, uint32_t tiles, float4* img, float* t_final,
                                  uint32_t* n_contrib, cudaStream_t s);
cudaError_t launch_dloss(const float4* img, const float4* target, uint32_t npix, float4* dimg, double* loss,
                         cudaStream_t s);
cudaError_t launch_dcomposite_bwd(const uint2* ranges, const uint32_t* tile_vals, const DiffRec* drec, uint32_t width,
                                  uint32_t height, uint32_t tiles_x, uint32_t tiles, const float4* dimg,
                                  const float* t_final, const uint32_t* n_contrib, DiffGrad2D* g2, cudaStream_t s);
cudaError_t launch_dproject_bwd(const DiffCamera& K, const DiffParams& P, const DiffLights& L, uint32_t n,
                                const DiffGrad2D* g2, const DiffRec* drec, const DiffGrads& G, cudaStream_t s);

}  // namespace sl
