// Display resolve, headless: the linear HDR image of a frame to 8-bit sRGB (shaders/display.wgsl:120-189, the pass
// after the composite): exposure, the frame's tone curve (frame.tone.x: 0 clamp, 1 AgX, 2 ACES filmic (Narkowicz's
// fit), 3 Reinhard on luminance, 4 Khronos PBR Neutral, 5 Hable filmic), the sRGB transfer function, and for the
// overdraw view the heat ramp of log2(1 + count) / 7.  Out: RGBA8, alpha 255, rounded to nearest.  The sky and
// light-disc background the reference adds where the splats leave the sky showing needs its environment sky model
// (probe bounce), outside this path: bare pixels stay black.
#include "sl_runtime.h"

namespace sl {
namespace {

constexpr int kThreads = 256;

struct C3 {
  float x, y, z;
};
__device__ __forceinline__ C3 c3(float x, float y, float z) { return C3{x, y, z}; }
__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
__device__ __forceinline__ C3 clamp3(C3 v) { return c3(clamp01(v.x), clamp01(v.y), clamp01(v.z)); }

__device__ __forceinline__ float srgb1(float c) {
  return c <= 0.0031308f ? c * 12.92f : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
}

__device__ __forceinline__ float hable1(float x) {
  return (x * (0.15f * x + 0.05f) + 0.004f) / (x * (0.15f * x + 0.5f) + 0.06f) - 0.02f / 0.3f;
}

__device__ C3 tone_map(C3 x, uint32_t mode) {
  if (mode == 1u) {  // AgX: inset, log2 encode over [-12.47, 4.03] EV, sigmoid polynomial, outset, 2.2 power
    const float m[3][3] = {{0.842479062253094f, 0.0784335999999992f, 0.0792237451477643f},
                           {0.0423282422610123f, 0.878468636469772f, 0.0791661274605434f},
                           {0.0423756549057051f, 0.0784336f, 0.879142973793104f}};
    const float mi[3][3] = {{1.19687900512017f, -0.0980208811401368f, -0.0990297440797205f},
                            {-0.0528968517574562f, 1.15190312990417f, -0.0989611768448433f},
                            {-0.0529716355144438f, -0.0980434501171241f, 1.15107367264116f}};
    const float lo = -12.47393f, hi = 4.026069f;
    const float v[3] = {x.x, x.y, x.z};
    float y[3];
    for (int r = 0; r < 3; r++) {
      float a = m[r][0] * v[0] + m[r][1] * v[1] + m[r][2] * v[2];
      float e = fminf(fmaxf(log2f(fmaxf(a, 1e-10f)), lo), hi);
      e = (e - lo) / (hi - lo);
      const float e2 = e * e, e4 = e2 * e2;
      y[r] = 15.5f * e4 * e2 - 40.14f * e4 * e + 31.96f * e4 - 6.868f * e2 * e + 0.4298f * e2 + 0.1191f * e - 0.00232f;
    }
    float o[3];
    for (int r = 0; r < 3; r++) {
      const float b = mi[r][0] * y[0] + mi[r][1] * y[1] + mi[r][2] * y[2];
      o[r] = clamp01(powf(fmaxf(b, 0.0f), 2.2f));
    }
    return c3(o[0], o[1], o[2]);
  }
  if (mode == 2u) {  // ACES filmic (Narkowicz)
    auto f = [](float v) { return clamp01(v * (2.51f * v + 0.03f) / (v * (2.43f * v + 0.59f) + 0.14f)); };
    return c3(f(x.x), f(x.y), f(x.z));
  }
  if (mode == 3u) {  // Reinhard on luminance
    const float l = 0.2126f * x.x + 0.7152f * x.y + 0.0722f * x.z;
    return clamp3(c3(x.x / (1.0f + l), x.y / (1.0f + l), x.z / (1.0f + l)));
  }
  if (mode == 4u) {  // Khronos PBR Neutral
    const float start = 0.8f - 0.04f, desat = 0.15f;
    const float lo = fminf(x.x, fminf(x.y, x.z));
    const float off = lo < 0.08f ? lo - 6.25f * lo * lo : 0.04f;
    C3 v = c3(x.x - off, x.y - off, x.z - off);
    const float peak = fmaxf(v.x, fmaxf(v.y, v.z));
    if (peak < start) return clamp3(v);
    const float d = 1.0f - start;
    const float np = 1.0f - d * d / (peak + d - start);
    const float s = np / peak;
    v = c3(v.x * s, v.y * s, v.z * s);
    const float g = 1.0f - 1.0f / (desat * (peak - np) + 1.0f);
    return clamp3(c3(v.x + (np - v.x) * g, v.y + (np - v.y) * g, v.z + (np - v.z) * g));
  }
  if (mode == 5u) {  // Hable filmic: bias 2, white 11.2
    const float w = hable1(11.2f);
    return clamp3(c3(hable1(2.0f * x.x) / w, hable1(2.0f * x.y) / w, hable1(2.0f * x.z) / w));
  }
  return clamp3(x);
}

__device__ __forceinline__ uint32_t to8(float v) { return (uint32_t)(clamp01(v) * 255.0f + 0.5f); }

__global__ void __launch_bounds__(kThreads) display_kernel(const float4* __restrict__ img, uint32_t n, float exposure,
                                                           uint32_t tone, uint32_t view_mode,
                                                           uchar4* __restrict__ out) {
  const uint32_t p = blockIdx.x * kThreads + threadIdx.x;
  if (p >= n) return;
  const float4 c = img[p];
  C3 rgb;
  if (view_mode == 2u) {  // heat ramp black -> blue -> green -> yellow -> red of log2(1 + count) / 7
    const float x = clamp01(log2f(1.0f + c.x) / 7.0f) * 4.0f;
    rgb = clamp3(c3(x - 2.0f, fminf(x - 1.0f, 4.0f - x), fminf(x, 2.0f - x)));
  } else {
    rgb = tone_map(c3(fmaxf(c.x * exposure, 0.0f), fmaxf(c.y * exposure, 0.0f), fmaxf(c.z * exposure, 0.0f)), tone);
    rgb = c3(srgb1(rgb.x), srgb1(rgb.y), srgb1(rgb.z));
  }
  out[p] = make_uchar4((unsigned char)to8(rgb.x), (unsigned char)to8(rgb.y), (unsigned char)to8(rgb.z), 255);
}

}  // namespace
}  // namespace sl

using namespace sl;

extern "C" int sl_display(const float* image_dev, uint32_t width, uint32_t height, const sl_render_frame* frame,
                          uint8_t* out_dev, void* stream) {
  if (!image_dev || !frame || !out_dev) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (frame->tone[0] > 5u) return fail(SL_ERR_INVALID_ARG, "tone curve must be 0..5");
  const uint64_t n = (uint64_t)width * height;
  if (n == 0 || n > (1ull << 31)) return fail(SL_ERR_INVALID_ARG, "bad image size");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  display_kernel<<<(uint32_t)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(
      reinterpret_cast<const float4*>(image_dev), (uint32_t)n, frame->exposure, frame->tone[0], frame->view_mode,
      reinterpret_cast<uchar4*>(out_dev));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sl_display");
  return SL_OK;
}
