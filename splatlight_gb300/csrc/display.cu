// Display resolve, headless: the linear HDR image of a frame to 8-bit sRGB (shaders/display.wgsl:120-189, the pass
// after the composite): exposure, the frame's tone curve (frame.tone.x: 0 clamp, 1 AgX, 2 ACES filmic (Narkowicz's
// fit), 3 Reinhard on luminance, 4 Khronos PBR Neutral, 5 Hable filmic), the sRGB transfer function, and for the
// overdraw view the heat ramp of log2(1 + count) / 7; with the environment (sl_display_env), in the lit view, the
// background sky (its own SH up to band 8 or the lighting sky, the glow round the sun, the horizon ring, the ground)
// and the distant lights' discs where the splats leave the sky showing (display.wgsl:22-133).  Out: RGBA8, alpha 255,
// rounded to nearest.
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

// sky_radiance (display.wgsl:22-32): the lighting sky, real SH bands 0-3, clamped at 0
__device__ C3 sky_radiance(const sl_display_sky& S, C3 w) {
  const float x = w.x, y = w.y, z = w.z;
  const float b[16] = {0.282095f, 0.488603f * y, 0.488603f * z, 0.488603f * x, 1.092548f * x * y, 1.092548f * y * z,
                       0.315392f * (3.0f * z * z - 1.0f), 1.092548f * x * z, 0.546274f * (x * x - y * y),
                       0.590044f * y * (3.0f * x * x - y * y), 2.890611f * x * y * z,
                       0.457046f * y * (5.0f * z * z - 1.0f), 0.373176f * z * (5.0f * z * z - 3.0f),
                       0.457046f * x * (5.0f * z * z - 1.0f), 1.445306f * z * (x * x - y * y),
                       0.590044f * x * (x * x - 3.0f * y * y)};
  C3 c = c3(0.0f, 0.0f, 0.0f);
  for (int k = 0; k < 16; k++)
    c = c3(c.x + b[k] * S.sky_sh[k][0], c.y + b[k] * S.sky_sh[k][1], c.z + b[k] * S.sky_sh[k][2]);
  return c3(fmaxf(c.x, 0.0f), fmaxf(c.y, 0.0f), fmaxf(c.z, 0.0f));
}

// sky_background (display.wgsl:36-80): the background SH by the associated-Legendre recurrence (index l l + l + m,
// m < 0 sine, m > 0 cosine, no Condon-Shortley phase), the glow, the horizon ring's lobes and the ground below
__device__ C3 sky_background(const sl_display_sky& S, C3 w) {
  const uint32_t n = S.bg_count < 81u ? S.bg_count : 81u;
  if (n == 0u) return sky_radiance(S, w);
  const uint32_t lmax = (uint32_t)rintf(sqrtf((float)n)) - 1u;
  C3 c = c3(0.0f, 0.0f, 0.0f);
  float cm = 1.0f, sm = 0.0f, pmm = 1.0f;
  for (uint32_t m = 0; m <= lmax; m++) {
    if (m > 0u) {
      const float c2 = cm * w.x - sm * w.y;
      sm = cm * w.y + sm * w.x;
      cm = c2;
      pmm *= (float)(2u * m - 1u);
    }
    float p_prev = 0.0f, p = pmm;
    float kf = 1.0f / (4.0f * 3.14159265f);
    for (uint32_t j = 1; j <= 2u * m; j++) kf /= (float)j;
    for (uint32_t l = m; l <= lmax; l++) {
      if (l == m + 1u) {
        p_prev = p;
        p = w.z * (float)(2u * m + 1u) * pmm;
      } else if (l > m + 1u) {
        const float pn = ((float)(2u * l - 1u) * w.z * p - (float)(l + m - 1u) * p_prev) / (float)(l - m);
        p_prev = p;
        p = pn;
        kf *= (float)(l - m) / (float)(l + m);
      }
      if (l == m + 1u) kf *= 1.0f / (float)(2u * m + 1u);
      const float k = sqrtf((float)(2u * l + 1u) * kf);
      const uint32_t i = l * l + l;
      if (m == 0u) {
        const float a = k * p;
        c = c3(c.x + a * S.bg_sh[i][0], c.y + a * S.bg_sh[i][1], c.z + a * S.bg_sh[i][2]);
      } else {
        const float a = 1.41421356f * k * p;
        c = c3(c.x + a * (cm * S.bg_sh[i + m][0] + sm * S.bg_sh[i - m][0]),
               c.y + a * (cm * S.bg_sh[i + m][1] + sm * S.bg_sh[i - m][1]),
               c.z + a * (cm * S.bg_sh[i + m][2] + sm * S.bg_sh[i - m][2]));
      }
    }
  }
  c = c3(fmaxf(c.x, 0.0f), fmaxf(c.y, 0.0f), fmaxf(c.z, 0.0f));
  if (S.glow_std > 0.0f) {
    const float s2 = S.glow_std * S.glow_std;
    const float e = expf((w.x * S.glow_dir[0] + w.y * S.glow_dir[1] + w.z * S.glow_dir[2] - 1.0f) / s2) /
                    (2.0f * 3.14159265f * s2);
    c = c3(c.x + S.glow[0] * e, c.y + S.glow[1] * e, c.z + S.glow[2] * e);
  }
  const uint32_t nr = S.ring_count < 8u ? S.ring_count : 8u;
  if (nr == 0u) return c;
  for (uint32_t k = 0; k < nr; k++) {
    const float a = 6.28318531f * (float)k / (float)nr;
    const float zx = cosf(a), zy = sinf(a);
    const float along = -w.x * zy + w.y * zx;
    const float e = fmaxf(w.x * zx + w.y * zy, 0.0f) * expf(-S.ring_par[0] * along * along - S.ring_par[1] * w.z * w.z);
    c = c3(c.x + S.ring[k][0] * e, c.y + S.ring[k][1] * e, c.z + S.ring[k][2] * e);
  }
  const float t = clamp01(w.z / S.ground_blend * 0.5f + 0.5f);
  return c3(S.ground[0] * (1.0f - t) + c.x * t, S.ground[1] * (1.0f - t) + c.y * t, S.ground[2] * (1.0f - t) + c.z * t);
}

// lights_radiance (display.wgsl:84-93): each distant light as an SG of its irradiance over its (disc's) angular size
__device__ C3 lights_radiance(const sl_display_sky& S, C3 w) {
  C3 c = c3(0.0f, 0.0f, 0.0f);
  for (uint32_t k = 0; k < S.n_lights && k < 4u; k++) {
    const float sd = S.disc_std[k] > 0.0f ? S.disc_std[k] : S.light_std[k];
    const float s2 = fmaxf(sd * sd, 1e-8f);
    const float e = expf((w.x * S.light_dir[k][0] + w.y * S.light_dir[k][1] + w.z * S.light_dir[k][2] - 1.0f) / s2) /
                    (2.0f * 3.14159265f * s2);
    c = c3(c.x + S.light_irr[k][0] * e, c.y + S.light_irr[k][1] * e, c.z + S.light_irr[k][2] * e);
  }
  return c;
}

struct DisplayView {
  float view[16];
  float vw, vh, fx, fy;
};

__global__ void __launch_bounds__(kThreads) display_kernel(const float4* __restrict__ img, uint32_t n, uint32_t width,
                                                           float exposure, uint32_t tone, uint32_t view_mode,
                                                           const DisplayView V,
                                                           const __grid_constant__ sl_display_sky S, uint32_t use_sky,
                                                           uchar4* __restrict__ out) {
  const uint32_t p = blockIdx.x * kThreads + threadIdx.x;
  if (p >= n) return;
  const float4 c = img[p];
  C3 rgb;
  if (view_mode == 2u) {  // heat ramp black -> blue -> green -> yellow -> red of log2(1 + count) / 7
    const float x = clamp01(log2f(1.0f + c.x) / 7.0f) * 4.0f;
    rgb = clamp3(c3(x - 2.0f, fminf(x - 1.0f, 4.0f - x), fminf(x, 2.0f - x)));
  } else {
    C3 lin = c3(c.x, c.y, c.z);
    if (use_sky && view_mode == 3u && (S.n_lights > 0u || S.has_sky)) {
      const float bare = 1.0f - clamp01(c.w);
      if (bare > 1.0f / 1024.0f) {  // where the splats leave the sky showing
        // view_dir (display.wgsl:95-99): the pixel centre's ray, into the world by the view matrix's transpose
        const float px = (float)(p % width) + 0.5f, py = (float)(p / width) + 0.5f;
        float vx = (px - 0.5f * V.vw) / V.fx, vy = -(py - 0.5f * V.vh) / V.fy, vz = -1.0f;
        float il = rsqrtf(vx * vx + vy * vy + vz * vz);
        vx *= il;
        vy *= il;
        vz *= il;
        C3 w = c3(V.view[0] * vx + V.view[1] * vy + V.view[2] * vz, V.view[4] * vx + V.view[5] * vy + V.view[6] * vz,
                  V.view[8] * vx + V.view[9] * vy + V.view[10] * vz);
        il = rsqrtf(w.x * w.x + w.y * w.y + w.z * w.z);
        w = c3(w.x * il, w.y * il, w.z * il);
        const C3 bg = S.has_sky ? sky_background(S, w) : c3(0.0f, 0.0f, 0.0f);
        const C3 li = lights_radiance(S, w);
        lin = c3(lin.x + bare * (bg.x + li.x), lin.y + bare * (bg.y + li.y), lin.z + bare * (bg.z + li.z));
      }
    }
    rgb = tone_map(c3(fmaxf(lin.x * exposure, 0.0f), fmaxf(lin.y * exposure, 0.0f), fmaxf(lin.z * exposure, 0.0f)),
                   tone);
    rgb = c3(srgb1(rgb.x), srgb1(rgb.y), srgb1(rgb.z));
  }
  out[p] = make_uchar4((unsigned char)to8(rgb.x), (unsigned char)to8(rgb.y), (unsigned char)to8(rgb.z), 255);
}

}  // namespace
}  // namespace sl

using namespace sl;

extern "C" int sl_display_env(const float* image_dev, uint32_t width, uint32_t height, const sl_render_frame* frame,
                              const sl_display_sky* sky, uint8_t* out_dev, void* stream) {
  if (!image_dev || !frame || !out_dev) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (frame->tone[0] > 5u) return fail(SL_ERR_INVALID_ARG, "tone curve must be 0..5");
  const uint64_t n = (uint64_t)width * height;
  if (n == 0 || n > (1ull << 31)) return fail(SL_ERR_INVALID_ARG, "bad image size");
  if (sky && (sky->bg_count > 81u || sky->ring_count > 8u || sky->n_lights > 4u))
    return fail(SL_ERR_INVALID_ARG, "sky: at most 81 background coefficients, 8 horizon lobes, 4 lights");
  if (sky && sky->ring_count && !(sky->ground_blend > 0.0f))
    return fail(SL_ERR_INVALID_ARG, "sky: the ground blend must be positive with a horizon ring");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  DisplayView V{};
  for (int k = 0; k < 16; k++) V.view[k] = frame->view[k];
  V.vw = frame->viewport[0];
  V.vh = frame->viewport[1];
  V.fx = frame->focal[0];
  V.fy = frame->focal[1];
  // the environment travels in the kernel's parameter block (1.5 KB)
  sl_display_sky S{};
  if (sky) S = *sky;
  display_kernel<<<(uint32_t)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(
      reinterpret_cast<const float4*>(image_dev), (uint32_t)n, width, frame->exposure, frame->tone[0],
      frame->view_mode, V, S, sky ? 1u : 0u, reinterpret_cast<uchar4*>(out_dev));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sl_display");
  return SL_OK;
}

extern "C" int sl_display(const float* image_dev, uint32_t width, uint32_t height, const sl_render_frame* frame,
                          uint8_t* out_dev, void* stream) {
  return sl_display_env(image_dev, width, height, frame, nullptr, out_dev, stream);
}
