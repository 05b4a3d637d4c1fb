/* Display resolve restated for the checks (test infrastructure): shaders/display.wgsl:107-189 -- exposure, the tone
 * curves (tone_map :140-150, hable :153-155, pbr_neutral :159-172, agx :176-189), srgb_encode (:107-111), the
 * overdraw heat ramp (:113-117, :122-125) -- in double precision, then rounded to 8 bits (nearest). */
#include <math.h>
#include <stdint.h>

#include "splatlight.h"

static double clamp01d(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }
static double srgb1d(double c) { return c <= 0.0031308 ? c * 12.92 : 1.055 * pow(c, 1.0 / 2.4) - 0.055; }
static double hable1d(double x) { return (x * (0.15 * x + 0.05) + 0.004) / (x * (0.15 * x + 0.5) + 0.06) - 0.02 / 0.3; }

static void tone_d(const double* x, uint32_t mode, double* o) {
  if (mode == 1u) {
    /* AgX: columns of the inset / outset matrices as display.wgsl:177-182 write them */
    const double m[3][3] = {{0.842479062253094, 0.0784335999999992, 0.0792237451477643},
                            {0.0423282422610123, 0.878468636469772, 0.0791661274605434},
                            {0.0423756549057051, 0.0784336, 0.879142973793104}};
    const double mi[3][3] = {{1.19687900512017, -0.0980208811401368, -0.0990297440797205},
                             {-0.0528968517574562, 1.15190312990417, -0.0989611768448433},
                             {-0.0529716355144438, -0.0980434501171241, 1.15107367264116}};
    const double lo = -12.47393, hi = 4.026069;
    double y[3];
    for (int r = 0; r < 3; r++) {
      double a = m[r][0] * x[0] + m[r][1] * x[1] + m[r][2] * x[2];
      double e = log2(a > 1e-10 ? a : 1e-10);
      e = e < lo ? lo : (e > hi ? hi : e);
      e = (e - lo) / (hi - lo);
      double e2 = e * e, e4 = e2 * e2;
      y[r] = 15.5 * e4 * e2 - 40.14 * e4 * e + 31.96 * e4 - 6.868 * e2 * e + 0.4298 * e2 + 0.1191 * e - 0.00232;
    }
    for (int r = 0; r < 3; r++) {
      double b = mi[r][0] * y[0] + mi[r][1] * y[1] + mi[r][2] * y[2];
      o[r] = clamp01d(pow(b > 0.0 ? b : 0.0, 2.2));
    }
    return;
  }
  if (mode == 2u) {
    for (int k = 0; k < 3; k++) o[k] = clamp01d(x[k] * (2.51 * x[k] + 0.03) / (x[k] * (2.43 * x[k] + 0.59) + 0.14));
    return;
  }
  if (mode == 3u) {
    double l = 0.2126 * x[0] + 0.7152 * x[1] + 0.0722 * x[2];
    for (int k = 0; k < 3; k++) o[k] = clamp01d(x[k] / (1.0 + l));
    return;
  }
  if (mode == 4u) {
    const double start = 0.8 - 0.04, desat = 0.15;
    double lo = fmin(x[0], fmin(x[1], x[2]));
    double off = lo < 0.08 ? lo - 6.25 * lo * lo : 0.04;
    double v[3] = {x[0] - off, x[1] - off, x[2] - off};
    double peak = fmax(v[0], fmax(v[1], v[2]));
    if (peak < start) {
      for (int k = 0; k < 3; k++) o[k] = clamp01d(v[k]);
      return;
    }
    double d = 1.0 - start, np = 1.0 - d * d / (peak + d - start);
    double g = 1.0 - 1.0 / (desat * (peak - np) + 1.0);
    for (int k = 0; k < 3; k++) {
      double t = v[k] * (np / peak);
      o[k] = clamp01d(t + (np - t) * g);
    }
    return;
  }
  if (mode == 5u) {
    double w = hable1d(11.2);
    for (int k = 0; k < 3; k++) o[k] = clamp01d(hable1d(2.0 * x[k]) / w);
    return;
  }
  for (int k = 0; k < 3; k++) o[k] = clamp01d(x[k]);
}

static uint8_t to8d(double v) { return (uint8_t)(clamp01d(v) * 255.0 + 0.5); }

void orc_display(const float* img, uint32_t n, float exposure, uint32_t tone, uint32_t view_mode, uint8_t* out) {
  for (uint32_t p = 0; p < n; p++) {
    const float* c = img + 4u * p;
    double rgb[3];
    if (view_mode == 2u) {
      double x = clamp01d(log2(1.0 + (double)c[0]) / 7.0) * 4.0;
      rgb[0] = clamp01d(x - 2.0);
      rgb[1] = clamp01d(fmin(x - 1.0, 4.0 - x));
      rgb[2] = clamp01d(fmin(x, 2.0 - x));
    } else {
      double x[3];
      for (int k = 0; k < 3; k++) {
        double v = (double)c[k] * (double)exposure;
        x[k] = v > 0.0 ? v : 0.0;
      }
      tone_d(x, tone, rgb);
      for (int k = 0; k < 3; k++) rgb[k] = srgb1d(rgb[k]);
    }
    for (int k = 0; k < 3; k++) out[4u * p + k] = to8d(rgb[k]);
    out[4u * p + 3] = 255;
  }
}

/* ---- the environment behind the splats (display.wgsl:22-133), FP64 ------------------------------------------- */

static void sky_radiance_d(const sl_display_sky* S, const double* w, double* c) {
  double x = w[0], y = w[1], z = w[2];
  double b[16] = {0.282095, 0.488603 * y, 0.488603 * z, 0.488603 * x, 1.092548 * x * y, 1.092548 * y * z,
                  0.315392 * (3.0 * z * z - 1.0), 1.092548 * x * z, 0.546274 * (x * x - y * y),
                  0.590044 * y * (3.0 * x * x - y * y), 2.890611 * x * y * z, 0.457046 * y * (5.0 * z * z - 1.0),
                  0.373176 * z * (5.0 * z * z - 3.0), 0.457046 * x * (5.0 * z * z - 1.0), 1.445306 * z * (x * x - y * y),
                  0.590044 * x * (x * x - 3.0 * y * y)};
  for (int ch = 0; ch < 3; ch++) {
    double a = 0.0;
    for (int k = 0; k < 16; k++) a += b[k] * S->sky_sh[k][ch];
    c[ch] = a > 0.0 ? a : 0.0;
  }
}

/* the background sky: the real SH basis in sky_radiance's order and signs (index l l + l + m, m < 0 sine, m > 0
 * cosine, no Condon-Shortley phase) by the associated-Legendre recurrence, then the glow, the ring and the ground */
static void sky_background_d(const sl_display_sky* S, const double* w, double* c) {
  uint32_t n = S->bg_count < 81u ? S->bg_count : 81u;
  if (n == 0u) {
    sky_radiance_d(S, w, c);
    return;
  }
  uint32_t lmax = (uint32_t)floor(sqrt((double)n) + 0.5) - 1u;
  double acc[3] = {0.0, 0.0, 0.0};
  double cm = 1.0, sm = 0.0, pmm = 1.0;
  for (uint32_t m = 0; m <= lmax; m++) {
    if (m > 0u) {
      double c2 = cm * w[0] - sm * w[1];
      sm = cm * w[1] + sm * w[0];
      cm = c2;
      pmm *= (double)(2u * m - 1u);
    }
    double p_prev = 0.0, p = pmm;
    double kf = 1.0 / (4.0 * M_PI);
    for (uint32_t j = 1; j <= 2u * m; j++) kf /= (double)j;
    for (uint32_t l = m; l <= lmax; l++) {
      if (l == m + 1u) {
        p_prev = p;
        p = w[2] * (double)(2u * m + 1u) * pmm;
      } else if (l > m + 1u) {
        double pn = ((double)(2u * l - 1u) * w[2] * p - (double)(l + m - 1u) * p_prev) / (double)(l - m);
        p_prev = p;
        p = pn;
        kf *= (double)(l - m) / (double)(l + m);
      }
      if (l == m + 1u) kf *= 1.0 / (double)(2u * m + 1u);
      double k = sqrt((double)(2u * l + 1u) * kf);
      uint32_t i = l * l + l;
      for (int ch = 0; ch < 3; ch++) {
        if (m == 0u) acc[ch] += k * p * S->bg_sh[i][ch];
        else acc[ch] += sqrt(2.0) * k * p * (cm * S->bg_sh[i + m][ch] + sm * S->bg_sh[i - m][ch]);
      }
    }
  }
  for (int ch = 0; ch < 3; ch++) c[ch] = acc[ch] > 0.0 ? acc[ch] : 0.0;
  if (S->glow_std > 0.0f) {
    double s2 = (double)S->glow_std * S->glow_std;
    double e = exp((w[0] * S->glow_dir[0] + w[1] * S->glow_dir[1] + w[2] * S->glow_dir[2] - 1.0) / s2) / (2.0 * M_PI * s2);
    for (int ch = 0; ch < 3; ch++) c[ch] += S->glow[ch] * e;
  }
  uint32_t nr = S->ring_count < 8u ? S->ring_count : 8u;
  if (nr == 0u) return;
  for (uint32_t k = 0; k < nr; k++) {
    double a = 2.0 * M_PI * (double)k / (double)nr;
    double zx = cos(a), zy = sin(a);
    double along = -w[0] * zy + w[1] * zx;
    double d = w[0] * zx + w[1] * zy;
    double e = (d > 0.0 ? d : 0.0) * exp(-S->ring_par[0] * along * along - S->ring_par[1] * w[2] * w[2]);
    for (int ch = 0; ch < 3; ch++) c[ch] += S->ring[k][ch] * e;
  }
  double t = clamp01d(w[2] / S->ground_blend * 0.5 + 0.5);
  for (int ch = 0; ch < 3; ch++) c[ch] = S->ground[ch] * (1.0 - t) + c[ch] * t;
}

static void lights_radiance_d(const sl_display_sky* S, const double* w, double* c) {
  for (int ch = 0; ch < 3; ch++) c[ch] = 0.0;
  for (uint32_t k = 0; k < S->n_lights && k < 4u; k++) {
    double sd = S->disc_std[k] > 0.0f ? S->disc_std[k] : S->light_std[k];
    double s2 = sd * sd > 1e-8 ? sd * sd : 1e-8;
    double e = exp((w[0] * S->light_dir[k][0] + w[1] * S->light_dir[k][1] + w[2] * S->light_dir[k][2] - 1.0) / s2) /
               (2.0 * M_PI * s2);
    for (int ch = 0; ch < 3; ch++) c[ch] += S->light_irr[k][ch] * e;
  }
}

/* orc_display with the environment behind the splats in the lit view (display.wgsl fs :120-133); view: the frame's
 * column-major view matrix, (vw, vh) the viewport, (fx, fy) the focal lengths */
void orc_display_env(const float* img, uint32_t width, uint32_t height, float exposure, uint32_t tone,
                     uint32_t view_mode, const float* view, float vw, float vh, float fx, float fy,
                     const sl_display_sky* sky, uint8_t* out) {
  uint32_t n = width * height;
  for (uint32_t p = 0; p < n; p++) {
    const float* c = img + 4u * p;
    double rgb[3];
    if (view_mode == 2u) {
      double x = clamp01d(log2(1.0 + (double)c[0]) / 7.0) * 4.0;
      rgb[0] = clamp01d(x - 2.0);
      rgb[1] = clamp01d(fmin(x - 1.0, 4.0 - x));
      rgb[2] = clamp01d(fmin(x, 2.0 - x));
    } else {
      double lin[3] = {c[0], c[1], c[2]};
      if (sky && view_mode == 3u && (sky->n_lights > 0u || sky->has_sky)) {
        double bare = 1.0 - clamp01d(c[3]);
        if (bare > 1.0 / 1024.0) {
          double px = (double)(p % width) + 0.5, py = (double)(p / width) + 0.5;
          double v[3] = {(px - 0.5 * vw) / fx, -(py - 0.5 * vh) / fy, -1.0};
          double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
          for (int k = 0; k < 3; k++) v[k] /= l;
          double w[3];
          for (int i = 0; i < 3; i++) w[i] = view[4 * i] * v[0] + view[4 * i + 1] * v[1] + view[4 * i + 2] * v[2];
          l = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
          for (int k = 0; k < 3; k++) w[k] /= l;
          double bg[3] = {0.0, 0.0, 0.0}, li[3];
          if (sky->has_sky) sky_background_d(sky, w, bg);
          lights_radiance_d(sky, w, li);
          for (int k = 0; k < 3; k++) lin[k] += bare * (bg[k] + li[k]);
        }
      }
      double x[3];
      for (int k = 0; k < 3; k++) {
        double v = lin[k] * (double)exposure;
        x[k] = v > 0.0 ? v : 0.0;
      }
      tone_d(x, tone, rgb);
      for (int k = 0; k < 3; k++) rgb[k] = srgb1d(rgb[k]);
    }
    for (int k = 0; k < 3; k++) out[4u * p + k] = to8d(rgb[k]);
    out[4u * p + 3] = 255;
  }
}
