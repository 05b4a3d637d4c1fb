/* Display resolve restated for the checks (test infrastructure): shaders/display.wgsl:107-189 -- exposure, the tone
 * curves (tone_map :140-150, hable :153-155, pbr_neutral :159-172, agx :176-189), srgb_encode (:107-111), the
 * overdraw heat ramp (:113-117, :122-125) -- in double precision, then rounded to 8 bits (nearest). */
#include <math.h>
#include <stdint.h>

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
