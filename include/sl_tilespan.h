/*
 * sl_tilespan.h -- which screen tiles of one tile row a splat can reach (shared by the CUDA binning kernels and the
 * CPU restatement, which must agree on every tile list bit for bit).
 *
 * A splat keeps the pixel centres p with q(p) = |(d.g0, d.g1)|^2 <= qcut, d = p - c: an ellipse with conic
 * M = g0 g0^T + g1 g1^T.  Its candidate rectangle (the ellipse's bounding box plus one pixel) bins a thin, tilted
 * ellipse into many tiles it never touches; per tile row the ellipse's horizontal extent over that row's band of
 * pixel centres is much tighter.  Over a band dy in [d0, d1] the right edge x_hi(dy) = (-b dy + sqrt(a Q - D dy^2))/a
 * (a = M00, b = M01, c = M11, D = det M) is concave, so its maximum is at dy* = -b sqrt(Q / (c D)) clamped into the
 * band; the left edge mirrors it.  The span is widened by one pixel plus 0.1% of the ellipse's half width, and Q by
 * 1e-4 relative, so float rounding (here or in the compositor's keep test) can never drop a kept pixel; nearly
 * degenerate conics (D below 1e-4 a c, where D loses its precision) keep the full rectangle row.
 *
 * Plain IEEE single-precision arithmetic only (+ - * / sqrt, floor, ceil): compile with contraction off
 * (nvcc --fmad=false, gcc -ffp-contract=off) so both sides round identically.
 */
#ifndef SL_TILESPAN_H
#define SL_TILESPAN_H

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SL_SPAN_FN __host__ __device__ __forceinline__
#else
#define SL_SPAN_FN static inline
#endif

/* The per-splat part of the row spans (the same for every tile row of the splat). */
typedef struct sl_span_prep {
  float cx, cy, a, b, D, Q, half_w, ylim, ys, m;
  int full; /* nearly degenerate conic: every row keeps the candidate rectangle's columns */
} sl_span_prep;

SL_SPAN_FN void sl_span_init(float cx, float cy, float g0x, float g0y, float g1x, float g1y, float qcut,
                             sl_span_prep* p) {
  const float a = g0x * g0x + g1x * g1x;
  const float b = g0x * g0y + g1x * g1y;
  const float c = g0y * g0y + g1y * g1y;
  const float ac = a * c;
  const float D = ac - b * b;
  p->cx = cx;
  p->cy = cy;
  p->a = a;
  p->b = b;
  p->D = D;
  p->full = (!(a > 0.0f) || !(c > 0.0f) || !(D > 1e-4f * ac)) ? 1 : 0;
  if (p->full) {
    p->Q = p->half_w = p->ylim = p->ys = p->m = 0.0f;
    return;
  }
  const float Q = qcut * 1.0001f;
  const float half_w = sqrtf(Q * c / D);   /* the ellipse's half width (x) */
  const float half_h = sqrtf(Q * a / D);   /* and half height (y) */
  p->Q = Q;
  p->half_w = half_w;
  p->ylim = half_h * 1.001f + 1.0f;
  p->ys = b * sqrtf(Q / (c * D));          /* the rightmost point sits at dy = -ys, the leftmost at +ys */
  p->m = 1.0f + 1e-3f * half_w;
}

/* Tile columns [*tx0, *tx1] of tile row ty (tiles tw x th pixels, tw a power of two: tile_shift = log2 tw) that the
 * prepared splat can reach, within the candidate rectangle's columns [rx0, rx1].  Returns 0 when the row holds
 * none. */
SL_SPAN_FN int sl_span_row(const sl_span_prep* p, uint32_t rx0, uint32_t rx1, uint32_t ty, uint32_t tw,
                           uint32_t tile_shift, uint32_t th, uint32_t* tx0, uint32_t* tx1) {
  *tx0 = rx0;
  *tx1 = rx1;
  if (p->full) return 1;
  const float d0 = ((float)(ty * th) + 0.5f) - p->cy;
  const float d1 = ((float)(ty * th + th) - 0.5f) - p->cy;
  if (d0 > p->ylim || d1 < -p->ylim) return 0;   /* the band lies beyond the ellipse's top or bottom */
  float yr = -p->ys, yl = p->ys;
  yr = yr < d0 ? d0 : (yr > d1 ? d1 : yr);
  yl = yl < d0 ? d0 : (yl > d1 ? d1 : yl);
  float ar = p->a * p->Q - p->D * (yr * yr);
  float al = p->a * p->Q - p->D * (yl * yl);
  ar = ar > 0.0f ? ar : 0.0f;
  al = al > 0.0f ? al : 0.0f;
  const float xh = p->cx + (sqrtf(ar) - p->b * yr) / p->a + p->m;
  const float xl = p->cx + (-sqrtf(al) - p->b * yl) / p->a - p->m;
  /* pixel columns whose centre ix + 0.5 lies in [xl, xh], then their tiles */
  const float fl = ceilf(xl - 0.5f), fh = floorf(xh - 0.5f);
  if (fh < fl) return 0;
  const float lo_t = (float)rx0 * (float)tw, hi_t = (float)(rx1 + 1u) * (float)tw - 1.0f;
  if (fh < lo_t || fl > hi_t) return 0;
  const uint32_t il = fl > lo_t ? (uint32_t)fl : rx0 * tw;
  const uint32_t ih = fh < hi_t ? (uint32_t)fh : (rx1 + 1u) * tw - 1u;
  *tx0 = il >> tile_shift;
  *tx1 = ih >> tile_shift;
  return 1;
}

SL_SPAN_FN uint32_t sl_tile_shift(uint32_t tw) {
  uint32_t s = 0;
  while ((1u << s) < tw) s++;
  return s;
}

/* Tile columns [*tx0, *tx1] of tile row ty (tiles tw x th pixels, tw a power of two) that the splat (centre cx, cy;
 * gradients g0, g1; cutoff qcut) can reach, within the candidate rectangle's columns [rx0, rx1].  Returns 0 when the
 * row holds none. */
SL_SPAN_FN int sl_row_tiles(float cx, float cy, float g0x, float g0y, float g1x, float g1y, float qcut, uint32_t rx0,
                            uint32_t rx1, uint32_t ty, uint32_t tw, uint32_t th, uint32_t* tx0, uint32_t* tx1) {
  sl_span_prep p;
  sl_span_init(cx, cy, g0x, g0y, g1x, g1y, qcut, &p);
  return sl_span_row(&p, rx0, rx1, ty, tw, sl_tile_shift(tw), th, tx0, tx1);
}

#endif /* SL_TILESPAN_H */
