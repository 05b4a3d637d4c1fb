/*
 * sl_oracle_light.c -- CPU restatement of the per-Gaussian lighting that the splat pipeline composites.  TEST
 * INFRASTRUCTURE (see sl_oracle.c).  fp32 with -ffp-contract=off; transcendental functions from sl_detmath.h so the
 * GPU kernels (compiled with --fmad=false and the same functions) can agree to the last bit wherever the operation
 * order is the same.  Host-side set-up (the emitter tree, the shadow-map frames) is float64, as the reference's JS.
 *
 * Follows, per stage:
 *   iso_init        runtime/wgsl/iso_init.wgsl:29-56 (per-leaf iso_norm into Node.pad0)
 *   emitter tree    src/lighting.js:99-169 buildEmitterTree (+ EIN3 :55-56, ASG_WIDEN :66), EmitParams :657-673
 *   light map A     runtime/wgsl/light_shadow.wgsl:69-143, 191-392 (lsm_splat, lsm_resolve, lsm_down, lsm_lookup);
 *                   host src/light_shadow.js:89-140 (resolution, mip levels, light point and spread)
 *   sun maps        runtime/wgsl/sun_map.wgsl:91-324; host src/sun_map.js:23-159 (layer plan, cascades, margin)
 *   motion blur     runtime/wgsl/motion_blur.wgsl:22-127 (blur_records: the records the map splats draw for a moving
 *                   part, stretched over the exposure); lighting.js:468-507 (bound to the opacity-map splats only,
 *                   the ?blurcut=0 form: every record stretched, its mass kept)
 *   shade_emit      runtime/wgsl/emissive.wgsl:123-150, 853-980 (M39 iso transfer, ASG specular on)
 *   env_direct      runtime/wgsl/environment.wgsl:207-308 (env_add)
 *   materials       runtime/wgsl/material_ext.wgsl:27-181; common.wgsl:113-254 (erfc, sym_mul, dirm, vgrid, ein,
 *                   footprint, quat_matrix)
 * Build-defined (no reference counterpart): a constant sky ambient, colour += albedo * sky_ambient for non-emissive
 * Gaussians (the reference's sky reaches Gaussians only through the probe bounce, which is outside this pipeline).
 */
#define _GNU_SOURCE
#include "sl_oracle_light.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "sl_detmath.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_F 3.14159265358979f
#define NONE_U32 0xFFFFFFFFu

typedef struct { float x, y, z; } f3;
typedef struct { float x, y; } f2;
typedef struct { f3 c[3]; } m3f;   /* columns */
typedef struct { f2 c[2]; } m2f;   /* columns */
typedef struct { float x, y, z, w; } f4;

static f3 F3(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static f2 F2(float x, float y) { f2 r = {x, y}; return r; }
static f3 add3(f3 a, f3 b) { return F3(a.x + b.x, a.y + b.y, a.z + b.z); }
static f3 sub3(f3 a, f3 b) { return F3(a.x - b.x, a.y - b.y, a.z - b.z); }
static f3 mul3(f3 a, float s) { return F3(a.x * s, a.y * s, a.z * s); }
static f3 mul3v(f3 a, f3 b) { return F3(a.x * b.x, a.y * b.y, a.z * b.z); }
static f3 div3(f3 a, float s) { return F3(a.x / s, a.y / s, a.z / s); }
static float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float len3(f3 a) { return sqrtf(dot3(a, a)); }
static f3 norm3(f3 a) { return div3(a, len3(a)); }
static f3 cross3(f3 a, f3 b) { return F3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static float dot2(f2 a, f2 b) { return a.x * b.x + a.y * b.y; }
static f2 sub2(f2 a, f2 b) { return F2(a.x - b.x, a.y - b.y); }
static f2 mul2(f2 a, float s) { return F2(a.x * s, a.y * s); }
static f2 div2(f2 a, float s) { return F2(a.x / s, a.y / s); }
static float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
static float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static f4 mix4(f4 a, f4 b, float t) {
  f4 r = {mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t), mixf(a.w, b.w, t)};
  return r;
}
static float smoothstepf(float e0, float e1, float x) {
  float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
static f3 m3_mulv(const m3f* m, f3 v) {
  return F3(m->c[0].x * v.x + m->c[1].x * v.y + m->c[2].x * v.z, m->c[0].y * v.x + m->c[1].y * v.y + m->c[2].y * v.z,
            m->c[0].z * v.x + m->c[1].z * v.y + m->c[2].z * v.z);
}
static m3f m3_mul(const m3f* a, const m3f* b) {
  m3f r;
  for (int j = 0; j < 3; j++) r.c[j] = m3_mulv(a, b->c[j]);
  return r;
}
static m3f m3_t(const m3f* a) {
  m3f r;
  r.c[0] = F3(a->c[0].x, a->c[1].x, a->c[2].x);
  r.c[1] = F3(a->c[0].y, a->c[1].y, a->c[2].y);
  r.c[2] = F3(a->c[0].z, a->c[1].z, a->c[2].z);
  return r;
}
static m3f m3_diag(f3 d) {
  m3f r;
  r.c[0] = F3(d.x, 0.0f, 0.0f);
  r.c[1] = F3(0.0f, d.y, 0.0f);
  r.c[2] = F3(0.0f, 0.0f, d.z);
  return r;
}
static f2 m2_mulv(const m2f* m, f2 v) { return F2(m->c[0].x * v.x + m->c[1].x * v.y, m->c[0].y * v.x + m->c[1].y * v.y); }
static m2f m2_mul(const m2f* a, const m2f* b) {
  m2f r;
  r.c[0] = m2_mulv(a, b->c[0]);
  r.c[1] = m2_mulv(a, b->c[1]);
  return r;
}
static m2f m2_t(const m2f* a) {
  m2f r;
  r.c[0] = F2(a->c[0].x, a->c[1].x);
  r.c[1] = F2(a->c[0].y, a->c[1].y);
  return r;
}
static m2f m2_scale(const m2f* a, float s) {
  m2f r;
  r.c[0] = mul2(a->c[0], s);
  r.c[1] = mul2(a->c[1], s);
  return r;
}
static float m2_det(const m2f* m) { return m->c[0].x * m->c[1].y - m->c[1].x * m->c[0].y; }
/* inv2 (light_shadow.wgsl:98-101) */
static m2f m2_inv(const m2f* m) {
  float d = m2_det(m);
  m2f r;
  r.c[0] = F2(m->c[1].y, -m->c[0].y);
  r.c[1] = F2(-m->c[1].x, m->c[0].x);
  return m2_scale(&r, 1.0f / d);
}
static float f16_to_f32(uint32_t h) {
  uint32_t e = (h >> 10) & 31u, m = h & 1023u;
  float s = (h & 0x8000u) ? -1.0f : 1.0f;
  if (e == 0) return s * (float)m * 5.9604644775390625e-08f;
  if (e == 31) return m ? NAN : s * INFINITY;
  return s * (1.0f + (float)m / 1024.0f) * sl_bits_to_float((uint32_t)(e - 15 + 127) << 23);
}

/* ---- runtime/wgsl/common.wgsl helpers ---------------------------------------------------------------------- */

static f3 xf_point(const float* m, f3 p) {
  return F3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
static f3 xf_dir_inv(const float* m, f3 d) {
  return add3(add3(mul3(F3(m[0], m[1], m[2]), d.x), mul3(F3(m[4], m[5], m[6]), d.y)), mul3(F3(m[8], m[9], m[10]), d.z));
}
/* erfc_pos, Numerical Recipes erfcc (common.wgsl:113-118) */
static float erfc_pos(float z) {
  float t = 1.0f / (1.0f + 0.5f * z);
  float p = -z * z - 1.26551223f +
            t * (1.00002368f +
                 t * (0.37409196f +
                      t * (0.09678418f +
                           t * (-0.18628806f +
                                t * (0.27886807f + t * (-1.13520398f + t * (1.48851587f + t * (-0.82215223f + t * 0.17087277f))))))));
  return t * sl_expf(p);
}
static f3 sym_mul(f3 d, f3 o, f3 v) {
  return F3(d.x * v.x + o.x * v.y + o.y * v.z, o.x * v.x + d.y * v.y + o.z * v.z, o.y * v.x + o.z * v.y + d.z * v.z);
}
static f3 nd_cinv_d(const sl_node* n) { return F3(n->cinv_diag[0], n->cinv_diag[1], n->cinv_diag[2]); }
static f3 nd_cinv_o(const sl_node* n) { return F3(n->cinv_off[0], n->cinv_off[1], n->cinv_off[2]); }
static f3 nd_sn_d(const sl_node* n) { return F3(n->sn_diag[0], n->sn_diag[1], n->sn_diag[2]); }
static f3 nd_sn_o(const sl_node* n) { return F3(n->sn_off[0], n->sn_off[1], n->sn_off[2]); }
static float dirm(const sl_node* n, f3 w) { return sqrtf(fmaxf(dot3(w, sym_mul(nd_sn_d(n), nd_sn_o(n), w)), 0.0f)); }
static float vgrid_cell(const sl_vgrid* v, uint32_t i, uint32_t j) {
  uint32_t k = i * 16u + j;
  return (float)((v->w[k >> 2u] >> ((k & 3u) * 8u)) & 0xFFu) * (1.0f / 255.0f);
}
/* vgrid_lookup (common.wgsl:162-177) */
static float vgrid_lookup(const sl_vgrid* v, f3 w) {
  float el = sl_asinf(clampf(w.z, -1.0f, 1.0f));
  float fi = clampf((0.5f * PI_F - el) / (PI_F / 8.0f) - 0.5f, 0.0f, 7.0f);
  uint32_t i0 = (uint32_t)fi;
  if (i0 > 6u) i0 = 6u;
  float ti = fi - (float)i0;
  float az = (fabsf(w.x) + fabsf(w.y) < 1e-30f) ? 0.0f : sl_atan2f(w.y, w.x);
  float fj = (az + PI_F) / (2.0f * PI_F) * 16.0f - 0.5f;
  float j0f = floorf(fj);
  float tj = fj - j0f;
  uint32_t j0 = (uint32_t)((int32_t)j0f + 16) % 16u;
  uint32_t j1 = (j0 + 1u) % 16u;
  float a = mixf(vgrid_cell(v, i0, j0), vgrid_cell(v, i0, j1), tj);
  float b = mixf(vgrid_cell(v, i0 + 1u, j0), vgrid_cell(v, i0 + 1u, j1), tj);
  return mixf(a, b, ti);
}
static f3 basis_k(f3 w) {
  f3 a = F3(0.0f, 0.0f, 1.0f);
  if (fabsf(w.z) >= 0.999f) a = F3(1.0f, 0.0f, 0.0f);
  return norm3(cross3(a, w));
}
/* quat_matrix (common.wgsl:218-223) */
static m3f quat_matrix(const float* q) {
  float x = q[0], y = q[1], z = q[2], w = q[3];
  m3f m;
  m.c[0] = F3(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + z * w), 2.0f * (x * z - y * w));
  m.c[1] = F3(2.0f * (x * y - z * w), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + x * w));
  m.c[2] = F3(2.0f * (x * z + y * w), 2.0f * (y * z - x * w), 1.0f - 2.0f * (x * x + y * y));
  return m;
}
/* ein (common.wgsl:226-239) */
static float ein(float x) {
  if (x < 1.0f) {
    float term = x, s = x;
    for (int k = 2; k <= 12; k++) {
      term *= -x / (float)k;
      s += term / (float)k;
    }
    return s;
  }
  float p = x * x * x * x + 8.5733287401f * x * x * x + 18.0590169730f * x * x + 8.6347608925f * x + 0.2677737343f;
  float q = x * x * x * x + 9.5733223454f * x * x * x + 25.6329561486f * x * x + 21.0996530827f * x + 3.9584969228f;
  return sl_logf(x) + 0.5772156649f + p / q / (x * sl_expf(x));
}
/* footprint (common.wgsl:242-246) */
static float footprint(const sl_node* n, float detC, f3 w) {
  float a = dot3(w, sym_mul(nd_cinv_d(n), nd_cinv_o(n), w));
  float K = n->kappa * dirm(n, w) * sqrtf(2.0f * PI_F / a);
  return 2.0f * PI_F * sqrtf(detC * a) * ein(K);
}
static float iso_norm(const sl_node* n) { return sl_bits_to_float(n->pad0); }

/* ---- material_ext.wgsl ------------------------------------------------------------------------------------- */

static float sym_det(f3 d, f3 o) {
  return d.x * (d.y * d.z - o.z * o.z) - o.x * (o.x * d.z - o.z * o.y) + o.y * (o.x * o.z - d.y * o.y);
}
static float sym_adj_quad(f3 d, f3 o, f3 w) {
  float a00 = d.y * d.z - o.z * o.z, a11 = d.x * d.z - o.y * o.y, a22 = d.x * d.y - o.x * o.x;
  float a01 = o.y * o.z - o.x * d.z, a02 = o.x * o.z - o.y * d.y, a12 = o.x * o.y - d.x * o.z;
  return a00 * w.x * w.x + a11 * w.y * w.y + a22 * w.z * w.z + 2.0f * (a01 * w.x * w.y + a02 * w.x * w.z + a12 * w.y * w.z);
}
static float phase_specular(f3 Sd, f3 So, f3 wi, f3 wo) {
  f3 h = add3(wi, wo);
  float hl = len3(h);
  if (hl < 1e-6f) return 0.0f;
  f3 wh = div3(h, hl);
  float det = fmaxf(sym_det(Sd, So), 1e-20f);
  float q = sym_adj_quad(Sd, So, wh) / det;
  float D = 1.0f / (PI_F * sqrtf(det) * q * q);
  float sigma = sqrtf(fmaxf(dot3(wi, sym_mul(Sd, So, wi)), 1e-12f));
  return D / (4.0f * sigma);
}
static float spec_weight(const sl_material* m) {
  if ((m->flags & 8u) == 0u || (m->flags & 1u) != 0u) return 0.0f;
  return clampf(f16_to_f32(m->pad0 & 0xFFFFu), 0.0f, 1.0f);
}
static float iso_lobe_from(float k, float p, float damp) { return (1.0f - k) + k * 4.0f * PI_F * p * damp; }
static float iso_damp(float inorm, float avr) { return fminf(1.0f, 1.0f / fmaxf(4.0f * PI_F * inorm * avr, 1e-30f)); }
static f3 mirror3(f3 wi, f3 n) { return sub3(mul3(n, 2.0f * dot3(wi, n)), wi); }
static void onb(f3 n, f3* b0, f3* b1) {
  float s = n.z >= 0.0f ? 1.0f : -1.0f;
  float a = -1.0f / (s + n.z);
  float b = n.x * n.y * a;
  *b0 = F3(1.0f + s * n.x * n.x * a, s * b, -s * n.x);
  *b1 = F3(b, s + n.y * n.y * a, -n.y);
}
typedef struct { float x, y, z; } s2m; /* symmetric 2x2 (xx, xy, yy) */
static float s2_det(s2m s) { return s.x * s.z - s.y * s.y; }
static float s2_quad(s2m s, f2 v) { return s.x * v.x * v.x + 2.0f * s.y * v.x * v.y + s.z * v.y * v.y; }
static float s2_quad_inv(s2m s, f2 v) {
  return (s.z * v.x * v.x - 2.0f * s.y * v.x * v.y + s.x * v.y * v.y) / fmaxf(s2_det(s), 1e-30f);
}
static s2m s2_xf(s2m s, f2 t0, f2 t1) {
  f2 a = F2(s.x * t0.x + s.y * t0.y, s.y * t0.x + s.z * t0.y);
  f2 b = F2(s.x * t1.x + s.y * t1.y, s.y * t1.x + s.z * t1.y);
  s2m r = {dot2(t0, a), dot2(t0, b), dot2(t1, b)};
  return r;
}
static s2m s2_add(s2m a, s2m b) { s2m r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static s2m s2_div(s2m a, float d) { s2m r = {a.x / d, a.y / d, a.z / d}; return r; }
static f3 s2_major(s2m s) {
  float h = 0.5f * (s.x - s.z);
  float lam = 0.5f * (s.x + s.z) + sqrtf(h * h + s.y * s.y);
  f2 v = s.x >= s.z ? F2(lam - s.z, s.y) : F2(s.y, lam - s.x);
  float l = sqrtf(dot2(v, v));
  f2 u = l > 1e-20f ? div2(v, l) : F2(1.0f, 0.0f);
  return F3(u.x, u.y, lam);
}
static float s2_minor(s2m s) {
  float h = 0.5f * (s.x - s.z);
  return 0.5f * (s.x + s.z) - sqrtf(h * h + s.y * s.y);
}
static f2 log_map(f3 c, f3 cb0, f3 cb1, f3 a) {
  float ca = clampf(dot3(c, a), -1.0f, 1.0f);
  f3 v = sub3(a, mul3(c, ca));
  float nv = len3(v);
  if (nv < 1e-9f) return F2(0.0f, 0.0f);
  float k = sl_acosf(ca) / nv;
  return F2(k * dot3(cb0, v), k * dot3(cb1, v));
}
/* asg_phase (material_ext.wgsl:127-181) */
static float asg_phase(f3 wi, f3 lb0, f3 lb1, s2m sl, f3 n0, f3 t1, f3 t2, f3 flake, f3 Sd, f3 So, f3 wo) {
  static const float ASG_W[3] = {0.61163f, 0.35083f, 0.0267f};
  static const float ASG_A[3] = {2.54696f, 0.6893f, 0.10727f};
  float pc = phase_specular(Sd, So, wi, wo);
  if (flake.x <= fmaxf(flake.y, flake.z) * 1.0001f) return pc;
  float co = dot3(n0, wo);
  f3 n = co >= 0.0f ? n0 : mul3(n0, -1.0f);
  float cos_o = fabsf(co);
  f3 wr = sub3(mul3(n, 2.0f * cos_o), wo);
  f3 rb0, rb1;
  onb(wr, &rb0, &rb1);
  f3 dw1 = add3(mul3(n, 2.0f * dot3(wo, t1)), mul3(t1, 2.0f * cos_o));
  f3 dw2 = add3(mul3(n, 2.0f * dot3(wo, t2)), mul3(t2, 2.0f * cos_o));
  f2 j0 = F2(dot3(rb0, dw1), dot3(rb0, dw2));
  f2 j1 = F2(dot3(rb1, dw1), dot3(rb1, dw2));
  f2 ia = F2(flake.y / (flake.x - flake.y), flake.z / (flake.x - flake.z));
  s2m s0 = {dot2(F2(j0.x * j0.x, j0.y * j0.y), ia), dot2(F2(j0.x * j1.x, j0.y * j1.y), ia),
            dot2(F2(j1.x * j1.x, j1.y * j1.y), ia)};
  float pk = flake.x * flake.x / (PI_F * sqrtf(flake.x * flake.y * flake.z)) /
             (4.0f * sqrtf(fmaxf(dot3(wr, sym_mul(Sd, So, wr)), 1e-12f)));
  f3 cs = add3(wi, wr);
  float cl = len3(cs);
  if (cl < 1e-4f) return pc;
  f3 c = div3(cs, cl);
  f3 cb0, cb1;
  onb(c, &cb0, &cb1);
  f2 dm = sub2(log_map(c, cb0, cb1, wr), log_map(c, cb0, cb1, wi));
  s2m sL = s2_xf(sl, F2(dot3(cb0, lb0), dot3(cb0, lb1)), F2(dot3(cb1, lb0), dot3(cb1, lb1)));
  s2m sR = s2_xf(s0, F2(dot3(cb0, rb0), dot3(cb0, rb1)), F2(dot3(cb1, rb0), dot3(cb1, rb1)));
  float ndm = fmaxf(sqrtf(dot2(dm, dm)), 1e-9f);
  float d = sqrtf(s2_quad_inv(s2_add(sL, s2_div(sR, 2.0f * ASG_A[2])), dm));
  float along = sqrtf(fmaxf(s2_quad(sL, dm), 0.0f)) / ndm;
  float far_ = smoothstepf(1.0f, 2.5f, d) * (1.0f - smoothstepf(0.15f, 0.3f, along / ndm));
  f3 maj = s2_major(sl);
  float ratio = sqrtf(maj.z / fmaxf(s2_minor(s0) / (2.0f * ASG_A[0]), 1e-30f));
  float t = fmaxf(far_, 1.0f - smoothstepf(0.12f, 0.3f, ratio));
  float p_asg = 0.0f;
  if (t < 1.0f) {
    for (int k = 0; k < 3; k++) {
      s2m sk = s2_div(sR, 2.0f * ASG_A[k]);
      s2m st = s2_add(sL, sk);
      p_asg += ASG_W[k] * sqrtf(fmaxf(s2_det(sk), 0.0f) / fmaxf(s2_det(st), 1e-30f)) * sl_expf(-0.5f * s2_quad_inv(st, dm));
    }
    p_asg *= pk;
  }
  float p_pt = pc;
  if (t > 0.0f) {
    f3 ax = mul3(add3(mul3(lb0, maj.x), mul3(lb1, maj.y)), sqrtf(3.0f * maj.z));
    p_pt = (2.0f / 3.0f) * pc + (1.0f / 6.0f) * (phase_specular(Sd, So, norm3(add3(wi, ax)), wo) +
                                                  phase_specular(Sd, So, norm3(sub3(wi, ax)), wo));
  }
  return mixf(p_asg, p_pt, t);
}

/* ---- iso_init.wgsl ----------------------------------------------------------------------------------------- */

void orc_iso_dirs(float* dirs /* 128 x 4: w.xyz, solid angle */) {
  for (int c = 0; c < 128; c++) {
    int i = c / 16, j = c % 16;
    double el = 0.5 * M_PI - (i + 0.5) * M_PI / 8.0;
    double az = -M_PI + (j + 0.5) * 2.0 * M_PI / 16.0;
    double top = 0.5 * M_PI - i * M_PI / 8.0;
    dirs[4 * c + 0] = (float)(cos(el) * cos(az));
    dirs[4 * c + 1] = (float)(cos(el) * sin(az));
    dirs[4 * c + 2] = (float)sin(el);
    dirs[4 * c + 3] = (float)((2.0 * M_PI / 16.0) * (sin(top) - sin(top - M_PI / 8.0)));
  }
}

static void iso_one(uint32_t g, const sl_gaussian* gs, sl_node* nodes, const sl_vgrid* vgrid, const float* dirs) {
  const sl_gaussian* G = &gs[g];
  const sl_node* nd = &nodes[g];
  float s3 = G->scale[0] * G->scale[1] * G->scale[2];
  float S = 0.0f, S0 = 0.0f;
  for (uint32_t c = 0; c < 128u; c++) {
    f3 w = F3(dirs[4 * c], dirs[4 * c + 1], dirs[4 * c + 2]);
    float om = dirs[4 * c + 3];
    uint32_t k = c; /* i * 16 + j */
    float v = (float)((vgrid[g].w[k >> 2u] >> ((k & 3u) * 8u)) & 0xFFu) * (1.0f / 255.0f);
    float a = footprint(nd, s3 * s3, w) * om;
    S += a * v;
    S0 += a;
  }
  float n = 1.0f / fmaxf(fmaxf(S, 0.02f * S0), 1e-30f);
  nodes[g].pad0 = sl_float_to_bits(n);
  nodes[g].pad1 = 0u;
}

/* ---- emitter tree (src/lighting.js:99-169) ---------------------------------------------------------------- */

typedef struct {
  double mu[3], C[6], M[6], Cs[6], mass, Le[3], radius;
  uint32_t lo, hi;
} tnode;

static double ein3(void) {
  double acc = 0.0;
  for (int i = 0; i < 3000; i++) {
    double x = (i + 0.5) * 0.001;
    acc += (1.0 - exp(-x)) / x * 0.001;
  }
  return acc;
}
static double sdet(const double* m) {
  double a = m[0], d = m[1], f = m[2], b = m[3], c = m[4], e = m[5];
  return a * (d * f - e * e) - b * (b * f - e * c) + c * (b * e - d * c);
}
static void sinv(const double* m, double* o) {
  double a = m[0], d = m[1], f = m[2], b = m[3], c = m[4], e = m[5], det = sdet(m);
  o[0] = (d * f - e * e) / det;
  o[1] = (a * f - c * c) / det;
  o[2] = (a * d - b * b) / det;
  o[3] = (c * e - b * f) / det;
  o[4] = (b * e - c * d) / det;
  o[5] = (b * c - a * e) / det;
}
static double squad(const double* m, const double* w) {
  return m[0] * w[0] * w[0] + m[1] * w[1] * w[1] + m[2] * w[2] * w[2] +
         2 * (m[3] * w[0] * w[1] + m[4] * w[0] * w[2] + m[5] * w[1] * w[2]);
}
/* symAxes: Jacobi rotations, 12 sweeps (lighting.js:75-89); axes[k] = eigenvector k */
static void sym_axes(const double* m, double axes[3][3]) {
  double A[3][3] = {{m[0], m[3], m[4]}, {m[3], m[1], m[5]}, {m[4], m[5], m[2]}};
  double V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  static const int PQ[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int sweep = 0; sweep < 12; sweep++) {
    for (int r = 0; r < 3; r++) {
      int p = PQ[r][0], q = PQ[r][1];
      if (fabs(A[p][q]) < 1e-30) continue;
      double th = 0.5 * atan2(2 * A[p][q], A[q][q] - A[p][p]);
      double c = cos(th), s = sin(th);
      for (int k = 0; k < 3; k++) { double x = A[k][p], y = A[k][q]; A[k][p] = c * x - s * y; A[k][q] = s * x + c * y; }
      for (int k = 0; k < 3; k++) { double x = A[p][k], y = A[q][k]; A[p][k] = c * x - s * y; A[q][k] = s * x + c * y; }
      for (int k = 0; k < 3; k++) { double x = V[k][p], y = V[k][q]; V[k][p] = c * x - s * y; V[k][q] = s * x + c * y; }
    }
  }
  for (int k = 0; k < 3; k++)
    for (int i = 0; i < 3; i++) axes[k][i] = V[i][k];
}
static double lum(const double* c) { return 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2]; }

typedef struct {
  const float* rec;
  tnode* info;
  float* out;   /* 24 floats per node */
  uint32_t next;
  double ein3, widen;
  uint32_t* idx_buf;
  const double* le_scale;  /* per emitter: multiplies its Le (NULL: 1) */
} tbuild;

static uint32_t t_write(tbuild* B, const tnode* nd) {
  uint32_t id = B->next++;
  float* f = B->out + 24u * id;
  uint32_t* u = (uint32_t*)f;
  f[0] = (float)nd->mu[0]; f[1] = (float)nd->mu[1]; f[2] = (float)nd->mu[2]; f[3] = (float)nd->radius;
  f[4] = (float)nd->M[0]; f[5] = (float)nd->M[1]; f[6] = (float)nd->M[2]; f[7] = 0.0f;
  f[8] = (float)nd->M[3]; f[9] = (float)nd->M[4]; f[10] = (float)nd->M[5]; u[11] = nd->lo;
  f[12] = (float)nd->Le[0]; f[13] = (float)nd->Le[1]; f[14] = (float)nd->Le[2]; u[15] = nd->hi;
  f[16] = (float)nd->Cs[0]; f[17] = (float)nd->Cs[1]; f[18] = (float)nd->Cs[2]; f[19] = 0.0f;
  f[20] = (float)nd->Cs[3]; f[21] = (float)nd->Cs[4]; f[22] = (float)nd->Cs[5]; f[23] = 0.0f;
  B->info[id] = *nd;
  return id;
}

static tnode t_leaf(tbuild* B, uint32_t i) {
  const float* o = B->rec + 16u * i;
  tnode nd;
  memset(&nd, 0, sizeof nd);
  double x = o[4], y = o[5], z = o[6], w = o[7];
  double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                    {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                    {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
  double s2[3] = {(double)o[8] * o[8], (double)o[9] * o[9], (double)o[10] * o[10]};
  static const int IJ[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  for (int j = 0; j < 6; j++) {
    int r = IJ[j][0], k = IJ[j][1];
    nd.C[j] = R[r][0] * R[k][0] * s2[0] + R[r][1] * R[k][1] * s2[1] + R[r][2] * R[k][2] * s2[2];
  }
  double g = pow(2 * M_PI * B->ein3, 2) * sdet(nd.C);
  double Ci[6];
  sinv(nd.C, Ci);
  for (int j = 0; j < 6; j++) nd.M[j] = Ci[j] * g;
  nd.mass = o[3] * pow(2 * M_PI, 1.5) * sqrt(sdet(nd.C));
  for (int j = 0; j < 6; j++) nd.Cs[j] = nd.C[j] * B->widen;
  nd.mu[0] = o[0]; nd.mu[1] = o[1]; nd.mu[2] = o[2];
  double ls = B->le_scale ? B->le_scale[i] : 1.0;
  nd.Le[0] = o[12] * ls; nd.Le[1] = o[13] * ls; nd.Le[2] = o[14] * ls;
  double smax = fmax(fmax(o[8], o[9]), o[10]);
  nd.radius = 3 * smax;
  nd.lo = NONE_U32;
  nd.hi = i;
  return nd;
}

static uint32_t t_build(tbuild* B, uint32_t* idx, uint32_t n) {
  if (n == 1) {
    tnode l = t_leaf(B, idx[0]);
    return t_write(B, &l);
  }
  double lo[3], hi[3];
  for (int k = 0; k < 3; k++) { lo[k] = INFINITY; hi[k] = -INFINITY; }
  for (uint32_t a = 0; a < n; a++)
    for (int k = 0; k < 3; k++) {
      double v = B->rec[16u * idx[a] + k];
      lo[k] = fmin(lo[k], v);
      hi[k] = fmax(hi[k], v);
    }
  int ax = 0;
  for (int k = 0; k < 3; k++)
    if (hi[k] - lo[k] > hi[ax] - lo[ax]) ax = k;
  /* the JS sort compares positions and is stable: ties keep the incoming order of idx */
  uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * n * 2);
  for (uint32_t a = 0; a < n; a++) { tmp[2 * a] = idx[a]; tmp[2 * a + 1] = a; }
  /* insertion sort by (position, incoming rank): stable and deterministic (n <= a few thousand emitters) */
  for (uint32_t a = 1; a < n; a++) {
    uint32_t k0 = tmp[2 * a], r0 = tmp[2 * a + 1];
    double v0 = B->rec[16u * k0 + ax];
    int64_t b = (int64_t)a - 1;
    while (b >= 0) {
      double vb = B->rec[16u * tmp[2 * b] + ax];
      if (vb > v0) {
        tmp[2 * (b + 1)] = tmp[2 * b];
        tmp[2 * (b + 1) + 1] = tmp[2 * b + 1];
        b--;
      } else {
        break;
      }
    }
    tmp[2 * (b + 1)] = k0;
    tmp[2 * (b + 1) + 1] = r0;
  }
  for (uint32_t a = 0; a < n; a++) idx[a] = tmp[2 * a];
  free(tmp);
  uint32_t half = n >> 1;
  uint32_t ia = t_build(B, idx, half);
  uint32_t ib = t_build(B, idx + half, n - half);
  const tnode* kids[2] = {&B->info[ia], &B->info[ib]};
  tnode nd;
  memset(&nd, 0, sizeof nd);
  double m = kids[0]->mass + kids[1]->mass;
  for (int k = 0; k < 3; k++) nd.mu[k] = (kids[0]->mass * kids[0]->mu[k] + kids[1]->mass * kids[1]->mu[k]) / m;
  static const int IJ[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  for (int j = 0; j < 6; j++) {
    int r = IJ[j][0], k = IJ[j][1];
    double acc = 0.0, accs = 0.0;
    for (int c = 0; c < 2; c++) {
      acc += kids[c]->mass * (kids[c]->C[j] + (kids[c]->mu[r] - nd.mu[r]) * (kids[c]->mu[k] - nd.mu[k]));
      accs += kids[c]->mass * (kids[c]->Cs[j] + (kids[c]->mu[r] - nd.mu[r]) * (kids[c]->mu[k] - nd.mu[k]));
    }
    nd.C[j] = acc / m;
    nd.Cs[j] = accs / m;
  }
  double axes[3][3];
  sym_axes(nd.C, axes);
  double tot[3], num[3] = {0, 0, 0}, den = 0.0;
  for (int k = 0; k < 3; k++) {
    tot[k] = 0.0;
    for (int c = 0; c < 2; c++) tot[k] += lum(kids[c]->Le) * sqrt(fmax(squad(kids[c]->M, axes[k]), 0.0));
  }
  for (int c = 0; c < 2; c++) {
    double sw = 0.0;
    for (int k = 0; k < 3; k++) sw += sqrt(fmax(squad(kids[c]->M, axes[k]), 0.0));
    for (int ch = 0; ch < 3; ch++) num[ch] += kids[c]->Le[ch] * sw;
    den += sw;
  }
  for (int ch = 0; ch < 3; ch++) nd.Le[ch] = num[ch] / den;
  double L = fmax(lum(nd.Le), 1e-12);
  for (int j = 0; j < 6; j++) nd.M[j] = 0.0;
  for (int k = 0; k < 3; k++) {
    double lam = pow(tot[k] / L, 2);
    for (int j = 0; j < 6; j++) nd.M[j] += lam * axes[k][IJ[j][0]] * axes[k][IJ[j][1]];
  }
  double rad = -INFINITY;
  for (int c = 0; c < 2; c++) {
    double dx = kids[c]->mu[0] - nd.mu[0], dy = kids[c]->mu[1] - nd.mu[1], dz = kids[c]->mu[2] - nd.mu[2];
    rad = fmax(rad, sqrt(dx * dx + dy * dy + dz * dz) + kids[c]->radius);
  }
  nd.radius = rad;
  nd.mass = m;
  nd.lo = ia;
  nd.hi = ib;
  return t_write(B, &nd);
}

/* The same tree in double precision with each emitter's Le scaled by le_scale (the differentiable path's
 * intensities): per node 16 doubles (mu xyz, radius, M xx yy zz xy xz yz, Le rgb, child_lo, child_hi, 0; children as
 * numbers, -1 for none).  Returns the root. */
uint32_t orc_emitter_tree_d(const float* rec, uint32_t n, const double* le_scale, double* nodes_out) {
  tbuild B;
  memset(&B, 0, sizeof B);
  B.rec = rec;
  B.info = (tnode*)calloc(2u * n, sizeof(tnode));
  float* tmp = (float*)calloc(24u * (2u * n), sizeof(float));
  B.out = tmp;
  B.ein3 = ein3();
  B.widen = B.ein3 / (1.0 - exp(-3.0));
  B.le_scale = le_scale;
  uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * n);
  for (uint32_t i = 0; i < n; i++) idx[i] = i;
  uint32_t root = t_build(&B, idx, n);
  for (uint32_t e = 0; e < 2 * n - 1; e++) {
    const tnode* t = &B.info[e];
    double* o = nodes_out + 16u * e;
    for (int k = 0; k < 3; k++) o[k] = t->mu[k];
    o[3] = t->radius;
    for (int j = 0; j < 6; j++) o[4 + j] = t->M[j];
    for (int k = 0; k < 3; k++) o[10 + k] = t->Le[k];
    o[13] = t->lo == NONE_U32 ? -1.0 : (double)t->lo;
    o[14] = t->lo == NONE_U32 ? -1.0 : (double)t->hi;
    o[15] = 0.0;
  }
  free(idx);
  free(tmp);
  free(B.info);
  return root;
}

uint32_t orc_emitter_tree(const float* rec, uint32_t n, float* nodes_out, float* root_cov) {
  tbuild B;
  memset(&B, 0, sizeof B);
  B.rec = rec;
  B.info = (tnode*)calloc(2u * n, sizeof(tnode));
  B.out = nodes_out;
  B.next = 0;
  B.ein3 = ein3();
  B.widen = B.ein3 / (1.0 - exp(-3.0));
  uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * n);
  for (uint32_t i = 0; i < n; i++) idx[i] = i;
  uint32_t root = t_build(&B, idx, n);
  if (root_cov)
    for (int j = 0; j < 6; j++) root_cov[j] = (float)B.info[root].Cs[j];
  free(idx);
  free(B.info);
  return root;
}

/* eig3 closed form (src/light_shadow.js:169-180), ascending */
static void eig3(const double* m, double* ev) {
  double a = m[0], d = m[1], f = m[2], b = m[3], c = m[4], e = m[5];
  double p1 = b * b + c * c + e * e;
  double q = (a + d + f) / 3;
  double p2 = (a - q) * (a - q) + (d - q) * (d - q) + (f - q) * (f - q) + 2 * p1;
  double p = sqrt(p2 / 6);
  if (p < 1e-30) { ev[0] = ev[1] = ev[2] = q; return; }
  double B[6] = {(a - q) / p, (d - q) / p, (f - q) / p, b / p, c / p, e / p};
  double r = (B[0] * (B[1] * B[2] - B[5] * B[5]) - B[3] * (B[3] * B[2] - B[5] * B[4]) + B[4] * (B[3] * B[5] - B[1] * B[4])) / 2;
  double phi = acos(fmin(1, fmax(-1, r))) / 3;
  double e1 = q + 2 * p * cos(phi), e3 = q + 2 * p * cos(phi + 2 * M_PI / 3);
  ev[0] = e3;
  ev[1] = 3 * q - e1 - e3;
  ev[2] = e1;
}

/* ---- opacity maps: shared splat / resolve / mips (light_shadow.wgsl:191-341, sun_map.wgsl:155-277) ------------ */

typedef struct {
  /* light map A: light frame */
  f3 center, normal, t1, t2;
  uint32_t hemi;
} lframe;

static f2 oct_uv(const lframe* L, f3 w) {
  f3 l = F3(dot3(w, L->t1), dot3(w, L->t2), dot3(w, L->normal));
  if (L->hemi) {
    float z = fmaxf(l.z, 0.0f);
    f2 p = div2(F2(l.x, l.y), fmaxf(fabsf(l.x) + fabsf(l.y) + z, 1e-12f));
    return F2(p.x + p.y, p.x - p.y);
  }
  f2 p = div2(F2(l.x, l.y), fmaxf(fabsf(l.x) + fabsf(l.y) + fabsf(l.z), 1e-12f));
  if (l.z < 0.0f) {
    float sx = p.x >= 0.0f ? 1.0f : -1.0f, sy = p.y >= 0.0f ? 1.0f : -1.0f;
    p = F2((1.0f - fabsf(p.y)) * sx, (1.0f - fabsf(p.x)) * sy);
  }
  return p;
}
static m2f oct_jac(const lframe* L, f3 w, f3 b0, f3 b1) {
  float e = 1e-3f;
  f2 u0 = oct_uv(L, w);
  f2 ua = oct_uv(L, norm3(add3(w, mul3(b0, e))));
  f2 ub = oct_uv(L, norm3(add3(w, mul3(b1, e))));
  m2f J;
  J.c[0] = div2(sub2(ua, u0), e);
  J.c[1] = div2(sub2(ub, u0), e);
  return J;
}
static f3 part_rot_col(const float* xf, int c) { return F3(xf[c], xf[4 + c], xf[8 + c]); }
/* ---- motion_blur.wgsl blur_records (:80-127) ------------------------------------------------------------------ */

static float m3_at(const m3f* m, int col, int row) {
  const f3* c = &m->c[col];
  return row == 0 ? c->x : (row == 1 ? c->y : c->z);
}
static void m3_set(m3f* m, int col, int row, float v) {
  f3* c = &m->c[col];
  if (row == 0) c->x = v; else if (row == 1) c->y = v; else c->z = v;
}
static m3f m3_identity(void) { return m3_diag(F3(1.0f, 1.0f, 1.0f)); }

/* cyclic Jacobi (8 sweeps over the pairs (0,1) (0,2) (1,2)): the columns of V are eigenvectors, the result the
 * eigenvalues (motion_blur.wgsl:37-60) */
static f3 blur_eig3(m3f A, m3f* V) {
  m3f Q = m3_identity();
  for (int sweep = 0; sweep < 8; sweep++)
    for (int k = 0; k < 3; k++) {
      const int pp = k == 2 ? 1 : 0, q = k == 2 ? 2 : k + 1;
      const float apq = m3_at(&A, q, pp);
      if (fabsf(apq) < 1e-30f) continue;
      const float theta = 0.5f * (m3_at(&A, q, q) - m3_at(&A, pp, pp)) / apq;
      const float sg = theta + (theta == 0.0f ? 1e-30f : 0.0f);
      const float sgn = sg > 0.0f ? 1.0f : (sg < 0.0f ? -1.0f : 0.0f);
      const float t = sgn / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
      const float c = 1.0f / sqrtf(t * t + 1.0f);
      const float sn = t * c;
      m3f J = m3_identity();
      m3_set(&J, pp, pp, c);
      m3_set(&J, q, q, c);
      m3_set(&J, q, pp, sn);
      m3_set(&J, pp, q, -sn);
      m3f Jt = m3_t(&J);
      m3f T1 = m3_mul(&Jt, &A);
      A = m3_mul(&T1, &J);
      Q = m3_mul(&Q, &J);
    }
  *V = Q;
  return F3(A.c[0].x, A.c[1].y, A.c[2].z);
}

/* column-major rotation -> quaternion (x, y, z, w), normalised (motion_blur.wgsl:62-78) */
static void blur_mat_to_quat(const m3f* m, float* q4) {
  const float m00 = m3_at(m, 0, 0), m11 = m3_at(m, 1, 1), m22 = m3_at(m, 2, 2);
  const float tr = m00 + m11 + m22;
  float q[4];
  if (tr > 0.0f) {
    const float s = sqrtf(tr + 1.0f) * 2.0f;
    q[0] = (m3_at(m, 1, 2) - m3_at(m, 2, 1)) / s;
    q[1] = (m3_at(m, 2, 0) - m3_at(m, 0, 2)) / s;
    q[2] = (m3_at(m, 0, 1) - m3_at(m, 1, 0)) / s;
    q[3] = 0.25f * s;
  } else if (m00 > m11 && m00 > m22) {
    const float s = sqrtf(1.0f + m00 - m11 - m22) * 2.0f;
    q[0] = 0.25f * s;
    q[1] = (m3_at(m, 1, 0) + m3_at(m, 0, 1)) / s;
    q[2] = (m3_at(m, 2, 0) + m3_at(m, 0, 2)) / s;
    q[3] = (m3_at(m, 1, 2) - m3_at(m, 2, 1)) / s;
  } else if (m11 > m22) {
    const float s = sqrtf(1.0f + m11 - m00 - m22) * 2.0f;
    q[0] = (m3_at(m, 1, 0) + m3_at(m, 0, 1)) / s;
    q[1] = 0.25f * s;
    q[2] = (m3_at(m, 2, 1) + m3_at(m, 1, 2)) / s;
    q[3] = (m3_at(m, 2, 0) - m3_at(m, 0, 2)) / s;
  } else {
    const float s = sqrtf(1.0f + m22 - m00 - m11) * 2.0f;
    q[0] = (m3_at(m, 2, 0) + m3_at(m, 0, 2)) / s;
    q[1] = (m3_at(m, 2, 1) + m3_at(m, 1, 2)) / s;
    q[2] = 0.25f * s;
    q[3] = (m3_at(m, 0, 1) - m3_at(m, 1, 0)) / s;
  }
  const float l = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int k = 0; k < 4; k++) q4[k] = q[k] / l;
}

void orc_blur_record(const sl_part* parts, uint32_t part_count, float shutter, const sl_gaussian* g_in,
                     const sl_node* n_in, sl_gaussian* g_out, sl_node* n_out) {
  sl_node nd = *n_in;
  sl_gaussian G = *g_in;
  /* blur_disp: the rest-frame displacement of the node's mean over the exposure */
  f3 d = F3(0.0f, 0.0f, 0.0f);
  const uint32_t p = nd.part;
  if (shutter > 0.0f && p < part_count && (parts[p].flags & 2u) != 0u) {
    const f3 x = F3(nd.mean[0], nd.mean[1], nd.mean[2]);
    const f3 a = xf_point(parts[p].xf, x), b = xf_point(parts[p].xf_prev, x);
    d = xf_dir_inv(parts[p].xf, F3(shutter * (a.x - b.x), shutter * (a.y - b.y), shutter * (a.z - b.z)));
  }
  const float dd = dot3(d, d);
  if (dd > 0.0f) {
    /* Sherman-Morrison: (C + d d^T / 12)^-1 from C^-1 */
    m3f Ci;
    Ci.c[0] = F3(nd.cinv_diag[0], nd.cinv_off[0], nd.cinv_off[1]);
    Ci.c[1] = F3(nd.cinv_off[0], nd.cinv_diag[1], nd.cinv_off[2]);
    Ci.c[2] = F3(nd.cinv_off[1], nd.cinv_off[2], nd.cinv_diag[2]);
    const f3 cd = m3_mulv(&Ci, d);
    const float m = dot3(d, cd);
    const float inv = 1.0f / (12.0f + m);
    const float cdv[3] = {cd.x, cd.y, cd.z};
    m3f Cn;
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) m3_set(&Cn, j, i, m3_at(&Ci, j, i) - (cdv[i] * cdv[j]) * inv);
    nd.mean[0] = nd.mean[0] - 0.5f * d.x;
    nd.mean[1] = nd.mean[1] - 0.5f * d.y;
    nd.mean[2] = nd.mean[2] - 0.5f * d.z;
    nd.cinv_diag[0] = m3_at(&Cn, 0, 0);
    nd.cinv_diag[1] = m3_at(&Cn, 1, 1);
    nd.cinv_diag[2] = m3_at(&Cn, 2, 2);
    nd.cinv_off[0] = m3_at(&Cn, 0, 1);
    nd.cinv_off[1] = m3_at(&Cn, 0, 2);
    nd.cinv_off[2] = m3_at(&Cn, 1, 2);
    nd.kappa = nd.kappa / sqrtf(1.0f + m / 12.0f);
    nd.smax = sqrtf(nd.smax * nd.smax + dd / 12.0f);
    nd.radius = sqrtf(nd.radius * nd.radius + 0.75f * dd);
    /* the Gaussian: the stretched covariance's eigen-frame, ascending, right-handed */
    m3f Rq = quat_matrix(G.quat);
    const f3 s2 = F3(G.scale[0] * G.scale[0], G.scale[1] * G.scale[1], G.scale[2] * G.scale[2]);
    m3f D = m3_diag(s2);
    m3f T1 = m3_mul(&Rq, &D);
    m3f RqT = m3_t(&Rq);
    m3f C = m3_mul(&T1, &RqT);
    const float dv[3] = {d.x, d.y, d.z};
    const float k12 = 1.0f / 12.0f;
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) m3_set(&C, j, i, m3_at(&C, j, i) + (dv[i] * dv[j]) * k12);
    m3f V;
    f3 ev = blur_eig3(C, &V);
    f3 c0 = V.c[0], c1 = V.c[1], c2 = V.c[2];
    if (ev.x > ev.y) { ev = F3(ev.y, ev.x, ev.z); f3 t = c0; c0 = c1; c1 = t; }
    if (ev.y > ev.z) { ev = F3(ev.x, ev.z, ev.y); f3 t = c1; c1 = c2; c2 = t; }
    if (ev.x > ev.y) { ev = F3(ev.y, ev.x, ev.z); f3 t = c0; c0 = c1; c1 = t; }
    c2 = cross3(c0, c1);
    G.mu[0] = G.mu[0] - 0.5f * d.x;
    G.mu[1] = G.mu[1] - 0.5f * d.y;
    G.mu[2] = G.mu[2] - 0.5f * d.z;
    G.kappa = nd.kappa;
    G.scale[0] = sqrtf(fmaxf(ev.x, 1e-12f));
    G.scale[1] = sqrtf(fmaxf(ev.y, 1e-12f));
    G.scale[2] = sqrtf(fmaxf(ev.z, 1e-12f));
    m3f R;
    R.c[0] = c0;
    R.c[1] = c1;
    R.c[2] = c2;
    blur_mat_to_quat(&R, G.quat);
  }
  *n_out = nd;
  *g_out = G;
}

/* world covariance R C R^T of a leaf (light_shadow.wgsl:125-137) */
static m3f leaf_cov_world(const sl_gaussian* G, const float* xf) {
  m3f R;
  for (int c = 0; c < 3; c++) R.c[c] = part_rot_col(xf, c);
  m3f Rq = quat_matrix(G->quat);
  f3 s2 = F3(G->scale[0] * G->scale[0], G->scale[1] * G->scale[1], G->scale[2] * G->scale[2]);
  m3f D = m3_diag(s2);
  m3f t0 = m3_mul(&Rq, &D);
  m3f RqT = m3_t(&Rq);
  m3f C = m3_mul(&t0, &RqT);
  m3f t1 = m3_mul(&R, &C);
  m3f RT = m3_t(&R);
  return m3_mul(&t1, &RT);
}

/* inv3 (light_shadow.wgsl:119-122) */
static m3f inv3(const m3f* m) {
  f3 r0 = cross3(m->c[1], m->c[2]), r1 = cross3(m->c[2], m->c[0]), r2 = cross3(m->c[0], m->c[1]);
  float id = 1.0f / dot3(m->c[0], r0);
  m3f r;
  r.c[0] = F3(r0.x * id, r1.x * id, r2.x * id);
  r.c[1] = F3(r0.y * id, r1.y * id, r2.y * id);
  r.c[2] = F3(r0.z * id, r1.z * id, r2.z * id);
  return r;
}
/* world covariance of record g: a leaf from its Gaussian, a tree node from its C^-1 (light_shadow.wgsl:125-137) */
static m3f rec_cov(const sl_gaussian* gs, const sl_node* nodes, uint32_t count, uint32_t g, const float* xf) {
  if (g < count) return leaf_cov_world(&gs[g], xf);
  const sl_node* n = &nodes[g];
  m3f S;
  S.c[0] = F3(n->cinv_diag[0], n->cinv_off[0], n->cinv_off[1]);
  S.c[1] = F3(n->cinv_off[0], n->cinv_diag[1], n->cinv_off[2]);
  S.c[2] = F3(n->cinv_off[1], n->cinv_off[2], n->cinv_diag[2]);
  m3f C = inv3(&S);
  m3f R;
  for (int c = 0; c < 3; c++) R.c[c] = part_rot_col(xf, c);
  m3f t = m3_mul(&R, &C);
  m3f RT = m3_t(&R);
  return m3_mul(&t, &RT);
}
/* the motion-blur cut of the map splats (light_shadow.wgsl:158-210, sun_map.wgsl:119-153) */
typedef struct {
  const sl_gaussian* g_rest;
  const sl_node* n_rest;
  const uint32_t* parent;
  uint32_t n_nodes;
  float k, shutter;
} bcut;
/* 0 = not splatted, 1 = as it is, 2 = keeping its rest coverage */
static int cut_verdict(const bcut* bc, const sl_part* parts, uint32_t count, uint32_t g, uint32_t p) {
  int leaf = g < count;
  float L = 0.0f;
  uint32_t root = parts[p].root;
  if (bc->k > 0.0f && bc->shutter > 0.0f && (parts[p].flags & 2u) != 0u && root < bc->n_nodes) {
    const sl_node* rn = &bc->n_rest[root];
    f3 x = F3(rn->mean[0], rn->mean[1], rn->mean[2]);
    f3 a = xf_point(parts[p].xf, x), b = xf_point(parts[p].xf_prev, x);
    L = bc->shutter * len3(sub3(a, b));
  }
  if (L <= 0.0f) return leaf ? 1 : 0;
  float thr = bc->k * L;
  if (!leaf && bc->n_rest[g].radius > thr) return 0;
  uint32_t par = bc->parent[g];
  if (g != root && par != NONE_U32 && bc->n_rest[par].radius <= thr) return 0;
  return 2;
}

static void atomic_add_u32(uint32_t* p, uint32_t v) {
#ifdef _OPENMP
#pragma omp atomic
#endif
  *p += v;
}
static uint32_t to_u32(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967040.0f) return 0xFFFFFF00u;
  return (uint32_t)x;
}

/* splat one leaf into light map A layer p (light_shadow.wgsl:212-286) */
static void lsm_splat_one(const lframe* L, uint32_t res, uint32_t g, uint32_t p, const sl_gaussian* gs,
                          const sl_node* nodes, const sl_part* parts, uint32_t count, const bcut* bc, int verdict,
                          uint32_t* acc) {
  const float FIX = 65536.0f, LOWPASS = 0.3f;
  const float* xf = parts[p].xf;
  const sl_node* nd = &nodes[g];
  f3 mu = g < count ? F3(gs[g].mu[0], gs[g].mu[1], gs[g].mu[2]) : F3(nd->mean[0], nd->mean[1], nd->mean[2]);
  f3 m = xf_point(xf, mu);
  f3 dv = sub3(m, L->center);
  float r = len3(dv);
  if (r < 1e-4f) return;
  f3 w = div3(dv, r);
  m3f C = rec_cov(gs, nodes, count, g, xf);
  if (L->hemi && dot3(dv, L->normal) < -3.0f * sqrtf(dot3(L->normal, m3_mulv(&C, L->normal)))) return;
  f3 b0 = basis_k(w), b1 = cross3(w, b0);
  f3 c0 = m3_mulv(&C, b0), c1 = m3_mulv(&C, b1);
  float cbbx = dot3(b0, c0), cbby = dot3(b0, c1), cbbz = dot3(b1, c1);
  f3 cw = m3_mulv(&C, w);
  f2 cbz = F2(dot3(b0, cw), dot3(b1, cw));
  float czz = dot3(w, cw);
  m2f Cbb;
  Cbb.c[0] = F2(cbbx, cbby);
  Cbb.c[1] = F2(cbby, cbbz);
  m2f Cbb_i = m2_inv(&Cbb);
  float sz2 = fmaxf(czz - dot2(cbz, m2_mulv(&Cbb_i, cbz)), 1e-12f);
  float tau0 = nd->kappa * dirm(nd, xf_dir_inv(xf, w)) * sqrtf(2.0f * PI_F * sz2);
  float half_res = 0.5f * (float)res;
  m2f J0 = oct_jac(L, w, b0, b1);
  m2f J = m2_scale(&J0, half_res);
  m2f Sang = m2_scale(&Cbb, 1.0f / (r * r));
  m2f t = m2_mul(&J, &Sang);
  m2f JT = m2_t(&J);
  m2f S = m2_mul(&t, &JT);
  float det0 = m2_det(&S);
  S.c[0].x += LOWPASS;
  S.c[1].y += LOWPASS;
  float det1 = m2_det(&S);
  tau0 *= sqrtf(fmaxf(det0, 0.0f) / det1);
  if (verdict == 2) {
    /* the rest record's peak opacity spread evenly over the stretched footprint: alpha' A' = alpha A */
    const sl_node* ndr = &bc->n_rest[g];
    m3f Cr = rec_cov(bc->g_rest, bc->n_rest, count, g, xf);
    f3 cwr = m3_mulv(&Cr, w);
    f3 r0 = m3_mulv(&Cr, b0), r1 = m3_mulv(&Cr, b1);
    m2f Cbr;
    Cbr.c[0] = F2(dot3(b0, r0), dot3(b0, r1));
    Cbr.c[1] = F2(dot3(b0, r1), dot3(b1, r1));
    f2 cbzr = F2(dot3(b0, cwr), dot3(b1, cwr));
    m2f Cbr_i = m2_inv(&Cbr);
    float szr = fmaxf(dot3(w, cwr) - dot2(cbzr, m2_mulv(&Cbr_i, cbzr)), 1e-12f);
    m2f Sa = m2_scale(&Cbr, 1.0f / (r * r));
    m2f tr = m2_mul(&J, &Sa);
    m2f Sr = m2_mul(&tr, &JT);
    float d0r = m2_det(&Sr);
    Sr.c[0].x += LOWPASS;
    Sr.c[1].y += LOWPASS;
    float d1r = m2_det(&Sr);
    float tau_r = ndr->kappa * dirm(ndr, xf_dir_inv(xf, w)) * sqrtf(2.0f * PI_F * szr) * sqrtf(fmaxf(d0r, 0.0f) / d1r);
    float a = fminf((1.0f - sl_expf(-tau_r)) * sqrtf(fmaxf(d1r, 1e-30f) / fmaxf(det1, 1e-30f)), 0.999f);
    tau0 = fminf(-sl_logf(1.0f - a), tau0);
  }
  m2f Si = m2_inv(&S);
  m2f Ji = m2_inv(&J);
  m2f JiT = m2_t(&Ji);
  f2 gz = m2_mulv(&JiT, mul2(m2_mulv(&Cbb_i, cbz), r));
  f2 uv = oct_uv(L, w);
  f2 ct = F2((uv.x * 0.5f + 0.5f) * (float)res, (uv.y * 0.5f + 0.5f) * (float)res);
  int hx = (int)ceilf(3.0f * sqrtf(S.c[0].x)), hy = (int)ceilf(3.0f * sqrtf(S.c[1].y));
  if (hx > 48) hx = 48;
  if (hy > 48) hy = 48;
  int cx = (int)floorf(ct.x), cy = (int)floorf(ct.y);
  uint32_t base = p * res * res;
  int ires = (int)res;
  for (int y = cy - hy > 0 ? cy - hy : 0; y <= (cy + hy < ires - 1 ? cy + hy : ires - 1); y++) {
    for (int x = cx - hx > 0 ? cx - hx : 0; x <= (cx + hx < ires - 1 ? cx + hx : ires - 1); x++) {
      f2 dt = sub2(F2((float)x + 0.5f, (float)y + 0.5f), ct);
      float q = dot2(dt, m2_mulv(&Si, dt));
      if (q > 9.0f) continue;
      float tt = fminf(tau0 * sl_expf(-0.5f * q), 64.0f);
      float t_fix = tt * FIX;
      if (t_fix < 0.5f) continue;
      float z = fmaxf(r + dot2(gz, dt), 0.0f);
      uint32_t k = (base + (uint32_t)y * res + (uint32_t)x) * 3u;
      atomic_add_u32(&acc[k], to_u32(t_fix + 0.5f));
      atomic_add_u32(&acc[k + 1], to_u32(t_fix * z + 0.5f));
      atomic_add_u32(&acc[k + 2], to_u32(t_fix * (z * z + sz2) + 0.5f));
    }
  }
}

static void resolve_layer(const uint32_t* acc, float fix, uint32_t texels, f4* mip0) {
  for (uint32_t i = 0; i < texels; i++) {
    float s0 = (float)acc[3 * i] / fix;
    f4 o = {0, 0, 0, 0};
    if (s0 > 1e-5f) {
      float a = 1.0f - sl_expf(-s0);
      o.x = a;
      o.y = a * (float)acc[3 * i + 1] / (fix * s0);
      o.z = a * (float)acc[3 * i + 2] / (fix * s0);
    }
    mip0[i] = o;
  }
}
static void mips_layer(f4* layer, const uint32_t* level_off, uint32_t levels, uint32_t res) {
  for (uint32_t k = 1; k < levels; k++) {
    uint32_t rk = res >> k, pr = rk * 2;
    for (uint32_t y = 0; y < rk; y++)
      for (uint32_t x = 0; x < rk; x++) {
        const f4* s = layer + level_off[k - 1] + (2 * y) * pr + 2 * x;
        f4 a = s[0], b = s[1], c = s[pr], d = s[pr + 1];
        f4 o = {0.25f * (a.x + b.x + c.x + d.x), 0.25f * (a.y + b.y + c.y + d.y), 0.25f * (a.z + b.z + c.z + d.z),
                0.25f * (a.w + b.w + c.w + d.w)};
        layer[level_off[k] + y * rk + x] = o;
      }
  }
}
static f4 mip_at(const f4* layer, const uint32_t* level_off, uint32_t res, uint32_t k, f2 tc) {
  uint32_t rk = res >> k;
  if (rk < 1u) rk = 1u;
  float sc = (float)(1u << k);
  float cxf = clampf(tc.x / sc - 0.5f, 0.0f, (float)(rk - 1u)), cyf = clampf(tc.y / sc - 0.5f, 0.0f, (float)(rk - 1u));
  uint32_t i0x = (uint32_t)floorf(cxf), i0y = (uint32_t)floorf(cyf);
  uint32_t i1x = i0x + 1u < rk - 1u ? i0x + 1u : rk - 1u, i1y = i0y + 1u < rk - 1u ? i0y + 1u : rk - 1u;
  float fx = cxf - (float)i0x, fy = cyf - (float)i0y;
  const f4* b = layer + level_off[k];
  f4 a = mix4(b[i0y * rk + i0x], b[i0y * rk + i1x], fx);
  f4 c = mix4(b[i1y * rk + i0x], b[i1y * rk + i1x], fx);
  return mix4(a, c, fy);
}
static f4 mip_tri(const f4* layer, const uint32_t* level_off, uint32_t res, uint32_t levels, float l, f2 tc) {
  float lc = clampf(l, 0.0f, (float)(levels - 1u));
  uint32_t k0 = (uint32_t)floorf(lc);
  uint32_t k1 = k0 + 1u < levels - 1u ? k0 + 1u : levels - 1u;
  return mix4(mip_at(layer, level_off, res, k0, tc), mip_at(layer, level_off, res, k1, tc), lc - (float)k0);
}
static float phi_cdf(float x) {
  float a = fabsf(x) * 0.70710678f;
  float h = 0.5f * erfc_pos(a);
  return x >= 0.0f ? 1.0f - h : h;
}

/* ---- the whole lighting update ------------------------------------------------------------------------------- */

static uint32_t mat_index(const sl_gaussian* G, uint32_t mat_count) {
  uint32_t m = G->flags & 0xFFFFu, top = (mat_count > 1u ? mat_count : 1u) - 1u;
  return m < top ? m : top;
}

int orc_lighting(const sl_gaussian* gs, uint32_t count, const sl_part* parts, uint32_t part_count, sl_node* nodes,
                 const sl_vgrid* vgrid, const sl_material* mats, uint32_t mat_count, const orc_light_setup* S,
                 float* colour, float* lamp_T, float* env_T, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  /* iso_init (once per asset) */
  float dirs[512];
  orc_iso_dirs(dirs);
  if (!S->shade_only) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 1024)
#endif
    for (int64_t g = 0; g < (int64_t)count; g++) iso_one((uint32_t)g, gs, nodes, vgrid, dirs);
  }

  /* emitter tree + params (lighting.js:657-673) */
  uint32_t n_emit = S->n_emit;
  float* tree = NULL;
  uint32_t root = 0;
  float root_cov[6] = {0, 0, 0, 0, 0, 0};
  if (n_emit) {
    tree = (float*)calloc((size_t)(2u * n_emit - 1u) * 24u, sizeof(float));
    root = orc_emitter_tree(S->emit_rec, n_emit, tree, root_cov);
  }

  /* motion blur for the lighting (motion_blur.wgsl, lighting.js:468-507): the opacity-map splats draw every record of
   * a moving part stretched over the exposure; the receivers (lookups, shading) keep their rest records */
  const sl_gaussian* gsp = gs;
  const sl_node* ndp = nodes;
  sl_gaussian* g_blur = NULL;
  sl_node* n_blur = NULL;
  const int have_tree = S->tree_nodes && S->n_tree > count;
  const uint32_t n_nodes = have_tree ? S->n_tree : count;
  bcut bc = {gs, have_tree ? S->tree_nodes : nodes, have_tree ? S->tree_parent : NULL, n_nodes, 0.0f,
             S->blur_shutter};
  uint32_t n_rec = count;
  if (S->blur_shutter > 0.0f && !S->shade_only) {
    g_blur = (sl_gaussian*)malloc(sizeof(sl_gaussian) * (count ? count : 1u));
    n_blur = (sl_node*)malloc(sizeof(sl_node) * (n_nodes ? n_nodes : 1u));
    for (uint32_t g = 0; g < count; g++)
      orc_blur_record(parts, part_count, S->blur_shutter, &gs[g], &bc.n_rest[g], &g_blur[g], &n_blur[g]);
    for (uint32_t i = count; i < n_nodes; i++) {  /* tree nodes: the node record alone */
      sl_gaussian dummy;
      memset(&dummy, 0, sizeof dummy);
      dummy.quat[3] = 1.0f;
      dummy.scale[0] = dummy.scale[1] = dummy.scale[2] = 1.0f;
      sl_gaussian unused;
      orc_blur_record(parts, part_count, S->blur_shutter, &dummy, &bc.n_rest[i], &unused, &n_blur[i]);
    }
    gsp = g_blur;
    ndp = n_blur;
    if (have_tree) {
      bc.k = S->cut_k;
      if (bc.k > 0.0f) n_rec = n_nodes;
    }
  }

  /* light map A (light_shadow.js:89-165): all layers dirty, then the lookup */
  if (!S->shade_only)
    for (uint32_t g = 0; g < count; g++) lamp_T[g] = 1.0f;
  if (n_emit && S->shadow_res && !S->shade_only) {
    uint32_t res = S->shadow_res, levels = 0, off = 0, level_off[16];
    for (uint32_t k = res; k >= 1u; k >>= 1) { level_off[levels++] = off; off += k * k; }
    uint32_t layer_texels = off;
    lframe L;
    L.center = F3(tree[24u * root], tree[24u * root + 1], tree[24u * root + 2]);
    double n[3] = {S->normal[0], S->normal[1], S->normal[2]};
    double nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; k++) n[k] /= nl;
    double a[3] = {fabs(n[0]) < 0.9 ? 1.0 : 0.0, fabs(n[0]) < 0.9 ? 0.0 : 1.0, 0.0};
    double t1[3] = {n[1] * a[2] - n[2] * a[1], n[2] * a[0] - n[0] * a[2], n[0] * a[1] - n[1] * a[0]};
    double tl = sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
    for (int k = 0; k < 3; k++) t1[k] /= tl;
    double t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
    L.normal = F3((float)n[0], (float)n[1], (float)n[2]);
    L.t1 = F3((float)t1[0], (float)t1[1], (float)t1[2]);
    L.t2 = F3((float)t2[0], (float)t2[1], (float)t2[2]);
    L.hemi = S->one_sided ? 1u : 0u;
    double cd[6] = {root_cov[0], root_cov[1], root_cov[2], root_cov[3], root_cov[4], root_cov[5]};
    double ev[3];
    eig3(cd, ev);
    float sigma_l = (float)sqrt(0.5 * (ev[1] + ev[2]));
    uint32_t* acc = (uint32_t*)calloc((size_t)part_count * res * res * 3u, sizeof(uint32_t));
    f4* mip = (f4*)calloc((size_t)part_count * layer_texels, sizeof(f4));
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
#endif
    for (int64_t gi = 0; gi < (int64_t)n_rec; gi++) {
      uint32_t g = (uint32_t)gi;
      uint32_t p = g < count ? (gsp[g].part_surface & 0xFFFFu) : bc.n_rest[g].part;
      if (p >= part_count || p == S->skip_part) continue;
      int verdict = cut_verdict(&bc, parts, count, g, p);
      if (verdict) lsm_splat_one(&L, res, g, p, gsp, ndp, parts, count, &bc, verdict, acc);
    }
    for (uint32_t p = 0; p < part_count; p++) {
      resolve_layer(acc + (size_t)p * res * res * 3u, 65536.0f, res * res, mip + (size_t)p * layer_texels);
      mips_layer(mip + (size_t)p * layer_texels, level_off, levels, res);
    }
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 1024)
#endif
    for (int64_t gi = 0; gi < (int64_t)count; gi++) {
      uint32_t g = (uint32_t)gi;
      const sl_gaussian* G = &gs[g];
      uint32_t own = G->part_surface & 0xFFFFu;
      f3 P = xf_point(parts[own].xf, F3(G->mu[0], G->mu[1], G->mu[2]));
      f3 dv = sub3(P, L.center);
      float z = len3(dv);
      if (z < 1e-4f) { lamp_T[g] = 1.0f; continue; }
      f3 w = div3(dv, z);
      f3 b0 = basis_k(w), b1 = cross3(w, b0);
      m2f J = oct_jac(&L, w, b0, b1);
      float tex_ang = (2.0f / (float)res) / sqrtf(fmaxf(fabsf(m2_det(&J)), 1e-12f));
      f2 uv = oct_uv(&L, w);
      f2 tc = F2((uv.x * 0.5f + 0.5f) * (float)res, (uv.y * 0.5f + 0.5f) * (float)res);
      float T = 1.0f;
      for (uint32_t p = 0; p < part_count; p++) {
        if (p == own || p == S->skip_part) continue;
        const float* bs = parts[p].bound;
        f3 bc = sub3(xf_point(parts[p].xf, F3(bs[0], bs[1], bs[2])), L.center);
        float dc = len3(bc);
        float zn = fmaxf(dc - bs[3], 0.02f);
        if (z <= zn) continue;
        float search = 2.0f * sigma_l * (z - zn) / (zn * z);
        if (dc > bs[3]) {
          float ang = sl_acosf(clampf(dot3(div3(bc, dc), w), -1.0f, 1.0f));
          if (ang > sl_asinf(bs[3] / dc) + search + 2.0f * tex_ang) continue;
        }
        const f4* layer = mip + (size_t)p * layer_texels;
        float ls = sl_log2f(fmaxf(2.0f * search / tex_ang, 1.0f));
        f4 a0 = mip_tri(layer, level_off, res, levels, ceilf(ls), tc);
        if (a0.x < 1e-4f) continue;
        float zb = fmaxf(a0.y / a0.x, 0.02f);
        float pen = sigma_l * fmaxf(z - zb, 0.0f) / (zb * z);
        f4 s = mip_tri(layer, level_off, res, levels, sl_log2f(fmaxf(2.0f * pen / tex_ang, 1.0f)), tc);
        if (s.x < 1e-5f) continue;
        float mu_ = s.y / s.x;
        float sd = sqrtf(fmaxf(s.z / s.x - mu_ * mu_, 1e-8f));
        T *= 1.0f - s.x * phi_cdf((z - mu_) / sd);
      }
      lamp_T[g] = T;
    }
    free(acc);
    free(mip);
  }

  /* sun maps (sun_map.js:23-159, sun_map.wgsl) */
  if (!S->shade_only)
    for (uint32_t g = 0; g < count; g++) env_T[4u * g] = env_T[4u * g + 1] = env_T[4u * g + 2] = env_T[4u * g + 3] = 1.0f;
  uint32_t K = S->n_lights < 4u ? S->n_lights : 4u;
  uint32_t Pn = part_count < 32u ? part_count : 32u;
  if (K && S->sun_res && !S->shade_only) {
    /* layer plan: per part with Gaussians, per light: cascades (8 m, 32 m) below 1.5 x the bound for large static
     * parts, then the fitted map */
    typedef struct { uint32_t p, k, kind; float c[2], half; } ldesc;
    ldesc* desc = (ldesc*)calloc((size_t)Pn * K * 3u, sizeof(ldesc));
    uint32_t nl = 0;
    double ext = 0.0, sig_max = 0.0;
    for (uint32_t p = 0; p < Pn; p++) {
      const float* b = parts[p].bound;
      ext = fmax(ext, sqrt((double)b[0] * b[0] + (double)b[1] * b[1] + (double)b[2] * b[2]) + b[3]);
    }
    for (uint32_t k = 0; k < K; k++) sig_max = fmax(sig_max, S->lights[k].std);
    float margin = (float)(3.0 * sig_max * 2.0 * ext);
    static const double CASC[2] = {8.0, 32.0};
    for (uint32_t p = 0; p < Pn; p++) {
      if (!(parts[p].g_hi > parts[p].g_lo)) continue;
      int big = parts[p].bound[3] > CASC[0] && (parts[p].flags & 1u);
      for (uint32_t k = 0; k < K; k++) {
        if (big)
          for (int c = 0; c < 2; c++) {
            if (!(CASC[c] < parts[p].bound[3] * 1.5)) continue;
            double L[3] = {S->lights[k].dir[0], S->lights[k].dir[1], S->lights[k].dir[2]};
            double aa[3] = {0, 0, 1};
            if (fabs(L[2]) >= 0.999) { aa[0] = 1; aa[2] = 0; }
            double t1[3] = {aa[1] * L[2] - aa[2] * L[1], aa[2] * L[0] - aa[0] * L[2], aa[0] * L[1] - aa[1] * L[0]};
            double tn = sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
            for (int q = 0; q < 3; q++) t1[q] /= tn;
            double t2[3] = {L[1] * t1[2] - L[2] * t1[1], L[2] * t1[0] - L[0] * t1[2], L[0] * t1[1] - L[1] * t1[0]};
            double h = CASC[c];
            double at[3] = {S->eye[0] + S->fwd[0] * h * 0.75, S->eye[1] + S->fwd[1] * h * 0.75,
                            S->eye[2] + S->fwd[2] * h * 0.75};
            ldesc* d = &desc[nl++];
            d->p = p;
            d->k = k;
            d->kind = 1;
            d->half = (float)h;
            d->c[0] = (float)(at[0] * t1[0] + at[1] * t1[1] + at[2] * t1[2]);
            d->c[1] = (float)(at[0] * t2[0] + at[1] * t2[1] + at[2] * t2[2]);
          }
        ldesc* d = &desc[nl++];
        d->p = p;
        d->k = k;
        d->kind = 0;
      }
    }
    uint32_t res = S->sun_res, levels = 0, off = 0, level_off[16];
    for (uint32_t k = res; k >= 1u; k >>= 1) { level_off[levels++] = off; off += k * k; }
    uint32_t layer_texels = off;
    /* sm_frame (sun_map.wgsl:91-107) */
    typedef struct { f2 c; float half, zref; f3 t1, t2; uint32_t part, light; } slayer;
    slayer* ly = (slayer*)calloc(nl ? nl : 1, sizeof(slayer));
    for (uint32_t l = 0; l < nl; l++) {
      f3 Ld = F3(S->lights[desc[l].k].dir[0], S->lights[desc[l].k].dir[1], S->lights[desc[l].k].dir[2]);
      f3 t1 = basis_k(Ld), t2 = cross3(Ld, t1);
      const float* b = parts[desc[l].p].bound;
      f3 c = xf_point(parts[desc[l].p].xf, F3(b[0], b[1], b[2]));
      f2 cc = F2(dot3(c, t1), dot3(c, t2));
      float half = b[3] + margin;
      if (desc[l].kind == 1u) { cc = F2(desc[l].c[0], desc[l].c[1]); half = desc[l].half; }
      ly[l].c = cc;
      ly[l].half = half;
      ly[l].zref = dot3(c, Ld) + b[3];
      ly[l].t1 = t1;
      ly[l].t2 = t2;
      ly[l].part = desc[l].p;
      ly[l].light = desc[l].k;
    }
    uint32_t* acc = (uint32_t*)calloc((size_t)(nl ? nl : 1) * res * res * 3u, sizeof(uint32_t));
    f4* mip = (f4*)calloc((size_t)(nl ? nl : 1) * layer_texels, sizeof(f4));
    const float SM_FIX = 4096.0f, SM_LOWPASS = 0.3f;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
#endif
    for (int64_t gi = 0; gi < (int64_t)n_rec; gi++) {
      uint32_t g = (uint32_t)gi;
      uint32_t p = g < count ? (gsp[g].part_surface & 0xFFFFu) : bc.n_rest[g].part;
      if (p >= Pn) continue;
      int verdict = cut_verdict(&bc, parts, count, g, p);
      if (!verdict) continue;
      for (uint32_t l = 0; l < nl; l++) {
        if (ly[l].part != p || !(S->lights[ly[l].light].shadows)) continue;
        /* sm_splat_one (sun_map.wgsl:155-219) */
        const float* xf = parts[p].xf;
        const sl_node* nd = &ndp[g];
        f3 mu = g < count ? F3(gsp[g].mu[0], gsp[g].mu[1], gsp[g].mu[2]) : F3(nd->mean[0], nd->mean[1], nd->mean[2]);
        f3 x = xf_point(xf, mu);
        f3 w = F3(S->lights[ly[l].light].dir[0], S->lights[ly[l].light].dir[1], S->lights[ly[l].light].dir[2]);
        f3 b0 = ly[l].t1, b1 = ly[l].t2;
        m3f C = rec_cov(gsp, ndp, count, g, xf);
        f3 c0 = m3_mulv(&C, b0), c1 = m3_mulv(&C, b1), cw = m3_mulv(&C, w);
        m2f Cbb;
        Cbb.c[0] = F2(dot3(b0, c0), dot3(b1, c0));
        Cbb.c[1] = F2(dot3(b0, c1), dot3(b1, c1));
        f2 cbz = F2(dot3(b0, cw), dot3(b1, cw));
        m2f Cbb_i = m2_inv(&Cbb);
        float sz2 = fmaxf(dot3(w, cw) - dot2(cbz, m2_mulv(&Cbb_i, cbz)), 1e-12f);
        float tex = (float)res / (2.0f * ly[l].half);
        m2f Sm = m2_scale(&Cbb, tex * tex);
        float det0 = m2_det(&Sm);
        Sm.c[0].x += SM_LOWPASS;
        Sm.c[1].y += SM_LOWPASS;
        float det1 = m2_det(&Sm);
        float tau0 = nd->kappa * dirm(nd, xf_dir_inv(xf, w)) * sqrtf(2.0f * PI_F * sz2) * sqrtf(fmaxf(det0, 0.0f) / det1);
        if (verdict == 2) { /* keep the rest record's coverage (sun_map.wgsl:178-193) */
          const sl_node* ndr = &bc.n_rest[g];
          m3f Cr = rec_cov(bc.g_rest, bc.n_rest, count, g, xf);
          f3 r0 = m3_mulv(&Cr, b0), r1 = m3_mulv(&Cr, b1), rw = m3_mulv(&Cr, w);
          m2f Cbr;
          Cbr.c[0] = F2(dot3(b0, r0), dot3(b1, r0));
          Cbr.c[1] = F2(dot3(b0, r1), dot3(b1, r1));
          f2 cbzr = F2(dot3(b0, rw), dot3(b1, rw));
          m2f Cbr_i = m2_inv(&Cbr);
          float szr = fmaxf(dot3(w, rw) - dot2(cbzr, m2_mulv(&Cbr_i, cbzr)), 1e-12f);
          m2f Sr = m2_scale(&Cbr, tex * tex);
          float d0r = m2_det(&Sr);
          Sr.c[0].x += SM_LOWPASS;
          Sr.c[1].y += SM_LOWPASS;
          float d1r = m2_det(&Sr);
          float tau_r = ndr->kappa * dirm(ndr, xf_dir_inv(xf, w)) * sqrtf(2.0f * PI_F * szr) *
                        sqrtf(fmaxf(d0r, 0.0f) / d1r);
          float a = fminf((1.0f - sl_expf(-tau_r)) * sqrtf(fmaxf(d1r, 1e-30f) / fmaxf(det1, 1e-30f)), 0.999f);
          tau0 = fminf(-sl_logf(1.0f - a), tau0);
        }
        m2f Si = m2_inv(&Sm);
        float z0 = ly[l].zref - dot3(x, w);
        f2 gz = div2(m2_mulv(&Cbb_i, cbz), tex);
        f2 ct = F2((dot3(x, b0) - ly[l].c.x + ly[l].half) * tex, (dot3(x, b1) - ly[l].c.y + ly[l].half) * tex);
        int hx = (int)ceilf(3.0f * sqrtf(Sm.c[0].x)), hy = (int)ceilf(3.0f * sqrtf(Sm.c[1].y));
        if (hx > 32) hx = 32;
        if (hy > 32) hy = 32;
        int cx = (int)floorf(ct.x), cy = (int)floorf(ct.y);
        uint32_t base = l * res * res;
        int ires = (int)res;
        for (int y = cy - hy > 0 ? cy - hy : 0; y <= (cy + hy < ires - 1 ? cy + hy : ires - 1); y++) {
          for (int xx = cx - hx > 0 ? cx - hx : 0; xx <= (cx + hx < ires - 1 ? cx + hx : ires - 1); xx++) {
            f2 dt = sub2(F2((float)xx + 0.5f, (float)y + 0.5f), ct);
            float q = dot2(dt, m2_mulv(&Si, dt));
            if (q > 9.0f) continue;
            float tt = fminf(tau0 * sl_expf(-0.5f * q), 64.0f);
            float t_fix = tt * SM_FIX;
            if (t_fix < 0.5f) continue;
            float z = fmaxf(z0 - dot2(gz, dt), 0.0f);
            uint32_t i = (base + (uint32_t)y * res + (uint32_t)xx) * 3u;
            atomic_add_u32(&acc[i], to_u32(t_fix + 0.5f));
            atomic_add_u32(&acc[i + 1], to_u32(t_fix * z + 0.5f));
            atomic_add_u32(&acc[i + 2], to_u32(t_fix * (z * z + sz2) + 0.5f));
          }
        }
      }
    }
    for (uint32_t l = 0; l < nl; l++) {
      resolve_layer(acc + (size_t)l * res * res * 3u, SM_FIX, res * res, mip + (size_t)l * layer_texels);
      mips_layer(mip + (size_t)l * layer_texels, level_off, levels, res);
    }
    /* sm_lookup (sun_map.wgsl:287-324) */
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 1024)
#endif
    for (int64_t gi = 0; gi < (int64_t)count; gi++) {
      uint32_t g = (uint32_t)gi;
      const sl_gaussian* G = &gs[g];
      uint32_t own = G->part_surface & 0xFFFFu;
      f3 P = xf_point(parts[own].xf, F3(G->mu[0], G->mu[1], G->mu[2]));
      float T[4] = {1, 1, 1, 1};
      uint32_t used = NONE_U32;
      for (uint32_t l = 0; l < nl; l++) {
        uint32_t key = ly[l].part * 8u + ly[l].light;
        if (ly[l].part == own || key == used || !(S->lights[ly[l].light].shadows)) continue;
        f3 w = F3(S->lights[ly[l].light].dir[0], S->lights[ly[l].light].dir[1], S->lights[ly[l].light].dir[2]);
        f2 uv = sub2(F2(dot3(P, ly[l].t1), dot3(P, ly[l].t2)), ly[l].c);
        float inner = (desc[l].kind == 1u ? 0.9f : 1.0f) * ly[l].half;
        if (fabsf(uv.x) >= inner || fabsf(uv.y) >= inner) continue;
        used = key;
        float z = ly[l].zref - dot3(P, w);
        if (z <= 0.0f) continue;
        float texel = 2.0f * ly[l].half / (float)res;
        f2 tc = F2((uv.x + ly[l].half) / texel, (uv.y + ly[l].half) / texel);
        float sig = S->lights[ly[l].light].std;
        float search = 2.0f * sig * z;
        const f4* layer = mip + (size_t)l * layer_texels;
        f4 a0 = mip_tri(layer, level_off, res, levels, sl_log2f(fmaxf(2.0f * search / texel, 1.0f)), tc);
        if (a0.x < 1e-4f) continue;
        float zb = a0.y / a0.x;
        float pen = sig * fmaxf(z - zb, 0.0f);
        f4 s = mip_tri(layer, level_off, res, levels, sl_log2f(fmaxf(2.0f * pen / texel, 1.0f)), tc);
        if (s.x < 1e-5f) continue;
        float mu_ = s.y / s.x;
        float sd = sqrtf(fmaxf(s.z / s.x - mu_ * mu_, 1e-8f));
        T[ly[l].light] *= 1.0f - s.x * phi_cdf((z - mu_) / sd);
      }
      for (int k = 0; k < 4; k++) env_T[4u * g + (uint32_t)k] = T[k];
    }
    free(acc);
    free(mip);
    free(ly);
    free(desc);
  }

  /* shade: shade_emit (emissive.wgsl:944-980) + env_direct (environment.wgsl:225-308) + sky ambient */
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 512)
#endif
  for (int64_t gi = 0; gi < (int64_t)count; gi++) {
    uint32_t g = (uint32_t)gi;
    const sl_gaussian* G = &gs[g];
    const sl_node* nd = &nodes[g];
    const sl_material* mat = &mats[mat_index(G, mat_count)];
    const float* xf = parts[G->part_surface & 0xFFFFu].xf;
    m3f Rq = quat_matrix(G->quat);
    m3f Dm = m3_diag(F3(mat->flake[0], mat->flake[1], mat->flake[2]));
    m3f t0 = m3_mul(&Rq, &Dm);
    m3f RqT = m3_t(&Rq);
    m3f Sloc = m3_mul(&t0, &RqT);
    float s3 = G->scale[0] * G->scale[1] * G->scale[2];
    float detC = s3 * s3;
    f3 P = xf_point(xf, F3(G->mu[0], G->mu[1], G->mu[2]));
    f3 n = Rq.c[0], t1 = Rq.c[1], t2 = Rq.c[2];
    f3 Sd = F3(Sloc.c[0].x, Sloc.c[1].y, Sloc.c[2].z), So = F3(Sloc.c[1].x, Sloc.c[2].x, Sloc.c[2].y);
    f3 flake = F3(mat->flake[0], mat->flake[1], mat->flake[2]);
    f3 alb = F3(G->albedo[0], G->albedo[1], G->albedo[2]);
    float ks = spec_weight(mat);
    int emissive = (mat->flags & 1u) != 0u;
    f3 eye = F3(S->eye[0], S->eye[1], S->eye[2]);
    f3 c = F3(0.0f, 0.0f, 0.0f);
    if (n_emit || emissive) {
      f3 wo0 = xf_dir_inv(xf, norm3(sub3(eye, P)));
      f3 acc = F3(0.0f, 0.0f, 0.0f);
      if (n_emit) {
        uint32_t stack[48];
        uint32_t sp = 1;
        stack[0] = root;
        int shape = S->asg && ks > 0.0f;
        while (sp > 0u) {
          sp--;
          const float* e = tree + 24u * stack[sp];
          uint32_t child_lo = sl_float_to_bits(e[11]), child_hi = sl_float_to_bits(e[15]);
          f3 emean = F3(e[0], e[1], e[2]);
          int use;
          if (child_lo == NONE_U32 || S->mode == 0u) {
            use = child_lo == NONE_U32;
          } else {
            f3 d = sub3(P, emean);
            use = dot3(d, d) > S->theta * S->theta * e[3] * e[3];
          }
          if (!use) {
            if (sp + 2u <= 48u) { stack[sp] = child_lo; stack[sp + 1u] = child_hi; sp += 2u; }
            continue;
          }
          f3 d = sub3(emean, P);
          float d2 = dot3(d, d);
          if (d2 < 1e-8f) continue;
          f3 ww = div3(d, sqrtf(d2));
          f3 wi = xf_dir_inv(xf, ww);
          float vi = vgrid_lookup(&vgrid[g], wi);
          if (vi <= 1e-7f) continue;
          float fp = footprint(nd, detC, wi);
          /* intensity(e, -ww) (emissive.wgsl:123-130): one-sided emitters fade over |cos| < edge_soft */
          f3 mw = mul3(ww, -1.0f);
          float s = 1.0f;
          if (S->one_sided) {
            f3 nn = F3(S->normal[0], S->normal[1], S->normal[2]);
            float cs = dot3(mw, nn);
            s = S->edge_soft > 0.0f ? smoothstepf(-S->edge_soft, S->edge_soft, cs) : (cs > 0.0f ? 1.0f : 0.0f);
          }
          float mq = sqrtf(fmaxf(dot3(mw, sym_mul(F3(e[4], e[5], e[6]), F3(e[8], e[9], e[10]), mw)), 0.0f));
          f3 I = mul3(F3(e[12], e[13], e[14]), s * S->scale * mq);
          f3 light = mul3(mul3(I, vi), fp / d2 * 1.0f);
          if (ks <= 0.0f) {
            acc = add3(acc, light);
            continue;
          }
          f3 wr = mirror3(wi, n);
          float damp = iso_damp(iso_norm(nd), footprint(nd, detC, wr) * vgrid_lookup(&vgrid[g], wr));
          if (shape) {
            f3 bw0, bw1;
            onb(ww, &bw0, &bw1);
            f3 cd = F3(e[16], e[17], e[18]), co = F3(e[20], e[21], e[22]);
            f3 cc0 = sym_mul(cd, co, bw0), cc1 = sym_mul(cd, co, bw1);
            s2m slm = {dot3(bw0, cc0) / d2, dot3(bw0, cc1) / d2, dot3(bw1, cc1) / d2};
            f3 lb0 = xf_dir_inv(xf, bw0), lb1 = xf_dir_inv(xf, bw1);
            float p = asg_phase(wi, lb0, lb1, slm, n, t1, t2, flake, Sd, So, wo0);
            acc = add3(acc, mul3(light, iso_lobe_from(ks, p, damp)));
            continue;
          }
          float k = ks;
          float lobe = k <= 0.0f ? 1.0f : iso_lobe_from(k, phase_specular(Sd, So, wi, wo0), damp);
          acc = add3(acc, mul3(light, lobe));
        }
      }
      float T = lamp_T[g];
      c = mul3(mul3v(alb, acc), T * iso_norm(nd));
      if (emissive && ((mat->flags & 4u) == 0u || dot3(wo0, n) > 0.0f)) {
        c = add3(c, F3(f16_to_f32(mat->pad0 & 0xFFFFu), f16_to_f32(mat->pad0 >> 16), f16_to_f32(mat->pad1 & 0xFFFFu)));
      }
    }
    /* env_direct (environment.wgsl:266-308) */
    if (K && !emissive) {
      float inorm = iso_norm(nd);
      if (ks <= 0.0f) {
        f3 dc = F3(0.0f, 0.0f, 0.0f);
        for (uint32_t k = 0; k < K; k++) {
          f3 wi = xf_dir_inv(xf, F3(S->lights[k].dir[0], S->lights[k].dir[1], S->lights[k].dir[2]));
          float v = vgrid_lookup(&vgrid[g], wi);
          if (v <= 1e-7f) continue;
          dc = add3(dc, mul3(F3(S->lights[k].irr[0], S->lights[k].irr[1], S->lights[k].irr[2]),
                             env_T[4u * g + k] * v * footprint(nd, detC, wi)));
        }
        c = add3(c, mul3(mul3v(alb, dc), inorm));
      } else {
        f3 wo = xf_dir_inv(xf, norm3(sub3(eye, P)));
        f3 diff = F3(0.0f, 0.0f, 0.0f), spec = F3(0.0f, 0.0f, 0.0f);
        for (uint32_t k = 0; k < K; k++) {
          f3 wi = xf_dir_inv(xf, F3(S->lights[k].dir[0], S->lights[k].dir[1], S->lights[k].dir[2]));
          float v = vgrid_lookup(&vgrid[g], wi);
          if (v <= 1e-7f) continue;
          f3 light = mul3(F3(S->lights[k].irr[0], S->lights[k].irr[1], S->lights[k].irr[2]),
                          env_T[4u * g + k] * v * footprint(nd, detC, wi));
          f3 wr = mirror3(wi, n);
          float damp = iso_damp(inorm, footprint(nd, detC, wr) * vgrid_lookup(&vgrid[g], wr));
          float s2 = S->lights[k].std * S->lights[k].std;
          f3 ob0, ob1;
          onb(wi, &ob0, &ob1);
          s2m slm = {s2, 0.0f, s2};
          float p = asg_phase(wi, ob0, ob1, slm, n, t1, t2, flake, Sd, So, wo);
          diff = add3(diff, mul3(light, 1.0f - ks));
          spec = add3(spec, mul3(light, iso_lobe_from(ks, p, damp) - (1.0f - ks)));
        }
        c = add3(c, mul3v(mul3(alb, inorm), add3(diff, spec)));
      }
    }
    if (!emissive && S->sky_ambient > 0.0f) c = add3(c, mul3(alb, S->sky_ambient));
    colour[4u * g] = c.x;
    colour[4u * g + 1] = c.y;
    colour[4u * g + 2] = c.z;
    colour[4u * g + 3] = 1.0f;
  }
  free(tree);
  free(g_blur);
  free(n_blur);
  return 0;
}

/* ---- probe bounce (runtime/wgsl/bounce.wgsl; host src/lighting.js:170-286, 723-816, 1018-1103) -------------------
 * The M39 stage-2 loop of the reference's non-sender-cut path (?sendercut=0) over the probe lattice, one frame per
 * call: iso_xfer (bounce.wgsl:993-1026), direct_dirs_emit (emissive.wgsl:1012-1016, 1066-1082) and env_dirs
 * (environment.wgsl:311-359) for a quarter of the Gaussians, node_leaf / node_up / node_sh2 (bounce.wgsl:1166-1236),
 * probe_gather (:1255-1410, no rectangle lamps), probe_valid (:1417-1447), probe_sh2 (:1029-1041), bounce_sh
 * (:1044-1095, with gloss_sh :1102-1125) and bounce_dirs (:887-985).  The probes: the lattice, 8 riding on each
 * movable part (part_probe_frame) and the static volumes' grids (vol_frame); near-field visibility is off
 * (near_byte = 1, the reference's default).  The WGSL pow(x, 3) of probe_cheb is taken as x x x.  The sender cut
 * (the reference's default) follows below. */

#define BN_NCELL 128u
#define BN_HIT_MAX 16u
#define BN_STACK 64u
#define BN_THETA 4.0f
#define BN_NEAR_R 0.3f
#define BN_G_VALID 0.95f
#define BN_GLOSS_SH_MIN 0.1f

static const double bn_d14_raw[14][3] = {{1, 0, 0}, {0, 1, 0}, {1e-4, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {1e-4, 0, -1},
                                         {1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                                         {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};

/* D14 (lighting.js:188-189: 6 axes, the verticals leaning 1e-4 off the pole, then the 8 diagonals / sqrt 3) and the
 * least-squares SH2 fit of values on them, pinv = (A^T A)^-1 A^T (lighting.js pinvD14, Gauss-Jordan), float64 */
void orc_bounce_tables(float* d14 /* 14 x 3 */, float* pinv /* 9 x 14 */) {
  double A[14][9], D[14][3];
  for (int k = 0; k < 14; k++) {
    double s = k < 6 ? 1.0 : 1.0 / sqrt(3.0);
    for (int c = 0; c < 3; c++) D[k][c] = bn_d14_raw[k][c] * s;
    double x = D[k][0], y = D[k][1], z = D[k][2];
    double b[9] = {0.282095, 0.488603 * y, 0.488603 * z, 0.488603 * x, 1.092548 * x * y, 1.092548 * y * z,
                   0.315392 * (3 * z * z - 1), 1.092548 * x * z, 0.546274 * (x * x - y * y)};
    for (int m = 0; m < 9; m++) A[k][m] = b[m];
    for (int c = 0; c < 3; c++) d14[3 * k + c] = (float)D[k][c];
  }
  double M[9][18];
  for (int i = 0; i < 9; i++)
    for (int j = 0; j < 9; j++) {
      double s = 0.0;
      for (int r = 0; r < 14; r++) s += A[r][i] * A[r][j];
      M[i][j] = s;
      M[i][9 + j] = i == j ? 1.0 : 0.0;
    }
  for (int c = 0; c < 9; c++) {
    int piv = c;
    for (int r = c + 1; r < 9; r++)
      if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
    for (int j = 0; j < 18; j++) {
      double t = M[c][j];
      M[c][j] = M[piv][j];
      M[piv][j] = t;
    }
    double dv = M[c][c];
    for (int j = 0; j < 18; j++) M[c][j] /= dv;
    for (int r = 0; r < 9; r++) {
      if (r == c) continue;
      double f = M[r][c];
      for (int j = 0; j < 18; j++) M[r][j] -= f * M[c][j];
    }
  }
  for (int m = 0; m < 9; m++)
    for (int k = 0; k < 14; k++) {
      double s = 0.0;
      for (int j = 0; j < 9; j++) s += M[m][9 + j] * A[k][j];
      pinv[14 * m + k] = (float)s;
    }
}

/* f32 -> f16 bits, round to nearest even (WGSL pack2x16float) */
uint32_t orc_f32_to_f16(float f) {
  uint32_t x = sl_float_to_bits(f);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ax = x & 0x7FFFFFFFu;
  if (ax >= 0x7F800000u) return sign | (ax > 0x7F800000u ? 0x7E00u : 0x7C00u);
  if (ax >= 0x477FF000u) return sign | 0x7C00u; /* rounds to >= 65520: infinity */
  if (ax < 0x38800000u) {                        /* below the smallest normal half: subnormal or zero */
    if (ax < 0x33000000u) return sign;           /* below half the smallest subnormal */
    /* the value is m 2^(e-150) and a half subnormal step is 2^-24: the step count is m 2^(e-126) */
    uint32_t e = ax >> 23, m = (ax & 0x7FFFFFu) | 0x800000u;
    uint32_t shift = 126u - e;
    uint32_t q = m >> shift, rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
    if (rem > halfway || (rem == halfway && (q & 1u))) q++;
    return sign | q;
  }
  uint32_t e = (ax >> 23) - 112u, m = ax & 0x7FFFFFu;
  uint32_t h = (e << 10) | (m >> 13), rem = m & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
  return sign | h;
}

static const float BN_PI = 3.14159265358979f;

static f3 bn_cell_dir(const float* cells, uint32_t c) { return F3(cells[4 * c], cells[4 * c + 1], cells[4 * c + 2]); }
static void bn_sh2(f3 d, float* b) {
  float x = d.x, y = d.y, z = d.z;
  b[0] = 0.282095f;
  b[1] = 0.488603f * y;
  b[2] = 0.488603f * z;
  b[3] = 0.488603f * x;
  b[4] = 1.092548f * x * y;
  b[5] = 1.092548f * y * z;
  b[6] = 0.315392f * (3.0f * z * z - 1.0f);
  b[7] = 1.092548f * x * z;
  b[8] = 0.546274f * (x * x - y * y);
}
static f3 bn_sky(const float* sh, f3 w) {
  float x = w.x, y = w.y, z = w.z;
  float b[16] = {0.282095f, 0.488603f * y, 0.488603f * z, 0.488603f * x, 1.092548f * x * y, 1.092548f * y * z,
                 0.315392f * (3.0f * z * z - 1.0f), 1.092548f * x * z, 0.546274f * (x * x - y * y),
                 0.590044f * y * (3.0f * x * x - y * y), 2.890611f * x * y * z, 0.457046f * y * (5.0f * z * z - 1.0f),
                 0.373176f * z * (5.0f * z * z - 3.0f), 0.457046f * x * (5.0f * z * z - 1.0f),
                 1.445306f * z * (x * x - y * y), 0.590044f * x * (x * x - 3.0f * y * y)};
  f3 c = F3(0.0f, 0.0f, 0.0f);
  for (int k = 0; k < 16; k++) c = add3(c, mul3(F3(sh[3 * k], sh[3 * k + 1], sh[3 * k + 2]), b[k]));
  return F3(fmaxf(c.x, 0.0f), fmaxf(c.y, 0.0f), fmaxf(c.z, 0.0f));
}
static float bn_seg_geom(const sl_node* nd, f3 P, f3 w, float t0, float t1) {
  f3 d = sub3(F3(nd->mean[0], nd->mean[1], nd->mean[2]), P);
  f3 cw = sym_mul(nd_cinv_d(nd), nd_cinv_o(nd), w);
  float a = dot3(cw, w);
  float m = dot3(cw, d) / a;
  f3 e = sub3(d, mul3(w, m));
  float q = fmaxf(dot3(e, sym_mul(nd_cinv_d(nd), nd_cinv_o(nd), e)), 0.0f);
  float s = sqrtf(0.5f * a);
  float x0 = s * (t0 - m), x1 = s * (t1 - m);
  float df;
  if (x0 > 0.0f) df = erfc_pos(x0) - erfc_pos(x1);
  else if (x1 < 0.0f) df = erfc_pos(-x1) - erfc_pos(-x0);
  else df = 2.0f - erfc_pos(x1) - erfc_pos(-x0);
  return sl_expf(-0.5f * q) * sqrtf(BN_PI / (2.0f * a)) * df;
}
static uint32_t bn_cell_of(f3 w) {
  float el = sl_asinf(clampf(w.z, -1.0f, 1.0f));
  float fi = fmaxf((0.5f * BN_PI - el) / (BN_PI / 8.0f), 0.0f);
  uint32_t i = (uint32_t)fi;
  i = i < 7u ? i : 7u;
  uint32_t j = ((uint32_t)sl_floorf((sl_atan2f(w.y, w.x) + BN_PI) / (2.0f * BN_PI) * 16.0f)) % 16u;
  return i * 16u + j;
}
static float bn_ground(const orc_probe_layout* L, uint32_t i, uint32_t j) {
  return L->ground ? L->ground[i * L->dims[1] + j] : 0.0f;
}
static f3 bn_lattice_pos(const orc_probe_layout* L, uint32_t p) {
  uint32_t i = p / (L->dims[1] * L->dims[2]), j = (p / L->dims[2]) % L->dims[1], k = p % L->dims[2];
  return F3(L->lo[0] + L->step[0] * (float)i, L->lo[1] + L->step[1] * (float)j, bn_ground(L, i, j) + L->levels[k]);
}

/* the probes after the lattice (bounce.wgsl:57-75, 217-268): 8 per part (part_probe_frame's 2x2x2 cube in the part's
 * rest frame), then the static volumes' grids (vol_frame) */
typedef struct {
  uint32_t nl, n_probes;                    /* lattice probes; all probes (lattice, 8 per part, volumes) */
  uint32_t vol_first[32], vol_dims[32][3];  /* per part: its volume's first probe after the lattice, grid (0: none) */
} bn_probes;

static bn_probes bn_probe_set(const orc_bounce_in* in) {
  bn_probes B;
  memset(&B, 0, sizeof(B));
  B.nl = in->lay.dims[0] * in->lay.dims[1] * in->lay.dims[2];
  uint32_t off = 8u * in->part_count;   /* the volumes follow every part's 8 (lighting.js:797-799) */
  for (uint32_t v = 0; v < in->lay.n_vols && v < 32u; v++) {
    uint32_t q = in->lay.vols[v][0];
    if (q >= 32u) continue;
    B.vol_first[q] = off;
    for (int c = 0; c < 3; c++) B.vol_dims[q][c] = in->lay.vols[v][1 + c];
    off += in->lay.vols[v][1] * in->lay.vols[v][2] * in->lay.vols[v][3];
  }
  B.n_probes = B.nl + off;
  return B;
}
/* is_part_probe_part (bounce.wgsl:264-266): a movable part's Gaussians read its own 8 probes */
static int bn_is_part_probe_part(const orc_bounce_in* in, uint32_t q) {
  return q < in->part_count && (in->parts[q].flags & 1u) == 0u && in->parts[q].root != NONE_U32;
}
static int bn_has_vol(const bn_probes* B, uint32_t q) { return q < 32u && B->vol_dims[q][0] > 0u; }
static float bn_sel(uint32_t o, float f) { return o ? f : 1.0f - f; }
static uint32_t bn_vol_of_probe(const orc_bounce_in* in, const bn_probes* B, uint32_t r) {
  for (uint32_t q = 0; q < in->part_count && q < 32u; q++) {
    uint32_t n = B->vol_dims[q][0] * B->vol_dims[q][1] * B->vol_dims[q][2];
    if (n > 0u && r >= B->vol_first[q] && r < B->vol_first[q] + n) return q;
  }
  return NONE_U32;
}
static void bn_part_frame(const orc_bounce_in* in, uint32_t q, f3* c, f3* h) {
  const sl_node* nd = &in->nodes[in->parts[q].root];
  f3 a = nd_cinv_d(nd), o = nd_cinv_o(nd);
  float det = a.x * (a.y * a.z - o.z * o.z) - o.x * (o.x * a.z - o.z * o.y) + o.y * (o.x * o.z - a.y * o.y);
  f3 var = div3(F3(a.y * a.z - o.z * o.z, a.x * a.z - o.y * o.y, a.x * a.y - o.x * o.x), fmaxf(det, 1e-30f));
  float hb = 0.5f * in->parts[q].bound[3];
  *c = F3(nd->mean[0], nd->mean[1], nd->mean[2]);
  *h = F3(fminf(0.95f * sqrtf(fmaxf(var.x, 0.0f)), hb), fminf(0.95f * sqrtf(fmaxf(var.y, 0.0f)), hb),
          fminf(0.95f * sqrtf(fmaxf(var.z, 0.0f)), hb));
}
static void bn_vol_frame(const orc_bounce_in* in, uint32_t q, f3* c, f3* h) {
  f3 h0;
  bn_part_frame(in, q, c, &h0);
  float R = in->parts[q].bound[3];
  *h = F3(fminf(1.6f * h0.x, R), fminf(1.6f * h0.y, R), fminf(1.6f * h0.z, R));
}
static f3 bn_probe_pos(const orc_bounce_in* in, const bn_probes* B, uint32_t p) {
  const uint32_t nl = B->nl;
  if (p >= nl + 8u * in->part_count) { /* a static volume's probe */
    uint32_t r = p - nl, q = bn_vol_of_probe(in, B, r);
    if (q == NONE_U32) return F3(0.0f, 0.0f, 0.0f);
    const uint32_t* d = B->vol_dims[q];
    uint32_t l = r - B->vol_first[q];
    f3 ijk = F3((float)(l / (d[1] * d[2])), (float)((l / d[2]) % d[1]), (float)(l % d[2]));
    f3 c, h;
    bn_vol_frame(in, q, &c, &h);
    f3 den = F3(fmaxf((float)d[0] - 1.0f, 1.0f), fmaxf((float)d[1] - 1.0f, 1.0f), fmaxf((float)d[2] - 1.0f, 1.0f));
    f3 t = mul3v(mul3(h, 2.0f), ijk);
    return xf_point(in->parts[q].xf, add3(sub3(c, h), F3(t.x / den.x, t.y / den.y, t.z / den.z)));
  }
  if (p >= nl) { /* a part's probe: the 2x2x2 cube, moving with the part */
    uint32_t q = (p - nl) / 8u, k = (p - nl) % 8u;
    f3 sgn = F3((float)(k >> 2u) * 2.0f - 1.0f, (float)((k >> 1u) & 1u) * 2.0f - 1.0f, (float)(k & 1u) * 2.0f - 1.0f);
    f3 c, h;
    bn_part_frame(in, q, &c, &h);
    return xf_point(in->parts[q].xf, add3(c, mul3v(sgn, h)));
  }
  return bn_lattice_pos(&in->lay, p);
}
static f3 bn_node_radiance(const uint32_t* node_sh, uint32_t ni, const float* b) {
  float h[28];
  for (uint32_t j = 0; j < 14u; j++) {
    uint32_t u = node_sh[ni * 14u + j];
    h[2 * j] = f16_to_f32(u & 0xFFFFu);
    h[2 * j + 1] = f16_to_f32(u >> 16);
  }
  f3 v = F3(0.0f, 0.0f, 0.0f);
  for (int m = 0; m < 9; m++) v = add3(v, mul3(F3(h[3 * m], h[3 * m + 1], h[3 * m + 2]), b[m]));
  return v;
}

static float bn_cheb(const orc_probe_layout* L, const float* pd, uint32_t p, f3 P) {
  f3 v = sub3(P, bn_lattice_pos(L, p));
  float dist = len3(v);
  const float* mm = pd + 8u * (p * BN_NCELL + bn_cell_of(div3(v, fmaxf(dist, 1e-9f)))) + 4u;
  float var = fmaxf(mm[1] - mm[0] * mm[0], 1e-4f);
  float dd = fmaxf(dist - 0.03f - mm[0], 0.0f);
  if (dd <= 0.0f) return 1.0f;
  float r = var / (var + dd * dd);
  return r * r * r;
}

typedef struct { uint32_t pid[8]; float w[8]; } bn_weights;

static bn_weights bn_probe_weights(const orc_probe_layout* L, const float* pd, f3 P) {
  const uint32_t* dm = L->dims;
  float fx = clampf((P.x - L->lo[0]) / L->step[0], 0.0f, (float)(dm[0] - 1u));
  float fy = clampf((P.y - L->lo[1]) / L->step[1], 0.0f, (float)(dm[1] - 1u));
  uint32_t i = (uint32_t)sl_floorf(fx), j = (uint32_t)sl_floorf(fy);
  i = i < dm[0] - 2u ? i : dm[0] - 2u;
  j = j < dm[1] - 2u ? j : dm[1] - 2u;
  float tx = fx - (float)i, ty = fy - (float)j;
  float g = mixf(mixf(bn_ground(L, i, j), bn_ground(L, i, j + 1u), ty),
                 mixf(bn_ground(L, i + 1u, j), bn_ground(L, i + 1u, j + 1u), ty), tx);
  float h = P.z - g;
  uint32_t k = 0;
  while (k + 2u < dm[2] && h > L->levels[k + 1u]) k++;
  float tz = clampf((h - L->levels[k]) / fmaxf(L->levels[k + 1u] - L->levels[k], 1e-6f), 0.0f, 1.0f);
  bn_weights out;
  float wsum = 0.0f;
  for (uint32_t c = 0; c < 8u; c++) {
    uint32_t ox = c >> 2u, oy = (c >> 1u) & 1u, oz = c & 1u;
    uint32_t p = ((i + ox) * dm[1] + (j + oy)) * dm[2] + (k + oz);
    out.pid[c] = p;
    float wx = ox ? tx : 1.0f - tx, wy = oy ? ty : 1.0f - ty, wz = oz ? tz : 1.0f - tz;
    float valid = pd[8u * (p * BN_NCELL) + 6u];
    float cw = wx * wy * wz * valid;
    out.w[c] = cw * fmaxf(bn_cheb(L, pd, p, P), 1e-3f);
    wsum += out.w[c];
  }
  if (wsum <= 0.0f) { /* probe_fallback: the 8 best valid probes of the 4x4x4 block */
    for (int c = 0; c < 8; c++) { out.pid[c] = 0u; out.w[c] = 0.0f; }
    for (uint32_t q = 0; q < 64u; q++) {
      int ii = (int)i + (int)(q >> 4u) - 1, jj = (int)j + (int)((q >> 2u) & 3u) - 1, kk = (int)k + (int)(q & 3u) - 1;
      if (ii < 0 || jj < 0 || kk < 0 || ii >= (int)dm[0] || jj >= (int)dm[1] || kk >= (int)dm[2]) continue;
      uint32_t p = ((uint32_t)ii * dm[1] + (uint32_t)jj) * dm[2] + (uint32_t)kk;
      if (pd[8u * (p * BN_NCELL) + 6u] <= 0.0f) continue;
      float d = fmaxf(len3(sub3(P, bn_lattice_pos(L, p))), 0.05f);
      float w = fmaxf(bn_cheb(L, pd, p, P), 1e-3f) / (d * d);
      if (w <= out.w[7]) continue;
      uint32_t at = 7u;
      while (at > 0u && out.w[at - 1u] < w) {
        out.w[at] = out.w[at - 1u];
        out.pid[at] = out.pid[at - 1u];
        at--;
      }
      out.w[at] = w;
      out.pid[at] = p;
    }
    float s = 0.0f;
    for (int c = 0; c < 8; c++) s += out.w[c];
    for (int c = 0; c < 8; c++) out.w[c] /= fmaxf(s, 1e-12f);
    return out;
  }
  for (int c = 0; c < 8; c++) out.w[c] /= fmaxf(wsum, 1e-12f);
  return out;
}

/* probe_weights (bounce.wgsl:813-885): a movable part's Gaussians trilinear over its own 8 probes, a static volume's
 * over its grid (neither with the Chebyshev test: those probes skip their own object), the rest over the lattice */
static bn_weights bn_weights_for(const orc_bounce_in* in, const bn_probes* B, const float* pd, f3 P, uint32_t own) {
  bn_weights out;
  if (bn_is_part_probe_part(in, own)) {
    f3 c, h;
    bn_part_frame(in, own, &c, &h);
    const float* xf = in->parts[own].xf;
    f3 lp = xf_dir_inv(xf, sub3(P, F3(xf[3], xf[7], xf[11])));
    f3 num = add3(sub3(lp, c), h);
    f3 f = F3(clampf(num.x / fmaxf(2.0f * h.x, 1e-6f), 0.0f, 1.0f), clampf(num.y / fmaxf(2.0f * h.y, 1e-6f), 0.0f, 1.0f),
              clampf(num.z / fmaxf(2.0f * h.z, 1e-6f), 0.0f, 1.0f));
    for (uint32_t k = 0; k < 8u; k++) {
      out.pid[k] = B->nl + own * 8u + k;
      out.w[k] = bn_sel(k >> 2u, f.x) * bn_sel((k >> 1u) & 1u, f.y) * bn_sel(k & 1u, f.z);
    }
    return out;
  }
  if (bn_has_vol(B, own)) {
    f3 c, h;
    bn_vol_frame(in, own, &c, &h);
    const float* xf = in->parts[own].xf;
    f3 lp = xf_dir_inv(xf, sub3(P, F3(xf[3], xf[7], xf[11])));
    const uint32_t* d = B->vol_dims[own];
    f3 num = add3(sub3(lp, c), h);
    f3 fq = F3(clampf(num.x / fmaxf(2.0f * h.x, 1e-6f), 0.0f, 1.0f) * ((float)d[0] - 1.0f),
               clampf(num.y / fmaxf(2.0f * h.y, 1e-6f), 0.0f, 1.0f) * ((float)d[1] - 1.0f),
               clampf(num.z / fmaxf(2.0f * h.z, 1e-6f), 0.0f, 1.0f) * ((float)d[2] - 1.0f));
    uint32_t fi[3] = {(uint32_t)sl_floorf(fq.x), (uint32_t)sl_floorf(fq.y), (uint32_t)sl_floorf(fq.z)};
    for (int a = 0; a < 3; a++) fi[a] = fi[a] < d[a] - 2u ? fi[a] : d[a] - 2u;
    f3 fr = F3(fq.x - (float)fi[0], fq.y - (float)fi[1], fq.z - (float)fi[2]);
    for (uint32_t k = 0; k < 8u; k++) {
      uint32_t ox = k >> 2u, oy = (k >> 1u) & 1u, oz = k & 1u;
      out.pid[k] = B->nl + B->vol_first[own] + ((fi[0] + ox) * d[1] + (fi[1] + oy)) * d[2] + (fi[2] + oz);
      out.w[k] = bn_sel(ox, fr.x) * bn_sel(oy, fr.y) * bn_sel(oz, fr.z);
    }
    return out;
  }
  return bn_probe_weights(&in->lay, pd, P);
}

/* emissive.wgsl DIRS14 (:107-112): the same directions with the diagonals' components written 0.57735 */
static const float bn_dirs14[14][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {1e-4f, 0.0f, 1.0f},
                                       {-1.0f, 0.0f, 0.0f}, {0.0f, -1.0f, 0.0f}, {1e-4f, 0.0f, -1.0f},
                                       {0.57735f, 0.57735f, 0.57735f}, {0.57735f, 0.57735f, -0.57735f},
                                       {0.57735f, -0.57735f, 0.57735f}, {0.57735f, -0.57735f, -0.57735f},
                                       {-0.57735f, 0.57735f, 0.57735f}, {-0.57735f, 0.57735f, -0.57735f},
                                       {-0.57735f, -0.57735f, 0.57735f}, {-0.57735f, -0.57735f, -0.57735f}};

/* direct_dirs_one (emissive.wgsl:1066-1082): shade_emitters toward DIRS14 (asg off; M39 transfer), each direction's
 * colour weighted by footprint x V toward it, then env_dirs_one's distant catch */
static void bn_direct_one(const orc_bounce_in* in, uint32_t g, float* lo_dir) {
  const sl_gaussian* G = &in->gs[g];
  const sl_node* nd = &in->nodes[g];
  const sl_material* mat = &in->mats[mat_index(G, in->mat_count)];
  const float* xf = in->parts[G->part_surface & 0xFFFFu].xf;
  m3f Rq = quat_matrix(G->quat);
  m3f Dm = m3_diag(F3(mat->flake[0], mat->flake[1], mat->flake[2]));
  m3f t0 = m3_mul(&Rq, &Dm);
  m3f RqT = m3_t(&Rq);
  m3f Sloc = m3_mul(&t0, &RqT);
  float s3 = G->scale[0] * G->scale[1] * G->scale[2];
  float detC = s3 * s3;
  f3 P = xf_point(xf, F3(G->mu[0], G->mu[1], G->mu[2]));
  f3 n = Rq.c[0];
  f3 Sd = F3(Sloc.c[0].x, Sloc.c[1].y, Sloc.c[2].z), So = F3(Sloc.c[1].x, Sloc.c[2].x, Sloc.c[2].y);
  f3 alb = F3(G->albedo[0], G->albedo[1], G->albedo[2]);
  float ks = spec_weight(mat);
  int emissive = (mat->flags & 1u) != 0u;
  f3 wo[14];
  f3 acc[14];
  for (int k = 0; k < 14; k++) {
    wo[k] = xf_dir_inv(xf, F3(bn_dirs14[k][0], bn_dirs14[k][1], bn_dirs14[k][2]));
    acc[k] = F3(0.0f, 0.0f, 0.0f);
  }
  if (in->n_emit) {
    uint32_t stack[48];
    uint32_t sp = 1;
    stack[0] = in->tree_root;
    while (sp > 0u) {
      sp--;
      const float* e = in->tree + 24u * stack[sp];
      uint32_t child_lo = sl_float_to_bits(e[11]), child_hi = sl_float_to_bits(e[15]);
      f3 emean = F3(e[0], e[1], e[2]);
      int use;
      if (child_lo == NONE_U32 || in->emit_mode == 0u) {
        use = child_lo == NONE_U32;
      } else {
        f3 d = sub3(P, emean);
        use = dot3(d, d) > in->emit_theta * in->emit_theta * e[3] * e[3];
      }
      if (!use) {
        if (sp + 2u <= 48u) { stack[sp] = child_lo; stack[sp + 1u] = child_hi; sp += 2u; }
        continue;
      }
      f3 d = sub3(emean, P);
      float d2 = dot3(d, d);
      if (d2 < 1e-8f) continue;
      f3 ww = div3(d, sqrtf(d2));
      f3 wi = xf_dir_inv(xf, ww);
      float vi = vgrid_lookup(&in->vgrid[g], wi);
      if (vi <= 1e-7f) continue;
      float fp = footprint(nd, detC, wi);
      f3 mw = mul3(ww, -1.0f);
      float s = 1.0f;
      if (in->one_sided) {
        f3 nn = F3(in->normal[0], in->normal[1], in->normal[2]);
        float cs = dot3(mw, nn);
        s = in->edge_soft > 0.0f ? smoothstepf(-in->edge_soft, in->edge_soft, cs) : (cs > 0.0f ? 1.0f : 0.0f);
      }
      float mq = sqrtf(fmaxf(dot3(mw, sym_mul(F3(e[4], e[5], e[6]), F3(e[8], e[9], e[10]), mw)), 0.0f));
      f3 I = mul3(F3(e[12], e[13], e[14]), s * in->emit_scale * mq);
      f3 light = mul3(mul3(I, vi), fp / d2 * 1.0f);
      if (ks <= 0.0f) {
        acc[0] = add3(acc[0], light);
        continue;
      }
      f3 wr = mirror3(wi, n);
      float damp = iso_damp(iso_norm(nd), footprint(nd, detC, wr) * vgrid_lookup(&in->vgrid[g], wr));
      for (int k = 0; k < 14; k++)
        acc[k] = add3(acc[k], mul3(light, iso_lobe_from(ks, phase_specular(Sd, So, wi, wo[k]), damp)));
    }
  }
  float T = in->lamp_T[g];
  float inorm = iso_norm(nd);
  f3 a0 = acc[0];
  f3 mean = F3(0.0f, 0.0f, 0.0f);
  float ws = 0.0f;
  f3 c0 = F3(0.0f, 0.0f, 0.0f);
  for (int k = 0; k < 14; k++) {
    f3 ck = mul3(mul3v(alb, ks <= 0.0f ? a0 : acc[k]), T * inorm);
    if (k == 0) c0 = ck;
    float w = footprint(nd, detC, wo[k]) * vgrid_lookup(&in->vgrid[g], wo[k]);
    mean = add3(mean, mul3(ck, w));
    ws += w;
  }
  f3 c = ws > 0.0f ? div3(mean, fmaxf(ws, 1e-20f)) : c0;
  /* env_dirs (environment.wgsl:353-359): the distant lights' catch, non-emissive Gaussians */
  if (in->n_lights && !emissive) {
    f3 dc = F3(0.0f, 0.0f, 0.0f);
    for (uint32_t k = 0; k < in->n_lights && k < 4u; k++) {
      f3 wi = xf_dir_inv(xf, F3(in->lights[k].dir[0], in->lights[k].dir[1], in->lights[k].dir[2]));
      float v = vgrid_lookup(&in->vgrid[g], wi);
      if (v <= 1e-7f) continue;
      dc = add3(dc, mul3(F3(in->lights[k].irr[0], in->lights[k].irr[1], in->lights[k].irr[2]),
                         in->env_T[4u * g + k] * v * footprint(nd, detC, wi)));
    }
    c = add3(c, mul3(mul3v(alb, dc), inorm));
  }
  lo_dir[4u * g] = c.x;
  lo_dir[4u * g + 1] = c.y;
  lo_dir[4u * g + 2] = c.z;
  lo_dir[4u * g + 3] = 0.0f;
}

/* the cells as lights (cell_asg_phase, bounce.wgsl:180-191): per cell the elevation and azimuth tangents and the
 * angular variances of a Gaussian CELL_STD of the cell across, float64 then rounded: 8 floats per cell */
static void bn_cell_asg_table(float* t) {
  const double CELL_STD = 0.4;
  for (int c = 0; c < 128; c++) {
    int i = c / 16, j = c % 16;
    double el = 0.5 * M_PI - (i + 0.5) * M_PI / 8.0, az = -M_PI + (j + 0.5) * 2.0 * M_PI / 16.0;
    double s_el = CELL_STD * M_PI / 8.0, s_az = CELL_STD * 2.0 * M_PI / 16.0 * fmax(cos(el), 0.05);
    float* o = t + 8 * c;
    o[0] = (float)(-sin(el) * cos(az));
    o[1] = (float)(-sin(el) * sin(az));
    o[2] = (float)cos(el);
    o[3] = (float)(-sin(az));
    o[4] = (float)cos(az);
    o[5] = 0.0f;
    o[6] = (float)(s_el * s_el);
    o[7] = (float)(s_az * s_az);
  }
}

/* bounce_dirs for a near-mirror Gaussian (bounce.wgsl:887-985, the M39 path): the 8 probes' per-cell radiance through
 * its transfer (V, footprint, solid angle) and the specular lobe toward D14 and the eye (the cells within about three
 * lobe widths of the eye's mirror direction as lights with a size when asg_cells) into lo_b */
static void bn_dirs_one(const orc_bounce_in* in, const bn_probes* PS, const float* cells, const float* casg,
                        const float* d14, orc_bounce_state* st, uint32_t g) {
  const sl_gaussian* G = &in->gs[g];
  const sl_node* nd = &in->nodes[g];
  const sl_material* mat = &in->mats[mat_index(G, in->mat_count)];
  uint32_t own = G->part_surface & 0xFFFFu;
  const float* xf = in->parts[own].xf;
  f3 P = xf_point(xf, F3(G->mu[0], G->mu[1], G->mu[2]));
  m3f Rq = quat_matrix(G->quat);
  m3f Dm = m3_diag(F3(mat->flake[0], mat->flake[1], mat->flake[2]));
  m3f t0 = m3_mul(&Rq, &Dm);
  m3f RqT = m3_t(&Rq);
  m3f Sloc = m3_mul(&t0, &RqT);
  f3 n = Rq.c[0], t1 = Rq.c[1], t2 = Rq.c[2];
  f3 Sd = F3(Sloc.c[0].x, Sloc.c[1].y, Sloc.c[2].z), So = F3(Sloc.c[1].x, Sloc.c[2].x, Sloc.c[2].y);
  f3 flake = F3(mat->flake[0], mat->flake[1], mat->flake[2]);
  float s3 = G->scale[0] * G->scale[1] * G->scale[2];
  float detC = s3 * s3;
  float ks = spec_weight(mat);
  float inorm = iso_norm(nd);
  bn_weights pw = bn_weights_for(in, PS, st->probe_data, P, own);
  float lobe_w = sqrtf(fminf(mat->flake[1], mat->flake[2]) / fmaxf(mat->flake[0], 1e-12f));
  float near_ang = fminf(3.0f * (0.4f * BN_PI / 8.0f + 2.0f * lobe_w), BN_PI);
  f3 wo[15];
  for (int k = 0; k < 14; k++) wo[k] = xf_dir_inv(xf, F3(d14[3 * k], d14[3 * k + 1], d14[3 * k + 2]));
  wo[14] = xf_dir_inv(xf, norm3(sub3(F3(in->eye[0], in->eye[1], in->eye[2]), P)));
  f3 acc[15];
  for (int k = 0; k < 15; k++) acc[k] = F3(0.0f, 0.0f, 0.0f);
  f3 wr_eye = mirror3(wo[14], n);
  for (uint32_t c = 0; c < BN_NCELL; c++) {
    f3 L = F3(0.0f, 0.0f, 0.0f);
    for (int k = 0; k < 8; k++) {
      if (pw.w[k] > 0.0f) {
        const float* r0 = st->probe_data + 8u * (pw.pid[k] * BN_NCELL + c);
        L = add3(L, mul3(F3(r0[0], r0[1], r0[2]), pw.w[k]));
      }
    }
    if (L.x + L.y + L.z <= 0.0f) continue;
    f3 u = xf_dir_inv(xf, bn_cell_dir(cells, c));
    float vis = vgrid_lookup(&in->vgrid[g], u) * 1.0f;
    if (vis <= 0.0f) continue;
    f3 lin = mul3(L, vis * footprint(nd, detC, u) * cells[4 * c + 3]);
    f3 ur = mirror3(u, n);
    float damp = iso_damp(inorm, footprint(nd, detC, ur) * vgrid_lookup(&in->vgrid[g], ur));
    for (int k = 0; k < 14; k++) acc[k] = add3(acc[k], mul3(lin, iso_lobe_from(ks, phase_specular(Sd, So, u, wo[k]), damp)));
    float lobe14;
    if (in->asg_cells && sl_acosf(clampf(dot3(u, wr_eye), -1.0f, 1.0f)) < near_ang) {
      const float* e = casg + 8 * c;
      f3 lb0 = xf_dir_inv(xf, F3(e[0], e[1], e[2])), lb1 = xf_dir_inv(xf, F3(e[3], e[4], e[5]));
      s2m sl = {e[6], 0.0f, e[7]};
      lobe14 = iso_lobe_from(ks, asg_phase(u, lb0, lb1, sl, n, t1, t2, flake, Sd, So, wo[14]), damp);
    } else {
      lobe14 = iso_lobe_from(ks, phase_specular(Sd, So, u, wo[14]), damp);
    }
    acc[14] = add3(acc[14], mul3(lin, lobe14));
  }
  f3 send = F3(0.0f, 0.0f, 0.0f);
  float ws = 0.0f;
  for (int k = 0; k < 14; k++) {
    float w = footprint(nd, detC, wo[k]) * vgrid_lookup(&in->vgrid[g], wo[k]);
    send = add3(send, mul3(acc[k], w));
    ws += w;
  }
  send = div3(send, fmaxf(ws, 1e-20f));
  f3 sc = mul3(F3(G->albedo[0], G->albedo[1], G->albedo[2]), inorm);
  f3 eyec = mul3v(sc, acc[14]), sendc = mul3v(sc, send);
  float* lb = st->lo_b + 12u * g;
  lb[0] = eyec.x; lb[1] = eyec.y; lb[2] = eyec.z; lb[3] = 0.0f;
  lb[4] = sendc.x; lb[5] = sendc.y; lb[6] = sendc.z; lb[7] = 0.0f;
  lb[8] = lb[9] = lb[10] = lb[11] = 0.0f;
}

/* ---- the sender cut (bounce.wgsl:1448-1730 sc_select .. node_sh2_sc; emissive.wgsl:1018-1065
 * direct_dirs_emit_sc / direct_dirs_nodes_sc; environment.wgsl:317-352 env_dirs_sc / env_dirs_nodes_sc; host
 * src/lighting.js:1057-1095), the reference's default level of detail for the probes' senders.
 * On a re-selection (the first frame, or one in which a part moved) every node of every part's tree is marked, top
 * down by depth: BELOW (above the parts, under a cut node or a cut leaf: never read), OPEN (some probe's gather opens
 * it), NODE (every probe uses it whole) or LEAF (a leaf whose parent is OPEN, or a part's root).  A cut node is lit as
 * one two-sided Gaussian (its nodeGaussians record and V grid), its shadow T the mean over 8 leaves reached by
 * mass-weighted random descents; its 14-direction sums come from that light plus the probes' SH2 at its centre through
 * its own two-face transfer; node_up sums the OPEN nodes only, and the gather reads zero under the cut.
 * Two choices here where the reference's result depends on the order its atomics hand out slots: the cut is not
 * capped (the reference stops at 2^18 cut nodes a frame, past which nodes open), and a cut node refreshes its shadow
 * and direct light in the frames with node % 4 == frame % 4 (the reference: its slot % 4). */
enum { SC_BELOW = 0u, SC_OPEN = 1u, SC_NODE = 2u, SC_LEAF = 3u };
#define SC_SAMPLES 8u

/* pcg_hash and to_unit (common.wgsl:98-104) */
static uint32_t sc_pcg(uint32_t x) {
  uint32_t s = x * 747796405u + 2891336453u;
  uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (w >> 22u) ^ w;
}
static float sc_to_unit(uint32_t x) { return (float)(x >> 8u) * (1.0f / 16777216.0f); }
/* sc_face (common.wgsl:342-345), SC_FACE_K 1 */
static float sc_face(float c) { return clampf(c * 1.0f, -1.0f, 1.0f); }
/* sc_mass (bounce.wgsl): kappa / sqrt(det cinv) */
static float sc_mass(const sl_node* nd) {
  return nd->kappa / sqrtf(fmaxf(sym_det(nd_cinv_d(nd), nd_cinv_o(nd)), 1e-30f));
}
static float sc_round(float x) { return rintf(x); } /* WGSL round: half to even */

/* sc_probe_dist (bounce.wgsl:1478-1516): the smallest (distance - margin) from world point P to the gather centres of
 * the probes that see part `own`: the room lattice's nearest 2x2x2 block centre less the block radius, the terrain's
 * 3 x 3 columns around P, each movable part's 8 probes but own's, each static volume's nearest grid probe */
static float sc_probe_dist(const orc_bounce_in* in, const bn_probes* PS, f3 P, uint32_t own, float brad) {
  const orc_probe_layout* L = &in->lay;
  float best = 1e30f;
  const float m = 0.0f; /* the gathers of probes that cut around themselves keep no margin (vol_info.y = 0) */
  if (!L->terrain) {
    const float Pv[3] = {P.x, P.y, P.z};
    float b[3];
    for (int a = 0; a < 3; a++) {
      float nb = (float)((L->dims[a] + 1u) / 2u);
      b[a] = clampf(sc_round(((Pv[a] - L->lo[a]) / fmaxf(L->step[a], 1e-6f) - 0.5f) * 0.5f), 0.0f, nb - 1.0f);
    }
    f3 cen = F3(L->lo[0] + L->step[0] * (2.0f * b[0] + 0.5f), L->lo[1] + L->step[1] * (2.0f * b[1] + 0.5f),
                L->lo[2] + L->step[2] * (2.0f * b[2] + 0.5f));
    best = len3(sub3(P, cen)) - brad;
  } else {
    float fx = clampf(sc_round((P.x - L->lo[0]) / fmaxf(L->step[0], 1e-6f)), -1e9f, 1e9f);
    float fy = clampf(sc_round((P.y - L->lo[1]) / fmaxf(L->step[1], 1e-6f)), -1e9f, 1e9f);
    int ci = (int)fx, cj = (int)fy;
    for (int di = -1; di <= 1; di++) {
      for (int dj = -1; dj <= 1; dj++) {
        int ii = ci + di, jj = cj + dj;
        uint32_t i = (uint32_t)(ii < 0 ? 0 : (ii > (int)L->dims[0] - 1 ? (int)L->dims[0] - 1 : ii));
        uint32_t j = (uint32_t)(jj < 0 ? 0 : (jj > (int)L->dims[1] - 1 ? (int)L->dims[1] - 1 : jj));
        float x = L->lo[0] + L->step[0] * (float)i, y = L->lo[1] + L->step[1] * (float)j;
        float gz = bn_ground(L, i, j);
        for (uint32_t k = 0; k < L->dims[2]; k++) best = fminf(best, len3(sub3(P, F3(x, y, gz + L->levels[k]))) - m);
      }
    }
  }
  for (uint32_t q = 0; q < in->part_count && q < 32u; q++) {
    if (q == own) continue;
    const float* xf = in->parts[q].xf;
    if (bn_is_part_probe_part(in, q)) {
      f3 c, h;
      bn_part_frame(in, q, &c, &h);
      if (len3(sub3(P, xf_point(xf, c))) - len3(h) - m >= best) continue;
      for (uint32_t k = 0; k < 8u; k++) best = fminf(best, len3(sub3(P, bn_probe_pos(in, PS, PS->nl + q * 8u + k))) - m);
    } else if (bn_has_vol(PS, q)) {
      f3 c, h;
      bn_vol_frame(in, q, &c, &h);
      const float d[3] = {(float)PS->vol_dims[q][0], (float)PS->vol_dims[q][1], (float)PS->vol_dims[q][2]};
      f3 lp = xf_dir_inv(xf, sub3(P, F3(xf[3], xf[7], xf[11])));
      const float lv[3] = {lp.x, lp.y, lp.z}, cv[3] = {c.x, c.y, c.z}, hv[3] = {h.x, h.y, h.z};
      float g[3];
      for (int a = 0; a < 3; a++) {
        float span = fmaxf(d[a] - 1.0f, 1.0f);
        float ijk = clampf(sc_round((lv[a] - cv[a] + hv[a]) / fmaxf(2.0f * hv[a], 1e-6f) * span), 0.0f, d[a] - 1.0f);
        g[a] = cv[a] - hv[a] + 2.0f * hv[a] * ijk / span;
      }
      best = fminf(best, len3(sub3(lp, F3(g[0], g[1], g[2]))) - m);
    }
  }
  return best;
}

/* sc_select (bounce.wgsl:1529-1548) for node n, its parent's mark already set */
static uint32_t sc_select_one(const orc_bounce_in* in, const bn_probes* PS, const uint32_t* parent,
                              const uint32_t* flag, uint32_t n, float brad) {
  const sl_node* nd = &in->nodes[n];
  uint32_t q = nd->part;
  if (q >= in->part_count) return SC_BELOW; /* scene nodes above the parts: the gather starts at part roots */
  if (in->parts[q].root != n && (parent[n] == NONE_U32 || flag[parent[n]] != SC_OPEN)) return SC_BELOW;
  if (n < in->count) return SC_LEAF;
  f3 P = xf_point(in->parts[q].xf, F3(nd->mean[0], nd->mean[1], nd->mean[2]));
  return sc_probe_dist(in, PS, P, q, brad) <= BN_THETA * nd->smax ? SC_OPEN : SC_NODE;
}

/* sc_xfer (bounce.wgsl:1631-1667): per cut node and face of its short axis the share of the SH2 transfer from its own
 * V grid and the face's exposure; 6 vec4: face 0 t0-3, t4-7, (t8, S, 0, 0), then face 1 */
static void sc_xfer_one(const orc_bounce_in* in, const float* cells, uint32_t n, float* X) {
  const uint32_t r = n - in->count;
  const sl_gaussian* G = &in->node_gs[r];
  const sl_node* nd = &in->nodes[n];
  const float* xf = in->parts[G->part_surface & 0xFFFFu].xf;
  m3f Rq = quat_matrix(G->quat);
  f3 nrm = Rq.c[0];
  float s3 = G->scale[0] * G->scale[1] * G->scale[2];
  float t[20];
  for (int i = 0; i < 20; i++) t[i] = 0.0f;
  float S0 = 0.0f;
  for (uint32_t cc = 0; cc < BN_NCELL; cc++) {
    f3 w = bn_cell_dir(cells, cc);
    f3 u = xf_dir_inv(xf, w);
    float a = footprint(nd, s3 * s3, u) * cells[4 * cc + 3];
    S0 += a;
    float v = vgrid_lookup(&in->node_vg[r], u);
    if (v <= 0.0f) continue;
    float h = 0.5f + 0.5f * sc_face(dot3(u, nrm));
    float y[9];
    bn_sh2(w, y);
    for (int i = 0; i < 9; i++) {
      t[i] += a * v * h * y[i];
      t[10 + i] += a * v * (1.0f - h) * y[i];
    }
    t[9] += a * v * h;
    t[19] += a * v * (1.0f - h);
  }
  float Smin = fmaxf(0.5f * 0.02f * S0, 1e-30f); /* iso_init.wgsl ISO_EPS, per face */
  for (int f = 0; f < 2; f++) {
    const float* o = t + 10 * f;
    float* x = X + 12 * f;
    x[0] = o[0]; x[1] = o[1]; x[2] = o[2]; x[3] = o[3];
    x[4] = o[4]; x[5] = o[5]; x[6] = o[6]; x[7] = o[7];
    x[8] = o[8]; x[9] = fmaxf(o[9], Smin); x[10] = 0.0f; x[11] = 0.0f;
  }
}

/* sc_shadow (bounce.wgsl:1566-1624): the mean lamp T and distant-light T over SC_SAMPLES leaves under n, each reached
 * by a descent that picks a child with probability by mass (a fixed hash per node and sample).  The Gaussians carry
 * one lamp T each here, so the reference's per-lamp slots reduce to that mean. */
static void sc_shadow_one(const orc_bounce_in* in, uint32_t n, float* T_out, float* E_out) {
  const uint32_t G = in->count;
  float T = 0.0f, E[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  for (uint32_t s = 0; s < SC_SAMPLES; s++) {
    uint32_t m = n, h = sc_pcg(n * SC_SAMPLES + s);
    for (uint32_t it = 0; it < 64u && m >= G; it++) {
      const sl_node* nd = &in->nodes[m];
      if (nd->child_hi <= nd->child_lo) break; /* no children to descend into: the sample counts T = 1 */
      float tot = 0.0f;
      for (uint32_t j = nd->child_lo; j < nd->child_hi; j++) tot += sc_mass(&in->nodes[in->kids[j]]);
      float u = sc_to_unit(h) * tot;
      h = sc_pcg(h);
      uint32_t pick = in->kids[nd->child_lo];
      for (uint32_t j = nd->child_lo; j < nd->child_hi; j++) {
        pick = in->kids[j];
        u -= sc_mass(&in->nodes[in->kids[j]]);
        if (u <= 0.0f) break;
      }
      m = pick;
    }
    /* trees are at most 64 levels deep (checked where the cut is set up), so m is a leaf */
    T += m < G ? in->lamp_T[m] : 1.0f;
    for (int c = 0; c < 4; c++) E[c] += m < G ? in->env_T[4u * m + c] : 1.0f;
  }
  *T_out = T / (float)SC_SAMPLES;
  for (int c = 0; c < 4; c++) E_out[c] = E[c] / (float)SC_SAMPLES;
}

/* direct_dirs_nodes_sc + env_dirs_nodes_sc: the light each face of cut node n catches, before albedo and exposure
 * (matte: shininess left out of the senders), into X's entries 6 and 7 */
static void sc_direct_node(const orc_bounce_in* in, uint32_t n, float T, const float* E, float* X) {
  const uint32_t r = n - in->count;
  const sl_gaussian* G = &in->node_gs[r];
  const sl_node* nd = &in->nodes[n];
  const float* xf = in->parts[G->part_surface & 0xFFFFu].xf;
  m3f Rq = quat_matrix(G->quat);
  f3 nrm = Rq.c[0];
  float s3 = G->scale[0] * G->scale[1] * G->scale[2];
  float detC = s3 * s3;
  f3 P = xf_point(xf, F3(G->mu[0], G->mu[1], G->mu[2]));
  f3 c0 = F3(0.0f, 0.0f, 0.0f), c1 = F3(0.0f, 0.0f, 0.0f);
  if (in->n_emit) {
    uint32_t stack[48];
    uint32_t sp = 1;
    stack[0] = in->tree_root;
    while (sp > 0u) {
      sp--;
      const float* e = in->tree + 24u * stack[sp];
      uint32_t child_lo = sl_float_to_bits(e[11]), child_hi = sl_float_to_bits(e[15]);
      f3 emean = F3(e[0], e[1], e[2]);
      int use;
      if (child_lo == NONE_U32 || in->emit_mode == 0u) {
        use = child_lo == NONE_U32;
      } else {
        f3 d = sub3(P, emean);
        use = dot3(d, d) > in->emit_theta * in->emit_theta * e[3] * e[3];
      }
      if (!use) {
        if (sp + 2u <= 48u) { stack[sp] = child_lo; stack[sp + 1u] = child_hi; sp += 2u; }
        continue;
      }
      f3 d = sub3(emean, P);
      float d2 = dot3(d, d);
      if (d2 < 1e-8f) continue;
      f3 ww = div3(d, sqrtf(d2));
      f3 wi = xf_dir_inv(xf, ww);
      float vi = vgrid_lookup(&in->node_vg[r], wi);
      if (vi <= 1e-7f) continue;
      f3 mw = mul3(ww, -1.0f);
      float s = 1.0f;
      if (in->one_sided) {
        f3 nn = F3(in->normal[0], in->normal[1], in->normal[2]);
        float cs = dot3(mw, nn);
        s = in->edge_soft > 0.0f ? smoothstepf(-in->edge_soft, in->edge_soft, cs) : (cs > 0.0f ? 1.0f : 0.0f);
      }
      float mq = sqrtf(fmaxf(dot3(mw, sym_mul(F3(e[4], e[5], e[6]), F3(e[8], e[9], e[10]), mw)), 0.0f));
      f3 I = mul3(F3(e[12], e[13], e[14]), s * in->emit_scale * mq);
      f3 light = mul3(I, vi * footprint(nd, detC, wi) / d2 * 1.0f);
      float h = 0.5f + 0.5f * sc_face(dot3(wi, nrm));
      c0 = add3(c0, mul3(light, h));
      c1 = add3(c1, mul3(light, 1.0f - h));
    }
  }
  c0 = mul3(c0, T);
  c1 = mul3(c1, T);
  const sl_material* mat = &in->mats[mat_index(G, in->mat_count)];
  if (in->n_lights && (mat->flags & 1u) == 0u) {
    for (uint32_t k = 0; k < in->n_lights && k < 4u; k++) {
      f3 wi = xf_dir_inv(xf, F3(in->lights[k].dir[0], in->lights[k].dir[1], in->lights[k].dir[2]));
      float v = vgrid_lookup(&in->node_vg[r], wi);
      if (v <= 1e-7f) continue;
      f3 c = mul3(F3(in->lights[k].irr[0], in->lights[k].irr[1], in->lights[k].irr[2]),
                  E[k] * v * footprint(nd, detC, wi));
      float h = 0.5f + 0.5f * sc_face(dot3(wi, nrm));
      c0 = add3(c0, mul3(c, h));
      c1 = add3(c1, mul3(c, 1.0f - h));
    }
  }
  X[24] = c0.x; X[25] = c0.y; X[26] = c0.z; X[27] = 0.0f;
  X[28] = c1.x; X[29] = c1.y; X[30] = c1.z; X[31] = 0.0f;
}

/* node_cut (bounce.wgsl:1669-1712): cut node n as one sender, each face's light (its direct light plus the probes'
 * SH2 at its centre through the face's transfer, over the face's exposure) shown toward each D_k by its share there */
static void sc_node_cut(const orc_bounce_in* in, const bn_probes* PS, const float* d14, const float* pd,
                        const float* probe_sh, uint32_t n, const float* X, float* acc) {
  const uint32_t r = n - in->count;
  const sl_gaussian* G = &in->node_gs[r];
  const sl_node* nd = &in->nodes[n];
  uint32_t own = G->part_surface & 0xFFFFu;
  const float* xf = in->parts[own].xf;
  f3 P = xf_point(xf, F3(G->mu[0], G->mu[1], G->mu[2]));
  m3f Rq = quat_matrix(G->quat);
  f3 nrm = Rq.c[0];
  float s3 = G->scale[0] * G->scale[1] * G->scale[2];
  bn_weights pw = bn_weights_for(in, PS, pd, P, own);
  f3 Lsh[9];
  for (int i = 0; i < 9; i++) Lsh[i] = F3(0.0f, 0.0f, 0.0f);
  for (int k = 0; k < 8; k++) {
    float w = pw.w[k];
    if (w <= 0.0f) continue;
    for (int i = 0; i < 9; i++) {
      const float* s = probe_sh + 4u * (9u * pw.pid[k] + (uint32_t)i);
      Lsh[i] = add3(Lsh[i], mul3(F3(s[0], s[1], s[2]), w));
    }
  }
  f3 col[2];
  f3 alb = F3(G->albedo[0], G->albedo[1], G->albedo[2]);
  for (int f = 0; f < 2; f++) {
    const float* x = X + 12 * f;
    f3 B = mul3(Lsh[0], x[0]);
    for (int i = 1; i < 9; i++) B = add3(B, mul3(Lsh[i], x[i]));
    B = F3(fmaxf(B.x, 0.0f), fmaxf(B.y, 0.0f), fmaxf(B.z, 0.0f));
    f3 Ld = add3(F3(X[24 + 4 * f], X[25 + 4 * f], X[26 + 4 * f]), B);
    Ld = F3(fmaxf(Ld.x, 0.0f), fmaxf(Ld.y, 0.0f), fmaxf(Ld.z, 0.0f));
    col[f] = div3(mul3v(alb, Ld), x[9]);
  }
  int dark = own == in->dark_part;
  for (int k = 0; k < 14; k++) {
    f3 wo = xf_dir_inv(xf, F3(d14[3 * k], d14[3 * k + 1], d14[3 * k + 2]));
    float w = footprint(nd, s3 * s3, wo) * vgrid_lookup(&in->node_vg[r], wo);
    float h = 0.5f + 0.5f * sc_face(dot3(wo, nrm));
    f3 L = dark ? F3(0.0f, 0.0f, 0.0f) : add3(mul3(col[0], h), mul3(col[1], 1.0f - h));
    float* o = acc + 4u * (14u * n + (uint32_t)k);
    o[0] = L.x * w;
    o[1] = L.y * w;
    o[2] = L.z * w;
    o[3] = w;
  }
}

int orc_bounce_frame(const orc_bounce_in* in, orc_bounce_state* st, int nthreads) {
  const orc_probe_layout* L = &in->lay;
  const uint32_t G = in->count, N = in->n_nodes;
  const bn_probes PS = bn_probe_set(in);
  const uint32_t NP = PS.n_probes, NL = PS.nl;
  float cells[4 * 128], d14[42], pinv[126], casg[8 * 128];
  orc_iso_dirs(cells);
  orc_bounce_tables(d14, pinv);
  bn_cell_asg_table(casg);
  (void)nthreads;

  /* iso_xfer: where something moved relative to the Gaussian, or forced */
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 256)
#endif
  for (int64_t gi = 0; gi < (int64_t)G; gi++) {
    uint32_t g = (uint32_t)gi;
    const sl_gaussian* Gs = &in->gs[g];
    uint32_t own = Gs->part_surface & 0xFFFFu;
    const float* xf = in->parts[own].xf;
    f3 P = xf_point(xf, F3(Gs->mu[0], Gs->mu[1], Gs->mu[2]));
    int stale = in->force || (own < 32u && ((in->moved_mask >> own) & 1u));
    for (uint32_t p = 0; p < in->part_count && p < 32u && !stale; p++) {
      if (p == own || ((in->moved_mask >> p) & 1u) == 0u) continue;
      const float* b = in->parts[p].bound;
      float r = b[3] + BN_NEAR_R;
      stale = len3(sub3(P, xf_point(in->parts[p].xf, F3(b[0], b[1], b[2])))) < r ||
              len3(sub3(P, xf_point(in->parts[p].xf_prev, F3(b[0], b[1], b[2])))) < r;
    }
    if (!stale) continue;
    const sl_node* nd = &in->nodes[g];
    float s3 = Gs->scale[0] * Gs->scale[1] * Gs->scale[2];
    float inorm = iso_norm(nd);
    float t[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t c = 0; c < BN_NCELL; c++) {
      f3 w = bn_cell_dir(cells, c);
      f3 u = xf_dir_inv(xf, w);
      float v = vgrid_lookup(&in->vgrid[g], u) * 1.0f;
      if (v <= 0.0f) continue;
      float a = inorm * footprint(nd, s3 * s3, u) * v * cells[4 * c + 3];
      float y[9];
      bn_sh2(w, y);
      for (int m = 0; m < 9; m++) t[m] += a * y[m];
    }
    float* xo = st->xfer + 12u * g;
    for (int m = 0; m < 9; m++) xo[m] = t[m];
    xo[9] = xo[10] = xo[11] = 0.0f;
  }

  /* the sender cut: re-selected top down by depth when a part moved (or on the first frame), with the cut nodes'
   * transfer; then the shadow T of the cut nodes that refresh this frame */
  const int sc = in->sender_cut != 0u;
  const uint32_t fq = in->frame % 4u;
  const int resel = sc && in->sc_reselect != 0u;
  const float sc_brad = L->terrain ? 0.0f : (float)(0.5 * sqrt((double)L->step[0] * L->step[0] +
                                                               (double)L->step[1] * L->step[1] +
                                                               (double)L->step[2] * L->step[2]));
  if (resel) {
    uint32_t* parent = (uint32_t*)malloc(sizeof(uint32_t) * N);
    uint32_t* by_depth = (uint32_t*)malloc(sizeof(uint32_t) * N);
    uint32_t dcount[257] = {0};
    if (!parent || !by_depth) return -1;
    for (uint32_t n = 0; n < N; n++) parent[n] = NONE_U32;
    for (uint32_t n = G; n < N; n++)
      for (uint32_t j = in->nodes[n].child_lo; j < in->nodes[n].child_hi; j++) parent[in->kids[j]] = n;
    for (uint32_t n = 0; n < N; n++) dcount[(in->nodes[n].depth < 255u ? in->nodes[n].depth : 255u) + 1u]++;
    for (int d = 1; d < 257; d++) dcount[d] += dcount[d - 1];
    uint32_t fill[256];
    for (int d = 0; d < 256; d++) fill[d] = dcount[d];
    for (uint32_t n = 0; n < N; n++) by_depth[fill[in->nodes[n].depth < 255u ? in->nodes[n].depth : 255u]++] = n;
    for (int d = 0; d < 256; d++) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
#endif
      for (int64_t t = dcount[d]; t < (int64_t)dcount[d + 1]; t++) {
        uint32_t n = by_depth[t];
        st->sc_flag[n] = sc_select_one(in, &PS, parent, st->sc_flag, n, sc_brad);
      }
    }
    free(parent);
    free(by_depth);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
#endif
    for (int64_t ni = G; ni < (int64_t)N; ni++)
      if (st->sc_flag[ni] == SC_NODE) sc_xfer_one(in, cells, (uint32_t)ni, st->sc_X + 32u * (uint32_t)(ni - G));
  }
  if (sc) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
#endif
    for (int64_t ni = G; ni < (int64_t)N; ni++) {
      uint32_t n = (uint32_t)ni;
      if (st->sc_flag[n] != SC_NODE || !(resel || n % 4u == fq)) continue;
      sc_shadow_one(in, n, st->sc_T + (n - G), st->sc_envT + 4u * (n - G));
    }
  }

  /* direct_dirs_emit + env_dirs: a quarter of the Gaussians (g % 4 == frame % 4); with the sender cut only the cut's
   * leaves among them (direct_dirs_emit_sc, env_dirs_sc), then the cut nodes that refresh this frame
   * (direct_dirs_nodes_sc, env_dirs_nodes_sc) */
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
#endif
  for (int64_t gi = in->frame % 4u; gi < (int64_t)G; gi += 4)
    if (!sc || st->sc_flag[gi] == SC_LEAF) bn_direct_one(in, (uint32_t)gi, st->lo_dir);
  if (sc) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
#endif
    for (int64_t ni = G; ni < (int64_t)N; ni++) {
      uint32_t n = (uint32_t)ni;
      if (st->sc_flag[n] != SC_NODE || !(resel || n % 4u == fq)) continue;
      sc_direct_node(in, n, st->sc_T[n - G], st->sc_envT + 4u * (n - G), st->sc_X + 32u * (n - G));
    }
  }

  /* node_leaf */
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 256)
#endif
  for (int64_t gi = 0; gi < (int64_t)G; gi++) {
    uint32_t g = (uint32_t)gi;
    if (sc && st->sc_flag[g] != SC_LEAF) continue; /* node_leaf_list: the cut's leaves */
    const sl_gaussian* Gs = &in->gs[g];
    const sl_node* nd = &in->nodes[g];
    const float* xf = in->parts[Gs->part_surface & 0xFFFFu].xf;
    float s3 = Gs->scale[0] * Gs->scale[1] * Gs->scale[2];
    int dark = (Gs->part_surface & 0xFFFFu) == in->dark_part; /* emitBounceFix (bounce.wgsl:1177-1187) */
    f3 Lr = dark ? F3(0.0f, 0.0f, 0.0f)
                 : add3(F3(st->lo_dir[4 * g], st->lo_dir[4 * g + 1], st->lo_dir[4 * g + 2]),
                        F3(st->lo_b[12 * g + 4], st->lo_b[12 * g + 5], st->lo_b[12 * g + 6]));
    for (int k = 0; k < 14; k++) {
      f3 wo = xf_dir_inv(xf, F3(d14[3 * k], d14[3 * k + 1], d14[3 * k + 2]));
      float w = footprint(nd, s3 * s3, wo) * vgrid_lookup(&in->vgrid[g], wo);
      float* o = st->node_acc + 4u * (14u * g + (uint32_t)k);
      o[0] = Lr.x * w;
      o[1] = Lr.y * w;
      o[2] = Lr.z * w;
      o[3] = w;
    }
  }
  /* node_cut: the cut nodes as senders, from the probes of the frame before */
  if (sc) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
#endif
    for (int64_t ni = G; ni < (int64_t)N; ni++)
      if (st->sc_flag[ni] == SC_NODE)
        sc_node_cut(in, &PS, d14, st->probe_data, st->probe_sh, (uint32_t)ni, st->sc_X + 32u * (uint32_t)(ni - G),
                    st->node_acc);
  }
  /* node_up: depths max_depth - 1 .. 1, children summed in kids order (with the sender cut the open nodes only) */
  for (int d = (int)in->max_depth - 1; d >= 1; d--) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 256)
#endif
    for (int64_t ii = G; ii < (int64_t)N; ii++) {
      const sl_node* nd = &in->nodes[ii];
      if (nd->depth != (uint32_t)d || nd->part == NONE_U32) continue;
      if (sc && st->sc_flag[ii] != SC_OPEN) continue;
      for (int k = 0; k < 14; k++) {
        float s[4] = {0, 0, 0, 0};
        for (uint32_t j = nd->child_lo; j < nd->child_hi; j++) {
          const float* c = st->node_acc + 4u * (14u * in->kids[j] + (uint32_t)k);
          for (int q = 0; q < 4; q++) s[q] += c[q];
        }
        float* o = st->node_acc + 4u * (14u * (uint32_t)ii + (uint32_t)k);
        for (int q = 0; q < 4; q++) o[q] = s[q];
      }
    }
  }
  /* node_sh2: the 14-direction means fitted to SH2, packed as 27 halves */
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 256)
#endif
  for (int64_t ii = 0; ii < (int64_t)N; ii++) {
    if (sc && st->sc_flag[ii] == SC_BELOW) { /* under the cut: the gather reads zero (the reference's null slot) */
      for (int j = 0; j < 14; j++) st->node_sh[14u * (uint32_t)ii + (uint32_t)j] = 0u;
      continue;
    }
    f3 Lk[14];
    for (int k = 0; k < 14; k++) {
      const float* a = st->node_acc + 4u * (14u * (uint32_t)ii + (uint32_t)k);
      Lk[k] = div3(F3(a[0], a[1], a[2]), fmaxf(a[3], 1e-12f));
    }
    float h[28];
    h[27] = 0.0f;
    for (int m = 0; m < 9; m++) {
      f3 c = F3(0.0f, 0.0f, 0.0f);
      for (int k = 0; k < 14; k++) c = add3(c, mul3(Lk[k], pinv[14 * m + k]));
      h[3 * m] = c.x;
      h[3 * m + 1] = c.y;
      h[3 * m + 2] = c.z;
    }
    for (int j = 0; j < 14; j++)
      st->node_sh[14u * (uint32_t)ii + (uint32_t)j] = orc_f32_to_f16(h[2 * j]) | (orc_f32_to_f16(h[2 * j + 1]) << 16);
  }

  /* probe_gather: every (probe, cell) ray of the lattice */
  /* block_rad: half the lattice cell's diagonal (lighting.js:794, float64); 0 for terrain probes (each cuts
   * around itself) */
  const float brad = L->terrain ? 0.0f : (float)(0.5 * sqrt((double)L->step[0] * L->step[0] +
                                                            (double)L->step[1] * L->step[1] +
                                                            (double)L->step[2] * L->step[2]));
  const float tmax = L->tmax;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
#endif
  for (int64_t id64 = 0; id64 < (int64_t)NP * BN_NCELL; id64++) {
    uint32_t id = (uint32_t)id64, p = id / BN_NCELL, c = id % BN_NCELL;
    /* a part probe skips its own part (and a static part's stay idle); a volume's probes skip their object */
    uint32_t skip = NONE_U32;
    if (p >= NL && p < NL + 8u * in->part_count) {
      skip = (p - NL) / 8u;
      if (!bn_is_part_probe_part(in, skip)) continue;
    } else if (p >= NL) {
      skip = bn_vol_of_probe(in, &PS, p - NL);
      if (skip == NONE_U32) continue;
    }
    f3 o = bn_probe_pos(in, &PS, p);
    f3 w = bn_cell_dir(cells, c);
    uint32_t dz = L->dims[2];
    f3 cen = o;
    if (!L->terrain && p < NL) {
      float bx = (float)((p / (L->dims[1] * dz)) / 2u), by = (float)(((p / dz) % L->dims[1]) / 2u),
            bz = (float)((p % dz) / 2u);
      cen = F3(L->lo[0] + L->step[0] * (2.0f * bx + 0.5f), L->lo[1] + L->step[1] * (2.0f * by + 0.5f),
               L->lo[2] + L->step[2] * (2.0f * bz + 0.5f));
    }
    float t1 = tmax;
    float ht[BN_HIT_MAX], hv[BN_HIT_MAX];
    uint32_t hn[BN_HIT_MAX];
    uint32_t k = 0;
    const float pbrad = p < NL ? brad : 0.0f;   /* probes off the lattice cut around themselves */
    for (uint32_t q = 0; q < in->part_count; q++) {
      if (q == skip) continue;
      const float* xf = in->parts[q].xf;
      f3 Po = xf_dir_inv(xf, sub3(o, F3(xf[3], xf[7], xf[11])));
      f3 wr = xf_dir_inv(xf, w);
      f3 cr = xf_dir_inv(xf, sub3(cen, F3(xf[3], xf[7], xf[11])));
      if (in->parts[q].root == NONE_U32) continue;
      uint32_t stack[BN_STACK];
      stack[0] = in->parts[q].root;
      uint32_t sp = 1;
      while (sp > 0u) {
        sp--;
        uint32_t ni = stack[sp];
        const sl_node* nd = &in->nodes[ni];
        f3 mean = F3(nd->mean[0], nd->mean[1], nd->mean[2]);
        f3 d = sub3(mean, Po);
        float tt = clampf(dot3(d, wr), 0.0f, t1);
        f3 e = sub3(d, mul3(wr, tt));
        if (dot3(e, e) > nd->radius * nd->radius) continue;
        int use_node = ni < G;
        if (!use_node) use_node = len3(sub3(cr, mean)) - pbrad > BN_THETA * nd->smax;
        if (use_node) {
          float tau = nd->kappa * dirm(nd, wr) * bn_seg_geom(nd, Po, wr, 0.0f, t1);
          if (tau > 1e-6f) {
            f3 cw = sym_mul(nd_cinv_d(nd), nd_cinv_o(nd), wr);
            float den = dot3(cw, wr);
            float tp = fabsf(den) > 1e-30f ? clampf(dot3(cw, d) / den, 0.0f, t1) : t1;
            uint32_t at = k < BN_HIT_MAX - 1u ? k : BN_HIT_MAX - 1u;
            uint32_t l = BN_HIT_MAX - 1u;
            if (k == BN_HIT_MAX && tp >= ht[l]) {
              ht[l] = fmaxf(ht[l], tp);
              hv[l] = fminf(hv[l] + tau, 64.0f);
              continue;
            }
            int full = k == BN_HIT_MAX;
            float sv = full ? hv[l] : 0.0f, stv = full ? ht[l] : 0.0f;
            while (at > 0u && ht[at - 1u] > tp) {
              ht[at] = ht[at - 1u];
              hv[at] = hv[at - 1u];
              hn[at] = hn[at - 1u];
              at--;
            }
            ht[at] = tp;
            hv[at] = tau;
            hn[at] = ni;
            if (full) {
              ht[l] = fmaxf(ht[l], stv);
              hv[l] = fminf(hv[l] + sv, 64.0f);
            }
            k = k + 1u < BN_HIT_MAX ? k + 1u : BN_HIT_MAX;
          }
        } else {
          for (uint32_t j = nd->child_lo; j < nd->child_hi; j++)
            if (sp < BN_STACK) stack[sp++] = in->kids[j];
        }
      }
    }
    float T = 1.0f, m1 = 0.0f, m2 = 0.0f, first_part = -1.0f, nearv = 0.0f;
    f3 acc = F3(0.0f, 0.0f, 0.0f);
    float bw[9];
    bn_sh2(mul3(w, -1.0f), bw);
    for (uint32_t i = 0; i < k; i++) {
      if (T <= 0.0f) break;
      float al = 1.0f - sl_expf(-hv[i]);
      f3 rad = bn_node_radiance(st->node_sh, hn[i], bw);
      rad = F3(fmaxf(rad.x, 0.0f), fmaxf(rad.y, 0.0f), fmaxf(rad.z, 0.0f));
      acc = add3(acc, mul3(rad, T * al));
      float dep = clampf(ht[i], 0.0f, t1);
      m1 += T * al * dep;
      m2 += T * al * dep * dep;
      float Tn = T * (1.0f - al);
      if (T >= 0.5f && Tn < 0.5f) {
        uint32_t hp = in->nodes[hn[i]].part;
        first_part = (float)hp;
        nearv = dep < 0.05f ? 1.0f : 0.0f;
        if (hn[i] < G && hp < in->part_count &&
            vgrid_lookup(&in->vgrid[hn[i]], xf_dir_inv(in->parts[hp].xf, mul3(w, -1.0f))) < 0.1f)
          nearv += 2.0f;
      }
      T = Tn;
    }
    if (in->sky_sh && t1 >= tmax * 0.999f) acc = add3(acc, mul3(bn_sky(in->sky_sh, w), T));
    m1 += T * t1;
    m2 += T * t1 * t1;
    float a = in->alpha;
    float* r0 = st->probe_data + 8u * id;
    float* r1 = r0 + 4;
    float* h = st->probe_hist + 16u * id; /* g1a, g1b, g2a, g2b */
    if (a < 0.0f) { /* FIR_TAPS (bounce.wgsl:1253, :1379-1393) */
      r0[0] = 0.5f * acc.x + 0.3f * h[0] + 0.2f * h[8];
      r0[1] = 0.5f * acc.y + 0.3f * h[1] + 0.2f * h[9];
      r0[2] = 0.5f * acc.z + 0.3f * h[2] + 0.2f * h[10];
      r0[3] = first_part;
      r1[0] = 0.5f * m1 + 0.3f * h[3] + 0.2f * h[11];
      r1[1] = 0.5f * m2 + 0.3f * h[4] + 0.2f * h[12];
      r1[3] = nearv;
      for (int q = 0; q < 8; q++) h[8 + q] = h[q];
      h[0] = acc.x; h[1] = acc.y; h[2] = acc.z; h[3] = m1;
      h[4] = m2; h[5] = h[6] = h[7] = 0.0f;
      continue;
    }
    r0[0] = mixf(r0[0], acc.x, a);
    r0[1] = mixf(r0[1], acc.y, a);
    r0[2] = mixf(r0[2], acc.z, a);
    r0[3] = first_part;
    r1[0] = mixf(r1[0], m1, a);
    r1[1] = mixf(r1[1], m2, a);
    r1[3] = nearv;
    if (a >= 1.0f) {
      h[0] = h[8] = acc.x; h[1] = h[9] = acc.y; h[2] = h[10] = acc.z; h[3] = h[11] = m1;
      h[4] = h[12] = m2; h[5] = h[6] = h[7] = h[13] = h[14] = h[15] = 0.0f;
    }
  }
  /* probe_valid */
  for (uint32_t p = 0; p < NP; p++) {
    if (p >= NL) { /* part and volume probes skip their own object, so never sit inside it */
      st->probe_data[8u * (p * BN_NCELL) + 6u] = 1.0f;
      continue;
    }
    uint32_t cnt[17] = {0};
    uint32_t nearc = 0, back = 0;
    for (uint32_t c = 0; c < BN_NCELL; c++) {
      const float* r0 = st->probe_data + 8u * (p * BN_NCELL + c);
      uint32_t fl = (uint32_t)(fmaxf(r0[7], 0.0f) + 0.5f);
      nearc += fl & 1u;
      back += (fl >> 1u) & 1u;
      if (r0[3] >= 0.0f) {
        uint32_t q = (uint32_t)r0[3];
        cnt[q < 16u ? q : 16u]++;
      }
    }
    int enclosed = 0;
    for (uint32_t q = 0; q < in->part_count && q < 16u; q++)
      if ((in->parts[q].flags & 1u) == 0u && (float)cnt[q] > BN_G_VALID * (float)BN_NCELL) enclosed = 1;
    st->probe_data[8u * (p * BN_NCELL) + 6u] = (enclosed || nearc * 2u > BN_NCELL || back * 2u > BN_NCELL) ? 0.0f : 1.0f;
  }
  /* probe_sh2 */
  for (uint32_t p = 0; p < NP; p++) {
    f3 c9[9];
    for (int m = 0; m < 9; m++) c9[m] = F3(0.0f, 0.0f, 0.0f);
    for (uint32_t c = 0; c < BN_NCELL; c++) {
      const float* r0 = st->probe_data + 8u * (p * BN_NCELL + c);
      f3 Lc = mul3(F3(r0[0], r0[1], r0[2]), cells[4 * c + 3]);
      float y[9];
      bn_sh2(bn_cell_dir(cells, c), y);
      for (int m = 0; m < 9; m++) c9[m] = add3(c9[m], mul3(Lc, y[m]));
    }
    for (int m = 0; m < 9; m++) {
      float* o = st->probe_sh + 4u * (9u * p + (uint32_t)m);
      o[0] = c9[m].x;
      o[1] = c9[m].y;
      o[2] = c9[m].z;
      o[3] = 0.0f;
    }
  }
  /* bounce_sh (+ gloss_sh) */
  f3 eye = F3(in->eye[0], in->eye[1], in->eye[2]);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 256)
#endif
  for (int64_t gi = 0; gi < (int64_t)G; gi++) {
    uint32_t g = (uint32_t)gi;
    const sl_gaussian* Gs = &in->gs[g];
    const sl_material* mat = &in->mats[mat_index(Gs, in->mat_count)];
    float ks = spec_weight(mat);
    float lw = sqrtf(fminf(mat->flake[1], mat->flake[2]) / fmaxf(mat->flake[0], 1e-12f));
    if (ks > 0.0f && !(lw >= BN_GLOSS_SH_MIN)) { /* near-mirror: bounce_dirs */
      bn_dirs_one(in, &PS, cells, casg, d14, st, g);
      continue;
    }
    uint32_t own = Gs->part_surface & 0xFFFFu;
    const float* xf = in->parts[own].xf;
    f3 P = xf_point(xf, F3(Gs->mu[0], Gs->mu[1], Gs->mu[2]));
    bn_weights pw = bn_weights_for(in, &PS, st->probe_data, P, own);
    f3 Lsh[9];
    for (int m = 0; m < 9; m++) Lsh[m] = F3(0.0f, 0.0f, 0.0f);
    for (int q = 0; q < 8; q++) {
      float wq = pw.w[q];
      if (wq <= 0.0f) continue;
      for (int m = 0; m < 9; m++) {
        const float* s = st->probe_sh + 4u * (9u * pw.pid[q] + (uint32_t)m);
        Lsh[m] = add3(Lsh[m], mul3(F3(s[0], s[1], s[2]), wq));
      }
    }
    const float* t = st->xfer + 12u * g;
    f3 cc = mul3(Lsh[0], t[0]);
    for (int m = 1; m < 9; m++) cc = add3(cc, mul3(Lsh[m], t[m]));
    f3 alb = F3(Gs->albedo[0], Gs->albedo[1], Gs->albedo[2]);
    f3 cb = mul3v(alb, F3(fmaxf(cc.x, 0.0f), fmaxf(cc.y, 0.0f), fmaxf(cc.z, 0.0f)));
    float* lb = st->lo_b + 12u * g;
    lb[0] = cb.x; lb[1] = cb.y; lb[2] = cb.z; lb[3] = 0.0f;
    lb[4] = cb.x; lb[5] = cb.y; lb[6] = cb.z; lb[7] = 0.0f;
    lb[8] = lb[9] = lb[10] = lb[11] = 0.0f;
    if (ks > 0.0f) {
      const sl_node* nd = &in->nodes[g];
      m3f Rq = quat_matrix(Gs->quat);
      f3 n = Rq.c[0];
      f3 wo = xf_dir_inv(xf, norm3(sub3(eye, P)));
      f3 wm = mirror3(wo, n);
      float s3 = Gs->scale[0] * Gs->scale[1] * Gs->scale[2];
      float detC = s3 * s3;
      float vis = vgrid_lookup(&in->vgrid[g], wm) * footprint(nd, detC, wm);
      f3 sp = F3(0.0f, 0.0f, 0.0f);
      if (vis > 0.0f) {
        float inorm = iso_norm(nd);
        float damp = iso_damp(inorm, footprint(nd, detC, wo) * vgrid_lookup(&in->vgrid[g], wo));
        float sg = 2.0f * lw;
        float a1 = sl_expf(-sg * sg), a2 = sl_expf(-3.0f * sg * sg);
        f3 wmw = F3(xf[0] * wm.x + xf[1] * wm.y + xf[2] * wm.z, xf[4] * wm.x + xf[5] * wm.y + xf[6] * wm.z,
                    xf[8] * wm.x + xf[9] * wm.y + xf[10] * wm.z);
        float y[9];
        bn_sh2(wmw, y);
        f3 Lm = mul3(Lsh[0], y[0]);
        for (int m = 1; m < 4; m++) Lm = add3(Lm, mul3(Lsh[m], a1 * y[m]));
        for (int m = 4; m < 9; m++) Lm = add3(Lm, mul3(Lsh[m], a2 * y[m]));
        f3 Lp = F3(fmaxf(Lm.x, 0.0f), fmaxf(Lm.y, 0.0f), fmaxf(Lm.z, 0.0f));
        sp = mul3(mul3v(mul3(mul3(mul3(mul3(mul3(alb, inorm), ks), 4.0f), BN_PI), damp), Lp), vis);
      }
      f3 eyec = add3(mul3(cb, 1.0f - ks), sp);
      lb[0] = eyec.x; lb[1] = eyec.y; lb[2] = eyec.z;
    }
  }
  return 0;
}
