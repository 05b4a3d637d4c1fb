// Device-side maths of the lighting kernels (runtime/wgsl/common.wgsl:79-254, material_ext.wgsl:12-181,
// light_shadow.wgsl:69-143).  fp32; the translation unit is compiled with --fmad=false and uses the deterministic
// transcendental functions of sl_detmath.h, so each expression rounds as written (sums left to right, matrix-vector
// as col0*v.x + col1*v.y + col2*v.z) and the results are reproducible on the CPU.
#pragma once

#include <cuda_fp16.h>

#include "sl_detmath.h"
#include "sl_internal.h"

namespace sl {
namespace lm {

// Transcendentals: the deterministic shared definitions by default (the opacity-map kernels must match the CPU
// restatement bit for bit); a translation unit that defines SL_FAST_SHADE (the shading pass, whose output is
// continuous in its inputs and checked to a tolerance) uses the hardware approximations instead.
#ifdef SL_FAST_SHADE
__device__ __forceinline__ float lm_exp(float x) { return __expf(x); }
__device__ __forceinline__ float lm_log(float x) { return __logf(x); }
__device__ __forceinline__ float lm_acos(float x) { return acosf(x); }
__device__ __forceinline__ float lm_asin(float x) { return asinf(x); }
__device__ __forceinline__ float lm_atan2(float y, float x) { return atan2f(y, x); }
#else
__device__ __forceinline__ float lm_exp(float x) { return sl_expf(x); }
__device__ __forceinline__ float lm_log(float x) { return sl_logf(x); }
__device__ __forceinline__ float lm_acos(float x) { return sl_acosf(x); }
__device__ __forceinline__ float lm_asin(float x) { return sl_asinf(x); }
__device__ __forceinline__ float lm_atan2(float y, float x) { return sl_atan2f(y, x); }
#endif

constexpr float kPi = 3.14159265358979f;
constexpr uint32_t kNone = 0xFFFFFFFFu;

struct f3 {
  float x, y, z;
};
struct f2 {
  float x, y;
};
struct m3 {
  f3 c[3];
};
struct m2 {
  f2 c[2];
};

__device__ __forceinline__ f3 F3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f2 F2(float x, float y) { return f2{x, y}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return F3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return F3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 mul3(f3 a, float s) { return F3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 mul3v(f3 a, f3 b) { return F3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 div3(f3 a, float s) { return F3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(f3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ f3 norm3(f3 a) { return div3(a, len3(a)); }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return F3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float dot2(f2 a, f2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) { return F2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ f2 mul2(f2 a, float s) { return F2(a.x * s, a.y * s); }
__device__ __forceinline__ f2 div2(f2 a, float s) { return F2(a.x / s, a.y / s); }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float4 mix4(float4 a, float4 b, float t) {
  return make_float4(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t), mixf(a.w, b.w, t));
}
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
  float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ f3 m3v(const m3& m, f3 v) {
  return F3(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z, m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
            m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z);
}
__device__ __forceinline__ m3 m3m(const m3& a, const m3& b) {
  m3 r;
  r.c[0] = m3v(a, b.c[0]);
  r.c[1] = m3v(a, b.c[1]);
  r.c[2] = m3v(a, b.c[2]);
  return r;
}
__device__ __forceinline__ m3 m3t(const m3& a) {
  m3 r;
  r.c[0] = F3(a.c[0].x, a.c[1].x, a.c[2].x);
  r.c[1] = F3(a.c[0].y, a.c[1].y, a.c[2].y);
  r.c[2] = F3(a.c[0].z, a.c[1].z, a.c[2].z);
  return r;
}
__device__ __forceinline__ m3 m3diag(f3 d) {
  m3 r;
  r.c[0] = F3(d.x, 0.0f, 0.0f);
  r.c[1] = F3(0.0f, d.y, 0.0f);
  r.c[2] = F3(0.0f, 0.0f, d.z);
  return r;
}
__device__ __forceinline__ f2 m2v(const m2& m, f2 v) {
  return F2(m.c[0].x * v.x + m.c[1].x * v.y, m.c[0].y * v.x + m.c[1].y * v.y);
}
__device__ __forceinline__ m2 m2m(const m2& a, const m2& b) {
  m2 r;
  r.c[0] = m2v(a, b.c[0]);
  r.c[1] = m2v(a, b.c[1]);
  return r;
}
__device__ __forceinline__ m2 m2t(const m2& a) {
  m2 r;
  r.c[0] = F2(a.c[0].x, a.c[1].x);
  r.c[1] = F2(a.c[0].y, a.c[1].y);
  return r;
}
__device__ __forceinline__ m2 m2s(const m2& a, float s) {
  m2 r;
  r.c[0] = mul2(a.c[0], s);
  r.c[1] = mul2(a.c[1], s);
  return r;
}
__device__ __forceinline__ float m2det(const m2& m) { return m.c[0].x * m.c[1].y - m.c[1].x * m.c[0].y; }
__device__ __forceinline__ m2 m2inv(const m2& m) {
  float d = m2det(m);
  m2 r;
  r.c[0] = F2(m.c[1].y, -m.c[0].y);
  r.c[1] = F2(-m.c[1].x, m.c[0].x);
  return m2s(r, 1.0f / d);
}
__device__ __forceinline__ float half_lo(uint32_t u) { return __half2float(__ushort_as_half((unsigned short)(u & 0xFFFFu))); }
__device__ __forceinline__ float half_hi(uint32_t u) { return __half2float(__ushort_as_half((unsigned short)(u >> 16))); }

// xf rows [R row | t] (common.wgsl:79-90)
__device__ __forceinline__ f3 xf_point(const float* m, f3 p) {
  return F3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
__device__ __forceinline__ f3 xf_dir_inv(const float* m, f3 d) {
  return add3(add3(mul3(F3(m[0], m[1], m[2]), d.x), mul3(F3(m[4], m[5], m[6]), d.y)), mul3(F3(m[8], m[9], m[10]), d.z));
}
__device__ __forceinline__ float erfc_pos(float z) {
  float t = 1.0f / (1.0f + 0.5f * z);
  float p = -z * z - 1.26551223f +
            t * (1.00002368f +
                 t * (0.37409196f +
                      t * (0.09678418f +
                           t * (-0.18628806f +
                                t * (0.27886807f + t * (-1.13520398f + t * (1.48851587f + t * (-0.82215223f + t * 0.17087277f))))))));
  return t * lm_exp(p);
}
__device__ __forceinline__ f3 sym_mul(f3 d, f3 o, f3 v) {
  return F3(d.x * v.x + o.x * v.y + o.y * v.z, o.x * v.x + d.y * v.y + o.z * v.z, o.y * v.x + o.z * v.y + d.z * v.z);
}

// the fields of a leaf Node the lighting reads (runtime/wgsl/common.wgsl:12-19)
struct Leaf {
  f3 cinv_d, cinv_o, sn_d, sn_o;
  float kappa, iso_norm;
};
__device__ __forceinline__ Leaf load_leaf(const sl_node* n) {
  Leaf l;
  l.cinv_d = F3(n->cinv_diag[0], n->cinv_diag[1], n->cinv_diag[2]);
  l.cinv_o = F3(n->cinv_off[0], n->cinv_off[1], n->cinv_off[2]);
  l.sn_d = F3(n->sn_diag[0], n->sn_diag[1], n->sn_diag[2]);
  l.sn_o = F3(n->sn_off[0], n->sn_off[1], n->sn_off[2]);
  l.kappa = n->kappa;
  l.iso_norm = __uint_as_float(n->pad0);
  return l;
}
__device__ __forceinline__ float dirm(const Leaf& n, f3 w) {
  return sqrtf(fmaxf(dot3(w, sym_mul(n.sn_d, n.sn_o, w)), 0.0f));
}
__device__ __forceinline__ float vgrid_cell(const sl_vgrid& v, uint32_t i, uint32_t j) {
  uint32_t k = i * 16u + j;
  return (float)((v.w[k >> 2u] >> ((k & 3u) * 8u)) & 0xFFu) * (1.0f / 255.0f);
}
// vgrid_lookup (common.wgsl:162-177)
__device__ __forceinline__ float vgrid_lookup(const sl_vgrid& v, f3 w) {
  float el = lm_asin(clampf(w.z, -1.0f, 1.0f));
  float fi = clampf((0.5f * kPi - el) / (kPi / 8.0f) - 0.5f, 0.0f, 7.0f);
  uint32_t i0 = (uint32_t)fi;
  i0 = i0 > 6u ? 6u : i0;
  float ti = fi - (float)i0;
  float az = (fabsf(w.x) + fabsf(w.y) < 1e-30f) ? 0.0f : lm_atan2(w.y, w.x);
  float fj = (az + kPi) / (2.0f * kPi) * 16.0f - 0.5f;
  float j0f = floorf(fj);
  float tj = fj - j0f;
  uint32_t j0 = (uint32_t)((int32_t)j0f + 16) % 16u;
  uint32_t j1 = (j0 + 1u) % 16u;
  float a = mixf(vgrid_cell(v, i0, j0), vgrid_cell(v, i0, j1), tj);
  float b = mixf(vgrid_cell(v, i0 + 1u, j0), vgrid_cell(v, i0 + 1u, j1), tj);
  return mixf(a, b, ti);
}
__device__ __forceinline__ f3 basis_k(f3 w) {
  f3 a = F3(0.0f, 0.0f, 1.0f);
  if (fabsf(w.z) >= 0.999f) a = F3(1.0f, 0.0f, 0.0f);
  return norm3(cross3(a, w));
}
// quat_matrix (common.wgsl:218-223)
__device__ __forceinline__ m3 quat_matrix(float x, float y, float z, float w) {
  m3 m;
  m.c[0] = F3(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + z * w), 2.0f * (x * z - y * w));
  m.c[1] = F3(2.0f * (x * y - z * w), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + x * w));
  m.c[2] = F3(2.0f * (x * z + y * w), 2.0f * (y * z - x * w), 1.0f - 2.0f * (x * x + y * y));
  return m;
}
// ein (common.wgsl:226-239): series below 1, else Abramowitz-Stegun 5.1.56
#ifdef SL_FAST_SHADE
// the same 12-term series Ein(x) = sum_k (-1)^(k+1) x^k / (k k!) evaluated by Horner's rule from its coefficients
__device__ __forceinline__ float ein(float x) {
  if (x < 1.0f) {
    constexpr float c[12] = {(float)(1.0), (float)(-1.0 / 4.0), (float)(1.0 / 18.0), (float)(-1.0 / 96.0),
                             (float)(1.0 / 600.0), (float)(-1.0 / 4320.0), (float)(1.0 / 35280.0),
                             (float)(-1.0 / 322560.0), (float)(1.0 / 3265920.0), (float)(-1.0 / 36288000.0),
                             (float)(1.0 / 439084800.0), (float)(-1.0 / 5748019200.0)};
    float s = c[11];
#pragma unroll
    for (int k = 10; k >= 0; k--) s = s * x + c[k];
    return s * x;
  }
  float p = (((x + 8.5733287401f) * x + 18.0590169730f) * x + 8.6347608925f) * x + 0.2677737343f;
  float q = (((x + 9.5733223454f) * x + 25.6329561486f) * x + 21.0996530827f) * x + 3.9584969228f;
  return lm_log(x) + 0.5772156649f + p / (q * x * lm_exp(x));
}
#else
__device__ __forceinline__ float ein(float x) {
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
#endif
// footprint (common.wgsl:242-246)
__device__ __forceinline__ float footprint(const Leaf& n, float detC, f3 w) {
  float a = dot3(w, sym_mul(n.cinv_d, n.cinv_o, w));
  float K = n.kappa * dirm(n, w) * sqrtf(2.0f * kPi / a);
  return 2.0f * kPi * sqrtf(detC * a) * ein(K);
}

// ---- material_ext.wgsl ---------------------------------------------------------------------------------------
__device__ __forceinline__ float sym_det(f3 d, f3 o) {
  return d.x * (d.y * d.z - o.z * o.z) - o.x * (o.x * d.z - o.z * o.y) + o.y * (o.x * o.z - d.y * o.y);
}
__device__ __forceinline__ float sym_adj_quad(f3 d, f3 o, f3 w) {
  float a00 = d.y * d.z - o.z * o.z, a11 = d.x * d.z - o.y * o.y, a22 = d.x * d.y - o.x * o.x;
  float a01 = o.y * o.z - o.x * d.z, a02 = o.x * o.z - o.y * d.y, a12 = o.x * o.y - d.x * o.z;
  return a00 * w.x * w.x + a11 * w.y * w.y + a22 * w.z * w.z + 2.0f * (a01 * w.x * w.y + a02 * w.x * w.z + a12 * w.y * w.z);
}
__device__ __forceinline__ float spec_weight(const sl_material& m) {
  if ((m.flags & 8u) == 0u || (m.flags & 1u) != 0u) return 0.0f;
  return clampf(half_lo(m.pad0), 0.0f, 1.0f);
}
__device__ __forceinline__ float iso_lobe_from(float k, float p, float damp) {
  return (1.0f - k) + k * 4.0f * kPi * p * damp;
}
__device__ __forceinline__ float iso_damp(float inorm, float avr) {
  return fminf(1.0f, 1.0f / fmaxf(4.0f * kPi * inorm * avr, 1e-30f));
}
__device__ __forceinline__ f3 mirror3(f3 wi, f3 n) { return sub3(mul3(n, 2.0f * dot3(wi, n)), wi); }
__device__ __forceinline__ void onb(f3 n, f3& b0, f3& b1) {
  float s = n.z >= 0.0f ? 1.0f : -1.0f;
  float a = -1.0f / (s + n.z);
  float b = n.x * n.y * a;
  b0 = F3(1.0f + s * n.x * n.x * a, s * b, -s * n.x);
  b1 = F3(b, s + n.y * n.y * a, -n.y);
}
struct s2m {
  float x, y, z;
};
__device__ __forceinline__ float s2_det(s2m s) { return s.x * s.z - s.y * s.y; }
__device__ __forceinline__ float s2_quad(s2m s, f2 v) { return s.x * v.x * v.x + 2.0f * s.y * v.x * v.y + s.z * v.y * v.y; }
__device__ __forceinline__ float s2_quad_inv(s2m s, f2 v) {
  return (s.z * v.x * v.x - 2.0f * s.y * v.x * v.y + s.x * v.y * v.y) / fmaxf(s2_det(s), 1e-30f);
}
__device__ __forceinline__ s2m s2_xf(s2m s, f2 t0, f2 t1) {
  f2 a = F2(s.x * t0.x + s.y * t0.y, s.y * t0.x + s.z * t0.y);
  f2 b = F2(s.x * t1.x + s.y * t1.y, s.y * t1.x + s.z * t1.y);
  return s2m{dot2(t0, a), dot2(t0, b), dot2(t1, b)};
}
__device__ __forceinline__ s2m s2_add(s2m a, s2m b) { return s2m{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ s2m s2_div(s2m a, float d) { return s2m{a.x / d, a.y / d, a.z / d}; }
__device__ __forceinline__ f3 s2_major(s2m s) {
  float h = 0.5f * (s.x - s.z);
  float lam = 0.5f * (s.x + s.z) + sqrtf(h * h + s.y * s.y);
  f2 v = s.x >= s.z ? F2(lam - s.z, s.y) : F2(s.y, lam - s.x);
  float l = sqrtf(dot2(v, v));
  f2 u = l > 1e-20f ? div2(v, l) : F2(1.0f, 0.0f);
  return F3(u.x, u.y, lam);
}
__device__ __forceinline__ float s2_minor(s2m s) {
  float h = 0.5f * (s.x - s.z);
  return 0.5f * (s.x + s.z) - sqrtf(h * h + s.y * s.y);
}
// ---- the specular and ASG phases (material_ext.wgsl:27-63, 127-181) with their per-Gaussian parts computed once
// (the shading pass evaluates them for every light of a Gaussian's cut; only the light's direction and lobe change
// between calls) ---------------------------------------------------------------------------------------------------
struct SpecPre {
  f3 Sd, So;
  float det, c0;                       // max(det S, 1e-20), pi sqrt(det)
  float a00, a11, a22, a01, a02, a12;  // adjugate of S
};
__device__ __forceinline__ SpecPre spec_prepare(f3 Sd, f3 So) {
  SpecPre p;
  p.Sd = Sd;
  p.So = So;
  p.det = fmaxf(sym_det(Sd, So), 1e-20f);
  p.c0 = kPi * sqrtf(p.det);
  p.a00 = Sd.y * Sd.z - So.z * So.z;
  p.a11 = Sd.x * Sd.z - So.y * So.y;
  p.a22 = Sd.x * Sd.y - So.x * So.x;
  p.a01 = So.y * So.z - So.x * Sd.z;
  p.a02 = So.x * So.z - So.y * Sd.y;
  p.a12 = So.x * So.y - Sd.x * So.z;
  return p;
}
__device__ __forceinline__ float phase_specular_p(const SpecPre& p, f3 wi, f3 wo) {
  f3 h = add3(wi, wo);
  float hl = len3(h);
  if (hl < 1e-6f) return 0.0f;
  f3 w = div3(h, hl);
  float adj = p.a00 * w.x * w.x + p.a11 * w.y * w.y + p.a22 * w.z * w.z +
              2.0f * (p.a01 * w.x * w.y + p.a02 * w.x * w.z + p.a12 * w.y * w.z);
  float q = adj / p.det;
  float D = 1.0f / (p.c0 * q * q);
  float sigma = sqrtf(fmaxf(dot3(wi, sym_mul(p.Sd, p.So, wi)), 1e-12f));
  return D / (4.0f * sigma);
}
struct AsgPre {
  bool aniso;
  f3 wr, rb0, rb1;
  s2m s0;
  float pk, minor0;
};
// the parts of asg_phase (material_ext.wgsl:127-181) that depend on the Gaussian and the view only
__device__ __forceinline__ AsgPre asg_prepare(f3 n0, f3 t1, f3 t2, f3 flake, f3 Sd, f3 So, f3 wo) {
  const float ASG_A0 = 2.54696f;
  AsgPre a;
  a.aniso = !(flake.x <= fmaxf(flake.y, flake.z) * 1.0001f);
  float co = dot3(n0, wo);
  f3 n = co >= 0.0f ? n0 : mul3(n0, -1.0f);
  float cos_o = fabsf(co);
  a.wr = sub3(mul3(n, 2.0f * cos_o), wo);
  onb(a.wr, a.rb0, a.rb1);
  f3 dw1 = add3(mul3(n, 2.0f * dot3(wo, t1)), mul3(t1, 2.0f * cos_o));
  f3 dw2 = add3(mul3(n, 2.0f * dot3(wo, t2)), mul3(t2, 2.0f * cos_o));
  f2 j0 = F2(dot3(a.rb0, dw1), dot3(a.rb0, dw2));
  f2 j1 = F2(dot3(a.rb1, dw1), dot3(a.rb1, dw2));
  f2 ia = F2(flake.y / (flake.x - flake.y), flake.z / (flake.x - flake.z));
  a.s0 = s2m{dot2(F2(j0.x * j0.x, j0.y * j0.y), ia), dot2(F2(j0.x * j1.x, j0.y * j1.y), ia),
             dot2(F2(j1.x * j1.x, j1.y * j1.y), ia)};
  a.pk = flake.x * flake.x / (kPi * sqrtf(flake.x * flake.y * flake.z)) /
         (4.0f * sqrtf(fmaxf(dot3(a.wr, sym_mul(Sd, So, a.wr)), 1e-12f)));
  a.minor0 = fmaxf(s2_minor(a.s0) / (2.0f * ASG_A0), 1e-30f);
  return a;
}
__device__ __forceinline__ float asg_phase_p(const AsgPre& a, const SpecPre& sp, f3 wi, f3 lb0, f3 lb1, s2m sl,
                                             f3 wo) {
  const float ASG_W[3] = {0.61163f, 0.35083f, 0.0267f};
  const float ASG_A[3] = {2.54696f, 0.6893f, 0.10727f};
  float pc = phase_specular_p(sp, wi, wo);
  if (!a.aniso) return pc;
  f3 cs = add3(wi, a.wr);
  float cl = len3(cs);
  if (cl < 1e-4f) return pc;
  // t = max(far, 1 - smoothstep(0.12, 0.3, ratio)) is 1 whenever ratio <= 0.12 (the light's angular extent small
  // against the reflection lobe: about half of the evaluations on the hill scene), and then neither the ASG sum nor
  // the `far` test is needed; the terms below are evaluated only when t can still be below 1
  f3 maj = s2_major(sl);
  float ratio = sqrtf(maj.z / a.minor0);
  float t = 1.0f - smoothstepf(0.12f, 0.3f, ratio);
  const float kInv2A[3] = {1.0f / (2.0f * ASG_A[0]), 1.0f / (2.0f * ASG_A[1]), 1.0f / (2.0f * ASG_A[2])};
  f2 dm = F2(0.0f, 0.0f);
  s2m sL{0.0f, 0.0f, 0.0f}, sR{0.0f, 0.0f, 0.0f};
  if (t < 1.0f) {
    f3 c = div3(cs, cl);
    f3 cb0, cb1;
    onb(c, cb0, cb1);
    // log_map(c, wr) - log_map(c, wi): c bisects wi and wr, so both make the same angle with c (one acos) and the
    // components along c cancel; the tangent-plane difference is (wr - wi) projected on (cb0, cb1), scaled by
    // angle / sin(angle)
    {
      const float ca = clampf(dot3(c, wi), -1.0f, 1.0f);
      const f3 v = sub3(wi, mul3(c, ca));
      const float nv = len3(v);
      if (!(nv < 1e-9f)) {
        const float k = lm_acos(ca) / nv;
        const f3 dw = sub3(a.wr, wi);
        dm = F2(k * dot3(cb0, dw), k * dot3(cb1, dw));
      }
    }
    sL = s2_xf(sl, F2(dot3(cb0, lb0), dot3(cb0, lb1)), F2(dot3(cb1, lb0), dot3(cb1, lb1)));
    sR = s2_xf(a.s0, F2(dot3(cb0, a.rb0), dot3(cb0, a.rb1)), F2(dot3(cb1, a.rb0), dot3(cb1, a.rb1)));
    float ndm = fmaxf(sqrtf(dot2(dm, dm)), 1e-9f);
    float d = sqrtf(s2_quad_inv(s2_add(sL, s2m{sR.x * kInv2A[2], sR.y * kInv2A[2], sR.z * kInv2A[2]}), dm));
    float along = sqrtf(fmaxf(s2_quad(sL, dm), 0.0f)) / ndm;
    float far_ = smoothstepf(1.0f, 2.5f, d) * (1.0f - smoothstepf(0.15f, 0.3f, along / ndm));
    t = fmaxf(far_, t);
  }
  float p_asg = 0.0f;
  if (t < 1.0f) {
    const float detR = fmaxf(s2_det(sR), 0.0f);
    for (int k = 0; k < 3; k++) {
      s2m sk = s2m{sR.x * kInv2A[k], sR.y * kInv2A[k], sR.z * kInv2A[k]};
      s2m st = s2_add(sL, sk);
      p_asg += ASG_W[k] * sqrtf(detR * (kInv2A[k] * kInv2A[k]) / fmaxf(s2_det(st), 1e-30f)) *
               lm_exp(-0.5f * s2_quad_inv(st, dm));
    }
    p_asg *= a.pk;
  }
  float p_pt = pc;
  if (t > 0.0f) {
    f3 ax = mul3(add3(mul3(lb0, maj.x), mul3(lb1, maj.y)), sqrtf(3.0f * maj.z));
    p_pt = (2.0f / 3.0f) * pc + (1.0f / 6.0f) * (phase_specular_p(sp, norm3(add3(wi, ax)), wo) +
                                                  phase_specular_p(sp, norm3(sub3(wi, ax)), wo));
  }
  return mixf(p_asg, p_pt, t);
}

__device__ __forceinline__ float phi_cdf(float x) {
  float a = fabsf(x) * 0.70710678f;
  float h = 0.5f * erfc_pos(a);
  return x >= 0.0f ? 1.0f - h : h;
}
__device__ __forceinline__ uint32_t to_u32(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967040.0f) return 0xFFFFFF00u;
  return (uint32_t)x;
}

}  // namespace lm
}  // namespace sl
