// The product's per-Gaussian lighting by emissive Gaussians (shade_leaf / shade_emitters,
// runtime/wgsl/emissive.wgsl:853-980: the light cut over the emitter tree, intensity Le scale sqrt(w^T M w) (:123-130),
// own-part visibility from the V grid (common.wgsl:162-177), the footprint transfer (common.wgsl:241-246) and, for a
// shiny material, the SGGX specular lobe with its iso damping (material_ext.wgsl:27-63)) as a function of free
// per-Gaussian parameters, written once for any scalar types: float for the differentiable path's forward, and Dual
// (value + one directional derivative) for forward-mode derivatives.  The backward takes the radiance's gradient in
// reverse mode, emitter_light_adj below: one walk of the light cut yields the adjoints of the receiver's position and
// fields, and receiver() in forward mode (no walk) carries those to the shape and material parameters; the all-Dual
// emitter_light stays as the forward-mode statement of the same derivative.  Two type parameters keep the dual
// arithmetic where a direction reaches:
// TP for the position and what follows from it alone (light directions and distances, V-grid lookups, the lights'
// intensities along those directions), TM for the Gaussian's shape and material (covariance, normal, SGGX matrix,
// opacity); a position direction runs with TM = float, the other directions with TP = float, and every mixed
// expression takes the dual type.  The Gaussian's leaf quantities follow from the parameters: rest-frame
// C^-1 = R diag(1/s^2) R^T, the SGGX S-hat = R diag(1, (s0/s1)^2, (s0/s2)^2) R^T, kappa = softplus(logit) /
// (sqrt(2 pi) s0), det C = (s0 s1 s2)^2; the material's flake is (1, r^2, r^2) of the roughness r.  The receiver's
// opacity-map transmittance T and its iso_norm (iso_init) are per-scene lighting state: inputs, held constant.  The
// ASG light-shape highlight (EmitParams bit 3) is not part of this model.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "splatlight.h"

namespace sl {
namespace dsh {

// ---- scalar types ---------------------------------------------------------------------------------------------
struct Dual {
  float v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const float r = 1.0f / b.v;
  return {a.v * r, (a.d - a.v * r * b.d) * r};
}
__device__ __forceinline__ Dual operator+(Dual a, float b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator-(Dual a, float b) { return {a.v - b, a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, float b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator/(Dual a, float b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ Dual operator+(float a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator-(float a, Dual b) { return {a - b.v, -b.d}; }
__device__ __forceinline__ Dual operator*(float a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator/(float a, Dual b) {
  const float r = 1.0f / b.v;
  return {a * r, -a * r * r * b.d};
}

// the type of a mixed expression: float only when both operands are
template <typename A, typename B> struct Promote {
  using type = Dual;
};
template <> struct Promote<float, float> {
  using type = float;
};
template <typename A, typename B> using Pr = typename Promote<A, B>::type;

__device__ __forceinline__ float val(float x) { return x; }
__device__ __forceinline__ float val(Dual x) { return x.v; }
template <typename T> __device__ __forceinline__ T cst(float x);
template <> __device__ __forceinline__ float cst<float>(float x) { return x; }
template <> __device__ __forceinline__ Dual cst<Dual>(float x) { return {x, 0.0f}; }

__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ Dual dsqrt(Dual x) {
  const float s = sqrtf(x.v);
  return {s, s > 0.0f ? 0.5f * x.d / s : 0.0f};
}
__device__ __forceinline__ float dexp(float x) { return expf(x); }
__device__ __forceinline__ Dual dexp(Dual x) {
  const float e = expf(x.v);
  return {e, e * x.d};
}
__device__ __forceinline__ float dlog(float x) { return logf(x); }
__device__ __forceinline__ Dual dlog(Dual x) { return {logf(x.v), x.d / x.v}; }
__device__ __forceinline__ float dlog1p(float x) { return log1pf(x); }
__device__ __forceinline__ Dual dlog1p(Dual x) { return {log1pf(x.v), x.d / (1.0f + x.v)}; }
__device__ __forceinline__ float dasin(float x) { return asinf(x); }
__device__ __forceinline__ Dual dasin(Dual x) {
  const float q = 1.0f - x.v * x.v;
  return {asinf(x.v), q > 0.0f ? x.d * rsqrtf(q) : 0.0f};
}
__device__ __forceinline__ float datan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ Dual datan2(Dual y, Dual x) {
  const float r = x.v * x.v + y.v * y.v;
  return {atan2f(y.v, x.v), r > 0.0f ? (x.v * y.d - y.v * x.d) / r : 0.0f};
}
__device__ __forceinline__ float dfloor(float x) { return floorf(x); }
__device__ __forceinline__ Dual dfloor(Dual x) { return {floorf(x.v), 0.0f}; }
// min / max / clamp: the branch taken by value (the derivative of the branch that is active)
template <typename T> __device__ __forceinline__ T dmax(T a, T b) { return val(a) >= val(b) ? a : b; }
template <typename T> __device__ __forceinline__ T dmin(T a, T b) { return val(a) <= val(b) ? a : b; }
template <typename T> __device__ __forceinline__ T dmaxc(T a, float b) { return val(a) >= b ? a : cst<T>(b); }
template <typename T> __device__ __forceinline__ T dminc(T a, float b) { return val(a) <= b ? a : cst<T>(b); }
template <typename T> __device__ __forceinline__ T dclamp(T x, float lo, float hi) { return dminc(dmaxc(x, lo), hi); }

template <typename T>
struct V3 {
  T x, y, z;
};
template <typename T> __device__ __forceinline__ V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <typename A, typename B> __device__ __forceinline__ V3<Pr<A, B>> add(V3<A> a, V3<B> b) {
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename A, typename B> __device__ __forceinline__ V3<Pr<A, B>> sub(V3<A> a, V3<B> b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename A, typename S> __device__ __forceinline__ V3<Pr<A, S>> mul(V3<A> a, S s) {
  return {a.x * s, a.y * s, a.z * s};
}
template <typename A, typename B> __device__ __forceinline__ Pr<A, B> dot(V3<A> a, V3<B> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename A, typename S> __device__ __forceinline__ V3<Pr<A, S>> dvd(V3<A> a, S s) {
  return {a.x / s, a.y / s, a.z / s};
}
template <typename A> __device__ __forceinline__ V3<A> nrm(V3<A> a) { return dvd(a, dsqrt(dot(a, a))); }
// symmetric 3x3 times a vector: diagonal d, off-diagonal o = (xy, xz, yz)
template <typename U, typename T>
__device__ __forceinline__ V3<Pr<T, U>> sym_mul(V3<U> d, V3<U> o, V3<T> v) {
  return {d.x * v.x + o.x * v.y + o.y * v.z, o.x * v.x + d.y * v.y + o.z * v.z, o.y * v.x + o.z * v.y + d.z * v.z};
}

// ---- inputs ----------------------------------------------------------------------------------------------------
// The emitter tree as the shading pass walks it: 24 floats per node (mean, radius, M diagonal, skip link, M off-
// diagonal, child_lo, Le, child_hi, ...; word 19 set where the walk's stack would be full), from the host build.
struct EmitTree {
  const float* nodes;
  uint32_t root, n_emit, mode;
  float theta, scale;
};

// Everything the radiance needs of one Gaussian, derived from its parameters: the position in TP, the rest in TM.
template <typename TP, typename TM>
struct Recv {
  V3<TP> P;                    // position
  V3<TM> n;                    // short axis (the normal the mirror direction uses)
  V3<TM> cinv_d, cinv_o, sn_d, sn_o, Sd, So;
  TM kappa, detC;
};

template <typename TP, typename TM>
__device__ __forceinline__ Recv<TP, TM> receiver(const TP mu[3], const TM ls[3], const TM q4[4], TM logit, TM rough) {
  Recv<TP, TM> r;
  r.P = v3(mu[0], mu[1], mu[2]);
  const TM qn = dsqrt(q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
  const TM x = q4[0] / qn, y = q4[1] / qn, z = q4[2] / qn, w = q4[3] / qn;
  // columns of R (common.wgsl:218-223)
  const V3<TM> c0 = v3(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + z * w), 2.0f * (x * z - y * w));
  const V3<TM> c1 = v3(2.0f * (x * y - z * w), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + x * w));
  const V3<TM> c2 = v3(2.0f * (x * z + y * w), 2.0f * (y * z - x * w), 1.0f - 2.0f * (x * x + y * y));
  r.n = c0;
  const TM s0 = dexp(ls[0]), s1 = dexp(ls[1]), s2 = dexp(ls[2]);
  const TM s3 = s0 * s1 * s2;
  r.detC = s3 * s3;
  // R diag(e) R^T for the three diagonals e
  auto symm = [&](TM e0, TM e1, TM e2, V3<TM>& d, V3<TM>& o) {
    d = v3(c0.x * c0.x * e0 + c1.x * c1.x * e1 + c2.x * c2.x * e2, c0.y * c0.y * e0 + c1.y * c1.y * e1 + c2.y * c2.y * e2,
           c0.z * c0.z * e0 + c1.z * c1.z * e1 + c2.z * c2.z * e2);
    o = v3(c0.x * c0.y * e0 + c1.x * c1.y * e1 + c2.x * c2.y * e2, c0.x * c0.z * e0 + c1.x * c1.z * e1 + c2.x * c2.z * e2,
           c0.y * c0.z * e0 + c1.y * c1.z * e1 + c2.y * c2.z * e2);
  };
  symm(1.0f / (s0 * s0), 1.0f / (s1 * s1), 1.0f / (s2 * s2), r.cinv_d, r.cinv_o);
  const TM a1 = s0 / s1, a2 = s0 / s2;
  symm(cst<TM>(1.0f), a1 * a1, a2 * a2, r.sn_d, r.sn_o);
  const TM fl = dmaxc(rough * rough, 1e-4f);
  symm(cst<TM>(1.0f), fl, fl, r.Sd, r.So);
  // kappa = softplus(logit) / (sqrt(2 pi) s0)
  const TM sp = val(logit) > 20.0f ? logit : dlog1p(dexp(logit));
  r.kappa = sp / (2.50662827463f * s0);
  return r;
}

// ein (common.wgsl:226-239): the 12-term series below 1, else Abramowitz-Stegun 5.1.56
template <typename T>
__device__ __forceinline__ T ein(T x) {
  if (val(x) < 1.0f) {
    T term = x, s = x;
    for (int k = 2; k <= 12; k++) {
      term = term * (-1.0f / (float)k) * x;
      s = s + term / (float)k;
    }
    return s;
  }
  const T x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
  const T p = x4 + 8.5733287401f * x3 + 18.0590169730f * x2 + 8.6347608925f * x + 0.2677737343f;
  const T q = x4 + 9.5733223454f * x3 + 25.6329561486f * x2 + 21.0996530827f * x + 3.9584969228f;
  return dlog(x) + 0.5772156649f + p / (q * x * dexp(x));
}

// footprint (common.wgsl:241-246)
template <typename TP, typename TM, typename TW>
__device__ __forceinline__ Pr<TW, TM> footprint(const Recv<TP, TM>& r, V3<TW> w) {
  using T = Pr<TW, TM>;
  const T a = dot(w, sym_mul(r.cinv_d, r.cinv_o, w));
  const T dm = dsqrt(dmaxc(T(dot(w, sym_mul(r.sn_d, r.sn_o, w))), 0.0f));
  const T K = r.kappa * dm * dsqrt(6.28318530718f / a);
  return 6.28318530718f * dsqrt(r.detC * a) * ein(K);
}

__device__ __forceinline__ float vcell(const sl_vgrid* v, uint32_t i, uint32_t j) {
  if (!v) return 1.0f;
  const uint32_t k = i * 16u + j;
  return (float)((v->w[k >> 2u] >> ((k & 3u) * 8u)) & 0xFFu) * (1.0f / 255.0f);
}

// vgrid_lookup (common.wgsl:162-177); a null grid sees everything
template <typename T>
__device__ __forceinline__ T vgrid(const sl_vgrid* v, V3<T> w) {
  if (!v) return cst<T>(1.0f);
  const float kPi = 3.14159265358979f;
  const T el = dasin(dclamp(w.z, -1.0f, 1.0f));
  const T fi = dclamp((0.5f * kPi - el) / (kPi / 8.0f) - 0.5f, 0.0f, 7.0f);
  uint32_t i0 = (uint32_t)val(fi);
  i0 = i0 > 6u ? 6u : i0;
  const T ti = fi - (float)i0;
  const T az = (fabsf(val(w.x)) + fabsf(val(w.y)) < 1e-30f) ? cst<T>(0.0f) : datan2(w.y, w.x);
  const T fj = (az + kPi) / (2.0f * kPi) * 16.0f - 0.5f;
  const T j0f = dfloor(fj);
  const T tj = fj - j0f;
  const uint32_t j0 = (uint32_t)((int32_t)val(j0f) + 16) % 16u, j1 = (j0 + 1u) % 16u;
  const T a = vcell(v, i0, j0) * (1.0f - tj) + vcell(v, i0, j1) * tj;
  const T b = vcell(v, i0 + 1u, j0) * (1.0f - tj) + vcell(v, i0 + 1u, j1) * tj;
  return a * (1.0f - ti) + b * ti;
}

// phase_specular (material_ext.wgsl:27-63, Heitz SGGX)
template <typename TP, typename TM, typename TW, typename TO>
__device__ __forceinline__ Pr<Pr<TW, TO>, TM> phase_specular(const Recv<TP, TM>& r, V3<TW> wi, V3<TO> wo) {
  using TH = Pr<TW, TO>;
  using T = Pr<TH, TM>;
  const V3<TH> h = add(wi, wo);
  const TH hl = dsqrt(dot(h, h));
  if (val(hl) < 1e-6f) return cst<T>(0.0f);
  const V3<TH> w = dvd(h, hl);
  const V3<TM>& d = r.Sd;
  const V3<TM>& o = r.So;
  const TM det = dmaxc(d.x * (d.y * d.z - o.z * o.z) - o.x * (o.x * d.z - o.z * o.y) + o.y * (o.x * o.z - d.y * o.y),
                       1e-20f);
  const TM a00 = d.y * d.z - o.z * o.z, a11 = d.x * d.z - o.y * o.y, a22 = d.x * d.y - o.x * o.x;
  const TM a01 = o.y * o.z - o.x * d.z, a02 = o.x * o.z - o.y * d.y, a12 = o.x * o.y - d.x * o.z;
  const T adj = a00 * (w.x * w.x) + a11 * (w.y * w.y) + a22 * (w.z * w.z) +
                2.0f * (a01 * (w.x * w.y) + a02 * (w.x * w.z) + a12 * (w.y * w.z));
  const T q = adj / det;
  const T D = 1.0f / (3.14159265358979f * dsqrt(det) * q * q);
  const Pr<TW, TM> sigma = dsqrt(dmaxc(Pr<TW, TM>(dot(wi, sym_mul(d, o, wi))), 1e-12f));
  return D / (4.0f * sigma);
}

// The emitter light gathered by one Gaussian (shade_emitters' acc, emissive.wgsl:873-929), rgb:
// acc = sum_e Le_e scale |w_e|_M f_e over the cut nodes e.  `visit(e, f_e, w_e, |w_e|_M)` is called once per cut node
// (f_e: everything but the node's intensity), so a caller can differentiate the intensities.
template <typename TP, typename TM, typename Visit>
__device__ __forceinline__ V3<Pr<TP, TM>> emitter_light(const EmitTree& E, const Recv<TP, TM>& r, const sl_vgrid* vg,
                                                        float ks, float iso_norm, V3<float> eye, Visit visit) {
  using T = Pr<TP, TM>;
  V3<T> acc = v3(cst<T>(0.0f), cst<T>(0.0f), cst<T>(0.0f));
  if (!E.n_emit) return acc;
  const V3<TP> wo0 = nrm(sub(eye, r.P));
  uint32_t node = E.root;
  for (uint32_t guard = 0; node != 0xFFFFFFFFu && guard < (1u << 16); guard++) {
    const float* e = E.nodes + 24u * node;
    const uint32_t child_lo = __float_as_uint(e[11]), child_hi = __float_as_uint(e[15]);
    const uint32_t skip = __float_as_uint(e[7]);
    const V3<float> emean = v3(e[0], e[1], e[2]);
    bool use;
    if (child_lo == 0xFFFFFFFFu || E.mode == 0u) {
      use = child_lo == 0xFFFFFFFFu;
    } else {
      const V3<TP> dd = sub(r.P, emean);
      use = val(dot(dd, dd)) > E.theta * E.theta * e[3] * e[3];
    }
    if (!use) {
      node = (child_lo != 0xFFFFFFFFu && __float_as_uint(e[19]) == 0u) ? child_hi : skip;
      continue;
    }
    const uint32_t used = node;  // the cut node lit by (and reported to visit); the walk goes on at its skip link
    node = skip;
    const V3<TP> d = sub(emean, r.P);
    const TP d2 = dot(d, d);
    if (val(d2) < 1e-8f) continue;
    const V3<TP> wi = dvd(d, dsqrt(d2));
    const TP vi = vgrid(vg, wi);
    if (val(vi) <= 1e-7f) continue;
    const T fp = footprint(r, wi);
    const V3<TP> mw = mul(wi, -1.0f);
    const V3<float> Md = v3(e[4], e[5], e[6]), Mo = v3(e[8], e[9], e[10]);
    const TP mq = dsqrt(dmaxc(TP(dot(mw, sym_mul(Md, Mo, mw))), 0.0f));
    T f = vi * fp / d2;
    if (ks > 0.0f) {
      const V3<T> wr = sub(mul(r.n, dot(wi, r.n) * 2.0f), wi);
      const T avr = footprint(r, wr) * vgrid(vg, wr);
      const T damp = dmin(cst<T>(1.0f), 1.0f / dmaxc(T(4.0f * 3.14159265358979f * iso_norm * avr), 1e-30f));
      const T lobe = (1.0f - ks) + ks * 4.0f * 3.14159265358979f * phase_specular(r, wi, wo0) * damp;
      f = f * lobe;
    }
    visit(used, f, mw, mq);
    const TP I = mq * E.scale;
    acc = add(acc, v3(e[12] * I * f, e[13] * I * f, e[14] * I * f));
  }
  return acc;
}

// ---- reverse mode: one walk of the cut gives the gradient of ga . acc with respect to the receiver -------------
// The same lighting in float, each cut node's contribution followed at once by its adjoint (the contributions are
// independent given the receiver, so no tape is kept): the adjoints of the position and of every receiver field
// accumulate in RecvAdj, and the caller takes the receiver's own Jacobian (receiver() in forward mode, no walk) to
// the parameters.  Branches (clamps, min / max) pass the derivative of the branch taken, as the Dual forms do.

struct RecvAdj {
  V3<float> P, n, cinv_d, cinv_o, sn_d, sn_o, Sd, So;
  float kappa, detC;
};

__device__ __forceinline__ V3<float> zero3() { return v3(0.0f, 0.0f, 0.0f); }

// the adjoint of a quadratic form w^T S w (S symmetric: d, o) weighted by g: into w and S's six fields
__device__ __forceinline__ void quad_adj(V3<float> d, V3<float> o, V3<float> w, float g, V3<float>& gw,
                                         V3<float>& gd, V3<float>& go) {
  const V3<float> Sw = sym_mul(d, o, w);
  gw = add(gw, mul(Sw, 2.0f * g));
  gd = add(gd, v3(g * (w.x * w.x), g * (w.y * w.y), g * (w.z * w.z)));
  go = add(go, v3(2.0f * g * (w.x * w.y), 2.0f * g * (w.x * w.z), 2.0f * g * (w.y * w.z)));
}

// footprint (common.wgsl:241-246) and its partials with respect to a = w^T C^-1 w, u = w^T S-hat w, kappa, det C
struct FootVG {
  float fp, pa, pu, pk, pd;
};
__device__ __forceinline__ FootVG footprint_vg(const Recv<float, float>& r, V3<float> w) {
  const float a = dot(w, sym_mul(r.cinv_d, r.cinv_o, w));
  const float u = dot(w, sym_mul(r.sn_d, r.sn_o, w));
  const float dm = sqrtf(u >= 0.0f ? u : 0.0f);
  const float s = sqrtf(6.28318530718f / a);
  const float K = r.kappa * dm * s;
  const float Ev = ein(K);
  const float Ed = K > 0.0f ? -expm1f(-K) / K : 1.0f;  // ein'(x) = (1 - e^-x) / x
  const float q = sqrtf(r.detC * a);
  FootVG o;
  o.fp = 6.28318530718f * q * Ev;
  const float gK = 6.28318530718f * q * Ed;  // d fp / d K
  const float gq = 6.28318530718f * Ev;      // d fp / d q
  o.pa = (q > 0.0f ? gq * r.detC * 0.5f / q : 0.0f) + gK * r.kappa * dm * (-0.5f * s / a);
  o.pu = (u >= 0.0f && dm > 0.0f) ? gK * r.kappa * s * 0.5f / dm : 0.0f;
  o.pk = gK * dm * s;
  o.pd = q > 0.0f ? gq * a * 0.5f / q : 0.0f;
  return o;
}
__device__ __forceinline__ void footprint_adj(const Recv<float, float>& r, V3<float> w, const FootVG& F, float g,
                                              V3<float>& gw, RecvAdj& ra) {
  if (g == 0.0f) return;
  quad_adj(r.cinv_d, r.cinv_o, w, g * F.pa, gw, ra.cinv_d, ra.cinv_o);
  quad_adj(r.sn_d, r.sn_o, w, g * F.pu, gw, ra.sn_d, ra.sn_o);
  ra.kappa += g * F.pk;
  ra.detC += g * F.pd;
}

// vgrid_lookup (common.wgsl:162-177) and its gradient with respect to the direction
__device__ __forceinline__ float vgrid_vg(const sl_vgrid* v, V3<float> w, V3<float>& grad) {
  grad = zero3();
  if (!v) return 1.0f;
  const float kPi = 3.14159265358979f;
  const bool zpass = w.z >= -1.0f && w.z <= 1.0f;
  const float zc = fminf(fmaxf(w.z, -1.0f), 1.0f);
  const float el = asinf(zc);
  const float xr = (0.5f * kPi - el) / (kPi / 8.0f) - 0.5f;
  const bool xpass = xr >= 0.0f && xr <= 7.0f;
  const float fi = fminf(fmaxf(xr, 0.0f), 7.0f);
  uint32_t i0 = (uint32_t)fi;
  i0 = i0 > 6u ? 6u : i0;
  const float ti = fi - (float)i0;
  const bool azpass = !(fabsf(w.x) + fabsf(w.y) < 1e-30f);
  const float az = azpass ? atan2f(w.y, w.x) : 0.0f;
  const float fj = (az + kPi) / (2.0f * kPi) * 16.0f - 0.5f;
  const float j0f = floorf(fj);
  const float tj = fj - j0f;
  const uint32_t j0 = (uint32_t)((int32_t)j0f + 16) % 16u, j1 = (j0 + 1u) % 16u;
  const float c00 = vcell(v, i0, j0), c01 = vcell(v, i0, j1), c10 = vcell(v, i0 + 1u, j0), c11 = vcell(v, i0 + 1u, j1);
  const float a = c00 * (1.0f - tj) + c01 * tj;
  const float b = c10 * (1.0f - tj) + c11 * tj;
  const float dti = b - a, dtj = (1.0f - ti) * (c01 - c00) + ti * (c11 - c10);
  const float qz = 1.0f - zc * zc;
  if (xpass && zpass && qz > 0.0f) grad.z = dti * (-8.0f / kPi) * rsqrtf(qz);
  const float rr = w.x * w.x + w.y * w.y;
  if (azpass && rr > 0.0f) {
    const float gaz = dtj * (16.0f / (2.0f * kPi));
    grad.x = -gaz * w.y / rr;
    grad.y = gaz * w.x / rr;
  }
  return a * (1.0f - ti) + b * ti;
}

// phase_specular's adjoint (material_ext.wgsl:27-63): g times its gradient into wi, wo and S (Sd, So)
__device__ __forceinline__ void phase_specular_adj(const Recv<float, float>& r, V3<float> wi, V3<float> wo, float g,
                                                   V3<float>& gwi, V3<float>& gwo, RecvAdj& ra) {
  if (g == 0.0f) return;
  const V3<float> h = add(wi, wo);
  const float hl = sqrtf(dot(h, h));
  if (hl < 1e-6f) return;
  const V3<float> w = dvd(h, hl);
  const V3<float>& d = r.Sd;
  const V3<float>& o = r.So;
  const float detr = d.x * (d.y * d.z - o.z * o.z) - o.x * (o.x * d.z - o.z * o.y) + o.y * (o.x * o.z - d.y * o.y);
  const bool detpass = detr >= 1e-20f;
  const float det = detpass ? detr : 1e-20f;
  const float a00 = d.y * d.z - o.z * o.z, a11 = d.x * d.z - o.y * o.y, a22 = d.x * d.y - o.x * o.x;
  const float a01 = o.y * o.z - o.x * d.z, a02 = o.x * o.z - o.y * d.y, a12 = o.x * o.y - d.x * o.z;
  const float adj = a00 * (w.x * w.x) + a11 * (w.y * w.y) + a22 * (w.z * w.z) +
                    2.0f * (a01 * (w.x * w.y) + a02 * (w.x * w.z) + a12 * (w.y * w.z));
  const float qq = adj / det;
  const float D = 1.0f / (3.14159265358979f * sqrtf(det) * qq * qq);
  const float sw = dot(wi, sym_mul(d, o, wi));
  const bool swpass = sw >= 1e-12f;
  const float sigma = sqrtf(swpass ? sw : 1e-12f);
  const float gD = g / (4.0f * sigma);
  const float gsig = -g * D / (4.0f * sigma * sigma);
  if (swpass) quad_adj(d, o, wi, gsig * 0.5f / sigma, gwi, ra.Sd, ra.So);
  float gdet = gD * (-0.5f * D / det);
  const float gqq = gD * (-2.0f * D / qq);
  const float gadj = gqq / det;
  gdet += -gqq * adj / (det * det);
  const V3<float> Aw = v3(a00 * w.x + a01 * w.y + a02 * w.z, a01 * w.x + a11 * w.y + a12 * w.z,
                          a02 * w.x + a12 * w.y + a22 * w.z);
  const V3<float> gw = mul(Aw, 2.0f * gadj);
  const float g00 = gadj * (w.x * w.x), g11 = gadj * (w.y * w.y), g22 = gadj * (w.z * w.z);
  const float g01 = 2.0f * gadj * (w.x * w.y), g02 = 2.0f * gadj * (w.x * w.z), g12 = 2.0f * gadj * (w.y * w.z);
  V3<float> gd = v3(g11 * d.z + g22 * d.y - g12 * o.z, g00 * d.z + g22 * d.x - g02 * o.y,
                    g00 * d.y + g11 * d.x - g01 * o.x);
  V3<float> go = v3(-2.0f * g22 * o.x - g01 * d.z + g02 * o.z + g12 * o.y,
                    -2.0f * g11 * o.y + g01 * o.z - g02 * d.y + g12 * o.x,
                    -2.0f * g00 * o.z + g01 * o.y + g02 * o.x - g12 * d.x);
  if (detpass) {
    gd = add(gd, v3(gdet * a00, gdet * a11, gdet * a22));
    go = add(go, v3(2.0f * gdet * a01, 2.0f * gdet * a02, 2.0f * gdet * a12));
  }
  ra.Sd = add(ra.Sd, gd);
  ra.So = add(ra.So, go);
  const V3<float> gh = dvd(sub(gw, mul(w, dot(w, gw))), hl);
  gwi = add(gwi, gh);
  gwo = add(gwo, gh);
}

// emitter_light in float with, per cut node, the adjoint of ga . (its contribution) into ra; returns acc.  visit as in
// emitter_light.
template <typename Visit>
__device__ __forceinline__ V3<float> emitter_light_adj(const EmitTree& E, const Recv<float, float>& r,
                                                       const sl_vgrid* vg, float ks, float iso_norm, V3<float> eye,
                                                       V3<float> ga, RecvAdj& ra, Visit visit) {
  V3<float> acc = zero3();
  ra.P = ra.n = ra.cinv_d = ra.cinv_o = ra.sn_d = ra.sn_o = ra.Sd = ra.So = zero3();
  ra.kappa = ra.detC = 0.0f;
  if (!E.n_emit) return acc;
  const float k4pi = 4.0f * 3.14159265358979f;
  const V3<float> vv = sub(eye, r.P);
  const float lv = sqrtf(dot(vv, vv));
  const V3<float> wo0 = dvd(vv, lv);
  V3<float> gwo0 = zero3();
  uint32_t node = E.root;
  for (uint32_t guard = 0; node != 0xFFFFFFFFu && guard < (1u << 16); guard++) {
    const float* e = E.nodes + 24u * node;
    const uint32_t child_lo = __float_as_uint(e[11]), child_hi = __float_as_uint(e[15]);
    const uint32_t skip = __float_as_uint(e[7]);
    const V3<float> emean = v3(e[0], e[1], e[2]);
    bool use;
    if (child_lo == 0xFFFFFFFFu || E.mode == 0u) {
      use = child_lo == 0xFFFFFFFFu;
    } else {
      const V3<float> dd = sub(r.P, emean);
      use = dot(dd, dd) > E.theta * E.theta * e[3] * e[3];
    }
    if (!use) {
      node = (child_lo != 0xFFFFFFFFu && __float_as_uint(e[19]) == 0u) ? child_hi : skip;
      continue;
    }
    const uint32_t used = node;
    node = skip;
    // ---- forward (the values emitter_light computes)
    const V3<float> d = sub(emean, r.P);
    const float d2 = dot(d, d);
    if (d2 < 1e-8f) continue;
    const float dl = sqrtf(d2);
    const V3<float> wi = dvd(d, dl);
    V3<float> gvi;
    const float vi = vgrid_vg(vg, wi, gvi);
    if (vi <= 1e-7f) continue;
    const FootVG Fi = footprint_vg(r, wi);
    const V3<float> mw = mul(wi, -1.0f);
    const V3<float> Md = v3(e[4], e[5], e[6]), Mo = v3(e[8], e[9], e[10]);
    const V3<float> Mmw = sym_mul(Md, Mo, mw);
    const float tq = dot(mw, Mmw);
    const float mq = sqrtf(tq >= 0.0f ? tq : 0.0f);
    const float f0 = vi * Fi.fp / d2;
    float f = f0, lobe = 1.0f, damp = 1.0f, ps = 0.0f, xd = 0.0f, vr = 1.0f, cwn = 0.0f;
    V3<float> wr = zero3(), gvr = zero3();
    FootVG Fr{};
    if (ks > 0.0f) {
      cwn = dot(wi, r.n);
      wr = sub(mul(r.n, cwn * 2.0f), wi);
      Fr = footprint_vg(r, wr);
      vr = vgrid_vg(vg, wr, gvr);
      xd = k4pi * iso_norm * (Fr.fp * vr);
      damp = fminf(1.0f, 1.0f / fmaxf(xd, 1e-30f));
      ps = phase_specular(r, wi, wo0);
      lobe = (1.0f - ks) + ks * k4pi * ps * damp;
      f = f0 * lobe;
    }
    visit(used, f, mw, mq);
    const float I = mq * E.scale;
    acc = add(acc, v3(e[12] * I * f, e[13] * I * f, e[14] * I * f));
    // ---- adjoint of ga . (Le I f)
    const float ce = E.scale * (ga.x * e[12] + ga.y * e[13] + ga.z * e[14]);
    const float gf = ce * mq, gmq = ce * f;
    V3<float> gwi = zero3();
    if (mq > 0.0f) gwi = sub(gwi, mul(Mmw, 2.0f * (gmq * 0.5f / mq)));  // t = mw^T M mw, mw = -wi
    const float gf0 = gf * lobe;
    if (ks > 0.0f) {
      const float globe = gf * f0;
      const float gps = globe * ks * k4pi * damp;
      const float gdamp = globe * ks * k4pi * ps;
      const float gx = (!(1.0f <= 1.0f / fmaxf(xd, 1e-30f)) && xd >= 1e-30f) ? -gdamp / (xd * xd) : 0.0f;
      const float gavr = gx * k4pi * iso_norm;
      V3<float> gwr = mul(gvr, gavr * Fr.fp);
      footprint_adj(r, wr, Fr, gavr * vr, gwr, ra);
      const float gwrn = dot(gwr, r.n);  // wr = 2 (wi . n) n - wi
      ra.n = add(ra.n, add(mul(wi, 2.0f * gwrn), mul(gwr, 2.0f * cwn)));
      gwi = add(gwi, sub(mul(r.n, 2.0f * gwrn), gwr));
      phase_specular_adj(r, wi, wo0, gps, gwi, gwo0, ra);
    }
    const float gvi_s = gf0 * Fi.fp / d2;
    const float gfpi = gf0 * vi / d2;
    const float gd2 = -gf0 * vi * Fi.fp / (d2 * d2);
    gwi = add(gwi, mul(gvi, gvi_s));
    footprint_adj(r, wi, Fi, gfpi, gwi, ra);
    // wi = d / |d|, d2 = d . d, d = emean - P
    const V3<float> gd = add(dvd(sub(gwi, mul(wi, dot(wi, gwi))), dl), mul(d, 2.0f * gd2));
    ra.P = sub(ra.P, gd);
  }
  // wo0 = (eye - P) / |eye - P|
  ra.P = sub(ra.P, dvd(sub(gwo0, mul(wo0, dot(wo0, gwo0))), lv));
  return acc;
}

}  // namespace dsh
}  // namespace sl
