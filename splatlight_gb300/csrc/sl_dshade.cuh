// The product's per-Gaussian lighting by emissive Gaussians (shade_leaf / shade_emitters,
// runtime/wgsl/emissive.wgsl:853-980: the light cut over the emitter tree, intensity Le scale sqrt(w^T M w) (:123-130),
// own-part visibility from the V grid (common.wgsl:162-177), the footprint transfer (common.wgsl:241-246) and, for a
// shiny material, the SGGX specular lobe with its iso damping (material_ext.wgsl:27-63)) as a function of free
// per-Gaussian parameters, written once for any scalar types: float for the differentiable path's forward, and Dual
// (value + one directional derivative) for its backward, which evaluates it once per parameter direction (forward
// mode) to get the Jacobian of the radiance.  Two type parameters keep the dual arithmetic where a direction reaches:
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

}  // namespace dsh
}  // namespace sl
