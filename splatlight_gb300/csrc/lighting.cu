// Per-Gaussian lighting kernels: iso_init, the emitter light's per-part opacity map (map A) and the sun's
// orthographic opacity maps, which give the shading pass (shade.cu) its shadow transmittances.  One thread per
// Gaussian (or per texel for resolve / mip passes); opacity maps accumulate u32 fixed-point atomics, so their sums do
// not depend on the order the Gaussians run in.
//
//   iso_kernel        runtime/wgsl/iso_init.wgsl:29-56
//   lsm_splat_kernel  runtime/wgsl/light_shadow.wgsl:191-286     lsm_lookup_kernel  :347-392
//   sm_splat_kernel   runtime/wgsl/sun_map.wgsl:127-219          sm_lookup_kernel   :287-324
//   resolve / down    light_shadow.wgsl:290-321, sun_map.wgsl:228-258
//   blur_records_kernel  runtime/wgsl/motion_blur.wgsl:22-127 (the records the map splats draw for a moving part)
// The shading pass lives in shade.cu.  Compiled with --fmad=false (see light_math.cuh): the opacity maps' mip-level
// selection (ceil of a log2) is discontinuous, so these kernels reproduce the CPU restatement's arithmetic exactly.
#include "light_math.cuh"
#include "sl_lighting.h"

namespace sl {

__constant__ float4 c_iso_dirs[128];  // iso_init cell directions (xyz) and solid angles (w)

namespace {

using namespace lm;
constexpr int kThreads = 256;

__device__ __forceinline__ f3 ld3(const float* p) { return F3(p[0], p[1], p[2]); }

__global__ void __launch_bounds__(kThreads) iso_kernel(const sl_gaussian* __restrict__ gs, sl_node* nodes,
                                                       const sl_vgrid* __restrict__ vgrid, uint32_t count) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= count) return;
  const sl_gaussian& G = gs[g];
  Leaf nd = load_leaf(&nodes[g]);
  const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
  float S = 0.0f, S0 = 0.0f;
  const sl_vgrid& vg = vgrid[g];
  for (uint32_t c = 0; c < 128u; c++) {
    const float4 d = c_iso_dirs[c];
    const float v = (float)((vg.w[c >> 2u] >> ((c & 3u) * 8u)) & 0xFFu) * (1.0f / 255.0f);
    const float a = footprint(nd, s3 * s3, F3(d.x, d.y, d.z)) * d.w;
    S += a * v;
    S0 += a;
  }
  const float n = 1.0f / fmaxf(fmaxf(S, 0.02f * S0), 1e-30f);
  nodes[g].pad0 = __float_as_uint(n);
  nodes[g].pad1 = 0u;
}

// ---- light map A -----------------------------------------------------------------------------------------------

__device__ __forceinline__ f2 oct_uv(const LightMapParams& L, f3 w) {
  f3 l = F3(dot3(w, ld3(L.t1)), dot3(w, ld3(L.t2)), dot3(w, ld3(L.normal)));
  if (L.hemi) {
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
__device__ __forceinline__ m2 oct_jac(const LightMapParams& L, f3 w, f3 b0, f3 b1) {
  const float e = 1e-3f;
  f2 u0 = oct_uv(L, w);
  f2 ua = oct_uv(L, norm3(add3(w, mul3(b0, e))));
  f2 ub = oct_uv(L, norm3(add3(w, mul3(b1, e))));
  m2 J;
  J.c[0] = div2(sub2(ua, u0), e);
  J.c[1] = div2(sub2(ub, u0), e);
  return J;
}
// world covariance R (Rq S^2 Rq^T) R^T of a leaf (light_shadow.wgsl:125-137)
__device__ __forceinline__ m3 leaf_cov_world(const sl_gaussian& G, const float* xf) {
  m3 R;
  R.c[0] = F3(xf[0], xf[4], xf[8]);
  R.c[1] = F3(xf[1], xf[5], xf[9]);
  R.c[2] = F3(xf[2], xf[6], xf[10]);
  m3 Rq = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]);
  m3 D = m3diag(F3(G.scale[0] * G.scale[0], G.scale[1] * G.scale[1], G.scale[2] * G.scale[2]));
  m3 t0 = m3m(Rq, D);
  m3 C = m3m(t0, m3t(Rq));
  m3 t1 = m3m(R, C);
  return m3m(t1, m3t(R));
}

// inv3 (light_shadow.wgsl:119-122): the adjugate's rows as columns, over the determinant
__device__ __forceinline__ m3 inv3(const m3& m) {
  const f3 r0 = cross3(m.c[1], m.c[2]), r1 = cross3(m.c[2], m.c[0]), r2 = cross3(m.c[0], m.c[1]);
  const float id = 1.0f / dot3(m.c[0], r0);
  m3 r;
  r.c[0] = F3(r0.x * id, r1.x * id, r2.x * id);
  r.c[1] = F3(r0.y * id, r1.y * id, r2.y * id);
  r.c[2] = F3(r0.z * id, r1.z * id, r2.z * id);
  return r;
}
// world covariance of record g: a leaf from its Gaussian, a tree node from its C^-1 (light_shadow.wgsl:125-137)
__device__ __forceinline__ m3 rec_cov(const sl_gaussian* gs, const sl_node* nodes, uint32_t count, uint32_t g,
                                      const float* xf) {
  if (g < count) return leaf_cov_world(gs[g], xf);
  const sl_node& n = nodes[g];
  m3 S;
  S.c[0] = F3(n.cinv_diag[0], n.cinv_off[0], n.cinv_off[1]);
  S.c[1] = F3(n.cinv_off[0], n.cinv_diag[1], n.cinv_off[2]);
  S.c[2] = F3(n.cinv_off[1], n.cinv_off[2], n.cinv_diag[2]);
  const m3 C = inv3(S);
  m3 R;
  R.c[0] = F3(xf[0], xf[4], xf[8]);
  R.c[1] = F3(xf[1], xf[5], xf[9]);
  R.c[2] = F3(xf[2], xf[6], xf[10]);
  return m3m(m3m(R, C), m3t(R));
}
// The cut's verdict for record g of part p: 0 = not splatted, 1 = splatted as it is, 2 = splatted keeping its rest
// coverage (light_shadow.wgsl:167-210 smear_len / lsm_splat)
__device__ __forceinline__ int cut_verdict(const BlurCut& bc, const sl_part* __restrict__ parts, uint32_t count,
                                           uint32_t g, uint32_t p) {
  const bool leaf = g < count;
  float L = 0.0f;
  const uint32_t root = parts[p].root;
  if (bc.k > 0.0f && bc.shutter > 0.0f && (parts[p].flags & 2u) != 0u && root < bc.n_nodes) {
    const sl_node& rn = bc.n_rest[root];
    const f3 x = F3(rn.mean[0], rn.mean[1], rn.mean[2]);
    const f3 a = xf_point(parts[p].xf, x), b = xf_point(parts[p].xf_prev, x);
    L = bc.shutter * len3(sub3(a, b));
  }
  if (L <= 0.0f) return leaf ? 1 : 0;
  const float thr = bc.k * L;
  if (!leaf && bc.n_rest[g].radius > thr) return 0;
  const uint32_t par = bc.parent[g];
  if (g != root && par != kNone && bc.n_rest[par].radius <= thr) return 0;
  return 2;
}

// One Gaussian's footprint in a map layer: the texels [x0, x1] x [y0, y1] around its centre ct (texels), the inverse of
// its low-passed texel covariance Si, its peak optical depth, the depth at the centre and its gradient, the depth
// variance along the light, the fixed-point scale and the layer's first texel.
struct Foot {
  m2 Si;
  f2 ct, gz;
  float tau0, zc, sz2, fix;
  uint32_t base, res;
  int x0, x1, y0, y1;
};

// One texel of a footprint: tau, tau z and tau (z^2 + sigma_z^2) in u32 fixed point, added atomically (the sums do
// not depend on the order).  kSun: the depth falls along the gradient (sun layers), else it rises (map A).
template <bool kSun>
__device__ __forceinline__ void splat_texel(const Foot& F, int x, int y, uint32_t* acc) {
  f2 dt = sub2(F2((float)x + 0.5f, (float)y + 0.5f), F.ct);
  float q = dot2(dt, m2v(F.Si, dt));
  if (q > 9.0f) return;
  float tt = fminf(F.tau0 * sl_expf(-0.5f * q), 64.0f);
  float t_fix = tt * F.fix;
  if (t_fix < 0.5f) return;
  float z = kSun ? fmaxf(F.zc - dot2(F.gz, dt), 0.0f) : fmaxf(F.zc + dot2(F.gz, dt), 0.0f);
  uint32_t i = (F.base + (uint32_t)y * F.res + (uint32_t)x) * 3u;
  atomicAdd(&acc[i], to_u32(t_fix + 0.5f));
  atomicAdd(&acc[i + 1], to_u32(t_fix * z + 0.5f));
  atomicAdd(&acc[i + 2], to_u32(t_fix * (z * z + F.sz2) + 0.5f));
}

__device__ __forceinline__ float shf(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ int shi(int v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// A warp's 32 footprints (`mine` false for lanes without one): small ones (at most 16 texels) by their own lane, the
// larger ones by the whole warp, one footprint at a time, a texel per lane -- footprints range from one texel to
// 97 x 97, and a lane looping over a large one alone would hold its warp's other lanes idle.
template <bool kSun>
__device__ __forceinline__ void splat_warp(bool mine, const Foot& F, uint32_t* acc) {
  const int w = F.x1 - F.x0 + 1, h = F.y1 - F.y0 + 1;
  const int n = (mine && w > 0 && h > 0) ? w * h : 0;
  if (n > 0 && n <= 16)
    for (int y = F.y0; y <= F.y1; y++)
      for (int x = F.x0; x <= F.x1; x++) splat_texel<kSun>(F, x, y, acc);
  uint32_t big = __ballot_sync(0xffffffffu, n > 16);
  const int lane = (int)(threadIdx.x & 31u);
  while (big) {
    const int src = __ffs(big) - 1;
    big &= big - 1u;
    Foot G;
    G.Si.c[0] = F2(shf(F.Si.c[0].x, src), shf(F.Si.c[0].y, src));
    G.Si.c[1] = F2(shf(F.Si.c[1].x, src), shf(F.Si.c[1].y, src));
    G.ct = F2(shf(F.ct.x, src), shf(F.ct.y, src));
    G.gz = F2(shf(F.gz.x, src), shf(F.gz.y, src));
    G.tau0 = shf(F.tau0, src);
    G.zc = shf(F.zc, src);
    G.sz2 = shf(F.sz2, src);
    G.fix = shf(F.fix, src);
    G.base = (uint32_t)shi((int)F.base, src);
    G.res = (uint32_t)shi((int)F.res, src);
    G.x0 = shi(F.x0, src);
    G.y0 = shi(F.y0, src);
    const int gw = shi(w, src), gn = shi(n, src);
    for (int k = lane; k < gn; k += 32) splat_texel<kSun>(G, G.x0 + k % gw, G.y0 + k / gw, acc);
  }
}

// map A (light_shadow.wgsl:191-286): Gaussian g's footprint in its part's octahedral layer; false when it has none
__device__ __forceinline__ bool lsm_foot(const LightMapParams& L, const sl_gaussian* __restrict__ gs,
                                         const sl_node* __restrict__ nodes, const sl_part* __restrict__ parts,
                                         uint32_t count, const BlurCut& bc, uint32_t g, Foot& F) {
  const bool leaf = g < count;
  const uint32_t p = leaf ? (gs[g].part_surface & 0xFFFFu) : bc.n_rest[g].part;
  if (p >= L.part_count || p == L.skip_part || ((L.dirty >> p) & 1u) == 0u) return false;
  const int verdict = cut_verdict(bc, parts, count, g, p);
  if (verdict == 0) return false;
  const float FIX = 65536.0f, LOWPASS = 0.3f;
  const float* xf = parts[p].xf;
  const Leaf nd = load_leaf(&nodes[g]);
  const f3 mu = leaf ? F3(gs[g].mu[0], gs[g].mu[1], gs[g].mu[2]) : F3(nodes[g].mean[0], nodes[g].mean[1], nodes[g].mean[2]);
  f3 m = xf_point(xf, mu);
  f3 dv = sub3(m, ld3(L.center));
  float r = len3(dv);
  if (r < 1e-4f) return false;
  f3 w = div3(dv, r);
  m3 C = rec_cov(gs, nodes, count, g, xf);
  if (L.hemi && dot3(dv, ld3(L.normal)) < -3.0f * sqrtf(dot3(ld3(L.normal), m3v(C, ld3(L.normal))))) return false;
  f3 b0 = basis_k(w), b1 = cross3(w, b0);
  f3 c0 = m3v(C, b0), c1 = m3v(C, b1);
  float cbbx = dot3(b0, c0), cbby = dot3(b0, c1), cbbz = dot3(b1, c1);
  f3 cw = m3v(C, w);
  f2 cbz = F2(dot3(b0, cw), dot3(b1, cw));
  float czz = dot3(w, cw);
  m2 Cbb;
  Cbb.c[0] = F2(cbbx, cbby);
  Cbb.c[1] = F2(cbby, cbbz);
  m2 Cbb_i = m2inv(Cbb);
  float sz2 = fmaxf(czz - dot2(cbz, m2v(Cbb_i, cbz)), 1e-12f);
  float tau0 = nd.kappa * dirm(nd, xf_dir_inv(xf, w)) * sqrtf(2.0f * kPi * sz2);
  float half_res = 0.5f * (float)L.res;
  m2 J = m2s(oct_jac(L, w, b0, b1), half_res);
  m2 Sang = m2s(Cbb, 1.0f / (r * r));
  m2 S = m2m(m2m(J, Sang), m2t(J));
  float det0 = m2det(S);
  S.c[0].x += LOWPASS;
  S.c[1].y += LOWPASS;
  float det1 = m2det(S);
  tau0 *= sqrtf(fmaxf(det0, 0.0f) / det1);
  if (verdict == 2) {
    // the rest record's peak opacity spread evenly over the stretched footprint: alpha' A' = alpha A
    const Leaf ndr = load_leaf(&bc.n_rest[g]);
    const m3 Cr = rec_cov(bc.g_rest, bc.n_rest, count, g, xf);
    const f3 cwr = m3v(Cr, w);
    const f3 r0 = m3v(Cr, b0), r1 = m3v(Cr, b1);
    m2 Cbr;
    Cbr.c[0] = F2(dot3(b0, r0), dot3(b0, r1));
    Cbr.c[1] = F2(dot3(b0, r1), dot3(b1, r1));
    const f2 cbzr = F2(dot3(b0, cwr), dot3(b1, cwr));
    const float szr = fmaxf(dot3(w, cwr) - dot2(cbzr, m2v(m2inv(Cbr), cbzr)), 1e-12f);
    m2 Sr = m2m(m2m(J, m2s(Cbr, 1.0f / (r * r))), m2t(J));
    const float d0r = m2det(Sr);
    Sr.c[0].x += LOWPASS;
    Sr.c[1].y += LOWPASS;
    const float d1r = m2det(Sr);
    const float tau_r = ndr.kappa * dirm(ndr, xf_dir_inv(xf, w)) * sqrtf(2.0f * kPi * szr) *
                        sqrtf(fmaxf(d0r, 0.0f) / d1r);
    const float a = fminf((1.0f - sl_expf(-tau_r)) * sqrtf(fmaxf(d1r, 1e-30f) / fmaxf(det1, 1e-30f)), 0.999f);
    tau0 = fminf(-sl_logf(1.0f - a), tau0);
  }
  m2 Si = m2inv(S);
  f2 gz = m2v(m2t(m2inv(J)), mul2(m2v(Cbb_i, cbz), r));
  f2 uv = oct_uv(L, w);
  f2 ct = F2((uv.x * 0.5f + 0.5f) * (float)L.res, (uv.y * 0.5f + 0.5f) * (float)L.res);
  int hx = (int)ceilf(3.0f * sqrtf(S.c[0].x)), hy = (int)ceilf(3.0f * sqrtf(S.c[1].y));
  hx = hx > 48 ? 48 : hx;
  hy = hy > 48 ? 48 : hy;
  int cx = (int)floorf(ct.x), cy = (int)floorf(ct.y);
  const uint32_t base = p * L.res * L.res;
  const int ires = (int)L.res;
  const int y0 = cy - hy > 0 ? cy - hy : 0, y1 = cy + hy < ires - 1 ? cy + hy : ires - 1;
  const int x0 = cx - hx > 0 ? cx - hx : 0, x1 = cx + hx < ires - 1 ? cx + hx : ires - 1;
  F.Si = Si;
  F.ct = ct;
  F.gz = gz;
  F.tau0 = tau0;
  F.zc = r;
  F.sz2 = sz2;
  F.fix = FIX;
  F.base = base;
  F.res = L.res;
  F.x0 = x0;
  F.x1 = x1;
  F.y0 = y0;
  F.y1 = y1;
  return true;
}

// One thread per record: the leaves, and with the motion-blur cut on also the tree's internal nodes.
__global__ void __launch_bounds__(kThreads) lsm_splat_kernel(const __grid_constant__ LightMapParams L,
                                                             const sl_gaussian* __restrict__ gs,
                                                             const sl_node* __restrict__ nodes,
                                                             const sl_part* __restrict__ parts, uint32_t count,
                                                             const BlurCut bc, uint32_t n_rec, uint32_t* acc) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  Foot F{};
  const bool mine = g < n_rec && lsm_foot(L, gs, nodes, parts, count, bc, g, F);
  splat_warp<false>(mine, F, acc);
}

// resolve: (alpha, alpha mu, alpha m2) per texel of every dirty layer (light_shadow.wgsl:290-304)
__global__ void __launch_bounds__(kThreads) resolve_kernel(const uint32_t* __restrict__ acc, float fix,
                                                           uint32_t texels, uint32_t layers, uint32_t layer_texels,
                                                           const uint32_t* __restrict__ dirty_layers,
                                                           float4* __restrict__ mip) {
  const uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= (uint64_t)texels * layers) return;
  const uint32_t l = (uint32_t)(i / texels);
  if (dirty_layers && !dirty_layers[l]) return;
  const uint32_t j = (uint32_t)(i - (uint64_t)l * texels);
  float s0 = (float)acc[3 * i] / fix;
  float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
  if (s0 > 1e-5f) {
    float a = 1.0f - sl_expf(-s0);
    o.x = a;
    o.y = a * (float)acc[3 * i + 1] / (fix * s0);
    o.z = a * (float)acc[3 * i + 2] / (fix * s0);
  }
  mip[(uint64_t)l * layer_texels + j] = o;
}

// one mip level from the level above, mean of 4 children (light_shadow.wgsl:307-321)
__global__ void __launch_bounds__(kThreads) down_kernel(float4* mip, uint32_t rk, uint32_t off_src, uint32_t off_dst,
                                                        uint32_t layers, uint32_t layer_texels,
                                                        const uint32_t* __restrict__ dirty_layers) {
  const uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  const uint32_t n = rk * rk;
  if (i >= (uint64_t)n * layers) return;
  const uint32_t l = (uint32_t)(i / n);
  if (dirty_layers && !dirty_layers[l]) return;
  const uint32_t j = (uint32_t)(i - (uint64_t)l * n);
  const uint32_t y = j / rk, x = j - y * rk, pr = rk * 2u;
  const float4* s = mip + (uint64_t)l * layer_texels + off_src + (2u * y) * pr + 2u * x;
  const float4 a = s[0], b = s[1], c = s[pr], d = s[pr + 1];
  mip[(uint64_t)l * layer_texels + off_dst + j] =
      make_float4(0.25f * (a.x + b.x + c.x + d.x), 0.25f * (a.y + b.y + c.y + d.y), 0.25f * (a.z + b.z + c.z + d.z),
                  0.25f * (a.w + b.w + c.w + d.w));
}

__device__ __forceinline__ float4 mip_at(const float4* layer, const uint32_t* level_off, uint32_t res, uint32_t k,
                                         f2 tc) {
  uint32_t rk = res >> k;
  rk = rk < 1u ? 1u : rk;
  float sc = (float)(1u << k);
  float cxf = clampf(tc.x / sc - 0.5f, 0.0f, (float)(rk - 1u)), cyf = clampf(tc.y / sc - 0.5f, 0.0f, (float)(rk - 1u));
  uint32_t i0x = (uint32_t)floorf(cxf), i0y = (uint32_t)floorf(cyf);
  uint32_t i1x = i0x + 1u < rk - 1u ? i0x + 1u : rk - 1u, i1y = i0y + 1u < rk - 1u ? i0y + 1u : rk - 1u;
  float fx = cxf - (float)i0x, fy = cyf - (float)i0y;
  const float4* b = layer + level_off[k];
  float4 a = mix4(b[i0y * rk + i0x], b[i0y * rk + i1x], fx);
  float4 c = mix4(b[i1y * rk + i0x], b[i1y * rk + i1x], fx);
  return mix4(a, c, fy);
}
__device__ __forceinline__ float4 mip_tri(const float4* layer, const uint32_t* level_off, uint32_t res,
                                          uint32_t levels, float l, f2 tc) {
  float lc = clampf(l, 0.0f, (float)(levels - 1u));
  uint32_t k0 = (uint32_t)floorf(lc);
  uint32_t k1 = k0 + 1u < levels - 1u ? k0 + 1u : levels - 1u;
  return mix4(mip_at(layer, level_off, res, k0, tc), mip_at(layer, level_off, res, k1, tc), lc - (float)k0);
}

__global__ void __launch_bounds__(kThreads) lsm_lookup_kernel(const __grid_constant__ LightMapParams L,
                                                              const sl_gaussian* __restrict__ gs,
                                                              const sl_part* __restrict__ parts, uint32_t count,
                                                              const float4* __restrict__ mip, float* __restrict__ lamp_T) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= count) return;
  const sl_gaussian& G = gs[g];
  const uint32_t own = G.part_surface & 0xFFFFu;
  f3 P = xf_point(parts[own].xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  f3 dv = sub3(P, ld3(L.center));
  float z = len3(dv);
  if (z < 1e-4f) {
    lamp_T[g] = 1.0f;
    return;
  }
  f3 w = div3(dv, z);
  f3 b0 = basis_k(w), b1 = cross3(w, b0);
  m2 J = oct_jac(L, w, b0, b1);
  float tex_ang = (2.0f / (float)L.res) / sqrtf(fmaxf(fabsf(m2det(J)), 1e-12f));
  f2 uv = oct_uv(L, w);
  f2 tc = F2((uv.x * 0.5f + 0.5f) * (float)L.res, (uv.y * 0.5f + 0.5f) * (float)L.res);
  float T = 1.0f;
  for (uint32_t p = 0; p < L.part_count; p++) {
    if (p == own || p == L.skip_part) continue;
    const float* bs = parts[p].bound;
    f3 bc = sub3(xf_point(parts[p].xf, F3(bs[0], bs[1], bs[2])), ld3(L.center));
    float dc = len3(bc);
    float zn = fmaxf(dc - bs[3], 0.02f);
    if (z <= zn) continue;
    float search = 2.0f * L.sigma_l * (z - zn) / (zn * z);
    if (dc > bs[3]) {
      float ang = sl_acosf(clampf(dot3(div3(bc, dc), w), -1.0f, 1.0f));
      if (ang > sl_asinf(bs[3] / dc) + search + 2.0f * tex_ang) continue;
    }
    const float4* layer = mip + (uint64_t)p * L.layer_texels;
    float ls = sl_log2f(fmaxf(2.0f * search / tex_ang, 1.0f));
    float4 a0 = mip_tri(layer, L.level_off, L.res, L.levels, ceilf(ls), tc);
    if (a0.x < 1e-4f) continue;
    float zb = fmaxf(a0.y / a0.x, 0.02f);
    float pen = L.sigma_l * fmaxf(z - zb, 0.0f) / (zb * z);
    float4 s = mip_tri(layer, L.level_off, L.res, L.levels, sl_log2f(fmaxf(2.0f * pen / tex_ang, 1.0f)), tc);
    if (s.x < 1e-5f) continue;
    float mu_ = s.y / s.x;
    float sd = sqrtf(fmaxf(s.z / s.x - mu_ * mu_, 1e-8f));
    T *= 1.0f - s.x * phi_cdf((z - mu_) / sd);
  }
  lamp_T[g] = T;
}

// ---- sun maps ----------------------------------------------------------------------------------------------------

// Gaussian g's footprint in sun layer l (sun_map.wgsl:127-219); false when it has none there
__device__ __forceinline__ bool sm_foot(const SunParams& SP, const SunLayer* __restrict__ layers,
                                        const sl_gaussian* __restrict__ gs, const sl_node* __restrict__ nodes,
                                        const sl_part* __restrict__ parts, uint32_t count, const BlurCut& bc,
                                        uint32_t g, uint32_t p, int verdict, uint32_t l, Foot& F) {
  const bool leaf = g < count;
  const float SM_FIX = 4096.0f, SM_LOWPASS = 0.3f;
  const SunLayer ly = layers[l];
  if (!ly.dirty || !SP.lights[ly.light].shadows) return false;
  const float* xf = parts[p].xf;
  const Leaf nd = load_leaf(&nodes[g]);
  const f3 mu = leaf ? F3(gs[g].mu[0], gs[g].mu[1], gs[g].mu[2]) : F3(nodes[g].mean[0], nodes[g].mean[1], nodes[g].mean[2]);
  f3 x = xf_point(xf, mu);
  f3 w = ld3(SP.lights[ly.light].dir);
  f3 b0 = ld3(ly.t1), b1 = ld3(ly.t2);
  m3 C = rec_cov(gs, nodes, count, g, xf);
  f3 c0 = m3v(C, b0), c1 = m3v(C, b1), cw = m3v(C, w);
  m2 Cbb;
  Cbb.c[0] = F2(dot3(b0, c0), dot3(b1, c0));
  Cbb.c[1] = F2(dot3(b0, c1), dot3(b1, c1));
  f2 cbz = F2(dot3(b0, cw), dot3(b1, cw));
  m2 Cbb_i = m2inv(Cbb);
  float sz2 = fmaxf(dot3(w, cw) - dot2(cbz, m2v(Cbb_i, cbz)), 1e-12f);
  float tex = (float)SP.res / (2.0f * ly.half);
  m2 Sm = m2s(Cbb, tex * tex);
  float det0 = m2det(Sm);
  Sm.c[0].x += SM_LOWPASS;
  Sm.c[1].y += SM_LOWPASS;
  float det1 = m2det(Sm);
  float tau0 = nd.kappa * dirm(nd, xf_dir_inv(xf, w)) * sqrtf(2.0f * kPi * sz2) * sqrtf(fmaxf(det0, 0.0f) / det1);
  if (verdict == 2) {  // keep the rest record's coverage (sun_map.wgsl:178-193)
    const Leaf ndr = load_leaf(&bc.n_rest[g]);
    const m3 Cr = rec_cov(bc.g_rest, bc.n_rest, count, g, xf);
    const f3 r0 = m3v(Cr, b0), r1 = m3v(Cr, b1), rw = m3v(Cr, w);
    m2 Cbr;
    Cbr.c[0] = F2(dot3(b0, r0), dot3(b1, r0));
    Cbr.c[1] = F2(dot3(b0, r1), dot3(b1, r1));
    const f2 cbzr = F2(dot3(b0, rw), dot3(b1, rw));
    const float szr = fmaxf(dot3(w, rw) - dot2(cbzr, m2v(m2inv(Cbr), cbzr)), 1e-12f);
    m2 Sr = m2s(Cbr, tex * tex);
    const float d0r = m2det(Sr);
    Sr.c[0].x += SM_LOWPASS;
    Sr.c[1].y += SM_LOWPASS;
    const float d1r = m2det(Sr);
    const float tau_r = ndr.kappa * dirm(ndr, xf_dir_inv(xf, w)) * sqrtf(2.0f * kPi * szr) *
                        sqrtf(fmaxf(d0r, 0.0f) / d1r);
    const float a = fminf((1.0f - sl_expf(-tau_r)) * sqrtf(fmaxf(d1r, 1e-30f) / fmaxf(det1, 1e-30f)), 0.999f);
    tau0 = fminf(-sl_logf(1.0f - a), tau0);
  }
  m2 Si = m2inv(Sm);
  float z0 = ly.zref - dot3(x, w);
  f2 gz = div2(m2v(Cbb_i, cbz), tex);
  f2 ct = F2((dot3(x, b0) - ly.c[0] + ly.half) * tex, (dot3(x, b1) - ly.c[1] + ly.half) * tex);
  int hx = (int)ceilf(3.0f * sqrtf(Sm.c[0].x)), hy = (int)ceilf(3.0f * sqrtf(Sm.c[1].y));
  hx = hx > 32 ? 32 : hx;
  hy = hy > 32 ? 32 : hy;
  int cx = (int)floorf(ct.x), cy = (int)floorf(ct.y);
  const int ires = (int)SP.res;
  F.Si = Si;
  F.ct = ct;
  F.gz = gz;
  F.tau0 = tau0;
  F.zc = z0;
  F.sz2 = sz2;
  F.fix = SM_FIX;
  F.base = l * SP.res * SP.res;
  F.res = SP.res;
  F.y0 = cy - hy > 0 ? cy - hy : 0;
  F.y1 = cy + hy < ires - 1 ? cy + hy : ires - 1;
  F.x0 = cx - hx > 0 ? cx - hx : 0;
  F.x1 = cx + hx < ires - 1 ? cx + hx : ires - 1;
  return true;
}

// Every layer of the Gaussian's part, warp-uniformly: the j-th layer of each lane's part at step j.
__global__ void __launch_bounds__(kThreads) sm_splat_kernel(const __grid_constant__ SunParams SP,
                                                            const SunLayer* __restrict__ layers,
                                                            const sl_gaussian* __restrict__ gs,
                                                            const sl_node* __restrict__ nodes,
                                                            const sl_part* __restrict__ parts, uint32_t count,
                                                            const BlurCut bc, uint32_t n_rec, uint32_t* acc) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  uint32_t p = 0, l_first = 0, n_layers = 0;
  int verdict = 0;
  if (g < n_rec) {
    p = g < count ? (gs[g].part_surface & 0xFFFFu) : bc.n_rest[g].part;
    if (p < SP.n_parts) {
      verdict = cut_verdict(bc, parts, count, g, p);
      if (verdict) {
        l_first = SP.part_first[p];
        n_layers = SP.part_layers[p];
      }
    }
  }
  const uint32_t steps = __reduce_max_sync(0xffffffffu, n_layers);
  for (uint32_t j = 0; j < steps; j++) {
    Foot F{};
    const bool mine = j < n_layers && sm_foot(SP, layers, gs, nodes, parts, count, bc, g, p, verdict, l_first + j, F);
    splat_warp<true>(mine, F, acc);
  }
}

__global__ void __launch_bounds__(kThreads) sm_lookup_kernel(const __grid_constant__ SunParams SP,
                                                             const SunLayer* __restrict__ layers,
                                                             const sl_gaussian* __restrict__ gs,
                                                             const sl_part* __restrict__ parts, uint32_t count,
                                                             const float4* __restrict__ mip, float4* __restrict__ env_T) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= count) return;
  const sl_gaussian& G = gs[g];
  const uint32_t own = G.part_surface & 0xFFFFu;
  f3 P = xf_point(parts[own].xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  float T[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  uint32_t used = kNone;
  for (uint32_t l = 0; l < SP.n_layers; l++) {
    const SunLayer ly = layers[l];
    const uint32_t key = ly.part * 8u + ly.light;
    if (ly.part == own || key == used || !SP.lights[ly.light].shadows) continue;
    f3 w = ld3(SP.lights[ly.light].dir);
    f2 uv = sub2(F2(dot3(P, ld3(ly.t1)), dot3(P, ld3(ly.t2))), F2(ly.c[0], ly.c[1]));
    float inner = (ly.kind == 1u ? 0.9f : 1.0f) * ly.half;
    if (fabsf(uv.x) >= inner || fabsf(uv.y) >= inner) continue;
    used = key;
    float z = ly.zref - dot3(P, w);
    if (z <= 0.0f) continue;
    float texel = 2.0f * ly.half / (float)SP.res;
    f2 tc = F2((uv.x + ly.half) / texel, (uv.y + ly.half) / texel);
    float sig = SP.lights[ly.light].std;
    float search = 2.0f * sig * z;
    const float4* layer = mip + (uint64_t)l * SP.layer_texels;
    float4 a0 = mip_tri(layer, SP.level_off, SP.res, SP.levels, sl_log2f(fmaxf(2.0f * search / texel, 1.0f)), tc);
    if (a0.x < 1e-4f) continue;
    float zb = a0.y / a0.x;
    float pen = sig * fmaxf(z - zb, 0.0f);
    float4 s = mip_tri(layer, SP.level_off, SP.res, SP.levels, sl_log2f(fmaxf(2.0f * pen / texel, 1.0f)), tc);
    if (s.x < 1e-5f) continue;
    float mu_ = s.y / s.x;
    float sd = sqrtf(fmaxf(s.z / s.x - mu_ * mu_, 1e-8f));
    T[ly.light] *= 1.0f - s.x * phi_cdf((z - mu_) / sd);
  }
  env_T[g] = make_float4(T[0], T[1], T[2], T[3]);
}

// ---- motion_blur.wgsl blur_records: the records the opacity-map splats draw, stretched along a moving part's motion
// over the exposure (the box-shutter average: covariance C + d d^T / 12 centred mid-exposure, mass kept) --------------

__device__ __forceinline__ float m3_at(const m3& m, int col, int row) {
  const f3& c = m.c[col];
  return row == 0 ? c.x : (row == 1 ? c.y : c.z);
}
__device__ __forceinline__ void m3_set(m3& m, int col, int row, float v) {
  f3& c = m.c[col];
  if (row == 0) c.x = v; else if (row == 1) c.y = v; else c.z = v;
}

// cyclic Jacobi, 8 sweeps over the pairs (0,1) (0,2) (1,2) (motion_blur.wgsl:37-60): eigenvectors in V's columns
__device__ f3 blur_eig3(m3 A, m3& V) {
  m3 Q = m3diag(F3(1.0f, 1.0f, 1.0f));
  for (int sweep = 0; sweep < 8; sweep++)
    for (int k = 0; k < 3; k++) {
      const int pp = k == 2 ? 1 : 0, q = k == 2 ? 2 : k + 1;
      const float apq = m3_at(A, q, pp);
      if (fabsf(apq) < 1e-30f) continue;
      const float theta = 0.5f * (m3_at(A, q, q) - m3_at(A, pp, pp)) / apq;
      const float sg = theta + (theta == 0.0f ? 1e-30f : 0.0f);
      const float sgn = sg > 0.0f ? 1.0f : (sg < 0.0f ? -1.0f : 0.0f);
      const float t = sgn / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
      const float c = 1.0f / sqrtf(t * t + 1.0f);
      const float sn = t * c;
      m3 J = m3diag(F3(1.0f, 1.0f, 1.0f));
      m3_set(J, pp, pp, c);
      m3_set(J, q, q, c);
      m3_set(J, q, pp, sn);
      m3_set(J, pp, q, -sn);
      A = m3m(m3m(m3t(J), A), J);
      Q = m3m(Q, J);
    }
  V = Q;
  return F3(A.c[0].x, A.c[1].y, A.c[2].z);
}

// column-major rotation -> normalised quaternion (x, y, z, w) (motion_blur.wgsl:62-78)
__device__ float4 blur_mat_to_quat(const m3& m) {
  const float m00 = m3_at(m, 0, 0), m11 = m3_at(m, 1, 1), m22 = m3_at(m, 2, 2);
  const float tr = m00 + m11 + m22;
  float q0, q1, q2, q3;
  if (tr > 0.0f) {
    const float s = sqrtf(tr + 1.0f) * 2.0f;
    q0 = (m3_at(m, 1, 2) - m3_at(m, 2, 1)) / s;
    q1 = (m3_at(m, 2, 0) - m3_at(m, 0, 2)) / s;
    q2 = (m3_at(m, 0, 1) - m3_at(m, 1, 0)) / s;
    q3 = 0.25f * s;
  } else if (m00 > m11 && m00 > m22) {
    const float s = sqrtf(1.0f + m00 - m11 - m22) * 2.0f;
    q0 = 0.25f * s;
    q1 = (m3_at(m, 1, 0) + m3_at(m, 0, 1)) / s;
    q2 = (m3_at(m, 2, 0) + m3_at(m, 0, 2)) / s;
    q3 = (m3_at(m, 1, 2) - m3_at(m, 2, 1)) / s;
  } else if (m11 > m22) {
    const float s = sqrtf(1.0f + m11 - m00 - m22) * 2.0f;
    q0 = (m3_at(m, 1, 0) + m3_at(m, 0, 1)) / s;
    q1 = 0.25f * s;
    q2 = (m3_at(m, 2, 1) + m3_at(m, 1, 2)) / s;
    q3 = (m3_at(m, 2, 0) - m3_at(m, 0, 2)) / s;
  } else {
    const float s = sqrtf(1.0f + m22 - m00 - m11) * 2.0f;
    q0 = (m3_at(m, 2, 0) + m3_at(m, 0, 2)) / s;
    q1 = (m3_at(m, 2, 1) + m3_at(m, 1, 2)) / s;
    q2 = 0.25f * s;
    q3 = (m3_at(m, 0, 1) - m3_at(m, 1, 0)) / s;
  }
  const float l = sqrtf(q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
  return make_float4(q0 / l, q1 / l, q2 / l, q3 / l);
}

// One thread per record (the leaves, then any tree nodes) of a part in `mask` (the parts that moved this frame or the
// last): its copy rewritten, stretched when the part moves (flags bit 1) and the shutter is open, else back to its
// rest record; a leaf's Gaussian is rewritten with its node.
__global__ void __launch_bounds__(kThreads) blur_records_kernel(const sl_part* __restrict__ parts, uint32_t part_count,
                                                                float shutter, uint32_t mask,
                                                                const sl_gaussian* __restrict__ g_src,
                                                                const sl_node* __restrict__ n_src,
                                                                sl_gaussian* __restrict__ g_dst,
                                                                sl_node* __restrict__ n_dst, uint32_t count,
                                                                uint32_t n_nodes) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n_nodes) return;
  sl_node nd = n_src[i];
  const uint32_t p = nd.part;
  if (p >= 32u || ((mask >> p) & 1u) == 0u) return;
  const bool leaf = i < count;
  sl_gaussian G;
  if (leaf) G = g_src[i];
  f3 d = F3(0.0f, 0.0f, 0.0f);
  if (shutter > 0.0f && p < part_count && (parts[p].flags & 2u) != 0u) {
    const f3 x = F3(nd.mean[0], nd.mean[1], nd.mean[2]);
    const f3 a = xf_point(parts[p].xf, x), b = xf_point(parts[p].xf_prev, x);
    d = xf_dir_inv(parts[p].xf, F3(shutter * (a.x - b.x), shutter * (a.y - b.y), shutter * (a.z - b.z)));
  }
  const float dd = dot3(d, d);
  if (dd > 0.0f) {
    m3 Ci;  // the node's C^-1; Sherman-Morrison gives (C + d d^T / 12)^-1
    Ci.c[0] = F3(nd.cinv_diag[0], nd.cinv_off[0], nd.cinv_off[1]);
    Ci.c[1] = F3(nd.cinv_off[0], nd.cinv_diag[1], nd.cinv_off[2]);
    Ci.c[2] = F3(nd.cinv_off[1], nd.cinv_off[2], nd.cinv_diag[2]);
    const f3 cd = m3v(Ci, d);
    const float m = dot3(d, cd);
    const float inv = 1.0f / (12.0f + m);
    const float cdv[3] = {cd.x, cd.y, cd.z};
    m3 Cn;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int r = 0; r < 3; r++) m3_set(Cn, j, r, m3_at(Ci, j, r) - (cdv[r] * cdv[j]) * inv);
    nd.mean[0] = nd.mean[0] - 0.5f * d.x;
    nd.mean[1] = nd.mean[1] - 0.5f * d.y;
    nd.mean[2] = nd.mean[2] - 0.5f * d.z;
    nd.cinv_diag[0] = m3_at(Cn, 0, 0);
    nd.cinv_diag[1] = m3_at(Cn, 1, 1);
    nd.cinv_diag[2] = m3_at(Cn, 2, 2);
    nd.cinv_off[0] = m3_at(Cn, 0, 1);
    nd.cinv_off[1] = m3_at(Cn, 0, 2);
    nd.cinv_off[2] = m3_at(Cn, 1, 2);
    nd.kappa = nd.kappa / sqrtf(1.0f + m / 12.0f);
    nd.smax = sqrtf(nd.smax * nd.smax + dd / 12.0f);
    nd.radius = sqrtf(nd.radius * nd.radius + 0.75f * dd);
  }
  if (dd > 0.0f && leaf) {
    // the Gaussian: the stretched covariance's eigen-frame, scales ascending, right-handed
    const m3 Rq = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]);
    const f3 s2 = F3(G.scale[0] * G.scale[0], G.scale[1] * G.scale[1], G.scale[2] * G.scale[2]);
    m3 C = m3m(m3m(Rq, m3diag(s2)), m3t(Rq));
    const float dv[3] = {d.x, d.y, d.z};
    const float k12 = 1.0f / 12.0f;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int r = 0; r < 3; r++) m3_set(C, j, r, m3_at(C, j, r) + (dv[r] * dv[j]) * k12);
    m3 V;
    f3 ev = blur_eig3(C, V);
    f3 c0 = V.c[0], c1 = V.c[1], c2 = V.c[2];
    if (ev.x > ev.y) { ev = F3(ev.y, ev.x, ev.z); const f3 t = c0; c0 = c1; c1 = t; }
    if (ev.y > ev.z) { ev = F3(ev.x, ev.z, ev.y); const f3 t = c1; c1 = c2; c2 = t; }
    if (ev.x > ev.y) { ev = F3(ev.y, ev.x, ev.z); const f3 t = c0; c0 = c1; c1 = t; }
    c2 = cross3(c0, c1);
    G.mu[0] = G.mu[0] - 0.5f * d.x;
    G.mu[1] = G.mu[1] - 0.5f * d.y;
    G.mu[2] = G.mu[2] - 0.5f * d.z;
    G.kappa = nd.kappa;
    G.scale[0] = sqrtf(fmaxf(ev.x, 1e-12f));
    G.scale[1] = sqrtf(fmaxf(ev.y, 1e-12f));
    G.scale[2] = sqrtf(fmaxf(ev.z, 1e-12f));
    m3 R;
    R.c[0] = c0;
    R.c[1] = c1;
    R.c[2] = c2;
    const float4 q = blur_mat_to_quat(R);
    G.quat[0] = q.x;
    G.quat[1] = q.y;
    G.quat[2] = q.z;
    G.quat[3] = q.w;
  }
  n_dst[i] = nd;
  if (leaf) g_dst[i] = G;
}

}  // namespace

cudaError_t upload_iso_dirs(const float* dirs128x4, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_iso_dirs, dirs128x4, sizeof(float) * 512, 0, cudaMemcpyHostToDevice, s);
}

static uint32_t blocks_for(uint64_t n) { return (uint32_t)((n + kThreads - 1) / kThreads); }

cudaError_t launch_iso(const sl_gaussian* gs, sl_node* nodes, const sl_vgrid* vgrid, uint32_t count, cudaStream_t s) {
  if (!count) return cudaSuccess;
  iso_kernel<<<blocks_for(count), kThreads, 0, s>>>(gs, nodes, vgrid, count);
  return cudaGetLastError();
}

cudaError_t launch_blur_records(const sl_part* parts, uint32_t part_count, float shutter, uint32_t mask,
                                const sl_gaussian* g_src, const sl_node* n_src, sl_gaussian* g_dst, sl_node* n_dst,
                                uint32_t count, uint32_t n_nodes, cudaStream_t s) {
  if (!n_nodes || !mask) return cudaSuccess;
  blur_records_kernel<<<blocks_for(n_nodes), kThreads, 0, s>>>(parts, part_count, shutter, mask, g_src, n_src, g_dst,
                                                                n_dst, count, n_nodes);
  return cudaGetLastError();
}

cudaError_t launch_lsm_splat(const LightMapParams& L, const sl_gaussian* gs, const sl_node* nodes,
                             const sl_part* parts, uint32_t count, const BlurCut& bc, uint32_t* acc, cudaStream_t s) {
  const uint32_t n_rec = bc.k > 0.0f && bc.n_nodes > count ? bc.n_nodes : count;
  if (!n_rec) return cudaSuccess;
  lsm_splat_kernel<<<blocks_for(n_rec), kThreads, 0, s>>>(L, gs, nodes, parts, count, bc, n_rec, acc);
  return cudaGetLastError();
}

cudaError_t launch_resolve(const uint32_t* acc, float fix, uint32_t texels, uint32_t layers, uint32_t layer_texels,
                           const uint32_t* dirty_layers, float4* mip, cudaStream_t s) {
  uint64_t n = (uint64_t)texels * layers;
  if (!n) return cudaSuccess;
  resolve_kernel<<<blocks_for(n), kThreads, 0, s>>>(acc, fix, texels, layers, layer_texels, dirty_layers, mip);
  return cudaGetLastError();
}

cudaError_t launch_mips(float4* mip, uint32_t res, uint32_t levels, const uint32_t* level_off, uint32_t layers,
                        uint32_t layer_texels, const uint32_t* dirty_layers, cudaStream_t s) {
  for (uint32_t k = 1; k < levels; k++) {
    uint32_t rk = res >> k;
    uint64_t n = (uint64_t)rk * rk * layers;
    down_kernel<<<blocks_for(n), kThreads, 0, s>>>(mip, rk, level_off[k - 1], level_off[k], layers, layer_texels,
                                                   dirty_layers);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_lsm_lookup(const LightMapParams& L, const sl_gaussian* gs, const sl_part* parts, uint32_t count,
                              const float4* mip, float* lamp_T, cudaStream_t s) {
  if (!count) return cudaSuccess;
  lsm_lookup_kernel<<<blocks_for(count), kThreads, 0, s>>>(L, gs, parts, count, mip, lamp_T);
  return cudaGetLastError();
}

cudaError_t launch_sm_splat(const SunParams& SP, const SunLayer* layers, const sl_gaussian* gs, const sl_node* nodes,
                            const sl_part* parts, uint32_t count, const BlurCut& bc, uint32_t* acc, cudaStream_t s) {
  const uint32_t n_rec = bc.k > 0.0f && bc.n_nodes > count ? bc.n_nodes : count;
  if (!n_rec) return cudaSuccess;
  sm_splat_kernel<<<blocks_for(n_rec), kThreads, 0, s>>>(SP, layers, gs, nodes, parts, count, bc, n_rec, acc);
  return cudaGetLastError();
}

cudaError_t launch_sm_lookup(const SunParams& SP, const SunLayer* layers, const sl_gaussian* gs, const sl_part* parts,
                             uint32_t count, const float4* mip, float4* env_T, cudaStream_t s) {
  if (!count) return cudaSuccess;
  sm_lookup_kernel<<<blocks_for(count), kThreads, 0, s>>>(SP, layers, gs, parts, count, mip, env_T);
  return cudaGetLastError();
}


}  // namespace sl
