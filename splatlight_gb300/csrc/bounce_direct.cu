// The light each Gaussian sends toward the probes (direct_dirs_emit + env_dirs: runtime/wgsl/emissive.wgsl:1012-1016,
// 1066-1082; environment.wgsl:311-359, 353-359), for the Gaussians g % 4 == frame % 4 (stage 2: a quarter a frame):
// shade_emitters toward the 14 fixed directions DIRS14 (the light cut, M39 transfer, ASG off), each direction's colour
// alb acc_k T iso_norm weighted by footprint x V toward it, then the distant lights' catch alb sum_k I_k T_k V A
// iso_norm for non-emissive Gaussians.  The quarter is taken in the shading pass's Morton order, so a warp's Gaussians
// share their light cuts.  A shiny Gaussian evaluates its specular lobe 14 times per light, so this
// translation unit is compiled for speed (fused multiply-add, approximate division and square root, hardware
// transcendentals), as the shading pass is: its output is continuous in its inputs and checked to a tolerance; the
// per-light parts of the lobe (the SGGX projected area along the light, the lobe's scale) are taken once per light.
#define SL_FAST_SHADE 1
#include "light_math.cuh"
#include "sl_bounce.h"

namespace sl {
namespace {

using namespace lm;
constexpr int kThreads = 128;

// emissive.wgsl DIRS14 (:107-112): the diagonals' components written 0.57735
__constant__ float c_dirs14[14][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {1e-4f, 0.0f, 1.0f},
                                      {-1.0f, 0.0f, 0.0f}, {0.0f, -1.0f, 0.0f}, {1e-4f, 0.0f, -1.0f},
                                      {0.57735f, 0.57735f, 0.57735f}, {0.57735f, 0.57735f, -0.57735f},
                                      {0.57735f, -0.57735f, 0.57735f}, {0.57735f, -0.57735f, -0.57735f},
                                      {-0.57735f, 0.57735f, 0.57735f}, {-0.57735f, 0.57735f, -0.57735f},
                                      {-0.57735f, -0.57735f, 0.57735f}, {-0.57735f, -0.57735f, -0.57735f}};

__device__ __forceinline__ f3 ld3(const float* p) { return F3(p[0], p[1], p[2]); }
__device__ __forceinline__ f3 dir14(const float* xf, int k) {
  return xf_dir_inv(xf, F3(c_dirs14[k][0], c_dirs14[k][1], c_dirs14[k][2]));
}

__global__ void __launch_bounds__(kThreads, 4) direct_kernel(const __grid_constant__ BounceParams B,
                                                             const __grid_constant__ ShadeParams SH,
                                                             const sl_gaussian* __restrict__ gs,
                                                             const sl_node* __restrict__ nodes,
                                                             const sl_vgrid* __restrict__ vgrid,
                                                             const sl_part* __restrict__ parts,
                                                             const sl_material* __restrict__ mats,
                                                             const float* __restrict__ tree,
                                                             const float* __restrict__ lamp_T,
                                                             const float4* __restrict__ env_T,
                                                             const uint32_t* __restrict__ quarter, uint32_t count,
                                                             const uint32_t* __restrict__ flag,
                                                             float4* __restrict__ lo_dir) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= count) return;
  const uint32_t g = quarter[i];
  if (flag && flag[g] != kScLeaf) return;  // direct_dirs_emit_sc / env_dirs_sc: the sender cut's leaves only
  const sl_gaussian& G = gs[g];
  const Leaf nd = load_leaf(&nodes[g]);
  uint32_t mi = G.flags & 0xFFFFu;
  const uint32_t mtop = (SH.material_count > 1u ? SH.material_count : 1u) - 1u;
  mi = mi < mtop ? mi : mtop;
  const sl_material mat = mats[mi];
  const float* xf = parts[G.part_surface & 0xFFFFu].xf;
  const m3 Rq = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]);
  const m3 Sloc = m3m(m3m(Rq, m3diag(F3(mat.flake[0], mat.flake[1], mat.flake[2]))), m3t(Rq));
  const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
  const float detC = s3 * s3;
  const f3 P = xf_point(xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  const f3 n = Rq.c[0];
  const f3 Sd = F3(Sloc.c[0].x, Sloc.c[1].y, Sloc.c[2].z), So = F3(Sloc.c[1].x, Sloc.c[2].x, Sloc.c[2].y);
  const f3 alb = F3(G.albedo[0], G.albedo[1], G.albedo[2]);
  const float ks = spec_weight(mat);
  const bool emissive = (mat.flags & 1u) != 0u;
  const sl_vgrid& vg = vgrid[g];
  f3 acc[14];
#pragma unroll
  for (int k = 0; k < 14; k++) acc[k] = F3(0.0f, 0.0f, 0.0f);
  SpecPre sp;
  if (ks > 0.0f) sp = spec_prepare(Sd, So);
  const float kl = ks * 4.0f * kPi;  // iso_lobe_from's k 4 pi
  if (SH.n_emit) {
    uint32_t node = SH.root;
    for (uint32_t guard = 0; node != kNone && guard < (1u << 16); guard++) {
      const float* e = tree + 24u * node;
      const uint32_t child_lo = __float_as_uint(e[11]), child_hi = __float_as_uint(e[15]);
      const uint32_t skip = __float_as_uint(e[7]);
      const f3 emean = F3(e[0], e[1], e[2]);
      bool use;
      if (child_lo == kNone || SH.mode == 0u) {
        use = child_lo == kNone;
      } else {
        const f3 d = sub3(P, emean);
        use = dot3(d, d) > SH.theta * SH.theta * e[3] * e[3];
      }
      if (!use) {
        node = (child_lo != kNone && __float_as_uint(e[19]) == 0u) ? child_hi : skip;
        continue;
      }
      node = skip;
      const f3 d = sub3(emean, P);
      const float d2 = dot3(d, d);
      if (d2 < 1e-8f) continue;
      const f3 ww = div3(d, sqrtf(d2));
      const f3 wi = xf_dir_inv(xf, ww);
      const float vi = vgrid_lookup(vg, wi);
      if (vi <= 1e-7f) continue;
      const float fp = footprint(nd, detC, wi);
      const f3 mw = mul3(ww, -1.0f);
      float s = 1.0f;
      if (SH.one_sided) {
        const float cs = dot3(mw, ld3(SH.normal));
        s = SH.edge_soft > 0.0f ? smoothstepf(-SH.edge_soft, SH.edge_soft, cs) : (cs > 0.0f ? 1.0f : 0.0f);
      }
      const float mq = sqrtf(fmaxf(dot3(mw, sym_mul(F3(e[4], e[5], e[6]), F3(e[8], e[9], e[10]), mw)), 0.0f));
      const f3 I = mul3(F3(e[12], e[13], e[14]), s * SH.scale * mq);
      const f3 light = mul3(mul3(I, vi), fp / d2);
      if (ks <= 0.0f) {
        acc[0] = add3(acc[0], light);
        continue;
      }
      const f3 wr = mirror3(wi, n);
      const float damp = iso_damp(nd.iso_norm, footprint(nd, detC, wr) * vgrid_lookup(vg, wr));
      // phase_specular (material_ext.wgsl:27-37) toward each direction: D(h) / (4 sigma(wi)), sigma per light
      const float inv4s = 0.25f * rsqrtf(fmaxf(dot3(wi, sym_mul(sp.Sd, sp.So, wi)), 1e-12f));
      const float cl = kl * damp * inv4s;
#pragma unroll
      for (int k = 0; k < 14; k++) {
        const f3 h = add3(wi, dir14(xf, k));
        const float hh = dot3(h, h);
        float p = 0.0f;
        if (hh >= 1e-12f) {
          const float adj = sp.a00 * h.x * h.x + sp.a11 * h.y * h.y + sp.a22 * h.z * h.z +
                            2.0f * (sp.a01 * h.x * h.y + sp.a02 * h.x * h.z + sp.a12 * h.y * h.z);
          const float q = adj / (sp.det * hh);  // the adjugate form of the normalised half vector
          p = 1.0f / (sp.c0 * q * q);
        }
        acc[k] = add3(acc[k], mul3(light, (1.0f - ks) + cl * p));
      }
    }
  }
  const float T = lamp_T[g];
  f3 mean = F3(0.0f, 0.0f, 0.0f), c0 = F3(0.0f, 0.0f, 0.0f);
  float ws = 0.0f;
#pragma unroll
  for (int k = 0; k < 14; k++) {
    const f3 ck = mul3(mul3v(alb, ks <= 0.0f ? acc[0] : acc[k]), T * nd.iso_norm);
    if (k == 0) c0 = ck;
    const f3 wo = dir14(xf, k);
    const float w = footprint(nd, detC, wo) * vgrid_lookup(vg, wo);
    mean = add3(mean, mul3(ck, w));
    ws += w;
  }
  f3 c = ws > 0.0f ? div3(mean, fmaxf(ws, 1e-20f)) : c0;
  if (SH.n_lights && !emissive) {
    const float4 et = env_T[g];
    const float Tk[4] = {et.x, et.y, et.z, et.w};
    f3 dc = F3(0.0f, 0.0f, 0.0f);
    for (uint32_t k = 0; k < SH.n_lights && k < 4u; k++) {
      const f3 wi = xf_dir_inv(xf, ld3(SH.lights[k].dir));
      const float v = vgrid_lookup(vg, wi);
      if (v <= 1e-7f) continue;
      dc = add3(dc, mul3(ld3(SH.lights[k].irr), Tk[k] * v * footprint(nd, detC, wi)));
    }
    c = add3(c, mul3(mul3v(alb, dc), nd.iso_norm));
  }
  lo_dir[g] = make_float4(c.x, c.y, c.z, 0.0f);
}

// direct_dirs_nodes_sc + env_dirs_nodes_sc (emissive.wgsl:1030-1065, environment.wgsl:329-352): the light each face of
// a cut node (its short axis' two sides) catches, before albedo and exposure, from the emitters' light cut (matte:
// shininess left out of the senders) times its sampled lamp T, then the distant lights' catch with its sampled T
__global__ void __launch_bounds__(kThreads, 4) direct_nodes_kernel(const __grid_constant__ BounceParams B,
                                                                   const __grid_constant__ ShadeParams SH,
                                                                   const uint32_t* __restrict__ list,
                                                                   const sl_node* __restrict__ tnodes,
                                                                   const sl_gaussian* __restrict__ sc_gs,
                                                                   const sl_vgrid* __restrict__ sc_vg,
                                                                   const sl_part* __restrict__ parts,
                                                                   const sl_material* __restrict__ mats,
                                                                   const float* __restrict__ tree,
                                                                   const float* __restrict__ sc_T,
                                                                   const float4* __restrict__ sc_E,
                                                                   float4* __restrict__ X) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= list[0]) return;
  const uint32_t n = list[1u + i];
  if (!(B.sc_reselect != 0u || n % 4u == B.frame % 4u)) return;
  const uint32_t r = n - B.G;
  const sl_gaussian& G = sc_gs[r];
  const Leaf nd = load_leaf(&tnodes[n]);
  const float* xf = parts[G.part_surface & 0xFFFFu].xf;
  const f3 nrm = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]).c[0];
  const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
  const float detC = s3 * s3;
  const f3 P = xf_point(xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  const sl_vgrid& vg = sc_vg[r];
  f3 c0 = F3(0.0f, 0.0f, 0.0f), c1 = F3(0.0f, 0.0f, 0.0f);
  if (SH.n_emit) {
    uint32_t node = SH.root;
    for (uint32_t guard = 0; node != kNone && guard < (1u << 16); guard++) {
      const float* e = tree + 24u * node;
      const uint32_t child_lo = __float_as_uint(e[11]), child_hi = __float_as_uint(e[15]);
      const uint32_t skip = __float_as_uint(e[7]);
      const f3 emean = F3(e[0], e[1], e[2]);
      bool use;
      if (child_lo == kNone || SH.mode == 0u) {
        use = child_lo == kNone;
      } else {
        const f3 d = sub3(P, emean);
        use = dot3(d, d) > SH.theta * SH.theta * e[3] * e[3];
      }
      if (!use) {
        node = (child_lo != kNone && __float_as_uint(e[19]) == 0u) ? child_hi : skip;
        continue;
      }
      node = skip;
      const f3 d = sub3(emean, P);
      const float d2 = dot3(d, d);
      if (d2 < 1e-8f) continue;
      const f3 ww = div3(d, sqrtf(d2));
      const f3 wi = xf_dir_inv(xf, ww);
      const float vi = vgrid_lookup(vg, wi);
      if (vi <= 1e-7f) continue;
      const f3 mw = mul3(ww, -1.0f);
      float s = 1.0f;
      if (SH.one_sided) {
        const float cs = dot3(mw, ld3(SH.normal));
        s = SH.edge_soft > 0.0f ? smoothstepf(-SH.edge_soft, SH.edge_soft, cs) : (cs > 0.0f ? 1.0f : 0.0f);
      }
      const float mq = sqrtf(fmaxf(dot3(mw, sym_mul(F3(e[4], e[5], e[6]), F3(e[8], e[9], e[10]), mw)), 0.0f));
      const f3 I = mul3(F3(e[12], e[13], e[14]), s * SH.scale * mq);
      const f3 light = mul3(I, vi * footprint(nd, detC, wi) / d2);
      const float h = 0.5f + 0.5f * clampf(dot3(wi, nrm), -1.0f, 1.0f);
      c0 = add3(c0, mul3(light, h));
      c1 = add3(c1, mul3(light, 1.0f - h));
    }
  }
  const float T = sc_T[r];
  c0 = mul3(c0, T);
  c1 = mul3(c1, T);
  uint32_t mi = G.flags & 0xFFFFu;
  const uint32_t mtop = (SH.material_count > 1u ? SH.material_count : 1u) - 1u;
  mi = mi < mtop ? mi : mtop;
  if (SH.n_lights && (mats[mi].flags & 1u) == 0u) {
    const float4 et = sc_E[r];
    const float Tk[4] = {et.x, et.y, et.z, et.w};
    for (uint32_t k = 0; k < SH.n_lights && k < 4u; k++) {
      const f3 wi = xf_dir_inv(xf, ld3(SH.lights[k].dir));
      const float v = vgrid_lookup(vg, wi);
      if (v <= 1e-7f) continue;
      const f3 c = mul3(ld3(SH.lights[k].irr), Tk[k] * v * footprint(nd, detC, wi));
      const float h = 0.5f + 0.5f * clampf(dot3(wi, nrm), -1.0f, 1.0f);
      c0 = add3(c0, mul3(c, h));
      c1 = add3(c1, mul3(c, 1.0f - h));
    }
  }
  X[8u * r + 6u] = make_float4(c0.x, c0.y, c0.z, 0.0f);
  X[8u * r + 7u] = make_float4(c1.x, c1.y, c1.z, 0.0f);
}

}  // namespace

cudaError_t launch_bounce_direct(const BounceParams& B, const ShadeParams& SH, const BounceBuffers& D, cudaStream_t s) {
  const uint32_t q = B.frame % 4u, count = D.quarter_off[q + 1] - D.quarter_off[q];
  const bool sc = B.sender_cut != 0u;
  if (count)
    direct_kernel<<<(count + kThreads - 1) / kThreads, kThreads, 0, s>>>(
        B, SH, D.gs, D.nodes, D.vgrid, D.parts, D.mats, D.tree, D.lamp_T, D.env_T, D.quarters + D.quarter_off[q],
        count, sc ? D.sc_flag : nullptr, D.lo_dir);
  const uint32_t I = B.N - B.G;
  if (sc && I)
    direct_nodes_kernel<<<(I + kThreads - 1) / kThreads, kThreads, 0, s>>>(B, SH, D.sc_list, D.tnodes, D.sc_gs,
                                                                          D.sc_vg, D.parts, D.mats, D.tree, D.sc_T,
                                                                          D.sc_E, D.sc_X);
  return cudaGetLastError();
}

}  // namespace sl
