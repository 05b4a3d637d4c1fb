// The shading pass: one thread per Gaussian sums the emissive-Gaussian lights over its light cut (shade_emit,
// runtime/wgsl/emissive.wgsl:853-980) and the distant lights (env_direct / env_add, environment.wgsl:207-308), plus
// the constant sky ambient, into the radiance the projection reads.  Unlike the opacity maps this output is
// continuous in its inputs, so the translation unit is compiled for speed (fused multiply-add, approximate division
// and square root): it agrees with the CPU restatement to ~1e-6 relative, not to the bit.
// A V grid of all 255 (no own-part occlusion) is recognised once per Gaussian: its lookup is exactly 1 for every
// direction (each cell is 255/255 = 1 and a mix of ones is one), so the three lookups per light are skipped.
#define SL_FAST_SHADE 1  // hardware exp/log/acos, Horner-form Ein: tolerance-checked output
#include "light_math.cuh"
#include "sl_lighting.h"

namespace sl {
namespace {

using namespace lm;
constexpr int kThreads = 128;

__device__ __forceinline__ f3 ld3(const float* p) { return F3(p[0], p[1], p[2]); }

__device__ __forceinline__ float vlook(const sl_vgrid& v, bool open, f3 w) { return open ? 1.0f : vgrid_lookup(v, w); }

// Radiance of Gaussian g seen from SH.eye (shade_leaf + env_add), rgb.
__device__ __forceinline__ f3 shade_one(const ShadeParams& SH, const sl_gaussian* __restrict__ gs,
                                        const sl_node* __restrict__ nodes, const sl_vgrid* __restrict__ vgrid,
                                        const sl_part* __restrict__ parts, const sl_material* __restrict__ mats,
                                        const float* __restrict__ tree, const float* __restrict__ lamp_T,
                                        const float4* __restrict__ env_T, uint32_t g) {
  const sl_gaussian& G = gs[g];
  const Leaf nd = load_leaf(&nodes[g]);
  uint32_t mi = G.flags & 0xFFFFu;
  const uint32_t mtop = (SH.material_count > 1u ? SH.material_count : 1u) - 1u;
  mi = mi < mtop ? mi : mtop;
  const sl_material mat = mats[mi];
  const float* xf = parts[G.part_surface & 0xFFFFu].xf;
  m3 Rq = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]);
  m3 Sloc = m3m(m3m(Rq, m3diag(F3(mat.flake[0], mat.flake[1], mat.flake[2]))), m3t(Rq));
  const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
  const float detC = s3 * s3;
  const f3 P = xf_point(xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  const f3 n = Rq.c[0], t1 = Rq.c[1], t2 = Rq.c[2];
  const f3 Sd = F3(Sloc.c[0].x, Sloc.c[1].y, Sloc.c[2].z), So = F3(Sloc.c[1].x, Sloc.c[2].x, Sloc.c[2].y);
  const f3 flake = F3(mat.flake[0], mat.flake[1], mat.flake[2]);
  const f3 alb = F3(G.albedo[0], G.albedo[1], G.albedo[2]);
  const float ks = spec_weight(mat);
  const bool emissive = (mat.flags & 1u) != 0u;
  const f3 eye = ld3(SH.eye);
  const sl_vgrid& vg = vgrid[g];
  bool open = true;
  {
    const uint4* w4 = reinterpret_cast<const uint4*>(vg.w);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const uint4 q = w4[k];
      open = open && (q.x & q.y & q.z & q.w) == 0xFFFFFFFFu;
    }
  }
  f3 c = F3(0.0f, 0.0f, 0.0f);
  const f3 wo0 = xf_dir_inv(xf, norm3(sub3(eye, P)));
  // per-Gaussian parts of the specular and ASG phases, shared by every light below
  SpecPre sp;
  AsgPre ap;
  if (ks > 0.0f) {
    sp = spec_prepare(Sd, So);
    ap = asg_prepare(n, t1, t2, flake, Sd, So, wo0);
  }
  if (SH.n_emit || emissive) {
    f3 acc = F3(0.0f, 0.0f, 0.0f);
    if (SH.n_emit) {
      // the cut walk of a 48-entry stack (hi child popped first), stackless: word 7 of a node is where the walk
      // goes once the node's subtree is done, word 19 marks nodes the full stack could not refine
      uint32_t node = SH.root;
      const bool shape = SH.asg && ks > 0.0f;
      for (uint32_t guard = 0; node != kNone && guard < (1u << 16); guard++) {
        const float* e = tree + 24u * node;
        const uint32_t child_lo = __float_as_uint(e[11]), child_hi = __float_as_uint(e[15]);
        const uint32_t skip = __float_as_uint(e[7]);
        const f3 emean = F3(e[0], e[1], e[2]);
        bool use;
        if (child_lo == kNone || SH.mode == 0u) {
          use = child_lo == kNone;
        } else {
          f3 d = sub3(P, emean);
          use = dot3(d, d) > SH.theta * SH.theta * e[3] * e[3];
        }
        if (!use) {
          node = (child_lo != kNone && __float_as_uint(e[19]) == 0u) ? child_hi : skip;
          continue;
        }
        node = skip;
        f3 d = sub3(emean, P);
        float d2 = dot3(d, d);
        if (d2 < 1e-8f) continue;
        f3 ww = div3(d, sqrtf(d2));
        f3 wi = xf_dir_inv(xf, ww);
        float vi = vlook(vg, open, wi);
        if (vi <= 1e-7f) continue;
        float fp = footprint(nd, detC, wi);
        f3 mw = mul3(ww, -1.0f);
        float s = 1.0f;
        if (SH.one_sided) {
          float cs = dot3(mw, ld3(SH.normal));
          s = SH.edge_soft > 0.0f ? smoothstepf(-SH.edge_soft, SH.edge_soft, cs) : (cs > 0.0f ? 1.0f : 0.0f);
        }
        float mq = sqrtf(fmaxf(dot3(mw, sym_mul(F3(e[4], e[5], e[6]), F3(e[8], e[9], e[10]), mw)), 0.0f));
        f3 I = mul3(F3(e[12], e[13], e[14]), s * SH.scale * mq);
        f3 light = mul3(mul3(I, vi), fp / d2 * 1.0f);
        if (ks <= 0.0f) {
          acc = add3(acc, light);
          continue;
        }
        f3 wr = mirror3(wi, n);
        float damp = iso_damp(nd.iso_norm, footprint(nd, detC, wr) * vlook(vg, open, wr));
        if (shape) {
          f3 bw0, bw1;
          onb(ww, bw0, bw1);
          f3 cd = F3(e[16], e[17], e[18]), co = F3(e[20], e[21], e[22]);
          f3 cc0 = sym_mul(cd, co, bw0), cc1 = sym_mul(cd, co, bw1);
          s2m slm{dot3(bw0, cc0) / d2, dot3(bw0, cc1) / d2, dot3(bw1, cc1) / d2};
          f3 lb0 = xf_dir_inv(xf, bw0), lb1 = xf_dir_inv(xf, bw1);
          float pp = asg_phase_p(ap, sp, wi, lb0, lb1, slm, wo0);
          acc = add3(acc, mul3(light, iso_lobe_from(ks, pp, damp)));
          continue;
        }
        float lobe = iso_lobe_from(ks, phase_specular_p(sp, wi, wo0), damp);
        acc = add3(acc, mul3(light, lobe));
      }
    }
    const float T = lamp_T[g];
    c = mul3(mul3v(alb, acc), T * nd.iso_norm);
    if (emissive && ((mat.flags & 4u) == 0u || dot3(wo0, n) > 0.0f))
      c = add3(c, F3(half_lo(mat.pad0), half_hi(mat.pad0), half_lo(mat.pad1)));
  }
  if (SH.n_lights && !emissive) {
    const float inorm = nd.iso_norm;
    const float4 et = env_T[g];
    const float Tk[4] = {et.x, et.y, et.z, et.w};
    if (ks <= 0.0f) {
      f3 dc = F3(0.0f, 0.0f, 0.0f);
      for (uint32_t k = 0; k < SH.n_lights; k++) {
        f3 wi = xf_dir_inv(xf, ld3(SH.lights[k].dir));
        float v = vlook(vg, open, wi);
        if (v <= 1e-7f) continue;
        dc = add3(dc, mul3(ld3(SH.lights[k].irr), Tk[k] * v * footprint(nd, detC, wi)));
      }
      c = add3(c, mul3(mul3v(alb, dc), inorm));
    } else {
      const f3 wo = wo0;
      f3 diff = F3(0.0f, 0.0f, 0.0f), spec = F3(0.0f, 0.0f, 0.0f);
      for (uint32_t k = 0; k < SH.n_lights; k++) {
        f3 wi = xf_dir_inv(xf, ld3(SH.lights[k].dir));
        float v = vlook(vg, open, wi);
        if (v <= 1e-7f) continue;
        f3 light = mul3(ld3(SH.lights[k].irr), Tk[k] * v * footprint(nd, detC, wi));
        f3 wr = mirror3(wi, n);
        float damp = iso_damp(inorm, footprint(nd, detC, wr) * vlook(vg, open, wr));
        float s2 = SH.lights[k].std * SH.lights[k].std;
        f3 ob0, ob1;
        onb(wi, ob0, ob1);
        float pp = asg_phase_p(ap, sp, wi, ob0, ob1, s2m{s2, 0.0f, s2}, wo);
        diff = add3(diff, mul3(light, 1.0f - ks));
        spec = add3(spec, mul3(light, iso_lobe_from(ks, pp, damp) - (1.0f - ks)));
      }
      c = add3(c, mul3v(mul3(alb, inorm), add3(diff, spec)));
    }
  }
  if (!emissive && SH.sky_ambient > 0.0f) c = add3(c, mul3(alb, SH.sky_ambient));
  return c;
}

__global__ void __launch_bounds__(kThreads, 4) shade_kernel(const __grid_constant__ ShadeParams SH,
                                                         const sl_gaussian* __restrict__ gs,
                                                         const sl_node* __restrict__ nodes,
                                                         const sl_vgrid* __restrict__ vgrid,
                                                         const sl_part* __restrict__ parts,
                                                         const sl_material* __restrict__ mats,
                                                         const float* __restrict__ tree,
                                                         const float* __restrict__ lamp_T,
                                                         const float4* __restrict__ env_T,
                                                         const uint32_t* __restrict__ order,
                                                         float4* __restrict__ colour, uint32_t count) {
  const uint32_t j = blockIdx.x * kThreads + threadIdx.x;
  if (j >= count) return;
  const uint32_t g = order[j];
  const f3 c = shade_one(SH, gs, nodes, vgrid, parts, mats, tree, lamp_T, env_T, g);
  colour[g] = make_float4(c.x, c.y, c.z, 1.0f);
}

// Batched: the marked scene Gaussians of every lit view (the coverage pass), shaded from the view's eye, with the
// palette and albedo scale the projection applies to bound radiance (project.wgsl:321-350), written into the splat
// records.
// MinB 128-thread blocks per SM (the autotuner's variants: 4 = at most 128 registers, 3 = uncapped at 143, 5 = at
// most 102; on the 64-view mix 4 measured 6.4 ms against 7.6 ms for 3).
template <int MinB>
__global__ void __launch_bounds__(kThreads, MinB) bshade_kernel(const BatchView* __restrict__ views,
                                                          const BatchScene* __restrict__ scenes,
                                                          const uint32_t* __restrict__ block_view,
                                                          const uint32_t* __restrict__ list,
                                                          const uint32_t* __restrict__ view_shade,
                                                          SplatRec* __restrict__ recs,
                                                          uint32_t* __restrict__ view_maxrad) {
  __shared__ ShadeParams sSH;
  __shared__ uint32_t s_max;
  const uint32_t v = block_view[blockIdx.x / 2];
  if (v == kNoView) return;
  const BatchView& V = views[v];
  const BatchScene& S = scenes[V.scene];
  if (V.P.view_mode != 3u || !S.lit) return;
  // this view's marked Gaussians: list[slot_base, slot_base + n)
  const uint32_t n = view_shade[v];
  const uint32_t j = (blockIdx.x / 2 - V.block_first) * 256u + (blockIdx.x & 1u) * kThreads + threadIdx.x;
  if ((blockIdx.x / 2 - V.block_first) * 256u + (blockIdx.x & 1u) * kThreads >= n) return;
  const int t = threadIdx.x;
  if (t == 0) {
    sSH = S.SH;
    sSH.eye[0] = V.eye[0];
    sSH.eye[1] = V.eye[1];
    sSH.eye[2] = V.eye[2];
    sSH.scale *= V.light_scale;  // the request's light state: every light's intensity scaled
    for (uint32_t k = 0; k < 4; k++)
      for (int c = 0; c < 3; c++) sSH.lights[k].irr[c] *= V.light_scale;
    s_max = 0u;
  }
  __syncthreads();
  float mx = 0.0f;
  uint32_t material = kEmitterMaterial, gslot = 0, i = 0;
  if (j < n) {
    gslot = list[V.slot_base + j];
    i = gslot - V.slot_base;
    const sl_gaussian& G = reinterpret_cast<const sl_gaussian*>(V.gaussians)[i];
    uint32_t part = G.part_surface & 0xffffu;
    part = part > kMaxParts - 1u ? kMaxParts - 1u : part;
    material = V.P.parts[part].material;
  }
  if (material != kEmitterMaterial) {  // emissive materials keep their albedo as radiance (the projection's rule)
    const f3 c = shade_one(sSH, reinterpret_cast<const sl_gaussian*>(V.gaussians), S.nodes, S.vgrid, S.parts, S.mats,
                           S.tree, S.lamp_T, S.env_T, i);
    // no bounce buffer on the batched path: radiance = shaded colour x palette x albedo scale
    float cr = c.x, cg = c.y, cb = c.z;
    if (material < 8u) {
      cr *= V.P.palette[material][0];
      cg *= V.P.palette[material][1];
      cb *= V.P.palette[material][2];
    }
    cr *= V.P.albedo_scale;
    cg *= V.P.albedo_scale;
    cb *= V.P.albedo_scale;
    float4 cc = recs[gslot].c;
    cc.x = cr;
    cc.y = cg;
    cc.z = cb;
    recs[gslot].c = cc;
    mx = fmaxf(fmaxf(cr, cg), fmaxf(cb, 0.0f));
  }
  if (mx > 0.0f) atomicMax(&s_max, __float_as_uint(mx));
  __syncthreads();
  if (t == 0 && s_max) atomicMax(&view_maxrad[v], s_max);
}

}  // namespace

cudaError_t launch_bshade(const BatchView* views, const BatchScene* scenes, const uint32_t* block_view,
                          uint32_t max_blocks, const uint32_t* list, const uint32_t* view_shade, SplatRec* recs,
                          uint32_t* view_maxrad, int variant, cudaStream_t s) {
  if (max_blocks == 0) return cudaSuccess;
  switch (kTuneMinBlocks[2][variant]) {
    case 4:
      bshade_kernel<4><<<2 * max_blocks, kThreads, 0, s>>>(views, scenes, block_view, list, view_shade, recs,
                                                           view_maxrad);
      break;
    case 3:
      bshade_kernel<3><<<2 * max_blocks, kThreads, 0, s>>>(views, scenes, block_view, list, view_shade, recs,
                                                           view_maxrad);
      break;
    case 5:
      bshade_kernel<5><<<2 * max_blocks, kThreads, 0, s>>>(views, scenes, block_view, list, view_shade, recs,
                                                           view_maxrad);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_shade(const ShadeParams& SH, const sl_gaussian* gs, const sl_node* nodes, const sl_vgrid* vgrid,
                         const sl_part* parts, const sl_material* mats, const float* tree, const float* lamp_T,
                         const float4* env_T, const uint32_t* order, float4* colour, uint32_t count, cudaStream_t s) {
  if (!count) return cudaSuccess;
  shade_kernel<<<(count + kThreads - 1) / kThreads, kThreads, 0, s>>>(SH, gs, nodes, vgrid, parts, mats, tree, lamp_T,
                                                                      env_T, order, colour, count);
  return cudaGetLastError();
}

}  // namespace sl
