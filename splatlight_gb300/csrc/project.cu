// Projection: one thread per slot turns a 3D Gaussian into a screen-space splat record, a 16-bit back-to-front
// depth key and a tile rectangle (shaders/project.wgsl:84-370, plain path).  A coalesced streaming kernel: each
// thread reads its 64-byte record as four 16-byte vector loads and writes a 48-byte splat, a 2-byte key and an
// 8-byte tile rectangle; the digit histograms the radix sort needs are reduced in shared memory and added once per
// block.
//
// Compiled with --fmad=false: every a*b+c rounds twice, as in the CPU restatement, so keys, tile rectangles and the
// per-fragment keep bound are bit-identical to it.  Sums evaluate left to right, matrix-vector products as
// col0*v.x + col1*v.y + col2*v.z, normalize(v) = v / sqrt(dot(v, v)), and ln comes from sl_detmath.h.
#include <cuda_fp16.h>

#include "sl_detmath.h"
#include "sl_internal.h"

namespace sl {
namespace {

struct V3 {
  float x, y, z;
};
struct M3 {
  V3 c[3];
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 scale3(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 mulv(const M3& m, V3 v) {
  return v3(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z, m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
            m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z);
}
__device__ __forceinline__ M3 mulm(const M3& a, const M3& b) {
  M3 r;
  r.c[0] = mulv(a, b.c[0]);
  r.c[1] = mulv(a, b.c[1]);
  r.c[2] = mulv(a, b.c[2]);
  return r;
}
// quat_to_mat, shaders/common.wgsl:83-89
__device__ __forceinline__ M3 quat_mat(float x, float y, float z, float w) {
  M3 m;
  m.c[0] = v3(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + w * z), 2.0f * (x * z - w * y));
  m.c[1] = v3(2.0f * (x * y - w * z), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + w * x));
  m.c[2] = v3(2.0f * (x * z + w * y), 2.0f * (y * z - w * x), 1.0f - 2.0f * (x * x + y * y));
  return m;
}
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

constexpr int kThreads = 256;

// A block's tallies of its slots' keys (in: the thread holds a slot): valid keys into the two depth-digit histograms
// (spread: shared atomics rarely collide), invalid keys (all digits 0xFF) and the visible count and radiance maximum
// one warp-aggregated add each, instead of 256 threads' atomics on one word.
__device__ __forceinline__ void block_tally(bool in, uint32_t key, float maxrad, uint32_t* h_lo, uint32_t* h_hi,
                                            uint32_t* s_visible, uint32_t* s_invalid, uint32_t* s_maxrad) {
  const bool vis = in && key != kInvalidKey16;
  if (vis) {
    atomicAdd(&h_lo[key & 0xffu], 1u);
    atomicAdd(&h_hi[key >> 8], 1u);
  }
  const uint32_t vmask = __ballot_sync(0xffffffffu, vis), imask = __ballot_sync(0xffffffffu, in && !vis);
  const uint32_t wmax = __reduce_max_sync(0xffffffffu, vis ? __float_as_uint(maxrad) : 0u);
  if ((threadIdx.x & 31u) == 0u) {
    if (vmask) atomicAdd(s_visible, (uint32_t)__popc(vmask));
    if (imask) atomicAdd(s_invalid, (uint32_t)__popc(imask));
    if (wmax) atomicMax(s_maxrad, wmax);
  }
}

// One slot i of project.wgsl main (:84-370, plain path): key (kInvalidKey16 when culled), tile rectangle and the
// largest radiance component; the splat record goes to *rec_out.  colour / lo_b may be null (radiance 0, filled in
// later by the batched shading pass).
__device__ __forceinline__ void project_slot(const ProjectParams& P, uint32_t i, const float4* __restrict__ gaussians,
                                             const float4* __restrict__ emitters, const float4* __restrict__ colour,
                                             const float4* __restrict__ lo_b, SplatRec* rec_out, uint32_t& key_out,
                                             ushort4& rect_out, float& maxrad_out,
                                             const LodDraw* lod = nullptr) {
  uint32_t key = kInvalidKey16;
  ushort4 rect = make_ushort4(1, 1, 0, 0);
  float maxrad = 0.0f;
  bool live = i < P.n_slots && i != P.count && i <= P.count + P.n_emit;
  // screen-space LOD (project.wgsl:90-109): slots from node_base are the tree's internal nodes; only the leaves and
  // nodes of the cut (flag 2) are drawn, and the emitter slots past the frame's emitters stay empty
  uint32_t node = 0xFFFFFFFFu;
  if (lod != nullptr && P.lod_on) {
    if (i >= P.node_base && i < P.n_slots) {
      node = i - P.node_base;
      live = node < P.n_int && lod->flags[P.count + node] == 2u;
    } else if (live && i < P.count && lod->flags[i] != 2u) {
      live = false;
    }
  }

  float4 g0, g1, g2, g3;
  uint32_t material = kEmitterMaterial;
  float keep = 1.0f;
  V3 mu;
  uint32_t part = 0xFFFFFFFFu;  // the Gaussian's part (its rotation is composed only for slots past the depth test)
  V3 vel = v3(0.0f, 0.0f, 0.0f);  // motion blur: world-space displacement over the exposure (project.wgsl:138-146)
  if (live) {
    const float4* src = node != 0xFFFFFFFFu ? reinterpret_cast<const float4*>(lod->nodes) + 4u * node
                        : (i > P.count) ? emitters + 4u * (i - P.count - 1u) : gaussians + 4u * i;
    g0 = __ldg(src + 0);
    g1 = __ldg(src + 1);
    g2 = __ldg(src + 2);
    g3 = __ldg(src + 3);
    if (i > P.count && node == 0xFFFFFFFFu) {  // project.wgsl:123-127
      mu = v3(g0.x, g0.y, g0.z);
    } else {  // :232-251
      part = __float_as_uint(g2.w) & 0xffffu;
      part = part > kMaxParts - 1u ? kMaxParts - 1u : part;
      const PartXf& p = P.parts[part];
      keep = p.keep;
      if ((p.flags & kPartHidden) != 0u || keep <= 0.0f) {
        live = false;
      } else {
        const float* a = p.xf;
        mu = v3(a[0] * g0.x + a[1] * g0.y + a[2] * g0.z + a[3] * 1.0f,
                a[4] * g0.x + a[5] * g0.y + a[6] * g0.z + a[7] * 1.0f,
                a[8] * g0.x + a[9] * g0.y + a[10] * g0.z + a[11] * 1.0f);
        material = p.material;
        if (P.shutter > 0.0f && (p.flags & 2u) != 0u) {
          const float* b = p.xf_prev;
          const V3 prev = v3(b[0] * g0.x + b[1] * g0.y + b[2] * g0.z + b[3] * 1.0f,
                             b[4] * g0.x + b[5] * g0.y + b[6] * g0.z + b[7] * 1.0f,
                             b[8] * g0.x + b[9] * g0.y + b[10] * g0.z + b[11] * 1.0f);
          vel = v3(P.shutter * (mu.x - prev.x), P.shutter * (mu.y - prev.y), P.shutter * (mu.z - prev.z));
          mu = v3(mu.x - 0.5f * vel.x, mu.y - 0.5f * vel.y, mu.z - 0.5f * vel.z);
        }
      }
    }
  }

  if (live) {
    const float* V = P.view;
    V3 tv = v3(V[0] * mu.x + V[4] * mu.y + V[8] * mu.z + V[12] * 1.0f,
               V[1] * mu.x + V[5] * mu.y + V[9] * mu.z + V[13] * 1.0f,
               V[2] * mu.x + V[6] * mu.y + V[10] * mu.z + V[14] * 1.0f);
    float depth = -tv.z;
    live = !(depth < P.near_plane || depth > P.far_plane);
    if (live) {
      M3 rot;
      if (part == 0xFFFFFFFFu) {
        rot = quat_mat(g1.x, g1.y, g1.z, g1.w);
      } else {
        const float* a = P.parts[part].xf;
        M3 R;
        R.c[0] = v3(a[0], a[4], a[8]);
        R.c[1] = v3(a[1], a[5], a[9]);
        R.c[2] = v3(a[2], a[6], a[10]);
        rot = mulm(R, quat_mat(g1.x, g1.y, g1.z, g1.w));
      }
      M3 W;
      W.c[0] = v3(V[0], V[1], V[2]);
      W.c[1] = v3(V[4], V[5], V[6]);
      W.c[2] = v3(V[8], V[9], V[10]);
      M3 wr = mulm(W, rot);
      const float sx = g2.x, sy = g2.y, sz = g2.z;
      V3 s2 = v3(sx * sx, sy * sy, sz * sz);
      V3 m0 = scale3(wr.c[0], sx), m1 = scale3(wr.c[1], sy), m2 = scale3(wr.c[2], sz);
      // cov[r][c] = sum_k m_k[r] m_k[c]
      const float mk0[3] = {m0.x, m0.y, m0.z}, mk1[3] = {m1.x, m1.y, m1.z}, mk2[3] = {m2.x, m2.y, m2.z};
      float cv[3][3];
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) cv[r][c] = mk0[r] * mk0[c] + mk1[r] * mk1[c] + mk2[r] * mk2[c];
      // the sharp covariance, kept for the coverage cap; blurred: + (W vel)(W vel)^T / 12 (project.wgsl:208-210)
      const bool blurred = vel.x != 0.0f || vel.y != 0.0f || vel.z != 0.0f;
      M3 cov_s;
      cov_s.c[0] = v3(cv[0][0], cv[1][0], cv[2][0]);
      cov_s.c[1] = v3(cv[0][1], cv[1][1], cv[2][1]);
      cov_s.c[2] = v3(cv[0][2], cv[1][2], cv[2][2]);
      if (blurred) {
        const V3 wv = mulv(W, vel);
        const float w3[3] = {wv.x, wv.y, wv.z};
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
          for (int c = 0; c < 3; c++) cv[r][c] = cv[r][c] + (w3[r] * w3[c]) * (1.0f / 12.0f);
      }
      M3 cov;
      cov.c[0] = v3(cv[0][0], cv[1][0], cv[2][0]);
      cov.c[1] = v3(cv[0][1], cv[1][1], cv[2][1]);
      cov.c[2] = v3(cv[0][2], cv[1][2], cv[2][2]);

      const float fx = P.focal[0], fy = P.focal[1];
      float iz = 1.0f / depth;
      float px = fx * tv.x * iz;
      float py = fy * tv.y * iz;
      float limx = 1.3f * P.viewport[0] * 0.5f;
      float limy = 1.3f * P.viewport[1] * 0.5f;
      float cxv = clampf(tv.x * iz, -limx / fx, limx / fx) * depth;
      float cyv = clampf(tv.y * iz, -limy / fy, limy / fy) * depth;
      V3 j0 = v3(fx * iz, 0.0f, fx * cxv * iz * iz);
      V3 j1 = v3(0.0f, fy * iz, fy * cyv * iz * iz);
      V3 cj0 = mulv(cov, j0), cj1 = mulv(cov, j1);
      float a = dot3(j0, cj0);
      float b = dot3(j0, cj1);
      float c = dot3(j1, cj1);
      float det0 = a * c - b * b;
      a += P.lowpass_px2;
      c += P.lowpass_px2;
      float det = a * c - b * b;
      live = det > 0.0f;
      float tau0 = 0.0f, qcut = 0.0f, r = 0.0f;
      const float kTauMin = -sl_logf(1.0f - 1.0f / 255.0f);
      if (live) {
        float dlen = sqrtf(dot3(tv, tv));
        V3 d = v3(tv.x / dlen, tv.y / dlen, tv.z / dlen);
        V3 dl = v3(dot3(wr.c[0], d), dot3(wr.c[1], d), dot3(wr.c[2], d));
        V3 is2 = v3(1.0f / s2.x, 1.0f / s2.y, 1.0f / s2.z);
        float q = dot3(v3(dl.x * dl.x, dl.y * dl.y, dl.z * dl.z), is2);
        const float q_s = q;
        float kappa = __uint_as_float(__float_as_uint(g0.w));
        if (blurred) {
          // Sigma' = Sigma + v v^T / 12 in the Gaussian's frame: Sherman-Morrison for the view ray's q, the
          // determinant lemma for the density that keeps the mass (project.wgsl:242-250)
          const V3 vl = v3(dot3(rot.c[0], vel), dot3(rot.c[1], vel), dot3(rot.c[2], vel));
          const float mv2 = dot3(v3(vl.x * vl.x, vl.y * vl.y, vl.z * vl.z), is2);
          const float dv = dot3(v3(dl.x * vl.x, dl.y * vl.y, dl.z * vl.z), is2);
          q -= dv * dv / (12.0f + mv2);
          kappa /= sqrtf(1.0f + mv2 / 12.0f);
        }
        const float kTwoPi = 6.283185307f;
        tau0 = kappa * sqrtf(kTwoPi / q) * sqrtf(fmaxf(det0, 0.0f) / det);
        if (blurred && P.blur_cov) {
          // coverage cap: a box shutter averages coverage, so the smear's peak alpha is capped at the sharp splat's
          // (same Jacobian) x sqrt(det_s / det) (project.wgsl:251-268)
          const V3 cs0 = mulv(cov_s, j0), cs1 = mulv(cov_s, j1);
          const float a_s = dot3(j0, cs0) + P.lowpass_px2;
          const float b_s = dot3(j0, cs1);
          const float c_s = dot3(j1, cs1) + P.lowpass_px2;
          const float det0_s = (a_s - P.lowpass_px2) * (c_s - P.lowpass_px2) - b_s * b_s;
          const float det_s = a_s * c_s - b_s * b_s;
          const float tau_s = __uint_as_float(__float_as_uint(g0.w)) * sqrtf(kTwoPi / q_s) *
                              sqrtf(fmaxf(det0_s, 0.0f) / det_s);
          const float ap = (1.0f - sl_expf(-tau_s)) * sqrtf(det_s / det);
          tau0 = fminf(tau0, -sl_logf(fmaxf(1.0f - ap, 1e-6f)));
        }
        tau0 *= keep;
        live = !(tau0 <= kTauMin);
      }
      if (live) {
        qcut = 2.0f * sl_logf(tau0 / kTauMin);
        r = sqrtf(qcut);
        float mid = 0.5f * (a + c);
        float disc = sqrtf(0.25f * (a - c) * (a - c) + b * b);
        float l0 = mid + disc;
        float l1 = fmaxf(det / l0, 1e-6f);
        float e0x = 1.0f, e0y = 0.0f;
        if (a >= c) {
          if (fabsf(b) > 0.0f || l0 > a) {
            float vx = l0 - c, vy = b, vl = sqrtf(vx * vx + vy * vy);
            e0x = vx / vl;
            e0y = vy / vl;
          }
        } else {
          float vx = b, vy = l0 - a, vl = sqrtf(vx * vx + vy * vy);
          e0x = vx / vl;
          e0y = vy / vl;
        }
        float e1x = -e0y, e1y = e0x;
        float sl0 = sqrtf(l0), sl1 = sqrtf(l1);
        float tnx = 2.0f / P.viewport[0], tny = 2.0f / P.viewport[1];
        float ax0 = e0x * sl0 * r * tnx, ay0 = e0y * sl0 * r * tny;
        float ax1 = e1x * sl1 * r * tnx, ay1 = e1y * sl1 * r * tny;
        float ccx = px * tnx, ccy = py * tny;
        float extx = fabsf(ax0) + fabsf(ax1), exty = fabsf(ay0) + fabsf(ay1);
        live = !(sl0 * r < 0.1f) && !(fabsf(ccx) - extx > 1.0f || fabsf(ccy) - exty > 1.0f);
        if (live) {
          // radiance (project.wgsl:317-350)
          float cr = g3.x, cg = g3.y, cb = g3.z;
          if (material == kEmitterMaterial) {
          } else if (P.view_mode == 3u) {
            if (node != 0xFFFFFFFFu) {  // a drawn node's lit colour, bounce included (lod_colour)
              const float4 nc = lod->colour[node];
              cr = nc.x;
              cg = nc.y;
              cb = nc.z;
            } else {
              float4 cl = colour ? colour[i] : make_float4(0.f, 0.f, 0.f, 0.f);
              float4 bo = lo_b ? lo_b[3u * i] : make_float4(0.f, 0.f, 0.f, 0.f);
              cr = cl.x + P.bounce_gain * bo.x;
              cg = cl.y + P.bounce_gain * bo.y;
              cb = cl.z + P.bounce_gain * bo.z;
            }
            if (material < 8u) {
              cr *= P.palette[material][0];
              cg *= P.palette[material][1];
              cb *= P.palette[material][2];
            }
          } else if (material < 8u && P.palette[material][3] > 0.5f) {
            cr = P.palette[material][0];
            cg = P.palette[material][1];
            cb = P.palette[material][2];
          }
          if (material != kEmitterMaterial) {
            cr *= P.albedo_scale;
            cg *= P.albedo_scale;
            cb *= P.albedo_scale;
          }
          // 16-bit log-depth key (project.wgsl:363-369)
          float lnr = sl_logf(P.far_plane / P.near_plane);
          float tt = clampf(sl_logf(depth / P.near_plane) / lnr, 0.0f, 1.0f);
          uint32_t k = 65535u - (uint32_t)(tt * 65535.0f + 0.5f);
          key = k > 0xfffeu ? 0xfffeu : k;
          if (P.view_mode == 1u) cr = cg = cb = 1.0f - tt;

          const float Wf = P.viewport[0], Hf = P.viewport[1];
          float cx = px + 0.5f * Wf;
          float cy = 0.5f * Hf - py;
          float a0x = e0x * sl0 * r, a0y = e0y * sl0 * r;
          float a1x = e1x * sl1 * r, a1y = e1y * sl1 * r;
          float n0 = fmaxf(a0x * a0x + a0y * a0y, 1e-12f);
          float n1 = fmaxf(a1x * a1x + a1y * a1y, 1e-12f);
          // candidate pixels: ellipse bounding box plus one pixel; tiles it overlaps
          float hx = r * sqrtf(a) + 1.0f, hy = r * sqrtf(c) + 1.0f;
          SplatRec rec;
          rec.a = make_float4(cx, cy, a0x * r / n0, -(a0y * r / n0));
          // half extents of that box, rounded up to half precision: the compositor's conservative block culling
          __half2 hxy = __halves2half2(__float2half_ru(hx), __float2half_ru(hy));
          rec.b = make_float4(a1x * r / n1, -(a1y * r / n1), *reinterpret_cast<float*>(&hxy), qcut);
          rec.c = make_float4(cr, cg, cb, tau0);
          *rec_out = rec;
          maxrad = fmaxf(fmaxf(cr, cg), fmaxf(cb, 0.0f));
          float xl = fmaxf(cx - hx - 0.5f, -1.0f), xh = fminf(cx + hx - 0.5f, Wf);
          float yl = fmaxf(cy - hy - 0.5f, -1.0f), yh = fminf(cy + hy - 0.5f, Hf);
          int ix0 = (int)ceilf(xl), ix1 = (int)floorf(xh);
          int iy0 = (int)ceilf(yl), iy1 = (int)floorf(yh);
          ix0 = ix0 < 0 ? 0 : ix0;
          iy0 = iy0 < 0 ? 0 : iy0;
          ix1 = ix1 > (int)Wf - 1 ? (int)Wf - 1 : ix1;
          iy1 = iy1 > (int)Hf - 1 ? (int)Hf - 1 : iy1;
          if (ix0 <= ix1 && iy0 <= iy1)
            rect = make_ushort4((unsigned short)(ix0 / (int)P.tile_w), (unsigned short)(iy0 / (int)P.tile_h),
                                (unsigned short)(ix1 / (int)P.tile_w), (unsigned short)(iy1 / (int)P.tile_h));
        }
      }
    }
  }

  key_out = key;
  rect_out = rect;
  maxrad_out = maxrad;
}

__global__ void __launch_bounds__(kThreads) project_kernel(const __grid_constant__ ProjectParams P,
                                                           const float4* __restrict__ gaussians,
                                                           const float4* __restrict__ emitters,
                                                           const float4* __restrict__ colour,
                                                           const float4* __restrict__ lo_b, uint16_t* __restrict__ key16,
                                                           SplatRec* __restrict__ recs, ushort4* __restrict__ rects,
                                                           uint32_t* __restrict__ digit_hist, FrameCounters* ctr,
                                                           const LodDraw lod) {
  __shared__ uint32_t h_lo[256], h_hi[256];
  __shared__ uint32_t s_visible, s_invalid, s_maxrad;
  const int t = threadIdx.x;
  h_lo[t] = 0u;
  h_hi[t] = 0u;
  if (t == 0) {
    s_visible = 0u;
    s_invalid = 0u;
    s_maxrad = 0u;
  }
  __syncthreads();

  const uint32_t i = blockIdx.x * kThreads + t;
  uint32_t key;
  ushort4 rect;
  float maxrad;
  project_slot(P, i, gaussians, emitters, colour, lo_b, recs + i, key, rect, maxrad, &lod);
  const bool in = i < P.n_slots;
  if (in) {
    key16[i] = (uint16_t)key;
    rects[i] = rect;
  }
  block_tally(in, key, maxrad, h_lo, h_hi, &s_visible, &s_invalid, &s_maxrad);
  __syncthreads();
  const uint32_t lo = h_lo[t] + (t == 255 ? s_invalid : 0u), hi = h_hi[t] + (t == 255 ? s_invalid : 0u);
  if (lo) atomicAdd(&digit_hist[t], lo);
  if (hi) atomicAdd(&digit_hist[256 + t], hi);
  if (t == 0) {
    if (s_visible) atomicAdd(&ctr->visible, s_visible);
    if (s_maxrad) atomicMax(&ctr->max_rad_bits, s_maxrad);
  }
}

// Batched: one block of 256 slots of one view; the view comes from block_view (kNoView: padding past the batch).
// Keys carry the view above the 16 depth bits, so one stable sort orders every view's slots exactly as the per-view
// sort does; lit radiance is filled in by the batched shading pass.
template <int MinB>
__global__ void __launch_bounds__(kThreads, MinB) bproject_kernel(const BatchView* __restrict__ views,
                                                            const uint32_t* __restrict__ block_view,
                                                            uint32_t* __restrict__ keys32, SplatRec* __restrict__ recs,
                                                            ushort4* __restrict__ rects, uint32_t* __restrict__ digit_hist,
                                                            uint32_t* __restrict__ view_maxrad,
                                                            uint32_t* __restrict__ view_visible,
                                                            uint32_t* __restrict__ block_valid) {
  __shared__ ProjectParams sP;
  __shared__ uint32_t h[2][256];
  __shared__ uint32_t s_visible, s_invalid, s_maxrad;
  const uint32_t v = block_view[blockIdx.x];
  if (v == kNoView) {
    if (threadIdx.x == 0) block_valid[blockIdx.x] = 0u;
    return;
  }
  const int t = threadIdx.x;
  const BatchView& V = views[v];
  {  // the frame's fields and the scene's parts only (every Gaussian's part is below part_count: checked at creation)
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&V.P);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&sP);
    const uint32_t np = V.P.part_count < kMaxParts ? V.P.part_count : kMaxParts;
    const uint32_t words = (uint32_t)((offsetof(ProjectParams, parts) + np * sizeof(PartXf)) / 4);
    for (uint32_t k = t; k < words; k += kThreads) dst[k] = src[k];
  }
  h[0][t] = 0u;
  h[1][t] = 0u;
  if (t == 0) {
    s_visible = 0u;
    s_invalid = 0u;
    s_maxrad = 0u;
  }
  __syncthreads();
  const uint32_t i = (blockIdx.x - V.block_first) * kThreads + t;
  const uint32_t gslot = V.slot_base + i;
  uint32_t key;
  ushort4 rect;
  float maxrad;
  project_slot(sP, i, V.gaussians, V.emitters, V.colour, V.lo_b, recs + gslot, key, rect, maxrad);
  const uint32_t key32 = (v << 16) | key;
  keys32[gslot] = key32;
  rects[gslot] = rect;
  block_tally(true, key, maxrad, h[0], h[1], &s_visible, &s_invalid, &s_maxrad);
  __syncthreads();
  // the digits of the valid keys only: the depth sort runs over the compacted valid keys (bcompact)
  if (h[0][t]) atomicAdd(&digit_hist[t], h[0][t]);
  if (h[1][t]) atomicAdd(&digit_hist[256 + t], h[1][t]);
  if (t == 0) {
    block_valid[blockIdx.x] = s_visible;
    if (s_visible) atomicAdd(&digit_hist[512 + v], s_visible);  // the view byte
    if (s_visible) atomicAdd(&view_visible[v], s_visible);
    if (s_maxrad) atomicMax(&view_maxrad[v], s_maxrad);
  }
}

}  // namespace

cudaError_t launch_bproject(const BatchView* views, const uint32_t* block_view, uint32_t max_blocks, uint32_t* keys32,
                            SplatRec* recs, ushort4* rects, uint32_t* digit_hist, uint32_t* view_maxrad,
                            uint32_t* view_visible, uint32_t* block_valid, int variant, cudaStream_t s) {
  if (max_blocks == 0) return cudaSuccess;
  switch (kTuneMinBlocks[0][variant]) {
    case 4:
      bproject_kernel<4><<<max_blocks, kThreads, 0, s>>>(views, block_view, keys32, recs, rects, digit_hist,
                                                         view_maxrad, view_visible, block_valid);
      break;
    case 3:
      bproject_kernel<3><<<max_blocks, kThreads, 0, s>>>(views, block_view, keys32, recs, rects, digit_hist,
                                                         view_maxrad, view_visible, block_valid);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_project(const ProjectParams& P, const sl_gaussian* gaussians, const sl_gaussian* emitters,
                           const float4* colour, const float4* lo_b, uint16_t* key16, SplatRec* recs,
                           ushort4* rects, uint32_t* digit_hist, FrameCounters* ctr, cudaStream_t s,
                           LodDraw lod) {
  if (P.n_slots == 0) return cudaSuccess;
  if (P.lod_on && (lod.flags == nullptr || lod.nodes == nullptr || lod.colour == nullptr)) return cudaErrorInvalidValue;
  uint32_t blocks = (P.n_slots + kThreads - 1) / kThreads;
  project_kernel<<<blocks, kThreads, 0, s>>>(P, reinterpret_cast<const float4*>(gaussians),
                                             reinterpret_cast<const float4*>(emitters), colour, lo_b, key16, recs,
                                             rects, digit_hist, ctr, lod);
  return cudaGetLastError();
}

}  // namespace sl
