// The differentiable splat path (inverse rendering): a forward pass over free parameters -- means, log-scales,
// quaternions, opacity logits, albedo, roughness and the emissive lights' intensities -- through the same projection
// (view-space covariance, 2D conic with the low-pass dilation, peak optical depth tau0 = softplus(logit) sqrt(det0 /
// det) / (s0 sqrt(q_d)), the model of shaders/project.wgsl:234-261), the product's per-Gaussian lighting by emissive
// Gaussian lights over the emitter tree's light cut (sl_dshade.cuh; emissive.wgsl shade_leaf), the same 16-bit depth
// keys, stable sort and tile lists, and front-to-back compositing; then hand-written gradients of an L2 image loss.
//
// Compositing for the differentiable path: alpha = min(1 - exp(-tau0 e^{-q/2}), 0.99), fragments with optical depth
// below 1e-6 skipped, a pixel stops before the fragment that would take its transmittance below 1e-4.  The forward
// stores per pixel only the final transmittance and the number of list entries it visited; the backward walks each
// tile list back to front, recovering T_f = T_{f+1} / (1 - alpha_f) and the colour behind each fragment, so no
// per-pixel fragment list is ever stored.  Per-splat gradients are reduced across the warp before one atomic add.
// The lighting's part of the chain rule is the Jacobian of the radiance with respect to the Gaussian's parameters,
// evaluated in forward mode (dual numbers through the lighting code itself, one parameter direction per pass), and
// with respect to the light intensities through the emitter tree's derivative table.
#include <cuda_fp16.h>

#include "sl_detmath.h"
#include "sl_diff.h"
#include "sl_internal.h"

namespace sl {
namespace {

constexpr int kThreads = 256;

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }

__device__ __forceinline__ void quat_rot(const float* q4, F3 R[3], float qh[4], float& qn) {
  const float n = sqrtf(q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
  qn = n;
  const float x = q4[0] / n, y = q4[1] / n, z = q4[2] / n, w = q4[3] / n;
  qh[0] = x;
  qh[1] = y;
  qh[2] = z;
  qh[3] = w;
  R[0] = f3(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + w * z), 2.0f * (x * z - w * y));
  R[1] = f3(2.0f * (x * y - w * z), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + w * x));
  R[2] = f3(2.0f * (x * z + w * y), 2.0f * (y * z - w * x), 1.0f - 2.0f * (x * x + y * y));
}

__device__ __forceinline__ float softplus(float x) { return x > 20.0f ? x : log1pf(expf(x)); }
__device__ __forceinline__ float sigmoid(float x) { return 1.0f / (1.0f + expf(-x)); }

// Everything the forward derives for one Gaussian (recomputed by the backward).
struct Geo {
  bool live;
  F3 t;            // view-space mean
  float depth, iz;
  F3 wr[3];        // rotation axes in view space
  float s[3];
  F3 j0, j1;
  bool clx, cly;   // Jacobian clamped in x / y
  float cxv, cyv;
  float cv[3][3];  // view-space covariance
  float a, b, c, det0, ap, cp, det;
  F3 d;            // unit view direction to the mean
  float tlen, dl[3], qd;
  float sp, tau0;
  float px, py;
};

__device__ __forceinline__ void geometry(const DiffCamera& K, const float* mu, const float* ls, const F3 R[3],
                                         float logit, Geo& g) {
  const float* V = K.view;
  g.t = f3(V[0] * mu[0] + V[4] * mu[1] + V[8] * mu[2] + V[12], V[1] * mu[0] + V[5] * mu[1] + V[9] * mu[2] + V[13],
           V[2] * mu[0] + V[6] * mu[1] + V[10] * mu[2] + V[14]);
  g.depth = -g.t.z;
  g.live = !(g.depth < K.near_plane || g.depth > K.far_plane);
  if (!g.live) return;
  const F3 W0 = f3(V[0], V[1], V[2]), W1 = f3(V[4], V[5], V[6]), W2 = f3(V[8], V[9], V[10]);
  for (int k = 0; k < 3; k++) {
    g.wr[k] = W0 * R[k].x + W1 * R[k].y + W2 * R[k].z;
    g.s[k] = expf(ls[k]);
  }
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      const float* a0 = &g.wr[0].x;
      const float* a1 = &g.wr[1].x;
      const float* a2 = &g.wr[2].x;
      g.cv[r][c] = g.s[0] * g.s[0] * a0[r] * a0[c] + g.s[1] * g.s[1] * a1[r] * a1[c] + g.s[2] * g.s[2] * a2[r] * a2[c];
    }
  const float fx = K.focal[0], fy = K.focal[1];
  g.iz = 1.0f / g.depth;
  g.px = fx * g.t.x * g.iz;
  g.py = fy * g.t.y * g.iz;
  const float limx = 1.3f * K.viewport[0] * 0.5f / fx, limy = 1.3f * K.viewport[1] * 0.5f / fy;
  const float ux = g.t.x * g.iz, uy = g.t.y * g.iz;
  g.clx = ux < -limx || ux > limx;
  g.cly = uy < -limy || uy > limy;
  g.cxv = fminf(fmaxf(ux, -limx), limx) * g.depth;
  g.cyv = fminf(fmaxf(uy, -limy), limy) * g.depth;
  g.j0 = f3(fx * g.iz, 0.0f, fx * g.cxv * g.iz * g.iz);
  g.j1 = f3(0.0f, fy * g.iz, fy * g.cyv * g.iz * g.iz);
  F3 cj0 = f3(dot(f3(g.cv[0][0], g.cv[0][1], g.cv[0][2]), g.j0), dot(f3(g.cv[1][0], g.cv[1][1], g.cv[1][2]), g.j0),
              dot(f3(g.cv[2][0], g.cv[2][1], g.cv[2][2]), g.j0));
  F3 cj1 = f3(dot(f3(g.cv[0][0], g.cv[0][1], g.cv[0][2]), g.j1), dot(f3(g.cv[1][0], g.cv[1][1], g.cv[1][2]), g.j1),
              dot(f3(g.cv[2][0], g.cv[2][1], g.cv[2][2]), g.j1));
  g.a = dot(g.j0, cj0);
  g.b = dot(g.j0, cj1);
  g.c = dot(g.j1, cj1);
  g.det0 = g.a * g.c - g.b * g.b;
  g.ap = g.a + K.lowpass;
  g.cp = g.c + K.lowpass;
  g.det = g.ap * g.cp - g.b * g.b;
  g.live = g.det > 0.0f && g.det0 > 0.0f;
  if (!g.live) return;
  g.tlen = sqrtf(dot(g.t, g.t));
  g.d = g.t * (1.0f / g.tlen);
  g.qd = 0.0f;
  for (int k = 0; k < 3; k++) {
    g.dl[k] = dot(g.wr[k], g.d);
    g.qd += g.dl[k] * g.dl[k] / (g.s[k] * g.s[k]);
  }
  g.sp = softplus(logit);
  g.tau0 = g.sp * sqrtf(g.det0 / g.det) / (g.s[0] * sqrtf(g.qd));
}

// Radiance of Gaussian i as the product's shading pass lights it: albedo (acc T iso_norm + ambient), acc the emitter
// light over its cut (sl_dshade.cuh).
__device__ __forceinline__ F3 lit_radiance(const DiffLights& L, const DiffParams& P, const DiffCamera& K, uint32_t i) {
  const float* m = P.means + 3 * i;
  const float* l = P.log_scales + 3 * i;
  const float* q = P.quats + 4 * i;
  const float mu[3] = {m[0], m[1], m[2]}, ls[3] = {l[0], l[1], l[2]}, q4[4] = {q[0], q[1], q[2], q[3]};
  const dsh::Recv<float, float> rv = dsh::receiver<float, float>(mu, ls, q4, P.opacity_logits[i], P.roughness[i]);
  const float iso = L.iso_norm ? L.iso_norm[i] : 1.0f, T = L.lamp_T ? L.lamp_T[i] : 1.0f;
  const dsh::V3<float> eye = dsh::v3(K.eye[0], K.eye[1], K.eye[2]);
  const dsh::V3<float> acc = dsh::emitter_light(L.tree, rv, L.vgrid ? L.vgrid + i : nullptr, L.ks, iso, eye,
                                                [](uint32_t, float, dsh::V3<float>, float) {});
  const float k = T * iso;
  const F3 alb = ld3(P.albedo + 3 * i);
  return f3(alb.x * (acc.x * k + L.ambient), alb.y * (acc.y * k + L.ambient), alb.z * (acc.z * k + L.ambient));
}

__global__ void __launch_bounds__(kThreads) dproject_kernel(const DiffCamera K, const DiffParams P, const DiffLights Lt,
                                                            uint32_t n, uint16_t* __restrict__ key16,
                                                            DiffRec* __restrict__ drec, SplatRec* __restrict__ recs,
                                                            ushort4* __restrict__ rects,
                                                            uint32_t* __restrict__ digit_hist, FrameCounters* ctr) {
  __shared__ uint32_t h_lo[256], h_hi[256];
  __shared__ uint32_t s_visible;
  const int t = threadIdx.x;
  h_lo[t] = 0u;
  h_hi[t] = 0u;
  if (t == 0) s_visible = 0u;
  __syncthreads();
  const uint32_t i = blockIdx.x * kThreads + t;
  if (i < n) {
    uint32_t key = 0xFFFFu;
    ushort4 rect = make_ushort4(1, 1, 0, 0);
    F3 R[3];
    float qh[4], qn;
    quat_rot(P.quats + 4 * i, R, qh, qn);
    Geo g;
    geometry(K, P.means + 3 * i, P.log_scales + 3 * i, R, P.opacity_logits[i], g);
    DiffRec d{};
    if (g.live && g.tau0 > kDiffTauMin) {
      const float W = K.viewport[0], H = K.viewport[1];
      d.cx = g.px + 0.5f * W;
      d.cy = 0.5f * H - g.py;
      d.A = g.cp / g.det;   // pixel (y-down) conic: q = A dx^2 + 2 B dx dy + C dy^2
      d.B = g.b / g.det;
      d.C = g.ap / g.det;
      d.tau0 = g.tau0;
      const F3 c = lit_radiance(Lt, P, K, i);
      d.r = c.x;
      d.g = c.y;
      d.bl = c.z;
      const float qcut = 2.0f * logf(g.tau0 / kDiffTauMin);
      d.hx = sqrtf(qcut * g.ap) + 1.0f;
      d.hy = sqrtf(qcut * g.cp) + 1.0f;
      // record for the shared tile binning: local frame by the Cholesky factor of the conic
      const float sa = sqrtf(d.A);
      const float g1y = sqrtf(fmaxf(d.C - d.B * d.B / d.A, 1e-30f));
      SplatRec rec;
      __half2 hxy = __halves2half2(__float2half_ru(d.hx), __float2half_ru(d.hy));
      rec.a = make_float4(d.cx, d.cy, sa, d.B / sa);
      rec.b = make_float4(0.0f, g1y, *reinterpret_cast<float*>(&hxy), qcut);
      rec.c = make_float4(c.x, c.y, c.z, g.tau0);
      recs[i] = rec;
      const float xl = fmaxf(d.cx - d.hx - 0.5f, -1.0f), xh = fminf(d.cx + d.hx - 0.5f, W);
      const float yl = fmaxf(d.cy - d.hy - 0.5f, -1.0f), yh = fminf(d.cy + d.hy - 0.5f, H);
      int ix0 = max((int)ceilf(xl), 0), ix1 = min((int)floorf(xh), (int)W - 1);
      int iy0 = max((int)ceilf(yl), 0), iy1 = min((int)floorf(yh), (int)H - 1);
      if (ix0 <= ix1 && iy0 <= iy1) {
        rect = make_ushort4((unsigned short)(ix0 / 16), (unsigned short)(iy0 / 16), (unsigned short)(ix1 / 16),
                            (unsigned short)(iy1 / 16));
        const float lnr = sl_logf(K.far_plane / K.near_plane);
        const float tt = fminf(fmaxf(sl_logf(g.depth / K.near_plane) / lnr, 0.0f), 1.0f);
        const uint32_t k = 65535u - (uint32_t)(tt * 65535.0f + 0.5f);
        key = k > 0xfffeu ? 0xfffeu : k;
      }
    }
    drec[i] = d;
    key16[i] = (uint16_t)key;
    rects[i] = rect;
    atomicAdd(&h_lo[key & 0xffu], 1u);
    atomicAdd(&h_hi[key >> 8], 1u);
    if (key != 0xFFFFu) atomicAdd(&s_visible, 1u);
  }
  __syncthreads();
  if (h_lo[t]) atomicAdd(&digit_hist[t], h_lo[t]);
  if (h_hi[t]) atomicAdd(&digit_hist[256 + t], h_hi[t]);
  if (t == 0 && s_visible) atomicAdd(&ctr->visible, s_visible);
}

// alpha of one fragment (shared by the forward and the backward so both round identically); false = skipped
__device__ __forceinline__ bool frag_alpha(const DiffRec& d, float pxc, float pyc, float& q, float& G, float& tau,
                                           float& alpha) {
  const float dx = pxc - d.cx, dy = pyc - d.cy;
  q = d.A * dx * dx + 2.0f * d.B * dx * dy + d.C * dy * dy;
  G = expf(-0.5f * q);
  tau = d.tau0 * G;
  if (!(tau >= kDiffTauMin)) return false;
  alpha = fminf(1.0f - expf(-tau), kDiffAlphaMax);
  return true;
}

__global__ void __launch_bounds__(kThreads) dcomposite_fwd_kernel(const uint2* __restrict__ ranges,
                                                                  const uint32_t* __restrict__ tile_vals,
                                                                  const DiffRec* __restrict__ drec, uint32_t width,
                                                                  uint32_t height, uint32_t tiles_x,
                                                                  float4* __restrict__ img, float* __restrict__ t_final,
                                                                  uint32_t* __restrict__ n_contrib) {
  __shared__ DiffRec buf[kThreads];
  const uint32_t tile = blockIdx.x;
  const uint32_t px = (tile % tiles_x) * 16 + (threadIdx.x & 15), py = (tile / tiles_x) * 16 + (threadIdx.x >> 4);
  const bool inside = px < width && py < height;
  const float pxc = (float)px + 0.5f, pyc = (float)py + 0.5f;
  const uint2 rg = ranges[tile];
  float T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f;
  uint32_t last = 0;
  bool done = !inside;
  const uint32_t n = rg.y - rg.x;
  for (uint32_t base = 0; base < n; base += kThreads) {
    if (__syncthreads_and(done)) break;
    const uint32_t f = base + threadIdx.x;  // front-to-back index f: entry rg.y - 1 - f
    if (f < n) buf[threadIdx.x] = drec[tile_vals[rg.y - 1u - f]];
    __syncthreads();
    const uint32_t m = min((uint32_t)kThreads, n - base);
    for (uint32_t k = 0; k < m && !done; k++) {
      float q, G, tau, alpha;
      if (!frag_alpha(buf[k], pxc, pyc, q, G, tau, alpha)) continue;
      const float tn = T * (1.0f - alpha);
      if (tn < kDiffTStop) {
        done = true;
        break;
      }
      const float w = T * alpha;
      cr += w * buf[k].r;
      cg += w * buf[k].g;
      cb += w * buf[k].bl;
      T = tn;
      last = base + k + 1u;
    }
  }
  if (inside) {
    const size_t p = (size_t)py * width + px;
    img[p] = make_float4(cr, cg, cb, 1.0f - T);
    t_final[p] = T;
    n_contrib[p] = last;
  }
}

// dL/dC = 2 (C - target) per pixel (rgb); the loss sum_p |C - target|^2 accumulated in double
__global__ void __launch_bounds__(kThreads) dloss_kernel(const float4* __restrict__ img,
                                                         const float4* __restrict__ target, uint32_t npix,
                                                         float4* __restrict__ dimg, double* loss) {
  __shared__ double red[kThreads / 32];
  const uint32_t p = blockIdx.x * kThreads + threadIdx.x;
  double l = 0.0;
  if (p < npix) {
    const float4 c = img[p], t = target[p];
    const float ex = c.x - t.x, ey = c.y - t.y, ez = c.z - t.z;
    dimg[p] = make_float4(2.0f * ex, 2.0f * ey, 2.0f * ez, 0.0f);
    l = (double)ex * ex + (double)ey * ey + (double)ez * ez;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kThreads / 32; w++) s += red[w];
    atomicAdd(loss, s);
  }
}

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kThreads) dcomposite_bwd_kernel(const uint2* __restrict__ ranges,
                                                                  const uint32_t* __restrict__ tile_vals,
                                                                  const DiffRec* __restrict__ drec, uint32_t width,
                                                                  uint32_t height, uint32_t tiles_x,
                                                                  const float4* __restrict__ dimg,
                                                                  const float* __restrict__ t_final,
                                                                  const uint32_t* __restrict__ n_contrib,
                                                                  DiffGrad2D* __restrict__ g2) {
  __shared__ DiffRec buf[kThreads];
  __shared__ uint32_t sidx[kThreads];
  const uint32_t tile = blockIdx.x;
  const uint32_t px = (tile % tiles_x) * 16 + (threadIdx.x & 15), py = (tile / tiles_x) * 16 + (threadIdx.x >> 4);
  const bool inside = px < width && py < height;
  const float pxc = (float)px + 0.5f, pyc = (float)py + 0.5f;
  const uint2 rg = ranges[tile];
  const size_t p = inside ? (size_t)py * width + px : 0;
  float T = inside ? t_final[p] : 1.0f;
  const uint32_t mine = inside ? n_contrib[p] : 0u;
  const float4 gC = inside ? dimg[p] : make_float4(0.f, 0.f, 0.f, 0.f);
  float Sr = 0.0f, Sg = 0.0f, Sb = 0.0f;  // colour behind the current fragment
  // the furthest entry any pixel of the tile visited
  uint32_t lim = mine;
  for (int o = 16; o > 0; o >>= 1) lim = max(lim, __shfl_xor_sync(0xffffffffu, lim, o));
  __shared__ uint32_t wl[kThreads / 32];
  if ((threadIdx.x & 31) == 0) wl[threadIdx.x >> 5] = lim;
  __syncthreads();
  lim = 0;
  for (int w = 0; w < kThreads / 32; w++) lim = max(lim, wl[w]);
  // back to front: front-to-back indices lim-1 .. 0, in chunks of kThreads
  for (int top = (int)lim; top > 0; top -= kThreads) {
    const int lo = max(top - kThreads, 0);
    __syncthreads();
    const int f = lo + (int)threadIdx.x;
    if (f < top) {
      const uint32_t slot = tile_vals[rg.y - 1u - (uint32_t)f];
      sidx[threadIdx.x] = slot;
      buf[threadIdx.x] = drec[slot];
    }
    __syncthreads();
    for (int f2 = top - 1; f2 >= lo; f2--) {
      const DiffRec& d = buf[f2 - lo];
      float q = 0.f, G = 0.f, tau = 0.f, alpha = 0.f;
      bool act = inside && (uint32_t)f2 < mine && frag_alpha(d, pxc, pyc, q, G, tau, alpha);
      float gcx = 0.f, gcy = 0.f, gA = 0.f, gB = 0.f, gCc = 0.f, gt = 0.f, gr = 0.f, gg = 0.f, gb = 0.f;
      if (act) {
        T = T / (1.0f - alpha);  // transmittance in front of this fragment
        const float w = T * alpha;
        gr = w * gC.x;
        gg = w * gC.y;
        gb = w * gC.z;
        const float dLda = T * ((d.r - Sr) * gC.x + (d.g - Sg) * gC.y + (d.bl - Sb) * gC.z);
        Sr = alpha * d.r + (1.0f - alpha) * Sr;
        Sg = alpha * d.g + (1.0f - alpha) * Sg;
        Sb = alpha * d.bl + (1.0f - alpha) * Sb;
        const float dLdtau = alpha < kDiffAlphaMax ? dLda * (1.0f - alpha) : 0.0f;
        gt = dLdtau * G;
        const float dLdq = -0.5f * dLdtau * tau;
        const float dx = pxc - d.cx, dy = pyc - d.cy;
        gcx = -dLdq * (2.0f * d.A * dx + 2.0f * d.B * dy);
        gcy = -dLdq * (2.0f * d.B * dx + 2.0f * d.C * dy);
        gA = dLdq * dx * dx;
        gB = dLdq * 2.0f * dx * dy;
        gCc = dLdq * dy * dy;
      }
      if (__any_sync(0xffffffffu, act)) {
        gcx = warp_sum(gcx);
        gcy = warp_sum(gcy);
        gA = warp_sum(gA);
        gB = warp_sum(gB);
        gCc = warp_sum(gCc);
        gt = warp_sum(gt);
        gr = warp_sum(gr);
        gg = warp_sum(gg);
        gb = warp_sum(gb);
        if ((threadIdx.x & 31) == 0) {
          DiffGrad2D* o = g2 + sidx[f2 - lo];
          atomicAdd(&o->cx, gcx);
          atomicAdd(&o->cy, gcy);
          atomicAdd(&o->A, gA);
          atomicAdd(&o->B, gB);
          atomicAdd(&o->C, gCc);
          atomicAdd(&o->tau0, gt);
          atomicAdd(&o->r, gr);
          atomicAdd(&o->g, gg);
          atomicAdd(&o->b, gb);
        }
      }
    }
  }
}

// Per-Gaussian chain rule from the 2D gradients to the parameters (and the lights' intensities).
// Two blocks per SM (at most 128 registers): the lighting's walk is latency-bound, and twice the resident warps
// (with some spilling) measured 13.6 ms per step against 15.6 ms at one block of 247 registers.
__global__ void __launch_bounds__(kThreads, 2) dproject_bwd_kernel(const DiffCamera K, const DiffParams P,
                                                                const DiffLights Lt, uint32_t n,
                                                                const DiffGrad2D* __restrict__ g2,
                                                                const DiffRec* __restrict__ drec, DiffGrads G) {
  __shared__ float s_lg[kMaxDiffLights];
  if (threadIdx.x < kMaxDiffLights) s_lg[threadIdx.x] = 0.0f;
  __syncthreads();
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i < n && drec[i].tau0 > 0.0f) {
    const DiffGrad2D gd = g2[i];
    F3 R[3];
    float qh[4], qn;
    quat_rot(P.quats + 4 * i, R, qh, qn);
    Geo g;
    const float logit = P.opacity_logits[i];
    geometry(K, P.means + 3 * i, P.log_scales + 3 * i, R, logit, g);
    // ---- conic and tau0 -> a, b, c (raw 2D covariance), the view direction terms, scales
    const float det = g.det, det2 = det * det;
    const float ap = g.ap, cp = g.cp, b = g.b;
    // A = cp/det, B = b/det, C = ap/det (det = ap cp - b^2)
    float dap = gd.A * (-cp * cp / det2) + gd.B * (-b * cp / det2) + gd.C * (-b * b / det2);
    float dcp = gd.A * (-b * b / det2) + gd.B * (-b * ap / det2) + gd.C * (-ap * ap / det2);
    float db = gd.A * (2.0f * b * cp / det2) + gd.B * ((det + 2.0f * b * b) / det2) + gd.C * (2.0f * b * ap / det2);
    // tau0 = sp sqrt(det0/det) / (s0 sqrt(qd))
    const float tau0 = g.tau0, gt = gd.tau0;
    const float ddet0 = gt * tau0 / (2.0f * g.det0);
    const float ddet = -gt * tau0 / (2.0f * det);
    const float dqd = -gt * tau0 / (2.0f * g.qd);
    float ds[3] = {-gt * tau0 / g.s[0], 0.0f, 0.0f};
    const float dlogit = gt * tau0 * sigmoid(logit) / g.sp;
    // det0 = a c - b^2, det = ap cp - b^2
    float da = ddet0 * g.c + ddet * cp + dap;
    float dc = ddet0 * g.a + ddet * ap + dcp;
    db += ddet0 * (-2.0f * b) + ddet * (-2.0f * b);
    // ---- a, b, c -> covariance and Jacobian
    float Gm[3][3];
    const float j0[3] = {g.j0.x, g.j0.y, g.j0.z}, j1[3] = {g.j1.x, g.j1.y, g.j1.z};
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) Gm[r][c] = da * j0[r] * j0[c] + db * j0[r] * j1[c] + dc * j1[r] * j1[c];
    float cj0[3], cj1[3];
    for (int r = 0; r < 3; r++) {
      cj0[r] = g.cv[r][0] * j0[0] + g.cv[r][1] * j0[1] + g.cv[r][2] * j0[2];
      cj1[r] = g.cv[r][0] * j1[0] + g.cv[r][1] * j1[1] + g.cv[r][2] * j1[2];
    }
    F3 dj0 = f3(2.0f * da * cj0[0] + db * cj1[0], 2.0f * da * cj0[1] + db * cj1[1], 2.0f * da * cj0[2] + db * cj1[2]);
    F3 dj1 = f3(db * cj0[0] + 2.0f * dc * cj1[0], db * cj0[1] + 2.0f * dc * cj1[1], db * cj0[2] + 2.0f * dc * cj1[2]);
    // covariance = sum_k s_k^2 wr_k wr_k^T
    F3 dwr[3];
    for (int k = 0; k < 3; k++) {
      const float w[3] = {g.wr[k].x, g.wr[k].y, g.wr[k].z};
      float v[3];
      for (int r = 0; r < 3; r++) v[r] = (Gm[r][0] + Gm[0][r]) * w[0] + (Gm[r][1] + Gm[1][r]) * w[1] + (Gm[r][2] + Gm[2][r]) * w[2];
      dwr[k] = f3(v[0], v[1], v[2]) * (g.s[k] * g.s[k]);
      float wGw = 0.0f;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) wGw += w[r] * Gm[r][c] * w[c];
      ds[k] += 2.0f * g.s[k] * wGw;
    }
    // qd = sum_k dl_k^2 / s_k^2, dl_k = wr_k . d
    F3 dd = f3(0.0f, 0.0f, 0.0f);
    for (int k = 0; k < 3; k++) {
      const float e = 2.0f * g.dl[k] / (g.s[k] * g.s[k]) * dqd;
      dwr[k] = dwr[k] + g.d * e;
      dd = dd + g.wr[k] * e;
      ds[k] += -2.0f * g.dl[k] * g.dl[k] / (g.s[k] * g.s[k] * g.s[k]) * dqd;
    }
    // d = t / |t|
    F3 dt = (dd - g.d * dot(g.d, dd)) * (1.0f / g.tlen);
    // Jacobian: j0 = (fx iz, 0, fx cxv iz^2), j1 = (0, fy iz, fy cyv iz^2), iz = 1/depth, depth = -t.z
    const float fx = K.focal[0], fy = K.focal[1], iz = g.iz;
    float ddepth = 0.0f;
    ddepth += dj0.x * (-fx * iz * iz) + dj1.y * (-fy * iz * iz);
    if (!g.clx) {
      dt.x += dj0.z * fx * iz * iz;
      ddepth += dj0.z * (-2.0f * fx * g.t.x * iz * iz * iz);
    } else {
      ddepth += dj0.z * (-fx * (g.cxv * iz) * iz * iz);
    }
    if (!g.cly) {
      dt.y += dj1.z * fy * iz * iz;
      ddepth += dj1.z * (-2.0f * fy * g.t.y * iz * iz * iz);
    } else {
      ddepth += dj1.z * (-fy * (g.cyv * iz) * iz * iz);
    }
    // screen centre: cx = fx t.x / depth + W/2, cy = H/2 - fy t.y / depth
    dt.x += gd.cx * fx * iz;
    dt.y += -gd.cy * fy * iz;
    ddepth += gd.cx * (-fx * g.t.x * iz * iz) + (-gd.cy) * (-fy * g.t.y * iz * iz);
    dt.z += -ddepth;
    // t = W mu + T -> dmu = W^T dt; wr_k = W R_k -> dR_k = W^T dwr_k
    const float* V = K.view;
    F3 dmu = f3(V[0] * dt.x + V[1] * dt.y + V[2] * dt.z, V[4] * dt.x + V[5] * dt.y + V[6] * dt.z,
                V[8] * dt.x + V[9] * dt.y + V[10] * dt.z);
    F3 dR[3];
    for (int k = 0; k < 3; k++)
      dR[k] = f3(V[0] * dwr[k].x + V[1] * dwr[k].y + V[2] * dwr[k].z, V[4] * dwr[k].x + V[5] * dwr[k].y + V[6] * dwr[k].z,
                 V[8] * dwr[k].x + V[9] * dwr[k].y + V[10] * dwr[k].z);
    // ---- lighting: dL/dacc = dL/dc x albedo x T x iso_norm; the radiance's Jacobian by forward mode, one of the
    // 12 directions (means 3, log-scales 3, quaternion 4, opacity logit, roughness) per pass
    const F3 gc = f3(gd.r, gd.g, gd.b);
    const F3 alb = ld3(P.albedo + 3 * i);
    const float Tl = Lt.lamp_T ? Lt.lamp_T[i] : 1.0f, iso = Lt.iso_norm ? Lt.iso_norm[i] : 1.0f;
    const sl_vgrid* vg = Lt.vgrid ? Lt.vgrid + i : nullptr;
    const float kk = Tl * iso;
    const F3 ga = f3(gc.x * alb.x * kk, gc.y * alb.y * kk, gc.z * alb.z * kk);
    const float* pm = P.means + 3 * i;
    const float* pl = P.log_scales + 3 * i;
    const float* pq = P.quats + 4 * i;
    const float mu0[3] = {pm[0], pm[1], pm[2]}, ls0[3] = {pl[0], pl[1], pl[2]};
    const float q40[4] = {pq[0], pq[1], pq[2], pq[3]}, rough0 = P.roughness[i];
    const dsh::V3<float> eyef = dsh::v3(K.eye[0], K.eye[1], K.eye[2]);
    float dlit[12];
    // one walk of the cut in reverse mode: the adjoint of ga . acc with respect to the position and every receiver field,
    // and (the visitor) the light intensities' gradient through the tree's derivative table (per cut node e and light
    // k: dI_e/ds_k = dLe_e/ds_k scale |w|_M + Le_e scale (w^T dM_e/ds_k w) / (2 |w|_M)); acc0 gives albedo's gradient
    dsh::RecvAdj ra;
    dsh::V3<float> acc0;
    {
      const dsh::Recv<float, float> rv = dsh::receiver<float, float>(mu0, ls0, q40, logit, rough0);
      const uint32_t nl = Lt.n;
      const float scale = Lt.tree.scale;
      acc0 = dsh::emitter_light_adj(
          Lt.tree, rv, vg, Lt.ks, iso, eyef, dsh::v3(ga.x, ga.y, ga.z), ra,
          [&](uint32_t node, float fe, dsh::V3<float> mw, float mq) {
            if (!Lt.dtab || !(mq > 0.0f) || node >= 2u * nl - 1u) return;  // (2 nl - 1 nodes in the table)
            const float* e = Lt.tree.nodes + 24u * node;
            for (uint32_t k = 0; k < nl; k++) {
              const float* t = Lt.dtab + ((size_t)node * nl + k) * 9u;
              const float dq = t[3] * mw.x * mw.x + t[4] * mw.y * mw.y + t[5] * mw.z * mw.z +
                               2.0f * (t[6] * mw.x * mw.y + t[7] * mw.x * mw.z + t[8] * mw.y * mw.z);
              const float dm = 0.5f * dq / mq;
              const float gI = ga.x * (t[0] * mq + e[12] * dm) + ga.y * (t[1] * mq + e[13] * dm) +
                               ga.z * (t[2] * mq + e[14] * dm);
              const float v = gI * scale * fe;
              if (v != 0.0f) atomicAdd(&s_lg[k], v);
            }
          });
    }
    dlit[0] = ra.P.x;
    dlit[1] = ra.P.y;
    dlit[2] = ra.P.z;
    // the receiver's fields against the shape and material parameters (log-scales 3, quaternion 4, opacity logit,
    // roughness), each in forward mode without a walk, dotted with the fields' adjoints
#pragma unroll 1
    for (int p = 3; p < 12; p++) {
      dsh::Dual ls[3], q4[4];
      for (int k = 0; k < 3; k++) ls[k] = dsh::Dual{ls0[k], p == 3 + k ? 1.0f : 0.0f};
      for (int k = 0; k < 4; k++) q4[k] = dsh::Dual{q40[k], p == 6 + k ? 1.0f : 0.0f};
      const dsh::Dual lg{logit, p == 10 ? 1.0f : 0.0f}, rg{rough0, p == 11 ? 1.0f : 0.0f};
      const dsh::Recv<float, dsh::Dual> rv = dsh::receiver<float, dsh::Dual>(mu0, ls, q4, lg, rg);
      auto dd = [](dsh::V3<float> g, dsh::V3<dsh::Dual> f) { return g.x * f.x.d + g.y * f.y.d + g.z * f.z.d; };
      dlit[p] = dd(ra.n, rv.n) + dd(ra.cinv_d, rv.cinv_d) + dd(ra.cinv_o, rv.cinv_o) + dd(ra.sn_d, rv.sn_d) +
                dd(ra.sn_o, rv.sn_o) + dd(ra.Sd, rv.Sd) + dd(ra.So, rv.So) + ra.kappa * rv.kappa.d +
                ra.detC * rv.detC.d;
    }
    const F3 dalb = f3(gc.x * (acc0.x * kk + Lt.ambient), gc.y * (acc0.y * kk + Lt.ambient),
                       gc.z * (acc0.z * kk + Lt.ambient));
    // ---- rotation matrix -> quaternion (normalised)
    const float x = qh[0], y = qh[1], z = qh[2], w = qh[3];
    // G[r][c] = dL/dR[r][c]; column k of R is R[k]
    const float G00 = dR[0].x, G10 = dR[0].y, G20 = dR[0].z;
    const float G01 = dR[1].x, G11 = dR[1].y, G21 = dR[1].z;
    const float G02 = dR[2].x, G12 = dR[2].y, G22 = dR[2].z;
    float dq[4];
    dq[0] = 2.0f * y * G10 + 2.0f * z * G20 + 2.0f * y * G01 - 4.0f * x * G11 + 2.0f * w * G21 + 2.0f * z * G02 -
            2.0f * w * G12 - 4.0f * x * G22;
    dq[1] = -4.0f * y * G00 + 2.0f * x * G10 - 2.0f * w * G20 + 2.0f * x * G01 + 2.0f * z * G21 + 2.0f * w * G02 +
            2.0f * z * G12 - 4.0f * y * G22;
    dq[2] = -4.0f * z * G00 + 2.0f * w * G10 + 2.0f * x * G20 - 2.0f * w * G01 - 4.0f * z * G11 + 2.0f * y * G21 +
            2.0f * x * G02 + 2.0f * y * G12;
    dq[3] = 2.0f * z * G10 - 2.0f * y * G20 - 2.0f * z * G01 + 2.0f * x * G21 + 2.0f * y * G02 - 2.0f * x * G12;
    const float proj = x * dq[0] + y * dq[1] + z * dq[2] + w * dq[3];
    for (int k = 0; k < 4; k++) G.quats[4 * i + k] = (dq[k] - qh[k] * proj) / qn + dlit[6 + k];
    G.means[3 * i + 0] = dmu.x + dlit[0];
    G.means[3 * i + 1] = dmu.y + dlit[1];
    G.means[3 * i + 2] = dmu.z + dlit[2];
    for (int k = 0; k < 3; k++) G.log_scales[3 * i + k] = ds[k] * g.s[k] + dlit[3 + k];
    G.opacity_logits[i] = dlogit + dlit[10];
    G.albedo[3 * i + 0] = dalb.x;
    G.albedo[3 * i + 1] = dalb.y;
    G.albedo[3 * i + 2] = dalb.z;
    G.roughness[i] = dlit[11];
  } else if (i < n) {
    for (int k = 0; k < 3; k++) {
      G.means[3 * i + k] = 0.0f;
      G.log_scales[3 * i + k] = 0.0f;
      G.albedo[3 * i + k] = 0.0f;
    }
    for (int k = 0; k < 4; k++) G.quats[4 * i + k] = 0.0f;
    G.opacity_logits[i] = 0.0f;
    G.roughness[i] = 0.0f;
  }
  __syncthreads();
  if (threadIdx.x < Lt.n && s_lg[threadIdx.x] != 0.0f) atomicAdd(&G.light_scale[threadIdx.x], s_lg[threadIdx.x]);
}

}  // namespace

cudaError_t launch_dproject(const DiffCamera& K, const DiffParams& P, const DiffLights& L, uint32_t n, uint16_t* key16,
                            DiffRec* drec, SplatRec* recs, ushort4* rects, uint32_t* digit_hist, FrameCounters* ctr,
                            cudaStream_t s) {
  if (!n) return cudaSuccess;
  dproject_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(K, P, L, n, key16, drec, recs, rects, digit_hist,
                                                                     ctr);
  return cudaGetLastError();
}

cudaError_t launch_dcomposite_fwd(const uint2* ranges, const uint32_t* tile_vals, const DiffRec* drec, uint32_t width,
                                  uint32_t height, uint32_t tiles_x, uint32_t tiles, float4* img, float* t_final,
                                  uint32_t* n_contrib, cudaStream_t s) {
  if (!tiles) return cudaSuccess;
  dcomposite_fwd_kernel<<<tiles, kThreads, 0, s>>>(ranges, tile_vals, drec, width, height, tiles_x, img, t_final,
                                                   n_contrib);
  return cudaGetLastError();
}

cudaError_t launch_dloss(const float4* img, const float4* target, uint32_t npix, float4* dimg, double* loss,
                         cudaStream_t s) {
  if (!npix) return cudaSuccess;
  dloss_kernel<<<(npix + kThreads - 1) / kThreads, kThreads, 0, s>>>(img, target, npix, dimg, loss);
  return cudaGetLastError();
}

cudaError_t launch_dcomposite_bwd(const uint2* ranges, const uint32_t* tile_vals, const DiffRec* drec, uint32_t width,
                                  uint32_t height, uint32_t tiles_x, uint32_t tiles, const float4* dimg,
                                  const float* t_final, const uint32_t* n_contrib, DiffGrad2D* g2, cudaStream_t s) {
  if (!tiles) return cudaSuccess;
  dcomposite_bwd_kernel<<<tiles, kThreads, 0, s>>>(ranges, tile_vals, drec, width, height, tiles_x, dimg, t_final,
                                                   n_contrib, g2);
  return cudaGetLastError();
}

cudaError_t launch_dproject_bwd(const DiffCamera& K, const DiffParams& P, const DiffLights& L, uint32_t n,
                                const DiffGrad2D* g2, const DiffRec* drec, const DiffGrads& G, cudaStream_t s) {
  if (!n) return cudaSuccess;
  dproject_bwd_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(K, P, L, n, g2, drec, G);
  return cudaGetLastError();
}

}  // namespace sl
