// Probe bounce (runtime/wgsl/bounce.wgsl, the M39 stage-2 loop; host src/lighting.js:723-816, 1018-1103): one frame
// per sl_lighting_update, in its dispatch order
//   xfer      iso_xfer (bounce.wgsl:993-1026): per Gaussian near something that moved (or on a forced refresh) the
//             SH2 of its transfer iso_norm A(w) V(w) over the 128 world cells
//   direct    direct_dirs_emit + env_dirs (bounce_direct.cu): a quarter of the Gaussians per frame, the light each
//             sends toward the probes
//   leaf / up / sh2  node_leaf, node_up (deepest depth first), node_sh2 (bounce.wgsl:1166-1236): per tree node the
//             14-direction sums of that light and their SH2 fit, packed as 27 halves
//   gather    probe_gather (:1255-1410): per (probe, cell) ray the conservative theta-4 cut of every part's tree,
//             the hits kept depth-sorted (16, the farthest folded into the last), composited front to back with the
//             nodes' SH2 radiance, the sky SH beyond; depth moments for the Chebyshev test
//   valid     probe_valid (:1417-1447); psh2: probe_sh2 (:1029-1041)
//   dirs      bounce_dirs (:887-985) for near-mirror Gaussians (flake lobe below 0.1 rad): the probes' per-cell
//             radiance through the Gaussian's transfer and specular lobe, the cells near the eye's mirror direction as
//             lights with a size (cell_asg_phase)
//   bounce    bounce_sh (:1044-1095) with gloss_sh (:1102-1125) for the others: the 8 surrounding probes (trilinear x
//             valid x Chebyshev with the 4x4x4 fallback; a movable part's own 8 probes; a static volume's grid) dotted
//             with the Gaussian's transfer into lo_b
// With the sender cut (sc_select .. node_sh2_sc, :1448-1730) the frame adds: on a re-selection sc_select per depth
// (top down) and sc_xfer for the cut nodes; sc_shadow; the cut's leaves and nodes' direct light (bounce_direct.cu);
// node_leaf on the cut's leaves; node_cut; node_up on the open nodes; node_sh2 zero under the cut.
// The translation unit is compiled with --fmad=false and the deterministic transcendentals of sl_detmath.h, so the
// CPU restatement reproduces it given the same light toward the probes (whose kernel is compiled for speed).
// Near-field visibility is off (the reference's default).
#include <cuda_fp16.h>

#include "light_math.cuh"
#include "sl_bounce.h"

namespace sl {
namespace {

using namespace lm;
constexpr uint32_t kCells = 128;
constexpr uint32_t kHitMax = 16;
constexpr uint32_t kStack = 64;
constexpr float kProbeTheta = 4.0f;
constexpr float kNearR = 0.3f;
constexpr float kGValid = 0.95f;
constexpr float kGlossShMin = 0.1f;

__device__ __forceinline__ f3 ld3(const float* p) { return F3(p[0], p[1], p[2]); }
__device__ __forceinline__ f3 max0(f3 a) { return F3(fmaxf(a.x, 0.0f), fmaxf(a.y, 0.0f), fmaxf(a.z, 0.0f)); }
__device__ __forceinline__ f3 cell_dir(const float* tab, uint32_t c) { return ld3(tab + kTabCells + 4u * c); }
__device__ __forceinline__ float cell_omega(const float* tab, uint32_t c) { return tab[kTabCells + 4u * c + 3u]; }

__device__ __forceinline__ void sh2_basis(f3 d, float* b) {
  const float x = d.x, y = d.y, z = d.z;
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

// sky_radiance (bounce.wgsl:148-160): real SH bands 0-3, clamped at 0
__device__ __forceinline__ f3 sky_radiance(const float* sh, f3 w) {
  const float x = w.x, y = w.y, z = w.z;
  const float b[16] = {0.282095f, 0.488603f * y, 0.488603f * z, 0.488603f * x, 1.092548f * x * y, 1.092548f * y * z,
                       0.315392f * (3.0f * z * z - 1.0f), 1.092548f * x * z, 0.546274f * (x * x - y * y),
                       0.590044f * y * (3.0f * x * x - y * y), 2.890611f * x * y * z,
                       0.457046f * y * (5.0f * z * z - 1.0f), 0.373176f * z * (5.0f * z * z - 3.0f),
                       0.457046f * x * (5.0f * z * z - 1.0f), 1.445306f * z * (x * x - y * y),
                       0.590044f * x * (x * x - 3.0f * y * y)};
  f3 c = F3(0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int k = 0; k < 16; k++) c = add3(c, mul3(ld3(sh + 3 * k), b[k]));
  return max0(c);
}

// a tree node's fields as the gather reads them
struct GNode {
  f3 mean, cinv_d, cinv_o, sn_d, sn_o;
  float radius, kappa, smax;
  uint32_t part, child_lo, child_hi;
};
__device__ __forceinline__ GNode load_gnode(const sl_node* n) {
  GNode g;
  g.mean = F3(n->mean[0], n->mean[1], n->mean[2]);
  g.radius = n->radius;
  g.cinv_d = F3(n->cinv_diag[0], n->cinv_diag[1], n->cinv_diag[2]);
  g.kappa = n->kappa;
  g.cinv_o = F3(n->cinv_off[0], n->cinv_off[1], n->cinv_off[2]);
  g.smax = n->smax;
  g.sn_d = F3(n->sn_diag[0], n->sn_diag[1], n->sn_diag[2]);
  g.part = n->part;
  g.sn_o = F3(n->sn_off[0], n->sn_off[1], n->sn_off[2]);
  g.child_lo = n->child_lo;
  g.child_hi = n->child_hi;
  return g;
}

// seg_geom (common.wgsl:133-151): int_t0^t1 exp(-q(t)/2) dt along P + t w
__device__ __forceinline__ float seg_geom(const GNode& nd, f3 P, f3 w, float t0, float t1) {
  const f3 d = sub3(nd.mean, P);
  const f3 cw = sym_mul(nd.cinv_d, nd.cinv_o, w);
  const float a = dot3(cw, w);
  const float m = dot3(cw, d) / a;
  const f3 e = sub3(d, mul3(w, m));
  const float q = fmaxf(dot3(e, sym_mul(nd.cinv_d, nd.cinv_o, e)), 0.0f);
  const float s = sqrtf(0.5f * a);
  const float x0 = s * (t0 - m), x1 = s * (t1 - m);
  float df;
  if (x0 > 0.0f) df = erfc_pos(x0) - erfc_pos(x1);
  else if (x1 < 0.0f) df = erfc_pos(-x1) - erfc_pos(-x0);
  else df = 2.0f - erfc_pos(x1) - erfc_pos(-x0);
  return lm_exp(-0.5f * q) * sqrtf(kPi / (2.0f * a)) * df;
}

__device__ __forceinline__ uint32_t cell_of(f3 w) {
  const float el = lm_asin(clampf(w.z, -1.0f, 1.0f));
  const float fi = fmaxf((0.5f * kPi - el) / (kPi / 8.0f), 0.0f);
  uint32_t i = (uint32_t)fi;
  i = i < 7u ? i : 7u;
  const uint32_t j = ((uint32_t)floorf((lm_atan2(w.y, w.x) + kPi) / (2.0f * kPi) * 16.0f)) % 16u;
  return i * 16u + j;
}

__device__ __forceinline__ float ground_at(const BounceParams& B, const float* ground, uint32_t i, uint32_t j) {
  return ground ? ground[i * B.dims[1] + j] : 0.0f;
}
__device__ __forceinline__ f3 lattice_pos(const BounceParams& B, const float* ground, uint32_t p) {
  const uint32_t i = p / (B.dims[1] * B.dims[2]), j = (p / B.dims[2]) % B.dims[1], k = p % B.dims[2];
  return F3(B.lo[0] + B.step[0] * (float)i, B.lo[1] + B.step[1] * (float)j, ground_at(B, ground, i, j) + B.levels[k]);
}

// is_part_probe_part (bounce.wgsl:264-266): a movable part's Gaussians read its own 8 probes
__device__ __forceinline__ bool part_probe_part(const BounceParams& B, const sl_part* parts, uint32_t q) {
  return q < B.part_count && (parts[q].flags & 1u) == 0u && parts[q].root != kNone;
}
__device__ __forceinline__ bool has_vol(const BounceParams& B, uint32_t q) { return q < 32u && B.vol_dims[q][0] > 0u; }
__device__ __forceinline__ uint32_t vol_of_probe(const BounceParams& B, uint32_t r) {
  for (uint32_t q = 0; q < B.part_count && q < 32u; q++) {
    const uint32_t n = B.vol_dims[q][0] * B.vol_dims[q][1] * B.vol_dims[q][2];
    if (n > 0u && r >= B.vol_first[q] && r < B.vol_first[q] + n) return q;
  }
  return kNone;
}
// part_probe_frame (bounce.wgsl:256-262): the part root's centre and 0.95 of its axis spreads, at most half its bound
__device__ __forceinline__ void part_frame(const sl_node* __restrict__ tnodes, const sl_part* parts, uint32_t q, f3& c,
                                           f3& h) {
  const sl_node* nd = &tnodes[parts[q].root];
  const f3 a = F3(nd->cinv_diag[0], nd->cinv_diag[1], nd->cinv_diag[2]);
  const f3 o = F3(nd->cinv_off[0], nd->cinv_off[1], nd->cinv_off[2]);
  const float det = a.x * (a.y * a.z - o.z * o.z) - o.x * (o.x * a.z - o.z * o.y) + o.y * (o.x * o.z - a.y * o.y);
  const f3 var = div3(F3(a.y * a.z - o.z * o.z, a.x * a.z - o.y * o.y, a.x * a.y - o.x * o.x), fmaxf(det, 1e-30f));
  const float hb = 0.5f * parts[q].bound[3];
  c = F3(nd->mean[0], nd->mean[1], nd->mean[2]);
  h = F3(fminf(0.95f * sqrtf(fmaxf(var.x, 0.0f)), hb), fminf(0.95f * sqrtf(fmaxf(var.y, 0.0f)), hb),
         fminf(0.95f * sqrtf(fmaxf(var.z, 0.0f)), hb));
}
// vol_frame (bounce.wgsl:69-73): the part frame widened to about the part's extent
__device__ __forceinline__ void vol_frame(const sl_node* __restrict__ tnodes, const sl_part* parts, uint32_t q, f3& c,
                                          f3& h) {
  f3 h0;
  part_frame(tnodes, parts, q, c, h0);
  const float R = parts[q].bound[3];
  h = F3(fminf(1.6f * h0.x, R), fminf(1.6f * h0.y, R), fminf(1.6f * h0.z, R));
}
// probe_pos (bounce.wgsl:217-244): the lattice, each part's 2x2x2 cube, the volumes' grids
__device__ __forceinline__ f3 probe_pos(const BounceParams& B, const float* ground, const sl_node* __restrict__ tnodes,
                                        const sl_part* parts, uint32_t p) {
  if (p >= B.NL + 8u * B.part_count) {
    const uint32_t r = p - B.NL, q = vol_of_probe(B, r);
    if (q == kNone) return F3(0.0f, 0.0f, 0.0f);
    const uint32_t* d = B.vol_dims[q];
    const uint32_t l = r - B.vol_first[q];
    const f3 ijk = F3((float)(l / (d[1] * d[2])), (float)((l / d[2]) % d[1]), (float)(l % d[2]));
    f3 c, h;
    vol_frame(tnodes, parts, q, c, h);
    const f3 den = F3(fmaxf((float)d[0] - 1.0f, 1.0f), fmaxf((float)d[1] - 1.0f, 1.0f), fmaxf((float)d[2] - 1.0f, 1.0f));
    const f3 t = mul3v(mul3(h, 2.0f), ijk);
    return xf_point(parts[q].xf, add3(sub3(c, h), F3(t.x / den.x, t.y / den.y, t.z / den.z)));
  }
  if (p >= B.NL) {
    const uint32_t q = (p - B.NL) / 8u, k = (p - B.NL) % 8u;
    const f3 sgn = F3((float)(k >> 2u) * 2.0f - 1.0f, (float)((k >> 1u) & 1u) * 2.0f - 1.0f,
                      (float)(k & 1u) * 2.0f - 1.0f);
    f3 c, h;
    part_frame(tnodes, parts, q, c, h);
    return xf_point(parts[q].xf, add3(c, mul3v(sgn, h)));
  }
  return lattice_pos(B, ground, p);
}

// probe_cheb (bounce.wgsl:759-768): DDGI Chebyshev visibility of P from probe p (pow(x, 3) as x x x)
__device__ __forceinline__ float probe_cheb(const BounceParams& B, const float* ground, const float4* pd, uint32_t p,
                                            f3 P) {
  const f3 v = sub3(P, lattice_pos(B, ground, p));
  const float dist = len3(v);
  const float4 mm = pd[2u * (p * kCells + cell_of(div3(v, fmaxf(dist, 1e-9f)))) + 1u];
  const float var = fmaxf(mm.y - mm.x * mm.x, 1e-4f);
  const float dd = fmaxf(dist - 0.03f - mm.x, 0.0f);
  if (dd <= 0.0f) return 1.0f;
  const float r = var / (var + dd * dd);
  return r * r * r;
}

struct Weights {
  uint32_t pid[8];
  float w[8];
};

// probe_weights, lattice path (bounce.wgsl:798-885, probe_fallback :771-796)
__device__ __forceinline__ Weights probe_weights(const BounceParams& B, const float* ground, const float4* pd, f3 P) {
  const uint32_t* dm = B.dims;
  const float fx = clampf((P.x - B.lo[0]) / B.step[0], 0.0f, (float)(dm[0] - 1u));
  const float fy = clampf((P.y - B.lo[1]) / B.step[1], 0.0f, (float)(dm[1] - 1u));
  uint32_t i = (uint32_t)floorf(fx), j = (uint32_t)floorf(fy);
  i = i < dm[0] - 2u ? i : dm[0] - 2u;
  j = j < dm[1] - 2u ? j : dm[1] - 2u;
  const float tx = fx - (float)i, ty = fy - (float)j;
  const float g = mixf(mixf(ground_at(B, ground, i, j), ground_at(B, ground, i, j + 1u), ty),
                       mixf(ground_at(B, ground, i + 1u, j), ground_at(B, ground, i + 1u, j + 1u), ty), tx);
  const float h = P.z - g;
  uint32_t k = 0;
  while (k + 2u < dm[2] && h > B.levels[k + 1u]) k++;
  const float tz = clampf((h - B.levels[k]) / fmaxf(B.levels[k + 1u] - B.levels[k], 1e-6f), 0.0f, 1.0f);
  Weights out;
  float wsum = 0.0f;
#pragma unroll
  for (uint32_t c = 0; c < 8u; c++) {
    const uint32_t ox = c >> 2u, oy = (c >> 1u) & 1u, oz = c & 1u;
    const uint32_t p = ((i + ox) * dm[1] + (j + oy)) * dm[2] + (k + oz);
    out.pid[c] = p;
    const float wx = ox ? tx : 1.0f - tx, wy = oy ? ty : 1.0f - ty, wz = oz ? tz : 1.0f - tz;
    const float valid = pd[2u * (p * kCells) + 1u].z;
    const float cw = wx * wy * wz * valid;
    out.w[c] = cw * fmaxf(probe_cheb(B, ground, pd, p, P), 1e-3f);
    wsum += out.w[c];
  }
  if (wsum <= 0.0f) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
      out.pid[c] = 0u;
      out.w[c] = 0.0f;
    }
    for (uint32_t q = 0; q < 64u; q++) {
      const int ii = (int)i + (int)(q >> 4u) - 1, jj = (int)j + (int)((q >> 2u) & 3u) - 1,
                kk = (int)k + (int)(q & 3u) - 1;
      if (ii < 0 || jj < 0 || kk < 0 || ii >= (int)dm[0] || jj >= (int)dm[1] || kk >= (int)dm[2]) continue;
      const uint32_t p = ((uint32_t)ii * dm[1] + (uint32_t)jj) * dm[2] + (uint32_t)kk;
      if (pd[2u * (p * kCells) + 1u].z <= 0.0f) continue;
      const float d = fmaxf(len3(sub3(P, lattice_pos(B, ground, p))), 0.05f);
      const float w = fmaxf(probe_cheb(B, ground, pd, p, P), 1e-3f) / (d * d);
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
#pragma unroll
    for (int c = 0; c < 8; c++) s += out.w[c];
#pragma unroll
    for (int c = 0; c < 8; c++) out.w[c] /= fmaxf(s, 1e-12f);
    return out;
  }
#pragma unroll
  for (int c = 0; c < 8; c++) out.w[c] /= fmaxf(wsum, 1e-12f);
  return out;
}

__device__ __forceinline__ float sel(uint32_t o, float f) { return o ? f : 1.0f - f; }

// probe_weights (bounce.wgsl:813-885): a movable part's Gaussians trilinear over its own 8 probes, a static volume's
// over its grid (neither with the Chebyshev test), the rest over the lattice
__device__ __forceinline__ Weights weights_for(const BounceParams& B, const float* ground, const float4* pd,
                                               const sl_node* __restrict__ tnodes, const sl_part* parts, f3 P,
                                               uint32_t own) {
  if (part_probe_part(B, parts, own)) {
    f3 c, h;
    part_frame(tnodes, parts, own, c, h);
    const float* xf = parts[own].xf;
    const f3 lp = xf_dir_inv(xf, sub3(P, F3(xf[3], xf[7], xf[11])));
    const f3 num = add3(sub3(lp, c), h);
    const f3 f = F3(clampf(num.x / fmaxf(2.0f * h.x, 1e-6f), 0.0f, 1.0f),
                    clampf(num.y / fmaxf(2.0f * h.y, 1e-6f), 0.0f, 1.0f),
                    clampf(num.z / fmaxf(2.0f * h.z, 1e-6f), 0.0f, 1.0f));
    Weights out;
#pragma unroll
    for (uint32_t k = 0; k < 8u; k++) {
      out.pid[k] = B.NL + own * 8u + k;
      out.w[k] = sel(k >> 2u, f.x) * sel((k >> 1u) & 1u, f.y) * sel(k & 1u, f.z);
    }
    return out;
  }
  if (has_vol(B, own)) {
    f3 c, h;
    vol_frame(tnodes, parts, own, c, h);
    const float* xf = parts[own].xf;
    const f3 lp = xf_dir_inv(xf, sub3(P, F3(xf[3], xf[7], xf[11])));
    const uint32_t* d = B.vol_dims[own];
    const f3 num = add3(sub3(lp, c), h);
    const f3 fq = F3(clampf(num.x / fmaxf(2.0f * h.x, 1e-6f), 0.0f, 1.0f) * ((float)d[0] - 1.0f),
                     clampf(num.y / fmaxf(2.0f * h.y, 1e-6f), 0.0f, 1.0f) * ((float)d[1] - 1.0f),
                     clampf(num.z / fmaxf(2.0f * h.z, 1e-6f), 0.0f, 1.0f) * ((float)d[2] - 1.0f));
    uint32_t fi[3] = {(uint32_t)floorf(fq.x), (uint32_t)floorf(fq.y), (uint32_t)floorf(fq.z)};
#pragma unroll
    for (int a = 0; a < 3; a++) fi[a] = fi[a] < d[a] - 2u ? fi[a] : d[a] - 2u;
    const f3 fr = F3(fq.x - (float)fi[0], fq.y - (float)fi[1], fq.z - (float)fi[2]);
    Weights out;
#pragma unroll
    for (uint32_t k = 0; k < 8u; k++) {
      const uint32_t ox = k >> 2u, oy = (k >> 1u) & 1u, oz = k & 1u;
      out.pid[k] = B.NL + B.vol_first[own] + ((fi[0] + ox) * d[1] + (fi[1] + oy)) * d[2] + (fi[2] + oz);
      out.w[k] = sel(ox, fr.x) * sel(oy, fr.y) * sel(oz, fr.z);
    }
    return out;
  }
  return probe_weights(B, ground, pd, P);
}

__device__ __forceinline__ uint32_t mat_index(const sl_gaussian& G, uint32_t mat_count) {
  const uint32_t mi = G.flags & 0xFFFFu, top = (mat_count > 1u ? mat_count : 1u) - 1u;
  return mi < top ? mi : top;
}

// ---- kernels ---------------------------------------------------------------------------------------------------

constexpr int kThreads = 128;

__global__ void __launch_bounds__(kThreads) xfer_kernel(const __grid_constant__ BounceParams B,
                                                        const sl_gaussian* __restrict__ gs,
                                                        const sl_node* __restrict__ nodes,
                                                        const sl_vgrid* __restrict__ vgrid,
                                                        const sl_part* __restrict__ parts,
                                                        const float* __restrict__ tab, float4* __restrict__ xfer,
                                                        float* __restrict__ leaf_w) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= B.G) return;
  const sl_gaussian& G = gs[g];
  const uint32_t own = G.part_surface & 0xFFFFu;
  const float* xf = parts[own].xf;
  const f3 P = xf_point(xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  bool stale = B.force || (own < 32u && ((B.moved_mask >> own) & 1u));
  for (uint32_t p = 0; p < B.part_count && p < 32u && !stale; p++) {
    if (p == own || ((B.moved_mask >> p) & 1u) == 0u) continue;
    const float* b = parts[p].bound;
    const float r = b[3] + kNearR;
    stale = len3(sub3(P, xf_point(parts[p].xf, F3(b[0], b[1], b[2])))) < r ||
            len3(sub3(P, xf_point(parts[p].xf_prev, F3(b[0], b[1], b[2])))) < r;
  }
  if (!stale) return;
  const Leaf nd = load_leaf(&nodes[g]);
  const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
  float t[9];
#pragma unroll
  for (int m = 0; m < 9; m++) t[m] = 0.0f;
  const sl_vgrid& vg = vgrid[g];
  for (uint32_t c = 0; c < kCells; c++) {
    const f3 w = cell_dir(tab, c);
    const f3 u = xf_dir_inv(xf, w);
    const float v = vgrid_lookup(vg, u) * 1.0f;
    if (v <= 0.0f) continue;
    const float a = nd.iso_norm * footprint(nd, s3 * s3, u) * v * cell_omega(tab, c);
    float y[9];
    sh2_basis(w, y);
#pragma unroll
    for (int m = 0; m < 9; m++) t[m] += a * y[m];
  }
  xfer[3u * g] = make_float4(t[0], t[1], t[2], t[3]);
  xfer[3u * g + 1u] = make_float4(t[4], t[5], t[6], t[7]);
  xfer[3u * g + 2u] = make_float4(t[8], 0.0f, 0.0f, 0.0f);
  // node_leaf's weights toward D14, footprint x V: like the transfer they change only when the part turns
  for (int k = 0; k < 14; k++) {
    const f3 wo = xf_dir_inv(xf, ld3(tab + kTabD14 + 3 * k));
    leaf_w[14u * g + (uint32_t)k] = footprint(nd, s3 * s3, wo) * vgrid_lookup(vg, wo);
  }
}

// node_leaf: per leaf and direction (L w, w), L its light toward the probes plus last frame's bounce
__global__ void __launch_bounds__(kThreads) leaf_kernel(const __grid_constant__ BounceParams B,
                                                        const sl_gaussian* __restrict__ gs,
                                                        const float* __restrict__ leaf_w,
                                                        const float4* __restrict__ lo_dir,
                                                        const float4* __restrict__ lo_b,
                                                        const uint32_t* __restrict__ flag, float4* __restrict__ acc) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= B.G) return;
  if (flag && flag[g] != kScLeaf) return;  // node_leaf_list: with the sender cut, the cut's leaves only
  const sl_gaussian& G = gs[g];
  const float4 ld = lo_dir[g], lb = lo_b[3u * g + 1u];
  // the emitters' own part sends nothing into the probes (PP.refl.w, emitBounceFix: their light reaches the scene as
  // direct light; the weights stay, so they still occlude)
  const bool dark = (G.part_surface & 0xFFFFu) == B.dark_part;
  const f3 L = dark ? F3(0.0f, 0.0f, 0.0f) : add3(F3(ld.x, ld.y, ld.z), F3(lb.x, lb.y, lb.z));
  for (int k = 0; k < 14; k++) {
    const float w = leaf_w[14u * g + (uint32_t)k];
    acc[14u * g + (uint32_t)k] = make_float4(L.x * w, L.y * w, L.z * w, w);
  }
}

// node_up for one depth: per (internal node, direction) the sum of its children's in kids order
__global__ void __launch_bounds__(kThreads) up_kernel(const sl_node* __restrict__ nodes,
                                                      const uint32_t* __restrict__ kids,
                                                      const uint32_t* __restrict__ list, uint32_t count,
                                                      const uint32_t* __restrict__ flag, float4* __restrict__ acc) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= count * 14u) return;
  const uint32_t i = list[t / 14u], k = t % 14u;
  if (flag && flag[i] != kScOpen) return;  // node_up_sc: the open nodes only
  const uint32_t lo = nodes[i].child_lo, hi = nodes[i].child_hi;
  float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  for (uint32_t j = lo; j < hi; j++) {
    const float4 c = acc[14u * kids[j] + k];
    s.x += c.x;
    s.y += c.y;
    s.z += c.z;
    s.w += c.w;
  }
  acc[14u * i + k] = s;
}

// node_sh2: the 14-direction means fitted to SH2 (pinv), 27 halves in 14 words
__global__ void __launch_bounds__(kThreads) sh2_kernel(uint32_t N, const float* __restrict__ tab,
                                                       const float4* __restrict__ acc,
                                                       const uint32_t* __restrict__ flag,
                                                       uint32_t* __restrict__ node_sh) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= N) return;
  if (flag && flag[i] == kScBelow) {  // under the sender cut: the gather reads zero (the reference's null slot)
#pragma unroll
    for (int j = 0; j < 14; j++) node_sh[14u * i + (uint32_t)j] = 0u;
    return;
  }
  f3 L[14];
#pragma unroll
  for (int k = 0; k < 14; k++) {
    const float4 a = acc[14u * i + (uint32_t)k];
    L[k] = div3(F3(a.x, a.y, a.z), fmaxf(a.w, 1e-12f));
  }
  float h[28];
  h[27] = 0.0f;
#pragma unroll
  for (int m = 0; m < 9; m++) {
    f3 c = F3(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < 14; k++) c = add3(c, mul3(L[k], tab[kTabPinv + 14 * m + k]));
    h[3 * m] = c.x;
    h[3 * m + 1] = c.y;
    h[3 * m + 2] = c.z;
  }
#pragma unroll
  for (int j = 0; j < 14; j++) {
    const uint32_t lo = __half_as_ushort(__float2half_rn(h[2 * j]));
    const uint32_t hi = __half_as_ushort(__float2half_rn(h[2 * j + 1]));
    node_sh[14u * i + (uint32_t)j] = lo | (hi << 16);
  }
}

__device__ __forceinline__ f3 node_radiance(const uint32_t* __restrict__ node_sh, uint32_t ni, const float* b) {
  float h[28];
#pragma unroll
  for (int j = 0; j < 14; j++) {
    const uint32_t u = node_sh[14u * ni + (uint32_t)j];
    h[2 * j] = __half2float(__ushort_as_half((unsigned short)(u & 0xFFFFu)));
    h[2 * j + 1] = __half2float(__ushort_as_half((unsigned short)(u >> 16)));
  }
  f3 v = F3(0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int m = 0; m < 9; m++) v = add3(v, mul3(F3(h[3 * m], h[3 * m + 1], h[3 * m + 2]), b[m]));
  return v;
}

// probe_gather: one (probe, cell) ray per thread
__global__ void __launch_bounds__(kThreads) gather_kernel(const __grid_constant__ BounceParams B,
                                                          const sl_node* __restrict__ tnodes,
                                                          const uint32_t* __restrict__ kids,
                                                          const sl_vgrid* __restrict__ vgrid,
                                                          const sl_part* __restrict__ parts,
                                                          const float* __restrict__ tab,
                                                          const float* __restrict__ ground,
                                                          const uint32_t* __restrict__ node_sh,
                                                          float4* __restrict__ pd, float4* __restrict__ hist) {
  const uint32_t id = blockIdx.x * kThreads + threadIdx.x;
  if (id >= B.NP * kCells) return;
  const uint32_t p = id / kCells, c = id % kCells;  // one probe per block; a warp takes two elevation rows of cells
  // a part probe skips its own part (a static part's stay idle); a volume's probes skip their object
  uint32_t skip = kNone;
  if (p >= B.NL && p < B.NL + 8u * B.part_count) {
    skip = (p - B.NL) / 8u;
    if (!part_probe_part(B, parts, skip)) return;
  } else if (p >= B.NL) {
    skip = vol_of_probe(B, p - B.NL);
    if (skip == kNone) return;
  }
  const f3 o = probe_pos(B, ground, tnodes, parts, p);
  const f3 w = cell_dir(tab, c);
  const float brad = p < B.NL ? B.brad : 0.0f;   // probes off the lattice cut around themselves
  f3 cen = o;
  if (!B.terrain && p < B.NL) {
    const uint32_t dz = B.dims[2];
    const float bx = (float)((p / (B.dims[1] * dz)) / 2u), by = (float)(((p / dz) % B.dims[1]) / 2u),
                bz = (float)((p % dz) / 2u);
    cen = F3(B.lo[0] + B.step[0] * (2.0f * bx + 0.5f), B.lo[1] + B.step[1] * (2.0f * by + 0.5f),
             B.lo[2] + B.step[2] * (2.0f * bz + 0.5f));
  }
  const float t1 = B.tmax;
  float ht[kHitMax], hv[kHitMax];
  uint32_t hn[kHitMax];
  uint32_t k = 0;
  // The warp's 32 rays belong to one probe, so whether a node is used whole or opened (the cut about the probe's
  // centre) is the same for all of them: the warp walks one depth-first stack, each entry carrying the lanes whose
  // rays met its parent, and a lane acts only on the entries in its mask.  Restricted to one lane this is exactly that
  // ray's own depth-first walk (the same nodes in the same order), so its hits, and everything after, are unchanged.
  __shared__ uint32_t s_node[kThreads / 32][kStack], s_mask[kThreads / 32][kStack];
  const uint32_t lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
  uint32_t* stn = s_node[wi];
  uint32_t* stm = s_mask[wi];
  for (uint32_t q = 0; q < B.part_count; q++) {
    const float* xf = parts[q].xf;
    const uint32_t root = parts[q].root;
    if (root == kNone || q == skip) continue;
    const f3 Po = xf_dir_inv(xf, sub3(o, F3(xf[3], xf[7], xf[11])));
    const f3 wr = xf_dir_inv(xf, w);
    const f3 cr = xf_dir_inv(xf, sub3(cen, F3(xf[3], xf[7], xf[11])));
    if (lane == 0) {
      stn[0] = root;
      stm[0] = 0xffffffffu;
    }
    __syncwarp();
    uint32_t sp = 1;
    // a tree visits each node once; the bound (warp-uniform) only keeps a malformed, cyclic tree from spinning
    for (uint32_t guard = 0; sp > 0u && guard < 4u * B.N + 64u; guard++) {
      sp--;
      const uint32_t ni = stn[sp], mask = stm[sp];
      __syncwarp();  // every lane has read the entry before a push may overwrite it
      // the bound test on one 16-byte load (mean, radius), by the lanes whose rays met the parent
      bool hit = false;
      f3 d = F3(0.0f, 0.0f, 0.0f);
      if ((mask >> lane) & 1u) {
        const float4 mr = __ldg(reinterpret_cast<const float4*>(&tnodes[ni]));
        d = sub3(F3(mr.x, mr.y, mr.z), Po);
        const float tt = clampf(dot3(d, wr), 0.0f, t1);
        const f3 e = sub3(d, mul3(wr, tt));
        hit = !(dot3(e, e) > mr.w * mr.w);
      }
      const uint32_t hits = __ballot_sync(0xffffffffu, hit);
      if (hits == 0u) continue;
      const GNode nd = load_gnode(&tnodes[ni]);
      bool use_node = ni < B.G;
      if (!use_node) use_node = len3(sub3(cr, nd.mean)) - brad > kProbeTheta * nd.smax;
      if (use_node) {
        if (hit) {
          const float tau = nd.kappa * sqrtf(fmaxf(dot3(wr, sym_mul(nd.sn_d, nd.sn_o, wr)), 0.0f)) *
                            seg_geom(nd, Po, wr, 0.0f, t1);
          if (tau > 1e-6f) {
            const f3 cw = sym_mul(nd.cinv_d, nd.cinv_o, wr);
            const float den = dot3(cw, wr);
            const float tp = fabsf(den) > 1e-30f ? clampf(dot3(cw, d) / den, 0.0f, t1) : t1;
            uint32_t at = k < kHitMax - 1u ? k : kHitMax - 1u;
            const uint32_t l = kHitMax - 1u;
            if (k == kHitMax && tp >= ht[l]) {
              ht[l] = fmaxf(ht[l], tp);
              hv[l] = fminf(hv[l] + tau, 64.0f);
            } else {
              const bool full = k == kHitMax;
              const float sv = full ? hv[l] : 0.0f, stv = full ? ht[l] : 0.0f;
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
              k = k + 1u < kHitMax ? k + 1u : kHitMax;
            }
          }
        }
      } else {
        for (uint32_t j = nd.child_lo; j < nd.child_hi; j++) {
          if (sp < kStack) {
            if (lane == 0) {
              stn[sp] = kids[j];
              stm[sp] = hits;
            }
            sp++;
          }
        }
        __syncwarp();
      }
    }
  }
  float T = 1.0f, m1 = 0.0f, m2 = 0.0f, first_part = -1.0f, nearv = 0.0f;
  f3 acc = F3(0.0f, 0.0f, 0.0f);
  float bw[9];
  sh2_basis(mul3(w, -1.0f), bw);
  for (uint32_t i = 0; i < k; i++) {
    if (T <= 0.0f) break;
    const float al = 1.0f - lm_exp(-hv[i]);
    const f3 rad = max0(node_radiance(node_sh, hn[i], bw));
    acc = add3(acc, mul3(rad, T * al));
    const float dep = clampf(ht[i], 0.0f, t1);
    m1 += T * al * dep;
    m2 += T * al * dep * dep;
    const float Tn = T * (1.0f - al);
    if (T >= 0.5f && Tn < 0.5f) {
      const uint32_t hp = tnodes[hn[i]].part;
      first_part = (float)hp;
      nearv = dep < 0.05f ? 1.0f : 0.0f;
      if (hn[i] < B.G && hp < B.part_count &&
          vgrid_lookup(vgrid[hn[i]], xf_dir_inv(parts[hp].xf, mul3(w, -1.0f))) < 0.1f)
        nearv += 2.0f;
    }
    T = Tn;
  }
  if (B.has_sky && t1 >= B.tmax * 0.999f) acc = add3(acc, mul3(sky_radiance(B.sky, w), T));
  m1 += T * t1;
  m2 += T * t1 * t1;
  // the history blend: an EMA of weight alpha (1: the gather as is), or alpha < 0 the tapered blend of this gather and
  // the two before it (FIR_TAPS 0.5, 0.3, 0.2: ?probeblend=fir); a gather with alpha >= 1 fills both history entries
  const float a = B.alpha;
  const float4 old0 = pd[2u * id], old1 = pd[2u * id + 1u];
  float4* hp = hist + 4u * id;
  if (a < 0.0f) {
    const float4 g1a = hp[0], g1b = hp[1], g2a = hp[2], g2b = hp[3];
    pd[2u * id] = make_float4(0.5f * acc.x + 0.3f * g1a.x + 0.2f * g2a.x, 0.5f * acc.y + 0.3f * g1a.y + 0.2f * g2a.y,
                              0.5f * acc.z + 0.3f * g1a.z + 0.2f * g2a.z, first_part);
    pd[2u * id + 1u] = make_float4(0.5f * m1 + 0.3f * g1a.w + 0.2f * g2a.w, 0.5f * m2 + 0.3f * g1b.x + 0.2f * g2b.x,
                                   old1.z, nearv);
    hp[2] = g1a;
    hp[3] = g1b;
    hp[0] = make_float4(acc.x, acc.y, acc.z, m1);
    hp[1] = make_float4(m2, 0.0f, 0.0f, 0.0f);
    return;
  }
  pd[2u * id] = make_float4(mixf(old0.x, acc.x, a), mixf(old0.y, acc.y, a), mixf(old0.z, acc.z, a), first_part);
  pd[2u * id + 1u] = make_float4(mixf(old1.x, m1, a), mixf(old1.y, m2, a), old1.z, nearv);
  if (a >= 1.0f) {
    hp[0] = hp[2] = make_float4(acc.x, acc.y, acc.z, m1);
    hp[1] = hp[3] = make_float4(m2, 0.0f, 0.0f, 0.0f);
  }
}

// probe_valid: one probe per thread
__global__ void __launch_bounds__(kThreads) valid_kernel(const __grid_constant__ BounceParams B,
                                                         const sl_part* __restrict__ parts, float4* __restrict__ pd) {
  const uint32_t p = blockIdx.x * kThreads + threadIdx.x;
  if (p >= B.NP) return;
  if (p >= B.NL) {  // part and volume probes skip their own object, so never sit inside it
    pd[2u * (p * kCells) + 1u].z = 1.0f;
    return;
  }
  uint32_t cnt[17];
#pragma unroll
  for (int i = 0; i < 17; i++) cnt[i] = 0u;
  uint32_t nearc = 0, back = 0;
  for (uint32_t c = 0; c < kCells; c++) {
    const float4 r0 = pd[2u * (p * kCells + c)], r1 = pd[2u * (p * kCells + c) + 1u];
    const uint32_t fl = (uint32_t)(fmaxf(r1.w, 0.0f) + 0.5f);
    nearc += fl & 1u;
    back += (fl >> 1u) & 1u;
    if (r0.w >= 0.0f) {
      const uint32_t q = (uint32_t)r0.w;
      cnt[q < 16u ? q : 16u]++;
    }
  }
  bool enclosed = false;
  for (uint32_t q = 0; q < B.part_count && q < 16u; q++)
    if ((parts[q].flags & 1u) == 0u && (float)cnt[q] > kGValid * (float)kCells) enclosed = true;
  const float valid = (enclosed || nearc * 2u > kCells || back * 2u > kCells) ? 0.0f : 1.0f;
  pd[2u * (p * kCells) + 1u].z = valid;
}

// probe_sh2: one probe per thread
__global__ void __launch_bounds__(kThreads) psh2_kernel(const __grid_constant__ BounceParams B,
                                                        const float* __restrict__ tab, const float4* __restrict__ pd,
                                                        float4* __restrict__ probe_sh) {
  const uint32_t p = blockIdx.x * kThreads + threadIdx.x;
  if (p >= B.NP) return;
  f3 c9[9];
#pragma unroll
  for (int m = 0; m < 9; m++) c9[m] = F3(0.0f, 0.0f, 0.0f);
  for (uint32_t c = 0; c < kCells; c++) {
    const float4 r0 = pd[2u * (p * kCells + c)];
    const f3 L = mul3(F3(r0.x, r0.y, r0.z), cell_omega(tab, c));
    float y[9];
    sh2_basis(cell_dir(tab, c), y);
#pragma unroll
    for (int m = 0; m < 9; m++) c9[m] = add3(c9[m], mul3(L, y[m]));
  }
#pragma unroll
  for (int m = 0; m < 9; m++) probe_sh[9u * p + (uint32_t)m] = make_float4(c9[m].x, c9[m].y, c9[m].z, 0.0f);
}

// bounce_sh + gloss_sh: one Gaussian per thread
__global__ void __launch_bounds__(kThreads) bounce_kernel(const __grid_constant__ BounceParams B,
                                                          const sl_gaussian* __restrict__ gs,
                                                          const sl_node* __restrict__ nodes,
                                                          const sl_vgrid* __restrict__ vgrid,
                                                          const sl_part* __restrict__ parts,
                                                          const sl_material* __restrict__ mats,
                                                          const sl_node* __restrict__ tnodes,
                                                          const float* __restrict__ ground,
                                                          const float4* __restrict__ pd,
                                                          const float4* __restrict__ probe_sh,
                                                          const float4* __restrict__ xfer, float4* __restrict__ lo_b) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= B.G) return;
  const sl_gaussian& G = gs[g];
  const sl_material mat = mats[mat_index(G, B.mat_count)];
  const float ks = spec_weight(mat);
  const float lw = sqrtf(fminf(mat.flake[1], mat.flake[2]) / fmaxf(mat.flake[0], 1e-12f));
  if (ks > 0.0f && !(lw >= kGlossShMin)) return;
  const uint32_t own = G.part_surface & 0xFFFFu;
  const float* xf = parts[own].xf;
  const f3 P = xf_point(xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  const Weights pw = weights_for(B, ground, pd, tnodes, parts, P, own);
  f3 Lsh[9];
#pragma unroll
  for (int m = 0; m < 9; m++) Lsh[m] = F3(0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const float wq = pw.w[q];
    if (wq <= 0.0f) continue;
#pragma unroll
    for (int m = 0; m < 9; m++) {
      const float4 s = probe_sh[9u * pw.pid[q] + (uint32_t)m];
      Lsh[m] = add3(Lsh[m], mul3(F3(s.x, s.y, s.z), wq));
    }
  }
  const float4 t0 = xfer[3u * g], t1 = xfer[3u * g + 1u], t2 = xfer[3u * g + 2u];
  const float t[9] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w, t2.x};
  f3 cc = mul3(Lsh[0], t[0]);
#pragma unroll
  for (int m = 1; m < 9; m++) cc = add3(cc, mul3(Lsh[m], t[m]));
  const f3 alb = F3(G.albedo[0], G.albedo[1], G.albedo[2]);
  const f3 cb = mul3v(alb, max0(cc));
  f3 eyec = cb;
  if (ks > 0.0f) {
    const Leaf nd = load_leaf(&nodes[g]);
    const m3 Rq = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]);
    const f3 n = Rq.c[0];
    const f3 wo = xf_dir_inv(xf, norm3(sub3(ld3(B.eye), P)));
    const f3 wm = mirror3(wo, n);
    const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
    const float detC = s3 * s3;
    const sl_vgrid& vg = vgrid[g];
    const float vis = vgrid_lookup(vg, wm) * footprint(nd, detC, wm);
    f3 sp = F3(0.0f, 0.0f, 0.0f);
    if (vis > 0.0f) {
      const float damp = iso_damp(nd.iso_norm, footprint(nd, detC, wo) * vgrid_lookup(vg, wo));
      const float sg = 2.0f * lw;
      const float a1 = lm_exp(-sg * sg), a2 = lm_exp(-3.0f * sg * sg);
      const f3 wmw = F3(xf[0] * wm.x + xf[1] * wm.y + xf[2] * wm.z, xf[4] * wm.x + xf[5] * wm.y + xf[6] * wm.z,
                        xf[8] * wm.x + xf[9] * wm.y + xf[10] * wm.z);
      float y[9];
      sh2_basis(wmw, y);
      f3 Lm = mul3(Lsh[0], y[0]);
#pragma unroll
      for (int m = 1; m < 4; m++) Lm = add3(Lm, mul3(Lsh[m], a1 * y[m]));
#pragma unroll
      for (int m = 4; m < 9; m++) Lm = add3(Lm, mul3(Lsh[m], a2 * y[m]));
      sp = mul3(mul3v(mul3(mul3(mul3(mul3(mul3(alb, nd.iso_norm), ks), 4.0f), kPi), damp), max0(Lm)), vis);
    }
    eyec = add3(mul3(cb, 1.0f - ks), sp);
  }
  lo_b[3u * g] = make_float4(eyec.x, eyec.y, eyec.z, 0.0f);
  lo_b[3u * g + 1u] = make_float4(cb.x, cb.y, cb.z, 0.0f);
  lo_b[3u * g + 2u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// bounce_dirs (bounce.wgsl:887-985, the M39 path), for near-mirror Gaussians (a specular flake lobe narrower than
// 0.1 rad, which the probes' SH2 cannot hold): the 8 probes' per-cell radiance through the Gaussian's transfer (V,
// footprint, solid angle) and its specular lobe toward D14 (their footprint x V weighted mean: toward the probes) and
// toward the eye (cells within about three lobe widths of the eye's mirror direction as lights with a size:
// cell_asg_phase) into lo_b; the other Gaussians are bounce_sh's
__global__ void __launch_bounds__(kThreads) dirs_kernel(const __grid_constant__ BounceParams B,
                                                        const sl_gaussian* __restrict__ gs,
                                                        const sl_node* __restrict__ nodes,
                                                        const sl_vgrid* __restrict__ vgrid,
                                                        const sl_part* __restrict__ parts,
                                                        const sl_material* __restrict__ mats,
                                                        const sl_node* __restrict__ tnodes,
                                                        const float* __restrict__ tab,
                                                        const float* __restrict__ ground,
                                                        const float4* __restrict__ pd, float4* __restrict__ lo_b) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g >= B.G) return;
  const sl_gaussian& G = gs[g];
  const sl_material mat = mats[mat_index(G, B.mat_count)];
  const float ks = spec_weight(mat);
  const float lw = sqrtf(fminf(mat.flake[1], mat.flake[2]) / fmaxf(mat.flake[0], 1e-12f));
  if (!(ks > 0.0f && !(lw >= kGlossShMin))) return;
  const uint32_t own = G.part_surface & 0xFFFFu;
  const float* xf = parts[own].xf;
  const f3 P = xf_point(xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  const Leaf nd = load_leaf(&nodes[g]);
  const m3 Rq = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]);
  const m3 Sloc = m3m(m3m(Rq, m3diag(F3(mat.flake[0], mat.flake[1], mat.flake[2]))), m3t(Rq));
  const f3 n = Rq.c[0];
  const f3 Sd = F3(Sloc.c[0].x, Sloc.c[1].y, Sloc.c[2].z), So = F3(Sloc.c[1].x, Sloc.c[2].x, Sloc.c[2].y);
  const f3 flake = F3(mat.flake[0], mat.flake[1], mat.flake[2]);
  const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
  const float detC = s3 * s3;
  const sl_vgrid& vg = vgrid[g];
  const Weights pw = weights_for(B, ground, pd, tnodes, parts, P, own);
  const float near_ang = fminf(3.0f * (0.4f * kPi / 8.0f + 2.0f * lw), kPi);
  const f3 wo14 = xf_dir_inv(xf, norm3(sub3(ld3(B.eye), P)));
  const f3 wr_eye = mirror3(wo14, n);
  const SpecPre sp = spec_prepare(Sd, So);
  const AsgPre ap = asg_prepare(n, Rq.c[1], Rq.c[2], flake, Sd, So, wo14);
  f3 acc[15];
#pragma unroll
  for (int k = 0; k < 15; k++) acc[k] = F3(0.0f, 0.0f, 0.0f);
  for (uint32_t c = 0; c < kCells; c++) {
    f3 L = F3(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (pw.w[k] > 0.0f) {
        const float4 r0 = pd[2u * (pw.pid[k] * kCells + c)];
        L = add3(L, mul3(F3(r0.x, r0.y, r0.z), pw.w[k]));
      }
    if (L.x + L.y + L.z <= 0.0f) continue;
    const f3 u = xf_dir_inv(xf, cell_dir(tab, c));
    const float vis = vgrid_lookup(vg, u) * 1.0f;
    if (vis <= 0.0f) continue;
    const f3 lin = mul3(L, vis * footprint(nd, detC, u) * cell_omega(tab, c));
    const f3 ur = mirror3(u, n);
    const float damp = iso_damp(nd.iso_norm, footprint(nd, detC, ur) * vgrid_lookup(vg, ur));
#pragma unroll
    for (int k = 0; k < 14; k++) {
      const f3 wo = xf_dir_inv(xf, ld3(tab + kTabD14 + 3 * k));
      acc[k] = add3(acc[k], mul3(lin, iso_lobe_from(ks, phase_specular_p(sp, u, wo), damp)));
    }
    float lobe14;
    if (B.asg_cells && lm_acos(clampf(dot3(u, wr_eye), -1.0f, 1.0f)) < near_ang) {
      const float* e = tab + kTabCellAsg + 8u * c;
      const f3 lb0 = xf_dir_inv(xf, ld3(e)), lb1 = xf_dir_inv(xf, ld3(e + 3));
      lobe14 = iso_lobe_from(ks, asg_phase_p(ap, sp, u, lb0, lb1, s2m{e[6], 0.0f, e[7]}, wo14), damp);
    } else {
      lobe14 = iso_lobe_from(ks, phase_specular_p(sp, u, wo14), damp);
    }
    acc[14] = add3(acc[14], mul3(lin, lobe14));
  }
  f3 send = F3(0.0f, 0.0f, 0.0f);
  float ws = 0.0f;
#pragma unroll
  for (int k = 0; k < 14; k++) {
    const f3 wo = xf_dir_inv(xf, ld3(tab + kTabD14 + 3 * k));
    const float w = footprint(nd, detC, wo) * vgrid_lookup(vg, wo);
    send = add3(send, mul3(acc[k], w));
    ws += w;
  }
  send = div3(send, fmaxf(ws, 1e-20f));
  const f3 sc = mul3(F3(G.albedo[0], G.albedo[1], G.albedo[2]), nd.iso_norm);
  const f3 eyec = mul3v(sc, acc[14]), sendc = mul3v(sc, send);
  lo_b[3u * g] = make_float4(eyec.x, eyec.y, eyec.z, 0.0f);
  lo_b[3u * g + 1u] = make_float4(sendc.x, sendc.y, sendc.z, 0.0f);
  lo_b[3u * g + 2u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// ---- the sender cut (bounce.wgsl:1448-1730) ------------------------------------------------------------------------

// pcg_hash and to_unit (common.wgsl:98-104); sc_face (common.wgsl:342-345, SC_FACE_K 1)
__device__ __forceinline__ uint32_t pcg_hash(uint32_t x) {
  const uint32_t s = x * 747796405u + 2891336453u;
  const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (w >> 22u) ^ w;
}
__device__ __forceinline__ float to_unit(uint32_t x) { return (float)(x >> 8u) * (1.0f / 16777216.0f); }
__device__ __forceinline__ float sc_face(float c) { return clampf(c * 1.0f, -1.0f, 1.0f); }
__device__ __forceinline__ float sc_mass(const sl_node* __restrict__ n) {
  return n->kappa / sqrtf(fmaxf(sym_det(F3(n->cinv_diag[0], n->cinv_diag[1], n->cinv_diag[2]),
                                        F3(n->cinv_off[0], n->cinv_off[1], n->cinv_off[2])),
                                1e-30f));
}
// a cut node refreshes its shadow and direct light when the cut was re-selected, else a quarter of them a frame
__device__ __forceinline__ bool sc_now(const BounceParams& B, uint32_t n) {
  return B.sc_reselect != 0u || n % 4u == B.frame % 4u;
}

// sc_probe_dist (bounce.wgsl:1478-1516): the smallest (distance - margin) from world point P to the gather centres of
// the probes that see part `own` (the room's nearest 2x2x2 block centre less the block radius; the terrain's 3 x 3
// columns around P; each movable part's 8 probes but own's; each static volume's nearest grid probe).  The gathers
// of probes that cut around themselves keep no margin (vol_info.y 0).  WGSL round is half to even: rintf.
__device__ float sc_probe_dist(const BounceParams& B, const float* __restrict__ ground,
                               const sl_node* __restrict__ tnodes, const sl_part* __restrict__ parts, f3 P,
                               uint32_t own) {
  float best = 1e30f;
  if (!B.terrain) {
    const float Pv[3] = {P.x, P.y, P.z};
    float b[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float nb = (float)((B.dims[a] + 1u) / 2u);
      b[a] = clampf(rintf(((Pv[a] - B.lo[a]) / fmaxf(B.step[a], 1e-6f) - 0.5f) * 0.5f), 0.0f, nb - 1.0f);
    }
    const f3 cen = F3(B.lo[0] + B.step[0] * (2.0f * b[0] + 0.5f), B.lo[1] + B.step[1] * (2.0f * b[1] + 0.5f),
                      B.lo[2] + B.step[2] * (2.0f * b[2] + 0.5f));
    best = len3(sub3(P, cen)) - B.brad;
  } else {
    const int ci = (int)clampf(rintf((P.x - B.lo[0]) / fmaxf(B.step[0], 1e-6f)), -1e9f, 1e9f);
    const int cj = (int)clampf(rintf((P.y - B.lo[1]) / fmaxf(B.step[1], 1e-6f)), -1e9f, 1e9f);
    for (int di = -1; di <= 1; di++) {
      for (int dj = -1; dj <= 1; dj++) {
        const int ii = min(max(ci + di, 0), (int)B.dims[0] - 1), jj = min(max(cj + dj, 0), (int)B.dims[1] - 1);
        const uint32_t i = (uint32_t)ii, j = (uint32_t)jj;
        const float x = B.lo[0] + B.step[0] * (float)i, y = B.lo[1] + B.step[1] * (float)j;
        const float gz = ground_at(B, ground, i, j);
        for (uint32_t k = 0; k < B.dims[2]; k++) best = fminf(best, len3(sub3(P, F3(x, y, gz + B.levels[k]))));
      }
    }
  }
  for (uint32_t q = 0; q < B.part_count && q < 32u; q++) {
    if (q == own) continue;
    const float* xf = parts[q].xf;
    if (part_probe_part(B, parts, q)) {
      f3 c, h;
      part_frame(tnodes, parts, q, c, h);
      if (len3(sub3(P, xf_point(xf, c))) - len3(h) >= best) continue;
      for (uint32_t k = 0; k < 8u; k++)
        best = fminf(best, len3(sub3(P, probe_pos(B, ground, tnodes, parts, B.NL + q * 8u + k))));
    } else if (has_vol(B, q)) {
      f3 c, h;
      vol_frame(tnodes, parts, q, c, h);
      const f3 lp = xf_dir_inv(xf, sub3(P, F3(xf[3], xf[7], xf[11])));
      const float lv[3] = {lp.x, lp.y, lp.z}, cv[3] = {c.x, c.y, c.z}, hv[3] = {h.x, h.y, h.z};
      float g[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        const float d = (float)B.vol_dims[q][a];
        const float span = fmaxf(d - 1.0f, 1.0f);
        const float ijk = clampf(rintf((lv[a] - cv[a] + hv[a]) / fmaxf(2.0f * hv[a], 1e-6f) * span), 0.0f, d - 1.0f);
        g[a] = cv[a] - hv[a] + 2.0f * hv[a] * ijk / span;
      }
      best = fminf(best, len3(sub3(lp, F3(g[0], g[1], g[2]))));
    }
  }
  return best;
}

// sc_select (bounce.wgsl:1529-1548) over one depth, the depth above already marked; the cut nodes join sc_list
__global__ void __launch_bounds__(kThreads) sc_select_kernel(const __grid_constant__ BounceParams B,
                                                             const sl_node* __restrict__ tnodes,
                                                             const sl_part* __restrict__ parts,
                                                             const float* __restrict__ ground,
                                                             const uint32_t* __restrict__ parent,
                                                             const uint32_t* __restrict__ level, uint32_t count,
                                                             uint32_t* __restrict__ flag, uint32_t* __restrict__ list) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= count) return;
  const uint32_t n = level[t];
  const sl_node& nd = tnodes[n];
  const uint32_t q = nd.part;
  uint32_t m;
  if (q >= B.part_count) {
    m = kScBelow;  // scene nodes above the parts: the gather starts at part roots
  } else if (parts[q].root != n && (parent[n] == kNone || flag[parent[n]] != kScOpen)) {
    m = kScBelow;
  } else if (n < B.G) {
    m = kScLeaf;
  } else {
    const f3 P = xf_point(parts[q].xf, F3(nd.mean[0], nd.mean[1], nd.mean[2]));
    m = sc_probe_dist(B, ground, tnodes, parts, P, q) <= kProbeTheta * nd.smax ? kScOpen : kScNode;
  }
  flag[n] = m;
  if (m == kScNode) list[1u + atomicAdd(&list[0], 1u)] = n;
}

// sc_xfer (bounce.wgsl:1631-1667): per cut node and face of its short axis, the SH2 transfer from its own V grid and
// the face's exposure (at least 1% of the whole): 6 vec4, face 0 t0-3, t4-7, (t8, S), then face 1
__global__ void __launch_bounds__(kThreads) sc_xfer_kernel(const __grid_constant__ BounceParams B,
                                                           const uint32_t* __restrict__ list,
                                                           const sl_node* __restrict__ tnodes,
                                                           const sl_gaussian* __restrict__ sc_gs,
                                                           const sl_vgrid* __restrict__ sc_vg,
                                                           const sl_part* __restrict__ parts,
                                                           const float* __restrict__ tab, float4* __restrict__ X) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= list[0]) return;
  const uint32_t n = list[1u + i], r = n - B.G;
  const sl_gaussian& G = sc_gs[r];
  const Leaf nd = load_leaf(&tnodes[n]);
  const float* xf = parts[G.part_surface & 0xFFFFu].xf;
  const f3 nrm = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]).c[0];
  const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
  const sl_vgrid& vg = sc_vg[r];
  float t[20];
#pragma unroll
  for (int m = 0; m < 20; m++) t[m] = 0.0f;
  float S0 = 0.0f;
  for (uint32_t c = 0; c < kCells; c++) {
    const f3 w = cell_dir(tab, c);
    const f3 u = xf_dir_inv(xf, w);
    const float a = footprint(nd, s3 * s3, u) * cell_omega(tab, c);
    S0 += a;
    const float v = vgrid_lookup(vg, u);
    if (v <= 0.0f) continue;
    const float h = 0.5f + 0.5f * sc_face(dot3(u, nrm));
    float y[9];
    sh2_basis(w, y);
#pragma unroll
    for (int m = 0; m < 9; m++) {
      t[m] += a * v * h * y[m];
      t[10 + m] += a * v * (1.0f - h) * y[m];
    }
    t[9] += a * v * h;
    t[19] += a * v * (1.0f - h);
  }
  const float Smin = fmaxf(0.5f * 0.02f * S0, 1e-30f);  // iso_init.wgsl ISO_EPS, per face
#pragma unroll
  for (int f = 0; f < 2; f++) {
    const float* o = t + 10 * f;
    X[8u * r + 3u * (uint32_t)f] = make_float4(o[0], o[1], o[2], o[3]);
    X[8u * r + 3u * (uint32_t)f + 1u] = make_float4(o[4], o[5], o[6], o[7]);
    X[8u * r + 3u * (uint32_t)f + 2u] = make_float4(o[8], fmaxf(o[9], Smin), 0.0f, 0.0f);
  }
}

// sc_shadow (bounce.wgsl:1566-1624): the mean lamp T and distant-light T of 8 leaves under the cut node, each reached
// by a descent that picks a child with probability by mass (a fixed hash per node and sample).  A Gaussian carries
// one lamp T here, so the reference's per-lamp slots reduce to that mean.
__global__ void __launch_bounds__(kThreads) sc_shadow_kernel(const __grid_constant__ BounceParams B,
                                                             const uint32_t* __restrict__ list,
                                                             const sl_node* __restrict__ tnodes,
                                                             const uint32_t* __restrict__ kids,
                                                             const float* __restrict__ lamp_T,
                                                             const float4* __restrict__ env_T,
                                                             float* __restrict__ sc_T, float4* __restrict__ sc_E) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= list[0]) return;
  const uint32_t n = list[1u + i];
  if (!sc_now(B, n)) return;
  float T = 0.0f;
  float4 E = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  for (uint32_t s = 0; s < 8u; s++) {
    uint32_t m = n, h = pcg_hash(n * 8u + s);
    for (uint32_t it = 0; it < 64u && m >= B.G; it++) {
      const uint32_t lo = tnodes[m].child_lo, hi = tnodes[m].child_hi;
      if (hi <= lo) break;  // no children to descend into: the sample counts T = 1
      float tot = 0.0f;
      for (uint32_t j = lo; j < hi; j++) tot += sc_mass(&tnodes[kids[j]]);
      float u = to_unit(h) * tot;
      h = pcg_hash(h);
      uint32_t pick = kids[lo];
      for (uint32_t j = lo; j < hi; j++) {
        pick = kids[j];
        u -= sc_mass(&tnodes[kids[j]]);
        if (u <= 0.0f) break;
      }
      m = pick;
    }
    // the tree is at most 64 levels deep (sl_lighting_set_sender_cut), so m is a leaf
    const float4 e = m < B.G ? env_T[m] : make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    T += m < B.G ? lamp_T[m] : 1.0f;
    E.x += e.x;
    E.y += e.y;
    E.z += e.z;
    E.w += e.w;
  }
  const uint32_t r = n - B.G;
  sc_T[r] = T / 8.0f;
  sc_E[r] = make_float4(E.x / 8.0f, E.y / 8.0f, E.z / 8.0f, E.w / 8.0f);
}

// node_cut (bounce.wgsl:1669-1712): a cut node as one sender, each face's light (its direct light plus the probes'
// SH2 at its centre through the face's transfer, over the face's exposure) shown toward each D_k by its share there
__global__ void __launch_bounds__(kThreads) node_cut_kernel(const __grid_constant__ BounceParams B,
                                                            const uint32_t* __restrict__ list,
                                                            const sl_node* __restrict__ tnodes,
                                                            const sl_gaussian* __restrict__ sc_gs,
                                                            const sl_vgrid* __restrict__ sc_vg,
                                                            const sl_part* __restrict__ parts,
                                                            const float* __restrict__ tab,
                                                            const float* __restrict__ ground,
                                                            const float4* __restrict__ pd,
                                                            const float4* __restrict__ probe_sh,
                                                            const float4* __restrict__ X, float4* __restrict__ acc) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= list[0]) return;
  const uint32_t n = list[1u + i], r = n - B.G;
  const sl_gaussian& G = sc_gs[r];
  const Leaf nd = load_leaf(&tnodes[n]);
  const uint32_t own = G.part_surface & 0xFFFFu;
  const float* xf = parts[own].xf;
  const f3 P = xf_point(xf, F3(G.mu[0], G.mu[1], G.mu[2]));
  const f3 nrm = quat_matrix(G.quat[0], G.quat[1], G.quat[2], G.quat[3]).c[0];
  const float s3 = G.scale[0] * G.scale[1] * G.scale[2];
  const Weights pw = weights_for(B, ground, pd, tnodes, parts, P, own);
  f3 Lsh[9];
#pragma unroll
  for (int m = 0; m < 9; m++) Lsh[m] = F3(0.0f, 0.0f, 0.0f);
  for (int k = 0; k < 8; k++) {
    const float w = pw.w[k];
    if (w <= 0.0f) continue;
#pragma unroll
    for (int m = 0; m < 9; m++) {
      const float4 c = probe_sh[9u * pw.pid[k] + (uint32_t)m];
      Lsh[m] = add3(Lsh[m], mul3(F3(c.x, c.y, c.z), w));
    }
  }
  const f3 alb = F3(G.albedo[0], G.albedo[1], G.albedo[2]);
  f3 col[2];
#pragma unroll
  for (int f = 0; f < 2; f++) {
    const float4 a = X[8u * r + 3u * (uint32_t)f], b = X[8u * r + 3u * (uint32_t)f + 1u],
                 c = X[8u * r + 3u * (uint32_t)f + 2u], d = X[8u * r + 6u + (uint32_t)f];
    const float x[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
    f3 Bv = mul3(Lsh[0], x[0]);
#pragma unroll
    for (int m = 1; m < 9; m++) Bv = add3(Bv, mul3(Lsh[m], x[m]));
    col[f] = div3(mul3v(alb, max0(add3(F3(d.x, d.y, d.z), max0(Bv)))), c.y);
  }
  const bool dark = own == B.dark_part;
  const sl_vgrid& vg = sc_vg[r];
  for (int k = 0; k < 14; k++) {
    const f3 wo = xf_dir_inv(xf, ld3(tab + kTabD14 + 3 * k));
    const float w = footprint(nd, s3 * s3, wo) * vgrid_lookup(vg, wo);
    const float h = 0.5f + 0.5f * sc_face(dot3(wo, nrm));
    const f3 L = dark ? F3(0.0f, 0.0f, 0.0f) : add3(mul3(col[0], h), mul3(col[1], 1.0f - h));
    acc[14u * n + (uint32_t)k] = make_float4(L.x * w, L.y * w, L.z * w, w);
  }
}

inline uint32_t blocks(uint64_t n) { return (uint32_t)((n + kThreads - 1) / kThreads); }

}  // namespace

cudaError_t launch_bounce_frame(const BounceParams& B, const ShadeParams& SH, const BounceBuffers& D,
                                const std::vector<uint32_t>& level_off, const std::vector<uint32_t>& level_cnt,
                                const std::vector<uint32_t>& sc_off, const std::vector<uint32_t>& sc_cnt,
                                cudaStream_t s) {
  if (B.G == 0) return cudaSuccess;
  // iso_xfer only where something may have changed a transfer: a forced refresh or a part that moved (lighting.js
  // :1036-1039 skips the dispatch otherwise)
  if (B.force || B.moved_mask)
    xfer_kernel<<<blocks(B.G), kThreads, 0, s>>>(B, D.gs, D.nodes, D.vgrid, D.parts, D.tab, D.xfer, D.leaf_w);
  // the sender cut: selected again top down when a part moved (or on its first frame), with the cut nodes'
  // transfer; then the shadow T of the cut nodes that refresh this frame.  Its kernels run over every internal node's
  // slot and stop past the cut's count.
  const bool sc = B.sender_cut != 0u;
  const uint32_t I = B.N - B.G;
  const uint32_t* flag = sc ? D.sc_flag : nullptr;
  if (sc && B.sc_reselect) {
    cudaMemsetAsync(D.sc_list, 0, 4, s);
    for (size_t d = 0; d < sc_cnt.size(); d++) {
      if (sc_cnt[d] == 0) continue;
      sc_select_kernel<<<blocks(sc_cnt[d]), kThreads, 0, s>>>(B, D.tnodes, D.parts, D.ground, D.parent,
                                                              D.sc_level + sc_off[d], sc_cnt[d], D.sc_flag, D.sc_list);
    }
    if (I) sc_xfer_kernel<<<blocks(I), kThreads, 0, s>>>(B, D.sc_list, D.tnodes, D.sc_gs, D.sc_vg, D.parts, D.tab,
                                                          D.sc_X);
  }
  if (sc && I)
    sc_shadow_kernel<<<blocks(I), kThreads, 0, s>>>(B, D.sc_list, D.tnodes, D.kids, D.lamp_T, D.env_T, D.sc_T,
                                                    D.sc_E);
  cudaError_t e = launch_bounce_direct(B, SH, D, s);
  if (e != cudaSuccess) return e;
  leaf_kernel<<<blocks(B.G), kThreads, 0, s>>>(B, D.gs, D.leaf_w, D.lo_dir, D.lo_b, flag, D.node_acc);
  if (sc && I)
    node_cut_kernel<<<blocks(I), kThreads, 0, s>>>(B, D.sc_list, D.tnodes, D.sc_gs, D.sc_vg, D.parts, D.tab,
                                                   D.ground, D.probe_data, D.probe_sh, D.sc_X, D.node_acc);
  for (int d = (int)level_cnt.size() - 1; d >= 1; d--) {
    const uint32_t n = level_cnt[(size_t)d];
    if (n == 0) continue;
    up_kernel<<<blocks(14ull * n), kThreads, 0, s>>>(D.tnodes, D.kids, D.up_list + level_off[(size_t)d], n, flag,
                                                     D.node_acc);
  }
  sh2_kernel<<<blocks(B.N), kThreads, 0, s>>>(B.N, D.tab, D.node_acc, flag, D.node_sh);
  if (B.NP) {
    gather_kernel<<<blocks((uint64_t)B.NP * kCells), kThreads, 0, s>>>(B, D.tnodes, D.kids, D.vgrid, D.parts, D.tab,
                                                                       D.ground, D.node_sh, D.probe_data,
                                                                       D.probe_hist);
    valid_kernel<<<blocks(B.NP), kThreads, 0, s>>>(B, D.parts, D.probe_data);
    psh2_kernel<<<blocks(B.NP), kThreads, 0, s>>>(B, D.tab, D.probe_data, D.probe_sh);
  }
  dirs_kernel<<<blocks(B.G), kThreads, 0, s>>>(B, D.gs, D.nodes, D.vgrid, D.parts, D.mats, D.tnodes, D.tab, D.ground,
                                               D.probe_data, D.lo_b);
  bounce_kernel<<<blocks(B.G), kThreads, 0, s>>>(B, D.gs, D.nodes, D.vgrid, D.parts, D.mats, D.tnodes, D.ground,
                                                 D.probe_data,
                                                 D.probe_sh, D.xfer, D.lo_b);
  return cudaGetLastError();
}

}  // namespace sl
