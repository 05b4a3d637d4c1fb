/*
 * sl_oracle.c -- CPU restatement of the reference splat pipeline (project -> stable radix order -> tile binning ->
 * back-to-front composite).  TEST INFRASTRUCTURE: only tests/, the smoke check and the benchmark's CPU-baseline
 * leg load this library; the product path never does.
 *
 * How it is pinned: the reference is WGSL on WebGPU (no graphics stack here to run it) and ships no tests or golden
 * vectors; it does ship two gs-runtime scenes (runtime/assets/cornell_sdf_room_plain_bin, hill_lite_bin).  This
 * restatement renders both as the reference's page shows them, and the GPU path is checked against it on both
 * (tests/test_gpu_assets.py); beside that, reading the cited lines, float64 brute-force and known-answer checks
 * (tests/test_oracle*.py) and the regression fixtures tests/golden/*.npz (tests/golden/make_golden.py).
 *
 * Arithmetic contract (shared with the CUDA kernels; both follow it independently):
 *   - fp32 throughout, compiled with -ffp-contract=off: every a*b+c below rounds twice unless written as fmaf();
 *   - sums and dot products evaluate left to right; matrix-vector products as col0*v.x + col1*v.y + col2*v.z;
 *   - normalize(v) = v / sqrt(dot(v, v)); natural log and exp come from sl_detmath.h (same bits as the device);
 *   - the fragment keep test alpha >= 1/255 is evaluated in its closed form q <= qcut = 2 ln(tau0 / tau_min), the
 *     bound shaders/project.wgsl:290-295 derives for the quad radius (r = sqrt(qcut)); in real arithmetic the two
 *     are the same test, in fp32 they can differ only for fragments whose alpha rounds to within an ulp of 1/255.
 *     The quad (|local| <= r per axis) circumscribes that ellipse, so it removes nothing the keep test keeps, up to
 *     the same rounding; it is therefore not tested separately.
 * Pixel geometry: framebuffer pixel (ix, iy), iy down from the top, centre (ix + 0.5, iy + 0.5); a splat's Mahalanobis
 * offset at a pixel is local = (d . g0, d . g1) with g = a r / |a|^2 per quad axis a in pixels -- the grad varying of
 * shaders/splat.wgsl:44-46 -- which equals the quad's interpolated `local` (shaders/splat.wgsl:43) in real arithmetic.
 */
#include "sl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "sl_detmath.h"
#include "sl_tilespan.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_INVALID 0xffffffffu
#define ORC_EMITTER_MATERIAL 254u
#define ORC_MAX_PARTS 32u
#define ORC_PART_HIDDEN 4u

typedef struct { float x, y, z; } v3;
typedef struct { v3 c[3]; } m3; /* columns */

static v3 v3_make(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static float v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 v3_scale(v3 a, float s) { return v3_make(a.x * s, a.y * s, a.z * s); }
/* M v = col0*v.x + col1*v.y + col2*v.z, per component left to right */
static v3 m3_mul_v(m3 m, v3 v) {
  return v3_make(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z,
                 m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
                 m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z);
}
static m3 m3_mul(m3 a, m3 b) {
  m3 r;
  for (int j = 0; j < 3; j++) r.c[j] = m3_mul_v(a, b.c[j]);
  return r;
}
/* M^T v: component k = dot(col_k, v) */
static v3 m3_tmul_v(m3 m, v3 v) { return v3_make(v3_dot(m.c[0], v), v3_dot(m.c[1], v), v3_dot(m.c[2], v)); }

/* quat_to_mat, shaders/common.wgsl:83-89 (columns) */
static m3 quat_to_mat(const float q[4]) {
  float x = q[0], y = q[1], z = q[2], w = q[3];
  m3 m;
  m.c[0] = v3_make(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + w * z), 2.0f * (x * z - w * y));
  m.c[1] = v3_make(2.0f * (x * y - w * z), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + w * x));
  m.c[2] = v3_make(2.0f * (x * z + w * y), 2.0f * (y * z - w * x), 1.0f - 2.0f * (x * x + y * y));
  return m;
}

/* part_rotation = transpose(mat3(xf[0].xyz, xf[1].xyz, xf[2].xyz)), shaders/common.wgsl:96-98 */
static m3 part_rotation(const sl_part* p) {
  m3 m;
  for (int c = 0; c < 3; c++) m.c[c] = v3_make(p->xf[0 * 4 + c], p->xf[1 * 4 + c], p->xf[2 * 4 + c]);
  return m;
}

/* part_apply: dot(xf[r], vec4(x, 1)), shaders/common.wgsl:100-103 */
static v3 part_apply(const sl_part* p, const float x[3]) {
  float o[3];
  for (int r = 0; r < 3; r++) {
    const float* a = p->xf + 4 * r;
    o[r] = a[0] * x[0] + a[1] * x[1] + a[2] * x[2] + a[3] * 1.0f;
  }
  return v3_make(o[0], o[1], o[2]);
}

/* the same with the pose at the start of the exposure (xf_prev), for motion blur (shaders/project.wgsl:140-145) */
static v3 part_apply_prev(const sl_part* p, const float x[3]) {
  float o[3];
  for (int r = 0; r < 3; r++) {
    const float* a = p->xf_prev + 4 * r;
    o[r] = a[0] * x[0] + a[1] * x[1] + a[2] * x[2] + a[3] * 1.0f;
  }
  return v3_make(o[0], o[1], o[2]);
}

/* palette_slot, shaders/project.wgsl:27-31 */
static const float* palette_slot(const sl_render_frame* f, uint32_t m) {
  static const float white0[4] = {1.0f, 1.0f, 1.0f, 0.0f};
  if (m < 3u) return f->palette[m];
  if (m >= 4u && m < 8u) return f->palette_ext[m - 4u];
  return white0;
}

static float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

/* one slot of shaders/project.wgsl main (:84-370), plain path; returns the key */
static uint32_t project_one(uint32_t i, const sl_gaussian* gaussians, uint32_t count, const sl_part* parts,
                            const sl_gaussian* emitters, const float* colour, const float* lo_b,
                            const sl_render_frame* f, orc_splat* out, const orc_lod* lod) {
  memset(out, 0, sizeof(*out));
  out->ix0 = 1;
  out->ix1 = 0;
  uint32_t n_emit = (uint32_t)f->palette[3][1];
  /* screen-space LOD (:90-109): slots from the node base are the tree's internal nodes, drawn when in the cut; leaves
   * are drawn when in the cut */
  uint32_t node = 0xFFFFFFFFu;
  if (lod && i >= lod->node_base) {
    node = i - lod->node_base;
    if (node >= lod->n_int || lod->flags[count + node] != 2u) return ORC_INVALID;
  } else {
    if (i == count || i > count + n_emit) return ORC_INVALID;
    if (lod && i < count && lod->flags[i] != 2u) return ORC_INVALID;
  }

  const sl_gaussian* g;
  v3 mu;
  m3 rot;
  uint32_t material = ORC_EMITTER_MATERIAL;
  float keep = 1.0f;
  v3 vel = v3_make(0.0f, 0.0f, 0.0f);
  if (i > count && node == 0xFFFFFFFFu) { /* :123-127 */
    g = &emitters[i - count - 1u];
    mu = v3_make(g->mu[0], g->mu[1], g->mu[2]);
    rot = quat_to_mat(g->quat);
  } else { /* :128-149 */
    g = node != 0xFFFFFFFFu ? &lod->nodes[node] : &gaussians[i];
    uint32_t part = g->part_surface & 0xffffu;
    if (part > ORC_MAX_PARTS - 1u) part = ORC_MAX_PARTS - 1u;
    const sl_part* p = &parts[part];
    if ((p->flags & ORC_PART_HIDDEN) != 0u) return ORC_INVALID;
    keep = 1.0f - clampf(f->part_fade[part], 0.0f, 1.0f);
    if (keep <= 0.0f) return ORC_INVALID;
    mu = part_apply(p, g->mu);
    rot = m3_mul(part_rotation(p), quat_to_mat(g->quat));
    material = part < 16u ? f->part_material[part] : f->part_material_ext[part - 16u];
    /* motion blur (:138-146): a box-shutter average of the move over the exposure, centred mid-exposure */
    float shutter = f->palette[3][2];
    if (shutter > 0.0f && (p->flags & 2u) != 0u) {
      v3 prev = part_apply_prev(p, g->mu);
      vel = v3_make(shutter * (mu.x - prev.x), shutter * (mu.y - prev.y), shutter * (mu.z - prev.z));
      mu = v3_make(mu.x - 0.5f * vel.x, mu.y - 0.5f * vel.y, mu.z - 0.5f * vel.z);
    }
  }

  /* tv = view * vec4(mu, 1) (:263) */
  const float* V = f->view;
  v3 tv = v3_make(V[0] * mu.x + V[4] * mu.y + V[8] * mu.z + V[12] * 1.0f,
                  V[1] * mu.x + V[5] * mu.y + V[9] * mu.z + V[13] * 1.0f,
                  V[2] * mu.x + V[6] * mu.y + V[10] * mu.z + V[14] * 1.0f);
  float depth = -tv.z;
  if (depth < f->near_plane || depth > f->far_plane) return ORC_INVALID; /* :199-200 */

  /* view-space covariance W R S^2 R^T W^T (:202-206) */
  m3 W;
  W.c[0] = v3_make(V[0], V[1], V[2]);
  W.c[1] = v3_make(V[4], V[5], V[6]);
  W.c[2] = v3_make(V[8], V[9], V[10]);
  m3 wr = m3_mul(W, rot);
  v3 s2 = v3_make(g->scale[0] * g->scale[0], g->scale[1] * g->scale[1], g->scale[2] * g->scale[2]);
  m3 m;
  m.c[0] = v3_scale(wr.c[0], g->scale[0]);
  m.c[1] = v3_scale(wr.c[1], g->scale[1]);
  m.c[2] = v3_scale(wr.c[2], g->scale[2]);
  float cv[3][3]; /* cv[row][col] = sum_k m_k[row] m_k[col] */
  {
    const float* mk[3] = {&m.c[0].x, &m.c[1].x, &m.c[2].x};
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) cv[r][c] = mk[0][r] * mk[0][c] + mk[1][r] * mk[1][c] + mk[2][r] * mk[2][c];
  }
  /* the sharp covariance (coverage cap); blurred: + (W vel)(W vel)^T / 12 (:208-210) */
  int blurred = vel.x != 0.0f || vel.y != 0.0f || vel.z != 0.0f;
  m3 cov_s;
  for (int c = 0; c < 3; c++) cov_s.c[c] = v3_make(cv[0][c], cv[1][c], cv[2][c]);
  if (blurred) {
    v3 wv = m3_mul_v(W, vel);
    float w3[3] = {wv.x, wv.y, wv.z};
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) cv[r][c] = cv[r][c] + (w3[r] * w3[c]) * (1.0f / 12.0f);
  }
  m3 cov;
  for (int c = 0; c < 3; c++) cov.c[c] = v3_make(cv[0][c], cv[1][c], cv[2][c]);

  /* EWA Jacobian, pixel units, y up (:212-232) */
  float fx = f->focal[0], fy = f->focal[1];
  float iz = 1.0f / depth;
  float px = fx * tv.x * iz;
  float py = fy * tv.y * iz;
  float limx = 1.3f * f->viewport[0] * 0.5f;
  float limy = 1.3f * f->viewport[1] * 0.5f;
  float cxv = clampf(tv.x * iz, -limx / fx, limx / fx) * depth;
  float cyv = clampf(tv.y * iz, -limy / fy, limy / fy) * depth;
  v3 j0 = v3_make(fx * iz, 0.0f, fx * cxv * iz * iz);
  v3 j1 = v3_make(0.0f, fy * iz, fy * cyv * iz * iz);
  v3 cj0 = m3_mul_v(cov, j0);
  v3 cj1 = m3_mul_v(cov, j1);
  float a = v3_dot(j0, cj0);
  float b = v3_dot(j0, cj1);
  float c = v3_dot(j1, cj1);
  float det0 = a * c - b * b;
  a += f->lowpass_px2;
  c += f->lowpass_px2;
  float det = a * c - b * b;
  if (det <= 0.0f) return ORC_INVALID;

  /* volumetric peak optical depth (:234-261) */
  float dlen = sqrtf(v3_dot(tv, tv));
  v3 d = v3_make(tv.x / dlen, tv.y / dlen, tv.z / dlen);
  v3 dl = m3_tmul_v(wr, d);
  v3 is2 = v3_make(1.0f / s2.x, 1.0f / s2.y, 1.0f / s2.z);
  float q = v3_dot(v3_make(dl.x * dl.x, dl.y * dl.y, dl.z * dl.z), is2);
  float q_s = q, kappa = g->kappa;
  if (blurred) { /* Sherman-Morrison for q, the determinant lemma for kappa (:242-250) */
    v3 vl = m3_tmul_v(rot, vel);
    float mv2 = v3_dot(v3_make(vl.x * vl.x, vl.y * vl.y, vl.z * vl.z), is2);
    float dv = v3_dot(v3_make(dl.x * vl.x, dl.y * vl.y, dl.z * vl.z), is2);
    q -= dv * dv / (12.0f + mv2);
    kappa /= sqrtf(1.0f + mv2 / 12.0f);
  }
  const float kTwoPi = 6.283185307f;
  float tau0 = kappa * sqrtf(kTwoPi / q) * sqrtf(fmaxf(det0, 0.0f) / det);
  if (blurred && f->palette[3][3] > 0.5f) { /* coverage cap (:251-268) */
    v3 cs0 = m3_mul_v(cov_s, j0), cs1 = m3_mul_v(cov_s, j1);
    float a_s = v3_dot(j0, cs0) + f->lowpass_px2;
    float b_s = v3_dot(j0, cs1);
    float c_s = v3_dot(j1, cs1) + f->lowpass_px2;
    float det0_s = (a_s - f->lowpass_px2) * (c_s - f->lowpass_px2) - b_s * b_s;
    float det_s = a_s * c_s - b_s * b_s;
    float tau_s = g->kappa * sqrtf(kTwoPi / q_s) * sqrtf(fmaxf(det0_s, 0.0f) / det_s);
    float ap = (1.0f - sl_expf(-tau_s)) * sqrtf(det_s / det);
    float tc = -sl_logf(fmaxf(1.0f - ap, 1e-6f));
    tau0 = fminf(tau0, tc);
  }
  tau0 *= keep; /* :384 */

  /* cutoff radius (:290-295) */
  const float kAlphaMin = 1.0f / 255.0f;
  float tau_min = -sl_logf(1.0f - kAlphaMin);
  float tau_cut = tau0;
  if (tau_cut <= tau_min) return ORC_INVALID;
  float qcut = 2.0f * sl_logf(tau_cut / tau_min);
  float r = sqrtf(qcut);

  /* eigen-axes of the 2x2 covariance (:297-309) */
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
  float tnx = 2.0f / f->viewport[0], tny = 2.0f / f->viewport[1];
  float ax0 = e0x * sl0 * r * tnx, ay0 = e0y * sl0 * r * tny;
  float ax1 = e1x * sl1 * r * tnx, ay1 = e1y * sl1 * r * tny;
  if (sl0 * r < 0.1f) return ORC_INVALID; /* :310-311 */
  float ccx = px * tnx, ccy = py * tny;   /* :313-315 */
  float extx = fabsf(ax0) + fabsf(ax1), exty = fabsf(ay0) + fabsf(ay1);
  if (fabsf(ccx) - extx > 1.0f || fabsf(ccy) - exty > 1.0f) return ORC_INVALID;

  /* colour (:317-350) */
  float rgb[3] = {g->albedo[0], g->albedo[1], g->albedo[2]};
  if (material == ORC_EMITTER_MATERIAL) {
    /* emitted radiance, shown as itself */
  } else if (f->view_mode == 3u) {
    float gain = f->palette[3][0];
    for (int k = 0; k < 3; k++) {
      if (node != 0xFFFFFFFFu) { /* a drawn node's lit colour, bounce included (lod_colour) */
        rgb[k] = lod->colour[4u * node + (uint32_t)k];
        continue;
      }
      float cl = colour ? colour[4u * i + (uint32_t)k] : 0.0f;
      float bo = lo_b ? lo_b[12u * i + (uint32_t)k] : 0.0f;
      rgb[k] = cl + gain * bo;
    }
    if (material < 8u) {
      const float* ps = palette_slot(f, material);
      for (int k = 0; k < 3; k++) rgb[k] *= ps[k];
    }
  } else if (material < 8u && palette_slot(f, material)[3] > 0.5f) {
    const float* ps = palette_slot(f, material);
    for (int k = 0; k < 3; k++) rgb[k] = ps[k];
  }
  if (material != ORC_EMITTER_MATERIAL)
    for (int k = 0; k < 3; k++) rgb[k] *= f->albedo_scale;

  /* 16-bit log-depth key (:363-369) */
  float lnr = sl_logf(f->far_plane / f->near_plane);
  float t = clampf(sl_logf(depth / f->near_plane) / lnr, 0.0f, 1.0f);
  uint32_t key = 65535u - (uint32_t)(t * 65535.0f + 0.5f);
  if (key > 0xfffeu) key = 0xfffeu;
  if (f->view_mode == 1u) /* depth view: splat.wgsl:28, 38-41, 76 */
    for (int k = 0; k < 3; k++) rgb[k] = 1.0f - t;

  /* pixel-space splat: centre, grad rows (splat.wgsl:44-46), y flipped to framebuffer rows */
  float W_ = f->viewport[0], H_ = f->viewport[1];
  out->cx = px + 0.5f * W_;
  out->cy = 0.5f * H_ - py;
  float a0x = e0x * sl0 * r, a0y = e0y * sl0 * r;
  float a1x = e1x * sl1 * r, a1y = e1y * sl1 * r;
  float n0 = fmaxf(a0x * a0x + a0y * a0y, 1e-12f);
  float n1 = fmaxf(a1x * a1x + a1y * a1y, 1e-12f);
  out->g0x = a0x * r / n0;
  out->g0y = -(a0y * r / n0);
  out->g1x = a1x * r / n1;
  out->g1y = -(a1y * r / n1);
  out->r = r;
  out->qcut = qcut;
  out->tau0 = tau0;
  out->rgb[0] = rgb[0];
  out->rgb[1] = rgb[1];
  out->rgb[2] = rgb[2];
  /* candidate pixels: the bounding box of the ellipse q <= r^2 (half widths r sqrt(a), r sqrt(c)) plus one pixel */
  float hx = r * sqrtf(a) + 1.0f, hy = r * sqrtf(c) + 1.0f;
  float xl = fmaxf(out->cx - hx - 0.5f, -1.0f), xh = fminf(out->cx + hx - 0.5f, W_);
  float yl = fmaxf(out->cy - hy - 0.5f, -1.0f), yh = fminf(out->cy + hy - 0.5f, H_);
  int32_t ix0 = (int32_t)ceilf(xl), ix1 = (int32_t)floorf(xh);
  int32_t iy0 = (int32_t)ceilf(yl), iy1 = (int32_t)floorf(yh);
  if (ix0 < 0) ix0 = 0;
  if (iy0 < 0) iy0 = 0;
  if (ix1 > (int32_t)W_ - 1) ix1 = (int32_t)W_ - 1;
  if (iy1 > (int32_t)H_ - 1) iy1 = (int32_t)H_ - 1;
  out->ix0 = ix0;
  out->ix1 = ix1;
  out->iy0 = iy0;
  out->iy1 = iy1;
  out->valid = 1;
  return key;
}

uint32_t orc_project_lod(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                         const sl_gaussian* emitters, const float* colour, const float* lo_b,
                         const sl_render_frame* frame, uint32_t n_slots, uint32_t* keys, orc_splat* splats,
                         int nthreads, const orc_lod* lod) {
  (void)part_count;
  uint32_t visible = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static, 4096) reduction(+ : visible)
#endif
  for (int64_t i = 0; i < (int64_t)n_slots; i++) {
    uint32_t k = project_one((uint32_t)i, gaussians, count, parts, emitters, colour, lo_b, frame, &splats[i], lod);
    keys[i] = k;
    if (k != ORC_INVALID) visible++;
  }
  return visible;
}

uint32_t orc_project(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                     const sl_gaussian* emitters, const float* colour, const float* lo_b,
                     const sl_render_frame* frame, uint32_t n_slots, uint32_t* keys, orc_splat* splats, int nthreads) {
  return orc_project_lod(gaussians, count, parts, part_count, emitters, colour, lo_b, frame, n_slots, keys, splats,
                         nthreads, NULL);
}

/* radix.wgsl: two stable 8-bit LSD passes over the low 16 key bits (shift 0 then 8, :44-59); the composition of
 * two stable passes is the stable order by the 16-bit key, which a single stable counting pass gives directly. */
void orc_sort16(const uint32_t* keys, uint32_t n, uint32_t* order) {
  uint32_t* hist = (uint32_t*)calloc(65537u, sizeof(uint32_t));
  for (uint32_t i = 0; i < n; i++) hist[(keys[i] & 0xffffu) + 1u]++;
  for (uint32_t d = 0; d < 65536u; d++) hist[d + 1u] += hist[d];
  for (uint32_t i = 0; i < n; i++) order[hist[keys[i] & 0xffffu]++] = i;
  free(hist);
}

/* Per-tile lists: every visible splat, in back-to-front order, joins the list of each tile its ellipse can reach
 * (sl_tilespan.h: per row of tiles inside its candidate rectangle, the columns the ellipse spans over that row). */
int64_t orc_bin(const orc_splat* splats, const uint32_t* order, uint32_t visible, uint32_t width, uint32_t height,
                uint32_t tile_w, uint32_t tile_h, uint32_t* ranges, uint32_t* entries, uint64_t cap) {
  uint32_t ntx = (width + tile_w - 1u) / tile_w, nty = (height + tile_h - 1u) / tile_h;
  uint32_t ntiles = ntx * nty;
  uint64_t* cnt = (uint64_t*)calloc((size_t)ntiles + 1u, sizeof(uint64_t));
  for (uint32_t p = 0; p < visible; p++) {
    const orc_splat* s = &splats[order[p]];
    if (s->ix0 > s->ix1 || s->iy0 > s->iy1) continue;
    for (uint32_t ty = (uint32_t)s->iy0 / tile_h; ty <= (uint32_t)s->iy1 / tile_h; ty++) {
      uint32_t t0, t1;
      if (!sl_row_tiles(s->cx, s->cy, s->g0x, s->g0y, s->g1x, s->g1y, s->qcut, (uint32_t)s->ix0 / tile_w,
                        (uint32_t)s->ix1 / tile_w, ty, tile_w, tile_h, &t0, &t1))
        continue;
      for (uint32_t tx = t0; tx <= t1; tx++) cnt[ty * ntx + tx + 1u]++;
    }
  }
  for (uint32_t t = 0; t < ntiles; t++) cnt[t + 1u] += cnt[t];
  uint64_t total = cnt[ntiles];
  if (ranges)
    for (uint32_t t = 0; t < ntiles; t++) {
      ranges[2u * t] = (uint32_t)cnt[t];
      ranges[2u * t + 1u] = (uint32_t)cnt[t + 1u];
    }
  if (entries) {
    if (total > cap) {
      free(cnt);
      return -1;
    }
    for (uint32_t p = 0; p < visible; p++) {
      const orc_splat* s = &splats[order[p]];
      if (s->ix0 > s->ix1 || s->iy0 > s->iy1) continue;
      for (uint32_t ty = (uint32_t)s->iy0 / tile_h; ty <= (uint32_t)s->iy1 / tile_h; ty++) {
        uint32_t t0, t1;
        if (!sl_row_tiles(s->cx, s->cy, s->g0x, s->g0y, s->g1x, s->g1y, s->qcut, (uint32_t)s->ix0 / tile_w,
                          (uint32_t)s->ix1 / tile_w, ty, tile_w, tile_h, &t0, &t1))
          continue;
        for (uint32_t tx = t0; tx <= t1; tx++) entries[cnt[ty * ntx + tx]++] = order[p];
      }
    }
  }
  free(cnt);
  return (int64_t)total;
}

int orc_row_tiles(const orc_splat* s, uint32_t ty, uint32_t tile_w, uint32_t tile_h, uint32_t* t0, uint32_t* t1) {
  return sl_row_tiles(s->cx, s->cy, s->g0x, s->g0y, s->g1x, s->g1y, s->qcut, (uint32_t)s->ix0 / tile_w,
                      (uint32_t)s->ix1 / tile_w, ty, tile_w, tile_h, t0, t1);
}

void orc_composite(const orc_splat* splats, const uint32_t* order, uint32_t visible, uint32_t width,
                   uint32_t height, float* rgba, uint32_t* counts, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (rgba) memset(rgba, 0, sizeof(float) * 4u * width * height);
  if (counts) memset(counts, 0, sizeof(uint32_t) * width * height);
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num(), nt = omp_get_num_threads();
#else
    int tid = 0, nt = 1;
#endif
    int32_t y_lo = (int32_t)((uint64_t)height * (uint64_t)tid / (uint64_t)nt);
    int32_t y_hi = (int32_t)((uint64_t)height * (uint64_t)(tid + 1) / (uint64_t)nt) - 1;
    for (uint32_t p = 0; p < visible; p++) { /* ascending key = far to near: back to front */
      const orc_splat* s = &splats[order[p]];
      if (s->ix0 > s->ix1) continue;
      int32_t ya = s->iy0 > y_lo ? s->iy0 : y_lo;
      int32_t yb = s->iy1 < y_hi ? s->iy1 : y_hi;
      for (int32_t iy = ya; iy <= yb; iy++) {
        float dy = ((float)iy + 0.5f) - s->cy;
        for (int32_t ix = s->ix0; ix <= s->ix1; ix++) {
          float dx = ((float)ix + 0.5f) - s->cx;
          float lx = fmaf(dx, s->g0x, dy * s->g0y);
          float ly = fmaf(dx, s->g1x, dy * s->g1y);
          float q = fmaf(lx, lx, ly * ly);
          if (q > s->qcut) continue; /* alpha < 1/255: discarded (splat.wgsl:73) */
          size_t pix = (size_t)iy * width + (size_t)ix;
          if (counts) counts[pix]++;
          if (rgba) {
            float e = sl_expf(-0.5f * q);
            float alpha = 1.0f - sl_expf(-(s->tau0 * e));
            float om = 1.0f - alpha;
            float* o = rgba + 4u * pix;
            /* premultiplied over: dst = (rgb alpha, alpha) + dst (1 - alpha) (src/renderer.js:140-142) */
            o[0] = s->rgb[0] * alpha + o[0] * om;
            o[1] = s->rgb[1] * alpha + o[1] * om;
            o[2] = s->rgb[2] * alpha + o[2] * om;
            o[3] = alpha + o[3] * om;
          }
        }
      }
    }
  }
}

int64_t orc_render_lod(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                       const sl_gaussian* emitters, const float* colour, const float* lo_b,
                       const sl_render_frame* frame, uint32_t tile_w, uint32_t tile_h,
                       uint32_t* keys, uint32_t* order, uint32_t* ranges, uint32_t* entries, uint64_t entries_cap,
                       uint64_t* n_entries, float* rgba, uint32_t* counts, int nthreads, const orc_lod* lod) {
  uint32_t n_emit = (uint32_t)frame->palette[3][1];
  uint32_t n = lod ? lod->node_base + lod->n_int : count + 1u + n_emit;
  uint32_t W = (uint32_t)frame->viewport[0], H = (uint32_t)frame->viewport[1];
  uint32_t* k = keys ? keys : (uint32_t*)malloc(sizeof(uint32_t) * n);
  uint32_t* o = order ? order : (uint32_t*)malloc(sizeof(uint32_t) * n);
  orc_splat* s = (orc_splat*)malloc(sizeof(orc_splat) * n);
  uint32_t visible =
      orc_project_lod(gaussians, count, parts, part_count, emitters, colour, lo_b, frame, n, k, s, nthreads, lod);
  orc_sort16(k, n, o);
  int64_t ne = orc_bin(s, o, visible, W, H, tile_w, tile_h, ranges, entries, entries_cap);
  if (n_entries) *n_entries = ne < 0 ? 0 : (uint64_t)ne;
  if (rgba || counts) orc_composite(s, o, visible, W, H, rgba, counts, nthreads);
  free(s);
  if (!keys) free(k);
  if (!order) free(o);
  return ne < 0 ? -8 : (int64_t)visible;
}

int64_t orc_render(const sl_gaussian* gaussians, uint32_t count, const sl_part* parts, uint32_t part_count,
                   const sl_gaussian* emitters, const float* colour, const float* lo_b,
                   const sl_render_frame* frame, uint32_t tile_w, uint32_t tile_h,
                   uint32_t* keys, uint32_t* order, uint32_t* ranges, uint32_t* entries, uint64_t entries_cap,
                   uint64_t* n_entries, float* rgba, uint32_t* counts, int nthreads) {
  return orc_render_lod(gaussians, count, parts, part_count, emitters, colour, lo_b, frame, tile_w, tile_h, keys, order,
                        ranges, entries, entries_cap, n_entries, rgba, counts, nthreads, NULL);
}

/* element-wise sl_logf / sl_expf, for the accuracy tests of the shared deterministic functions */
void orc_logf_n(const float* x, float* y, uint64_t n) {
  for (uint64_t i = 0; i < n; i++) y[i] = sl_logf(x[i]);
}
void orc_expf_n(const float* x, float* y, uint64_t n) {
  for (uint64_t i = 0; i < n; i++) y[i] = sl_expf(x[i]);
}
void orc_atan2f_n(const float* y, const float* x, float* out, uint64_t n) {
  for (uint64_t i = 0; i < n; i++) out[i] = sl_atan2f(y[i], x[i]);
}
void orc_asinf_n(const float* x, float* y, uint64_t n) {
  for (uint64_t i = 0; i < n; i++) y[i] = sl_asinf(x[i]);
}
void orc_acosf_n(const float* x, float* y, uint64_t n) {
  for (uint64_t i = 0; i < n; i++) y[i] = sl_acosf(x[i]);
}
