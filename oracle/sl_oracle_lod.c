/*
 * sl_oracle_lod.c -- CPU restatement of the reference's screen-space LOD (src/lod.js nodeGaussians, Lod;
 * runtime/wgsl/lod.wgsl lod_select, lod_colour).  TEST INFRASTRUCTURE ONLY: the parity tests link this; the product
 * never does.  Parity unpinned against the reference itself (WebGPU; no tests or golden vectors there): pinned by
 * reading the cited code and by the tree invariant tests (every leaf covered exactly once by the cut).
 *
 * The node records are made in float64 (as lod.js does in JS doubles) with the C library's atan2, cos, sin and sqrt;
 * the cut and the colours in float32 in written order, the on-screen size from include/sl_lodsize.h.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "sl_lodsize.h"
#include "sl_oracle.h"

/* src/lod.js:9-23: cyclic Jacobi, values ascending (stable), vecs[k] = k-th column */
static void orc_eig3(const double A[3][3], double vals[3], double vecs[3][3]) {
  double a[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  memcpy(a, A, sizeof(a));
  for (int sweep = 0; sweep < 20; sweep++) {
    double off = 0.0;
    for (int p = 0; p < 3; p++)
      for (int q = p + 1; q < 3; q++) off += a[p][q] * a[p][q];
    if (off < 1e-30) break;
    for (int p = 0; p < 3; p++)
      for (int q = p + 1; q < 3; q++) {
        if (fabs(a[p][q]) < 1e-30) continue;
        double th = 0.5 * atan2(2.0 * a[p][q], a[q][q] - a[p][p]), c = cos(th), s = sin(th);
        for (int k = 0; k < 3; k++) {
          double x = a[k][p], y = a[k][q];
          a[k][p] = c * x - s * y;
          a[k][q] = s * x + c * y;
        }
        for (int k = 0; k < 3; k++) {
          double x = a[p][k], y = a[q][k];
          a[p][k] = c * x - s * y;
          a[q][k] = s * x + c * y;
        }
        for (int k = 0; k < 3; k++) {
          double x = V[k][p], y = V[k][q];
          V[k][p] = c * x - s * y;
          V[k][q] = s * x + c * y;
        }
      }
  }
  int idx[3] = {0, 1, 2};
  for (int i = 1; i < 3; i++) /* insertion sort: stable */
    for (int j = i; j > 0 && a[idx[j]][idx[j]] < a[idx[j - 1]][idx[j - 1]]; j--) {
      int t = idx[j];
      idx[j] = idx[j - 1];
      idx[j - 1] = t;
    }
  for (int k = 0; k < 3; k++) {
    vals[k] = a[idx[k]][idx[k]];
    for (int r = 0; r < 3; r++) vecs[k][r] = V[r][idx[k]];
  }
}

/* src/lod.js:26-37 */
static void orc_quat_cols(const double c[3][3], double q[4]) {
  double m00 = c[0][0], m11 = c[1][1], m22 = c[2][2];
  double m10 = c[0][1], m20 = c[0][2], m01 = c[1][0], m21 = c[1][2], m02 = c[2][0], m12 = c[2][1];
  double tr = m00 + m11 + m22, x, y, z, w;
  if (tr > 0) {
    double s = 2.0 * sqrt(tr + 1.0);
    w = s / 4.0; x = (m21 - m12) / s; y = (m02 - m20) / s; z = (m10 - m01) / s;
  } else if (m00 > m11 && m00 > m22) {
    double s = 2.0 * sqrt(1.0 + m00 - m11 - m22);
    x = s / 4.0; w = (m21 - m12) / s; y = (m01 + m10) / s; z = (m02 + m20) / s;
  } else if (m11 > m22) {
    double s = 2.0 * sqrt(1.0 + m11 - m00 - m22);
    y = s / 4.0; w = (m02 - m20) / s; x = (m01 + m10) / s; z = (m12 + m21) / s;
  } else {
    double s = 2.0 * sqrt(1.0 + m22 - m00 - m11);
    z = s / 4.0; w = (m10 - m01) / s; x = (m02 + m20) / s; y = (m12 + m21) / s;
  }
  double l = sqrt(x * x + y * y + z * z + w * w);
  if (!(l > 0.0)) l = 1.0;
  q[0] = x / l; q[1] = y / l; q[2] = z / l; q[3] = w / l;
}

/* src/lod.js:52-62: inverse of the node's cinv by the adjugate, and det(cinv) */
static double orc_node_cov(const sl_node* nd, double C[3][3]) {
  double M[3][3] = {{nd->cinv_diag[0], nd->cinv_off[0], nd->cinv_off[1]},
                    {nd->cinv_off[0], nd->cinv_diag[1], nd->cinv_off[2]},
                    {nd->cinv_off[1], nd->cinv_off[2], nd->cinv_diag[2]}};
  double det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
               M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
  double inv[3][3] = {{M[1][1] * M[2][2] - M[1][2] * M[2][1], M[0][2] * M[2][1] - M[0][1] * M[2][2],
                       M[0][1] * M[1][2] - M[0][2] * M[1][1]},
                      {M[1][2] * M[2][0] - M[1][0] * M[2][2], M[0][0] * M[2][2] - M[0][2] * M[2][0],
                       M[0][2] * M[1][0] - M[0][0] * M[1][2]},
                      {M[1][0] * M[2][1] - M[1][1] * M[2][0], M[0][1] * M[2][0] - M[0][0] * M[2][1],
                       M[0][0] * M[1][1] - M[0][1] * M[1][0]}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) C[i][j] = inv[i][j] / det;
  return det;
}

int orc_lod_records(const sl_gaussian* gauss, uint32_t G, const sl_node* nodes, uint32_t N, const uint32_t* kids,
                    sl_gaussian* out) {
  double* mass = (double*)calloc(N, sizeof(double));
  double* alb = (double*)calloc(3u * (size_t)N, sizeof(double));
  uint32_t* mat = (uint32_t*)calloc(N, sizeof(uint32_t));
  uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (N > G ? N - G : 1));
  if (!mass || !alb || !mat || !order) return -1;
  for (uint32_t g = 0; g < G; g++) {
    double C[3][3];
    double det = orc_node_cov(&nodes[g], C);
    mass[g] = (double)nodes[g].kappa / sqrt(det > 1e-30 ? det : 1e-30);
    for (int c = 0; c < 3; c++) alb[3u * g + c] = gauss[g].albedo[c];
    mat[g] = gauss[g].flags & 0xFFFFu;
  }
  /* internal nodes, deepest first, ties in index order (a stable sort by depth, descending) */
  uint32_t max_d = 0, k = 0;
  for (uint32_t n = G; n < N; n++)
    if (nodes[n].depth > max_d) max_d = nodes[n].depth;
  for (int64_t d = max_d; d >= 0; d--)
    for (uint32_t n = G; n < N; n++)
      if (nodes[n].depth == (uint32_t)d) order[k++] = n;
  for (uint32_t t = 0; t < N - G; t++) {
    uint32_t n = order[t], lo = nodes[n].child_lo, hi = nodes[n].child_hi;
    double m = 0.0, c[3] = {0.0, 0.0, 0.0};
    for (uint32_t j = lo; j < hi; j++) {
      uint32_t ch = kids[j];
      m += mass[ch];
      for (int q = 0; q < 3; q++) c[q] += mass[ch] * alb[3u * ch + q];
    }
    mass[n] = m;
    for (int q = 0; q < 3; q++) alb[3u * n + q] = c[q] / (m > 1e-30 ? m : 1e-30);
    mat[n] = hi > lo ? mat[kids[lo]] : 0u;
    double C[3][3], vals[3], cols[3][3], q4[4];
    orc_node_cov(&nodes[n], C);
    orc_eig3((const double(*)[3])C, vals, cols);
    double det = cols[0][0] * (cols[1][1] * cols[2][2] - cols[1][2] * cols[2][1]) -
                 cols[1][0] * (cols[0][1] * cols[2][2] - cols[0][2] * cols[2][1]) +
                 cols[2][0] * (cols[0][1] * cols[1][2] - cols[0][2] * cols[1][1]);
    if (det < 0)
      for (int r = 0; r < 3; r++) cols[2][r] = -cols[2][r];
    orc_quat_cols((const double(*)[3])cols, q4);
    sl_gaussian* o = &out[n - G];
    memset(o, 0, sizeof(*o));
    for (int q = 0; q < 3; q++) o->mu[q] = nodes[n].mean[q];
    o->kappa = nodes[n].kappa;
    for (int q = 0; q < 4; q++) o->quat[q] = (float)q4[q];
    for (int q = 0; q < 3; q++) o->scale[q] = (float)sqrt(vals[q] > 1e-12 ? vals[q] : 1e-12);
    o->part_surface = nodes[n].part & 0xFFFFu;
    for (int q = 0; q < 3; q++) o->albedo[q] = (float)alb[3u * n + q];
    o->flags = mat[n];
  }
  free(mass);
  free(alb);
  free(mat);
  free(order);
  return 0;
}

/* nodeGaussians' node V grids (src/lod.js:47-50, 86-88, 99-103): per internal node, deepest first, the mass-weighted
 * mean of its children's cells, kept as float32 (each addition rounded there), then rounded half up and clamped at 255 */
int orc_lod_vgrids(uint32_t G, const sl_node* nodes, uint32_t N, const uint32_t* kids, const sl_vgrid* leaf_vg,
                   sl_vgrid* out) {
  if (N <= G) return 0;
  double* mass = (double*)calloc(N, sizeof(double));
  float* V = (float*)calloc((size_t)(N - G) * 128u, sizeof(float));
  uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (N - G));
  if (!mass || !V || !order) return -1;
  for (uint32_t g = 0; g < G; g++) {
    double C[3][3];
    double det = orc_node_cov(&nodes[g], C);
    mass[g] = (double)nodes[g].kappa / sqrt(det > 1e-30 ? det : 1e-30);
  }
  uint32_t max_d = 0, k = 0;
  for (uint32_t n = G; n < N; n++)
    if (nodes[n].depth > max_d) max_d = nodes[n].depth;
  for (int64_t d = max_d; d >= 0; d--)
    for (uint32_t n = G; n < N; n++)
      if (nodes[n].depth == (uint32_t)d) order[k++] = n;
  for (uint32_t t = 0; t < N - G; t++) {
    uint32_t n = order[t], lo = nodes[n].child_lo, hi = nodes[n].child_hi;
    double m = 0.0;
    for (uint32_t j = lo; j < hi; j++) m += mass[kids[j]];
    mass[n] = m;
    float* vn = V + (size_t)(n - G) * 128u;
    for (uint32_t j = lo; j < hi; j++) {
      uint32_t ch = kids[j];
      double w = mass[ch] / (m > 1e-30 ? m : 1e-30);
      const uint8_t* lb = ch < G ? (const uint8_t*)&leaf_vg[ch] : NULL;
      const float* vc = ch < G ? NULL : V + (size_t)(ch - G) * 128u;
      for (int q = 0; q < 128; q++) vn[q] = (float)((double)vn[q] + w * (double)(lb ? (float)lb[q] : vc[q]));
    }
  }
  for (uint32_t r = 0; r < N - G; r++) {
    uint8_t* o = (uint8_t*)&out[r];
    for (int q = 0; q < 128; q++) {
      double v = floor((double)V[(size_t)r * 128u + q] + 0.5);
      o[q] = (uint8_t)(v > 255.0 ? 255.0 : (v < 0.0 ? 0.0 : v));
    }
  }
  free(mass);
  free(V);
  free(order);
  return 0;
}

enum { ORC_NONE = 0, ORC_OPEN = 1, ORC_DRAW = 2, ORC_CAND = 3, ORC_UNDER = 4 };

/* lod.wgsl lod_select (:169-225), one depth after the other from the roots down */
void orc_lod_select(const sl_node* nodes, uint32_t N, uint32_t G, const uint32_t* kids, const sl_part* parts,
                    uint32_t part_count, const sl_render_frame* f, uint32_t emit_part, uint32_t size_rule,
                    float blur_lod, uint32_t* flags) {
  uint32_t max_d = 0;
  for (uint32_t n = 0; n < N; n++)
    if (nodes[n].depth > max_d) max_d = nodes[n].depth;
  float thr0;
  memcpy(&thr0, &f->lod[0], 4);
  for (uint32_t d = 0; d <= max_d; d++)
    for (uint32_t n = 0; n < N; n++) {
      const sl_node* nd = &nodes[n];
      if (nd->depth != d) continue;
      uint32_t fl = flags[n], part = nd->part;
      int root = part < 32u && part < part_count && parts[part].root == n;
      if (!root && fl != ORC_CAND) {
        int under = fl == ORC_UNDER;
        if (!under) flags[n] = ORC_NONE;
        if (n >= G)
          for (uint32_t k = nd->child_lo; k < nd->child_hi; k++) flags[kids[k]] = under ? ORC_UNDER : ORC_NONE;
        continue;
      }
      if (n < G) {
        flags[n] = ORC_DRAW;
        continue;
      }
      int open = part == emit_part;
      if (!open) {
        const sl_part* pt = &parts[part < 32u ? part : 31u];
        float w[3], z;
        float size = sl_lod_size(nd->mean, nd->radius, nd->cinv_diag, nd->cinv_off, pt->xf, f->view, f->focal[1],
                                 f->near_plane, size_rule & 1u, w, &z);
        float thr = thr0, shutter = f->palette[3][2];
        if (blur_lod > 0.0f && shutter > 0.0f && (pt->flags & 2u) != 0u) {
          float wp[3];
          for (int r = 0; r < 3; r++)
            wp[r] = pt->xf_prev[4 * r + 0] * nd->mean[0] + pt->xf_prev[4 * r + 1] * nd->mean[1] +
                    pt->xf_prev[4 * r + 2] * nd->mean[2] + pt->xf_prev[4 * r + 3] * 1.0f;
          float dx = w[0] - wp[0], dy = w[1] - wp[1], dz = w[2] - wp[2];
          float zr = z - nd->radius;
          float smear = f->focal[1] * shutter * sqrtf(dx * dx + dy * dy + dz * dz) / (zr > f->near_plane ? zr : f->near_plane);
          float b = blur_lod * smear;
          thr = thr > b ? thr : b;
        }
        open = size > thr;
      }
      flags[n] = open ? ORC_OPEN : ORC_DRAW;
      for (uint32_t k = nd->child_lo; k < nd->child_hi; k++) flags[kids[k]] = open ? ORC_CAND : ORC_UNDER;
    }
}

static float orc_node_mass(const sl_node* nd) {
  const float* a = nd->cinv_diag;
  const float* o = nd->cinv_off;
  float det_inv = a[0] * (a[1] * a[2] - o[2] * o[2]) - o[0] * (o[0] * a[2] - o[2] * o[1]) + o[1] * (o[0] * o[2] - a[1] * o[1]);
  return nd->kappa / sqrtf(det_inv > 1e-30f ? det_inv : 1e-30f);
}

/* lod.wgsl lod_colour (:90-110), deepest first */
void orc_lod_colour(const sl_node* nodes, uint32_t N, uint32_t G, const uint32_t* kids, const uint32_t* flags,
                    const float* colour, const float* lo_b, float gain, uint32_t colour_all, float* ncolour) {
  uint32_t max_d = 0;
  for (uint32_t n = G; n < N; n++)
    if (nodes[n].depth > max_d) max_d = nodes[n].depth;
  for (int64_t d = max_d; d >= 0; d--)
    for (uint32_t n = G; n < N; n++) {
      if (nodes[n].depth != (uint32_t)d) continue;
      uint32_t fl = flags[n];
      if (fl != ORC_DRAW && fl != ORC_UNDER && !colour_all) continue;
      float c[3] = {0.0f, 0.0f, 0.0f}, w = 0.0f;
      for (uint32_t k = nodes[n].child_lo; k < nodes[n].child_hi; k++) {
        uint32_t ch = kids[k];
        float m = orc_node_mass(&nodes[ch]), sc[3];
        for (int q = 0; q < 3; q++) {
          if (ch < G) {
            float cl = colour ? colour[4u * ch + q] : 0.0f;
            float bo = lo_b ? lo_b[12u * ch + q] : 0.0f;
            sc[q] = cl + gain * bo;
          } else {
            sc[q] = ncolour[4u * (ch - G) + q];
          }
        }
        for (int q = 0; q < 3; q++) c[q] = c[q] + m * sc[q];
        w = w + m;
      }
      float dv = w > 1e-30f ? w : 1e-30f;
      for (int q = 0; q < 3; q++) ncolour[4u * (n - G) + q] = c[q] / dv;
      ncolour[4u * (n - G) + 3] = 1.0f;
    }
}
