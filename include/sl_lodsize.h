/*
 * sl_lodsize.h -- the on-screen size of a tree node that the screen-space LOD cut compares with its threshold
 * (runtime/wgsl/lod.wgsl lod_select :179-216 and screen_cov :146-167), shared by the CUDA select kernel and the CPU
 * restatement, which must agree on every open/draw decision bit for bit.
 *
 * size = (2/3) f R / max(z - R, near), R the node's bounding radius, z its depth; with the projected-area rule (the
 * reference's default) and the node in front of the near plane, size is scaled by sqrt(sqrt(short / long)) of the
 * node's on-screen covariance ellipse (short = det / long), so long thin nodes collapse once they are thin on screen.
 *
 * Plain IEEE single-precision arithmetic in written order (+ - * / sqrt): compile with contraction off (nvcc
 * --fmad=false, gcc -ffp-contract=off).  Matrices are column-major 3x3 (c[col][row]); A * v = c0 v.x + c1 v.y + c2 v.z,
 * sums left to right.
 */
#ifndef SL_LODSIZE_H
#define SL_LODSIZE_H

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SL_LOD_FN __host__ __device__ __forceinline__
#else
#define SL_LOD_FN static inline
#endif

typedef struct sl_lod_m3 {
  float c[3][3];
} sl_lod_m3;

SL_LOD_FN void sl_lod_mv(const sl_lod_m3* m, const float v[3], float out[3]) {
  for (int r = 0; r < 3; r++) out[r] = m->c[0][r] * v[0] + m->c[1][r] * v[1] + m->c[2][r] * v[2];
}

SL_LOD_FN sl_lod_m3 sl_lod_mm(const sl_lod_m3* a, const sl_lod_m3* b) {
  sl_lod_m3 o;
  for (int j = 0; j < 3; j++) sl_lod_mv(a, b->c[j], o.c[j]);
  return o;
}

SL_LOD_FN sl_lod_m3 sl_lod_tr(const sl_lod_m3* a) {
  sl_lod_m3 o;
  for (int j = 0; j < 3; j++)
    for (int r = 0; r < 3; r++) o.c[j][r] = a->c[r][j];
  return o;
}

SL_LOD_FN void sl_lod_cross(const float a[3], const float b[3], float o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

SL_LOD_FN float sl_lod_dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* The node's world mean w under its part's pose xf (three rows of 4, rows . (mean, 1)) and its view depth z. */
SL_LOD_FN void sl_lod_world(const float mean[3], const float xf[12], const float view[16], float w[3], float* z) {
  for (int r = 0; r < 3; r++)
    w[r] = xf[4 * r + 0] * mean[0] + xf[4 * r + 1] * mean[1] + xf[4 * r + 2] * mean[2] + xf[4 * r + 3] * 1.0f;
  *z = -(view[2] * w[0] + view[6] * w[1] + view[10] * w[2] + view[14] * 1.0f);
}

/* lod.wgsl screen_cov: the node's covariance (inverse of cinv, by the adjugate) posed by the part, seen through the
 * view, projected by the pinhole Jacobian at w: the 2x2 screen covariance (px^2), columns (s00, s10) and (s01, s11)
 * (s10 = j1 . C j0 and s01 = j0 . C j1, equal up to rounding). */
SL_LOD_FN void sl_lod_screen_cov(const float cinv_diag[3], const float cinv_off[3], const float xf[12],
                                 const float view[16], float focal, const float w[3], float* s00, float* s10,
                                 float* s01, float* s11) {
  const float ci0[3] = {cinv_diag[0], cinv_off[0], cinv_off[1]};
  const float ci1[3] = {cinv_off[0], cinv_diag[1], cinv_off[2]};
  const float ci2[3] = {cinv_off[1], cinv_off[2], cinv_diag[2]};
  float r0[3], r1[3], r2[3];
  sl_lod_cross(ci1, ci2, r0);
  sl_lod_cross(ci2, ci0, r1);
  sl_lod_cross(ci0, ci1, r2);
  const float inv_det = 1.0f / sl_lod_dot3(ci0, r0);
  sl_lod_m3 C; /* transpose(mat3(r0, r1, r2)) * inv_det: column j = (r0[j], r1[j], r2[j]) */
  for (int j = 0; j < 3; j++) {
    C.c[j][0] = r0[j] * inv_det;
    C.c[j][1] = r1[j] * inv_det;
    C.c[j][2] = r2[j] * inv_det;
  }
  sl_lod_m3 Rp; /* transpose(mat3(xf rows)): column j = row j's xyz transposed, i.e. Rp[j][r] = xf[r][j] */
  for (int j = 0; j < 3; j++)
    for (int r = 0; r < 3; r++) Rp.c[j][r] = xf[4 * r + j];
  sl_lod_m3 V;
  for (int j = 0; j < 3; j++)
    for (int r = 0; r < 3; r++) V.c[j][r] = view[4 * j + r];
  const sl_lod_m3 M = sl_lod_mm(&V, &Rp);
  const sl_lod_m3 MC = sl_lod_mm(&M, &C);
  const sl_lod_m3 Mt = sl_lod_tr(&M);
  const sl_lod_m3 Cv = sl_lod_mm(&MC, &Mt);
  float pv[3];
  for (int r = 0; r < 3; r++)
    pv[r] = view[0 + r] * w[0] + view[4 + r] * w[1] + view[8 + r] * w[2] + view[12 + r] * 1.0f;
  const float z = -pv[2];
  const float f = focal;
  const float j0[3] = {f / z, 0.0f, f * pv[0] / (z * z)};
  const float j1[3] = {0.0f, f / z, f * pv[1] / (z * z)};
  float c0[3], c1[3];
  sl_lod_mv(&Cv, j0, c0);
  sl_lod_mv(&Cv, j1, c1);
  *s00 = sl_lod_dot3(j0, c0);
  *s10 = sl_lod_dot3(j1, c0);
  *s01 = sl_lod_dot3(j0, c1);
  *s11 = sl_lod_dot3(j1, c1);
}

/* The size lod_select compares with the threshold (px).  area_rule: 1 projected area (default), 0 bounding radius. */
SL_LOD_FN float sl_lod_size(const float mean[3], float radius, const float cinv_diag[3], const float cinv_off[3],
                            const float xf[12], const float view[16], float focal, float near_plane,
                            uint32_t area_rule, float w_out[3], float* z_out) {
  float w[3], z;
  sl_lod_world(mean, xf, view, w, &z);
  const float R = radius;
  const float zr = z - R;
  float size = (2.0f / 3.0f) * focal * R / (zr > near_plane ? zr : near_plane);
  if (area_rule && zr > near_plane) {
    float s00, s10, s01, s11;
    sl_lod_screen_cov(cinv_diag, cinv_off, xf, view, focal, w, &s00, &s10, &s01, &s11);
    const float tr = s00 + s11;
    float dt = s00 * s11 - s01 * s10; /* determinant of the 2x2 (columns (s00, s10), (s01, s11)) */
    dt = dt > 0.0f ? dt : 0.0f;
    float q = 0.25f * (s00 - s11) * (s00 - s11) + s10 * s10;
    const float disc = sqrtf(q > 0.0f ? q : 0.0f);
    float l1 = 0.5f * tr + disc;
    l1 = l1 > 1e-12f ? l1 : 1e-12f;
    float ratio = dt / l1;
    ratio = ratio > 0.0f ? ratio : 0.0f;
    size *= sqrtf(sqrtf(ratio / l1));
  }
  for (int k = 0; k < 3; k++) w_out[k] = w[k];
  *z_out = z;
  return size;
}

#endif /* SL_LODSIZE_H */
