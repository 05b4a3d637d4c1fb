/* The differentiable splat path's forward in double precision with a naive dense compositor (test infrastructure:
 * the reference for finite-difference checks of the hand-written backward).  The model restated from the GPU
 * path's definition (include/splatlight.h, sl_diff_*): projection as shaders/project.wgsl:84-300 with
 * kappa = softplus(logit) / (sqrt(2 pi) s0); lighting as the product's shading pass lights a Gaussian with emissive
 * Gaussian lights (runtime/wgsl/emissive.wgsl:853-980 shade_leaf: the light cut over the emitter tree built from the
 * lights at their current intensities -- src/lighting.js:99-169, restated in sl_oracle_light.c -- intensity
 * Le sqrt(w^T M w) (:123-130), the V grid (common.wgsl:162-177), the footprint transfer (common.wgsl:241-246), the
 * SGGX specular lobe with its iso damping (material_ext.wgsl:27-63)), with the receiver's leaf quantities derived
 * from its parameters, times its opacity-map T and iso_norm (inputs), plus albedo x ambient;
 * alpha = min(1 - exp(-tau0 e^{-q/2}), 0.99), fragments below optical depth 1e-6 skipped, a pixel stopping before its
 * transmittance would drop below 1e-4.  Dense: every Gaussian of `order` (far to near) is evaluated at every pixel;
 * no tiles, no candidate rectangles, no depth keys (the order is an input, so finite differences see a fixed
 * order, as the gradient of a sort does). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double cx, cy, A, B, C, tau0, rgb[3];
  int live;
} dsplat;

static double softplus_d(double x) { return x > 30.0 ? x : log1p(exp(x)); }

static void quat_rot_d(const double* q, double R[3][3]) {
  double n = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double x = q[0] / n, y = q[1] / n, z = q[2] / n, w = q[3] / n;
  /* R[k] = column k */
  R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y + w * z); R[0][2] = 2 * (x * z - w * y);
  R[1][0] = 2 * (x * y - w * z); R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z + w * x);
  R[2][0] = 2 * (x * z + w * y); R[2][1] = 2 * (y * z - w * x); R[2][2] = 1 - 2 * (x * x + y * y);
}

static double dot3d(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

uint32_t orc_emitter_tree_d(const float* rec, uint32_t n, const double* le_scale, double* nodes_out);

/* the lighting of the differentiable path: the tree (16 doubles per node, orc_emitter_tree_d), the per-Gaussian
 * state held constant (V grids, opacity-map T, iso_norm; NULL = visible / 1 / 1) */
typedef struct {
  const double* tree;
  uint32_t root, n;
  double ambient, ks;
  const uint32_t* vgrid;
  const double* lamp_T;
  const double* iso_norm;
} dlight;

typedef struct {
  double P[3], n[3], cinv_d[3], cinv_o[3], sn_d[3], sn_o[3], Sd[3], So[3], kappa, detC;
} drecv;

static void symm_d(const double R[3][3], double e0, double e1, double e2, double* d, double* o) {
  const double* c0 = R[0];
  const double* c1 = R[1];
  const double* c2 = R[2];
  d[0] = c0[0] * c0[0] * e0 + c1[0] * c1[0] * e1 + c2[0] * c2[0] * e2;
  d[1] = c0[1] * c0[1] * e0 + c1[1] * c1[1] * e1 + c2[1] * c2[1] * e2;
  d[2] = c0[2] * c0[2] * e0 + c1[2] * c1[2] * e1 + c2[2] * c2[2] * e2;
  o[0] = c0[0] * c0[1] * e0 + c1[0] * c1[1] * e1 + c2[0] * c2[1] * e2;
  o[1] = c0[0] * c0[2] * e0 + c1[0] * c1[2] * e1 + c2[0] * c2[2] * e2;
  o[2] = c0[1] * c0[2] * e0 + c1[1] * c1[2] * e1 + c2[1] * c2[2] * e2;
}

static void sym_mul_d(const double* d, const double* o, const double* v, double* r) {
  r[0] = d[0] * v[0] + o[0] * v[1] + o[1] * v[2];
  r[1] = o[0] * v[0] + d[1] * v[1] + o[2] * v[2];
  r[2] = o[1] * v[0] + o[2] * v[1] + d[2] * v[2];
}

static double ein_d(double x) { /* common.wgsl:226-239 */
  if (x < 1.0) {
    double term = x, s = x;
    for (int k = 2; k <= 12; k++) {
      term *= -x / k;
      s += term / k;
    }
    return s;
  }
  double p = x * x * x * x + 8.5733287401 * x * x * x + 18.0590169730 * x * x + 8.6347608925 * x + 0.2677737343;
  double q = x * x * x * x + 9.5733223454 * x * x * x + 25.6329561486 * x * x + 21.0996530827 * x + 3.9584969228;
  return log(x) + 0.5772156649 + p / (q * x * exp(x));
}

static double footprint_d(const drecv* r, const double* w) { /* common.wgsl:241-246 */
  double t[3];
  sym_mul_d(r->cinv_d, r->cinv_o, w, t);
  double a = dot3d(w, t);
  sym_mul_d(r->sn_d, r->sn_o, w, t);
  double dm = sqrt(fmax(dot3d(w, t), 0.0));
  double K = r->kappa * dm * sqrt(2.0 * M_PI / a);
  return 2.0 * M_PI * sqrt(r->detC * a) * ein_d(K);
}

static double vcell_d(const uint32_t* v, uint32_t i, uint32_t j) {
  uint32_t k = i * 16u + j;
  return (double)((v[k >> 2u] >> ((k & 3u) * 8u)) & 0xFFu) / 255.0;
}

static double vgrid_d(const uint32_t* v, const double* w) { /* common.wgsl:162-177 */
  if (!v) return 1.0;
  double el = asin(fmin(fmax(w[2], -1.0), 1.0));
  double fi = fmin(fmax((0.5 * M_PI - el) / (M_PI / 8.0) - 0.5, 0.0), 7.0);
  uint32_t i0 = (uint32_t)fi;
  if (i0 > 6u) i0 = 6u;
  double ti = fi - i0;
  double az = (fabs(w[0]) + fabs(w[1]) < 1e-30) ? 0.0 : atan2(w[1], w[0]);
  double fj = (az + M_PI) / (2.0 * M_PI) * 16.0 - 0.5;
  double j0f = floor(fj), tj = fj - j0f;
  uint32_t j0 = (uint32_t)((int32_t)j0f + 16) % 16u, j1 = (j0 + 1u) % 16u;
  double a = vcell_d(v, i0, j0) * (1.0 - tj) + vcell_d(v, i0, j1) * tj;
  double b = vcell_d(v, i0 + 1u, j0) * (1.0 - tj) + vcell_d(v, i0 + 1u, j1) * tj;
  return a * (1.0 - ti) + b * ti;
}

static double phase_d(const drecv* r, const double* wi, const double* wo) { /* material_ext.wgsl:27-63 */
  double h[3] = {wi[0] + wo[0], wi[1] + wo[1], wi[2] + wo[2]};
  double hl = sqrt(dot3d(h, h));
  if (hl < 1e-6) return 0.0;
  double w[3] = {h[0] / hl, h[1] / hl, h[2] / hl};
  const double *d = r->Sd, *o = r->So;
  double det = fmax(d[0] * (d[1] * d[2] - o[2] * o[2]) - o[0] * (o[0] * d[2] - o[2] * o[1]) +
                        o[1] * (o[0] * o[2] - d[1] * o[1]),
                    1e-20);
  double a00 = d[1] * d[2] - o[2] * o[2], a11 = d[0] * d[2] - o[1] * o[1], a22 = d[0] * d[1] - o[0] * o[0];
  double a01 = o[1] * o[2] - o[0] * d[2], a02 = o[0] * o[2] - o[1] * d[1], a12 = o[0] * o[1] - d[0] * o[2];
  double adj = a00 * w[0] * w[0] + a11 * w[1] * w[1] + a22 * w[2] * w[2] +
               2.0 * (a01 * w[0] * w[1] + a02 * w[0] * w[2] + a12 * w[1] * w[2]);
  double q = adj / det, D = 1.0 / (M_PI * sqrt(det) * q * q), t[3];
  sym_mul_d(d, o, wi, t);
  double sigma = sqrt(fmax(dot3d(wi, t), 1e-12));
  return D / (4.0 * sigma);
}

/* shade_emitters over the cut below `node` (emissive.wgsl:873-929; cut rule use_node :133-137, theta 4) */
static void cut_d(const dlight* L, const drecv* r, const uint32_t* vg, double iso, const double* wo0, uint32_t node,
                  double* acc) {
  const double* e = L->tree + 16u * node;
  int leaf = e[13] < 0.0;
  double dd[3] = {r->P[0] - e[0], r->P[1] - e[1], r->P[2] - e[2]};
  if (!leaf && !(dot3d(dd, dd) > 16.0 * e[3] * e[3])) {
    cut_d(L, r, vg, iso, wo0, (uint32_t)e[14], acc);
    cut_d(L, r, vg, iso, wo0, (uint32_t)e[13], acc);
    return;
  }
  double d[3] = {-dd[0], -dd[1], -dd[2]};
  double d2 = dot3d(d, d);
  if (d2 < 1e-8) return;
  double dl = sqrt(d2), wi[3] = {d[0] / dl, d[1] / dl, d[2] / dl};
  double vi = vgrid_d(vg, wi);
  if (vi <= 1e-7) return;
  double fp = footprint_d(r, wi);
  double mw[3] = {-wi[0], -wi[1], -wi[2]}, Md[3] = {e[4], e[5], e[6]}, Mo[3] = {e[7], e[8], e[9]}, t[3];
  sym_mul_d(Md, Mo, mw, t);
  double mq = sqrt(fmax(dot3d(mw, t), 0.0));
  double f = vi * fp / d2;
  if (L->ks > 0.0) {
    double cw = dot3d(wi, r->n);
    double wr[3] = {2.0 * cw * r->n[0] - wi[0], 2.0 * cw * r->n[1] - wi[1], 2.0 * cw * r->n[2] - wi[2]};
    double avr = footprint_d(r, wr) * vgrid_d(vg, wr);
    double damp = fmin(1.0, 1.0 / fmax(4.0 * M_PI * iso * avr, 1e-30));
    f *= (1.0 - L->ks) + L->ks * 4.0 * M_PI * phase_d(r, wi, wo0) * damp;
  }
  for (int k = 0; k < 3; k++) acc[k] += e[10 + k] * mq * f;
}

/* the radiance of Gaussian i: albedo (acc T iso_norm + ambient) */
static void light_d(const dlight* L, uint32_t i, const double* mu, const double* ls, const double R[3][3],
                    double logit, double rough, const double* alb, const double* eye, double* rgb) {
  drecv r;
  for (int k = 0; k < 3; k++) {
    r.P[k] = mu[k];
    r.n[k] = R[0][k];
  }
  double s0 = exp(ls[0]), s1 = exp(ls[1]), s2 = exp(ls[2]), s3 = s0 * s1 * s2;
  r.detC = s3 * s3;
  symm_d(R, 1.0 / (s0 * s0), 1.0 / (s1 * s1), 1.0 / (s2 * s2), r.cinv_d, r.cinv_o);
  symm_d(R, 1.0, (s0 / s1) * (s0 / s1), (s0 / s2) * (s0 / s2), r.sn_d, r.sn_o);
  double fl = fmax(rough * rough, 1e-4);
  symm_d(R, 1.0, fl, fl, r.Sd, r.So);
  r.kappa = softplus_d(logit) / (sqrt(2.0 * M_PI) * s0);
  double iso = L->iso_norm ? L->iso_norm[i] : 1.0, T = L->lamp_T ? L->lamp_T[i] : 1.0;
  double acc[3] = {0, 0, 0};
  if (L->n) {
    double ve[3] = {eye[0] - mu[0], eye[1] - mu[1], eye[2] - mu[2]};
    double vl = sqrt(dot3d(ve, ve)), wo0[3] = {ve[0] / vl, ve[1] / vl, ve[2] / vl};
    cut_d(L, &r, L->vgrid ? L->vgrid + 32u * i : NULL, iso, wo0, L->root, acc);
  }
  for (int k = 0; k < 3; k++) rgb[k] = alb[k] * (acc[k] * T * iso + L->ambient);
}

static void splat_d(uint32_t i, const double* mu, const double* ls, const double* q4, double logit, const double* alb,
                    double rough, const dlight* L, const double* V, const double* focal, const double* vp,
                    double nearp, double farp, double lowpass, const double* eye, dsplat* o) {
  memset(o, 0, sizeof(*o));
  double t[3];
  for (int k = 0; k < 3; k++) t[k] = V[k] * mu[0] + V[4 + k] * mu[1] + V[8 + k] * mu[2] + V[12 + k];
  double depth = -t[2];
  if (depth < nearp || depth > farp) return;
  double R[3][3];
  quat_rot_d(q4, R);
  double wr[3][3], s[3];
  for (int k = 0; k < 3; k++) {
    for (int r = 0; r < 3; r++) wr[k][r] = V[r] * R[k][0] + V[4 + r] * R[k][1] + V[8 + r] * R[k][2];
    s[k] = exp(ls[k]);
  }
  double cv[3][3];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++)
      cv[r][c] = s[0] * s[0] * wr[0][r] * wr[0][c] + s[1] * s[1] * wr[1][r] * wr[1][c] + s[2] * s[2] * wr[2][r] * wr[2][c];
  double fx = focal[0], fy = focal[1], iz = 1.0 / depth;
  double limx = 1.3 * vp[0] * 0.5 / fx, limy = 1.3 * vp[1] * 0.5 / fy;
  double ux = t[0] * iz, uy = t[1] * iz;
  double cxv = fmin(fmax(ux, -limx), limx) * depth, cyv = fmin(fmax(uy, -limy), limy) * depth;
  double j0[3] = {fx * iz, 0.0, fx * cxv * iz * iz}, j1[3] = {0.0, fy * iz, fy * cyv * iz * iz};
  double cj0[3], cj1[3];
  for (int r = 0; r < 3; r++) {
    cj0[r] = cv[r][0] * j0[0] + cv[r][1] * j0[1] + cv[r][2] * j0[2];
    cj1[r] = cv[r][0] * j1[0] + cv[r][1] * j1[1] + cv[r][2] * j1[2];
  }
  double a = dot3d(j0, cj0), b = dot3d(j0, cj1), c = dot3d(j1, cj1);
  double det0 = a * c - b * b, ap = a + lowpass, cp = c + lowpass, det = ap * cp - b * b;
  if (!(det > 0.0) || !(det0 > 0.0)) return;
  double tl = sqrt(dot3d(t, t)), d[3] = {t[0] / tl, t[1] / tl, t[2] / tl}, qd = 0.0;
  for (int k = 0; k < 3; k++) {
    double dl = dot3d(wr[k], d);
    qd += dl * dl / (s[k] * s[k]);
  }
  o->tau0 = softplus_d(logit) * sqrt(det0 / det) / (s[0] * sqrt(qd));
  o->cx = fx * t[0] * iz + 0.5 * vp[0];
  o->cy = 0.5 * vp[1] - fy * t[1] * iz;
  o->A = cp / det;
  o->B = b / det;
  o->C = ap / det;
  light_d(L, i, mu, ls, R, logit, rough, alb, eye, o->rgb);
  o->live = 1;
}

/* Renders W x H x 4 (rgb, 1 - T) into img (double) and returns the L2 loss against target (float, W x H x 4; rgb),
 * or 0 when target is NULL.  Arrays are per Gaussian (means n x 3 ...); camera as the RenderFrame holds it. */
double orc_diff_render(const double* means, const double* log_scales, const double* quats, const double* logits,
                       const double* albedo, const double* rough, uint32_t n, const float* light_rec,
                       const double* lscale, uint32_t nl, double ambient, double ks, const uint32_t* vgrid,
                       const double* lamp_T, const double* iso_norm, const float* view16, const float* focal,
                       const float* viewport, float nearp, float farp, float lowpass, const double* eye,
                       const uint32_t* order, uint32_t n_order, const float* target, double* img, int nthreads) {
  double V[16], fo[2] = {focal[0], focal[1]}, vp[2] = {viewport[0], viewport[1]};
  (void)n;
  double* tree = (double*)calloc(16u * (2u * (nl ? nl : 1u)), sizeof(double));
  dlight L = {tree, 0u, nl, ambient, ks, vgrid, lamp_T, iso_norm};
  if (nl) L.root = orc_emitter_tree_d(light_rec, nl, lscale, tree);
  for (int k = 0; k < 16; k++) V[k] = view16[k];
  const uint32_t W = (uint32_t)viewport[0], H = (uint32_t)viewport[1];
  dsplat* sp = (dsplat*)malloc(sizeof(dsplat) * (n_order ? n_order : 1));
  for (uint32_t k = 0; k < n_order; k++) {
    uint32_t i = order[k];
    splat_d(i, means + 3 * i, log_scales + 3 * i, quats + 4 * i, logits[i], albedo + 3 * i, rough[i], &L, V, fo, vp,
            nearp, farp, lowpass, eye, &sp[k]);
  }
  if (nthreads < 1) nthreads = 1;
  double loss = 0.0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) reduction(+ : loss) schedule(dynamic, 4)
#endif
  for (int64_t py = 0; py < (int64_t)H; py++) {
    for (uint32_t px = 0; px < W; px++) {
      double T = 1.0, C[3] = {0, 0, 0};
      const double xc = px + 0.5, yc = py + 0.5;
      for (int64_t k = (int64_t)n_order - 1; k >= 0; k--) { /* near to far */
        const dsplat* s = &sp[k];
        if (!s->live) continue;
        double dx = xc - s->cx, dy = yc - s->cy;
        double q = s->A * dx * dx + 2.0 * s->B * dx * dy + s->C * dy * dy;
        double tau = s->tau0 * exp(-0.5 * q);
        if (!(tau >= 1e-6)) continue;
        double al = fmin(1.0 - exp(-tau), 0.99);
        double tn = T * (1.0 - al);
        if (tn < 1e-4) break;
        for (int c = 0; c < 3; c++) C[c] += T * al * s->rgb[c];
        T = tn;
      }
      size_t p = (size_t)py * W + px;
      if (img) {
        img[4 * p] = C[0];
        img[4 * p + 1] = C[1];
        img[4 * p + 2] = C[2];
        img[4 * p + 3] = 1.0 - T;
      }
      if (target)
        for (int c = 0; c < 3; c++) {
          double e = C[c] - (double)target[4 * p + c];
          loss += e * e;
        }
    }
  }
  free(sp);
  free(tree);
  return loss;
}
