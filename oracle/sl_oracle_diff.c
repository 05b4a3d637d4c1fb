/* The differentiable splat path's forward in double precision with a naive dense compositor (test infrastructure:
 * the reference for finite-difference checks of the hand-written backward).  The model restated from the GPU
 * path's definition (include/splatlight.h, sl_diff_*): projection as shaders/project.wgsl:84-300 with
 * kappa = softplus(logit) / (sqrt(2 pi) s0), point-emitter shading (Lambert + normalised spherical-Gaussian lobe),
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

static void splat_d(const double* mu, const double* ls, const double* q4, double logit, const double* alb, double rough,
                    const double* lpos, const double* lle, const double* lscale, uint32_t nl, double ambient,
                    double ks, const double* V, const double* focal, const double* vp, double nearp, double farp,
                    double lowpass, const double* eye, dsplat* o) {
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
  /* shading */
  double ve[3] = {eye[0] - mu[0], eye[1] - mu[1], eye[2] - mu[2]};
  double vl = sqrt(dot3d(ve, ve)), v[3] = {ve[0] / vl, ve[1] / vl, ve[2] / vl};
  double n[3] = {R[0][0], R[0][1], R[0][2]};
  if (dot3d(n, v) < 0.0)
    for (int k = 0; k < 3; k++) n[k] = -n[k];
  double r2 = rough * rough, dif[3] = {0, 0, 0}, spc[3] = {0, 0, 0};
  for (uint32_t l = 0; l < nl; l++) {
    double D[3] = {lpos[3 * l] - mu[0], lpos[3 * l + 1] - mu[1], lpos[3 * l + 2] - mu[2]};
    double d2 = dot3d(D, D), dl = sqrt(d2), w[3] = {D[0] / dl, D[1] / dl, D[2] / dl};
    double cs = dot3d(n, w);
    if (!(cs > 0.0)) continue;
    double hh[3] = {w[0] + v[0], w[1] + v[1], w[2] + v[2]};
    double hl = sqrt(dot3d(hh, hh)), h[3] = {hh[0] / hl, hh[1] / hl, hh[2] / hl};
    double nh = dot3d(n, h);
    double Dl = exp((nh - 1.0) / r2) / (M_PI * r2);
    for (int k = 0; k < 3; k++) {
      double E = lle[3 * l + k] * lscale[l] * cs / d2;
      dif[k] += E / M_PI;
      spc[k] += E * Dl;
    }
  }
  for (int k = 0; k < 3; k++) o->rgb[k] = alb[k] * (ambient + dif[k]) + ks * spc[k];
  o->live = 1;
}

/* Renders W x H x 4 (rgb, 1 - T) into img (double) and returns the L2 loss against target (float, W x H x 4; rgb),
 * or 0 when target is NULL.  Arrays are per Gaussian (means n x 3 ...); camera as the RenderFrame holds it. */
double orc_diff_render(const double* means, const double* log_scales, const double* quats, const double* logits,
                       const double* albedo, const double* rough, uint32_t n, const double* lpos, const double* lle,
                       const double* lscale, uint32_t nl, double ambient, double ks, const float* view16,
                       const float* focal, const float* viewport, float nearp, float farp, float lowpass,
                       const double* eye, const uint32_t* order, uint32_t n_order, const float* target, double* img,
                       int nthreads) {
  double V[16], fo[2] = {focal[0], focal[1]}, vp[2] = {viewport[0], viewport[1]};
  for (int k = 0; k < 16; k++) V[k] = view16[k];
  const uint32_t W = (uint32_t)viewport[0], H = (uint32_t)viewport[1];
  dsplat* sp = (dsplat*)malloc(sizeof(dsplat) * (n_order ? n_order : 1));
  for (uint32_t k = 0; k < n_order; k++) {
    uint32_t i = order[k];
    splat_d(means + 3 * i, log_scales + 3 * i, quats + 4 * i, logits[i], albedo + 3 * i, rough[i], lpos, lle, lscale,
            nl, ambient, ks, V, fo, vp, nearp, farp, lowpass, eye, &sp[k]);
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
  return loss;
}
