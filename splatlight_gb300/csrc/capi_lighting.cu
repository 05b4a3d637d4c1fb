// C ABI of the lighting (src/lighting.js Lighting, src/light_shadow.js LightShadow, src/sun_map.js SunMap,
// src/environment.js Environment): the host-side emitter tree, the opacity-map plans, and the per-frame update that
// launches the lighting kernels of lighting.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "sl_lighting.h"
#include "sl_runtime.h"


namespace sl {
namespace {

// ---- emitter tree: src/lighting.js:99-169 buildEmitterTree (float64, as the JS) ---------------------------------

struct TNode {
  double mu[3], C[6], M[6], Cs[6], mass, Le[3], radius;
  uint32_t lo, hi;
};

double ein3() {
  double acc = 0.0;
  for (int i = 0; i < 3000; i++) {
    double x = (i + 0.5) * 0.001;
    acc += (1.0 - std::exp(-x)) / x * 0.001;
  }
  return acc;
}
double sym_det(const double* m) {
  double a = m[0], d = m[1], f = m[2], b = m[3], c = m[4], e = m[5];
  return a * (d * f - e * e) - b * (b * f - e * c) + c * (b * e - d * c);
}
void sym_inv(const double* m, double* o) {
  double a = m[0], d = m[1], f = m[2], b = m[3], c = m[4], e = m[5], det = sym_det(m);
  o[0] = (d * f - e * e) / det;
  o[1] = (a * f - c * c) / det;
  o[2] = (a * d - b * b) / det;
  o[3] = (c * e - b * f) / det;
  o[4] = (b * e - c * d) / det;
  o[5] = (b * c - a * e) / det;
}
double sym_quad(const double* m, const double* w) {
  return m[0] * w[0] * w[0] + m[1] * w[1] * w[1] + m[2] * w[2] * w[2] +
         2 * (m[3] * w[0] * w[1] + m[4] * w[0] * w[2] + m[5] * w[1] * w[2]);
}
// principal axes by Jacobi rotations, 12 sweeps (lighting.js:75-89)
void sym_axes(const double* m, double axes[3][3]) {
  double A[3][3] = {{m[0], m[3], m[4]}, {m[3], m[1], m[5]}, {m[4], m[5], m[2]}};
  double V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  const int PQ[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int sweep = 0; sweep < 12; sweep++) {
    for (auto& pq : PQ) {
      int p = pq[0], q = pq[1];
      if (std::fabs(A[p][q]) < 1e-30) continue;
      double th = 0.5 * std::atan2(2 * A[p][q], A[q][q] - A[p][p]);
      double c = std::cos(th), s = std::sin(th);
      for (int k = 0; k < 3; k++) {
        double x = A[k][p], y = A[k][q];
        A[k][p] = c * x - s * y;
        A[k][q] = s * x + c * y;
      }
      for (int k = 0; k < 3; k++) {
        double x = A[p][k], y = A[q][k];
        A[p][k] = c * x - s * y;
        A[q][k] = s * x + c * y;
      }
      for (int k = 0; k < 3; k++) {
        double x = V[k][p], y = V[k][q];
        V[k][p] = c * x - s * y;
        V[k][q] = s * x + c * y;
      }
    }
  }
  for (int k = 0; k < 3; k++)
    for (int i = 0; i < 3; i++) axes[k][i] = V[i][k];
}
double lum(const double* c) { return 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2]; }
const int kIJ[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};

struct TreeBuilder {
  const float* rec;
  const double* le_scale = nullptr;  // per emitter: multiplies its Le (the differentiable path's intensities)
  std::vector<TNode> info;
  std::vector<float> out;  // 24 floats per node (EmitNode + its ASG covariance, lighting.js packEmitNodes)
  uint32_t next = 0;
  double e3, widen;

  uint32_t write(const TNode& nd) {
    uint32_t id = next++;
    float* f = &out[24u * id];
    f[0] = (float)nd.mu[0];
    f[1] = (float)nd.mu[1];
    f[2] = (float)nd.mu[2];
    f[3] = (float)nd.radius;
    f[4] = (float)nd.M[0];
    f[5] = (float)nd.M[1];
    f[6] = (float)nd.M[2];
    f[7] = 0.0f;
    f[8] = (float)nd.M[3];
    f[9] = (float)nd.M[4];
    f[10] = (float)nd.M[5];
    memcpy(&f[11], &nd.lo, 4);
    f[12] = (float)nd.Le[0];
    f[13] = (float)nd.Le[1];
    f[14] = (float)nd.Le[2];
    memcpy(&f[15], &nd.hi, 4);
    f[16] = (float)nd.Cs[0];
    f[17] = (float)nd.Cs[1];
    f[18] = (float)nd.Cs[2];
    f[19] = 0.0f;
    f[20] = (float)nd.Cs[3];
    f[21] = (float)nd.Cs[4];
    f[22] = (float)nd.Cs[5];
    f[23] = 0.0f;
    info[id] = nd;
    return id;
  }

  TNode leaf(uint32_t i) {
    const float* o = rec + 16u * i;
    TNode nd{};
    double x = o[4], y = o[5], z = o[6], w = o[7];
    double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                      {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                      {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    double s2[3] = {(double)o[8] * o[8], (double)o[9] * o[9], (double)o[10] * o[10]};
    for (int j = 0; j < 6; j++) {
      int r = kIJ[j][0], k = kIJ[j][1];
      nd.C[j] = R[r][0] * R[k][0] * s2[0] + R[r][1] * R[k][1] * s2[1] + R[r][2] * R[k][2] * s2[2];
    }
    double g = std::pow(2 * M_PI * e3, 2) * sym_det(nd.C);
    double Ci[6];
    sym_inv(nd.C, Ci);
    for (int j = 0; j < 6; j++) nd.M[j] = Ci[j] * g;
    nd.mass = o[3] * std::pow(2 * M_PI, 1.5) * std::sqrt(sym_det(nd.C));
    for (int j = 0; j < 6; j++) nd.Cs[j] = nd.C[j] * widen;
    for (int k = 0; k < 3; k++) {
      nd.mu[k] = o[k];
      nd.Le[k] = le_scale ? o[12 + k] * le_scale[i] : o[12 + k];
    }
    nd.radius = 3 * std::max(std::max((double)o[8], (double)o[9]), (double)o[10]);
    nd.lo = 0xFFFFFFFFu;
    nd.hi = i;
    return nd;
  }

  uint32_t build(std::vector<uint32_t> idx) {
    const uint32_t n = (uint32_t)idx.size();
    if (n == 1) return write(leaf(idx[0]));
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i : idx)
      for (int k = 0; k < 3; k++) {
        lo[k] = std::min(lo[k], (double)rec[16u * i + k]);
        hi[k] = std::max(hi[k], (double)rec[16u * i + k]);
      }
    int ax = 0;
    for (int k = 0; k < 3; k++)
      if (hi[k] - lo[k] > hi[ax] - lo[ax]) ax = k;
    // median split on the longest axis; std::stable_sort keeps ties in their incoming order, as JS's stable sort
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t p, uint32_t q) {
      return (double)rec[16u * p + ax] < (double)rec[16u * q + ax];
    });
    const uint32_t half = n >> 1;
    uint32_t ia = build(std::vector<uint32_t>(idx.begin(), idx.begin() + half));
    uint32_t ib = build(std::vector<uint32_t>(idx.begin() + half, idx.end()));
    const TNode* kids[2] = {&info[ia], &info[ib]};
    TNode nd{};
    double m = kids[0]->mass + kids[1]->mass;
    for (int k = 0; k < 3; k++) nd.mu[k] = (kids[0]->mass * kids[0]->mu[k] + kids[1]->mass * kids[1]->mu[k]) / m;
    for (int j = 0; j < 6; j++) {
      int r = kIJ[j][0], k = kIJ[j][1];
      double acc = 0.0, accs = 0.0;
      for (const TNode* ch : kids) {
        acc += ch->mass * (ch->C[j] + (ch->mu[r] - nd.mu[r]) * (ch->mu[k] - nd.mu[k]));
        accs += ch->mass * (ch->Cs[j] + (ch->mu[r] - nd.mu[r]) * (ch->mu[k] - nd.mu[k]));
      }
      nd.C[j] = acc / m;
      nd.Cs[j] = accs / m;
    }
    double axes[3][3];
    sym_axes(nd.C, axes);
    double tot[3], num[3] = {0, 0, 0}, den = 0.0;
    for (int k = 0; k < 3; k++) {
      tot[k] = 0.0;
      for (const TNode* ch : kids) tot[k] += lum(ch->Le) * std::sqrt(std::max(sym_quad(ch->M, axes[k]), 0.0));
    }
    for (const TNode* ch : kids) {
      double sw = 0.0;
      for (int k = 0; k < 3; k++) sw += std::sqrt(std::max(sym_quad(ch->M, axes[k]), 0.0));
      for (int c = 0; c < 3; c++) num[c] += ch->Le[c] * sw;
      den += sw;
    }
    for (int c = 0; c < 3; c++) nd.Le[c] = num[c] / den;
    double L = std::max(lum(nd.Le), 1e-12);
    for (int k = 0; k < 3; k++) {
      double lam = std::pow(tot[k] / L, 2);
      for (int j = 0; j < 6; j++) nd.M[j] += lam * axes[k][kIJ[j][0]] * axes[k][kIJ[j][1]];
    }
    double rad = -INFINITY;
    for (const TNode* ch : kids) {
      double dx = ch->mu[0] - nd.mu[0], dy = ch->mu[1] - nd.mu[1], dz = ch->mu[2] - nd.mu[2];
      rad = std::max(rad, std::sqrt(dx * dx + dy * dy + dz * dz) + ch->radius);
    }
    nd.radius = rad;
    nd.mass = m;
    nd.lo = ia;
    nd.hi = ib;
    return write(nd);
  }
};

// eigenvalues of a symmetric 3x3, ascending (src/light_shadow.js:169-180)
void eig3(const double* m, double* ev) {
  double a = m[0], d = m[1], f = m[2], b = m[3], c = m[4], e = m[5];
  double p1 = b * b + c * c + e * e;
  double q = (a + d + f) / 3;
  double p2 = (a - q) * (a - q) + (d - q) * (d - q) + (f - q) * (f - q) + 2 * p1;
  double p = std::sqrt(p2 / 6);
  if (p < 1e-30) {
    ev[0] = ev[1] = ev[2] = q;
    return;
  }
  double B[6] = {(a - q) / p, (d - q) / p, (f - q) / p, b / p, c / p, e / p};
  double r = (B[0] * (B[1] * B[2] - B[5] * B[5]) - B[3] * (B[3] * B[2] - B[5] * B[4]) + B[4] * (B[3] * B[5] - B[1] * B[4])) / 2;
  double phi = std::acos(std::min(1.0, std::max(-1.0, r))) / 3;
  double e1 = q + 2 * p * std::cos(phi), e3 = q + 2 * p * std::cos(phi + 2 * M_PI / 3);
  ev[0] = e3;
  ev[1] = 3 * q - e1 - e3;
  ev[2] = e1;
}

void levels_for(uint32_t res, uint32_t& levels, uint32_t* level_off, uint32_t& layer_texels) {
  uint32_t off = 0;
  levels = 0;
  for (uint32_t k = res; k >= 1u; k >>= 1) {
    level_off[levels++] = off;
    off += k * k;
  }
  layer_texels = off;
}

// basisK of src/sun_map.js:165-169 (float64)
void basis_k64(const double* w, double* t1) {
  double a[3] = {0, 0, 1};
  if (std::fabs(w[2]) >= 0.999) {
    a[0] = 1;
    a[2] = 0;
  }
  double c[3] = {a[1] * w[2] - a[2] * w[1], a[2] * w[0] - a[0] * w[2], a[0] * w[1] - a[1] * w[0]};
  double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  for (int k = 0; k < 3; k++) t1[k] = c[k] / l;
}
// float32 basis_k / cross of sun_map.wgsl sm_frame (common.wgsl:181-185), with the kernels' rounding order
void basis_k32(const float* w, float* t1, float* t2) {
  float a[3] = {0.0f, 0.0f, 1.0f};
  if (std::fabs(w[2]) >= 0.999f) {
    a[0] = 1.0f;
    a[2] = 0.0f;
  }
  volatile float c0 = a[1] * w[2] - a[2] * w[1], c1 = a[2] * w[0] - a[0] * w[2], c2 = a[0] * w[1] - a[1] * w[0];
  volatile float l = std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  t1[0] = c0 / l;
  t1[1] = c1 / l;
  t1[2] = c2 / l;
  t2[0] = w[1] * t1[2] - w[2] * t1[1];
  t2[1] = w[2] * t1[0] - w[0] * t1[2];
  t2[2] = w[0] * t1[1] - w[1] * t1[0];
}

}  // namespace
}  // namespace sl

namespace sl {

// iso_init cell directions and solid angles (iso_init.wgsl:39-45), float64 then rounded
void iso_dirs(float* d) {
  for (int c = 0; c < 128; c++) {
    int i = c / 16, j = c % 16;
    double el = 0.5 * M_PI - (i + 0.5) * M_PI / 8.0;
    double az = -M_PI + (j + 0.5) * 2.0 * M_PI / 16.0;
    double top = 0.5 * M_PI - i * M_PI / 8.0;
    d[4 * c + 0] = (float)(std::cos(el) * std::cos(az));
    d[4 * c + 1] = (float)(std::cos(el) * std::sin(az));
    d[4 * c + 2] = (float)std::sin(el);
    d[4 * c + 3] = (float)((2.0 * M_PI / 16.0) * (std::sin(top) - std::sin(top - M_PI / 8.0)));
  }
}

// D14 (lighting.js:188-189: the 6 axes, the verticals leaning 1e-4 off the pole, and the 8 diagonals / sqrt 3) and
// pinvD14 (:192-207): the least-squares SH2 fit (A^T A)^-1 A^T of values on them, Gauss-Jordan with partial pivoting
void bounce_tables(float* d14, float* pinv) {
  static const double raw[14][3] = {{1, 0, 0}, {0, 1, 0}, {1e-4, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {1e-4, 0, -1},
                                    {1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                                    {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
  double A[14][9];
  for (int k = 0; k < 14; k++) {
    const double s = k < 6 ? 1.0 : 1.0 / std::sqrt(3.0);
    const double x = raw[k][0] * s, y = raw[k][1] * s, z = raw[k][2] * s;
    const double b[9] = {0.282095, 0.488603 * y, 0.488603 * z, 0.488603 * x, 1.092548 * x * y, 1.092548 * y * z,
                         0.315392 * (3 * z * z - 1), 1.092548 * x * z, 0.546274 * (x * x - y * y)};
    for (int m = 0; m < 9; m++) A[k][m] = b[m];
    d14[3 * k] = (float)x;
    d14[3 * k + 1] = (float)y;
    d14[3 * k + 2] = (float)z;
  }
  double M[9][18];
  for (int i = 0; i < 9; i++)
    for (int j = 0; j < 9; j++) {
      double acc = 0.0;
      for (int r = 0; r < 14; r++) acc += A[r][i] * A[r][j];
      M[i][j] = acc;
      M[i][9 + j] = i == j ? 1.0 : 0.0;
    }
  for (int c = 0; c < 9; c++) {
    int piv = c;
    for (int r = c + 1; r < 9; r++)
      if (std::fabs(M[r][c]) > std::fabs(M[piv][c])) piv = r;
    for (int j = 0; j < 18; j++) std::swap(M[c][j], M[piv][j]);
    const double dv = M[c][c];
    for (int j = 0; j < 18; j++) M[c][j] /= dv;
    for (int r = 0; r < 9; r++) {
      if (r == c) continue;
      const double f = M[r][c];
      for (int j = 0; j < 18; j++) M[r][j] -= f * M[c][j];
    }
  }
  for (int m = 0; m < 9; m++)
    for (int k = 0; k < 14; k++) {
      double acc = 0.0;
      for (int j = 0; j < 9; j++) acc += M[m][9 + j] * A[k][j];
      pinv[14 * m + k] = (float)acc;
    }
}

void cell_asg_table(float* t) {
  const double kCellStd = 0.4;
  for (int c = 0; c < 128; c++) {
    const int i = c / 16, j = c % 16;
    const double el = 0.5 * M_PI - (i + 0.5) * M_PI / 8.0, az = -M_PI + (j + 0.5) * 2.0 * M_PI / 16.0;
    const double s_el = kCellStd * M_PI / 8.0, s_az = kCellStd * 2.0 * M_PI / 16.0 * std::max(std::cos(el), 0.05);
    float* o = t + 8 * c;
    o[0] = (float)(-std::sin(el) * std::cos(az));
    o[1] = (float)(-std::sin(el) * std::sin(az));
    o[2] = (float)std::cos(el);
    o[3] = (float)(-std::sin(az));
    o[4] = (float)std::cos(az);
    o[5] = 0.0f;
    o[6] = (float)(s_el * s_el);
    o[7] = (float)(s_az * s_az);
  }
}

// Skip links for a stackless walk of the light cut (the GPU shading pass).  The cut is the walk of a 48-entry stack
// that pushes (lo, hi) and so pops hi first: node order = preorder with the hi subtree before the lo one.  Per node,
// word 7 = the node that walk reaches once this node's subtree is done (its skip); word 19 = 1 when the stack would
// be full there (depth of pending lo siblings + 2 > 48), where the stack walk neither uses nor refines the node.
constexpr uint32_t kNoChild = 0xFFFFFFFFu;

void link_tree(std::vector<float>& out, uint32_t node, uint32_t skip, uint32_t pending) {
  for (;;) {
    float* f = &out[24u * node];
    memcpy(&f[7], &skip, 4);
    const uint32_t full = pending + 2u > 48u ? 1u : 0u;
    memcpy(&f[19], &full, 4);
    uint32_t lo, hi;
    memcpy(&lo, &f[11], 4);
    memcpy(&hi, &f[15], 4);
    if (lo == kNoChild) return;
    link_tree(out, hi, lo, pending + 1u);  // hi first; lo is pending meanwhile
    node = lo;                              // then lo, which ends where this node ends
  }
}

// The emitter tree of n records (16 floats each, albedo = Le) with each emitter's Le scaled by le_scale[k] (NULL: 1),
// laid out as the shading pass walks it (24 floats per node, skip links set); returns the root.  With dtab non-null
// it also receives, per node e and emitter k, the derivatives of the node's Le (3) and M (6: xx yy zz xy xz yz) with
// respect to le_scale[k], [e][k][9]: central differences of the float64 build (relative step 1e-6; the split
// structure and the moment-matched shapes do not depend on the intensities, only Le and M do).
uint32_t build_emitter_tree(const float* rec, uint32_t n, const double* le_scale, std::vector<float>& out,
                            std::vector<float>* dtab) {
  const double e3 = ein3();
  auto run = [&](const double* sc, std::vector<TNode>* info_out, std::vector<float>* packed) {
    TreeBuilder B;
    B.rec = rec;
    B.le_scale = sc;
    B.info.resize(2ull * n);
    B.out.assign(24ull * (2 * n - 1), 0.0f);
    B.e3 = e3;
    B.widen = e3 / (1.0 - std::exp(-3.0));
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    const uint32_t root = B.build(idx);
    if (packed) {
      link_tree(B.out, root, kNoChild, 0);
      *packed = std::move(B.out);
    }
    if (info_out) *info_out = std::move(B.info);
    return root;
  };
  std::vector<double> sc(n, 1.0);
  if (le_scale)
    for (uint32_t k = 0; k < n; k++) sc[k] = le_scale[k];
  const uint32_t root = run(sc.data(), nullptr, &out);
  if (dtab) {
    const uint32_t nodes = 2 * n - 1;
    dtab->assign((size_t)nodes * n * 9, 0.0f);
    std::vector<TNode> ip, im;
    for (uint32_t k = 0; k < n; k++) {
      const double h = 1e-6 * std::max(std::fabs(sc[k]), 1e-3);
      std::vector<double> sp = sc, sm = sc;
      sp[k] += h;
      sm[k] -= h;
      run(sp.data(), &ip, nullptr);
      run(sm.data(), &im, nullptr);
      for (uint32_t e = 0; e < nodes; e++) {
        float* o = &(*dtab)[((size_t)e * n + k) * 9];
        for (int c = 0; c < 3; c++) o[c] = (float)((ip[e].Le[c] - im[e].Le[c]) / (2 * h));
        for (int j = 0; j < 6; j++) o[3 + j] = (float)((ip[e].M[j] - im[e].M[j]) / (2 * h));
      }
    }
  }
  return root;
}

// Shading order: the Gaussians sorted by a 30-bit Morton code of their model-space means over the scene's bounds,
// so a warp's threads shade nearby points whose light cuts agree (less divergence in the cut walk).
cudaError_t build_shade_order(sl_lighting* l) {
  const uint32_t G = l->count;
  std::vector<sl_gaussian> g(G);
  cudaError_t e = cudaMemcpy(g.data(), l->r->gaussians.ptr, sizeof(sl_gaussian) * (size_t)G, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (const sl_gaussian& x : g)
    for (int k = 0; k < 3; k++)
      if (std::isfinite(x.mu[k])) {
        lo[k] = std::min(lo[k], x.mu[k]);
        hi[k] = std::max(hi[k], x.mu[k]);
      }
  auto spread = [](uint32_t v) {  // 10 bits -> every third bit
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
  };
  std::vector<uint64_t> key(G);
  for (uint32_t i = 0; i < G; i++) {
    uint32_t q[3];
    for (int k = 0; k < 3; k++) {
      const float span = hi[k] > lo[k] ? hi[k] - lo[k] : 1.0f;
      float t = std::isfinite(g[i].mu[k]) ? (g[i].mu[k] - lo[k]) / span : 0.0f;
      t = std::min(std::max(t, 0.0f), 1.0f);
      q[k] = (uint32_t)(t * 1023.0f);
    }
    const uint32_t m = spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2);
    key[i] = ((uint64_t)m << 32) | i;
  }
  std::sort(key.begin(), key.end());
  std::vector<uint32_t> order(G);
  for (uint32_t i = 0; i < G; i++) order[i] = (uint32_t)key[i];
  if ((e = l->order.ensure(4ull * G + 16)) != cudaSuccess) return e;
  return cudaMemcpy(l->order.ptr, order.data(), 4ull * G, cudaMemcpyHostToDevice);
}

void shade_params(const sl_lighting* l, const float* eye, ShadeParams& SH) {
  memset(&SH, 0, sizeof(SH));
  for (int k = 0; k < 3; k++) {
    SH.eye[k] = eye ? eye[k] : 0.0f;
    SH.normal[k] = l->normal[k];
  }
  SH.n_emit = l->n_emit;
  SH.root = l->root;
  SH.mode = l->mode;
  SH.asg = l->asg;
  SH.one_sided = l->one_sided;
  SH.material_count = l->material_count;
  SH.scale = l->scale;
  SH.theta = l->theta;
  SH.edge_soft = l->edge_soft;
  SH.sky_ambient = l->sky_ambient;
  const uint32_t K = (uint32_t)std::min<size_t>(l->lights.size(), 4);
  SH.n_lights = K;
  for (uint32_t k = 0; k < K; k++) {
    for (int c = 0; c < 3; c++) {
      SH.lights[k].dir[c] = l->lights[k].dir[c];
      SH.lights[k].irr[c] = l->lights[k].irradiance[c];
    }
    SH.lights[k].std = l->lights[k].std;
    SH.lights[k].shadows = l->lights[k].casts_shadows ? 1u : 0u;
  }
}

}  // namespace sl

using namespace sl;

#define SL_CHECK_CUDA(expr, what)                          \
  do {                                                     \
    cudaError_t _e = (expr);                               \
    if (_e != cudaSuccess) return cuda_fail(_e, what);     \
  } while (0)

extern "C" {

int sl_lighting_create(sl_renderer* r, const sl_node* nodes, const sl_vgrid* vgrid, const sl_material* materials,
                       uint32_t material_count, sl_lighting** out) {
  if (!out) return fail(SL_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  if (!r || !nodes || !vgrid || !materials || material_count == 0 || material_count > 256)
    return fail(SL_ERR_INVALID_ARG, "bad lighting arguments");
  cudaSetDevice(r->device);
  sl_lighting* l = new sl_lighting();
  l->r = r;
  l->device = r->device;
  l->count = r->count;
  l->material_count = material_count;
  cudaError_t e = l->nodes.ensure(sizeof(sl_node) * (size_t)r->count);
  if (e == cudaSuccess) e = cudaMemcpy(l->nodes.ptr, nodes, sizeof(sl_node) * (size_t)r->count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = l->vgrid.ensure(sizeof(sl_vgrid) * (size_t)r->count);
  if (e == cudaSuccess) e = cudaMemcpy(l->vgrid.ptr, vgrid, sizeof(sl_vgrid) * (size_t)r->count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = l->materials.ensure(sizeof(sl_material) * material_count);
  if (e == cudaSuccess) e = cudaMemcpy(l->materials.ptr, materials, sizeof(sl_material) * material_count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = l->parts.ensure(sizeof(sl_part) * kMaxParts);
  if (e == cudaSuccess) e = l->lamp_T.ensure(4ull * r->count);
  if (e == cudaSuccess) e = l->env_T.ensure(16ull * r->count);
  if (e == cudaSuccess) e = l->colour.ensure(16ull * r->count);
  if (e == cudaSuccess) e = l->tree.ensure(4 * 24);
  if (e == cudaSuccess) e = build_shade_order(l);
  if (e != cudaSuccess) {
    delete l;
    return cuda_fail(e, "sl_lighting_create");
  }
  *out = l;
  return SL_OK;
}

int sl_lighting_destroy(sl_lighting* l) {
  if (!l) return SL_OK;
  cudaSetDevice(l->device);
  cudaDeviceSynchronize();
  if (l->r && l->r->lighting == l) {
    l->r->lighting = nullptr;
    l->r->colour = nullptr;
  }
  if (l->r && l->r->lo_b == l->lo_b.as<float4>()) l->r->lo_b = nullptr;
  sl::DevBuf* all[] = {&l->nodes, &l->vgrid, &l->materials, &l->parts, &l->tree, &l->lamp_T, &l->env_T, &l->colour,
                       &l->lm_acc, &l->lm_mip, &l->sm_acc, &l->sm_mip, &l->sm_layers, &l->sm_dirty, &l->order,
                       &l->g_blur, &l->n_blur, &l->tree_nodes, &l->node_parent, &l->kids, &l->bn_tab,
                       &l->bn_ground, &l->bn_up, &l->probe_data, &l->probe_sh, &l->xfer, &l->lo_dir, &l->lo_b,
                       &l->node_acc, &l->node_sh, &l->bn_quarters, &l->bn_leaf_w, &l->probe_hist,
                       &l->sc_level, &l->sc_gs, &l->sc_vg, &l->sc_flag, &l->sc_X, &l->sc_T, &l->sc_E, &l->sc_list};
  for (sl::DevBuf* b : all) b->release();
  delete l;
  return SL_OK;
}

int sl_emitter_tree(const sl_gaussian* emitters, uint32_t n, const double* le_scale, float* nodes_out,
                    float* dtab_out, uint32_t* root) {
  if (!emitters || !nodes_out || !root || n == 0) return fail(SL_ERR_INVALID_ARG, "null argument or no emitters");
  if (n > 16384) return fail(SL_ERR_INVALID_ARG, "more than MAX_EMITTERS (16384) emitters");
  std::vector<float> out, dtab;
  *root = build_emitter_tree(reinterpret_cast<const float*>(emitters), n, le_scale, out, dtab_out ? &dtab : nullptr);
  memcpy(nodes_out, out.data(), out.size() * 4);
  if (dtab_out) memcpy(dtab_out, dtab.data(), dtab.size() * 4);
  return SL_OK;
}

int sl_lighting_set_emitters(sl_lighting* l, const sl_gaussian* emitters, uint32_t n, float scale, int one_sided,
                             const float* normal, uint32_t skip_part) {
  if (!l || (n && !emitters)) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n > 16384) return fail(SL_ERR_INVALID_ARG, "more than MAX_EMITTERS (16384) emitters");
  cudaSetDevice(l->device);
  l->n_emit = n;
  l->scale = scale;
  l->one_sided = one_sided ? 1u : 0u;
  if (normal) {
    l->normal[0] = normal[0];
    l->normal[1] = normal[1];
    l->normal[2] = normal[2];
  }
  l->skip_part = skip_part;
  l->rec.assign(reinterpret_cast<const float*>(emitters), reinterpret_cast<const float*>(emitters) + 16ull * n);
  if (n) {
    TreeBuilder B;
    B.rec = l->rec.data();
    B.info.resize(2ull * n);
    B.out.assign(24ull * (2 * n - 1), 0.0f);
    B.e3 = ein3();
    B.widen = B.e3 / (1.0 - std::exp(-3.0));
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    l->root = B.build(idx);
    for (int j = 0; j < 6; j++) l->root_cov[j] = (double)(float)B.info[l->root].Cs[j];
    link_tree(B.out, l->root, kNoChild, 0);
    SL_CHECK_CUDA(l->tree.ensure(B.out.size() * 4), "emitter tree");
    SL_CHECK_CUDA(cudaMemcpy(l->tree.ptr, B.out.data(), B.out.size() * 4, cudaMemcpyHostToDevice), "emitter tree");
  }
  // the renderer draws the same emitters in slots count+1 .. count+n (bindColour's emitterBuf, renderer.js:264-268)
  if (n <= l->r->max_emitters) {
    int rc = sl_renderer_set_emitters(l->r, emitters, n);
    if (rc) return rc;
  }
  l->lm_dirty = true;
  return SL_OK;
}

int sl_lighting_set_environment(sl_lighting* l, const sl_env_light* lights, uint32_t n, float sky_ambient) {
  if (!l || (n && !lights)) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n > 4) return fail(SL_ERR_INVALID_ARG, "at most 4 distant lights (environment.wgsl Env.lights)");
  l->lights.assign(lights, lights + n);
  l->sky_ambient = sky_ambient;
  l->sm_dirty_all = true;
  l->have_center.clear();
  return SL_OK;
}

int sl_lighting_set_options(sl_lighting* l, uint32_t shadow_res, uint32_t sun_res, uint32_t mode, float theta,
                            int asg) {
  if (!l) return fail(SL_ERR_INVALID_ARG, "null lighting");
  auto pow2 = [](uint32_t x) { return x == 0 || ((x & (x - 1)) == 0 && x >= 64 && x <= 8192); };
  if (!pow2(shadow_res) || !pow2(sun_res)) return fail(SL_ERR_INVALID_ARG, "map resolutions: 0 or a power of two in [64, 8192]");
  if (mode > 1) return fail(SL_ERR_INVALID_ARG, "mode must be 0 (every emitter) or 1 (light cut)");
  l->shadow_res = shadow_res;
  l->sun_res = sun_res;
  l->mode = mode;
  l->theta = theta;
  l->asg = asg ? 1u : 0u;
  l->lm_dirty = true;
  l->sm_dirty_all = true;
  l->have_center.clear();
  return SL_OK;
}

int sl_lighting_set_blur(sl_lighting* l, float shutter, float cut_k) {
  if (!l) return fail(SL_ERR_INVALID_ARG, "null lighting");
  if (!(shutter >= 0.0f && shutter <= 1.0f)) return fail(SL_ERR_INVALID_ARG, "shutter outside [0, 1]");
  if (!(cut_k >= 0.0f && cut_k <= 1e6f)) return fail(SL_ERR_INVALID_ARG, "bad cut factor");
  if (shutter != l->blur_shutter || cut_k != l->cut_k) {
    l->blur_shutter = shutter;
    l->cut_k = cut_k;
    l->blur_init = false;
    l->blur_prev = 0;
    l->lm_dirty = true;
    l->sm_dirty_all = true;
  }
  return SL_OK;
}

int sl_lighting_set_tree(sl_lighting* l, const sl_node* nodes, uint32_t n_nodes, const uint32_t* kids,
                         uint32_t n_kids) {
  if (!l || !nodes || (n_kids && !kids)) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n_nodes < l->count) return fail(SL_ERR_INVALID_ARG, "the tree must start with the scene's leaves");
  cudaSetDevice(l->device);
  // every node's parent (lighting.js initNodeParents): for an internal node with a part, its children's
  std::vector<uint32_t> parent(n_nodes, 0xFFFFFFFFu);
  for (uint32_t i = l->count; i < n_nodes; i++) {
    if (nodes[i].part == 0xFFFFFFFFu) continue;
    if (nodes[i].child_lo > nodes[i].child_hi || nodes[i].child_hi > n_kids)
      return fail(SL_ERR_INVALID_ARG, "node children outside kids");
    for (uint32_t j = nodes[i].child_lo; j < nodes[i].child_hi; j++) {
      if (kids[j] >= n_nodes) return fail(SL_ERR_INVALID_ARG, "kid index outside the tree");
      parent[kids[j]] = i;
    }
  }
  SL_CHECK_CUDA(l->tree_nodes.ensure(sizeof(sl_node) * (size_t)n_nodes), "tree nodes");
  SL_CHECK_CUDA(l->node_parent.ensure(4ull * n_nodes), "node parents");
  SL_CHECK_CUDA(l->kids.ensure(4ull * n_kids + 16), "kids");
  SL_CHECK_CUDA(cudaMemcpy(l->tree_nodes.ptr, nodes, sizeof(sl_node) * (size_t)n_nodes, cudaMemcpyHostToDevice),
                "tree nodes");
  SL_CHECK_CUDA(cudaMemcpy(l->node_parent.ptr, parent.data(), 4ull * n_nodes, cudaMemcpyHostToDevice), "node parents");
  if (n_kids) SL_CHECK_CUDA(cudaMemcpy(l->kids.ptr, kids, 4ull * n_kids, cudaMemcpyHostToDevice), "kids");
  l->tree_depth.resize(n_nodes);
  l->tree_part.resize(n_nodes);
  for (uint32_t i = 0; i < n_nodes; i++) {
    l->tree_depth[i] = nodes[i].depth;
    l->tree_part[i] = nodes[i].part;
  }
  l->n_tree = n_nodes;
  l->n_kids = n_kids;
  l->bounce_on = false;  // the probes are laid over a tree: set them again
  l->bn_sc = false;      // so is the sender cut's node data
  l->blur_init = false;
  l->lm_dirty = true;
  l->sm_dirty_all = true;
  return SL_OK;
}

int sl_lighting_update(sl_lighting* l, const float* eye, const float* forward, uint32_t moved_mask, void* stream) {
  if (!l || !eye) return fail(SL_ERR_INVALID_ARG, "null argument");
  cudaSetDevice(l->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  sl_renderer* r = l->r;
  const uint32_t G = l->count, P = r->part_count;
  const sl_gaussian* gs = r->gaussians.as<sl_gaussian>();
  sl_part* parts = l->parts.as<sl_part>();
  SL_CHECK_CUDA(cudaMemcpyAsync(parts, r->parts.data(), sizeof(sl_part) * P, cudaMemcpyHostToDevice, s), "parts");

  if (!l->iso_done) {  // iso_init: once per asset (lighting.js:529-555)
    float dirs[512];
    iso_dirs(dirs);
    SL_CHECK_CUDA(upload_iso_dirs(dirs, s), "iso directions");
    SL_CHECK_CUDA(launch_iso(gs, l->nodes.as<sl_node>(), l->vgrid.as<sl_vgrid>(), G, s), "iso_init");
    l->iso_done = true;
  }

  // motion blur: the copies the map splats draw, rewritten for the parts that moved now or in the last update
  // (lighting.js encodeBlur); every part on the first update after blur was switched on
  const sl_gaussian* gsp = gs;
  const sl_node* ndp = l->nodes.as<sl_node>();
  uint32_t blur_mask = 0;
  const bool tree = l->n_tree > G;
  const uint32_t N = tree ? l->n_tree : G;  // records: the leaves, then the tree's internal nodes
  const sl_node* n_rest = tree ? l->tree_nodes.as<sl_node>() : l->nodes.as<sl_node>();
  BlurCut bc{gs, n_rest, tree ? l->node_parent.as<uint32_t>() : nullptr, N, 0.0f, l->blur_shutter};
  if (l->blur_shutter > 0.0f) {
    SL_CHECK_CUDA(l->g_blur.ensure(sizeof(sl_gaussian) * (size_t)G), "blur copies");
    SL_CHECK_CUDA(l->n_blur.ensure(sizeof(sl_node) * (size_t)N), "blur copies");
    const uint32_t all = P >= 32 ? 0xFFFFFFFFu : ((1u << P) - 1u);
    if (!l->blur_init) {
      SL_CHECK_CUDA(cudaMemcpyAsync(l->g_blur.ptr, gs, sizeof(sl_gaussian) * (size_t)G, cudaMemcpyDeviceToDevice, s),
                    "blur copies");
      SL_CHECK_CUDA(cudaMemcpyAsync(l->n_blur.ptr, n_rest, sizeof(sl_node) * (size_t)N, cudaMemcpyDeviceToDevice, s),
                    "blur copies");
      blur_mask = all;
      l->blur_init = true;
    } else {
      blur_mask = (moved_mask | l->blur_prev) & all;
    }
    l->blur_prev = moved_mask;
    SL_CHECK_CUDA(launch_blur_records(parts, P, l->blur_shutter, blur_mask, gs, n_rest, l->g_blur.as<sl_gaussian>(),
                                      l->n_blur.as<sl_node>(), G, N, s),
                  "blur_records");
    gsp = l->g_blur.as<sl_gaussian>();
    ndp = l->n_blur.as<sl_node>();
    if (tree) bc.k = l->cut_k;
  }
  const uint32_t resplat = moved_mask | blur_mask;

  // light map A (light_shadow.js:113-165): re-splat every layer when the light changed, else the moved parts'
  const bool lmap = l->n_emit && l->shadow_res;
  if (lmap && (l->lm_dirty || resplat)) {
    LightMapParams& L = l->LP;
    memset(&L, 0, sizeof(L));
    const float* t = reinterpret_cast<const float*>(l->tree.ptr);
    std::vector<float> root(24);
    SL_CHECK_CUDA(cudaMemcpy(root.data(), t + 24u * l->root, 96, cudaMemcpyDeviceToHost), "tree root");
    L.center[0] = root[0];
    L.center[1] = root[1];
    L.center[2] = root[2];
    double n[3] = {l->normal[0], l->normal[1], l->normal[2]};
    double nl = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (double& v : n) v /= nl;
    double a[3] = {std::fabs(n[0]) < 0.9 ? 1.0 : 0.0, std::fabs(n[0]) < 0.9 ? 0.0 : 1.0, 0.0};
    double t1[3] = {n[1] * a[2] - n[2] * a[1], n[2] * a[0] - n[0] * a[2], n[0] * a[1] - n[1] * a[0]};
    double tl = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
    for (double& v : t1) v /= tl;
    double t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
    for (int k = 0; k < 3; k++) {
      L.normal[k] = (float)n[k];
      L.t1[k] = (float)t1[k];
      L.t2[k] = (float)t2[k];
    }
    double ev[3];
    eig3(l->root_cov, ev);
    L.sigma_l = (float)std::sqrt(0.5 * (ev[1] + ev[2]));
    L.hemi = l->one_sided;
    L.res = l->shadow_res;
    levels_for(L.res, L.levels, L.level_off, L.layer_texels);
    L.part_count = P;
    L.skip_part = l->skip_part;
    L.dirty = l->lm_dirty ? (P >= 32 ? 0xFFFFFFFFu : ((1u << P) - 1u)) : resplat;
    const size_t acc_layer = 12ull * L.res * L.res;
    SL_CHECK_CUDA(l->lm_acc.ensure(acc_layer * P), "light map");
    SL_CHECK_CUDA(l->lm_mip.ensure(16ull * L.layer_texels * P), "light map mips");
    for (uint32_t p = 0; p < P; p++)
      if ((L.dirty >> p) & 1u)
        SL_CHECK_CUDA(cudaMemsetAsync(l->lm_acc.as<char>() + acc_layer * p, 0, acc_layer, s), "clear light map");
    SL_CHECK_CUDA(launch_lsm_splat(L, gsp, ndp, parts, G, bc, l->lm_acc.as<uint32_t>(), s), "lsm_splat");
    SL_CHECK_CUDA(launch_resolve(l->lm_acc.as<uint32_t>(), 65536.0f, L.res * L.res, P, L.layer_texels, nullptr,
                                 l->lm_mip.as<float4>(), s),
                  "lsm_resolve");
    SL_CHECK_CUDA(launch_mips(l->lm_mip.as<float4>(), L.res, L.levels, L.level_off, P, L.layer_texels, nullptr, s),
                  "lsm_down");
    SL_CHECK_CUDA(launch_lsm_lookup(L, gs, parts, G, l->lm_mip.as<float4>(), l->lamp_T.as<float>(), s), "lsm_lookup");
    l->lm_dirty = false;
    l->lamp_filled = true;
  } else if (!lmap && !l->lamp_filled) {
    std::vector<float> ones(G, 1.0f);
    SL_CHECK_CUDA(cudaMemcpy(l->lamp_T.ptr, ones.data(), 4ull * G, cudaMemcpyHostToDevice), "lamp T");
    l->lamp_filled = true;
  }

  // sun maps (sun_map.js:23-159)
  const uint32_t K = (uint32_t)std::min<size_t>(l->lights.size(), 4);
  const uint32_t Pn = std::min<uint32_t>(P, 32u);
  if (K && l->sun_res) {
    SunParams& SP = l->SP;
    memset(&SP, 0, sizeof(SP));
    SP.res = l->sun_res;
    levels_for(SP.res, SP.levels, SP.level_off, SP.layer_texels);
    SP.n_parts = Pn;
    for (uint32_t k = 0; k < K; k++) {
      for (int c = 0; c < 3; c++) {
        SP.lights[k].dir[c] = l->lights[k].dir[c];
        SP.lights[k].irr[c] = l->lights[k].irradiance[c];
      }
      SP.lights[k].std = l->lights[k].std;
      SP.lights[k].shadows = l->lights[k].casts_shadows ? 1u : 0u;
    }
    // the layer plan: per part with Gaussians and per light, cascades then the fitted map (sun_map.js:40-52)
    double ext = 0.0, sig_max = 0.0;
    for (uint32_t p = 0; p < Pn; p++) {
      const float* b = r->parts[p].bound;
      ext = std::max(ext, std::sqrt((double)b[0] * b[0] + (double)b[1] * b[1] + (double)b[2] * b[2]) + b[3]);
    }
    for (uint32_t k = 0; k < K; k++) sig_max = std::max(sig_max, (double)l->lights[k].std);
    const float margin = (float)(3.0 * sig_max * 2.0 * ext);
    const double kCasc[2] = {8.0, 32.0};
    std::vector<SunLayer> plan;
    for (uint32_t p = 0; p < Pn; p++) {
      SP.part_first[p] = (uint32_t)plan.size();
      const sl_part& part = r->parts[p];
      if (part.g_hi > part.g_lo) {
        const bool big = part.bound[3] > kCasc[0] && (part.flags & 1u);
        for (uint32_t k = 0; k < K; k++) {
          float Ld[3] = {l->lights[k].dir[0], l->lights[k].dir[1], l->lights[k].dir[2]};
          float t1[3], t2[3];
          basis_k32(Ld, t1, t2);
          if (big)
            for (int c = 0; c < 2; c++) {
              if (!(kCasc[c] < part.bound[3] * 1.5)) continue;
              double L64[3] = {Ld[0], Ld[1], Ld[2]}, c1[3];
              basis_k64(L64, c1);
              double c2[3] = {L64[1] * c1[2] - L64[2] * c1[1], L64[2] * c1[0] - L64[0] * c1[2], L64[0] * c1[1] - L64[1] * c1[0]};
              double h = kCasc[c];
              double at[3];
              for (int q = 0; q < 3; q++) at[q] = (double)eye[q] + (forward ? (double)forward[q] : 0.0) * h * 0.75;
              SunLayer ly{};
              ly.c[0] = (float)(at[0] * c1[0] + at[1] * c1[1] + at[2] * c1[2]);
              ly.c[1] = (float)(at[0] * c2[0] + at[1] * c2[1] + at[2] * c2[2]);
              ly.half = (float)h;
              ly.kind = 1;
              ly.part = p;
              ly.light = k;
              plan.push_back(ly);
            }
          SunLayer ly{};
          ly.kind = 0;
          ly.part = p;
          ly.light = k;
          plan.push_back(ly);
        }
      }
      SP.part_layers[p] = (uint32_t)plan.size() - SP.part_first[p];
    }
    // sm_frame (sun_map.wgsl:91-107) on the host, in float32 with the kernels' rounding order; dirty flags
    const size_t nl = plan.size();
    if (l->layers.size() != nl) {
      l->layers.assign(nl, SunLayer{});
      l->have_center.assign(nl, 0);
      l->sm_dirty_all = true;
    }
    bool any = false;
    for (size_t li = 0; li < nl; li++) {
      SunLayer& ly = plan[li];
      const sl_part& part = r->parts[ly.part];
      float Ld[3] = {l->lights[ly.light].dir[0], l->lights[ly.light].dir[1], l->lights[ly.light].dir[2]};
      basis_k32(Ld, ly.t1, ly.t2);
      const float* b = part.bound;
      const float* xf = part.xf;
      volatile float cx = xf[0] * b[0] + xf[1] * b[1] + xf[2] * b[2] + xf[3];
      volatile float cy = xf[4] * b[0] + xf[5] * b[1] + xf[6] * b[2] + xf[7];
      volatile float cz = xf[8] * b[0] + xf[9] * b[1] + xf[10] * b[2] + xf[11];
      bool dirty = l->sm_dirty_all || ((resplat >> ly.part) & 1u);
      if (ly.kind == 1u) {
        const SunLayer& old = l->layers[li];
        const float h = ly.half;
        if (l->have_center[li] && !l->sm_dirty_all &&
            std::hypot((double)ly.c[0] - old.c[0], (double)ly.c[1] - old.c[1]) <= h / 4) {
          ly.c[0] = old.c[0];
          ly.c[1] = old.c[1];
        } else {
          dirty = true;
        }
        l->have_center[li] = 1;
      } else {
        volatile float d0 = cx * ly.t1[0] + cy * ly.t1[1] + cz * ly.t1[2];
        volatile float d1 = cx * ly.t2[0] + cy * ly.t2[1] + cz * ly.t2[2];
        ly.c[0] = d0;
        ly.c[1] = d1;
        ly.half = b[3] + margin;
      }
      volatile float zr = cx * Ld[0] + cy * Ld[1] + cz * Ld[2];
      ly.zref = zr + b[3];
      ly.dirty = dirty ? 1u : 0u;
      any = any || dirty;
    }
    SP.n_layers = (uint32_t)nl;
    if (any) {
      const size_t acc_layer = 12ull * SP.res * SP.res;
      SL_CHECK_CUDA(l->sm_acc.ensure(acc_layer * std::max<size_t>(nl, 1)), "sun map");
      SL_CHECK_CUDA(l->sm_mip.ensure(16ull * SP.layer_texels * std::max<size_t>(nl, 1)), "sun map mips");
      SL_CHECK_CUDA(l->sm_layers.ensure(sizeof(SunLayer) * std::max<size_t>(nl, 1)), "sun layers");
      SL_CHECK_CUDA(l->sm_dirty.ensure(4 * std::max<size_t>(nl, 1)), "sun dirty");
      std::vector<uint32_t> dl(nl);
      for (size_t li = 0; li < nl; li++) {
        dl[li] = plan[li].dirty;
        if (plan[li].dirty)
          SL_CHECK_CUDA(cudaMemsetAsync(l->sm_acc.as<char>() + acc_layer * li, 0, acc_layer, s), "clear sun map");
      }
      SL_CHECK_CUDA(cudaMemcpyAsync(l->sm_layers.ptr, plan.data(), sizeof(SunLayer) * nl, cudaMemcpyHostToDevice, s),
                    "sun layers");
      SL_CHECK_CUDA(cudaMemcpyAsync(l->sm_dirty.ptr, dl.data(), 4 * nl, cudaMemcpyHostToDevice, s), "sun dirty");
      SL_CHECK_CUDA(launch_sm_splat(SP, l->sm_layers.as<SunLayer>(), gsp, ndp, parts, G, bc, l->sm_acc.as<uint32_t>(),
                                    s),
                    "sm_splat");
      SL_CHECK_CUDA(launch_resolve(l->sm_acc.as<uint32_t>(), 4096.0f, SP.res * SP.res, (uint32_t)nl, SP.layer_texels,
                                   l->sm_dirty.as<uint32_t>(), l->sm_mip.as<float4>(), s),
                    "sm_resolve");
      SL_CHECK_CUDA(launch_mips(l->sm_mip.as<float4>(), SP.res, SP.levels, SP.level_off, (uint32_t)nl, SP.layer_texels,
                                l->sm_dirty.as<uint32_t>(), s),
                    "sm_down");
      SL_CHECK_CUDA(launch_sm_lookup(SP, l->sm_layers.as<SunLayer>(), gs, parts, G, l->sm_mip.as<float4>(),
                                     l->env_T.as<float4>(), s),
                    "sm_lookup");
      SL_CHECK_CUDA(cudaStreamSynchronize(s), "sun maps");  // plan/dl host vectors go out of scope
      l->layers = plan;
      l->sm_dirty_all = false;
      l->env_filled = true;
    }
  } else if (!l->env_filled) {
    std::vector<float> ones(4ull * G, 1.0f);
    SL_CHECK_CUDA(cudaMemcpy(l->env_T.ptr, ones.data(), 16ull * G, cudaMemcpyHostToDevice), "env T");
    l->env_filled = true;
  }

  // shade (emissive.wgsl shade_emit + environment.wgsl env_direct + the constant sky ambient)
  ShadeParams SH;
  shade_params(l, eye, SH);
  SL_CHECK_CUDA(launch_shade(SH, gs, l->nodes.as<sl_node>(), l->vgrid.as<sl_vgrid>(), parts, l->materials.as<sl_material>(),
                             l->tree.as<float>(), l->lamp_T.as<float>(), l->env_T.as<float4>(), l->order.as<uint32_t>(),
                             l->colour.as<float4>(), G, s),
                "shade");
  if (l->bounce_on) {  // the probe bounce after the shading (lighting.js encodeBounce)
    for (uint32_t q = 0; q < P; q++)
      if (r->parts[q].root != 0xFFFFFFFFu && r->parts[q].root >= l->n_tree)
        return fail(SL_ERR_INVALID_ARG, "a part's tree root lies outside the tree set by sl_lighting_set_tree");
    if (P != l->BP.part_count)
      return fail(SL_ERR_INVALID_ARG, "the part count changed since sl_lighting_set_probes: set the probes again");
    BounceParams B = l->BP;
    B.alpha = l->bn_first ? 1.0f : l->bn_blend;
    B.frame = l->bn_frame;
    B.force = l->bn_first ? 1u : 0u;
    B.moved_mask = moved_mask;
    B.has_sky = l->has_sky ? 1u : 0u;
    B.dark_part = l->bn_emit_dark ? l->skip_part : 0xFFFFFFFFu;
    B.asg_cells = l->asg ? 1u : 0u;
    B.sender_cut = l->bn_sc ? 1u : 0u;
    B.sc_reselect = l->bn_sc && (l->bn_sc_stale || moved_mask != 0u) ? 1u : 0u;
    memcpy(B.sky, l->sky, sizeof(B.sky));
    for (int k = 0; k < 3; k++) B.eye[k] = eye[k];
    ShadeParams SHd;
    shade_params(l, eye, SHd);
    BounceBuffers D{};
    D.gs = gs;
    D.nodes = l->nodes.as<sl_node>();
    D.tnodes = l->tree_nodes.as<sl_node>();
    D.kids = l->kids.as<uint32_t>();
    D.vgrid = l->vgrid.as<sl_vgrid>();
    D.parts = parts;
    D.mats = l->materials.as<sl_material>();
    D.tree = l->tree.as<float>();
    D.lamp_T = l->lamp_T.as<float>();
    D.env_T = l->env_T.as<float4>();
    D.tab = l->bn_tab.as<float>();
    D.ground = l->bn_ground.as<float>();
    D.up_list = l->bn_up.as<uint32_t>();
    D.quarters = l->bn_quarters.as<uint32_t>();
    D.leaf_w = l->bn_leaf_w.as<float>();
    D.probe_hist = l->probe_hist.as<float4>();
    for (int q = 0; q < 5; q++) D.quarter_off[q] = l->bn_quarter_off[q];
    D.xfer = l->xfer.as<float4>();
    D.lo_dir = l->lo_dir.as<float4>();
    D.lo_b = l->lo_b.as<float4>();
    D.node_acc = l->node_acc.as<float4>();
    D.probe_data = l->probe_data.as<float4>();
    D.probe_sh = l->probe_sh.as<float4>();
    D.node_sh = l->node_sh.as<uint32_t>();
    if (l->bn_sc) {
      D.sc_level = l->sc_level.as<uint32_t>();
      D.parent = l->node_parent.as<uint32_t>();
      D.sc_gs = l->sc_gs.as<sl_gaussian>();
      D.sc_vg = l->sc_vg.as<sl_vgrid>();
      D.sc_flag = l->sc_flag.as<uint32_t>();
      D.sc_X = l->sc_X.as<float4>();
      D.sc_T = l->sc_T.as<float>();
      D.sc_E = l->sc_E.as<float4>();
      D.sc_list = l->sc_list.as<uint32_t>();
    }
    SL_CHECK_CUDA(launch_bounce_frame(B, SHd, D, l->bn_level_off, l->bn_level_cnt, l->sc_level_off, l->sc_level_cnt,
                                      s),
                  "probe bounce");
    l->bn_first = false;
    if (B.sc_reselect) l->bn_sc_stale = false;
    l->bn_frame++;
  }
  return SL_OK;
}

int sl_lighting_shade(sl_lighting* l, const float* eye, void* stream) {
  if (!l || !eye) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (!l->iso_done) return fail(SL_ERR_INVALID_ARG, "shade needs a prior sl_lighting_update (maps, iso_norm)");
  cudaSetDevice(l->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  ShadeParams SH;
  shade_params(l, eye, SH);
  SL_CHECK_CUDA(launch_shade(SH, l->r->gaussians.as<sl_gaussian>(), l->nodes.as<sl_node>(), l->vgrid.as<sl_vgrid>(),
                             l->parts.as<sl_part>(), l->materials.as<sl_material>(), l->tree.as<float>(),
                             l->lamp_T.as<float>(), l->env_T.as<float4>(), l->order.as<uint32_t>(),
                             l->colour.as<float4>(), l->count, s),
                "shade");
  return SL_OK;
}

int sl_lighting_read(sl_lighting* l, float* colour, float* lamp_T, float* env_T, sl_node* nodes) {
  if (!l) return fail(SL_ERR_INVALID_ARG, "null lighting");
  cudaSetDevice(l->device);
  SL_CHECK_CUDA(cudaDeviceSynchronize(), "sync");
  const size_t G = l->count;
  if (colour) SL_CHECK_CUDA(cudaMemcpy(colour, l->colour.ptr, 16 * G, cudaMemcpyDeviceToHost), "colour");
  if (lamp_T) SL_CHECK_CUDA(cudaMemcpy(lamp_T, l->lamp_T.ptr, 4 * G, cudaMemcpyDeviceToHost), "lamp T");
  if (env_T) SL_CHECK_CUDA(cudaMemcpy(env_T, l->env_T.ptr, 16 * G, cudaMemcpyDeviceToHost), "env T");
  if (nodes) SL_CHECK_CUDA(cudaMemcpy(nodes, l->nodes.ptr, sizeof(sl_node) * G, cudaMemcpyDeviceToHost), "nodes");
  return SL_OK;
}

int sl_renderer_bind_lighting(sl_renderer* r, sl_lighting* l) {
  if (!r || !l) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (l->r != r) return fail(SL_ERR_INVALID_ARG, "the lighting object belongs to another renderer");
  r->lighting = l;
  r->colour = l->colour.as<float4>();
  r->lo_b = l->bounce_on ? l->lo_b.as<float4>() : nullptr;
  return SL_OK;
}

int sl_lighting_set_probes(sl_lighting* l, const sl_probe_layout* lay, uint32_t max_depth, float blend,
                           int emitters_dark) {
  if (!l || !lay) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (l->n_tree < l->count || l->tree_depth.size() != l->n_tree)
    return fail(SL_ERR_INVALID_ARG, "the probe gather walks the scene's tree: sl_lighting_set_tree first");
  const uint32_t dx = lay->dims[0], dy = lay->dims[1], dz = lay->dims[2];
  if (dx < 2 || dy < 2 || dz < 2 || dz > 16 || (uint64_t)dx * dy > 1024)
    return fail(SL_ERR_INVALID_ARG, "probe layout: 2..16 levels and 2 x 2 .. 1024 columns");
  if (!(lay->tmax > 0.0f) || !(lay->step[0] > 0.0f) || !(lay->step[1] > 0.0f))
    return fail(SL_ERR_INVALID_ARG, "probe layout: positive spacing and ray length");
  for (uint32_t k = 0; k + 1 < dz; k++)
    if (!(lay->levels[k + 1] > lay->levels[k])) return fail(SL_ERR_INVALID_ARG, "probe levels must ascend");
  if (!((blend > 0.0f && blend <= 1.0f) || blend == -1.0f))
    return fail(SL_ERR_INVALID_ARG, "blend must be in (0, 1], or -1 (the FIR blend)");
  if (lay->n_vols > 32) return fail(SL_ERR_INVALID_ARG, "at most 32 probe volumes");
  cudaSetDevice(l->device);
  const uint32_t G = l->count, N = l->n_tree, NL = dx * dy * dz, P = l->r->part_count;
  BounceParams& B = l->BP;
  B = BounceParams{};
  // the probes after the lattice: 8 per part, then the volumes' grids (lighting.js:739-740, 797-799)
  uint32_t off = 8u * P;
  for (uint32_t v = 0; v < lay->n_vols; v++) {
    const uint32_t q = lay->vols[v][0], nx = lay->vols[v][1], ny = lay->vols[v][2], nz = lay->vols[v][3];
    if (q >= 32 || q >= P) return fail(SL_ERR_INVALID_ARG, "a probe volume names a part outside 0-31 or the scene");
    if (l->r->parts[q].root >= N) return fail(SL_ERR_INVALID_ARG, "a probe volume's part has no tree root");
    if (nx < 2 || ny < 2 || nz < 2 || nx > 64 || ny > 64 || nz > 64)
      return fail(SL_ERR_INVALID_ARG, "probe volume grids take 2-64 probes per axis");
    if (B.vol_dims[q][0]) return fail(SL_ERR_INVALID_ARG, "two probe volumes on one part");
    B.vol_first[q] = off;
    B.vol_dims[q][0] = nx;
    B.vol_dims[q][1] = ny;
    B.vol_dims[q][2] = nz;
    off += nx * ny * nz;
  }
  const uint32_t NP = NL + off;
  B.G = G;
  B.N = N;
  B.NP = NP;
  B.NL = NL;
  B.part_count = P;
  B.mat_count = l->material_count;
  B.dims[0] = dx;
  B.dims[1] = dy;
  B.dims[2] = dz;
  B.terrain = lay->terrain ? 1u : 0u;
  for (int k = 0; k < 3; k++) {
    B.lo[k] = lay->lo[k];
    B.step[k] = lay->step[k];
  }
  for (uint32_t k = 0; k < 16; k++) B.levels[k] = lay->levels[k];
  B.tmax = lay->tmax;
  // block_rad (lighting.js:794): half the cell diagonal, float64; terrain probes each cut around themselves
  B.brad = B.terrain ? 0.0f
                     : (float)(0.5 * std::sqrt((double)B.step[0] * B.step[0] + (double)B.step[1] * B.step[1] +
                                               (double)B.step[2] * B.step[2]));
  // node_up's lists: internal nodes with a part at depths 1 .. max_depth - 1 (lighting.js:771-789)
  uint32_t md = max_depth;
  if (md == 0)
    for (uint32_t i = G; i < N; i++) md = std::max(md, l->tree_depth[i] + 1u);
  std::vector<std::vector<uint32_t>> by(md + 1);
  for (uint32_t i = G; i < N; i++)
    if (l->tree_part[i] != 0xFFFFFFFFu && l->tree_depth[i] <= md) by[l->tree_depth[i]].push_back(i);
  std::vector<uint32_t> up;
  l->bn_level_off.assign(md, 0);
  l->bn_level_cnt.assign(md, 0);
  for (uint32_t d = 0; d < md; d++) {
    l->bn_level_off[d] = (uint32_t)up.size();
    l->bn_level_cnt[d] = (uint32_t)by[d].size();
    up.insert(up.end(), by[d].begin(), by[d].end());
  }
  // direct_dirs_emit's quarters (g % 4 == frame % 4), each in the shading pass's Morton order so a warp's Gaussians
  // share their light cuts
  {
    std::vector<uint32_t> order(G), q4;
    q4.reserve(G);
    SL_CHECK_CUDA(cudaMemcpy(order.data(), l->order.ptr, 4ull * G, cudaMemcpyDeviceToHost), "shading order");
    for (uint32_t q = 0; q < 4; q++) {
      l->bn_quarter_off[q] = (uint32_t)q4.size();
      for (uint32_t g : order)
        if (g % 4u == q) q4.push_back(g);
    }
    l->bn_quarter_off[4] = (uint32_t)q4.size();
    SL_CHECK_CUDA(l->bn_quarters.ensure(4ull * G + 16), "quarters");
    if (G) SL_CHECK_CUDA(cudaMemcpy(l->bn_quarters.ptr, q4.data(), 4ull * G, cudaMemcpyHostToDevice), "quarters");
  }
  float tab[kTabFloats];
  iso_dirs(tab + kTabCells);
  bounce_tables(tab + kTabD14, tab + kTabPinv);
  cell_asg_table(tab + kTabCellAsg);
  SL_CHECK_CUDA(l->bn_tab.ensure(sizeof(tab)), "bounce table");
  SL_CHECK_CUDA(cudaMemcpy(l->bn_tab.ptr, tab, sizeof(tab), cudaMemcpyHostToDevice), "bounce table");
  SL_CHECK_CUDA(l->bn_up.ensure(4ull * up.size() + 16), "node_up lists");
  if (!up.empty()) SL_CHECK_CUDA(cudaMemcpy(l->bn_up.ptr, up.data(), 4ull * up.size(), cudaMemcpyHostToDevice), "lists");
  SL_CHECK_CUDA(l->bn_ground.ensure(4ull * dx * dy), "ground");
  std::vector<float> ground(dx * dy, 0.0f);
  if (lay->ground) memcpy(ground.data(), lay->ground, 4ull * dx * dy);
  SL_CHECK_CUDA(cudaMemcpy(l->bn_ground.ptr, ground.data(), 4ull * dx * dy, cudaMemcpyHostToDevice), "ground");
  struct Sz {
    sl::DevBuf* b;
    size_t bytes;
  } bufs[] = {{&l->probe_data, 32ull * NP * 128}, {&l->probe_sh, 144ull * NP}, {&l->xfer, 48ull * G},
              {&l->lo_dir, 16ull * G}, {&l->lo_b, 48ull * G}, {&l->node_acc, 224ull * N}, {&l->node_sh, 56ull * N},
              {&l->bn_leaf_w, 56ull * G}, {&l->probe_hist, 64ull * NP * 128}};
  for (const Sz& z : bufs) {
    SL_CHECK_CUDA(z.b->ensure(z.bytes), "bounce buffers");
    SL_CHECK_CUDA(cudaMemset(z.b->ptr, 0, z.bytes), "bounce buffers");
  }
  l->bn_blend = blend;
  l->bn_emit_dark = emitters_dark != 0;
  l->bn_first = true;
  l->bn_sc_stale = true;  // the cut is selected over the new probes
  l->bn_frame = 0;
  l->bounce_on = true;
  if (l->r && l->r->lighting == l) l->r->lo_b = l->lo_b.as<float4>();
  return SL_OK;
}

int sl_lighting_set_sky(sl_lighting* l, const float* sh_rgb, uint32_t n_coef) {
  if (!l || (n_coef && !sh_rgb)) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (n_coef > 16) return fail(SL_ERR_INVALID_ARG, "the probes' sky holds SH bands 0-3 (16 coefficients)");
  memset(l->sky, 0, sizeof(l->sky));
  if (n_coef) memcpy(l->sky, sh_rgb, 12ull * n_coef);
  l->has_sky = n_coef > 0;
  l->bn_first = true;  // the probes re-gather the new sky (environment.js:151)
  return SL_OK;
}

int sl_lighting_set_sender_cut(sl_lighting* l, uint32_t on) {
  if (!l) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (!on) {
    l->bn_sc = false;
    return SL_OK;
  }
  if (!l->bounce_on) return fail(SL_ERR_INVALID_ARG, "the sender cut selects over the probes: sl_lighting_set_probes first");
  if (!l->r) return fail(SL_ERR_INVALID_ARG, "the sender cut needs the renderer bound (its Gaussians)");
  cudaSetDevice(l->device);
  const uint32_t G = l->count, N = l->n_tree;
  std::vector<sl_node> nodes(N);
  std::vector<uint32_t> kids(l->n_kids);
  std::vector<sl_gaussian> gs(G);
  std::vector<sl_vgrid> vg(G);
  SL_CHECK_CUDA(cudaDeviceSynchronize(), "sync");
  SL_CHECK_CUDA(cudaMemcpy(nodes.data(), l->tree_nodes.ptr, sizeof(sl_node) * (size_t)N, cudaMemcpyDeviceToHost), "tree");
  if (l->n_kids)
    SL_CHECK_CUDA(cudaMemcpy(kids.data(), l->kids.ptr, 4ull * l->n_kids, cudaMemcpyDeviceToHost), "kids");
  SL_CHECK_CUDA(cudaMemcpy(gs.data(), l->r->gaussians.ptr, sizeof(sl_gaussian) * (size_t)G, cudaMemcpyDeviceToHost),
                "gaussians");
  SL_CHECK_CUDA(cudaMemcpy(vg.data(), l->vgrid.ptr, sizeof(sl_vgrid) * (size_t)G, cudaMemcpyDeviceToHost), "vgrid");
  // sc_shadow's descents take at most 64 steps, and each picks among a node's children
  uint32_t maxd = 0;
  for (uint32_t n = 0; n < N; n++) {
    maxd = std::max(maxd, nodes[n].depth);
    if (n >= G && nodes[n].part != 0xFFFFFFFFu && nodes[n].child_hi <= nodes[n].child_lo)
      return fail(SL_ERR_INVALID_ARG, "the sender cut needs every internal node of a part to have children");
  }
  if (maxd > 64u) return fail(SL_ERR_INVALID_ARG, "the sender cut's shadow descents reach 64 levels: tree too deep");
  std::vector<sl_gaussian> recs;
  std::vector<sl_vgrid> nvg;
  int rc = sl::node_records(gs.data(), G, nodes.data(), N, kids.data(), l->n_kids, recs, vg.data(), &nvg);
  if (rc != SL_OK) return rc;
  // sc_select's levels: every node by depth, index order within a depth
  std::vector<std::vector<uint32_t>> by(maxd + 1);
  for (uint32_t n = 0; n < N; n++) by[nodes[n].depth].push_back(n);
  std::vector<uint32_t> level;
  level.reserve(N);
  l->sc_level_off.assign(maxd + 1, 0);
  l->sc_level_cnt.assign(maxd + 1, 0);
  for (uint32_t d = 0; d <= maxd; d++) {
    l->sc_level_off[d] = (uint32_t)level.size();
    l->sc_level_cnt[d] = (uint32_t)by[d].size();
    level.insert(level.end(), by[d].begin(), by[d].end());
  }
  const size_t I = N - G;
  SL_CHECK_CUDA(l->sc_level.ensure(4ull * N + 16), "sender cut");
  SL_CHECK_CUDA(l->sc_gs.ensure(sizeof(sl_gaussian) * I + 16), "sender cut");
  SL_CHECK_CUDA(l->sc_vg.ensure(sizeof(sl_vgrid) * I + 16), "sender cut");
  SL_CHECK_CUDA(l->sc_flag.ensure(4ull * N + 16), "sender cut");
  SL_CHECK_CUDA(l->sc_X.ensure(128ull * I + 16), "sender cut");
  SL_CHECK_CUDA(l->sc_T.ensure(4ull * I + 16), "sender cut");
  SL_CHECK_CUDA(l->sc_E.ensure(16ull * I + 16), "sender cut");
  SL_CHECK_CUDA(l->sc_list.ensure(4ull * I + 16), "sender cut");
  if (N) SL_CHECK_CUDA(cudaMemcpy(l->sc_level.ptr, level.data(), 4ull * N, cudaMemcpyHostToDevice), "sender cut");
  if (I) {
    SL_CHECK_CUDA(cudaMemcpy(l->sc_gs.ptr, recs.data(), sizeof(sl_gaussian) * I, cudaMemcpyHostToDevice), "sender cut");
    SL_CHECK_CUDA(cudaMemcpy(l->sc_vg.ptr, nvg.data(), sizeof(sl_vgrid) * I, cudaMemcpyHostToDevice), "sender cut");
  }
  SL_CHECK_CUDA(cudaMemset(l->sc_flag.ptr, 0, 4ull * N + 16), "sender cut");
  SL_CHECK_CUDA(cudaMemset(l->sc_X.ptr, 0, 128ull * I + 16), "sender cut");
  SL_CHECK_CUDA(cudaMemset(l->sc_T.ptr, 0, 4ull * I + 16), "sender cut");
  SL_CHECK_CUDA(cudaMemset(l->sc_E.ptr, 0, 16ull * I + 16), "sender cut");
  SL_CHECK_CUDA(cudaMemset(l->sc_list.ptr, 0, 4ull * I + 16), "sender cut");
  l->bn_sc = true;
  l->bn_sc_stale = true;
  return SL_OK;
}

int sl_lighting_read_bounce(sl_lighting* l, uint32_t what, void* dst, size_t bytes) {
  if (!l || !dst) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (!l->bounce_on) return fail(SL_ERR_INVALID_ARG, "no probes set");
  const size_t G = l->count, N = l->n_tree, NP = l->BP.NP, I = N - G;
  const sl::DevBuf* src[] = {&l->lo_b, &l->lo_dir, &l->xfer, &l->probe_sh, &l->probe_data, &l->node_sh,
                             &l->node_acc, &l->sc_flag, &l->sc_X, &l->sc_T, &l->sc_E};
  const size_t size[] = {48 * G, 16 * G, 48 * G, 144 * NP, 32 * NP * 128, 56 * N, 224 * N, 4 * N, 128 * I, 4 * I,
                         16 * I};
  if (what >= 11) return fail(SL_ERR_INVALID_ARG, "unknown bounce buffer");
  if (what >= 7 && !l->bn_sc) return fail(SL_ERR_INVALID_ARG, "the sender cut is off");
  if (bytes > size[what]) return fail(SL_ERR_INVALID_ARG, "read past the bounce buffer");
  cudaSetDevice(l->device);
  SL_CHECK_CUDA(cudaDeviceSynchronize(), "sync");
  SL_CHECK_CUDA(cudaMemcpy(dst, src[what]->ptr, bytes, cudaMemcpyDeviceToHost), "bounce read");
  return SL_OK;
}

}  // extern "C"
