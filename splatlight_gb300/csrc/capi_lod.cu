// Screen-space LOD (C ABI): src/lod.js's nodeGaussians (the internal nodes of the scene's tree as Gaussian records,
// float64 on the host) and Lod (the per-depth node lists; encodeSelect / encodeColour as one kernel launch per large
// depth and one for the small top depths together, csrc/lod.cu).  The renderer's projection draws the cut for frames with frame.lod on (csrc/project.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sl_runtime.h"

namespace sl {
namespace {

using M3d = double[3][3];

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (src/lod.js:9-23): values ascending, vectors[k] the
// k-th column (ties keep index order).
void eig3(const M3d A, double vals[3], double vecs[3][3]) {
  double a[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  memcpy(a, A, sizeof(a));
  for (int sweep = 0; sweep < 20; sweep++) {
    double off = 0.0;
    for (int p = 0; p < 3; p++)
      for (int q = p + 1; q < 3; q++) off += a[p][q] * a[p][q];
    if (off < 1e-30) break;
    for (int p = 0; p < 3; p++)
      for (int q = p + 1; q < 3; q++) {
        if (std::fabs(a[p][q]) < 1e-30) continue;
        const double th = 0.5 * std::atan2(2.0 * a[p][q], a[q][q] - a[p][p]);
        const double c = std::cos(th), s = std::sin(th);
        for (int k = 0; k < 3; k++) {
          const double x = a[k][p], y = a[k][q];
          a[k][p] = c * x - s * y;
          a[k][q] = s * x + c * y;
        }
        for (int k = 0; k < 3; k++) {
          const double x = a[p][k], y = a[q][k];
          a[p][k] = c * x - s * y;
          a[q][k] = s * x + c * y;
        }
        for (int k = 0; k < 3; k++) {
          const double x = V[k][p], y = V[k][q];
          V[k][p] = c * x - s * y;
          V[k][q] = s * x + c * y;
        }
      }
  }
  int idx[3] = {0, 1, 2};
  std::stable_sort(idx, idx + 3, [&](int i, int j) { return a[i][i] < a[j][j]; });
  for (int k = 0; k < 3; k++) {
    vals[k] = a[idx[k]][idx[k]];
    for (int r = 0; r < 3; r++) vecs[k][r] = V[r][idx[k]];
  }
}

// The rotation with columns c[0..2] as a quaternion (x, y, z, w), quat_to_mat's convention (src/lod.js:26-37).
void quat_from_columns(const double c[3][3], double q[4]) {
  const double m00 = c[0][0], m11 = c[1][1], m22 = c[2][2];
  const double m10 = c[0][1], m20 = c[0][2], m01 = c[1][0], m21 = c[1][2], m02 = c[2][0], m12 = c[2][1];
  const double tr = m00 + m11 + m22;
  double x, y, z, w;
  if (tr > 0) {
    const double s = 2.0 * std::sqrt(tr + 1.0);
    w = s / 4.0;
    x = (m21 - m12) / s;
    y = (m02 - m20) / s;
    z = (m10 - m01) / s;
  } else if (m00 > m11 && m00 > m22) {
    const double s = 2.0 * std::sqrt(1.0 + m00 - m11 - m22);
    x = s / 4.0;
    w = (m21 - m12) / s;
    y = (m01 + m10) / s;
    z = (m02 + m20) / s;
  } else if (m11 > m22) {
    const double s = 2.0 * std::sqrt(1.0 + m11 - m00 - m22);
    y = s / 4.0;
    w = (m02 - m20) / s;
    x = (m01 + m10) / s;
    z = (m12 + m21) / s;
  } else {
    const double s = 2.0 * std::sqrt(1.0 + m22 - m00 - m11);
    z = s / 4.0;
    w = (m10 - m01) / s;
    x = (m02 + m20) / s;
    y = (m12 + m21) / s;
  }
  double l = std::sqrt(x * x + y * y + z * z + w * w);
  if (!(l > 0.0)) l = 1.0;
  q[0] = x / l;
  q[1] = y / l;
  q[2] = z / l;
  q[3] = w / l;
}

// A node's covariance (the inverse of its cinv, by the adjugate) and det(cinv) (src/lod.js:52-62).
void node_cov(const sl_node& nd, M3d C, double* det_out) {
  const double M[3][3] = {{nd.cinv_diag[0], nd.cinv_off[0], nd.cinv_off[1]},
                          {nd.cinv_off[0], nd.cinv_diag[1], nd.cinv_off[2]},
                          {nd.cinv_off[1], nd.cinv_off[2], nd.cinv_diag[2]}};
  const double det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                     M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                     M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
  const double inv[3][3] = {{M[1][1] * M[2][2] - M[1][2] * M[2][1], M[0][2] * M[2][1] - M[0][1] * M[2][2],
                             M[0][1] * M[1][2] - M[0][2] * M[1][1]},
                            {M[1][2] * M[2][0] - M[1][0] * M[2][2], M[0][0] * M[2][2] - M[0][2] * M[2][0],
                             M[0][2] * M[1][0] - M[0][0] * M[1][2]},
                            {M[1][0] * M[2][1] - M[1][1] * M[2][0], M[0][1] * M[2][0] - M[0][0] * M[2][1],
                             M[0][0] * M[1][1] - M[0][1] * M[1][0]}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) C[i][j] = inv[i][j] / det;
  *det_out = det;
}

}  // namespace

// nodeGaussians (src/lod.js:44-107): internal nodes G..N-1 as Gaussian records, children before parents; with vg
// their V grids too (lod.js:47-50, 86-88, 99-103): per cell the mass-weighted mean of the children's, kept as float32
// (each addition rounded there), then rounded half up and clamped at 255.
int node_records(const sl_gaussian* gauss, uint32_t G, const sl_node* nodes, uint32_t N, const uint32_t* kids,
                 uint32_t n_kids, std::vector<sl_gaussian>& out, const sl_vgrid* leaf_vg,
                 std::vector<sl_vgrid>* vg) {
  std::vector<float> V;
  if (vg) V.assign((size_t)(N - G) * 128u, 0.0f);
  std::vector<double> mass(N), alb(3 * (size_t)N);
  std::vector<uint32_t> mat(N, 0);
  for (uint32_t g = 0; g < G; g++) {
    M3d C;
    double det;
    node_cov(nodes[g], C, &det);
    mass[g] = (double)nodes[g].kappa / std::sqrt(std::max(det, 1e-30));
    for (int c = 0; c < 3; c++) alb[3 * (size_t)g + c] = gauss[g].albedo[c];
    mat[g] = gauss[g].flags & 0xFFFFu;
  }
  std::vector<uint32_t> order;
  for (uint32_t n = G; n < N; n++) order.push_back(n);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return nodes[a].depth > nodes[b].depth; });
  out.assign(N - G, sl_gaussian{});
  for (uint32_t n : order) {
    const uint32_t lo = nodes[n].child_lo, hi = nodes[n].child_hi;
    if (lo > hi || hi > n_kids) return fail(SL_ERR_INVALID_ARG, "node " + std::to_string(n) + ": children out of range");
    double m = 0.0, c[3] = {0.0, 0.0, 0.0};
    for (uint32_t k = lo; k < hi; k++) {
      const uint32_t ch = kids[k];
      if (ch >= N) return fail(SL_ERR_INVALID_ARG, "kids: node index out of range");
      m += mass[ch];
      for (int j = 0; j < 3; j++) c[j] += mass[ch] * alb[3 * (size_t)ch + j];
    }
    mass[n] = m;
    for (int j = 0; j < 3; j++) alb[3 * (size_t)n + j] = c[j] / std::max(m, 1e-30);
    if (vg) {
      float* vn = V.data() + (size_t)(n - G) * 128u;
      for (uint32_t k = lo; k < hi; k++) {
        const uint32_t ch = kids[k];
        const double w = mass[ch] / std::max(m, 1e-30);
        const uint8_t* lb = ch < G ? reinterpret_cast<const uint8_t*>(&leaf_vg[ch]) : nullptr;
        const float* vc = ch < G ? nullptr : V.data() + (size_t)(ch - G) * 128u;
        for (int q = 0; q < 128; q++) vn[q] = (float)((double)vn[q] + w * (double)(lb ? (float)lb[q] : vc[q]));
      }
    }
    mat[n] = hi > lo ? mat[kids[lo]] : 0u;
    M3d C;
    double det_unused;
    node_cov(nodes[n], C, &det_unused);
    double vals[3], cols[3][3];
    eig3(C, vals, cols);
    const double det = cols[0][0] * (cols[1][1] * cols[2][2] - cols[1][2] * cols[2][1]) -
                       cols[1][0] * (cols[0][1] * cols[2][2] - cols[0][2] * cols[2][1]) +
                       cols[2][0] * (cols[0][1] * cols[1][2] - cols[0][2] * cols[1][1]);
    if (det < 0)
      for (int r = 0; r < 3; r++) cols[2][r] = -cols[2][r];
    double q[4];
    quat_from_columns(cols, q);
    sl_gaussian& o = out[n - G];
    for (int j = 0; j < 3; j++) o.mu[j] = nodes[n].mean[j];
    o.kappa = nodes[n].kappa;
    for (int j = 0; j < 4; j++) o.quat[j] = (float)q[j];
    for (int j = 0; j < 3; j++) o.scale[j] = (float)std::sqrt(std::max(vals[j], 1e-12));
    o.part_surface = nodes[n].part & 0xFFFFu;
    for (int j = 0; j < 3; j++) o.albedo[j] = (float)alb[3 * (size_t)n + j];
    o.flags = mat[n];
  }
  if (vg) {
    vg->assign(N - G, sl_vgrid{});
    for (size_t r = 0; r < (size_t)(N - G); r++) {
      uint8_t* o = reinterpret_cast<uint8_t*>(&(*vg)[r]);
      for (int q = 0; q < 128; q++) o[q] = (uint8_t)std::min(255.0, std::floor((double)V[r * 128u + q] + 0.5));
    }
  }
  return SL_OK;
}

}  // namespace sl

using namespace sl;

extern "C" {

int sl_lod_create(sl_renderer* r, const sl_node* nodes, uint32_t n_nodes, const uint32_t* kids, uint32_t n_kids,
                  sl_lod** out) {
  if (!out) return fail(SL_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  if (!r || !nodes || (!kids && n_kids)) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (r->lod) return fail(SL_ERR_INVALID_ARG, "this renderer already has a LOD");
  if (n_nodes < r->count || n_nodes > (1u << 26)) return fail(SL_ERR_INVALID_ARG, "node count below the Gaussian count");
  if (r->part_count > kMaxParts) return fail(SL_ERR_INVALID_ARG, "screen-space LOD needs at most 32 parts");
  const uint32_t G = r->count, N = n_nodes;
  for (uint32_t n = 0; n < N; n++) {
    if (n < G && nodes[n].child_hi != nodes[n].child_lo)
      return fail(SL_ERR_INVALID_ARG, "leaf " + std::to_string(n) + " has children");
    if (nodes[n].depth > 4096u) return fail(SL_ERR_INVALID_ARG, "tree deeper than 4096");
  }
  cudaSetDevice(r->device);
  std::vector<sl_gaussian> gauss(G);
  cudaError_t e = cudaMemcpy(gauss.data(), r->gaussians.ptr, sizeof(sl_gaussian) * G, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "reading the scene's Gaussians");
  std::vector<sl_gaussian> recs;
  int rc = node_records(gauss.data(), G, nodes, N, kids, n_kids, recs);
  if (rc) return rc;
  // nodes by depth: each depth's internal nodes, then its leaves (src/lod.js:114-125)
  uint32_t max_depth = 0;
  for (uint32_t n = 0; n < N; n++) max_depth = std::max(max_depth, nodes[n].depth);
  std::vector<std::vector<uint32_t>> inner(max_depth + 1), leaves(max_depth + 1);
  for (uint32_t n = 0; n < N; n++) (n < G ? leaves : inner)[nodes[n].depth].push_back(n);
  sl_lod* l = new sl_lod();
  l->r = r;
  l->device = r->device;
  l->N = N;
  l->G = G;
  l->n_int = N - G;
  std::vector<uint32_t> level;
  level.reserve(N);
  for (uint32_t d = 0; d <= max_depth; d++) {
    l->lvl_off.push_back((uint32_t)level.size());
    l->lvl_int.push_back((uint32_t)inner[d].size());
    l->lvl_all.push_back((uint32_t)(inner[d].size() + leaves[d].size()));
    level.insert(level.end(), inner[d].begin(), inner[d].end());
    level.insert(level.end(), leaves[d].begin(), leaves[d].end());
  }
  while (l->top < l->lvl_all.size() && l->lvl_all[l->top] <= kLodTopNodes) l->top++;
  std::vector<uint32_t> tables(l->lvl_off);
  tables.insert(tables.end(), l->lvl_all.begin(), l->lvl_all.end());
  tables.insert(tables.end(), l->lvl_int.begin(), l->lvl_int.end());
  auto up = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t e1 = b.ensure(std::max<size_t>(bytes, 16));
    if (e1 == cudaSuccess && bytes) e1 = cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice);
    return e1;
  };
  if ((e = up(l->nodes, nodes, sizeof(sl_node) * N)) != cudaSuccess ||
      (e = up(l->kids, kids, 4ull * n_kids)) != cudaSuccess ||
      (e = up(l->records, recs.data(), sizeof(sl_gaussian) * recs.size())) != cudaSuccess ||
      (e = up(l->level, level.data(), 4ull * level.size())) != cudaSuccess ||
      (e = up(l->tables, tables.data(), 4ull * tables.size())) != cudaSuccess ||
      (e = l->flags.ensure(4ull * N + 16)) != cudaSuccess || (e = l->colour.ensure(16ull * l->n_int + 16)) != cudaSuccess ||
      (e = cudaMemset(l->flags.ptr, 0, 4ull * N)) != cudaSuccess ||
      (e = cudaMemset(l->colour.ptr, 0, 16ull * l->n_int)) != cudaSuccess) {
    sl_lod_destroy(l);
    return e == cudaErrorMemoryAllocation ? fail(SL_ERR_OOM, "LOD buffers") : cuda_fail(e, "LOD buffers");
  }
  r->lod = l;
  *out = l;
  return SL_OK;
}

int sl_lod_destroy(sl_lod* l) {
  if (!l) return SL_OK;
  cudaSetDevice(l->device);
  cudaDeviceSynchronize();
  if (l->r && l->r->lod == l) l->r->lod = nullptr;
  DevBuf* all[] = {&l->nodes, &l->kids, &l->flags, &l->records, &l->colour, &l->level, &l->tables};
  for (DevBuf* b : all) b->release();
  delete l;
  return SL_OK;
}

int sl_lod_select(sl_lod* l, const sl_render_frame* f, uint32_t emit_part, uint32_t size_rule, float blur_lod,
                  void* stream) {
  if (!l || !f) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (!l->r) return fail(SL_ERR_INVALID_ARG, "the LOD's renderer was destroyed");
  if (!(f->near_plane > 0.0f) || !(f->focal[1] > 0.0f)) return fail(SL_ERR_INVALID_ARG, "bad frame");
  sl_renderer* r = l->r;
  cudaSetDevice(l->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  LodSelectParams P;
  memset(&P, 0, sizeof(P));
  memcpy(P.view, f->view, sizeof(P.view));
  P.focal = f->focal[1];  // lod.js is given the frame's focal in px (src/main.js:545-547: H / (2 tan(fovy / 2)))
  P.near_plane = f->near_plane;
  float thr;
  memcpy(&thr, &f->lod[0], 4);
  P.threshold = thr;
  P.shutter = f->palette[3][2];
  P.blur_lod = blur_lod;
  P.G = l->G;
  P.emit_part = emit_part;
  P.size_rule = size_rule;
  P.part_count = (uint32_t)r->parts.size();
  for (uint32_t p = 0; p < P.part_count && p < kMaxParts; p++) {
    memcpy(P.parts[p].xf, r->parts[p].xf, sizeof(P.parts[p].xf));
    memcpy(P.parts[p].xf_prev, r->parts[p].xf_prev, sizeof(P.parts[p].xf_prev));
    P.parts[p].root = r->parts[p].root;
    P.parts[p].flags = r->parts[p].flags;
  }
  const uint32_t D = (uint32_t)l->lvl_off.size();
  const uint32_t* tab = l->tables.as<uint32_t>();
  cudaError_t e = launch_lod_select_top(P, l->nodes.as<sl_node>(), l->kids.as<uint32_t>(), l->level.as<uint32_t>(), tab,
                                        tab + D, l->top, l->flags.as<uint32_t>(), s);
  if (e != cudaSuccess) return cuda_fail(e, "lod_select");
  for (uint32_t d = l->top; d < D; d++) {
    e = launch_lod_select(P, l->nodes.as<sl_node>(), l->kids.as<uint32_t>(), l->level.as<uint32_t>(), l->lvl_off[d],
                          l->lvl_all[d], l->flags.as<uint32_t>(), s);
    if (e != cudaSuccess) return cuda_fail(e, "lod_select");
  }
  return SL_OK;
}

int sl_lod_colour(sl_lod* l, const sl_render_frame* f, uint32_t colour_all, void* stream) {
  if (!l || !f) return fail(SL_ERR_INVALID_ARG, "null argument");
  if (!l->r) return fail(SL_ERR_INVALID_ARG, "the LOD's renderer was destroyed");
  cudaSetDevice(l->device);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float gain = f->palette[3][0];
  const uint32_t D = (uint32_t)l->lvl_off.size();
  for (uint32_t d = D; d-- > l->top;) {
    if (l->lvl_int[d] == 0) continue;
    cudaError_t e = launch_lod_colour(l->G, gain, colour_all, l->nodes.as<sl_node>(), l->kids.as<uint32_t>(),
                                      l->level.as<uint32_t>(), l->lvl_off[d], l->lvl_int[d], l->flags.as<uint32_t>(),
                                      l->r->colour, l->r->lo_b, l->colour.as<float4>(), s);
    if (e != cudaSuccess) return cuda_fail(e, "lod_colour");
  }
  const uint32_t* tab = l->tables.as<uint32_t>();
  cudaError_t e = launch_lod_colour_top(l->G, gain, colour_all, l->nodes.as<sl_node>(), l->kids.as<uint32_t>(),
                                        l->level.as<uint32_t>(), tab, tab + 2 * D, l->top, l->flags.as<uint32_t>(),
                                        l->r->colour, l->r->lo_b, l->colour.as<float4>(), s);
  if (e != cudaSuccess) return cuda_fail(e, "lod_colour");
  return SL_OK;
}

int sl_lod_read(sl_lod* l, uint32_t* flags, float* node_colour, sl_gaussian* records) {
  if (!l) return fail(SL_ERR_INVALID_ARG, "null LOD");
  cudaSetDevice(l->device);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess && flags) e = cudaMemcpy(flags, l->flags.ptr, 4ull * l->N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && node_colour)
    e = cudaMemcpy(node_colour, l->colour.ptr, 16ull * l->n_int, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && records)
    e = cudaMemcpy(records, l->records.ptr, sizeof(sl_gaussian) * l->n_int, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "LOD read-back");
  return SL_OK;
}

}  // extern "C"
