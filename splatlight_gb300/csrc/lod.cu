// Screen-space LOD (runtime/wgsl/lod.wgsl): the cut over the scene's tree and the lit colours of its nodes.
//   lod_select  top-down, one launch per tree depth over that depth's nodes: a part root or a node flagged a candidate
//               opens when its on-screen size (include/sl_lodsize.h) exceeds the threshold (its children become
//               candidates) and is drawn otherwise (its subtree is flagged "under"); a candidate leaf is drawn; every
//               other node passes "under" or "none" on to its children, so no flag from an earlier frame survives.
//   lod_colour  bottom-up, one launch per depth (deepest first) over its internal nodes that are drawn or under a
//               drawn node: the mass-weighted mean (mass = kappa / sqrt(det cinv)) of the children's shown colours.
// Each node writes only its own flag and its children's, and a depth's nodes share no children, so one launch per
// depth needs no atomics; the small top depths (a tree's first dozen) run in one CTA with a barrier between depths,
// so a frame costs a launch per large depth only.  Compiled with --fmad=false: the open/draw decisions and the colour sums match the CPU
// restatement bit for bit.
#include "sl_internal.h"
#include "sl_lodsize.h"

namespace sl {
namespace {

constexpr int kThreads = 256;
constexpr int kBlock = 1024;  // the single CTA of the small top depths
constexpr uint32_t kNone = 0u, kOpen = 1u, kDraw = 2u, kCand = 3u, kUnder = 4u;

__device__ __forceinline__ void select_node(const LodSelectParams& P, const sl_node* __restrict__ nodes,
                                            const uint32_t* __restrict__ kids, uint32_t n,
                                            uint32_t* __restrict__ flags) {
  const sl_node& nd = nodes[n];
  const uint32_t f = flags[n];
  const uint32_t part = nd.part;
  const bool root = part < kMaxParts && part < P.part_count && P.parts[part].root == n;
  if (!root && f != kCand) {
    const bool under = f == kUnder;
    if (!under) flags[n] = kNone;
    if (n >= P.G)
      for (uint32_t k = nd.child_lo; k < nd.child_hi; k++) flags[kids[k]] = under ? kUnder : kNone;
    return;
  }
  if (n < P.G) {
    flags[n] = kDraw;
    return;
  }
  bool open = part == P.emit_part;
  if (!open) {
    const LodPart& pt = P.parts[part < kMaxParts ? part : kMaxParts - 1u];
    float w[3], z;
    const float size = sl_lod_size(nd.mean, nd.radius, nd.cinv_diag, nd.cinv_off, pt.xf, P.view, P.focal, P.near_plane,
                                   P.size_rule & 1u, w, &z);
    float thr = P.threshold;
    if (P.blur_lod > 0.0f && P.shutter > 0.0f && (pt.flags & 2u) != 0u) {
      // motion blur variant D: a moving part opens only nodes larger than blur_lod x its smear this exposure
      float wp[3];
      for (int r = 0; r < 3; r++)
        wp[r] = pt.xf_prev[4 * r + 0] * nd.mean[0] + pt.xf_prev[4 * r + 1] * nd.mean[1] +
                pt.xf_prev[4 * r + 2] * nd.mean[2] + pt.xf_prev[4 * r + 3] * 1.0f;
      const float dx = w[0] - wp[0], dy = w[1] - wp[1], dz = w[2] - wp[2];
      const float zr = z - nd.radius;
      const float smear = P.focal * P.shutter * sqrtf(dx * dx + dy * dy + dz * dz) / (zr > P.near_plane ? zr : P.near_plane);
      const float b = P.blur_lod * smear;
      thr = thr > b ? thr : b;
    }
    open = size > thr;
  }
  flags[n] = open ? kOpen : kDraw;
  for (uint32_t k = nd.child_lo; k < nd.child_hi; k++) flags[kids[k]] = open ? kCand : kUnder;
}

__global__ void __launch_bounds__(kThreads) lod_select_kernel(const __grid_constant__ LodSelectParams P,
                                                              const sl_node* __restrict__ nodes,
                                                              const uint32_t* __restrict__ kids,
                                                              const uint32_t* __restrict__ level, uint32_t off,
                                                              uint32_t n_all, uint32_t* __restrict__ flags) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g < n_all) select_node(P, nodes, kids, level[off + g], flags);
}

// The small top depths in one CTA, a barrier between depths (their flags are written and read by this CTA alone).
__global__ void __launch_bounds__(kBlock) lod_select_top_kernel(const __grid_constant__ LodSelectParams P,
                                                                const sl_node* __restrict__ nodes,
                                                                const uint32_t* __restrict__ kids,
                                                                const uint32_t* __restrict__ level,
                                                                const uint32_t* __restrict__ lvl_off,
                                                                const uint32_t* __restrict__ lvl_all, uint32_t depths,
                                                                uint32_t* __restrict__ flags) {
  for (uint32_t d = 0; d < depths; d++) {
    const uint32_t off = lvl_off[d], n_all = lvl_all[d];
    for (uint32_t g = threadIdx.x; g < n_all; g += kBlock) select_node(P, nodes, kids, level[off + g], flags);
    __syncthreads();
  }
}

__device__ __forceinline__ float node_mass(const sl_node& nd) {
  const float* a = nd.cinv_diag;
  const float* o = nd.cinv_off;
  const float det_inv = a[0] * (a[1] * a[2] - o[2] * o[2]) - o[0] * (o[0] * a[2] - o[2] * o[1]) +
                        o[1] * (o[0] * o[2] - a[1] * o[1]);
  return nd.kappa / sqrtf(det_inv > 1e-30f ? det_inv : 1e-30f);
}

__device__ __forceinline__ void colour_node(uint32_t G, float gain, uint32_t colour_all,
                                            const sl_node* __restrict__ nodes, const uint32_t* __restrict__ kids,
                                            uint32_t n, const uint32_t* __restrict__ flags,
                                            const float4* __restrict__ colour, const float4* __restrict__ lo_b,
                                            float4* __restrict__ ncolour) {
  const uint32_t f = flags[n];
  if (f != kDraw && f != kUnder && !colour_all) return;
  const sl_node& nd = nodes[n];
  float cr = 0.0f, cg = 0.0f, cb = 0.0f, w = 0.0f;
  for (uint32_t k = nd.child_lo; k < nd.child_hi; k++) {
    const uint32_t ch = kids[k];
    const float m = node_mass(nodes[ch]);
    float sr, sg, sb;
    if (ch < G) {  // a leaf as the projection shows it: radiance + gain x the bounce toward the eye
      const float4 c = colour ? colour[ch] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      const float4 b = lo_b ? lo_b[3u * ch] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      sr = c.x + gain * b.x;
      sg = c.y + gain * b.y;
      sb = c.z + gain * b.z;
    } else {
      const float4 c = ncolour[ch - G];
      sr = c.x;
      sg = c.y;
      sb = c.z;
    }
    cr = cr + m * sr;
    cg = cg + m * sg;
    cb = cb + m * sb;
    w = w + m;
  }
  const float d = w > 1e-30f ? w : 1e-30f;
  ncolour[n - G] = make_float4(cr / d, cg / d, cb / d, 1.0f);
}

__global__ void __launch_bounds__(kThreads) lod_colour_kernel(uint32_t G, float gain, uint32_t colour_all,
                                                              const sl_node* __restrict__ nodes,
                                                              const uint32_t* __restrict__ kids,
                                                              const uint32_t* __restrict__ level, uint32_t off,
                                                              uint32_t n_int, const uint32_t* __restrict__ flags,
                                                              const float4* __restrict__ colour,
                                                              const float4* __restrict__ lo_b,
                                                              float4* __restrict__ ncolour) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g < n_int) colour_node(G, gain, colour_all, nodes, kids, level[off + g], flags, colour, lo_b, ncolour);
}

// The small top depths bottom-up in one CTA (after the larger depths below them).
__global__ void __launch_bounds__(kBlock) lod_colour_top_kernel(uint32_t G, float gain, uint32_t colour_all,
                                                                const sl_node* __restrict__ nodes,
                                                                const uint32_t* __restrict__ kids,
                                                                const uint32_t* __restrict__ level,
                                                                const uint32_t* __restrict__ lvl_off,
                                                                const uint32_t* __restrict__ lvl_int, uint32_t depths,
                                                                const uint32_t* __restrict__ flags,
                                                                const float4* __restrict__ colour,
                                                                const float4* __restrict__ lo_b,
                                                                float4* __restrict__ ncolour) {
  for (uint32_t d = depths; d-- > 0;) {
    const uint32_t off = lvl_off[d], n_int = lvl_int[d];
    for (uint32_t g = threadIdx.x; g < n_int; g += kBlock)
      colour_node(G, gain, colour_all, nodes, kids, level[off + g], flags, colour, lo_b, ncolour);
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_lod_select(const LodSelectParams& P, const sl_node* nodes, const uint32_t* kids,
                              const uint32_t* level, uint32_t off, uint32_t n_all, uint32_t* flags, cudaStream_t s) {
  if (n_all == 0) return cudaSuccess;
  lod_select_kernel<<<(n_all + kThreads - 1) / kThreads, kThreads, 0, s>>>(P, nodes, kids, level, off, n_all, flags);
  return cudaGetLastError();
}

cudaError_t launch_lod_select_top(const LodSelectParams& P, const sl_node* nodes, const uint32_t* kids,
                                  const uint32_t* level, const uint32_t* lvl_off, const uint32_t* lvl_all,
                                  uint32_t depths, uint32_t* flags, cudaStream_t s) {
  if (depths == 0) return cudaSuccess;
  lod_select_top_kernel<<<1, kBlock, 0, s>>>(P, nodes, kids, level, lvl_off, lvl_all, depths, flags);
  return cudaGetLastError();
}

cudaError_t launch_lod_colour_top(uint32_t G, float gain, uint32_t colour_all, const sl_node* nodes,
                                  const uint32_t* kids, const uint32_t* level, const uint32_t* lvl_off,
                                  const uint32_t* lvl_int, uint32_t depths, const uint32_t* flags,
                                  const float4* colour, const float4* lo_b, float4* ncolour, cudaStream_t s) {
  if (depths == 0) return cudaSuccess;
  lod_colour_top_kernel<<<1, kBlock, 0, s>>>(G, gain, colour_all, nodes, kids, level, lvl_off, lvl_int, depths, flags,
                                             colour, lo_b, ncolour);
  return cudaGetLastError();
}

cudaError_t launch_lod_colour(uint32_t G, float gain, uint32_t colour_all, const sl_node* nodes, const uint32_t* kids,
                              const uint32_t* level, uint32_t off, uint32_t n_int, const uint32_t* flags,
                              const float4* colour, const float4* lo_b, float4* ncolour, cudaStream_t s) {
  if (n_int == 0) return cudaSuccess;
  lod_colour_kernel<<<(n_int + kThreads - 1) / kThreads, kThreads, 0, s>>>(G, gain, colour_all, nodes, kids, level,
                                                                           off, n_int, flags, colour, lo_b, ncolour);
  return cudaGetLastError();
}

}  // namespace sl
