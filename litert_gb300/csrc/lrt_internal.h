// Internal declarations shared by the host library (C++) and the CUDA kernels.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/lrt_gpu.h"

namespace lrt {

constexpr uint32_t kLeafBit = 0x80000000u;     // LEAF_BIT, raytrace_common.h:43
constexpr uint32_t kEmptyChild = 0xFFFFFFFFu;  // unused slot of a wide node
constexpr uint32_t kMiss = 0xFFFFFFFFu;        // primId of a miss, Renderer/eye_ray.cpp:174
constexpr int kStackSize = 64;                 // traversal stack entries per ray

// 4-wide BVH node, one 128-byte line.  Child boxes are stored axis-major so a
// lane reads each slab bound of all four children with one 16-byte load.
// child[i]: internal -> wide node index; leaf -> kLeafBit | payload (box id for
// SBS/SVS, (count << 24) | start for triangle ranges); empty -> kEmptyChild.
struct alignas(128) WNode4 {
  float lo_x[4], hi_x[4], lo_y[4], hi_y[4], lo_z[4], hi_z[4];
  uint32_t child[4];
  uint32_t pad[4];
};
static_assert(sizeof(WNode4) == 128, "WNode4 must be one 128-byte line");

struct SbsData {
  lrt_sbs_header hdr;
  std::vector<lrt_sbs_node> nodes;
  std::vector<uint32_t> values;
};

struct BvhData {
  std::vector<WNode4> wnodes;            // root at 0
  std::vector<uint32_t> order;           // primitive order of the leaves
  std::vector<lrt_bvh_pair> pairs;       // reference fat-pair layout
  std::vector<uint32_t> leaf_start_count;  // triangles: per fat-pair leaf
  uint32_t max_depth = 0;                // wide-node depth
  std::vector<uint32_t> level_start;     // first wide node of each depth (nodes are breadth first)
};

float sdf_eval(const lrt_sdf_desc &f, float x, float y, float z);
lrt_status build_sbs(const lrt_sdf_desc &f, uint32_t depth, const lrt_sbs_header &hdr, int threads, SbsData &out);
lrt_status build_svs(const lrt_sdf_desc &f, uint32_t depth, int threads, std::vector<lrt_svs_node> &out);
// the same on the current device (build_gpu.cu); depth >= 4, arguments validated by the caller
lrt_status build_sbs_gpu(const lrt_sdf_desc &f, uint32_t depth, const lrt_sbs_header &hdr, SbsData &out,
                         std::string &err);
lrt_status build_svs_gpu(const lrt_sdf_desc &f, uint32_t depth, std::vector<lrt_svs_node> &out, std::string &err);
// Voxel occupancy of every brick: bit (i*bs + j)*bs + k of brick b is set when
// the smallest of the voxel's 8 decoded corner values is <= 0 -- exactly the
// voxel test of OctreeBrickIntersect (BVH/BVH2Common.cpp:821).
void build_occupancy(const SbsData &sbs, const std::vector<float> &values_f, uint32_t occ_words,
                     std::vector<uint32_t> &occ);
// boxes6: n x (min xyz, max xyz).  boxes=true: one box per leaf, payload = box
// id; boxes=false: triangles, up to two per leaf, payload = range in `order`.
lrt_status build_bvh(const float *boxes6, uint32_t n, bool boxes, BvhData &out);

// The same wide BVH layout built on the device (bvh_gpu.cu).  sah: build_bvh's
// binned SAH restated level by level (the same tree, nodes, order and fat pairs;
// cudaErrorNotSupported when an object-median split too large for the device
// path occurs, and the caller builds on the host); otherwise a linear BVH over
// Morton codes with one primitive per leaf.  Both collapse like build_bvh.  All
// pointers are device memory: d_boxes6 n x 6 floats; d_wnodes room for
// max(1, n-1) nodes; optional outputs d_order (n: primitive of each leaf-order
// position), d_pairs (max(1, n-1): the reference fat-pair layout) and, for
// triangles, d_leaf_start_count (n).  Synchronises the stream.
struct GpuBvhInfo {
  uint32_t n_wnodes = 0, max_depth = 0;
  uint32_t n_pairs = 0, n_leaves = 0;  // fat pairs written, leaves (leaf_start_count entries)
  std::vector<uint32_t> level_start;   // first wide node of each depth
};
cudaError_t build_bvh_gpu(const float *d_boxes6, uint32_t n, bool boxes, bool sah, WNode4 *d_wnodes,
                          uint32_t *d_order, lrt_bvh_pair *d_pairs, uint32_t *d_leaf_start_count, GpuBvhInfo &info,
                          cudaStream_t st);
// New slot boxes for an existing wide tree (host- or device-built) from new
// primitive boxes; triangle leaf ranges index d_order (null: identity).
cudaError_t refit_bvh_gpu(const float *d_boxes6, bool boxes, const uint32_t *d_order, WNode4 *d_wnodes,
                          const std::vector<uint32_t> &level_start, uint32_t n_wnodes, cudaStream_t st);
// boxes of the gathered triangles; gather of the triangles' vertices in BVH order
cudaError_t triangle_boxes_gpu(const float4 *d_tri_verts, uint32_t n, float *d_boxes6, cudaStream_t st);
cudaError_t gather_triangles_gpu(const float4 *d_vpos, const uint32_t *d_indices, const uint32_t *d_order, uint32_t n,
                                 float4 *d_tri_verts, cudaStream_t st);
// exclusive scan of n words on the device; *total (host, optional) receives the sum
cudaError_t gpu_exclusive_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint64_t *total, cudaStream_t st);

// ------------------------------------------------------------------ device side
// One instance of the committed geometry: its box in world space and the
// inverse matrix (and its transpose) of AddInstance (BVH/BVH2Common_host.cpp:1450-1487).
struct DevInst {
  float bmin[3], bmax[3];
  float inv[16], inv_t[16];
  float _pad[2];
};

// Scene as the kernels see it (all pointers device memory).
struct DevScene {
  uint32_t type;                 // LRT_TYPE_*
  uint32_t geom_id;              // geometry id reported in hits
  const WNode4 *nodes;
  // SBS
  lrt_sbs_header sbs_hdr;
  const lrt_sbs_node *bricks;
  const float4 *leaf_boxes;      // per brick: (min xyz, -), (max xyz, -) exactly as the BVH leaf box
  const uint32_t *occ;           // per brick: one bit per voxel, set when a corner value is <= 0
  uint32_t occ_words;            // 32-bit words of occupancy per brick
  const uint32_t *values;
  const float *values_f;
  // SVS
  const lrt_svs_node *svs;
  // triangles: vertex positions gathered per reordered triangle (A,B,C as float4)
  const float4 *tri_verts;
  const uint32_t *prim_indices;  // reordered -> original triangle id
  // instance 0 (the only one, or the one the shading functions read)
  float inst_bmin[3], inst_bmax[3];
  float inst_inv[16], inst_inv_t[16];
  // all instances of the geometry, when there are several (kernels instantiated
  // with FEAT bit 3 walk them; null otherwise)
  const DevInst *insts;
  uint32_t n_inst;
  lrt_preset preset;
  uint32_t seed;                 // MultiRenderer::m_seed (setSeed), for RAY_GEN_MODE_RANDOM
  // the BVH2 in the reference's fat-pair layout (4 float4 per pair), for the
  // first-hit walk of the "first_hit" tuning (null until that walk is used)
  const float4 *pairs;
  uint32_t n_pairs;
};

// A view prepared for the kernel: inverse matrices and its place in the
// flattened pixel and tile spaces.
struct DevView {
  uint32_t width, height;
  uint32_t pix_offset;   // first pixel in the batched outputs
  uint32_t tile_offset;  // first tile in the global tile space
  uint32_t tiles_x;      // tiles per row
  uint32_t tile_w_log2;  // a warp's tile is (1 << tile_w_log2) x (32 >> tile_w_log2) pixels
  // outputs published in chunks (RenderLaunch::chunk_done): the view's tile rows
  // r * rows_per_chunk .. (r + 1) * rows_per_chunk - 1 form chunk chunk_offset + r
  uint32_t chunk_offset;
  uint32_t rows_per_chunk;
  float proj_inv[16];
  float wv_inv[16];
};

struct RenderLaunch {
  const DevView *views;  // device
  uint32_t n_views;
  uint32_t total_tiles;
  lrt_hit16 *hits16;
  float4 *rgba;
  uint32_t *rgba8;
  uint32_t *tile_counter;       // scratch: persistent work queue head (zeroed before launch)
  unsigned long long *counters; // optional traversal counters [4]
  // optional, zeroed before launch: per output chunk, the warp tiles whose outputs
  // are written and fenced (render_kernel only; other kernels leave it untouched)
  uint32_t *chunk_done = nullptr;
  // optional: pixels from direct_from on are written through these pointers
  // instead (page-locked host outputs, mapped: the batch's tail, which would
  // otherwise be copied after the kernel)
  uint64_t direct_from = ~0ull;
  lrt_hit16 *hits16_direct = nullptr;
  float4 *rgba_direct = nullptr;
  uint32_t *rgba8_direct = nullptr;
};

// Launch-shape and kernel choices (set through lrt_set_tuning).
struct Tuning {
  int variant = 0;          // render kernel: 0 = one ray per lane (while-while), 1 = warp packet traversal,
                            // 2 = one ray per lane with per-lane ray refill
  int block_warps = 4;      // warps per block
  int stage = 0;            // packet kernel: 1 = stage each brick in shared memory, 0 = read corners from global
  int tile_w = 8;           // warp tile width in pixels (4, 8, 16 or 32; height 32 / tile_w)
  int stack = 64;           // per-ray traversal stack entries (32 or 64; 32 only for shallow trees)
  int refill = 8;           // variant 2: idle lanes of a warp that trigger fetching new rays
  int host_copy = 1;        // lrt_render_host into page-locked memory: 1 = render into device memory and copy
                            // each finished chunk while the rest renders, 0 = the kernel writes host memory
  int fma = 0;              // 1: variant 0 without counters runs the kernels compiled with FP contraction
  int first_hit = 0;        // 1: SBS / SVS renders and queries walk the BVH2 in the reference's order and
                            // stop at the first SDF leaf that hits (BVH2TraverseF32's result)
  int tc_wait = 1 << 20;    // tcgen05 network engine: mbarrier polls (up to ~1 us each) before a timeout
  int proposal_target = 0; // training target of collected triples: 0 crossing fraction, 1 first finder voxel
};

// Whether launch_render runs render_kernel for this launch (the kernel that
// publishes RenderLaunch::chunk_done); `color`: an rgba or rgba8 output.
bool render_publishes_chunks(const DevScene &s, bool color, uint32_t total_tiles, const Tuning &tu);
cudaError_t launch_render(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool count,
                          const Tuning &tu);
// NORMAL_MODE_SDF_SMOOTHED applies: the neighbour layout and a mode that needs normals
// (BVH/BVH2Common.cpp:838-840; trilinear interpolation is the only one supported)
inline bool smoothed_normals(const DevScene &s) {
  const uint32_t m = s.preset.render_mode;
  return s.type != LRT_TYPE_MESH_TRIANGLE && s.type != LRT_TYPE_SDF_SVS &&
         s.sbs_hdr.aux_data == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN && s.preset.normal_mode == 2 &&
         (m == 1 || m == 8 || m == 12 || m == 17 || m == 18);
}
// Kernel features an SBS scene needs: 1 smoothed normals; 2 brick colours computed in
// the leaf loop (ST_ITERATIONS stores the iteration count in primId, so the final
// hit no longer names its brick); 0 neither.
inline int render_features(const DevScene &s) {
  if (smoothed_normals(s)) return 1;
  const uint32_t layout = s.sbs_hdr.aux_data & 0xFF000000u;
  if (s.type != LRT_TYPE_MESH_TRIANGLE && s.type != LRT_TYPE_SDF_SVS && s.preset.render_mode == 10 &&
      layout != LRT_SBS_LAYOUT_DX && layout != LRT_SBS_LAYOUT_UNDEFINED)
    return 2;
  return 0;
}
// The variant-0 render kernel compiled with FP contraction (trace_fused.cu).
cudaError_t launch_render_fused(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                const Tuning &tu);
// Variant 3: the block-regrouped SBS kernel (render_lq.cuh), uncontracted (trace.cu)
// and contracted (trace_fused.cu).
cudaError_t launch_render_lq(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, const Tuning &tu);
cudaError_t launch_render_lq_fused(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                   const Tuning &tu);
// Warp-packet SBS render kernel (trace_pkt.cu).
cudaError_t launch_render_packet(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool count,
                                 const Tuning &tu);
// lrt_render_noalloc: same kernels, scratch in a file-scope device array (trace.cu).
cudaError_t launch_render_noalloc(const DevScene &s, const DevView *host_views, uint32_t n_views,
                                  uint32_t total_tiles, lrt_hit16 *hits16, float4 *rgba, uint32_t *rgba8,
                                  int device, int num_sms, cudaStream_t st, const Tuning &tu, bool first_hit);
cudaError_t launch_query(const DevScene &s, const float4 *pos_near, const float4 *dir_far, uint32_t n,
                         lrt_hit *out, cudaStream_t st);
// The same two launches with the reference's first-hit BVH2 walk (trace_ref.cu);
// SBS and SVS scenes whose s.pairs is set.
cudaError_t launch_render_ref(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st);
cudaError_t launch_query_ref(const DevScene &s, const float4 *pos_near, const float4 *dir_far, uint32_t n,
                             lrt_hit *out, cudaStream_t st);
inline bool sdf_scene(const DevScene &s) { return s.type != LRT_TYPE_MESH_TRIANGLE; }
// The same launches for a scene with several instances of its geometry (trace_inst.cu);
// first_hit: the reference's BVH2 walk per instance (SDF scenes whose s.pairs is set).
cudaError_t launch_render_inst(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool first_hit);
cudaError_t launch_query_inst(const DevScene &s, const float4 *pos_near, const float4 *dir_far, uint32_t n,
                              lrt_hit *out, cudaStream_t st, bool first_hit);

}  // namespace lrt

// host-side results of the SBS / SVS builders and loaders (opaque in the C ABI)
struct lrt_sbs { lrt::SbsData d; };
struct lrt_svs { std::vector<lrt_svs_node> nodes; };
