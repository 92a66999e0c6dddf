// C ABI of the GB300 ray-query engine: context, scene staging and commit
// (the BVHRT host side, BVH/BVH2Common_host.cpp), batched rendering and ray
// queries.  Host code only; kernels live in trace.cu.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx_internal.h"
#include "lrt_internal.h"

using namespace lrt;

// ---------------------------------------------------------------- matrices
static void mat_mul_vec4(const float m[16], const float v[4], float r[4]) {
  for (int i = 0; i < 4; i++) r[i] = m[i * 4 + 0] * v[0] + m[i * 4 + 1] * v[1] + m[i * 4 + 2] * v[2] + m[i * 4 + 3] * v[3];
}

extern "C" void lrt_inverse4x4(const float m[16], float out[16]) {
  double a[4][8];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 8; j++) a[i][j] = j < 4 ? double(m[i * 4 + j]) : (j - 4 == i ? 1.0 : 0.0);
  for (int c = 0; c < 4; c++) {
    int p = c;
    for (int r = c + 1; r < 4; r++)
      if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
    if (p != c)
      for (int j = 0; j < 8; j++) std::swap(a[c][j], a[p][j]);
    const double inv = 1.0 / a[c][c];
    for (int j = 0; j < 8; j++) a[c][j] *= inv;
    for (int r = 0; r < 4; r++)
      if (r != c) {
        const double f = a[r][c];
        for (int j = 0; j < 8; j++) a[r][j] -= f * a[c][j];
      }
  }
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) out[i * 4 + j] = float(a[i][j + 4]);
}

extern "C" void lrt_perspective(float fov_deg, float aspect, float znear, float zfar, float out[16]) {
  std::memset(out, 0, 16 * sizeof(float));
  const float ymax = znear * std::tan(fov_deg * 3.14159265358979323846f / 180.0f * 0.5f);
  const float xmax = ymax * aspect;
  const float l = -xmax, r = xmax, b = -ymax, t = ymax;
  out[0] = 2.0f * znear / (r - l);
  out[2] = (r + l) / (r - l);
  out[5] = 2.0f * znear / (t - b);
  out[6] = (t + b) / (t - b);
  out[10] = (-zfar - znear) / (zfar - znear);
  out[11] = (-2.0f * znear * zfar) / (zfar - znear);
  out[14] = -1.0f;
}

extern "C" void lrt_look_at(const float eye[3], const float center[3], const float up[3], float out[16]) {
  float z[3] = {eye[0] - center[0], eye[1] - center[1], eye[2] - center[2]};
  const float lz = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
  for (float &v : z) v /= lz;
  float x[3] = {up[1] * z[2] - up[2] * z[1], up[2] * z[0] - up[0] * z[2], up[0] * z[1] - up[1] * z[0]};
  const float lx = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  for (float &v : x) v /= lx;
  const float y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
  std::memset(out, 0, 16 * sizeof(float));
  for (int i = 0; i < 3; i++) {
    out[i] = x[i];
    out[4 + i] = y[i];
    out[8 + i] = z[i];
  }
  out[3] = -(x[0] * eye[0] + x[1] * eye[1] + x[2] * eye[2]);
  out[7] = -(y[0] * eye[0] + y[1] * eye[1] + y[2] * eye[2]);
  out[11] = -(z[0] * eye[0] + z[1] * eye[1] + z[2] * eye[2]);
  out[15] = 1.0f;
}

// ---------------------------------------------------------------- context
extern "C" const char *lrt_status_string(lrt_status s) {
  switch (s) {
    case LRT_OK: return "ok";
    case LRT_ERR_INVALID: return "invalid argument";
    case LRT_ERR_OOM: return "out of memory";
    case LRT_ERR_CUDA: return "CUDA error";
    case LRT_ERR_UNSUPPORTED: return "unsupported";
    case LRT_ERR_TIMEOUT: return "device wait timed out";
    case LRT_ERR_BOUNDS: return "device bounds check failed";
    case LRT_ERR_STATE: return "bad call order";
  }
  return "unknown";
}

extern "C" lrt_status lrt_create(lrt_ctx **out, int device) {
  if (!out) return LRT_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return LRT_ERR_CUDA;
  if (device < 0 || device >= n) return LRT_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return LRT_ERR_CUDA;
  lrt_ctx *ctx = new (std::nothrow) lrt_ctx();
  if (!ctx) return LRT_ERR_OOM;
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  ctx->preset.render_mode = LRT_RENDER_MODE_LAMBERT_NO_TEX;   // getDefaultPreset, render_settings.h:97-108
  ctx->preset.sdf_node_intersect = LRT_INTERSECT_ST;
  ctx->preset.normal_mode = 0;
  ctx->preset.ray_gen_mode = 0;
  ctx->preset.interpolation_mode = 0;
  ctx->preset.representation_mode = 1;
  ctx->preset.spp = 1;
  if (ctx->d_tile_counter.ensure(1) != cudaSuccess || ctx->d_counters.ensure(4) != cudaSuccess) {
    delete ctx;
    return LRT_ERR_OOM;
  }
  *out = ctx;
  return LRT_OK;
}

static void release_scene(lrt_ctx *ctx) {
  ctx->d_nodes.release();
  ctx->d_bricks.release();
  ctx->d_leaf_boxes.release();
  ctx->d_occ.release();
  ctx->d_values.release();
  ctx->d_values_f.release();
  ctx->d_svs.release();
  ctx->d_tri_verts.release();
  ctx->d_prim_indices.release();
  ctx->d_boxes6.release();
  ctx->d_pairs.release();
  ctx->d_leaf_start_count.release();
  ctx->d_vpos.release();
  ctx->d_tri_indices.release();
  ctx->d_ref_pairs.release();
  ctx->d_insts.release();
  ctx->bvh_on_device = ctx->bvh_refit = ctx->tri_indices_on_device = false;
  ctx->ref_pairs_ready = false;
  ctx->dev.pairs = nullptr;
  ctx->dev.n_pairs = 0;
  ctx->committed = false;
}

extern "C" void lrt_destroy(lrt_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  lrt::dr_state_free(ctx->dr);
  ctx->dr = nullptr;
  lrt::proposal_state_free(ctx->prop);
  ctx->prop = nullptr;
  release_scene(ctx);
  ctx->d_tile_counter.release();
  ctx->d_views.release();
  ctx->d_counters.release();
  ctx->d_out_hits.release();
  ctx->d_out_rgba.release();
  ctx->d_out_rgba8.release();
  ctx->d_q_pos.release();
  ctx->d_q_dir.release();
  ctx->d_q_out.release();
  ctx->d_chunk_done.release();
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->chunks_zeroed) cudaEventDestroy(ctx->chunks_zeroed);
  if (ctx->render_done) cudaEventDestroy(ctx->render_done);
  if (ctx->h_views) cudaFreeHost(ctx->h_views);
  delete ctx;
}

extern "C" const char *lrt_last_error(const lrt_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }
extern "C" uint32_t lrt_last_launch_count(const lrt_ctx *ctx) { return ctx ? ctx->last_launches : 0; }

// ---------------------------------------------------------------- geometry
extern "C" lrt_status lrt_clear_geom(lrt_ctx *ctx) {
  if (!ctx) return LRT_ERR_INVALID;
  ctx->geoms.clear();
  ctx->insts.clear();
  return LRT_OK;
}

extern "C" lrt_status lrt_add_sbs(lrt_ctx *ctx, const lrt_sbs_header *hdr, const lrt_sbs_node *nodes, uint32_t n_nodes,
                                  const uint32_t *values, uint32_t n_values, const float *values_f, uint32_t n_values_f,
                                  uint32_t *geom_id) {
  if (!ctx) return LRT_ERR_INVALID;
  if (!hdr || !nodes || !values || n_nodes == 0 || n_values == 0)
    return fail(ctx, LRT_ERR_INVALID, "lrt_add_sbs: empty SBS");
  // BVH/BVH2Common_host.cpp:569-570
  if (n_nodes >= (1u << 28) || n_values >= (1u << 28)) return fail(ctx, LRT_ERR_INVALID, "lrt_add_sbs: SBS too large");
  if (hdr->brick_size < 1 || hdr->brick_size > 16 || hdr->brick_pad > 1 ||
      !(hdr->bytes_per_value == 1 || hdr->bytes_per_value == 2 || hdr->bytes_per_value == 4))
    return fail(ctx, LRT_ERR_INVALID, "lrt_add_sbs: bad header");
  const uint32_t layout = hdr->aux_data & 0xFF000000u;
  uint32_t type;
  const bool indexed = layout == LRT_SBS_LAYOUT_ID32F_IRGB32F || layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN;
  const bool extra8 = layout == LRT_SBS_LAYOUT_DX_UV16 || layout == LRT_SBS_LAYOUT_DX_RGB8;   // + 8 words per brick
  // AddGeom_SdfSBS, BVH/BVH2Common_host.cpp:572-592
  if (layout == LRT_SBS_LAYOUT_UNDEFINED || layout == LRT_SBS_LAYOUT_DX) type = LRT_TYPE_SDF_SBS;
  else if (layout == LRT_SBS_LAYOUT_DX_UV16) type = LRT_TYPE_SDF_SBS_TEX;
  else if (indexed || layout == LRT_SBS_LAYOUT_DX_RGB8) type = LRT_TYPE_SDF_SBS_COL;
  else return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_add_sbs: unknown node layout");
  if (indexed && (!values_f || n_values_f == 0))
    return fail(ctx, LRT_ERR_INVALID, "lrt_add_sbs: indexed layout needs values_f");
  // every brick's data must lie inside `values`
  const uint32_t v_size = hdr->brick_size + 2 * hdr->brick_pad + 1, v3 = v_size * v_size * v_size;
  const uint32_t words = indexed ? v3 + 8 + (layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN ? 27 : 0)
                                 : (v3 + 4 / hdr->bytes_per_value - 1) / (4 / hdr->bytes_per_value) + (extra8 ? 8 : 0);
  for (uint32_t i = 0; i < n_nodes; i++) {
    if (uint64_t(nodes[i].data_offset) + words > n_values)
      return fail(ctx, LRT_ERR_INVALID, "lrt_add_sbs: brick data_offset out of range");
    if ((nodes[i].pos_z_lod_size & 0xFFFF) == 0) return fail(ctx, LRT_ERR_INVALID, "lrt_add_sbs: zero LOD size");
  }
  if (indexed) {   // distance indices, then 8 colour indices (3 floats each) per brick
    for (uint32_t i = 0; i < n_nodes; i++) {
      const uint32_t *w = values + nodes[i].data_offset;
      for (uint32_t j = 0; j < v3; j++)
        if (w[j] >= n_values_f) return fail(ctx, LRT_ERR_INVALID, "lrt_add_sbs: distance index out of range");
      for (uint32_t j = v3; j < v3 + 8; j++)
        if (uint64_t(w[j]) + 3 > n_values_f) return fail(ctx, LRT_ERR_INVALID, "lrt_add_sbs: colour index out of range");
    }
  }
  Geom g;
  g.type = type;
  g.sbs.hdr = *hdr;
  g.sbs.nodes.assign(nodes, nodes + n_nodes);
  g.sbs.values.assign(values, values + n_values);
  if (indexed) g.values_f.assign(values_f, values_f + n_values_f);
  ctx->geoms.push_back(std::move(g));
  if (geom_id) *geom_id = uint32_t(ctx->geoms.size() - 1);
  ctx->committed = false;
  return LRT_OK;
}

extern "C" lrt_status lrt_add_svs(lrt_ctx *ctx, const lrt_svs_node *nodes, uint32_t n_nodes, uint32_t *geom_id) {
  if (!ctx) return LRT_ERR_INVALID;
  if (!nodes || n_nodes == 0) return fail(ctx, LRT_ERR_INVALID, "lrt_add_svs: empty SVS");
  if (n_nodes >= (1u << 28)) return fail(ctx, LRT_ERR_INVALID, "lrt_add_svs: SVS too large");
  for (uint32_t i = 0; i < n_nodes; i++)
    if ((nodes[i].pos_z_lod_size & 0xFFFF) == 0) return fail(ctx, LRT_ERR_INVALID, "lrt_add_svs: zero LOD size");
  Geom g;
  g.type = LRT_TYPE_SDF_SVS;
  g.svs.assign(nodes, nodes + n_nodes);
  ctx->geoms.push_back(std::move(g));
  if (geom_id) *geom_id = uint32_t(ctx->geoms.size() - 1);
  ctx->committed = false;
  return LRT_OK;
}

extern "C" lrt_status lrt_add_triangles(lrt_ctx *ctx, const float *vpos, size_t n_vert, size_t v_byte_stride,
                                        const uint32_t *indices, size_t n_indices, uint32_t *geom_id) {
  if (!ctx) return LRT_ERR_INVALID;
  if (!vpos || !indices || n_vert == 0 || n_indices < 3 || n_indices % 3 != 0 || v_byte_stride < 12 ||
      v_byte_stride % 4 != 0)
    return fail(ctx, LRT_ERR_INVALID, "lrt_add_triangles: bad mesh");
  if (n_indices / 3 >= (1u << 24)) return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_add_triangles: too many triangles");
  for (size_t i = 0; i < n_indices; i++)
    if (indices[i] >= n_vert) return fail(ctx, LRT_ERR_INVALID, "lrt_add_triangles: index out of range");
  Geom g;
  g.type = LRT_TYPE_MESH_TRIANGLE;
  const size_t st = v_byte_stride / 4;
  g.vpos.resize(4 * n_vert);
  for (int k = 0; k < 3; k++) { g.bmin[k] = 3.4e38f; g.bmax[k] = -3.4e38f; }
  for (size_t i = 0; i < n_vert; i++) {
    for (int k = 0; k < 3; k++) {
      const float v = vpos[i * st + k];
      g.vpos[4 * i + k] = v;
      g.bmin[k] = std::min(g.bmin[k], v);
      g.bmax[k] = std::max(g.bmax[k], v);
    }
    g.vpos[4 * i + 3] = 1.0f;
  }
  g.indices.assign(indices, indices + n_indices);
  ctx->geoms.push_back(std::move(g));
  if (geom_id) *geom_id = uint32_t(ctx->geoms.size() - 1);
  ctx->committed = false;
  return LRT_OK;
}

extern "C" lrt_status lrt_clear_scene(lrt_ctx *ctx) {
  if (!ctx) return LRT_ERR_INVALID;
  ctx->insts.clear();
  ctx->committed = false;
  return LRT_OK;
}

// transformed corners of the geometry box, BVH/BVH2Common_host.cpp:1460-1475
static void instance_bounds(const Geom &g, Inst &in) {
  for (int k = 0; k < 3; k++) { in.bmin[k] = 3.4e38f; in.bmax[k] = -3.4e38f; }
  for (int c = 0; c < 8; c++) {
    const float v[4] = {(c & 1) ? g.bmax[0] : g.bmin[0], (c & 2) ? g.bmax[1] : g.bmin[1], (c & 4) ? g.bmax[2] : g.bmin[2], 1.0f};
    float r[4];
    mat_mul_vec4(in.m, v, r);
    for (int k = 0; k < 3; k++) { in.bmin[k] = std::min(in.bmin[k], r[k]); in.bmax[k] = std::max(in.bmax[k], r[k]); }
  }
}

static void dev_inst(const Inst &in, DevInst &o) {
  std::memset(&o, 0, sizeof(o));
  for (int k = 0; k < 3; k++) { o.bmin[k] = in.bmin[k]; o.bmax[k] = in.bmax[k]; }
  std::memcpy(o.inv, in.inv, sizeof(o.inv));
  std::memcpy(o.inv_t, in.inv_t, sizeof(o.inv_t));
}

extern "C" lrt_status lrt_add_instance(lrt_ctx *ctx, uint32_t geom_id, const float matrix[16], uint32_t *inst_id) {
  if (!ctx) return LRT_ERR_INVALID;
  geom_id &= 0x7fffffffu;   // CRT_GEOM_MASK_AABB_BIT, BVH/BVH2Common_host.cpp:1452-1453
  if (geom_id >= ctx->geoms.size() || !matrix) return fail(ctx, LRT_ERR_INVALID, "lrt_add_instance: bad geometry id");
  const Geom &g = ctx->geoms[geom_id];
  Inst in;
  in.geom = geom_id;
  std::memcpy(in.m, matrix, sizeof(in.m));
  lrt_inverse4x4(matrix, in.inv);
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) in.inv_t[i * 4 + j] = in.inv[j * 4 + i];
  instance_bounds(g, in);
  ctx->insts.push_back(in);
  if (inst_id) *inst_id = uint32_t(ctx->insts.size() - 1);
  ctx->committed = false;
  return LRT_OK;
}

template <typename T>
static cudaError_t upload(DevBuf<T> &b, const T *src, size_t n) {
  if (inject_fault("upload")) return cudaErrorInvalidValue;
  cudaError_t e = b.ensure(n);
  if (e != cudaSuccess || n == 0) return e;
  return cudaMemcpy(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

// BVH of the committed geometry built on the device: wide nodes straight into
// d_nodes, the sorted triangle order into d_prim_indices, the fat pairs kept on
// the device until lrt_get_bvh2 asks for them.
static lrt_status device_bvh(lrt_ctx *ctx, const std::vector<float> &boxes, bool tri) {
  const Geom &g = ctx->geoms[ctx->insts[0].geom];
  const uint32_t n = uint32_t(boxes.size() / 6);
  if (n == 0) return fail(ctx, LRT_ERR_INVALID, "lrt_commit_scene: empty geometry");
  if (!tri && n >= (1u << 31)) return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_commit_scene: too many boxes");
  const uint32_t n_int = std::max<uint32_t>(1, n - 1);
  cudaError_t e;
  if ((e = upload(ctx->d_boxes6, boxes.data(), boxes.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload boxes");
  LRT_CUDA(ctx, ctx->d_nodes.ensure(n_int));
  LRT_CUDA(ctx, ctx->d_pairs.ensure(n_int));
  if (tri) {
    LRT_CUDA(ctx, ctx->d_prim_indices.ensure(n));
    LRT_CUDA(ctx, ctx->d_leaf_start_count.ensure(n));
    if ((e = upload(ctx->d_vpos, reinterpret_cast<const float4 *>(g.vpos.data()), g.vpos.size() / 4)) != cudaSuccess)
      return cuda_fail(ctx, e, "upload vertices");
    if ((e = upload(ctx->d_tri_indices, g.indices.data(), g.indices.size())) != cudaSuccess)
      return cuda_fail(ctx, e, "upload indices");
    ctx->tri_indices_on_device = true;
  }
  GpuBvhInfo info;
  e = build_bvh_gpu(ctx->d_boxes6.p, n, !tri, ctx->bvh_builder == 1, ctx->d_nodes.p,
                    tri ? ctx->d_prim_indices.p : nullptr, ctx->d_pairs.p, tri ? ctx->d_leaf_start_count.p : nullptr,
                    info, 0);
  if (e == cudaErrorNotSupported) {   // a split the device path does not take: the host builder, same tree
    (void)cudaGetLastError();
    return LRT_ERR_UNSUPPORTED;
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "lrt_commit_scene: device BVH build");
  ctx->bvh = BvhData{};
  ctx->bvh.max_depth = info.max_depth;
  ctx->bvh.level_start = info.level_start;
  ctx->n_wnodes = info.n_wnodes;
  ctx->n_pairs = info.n_pairs;
  ctx->n_leaf_start_count = tri ? info.n_leaves : 0;
  ctx->bvh_on_device = true;
  return LRT_OK;
}

extern "C" lrt_status lrt_commit_scene(lrt_ctx *ctx) {
  if (!ctx) return LRT_ERR_INVALID;
  if (ctx->insts.empty()) return fail(ctx, LRT_ERR_STATE, "lrt_commit_scene: no instance");
  for (const Inst &i : ctx->insts)
    if (i.geom != ctx->insts[0].geom)
      return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_commit_scene: the instances of a scene must share one geometry");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  release_scene(ctx);
  const Inst &in = ctx->insts[0];
  const Geom &g = ctx->geoms[in.geom];
  std::vector<float> boxes;
  DevScene s{};
  s.type = g.type;
  s.geom_id = in.geom;
  lrt_status st = LRT_OK;
  if (g.type == LRT_TYPE_MESH_TRIANGLE) {
    const size_t nt = g.indices.size() / 3;
    boxes.resize(6 * nt);
    for (size_t t = 0; t < nt; t++)
      for (int k = 0; k < 3; k++) {
        float lo = 3.4e38f, hi = -3.4e38f;
        for (int v = 0; v < 3; v++) {
          const float x = g.vpos[4 * size_t(g.indices[3 * t + v]) + k];
          lo = std::min(lo, x);
          hi = std::max(hi, x);
        }
        boxes[6 * t + k] = lo;
        boxes[6 * t + 3 + k] = hi;
      }
  } else {
    // one AABB per brick / voxel, BVH/BVH2Common_host.cpp:546-555, 640-653
    const bool sbs = g.type != LRT_TYPE_SDF_SVS;
    const size_t n = sbs ? g.sbs.nodes.size() : g.svs.size();
    boxes.resize(6 * n);
    for (size_t i = 0; i < n; i++) {
      const uint32_t pxy = sbs ? g.sbs.nodes[i].pos_xy : g.svs[i].pos_xy;
      const uint32_t pzl = sbs ? g.sbs.nodes[i].pos_z_lod_size : g.svs[i].pos_z_lod_size;
      const float px = float(pxy >> 16), py = float(pxy & 0x0000FFFF), pz = float(pzl >> 16), sz = float(pzl & 0x0000FFFF);
      const float lo[3] = {-1 + 2.0f * px / sz, -1 + 2.0f * py / sz, -1 + 2.0f * pz / sz};
      for (int k = 0; k < 3; k++) {
        boxes[6 * i + k] = lo[k];
        boxes[6 * i + 3 + k] = lo[k] + 2.0f * 1 / sz;
      }
    }
  }
  const bool tri = g.type == LRT_TYPE_MESH_TRIANGLE;
  const uint32_t n_prims = uint32_t(boxes.size() / 6);
  cudaError_t e;
  if (ctx->bvh_builder != 0) st = device_bvh(ctx, boxes, tri);
  if (ctx->bvh_builder != 0 && st != LRT_ERR_UNSUPPORTED) {
    if (st != LRT_OK) return st;
  } else {
    st = build_bvh(boxes.data(), n_prims, !tri, ctx->bvh);
    if (st != LRT_OK) return fail(ctx, st, "lrt_commit_scene: BVH build failed");
    ctx->n_wnodes = uint32_t(ctx->bvh.wnodes.size());
  }
  if (3 * int(ctx->bvh.max_depth) + 4 > kStackSize)
    return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_commit_scene: BVH deeper than the traversal stack");

  if (!ctx->bvh_on_device && (e = upload(ctx->d_nodes, ctx->bvh.wnodes.data(), ctx->bvh.wnodes.size())) != cudaSuccess)
    return cuda_fail(ctx, e, "upload nodes");
  s.nodes = ctx->d_nodes.p;
  if (tri && ctx->bvh_on_device) {
    const size_t nt = g.indices.size() / 3;
    LRT_CUDA(ctx, ctx->d_tri_verts.ensure(3 * nt));
    LRT_CUDA(ctx, gather_triangles_gpu(ctx->d_vpos.p, ctx->d_tri_indices.p, ctx->d_prim_indices.p, uint32_t(nt),
                                       ctx->d_tri_verts.p, 0));
    LRT_CUDA(ctx, cudaDeviceSynchronize());
    s.tri_verts = ctx->d_tri_verts.p;
    s.prim_indices = ctx->d_prim_indices.p;
  } else if (tri) {
    const size_t nt = g.indices.size() / 3;
    std::vector<float4> tv(3 * nt);
    for (size_t r = 0; r < nt; r++) {
      const uint32_t t = ctx->bvh.order[r];
      for (int v = 0; v < 3; v++) {
        const float *p = &g.vpos[4 * size_t(g.indices[3 * size_t(t) + v])];
        tv[3 * r + v] = make_float4(p[0], p[1], p[2], p[3]);
      }
    }
    if ((e = upload(ctx->d_tri_verts, tv.data(), tv.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload tris");
    if ((e = upload(ctx->d_prim_indices, ctx->bvh.order.data(), ctx->bvh.order.size())) != cudaSuccess)
      return cuda_fail(ctx, e, "upload prim indices");
    s.tri_verts = ctx->d_tri_verts.p;
    s.prim_indices = ctx->d_prim_indices.p;
  } else if (g.type == LRT_TYPE_SDF_SVS) {
    if ((e = upload(ctx->d_svs, g.svs.data(), g.svs.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload svs");
    s.svs = ctx->d_svs.p;
  } else {
    // Device layout: every brick's words start on a 16-byte boundary (stride
    // rounded up to 4 words) so a warp can stage a brick with 16-byte loads.
    const lrt_sbs_header &hd = g.sbs.hdr;
    const uint32_t layout = hd.aux_data & 0xFF000000u;
    const uint32_t v_size = hd.brick_size + 2 * hd.brick_pad + 1, v3 = v_size * v_size * v_size;
    const bool indexed = layout == LRT_SBS_LAYOUT_ID32F_IRGB32F || layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN;
    const uint32_t vpi = 4 / hd.bytes_per_value;
    const bool extra8 = layout == LRT_SBS_LAYOUT_DX_UV16 || layout == LRT_SBS_LAYOUT_DX_RGB8;
    const uint32_t words = indexed ? v3 + 8 + (layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN ? 27 : 0)
                                   : (v3 + vpi - 1) / vpi + (extra8 ? 8 : 0);
    const uint32_t stride = (words + 3u) & ~3u;
    const size_t nb = g.sbs.nodes.size();
    if (uint64_t(nb) * stride >= (1ull << 32))
      return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_commit_scene: brick data exceeds 2^32 words");
    std::vector<uint32_t> dv(nb * stride, 0u);
    std::vector<lrt_sbs_node> dn(g.sbs.nodes);
    for (size_t i = 0; i < nb; i++) {
      std::memcpy(&dv[i * stride], &g.sbs.values[g.sbs.nodes[i].data_offset], size_t(words) * 4);
      dn[i].data_offset = uint32_t(i * stride);
    }
    ctx->brick_stride = stride;
    std::vector<float4> lb(2 * nb);   // the BVH leaf boxes computed above
    for (size_t i = 0; i < nb; i++) {
      lb[2 * i] = make_float4(boxes[6 * i], boxes[6 * i + 1], boxes[6 * i + 2], 0.0f);
      lb[2 * i + 1] = make_float4(boxes[6 * i + 3], boxes[6 * i + 4], boxes[6 * i + 5], 0.0f);
    }
    if ((e = upload(ctx->d_leaf_boxes, lb.data(), lb.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload boxes");
    s.leaf_boxes = ctx->d_leaf_boxes.p;
    const uint32_t occ_words = (hd.brick_size * hd.brick_size * hd.brick_size + 31u) / 32u;
    std::vector<uint32_t> occ;
    build_occupancy(g.sbs, g.values_f, occ_words, occ);
    if ((e = upload(ctx->d_occ, occ.data(), occ.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload occupancy");
    s.occ = ctx->d_occ.p;
    s.occ_words = occ_words;
    if ((e = upload(ctx->d_bricks, dn.data(), dn.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload bricks");
    if ((e = upload(ctx->d_values, dv.data(), dv.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload values");
    if (!g.values_f.empty() && (e = upload(ctx->d_values_f, g.values_f.data(), g.values_f.size())) != cudaSuccess)
      return cuda_fail(ctx, e, "upload values_f");
    s.sbs_hdr = g.sbs.hdr;
    s.bricks = ctx->d_bricks.p;
    s.values = ctx->d_values.p;
    s.values_f = ctx->d_values_f.p;
  }
  for (int k = 0; k < 3; k++) { s.inst_bmin[k] = in.bmin[k]; s.inst_bmax[k] = in.bmax[k]; }
  std::memcpy(s.inst_inv, in.inv, sizeof(s.inst_inv));
  std::memcpy(s.inst_inv_t, in.inv_t, sizeof(s.inst_inv_t));
  s.n_inst = uint32_t(ctx->insts.size());
  s.insts = nullptr;
  if (s.n_inst > 1) {
    std::vector<DevInst> di(ctx->insts.size());
    for (size_t i = 0; i < di.size(); i++) dev_inst(ctx->insts[i], di[i]);
    if ((e = upload(ctx->d_insts, di.data(), di.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload instances");
    s.insts = ctx->d_insts.p;
  }
  s.preset = ctx->preset;
  s.seed = ctx->seed;
  ctx->dev = s;
  ctx->committed = true;
  return LRT_OK;
}

extern "C" lrt_status lrt_set_preset(lrt_ctx *ctx, const lrt_preset *preset) {
  if (!ctx || !preset) return LRT_ERR_INVALID;
  if (preset->sdf_node_intersect > LRT_INTERSECT_IT) return fail(ctx, LRT_ERR_INVALID, "lrt_set_preset: bad intersect mode");
  if (preset->interpolation_mode != 0)
    return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_set_preset: only trilinear interpolation is supported");
  if (preset->ray_gen_mode > 1) return fail(ctx, LRT_ERR_INVALID, "lrt_set_preset: ray_gen_mode is 0 or 1");
  if (preset->spp == 0 || preset->spp > 1024) return fail(ctx, LRT_ERR_INVALID, "lrt_set_preset: bad spp");
  switch (preset->render_mode) {   // kernel_RayTrace's modes for the geometry types of this path
    case LRT_RENDER_MODE_MASK: case LRT_RENDER_MODE_LAMBERT_NO_TEX: case LRT_RENDER_MODE_DEPTH:
    case LRT_RENDER_MODE_LINEAR_DEPTH: case LRT_RENDER_MODE_INVERSE_LINEAR_DEPTH: case LRT_RENDER_MODE_PRIMITIVE:
    case LRT_RENDER_MODE_TYPE: case LRT_RENDER_MODE_GEOM: case LRT_RENDER_MODE_NORMAL:
    case LRT_RENDER_MODE_BARYCENTRIC: case LRT_RENDER_MODE_ST_ITERATIONS: case LRT_RENDER_MODE_PHONG_NO_TEX:
    case LRT_RENDER_MODE_DIFFUSE: case LRT_RENDER_MODE_LAMBERT: case LRT_RENDER_MODE_PHONG:
    case LRT_RENDER_MODE_HSV_DEPTH:
      break;
    default:   // radiance-field, Gaussian-splat and texture-coordinate modes
      return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_set_preset: render mode not supported");
  }
  ctx->preset = *preset;
  ctx->dev.preset = *preset;
  return LRT_OK;
}

extern "C" lrt_status lrt_set_tuning(lrt_ctx *ctx, const char *key, int value) {
  if (!ctx || !key) return LRT_ERR_INVALID;
  const std::string k(key);
  if (k == "variant") {
    if (value < 0 || value > 3) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: variant is 0, 1, 2 or 3");
    ctx->tuning.variant = value;
  } else if (k == "block_warps") {
    if (value < 1 || value > 8) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: block_warps in 1..8");
    ctx->tuning.block_warps = value;
  } else if (k == "stage") {
    if (value < 0 || value > 1) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: stage is 0 or 1");
    ctx->tuning.stage = value;
  } else if (k == "tile_w") {
    if (value != 4 && value != 8 && value != 16 && value != 32)
      return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: tile_w is 4, 8, 16 or 32");
    ctx->tuning.tile_w = value;
  } else if (k == "stack") {
    if (value != 32 && value != 64) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: stack is 32 or 64");
    ctx->tuning.stack = value;
  } else if (k == "refill") {
    if (value < 1 || value > 32) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: refill in 1..32");
    ctx->tuning.refill = value;
  } else if (k == "fma") {
    if (value < 0 || value > 1) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: fma is 0 or 1");
    ctx->tuning.fma = value;
  } else if (k == "bvh_builder") {
    if (value < 0 || value > 2) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: bvh_builder is 0, 1 or 2");
    ctx->bvh_builder = value;
  } else if (k == "host_copy") {
    if (value < 0 || value > 1) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: host_copy is 0 or 1");
    ctx->tuning.host_copy = value;
  } else if (k == "proposal_target") {
    if (value < 0 || value > 1) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: proposal_target is 0 or 1");
    ctx->tuning.proposal_target = value;
  } else if (k == "first_hit") {
    if (value < 0 || value > 1) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: first_hit is 0 or 1");
    ctx->tuning.first_hit = value;
  } else if (k == "tc_wait") {
    if (value < 0) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: tc_wait is a poll count >= 0");
    ctx->tuning.tc_wait = value;
  } else if (k == "proposal") {
    if (value < 0 || value > 1) return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: proposal is 0 or 1");
    ctx->use_proposal = value;
  } else {
    return fail(ctx, LRT_ERR_INVALID, "lrt_set_tuning: unknown key " + k);
  }
  return LRT_OK;
}

extern "C" lrt_status lrt_refit_triangles(lrt_ctx *ctx, const float *vpos, size_t n_vert, size_t v_byte_stride) {
  if (!ctx) return LRT_ERR_INVALID;
  if (!ctx->committed) return fail(ctx, LRT_ERR_STATE, "lrt_refit_triangles: no committed scene");
  Inst &in = ctx->insts[0];
  Geom &g = ctx->geoms[in.geom];
  if (g.type != LRT_TYPE_MESH_TRIANGLE)
    return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_refit_triangles: the committed geometry is not a triangle mesh");
  if (!vpos || v_byte_stride < 12 || v_byte_stride % 4 != 0 || n_vert != g.vpos.size() / 4)
    return fail(ctx, LRT_ERR_INVALID, "lrt_refit_triangles: vertex count or stride differs from the mesh");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t sv = v_byte_stride / 4;
  for (int k = 0; k < 3; k++) { g.bmin[k] = 3.4e38f; g.bmax[k] = -3.4e38f; }
  for (size_t i = 0; i < n_vert; i++)
    for (int k = 0; k < 3; k++) {
      const float v = vpos[i * sv + k];
      g.vpos[4 * i + k] = v;
      g.bmin[k] = std::min(g.bmin[k], v);
      g.bmax[k] = std::max(g.bmax[k], v);
    }
  for (Inst &i : ctx->insts) instance_bounds(g, i);
  for (int k = 0; k < 3; k++) { ctx->dev.inst_bmin[k] = in.bmin[k]; ctx->dev.inst_bmax[k] = in.bmax[k]; }
  cudaError_t e;
  if (ctx->dev.n_inst > 1) {
    std::vector<DevInst> di(ctx->insts.size());
    for (size_t i = 0; i < di.size(); i++) dev_inst(ctx->insts[i], di[i]);
    if ((e = upload(ctx->d_insts, di.data(), di.size())) != cudaSuccess) return cuda_fail(ctx, e, "upload instances");
  }
  if ((e = upload(ctx->d_vpos, reinterpret_cast<const float4 *>(g.vpos.data()), n_vert)) != cudaSuccess)
    return cuda_fail(ctx, e, "lrt_refit_triangles: upload vertices");
  if (!ctx->tri_indices_on_device) {
    if ((e = upload(ctx->d_tri_indices, g.indices.data(), g.indices.size())) != cudaSuccess)
      return cuda_fail(ctx, e, "lrt_refit_triangles: upload indices");
    ctx->tri_indices_on_device = true;
  }
  const uint32_t nt = uint32_t(g.indices.size() / 3);
  LRT_CUDA(ctx, ctx->d_boxes6.ensure(6 * size_t(nt)));
  LRT_CUDA(ctx, gather_triangles_gpu(ctx->d_vpos.p, ctx->d_tri_indices.p, ctx->d_prim_indices.p, nt,
                                     ctx->d_tri_verts.p, 0));
  LRT_CUDA(ctx, triangle_boxes_gpu(ctx->d_tri_verts.p, nt, ctx->d_boxes6.p, 0));
  LRT_CUDA(ctx, refit_bvh_gpu(ctx->d_boxes6.p, false, nullptr, ctx->d_nodes.p, ctx->bvh.level_start, ctx->n_wnodes, 0));
  LRT_CUDA(ctx, cudaDeviceSynchronize());
  ctx->bvh_refit = true;
  ctx->last_launches = 2 + uint32_t(ctx->bvh.level_start.size());
  return LRT_OK;
}

extern "C" lrt_status lrt_get_bvh2(lrt_ctx *ctx, const lrt_bvh_pair **pairs, uint32_t *n_pairs) {
  if (!ctx || !pairs || !n_pairs) return LRT_ERR_INVALID;
  if (!ctx->committed) return fail(ctx, LRT_ERR_STATE, "lrt_get_bvh2: no committed scene");
  if (ctx->bvh_refit)
    return fail(ctx, LRT_ERR_STATE, "lrt_get_bvh2: the BVH was refit; the fat-pair layout is only made at commit");
  if (ctx->bvh_on_device && ctx->bvh.pairs.empty()) {   // device-built: fetch once
    LRT_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->bvh.pairs.resize(ctx->n_pairs);
    ctx->bvh.leaf_start_count.resize(ctx->n_leaf_start_count);
    LRT_CUDA(ctx, cudaMemcpy(ctx->bvh.pairs.data(), ctx->d_pairs.p, size_t(ctx->n_pairs) * sizeof(lrt_bvh_pair),
                             cudaMemcpyDeviceToHost));
    if (ctx->n_leaf_start_count)
      LRT_CUDA(ctx, cudaMemcpy(ctx->bvh.leaf_start_count.data(), ctx->d_leaf_start_count.p,
                               size_t(ctx->n_leaf_start_count) * 4, cudaMemcpyDeviceToHost));
  }
  *pairs = ctx->bvh.pairs.data();
  *n_pairs = uint32_t(ctx->bvh.pairs.size());
  return LRT_OK;
}

// A BVH2 the first-hit walk can follow: pair 0 is the root, every inner child
// names a pair that no other node names (a tree: the walk ends), every leaf names
// a primitive of the committed geometry (or is the empty marker 0xFFFFFFFF), and
// no path holds more inner pairs than the walk's 80-entry stack.
static bool check_bvh2(const lrt_bvh_pair *pairs, uint32_t n_pairs, uint32_t n_prims, std::string &why) {
  if (n_pairs == 0) { why = "no pairs"; return false; }
  std::vector<uint8_t> seen(n_pairs, 0);
  std::vector<std::pair<uint32_t, uint32_t>> todo{{0u, 1u}};   // (pair, inner pairs on the path)
  seen[0] = 1;
  while (!todo.empty()) {
    const auto [p, depth] = todo.back();
    todo.pop_back();
    if (depth > 80) { why = "a path needs more than 80 stack entries"; return false; }
    for (const lrt_bvh_node *c : {&pairs[p].left, &pairs[p].right}) {
      const uint32_t off = c->leftOffset;
      if (off & 0x80000000u) {
        if (off != 0xFFFFFFFFu && (off & 0x00FFFFFFu) >= n_prims) { why = "leaf names no primitive"; return false; }
      } else {
        if (off >= n_pairs || seen[off]) { why = "child index out of range or shared"; return false; }
        seen[off] = 1;
        todo.push_back({off, depth + 1});
      }
    }
  }
  return true;
}

static uint32_t committed_prims(const lrt_ctx *ctx) {
  const Geom &g = ctx->geoms[ctx->insts[0].geom];
  return g.type == LRT_TYPE_SDF_SVS ? uint32_t(g.svs.size()) : uint32_t(g.sbs.nodes.size());
}

static lrt_status upload_ref_pairs(lrt_ctx *ctx, const lrt_bvh_pair *pairs, uint32_t n_pairs) {
  std::string why;
  if (!check_bvh2(pairs, n_pairs, committed_prims(ctx), why)) return fail(ctx, LRT_ERR_INVALID, "BVH2: " + why);
  cudaError_t e = upload(ctx->d_ref_pairs, pairs, n_pairs);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "upload BVH2");
  ctx->dev.pairs = reinterpret_cast<const float4 *>(ctx->d_ref_pairs.p);
  ctx->dev.n_pairs = n_pairs;
  ctx->ref_pairs_ready = true;
  return LRT_OK;
}

// The first-hit walk's tree, on its first use after a commit: the committed BVH's
// own fat pairs (the tree the closest-hit kernels collapse into 4-wide nodes).
static lrt_status ensure_walk(lrt_ctx *ctx) {
  if (!ctx->tuning.first_hit || !sdf_scene(ctx->dev) || ctx->ref_pairs_ready) return LRT_OK;
  const lrt_bvh_pair *p = nullptr;
  uint32_t n = 0;
  lrt_status s = lrt_get_bvh2(ctx, &p, &n);
  if (s != LRT_OK) return s;
  return upload_ref_pairs(ctx, p, n);
}

extern "C" lrt_status lrt_set_bvh2(lrt_ctx *ctx, const lrt_bvh_pair *pairs, uint32_t n_pairs) {
  if (!ctx || !pairs) return LRT_ERR_INVALID;
  if (!ctx->committed) return fail(ctx, LRT_ERR_STATE, "lrt_set_bvh2: commit the scene first");
  if (!sdf_scene(ctx->dev))
    return fail(ctx, LRT_ERR_UNSUPPORTED, "lrt_set_bvh2: triangle meshes have no first-hit walk");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  return upload_ref_pairs(ctx, pairs, n_pairs);
}

extern "C" lrt_status lrt_set_seed(lrt_ctx *ctx, uint32_t seed) {
  if (!ctx) return LRT_ERR_INVALID;
  ctx->seed = seed;
  ctx->dev.seed = seed;
  return LRT_OK;
}

extern "C" lrt_status lrt_update_instance(lrt_ctx *ctx, uint32_t inst_id, const float matrix[16]) {
  if (!ctx || !matrix) return LRT_ERR_INVALID;
  if (inst_id >= ctx->insts.size()) return fail(ctx, LRT_ERR_INVALID, "lrt_update_instance: bad instance id");
  Inst &in = ctx->insts[inst_id];
  std::memcpy(in.m, matrix, sizeof(in.m));
  lrt_inverse4x4(matrix, in.inv);
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) in.inv_t[i * 4 + j] = in.inv[j * 4 + i];
  instance_bounds(ctx->geoms[in.geom], in);
  if (!ctx->committed) return LRT_OK;
  // the committed scene follows at once: no rebuild (the BLAS is in object space)
  if (inst_id == 0) {
    for (int k = 0; k < 3; k++) { ctx->dev.inst_bmin[k] = in.bmin[k]; ctx->dev.inst_bmax[k] = in.bmax[k]; }
    std::memcpy(ctx->dev.inst_inv, in.inv, sizeof(in.inv));
    std::memcpy(ctx->dev.inst_inv_t, in.inv_t, sizeof(in.inv_t));
  }
  if (ctx->dev.n_inst > 1) {
    DevInst di;
    dev_inst(in, di);
    LRT_CUDA(ctx, cudaSetDevice(ctx->device));
    LRT_CUDA(ctx, cudaMemcpy(ctx->d_insts.p + inst_id, &di, sizeof(di), cudaMemcpyHostToDevice));
  }
  return LRT_OK;
}

extern "C" lrt_status lrt_update_geom_triangles(lrt_ctx *ctx, uint32_t geom_id, const float *vpos, size_t n_vert,
                                                const uint32_t *indices, size_t n_indices, size_t v_byte_stride) {
  if (!ctx) return LRT_ERR_INVALID;
  if (geom_id >= ctx->geoms.size() || ctx->geoms[geom_id].type != LRT_TYPE_MESH_TRIANGLE)
    return fail(ctx, LRT_ERR_INVALID, "lrt_update_geom_triangles: not a triangle geometry");
  const Geom &g = ctx->geoms[geom_id];
  if (indices && (n_indices != g.indices.size() || !std::equal(g.indices.begin(), g.indices.end(), indices)))
    return fail(ctx, LRT_ERR_UNSUPPORTED,
                "lrt_update_geom_triangles: new connectivity needs lrt_add_triangles and a commit");
  if (!ctx->committed || ctx->insts[0].geom != geom_id)
    return fail(ctx, LRT_ERR_STATE, "lrt_update_geom_triangles: the geometry is not the committed one");
  return lrt_refit_triangles(ctx, vpos, n_vert, v_byte_stride);
}

extern "C" lrt_status lrt_add_aabb(lrt_ctx *ctx, uint32_t type_id, const float *boxes8, size_t n_boxes,
                                   uint32_t *geom_id) {
  (void)type_id; (void)boxes8; (void)n_boxes;
  if (geom_id) *geom_id = 0xFFFFFFFFu;
  return fail(ctx, LRT_ERR_UNSUPPORTED,
              "lrt_add_aabb: custom-box geometry has no intersector on this path (the reference's AddGeom_AABB "
              "registers boxes but no geometry object to intersect them)");
}

// ---------------------------------------------------------------- rendering
static lrt_status prepare_views(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, cudaStream_t st,
                                uint32_t *total_tiles, uint64_t *total_pix) {
  if (!views || n_views == 0) return fail(ctx, LRT_ERR_INVALID, "render: no views");
  if (ctx->h_views_cap < n_views) {
    if (ctx->h_views) cudaFreeHost(ctx->h_views);
    ctx->h_views = nullptr;
    ctx->h_views_cap = 0;
    LRT_CUDA(ctx, cudaMallocHost(&ctx->h_views, n_views * sizeof(DevView)));
    ctx->h_views_cap = n_views;
  }
  // The pinned staging buffer is reused; wait for the previous upload to finish.
  LRT_CUDA(ctx, cudaStreamSynchronize(st));
  uint64_t all_pix = 0;
  for (uint32_t v = 0; v < n_views; v++) all_pix += uint64_t(views[v].width) * views[v].height;
  // output chunks for lrt_render_host's overlapped copies: whole tile rows of one
  // view, about 1/48 of the batch each (at least 64 Ki pixels)
  const uint64_t chunk_pix = std::max<uint64_t>(all_pix / 48, 65536);
  ctx->chunks.clear();
  uint64_t pix = 0, tiles = 0;
  for (uint32_t v = 0; v < n_views; v++) {
    const lrt_view &in = views[v];
    if (in.width == 0 || in.height == 0 || in.width > 65535 || in.height > 65535)
      return fail(ctx, LRT_ERR_INVALID, "render: bad view size");
    DevView &o = ctx->h_views[v];
    std::memset(&o, 0, sizeof(o));
    o.width = in.width;
    o.height = in.height;
    o.pix_offset = uint32_t(pix);
    o.tile_offset = uint32_t(tiles);
    const uint32_t tw = uint32_t(ctx->tuning.tile_w), th = 32u / tw;
    o.tile_w_log2 = tw == 4 ? 2u : tw == 16 ? 4u : tw == 32 ? 5u : 3u;
    o.tiles_x = (in.width + tw - 1) / tw;
    lrt_inverse4x4(in.proj, o.proj_inv);       // UpdateCamera, Renderer/eye_ray_host.cpp:59-65
    lrt_inverse4x4(in.world_view, o.wv_inv);
    const uint32_t tile_rows = (in.height + th - 1) / th;
    o.rows_per_chunk = uint32_t(std::min<uint64_t>(
        tile_rows, std::max<uint64_t>(1, chunk_pix / (uint64_t(in.width) * th))));
    o.chunk_offset = uint32_t(ctx->chunks.size());
    for (uint32_t r = 0; r < tile_rows; r += o.rows_per_chunk) {
      const uint32_t r1 = std::min(tile_rows, r + o.rows_per_chunk);
      ctx->chunks.push_back({(r1 - r) * o.tiles_x, pix + uint64_t(r) * th * in.width,
                             pix + uint64_t(std::min(r1 * th, in.height)) * in.width});
    }
    pix += uint64_t(in.width) * in.height;
    tiles += uint64_t(o.tiles_x) * tile_rows;
  }
  if (pix >= (1ull << 32) || tiles >= (1ull << 32)) return fail(ctx, LRT_ERR_INVALID, "render: batch too large");
  LRT_CUDA(ctx, ctx->d_views.ensure(n_views));
  LRT_CUDA(ctx, cudaMemcpyAsync(ctx->d_views.p, ctx->h_views, n_views * sizeof(DevView), cudaMemcpyHostToDevice, st));
  *total_tiles = uint32_t(tiles);
  *total_pix = pix;
  return LRT_OK;
}

// the tuned stack must hold the committed tree: (W-1)*depth + 1 entries, plus slack
static bool stack_fits(const lrt_ctx *ctx) { return 3 * int(ctx->bvh.max_depth) + 4 <= ctx->tuning.stack; }

// Page-locked host outputs (mapped device addresses) the kernel writes directly.
struct HostOutputs {
  lrt_hit16 *hits16;
  float *rgba;
  uint32_t *rgba8;
};

// chunked: count finished tiles per output chunk (ctx->chunks) in d_chunk_done:
// zeroed before the launch (event chunks_zeroed), and every count set to
// 0x7F7F7F7F after it (event render_done), so that a wait for any chunk's count
// ends once the render has, whatever the kernel published.  With `tail`, the
// last whole chunks (at most 1/16 of the batch) are written to those host
// outputs by the kernel itself; ctx->chunk_copy_end is the first of them.
static lrt_status render_impl(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, lrt_hit16 *hits16, float *rgba,
                              uint32_t *rgba8, cudaStream_t st, unsigned long long *counters, bool chunked = false,
                              const HostOutputs *tail = nullptr) {
  if (!ctx->committed) return fail(ctx, LRT_ERR_STATE, "render: commit the scene first");
  if (!stack_fits(ctx)) return fail(ctx, LRT_ERR_UNSUPPORTED, "render: the tuned stack is too small for this BVH");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  uint32_t tiles = 0;
  uint64_t pix = 0;
  lrt_status s = prepare_views(ctx, views, n_views, st, &tiles, &pix);
  if (s != LRT_OK) return s;
  if ((s = ensure_walk(ctx)) != LRT_OK) return s;
  RenderLaunch L;
  L.views = ctx->d_views.p;
  L.n_views = n_views;
  L.total_tiles = tiles;
  L.hits16 = hits16;
  L.rgba = reinterpret_cast<float4 *>(rgba);
  L.rgba8 = rgba8;
  L.tile_counter = ctx->d_tile_counter.p;
  L.counters = counters;
  const size_t chunk_bytes = ctx->chunks.size() * sizeof(uint32_t);
  ctx->chunk_copy_end = ctx->chunks.size();
  if (chunked && tail) {
    uint64_t direct = 0;
    while (ctx->chunk_copy_end > 1) {
      const lrt_ctx::Chunk &k = ctx->chunks[ctx->chunk_copy_end - 1];
      if (direct + (k.end_pixel - k.first_pixel) > pix / 16) break;
      direct += k.end_pixel - k.first_pixel;
      ctx->chunk_copy_end--;
    }
    if (ctx->chunk_copy_end < ctx->chunks.size()) {
      L.direct_from = ctx->chunks[ctx->chunk_copy_end].first_pixel;
      L.hits16_direct = tail->hits16;
      L.rgba_direct = reinterpret_cast<float4 *>(tail->rgba);
      L.rgba8_direct = tail->rgba8;
    }
  }
  if (chunked) {
    LRT_CUDA(ctx, ctx->d_chunk_done.ensure(ctx->chunks.size()));
    LRT_CUDA(ctx, cudaMemsetAsync(ctx->d_chunk_done.p, 0, chunk_bytes, st));
    LRT_CUDA(ctx, cudaEventRecord(ctx->chunks_zeroed, st));
    L.chunk_done = ctx->d_chunk_done.p;
  }
  LRT_CUDA(ctx, cudaMemsetAsync(ctx->d_tile_counter.p, 0, sizeof(uint32_t), st));
  LRT_CUDA(ctx, dispatch_render(ctx, L, st, counters != nullptr));
  if (chunked) {
    LRT_CUDA(ctx, cudaMemsetAsync(ctx->d_chunk_done.p, 0x7F, chunk_bytes, st));
    LRT_CUDA(ctx, cudaEventRecord(ctx->render_done, st));
  }
  ctx->last_launches = 1;
  return LRT_OK;
}

extern "C" lrt_status lrt_render(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, lrt_hit16 *hits16, float *rgba,
                                 uint32_t *rgba8, void *stream) {
  if (!ctx) return LRT_ERR_INVALID;
  return render_impl(ctx, views, n_views, hits16, rgba, rgba8, static_cast<cudaStream_t>(stream), nullptr);
}

// Device address of a page-locked host buffer (cudaHostAlloc / cudaHostRegister,
// mapped under unified addressing), or null for pageable memory.
static void *mapped_host(const void *host) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// cuStreamWaitValue32 (driver API, resolved at run time: the library does not
// link the driver), or null where it is unavailable
using WaitValue32Fn = CUresult (*)(CUstream, CUdeviceptr, cuuint32_t, unsigned int);
static WaitValue32Fn stream_wait_value32() {
  static const WaitValue32Fn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuStreamWaitValue32", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return WaitValue32Fn(nullptr);
    }
    return reinterpret_cast<WaitValue32Fn>(p);
  }();
  return fn;
}

// Page-locked outputs of a render whose kernel publishes chunk counts: the kernel
// writes device buffers, and a non-blocking copy stream moves each chunk to the
// host as soon as its tiles are counted, while later tiles render; the kernel
// writes the batch's last chunks (at most 1/16 of it) to the host outputs
// itself, so no copy is left once it ends.  Every operation of the render stream
// is enqueued before the copy stream's waits, and the render stream ends by
// releasing every count, so the waits end whenever the render does.
static lrt_status render_host_chunked(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, uint64_t pix,
                                      lrt_hit16 *hits16, float *rgba, uint32_t *rgba8, const HostOutputs &mapped,
                                      WaitValue32Fn wait) {
  const cudaStream_t st = nullptr;
  if (!ctx->copy_stream) LRT_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  if (!ctx->chunks_zeroed) LRT_CUDA(ctx, cudaEventCreateWithFlags(&ctx->chunks_zeroed, cudaEventDisableTiming));
  if (!ctx->render_done) LRT_CUDA(ctx, cudaEventCreateWithFlags(&ctx->render_done, cudaEventDisableTiming));
  if (hits16) LRT_CUDA(ctx, ctx->d_out_hits.ensure(pix));
  if (rgba) LRT_CUDA(ctx, ctx->d_out_rgba.ensure(pix));
  if (rgba8) LRT_CUDA(ctx, ctx->d_out_rgba8.ensure(pix));
  lrt_status s = render_impl(ctx, views, n_views, hits16 ? ctx->d_out_hits.p : nullptr,
                             rgba ? reinterpret_cast<float *>(ctx->d_out_rgba.p) : nullptr,
                             rgba8 ? ctx->d_out_rgba8.p : nullptr, st, nullptr, true, &mapped);
  if (s != LRT_OK) return s;
  const cudaStream_t cs = ctx->copy_stream;
  cudaError_t e = cudaStreamWaitEvent(cs, ctx->chunks_zeroed, 0);
  bool waiting = true;   // false: a wait could not be enqueued; copy after the render instead
  for (size_t c = 0; c < ctx->chunk_copy_end && e == cudaSuccess; c++) {
    const lrt_ctx::Chunk &k = ctx->chunks[c];
    // the last chunk is finished when the kernel is: its copy waits for the event
    if (waiting && (c + 1 == ctx->chunks.size() ||
                    wait(reinterpret_cast<CUstream>(cs), reinterpret_cast<CUdeviceptr>(ctx->d_chunk_done.p + c),
                         k.tiles, CU_STREAM_WAIT_VALUE_GEQ) != CUDA_SUCCESS)) {
      waiting = false;
      e = cudaStreamWaitEvent(cs, ctx->render_done, 0);
    }
    const uint64_t p0 = k.first_pixel, n = k.end_pixel - k.first_pixel;
    if (hits16 && e == cudaSuccess)
      e = cudaMemcpyAsync(hits16 + p0, ctx->d_out_hits.p + p0, n * sizeof(lrt_hit16), cudaMemcpyDeviceToHost, cs);
    if (rgba && e == cudaSuccess)
      e = cudaMemcpyAsync(rgba + 4 * p0, ctx->d_out_rgba.p + p0, n * sizeof(float4), cudaMemcpyDeviceToHost, cs);
    if (rgba8 && e == cudaSuccess)
      e = cudaMemcpyAsync(rgba8 + p0, ctx->d_out_rgba8.p + p0, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, cs);
  }
  // both streams drain whatever was enqueued (the render stream's release ends any wait)
  const cudaError_t e1 = cudaStreamSynchronize(cs), e2 = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = e1 != cudaSuccess ? e1 : e2;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "lrt_render_host");
  return LRT_OK;
}

// Outputs in page-locked host memory: rendered into device buffers and copied
// chunk by chunk while the render runs (render_host_chunked), or, where the
// kernel does not publish chunks ("host_copy" 0, the packet / refill / leaf-queue
// / proposal kernels), written by the kernel itself across the host link.
// Pageable outputs are rendered into device buffers and copied back.
extern "C" lrt_status lrt_render_host(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, lrt_hit16 *hits16,
                                      float *rgba, uint32_t *rgba8) {
  if (!ctx) return LRT_ERR_INVALID;
  if (!views || n_views == 0) return fail(ctx, LRT_ERR_INVALID, "render: no views");
  uint64_t pix = 0, tiles = 0;
  const uint32_t tw = uint32_t(ctx->tuning.tile_w), th = 32u / tw;
  for (uint32_t v = 0; v < n_views; v++) {
    pix += uint64_t(views[v].width) * views[v].height;
    tiles += uint64_t((views[v].width + tw - 1) / tw) * ((views[v].height + th - 1) / th);
  }
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  lrt_hit16 *m_hits = hits16 ? static_cast<lrt_hit16 *>(mapped_host(hits16)) : nullptr;
  float *m_rgba = rgba ? static_cast<float *>(mapped_host(rgba)) : nullptr;
  uint32_t *m_rgba8 = rgba8 ? static_cast<uint32_t *>(mapped_host(rgba8)) : nullptr;
  const WaitValue32Fn wait = ctx->tuning.host_copy ? stream_wait_value32() : nullptr;
  if (wait && ctx->committed && (hits16 || rgba || rgba8) && (!hits16 || m_hits) && (!rgba || m_rgba) &&
      (!rgba8 || m_rgba8) && n_views <= 256 && tiles < (1ull << 32) &&
      dispatch_publishes_chunks(ctx, rgba || rgba8, uint32_t(tiles)))
    return render_host_chunked(ctx, views, n_views, pix, hits16, rgba, rgba8, HostOutputs{m_hits, m_rgba, m_rgba8},
                               wait);
  if (hits16 && !m_hits) LRT_CUDA(ctx, ctx->d_out_hits.ensure(pix));
  if (rgba && !m_rgba) LRT_CUDA(ctx, ctx->d_out_rgba.ensure(pix));
  if (rgba8 && !m_rgba8) LRT_CUDA(ctx, ctx->d_out_rgba8.ensure(pix));
  const cudaStream_t st = nullptr;
  lrt_status s = render_impl(ctx, views, n_views, hits16 ? (m_hits ? m_hits : ctx->d_out_hits.p) : nullptr,
                             rgba ? (m_rgba ? m_rgba : reinterpret_cast<float *>(ctx->d_out_rgba.p)) : nullptr,
                             rgba8 ? (m_rgba8 ? m_rgba8 : ctx->d_out_rgba8.p) : nullptr, st, nullptr);
  if (s != LRT_OK) return s;
  if (hits16 && !m_hits)
    LRT_CUDA(ctx, cudaMemcpyAsync(hits16, ctx->d_out_hits.p, pix * sizeof(lrt_hit16), cudaMemcpyDeviceToHost, st));
  if (rgba && !m_rgba)
    LRT_CUDA(ctx, cudaMemcpyAsync(rgba, ctx->d_out_rgba.p, pix * sizeof(float4), cudaMemcpyDeviceToHost, st));
  if (rgba8 && !m_rgba8)
    LRT_CUDA(ctx, cudaMemcpyAsync(rgba8, ctx->d_out_rgba8.p, pix * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  LRT_CUDA(ctx, cudaStreamSynchronize(st));
  return LRT_OK;
}

// No allocation anywhere on this path: the view table is built in a stack array
// and handed by value to a set-up kernel that writes it into the file-scope
// scratch array of trace.cu; errors are returned as codes only.
extern "C" lrt_status lrt_render_noalloc(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, lrt_hit16 *hits16,
                                         float *rgba, uint32_t *rgba8, void *stream) {
  if (!ctx || !views || n_views == 0 || n_views > LRT_NOALLOC_MAX_VIEWS) return LRT_ERR_INVALID;
  if (!ctx->committed) return LRT_ERR_STATE;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return LRT_ERR_CUDA;
  DevView hv[LRT_NOALLOC_MAX_VIEWS];
  uint64_t pix = 0, tiles = 0;
  for (uint32_t v = 0; v < n_views; v++) {
    const lrt_view &in = views[v];
    if (in.width == 0 || in.height == 0 || in.width > 65535 || in.height > 65535) return LRT_ERR_INVALID;
    DevView &o = hv[v];
    std::memset(&o, 0, sizeof(o));
    o.width = in.width;
    o.height = in.height;
    o.pix_offset = uint32_t(pix);
    o.tile_offset = uint32_t(tiles);
    const uint32_t tw = uint32_t(ctx->tuning.tile_w), th = 32u / tw;
    o.tile_w_log2 = tw == 4 ? 2u : tw == 16 ? 4u : tw == 32 ? 5u : 3u;
    o.tiles_x = (in.width + tw - 1) / tw;
    lrt_inverse4x4(in.proj, o.proj_inv);       // UpdateCamera, Renderer/eye_ray_host.cpp:59-65
    lrt_inverse4x4(in.world_view, o.wv_inv);
    pix += uint64_t(in.width) * in.height;
    tiles += uint64_t(o.tiles_x) * ((in.height + th - 1) / th);
  }
  if (pix >= (1ull << 32) || tiles >= (1ull << 32)) return LRT_ERR_INVALID;
  if (!stack_fits(ctx)) return LRT_ERR_UNSUPPORTED;
  // "first_hit": the reference's walk needs its tree on the device; uploading it
  // would allocate, so an earlier call must have done so
  const bool first_hit = ctx->tuning.first_hit && sdf_scene(ctx->dev);
  if (first_hit && !ctx->ref_pairs_ready) return LRT_ERR_STATE;
  const cudaError_t e = launch_render_noalloc(ctx->dev, hv, n_views, uint32_t(tiles), hits16,
                                              reinterpret_cast<float4 *>(rgba), rgba8, ctx->device, ctx->num_sms,
                                              static_cast<cudaStream_t>(stream), ctx->tuning, first_hit);
  if (e != cudaSuccess) return e == cudaErrorInvalidValue ? LRT_ERR_INVALID : LRT_ERR_CUDA;
  ctx->last_launches = 2;   // set-up kernel + render kernel
  return LRT_OK;
}

extern "C" lrt_status lrt_render_counters(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, uint64_t out[4]) {
  if (!ctx || !out) return LRT_ERR_INVALID;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, cudaMemset(ctx->d_counters.p, 0, 4 * sizeof(unsigned long long)));
  lrt_status s = render_impl(ctx, views, n_views, nullptr, nullptr, nullptr, nullptr, ctx->d_counters.p);
  if (s != LRT_OK) return s;
  unsigned long long h[4];
  LRT_CUDA(ctx, cudaMemcpy(h, ctx->d_counters.p, sizeof(h), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 4; i++) out[i] = h[i];
  return LRT_OK;
}

extern "C" lrt_status lrt_query_rays(lrt_ctx *ctx, const float *pos_near, const float *dir_far, uint32_t n,
                                     lrt_hit *out, int device_ptrs, void *stream) {
  if (!ctx) return LRT_ERR_INVALID;
  if (!ctx->committed) return fail(ctx, LRT_ERR_STATE, "lrt_query_rays: commit the scene first");
  if (n == 0) return LRT_OK;
  if (!pos_near || !dir_far || !out) return fail(ctx, LRT_ERR_INVALID, "lrt_query_rays: null array");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  lrt_status ws = ensure_walk(ctx);
  if (ws != LRT_OK) return ws;
  const bool ref = ctx->tuning.first_hit && sdf_scene(ctx->dev);
  auto launch_q = [&](const float4 *p, const float4 *d, lrt_hit *o) {
    return ref ? launch_query_ref(ctx->dev, p, d, n, o, st) : launch_query(ctx->dev, p, d, n, o, st);
  };
  if (device_ptrs) {
    LRT_CUDA(ctx, launch_q(reinterpret_cast<const float4 *>(pos_near), reinterpret_cast<const float4 *>(dir_far), out));
    ctx->last_launches = 1;
    return LRT_OK;
  }
  LRT_CUDA(ctx, ctx->d_q_pos.ensure(n));
  LRT_CUDA(ctx, ctx->d_q_dir.ensure(n));
  LRT_CUDA(ctx, ctx->d_q_out.ensure(n));
  LRT_CUDA(ctx, cudaMemcpyAsync(ctx->d_q_pos.p, pos_near, size_t(n) * 16, cudaMemcpyHostToDevice, st));
  LRT_CUDA(ctx, cudaMemcpyAsync(ctx->d_q_dir.p, dir_far, size_t(n) * 16, cudaMemcpyHostToDevice, st));
  LRT_CUDA(ctx, launch_q(ctx->d_q_pos.p, ctx->d_q_dir.p, ctx->d_q_out.p));
  LRT_CUDA(ctx, cudaMemcpyAsync(out, ctx->d_q_out.p, size_t(n) * sizeof(lrt_hit), cudaMemcpyDeviceToHost, st));
  LRT_CUDA(ctx, cudaStreamSynchronize(st));
  ctx->last_launches = 1;
  return LRT_OK;
}

extern "C" lrt_status lrt_build_bvh2(const float *boxes6, uint32_t n, uint32_t prims_per_leaf, lrt_bvh_pair **pairs,
                                     uint32_t *n_pairs, uint32_t **leaf_start_count, uint32_t *n_leaves,
                                     uint32_t **order) {
  if (!boxes6 || n == 0 || !pairs || !n_pairs || (prims_per_leaf != 1 && prims_per_leaf != 2)) return LRT_ERR_INVALID;
  BvhData b;
  const lrt_status s = build_bvh(boxes6, n, prims_per_leaf == 1, b);
  if (s != LRT_OK) return s;
  *pairs = static_cast<lrt_bvh_pair *>(std::malloc(b.pairs.size() * sizeof(lrt_bvh_pair)));
  if (!*pairs) return LRT_ERR_OOM;
  std::memcpy(*pairs, b.pairs.data(), b.pairs.size() * sizeof(lrt_bvh_pair));
  *n_pairs = uint32_t(b.pairs.size());
  if (leaf_start_count) {
    *leaf_start_count = static_cast<uint32_t *>(std::malloc(std::max<size_t>(1, b.leaf_start_count.size()) * 4));
    std::memcpy(*leaf_start_count, b.leaf_start_count.data(), b.leaf_start_count.size() * 4);
  }
  if (n_leaves) *n_leaves = uint32_t(b.leaf_start_count.size());
  if (order) {
    *order = static_cast<uint32_t *>(std::malloc(b.order.size() * 4));
    std::memcpy(*order, b.order.data(), b.order.size() * 4);
  }
  return LRT_OK;
}

extern "C" void lrt_free(void *p) { std::free(p); }

// ---------------------------------------------------------------- scene construction

extern "C" lrt_status lrt_sbs_build_from_sdf(const lrt_sdf_desc *sdf, uint32_t depth, const lrt_sbs_header *hdr,
                                             int threads, lrt_sbs **out) {
  if (!sdf || !hdr || !out || (sdf->n_spheres + sdf->n_boxes) == 0) return LRT_ERR_INVALID;
  lrt_sbs *r = new (std::nothrow) lrt_sbs();
  if (!r) return LRT_ERR_OOM;
  lrt_status s = build_sbs(*sdf, depth, *hdr, threads, r->d);
  if (s != LRT_OK) { delete r; return s; }
  *out = r;
  return LRT_OK;
}

extern "C" lrt_status lrt_sbs_data(const lrt_sbs *sbs, lrt_sbs_header *hdr, const lrt_sbs_node **nodes, uint32_t *n_nodes,
                                   const uint32_t **values, uint32_t *n_values) {
  if (!sbs) return LRT_ERR_INVALID;
  if (hdr) *hdr = sbs->d.hdr;
  if (nodes) *nodes = sbs->d.nodes.data();
  if (n_nodes) *n_nodes = uint32_t(sbs->d.nodes.size());
  if (values) *values = sbs->d.values.data();
  if (n_values) *n_values = uint32_t(sbs->d.values.size());
  return LRT_OK;
}

extern "C" void lrt_sbs_free(lrt_sbs *sbs) { delete sbs; }

extern "C" lrt_status lrt_svs_build_from_sdf(const lrt_sdf_desc *sdf, uint32_t depth, int threads, lrt_svs **out) {
  if (!sdf || !out || (sdf->n_spheres + sdf->n_boxes) == 0) return LRT_ERR_INVALID;
  lrt_svs *r = new (std::nothrow) lrt_svs();
  if (!r) return LRT_ERR_OOM;
  lrt_status s = build_svs(*sdf, depth, threads, r->nodes);
  if (s != LRT_OK) { delete r; return s; }
  *out = r;
  return LRT_OK;
}

// The GPU builders report errors through their return code only (no context);
// the message of the last failure on this thread is kept for lrt_build_last_error.
static thread_local std::string g_build_error;

extern "C" const char *lrt_build_last_error(void) { return g_build_error.c_str(); }

static bool sdf_args_ok(const lrt_sdf_desc *sdf) {
  if (!sdf || (sdf->n_spheres + sdf->n_boxes) == 0) return false;
  if ((sdf->n_spheres && !sdf->spheres) || (sdf->n_boxes && !sdf->boxes)) return false;
  return true;
}

extern "C" lrt_status lrt_sbs_build_from_sdf_gpu(int device, const lrt_sdf_desc *sdf, uint32_t depth,
                                                 const lrt_sbs_header *hdr, lrt_sbs **out) {
  g_build_error.clear();
  if (!sdf_args_ok(sdf) || !hdr || !out) return LRT_ERR_INVALID;
  if (hdr->brick_size < 1 || hdr->brick_size > 16 || hdr->brick_pad > 1 ||
      !(hdr->bytes_per_value == 1 || hdr->bytes_per_value == 2 || hdr->bytes_per_value == 4) || depth > 15)
    return LRT_ERR_INVALID;
  if ((hdr->aux_data & 0xFF000000u) != LRT_SBS_LAYOUT_DX && (hdr->aux_data & 0xFF000000u) != LRT_SBS_LAYOUT_UNDEFINED)
    return LRT_ERR_UNSUPPORTED;
  if (depth < 4) {
    g_build_error = "the GPU builder needs depth >= 4 (use lrt_sbs_build_from_sdf)";
    return LRT_ERR_UNSUPPORTED;
  }
  if (cudaSetDevice(device) != cudaSuccess) return LRT_ERR_CUDA;
  lrt_sbs *r = new (std::nothrow) lrt_sbs();
  if (!r) return LRT_ERR_OOM;
  lrt_status s = build_sbs_gpu(*sdf, depth, *hdr, r->d, g_build_error);
  if (s != LRT_OK) { delete r; return s; }
  *out = r;
  return LRT_OK;
}

extern "C" lrt_status lrt_svs_build_from_sdf_gpu(int device, const lrt_sdf_desc *sdf, uint32_t depth, lrt_svs **out) {
  g_build_error.clear();
  if (!sdf_args_ok(sdf) || !out || depth > 15) return LRT_ERR_INVALID;
  if (depth < 4) {
    g_build_error = "the GPU builder needs depth >= 4 (use lrt_svs_build_from_sdf)";
    return LRT_ERR_UNSUPPORTED;
  }
  if (cudaSetDevice(device) != cudaSuccess) return LRT_ERR_CUDA;
  lrt_svs *r = new (std::nothrow) lrt_svs();
  if (!r) return LRT_ERR_OOM;
  lrt_status s = build_svs_gpu(*sdf, depth, r->nodes, g_build_error);
  if (s != LRT_OK) { delete r; return s; }
  *out = r;
  return LRT_OK;
}

extern "C" lrt_status lrt_svs_data(const lrt_svs *svs, const lrt_svs_node **nodes, uint32_t *n_nodes) {
  if (!svs) return LRT_ERR_INVALID;
  if (nodes) *nodes = svs->nodes.data();
  if (n_nodes) *n_nodes = uint32_t(svs->nodes.size());
  return LRT_OK;
}

extern "C" void lrt_svs_free(lrt_svs *svs) { delete svs; }

// ---------------------------------------------------------------- CUDA graph of a batched render
// The persistent launch of a fixed view batch captured once (work-queue reset +
// kernel) and replayed; the graph owns its view table and queue head, so
// replays and ordinary renders on the same context do not interfere.
struct lrt_graph {
  int device = 0;
  uint32_t n_views = 0;
  std::vector<lrt_view> views;
  DevBuf<DevView> d_views;
  DevBuf<uint32_t> d_head;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

static lrt_status fill_views(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, std::vector<DevView> &out,
                             uint32_t *total_tiles) {
  uint64_t pix = 0, tiles = 0;
  out.assign(n_views, DevView{});
  const uint32_t tw = uint32_t(ctx->tuning.tile_w), th = 32u / tw;
  for (uint32_t v = 0; v < n_views; v++) {
    const lrt_view &in = views[v];
    if (in.width == 0 || in.height == 0 || in.width > 65535 || in.height > 65535)
      return fail(ctx, LRT_ERR_INVALID, "render: bad view size");
    DevView &o = out[v];
    o.width = in.width;
    o.height = in.height;
    o.pix_offset = uint32_t(pix);
    o.tile_offset = uint32_t(tiles);
    o.tile_w_log2 = tw == 4 ? 2u : tw == 16 ? 4u : tw == 32 ? 5u : 3u;
    o.tiles_x = (in.width + tw - 1) / tw;
    lrt_inverse4x4(in.proj, o.proj_inv);
    lrt_inverse4x4(in.world_view, o.wv_inv);
    pix += uint64_t(in.width) * in.height;
    tiles += uint64_t(o.tiles_x) * ((in.height + th - 1) / th);
  }
  if (pix >= (1ull << 32) || tiles >= (1ull << 32)) return fail(ctx, LRT_ERR_INVALID, "render: batch too large");
  *total_tiles = uint32_t(tiles);
  return LRT_OK;
}

extern "C" void lrt_render_graph_destroy(lrt_graph *g) {
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  g->d_views.release();
  g->d_head.release();
  delete g;
}

extern "C" lrt_status lrt_render_graph_create(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views,
                                              lrt_hit16 *hits16, float *rgba, uint32_t *rgba8, lrt_graph **out) {
  if (!ctx || !views || n_views == 0 || !out) return LRT_ERR_INVALID;
  if (!ctx->committed) return fail(ctx, LRT_ERR_STATE, "graph: commit the scene first");
  if (!stack_fits(ctx)) return fail(ctx, LRT_ERR_UNSUPPORTED, "graph: the tuned stack is too small for this BVH");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  std::vector<DevView> hv;
  uint32_t tiles = 0;
  lrt_status s = fill_views(ctx, views, n_views, hv, &tiles);
  if (s != LRT_OK) return s;
  if ((s = ensure_walk(ctx)) != LRT_OK) return s;
  lrt_graph *g = new (std::nothrow) lrt_graph();
  if (!g) return fail(ctx, LRT_ERR_OOM, "graph allocation failed");
  g->device = ctx->device;
  g->n_views = n_views;
  g->views.assign(views, views + n_views);
  cudaError_t e = g->d_views.ensure(n_views);
  if (e == cudaSuccess) e = g->d_head.ensure(1);
  if (e == cudaSuccess) e = cudaMemcpy(g->d_views.p, hv.data(), n_views * sizeof(DevView), cudaMemcpyHostToDevice);
  cudaStream_t cs = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    RenderLaunch L;
    L.views = g->d_views.p;
    L.n_views = n_views;
    L.total_tiles = tiles;
    L.hits16 = hits16;
    L.rgba = reinterpret_cast<float4 *>(rgba);
    L.rgba8 = rgba8;
    L.tile_counter = g->d_head.p;
    L.counters = nullptr;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
      cudaError_t e1 = cudaMemsetAsync(g->d_head.p, 0, sizeof(uint32_t), cs);
      cudaError_t e2 = e1 == cudaSuccess ? dispatch_render(ctx, L, cs, false) : e1;
      e = cudaStreamEndCapture(cs, &g->graph);
      if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = inject_fault("graph") ? cudaErrorInvalidValue : cudaGraphInstantiate(&g->exec, g->graph, 0);
  }
  if (cs) cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    lrt_render_graph_destroy(g);
    return cuda_fail(ctx, e, "lrt_render_graph_create");
  }
  *out = g;
  return LRT_OK;
}

extern "C" lrt_status lrt_render_graph_launch(lrt_ctx *ctx, lrt_graph *g, void *stream) {
  if (!ctx || !g) return LRT_ERR_INVALID;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)));
  ctx->last_launches = 1;
  return LRT_OK;
}

extern "C" lrt_status lrt_render_graph_set_views(lrt_ctx *ctx, lrt_graph *g, const lrt_view *views, uint32_t n_views) {
  if (!ctx || !g || !views || n_views != g->n_views) return fail(ctx, LRT_ERR_INVALID, "graph: view count differs");
  for (uint32_t v = 0; v < n_views; v++)
    if (views[v].width != g->views[v].width || views[v].height != g->views[v].height)
      return fail(ctx, LRT_ERR_INVALID, "graph: view sizes are fixed at capture");
  std::vector<DevView> hv;
  uint32_t tiles = 0;
  lrt_status s = fill_views(ctx, views, n_views, hv, &tiles);
  if (s != LRT_OK) return s;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, cudaMemcpy(g->d_views.p, hv.data(), n_views * sizeof(DevView), cudaMemcpyHostToDevice));
  g->views.assign(views, views + n_views);
  return LRT_OK;
}

// ---------------------------------------------------------------- autotuner
// Times each candidate launch shape on the given views (device hit buffer,
// CUDA events, median of `reps` after one warm-up), keeps the fastest in the
// context and reports every candidate.  Results do not depend on the choice.
extern "C" lrt_status lrt_autotune(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, uint32_t reps,
                                   lrt_tuning_choice *best, lrt_tuning_choice *all, uint32_t cap, uint32_t *n_tried) {
  if (!ctx || !views || n_views == 0 || reps == 0 || !best) return LRT_ERR_INVALID;
  if (!ctx->committed) return fail(ctx, LRT_ERR_STATE, "autotune: commit the scene first");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  uint64_t pix = 0;
  for (uint32_t v = 0; v < n_views; v++) pix += uint64_t(views[v].width) * views[v].height;
  LRT_CUDA(ctx, ctx->d_out_hits.ensure(size_t(pix)));
  const bool sbs = ctx->dev.type == LRT_TYPE_SDF_SBS || ctx->dev.type == LRT_TYPE_SDF_SBS_COL ||
                   ctx->dev.type == LRT_TYPE_SDF_SBS_TEX;
  std::vector<lrt_tuning_choice> cand;
  for (int tw : {4, 8, 16})
    for (int stk : {32, 64}) cand.push_back(lrt_tuning_choice{0, 4, 0, tw, stk, 0.0f});
  for (int tw : {4, 8})
    for (int stk : {32, 64}) cand.push_back(lrt_tuning_choice{2, 4, 0, tw, stk, 0.0f});
  if (sbs)
    for (int stage : {0, 1})
      for (int bw : {2, 4}) cand.push_back(lrt_tuning_choice{1, bw, stage, 8, 64, 0.0f});
  const Tuning saved = ctx->tuning;
  cudaEvent_t a = nullptr, b = nullptr;
  LRT_CUDA(ctx, cudaEventCreate(&a));
  LRT_CUDA(ctx, cudaEventCreate(&b));
  lrt_tuning_choice win{};
  win.ms = 3.0e38f;
  uint32_t tried = 0;
  lrt_status st = LRT_OK;
  for (lrt_tuning_choice &c : cand) {
    ctx->tuning.variant = c.variant;
    ctx->tuning.block_warps = c.block_warps;
    ctx->tuning.stage = c.stage;
    ctx->tuning.tile_w = c.tile_w;
    ctx->tuning.stack = c.stack;
    if (!stack_fits(ctx)) continue;
    std::vector<float> ts;
    for (uint32_t r = 0; r <= reps && st == LRT_OK; r++) {
      cudaEventRecord(a, nullptr);
      st = render_impl(ctx, views, n_views, ctx->d_out_hits.p, nullptr, nullptr, nullptr, nullptr);
      cudaEventRecord(b, nullptr);
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (r > 0) ts.push_back(ms);
    }
    if (st != LRT_OK) break;
    std::sort(ts.begin(), ts.end());
    c.ms = ts[ts.size() / 2];
    if (all && tried < cap) all[tried] = c;
    tried++;
    if (c.ms < win.ms) win = c;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (st != LRT_OK) {
    ctx->tuning = saved;
    return st;
  }
  ctx->tuning.variant = win.variant;
  ctx->tuning.block_warps = win.block_warps;
  ctx->tuning.stage = win.stage;
  ctx->tuning.tile_w = win.tile_w;
  ctx->tuning.stack = win.stack;
  *best = win;
  if (n_tried) *n_tried = tried;
  return LRT_OK;
}
