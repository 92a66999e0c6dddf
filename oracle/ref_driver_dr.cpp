// Driver around the reference's differentiable renderer and scene builders,
// compiled in place (oracle pinning only; built by oracle/build_ref.py into
// oracle/_ref/libref_dr.so where the reference tree is present).
//
// Compiled in place beside this file: BVH/BVH2Common.cpp, diff_render/BVH2DR.cpp,
// Renderer/eye_ray.cpp (pixel packing, eye rays, rand2), diff_render/MultiRendererDR.cpp
// (RenderDR, CastRayWithGrad, the border integral, OptimizeStepAdam,
// OptimizeFixedStructure), diff_render/DR_common.cpp (create_grid_sbs) and
// utils/sparse_octree_builder.cpp (frame octree, frame_octree_to_SBS / _SVS,
// SBS_ind_to_SBS_ind_with_neighbors).
//
// This file supplies what those units take from translation units that cannot be
// compiled here (they need LiteScene, Hydra, Embree): the MultiRenderer members
// of Renderer/eye_ray_host.cpp and the BVHRT members of BVH/BVH2Common_host.cpp
// that OptimizeFixedStructure reaches, restated line by line (the BVH itself
// comes from the caller: the reference builds it with Embree, which is absent),
// stubs for members off these paths, and a C interface for the tests.
#include <omp.h>

#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "BVH/BVH2Common.h"
#include "diff_render/BVH2DR.h"
#include "diff_render/MultiRendererDR.h"
#include "diff_render/DR_common.h"
#include "utils/sparse_octree_builder.h"
#include "utils/points_visualizer.h"

using LiteMath::float2;
using LiteMath::float3;
using LiteMath::float4;
using LiteMath::float4x4;

namespace {
// the BVH2 the next AddGeom_AABB installs (the caller's tree for the bricks)
std::vector<BVHNodePair> g_next_pairs;
}

// ---------------------------------------------------------------- BVHRT host members
// BVHRT::ClearGeom, BVH/BVH2Common_host.cpp:82-108
void BVHRT::ClearGeom() {
  m_geomData.resize(0);
  m_abstractObjectPtrs.resize(0);
  startEnd.resize(0);
  m_indices.resize(0);
  m_vertPos.resize(0);
  m_primIndices.resize(0);
  m_allNodePairs.resize(0);
  m_abstractObjects.resize(0);
  ClearScene();
}
// BVHRT::ClearScene, :1382-1388
void BVHRT::ClearScene() {
  m_instanceData.resize(0);
  m_firstSceneCommit = true;
}
// BVHRT::AddGeom_AABB, :264-280, with the caller's fat pairs in place of
// BuildBVHFatCustom (Embree): leaf payloads are the box indices.
uint32_t BVHRT::AddGeom_AABB(uint32_t, const CRT_AABB *, size_t a_boxNumber, void **, size_t) {
  m_allNodePairs.insert(m_allNodePairs.end(), g_next_pairs.begin(), g_next_pairs.end());
  const size_t oldSize = m_primIdCount.size();
  m_primIdCount.resize(oldSize + a_boxNumber);
  for (size_t i = 0; i < a_boxNumber; i++) m_primIdCount[oldSize + i] = uint32_t(i);
  startEnd.push_back(uint2(uint32_t(oldSize), uint32_t(m_primIdCount.size())));
  return uint32_t(startEnd.size() - 1);
}
// BVHRT::AddGeom_SdfSBS, :567-666
uint32_t BVHRT::AddGeom_SdfSBS(SdfSBSView octree, ISceneObject *fake_this, BuildOptions) {
  uint32_t type = TYPE_SDF_SBS;
  const uint32_t node_layout = octree.header.aux_data & SDF_SBS_NODE_LAYOUT_MASK;
  if (node_layout == SDF_SBS_NODE_LAYOUT_DX_UV16)
    type = TYPE_SDF_SBS_TEX;
  else if (node_layout == SDF_SBS_NODE_LAYOUT_DX_RGB8 || node_layout == SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F ||
           node_layout == SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F_IN)
    type = TYPE_SDF_SBS_COL;
  const float4 mn = float4(-1, -1, -1, 1), mx = float4(1, 1, 1, 1);
  m_abstractObjects.resize(m_abstractObjects.size() + 1);
  const uint32_t typeTag = AbstractObject::TAG_SDF_BRICK;   // type_to_tag, :24-80, for the three SBS types
  new (m_abstractObjects.data() + m_abstractObjects.size() - 1) GeomDataSdfBrick();
  m_abstractObjects.back().geomId = m_abstractObjects.size() - 1;
  m_abstractObjects.back().m_tag = typeTag;
  m_geomData.emplace_back();
  m_geomData.back().boxMin = mn;
  m_geomData.back().boxMax = mx;
  m_geomData.back().offset = uint2(m_SdfSBSRoots.size(), 0);
  m_geomData.back().bvhOffset = m_allNodePairs.size();
  m_geomData.back().type = type;
  const unsigned n_offset = m_SdfSBSNodes.size(), v_offset = m_SdfSBSData.size();
  m_SdfSBSRoots.push_back(n_offset);
  m_SdfSBSHeaders.push_back(octree.header);
  m_SdfSBSNodes.insert(m_SdfSBSNodes.end(), octree.nodes, octree.nodes + octree.size);
  m_SdfSBSData.insert(m_SdfSBSData.end(), octree.values, octree.values + octree.values_count);
  for (size_t i = n_offset; i < m_SdfSBSNodes.size(); i++) m_SdfSBSNodes[i].data_offset += v_offset;
  if (node_layout == SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F || node_layout == SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F_IN) {
    const unsigned f_offset = m_SdfSBSDataF.size();
    m_SdfSBSDataF.insert(m_SdfSBSDataF.end(), octree.values_f, octree.values_f + octree.values_f_count);
    for (size_t i = v_offset; i < m_SdfSBSData.size(); i++) m_SdfSBSData[i] += f_offset;
  }
  std::vector<BVHNode> orig_nodes(octree.size);
  for (size_t i = 0; i < octree.size; i++) {
    const float px = octree.nodes[i].pos_xy >> 16, py = octree.nodes[i].pos_xy & 0x0000FFFF;
    const float pz = octree.nodes[i].pos_z_lod_size >> 16, sz = octree.nodes[i].pos_z_lod_size & 0x0000FFFF;
    orig_nodes[i].boxMin = float3(-1, -1, -1) + 2.0f * float3(px, py, pz) / sz;
    orig_nodes[i].boxMax = orig_nodes[i].boxMin + 2.0f * float3(1, 1, 1) / sz;
  }
  return fake_this->AddGeom_AABB(typeTag, (const CRT_AABB *)orig_nodes.data(), orig_nodes.size(), nullptr, 1);
}
// BVHRT::AddInstance, :1450-1487
uint32_t BVHRT::AddInstance(uint32_t a_geomId, const float4x4 &a_matrix) {
  if (a_geomId & CRT_GEOM_MASK_AABB_BIT) a_geomId = (a_geomId & 0x7fffffff);
  const auto &boxMin = m_geomData[a_geomId].boxMin;
  const auto &boxMax = m_geomData[a_geomId].boxMax;
  const float4 v[8] = {a_matrix * float4{boxMin.x, boxMin.y, boxMin.z, 1.0f}, a_matrix * float4{boxMax.x, boxMin.y, boxMin.z, 1.0f},
                       a_matrix * float4{boxMin.x, boxMax.y, boxMin.z, 1.0f}, a_matrix * float4{boxMin.x, boxMin.y, boxMax.z, 1.0f},
                       a_matrix * float4{boxMax.x, boxMax.y, boxMin.z, 1.0f}, a_matrix * float4{boxMax.x, boxMin.y, boxMax.z, 1.0f},
                       a_matrix * float4{boxMin.x, boxMax.y, boxMax.z, 1.0f}, a_matrix * float4{boxMax.x, boxMax.y, boxMax.z, 1.0f}};
  Box4f newBox;
  for (int i = 0; i < 8; i++) newBox.include(v[i]);
  const uint32_t oldSize = uint32_t(m_instanceData.size());
  InstanceData instance;
  std::memset(&instance, 0, sizeof(instance));
  instance.boxMin = newBox.boxMin;
  instance.boxMax = newBox.boxMax;
  instance.geomId = a_geomId;
  instance.transform = a_matrix;
  instance.transformInv = inverse4x4(a_matrix);
  instance.transformInvTransposed = transpose(inverse4x4(a_matrix));
  m_instanceData.push_back(instance);
  return oldSize;
}
// BVHRT::CommitScene, :1416-1448 (one instance: the TLAS is one leaf node)
void BVHRT::CommitScene(uint32_t) {
  m_nodesTLAS.clear();
  m_nodesTLAS.emplace_back();
  m_nodesTLAS[0].boxMin = to_float3(m_instanceData[0].boxMin);
  m_nodesTLAS[0].boxMax = to_float3(m_instanceData[0].boxMax);
  m_nodesTLAS[0].leftOffset = LEAF_BIT;
  m_nodesTLAS[0].escapeIndex = LEAF_NORMAL;
  m_firstSceneCommit = false;
  m_abstractObjectPtrs.resize(m_abstractObjects.size());
  for (size_t i = 0; i < m_abstractObjects.size(); i++) m_abstractObjectPtrs[i] = m_abstractObjects.data() + i;
}
// off the pinned paths
uint32_t BVHRT::AddCustomGeom_FromFile(const char *, const char *, ISceneObject *) { std::abort(); }
uint32_t BVHRT::AddGeom_Triangles3f(const float *, size_t, const uint32_t *, size_t, uint32_t, size_t) { std::abort(); }
void BVHRT::UpdateGeom_Triangles3f(uint32_t, const float *, size_t, const uint32_t *, size_t, uint32_t, size_t) {}
void BVHRT::UpdateGeom_AABB(uint32_t, uint32_t, const CRT_AABB *, size_t, void **, size_t) {}
void BVHRT::UpdateInstance(uint32_t, const float4x4 &) {}
void BVHRT::AppendTreeData(const std::vector<BVHNodePair> &, const std::vector<uint32_t> &, const uint32_t *, size_t) {}
float BVHRT::eval_distance(float3) { std::abort(); }
void BVHRT::init(SdfGridView) {}

// ---------------------------------------------------------------- MultiRenderer host members
// MultiRenderer::MultiRenderer, Renderer/eye_ray_host.cpp:21-41 (the accel
// structure is set by the caller -- OptimizeFixedStructure sets a BVHDR -- and no
// texture or material is used by the differentiable renderer)
MultiRenderer::MultiRenderer(uint32_t maxPrimitives) {
  m_maxPrimitives = maxPrimitives;
  m_preset = getDefaultPreset();
  m_seed = 0;
  m_lights = {create_direct_light(float3(1, 1, 1), float3(2.0f / 3.0f)),
              create_ambient_light(float3(0.25, 0.25, 0.25))};
}
// :43-50
void MultiRenderer::SetViewport(int, int, int a_width, int a_height) {
  m_width = a_width;
  m_height = a_height;
  m_packedXY_width = PACK_XY_BLOCK_SIZE * ((a_width + PACK_XY_BLOCK_SIZE - 1) / PACK_XY_BLOCK_SIZE);
  m_packedXY_height = PACK_XY_BLOCK_SIZE * ((a_height + PACK_XY_BLOCK_SIZE - 1) / PACK_XY_BLOCK_SIZE);
  m_packedXY.resize(m_packedXY_width * m_packedXY_height);
}
// :59-65
void MultiRenderer::UpdateCamera(const float4x4 &worldView, const float4x4 &proj) {
  m_proj = proj;
  m_worldView = worldView;
  m_projInv = inverse4x4(proj);
  m_worldViewInv = inverse4x4(worldView);
}
// :549-556
void MultiRenderer::SetPreset(const MultiRenderPreset &a_preset) {
  m_preset = a_preset;
  auto *bvhrt = dynamic_cast<BVHRT *>(m_pAccelStruct->UnderlyingImpl(0));
  if (bvhrt) bvhrt->SetPreset(a_preset);
}
// :678-682
uint32_t MultiRenderer::AddInstance(uint32_t a_geomId, const float4x4 &a_matrix) {
  m_instanceTransformInvTransposed.push_back(transpose(inverse4x4(a_matrix)));
  return m_pAccelStruct->AddInstance(a_geomId, a_matrix);
}
// :362-376
void MultiRenderer::SetScene(SdfSBSView scene) {
  BVHRT *bvhrt = dynamic_cast<BVHRT *>(m_pAccelStruct->UnderlyingImpl(0));
  SetPreset(m_preset);
  m_pAccelStruct->ClearGeom();
  auto geomId = bvhrt->AddGeom_SdfSBS(scene, m_pAccelStruct.get());
  m_pAccelStruct->ClearScene();
  AddInstance(geomId, float4x4());
  m_pAccelStruct->CommitScene();
}
// :257-282, serial
void MultiRenderer::CastRaySingleBlock(uint32_t tidX, uint32_t *out_color, uint32_t) {
  for (uint32_t i = 0; i < tidX; i++) CastRaySingle(i, out_color);
}
void MultiRenderer::CastRayFloatSingleBlock(uint32_t tidX, float4 *out_color, uint32_t) {
  for (uint32_t i = 0; i < tidX; i++) CastRayFloatSingle(i, out_color);
}
void MultiRenderer::Render(uint32_t *a_outColor, uint32_t, uint32_t, const char *, int a_passNum) {
  for (int i = 0; i < a_passNum; i++) CastRaySingleBlock(m_packedXY_width * m_packedXY_height, a_outColor, a_passNum);
}
// :575-585
void MultiRenderer::RenderFloat(float4 *imageData, uint32_t a_width, uint32_t a_height, const float4x4 &a_worldView,
                                const float4x4 &a_proj, MultiRenderPreset preset, int a_passNum) {
  SetViewport(0, 0, a_width, a_height);
  UpdateCamera(a_worldView, a_proj);
  SetPreset(preset);
  CommitDeviceData();
  Clear(a_width, a_height, "color");
  RenderFloat(imageData, a_width, a_height, "color", a_passNum);
}
void MultiRenderer::RenderFloat(float4 *a_outColor, uint32_t, uint32_t, const char *, int a_passNum) {
  for (int i = 0; i < a_passNum; i++)
    CastRayFloatSingleBlock(m_packedXY_width * m_packedXY_height, a_outColor, a_passNum);
}
const char *MultiRenderer::Name() const { return "MultiRenderer"; }
bool MultiRenderer::LoadScene(const char *) { return false; }
void MultiRenderer::GetExecutionTime(const char *, float a_out[4]) { a_out[0] = 0.0f; }

// mesh helpers and debug drawing, off the pinned paths
namespace cmesh4 {
float3 closest_point_triangle(const float3 &, const float3 &, const float3 &, const float3 &) { std::abort(); }
float3 barycentric(const float3 &, const float3 &, const float3 &, const float3 &) { std::abort(); }
}  // namespace cmesh4
void draw_points(std::vector<float4> &, std::vector<float4> &, LiteImage::Image2D<float4> &) {}
void draw_line(float2, float2, float, float4, LiteImage::Image2D<float4> &) {}

// ---------------------------------------------------------------- C interface for the tests
namespace {
using SdfFn = float (*)(const void *ctx, float x, float y, float z);

struct RefSbs {
  SdfSBSHeader header;
  std::vector<SdfSBSNode> nodes;
  std::vector<uint32_t> values;
  std::vector<float> values_f;
};

RefSbs *export_sbs(const SdfSBS &s) {
  RefSbs *r = new RefSbs();
  r->header = s.header;
  r->nodes = s.nodes;
  r->values = s.values;
  r->values_f = s.values_f;
  return r;
}
}  // namespace

extern "C" {

// create_sdf_SBS(settings, header, sdf), utils/sdf_converter.cpp:162-181: the
// frame octree to `depth` (brick level), node limit, frame_octree_to_SBS.
void *ref_build_sbs(SdfFn fn, const void *ctx, uint32_t depth, uint32_t brick_size, uint32_t brick_pad,
                    uint32_t bytes_per_value, uint32_t threads) {
  SparseOctreeSettings settings(SparseOctreeBuildType::DEFAULT, depth);
  SdfSBSHeader header;
  header.brick_size = brick_size;
  header.brick_pad = brick_pad;
  header.bytes_per_value = bytes_per_value;
  header.aux_data = SDF_SBS_NODE_LAYOUT_DX;
  sdf_converter::MultithreadedDistanceFunction sdf = [&](const float3 &p, unsigned) -> float { return fn(ctx, p.x, p.y, p.z); };
  auto frame = sdf_converter::construct_sdf_frame_octree(settings, sdf, threads);
  sdf_converter::frame_octree_limit_nodes(frame, settings.nodes_limit, true);
  return export_sbs(sdf_converter::frame_octree_to_SBS(sdf, threads, frame, header));
}

// create_sdf_SVS(settings, sdf), utils/sdf_converter.cpp:118-134
void *ref_build_svs(SdfFn fn, const void *ctx, uint32_t depth, uint32_t threads, uint32_t *n_nodes) {
  SparseOctreeSettings settings(SparseOctreeBuildType::DEFAULT, depth);
  sdf_converter::MultithreadedDistanceFunction sdf = [&](const float3 &p, unsigned) -> float { return fn(ctx, p.x, p.y, p.z); };
  auto frame = sdf_converter::construct_sdf_frame_octree(settings, sdf, threads);
  sdf_converter::frame_octree_limit_nodes(frame, settings.nodes_limit, true);
  auto *nodes = new std::vector<SdfSVSNode>();
  sdf_converter::frame_octree_to_SVS_rec(frame, *nodes, 0, uint3(0, 0, 0), 1);
  *n_nodes = uint32_t(nodes->size());
  return nodes;
}
void ref_svs_copy(void *p, SdfSVSNode *out) {
  auto *v = static_cast<std::vector<SdfSVSNode> *>(p);
  std::memcpy(out, v->data(), v->size() * sizeof(SdfSVSNode));
}
void ref_svs_free(void *p) { delete static_cast<std::vector<SdfSVSNode> *>(p); }

// create_grid_sbs, diff_render/DR_common.cpp:47-146: a dense grid of bricks around
// circle_sdf(center, radius), colours single_color (0) or gradient_color (1).
void *ref_grid_sbs(uint32_t brick_count, uint32_t brick_size, float cx, float cy, float cz, float radius,
                   uint32_t color_mode) {
  auto sdf = [=](float3 p) { return dr::circle_sdf(float3(cx, cy, cz), radius, p); };
  std::function<float3(float3)> col = color_mode ? std::function<float3(float3)>(dr::gradient_color)
                                                 : std::function<float3(float3)>(dr::single_color);
  return export_sbs(dr::create_grid_sbs(brick_count, brick_size, sdf, col));
}

void ref_sbs_sizes(void *p, SdfSBSHeader *hdr, uint32_t *n_nodes, uint32_t *n_values, uint32_t *n_values_f) {
  const RefSbs *s = static_cast<RefSbs *>(p);
  *hdr = s->header;
  *n_nodes = uint32_t(s->nodes.size());
  *n_values = uint32_t(s->values.size());
  *n_values_f = uint32_t(s->values_f.size());
}
void ref_sbs_copy(void *p, SdfSBSNode *nodes, uint32_t *values, float *values_f) {
  const RefSbs *s = static_cast<RefSbs *>(p);
  std::memcpy(nodes, s->nodes.data(), s->nodes.size() * sizeof(SdfSBSNode));
  std::memcpy(values, s->values.data(), s->values.size() * 4);
  if (!s->values_f.empty()) std::memcpy(values_f, s->values_f.data(), s->values_f.size() * 4);
}
void ref_sbs_free(void *p) { delete static_cast<RefSbs *>(p); }

// The differentiable renderer's settings a test varies; the rest stay at
// getDefaultPresetDR (diff_render/MultiRendererDR.h:9-75).
struct RefDrSettings {
  uint32_t render_mode, reconstruction_flags, loss_function, input_type, border_sampling, raycasting_mask;
  uint32_t spp, border_spp, iterations, image_batch_size, reg_function, redistancing_enable;
  float border_relax_eps, lr, reg_lambda, reg_power;
};

// MultiRendererDR::OptimizeFixedStructure (diff_render/MultiRendererDR.cpp:278-576)
// on an indexed SBS with the caller's BVH2, reference images and cameras, with
// setSeed(seed) and one thread.  Outputs: the parameters after the last Adam
// step, getLastdLoss_dS (the last iteration's gradient as handed to Adam) and
// the last rendered image of every view.
void ref_dr_optimize(const SdfSBSHeader *hdr, const SdfSBSNode *nodes, uint32_t n_nodes, const uint32_t *values,
                     uint32_t n_values, const float *values_f, uint32_t n_values_f, const BVHNodePair *pairs,
                     uint32_t n_pairs, uint32_t n_views, uint32_t width, uint32_t height, const float *images,
                     const float *world_view, const float *proj, const RefDrSettings *st, uint32_t seed,
                     float *out_values_f, float *out_grad, float *out_images) {
  g_next_pairs.assign(pairs, pairs + n_pairs);
  omp_set_num_threads(1);   // one gradient slice, pixels in the packed order: reproducible sums
  dr::MultiRendererDR R;
  R.setSeed(seed);
  std::vector<LiteImage::Image2D<float4>> imgs;
  std::vector<float4x4> wv, pj;
  for (uint32_t v = 0; v < n_views; v++) {
    LiteImage::Image2D<float4> im(width, height);
    std::memcpy(im.data(), images + size_t(v) * width * height * 4, size_t(width) * height * 16);
    imgs.push_back(im);
    wv.push_back(float4x4(world_view + 16 * v));
    pj.push_back(float4x4(proj + 16 * v));
  }
  R.SetReference(imgs, wv, pj);
  dr::MultiRendererDRPreset p = dr::getDefaultPresetDR();
  p.dr_render_mode = st->render_mode;
  p.dr_reconstruction_flags = st->reconstruction_flags;
  p.dr_loss_function = st->loss_function;
  p.dr_input_type = st->input_type;
  p.dr_border_sampling = st->border_sampling;
  p.dr_raycasting_mask = st->raycasting_mask;
  p.spp = st->spp;
  p.border_spp = st->border_spp;
  p.border_relax_eps = st->border_relax_eps;
  p.opt_lr = st->lr;
  p.opt_iterations = st->iterations;
  p.image_batch_size = st->image_batch_size;
  p.reg_function = st->reg_function;
  p.reg_lambda = st->reg_lambda;
  p.reg_power = st->reg_power;
  p.redistancing_enable = st->redistancing_enable != 0;
  p.debug_print = false;
  SdfSBS sbs;
  sbs.header = *hdr;
  sbs.nodes.assign(nodes, nodes + n_nodes);
  sbs.values.assign(values, values + n_values);
  sbs.values_f.assign(values_f, values_f + n_values_f);
  R.OptimizeFixedStructure(p, sbs);
  std::memcpy(out_values_f, sbs.values_f.data(), sbs.values_f.size() * 4);
  std::memcpy(out_grad, R.getLastdLoss_dS(), size_t(n_values_f) * 4);
  for (uint32_t v = 0; v < n_views; v++)
    std::memcpy(out_images + size_t(v) * width * height * 4, R.getLastImage(v).data(), size_t(width) * height * 16);
}

// MultiRenderer::RenderFloat (Renderer/eye_ray_host.cpp:575-585 -> CastRayFloatSingle,
// Renderer/eye_ray.cpp:118-142, one thread) of a DX-layout SBS with the caller's
// BVH2: the spp loop with the regular grid or RAY_GEN_MODE_RANDOM's rand2 offsets
// (setSeed(seed)), kernel_InitEyeRay, RayQuery_NearestHit and kernel_RayTrace's
// geometric modes (MASK, DEPTH, LINEAR_DEPTH, NORMAL: no textures are sampled).
void ref_render_float(const SdfSBSHeader *hdr, const SdfSBSNode *nodes, uint32_t n_nodes, const uint32_t *values,
                      uint32_t n_values, const BVHNodePair *pairs, uint32_t n_pairs, uint32_t width, uint32_t height,
                      const float *world_view, const float *proj, uint32_t render_mode, uint32_t intersect,
                      uint32_t spp, uint32_t ray_gen_mode, uint32_t seed, float *out_rgba) {
  g_next_pairs.assign(pairs, pairs + n_pairs);
  omp_set_num_threads(1);
  MultiRenderer R(10000000);
  R.SetAccelStruct(std::make_shared<BVHRT>());
  MultiRenderPreset p = getDefaultPreset();
  p.render_mode = render_mode;
  p.sdf_node_intersect = intersect;
  p.spp = spp;
  p.ray_gen_mode = ray_gen_mode;
  R.SetPreset(p);
  SdfSBSView view;
  view.header = *hdr;
  view.size = n_nodes;
  view.nodes = nodes;
  view.values_count = n_values;
  view.values = values;
  view.values_f_count = 0;
  view.values_f = nullptr;
  R.SetScene(view);
  R.setSeed(seed);
  R.RenderFloat(reinterpret_cast<float4 *>(out_rgba), width, height, float4x4(world_view), float4x4(proj), p, 1);
}

// MultiRendererDR::OptimizeStepAdam (diff_render/MultiRendererDR.cpp:828-853) on
// the caller's arrays: state holds V then S (2n floats).
struct AdamProbe : dr::MultiRendererDR {
  void step(unsigned iter, const float *g, float *x, float *state, unsigned n, dr::MultiRendererDRPreset p) {
    OptimizeStepAdam(iter, g, x, state, n, p);
  }
};
void ref_dr_adam(uint32_t iter, const float *g, float *x, float *state, uint32_t n, float lr, float b1, float b2,
                 float eps) {
  AdamProbe a;
  dr::MultiRendererDRPreset p = dr::getDefaultPresetDR();
  p.opt_lr = lr;
  p.opt_beta_1 = b1;
  p.opt_beta_2 = b2;
  p.opt_eps = eps;
  a.step(iter, g, x, state, n, p);
}

}  // extern "C"
