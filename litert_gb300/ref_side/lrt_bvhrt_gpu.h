// The reference-side binding of the lrt C ABI: what a LiteRT maintainer adds to
// the reference tree to run its ray-query path on this engine.
//
//   BVHRT_GPU         an ISceneObject (the CrossRT interface BVHRT implements,
//                     BVH/BVH2Common.h:100-173) whose every member forwards to
//                     include/lrt_gpu.h, plus BVHRT's non-virtual SDF adders
//                     (AddGeom_SdfSBS / AddGeom_SdfSVS) and a batched query.
//   MultiRendererGPU  a MultiRenderer (Renderer/eye_ray.h:77-250) whose pixel
//                     loops (CastRaySingleBlock / CastRayFloatSingleBlock, the
//                     virtual members Render / RenderFloat end in,
//                     Renderer/eye_ray_host.cpp:247-282) render the whole image in
//                     one launch through lrt_render_host, with the renderer's
//                     camera, preset and seed.
//
// Header-only: include it after the reference's BVH/BVH2Common.h and
// Renderer/eye_ray.h and link liblrt_gb300.so.  Errors of the engine are kept in
// last_error() (the reference's interface has no error channel: a failed query
// returns a miss, a failed render leaves the image untouched).
#pragma once
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "lrt_gpu.h"

class BVHRT_GPU : public ISceneObject {
 public:
  explicit BVHRT_GPU(int device = 0) {
    if (lrt_create(&m_ctx, device) != LRT_OK) m_err = "lrt_create failed (no usable GPU)";
  }
  ~BVHRT_GPU() override {
    if (m_ctx) lrt_destroy(m_ctx);
  }
  BVHRT_GPU(const BVHRT_GPU &) = delete;
  BVHRT_GPU &operator=(const BVHRT_GPU &) = delete;

  bool ok() const { return m_ctx != nullptr; }
  const std::string &last_error() const { return m_err; }
  lrt_ctx *context() { return m_ctx; }

  const char *Name() const override { return "BVHRT_GPU"; }
  ISceneObject *UnderlyingImpl(uint32_t) override { return this; }

  void ClearGeom() override { check(lrt_clear_geom(m_ctx)); }
  uint32_t AddCustomGeom_FromFile(const char *, const char *, ISceneObject *) override {
    m_err = "AddCustomGeom_FromFile: custom geometry files are outside this path";
    return kBad;
  }
  uint32_t AddGeom_Triangles3f(const float *vpos, size_t n_vert, const uint32_t *idx, size_t n_idx, uint32_t,
                               size_t stride) override {
    uint32_t id = kBad;
    check(lrt_add_triangles(m_ctx, vpos, n_vert, stride, idx, n_idx, &id));
    return id;
  }
  void UpdateGeom_Triangles3f(uint32_t geom, const float *vpos, size_t n_vert, const uint32_t *idx, size_t n_idx,
                              uint32_t, size_t stride) override {
    check(lrt_update_geom_triangles(m_ctx, geom, vpos, n_vert, idx, n_idx, stride));
  }
  uint32_t AddGeom_AABB(uint32_t type, const CRT_AABB *boxes, size_t n, void **, size_t) override {
    uint32_t id = kBad;
    check(lrt_add_aabb(m_ctx, type, reinterpret_cast<const float *>(boxes), n, &id));
    return id;
  }
  void UpdateGeom_AABB(uint32_t, uint32_t, const CRT_AABB *, size_t, void **, size_t) override {
    m_err = "UpdateGeom_AABB: not supported (the reference leaves it unimplemented)";
  }
  void ClearScene() override { check(lrt_clear_scene(m_ctx)); }
  void CommitScene(uint32_t = BUILD_HIGH) override { check(lrt_commit_scene(m_ctx)); }
  uint32_t AddInstance(uint32_t geom, const LiteMath::float4x4 &m) override {
    float a[16];
    rows(m, a);
    uint32_t id = kBad;
    check(lrt_add_instance(m_ctx, geom, a, &id));
    return id;
  }
  uint32_t AddInstanceMotion(uint32_t geom, const LiteMath::float4x4 *ms, uint32_t) override {
    return AddInstance(geom, ms[0]);   // as BVHRT does (BVH/BVH2Common.h:162-163)
  }
  void UpdateInstance(uint32_t inst, const LiteMath::float4x4 &m) override {
    float a[16];
    rows(m, a);
    check(lrt_update_instance(m_ctx, inst, a));
  }

  // One ray: a host round trip per call.  Callers with many rays use the batch below.
  CRT_Hit RayQuery_NearestHit(LiteMath::float4 pos_near, LiteMath::float4 dir_far) override {
    CRT_Hit h;
    RayQuery_NearestHitBatch(&pos_near, &dir_far, 1, &h);
    return h;
  }
  CRT_Hit RayQuery_NearestHitMotion(LiteMath::float4 p, LiteMath::float4 d, float) override {
    return RayQuery_NearestHit(p, d);
  }
  bool RayQuery_AnyHit(LiteMath::float4 p, LiteMath::float4 d) override {   // :3561-3566
    d.w *= -1.0f;
    return RayQuery_NearestHit(p, d).geomId != uint32_t(-1);
  }
  bool RayQuery_AnyHitMotion(LiteMath::float4 p, LiteMath::float4 d, float) override { return RayQuery_AnyHit(p, d); }

  // n rays in one launch (lrt_query_rays on host arrays); a failure returns misses.
  void RayQuery_NearestHitBatch(const LiteMath::float4 *pos_near, const LiteMath::float4 *dir_far, uint32_t n,
                                CRT_Hit *out) {
    static_assert(sizeof(CRT_Hit) == sizeof(lrt_hit), "CRT_Hit and lrt_hit share their layout");
    std::vector<float> p(4 * size_t(n)), d(4 * size_t(n));
    for (uint32_t i = 0; i < n; i++)
      for (int k = 0; k < 4; k++) {
        p[4 * size_t(i) + k] = pos_near[i][k];
        d[4 * size_t(i) + k] = dir_far[i][k];
      }
    if (!check(lrt_query_rays(m_ctx, p.data(), d.data(), n, reinterpret_cast<lrt_hit *>(out), 0, nullptr)))
      for (uint32_t i = 0; i < n; i++) {
        out[i].t = dir_far[i].w;
        out[i].primId = out[i].instId = out[i].geomId = uint32_t(-1);
        out[i].coords[0] = 1.0f;
        out[i].coords[1] = out[i].coords[2] = out[i].coords[3] = 0.0f;
      }
  }

  // BVHRT's non-virtual SDF adders (BVH/BVH2Common_host.cpp:502-666)
  uint32_t AddGeom_SdfSBS(SdfSBSView v, ISceneObject * = nullptr, BuildOptions = BUILD_HIGH) {
    uint32_t id = kBad;
    check(lrt_add_sbs(m_ctx, reinterpret_cast<const lrt_sbs_header *>(&v.header),
                      reinterpret_cast<const lrt_sbs_node *>(v.nodes), uint32_t(v.size), v.values,
                      uint32_t(v.values_count), v.values_f, uint32_t(v.values_f_count), &id));
    return id;
  }
  uint32_t AddGeom_SdfSVS(SdfSVSView v, ISceneObject * = nullptr, BuildOptions = BUILD_HIGH) {
    uint32_t id = kBad;
    check(lrt_add_svs(m_ctx, reinterpret_cast<const lrt_svs_node *>(v.nodes), uint32_t(v.size), &id));
    return id;
  }
  void SetPreset(const MultiRenderPreset &p) { check(lrt_set_preset(m_ctx, reinterpret_cast<const lrt_preset *>(&p))); }
  // the reference's first-hit result on a given BVH2 (e.g. the pairs its own builder made)
  void SetFirstHit(bool on) { check(lrt_set_tuning(m_ctx, "first_hit", on ? 1 : 0)); }
  void SetBVH2(const BVHNodePair *pairs, uint32_t n) {
    check(lrt_set_bvh2(m_ctx, reinterpret_cast<const lrt_bvh_pair *>(pairs), n));
  }

  static void rows(const LiteMath::float4x4 &m, float a[16]) {
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) a[4 * i + j] = m(i, j);
  }

 private:
  static constexpr uint32_t kBad = 0xFFFFFFFFu;
  bool check(lrt_status s) {
    if (s == LRT_OK) return true;
    m_err = m_ctx ? lrt_last_error(m_ctx) : "no context";
    return false;
  }
  lrt_ctx *m_ctx = nullptr;
  std::string m_err;
};

class MultiRendererGPU : public MultiRenderer {
 public:
  explicit MultiRendererGPU(int device = 0, uint32_t max_primitives = 10'000'000)
      : MultiRenderer(max_primitives), m_gpu(std::make_shared<BVHRT_GPU>(device)) {
    SetAccelStruct(m_gpu);
  }
  BVHRT_GPU &gpu() { return *m_gpu; }

  // SetScene(SdfSBSView / SdfSVSView / mesh), Renderer/eye_ray_host.cpp:297-375,
  // on the GPU scene
  void SetScene(SdfSBSView scene) { commit(m_gpu->AddGeom_SdfSBS(scene)); }
  void SetScene(SdfSVSView scene) { commit(m_gpu->AddGeom_SdfSVS(scene)); }
  void SetScene(const float *vpos4, size_t n_vert, const uint32_t *idx, size_t n_idx) {
    commit(m_gpu->AddGeom_Triangles3f(vpos4, n_vert, idx, n_idx, BUILD_HIGH, 16));
  }

 protected:
  // Render (uint32 RGBA8) and RenderFloat end in these two loops over the packed
  // pixels; here the whole image is one batched launch.
  void CastRaySingleBlock(uint32_t, uint32_t *out_color, uint32_t) override { render(nullptr, out_color); }
  void CastRayFloatSingleBlock(uint32_t, LiteMath::float4 *out_color, uint32_t) override {
    render(reinterpret_cast<float *>(out_color), nullptr);
  }

 private:
  void commit(uint32_t geom) {
    m_gpu->ClearScene();
    m_gpu->AddInstance(geom, LiteMath::float4x4());
    m_gpu->CommitScene();
  }
  void render(float *rgba, uint32_t *rgba8) {
    lrt_view v;
    v.width = m_width;
    v.height = m_height;
    BVHRT_GPU::rows(m_worldView, v.world_view);
    BVHRT_GPU::rows(m_proj, v.proj);
    m_gpu->SetPreset(m_preset);
    lrt_set_seed(m_gpu->context(), m_seed);
    lrt_render_host(m_gpu->context(), &v, 1, nullptr, rgba, rgba8);
  }
  std::shared_ptr<BVHRT_GPU> m_gpu;
};
