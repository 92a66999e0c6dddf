// Driver around the reference's own BVH/BVH2Common.cpp, compiled in place
// (oracle pinning only; built by oracle/build_ref.py into oracle/_ref/ where the
// reference tree is present).  It fills BVHRT's flat arrays the way
// AddGeom_SdfSBS / AddGeom_SdfSVS / AddGeom_Triangles3f + AddInstance +
// CommitScene do (BVH/BVH2Common_host.cpp:205-280, 502-666, 1416-1487), from
// data and a BVH2 supplied by the caller, then answers ray queries with the
// reference's BVHRT::RayQuery_NearestHit and eye rays with render_common.h.
// BVHRT members that live in the host TU and are off the ray-query path
// (geometry adders, builders, SDF-grid evaluation) are stubs here.
#include <new>
#include <vector>

#include "BVH/BVH2Common.h"
#include "diff_render/BVH2DR.h"
#include "render_common.h"

// ---- off-path members of BVHRT (BVH/BVH2Common_host.cpp), stubbed ----
void BVHRT::ClearGeom() {}
uint32_t BVHRT::AddCustomGeom_FromFile(const char *, const char *, ISceneObject *) { return 0; }
uint32_t BVHRT::AddGeom_Triangles3f(const float *, size_t, const uint32_t *, size_t, uint32_t, size_t) { return 0; }
void BVHRT::UpdateGeom_Triangles3f(uint32_t, const float *, size_t, const uint32_t *, size_t, uint32_t, size_t) {}
uint32_t BVHRT::AddGeom_AABB(uint32_t, const CRT_AABB *, size_t, void **, size_t) { return 0; }
void BVHRT::UpdateGeom_AABB(uint32_t, uint32_t, const CRT_AABB *, size_t, void **, size_t) {}
float BVHRT::eval_distance(float3) { return 0.0f; }
void BVHRT::init(SdfGridView) {}
void BVHRT::ClearScene() {}
void BVHRT::CommitScene(uint32_t) {}
uint32_t BVHRT::AddInstance(uint32_t, const float4x4 &) { return 0; }
void BVHRT::UpdateInstance(uint32_t, const float4x4 &) {}
void BVHRT::AppendTreeData(const std::vector<BVHNodePair> &, const std::vector<uint32_t> &, const uint32_t *, size_t) {}

namespace {
struct RefScene {
  dr::BVHDR rt;   // BVHDR adds only non-virtual gradient queries to BVHRT
};

template <typename T>
void place_object(BVHRT &rt) {
  rt.m_abstractObjects.resize(1);
  new (rt.m_abstractObjects.data()) T();   // the way BVHRT::AddGeom_* creates them
  rt.m_abstractObjects[0].geomId = 0;
  rt.m_abstractObjectPtrs.assign(1, rt.m_abstractObjects.data());
}

void finish(BVHRT &rt, const BVHNodePair *pairs, uint32_t n_pairs, float4 gmin, float4 gmax, uint32_t type,
            const MultiRenderPreset &preset) {
  rt.m_allNodePairs.assign(pairs, pairs + n_pairs);
  GeomData gd;
  gd.boxMin = gmin;
  gd.boxMax = gmax;
  gd.bvhOffset = 0;
  gd.type = type;
  gd.offset = uint2(0, 0);
  rt.m_geomData.assign(1, gd);
  InstanceData inst;
  std::memset(&inst, 0, sizeof(inst));
  inst.boxMin = gmin;
  inst.boxMax = gmax;
  inst.geomId = 0;
  inst.transform = float4x4();
  inst.transformInv = float4x4();
  inst.transformInvTransposed = float4x4();
  rt.m_instanceData.assign(1, inst);
  BVHNode tlas;
  tlas.boxMin = to_float3(gmin);
  tlas.boxMax = to_float3(gmax);
  tlas.leftOffset = LEAF_BIT;
  tlas.escapeIndex = LEAF_NORMAL;
  rt.m_nodesTLAS.assign(1, tlas);
  rt.SetPreset(preset);
}
}  // namespace

extern "C" {

// SBS geometry (AddGeom_SdfSBS, single SBS: roots 0, data offsets as given).
void *ref_make_sbs(const SdfSBSHeader *hdr, const SdfSBSNode *nodes, uint32_t n_nodes, const uint32_t *values,
                   uint32_t n_values, const float *values_f, uint32_t n_values_f, const BVHNodePair *pairs,
                   uint32_t n_pairs, const MultiRenderPreset *preset) {
  RefScene *s = new RefScene();
  BVHRT &rt = s->rt;
  const uint32_t layout = hdr->aux_data & SDF_SBS_NODE_LAYOUT_MASK;
  uint32_t type = TYPE_SDF_SBS;   // BVH/BVH2Common_host.cpp:572-592
  if (layout == SDF_SBS_NODE_LAYOUT_DX_UV16)
    type = TYPE_SDF_SBS_TEX;
  else if (layout == SDF_SBS_NODE_LAYOUT_DX_RGB8 || layout == SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F ||
           layout == SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F_IN)
    type = TYPE_SDF_SBS_COL;
  place_object<GeomDataSdfBrick>(rt);
  rt.m_SdfSBSRoots.assign(1, 0u);
  rt.m_SdfSBSHeaders.assign(1, *hdr);
  rt.m_SdfSBSNodes.assign(nodes, nodes + n_nodes);
  rt.m_SdfSBSData.assign(values, values + n_values);
  if (values_f) rt.m_SdfSBSDataF.assign(values_f, values_f + n_values_f);
  rt.m_primIdCount.resize(n_nodes);
  for (uint32_t i = 0; i < n_nodes; i++) rt.m_primIdCount[i] = i;
  rt.startEnd.assign(1, uint2(0, n_nodes));
  finish(rt, pairs, n_pairs, float4(-1, -1, -1, 1), float4(1, 1, 1, 1), type, *preset);
  return s;
}

// SVS geometry (AddGeom_SdfSVS).
void *ref_make_svs(const SdfSVSNode *nodes, uint32_t n_nodes, const BVHNodePair *pairs, uint32_t n_pairs,
                   const MultiRenderPreset *preset) {
  RefScene *s = new RefScene();
  BVHRT &rt = s->rt;
  place_object<GeomDataSdfNode>(rt);
  rt.m_SdfSVSRoots.assign(1, 0u);
  rt.m_SdfSVSNodes.assign(nodes, nodes + n_nodes);
  rt.m_primIdCount.resize(n_nodes);
  for (uint32_t i = 0; i < n_nodes; i++) rt.m_primIdCount[i] = i;
  rt.startEnd.assign(1, uint2(0, n_nodes));
  finish(rt, pairs, n_pairs, float4(-1, -1, -1, 1), float4(1, 1, 1, 1), TYPE_SDF_SVS, *preset);
  return s;
}

// Triangles (AddGeom_Triangles3f + AppendTreeData): vertices as float4, the
// triangle order of the BVH leaves, per-leaf PackOffsetAndSize(start, count).
void *ref_make_tris(const float *vpos4, uint32_t n_vert, const uint32_t *indices, uint32_t n_tris,
                    const uint32_t *order, const uint32_t *leaf_start_count, uint32_t n_leaves,
                    const BVHNodePair *pairs, uint32_t n_pairs, const MultiRenderPreset *preset) {
  RefScene *s = new RefScene();
  BVHRT &rt = s->rt;
  place_object<GeomDataTriangle>(rt);
  Box4f bbox;
  rt.m_vertPos.resize(n_vert);
  rt.m_vertNorm.assign(n_vert, float4(1, 0, 0, 1));
  for (uint32_t i = 0; i < n_vert; i++) {
    rt.m_vertPos[i] = float4(vpos4[4 * i], vpos4[4 * i + 1], vpos4[4 * i + 2], 1.0f);
    bbox.include(rt.m_vertPos[i]);
  }
  rt.m_primIndices.assign(order, order + n_tris);
  rt.m_indices.resize(size_t(n_tris) * 3);
  for (uint32_t i = 0; i < n_tris; i++)
    for (int k = 0; k < 3; k++) rt.m_indices[3 * size_t(i) + k] = indices[3 * size_t(order[i]) + k];
  rt.m_primIdCount.assign(leaf_start_count, leaf_start_count + n_leaves);
  rt.startEnd.assign(1, uint2(0, n_leaves));
  finish(rt, pairs, n_pairs, bbox.boxMin, bbox.boxMax, TYPE_MESH_TRIANGLE, *preset);
  return s;
}

void ref_free(void *p) { delete static_cast<RefScene *>(p); }

// BVHRT::RayQuery_NearestHit on n rays (float4 pos+tNear, float4 dir+tFar).
void ref_query(void *p, const float *pos_near, const float *dir_far, uint32_t n, CRT_Hit *out) {
  BVHRT &rt = static_cast<RefScene *>(p)->rt;
  for (uint32_t i = 0; i < n; i++) {
    const float *a = pos_near + 4 * size_t(i), *b = dir_far + 4 * size_t(i);
    out[i] = rt.RayQuery_NearestHit(float4(a[0], a[1], a[2], a[3]), float4(b[0], b[1], b[2], b[3]));
  }
}

// dr::BVHDR::RayQuery_NearestHitWithGrad (diff_render/BVH2DR.cpp:12-102) on n
// rays with the given DR_RAY_FLAG_* bits.  Each ray writes one flat record of
// 576 32-bit words: [0,14) the hit, [14,28) payload.missed_hit (each as t,
// primId, instId, geomId, color.xyz, sdf, normal.xyz, check_vox_border),
// [28,36) missed_indices, [36,44) missed_dSDF_dtheta, [44,60) dDiffuse_dSc as
// (index, value) pairs, [60,572) dDiffuseNormal_dSd as (dDiffuse.xyz, index,
// dNorm.xyz, dDist), [572,576) zero.
static void put_hit(uint32_t *o, const dr::CRT_HitDR &h) {
  std::memcpy(o + 0, &h.t, 4);
  o[1] = h.primId; o[2] = h.instId; o[3] = h.geomId;
  std::memcpy(o + 4, &h.color.x, 4); std::memcpy(o + 5, &h.color.y, 4); std::memcpy(o + 6, &h.color.z, 4);
  std::memcpy(o + 7, &h.sdf, 4);
  std::memcpy(o + 8, &h.normal.x, 4); std::memcpy(o + 9, &h.normal.y, 4); std::memcpy(o + 10, &h.normal.z, 4);
  o[11] = h.check_vox_border;
  o[12] = o[13] = 0;
}

void ref_dr_query(void *p, uint32_t ray_flags, const float *pos_near, const float *dir_far, uint32_t n,
                  uint32_t *out) {
  dr::BVHDR &rt = static_cast<RefScene *>(p)->rt;
  for (uint32_t i = 0; i < n; i++) {
    const float *a = pos_near + 4 * size_t(i), *b = dir_far + 4 * size_t(i);
    dr::RayDiffPayload pl;
    std::memset(&pl, 0, sizeof(pl));
    const dr::CRT_HitDR h = rt.RayQuery_NearestHitWithGrad(ray_flags, float4(a[0], a[1], a[2], a[3]),
                                                           float4(b[0], b[1], b[2], b[3]), &pl);
    uint32_t *o = out + 576 * size_t(i);
    std::memset(o, 0, 576 * 4);
    put_hit(o, h);
    put_hit(o + 14, pl.missed_hit);
    for (int k = 0; k < 8; k++) {
      o[28 + k] = pl.missed_indices[k];
      std::memcpy(o + 36 + k, &pl.missed_dSDF_dtheta[k], 4);
      o[44 + 2 * k] = pl.dDiffuse_dSc[k].index;
      std::memcpy(o + 45 + 2 * k, &pl.dDiffuse_dSc[k].value, 4);
    }
    for (int k = 0; k < 64; k++) {
      const dr::PDDist &d = pl.dDiffuseNormal_dSd[k];
      uint32_t *q = o + 60 + 8 * k;
      std::memcpy(q + 0, &d.dDiffuse.x, 4); std::memcpy(q + 1, &d.dDiffuse.y, 4); std::memcpy(q + 2, &d.dDiffuse.z, 4);
      q[3] = d.index;
      std::memcpy(q + 4, &d.dNorm.x, 4); std::memcpy(q + 5, &d.dNorm.y, 4); std::memcpy(q + 6, &d.dNorm.z, 4);
      std::memcpy(q + 7, &d.dDist, 4);
    }
  }
}

// kernel_InitEyeRay (Renderer/eye_ray.cpp:146-160) with the reference's
// EyeRayDirNormalized and transform_ray3f (render_common.h:25-55).
void ref_eye_rays(uint32_t w, uint32_t h, const float *proj_inv, const float *wv_inv, const uint32_t *pix,
                  uint32_t n, float dx, float dy, float *pos_near, float *dir_far) {
  const float4x4 pi(proj_inv), wi(wv_inv);
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t x = pix[i] % w, y = pix[i] / w;
    float3 rayDir = EyeRayDirNormalized((float(x) + dx) / float(w), (float(y) + dy) / float(h), pi);
    float3 rayPos = float3(0, 0, 0);
    transform_ray3f(wi, &rayPos, &rayDir);
    float *p = pos_near + 4 * size_t(i), *d = dir_far + 4 * size_t(i);
    p[0] = rayPos.x; p[1] = rayPos.y; p[2] = rayPos.z; p[3] = 0.0f;
    d[0] = rayDir.x; d[1] = rayDir.y; d[2] = rayDir.z; d[3] = 1e9f;
  }
}

}  // extern "C"
