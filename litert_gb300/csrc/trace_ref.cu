// Renders and batched queries with the reference's own traversal result: the
// BVH2 fat pairs walked in BVH2TraverseF32's order with its first-hit early-out
// for SDF leaves (BVH/BVH2Common.cpp:3402-3405, 3407-3488), selected by the
// "first_hit" tuning key.  The default kernels return the closest hit, which does
// not depend on the tree; the reference stops at the first SDF leaf that reports
// a hit, which does (where sibling boxes overlap, a farther brick can be reached
// first).  Given the same BVH2 -- the engine's own, or the caller's through
// lrt_set_bvh2 -- these kernels return the reference's records bit for bit.
// Eye rays, leaves, shading and the persistent tile queue are those of
// trace.cu (uncontracted arithmetic).
#include "render_kernel.cuh"

namespace lrt {

template <int TYPE, int MODE, bool PHONG, int FEAT>
static cudaError_t launch_ref_m(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, dev::render_kernel<TYPE, false, MODE, kStackSize, 0, PHONG, FEAT | 4>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_kernel<TYPE, false, MODE, kStackSize, 0, PHONG, FEAT | 4><<<blocks, 128, 0, st>>>(s, L);
  return cudaGetLastError();
}

template <int TYPE, bool PHONG, int FEAT>
static cudaError_t launch_ref_t(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  switch (s.preset.sdf_node_intersect) {
    case LRT_INTERSECT_NEWTON: return launch_ref_m<TYPE, LRT_INTERSECT_NEWTON, PHONG, FEAT>(s, L, num_sms, st);
    case LRT_INTERSECT_ST: return launch_ref_m<TYPE, LRT_INTERSECT_ST, PHONG, FEAT>(s, L, num_sms, st);
    default: return launch_ref_m<TYPE, -1, PHONG, FEAT>(s, L, num_sms, st);
  }
}

cudaError_t launch_render_ref(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  if (!s.pairs || !sdf_scene(s)) return cudaErrorInvalidValue;
  if (s.n_inst > 1) return launch_render_inst(s, L, num_sms, st, true);
  const uint32_t rm = s.preset.render_mode;
  const bool phong = (rm == LRT_RENDER_MODE_PHONG || rm == LRT_RENDER_MODE_PHONG_NO_TEX) && (L.rgba || L.rgba8);
  if (s.type == LRT_TYPE_SDF_SVS)
    return phong ? launch_ref_t<LRT_TYPE_SDF_SVS, true, 0>(s, L, num_sms, st)
                 : launch_ref_t<LRT_TYPE_SDF_SVS, false, 0>(s, L, num_sms, st);
  switch (render_features(s)) {
    case 1:
      return phong ? launch_ref_t<LRT_TYPE_SDF_SBS, true, 1>(s, L, num_sms, st)
                   : launch_ref_t<LRT_TYPE_SDF_SBS, false, 1>(s, L, num_sms, st);
    case 2: return launch_ref_t<LRT_TYPE_SDF_SBS, false, 2>(s, L, num_sms, st);
    default:
      return phong ? launch_ref_t<LRT_TYPE_SDF_SBS, true, 0>(s, L, num_sms, st)
                   : launch_ref_t<LRT_TYPE_SDF_SBS, false, 0>(s, L, num_sms, st);
  }
}

cudaError_t launch_query_ref(const DevScene &s, const float4 *pos_near, const float4 *dir_far, uint32_t n,
                             lrt_hit *out, cudaStream_t st) {
  if (!s.pairs || !sdf_scene(s)) return cudaErrorInvalidValue;
  if (s.n_inst > 1) return launch_query_inst(s, pos_near, dir_far, n, out, st, true);
  if (n == 0) return cudaSuccess;
  const uint32_t blocks = (n + 127) / 128;
  if (s.type == LRT_TYPE_SDF_SVS) {
    dev::query_kernel<LRT_TYPE_SDF_SVS, 4><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out);
  } else {
    switch (render_features(s)) {
      case 1: dev::query_kernel<LRT_TYPE_SDF_SBS, 5><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
      case 2: dev::query_kernel<LRT_TYPE_SDF_SBS, 6><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
      default: dev::query_kernel<LRT_TYPE_SDF_SBS, 4><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
    }
  }
  return cudaGetLastError();
}

}  // namespace lrt
