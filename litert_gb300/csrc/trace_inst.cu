// Renders and batched queries of a scene holding several instances of its
// geometry (the TLAS of RayQuery_NearestHit, BVH/BVH2Common.cpp:3508-3547):
// the render and query kernels of trace.cu / trace_ref.cu instantiated with
// FEAT bit 3, which walks every instance whose box the ray enters, in instance
// order, each in its own object space, with the closest hit so far, and shades
// the hit in the frame of the instance it belongs to.  The finder mode is read
// at run time here (these kernels are not the benchmark's), uncontracted
// arithmetic as in trace.cu.
#include "render_kernel.cuh"

namespace lrt {

template <int TYPE, bool PHONG, int FEAT>
static cudaError_t launch_inst_m(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, dev::render_kernel<TYPE, false, -1, kStackSize, 0, PHONG, FEAT | 8>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_kernel<TYPE, false, -1, kStackSize, 0, PHONG, FEAT | 8><<<blocks, 128, 0, st>>>(s, L);
  return cudaGetLastError();
}

template <bool PHONG>
static cudaError_t launch_inst_p(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                 bool first_hit) {
  switch (s.type) {
    case LRT_TYPE_MESH_TRIANGLE: return launch_inst_m<LRT_TYPE_MESH_TRIANGLE, PHONG, 0>(s, L, num_sms, st);
    case LRT_TYPE_SDF_SVS:
      return first_hit ? launch_inst_m<LRT_TYPE_SDF_SVS, PHONG, 4>(s, L, num_sms, st)
                       : launch_inst_m<LRT_TYPE_SDF_SVS, PHONG, 0>(s, L, num_sms, st);
    default:
      if (render_features(s) == 1)
        return first_hit ? launch_inst_m<LRT_TYPE_SDF_SBS, PHONG, 5>(s, L, num_sms, st)
                         : launch_inst_m<LRT_TYPE_SDF_SBS, PHONG, 1>(s, L, num_sms, st);
      return first_hit ? launch_inst_m<LRT_TYPE_SDF_SBS, PHONG, 4>(s, L, num_sms, st)
                       : launch_inst_m<LRT_TYPE_SDF_SBS, PHONG, 0>(s, L, num_sms, st);
  }
}

cudaError_t launch_render_inst(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool first_hit) {
  if (!s.insts || s.n_inst == 0 || (first_hit && !s.pairs) || render_features(s) == 2) return cudaErrorInvalidValue;
  const uint32_t rm = s.preset.render_mode;
  const bool phong = (rm == LRT_RENDER_MODE_PHONG || rm == LRT_RENDER_MODE_PHONG_NO_TEX) && (L.rgba || L.rgba8);
  return phong ? launch_inst_p<true>(s, L, num_sms, st, first_hit) : launch_inst_p<false>(s, L, num_sms, st, first_hit);
}

cudaError_t launch_query_inst(const DevScene &s, const float4 *pos_near, const float4 *dir_far, uint32_t n,
                              lrt_hit *out, cudaStream_t st, bool first_hit) {
  if (!s.insts || s.n_inst == 0 || (first_hit && !s.pairs) || render_features(s) == 2) return cudaErrorInvalidValue;
  if (n == 0) return cudaSuccess;
  const uint32_t blocks = (n + 127) / 128;
  switch (s.type) {
    case LRT_TYPE_MESH_TRIANGLE:
      dev::query_kernel<LRT_TYPE_MESH_TRIANGLE, 8><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out);
      break;
    case LRT_TYPE_SDF_SVS:
      if (first_hit) dev::query_kernel<LRT_TYPE_SDF_SVS, 12><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out);
      else dev::query_kernel<LRT_TYPE_SDF_SVS, 8><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out);
      break;
    default:
      if (render_features(s) == 1) {
        if (first_hit) dev::query_kernel<LRT_TYPE_SDF_SBS, 13><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out);
        else dev::query_kernel<LRT_TYPE_SDF_SBS, 9><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out);
      } else {
        if (first_hit) dev::query_kernel<LRT_TYPE_SDF_SBS, 12><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out);
        else dev::query_kernel<LRT_TYPE_SDF_SBS, 8><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out);
      }
      break;
  }
  return cudaGetLastError();
}

}  // namespace lrt
