// The persistent render kernel compiled with floating-point contraction: every
// a * b + c of the traversal, the leaf finders and the shading is one FMA (a
// single rounding) instead of a product and a sum rounded separately.  Results
// are no longer bit-identical to the reference's x86-64 build (which does not
// contract); they stay within the forward parity tolerance (hit mask, depth
// within 1e-4 of the scene extent, normals within 1e-3, apart from grazing and
// crease pixels).  Selected by the "fma" tuning key for SBS and SVS scenes
// (triangle scenes keep the uncontracted kernel: a contracted edge test can let
// a ray through the crack between two triangles); spp loop, outputs and work
// distribution are those of trace.cu's instantiations.
#include "render_kernel.cuh"
#include "render_lq.cuh"

namespace lrt {

template <int TYPE, int MODE, int STACK>
static cudaError_t launch_fused_m(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e =
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_kernel<TYPE, false, MODE, STACK, 1>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_kernel<TYPE, false, MODE, STACK, 1><<<blocks, 128, 0, st>>>(s, L);
  return cudaGetLastError();
}

template <int TYPE>
static cudaError_t launch_fused_t(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                  const Tuning &tu) {
  switch (s.preset.sdf_node_intersect) {
    case LRT_INTERSECT_NEWTON:
      if (TYPE == LRT_TYPE_SDF_SBS && tu.stack == 32)
        return launch_fused_m<TYPE, LRT_INTERSECT_NEWTON, 32>(s, L, num_sms, st);
      return launch_fused_m<TYPE, LRT_INTERSECT_NEWTON, kStackSize>(s, L, num_sms, st);
    case LRT_INTERSECT_ST: return launch_fused_m<TYPE, LRT_INTERSECT_ST, kStackSize>(s, L, num_sms, st);
    default: return launch_fused_m<TYPE, -1, kStackSize>(s, L, num_sms, st);
  }
}

template <int MODE, int STACK>
static cudaError_t launch_lq_m1(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_lq_kernel<MODE, STACK, 1>,
                                                                dev::kLqThreads, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_lq_kernel<MODE, STACK, 1><<<blocks, dev::kLqThreads, 0, st>>>(s, L);
  return cudaGetLastError();
}

// variant 3: traversal and leaf phases regrouped across the block (render_lq.cuh)
cudaError_t launch_render_lq_fused(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                              const Tuning &tu) {
  switch (s.preset.sdf_node_intersect) {
    case LRT_INTERSECT_NEWTON:
      if (tu.stack == 32) return launch_lq_m1<LRT_INTERSECT_NEWTON, 32>(s, L, num_sms, st);
      return launch_lq_m1<LRT_INTERSECT_NEWTON, kStackSize>(s, L, num_sms, st);
    case LRT_INTERSECT_ST: return launch_lq_m1<LRT_INTERSECT_ST, kStackSize>(s, L, num_sms, st);
    default: return launch_lq_m1<-1, kStackSize>(s, L, num_sms, st);
  }
}

cudaError_t launch_render_fused(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                const Tuning &tu) {
  switch (s.type) {
    case LRT_TYPE_SDF_SVS: return launch_fused_t<LRT_TYPE_SDF_SVS>(s, L, num_sms, st, tu);
    default: return launch_fused_t<LRT_TYPE_SDF_SBS>(s, L, num_sms, st, tu);
  }
}

}  // namespace lrt
