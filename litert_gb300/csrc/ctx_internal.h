// Host-side context of the C ABI (lrt_ctx) and its helpers, shared by the
// ray-query driver (lrt_api.cpp) and the differentiable-render driver
// (dr_api.cpp).  Host code only.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lrt_internal.h"

namespace lrt {
struct DrState;
void dr_state_free(DrState *st);
struct ProposalState;
void proposal_state_free(ProposalState *st);
// the batched render launch of the context's kernel choice (plain or proposal)
cudaError_t dispatch_render(struct ::lrt_ctx *ctx, const RenderLaunch &L, cudaStream_t st, bool count);
// whether that launch (without counters) counts finished tiles in RenderLaunch::chunk_done
bool dispatch_publishes_chunks(const struct ::lrt_ctx *ctx, bool color, uint32_t total_tiles);
}  // namespace lrt

namespace lrt {

// Host-side fault injection for the failure-path tests: while the environment
// variable LRT_INJECT_FAULT names a site ("alloc": device buffer allocation,
// "upload": host-to-device scene upload, "graph": CUDA-graph instantiation), every
// call through that site fails as the CUDA runtime would (cudaErrorMemoryAllocation
// / cudaErrorInvalidValue), before any device work.  Read on each call (cold
// paths only); unset, it costs one getenv.
inline bool inject_fault(const char *site) {
  const char *v = std::getenv("LRT_INJECT_FAULT");
  return v && std::strcmp(v, site) == 0;
}

struct Geom {
  uint32_t type = 0;
  SbsData sbs;
  std::vector<float> values_f;
  std::vector<lrt_svs_node> svs;
  std::vector<float> vpos;        // float4 per vertex
  std::vector<uint32_t> indices;  // 3 per triangle
  float bmin[3] = {-1, -1, -1}, bmax[3] = {1, 1, 1};
};

struct Inst {
  uint32_t geom = 0;
  float m[16], inv[16], inv_t[16];
  float bmin[3], bmax[3];
};

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t cap = 0;  // elements
  cudaError_t ensure(size_t n) {
    if (n <= cap) return cudaSuccess;
    if (inject_fault("alloc")) return cudaErrorMemoryAllocation;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) cap = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

}  // namespace lrt

using namespace lrt;   // internal header: the context is built from lrt:: types

struct lrt_ctx {
  int device = 0;
  int num_sms = 0;
  std::string err;
  std::vector<Geom> geoms;
  std::vector<Inst> insts;
  lrt_preset preset{};
  bool committed = false;
  DevScene dev{};
  BvhData bvh;
  // committed scene buffers
  DevBuf<WNode4> d_nodes;
  DevBuf<lrt_sbs_node> d_bricks;
  DevBuf<float4> d_leaf_boxes;
  DevBuf<uint32_t> d_occ;
  DevBuf<uint32_t> d_values;
  DevBuf<float> d_values_f;
  DevBuf<lrt_svs_node> d_svs;
  DevBuf<float4> d_tri_verts;
  DevBuf<uint32_t> d_prim_indices;
  // BVH built on the device (bvh_builder = 1) and triangle refit
  DevBuf<float> d_boxes6;              // primitive boxes (build input / refit scratch)
  DevBuf<lrt_bvh_pair> d_pairs;        // reference fat-pair layout of a device-built BVH
  DevBuf<uint32_t> d_leaf_start_count;
  DevBuf<float4> d_vpos;               // mesh vertices (refit)
  DevBuf<uint32_t> d_tri_indices;      // mesh indices (refit)
  int bvh_builder = 0;                 // 0: host binned SAH, 1: device linear BVH
  bool bvh_on_device = false;          // the committed BVH was built on the device
  bool bvh_refit = false;              // slot boxes refit since the commit (fat pairs not refit)
  bool tri_indices_on_device = false;
  uint32_t n_wnodes = 0, n_pairs = 0, n_leaf_start_count = 0;
  // per-call scratch
  DevBuf<uint32_t> d_tile_counter;
  DevBuf<DevView> d_views;
  DevBuf<unsigned long long> d_counters;
  DevView *h_views = nullptr;  // pinned staging for view uploads
  size_t h_views_cap = 0;
  // output chunks of the last prepared batch (whole tile rows of one view each):
  // the tiles that make a chunk and its pixel range in the batched outputs
  struct Chunk {
    uint32_t tiles;
    uint64_t first_pixel, end_pixel;
  };
  std::vector<Chunk> chunks;
  size_t chunk_copy_end = 0;   // chunks from here on are written to the host by the kernel
  DevBuf<uint32_t> d_chunk_done;
  cudaStream_t copy_stream = nullptr;   // lrt_render_host's chunk copies (non-blocking)
  cudaEvent_t chunks_zeroed = nullptr;  // chunk counts cleared on the render stream
  cudaEvent_t render_done = nullptr;    // the render and the counts' release
  // host-buffer entry points
  DevBuf<lrt_hit16> d_out_hits;
  DevBuf<float4> d_out_rgba;
  DevBuf<uint32_t> d_out_rgba8;
  DevBuf<float4> d_q_pos, d_q_dir;
  DevBuf<lrt_hit> d_q_out;
  uint32_t last_launches = 0;
  uint32_t brick_stride = 0;   // device words per brick (16-byte multiple)
  Tuning tuning;
  lrt::DrState *dr = nullptr;  // differentiable-render state (dr_api.cpp)
  lrt::ProposalState *prop = nullptr;   // learned proposal (proposal_api.cpp)
  int use_proposal = 0;        // render SBS leaves with the proposal kernel
  uint32_t seed = 0;           // MultiRenderer::setSeed
  // the BVH2 of the first-hit walk ("first_hit" tuning): checked and uploaded on
  // first use, or given by the caller (lrt_set_bvh2); reset by a commit
  DevBuf<lrt_bvh_pair> d_ref_pairs;
  DevBuf<DevInst> d_insts;     // all instances, when the scene has several
  bool ref_pairs_ready = false;
};

static inline lrt_status fail(lrt_ctx *ctx, lrt_status s, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return s;
}

static inline lrt_status cuda_fail(lrt_ctx *ctx, cudaError_t e, const char *where) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? LRT_ERR_OOM : LRT_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

#define LRT_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);  \
  } while (0)

