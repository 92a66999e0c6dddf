// Device-side state of the learned proposal (proposal.cu), shared with the host
// driver (proposal_api.cpp).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "lrt_internal.h"

namespace lrt {

// Training triples: 16 bf16 features and the crossing fraction per sample.
// Features are stored in tiles of 128 samples, 4 KB each: the 16-byte halves
// holding features 0-7 of the tile's 128 samples, then the halves holding
// features 8-15.  One 4 KB bulk copy of a tile is then the tcgen05 A operand
// in the no-swizzle K-major layout (8-row x 16-byte core matrices, 16 bytes
// between rows, 2 KB between the two K halves).  Index of a half in 16-byte
// units:
__host__ __device__ inline uint64_t feat_u4(uint64_t row, uint32_t half) {
  return (row >> 7) * 256u + uint64_t(half) * 128u + (row & 127u);
}
// bf16 elements a store of n samples occupies (whole tiles)
__host__ __device__ inline uint64_t feat_elems(uint64_t n) { return ((n + 127u) >> 7) * 2048u; }

struct TripleBuf {
  __nv_bfloat16 *feat;
  float *target;
  unsigned long long *count;   // samples written (may exceed capacity: extra ones are dropped)
  unsigned long long capacity;
};
// Samples [first, first + n) of a store (feat and target point at the store's start).
struct TripleView {
  const __nv_bfloat16 *feat;
  const float *target;
  uint64_t first, n;
};

// Network parameters and optimiser state (device).
struct MlpState {
  float *master;            // 1633 FP32 parameters
  __nv_bfloat16 *wbf;       // BF16 weight image (W1 | W2 | W3 padded to 8 rows)
  float *grad;              // gradient accumulator
  float *adam_m, *adam_v;
  unsigned int *ticket;     // blocks finished in the current step
  float *loss;              // where a step adds its mean loss (may be null)
};

cudaError_t launch_gen_triples(const DevScene &s, const DevView *views, uint32_t n_views, uint64_t total_pix,
                               const TripleBuf &out, uint32_t target, cudaStream_t st);
cudaError_t launch_mlp_step(const TripleView &data, const MlpState &m, uint32_t batch, uint32_t step, uint32_t seed,
                            bool random, bool update, float lr, float b1, float b2, float eps, cudaStream_t st);
cudaError_t launch_mlp_infer(const TripleView &data, const MlpState &m, float *out, cudaStream_t st);
cudaError_t launch_mlp_infer_tc(const TripleView &data, const MlpState &m, float *out, unsigned int *status,
                                cudaStream_t st,
                                uint32_t wait_limit);
cudaError_t launch_render_proposal(const DevScene &s, const RenderLaunch &L, const MlpState &m,
                                   unsigned long long *stats, int num_sms, cudaStream_t st);

}  // namespace lrt
