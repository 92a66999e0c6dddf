/*
 * lrt — learned proposal for the SBS leaf phase, C ABI.
 *
 * A per-(ray, brick) network (16 inputs: the segment's entry and exit in brick
 * units, the brick's 8 corner distances and the segment length in brick edges,
 * the smallest corner distance; two hidden ReLU layers of 32; one output: the
 * crossing's fraction along the segment) with BF16 weights on the tensor cores
 * and FP32 accumulation.  It is trained on the GPU from (ray, brick, t) triples
 * the plain finder produces.  Rendering with it (lrt_set_tuning(ctx,
 * "proposal", 1)) starts a brick's voxel walk at the predicted voxel when the
 * brick's occupancy mask shows that every voxel before it is empty, and falls
 * back to the plain walk otherwise; the reference finder refines the crossing
 * in either case, so hits are identical to the plain kernel's.  SBS scenes in a
 * DX layout with the NEWTON finder only; other scenes render with the plain
 * kernel.  No counterpart in the reference.
 */
#ifndef LRT_PROPOSAL_H
#define LRT_PROPOSAL_H
#include "lrt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LRT_MLP_PARAMS 1633   /* W1[32][16], b1[32], W2[32][32], b2[32], W3[32], b3 */
#define LRT_MLP_FEATURES 16

/* FP32 parameters in the layout above; setting them resets the optimiser. */
lrt_status lrt_proposal_set_weights(lrt_ctx *ctx, const float *params);
lrt_status lrt_proposal_get_weights(lrt_ctx *ctx, float *params);

/* Triples from the plain finder: renders the views (pixel centres) of the
 * committed SBS scene and appends, for every hit, the features of the hit
 * brick's segment and a target fraction of the segment, keeping at most
 * `capacity` triples in the context.  *n_total: triples held afterwards.
 * The target follows the "proposal_target" tuning key: 0 (default) the
 * crossing; 1 the middle of the first voxel in which the walk would run the
 * finder (occupied and entered past the ray's start), the farthest point a
 * jump can be certified to. */
lrt_status lrt_proposal_collect(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, uint64_t capacity,
                                uint64_t *n_total);
/* Drops every triple held. */
lrt_status lrt_proposal_clear(lrt_ctx *ctx);
/* Replaces the triples with host data (n x 16 features, rounded to BF16, and n targets). */
lrt_status lrt_proposal_set_triples(lrt_ctx *ctx, const float *features, const float *targets, uint64_t n);
/* Copies triples [first, first + n) out (features widened to FP32). */
lrt_status lrt_proposal_get_triples(lrt_ctx *ctx, uint64_t first, uint64_t n, float *features, float *targets);

/* Adam training: `steps` steps numbered first_step.. (bias correction), each on
 * `batch` samples (a multiple of 32) drawn uniformly with replacement from the
 * triples by a hash of (seed, step, sample), mean squared error.  losses
 * (steps floats, may be NULL) receives each step's loss. */
lrt_status lrt_proposal_train(lrt_ctx *ctx, uint32_t first_step, uint32_t steps, uint32_t batch, float lr,
                              uint32_t seed, float *losses);
/* Loss and gradient (LRT_MLP_PARAMS floats) over the first n triples, in order, without an update. */
lrt_status lrt_proposal_gradient(lrt_ctx *ctx, uint32_t n, float *grad, float *loss);
/* Network outputs for triples [first, first + n). */
lrt_status lrt_proposal_infer(lrt_ctx *ctx, uint64_t first, uint64_t n, float *out);
/* The same on a chosen tensor-core engine: LRT_MLP_ENGINE_MMA (warp-level
 * mma.sync, 32 samples a warp) or LRT_MLP_ENGINE_TCGEN05 (128-sample tiles,
 * single-thread tcgen05.mma into TMEM).  Both round to BF16 at the same points;
 * FP32 accumulation order inside the tensor core may differ.  ms (may be NULL)
 * receives the kernel's device time. */
#define LRT_MLP_ENGINE_MMA 0
#define LRT_MLP_ENGINE_TCGEN05 1
lrt_status lrt_proposal_infer_ex(lrt_ctx *ctx, uint64_t first, uint64_t n, float *out, int engine, float *ms);
/* Counters of the proposal renders since the last call: proposals made, walks
 * started at the predicted voxel, of those the ones that ended in a hit, and the
 * voxel steps those jumps skipped (voxel faces between the entry voxel and the
 * predicted one) -- the work the network saves. */
lrt_status lrt_proposal_stats(lrt_ctx *ctx, unsigned long long out[4]);

#ifdef __cplusplus
}
#endif
#endif
