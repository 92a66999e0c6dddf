/*
 * lrt — GB300 ray-query engine, C ABI.
 *
 * Plain pointers and sizes only.  Every call returns an lrt_status; on failure
 * lrt_last_error(ctx) holds a message.  One context per host thread; all device
 * work of a call is issued on the stream passed in (NULL = the legacy default
 * stream).  Each entry point names the reference interface it replaces.
 */
#ifndef LRT_GPU_H
#define LRT_GPU_H
#include "lrt_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  LRT_OK = 0,
  LRT_ERR_INVALID = 1,      /* bad argument */
  LRT_ERR_OOM = 2,          /* device or host allocation failed */
  LRT_ERR_CUDA = 3,         /* CUDA runtime error */
  LRT_ERR_UNSUPPORTED = 4,  /* input the engine does not handle (layout, type, ...) */
  LRT_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
  LRT_ERR_BOUNDS = 6,       /* a device-side index check failed */
  LRT_ERR_STATE = 7         /* call order (e.g. render before commit) */
} lrt_status;

typedef struct lrt_ctx lrt_ctx;

/* ---- context (replaces CreateSceneRT / CreateMultiRenderer(DEVICE_GPU):
 *      ISceneObject.h:14, BVH/BVH2Common_host.cpp:1799-1802,
 *      Renderer/eye_ray_host.cpp:684-753) ---- */
lrt_status  lrt_create(lrt_ctx **out, int device);
void        lrt_destroy(lrt_ctx *ctx);
const char *lrt_last_error(const lrt_ctx *ctx);
const char *lrt_status_string(lrt_status s);

/* ---- scene (ISceneObject / BVHRT surface, BVH/BVH2Common.h:100-173) ---- */
/* BVHRT::ClearGeom, BVH/BVH2Common_host.cpp:82-108 */
lrt_status lrt_clear_geom(lrt_ctx *ctx);
/* BVHRT::AddGeom_SdfSBS, BVH/BVH2Common_host.cpp:567-666.  Layouts DX (1/2/4 bytes),
 * ID32F_IRGB32F and ID32F_IRGB32F_IN.  Data are copied. */
lrt_status lrt_add_sbs(lrt_ctx *ctx, const lrt_sbs_header *hdr, const lrt_sbs_node *nodes, uint32_t n_nodes,
                       const uint32_t *values, uint32_t n_values, const float *values_f,
                       uint32_t n_values_f, uint32_t *geom_id);
/* BVHRT::AddGeom_SdfSVS, BVH/BVH2Common_host.cpp:502-565 */
lrt_status lrt_add_svs(lrt_ctx *ctx, const lrt_svs_node *nodes, uint32_t n_nodes, uint32_t *geom_id);
/* BVHRT::AddGeom_Triangles3f, BVH/BVH2Common_host.cpp:205-257 (primsInLeaf 2) */
lrt_status lrt_add_triangles(lrt_ctx *ctx, const float *vpos, size_t n_vert, size_t v_byte_stride,
                             const uint32_t *indices, size_t n_indices, uint32_t *geom_id);
/* BVHRT::ClearScene, BVH/BVH2Common_host.cpp:1382-1388 */
lrt_status lrt_clear_scene(lrt_ctx *ctx);
/* BVHRT::AddInstance, BVH/BVH2Common_host.cpp:1450-1487 (matrix row-major) */
lrt_status lrt_add_instance(lrt_ctx *ctx, uint32_t geom_id, const float matrix[16], uint32_t *inst_id);
/* BVHRT::CommitScene, BVH/BVH2Common_host.cpp:1416-1448: builds the BVH and
 * uploads the scene to the device.  Any number of instances, all of one
 * geometry (instances of different geometries: LRT_ERR_UNSUPPORTED); with
 * several, every ray tests each instance box in instance order and walks the
 * instances it enters with the closest hit so far (the reference's TLAS walk,
 * BVH/BVH2Common.cpp:3508-3547, gives the same closest hit), and query records
 * carry the instance in instId. */
lrt_status lrt_commit_scene(lrt_ctx *ctx);
/* BVHRT::SetPreset / MultiRenderer::SetPreset, Renderer/eye_ray_host.cpp:549-556.
 * ray_gen_mode 0 (regular sub-pixel grid) or 1 (RAY_GEN_MODE_RANDOM, see
 * lrt_set_seed); interpolation_mode 0 (trilinear) only. */
lrt_status lrt_set_preset(lrt_ctx *ctx, const lrt_preset *preset);

/* Launch-shape and kernel choices; no reference counterpart (the reference's
 * device path is generated by kernel_slicer).  Keys: "variant" (0 = one ray per
 * lane, default; 1 = warp packet traversal; 2 = one ray per lane with per-lane
 * ray refill), "refill" (variant 2: idle lanes that trigger a refill, 1..32),
 * "stage" (packet kernel: 1 = stage each brick in shared memory), "block_warps"
 * (1..8), "tile_w" (a warp's pixel tile is tile_w x 32/tile_w: 4, 8 (default),
 * 16, 32), "stack" (traversal stack entries: 64 (default) or 32, which renders
 * refuse for trees too deep for it).  Results do not depend on these.
 * "fma" (0 = default; 1 = variant-0 renders of SBS and SVS scenes run kernels compiled with
 * floating-point contraction: faster, no longer bit-identical to the reference's
 * x86-64 build, within the forward parity tolerance: same hit mask, depth within
 * 1e-4 of the scene extent, normals within 1e-3, apart from grazing and crease
 * pixels).  "proposal": see lrt_proposal.h.
 * "bvh_builder" (read by lrt_commit_scene and lrt_dr_set_scene: 0 = host
 * binned-SAH build, default, standing in for the reference's Embree build
 * (BVH/cbvh.cpp:591-657); 1 = the same binned SAH on the device, level by level:
 * the same tree, fat pairs and hits (a rare object-median split of more than
 * 4096 primitives sends the build back to the host, with the same result);
 * 2 = a linear BVH on the device: Morton codes of the primitive centroids, a
 * radix sort, a binary radix tree and the same 4-wide collapse, one primitive
 * per leaf; hits are the same apart from exact ties between primitives, and
 * traversal is a few percent slower).
 * "first_hit" (0 = default: the closest hit, independent of the BVH's shape;
 * 1 = SBS and SVS renders, queries and graphs walk the BVH2 fat pairs in
 * BVH2TraverseF32's order and stop at the first SDF leaf that reports a hit,
 * BVH/BVH2Common.cpp:3402-3405, 3407-3488 -- the reference's own result, which
 * depends on the tree: the committed BVH's pairs, or the caller's through
 * lrt_set_bvh2.  Triangle meshes have no early-out in the reference and keep
 * the closest hit.  Not used by lrt_render_counters or the autotuner;
 * lrt_render_noalloc uses it once the BVH2 is on the device).
 * "proposal_target": lrt_proposal_collect's target (see lrt_proposal.h).
 * "host_copy" (1 = default: lrt_render_host copies page-locked outputs chunk by
 * chunk while the render runs; 0 = the kernel writes them across the host link).
 * "tc_wait" (default 1048576): how many times the tcgen05 network engine polls
 * a completion barrier before it gives up (a poll sleeps up to about 1 us, so
 * the default bounds a wait near one second); a timeout makes
 * lrt_proposal_infer_ex return LRT_ERR_TIMEOUT after the block has drained its
 * issued tensor-core work and freed its tensor memory (the next call runs
 * normally).  0 makes every block give up at its first wait: the failure path,
 * for tests. */
lrt_status lrt_set_tuning(lrt_ctx *ctx, const char *key, int value);

/* MultiRenderer::setSeed (Renderer/eye_ray.h:173): the seed of the sub-pixel
 * offsets of RAY_GEN_MODE_RANDOM (preset ray_gen_mode 1), drawn as the
 * reference does with rand2(x, y, i + seed % 2) (Renderer/eye_ray.cpp:53-80,
 * 100-107).  Default 0 (the reference seeds from rand()). */
lrt_status lrt_set_seed(lrt_ctx *ctx, uint32_t seed);

/* The BVH2 of the first-hit walk ("first_hit" tuning) for the committed SBS or
 * SVS scene, in the reference's fat-pair layout (root pair at 0, leaf payload
 * PackOffsetAndSize(brick, 1)) -- e.g. the tree the reference's own builder made
 * for the same bricks (BVHRT::m_allNodePairs), so that renders reproduce the
 * reference's first hits exactly.  Copied; checked first (a tree rooted at pair
 * 0, every index in range, at most 80 inner pairs on a path: LRT_ERR_INVALID
 * otherwise).  Valid until the next commit.  No reference counterpart. */
lrt_status lrt_set_bvh2(lrt_ctx *ctx, const lrt_bvh_pair *pairs, uint32_t n_pairs);

/* BVHRT::UpdateInstance, BVH/BVH2Common_host.cpp:1489-1520: a new matrix for an
 * instance; the committed scene follows at once (no rebuild: the instance box
 * and inverse matrices are recomputed). */
lrt_status lrt_update_instance(lrt_ctx *ctx, uint32_t inst_id, const float matrix[16]);

/* BVHRT::UpdateGeom_Triangles3f, BVH/BVH2Common_host.cpp:258-261 (which the
 * reference leaves unimplemented): new vertex positions for the committed mesh,
 * refit on the device as lrt_refit_triangles does.  `indices` may be NULL or
 * must equal the committed ones (new connectivity: LRT_ERR_UNSUPPORTED; add the
 * mesh again and commit). */
lrt_status lrt_update_geom_triangles(lrt_ctx *ctx, uint32_t geom_id, const float *vpos, size_t n_vert,
                                     const uint32_t *indices, size_t n_indices, size_t v_byte_stride);

/* BVHRT::AddGeom_AABB, BVH/BVH2Common_host.cpp:264-280: always
 * LRT_ERR_UNSUPPORTED.  The reference builds a BVH over the boxes but registers
 * no geometry object for them, so its traversal has no intersector to call for
 * such a leaf; this path has none either (custom primitives are outside the
 * SBS / SVS / triangle leaves it accelerates). */
lrt_status lrt_add_aabb(lrt_ctx *ctx, uint32_t type_id, const float *boxes8, size_t n_boxes, uint32_t *geom_id);

/* New vertex positions for the committed triangle mesh (same vertex count and
 * indices; n_vert positions, v_byte_stride bytes apart): the BVH keeps its
 * topology and its boxes are refit on the device, deepest level first; the
 * instance box follows the new geometry box.  No reference counterpart (the
 * reference rebuilds).  Afterwards lrt_get_bvh2 fails (the fat pairs are made
 * at commit only) and graphs captured earlier must be created again. */
lrt_status lrt_refit_triangles(lrt_ctx *ctx, const float *vpos, size_t n_vert, size_t v_byte_stride);

/* One launch shape and its median time. */
typedef struct { int variant, block_warps, stage, tile_w, stack; float ms; } lrt_tuning_choice;
/* Autotuner: renders the views into a device buffer with each candidate shape
 * (tile shapes 4x8/8x4/16x2 x stack 32/64 for the per-lane kernel; the packet
 * kernel with and without brick staging at 2 and 4 warps per block), `reps`
 * timed runs each after a warm-up, sets the fastest on the context and returns
 * it; `all` (capacity cap, may be NULL) receives every candidate tried. */
lrt_status lrt_autotune(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, uint32_t reps, lrt_tuning_choice *best,
                        lrt_tuning_choice *all, uint32_t cap, uint32_t *n_tried);

/* A batched render captured as a CUDA graph (work-queue reset + the persistent
 * kernel) for a fixed set of view sizes and output pointers (device memory),
 * with the context's tuning at capture time.  Launch replays it on `stream`;
 * set_views changes the cameras (same sizes) for later replays.  The graph owns
 * its view table; destroy it before the context. */
typedef struct lrt_graph lrt_graph;
lrt_status lrt_render_graph_create(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, lrt_hit16 *hits16,
                                   float *rgba, uint32_t *rgba8, lrt_graph **out);
lrt_status lrt_render_graph_launch(lrt_ctx *ctx, lrt_graph *graph, void *stream);
lrt_status lrt_render_graph_set_views(lrt_ctx *ctx, lrt_graph *graph, const lrt_view *views, uint32_t n_views);
void       lrt_render_graph_destroy(lrt_graph *graph);

/* ---- queries ---- */
/* BVHRT::RayQuery_NearestHit, BVH/BVH2Common.cpp:3490-3559, batched: n rays of
 * float4 (pos, tNear) and float4 (dir, tFar); tFar <= 0 requests any-hit
 * (RayQuery_AnyHit, :3561-3566).  device_ptrs != 0: all three arrays are device
 * memory and the call is asynchronous on `stream`; otherwise host memory and the
 * call returns after the copy back. */
lrt_status lrt_query_rays(lrt_ctx *ctx, const float *pos_near, const float *dir_far, uint32_t n,
                          lrt_hit *out, int device_ptrs, void *stream);

/* ---- rendering (MultiRenderer::Render / RenderFloat, Renderer/eye_ray_host.cpp:563-585,
 *      batched over views in one persistent launch) ---- */
/* Output offsets: view v starts at sum_{u<v} width_u*height_u pixels, row-major
 * within a view.  Any of hits16 / rgba / rgba8 may be NULL.  All output pointers
 * are device memory; asynchronous on `stream`. */
lrt_status lrt_render(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, lrt_hit16 *hits16,
                      float *rgba, uint32_t *rgba8, void *stream);
/* Same, with host output buffers, synchronous.  Page-locked buffers (cudaHostAlloc,
 * cudaHostRegister): the kernel renders into device buffers and counts each
 * finished chunk of whole tile rows (about 1/48 of the batch), and a copy stream
 * of the context moves each chunk to the host as soon as it is counted, while
 * the rest renders (stream memory waits through the driver entry point
 * cuStreamWaitValue32; the render stream releases every wait once the kernel has
 * finished); the batch's last chunks, at most 1/16 of it, the kernel writes to
 * the host buffers itself, so that no copy is left once it ends.  Where the chosen kernel does not count chunks (variant 1, 2 or 3,
 * the proposal kernel), with more than 256 views, or with "host_copy" 0, the
 * kernel writes the page-locked buffers itself across the host link.  Pageable
 * buffers receive a copy of device buffers after the render.  The results are
 * the same on every path. */
lrt_status lrt_render_host(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, lrt_hit16 *hits16,
                           float *rgba, uint32_t *rgba8);
/* Rendering that allocates nothing.  No counterpart in the reference.
 *
 * For callers that must not allocate device memory during rendering: a host
 * application whose own pool allocator has reserved the GPU's memory up front
 * (a cudaMalloc from the library would fail or fragment that pool), and a
 * real-time frame loop where cudaMalloc's implicit device synchronisation and
 * latency are not acceptable.  Same results as lrt_render for the committed
 * scene (the inputs were allocated once, by lrt_commit_scene), rendered with
 * the plain finder: the "proposal" tuning key is ignored here (the proposal
 * kernels need the network's buffers, which this call does not touch).  With
 * "first_hit" set it renders the reference's first-hit walk like lrt_render,
 * whose tree is put on the device by the first lrt_render, lrt_query_rays or
 * lrt_set_bvh2 call after a commit; before that, this call returns
 * LRT_ERR_STATE rather than allocate it.  The
 * per-call scratch -- the persistent kernel's work-queue head and the per-view
 * table -- lives in one file-scope device array of 256 +
 * LRT_NOALLOC_MAX_VIEWS * 160 bytes that every GPU loading the library keeps
 * until exit.  At most LRT_NOALLOC_MAX_VIEWS views per call; more returns
 * LRT_ERR_INVALID.  The view table is passed to a small set-up kernel by
 * value (two launches per call: set-up, render), so the `views` array may be
 * reused as soon as the call returns.  The first call on a device looks up
 * the array's device address and keeps it for the life of the process: make
 * that first call before any stream capture, and do not use the library on a
 * device after cudaDeviceReset (which also invalidates every context's device
 * buffers).  All calls share the array, which keeps the last call's contents
 * (the queue head is cleared on every call): calls whose GPU work overlaps --
 * on different streams, or from several host threads -- race on it; serialise
 * them on one stream.  Outputs are device memory, as in lrt_render;
 * asynchronous on `stream`.  Errors are reported through the status only
 * (lrt_last_error is not updated, which could allocate). */
#define LRT_NOALLOC_MAX_VIEWS 64
lrt_status lrt_render_noalloc(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, lrt_hit16 *hits16,
                              float *rgba, uint32_t *rgba8, void *stream);
/* Number of our kernels launched by the last lrt_render / lrt_query_rays call. */
uint32_t lrt_last_launch_count(const lrt_ctx *ctx);
/* Per-ray traversal counters of the committed scene for the given views (a
 * counting variant of the render kernel, not for timing): fat-node visits
 * (BVH2-equivalent), leaf visits, voxel visits, finder calls.  out[4], summed. */
lrt_status lrt_render_counters(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, uint64_t out[4]);

/* The committed scene's BVH2 in the reference's fat-pair layout (root pair at 0),
 * as CreateFatTreeArray produces it (BVH/cbvh_fat.cpp:100-142).  Host pointer
 * owned by ctx, valid until the next commit.  A device-built BVH numbers pair i
 * after internal node i of its radix tree and is copied from the device on the
 * first call. */
lrt_status lrt_get_bvh2(lrt_ctx *ctx, const lrt_bvh_pair **pairs, uint32_t *n_pairs);

/* The BVH builder alone, no device needed: fat pairs for n boxes (n x 6 floats,
 * min xyz then max xyz).  prims_per_leaf 1: leaf payload is the box id; 2: leaf
 * payload indexes *leaf_start_count (PackOffsetAndSize(start, count) into
 * *order, the reordered primitive ids).  Arrays are malloc'd; free with
 * lrt_free.  Replaces BuildBVHFatCustom / BuildBVHFat (BVH/cbvh_fat.cpp:148-183). */
lrt_status lrt_build_bvh2(const float *boxes6, uint32_t n, uint32_t prims_per_leaf, lrt_bvh_pair **pairs,
                          uint32_t *n_pairs, uint32_t **leaf_start_count, uint32_t *n_leaves, uint32_t **order);
void lrt_free(void *p);

/* ---- scene construction (utils/sdf_converter.cpp:118-181,
 *      utils/sparse_octree_builder.cpp:72-444, :2346-2387) ---- */
typedef struct lrt_sbs lrt_sbs;
typedef struct lrt_svs lrt_svs;
/* create_sdf_SBS: frame octree to `depth`, border bricks, DX layout quantisation. */
lrt_status lrt_sbs_build_from_sdf(const lrt_sdf_desc *sdf, uint32_t depth, const lrt_sbs_header *hdr,
                                  int threads, lrt_sbs **out);
lrt_status lrt_sbs_data(const lrt_sbs *sbs, lrt_sbs_header *hdr, const lrt_sbs_node **nodes, uint32_t *n_nodes,
                        const uint32_t **values, uint32_t *n_values);
void       lrt_sbs_free(lrt_sbs *sbs);
/* create_sdf_SVS */
lrt_status lrt_svs_build_from_sdf(const lrt_sdf_desc *sdf, uint32_t depth, int threads, lrt_svs **out);
lrt_status lrt_svs_data(const lrt_svs *svs, const lrt_svs_node **nodes, uint32_t *n_nodes);
void       lrt_svs_free(lrt_svs *svs);
/* The same two builders on GPU `device`: the same frame octree, bricks and voxels
 * in the same order, bit for bit (the octree grows level by level, one thread per
 * node; brick values one block per leaf).  depth >= 4 (shallower sets are a few
 * thousand nodes: use the host builders); results in host memory as above.
 * lrt_build_last_error() describes the last failure of these calls on the calling
 * thread. */
lrt_status lrt_sbs_build_from_sdf_gpu(int device, const lrt_sdf_desc *sdf, uint32_t depth, const lrt_sbs_header *hdr,
                                      lrt_sbs **out);
lrt_status lrt_svs_build_from_sdf_gpu(int device, const lrt_sdf_desc *sdf, uint32_t depth, lrt_svs **out);
const char *lrt_build_last_error(void);

/* Files in the reference's binary layout (save_sdf_SBS / load_sdf_SBS /
 * save_sdf_SVS / load_sdf_SVS, sdfScene/sdf_scene.cpp:121-175): SBS = header,
 * u32 node count, nodes, u32 value count, values; SVS = u32 node count, nodes.
 * Loads check every count against the file size (LRT_ERR_INVALID for a short or
 * foreign file) and return the same objects as the builders. */
lrt_status lrt_sbs_save(const char *path, const lrt_sbs_header *hdr, const lrt_sbs_node *nodes, uint32_t n_nodes,
                        const uint32_t *values, uint32_t n_values);
lrt_status lrt_sbs_load(const char *path, lrt_sbs **out);
lrt_status lrt_svs_save(const char *path, const lrt_svs_node *nodes, uint32_t n_nodes);
lrt_status lrt_svs_load(const char *path, lrt_svs **out);

/* ---- camera helpers (LiteMath::perspectiveMatrix / lookAt / inverse4x4 as used
 *      by tests/tests.cpp:29-41 and Renderer/eye_ray_host.cpp:59-65) ---- */
void lrt_perspective(float fov_deg, float aspect, float znear, float zfar, float out[16]);
void lrt_look_at(const float eye[3], const float center[3], const float up[3], float out[16]);
void lrt_inverse4x4(const float m[16], float out[16]);

#ifdef __cplusplus
}
#endif
#endif
