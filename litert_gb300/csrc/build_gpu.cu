// GPU construction of sparse brick sets (SBS) and sparse voxel sets (SVS) from
// analytic SDFs: the same frame octree, bricks and voxels as the host builder
// (scene_build.cpp, a restatement of utils/sparse_octree_builder.cpp:72-444 and
// :2346-2387 entered through utils/sdf_converter.cpp:118-181), in the same order
// and bit for bit.
//
// The frame octree is grown level by level.  Levels 0-4 are the reference's
// "large" nodes (a full octree); each level-4 node whose centre distance is
// below sqrt(3) 2^-4 roots a subtree that add_node_rec splits while the node's
// centre distance is below sqrt(3) d or its corner values change sign.  Every
// node is one thread of a level pass; split nodes emit their 8 children into the
// next level's array at positions given by an exclusive scan.
//
// Order.  The host builder appends each subtree after the large nodes in
// large-node order, and inside a subtree allocates a split node's 8 children as
// one block when the depth-first recursion reaches that node, so a leaf's place
// among the frame nodes is base(subtree) + 8 rank(parent) + child, where
// rank(parent) is the parent's position among the subtree's split nodes in
// depth-first pre-order.  Ranks come from per-node split counts (a bottom-up
// pass) distributed top-down over each split node's children.  Kept bricks are
// written in frame order by an exclusive scan over a per-frame-node flag.  The
// SVS writer walks the octree depth first from the root (svs_rec), i.e. leaves in
// lexicographic path order: kept-leaf counts bottom-up, offsets top-down.
//
// All arithmetic follows the host builder's expression order; this unit is
// compiled without contraction, with IEEE division and square root, so the
// values equal the host's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "lrt_internal.h"

namespace lrt {
namespace bld {

constexpr uint32_t kNoParent = 0xFFFFFFFFu;
constexpr uint32_t kLargeLevels = 4;                         // levels 0..4 are the large nodes
constexpr uint32_t kLargeCount = 1 + 8 + 64 + 512 + 4096;    // 4681
constexpr uint32_t kLevel4First = 1 + 8 + 64 + 512;          // BFS index of the first level-4 node

struct Sdf {
  const float *spheres;
  const float *boxes;
  uint32_t ns, nb;
  float k;
};

// ---- the SDF, as scene_build.cpp evaluates it ----
__device__ __forceinline__ float sdf_sphere(const float *s, float x, float y, float z) {
  const float dx = x - __ldg(s), dy = y - __ldg(s + 1), dz = z - __ldg(s + 2);
  return sqrtf(dx * dx + dy * dy + dz * dz) - __ldg(s + 3);
}
__device__ __forceinline__ float sdf_round_box(const float *b, float x, float y, float z) {
  const float px = x - __ldg(b), py = y - __ldg(b + 1), pz = z - __ldg(b + 2);
  const float *R = b + 7;
  const float lx = __ldg(R) * px + __ldg(R + 1) * py + __ldg(R + 2) * pz;
  const float ly = __ldg(R + 3) * px + __ldg(R + 4) * py + __ldg(R + 5) * pz;
  const float lz = __ldg(R + 6) * px + __ldg(R + 7) * py + __ldg(R + 8) * pz;
  const float r = __ldg(b + 6);
  const float qx = fabsf(lx) - (__ldg(b + 3) - r), qy = fabsf(ly) - (__ldg(b + 4) - r), qz = fabsf(lz) - (__ldg(b + 5) - r);
  const float mx = qx > 0 ? qx : 0, my = qy > 0 ? qy : 0, mz = qz > 0 ? qz : 0;
  const float outside = sqrtf(mx * mx + my * my + mz * mz);
  float m = qx > qy ? qx : qy;
  m = m > qz ? m : qz;
  const float inside = m < 0 ? m : 0;
  return outside + inside - r;
}
__device__ __forceinline__ float smooth_min(float a, float b, float k) {
  const float m = a < b ? a : b;
  if (k <= 0.0f) return m;
  float h = k - fabsf(a - b);
  h = h > 0 ? h : 0;
  h = h / k;
  return m - h * h * k * 0.25f;
}
__device__ float sdf_eval(const Sdf &f, float x, float y, float z) {
  float d = 1e10f;
  bool first = true;
  for (uint32_t i = 0; i < f.ns; i++) {
    const float v = sdf_sphere(f.spheres + 4 * i, x, y, z);
    d = first ? v : smooth_min(d, v, f.k);
    first = false;
  }
  for (uint32_t i = 0; i < f.nb; i++) {
    const float v = sdf_round_box(f.boxes + 16 * i, x, y, z);
    d = first ? v : smooth_min(d, v, f.k);
    first = false;
  }
  return d;
}
// sdf(2 ((p + c) d) - 1), utils/sparse_octree_builder.cpp:75,80
__device__ __forceinline__ float node_point(const Sdf &f, float px, float py, float pz, float cx, float cy, float cz,
                                            float d) {
  return sdf_eval(f, 2.0f * ((px + cx) * d) - 1.0f, 2.0f * ((py + cy) * d) - 1.0f, 2.0f * ((pz + cz) * d) - 1.0f);
}

__device__ __forceinline__ float fmin_ref(float a, float b) { return b < a ? b : a; }   // std::min
__device__ __forceinline__ float fmax_ref(float a, float b) { return a < b ? b : a; }   // std::max

// octal digit of a level-4 BFS rank -> coordinates, and back
__device__ __forceinline__ uint3 l4_coords(uint32_t r) {
  uint32_t x = 0, y = 0, z = 0;
  for (int lev = 0; lev < 4; lev++) {
    const uint32_t c = (r >> (3 * (3 - lev))) & 7u;
    x = 2 * x + ((c >> 2) & 1u);
    y = 2 * y + ((c >> 1) & 1u);
    z = 2 * z + (c & 1u);
  }
  return make_uint3(x, y, z);
}
__device__ __forceinline__ uint32_t l4_rank(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t r = 0;
  for (int b = 3; b >= 0; b--) r = 8 * r + ((((x >> b) & 1u) << 2) | (((y >> b) & 1u) << 1) | ((z >> b) & 1u));
  return r;
}

// one level of the octree (device arrays)
struct LevelView {
  uint32_t n, level;
  uint4 *pos;       // x, y, z at this level; parent index in the level above
  uint32_t *meta;   // bits 0-2 child index, bit 3 split, bit 4 large-node border (level 4)
  float4 *vals;     // 8 corner values (2 float4)
  uint32_t *base;   // first child in the next level (split nodes)
  uint32_t *cnt;    // split nodes in the subtree (SBS) / kept leaves in the subtree (SVS)
  uint32_t *rank;   // depth-first rank among split nodes of the subtree (SBS) / output offset (SVS)
};

__global__ void init_level4(LevelView L) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= L.n) return;
  const uint3 c = l4_coords(r);
  L.pos[r] = make_uint4(c.x, c.y, c.z, kNoParent);
  L.meta[r] = 0;
}

// corner values, the large-node border test (level 4) and add_node_rec's split test
__global__ void eval_level(Sdf f, LevelView L, uint32_t max_depth) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  const uint4 p = L.pos[i];
  const float d = ldexpf(1.0f, -int(L.level));
  const float px = float(p.x), py = float(p.y), pz = float(p.z);
  const float vc = node_point(f, px, py, pz, 0.5f, 0.5f, 0.5f, d);
  float v[8];
  float mn = 1000, mx = -1000;
#pragma unroll 1
  for (int c = 0; c < 8; c++) {
    v[c] = node_point(f, px, py, pz, float((c & 4) >> 2), float((c & 2) >> 1), float(c & 1), d);
    mn = fmin_ref(mn, v[c]);
    mx = fmax_ref(mx, v[c]);
  }
  L.vals[2 * i] = make_float4(v[0], v[1], v[2], v[3]);
  L.vals[2 * i + 1] = make_float4(v[4], v[5], v[6], v[7]);
  uint32_t meta = L.meta[i] & 7u;
  bool may_split = true;
  if (L.level == kLargeLevels) {   // is_border of a large leaf (:38-41), in double as there
    const bool border = fabs(double(vc)) < sqrt(3.0) * ldexp(1.0, -int(L.level));
    if (border) meta |= 16u;
    may_split = border;
  }
  const bool split = may_split && L.level < max_depth && (fabsf(vc) < sqrtf(3.0f) * d || mn * mx <= 0);
  if (split) meta |= 8u;
  L.meta[i] = meta;
}

__global__ void split_flags(LevelView L, uint32_t *flag) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < L.n) flag[i] = (L.meta[i] >> 3) & 1u;
}

__global__ void emit_children(LevelView L, const uint32_t *scan, LevelView N) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n || !((L.meta[i] >> 3) & 1u)) return;
  const uint32_t b = 8 * scan[i];
  L.base[i] = b;
  const uint4 p = L.pos[i];
#pragma unroll
  for (uint32_t c = 0; c < 8; c++) {
    N.pos[b + c] = make_uint4(2 * p.x + ((c & 4) >> 2), 2 * p.y + ((c & 2) >> 1), 2 * p.z + (c & 1), i);
    N.meta[b + c] = c;
  }
}

// split nodes per subtree, bottom-up (next = the level below; null at the deepest)
__global__ void count_splits(LevelView L, LevelView N, bool has_next) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  uint32_t c = 0;
  if ((L.meta[i] >> 3) & 1u) {
    c = 1;
    if (has_next)
      for (uint32_t k = 0; k < 8; k++) c += N.cnt[L.base[i] + k];
  }
  L.cnt[i] = c;
}

// depth-first ranks of the children of each split node
__global__ void rank_children(LevelView L, LevelView N) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n || !((L.meta[i] >> 3) & 1u)) return;
  uint32_t acc = L.rank[i] + 1;
  for (uint32_t k = 0; k < 8; k++) {
    N.rank[L.base[i] + k] = acc;
    acc += N.cnt[L.base[i] + k];
  }
}

__global__ void subtree_sizes(LevelView L4, uint32_t *app) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < L4.n) app[r] = 8u * L4.cnt[r];
}

struct BrickParams {
  uint32_t bs, pad, v, v3, words, vals_per_int, bits, max_q;
};

// frame index of a leaf (scene_build.cpp build_frame's node order)
__device__ __forceinline__ uint32_t frame_index(const LevelView &L, const LevelView &P, const uint32_t *sub_base,
                                                uint32_t i) {
  const uint4 p = L.pos[i];
  if (L.level == kLargeLevels) return kLevel4First + i;
  const uint32_t sh = L.level - kLargeLevels;
  const uint32_t r = l4_rank(p.x >> sh, p.y >> sh, p.z >> sh);
  return sub_base[r] + 8u * P.rank[p.w] + (L.meta[i] & 7u);
}

// One block per node of a level: the brick values of a leaf (frame_octree_to_SBS,
// :291-444), the is_border_node test (:49-53) and, for a kept brick, its
// quantised words in a slot of the unordered staging buffer.
__global__ void __launch_bounds__(256) brick_values(Sdf f, LevelView L, LevelView P, const uint32_t *sub_base,
                                                    BrickParams bp, uint32_t *slot_of_frame, uint32_t *slot_counter,
                                                    uint32_t *stage_words, lrt_sbs_node *stage_nodes,
                                                    uint32_t stage_cap) {
  extern __shared__ float vals[];
  __shared__ float red_mn[8], red_mx[8];
  __shared__ uint32_t slot_sh;
  const uint32_t i = blockIdx.x;
  if ((L.meta[i] >> 3) & 1u) return;   // split: not a leaf (uniform over the block)
  const uint4 p = L.pos[i];
  const float d = ldexpf(1.0f, -int(L.level));
  const float4 c0 = L.vals[2 * i], c1 = L.vals[2 * i + 1];
  const float nv[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
  const float p0x = 2.0f * (d * float(p.x)) - 1.0f, p0y = 2.0f * (d * float(p.y)) - 1.0f,
              p0z = 2.0f * (d * float(p.z)) - 1.0f;
  const float dp = 2.0f * d / float(bp.bs);
  const int B = int(bp.bs), pad = int(bp.pad), V = int(bp.v);
  float mn = 1000, mx = -1000;
  for (int k = 0; k < 8; k++) { mn = fmin_ref(mn, nv[k]); mx = fmax_ref(mx, nv[k]); }
  for (uint32_t idx = threadIdx.x; idx < bp.v3; idx += blockDim.x) {
    const int i3 = int(idx) / (V * V) - pad, j3 = (int(idx) / V) % V - pad, k3 = int(idx) % V - pad;
    float val = 2e6f;
    if (i3 == 0) {
      if (j3 == 0) { if (k3 == 0) val = nv[0]; else if (k3 == B) val = nv[1]; }
      else if (j3 == B) { if (k3 == 0) val = nv[2]; else if (k3 == B) val = nv[3]; }
    } else if (i3 == B) {
      if (j3 == 0) { if (k3 == 0) val = nv[4]; else if (k3 == B) val = nv[5]; }
      else if (j3 == B) { if (k3 == 0) val = nv[6]; else if (k3 == B) val = nv[7]; }
    }
    if (val > 1e6f) val = sdf_eval(f, p0x + dp * float(i3), p0y + dp * float(j3), p0z + dp * float(k3));
    vals[idx] = val;
    mn = fmin_ref(mn, val);
    mx = fmax_ref(mx, val);
  }
  // min and max are exact, so the reduction order does not matter
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin_ref(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax_ref(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) { red_mn[threadIdx.x >> 5] = mn; red_mx[threadIdx.x >> 5] = mx; }
  __syncthreads();
  mn = red_mn[0];
  mx = red_mx[0];
  for (uint32_t w = 1; w < (blockDim.x >> 5); w++) { mn = fmin_ref(mn, red_mn[w]); mx = fmax_ref(mx, red_mx[w]); }
  const uint32_t level_size = uint32_t(1 / d);
  const float bd_max = float(2 * sqrt(3.0) / double(level_size));
  if (!((mn <= 0) && (mx > -bd_max))) return;   // uniform
  if (threadIdx.x == 0) {
    const uint32_t s = atomicAdd(slot_counter, 1u);
    slot_sh = s;
    if (s < stage_cap) {
      slot_of_frame[frame_index(L, P, sub_base, i)] = s + 1;
      const uint32_t lod_size = uint32_t(1.0f / d);
      lrt_sbs_node nd;
      nd.pos_xy = (p.x << 16) | p.y;
      nd.pos_z_lod_size = (p.z << 16) | lod_size;
      nd.data_offset = 0;
      nd._pad = 0;
      stage_nodes[s] = nd;
    }
  }
  __syncthreads();
  const uint32_t s = slot_sh;
  if (s >= stage_cap) return;   // counted; the host reports the overflow
  const uint32_t lod_size = uint32_t(1.0f / d);
  const float d_max = float(2 * sqrt(3.0) / double(lod_size));
  uint32_t *w = stage_words + size_t(s) * bp.words;
  for (uint32_t wi = threadIdx.x; wi < bp.words; wi += blockDim.x) {
    uint32_t word = 0;
    for (uint32_t e = 0; e < bp.vals_per_int; e++) {
      const uint32_t vi = wi * bp.vals_per_int + e;
      if (vi >= bp.v3) break;
      float fq = float(bp.max_q) * ((vals[vi] + d_max) / (2 * d_max));
      fq = fmax_ref(0.0f, fq);
      uint32_t q = fq >= 4294967296.0f ? 0xFFFFFFFFu : uint32_t(fq);
      q = q < bp.max_q ? q : bp.max_q;
      word |= q << (bp.bits * e);
    }
    w[wi] = word;
  }
}

__global__ void nonzero_flags(const uint32_t *in, uint32_t *out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i] != 0 ? 1u : 0u;
}

// kept bricks from their staging slots to frame order
__global__ void place_bricks(const uint32_t *slot_of_frame, const uint32_t *pos_of_frame, uint32_t n_frame,
                             const lrt_sbs_node *stage_nodes, const uint32_t *stage_words, uint32_t words,
                             lrt_sbs_node *out_nodes, uint32_t *out_words) {
  for (uint32_t fi = blockIdx.x; fi < n_frame; fi += gridDim.x) {
    const uint32_t s1 = slot_of_frame[fi];
    if (s1 == 0) continue;   // uniform over the block
    const uint32_t s = s1 - 1, o = pos_of_frame[fi];
    if (threadIdx.x == 0) {
      lrt_sbs_node nd = stage_nodes[s];
      nd.data_offset = o * words;
      out_nodes[o] = nd;
    }
    for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) out_words[size_t(o) * words + w] = stage_words[size_t(s) * words + w];
  }
}

// ---- SVS (frame_octree_to_SVS_rec, :2346-2387) ----
__device__ __forceinline__ bool svs_keep(const float4 &c0, const float4 &c1, float d_max) {
  const float v[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
  float mn = 1000, mx = -1000;
  for (int k = 0; k < 8; k++) { mn = fmin_ref(mn, v[k]); mx = fmax_ref(mx, v[k]); }
  return (mn <= 0) && (mx > -d_max);
}
__device__ __forceinline__ float svs_dmax(uint32_t level) {
  return float(2 * sqrt(3.0) / double(1u << level));
}
__global__ void svs_count(LevelView L, LevelView N, bool has_next) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  uint32_t c = 0;
  if ((L.meta[i] >> 3) & 1u) {
    if (has_next)
      for (uint32_t k = 0; k < 8; k++) c += N.cnt[L.base[i] + k];
  } else {
    c = svs_keep(L.vals[2 * i], L.vals[2 * i + 1], svs_dmax(L.level)) ? 1u : 0u;
  }
  L.cnt[i] = c;
}
__global__ void svs_offsets(LevelView L, LevelView N) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n || !((L.meta[i] >> 3) & 1u)) return;
  uint32_t acc = L.rank[i];
  for (uint32_t k = 0; k < 8; k++) {
    N.rank[L.base[i] + k] = acc;
    acc += N.cnt[L.base[i] + k];
  }
}
__global__ void svs_write(LevelView L, lrt_svs_node *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n || ((L.meta[i] >> 3) & 1u) || L.cnt[i] == 0) return;
  const float4 c0 = L.vals[2 * i], c1 = L.vals[2 * i + 1];
  const float v[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
  const uint32_t lod = 1u << L.level;
  const float d_max = svs_dmax(L.level);
  const uint4 p = L.pos[i];
  lrt_svs_node s;
  s.pos_xy = (p.x << 16) | p.y;
  s.pos_z_lod_size = (p.z << 16) | lod;
  s.values[0] = 0u;
  s.values[1] = 0u;
  for (int k = 0; k < 8; k++) {
    const float fq = fmax_ref(0.0f, 255 * ((v[k] + d_max) / (2 * d_max)) + 0.5f);
    uint32_t q = uint32_t(fq);
    q = q < 255u ? q : 255u;
    s.values[k / 4] |= q << (8 * (k % 4));
  }
  out[L.rank[i]] = s;
}

// ---- exclusive scan of uint32 (block scan of 4096 elements, recursive over block sums) ----
constexpr uint32_t kScanThreads = 1024, kScanItems = 4;
__global__ void __launch_bounds__(kScanThreads) scan_blocks(const uint32_t *in, uint32_t *out, uint32_t n,
                                                            uint32_t *block_sums) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  const uint32_t base = blockIdx.x * kScanThreads * kScanItems + threadIdx.x * kScanItems;
  uint32_t v[kScanItems], s = 0;
#pragma unroll
  for (uint32_t k = 0; k < kScanItems; k++) {
    v[k] = (base + k < n) ? in[base + k] : 0u;
    s += v[k];
  }
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t incl = s;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= uint32_t(o)) incl += t;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t t = warp_tot[lane], ti = t;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, ti, o);
      if (lane >= uint32_t(o)) ti += u;
    }
    warp_tot[lane] = ti - t;   // exclusive warp offsets
    if (lane == 31 && block_sums) block_sums[blockIdx.x] = ti;
  }
  __syncthreads();
  uint32_t run = warp_tot[w] + incl - s;
#pragma unroll
  for (uint32_t k = 0; k < kScanItems; k++) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}
__global__ void scan_add(uint32_t *out, uint32_t n, const uint32_t *block_offsets) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += block_offsets[i / (kScanThreads * kScanItems)];
}

}  // namespace bld

namespace {

using namespace bld;

template <typename T>
struct Buf {
  T *p = nullptr;
  cudaError_t alloc(size_t n) {
    if (p) cudaFree(p);
    p = nullptr;
    return cudaMalloc(&p, (n ? n : 1) * sizeof(T));
  }
  ~Buf() {
    if (p) cudaFree(p);
  }
};

struct LevelBufs {
  Buf<uint4> pos;
  Buf<uint32_t> meta, base, cnt, rank;
  Buf<float4> vals;
  uint32_t n = 0, level = 0;
  LevelView view() { return LevelView{n, level, pos.p, meta.p, vals.p, base.p, cnt.p, rank.p}; }
  cudaError_t alloc(uint32_t count, uint32_t lev) {
    n = count;
    level = lev;
    cudaError_t e;
    if ((e = pos.alloc(count)) != cudaSuccess) return e;
    if ((e = meta.alloc(count)) != cudaSuccess) return e;
    if ((e = base.alloc(count)) != cudaSuccess) return e;
    if ((e = cnt.alloc(count)) != cudaSuccess) return e;
    if ((e = rank.alloc(count)) != cudaSuccess) return e;
    return vals.alloc(size_t(count) * 2);
  }
};

inline unsigned grid(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

// exclusive scan; *total (host) receives the sum
cudaError_t exclusive_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint64_t *total, cudaStream_t st) {
  if (n == 0) {
    if (total) *total = 0;
    return cudaSuccess;
  }
  const uint32_t per = kScanThreads * kScanItems, nb = (n + per - 1) / per;
  Buf<uint32_t> sums, offs;
  cudaError_t e;
  if ((e = sums.alloc(nb)) != cudaSuccess) return e;
  scan_blocks<<<nb, kScanThreads, 0, st>>>(in, out, n, sums.p);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (nb > 1) {
    if ((e = offs.alloc(nb)) != cudaSuccess) return e;
    uint64_t t = 0;
    if ((e = exclusive_scan(sums.p, offs.p, nb, &t, st)) != cudaSuccess) return e;
    scan_add<<<grid(n, 256), 256, 0, st>>>(out, n, offs.p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (total) *total = t;
    return cudaSuccess;
  }
  if (total) {
    uint32_t t = 0;
    if ((e = cudaMemcpyAsync(&t, sums.p, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    *total = t;
  }
  return cudaSuccess;
}

struct DevSdf {
  Buf<float> spheres, boxes;
  Sdf f{};
  cudaError_t upload(const lrt_sdf_desc &d) {
    cudaError_t e;
    if ((e = spheres.alloc(size_t(d.n_spheres) * 4)) != cudaSuccess) return e;
    if ((e = boxes.alloc(size_t(d.n_boxes) * 16)) != cudaSuccess) return e;
    if (d.n_spheres && (e = cudaMemcpy(spheres.p, d.spheres, size_t(d.n_spheres) * 16, cudaMemcpyHostToDevice)) != cudaSuccess)
      return e;
    if (d.n_boxes && (e = cudaMemcpy(boxes.p, d.boxes, size_t(d.n_boxes) * 64, cudaMemcpyHostToDevice)) != cudaSuccess)
      return e;
    f = Sdf{spheres.p, boxes.p, d.n_spheres, d.n_boxes, d.k};
    return cudaSuccess;
  }
};

// levels 4..depth of the frame octree
cudaError_t grow_levels(const Sdf &f, uint32_t depth, std::vector<LevelBufs> &lv, cudaStream_t st) {
  lv.clear();
  lv.resize(depth - kLargeLevels + 1);
  cudaError_t e;
  if ((e = lv[0].alloc(4096, kLargeLevels)) != cudaSuccess) return e;
  init_level4<<<grid(4096, 256), 256, 0, st>>>(lv[0].view());
  Buf<uint32_t> flag, scan;
  for (uint32_t li = 0; li < lv.size(); li++) {
    LevelBufs &L = lv[li];
    eval_level<<<grid(L.n, 128), 128, 0, st>>>(f, L.view(), depth);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (li + 1 == lv.size()) break;
    if ((e = flag.alloc(L.n)) != cudaSuccess) return e;
    if ((e = scan.alloc(L.n)) != cudaSuccess) return e;
    split_flags<<<grid(L.n, 256), 256, 0, st>>>(L.view(), flag.p);
    uint64_t n_split = 0;
    if ((e = exclusive_scan(flag.p, scan.p, L.n, &n_split, st)) != cudaSuccess) return e;
    if (n_split * 8 > 0xFFFFFFFFull) return cudaErrorMemoryAllocation;
    if ((e = lv[li + 1].alloc(uint32_t(n_split * 8), L.level + 1)) != cudaSuccess) return e;
    if (n_split == 0) {
      lv.resize(li + 1);   // no deeper nodes
      break;
    }
    emit_children<<<grid(L.n, 256), 256, 0, st>>>(L.view(), scan.p, lv[li + 1].view());
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace

// create_sdf_SBS on the GPU (depth >= 4; the caller validates the header)
lrt_status build_sbs_gpu(const lrt_sdf_desc &sd, uint32_t depth, const lrt_sbs_header &hdr, SbsData &out,
                         std::string &err) {
  const cudaStream_t st = nullptr;
  DevSdf dsdf;
  cudaError_t e = dsdf.upload(sd);
  std::vector<LevelBufs> lv;
  if (e == cudaSuccess) e = grow_levels(dsdf.f, depth, lv, st);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return LRT_ERR_CUDA; }
  const uint32_t nl = uint32_t(lv.size());
  // split counts bottom-up, depth-first ranks top-down
  for (int li = int(nl) - 1; li >= 0; li--) {
    const bool has_next = uint32_t(li + 1) < nl;
    count_splits<<<grid(lv[li].n, 256), 256, 0, st>>>(lv[li].view(), has_next ? lv[li + 1].view() : lv[li].view(),
                                                      has_next);
  }
  cudaMemsetAsync(lv[0].rank.p, 0, 4096 * 4, st);
  for (uint32_t li = 0; li + 1 < nl; li++)
    rank_children<<<grid(lv[li].n, 256), 256, 0, st>>>(lv[li].view(), lv[li + 1].view());
  // subtree bases in large-node order
  Buf<uint32_t> app, sub_base;
  uint64_t appended = 0;
  if ((e = app.alloc(4096)) == cudaSuccess && (e = sub_base.alloc(4096)) == cudaSuccess) {
    subtree_sizes<<<grid(4096, 256), 256, 0, st>>>(lv[0].view(), app.p);
    e = exclusive_scan(app.p, sub_base.p, 4096, &appended, st);
  }
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return LRT_ERR_CUDA; }
  const uint64_t n_frame = uint64_t(kLargeCount) + appended;
  if (n_frame > 0xFFFFFFFFull) { err = "frame octree too large"; return LRT_ERR_INVALID; }
  {  // sub_base += number of large nodes
    std::vector<uint32_t> h(4096);
    if ((e = cudaMemcpy(h.data(), sub_base.p, 4096 * 4, cudaMemcpyDeviceToHost)) != cudaSuccess) {
      err = cudaGetErrorString(e);
      return LRT_ERR_CUDA;
    }
    for (auto &x : h) x += kLargeCount;
    if ((e = cudaMemcpy(sub_base.p, h.data(), 4096 * 4, cudaMemcpyHostToDevice)) != cudaSuccess) {
      err = cudaGetErrorString(e);
      return LRT_ERR_CUDA;
    }
  }
  BrickParams bp;
  bp.bs = hdr.brick_size;
  bp.pad = hdr.brick_pad;
  bp.v = bp.bs + 2 * bp.pad + 1;
  bp.v3 = bp.v * bp.v * bp.v;
  bp.vals_per_int = 4 / hdr.bytes_per_value;
  bp.bits = 8 * hdr.bytes_per_value;
  bp.max_q = hdr.bytes_per_value == 4 ? 0xFFFFFFFFu : ((1u << bp.bits) - 1);
  bp.words = (bp.v3 + bp.vals_per_int - 1) / bp.vals_per_int;
  // every leaf may become a brick: the staging buffer holds one per node (an upper bound)
  uint64_t leaves = 0;
  for (uint32_t li = 0; li < nl; li++) leaves += lv[li].n;
  Buf<uint32_t> slot_of_frame, pos_of_frame, counter, stage_words, out_words;
  Buf<lrt_sbs_node> stage_nodes, out_nodes;
  uint32_t cap = uint32_t(std::min<uint64_t>(leaves, 0xFFFFFFFFull / std::max<uint32_t>(bp.words, 1)));
  // staging sized for the leaves, bounded by 8 GB
  const uint64_t max_stage_words = (8ull << 30) / 4;
  if (uint64_t(cap) * bp.words > max_stage_words) cap = uint32_t(max_stage_words / bp.words);
  if ((e = slot_of_frame.alloc(n_frame)) != cudaSuccess || (e = pos_of_frame.alloc(n_frame)) != cudaSuccess ||
      (e = counter.alloc(1)) != cudaSuccess || (e = stage_words.alloc(size_t(cap) * bp.words)) != cudaSuccess ||
      (e = stage_nodes.alloc(cap)) != cudaSuccess) {
    err = cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? LRT_ERR_OOM : LRT_ERR_CUDA;
  }
  cudaMemsetAsync(slot_of_frame.p, 0, n_frame * 4, st);
  cudaMemsetAsync(counter.p, 0, 4, st);
  const size_t smem = size_t(bp.v3) * 4;
  if (smem > 48 * 1024) cudaFuncSetAttribute(brick_values, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  for (uint32_t li = 0; li < nl; li++) {
    if (lv[li].n == 0) continue;
    const LevelView P = li > 0 ? lv[li - 1].view() : lv[li].view();
    brick_values<<<lv[li].n, 256, smem, st>>>(dsdf.f, lv[li].view(), P, sub_base.p, bp, slot_of_frame.p, counter.p,
                                              stage_words.p, stage_nodes.p, cap);
    if ((e = cudaGetLastError()) != cudaSuccess) { err = cudaGetErrorString(e); return LRT_ERR_CUDA; }
  }
  uint32_t kept = 0;
  if ((e = cudaMemcpy(&kept, counter.p, 4, cudaMemcpyDeviceToHost)) != cudaSuccess) {
    err = cudaGetErrorString(e);
    return LRT_ERR_CUDA;
  }
  if (kept > cap) { err = "more bricks than the staging buffer holds"; return LRT_ERR_OOM; }
  // frame-order positions of the kept bricks
  Buf<uint32_t> nz;
  if ((e = nz.alloc(n_frame)) != cudaSuccess) { err = cudaGetErrorString(e); return LRT_ERR_OOM; }
  nonzero_flags<<<grid(n_frame, 256), 256, 0, st>>>(slot_of_frame.p, nz.p, uint32_t(n_frame));
  uint64_t total = 0;
  if ((e = exclusive_scan(nz.p, pos_of_frame.p, uint32_t(n_frame), &total, st)) != cudaSuccess) {
    err = cudaGetErrorString(e);
    return LRT_ERR_CUDA;
  }
  if ((e = out_nodes.alloc(kept)) != cudaSuccess || (e = out_words.alloc(size_t(kept) * bp.words)) != cudaSuccess) {
    err = cudaGetErrorString(e);
    return LRT_ERR_OOM;
  }
  if (kept) {
    place_bricks<<<std::min<uint64_t>(n_frame, 65535u * 16u), 128, 0, st>>>(
        slot_of_frame.p, pos_of_frame.p, uint32_t(n_frame), stage_nodes.p, stage_words.p, bp.words, out_nodes.p,
        out_words.p);
  }
  out.hdr = hdr;
  out.nodes.resize(kept);
  out.values.resize(size_t(kept) * bp.words);
  if (kept && ((e = cudaMemcpy(out.nodes.data(), out_nodes.p, size_t(kept) * sizeof(lrt_sbs_node),
                               cudaMemcpyDeviceToHost)) != cudaSuccess ||
               (e = cudaMemcpy(out.values.data(), out_words.p, size_t(kept) * bp.words * 4, cudaMemcpyDeviceToHost)) !=
                   cudaSuccess)) {
    err = cudaGetErrorString(e);
    return LRT_ERR_CUDA;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) { err = cudaGetErrorString(e); return LRT_ERR_CUDA; }
  return LRT_OK;
}

// create_sdf_SVS on the GPU (depth >= 4)
lrt_status build_svs_gpu(const lrt_sdf_desc &sd, uint32_t depth, std::vector<lrt_svs_node> &out, std::string &err) {
  const cudaStream_t st = nullptr;
  DevSdf dsdf;
  cudaError_t e = dsdf.upload(sd);
  std::vector<LevelBufs> lv;
  if (e == cudaSuccess) e = grow_levels(dsdf.f, depth, lv, st);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return LRT_ERR_CUDA; }
  const uint32_t nl = uint32_t(lv.size());
  for (int li = int(nl) - 1; li >= 0; li--) {
    const bool has_next = uint32_t(li + 1) < nl;
    svs_count<<<grid(lv[li].n, 256), 256, 0, st>>>(lv[li].view(), has_next ? lv[li + 1].view() : lv[li].view(),
                                                   has_next);
  }
  // level-4 nodes in breadth-first order are the large octree's leaves in depth-first order
  uint64_t total = 0;
  if ((e = exclusive_scan(lv[0].cnt.p, lv[0].rank.p, 4096, &total, st)) != cudaSuccess) {
    err = cudaGetErrorString(e);
    return LRT_ERR_CUDA;
  }
  for (uint32_t li = 0; li + 1 < nl; li++)
    svs_offsets<<<grid(lv[li].n, 256), 256, 0, st>>>(lv[li].view(), lv[li + 1].view());
  Buf<lrt_svs_node> d_out;
  if ((e = d_out.alloc(total)) != cudaSuccess) { err = cudaGetErrorString(e); return LRT_ERR_OOM; }
  for (uint32_t li = 0; li < nl; li++)
    if (lv[li].n) svs_write<<<grid(lv[li].n, 256), 256, 0, st>>>(lv[li].view(), d_out.p);
  out.resize(total);
  if (total && (e = cudaMemcpy(out.data(), d_out.p, total * sizeof(lrt_svs_node), cudaMemcpyDeviceToHost)) != cudaSuccess) {
    err = cudaGetErrorString(e);
    return LRT_ERR_CUDA;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) { err = cudaGetErrorString(e); return LRT_ERR_CUDA; }
  return LRT_OK;
}

cudaError_t gpu_exclusive_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint64_t *total, cudaStream_t st) {
  return exclusive_scan(in, out, n, total, st);
}

}  // namespace lrt
