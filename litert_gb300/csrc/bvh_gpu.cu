// BVH construction and refit on the device.
//
// The reference builds its bottom-level BVH on the host with Embree
// (BVH/cbvh.cpp:591-657, BVH/cbvh_embree2.cpp:287-332) and builds it again from
// scratch every time the brick set changes (diff_render/MultiRendererDR.cpp:
// 228-277, OptimizeGrid).  This unit builds a linear BVH on the device instead:
//   1. bounds of the primitive centroids (warp reductions, order-preserving
//      integer atomics);
//   2. a 30-bit Morton code per centroid, 10 bits per axis inside those bounds;
//   3. a stable least-significant-digit radix sort of (code, primitive id),
//      4 bits per pass, tiles of 2048 keys per block;
//   4. the binary radix tree over the sorted codes, one thread per internal
//      node (T. Karras, "Maximizing Parallelism in the Construction of BVHs,
//      Octrees, and k-d Trees", HPG 2012); equal codes are ordered by their
//      sorted position, so every key is distinct;
//   5. node boxes bottom-up: of the two threads reaching a node, the second
//      merges the children's boxes and climbs on;
//   6. the host builder's 4-wide collapse (open the internal child of largest
//      surface area until a node has four children), one level of the wide
//      tree per pass, wide nodes numbered breadth first as on the host;
//   7. optionally the reference's fat-pair layout, pair i = internal node i
//      (pair 0 is the root, as in BVH/cbvh.h:29-33 BVHNodePair).
// Every leaf holds one primitive (box id, or a one-triangle range of the sorted
// order).  Refit recomputes the slot boxes of an existing wide tree from new
// primitive boxes, deepest level first.
//
// Box unions are exact (min/max); areas follow the host builder's expression,
// so for the same binary tree both collapses pick the same children.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <utility>
#include <vector>

#include "lrt_internal.h"

namespace lrt {
namespace bvhg {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kSortThreads = 256, kSortItems = 8, kSortTile = kSortThreads * kSortItems;

// float <-> unsigned with the same order (for atomicMin / atomicMax)
__device__ __forceinline__ uint32_t ord(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__global__ void bounds_init(uint32_t *ob) {
  if (threadIdx.x < 3) ob[threadIdx.x] = 0xFFFFFFFFu;
  else if (threadIdx.x < 6) ob[threadIdx.x] = 0u;
}

__global__ void centroid_bounds(const float *b6, uint32_t n, uint32_t *ob) {
  float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float c = 0.5f * (b6[6 * size_t(i) + k] + b6[6 * size_t(i) + 3 + k]);
      lo[k] = fminf(lo[k], c);
      hi[k] = fmaxf(hi[k], c);
    }
#pragma unroll
  for (int k = 0; k < 3; k++)
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  if ((threadIdx.x & 31) == 0 && lo[0] <= hi[0])
    for (int k = 0; k < 3; k++) {
      atomicMin(&ob[k], ord(lo[k]));
      atomicMax(&ob[3 + k], ord(hi[k]));
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {   // bit b -> bit 3b
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void morton_codes(const float *b6, uint32_t n, const uint32_t *ob, uint32_t *code, uint32_t *id) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t q[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float lo = unord(ob[k]), ext = unord(ob[3 + k]) - lo;
    const float c = 0.5f * (b6[6 * size_t(i) + k] + b6[6 * size_t(i) + 3 + k]);
    const float x = ext > 0.0f ? (c - lo) / ext : 0.0f;
    q[k] = uint32_t(min(max(int(x * 1024.0f), 0), 1023));
  }
  code[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  id[i] = i;
}

// ---- stable radix sort pass: digit counts per tile, then a stable scatter ----
__global__ void __launch_bounds__(kSortThreads) radix_count(const uint32_t *key, uint32_t n, uint32_t shift,
                                                            uint32_t nblk, uint32_t *hist) {
  __shared__ uint32_t c[16];
  if (threadIdx.x < 16) c[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * kSortTile;
  for (uint32_t k = threadIdx.x; k < kSortTile; k += kSortThreads)
    if (base + k < n) atomicAdd(&c[(key[base + k] >> shift) & 15u], 1u);
  __syncthreads();
  if (threadIdx.x < 16) hist[threadIdx.x * nblk + blockIdx.x] = c[threadIdx.x];
}

// Each thread owns 8 consecutive keys of the tile.  Per-digit counts are packed
// two 16-bit lanes to a word (a tile holds at most 2048 keys, so no lane
// carries into the next); a block-wide exclusive scan of the packed counts
// gives each thread the number of equal digits ahead of it in the tile.
__global__ void __launch_bounds__(kSortThreads) radix_scatter(const uint32_t *kin, const uint32_t *vin, uint32_t *kout,
                                                              uint32_t *vout, uint32_t n, uint32_t shift,
                                                              uint32_t nblk, const uint32_t *offs) {
  __shared__ uint32_t goff[16];
  __shared__ uint32_t wtot[kSortThreads / 32][8];
  if (threadIdx.x < 16) goff[threadIdx.x] = offs[threadIdx.x * nblk + blockIdx.x];
  const uint32_t base = blockIdx.x * kSortTile + threadIdx.x * kSortItems;
  uint32_t k[kSortItems], v[kSortItems], cnt[8];
#pragma unroll
  for (int w = 0; w < 8; w++) cnt[w] = 0;
#pragma unroll
  for (uint32_t j = 0; j < kSortItems; j++) {
    k[j] = 0;
    v[j] = 0;
    if (base + j < n) {
      k[j] = kin[base + j];
      v[j] = vin[base + j];
      const uint32_t d = (k[j] >> shift) & 15u, inc = 1u << ((d & 1u) * 16u);
#pragma unroll
      for (uint32_t w = 0; w < 8; w++) cnt[w] += (w == (d >> 1)) ? inc : 0u;
    }
  }
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t incl[8];
#pragma unroll
  for (int w = 0; w < 8; w++) incl[w] = cnt[w];
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
#pragma unroll
    for (int w = 0; w < 8; w++) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl[w], o);
      if (lane >= uint32_t(o)) incl[w] += t;
    }
  if (lane == 31)
#pragma unroll
    for (int w = 0; w < 8; w++) wtot[wid][w] = incl[w];
  __syncthreads();
  uint32_t pre[8];
#pragma unroll
  for (int w = 0; w < 8; w++) {
    uint32_t s = 0;
    for (uint32_t x = 0; x < wid; x++) s += wtot[x][w];
    pre[w] = s + incl[w] - cnt[w];
  }
#pragma unroll
  for (uint32_t j = 0; j < kSortItems; j++) {
    if (base + j >= n) continue;
    const uint32_t d = (k[j] >> shift) & 15u, sh = (d & 1u) * 16u;
    uint32_t word = 0;
#pragma unroll
    for (uint32_t w = 0; w < 8; w++) word = (w == (d >> 1)) ? pre[w] : word;
    const uint32_t pos = goff[d] + ((word >> sh) & 0xFFFFu);
    kout[pos] = k[j];
    vout[pos] = v[j];
#pragma unroll
    for (uint32_t w = 0; w < 8; w++) pre[w] += (w == (d >> 1)) ? (1u << sh) : 0u;
  }
}

// ---- binary radix tree (Karras 2012, algorithm of section 4) ----
// Length of the common prefix of keys i and j, -1 outside [0, n).  Equal codes
// continue with the bits of the positions.
__device__ __forceinline__ int prefix(const uint32_t *code, int64_t n, int64_t i, int64_t j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = code[i], b = code[j];
  if (a != b) return __clz(a ^ b);
  return 32 + __clz(uint32_t(i ^ j));
}

__global__ void radix_tree(const uint32_t *code, uint32_t n, uint32_t *child, uint32_t *parent_int,
                           uint32_t *parent_leaf) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t nn = n;
  if (i >= nn - 1) return;
  if (i == 0) parent_int[0] = kNone;
  const int d = prefix(code, nn, i, i + 1) > prefix(code, nn, i, i - 1) ? 1 : -1;
  const int pmin = prefix(code, nn, i, i - d);
  int64_t lmax = 2;
  while (prefix(code, nn, i, i + lmax * d) > pmin) lmax <<= 1;
  int64_t l = 0;
  for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
    if (prefix(code, nn, i, i + (l + t) * d) > pmin) l += t;
  const int64_t j = i + l * d;
  const int pnode = prefix(code, nn, i, j);
  int64_t s = 0;
  for (int64_t div = 2;; div <<= 1) {
    const int64_t t = (l + div - 1) / div;
    if (prefix(code, nn, i, i + (s + t) * d) > pnode) s += t;
    if (t <= 1) break;
  }
  const int64_t g = i + s * d + (d < 0 ? -1 : 0);
  const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
  const uint32_t left = lo == g ? (kLeafBit | uint32_t(g)) : uint32_t(g);
  const uint32_t right = hi == g + 1 ? (kLeafBit | uint32_t(g + 1)) : uint32_t(g + 1);
  child[2 * i] = left;
  child[2 * i + 1] = right;
  if (left & kLeafBit) parent_leaf[g] = uint32_t(i); else parent_int[g] = uint32_t(i);
  if (right & kLeafBit) parent_leaf[g + 1] = uint32_t(i); else parent_int[g + 1] = uint32_t(i);
}

struct Box {
  float lo[3], hi[3];
};
__device__ __forceinline__ Box prim_box(const float *b6, uint32_t p) {
  Box b;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    b.lo[k] = b6[6 * size_t(p) + k];
    b.hi[k] = b6[6 * size_t(p) + 3 + k];
  }
  return b;
}
__device__ __forceinline__ Box node_box(const float *nb, uint32_t c) {   // written by another thread: L2 loads
  Box b;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    b.lo[k] = __ldcg(nb + 6 * size_t(c) + k);
    b.hi[k] = __ldcg(nb + 6 * size_t(c) + 3 + k);
  }
  return b;
}
__device__ __forceinline__ Box child_box(const float *b6, const uint32_t *sid, const float *nb, uint32_t c) {
  return (c & kLeafBit) ? prim_box(b6, sid[c & ~kLeafBit]) : node_box(nb, c);
}

// One thread per leaf climbs towards the root; the first thread to reach a node
// stops there, the second (which sees both children finished) writes its box.
__global__ void node_boxes(const float *b6, const uint32_t *sid, uint32_t n, const uint32_t *child,
                           const uint32_t *parent_int, const uint32_t *parent_leaf, float *nb, uint32_t *visits,
                           uint32_t *err) {
  const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= n) return;
  uint32_t p = parent_leaf[leaf];
  for (uint32_t it = 0; p != kNone; it++) {
    if (it >= n || p >= n - 1) {   // a parent chain longer than the tree: never for a valid tree
      atomicOr(err, 1u);
      return;
    }
    __threadfence();
    if (atomicAdd(&visits[p], 1u) == 0) return;
    __threadfence();
    const Box a = child_box(b6, sid, nb, child[2 * p]), b = child_box(b6, sid, nb, child[2 * p + 1]);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      __stcg(nb + 6 * size_t(p) + k, fminf(a.lo[k], b.lo[k]));
      __stcg(nb + 6 * size_t(p) + 3 + k, fmaxf(a.hi[k], b.hi[k]));
    }
    p = parent_int[p];
  }
}

// ---- leaves of the radix tree in the common BVH2 form ----
// Leaf i (sorted position i) holds primitive sid[i]: its box, and the payload a
// wide node stores for it (box id, or a one-triangle range of the sorted order).
__global__ void lbvh_leaves(const float *b6, const uint32_t *sid, uint32_t n, bool boxes, float *lbox,
                            uint32_t *lpay) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t p = sid[i];
#pragma unroll
  for (int k = 0; k < 6; k++) lbox[6 * size_t(i) + k] = b6[6 * size_t(p) + k];
  lpay[i] = boxes ? (kLeafBit | p) : (kLeafBit | (1u << 24) | i);
}

// ---- exact binned SAH, one tree level per pass (the host builder restated) ----
// Segment k of a level is the primitive range [seg_b, seg_e) of `order` under
// one BVH2 node.  A block per segment: box and centroid bounds, the 32 bins of
// every axis with a non-zero centroid extent (the host's expressions), the cost
// sweep on one thread in the host's order, and a stable partition (or the object
// median by (centroid, id) when no split is found or below depth 40).  The tree's
// shape depends only on these sets, so it is the host builder's tree.
constexpr int kNB = 32;
constexpr uint32_t kSahThreads = 128;
constexpr uint32_t kMedianMax = 4096;   // larger median-fallback segments go back to the host builder
constexpr uint32_t kBigMin = 16384;     // node ranges at least this large are split by many blocks
constexpr uint32_t kBigMaxSegs = 64;    // ... looked for on levels of at most this many ranges

__device__ __forceinline__ float fmn(float a, float b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ float fmx(float a, float b) { return (a < b) ? b : a; }   // std::max
__device__ __forceinline__ float area6(const float lo[3], const float hi[3]) {
  const float dx = fmx(0.0f, hi[0] - lo[0]), dy = fmx(0.0f, hi[1] - lo[1]), dz = fmx(0.0f, hi[2] - lo[2]);
  return 2.0f * (dx * dy + dy * dz + dz * dx);
}

__global__ void centroids(const float *b6, uint32_t n, float *cent, uint32_t *order) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int k = 0; k < 3; k++) cent[3 * size_t(i) + k] = 0.5f * (b6[6 * size_t(i) + k] + b6[6 * size_t(i) + 3 + k]);
  order[i] = i;
}

// block-wide min of v[0..5] and max of v[6..11] (12 values), result in out[12]
__device__ void block_minmax12(float v[12], float *sh /* [kSahThreads/32][12] */, float out[12]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 12; k++)
    for (int o = 16; o > 0; o >>= 1) {
      const float u = __shfl_xor_sync(0xffffffffu, v[k], o);
      v[k] = k < 6 ? fminf(v[k], u) : fmaxf(v[k], u);
    }
  if (lane == 0)
    for (int k = 0; k < 12; k++) sh[w * 12 + k] = v[k];
  __syncthreads();
  for (int k = 0; k < 12; k++) {
    float r = sh[k];
    for (uint32_t x = 1; x < kSahThreads / 32; x++) r = k < 6 ? fminf(r, sh[x * 12 + k]) : fmaxf(r, sh[x * 12 + k]);
    out[k] = r;
  }
  __syncthreads();
}

// The cost sweep of Builder::split over the bins of one node range (bl / bh:
// [3][kNB][3] ordered box bounds, bc: [3][kNB] counts, shared or global memory),
// in the host's order; no split (or below depth 40: use all false) selects the
// object median on the widest centroid axis.
__device__ void sah_sweep(const uint32_t *bl, const uint32_t *bh, const uint32_t *bc, const bool use[3],
                          const float cl[3], const float ch[3], uint32_t m, int &axis, int &bin, int &median,
                          uint32_t &nleft) {
  float best_cost = 3.4e38f;
  int best_axis = -1, best_bin = -1;
  for (int a = 0; a < 3; a++) {
    if (!use[a]) continue;
    float rA[kNB];
    uint32_t rN[kNB];
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    uint32_t cnt = 0;
    for (int i = kNB - 1; i > 0; i--) {
      for (int c = 0; c < 3; c++) {
        lo[c] = fmn(lo[c], unord(bl[(a * kNB + i) * 3 + c]));
        hi[c] = fmx(hi[c], unord(bh[(a * kNB + i) * 3 + c]));
      }
      cnt += bc[a * kNB + i];
      rA[i] = area6(lo, hi);
      rN[i] = cnt;
    }
    for (int c = 0; c < 3; c++) { lo[c] = 3.4e38f; hi[c] = -3.4e38f; }
    cnt = 0;
    for (int i = 0; i < kNB - 1; i++) {
      for (int c = 0; c < 3; c++) {
        lo[c] = fmn(lo[c], unord(bl[(a * kNB + i) * 3 + c]));
        hi[c] = fmx(hi[c], unord(bh[(a * kNB + i) * 3 + c]));
      }
      cnt += bc[a * kNB + i];
      if (cnt == 0 || rN[i + 1] == 0) continue;
      const float cost = area6(lo, hi) * float(cnt) + rA[i + 1] * float(rN[i + 1]);
      if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = i; }
    }
  }
  median = best_axis < 0;
  if (best_axis < 0) {
    int ax = 0;
    for (int c = 1; c < 3; c++) if (ch[c] - cl[c] > ch[ax] - cl[ax]) ax = c;
    best_axis = ax;
    nleft = m / 2;
  } else {
    uint32_t nl = 0;
    for (int i = 0; i <= best_bin; i++) nl += bc[best_axis * kNB + i];
    nleft = nl;
  }
  axis = best_axis;
  bin = best_bin;
}

__global__ void __launch_bounds__(kSahThreads) sah_level(const float *b6, const float *cent, uint32_t *order,
                                                         uint32_t *tmp, uint32_t *rank, const uint32_t *seg_b,
                                                         const uint32_t *seg_e,
                                                         uint32_t depth, uint32_t max_leaf, float *seg_box,
                                                         uint32_t *seg_split, uint32_t *seg_flag, uint32_t *err,
                                                         uint32_t big_min) {
  __shared__ float red[kSahThreads / 32 * 12];
  __shared__ uint32_t bl[3][kNB][3], bh[3][kNB][3], bc[3][kNB];
  __shared__ int s_axis, s_bin, s_median;
  __shared__ uint32_t s_nleft, s_run, s_wsum[kSahThreads / 32];
  const uint32_t k = blockIdx.x, b = seg_b[k], e = seg_e[k], m = e - b, tid = threadIdx.x;
  if (m >= big_min) return;   // done by the multi-block path (sah_big_*)
  // 1. node box and centroid bounds
  float v[12];
  for (int q = 0; q < 6; q++) { v[q] = 3.4e38f; v[6 + q] = -3.4e38f; }
  for (uint32_t i = b + tid; i < e; i += kSahThreads) {
    const uint32_t p = order[i];
    for (int a = 0; a < 3; a++) {
      v[a] = fminf(v[a], b6[6 * size_t(p) + a]);
      v[6 + a] = fmaxf(v[6 + a], b6[6 * size_t(p) + 3 + a]);
      v[3 + a] = fminf(v[3 + a], cent[3 * size_t(p) + a]);
      v[9 + a] = fmaxf(v[9 + a], cent[3 * size_t(p) + a]);
    }
  }
  float r[12];
  block_minmax12(v, red, r);   // r: box lo 0-2, cb lo 3-5, box hi 6-8, cb hi 9-11
  if (tid == 0) {
    for (int a = 0; a < 3; a++) { seg_box[6 * size_t(k) + a] = r[a]; seg_box[6 * size_t(k) + 3 + a] = r[6 + a]; }
    seg_flag[k] = m > max_leaf ? 1u : 0u;
  }
  if (m <= max_leaf) return;
  const float cl[3] = {r[3], r[4], r[5]}, ch[3] = {r[9], r[10], r[11]};
  float sc[3];
  bool use[3];
  for (int a = 0; a < 3; a++) {
    const float ext = ch[a] - cl[a];
    use[a] = depth < 40 && ext > 0;
    sc[a] = use[a] ? kNB / ext : 0.0f;
  }
  // 2. bins: counts and boxes (ordered-integer atomics; empty bins stay the reset box)
  for (uint32_t q = tid; q < 3 * kNB; q += kSahThreads) {
    const uint32_t a = q / kNB, i = q % kNB;
    bc[a][i] = 0;
    for (int c = 0; c < 3; c++) { bl[a][i][c] = ord(3.4e38f); bh[a][i][c] = ord(-3.4e38f); }
  }
  __syncthreads();
  for (uint32_t i = b + tid; i < e; i += kSahThreads) {
    const uint32_t p = order[i];
    for (int a = 0; a < 3; a++) {
      if (!use[a]) continue;
      int bi = int((cent[3 * size_t(p) + a] - cl[a]) * sc[a]);
      bi = min(max(bi, 0), kNB - 1);
      atomicAdd(&bc[a][bi], 1u);
      for (int c = 0; c < 3; c++) {
        atomicMin(&bl[a][bi][c], ord(b6[6 * size_t(p) + c]));
        atomicMax(&bh[a][bi][c], ord(b6[6 * size_t(p) + 3 + c]));
      }
    }
  }
  __syncthreads();
  // 3. cost sweep (Builder::split), one thread
  if (tid == 0) {
    int best_axis, best_bin, med;
    uint32_t nl;
    sah_sweep(&bl[0][0][0], &bh[0][0][0], &bc[0][0], use, cl, ch, m, best_axis, best_bin, med, nl);
    s_median = med;
    s_nleft = nl;
    s_axis = best_axis;
    s_bin = best_bin;
    s_run = 0;
  }
  __syncthreads();
  const int ax = s_axis, bin = s_bin;
  const bool median = s_median;
  const uint32_t nleft = s_nleft;
  if (median && m > kMedianMax) {   // too large for the quadratic rank below: the caller builds on the host
    if (tid == 0) {
      atomicOr(err, 1u);
      seg_flag[k] = 0;   // closed as a leaf so the level stays well formed
    }
    return;
  }
  // median: rank of every element by (centroid, id) among the segment
  if (median) {
    for (uint32_t i = b + tid; i < e; i += kSahThreads) {
      const uint32_t p = order[i];
      const float cp = cent[3 * size_t(p) + ax];
      uint32_t r = 0;
      for (uint32_t j = b; j < e; j++) {
        const uint32_t q = order[j];
        const float cq = cent[3 * size_t(q) + ax];
        r += (cq < cp || (cq == cp && q < p)) ? 1u : 0u;
      }
      rank[i] = r;
    }
    __syncthreads();
  }
  // 4. stable partition into tmp, chunk by chunk, then back into order
  const uint32_t lane = tid & 31, w = tid >> 5;
  for (uint32_t base = b; base < e; base += kSahThreads) {
    const uint32_t i = base + tid;
    bool in = i < e, left = false;
    uint32_t p = 0;
    if (in) {
      p = order[i];
      if (median) {
        left = rank[i] < nleft;
      } else {
        int bi = int((cent[3 * size_t(p) + ax] - cl[ax]) * sc[ax]);
        bi = min(max(bi, 0), kNB - 1);
        left = bi <= bin;
      }
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, in && left);
    if (lane == 0) s_wsum[w] = __popc(bal);
    __syncthreads();
    uint32_t before = s_run, chunk_left = 0;
    for (uint32_t x = 0; x < kSahThreads / 32; x++) {
      if (x < w) before += s_wsum[x];
      chunk_left += s_wsum[x];
    }
    before += __popc(bal & ((1u << lane) - 1u));
    __syncthreads();
    if (in) {   // left: slot b + (lefts before it); right: slot b + nleft + (rights before it)
      const uint32_t pos = left ? b + before : b + nleft + ((i - b) - before);
      tmp[pos] = p;
    }
    if (tid == 0) s_run += chunk_left;
    __syncthreads();
  }
  for (uint32_t i = b + tid; i < e; i += kSahThreads) order[i] = tmp[i];
  if (tid == 0) seg_split[k] = b + nleft;
}

// ---- the same split for one large node range, spread over many blocks ----
// Scratch layout (words): [0, 12) ordered bounds (box lo, centroid lo: min; box hi,
// centroid hi: max), then bin lows [3][kNB][3], bin highs [3][kNB][3], bin counts
// [3][kNB], then the sweep's axis, bin, median flag and left count.
constexpr uint32_t kBigBL = 12, kBigBH = kBigBL + 3 * kNB * 3, kBigBC = kBigBH + 3 * kNB * 3,
                   kBigRes = kBigBC + 3 * kNB, kBigWords = kBigRes + 4;

__global__ void sah_big_init(uint32_t *sc) {
  for (uint32_t i = threadIdx.x; i < kBigWords; i += blockDim.x) {
    uint32_t v = 0;
    if (i < 6) v = 0xFFFFFFFFu;
    else if (i < 12) v = 0u;
    else if (i < kBigBH) v = ord(3.4e38f);
    else if (i < kBigBC) v = ord(-3.4e38f);
    sc[i] = v;
  }
}

__global__ void sah_big_bounds(const float *b6, const float *cent, const uint32_t *order, uint32_t b, uint32_t e,
                               uint32_t *sc) {
  float v[12];
  for (int q = 0; q < 6; q++) { v[q] = 3.4e38f; v[6 + q] = -3.4e38f; }
  for (uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
    const uint32_t p = order[i];
    for (int a = 0; a < 3; a++) {
      v[a] = fminf(v[a], b6[6 * size_t(p) + a]);
      v[6 + a] = fmaxf(v[6 + a], b6[6 * size_t(p) + 3 + a]);
      v[3 + a] = fminf(v[3 + a], cent[3 * size_t(p) + a]);
      v[9 + a] = fmaxf(v[9 + a], cent[3 * size_t(p) + a]);
    }
  }
  for (int q = 0; q < 12; q++)
    for (int o = 16; o > 0; o >>= 1) {
      const float u = __shfl_xor_sync(0xffffffffu, v[q], o);
      v[q] = q < 6 ? fminf(v[q], u) : fmaxf(v[q], u);
    }
  if ((threadIdx.x & 31) == 0 && v[0] <= v[6])
    for (int q = 0; q < 12; q++) {
      if (q < 6) atomicMin(&sc[q], ord(v[q]));
      else atomicMax(&sc[q], ord(v[q]));
    }
}

__device__ __forceinline__ void big_axes(const uint32_t *sc, uint32_t depth, float cl[3], float ch[3], bool use[3],
                                         float scl[3]) {
  for (int a = 0; a < 3; a++) {
    cl[a] = unord(sc[3 + a]);
    ch[a] = unord(sc[9 + a]);
    const float ext = ch[a] - cl[a];
    use[a] = depth < 40 && ext > 0;
    scl[a] = use[a] ? kNB / ext : 0.0f;
  }
}

__global__ void __launch_bounds__(256) sah_big_bins(const float *b6, const float *cent, const uint32_t *order,
                                                    uint32_t b, uint32_t e, uint32_t depth, uint32_t *sc) {
  __shared__ uint32_t bl[3 * kNB * 3], bh[3 * kNB * 3], bc[3 * kNB];
  float cl[3], ch[3], scl[3];
  bool use[3];
  big_axes(sc, depth, cl, ch, use, scl);
  for (uint32_t q = threadIdx.x; q < 3 * kNB * 3; q += blockDim.x) { bl[q] = ord(3.4e38f); bh[q] = ord(-3.4e38f); }
  for (uint32_t q = threadIdx.x; q < 3 * kNB; q += blockDim.x) bc[q] = 0;
  __syncthreads();
  for (uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
    const uint32_t p = order[i];
    for (int a = 0; a < 3; a++) {
      if (!use[a]) continue;
      int bi = int((cent[3 * size_t(p) + a] - cl[a]) * scl[a]);
      bi = min(max(bi, 0), kNB - 1);
      atomicAdd(&bc[a * kNB + bi], 1u);
      for (int c = 0; c < 3; c++) {
        atomicMin(&bl[(a * kNB + bi) * 3 + c], ord(b6[6 * size_t(p) + c]));
        atomicMax(&bh[(a * kNB + bi) * 3 + c], ord(b6[6 * size_t(p) + 3 + c]));
      }
    }
  }
  __syncthreads();
  for (uint32_t q = threadIdx.x; q < 3 * kNB; q += blockDim.x) {
    if (bc[q] == 0) continue;
    atomicAdd(&sc[kBigBC + q], bc[q]);
    for (int c = 0; c < 3; c++) {
      atomicMin(&sc[kBigBL + q * 3 + c], bl[q * 3 + c]);
      atomicMax(&sc[kBigBH + q * 3 + c], bh[q * 3 + c]);
    }
  }
}

__global__ void sah_big_sweep(uint32_t k, uint32_t b, uint32_t e, uint32_t depth, uint32_t *sc, float *seg_box,
                              uint32_t *seg_split, uint32_t *seg_flag, uint32_t *err) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float cl[3], ch[3], scl[3];
  bool use[3];
  big_axes(sc, depth, cl, ch, use, scl);
  int axis, bin, median;
  uint32_t nleft;
  sah_sweep(sc + kBigBL, sc + kBigBH, sc + kBigBC, use, cl, ch, e - b, axis, bin, median, nleft);
  for (int a = 0; a < 3; a++) {
    seg_box[6 * size_t(k) + a] = unord(sc[a]);
    seg_box[6 * size_t(k) + 3 + a] = unord(sc[6 + a]);
  }
  sc[kBigRes + 0] = uint32_t(axis);
  sc[kBigRes + 1] = uint32_t(bin);
  sc[kBigRes + 2] = uint32_t(median);
  sc[kBigRes + 3] = nleft;
  if (median) {   // an object median this large: the caller builds on the host
    atomicOr(err, 1u);
    seg_flag[k] = 0;
    return;
  }
  seg_flag[k] = 1;
  seg_split[k] = b + nleft;
}

__global__ void sah_big_flags(const float *cent, const uint32_t *order, uint32_t b, uint32_t e, uint32_t depth,
                              const uint32_t *sc, uint32_t *flag) {
  if (sc[kBigRes + 2]) return;
  float cl[3], ch[3], scl[3];
  bool use[3];
  big_axes(sc, depth, cl, ch, use, scl);
  const int ax = int(sc[kBigRes + 0]), bin = int(sc[kBigRes + 1]);
  for (uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
    const uint32_t p = order[i];
    int bi = int((cent[3 * size_t(p) + ax] - cl[ax]) * scl[ax]);
    bi = min(max(bi, 0), kNB - 1);
    flag[i - b] = bi <= bin ? 1u : 0u;
  }
}

__global__ void sah_big_scatter(const uint32_t *order, uint32_t b, uint32_t e, const uint32_t *sc,
                                const uint32_t *flag, const uint32_t *excl, uint32_t *tmp) {
  if (sc[kBigRes + 2]) return;
  const uint32_t nleft = sc[kBigRes + 3];
  for (uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
    const uint32_t o = i - b, before = excl[o];
    tmp[flag[o] ? b + before : b + nleft + (o - before)] = order[i];
  }
}

__global__ void sah_big_copy(uint32_t *order, const uint32_t *tmp, uint32_t b, uint32_t e, const uint32_t *sc) {
  if (sc[kBigRes + 2]) return;
  for (uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) order[i] = tmp[i];
}

// After a level's scan of seg_flag: internal nodes and leaves get their ids (level
// order, the host builder's breadth-first pair order), parents learn their
// children, split segments emit their two halves for the next level.
__global__ void sah_link(uint32_t nseg, const uint32_t *seg_b, const uint32_t *seg_e, const uint32_t *seg_parent,
                         const float *seg_box, const uint32_t *seg_split, const uint32_t *seg_flag,
                         const uint32_t *excl, uint32_t int_base, uint32_t leaf_base, const uint32_t *order,
                         bool boxes, uint32_t *child, float *ibox, float *lbox, uint32_t *lpay, uint32_t *nb_,
                         uint32_t *ne_, uint32_t *np_) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nseg) return;
  const uint32_t b = seg_b[k], e = seg_e[k];
  uint32_t ref;
  if (seg_flag[k]) {
    const uint32_t q = int_base + excl[k];
    ref = q;
    for (int c = 0; c < 6; c++) ibox[6 * size_t(q) + c] = seg_box[6 * size_t(k) + c];
    const uint32_t j = 2 * excl[k], m = seg_split[k];
    nb_[j] = b; ne_[j] = m; np_[j] = 2 * q;
    nb_[j + 1] = m; ne_[j + 1] = e; np_[j + 1] = 2 * q + 1;
  } else {
    const uint32_t l = leaf_base + (k - excl[k]);
    ref = kLeafBit | l;
    for (int c = 0; c < 6; c++) lbox[6 * size_t(l) + c] = seg_box[6 * size_t(k) + c];
    lpay[l] = boxes ? (kLeafBit | order[b]) : (kLeafBit | (((e - b) & 0x7Fu) << 24) | (b & 0x00FFFFFFu));
  }
  if (seg_parent[k] != kNone) child[seg_parent[k]] = ref;
}

// ---- collapse into 4-wide nodes, one wide level per pass (the host builder's) ----
// child: 2 per internal node, internal id or kLeafBit | leaf id; ibox / lbox:
// 6 floats per internal node / leaf; lpay: the leaf's wide-node payload.
__global__ void collapse_pick(const uint32_t *front, uint32_t nf, const uint32_t *child, const float *ibox,
                              uint32_t *pick, uint32_t *n_internal) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nf) return;
  const uint32_t r = front[k];
  uint32_t ch[4] = {kEmptyChild, kEmptyChild, kEmptyChild, kEmptyChild};
  int nc = 0;
  if (r & kLeafBit) {
    ch[nc++] = r;
  } else {
    ch[nc++] = child[2 * r];
    ch[nc++] = child[2 * r + 1];
    while (nc < 4) {   // open the internal child with the largest surface area (first on ties)
      int best = -1;
      float best_a = -1.0f;
      for (int i = 0; i < nc; i++)
        if (!(ch[i] & kLeafBit)) {
          float lo[3], hi[3];
          for (int c = 0; c < 3; c++) { lo[c] = ibox[6 * size_t(ch[i]) + c]; hi[c] = ibox[6 * size_t(ch[i]) + 3 + c]; }
          const float a = area6(lo, hi);
          if (a > best_a) {
            best_a = a;
            best = i;
          }
        }
      if (best < 0) break;
      const uint32_t x = ch[best];
      ch[best] = child[2 * x];
      ch[nc++] = child[2 * x + 1];
    }
  }
  uint32_t m = 0;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    pick[4 * size_t(k) + i] = ch[i];
    m += (ch[i] != kEmptyChild && !(ch[i] & kLeafBit)) ? 1u : 0u;
  }
  n_internal[k] = m;
}

__global__ void collapse_write(const uint32_t *pick, uint32_t nf, const uint32_t *off, uint32_t level_base,
                               uint32_t next_base, const float *ibox, const float *lbox, const uint32_t *lpay,
                               WNode4 *wn, uint32_t *next_front) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nf) return;
  WNode4 w;
  uint32_t j = 0;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const uint32_t c = pick[4 * size_t(k) + i];
    w.pad[i] = 0;
    if (c == kEmptyChild) {   // a point box far beyond any ray's tFar, never entered
      w.lo_x[i] = w.lo_y[i] = w.lo_z[i] = 1e30f;
      w.hi_x[i] = w.hi_y[i] = w.hi_z[i] = 1e30f;
      w.child[i] = kEmptyChild;
      continue;
    }
    const bool leaf = (c & kLeafBit) != 0;
    const uint32_t id = c & ~kLeafBit;
    const float *bx = leaf ? lbox + 6 * size_t(id) : ibox + 6 * size_t(id);
    w.lo_x[i] = bx[0]; w.lo_y[i] = bx[1]; w.lo_z[i] = bx[2];
    w.hi_x[i] = bx[3]; w.hi_y[i] = bx[4]; w.hi_z[i] = bx[5];
    if (leaf) {
      w.child[i] = lpay[id];
    } else {
      w.child[i] = next_base + off[k] + j;
      next_front[off[k] + j] = c;
      j++;
    }
  }
  wn[level_base + k] = w;
}

// ---- reference fat-pair layout: pair i holds the two children of internal node i ----
// (breadth-first over internal nodes, leaves numbered in the same order, as
// BVH/cbvh_fat.cpp:100-142 numbers them)
__device__ __forceinline__ void pair_side(lrt_bvh_node &s, uint32_t c, const float *ibox, const float *lbox,
                                          const uint32_t *lpay, bool boxes, uint32_t *lsc) {
  const bool leaf = (c & kLeafBit) != 0;
  const uint32_t id = c & ~kLeafBit;
  const float *bx = leaf ? lbox + 6 * size_t(id) : ibox + 6 * size_t(id);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s.boxMin[k] = bx[k];
    s.boxMax[k] = bx[3 + k];
  }
  s.escapeIndex = 0;
  if (leaf) {
    if (boxes) {
      s.leftOffset = kLeafBit | (1u << 24) | ((lpay[id] & ~kLeafBit) & 0x00FFFFFFu);
    } else {
      s.leftOffset = kLeafBit | (1u << 24) | (id & 0x00FFFFFFu);
      if (lsc) lsc[id] = lpay[id];
    }
  } else {
    s.leftOffset = c;
  }
}

__global__ void fat_pairs(uint32_t n_int, uint32_t root, const uint32_t *child, const float *ibox, const float *lbox,
                          const uint32_t *lpay, bool boxes, lrt_bvh_pair *pairs, uint32_t *lsc) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (root & kLeafBit) {   // a single leaf: both sides are the root leaf
    if (i == 0) {
      pair_side(pairs[0].left, root, ibox, lbox, lpay, boxes, lsc);
      pairs[0].right = pairs[0].left;
    }
    return;
  }
  if (i >= n_int) return;
  pair_side(pairs[i].left, child[2 * i], ibox, lbox, lpay, boxes, lsc);
  pair_side(pairs[i].right, child[2 * i + 1], ibox, lbox, lpay, boxes, lsc);
}

// ---- refit of a wide tree, one level (deepest first) ----
__global__ void refit_level(WNode4 *wn, uint32_t first, uint32_t count, const float *b6, const uint32_t *order,
                            bool boxes) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  WNode4 &w = wn[first + k];
  for (int i = 0; i < 4; i++) {
    const uint32_t c = w.child[i];
    if (c == kEmptyChild) continue;
    Box b;
    if (c & kLeafBit) {
      if (boxes) {
        b = prim_box(b6, c & ~kLeafBit);
      } else {
        const uint32_t cnt = (c >> 24) & 0x7Fu, start = c & 0x00FFFFFFu;
        b = prim_box(b6, order ? order[start] : start);
        for (uint32_t q = 1; q < cnt; q++) {
          const Box e = prim_box(b6, order ? order[start + q] : start + q);
#pragma unroll
          for (int a = 0; a < 3; a++) {
            b.lo[a] = fminf(b.lo[a], e.lo[a]);
            b.hi[a] = fmaxf(b.hi[a], e.hi[a]);
          }
        }
      }
    } else {
      const WNode4 &x = wn[c];
      b.lo[0] = b.lo[1] = b.lo[2] = 3.4e38f;
      b.hi[0] = b.hi[1] = b.hi[2] = -3.4e38f;
      for (int q = 0; q < 4; q++) {
        if (x.child[q] == kEmptyChild) continue;
        b.lo[0] = fminf(b.lo[0], x.lo_x[q]); b.hi[0] = fmaxf(b.hi[0], x.hi_x[q]);
        b.lo[1] = fminf(b.lo[1], x.lo_y[q]); b.hi[1] = fmaxf(b.hi[1], x.hi_y[q]);
        b.lo[2] = fminf(b.lo[2], x.lo_z[q]); b.hi[2] = fmaxf(b.hi[2], x.hi_z[q]);
      }
    }
    w.lo_x[i] = b.lo[0]; w.lo_y[i] = b.lo[1]; w.lo_z[i] = b.lo[2];
    w.hi_x[i] = b.hi[0]; w.hi_y[i] = b.hi[1]; w.hi_z[i] = b.hi[2];
  }
}

// triangle boxes of the sorted triangle array (3 float4 vertices per triangle)
__global__ void triangle_boxes(const float4 *tv, uint32_t n, float *b6) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float4 a = tv[3 * size_t(t)], b = tv[3 * size_t(t) + 1], c = tv[3 * size_t(t) + 2];
  float *o = b6 + 6 * size_t(t);
  o[0] = fminf(fminf(a.x, b.x), c.x); o[1] = fminf(fminf(a.y, b.y), c.y); o[2] = fminf(fminf(a.z, b.z), c.z);
  o[3] = fmaxf(fmaxf(a.x, b.x), c.x); o[4] = fmaxf(fmaxf(a.y, b.y), c.y); o[5] = fmaxf(fmaxf(a.z, b.z), c.z);
}

// gather the vertices of each sorted triangle from the indexed mesh
__global__ void gather_triangles(const float4 *vpos, const uint32_t *indices, const uint32_t *order, uint32_t n,
                                 float4 *tv) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const uint32_t t = order[r];
#pragma unroll
  for (int v = 0; v < 3; v++) tv[3 * size_t(r) + v] = vpos[indices[3 * size_t(t) + v]];
}

}  // namespace bvhg

namespace {

using namespace bvhg;

inline unsigned blocks(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

template <typename T>
struct Tmp {
  T *p = nullptr;
  cudaError_t alloc(size_t n, cudaStream_t st) { return cudaMallocAsync(&p, (n ? n : 1) * sizeof(T), st); }
  cudaStream_t st = nullptr;
  ~Tmp() {
    if (p) cudaFreeAsync(p, st);
  }
};

}  // namespace

#define LRT_TRY(x)                          \
  do {                                      \
    cudaError_t e_ = (x);                   \
    if (e_ != cudaSuccess) return e_;       \
  } while (0)

cudaError_t build_bvh_gpu(const float *d_boxes6, uint32_t n, bool boxes, bool sah, WNode4 *d_wnodes,
                          uint32_t *d_order, lrt_bvh_pair *d_pairs, uint32_t *d_leaf_start_count, GpuBvhInfo &info,
                          cudaStream_t st) {
  info = GpuBvhInfo{};
  if (n == 0) return cudaErrorInvalidValue;
  const uint32_t n_cap = n > 1 ? n - 1 : 1;   // internal nodes at most
  // the BVH2 in common form
  Tmp<uint32_t> child, lpay, sidb, err;
  Tmp<float> ibox, lbox;
  for (auto *t : {&child, &lpay, &sidb, &err}) t->st = st;
  ibox.st = lbox.st = st;
  LRT_TRY(child.alloc(2 * size_t(n_cap), st));
  LRT_TRY(ibox.alloc(6 * size_t(n_cap), st));
  LRT_TRY(lbox.alloc(6 * size_t(n), st));
  LRT_TRY(lpay.alloc(n, st));
  LRT_TRY(sidb.alloc(n, st));
  LRT_TRY(err.alloc(1, st));
  LRT_TRY(cudaMemsetAsync(err.p, 0, 4, st));
  uint32_t root = 0, n_int = 0, n_leaf = 0;
  if (sah) {
    // exact binned SAH, level by level
    const uint32_t max_leaf = boxes ? 1u : 2u;
    Tmp<float> cent, sbox;
    Tmp<uint32_t> tmp, rank, sb, se, sp, nb_, ne_, np_, split, flag, excl, bflag, bscan, big;
    cent.st = sbox.st = st;
    for (auto *t : {&tmp, &rank, &sb, &se, &sp, &nb_, &ne_, &np_, &split, &flag, &excl, &bflag, &bscan, &big})
      t->st = st;
    LRT_TRY(cent.alloc(3 * size_t(n), st));
    LRT_TRY(sbox.alloc(6 * size_t(n), st));
    for (auto *t : {&tmp, &rank, &sb, &se, &sp, &nb_, &ne_, &np_, &split, &flag, &excl, &bflag, &bscan})
      LRT_TRY(t->alloc(n, st));
    LRT_TRY(big.alloc(kBigWords, st));
    centroids<<<blocks(n, 256), 256, 0, st>>>(d_boxes6, n, cent.p, sidb.p);
    const uint32_t seg0[3] = {0u, n, kNone};
    LRT_TRY(cudaMemcpyAsync(sb.p, &seg0[0], 4, cudaMemcpyHostToDevice, st));
    LRT_TRY(cudaMemcpyAsync(se.p, &seg0[1], 4, cudaMemcpyHostToDevice, st));
    LRT_TRY(cudaMemcpyAsync(sp.p, &seg0[2], 4, cudaMemcpyHostToDevice, st));
    uint32_t nseg = 1, depth = 0;
    uint32_t *cb = sb.p, *ce = se.p, *cp = sp.p, *xb = nb_.p, *xe = ne_.p, *xp = np_.p;
    while (nseg > 0) {
      // node ranges of kBigMin primitives or more (the top levels) are split by many
      // blocks each; the level kernel skips them
      if (nseg <= kBigMaxSegs) {
        uint32_t hb[kBigMaxSegs], he[kBigMaxSegs];
        LRT_TRY(cudaMemcpyAsync(hb, cb, nseg * 4, cudaMemcpyDeviceToHost, st));
        LRT_TRY(cudaMemcpyAsync(he, ce, nseg * 4, cudaMemcpyDeviceToHost, st));
        LRT_TRY(cudaStreamSynchronize(st));
        for (uint32_t k = 0; k < nseg; k++) {
          const uint32_t b = hb[k], e = he[k], m = e - b;
          if (m < kBigMin) continue;
          const unsigned g = std::min<unsigned>(blocks(m, 1024), 1024);
          sah_big_init<<<1, 256, 0, st>>>(big.p);
          sah_big_bounds<<<g, 256, 0, st>>>(d_boxes6, cent.p, sidb.p, b, e, big.p);
          sah_big_bins<<<g, 256, 0, st>>>(d_boxes6, cent.p, sidb.p, b, e, depth, big.p);
          sah_big_sweep<<<1, 32, 0, st>>>(k, b, e, depth, big.p, sbox.p, split.p, flag.p, err.p);
          sah_big_flags<<<g, 256, 0, st>>>(cent.p, sidb.p, b, e, depth, big.p, bflag.p);
          LRT_TRY(cudaGetLastError());
          LRT_TRY(gpu_exclusive_scan(bflag.p, bscan.p, m, nullptr, st));
          sah_big_scatter<<<g, 256, 0, st>>>(sidb.p, b, e, big.p, bflag.p, bscan.p, tmp.p);
          sah_big_copy<<<g, 256, 0, st>>>(sidb.p, tmp.p, b, e, big.p);
          LRT_TRY(cudaGetLastError());
        }
      }
      sah_level<<<nseg, kSahThreads, 0, st>>>(d_boxes6, cent.p, sidb.p, tmp.p, rank.p, cb, ce, depth, max_leaf, sbox.p,
                                              split.p, flag.p, err.p, nseg <= kBigMaxSegs ? kBigMin : 0xFFFFFFFFu);
      LRT_TRY(cudaGetLastError());
      uint64_t n_split = 0;
      LRT_TRY(gpu_exclusive_scan(flag.p, excl.p, nseg, &n_split, st));
      sah_link<<<blocks(nseg, 128), 128, 0, st>>>(nseg, cb, ce, cp, sbox.p, split.p, flag.p, excl.p, n_int, n_leaf,
                                                  sidb.p, boxes, child.p, ibox.p, lbox.p, lpay.p, xb, xe, xp);
      LRT_TRY(cudaGetLastError());
      n_int += uint32_t(n_split);
      n_leaf += nseg - uint32_t(n_split);
      nseg = 2 * uint32_t(n_split);
      std::swap(cb, xb);
      std::swap(ce, xe);
      std::swap(cp, xp);
      depth++;
    }
    uint32_t herr = 0;
    LRT_TRY(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, st));
    LRT_TRY(cudaStreamSynchronize(st));
    if (herr) return cudaErrorNotSupported;   // a median split too large for the device path
    root = n > max_leaf ? 0u : kLeafBit;
  } else {
    // linear BVH: Morton codes, radix sort, radix tree, node boxes
    Tmp<uint32_t> ob, code, code2, id2, hist, hoff, par_i, par_l, visits;
    for (auto *t : {&ob, &code, &code2, &id2, &hist, &hoff, &par_i, &par_l, &visits}) t->st = st;
    const uint32_t nblk = blocks(n, kSortTile);
    LRT_TRY(ob.alloc(6, st));
    LRT_TRY(code.alloc(n, st));
    LRT_TRY(code2.alloc(n, st));
    LRT_TRY(id2.alloc(n, st));
    LRT_TRY(hist.alloc(16 * size_t(nblk), st));
    LRT_TRY(hoff.alloc(16 * size_t(nblk), st));
    LRT_TRY(par_i.alloc(n_cap, st));
    LRT_TRY(par_l.alloc(n, st));
    LRT_TRY(visits.alloc(n_cap, st));
    bounds_init<<<1, 32, 0, st>>>(ob.p);
    centroid_bounds<<<std::min<uint32_t>(blocks(n, 256), 2048), 256, 0, st>>>(d_boxes6, n, ob.p);
    morton_codes<<<blocks(n, 256), 256, 0, st>>>(d_boxes6, n, ob.p, code.p, sidb.p);
    LRT_TRY(cudaGetLastError());
    // radix sort, 8 passes of 4 bits (an even count: the result ends in code / sidb)
    uint32_t *ki = code.p, *vi = sidb.p, *ko = code2.p, *vo = id2.p;
    for (uint32_t shift = 0; shift < 32; shift += 4) {
      radix_count<<<nblk, kSortThreads, 0, st>>>(ki, n, shift, nblk, hist.p);
      LRT_TRY(cudaGetLastError());
      LRT_TRY(gpu_exclusive_scan(hist.p, hoff.p, 16 * nblk, nullptr, st));
      radix_scatter<<<nblk, kSortThreads, 0, st>>>(ki, vi, ko, vo, n, shift, nblk, hoff.p);
      LRT_TRY(cudaGetLastError());
      std::swap(ki, ko);
      std::swap(vi, vo);
    }
    if (n > 1) {
      radix_tree<<<blocks(n - 1, 256), 256, 0, st>>>(ki, n, child.p, par_i.p, par_l.p);
      LRT_TRY(cudaMemsetAsync(visits.p, 0, size_t(n_cap) * 4, st));
      node_boxes<<<blocks(n, 256), 256, 0, st>>>(d_boxes6, sidb.p, n, child.p, par_i.p, par_l.p, ibox.p, visits.p,
                                                 err.p);
      LRT_TRY(cudaGetLastError());
    }
    lbvh_leaves<<<blocks(n, 256), 256, 0, st>>>(d_boxes6, sidb.p, n, boxes, lbox.p, lpay.p);
    LRT_TRY(cudaGetLastError());
    uint32_t herr = 0;
    LRT_TRY(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, st));
    LRT_TRY(cudaStreamSynchronize(st));
    if (herr) return cudaErrorUnknown;
    root = n > 1 ? 0u : kLeafBit;
    n_int = n > 1 ? n - 1 : 0;
    n_leaf = n;
  }
  // collapse, level by level
  Tmp<uint32_t> front, front2, pick, cnt, off;
  for (auto *t : {&front, &front2, &pick, &cnt, &off}) t->st = st;
  LRT_TRY(front.alloc(n, st));
  LRT_TRY(front2.alloc(n, st));
  LRT_TRY(pick.alloc(4 * size_t(n), st));
  LRT_TRY(cnt.alloc(n, st));
  LRT_TRY(off.alloc(n, st));
  LRT_TRY(cudaMemcpyAsync(front.p, &root, 4, cudaMemcpyHostToDevice, st));
  uint32_t nf = 1, level_base = 0;
  uint32_t *fr = front.p, *fr2 = front2.p;
  while (nf > 0) {
    info.level_start.push_back(level_base);
    collapse_pick<<<blocks(nf, 128), 128, 0, st>>>(fr, nf, child.p, ibox.p, pick.p, cnt.p);
    LRT_TRY(cudaGetLastError());
    uint64_t total = 0;
    LRT_TRY(gpu_exclusive_scan(cnt.p, off.p, nf, &total, st));
    collapse_write<<<blocks(nf, 128), 128, 0, st>>>(pick.p, nf, off.p, level_base, level_base + nf, ibox.p, lbox.p,
                                                    lpay.p, d_wnodes, fr2);
    LRT_TRY(cudaGetLastError());
    level_base += nf;
    nf = uint32_t(total);
    std::swap(fr, fr2);
  }
  info.n_wnodes = level_base;
  info.max_depth = uint32_t(info.level_start.size()) - 1;
  info.n_pairs = std::max<uint32_t>(1, n_int);
  info.n_leaves = n_leaf;
  if (d_order) LRT_TRY(cudaMemcpyAsync(d_order, sidb.p, size_t(n) * 4, cudaMemcpyDeviceToDevice, st));
  if (d_pairs) {
    fat_pairs<<<blocks(info.n_pairs, 256), 256, 0, st>>>(n_int, root, child.p, ibox.p, lbox.p, lpay.p, boxes, d_pairs,
                                                         boxes ? nullptr : d_leaf_start_count);
    LRT_TRY(cudaGetLastError());
  }
  return cudaStreamSynchronize(st);
}

cudaError_t refit_bvh_gpu(const float *d_boxes6, bool boxes, const uint32_t *d_order, WNode4 *d_wnodes,
                          const std::vector<uint32_t> &level_start, uint32_t n_wnodes, cudaStream_t st) {
  for (size_t l = level_start.size(); l-- > 0;) {
    const uint32_t first = level_start[l];
    const uint32_t last = l + 1 < level_start.size() ? level_start[l + 1] : n_wnodes;
    if (last <= first) continue;
    refit_level<<<blocks(last - first, 128), 128, 0, st>>>(d_wnodes, first, last - first, d_boxes6, d_order, boxes);
    LRT_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

cudaError_t triangle_boxes_gpu(const float4 *d_tri_verts, uint32_t n, float *d_boxes6, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  triangle_boxes<<<blocks(n, 256), 256, 0, st>>>(d_tri_verts, n, d_boxes6);
  return cudaGetLastError();
}

cudaError_t gather_triangles_gpu(const float4 *d_vpos, const uint32_t *d_indices, const uint32_t *d_order, uint32_t n,
                                 float4 *d_tri_verts, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  gather_triangles<<<blocks(n, 256), 256, 0, st>>>(d_vpos, d_indices, d_order, n, d_tri_verts);
  return cudaGetLastError();
}

}  // namespace lrt
