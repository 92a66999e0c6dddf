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
__device__ __forceinline__ float area(const Box &b) {   // the host builder's Aabb::area
  const float dx = fmaxf(0.0f, b.hi[0] - b.lo[0]), dy = fmaxf(0.0f, b.hi[1] - b.lo[1]),
              dz = fmaxf(0.0f, b.hi[2] - b.lo[2]);
  return 2.0f * (dx * dy + dy * dz + dz * dx);
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

// ---- collapse into 4-wide nodes, one wide level per pass ----
__global__ void collapse_pick(const uint32_t *front, uint32_t nf, const uint32_t *child, const float *b6,
                              const uint32_t *sid, const float *nb, uint32_t *pick, uint32_t *n_internal) {
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
          const float a = area(child_box(b6, sid, nb, ch[i]));
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
                               uint32_t next_base, const float *b6, const uint32_t *sid, const float *nb, bool boxes,
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
    const Box b = child_box(b6, sid, nb, c);
    w.lo_x[i] = b.lo[0]; w.lo_y[i] = b.lo[1]; w.lo_z[i] = b.lo[2];
    w.hi_x[i] = b.hi[0]; w.hi_y[i] = b.hi[1]; w.hi_z[i] = b.hi[2];
    if (c & kLeafBit) {
      const uint32_t pos = c & ~kLeafBit;
      w.child[i] = boxes ? (kLeafBit | sid[pos]) : (kLeafBit | (1u << 24) | pos);
    } else {
      w.child[i] = next_base + off[k] + j;
      next_front[off[k] + j] = c;
      j++;
    }
  }
  wn[level_base + k] = w;
}

// ---- reference fat-pair layout: pair i holds the two children of internal node i ----
__device__ __forceinline__ void pair_side(lrt_bvh_node &s, uint32_t c, const float *b6, const uint32_t *sid,
                                          const float *nb, bool boxes, uint32_t *lsc) {
  const Box b = child_box(b6, sid, nb, c);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s.boxMin[k] = b.lo[k];
    s.boxMax[k] = b.hi[k];
  }
  s.escapeIndex = 0;
  if (c & kLeafBit) {
    const uint32_t pos = c & ~kLeafBit;
    if (boxes) {
      s.leftOffset = kLeafBit | (1u << 24) | (sid[pos] & 0x00FFFFFFu);
    } else {
      s.leftOffset = kLeafBit | (1u << 24) | (pos & 0x00FFFFFFu);
      if (lsc) lsc[pos] = kLeafBit | (1u << 24) | (pos & 0x00FFFFFFu);
    }
  } else {
    s.leftOffset = c;
  }
}

__global__ void fat_pairs(uint32_t n, const uint32_t *child, const float *b6, const uint32_t *sid, const float *nb,
                          bool boxes, lrt_bvh_pair *pairs, uint32_t *lsc) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (n == 1) {   // a single leaf: both sides are the root leaf
    if (i == 0) {
      pair_side(pairs[0].left, kLeafBit, b6, sid, nb, boxes, lsc);
      pairs[0].right = pairs[0].left;
    }
    return;
  }
  if (i >= n - 1) return;
  pair_side(pairs[i].left, child[2 * i], b6, sid, nb, boxes, lsc);
  pair_side(pairs[i].right, child[2 * i + 1], b6, sid, nb, boxes, lsc);
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

cudaError_t build_bvh_gpu(const float *d_boxes6, uint32_t n, bool boxes, WNode4 *d_wnodes, uint32_t *d_order,
                          lrt_bvh_pair *d_pairs, uint32_t *d_leaf_start_count, GpuBvhInfo &info, cudaStream_t st) {
  info = GpuBvhInfo{};
  if (n == 0) return cudaErrorInvalidValue;
  const uint32_t n_int = n > 1 ? n - 1 : 1;
  Tmp<uint32_t> ob, code, id, code2, id2, hist, hoff, child, par_i, par_l, visits, err, front, front2, pick, cnt, off;
  Tmp<float> nb;
  for (auto *t : {&ob, &code, &id, &code2, &id2, &hist, &hoff, &child, &par_i, &par_l, &visits, &err, &front, &front2,
                  &pick, &cnt, &off})
    t->st = st;
  nb.st = st;
  const uint32_t nblk = blocks(n, kSortTile);
  LRT_TRY(ob.alloc(6, st));
  LRT_TRY(code.alloc(n, st));
  LRT_TRY(id.alloc(n, st));
  LRT_TRY(code2.alloc(n, st));
  LRT_TRY(id2.alloc(n, st));
  LRT_TRY(hist.alloc(16 * size_t(nblk), st));
  LRT_TRY(hoff.alloc(16 * size_t(nblk), st));
  LRT_TRY(child.alloc(2 * size_t(n_int), st));
  LRT_TRY(par_i.alloc(n_int, st));
  LRT_TRY(par_l.alloc(n, st));
  LRT_TRY(visits.alloc(n_int, st));
  LRT_TRY(err.alloc(1, st));
  LRT_TRY(nb.alloc(6 * size_t(n_int), st));
  LRT_TRY(front.alloc(n, st));
  LRT_TRY(front2.alloc(n, st));
  LRT_TRY(pick.alloc(4 * size_t(n), st));
  LRT_TRY(cnt.alloc(n, st));
  LRT_TRY(off.alloc(n, st));

  // 1-2. centroid bounds, Morton codes
  bounds_init<<<1, 32, 0, st>>>(ob.p);
  centroid_bounds<<<std::min<uint32_t>(blocks(n, 256), 2048), 256, 0, st>>>(d_boxes6, n, ob.p);
  morton_codes<<<blocks(n, 256), 256, 0, st>>>(d_boxes6, n, ob.p, code.p, id.p);
  LRT_TRY(cudaGetLastError());
  // 3. radix sort, 8 passes of 4 bits (an even count: the result ends in code/id)
  uint32_t *ki = code.p, *vi = id.p, *ko = code2.p, *vo = id2.p;
  for (uint32_t shift = 0; shift < 32; shift += 4) {
    radix_count<<<nblk, kSortThreads, 0, st>>>(ki, n, shift, nblk, hist.p);
    LRT_TRY(cudaGetLastError());
    LRT_TRY(gpu_exclusive_scan(hist.p, hoff.p, 16 * nblk, nullptr, st));
    radix_scatter<<<nblk, kSortThreads, 0, st>>>(ki, vi, ko, vo, n, shift, nblk, hoff.p);
    LRT_TRY(cudaGetLastError());
    std::swap(ki, ko);
    std::swap(vi, vo);
  }
  const uint32_t *sid = vi;
  // 4-5. radix tree and node boxes
  if (n > 1) {
    radix_tree<<<blocks(n - 1, 256), 256, 0, st>>>(ki, n, child.p, par_i.p, par_l.p);
    LRT_TRY(cudaMemsetAsync(visits.p, 0, size_t(n_int) * 4, st));
    LRT_TRY(cudaMemsetAsync(err.p, 0, 4, st));
    node_boxes<<<blocks(n, 256), 256, 0, st>>>(d_boxes6, sid, n, child.p, par_i.p, par_l.p, nb.p, visits.p, err.p);
    LRT_TRY(cudaGetLastError());
    uint32_t herr = 0;
    LRT_TRY(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, st));
    LRT_TRY(cudaStreamSynchronize(st));
    if (herr) return cudaErrorUnknown;
  }
  // 6. collapse, level by level
  const uint32_t root = n > 1 ? 0u : kLeafBit;
  LRT_TRY(cudaMemcpyAsync(front.p, &root, 4, cudaMemcpyHostToDevice, st));
  uint32_t nf = 1, level_base = 0;
  uint32_t *fr = front.p, *fr2 = front2.p;
  while (nf > 0) {
    info.level_start.push_back(level_base);
    collapse_pick<<<blocks(nf, 128), 128, 0, st>>>(fr, nf, child.p, d_boxes6, sid, nb.p, pick.p, cnt.p);
    LRT_TRY(cudaGetLastError());
    uint64_t total = 0;
    LRT_TRY(gpu_exclusive_scan(cnt.p, off.p, nf, &total, st));
    collapse_write<<<blocks(nf, 128), 128, 0, st>>>(pick.p, nf, off.p, level_base, level_base + nf, d_boxes6, sid,
                                                    nb.p, boxes, d_wnodes, fr2);
    LRT_TRY(cudaGetLastError());
    level_base += nf;
    nf = uint32_t(total);
    std::swap(fr, fr2);
  }
  info.n_wnodes = level_base;
  info.max_depth = uint32_t(info.level_start.size()) - 1;
  // 7. outputs
  if (d_order) LRT_TRY(cudaMemcpyAsync(d_order, sid, size_t(n) * 4, cudaMemcpyDeviceToDevice, st));
  if (d_pairs) {
    fat_pairs<<<blocks(n_int, 256), 256, 0, st>>>(n, child.p, d_boxes6, sid, nb.p, boxes, d_pairs,
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
