// BVH construction on the host.  The reference builds a binary SAH BVH with
// Embree's rtcBuildBVH (BVH/cbvh_embree2.cpp:287-332) and re-packs it into
// 64-byte fat node pairs (BVH/cbvh_fat.cpp:100-142).  Embree is not available;
// this is a binned-SAH BVH2 builder of our own, followed by a collapse into
// 4-wide nodes laid out for the GPU (one 128-byte line per node, child boxes in
// structure-of-arrays order).  The fat-pair form is still produced for callers
// that read the reference layout.
//
// Leaf payloads follow the reference: for box geometry (SBS bricks, SVS voxels)
// a leaf holds one box and its id (BVH/cbvh.cpp:628-637, primsInLeaf = 1); for
// triangles a leaf holds up to two triangles of the reordered triangle array
// (BVH/cbvh.cpp:508-516, "cbvh_embree2" -> primsInLeaf = 2).
#include "lrt_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace lrt {

namespace {

struct Aabb {
  float lo[3], hi[3];
  void reset() { lo[0] = lo[1] = lo[2] = 3.4e38f; hi[0] = hi[1] = hi[2] = -3.4e38f; }
  void grow(const Aabb &b) {
    for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
  }
  void grow_pt(const float p[3]) {
    for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
  }
  float area() const {
    const float dx = std::max(0.0f, hi[0] - lo[0]), dy = std::max(0.0f, hi[1] - lo[1]), dz = std::max(0.0f, hi[2] - lo[2]);
    return 2.0f * (dx * dy + dy * dz + dz * dx);
  }
};

struct Node2 {
  Aabb box;
  int32_t left = -1, right = -1;  // internal: child node indices
  uint32_t start = 0, count = 0;  // leaf: range in prim order
  bool leaf() const { return left < 0; }
};

struct Builder {
  const std::vector<Aabb> &prims;
  std::vector<float> cent;      // 3 per prim
  std::vector<uint32_t> order;  // prim ids
  std::vector<Node2> nodes;
  uint32_t max_leaf;
  uint32_t max_depth_seen = 0;

  Builder(const std::vector<Aabb> &p, uint32_t ml) : prims(p), max_leaf(ml) {
    const size_t n = p.size();
    cent.resize(3 * n);
    order.resize(n);
    for (size_t i = 0; i < n; i++) {
      order[i] = uint32_t(i);
      for (int k = 0; k < 3; k++) cent[3 * i + k] = 0.5f * (p[i].lo[k] + p[i].hi[k]);
    }
  }

  Aabb range_box(uint32_t b, uint32_t e) const {
    Aabb a; a.reset();
    for (uint32_t i = b; i < e; i++) a.grow(prims[order[i]]);
    return a;
  }

  // split [b,e) in place; returns the split position (b < m < e)
  uint32_t split(uint32_t b, uint32_t e, uint32_t depth) {
    Aabb cb; cb.reset();
    for (uint32_t i = b; i < e; i++) cb.grow_pt(&cent[3 * size_t(order[i])]);
    constexpr int NB = 32;
    float best_cost = 3.4e38f;
    int best_axis = -1, best_bin = -1;
    if (depth < 40) {
      for (int ax = 0; ax < 3; ax++) {
        const float ext = cb.hi[ax] - cb.lo[ax];
        if (!(ext > 0)) continue;
        Aabb bins[NB]; uint32_t cnt[NB] = {0};
        for (int i = 0; i < NB; i++) bins[i].reset();
        const float sc = NB / ext;
        for (uint32_t i = b; i < e; i++) {
          const uint32_t id = order[i];
          int bi = int((cent[3 * size_t(id) + ax] - cb.lo[ax]) * sc);
          bi = std::min(std::max(bi, 0), NB - 1);
          bins[bi].grow(prims[id]);
          cnt[bi]++;
        }
        float rA[NB]; uint32_t rN[NB];
        Aabb acc; acc.reset(); uint32_t n = 0;
        for (int i = NB - 1; i > 0; i--) { acc.grow(bins[i]); n += cnt[i]; rA[i] = acc.area(); rN[i] = n; }
        acc.reset(); n = 0;
        for (int i = 0; i < NB - 1; i++) {
          acc.grow(bins[i]); n += cnt[i];
          if (n == 0 || rN[i + 1] == 0) continue;
          const float cost = acc.area() * float(n) + rA[i + 1] * float(rN[i + 1]);
          if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = i; }
        }
      }
    }
    if (best_axis >= 0) {
      const int ax = best_axis;
      const float ext = cb.hi[ax] - cb.lo[ax];
      const float sc = NB / ext;
      auto mid = std::stable_partition(order.begin() + b, order.begin() + e, [&](uint32_t id) {
        int bi = int((cent[3 * size_t(id) + ax] - cb.lo[ax]) * sc);
        bi = std::min(std::max(bi, 0), NB - 1);
        return bi <= best_bin;
      });
      const uint32_t m = uint32_t(mid - order.begin());
      if (m > b && m < e) return m;
    }
    // object median on the widest centroid axis (also the fallback below depth 40)
    int ax = 0;
    for (int k = 1; k < 3; k++) if (cb.hi[k] - cb.lo[k] > cb.hi[ax] - cb.lo[ax]) ax = k;
    const uint32_t m = b + (e - b) / 2;
    std::nth_element(order.begin() + b, order.begin() + m, order.begin() + e, [&](uint32_t x, uint32_t y) {
      const float cx = cent[3 * size_t(x) + ax], cy = cent[3 * size_t(y) + ax];
      return cx < cy || (cx == cy && x < y);
    });
    return m;
  }

  void build() {
    const uint32_t n = uint32_t(prims.size());
    nodes.clear();
    nodes.reserve(2 * size_t(n) + 1);
    nodes.emplace_back();
    struct Task { uint32_t node, b, e, depth; };
    std::vector<Task> st;
    st.push_back({0, 0, n, 0});
    while (!st.empty()) {
      Task t = st.back(); st.pop_back();
      nodes[t.node].box = range_box(t.b, t.e);
      max_depth_seen = std::max(max_depth_seen, t.depth);
      if (t.e - t.b <= max_leaf) {
        nodes[t.node].start = t.b;
        nodes[t.node].count = t.e - t.b;
        continue;
      }
      const uint32_t m = split(t.b, t.e, t.depth);
      const int32_t l = int32_t(nodes.size());
      nodes.emplace_back();
      nodes.emplace_back();
      nodes[t.node].left = l;
      nodes[t.node].right = l + 1;
      st.push_back({uint32_t(l + 1), m, t.e, t.depth + 1});
      st.push_back({uint32_t(l), t.b, m, t.depth + 1});
    }
  }
};

}  // namespace

// Leaf reference stored in a wide node: LEAF_BIT | payload.
static inline uint32_t leaf_ref(const Node2 &nd, const std::vector<uint32_t> &order, bool boxes) {
  if (boxes) return kLeafBit | order[nd.start];                                   // box / brick id
  return kLeafBit | ((nd.count & 0x7Fu) << 24) | (nd.start & 0x00FFFFFFu);       // triangle range
}

lrt_status build_bvh(const float *boxes6, uint32_t n, bool boxes, BvhData &out) {
  if (n == 0) return LRT_ERR_INVALID;
  if (!boxes && n >= (1u << 24)) return LRT_ERR_UNSUPPORTED;
  if (boxes && n >= (1u << 31)) return LRT_ERR_UNSUPPORTED;
  std::vector<Aabb> prims(n);
  for (uint32_t i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) { prims[i].lo[k] = boxes6[6 * size_t(i) + k]; prims[i].hi[k] = boxes6[6 * size_t(i) + 3 + k]; }
  Builder B(prims, boxes ? 1u : 2u);
  B.build();
  out.order = B.order;

  // ---- 4-wide collapse (GPU layout) ----
  // Wide node k is built from BVH2 node pend[k]; children are appended to pend
  // in breadth-first order, so a child's wide index is its position in pend.
  std::vector<int32_t> pend(1, 0);
  std::vector<uint32_t> wdepth(1, 0);
  std::vector<WNode4> &wn = out.wnodes;
  wn.clear();
  out.level_start.assign(1, 0);
  uint32_t max_wdepth = 0;
  for (size_t wi = 0; wi < pend.size(); wi++) {
    const Node2 &root = B.nodes[pend[wi]];
    int32_t ch[4];
    int nc = 0;
    if (root.leaf()) {
      ch[nc++] = pend[wi];
    } else {
      ch[nc++] = root.left;
      ch[nc++] = root.right;
      while (nc < 4) {   // open the internal child with the largest surface area
        int best = -1;
        float best_a = -1;
        for (int i = 0; i < nc; i++)
          if (!B.nodes[ch[i]].leaf() && B.nodes[ch[i]].box.area() > best_a) { best_a = B.nodes[ch[i]].box.area(); best = i; }
        if (best < 0) break;
        const Node2 &x = B.nodes[ch[best]];
        ch[best] = x.left;
        ch[nc++] = x.right;
      }
    }
    WNode4 w;
    for (int i = 0; i < 4; i++) {
      w.pad[i] = 0;
      if (i < nc) {
        const Node2 &c = B.nodes[ch[i]];
        w.lo_x[i] = c.box.lo[0]; w.lo_y[i] = c.box.lo[1]; w.lo_z[i] = c.box.lo[2];
        w.hi_x[i] = c.box.hi[0]; w.hi_y[i] = c.box.hi[1]; w.hi_z[i] = c.box.hi[2];
        if (c.leaf()) {
          w.child[i] = leaf_ref(c, B.order, boxes);
        } else {
          w.child[i] = uint32_t(pend.size());
          if (wdepth[wi] + 1 == out.level_start.size()) out.level_start.push_back(uint32_t(pend.size()));
          pend.push_back(ch[i]);
          wdepth.push_back(wdepth[wi] + 1);
          max_wdepth = std::max(max_wdepth, wdepth[wi] + 1);
        }
      } else {
        // empty slot: a point box far beyond any ray's tFar, never entered
        w.lo_x[i] = w.lo_y[i] = w.lo_z[i] = 1e30f;
        w.hi_x[i] = w.hi_y[i] = w.hi_z[i] = 1e30f;
        w.child[i] = kEmptyChild;
      }
    }
    wn.push_back(w);
  }
  out.max_depth = max_wdepth;

  // ---- reference fat-pair layout (root pair = root's two children) ----
  out.pairs.clear();
  out.leaf_start_count.clear();
  if (B.nodes[0].leaf()) {
    lrt_bvh_pair p;
    const Node2 &r = B.nodes[0];
    for (int k = 0; k < 3; k++) { p.left.boxMin[k] = r.box.lo[k]; p.left.boxMax[k] = r.box.hi[k]; }
    if (boxes) p.left.leftOffset = kLeafBit | (1u << 24) | (B.order[r.start] & 0x00FFFFFFu);
    else { p.left.leftOffset = kLeafBit | (1u << 24); out.leaf_start_count.push_back(kLeafBit | ((r.count & 0x7Fu) << 24) | r.start); }
    p.left.escapeIndex = 0;
    p.right = p.left;
    out.pairs.push_back(p);
  } else {
    std::vector<int32_t> q;    // BVH2 internal node per pair
    q.push_back(0);
    out.pairs.emplace_back();
    for (size_t pi = 0; pi < q.size(); pi++) {
      const Node2 &nd = B.nodes[q[pi]];
      lrt_bvh_pair p;
      lrt_bvh_node *sides[2] = {&p.left, &p.right};
      const int32_t kids[2] = {nd.left, nd.right};
      for (int s = 0; s < 2; s++) {
        const Node2 &c = B.nodes[kids[s]];
        for (int k = 0; k < 3; k++) { sides[s]->boxMin[k] = c.box.lo[k]; sides[s]->boxMax[k] = c.box.hi[k]; }
        sides[s]->escapeIndex = 0;
        if (c.leaf()) {
          if (boxes) sides[s]->leftOffset = kLeafBit | (1u << 24) | (B.order[c.start] & 0x00FFFFFFu);
          else {
            sides[s]->leftOffset = kLeafBit | (1u << 24) | (uint32_t(out.leaf_start_count.size()) & 0x00FFFFFFu);
            out.leaf_start_count.push_back(kLeafBit | ((c.count & 0x7Fu) << 24) | (c.start & 0x00FFFFFFu));
          }
        } else {
          sides[s]->leftOffset = uint32_t(q.size());
          q.push_back(kids[s]);
          out.pairs.emplace_back();
        }
      }
      out.pairs[pi] = p;
    }
  }
  return LRT_OK;
}

}  // namespace lrt
