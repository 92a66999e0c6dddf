// Host construction of sparse brick sets (SBS) and sparse voxel sets (SVS) from
// analytic SDFs: a restatement of the reference's frame-octree builder
// (utils/sparse_octree_builder.cpp:72-252), SBS conversion (:291-444) and SVS
// conversion (:2346-2387), entered through create_sdf_SBS / create_sdf_SVS
// (utils/sdf_converter.cpp:118-181).
//
// The reference builds per-thread subtrees and appends bricks under an OpenMP
// critical section, so its brick order depends on scheduling.  Here every
// parallel stage writes into per-task slots that are concatenated in task
// order, which yields the order a single-threaded run of the reference gives.
// Compiled with -ffp-contract=off so that results are identical on x86-64 and
// aarch64 hosts.
#include "lrt_internal.h"

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace lrt {

// ---------------------------------------------------------------- SDFs
static inline float sdf_sphere(const float *s, float x, float y, float z) {
  const float dx = x - s[0], dy = y - s[1], dz = z - s[2];
  return std::sqrt(dx * dx + dy * dy + dz * dz) - s[3];
}

// rounded box {c[3], half[3], r, R[9]} evaluated in the box frame
static inline float sdf_round_box(const float *b, float x, float y, float z) {
  const float px = x - b[0], py = y - b[1], pz = z - b[2];
  const float *R = b + 7;
  const float lx = R[0] * px + R[1] * py + R[2] * pz;
  const float ly = R[3] * px + R[4] * py + R[5] * pz;
  const float lz = R[6] * px + R[7] * py + R[8] * pz;
  const float qx = std::fabs(lx) - (b[3] - b[6]), qy = std::fabs(ly) - (b[4] - b[6]),
              qz = std::fabs(lz) - (b[5] - b[6]);
  const float mx = qx > 0 ? qx : 0, my = qy > 0 ? qy : 0, mz = qz > 0 ? qz : 0;
  const float outside = std::sqrt(mx * mx + my * my + mz * mz);
  float m = qx > qy ? qx : qy;
  m = m > qz ? m : qz;
  const float inside = m < 0 ? m : 0;
  return outside + inside - b[6];
}

// polynomial smooth minimum (quadratic kernel)
static inline float smooth_min(float a, float b, float k) {
  const float m = a < b ? a : b;
  if (k <= 0.0f) return m;
  float h = k - std::fabs(a - b);
  h = h > 0 ? h : 0;
  h = h / k;
  return m - h * h * k * 0.25f;
}

float sdf_eval(const lrt_sdf_desc &f, float x, float y, float z) {
  float d = 1e10f;
  bool first = true;
  for (uint32_t i = 0; i < f.n_spheres; i++) {
    const float v = sdf_sphere(f.spheres + 4 * i, x, y, z);
    d = first ? v : smooth_min(d, v, f.k);
    first = false;
  }
  for (uint32_t i = 0; i < f.n_boxes; i++) {
    const float v = sdf_round_box(f.boxes + 16 * i, x, y, z);
    d = first ? v : smooth_min(d, v, f.k);
    first = false;
  }
  return d;
}

// ---------------------------------------------------------------- frame octree
struct FrameNode {
  float values[8];
  uint32_t offset;  // first child (8 consecutive), 0 = leaf
};

static inline float sdf_node_point(const lrt_sdf_desc &f, const float p[3], float cx, float cy, float cz, float d) {
  // sdf(2.0f * ((p + c) * d) - 1), utils/sparse_octree_builder.cpp:75,80
  return sdf_eval(f, 2.0f * ((p[0] + cx) * d) - 1.0f, 2.0f * ((p[1] + cy) * d) - 1.0f,
                  2.0f * ((p[2] + cz) * d) - 1.0f);
}

// add_node_rec, utils/sparse_octree_builder.cpp:72-96
static void add_node_rec(std::vector<FrameNode> &nodes, const lrt_sdf_desc &f, uint32_t idx, uint32_t depth,
                         uint32_t max_depth, const float p[3], float d) {
  const float vc = sdf_node_point(f, p, 0.5f, 0.5f, 0.5f, d);
  float mn = 1000, mx = -1000;
  for (int c = 0; c < 8; c++) {
    const float v = sdf_node_point(f, p, float((c & 4) >> 2), float((c & 2) >> 1), float(c & 1), d);
    nodes[idx].values[c] = v;
    mn = std::min(mn, v);
    mx = std::max(mx, v);
  }
  if (depth < max_depth && (std::fabs(vc) < std::sqrt(3.0f) * d || mn * mx <= 0)) {
    const uint32_t off = uint32_t(nodes.size());
    nodes[idx].offset = off;
    nodes.resize(nodes.size() + 8);
    for (uint32_t c = 0; c < 8; c++) {
      const float cp[3] = {2 * p[0] + float((c & 4) >> 2), 2 * p[1] + float((c & 2) >> 1), 2 * p[2] + float(c & 1)};
      add_node_rec(nodes, f, off + c, depth + 1, max_depth, cp, d / 2);
    }
  }
}

struct Frame {
  std::vector<FrameNode> nodes;
  std::vector<float> pd;  // (p.xyz, d) per node
};

// construct_sdf_frame_octree, utils/sparse_octree_builder.cpp:125-252
static Frame build_frame(const lrt_sdf_desc &f, uint32_t depth, int threads) {
  struct Large { float p[3]; float d, value; uint32_t level, children; };
  const uint32_t min_remove_level = std::min(depth, 4u);
  std::vector<Large> L;
  L.push_back({{0, 0, 0}, 1.0f, 1000.0f, 0, 0});
  for (size_t i = 0; i < L.size(); i++) {
    if (L[i].level < min_remove_level) {
      L[i].children = uint32_t(L.size());
      for (int j = 0; j < 8; j++) {
        Large c;
        c.d = L[i].d / 2;
        c.p[0] = 2 * L[i].p[0] + float((j & 4) >> 2);
        c.p[1] = 2 * L[i].p[1] + float((j & 2) >> 1);
        c.p[2] = 2 * L[i].p[2] + float(j & 1);
        c.level = L[i].level + 1;
        c.children = 0;
        c.value = 1000.0f;
        L.push_back(c);
      }
    }
  }
  const long nl = long(L.size());
  std::vector<char> border(nl, 0);
  // is_border, :38-41
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
  for (long i = 0; i < nl; i++) {
    L[i].value = sdf_node_point(f, L[i].p, 0.5f, 0.5f, 0.5f, L[i].d);
    const bool isb = L[i].level < 2 ? true
                                    : (std::fabs(double(L[i].value)) < std::sqrt(3.0) * std::pow(2.0, -double(L[i].level)));
    border[i] = (L[i].children == 0 && isb) ? 1 : 0;
  }
  // subtrees of border large nodes, one task each
  std::vector<std::vector<FrameNode>> sub(nl);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (long i = 0; i < nl; i++) {
    if (!border[i]) continue;
    sub[i].resize(1);
    std::memset(sub[i].data(), 0, sizeof(FrameNode));
    add_node_rec(sub[i], f, 0, L[i].level, depth, L[i].p, L[i].d);
  }
  Frame fr;
  fr.nodes.resize(nl);
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long i = 0; i < nl; i++) {
    for (int c = 0; c < 8; c++)
      fr.nodes[i].values[c] = sdf_node_point(f, L[i].p, float((c & 4) >> 2), float((c & 2) >> 1), float(c & 1), L[i].d);
    fr.nodes[i].offset = L[i].children;
  }
  for (long i = 0; i < nl; i++) {
    if (!border[i] || sub[i].size() <= 1) continue;
    const size_t prev = fr.nodes.size();
    const long shift = long(prev) - 1;
    fr.nodes[i].offset = uint32_t(long(sub[i][0].offset) + shift);
    fr.nodes.insert(fr.nodes.end(), sub[i].begin() + 1, sub[i].end());
    for (size_t j = prev; j < fr.nodes.size(); j++)
      if (fr.nodes[j].offset != 0) fr.nodes[j].offset = uint32_t(long(fr.nodes[j].offset) + shift);
    std::vector<FrameNode>().swap(sub[i]);
  }
  // octree_to_layers, :262-275
  fr.pd.assign(fr.nodes.size() * 4, 0.0f);
  fr.pd[3] = 1.0f;
  std::vector<size_t> stk;
  stk.push_back(0);
  while (!stk.empty()) {
    const size_t idx = stk.back();
    stk.pop_back();
    const uint32_t ofs = fr.nodes[idx].offset;
    if (ofs == 0 || (ofs & 0x80000000u)) continue;
    for (int c = 0; c < 8; c++) {
      float *q = &fr.pd[4 * size_t(ofs + c)];
      q[0] = 2 * fr.pd[4 * idx + 0] + float((c & 4) >> 2);
      q[1] = 2 * fr.pd[4 * idx + 1] + float((c & 2) >> 1);
      q[2] = 2 * fr.pd[4 * idx + 2] + float(c & 1);
      q[3] = fr.pd[4 * idx + 3] / 2;
      stk.push_back(ofs + c);
    }
  }
  return fr;
}

static inline bool frame_is_leaf(uint32_t ofs) { return ofs == 0 || (ofs & 0x80000000u); }

// frame_octree_to_SBS, utils/sparse_octree_builder.cpp:291-444
lrt_status build_sbs(const lrt_sdf_desc &f, uint32_t depth, const lrt_sbs_header &hdr, int threads, SbsData &out) {
  if (hdr.brick_size < 1 || hdr.brick_size > 16 || hdr.brick_pad > 1 ||
      !(hdr.bytes_per_value == 1 || hdr.bytes_per_value == 2 || hdr.bytes_per_value == 4) || depth < 2 || depth > 15)
    return LRT_ERR_INVALID;
  if ((hdr.aux_data & 0xFF000000u) != LRT_SBS_LAYOUT_DX && (hdr.aux_data & 0xFF000000u) != LRT_SBS_LAYOUT_UNDEFINED)
    return LRT_ERR_UNSUPPORTED;
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#else
  threads = 1;
#endif
  Frame fr = build_frame(f, depth, threads);
  std::vector<uint32_t> leaves;
  for (size_t i = 0; i < fr.nodes.size(); i++)
    if (frame_is_leaf(fr.nodes[i].offset)) leaves.push_back(uint32_t(i));

  const uint32_t bs = hdr.brick_size, pad = hdr.brick_pad;
  const uint32_t v_size = bs + 2 * pad + 1, v3 = v_size * v_size * v_size;
  const uint32_t vals_per_int = 4 / hdr.bytes_per_value, bits = 8 * hdr.bytes_per_value;
  const uint32_t max_q = hdr.bytes_per_value == 4 ? 0xFFFFFFFFu : ((1u << bits) - 1);
  const uint32_t words = (v3 + vals_per_int - 1) / vals_per_int;

  out.hdr = hdr;
  out.nodes.clear();
  out.values.clear();
  const size_t chunk = 4096;
  std::vector<uint32_t> cwords;
  std::vector<lrt_sbs_node> cnodes;
  std::vector<char> keep;
  for (size_t c0 = 0; c0 < leaves.size(); c0 += chunk) {
    const size_t cn = std::min(chunk, leaves.size() - c0);
    cwords.assign(cn * words, 0u);
    cnodes.assign(cn, lrt_sbs_node{0, 0, 0, 0});
    keep.assign(cn, 0);
#pragma omp parallel num_threads(threads)
    {
      std::vector<float> values(v3);
#pragma omp for schedule(dynamic, 8)
      for (long li = 0; li < long(cn); li++) {
        const uint32_t idx = leaves[c0 + li];
        const FrameNode &nd = fr.nodes[idx];
        const uint32_t p[3] = {uint32_t(fr.pd[4 * size_t(idx)]), uint32_t(fr.pd[4 * size_t(idx) + 1]),
                               uint32_t(fr.pd[4 * size_t(idx) + 2])};
        const float d = fr.pd[4 * size_t(idx) + 3];
        float mn = 1000, mx = -1000;
        for (int i = 0; i < 8; i++) { mn = std::min(mn, nd.values[i]); mx = std::max(mx, nd.values[i]); }
        const float p0x = 2.0f * (d * float(p[0])) - 1.0f, p0y = 2.0f * (d * float(p[1])) - 1.0f,
                    p0z = 2.0f * (d * float(p[2])) - 1.0f;
        const float dp = 2.0f * d / float(bs);
        for (int i = -int(pad); i <= int(bs + pad); i++)
          for (int j = -int(pad); j <= int(bs + pad); j++)
            for (int k = -int(pad); k <= int(bs + pad); k++) {
              float val = 2e6f;
              const int B = int(bs);
              if (i == 0) {
                if (j == 0) { if (k == 0) val = nd.values[0]; else if (k == B) val = nd.values[1]; }
                else if (j == B) { if (k == 0) val = nd.values[2]; else if (k == B) val = nd.values[3]; }
              } else if (i == B) {
                if (j == 0) { if (k == 0) val = nd.values[4]; else if (k == B) val = nd.values[5]; }
                else if (j == B) { if (k == 0) val = nd.values[6]; else if (k == B) val = nd.values[7]; }
              }
              if (val > 1e6f) val = sdf_eval(f, p0x + dp * float(i), p0y + dp * float(j), p0z + dp * float(k));
              const uint32_t vid = uint32_t(i + int(pad)) * v_size * v_size + uint32_t(j + int(pad)) * v_size +
                                   uint32_t(k + int(pad));
              values[vid] = val;
              mn = std::min(mn, val);
              mx = std::max(mx, val);
            }
        // is_border_node, :49-53
        const uint32_t level_size = uint32_t(1 / d);
        const float bd_max = float(2 * std::sqrt(3.0) / level_size);
        if (!((mn <= 0) && (mx > -bd_max))) continue;
        const uint32_t lod_size = uint32_t(1.0f / d);
        const float d_max = float(2 * std::sqrt(3.0) / lod_size);
        keep[li] = 1;
        cnodes[li].pos_xy = (p[0] << 16) | p[1];
        cnodes[li].pos_z_lod_size = (p[2] << 16) | lod_size;
        uint32_t *w = &cwords[size_t(li) * words];
        for (uint32_t i = 0; i < v3; i++) {
          // float->unsigned of values >= 2^32 is undefined in the reference; saturate
          float fq = float(max_q) * ((values[i] + d_max) / (2 * d_max));
          fq = std::max(0.0f, fq);
          uint32_t q = fq >= 4294967296.0f ? 0xFFFFFFFFu : uint32_t(fq);
          q = std::min(q, max_q);
          w[i / vals_per_int] |= q << (bits * (i % vals_per_int));
        }
      }
    }
    for (size_t li = 0; li < cn; li++) {
      if (!keep[li]) continue;
      lrt_sbs_node nd = cnodes[li];
      nd.data_offset = uint32_t(out.values.size());
      out.nodes.push_back(nd);
      out.values.insert(out.values.end(), cwords.begin() + li * words, cwords.begin() + (li + 1) * words);
    }
  }
  return LRT_OK;
}

void build_occupancy(const SbsData &sbs, const std::vector<float> &values_f, uint32_t occ_words,
                     std::vector<uint32_t> &occ) {
  const lrt_sbs_header &h = sbs.hdr;
  const uint32_t bs = h.brick_size, pad = h.brick_pad, v = bs + 2 * pad + 1;
  const uint32_t layout = h.aux_data & 0xFF000000u;
  const bool indexed = layout == LRT_SBS_LAYOUT_ID32F_IRGB32F || layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN;
  const uint32_t vpi = 4 / h.bytes_per_value, bits = 8 * h.bytes_per_value;
  const uint32_t max_val = h.bytes_per_value == 4 ? 0xFFFFFFFFu : ((1u << bits) - 1);
  const long nb = long(sbs.nodes.size());
  occ.assign(size_t(nb) * occ_words, 0u);
#pragma omp parallel for schedule(dynamic, 256)
  for (long b = 0; b < nb; b++) {
    const lrt_sbs_node &nd = sbs.nodes[b];
    const float sz = float(nd.pos_z_lod_size & 0x0000FFFF);
    const float sz_inv = 2.0f / sz;
    const float d_max = 1.73205081f * sz_inv;          // load_distance_values, BVH/BVH2Common.cpp:749-759
    const float mult = 2 * d_max / float(max_val);
    auto value = [&](uint32_t vid) -> float {
      if (indexed) return values_f[sbs.values[nd.data_offset + vid]];
      const uint32_t q = (sbs.values[nd.data_offset + vid / vpi] >> (bits * (vid % vpi))) & max_val;
      return -d_max + mult * float(q);
    };
    uint32_t *o = &occ[size_t(b) * occ_words];
    for (uint32_t i = 0; i < bs; i++)
      for (uint32_t j = 0; j < bs; j++)
        for (uint32_t k = 0; k < bs; k++) {
          bool any = false;
          for (int c = 0; c < 8 && !any; c++) {
            const uint32_t vid = (i + ((c & 4) >> 2) + pad) * v * v + (j + ((c & 2) >> 1) + pad) * v + (k + (c & 1) + pad);
            any = value(vid) <= 0.0f;
          }
          const uint32_t bit = (i * bs + j) * bs + k;
          if (any) o[bit >> 5] |= 1u << (bit & 31);
        }
  }
}

// frame_octree_to_SVS_rec, utils/sparse_octree_builder.cpp:2346-2387
static void svs_rec(const Frame &fr, uint32_t idx, uint32_t px, uint32_t py, uint32_t pz, uint32_t lod,
                    std::vector<lrt_svs_node> &out) {
  const uint32_t ofs = fr.nodes[idx].offset;
  if (frame_is_leaf(ofs)) {
    const float d_max = float(2 * std::sqrt(3.0) / lod);
    float mn = 1000, mx = -1000;
    for (int i = 0; i < 8; i++) { mn = std::min(mn, fr.nodes[idx].values[i]); mx = std::max(mx, fr.nodes[idx].values[i]); }
    if ((mn <= 0) && (mx > -d_max)) {
      lrt_svs_node s;
      s.pos_xy = (px << 16) | py;
      s.pos_z_lod_size = (pz << 16) | lod;
      s.values[0] = 0u;
      s.values[1] = 0u;
      for (int i = 0; i < 8; i++) {
        const float fq = std::max(0.0f, 255 * ((fr.nodes[idx].values[i] + d_max) / (2 * d_max)) + 0.5f);
        uint32_t q = uint32_t(fq);
        q = std::min(q, 255u);
        s.values[i / 4] |= q << (8 * (i % 4));
      }
      out.push_back(s);
    }
  } else {
    for (int i = 0; i < 8; i++)
      svs_rec(fr, ofs + i, 2 * px + ((i & 4) >> 2), 2 * py + ((i & 2) >> 1), 2 * pz + (i & 1), 2 * lod, out);
  }
}

lrt_status build_svs(const lrt_sdf_desc &f, uint32_t depth, int threads, std::vector<lrt_svs_node> &out) {
  if (depth < 2 || depth > 15) return LRT_ERR_INVALID;
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#else
  threads = 1;
#endif
  Frame fr = build_frame(f, depth, threads);
  out.clear();
  svs_rec(fr, 0, 0, 0, 0, 1, out);
  return LRT_OK;
}

}  // namespace lrt
