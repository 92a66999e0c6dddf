/*
 * CPU oracle, scene side — TEST INFRASTRUCTURE ONLY (see lrt_oracle.h).
 * Restates the reference's SDF -> frame octree -> SBS/SVS construction
 * (utils/sparse_octree_builder.cpp) single-threaded, plus a deliberately simple
 * median-split BVH2 builder (the reference uses Embree's SAH builder, which is
 * absent; with closest-hit traversal the topology does not change results).
 */
#include "lrt_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------- analytic SDFs used by the configs ---------------- */
static float sd_sphere(const float *s, float x, float y, float z) {
  float dx = x - s[0], dy = y - s[1], dz = z - s[2];
  return sqrtf(dx * dx + dy * dy + dz * dz) - s[3];
}

/* rounded box {c[3], half[3], r, R[9]}: q = |R(p-c)| - (half - r);
 * length(max(q,0)) + min(max(q.x,max(q.y,q.z)),0) - r */
static float sd_round_box(const float *b, float x, float y, float z) {
  float px = x - b[0], py = y - b[1], pz = z - b[2];
  const float *R = b + 7;
  float lx = R[0] * px + R[1] * py + R[2] * pz;
  float ly = R[3] * px + R[4] * py + R[5] * pz;
  float lz = R[6] * px + R[7] * py + R[8] * pz;
  float qx = fabsf(lx) - (b[3] - b[6]), qy = fabsf(ly) - (b[4] - b[6]), qz = fabsf(lz) - (b[5] - b[6]);
  float mx = qx > 0 ? qx : 0, my = qy > 0 ? qy : 0, mz = qz > 0 ? qz : 0;
  float outside = sqrtf(mx * mx + my * my + mz * mz);
  float m = qx > qy ? qx : qy; m = m > qz ? m : qz;
  float inside = m < 0 ? m : 0;
  return outside + inside - b[6];
}

/* polynomial smooth minimum: h = max(k-|a-b|,0)/k; min(a,b) - h*h*k*0.25 */
static float smin_poly(float a, float b, float k) {
  float m = a < b ? a : b;
  if (k <= 0.0f) return m;
  float h = k - fabsf(a - b); h = h > 0 ? h : 0; h = h / k;
  return m - h * h * k * 0.25f;
}

float orc_sdf_eval(const orc_sdf *f, float x, float y, float z) {
  float d = 1e10f;
  int first = 1;
  for (uint32_t i = 0; i < f->n_spheres; i++) {
    float v = sd_sphere(f->spheres + 4 * i, x, y, z);
    d = first ? v : smin_poly(d, v, f->k); first = 0;
  }
  for (uint32_t i = 0; i < f->n_boxes; i++) {
    float v = sd_round_box(f->boxes + 16 * i, x, y, z);
    d = first ? v : smin_poly(d, v, f->k); first = 0;
  }
  return d;
}

/* ---------------- frame octree (utils/sparse_octree_builder.cpp:72-252) ---------------- */
typedef struct { float values[8]; uint32_t offset; } fnode;   /* SdfFrameOctreeNode subset */
typedef struct { fnode *v; size_t n, cap; } fvec;
static void fv_resize(fvec *a, size_t n) {
  if (n > a->cap) { size_t c = a->cap ? a->cap : 1024; while (c < n) c *= 2; a->v = (fnode *)realloc(a->v, c * sizeof(fnode)); a->cap = c; }
  for (size_t i = a->n; i < n; i++) { memset(&a->v[i], 0, sizeof(fnode)); }
  a->n = n;
}

static inline float sdf_at(const orc_sdf *f, float px, float py, float pz, float cx, float cy, float cz, float d) {
  /* sdf(2.0f * ((p + c) * d) - float3(1, 1, 1)) */
  return orc_sdf_eval(f, 2.0f * ((px + cx) * d) - 1.0f, 2.0f * ((py + cy) * d) - 1.0f, 2.0f * ((pz + cz) * d) - 1.0f);
}

/* add_node_rec, :72-96 */
static void add_node_rec(fvec *nodes, const orc_sdf *f, uint32_t idx, uint32_t depth, uint32_t max_depth,
                         float px, float py, float pz, float d) {
  float vc = sdf_at(f, px, py, pz, 0.5f, 0.5f, 0.5f, d);
  float mn = 1000, mx = -1000;
  for (int c = 0; c < 8; c++) {
    float v = sdf_at(f, px, py, pz, (float)((c & 4) >> 2), (float)((c & 2) >> 1), (float)(c & 1), d);
    nodes->v[idx].values[c] = v;
    mn = mn < v ? mn : v; mx = mx < v ? v : mx;
  }
  if (depth < max_depth && (fabsf(vc) < sqrtf(3.0f) * d || mn * mx <= 0)) {
    uint32_t off = (uint32_t)nodes->n;
    nodes->v[idx].offset = off;
    fv_resize(nodes, nodes->n + 8);
    for (uint32_t c = 0; c < 8; c++)
      add_node_rec(nodes, f, off + c, depth + 1, max_depth, 2 * px + (float)((c & 4) >> 2),
                   2 * py + (float)((c & 2) >> 1), 2 * pz + (float)(c & 1), d / 2);
  }
}

typedef struct { float p[3], d, value; uint32_t level, children; } lnode;

/* construct_sdf_frame_octree, :125-252, as if run with one thread.  Leaves'
 * (p, d) are returned through *out_pd (4 floats per node). */
static fnode *build_frame(const orc_sdf *f, uint32_t depth, size_t *out_n, float **out_pd) {
  uint32_t min_remove_level = depth < 4 ? depth : 4;
  size_t nl = 0, capl = 16;
  lnode *L = (lnode *)malloc(capl * sizeof(lnode));
  L[0].p[0] = L[0].p[1] = L[0].p[2] = 0; L[0].d = 1.0f; L[0].level = 0; L[0].children = 0; L[0].value = 1000.0f;
  nl = 1;
  for (size_t i = 0; i < nl; i++) {
    if (L[i].level < min_remove_level) {
      L[i].children = (uint32_t)nl;
      for (int j = 0; j < 8; j++) {
        if (nl == capl) { capl *= 2; L = (lnode *)realloc(L, capl * sizeof(lnode)); }
        lnode c; c.d = L[i].d / 2;
        c.p[0] = 2 * L[i].p[0] + (float)((j & 4) >> 2); c.p[1] = 2 * L[i].p[1] + (float)((j & 2) >> 1);
        c.p[2] = 2 * L[i].p[2] + (float)(j & 1);
        c.level = L[i].level + 1; c.children = 0; c.value = 1000.0f;
        L[nl++] = c;
      }
    }
  }
  /* is_border, :38-41 */
  unsigned char *border = (unsigned char *)calloc(nl, 1);
  for (size_t i = 0; i < nl; i++) {
    L[i].value = sdf_at(f, L[i].p[0], L[i].p[1], L[i].p[2], 0.5f, 0.5f, 0.5f, L[i].d);
    int isb = L[i].level < 2 ? 1 : (fabs((double)L[i].value) < sqrt(3.0) * pow(2.0, -(double)L[i].level));
    border[i] = (L[i].children == 0 && isb);
  }
  fvec res = {0, 0, 0};
  fv_resize(&res, nl);
  for (size_t i = 0; i < nl; i++) {
    for (int c = 0; c < 8; c++)
      res.v[i].values[c] = sdf_at(f, L[i].p[0], L[i].p[1], L[i].p[2], (float)((c & 4) >> 2),
                                  (float)((c & 2) >> 1), (float)(c & 1), L[i].d);
    res.v[i].offset = L[i].children;
    if (border[i]) {
      /* a local subtree built by add_node_rec, root at local index 0 */
      fvec sub = {0, 0, 0};
      fv_resize(&sub, 1);
      add_node_rec(&sub, f, 0, L[i].level, depth, L[i].p[0], L[i].p[1], L[i].p[2], L[i].d);
      if (sub.n > 1) {
        size_t prev = res.n;
        long shift = (long)prev - 1;   /* local index 1 lands at prev */
        res.v[i].offset = (uint32_t)((long)sub.v[0].offset + shift);
        fv_resize(&res, prev + sub.n - 1);
        memcpy(res.v + prev, sub.v + 1, (sub.n - 1) * sizeof(fnode));
        for (size_t j = prev; j < res.n; j++)
          if (res.v[j].offset != 0) res.v[j].offset = (uint32_t)((long)res.v[j].offset + shift);
      }
      free(sub.v);
    }
  }
  /* layers: (p, d) per node (octree_to_layers, :262-275) */
  float *pd = (float *)malloc(res.n * 4 * sizeof(float));
  size_t *stk = (size_t *)malloc((res.n + 8) * sizeof(size_t));
  size_t sp = 0;
  pd[0] = pd[1] = pd[2] = 0; pd[3] = 1.0f;
  stk[sp++] = 0;
  while (sp) {
    size_t idx = stk[--sp];
    uint32_t ofs = res.v[idx].offset;
    if (!(ofs == 0 || (ofs & 0x80000000u))) {
      for (int c = 0; c < 8; c++) {
        float *q = pd + 4 * (ofs + c);
        q[0] = 2 * pd[4 * idx + 0] + (float)((c & 4) >> 2);
        q[1] = 2 * pd[4 * idx + 1] + (float)((c & 2) >> 1);
        q[2] = 2 * pd[4 * idx + 2] + (float)(c & 1);
        q[3] = pd[4 * idx + 3] / 2;
        stk[sp++] = ofs + c;
      }
    }
  }
  free(stk); free(L); free(border);
  *out_n = res.n; *out_pd = pd;
  return res.v;
}

/* frame_octree_to_SBS, :291-444 (brick order = frame node order, one thread) */
uint32_t orc_build_sbs(const orc_sdf *f, uint32_t depth, orc_sbs_header hdr, orc_sbs_node **out_nodes,
                       uint32_t **out_values, uint32_t *out_n_values) {
  size_t nn; float *pd;
  fnode *nodes = build_frame(f, depth, &nn, &pd);
  const uint32_t bs = hdr.brick_size, pad = hdr.brick_pad;
  const uint32_t v_size = bs + 2 * pad + 1, v3 = v_size * v_size * v_size;
  const uint32_t vals_per_int = 4 / hdr.bytes_per_value, bits = 8 * hdr.bytes_per_value;
  const uint32_t max_q = hdr.bytes_per_value == 4 ? 0xFFFFFFFFu : ((1u << bits) - 1);
  const uint32_t words = (v3 + vals_per_int - 1) / vals_per_int;
  size_t cap = 1024, n = 0;
  orc_sbs_node *out = (orc_sbs_node *)malloc(cap * sizeof(orc_sbs_node));
  uint32_t *vals = (uint32_t *)malloc(cap * words * sizeof(uint32_t));
  float *values = (float *)malloc(v3 * sizeof(float));
  for (size_t idx = 0; idx < nn; idx++) {
    uint32_t ofs = nodes[idx].offset;
    if (!(ofs == 0 || (ofs & 0x80000000u))) continue;
    uint32_t p[3] = {(uint32_t)pd[4 * idx], (uint32_t)pd[4 * idx + 1], (uint32_t)pd[4 * idx + 2]};
    float d = pd[4 * idx + 3];
    float mn = 1000, mx = -1000;
    for (int i = 0; i < 8; i++) { float v = nodes[idx].values[i]; mn = mn < v ? mn : v; mx = mx < v ? v : mx; }
    float p0x = 2.0f * (d * (float)p[0]) - 1.0f, p0y = 2.0f * (d * (float)p[1]) - 1.0f, p0z = 2.0f * (d * (float)p[2]) - 1.0f;
    float dp = 2.0f * d / (float)bs;
    for (int i = -(int)pad; i <= (int)(bs + pad); i++)
      for (int j = -(int)pad; j <= (int)(bs + pad); j++)
        for (int k = -(int)pad; k <= (int)(bs + pad); k++) {
          float val = 2e6f;
          if (i == 0) {
            if (j == 0) { if (k == 0) val = nodes[idx].values[0]; else if (k == (int)bs) val = nodes[idx].values[1]; }
            else if (j == (int)bs) { if (k == 0) val = nodes[idx].values[2]; else if (k == (int)bs) val = nodes[idx].values[3]; }
          } else if (i == (int)bs) {
            if (j == 0) { if (k == 0) val = nodes[idx].values[4]; else if (k == (int)bs) val = nodes[idx].values[5]; }
            else if (j == (int)bs) { if (k == 0) val = nodes[idx].values[6]; else if (k == (int)bs) val = nodes[idx].values[7]; }
          }
          if (val > 1e6f) val = orc_sdf_eval(f, p0x + dp * (float)i, p0y + dp * (float)j, p0z + dp * (float)k);
          uint32_t vid = ((uint32_t)(i + (int)pad)) * v_size * v_size + ((uint32_t)(j + (int)pad)) * v_size + (uint32_t)(k + (int)pad);
          values[vid] = val;
          mn = mn < val ? mn : val; mx = mx < val ? val : mx;
        }
    /* is_border_node, :49-53 */
    uint32_t level_size = (uint32_t)(1 / d);
    float bd_max = (float)(2 * sqrt(3.0) / level_size);
    if (!((mn <= 0) && (mx > -bd_max))) continue;
    uint32_t lod_size = (uint32_t)(1.0f / d);
    float d_max = (float)(2 * sqrt(3.0) / lod_size);
    if (n == cap) { cap *= 2; out = (orc_sbs_node *)realloc(out, cap * sizeof(orc_sbs_node)); vals = (uint32_t *)realloc(vals, cap * words * sizeof(uint32_t)); }
    out[n].data_offset = (uint32_t)(n * words);
    out[n].pos_xy = (p[0] << 16) | p[1];
    out[n].pos_z_lod_size = (p[2] << 16) | lod_size;
    out[n].pad = 0;
    uint32_t *w = vals + n * words;
    memset(w, 0, words * sizeof(uint32_t));
    for (uint32_t i = 0; i < v3; i++) {
      /* max_val*((v+d_max)/(2*d_max)) in float, clamped at 0; float->unsigned
       * conversion of values >= 2^32 is undefined in C++, here it saturates */
      float fq = (float)max_q * ((values[i] + d_max) / (2 * d_max));
      fq = 0.0f < fq ? fq : 0.0f;
      uint32_t q = fq >= 4294967296.0f ? 0xFFFFFFFFu : (uint32_t)fq;
      q = q < max_q ? q : max_q;
      w[i / vals_per_int] |= q << (bits * (i % vals_per_int));
    }
    n++;
  }
  free(values); free(nodes); free(pd);
  *out_nodes = out; *out_values = vals; *out_n_values = (uint32_t)(n * words);
  return (uint32_t)n;
}

/* frame_octree_to_SVS_rec, :2346-2387 */
static void svs_rec(const fnode *fr, uint32_t idx, uint32_t px, uint32_t py, uint32_t pz, uint32_t lod,
                    orc_svs_node **out, size_t *n, size_t *cap) {
  uint32_t ofs = fr[idx].offset;
  if (ofs == 0 || (ofs & 0x80000000u)) {
    float d_max = (float)(2 * sqrt(3.0) / lod);
    float mn = 1000, mx = -1000;
    for (int i = 0; i < 8; i++) { float v = fr[idx].values[i]; mn = mn < v ? mn : v; mx = mx < v ? v : mx; }
    float bd_max = (float)(2 * sqrt(3.0) / lod);
    if ((mn <= 0) && (mx > -bd_max)) {
      if (*n == *cap) { *cap *= 2; *out = (orc_svs_node *)realloc(*out, *cap * sizeof(orc_svs_node)); }
      orc_svs_node *s = &(*out)[(*n)++];
      s->pos_xy = (px << 16) | py;
      s->pos_z_lod_size = (pz << 16) | lod;
      s->values[0] = 0u; s->values[1] = 0u;
      for (int i = 0; i < 8; i++) {
        float fq = 255 * ((fr[idx].values[i] + d_max) / (2 * d_max)) + 0.5f;
        fq = 0.0f < fq ? fq : 0.0f;
        uint32_t q = (uint32_t)fq;
        q = q < 255u ? q : 255u;
        s->values[i / 4] |= q << (8 * (i % 4));
      }
    }
  } else {
    for (int i = 0; i < 8; i++)
      svs_rec(fr, ofs + i, 2 * px + ((i & 4) >> 2), 2 * py + ((i & 2) >> 1), 2 * pz + (i & 1), 2 * lod, out, n, cap);
  }
}

uint32_t orc_build_svs(const orc_sdf *f, uint32_t depth, orc_svs_node **out_nodes) {
  size_t nn; float *pd;
  fnode *nodes = build_frame(f, depth, &nn, &pd);
  size_t n = 0, cap = 1024;
  orc_svs_node *out = (orc_svs_node *)malloc(cap * sizeof(orc_svs_node));
  svs_rec(nodes, 0, 0, 0, 0, 1, &out, &n, &cap);
  free(nodes); free(pd);
  *out_nodes = out;
  return (uint32_t)n;
}

/* ---------------- BVH2: recursive median split ---------------- */
typedef struct {
  const float *boxes; uint32_t *ids; uint32_t prims_in_leaf;
  orc_bvh_pair *pairs; uint32_t n_pairs;
  uint32_t *leaf_sc; uint32_t n_leaves;
} bctx;

static int g_axis; static const float *g_boxes;
static int cmp_centroid(const void *a, const void *b) {
  uint32_t ia = *(const uint32_t *)a, ib = *(const uint32_t *)b;
  float ca = g_boxes[6 * ia + g_axis] + g_boxes[6 * ia + 3 + g_axis];
  float cb = g_boxes[6 * ib + g_axis] + g_boxes[6 * ib + 3 + g_axis];
  if (ca < cb) return -1;
  if (ca > cb) return 1;
  return ia < ib ? -1 : (ia > ib ? 1 : 0);
}

static void bounds_of(const bctx *c, uint32_t b, uint32_t e, orc_bvh_node *nd) {
  for (int k = 0; k < 3; k++) { nd->bmin[k] = 3.4e38f; nd->bmax[k] = -3.4e38f; }
  for (uint32_t i = b; i < e; i++) {
    const float *bx = c->boxes + 6 * c->ids[i];
    for (int k = 0; k < 3; k++) {
      nd->bmin[k] = bx[k] < nd->bmin[k] ? bx[k] : nd->bmin[k];
      nd->bmax[k] = bx[3 + k] > nd->bmax[k] ? bx[3 + k] : nd->bmax[k];
    }
  }
}

/* returns the child reference (pair index, or LEAF_BIT|payload) for range [b,e) */
static uint32_t build_rec(bctx *c, uint32_t b, uint32_t e);

static uint32_t make_leaf(bctx *c, uint32_t b, uint32_t e) {
  if (c->prims_in_leaf == 1) return 0x80000000u | (1u << 24) | (c->ids[b] & 0x00FFFFFFu);
  c->leaf_sc[c->n_leaves] = 0x80000000u | (((e - b) << 24) & 0x7F000000u) | (b & 0x00FFFFFFu);
  return 0x80000000u | (1u << 24) | (c->n_leaves++ & 0x00FFFFFFu);
}

static uint32_t build_pair(bctx *c, uint32_t b, uint32_t m, uint32_t e) {
  uint32_t me = c->n_pairs++;
  bounds_of(c, b, m, &c->pairs[me].l);
  bounds_of(c, m, e, &c->pairs[me].r);
  c->pairs[me].l.escape = c->pairs[me].r.escape = 0;
  uint32_t l = (m - b <= c->prims_in_leaf) ? make_leaf(c, b, m) : build_rec(c, b, m);
  uint32_t r = (e - m <= c->prims_in_leaf) ? make_leaf(c, m, e) : build_rec(c, m, e);
  c->pairs[me].l.left_offset = l;
  c->pairs[me].r.left_offset = r;
  return me;
}

static uint32_t build_rec(bctx *c, uint32_t b, uint32_t e) {
  float cmin[3] = {3.4e38f, 3.4e38f, 3.4e38f}, cmax[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (uint32_t i = b; i < e; i++)
    for (int k = 0; k < 3; k++) {
      float cc = c->boxes[6 * c->ids[i] + k] + c->boxes[6 * c->ids[i] + 3 + k];
      cmin[k] = cc < cmin[k] ? cc : cmin[k]; cmax[k] = cc > cmax[k] ? cc : cmax[k];
    }
  int ax = 0;
  for (int k = 1; k < 3; k++) if (cmax[k] - cmin[k] > cmax[ax] - cmin[ax]) ax = k;
  g_axis = ax; g_boxes = c->boxes;
  qsort(c->ids + b, e - b, sizeof(uint32_t), cmp_centroid);
  return build_pair(c, b, b + (e - b) / 2, e);
}

uint32_t orc_bvh2_build(const float *boxes, uint32_t n, uint32_t prims_in_leaf, orc_bvh_pair **out_pairs,
                        uint32_t **out_leaf_start_count, uint32_t **out_order, uint32_t *out_n_leaves) {
  bctx c;
  c.boxes = boxes; c.prims_in_leaf = prims_in_leaf ? prims_in_leaf : 1;
  c.ids = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
  for (uint32_t i = 0; i < n; i++) c.ids[i] = i;
  c.pairs = (orc_bvh_pair *)calloc(n + 2, sizeof(orc_bvh_pair));
  c.n_pairs = 0;
  c.leaf_sc = (uint32_t *)malloc((n + 2) * sizeof(uint32_t));
  c.n_leaves = 0;
  if (n <= c.prims_in_leaf) {
    /* a single leaf: duplicate it into both children of the root pair */
    uint32_t me = c.n_pairs++;
    bounds_of(&c, 0, n, &c.pairs[me].l);
    uint32_t lf = make_leaf(&c, 0, n);
    c.pairs[me].l.left_offset = lf;
    c.pairs[me].r = c.pairs[me].l;
  } else {
    uint32_t root_b = 0, root_e = n;
    /* root pair holds the two halves of the first split */
    float cmin[3] = {3.4e38f, 3.4e38f, 3.4e38f}, cmax[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (uint32_t i = 0; i < n; i++)
      for (int k = 0; k < 3; k++) {
        float cc = boxes[6 * i + k] + boxes[6 * i + 3 + k];
        cmin[k] = cc < cmin[k] ? cc : cmin[k]; cmax[k] = cc > cmax[k] ? cc : cmax[k];
      }
    int ax = 0;
    for (int k = 1; k < 3; k++) if (cmax[k] - cmin[k] > cmax[ax] - cmin[ax]) ax = k;
    g_axis = ax; g_boxes = boxes;
    qsort(c.ids, n, sizeof(uint32_t), cmp_centroid);
    build_pair(&c, root_b, root_e / 2, root_e);
  }
  *out_pairs = c.pairs;
  if (out_leaf_start_count) *out_leaf_start_count = c.leaf_sc; else free(c.leaf_sc);
  if (out_order) *out_order = c.ids; else free(c.ids);
  if (out_n_leaves) *out_n_leaves = c.n_leaves;
  return c.n_pairs;
}

/* ---------------- camera matrices ---------------- */
void orc_perspective(float fov_deg, float aspect, float znear, float zfar, float out[16]) {
  memset(out, 0, 16 * sizeof(float));
  const float ymax = znear * tanf(fov_deg * 3.14159265358979323846f / 180.0f * 0.5f);
  const float xmax = ymax * aspect;
  const float l = -xmax, r = xmax, b = -ymax, t = ymax;
  out[0] = 2.0f * znear / (r - l);
  out[2] = (r + l) / (r - l);
  out[5] = 2.0f * znear / (t - b);
  out[6] = (t + b) / (t - b);
  out[10] = (-zfar - znear) / (zfar - znear);
  out[11] = (-2.0f * znear * zfar) / (zfar - znear);
  out[14] = -1.0f;
}

void orc_look_at(const float eye[3], const float center[3], const float up[3], float out[16]) {
  float z[3] = {eye[0] - center[0], eye[1] - center[1], eye[2] - center[2]};
  float lz = sqrtf(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
  for (int i = 0; i < 3; i++) z[i] /= lz;
  float x[3] = {up[1] * z[2] - up[2] * z[1], up[2] * z[0] - up[0] * z[2], up[0] * z[1] - up[1] * z[0]};
  float lx = sqrtf(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  for (int i = 0; i < 3; i++) x[i] /= lx;
  float y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
  memset(out, 0, 16 * sizeof(float));
  for (int i = 0; i < 3; i++) { out[i] = x[i]; out[4 + i] = y[i]; out[8 + i] = z[i]; }
  out[3] = -(x[0] * eye[0] + x[1] * eye[1] + x[2] * eye[2]);
  out[7] = -(y[0] * eye[0] + y[1] * eye[1] + y[2] * eye[2]);
  out[11] = -(z[0] * eye[0] + z[1] * eye[1] + z[2] * eye[2]);
  out[15] = 1.0f;
}

void orc_inverse4x4(const float m[16], float out[16]) {
  double a[4][8];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 8; j++) a[i][j] = j < 4 ? (double)m[i * 4 + j] : (j - 4 == i ? 1.0 : 0.0);
  for (int c = 0; c < 4; c++) {
    int p = c;
    for (int r = c + 1; r < 4; r++) if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
    if (p != c) for (int j = 0; j < 8; j++) { double t = a[c][j]; a[c][j] = a[p][j]; a[p][j] = t; }
    double inv = 1.0 / a[c][c];
    for (int j = 0; j < 8; j++) a[c][j] *= inv;
    for (int r = 0; r < 4; r++) if (r != c) { double f = a[r][c]; for (int j = 0; j < 8; j++) a[r][j] -= f * a[c][j]; }
  }
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) out[i * 4 + j] = (float)a[i][j + 4];
}
