/*
 * CPU oracle for the LiteRT ray-query hot path — TEST INFRASTRUCTURE ONLY.
 * Plain-C restatement of the reference algorithm; see lrt_oracle.h for scope
 * and pinning.  Compiled with -ffp-contract=off so that x86-64 and aarch64
 * hosts produce identical float results (the reference's own x86-64 build
 * performs no contraction).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU legs load this library.
 */
#include "lrt_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "lrt_oracle_math.h"

/* ---------------- BVH/BVH2Common.cpp ---------------- */
static int need_normal(const orc_preset *p) {   /* BVH/BVH2Common.cpp:20-27 */
  return p->render_mode == 1 || p->render_mode == 8 || p->render_mode == 12 ||
         p->render_mode == 17 || p->render_mode == 18;
}

/* encode_normal, BVH/BVH2Common.cpp:29-35 */
static f2 encode_normal(f3 v) {
  const float s = 1.0f / (fabsf(v.x) + fabsf(v.y) + fabsf(v.z));
  f2 p; p.x = v.x * s; p.y = v.y * s;
  const float sx = (p.x >= 0.0f) ? 1.0f : -1.0f, sy = (p.y >= 0.0f) ? 1.0f : -1.0f;
  if (v.z <= 0.0f) { f2 r; r.x = (1.0f - fabsf(p.y)) * sx; r.y = (1.0f - fabsf(p.x)) * sy; return r; }
  return p;
}


/* LocalSurfaceIntersection, BVH/BVH2Common.cpp:274-631 (modes ST, ANALYTIC, NEWTON,
 * BBOX, IT; trilinear).  Writes *hit when the crossing is closer than hit->t. */
static void local_surface_intersection(const orc_scene *s, uint32_t type, f3 ray_dir, uint32_t geom_id,
                                       const float values[8], uint32_t prim_id, float d, float qNear,
                                       float qFar, f2 fNearFar, f3 start_q, orc_hit *hit,
                                       orc_counters *cnt) {
  const orc_preset *pr = &s->preset;
  const float EPS = 1e-6f;
  float d_inv = 1.0f / d;
  float t = qNear;
  int is_hit = 0;
  unsigned iter = 0;
  float start_sign = 1;
  float start_dist = eval_trilinear(values, add3(start_q, scl3(t, ray_dir)));
  if (cnt) cnt->n_finder++;
  if (pr->representation_mode == 0 /*SURFACE*/) start_sign = signf_(start_dist);
  start_dist *= start_sign;

  if (start_dist <= EPS || pr->sdf_node_intersect == 3 /*BBOX*/) {
    is_hit = 1;
  } else if (pr->sdf_node_intersect == 0 /*ST*/) {                      /* :301-317 */
    const unsigned ST_max_iters = 256;
    float dist = start_dist;
    while (t < qFar && dist > EPS && iter < ST_max_iters) {
      t += dist * d_inv;
      dist = start_sign * eval_trilinear(values, add3(start_q, scl3(t, ray_dir)));
      iter++;
    }
    is_hit = (dist <= EPS);
  } else {
    /* cubic coefficients, JCGT 2022 (:327-361) */
    float s000 = values[0] * d_inv, s001 = values[1] * d_inv, s010 = values[2] * d_inv, s011 = values[3] * d_inv;
    float s100 = values[4] * d_inv, s101 = values[5] * d_inv, s110 = values[6] * d_inv, s111 = values[7] * d_inv;
    float a = s101 - s001;
    float k0 = s000, k1 = s100 - s000, k2 = s010 - s000, k3 = s110 - s010 - k1;
    float k4 = k0 - s001, k5 = k1 - a, k6 = k2 - (s011 - s001), k7 = k3 - (s111 - s011 - a);
    f3 o = start_q, d3 = ray_dir;
    float m0 = o.x * o.y, m1 = d3.x * d3.y, m2 = o.x * d3.y + o.y * d3.x;
    float m3 = k5 * o.z - k1, m4 = k6 * o.z - k2, m5 = k7 * o.z - k3;
    float c0 = (k4 * o.z - k0) + o.x * m3 + o.y * m4 + m0 * m5;
    float c1 = d3.x * m3 + d3.y * m4 + m2 * m5 + d3.z * (k4 + k5 * o.x + k6 * o.y + k7 * m0);
    float c2 = m1 * m5 + d3.z * (k5 * d3.x + k6 * d3.y + k7 * m2);
    float c3 = k7 * m1 * d3.z;

    if (pr->sdf_node_intersect == 1 /*ANALYTIC*/) {                       /* :367-436 */
      float x1 = 1000, x2 = 1000, x3 = 1000;
      if (fabsf(c3) > 1e-2) {
        float aa = c2 / c3, b = c1 / c3, c = c0 / c3;
        float Q = (aa * aa - 3 * b) / 9;
        float R = (2 * aa * aa - 9 * aa * b + 27 * c) / 54;
        float Q3 = Q * Q * Q;
        /* The reference's unqualified sqrt(float) resolves to ::sqrt(double), which
         * promotes these expressions to double; std::acos/std::pow then take the
         * double overloads, std::cos(float) stays float.  LiteMath::M_PI is float. */
        if (R * R < Q3) {
          float theta = (float)acos((double)R / sqrt((double)Q3));
          x1 = (float)(-2 * sqrt((double)Q) * (double)cosf(theta / 3) - (double)(aa / 3));
          x2 = (float)(-2 * sqrt((double)Q) * (double)cosf((theta + 2 * 3.14159265358979323846f) / 3) - (double)(aa / 3));
          x3 = (float)(-2 * sqrt((double)Q) * (double)cosf((theta - 2 * 3.14159265358979323846f) / 3) - (double)(aa / 3));
        } else {
          float A = (float)((double)(-signf_(R)) *
                            pow((double)fabsf(R) + sqrt((double)(R * R - Q3)), (double)(1.0f / 3.0f)));
          float B = fabsf(A) > EPS ? Q / A : 0;
          x1 = A + B - aa / 3;
        }
      } else if (fabsf(c2) > 1e-4) {
        float aa = c2, b = c1, c = c0;
        float D = b * b - 4 * aa * c;
        if (D > 0) {
          float q = -0.5f * (b + signf_(b) * sqrtf(D));
          x1 = q / aa;
          if (fabsf(q) > EPS) x2 = c / q;
        }
      } else if (fabsf(c1) > EPS) {
        x1 = -c0 / c1;
      }
      x1 = x1 < 0 ? 1000 : x1;
      x2 = x2 < 0 ? 1000 : x2;
      x3 = x3 < 0 ? 1000 : x3;
      t = fminf_(x1, fminf_(x2, x3));
      is_hit = (t >= 0 && t <= qFar);
    } else if (pr->sdf_node_intersect == 2 /*NEWTON*/) {                  /* :437-522 */
      float aa = 3 * c3, b = 2 * c2, c = c1;
      float t0 = 0, t1 = qFar, t2 = qFar, t3 = qFar;
      float D = b * b - 4 * aa * c;
      if (D >= 0) {
        float q = -0.5f * (b + signf_(b) * sqrtf(D));
        t1 = fabsf(aa) > EPS ? q / aa : t0;
        t2 = fabsf(q) > EPS ? c / q : qFar;
        float tmp = fminf_(t1, t2);
        t2 = fmaxf_(t1, t2);
        t1 = tmp;
        t1 = clampf_(t1, t0, t3);
        t2 = clampf_(t2, t0, t3);
      }
      int s0 = c0 > 0;
      int s1 = (c0 + t1 * (c1 + t1 * (c2 + t1 * c3))) > 0;
      int s2 = (c0 + t2 * (c1 + t2 * (c2 + t2 * c3))) > 0;
      int s3 = (c0 + t3 * (c1 + t3 * (c2 + t3 * c3))) > 0;
      float nwt_min = t0, nwt_max = t0;
      if (s0 != s1) { nwt_min = t0; nwt_max = t1; }
      else if (s1 != s2) { nwt_min = t1; nwt_max = t2; }
      else if (s2 != s3) { nwt_min = t2; nwt_max = t3; }
      if (nwt_min < nwt_max) {
        const unsigned max_iters = 10;
        unsigned it = 0;
        float rtn = 0.5f * (nwt_min + nwt_max);
        float f = 1000;
        while (it < max_iters && fabsf(f) >= EPS) {
          f = c0 + rtn * (c1 + rtn * (c2 + rtn * c3));
          float df = c1 + rtn * (2 * c2 + rtn * 3 * c3);
          float dx = f / (df + signf_(df) * 1e-9f);
          rtn -= dx;
          it++;
        }
        t = rtn;
        is_hit = (t >= 0 && t <= qFar && fabsf(f) < EPS);
      } else {
        is_hit = 0;
      }
    } else {                                                              /* IT, :523-550 */
      const unsigned IT_max_iters = 256;
      const float k = 2;
      float e = 0.1f * qFar;
      float t_max = fabsf(c3) < EPS ? 1e6f : -c2 / (3 * c3);
      float df_max = 3 * c3 * t_max * t_max + 2 * c2 * t_max + c1;
      float dist = start_dist;
      while (t < qFar && dist > EPS && iter < IT_max_iters) {
        float df_1 = 3 * c3 * t * t + 2 * c2 * t + c1;
        float df_2 = 3 * c3 * (t + e) * (t + e) + 2 * c2 * (t + e) + c1;
        float L = (t_max > t && t_max < t + e) ? fmaxf_(df_max, fmaxf_(df_1, df_2)) : fmaxf_(df_1, df_2);
        L = fmaxf_(L, EPS);
        float st = fminf_((dist * d_inv) / L, e);
        t += st;
        e = k * st;
        dist = start_sign * eval_trilinear(values, add3(start_q, scl3(t, ray_dir)));
        iter++;
      }
      is_hit = (dist <= EPS);
    }
  }

  float tReal = fNearFar.x + d * t;
  if (t <= qFar && is_hit && tReal < hit->t) {                            /* :569-601 */
    f3 norm = mk3(0, 0, 1);
    if (need_normal(pr)) {
      f3 p0 = add3(start_q, scl3(t, ray_dir));
      const float h = 0.001f;
      float ddx = (eval_trilinear(values, add3(p0, mk3(h, 0, 0))) - eval_trilinear(values, add3(p0, mk3(-h, 0, 0)))) / (2 * h);
      float ddy = (eval_trilinear(values, add3(p0, mk3(0, h, 0))) - eval_trilinear(values, add3(p0, mk3(0, -h, 0)))) / (2 * h);
      float ddz = (eval_trilinear(values, add3(p0, mk3(0, 0, h))) - eval_trilinear(values, add3(p0, mk3(0, 0, -h)))) / (2 * h);
      norm = scl3(start_sign, normalize3(matmul4x3(s->inst_inv_t, mk3(ddx, ddy, ddz))));
    }
    f2 en = encode_normal(norm);
    hit->t = tReal;
    hit->prim_id = prim_id;
    hit->inst_id = 0;
    hit->geom_id = geom_id | (type << 24);
    hit->coords[0] = 0; hit->coords[1] = 0;
    hit->coords[2] = en.x; hit->coords[3] = en.y;
    if (pr->render_mode == 10 /*ST_ITERATIONS*/) hit->prim_id = iter;
  }
}

/* load_distance_values, BVH/BVH2Common.cpp:725-762 (+ SBS_v_to_i, sdfScene/sdf_scene.h:201-204) */
static float load_distance_values(const orc_scene *s, uint32_t node_id, f3 voxelPos, uint32_t v_size,
                                  float sz_inv, float values[8]) {
  const orc_sbs_header *h = &s->sbs_hdr;
  float vmin = 1e6f;
  uint32_t v_off = s->sbs_nodes[node_id].data_offset;
  const uint32_t layout = h->aux_data & 0xFF000000u;
  if (layout == (4u << 24) || layout == (5u << 24)) {
    for (int i = 0; i < 8; i++) {
      uint32_t vx = (uint32_t)voxelPos.x + ((i & 4) >> 2), vy = (uint32_t)voxelPos.y + ((i & 2) >> 1), vz = (uint32_t)voxelPos.z + (i & 1);
      uint32_t vId = (vx + h->brick_pad) * v_size * v_size + (vy + h->brick_pad) * v_size + (vz + h->brick_pad);
      values[i] = s->sbs_values_f[s->sbs_values[v_off + vId]];
      vmin = fminf_(vmin, values[i]);
    }
  } else {
    uint32_t vals_per_int = 4 / h->bytes_per_value;
    uint32_t bits = 8 * h->bytes_per_value;
    uint32_t max_val = h->bytes_per_value == 4 ? 0xFFFFFFFFu : ((1u << bits) - 1);
    float d_max = 1.73205081f * sz_inv;
    float mult = 2 * d_max / (float)max_val;
    for (int i = 0; i < 8; i++) {
      uint32_t vx = (uint32_t)voxelPos.x + ((i & 4) >> 2), vy = (uint32_t)voxelPos.y + ((i & 2) >> 1), vz = (uint32_t)voxelPos.z + (i & 1);
      uint32_t vId = (vx + h->brick_pad) * v_size * v_size + (vy + h->brick_pad) * v_size + (vz + h->brick_pad);
      uint32_t q = (s->sbs_values[v_off + vId / vals_per_int] >> (bits * (vId % vals_per_int))) & max_val;
      values[i] = -d_max + mult * (float)q;
      vmin = fminf_(vmin, values[i]);
    }
  }
  return vmin;
}

/* eval_dist_trilinear_diff (BVH/BVH2Common.cpp:656-686); a + -(b) is a - b exactly */
static f3 tri_diff(const float v[8], f3 dp) {
  float dx = -(1 - dp.y) * (1 - dp.z) * v[0] - (1 - dp.y) * (dp.z) * v[1] - (dp.y) * (1 - dp.z) * v[2] -
             (dp.y) * (dp.z) * v[3] + (1 - dp.y) * (1 - dp.z) * v[4] + (1 - dp.y) * (dp.z) * v[5] +
             (dp.y) * (1 - dp.z) * v[6] + (dp.y) * (dp.z) * v[7];
  float dy = -(1 - dp.x) * (1 - dp.z) * v[0] - (1 - dp.x) * (dp.z) * v[1] + (1 - dp.x) * (1 - dp.z) * v[2] +
             (1 - dp.x) * (dp.z) * v[3] - (dp.x) * (1 - dp.z) * v[4] - (dp.x) * (dp.z) * v[5] +
             (dp.x) * (1 - dp.z) * v[6] + (dp.x) * (dp.z) * v[7];
  float dz = -(1 - dp.x) * (1 - dp.y) * v[0] + (1 - dp.x) * (1 - dp.y) * v[1] - (1 - dp.x) * (dp.y) * v[2] +
             (1 - dp.x) * (dp.y) * v[3] - (dp.x) * (1 - dp.y) * v[4] + (dp.x) * (1 - dp.y) * v[5] -
             (dp.x) * (dp.y) * v[6] + (dp.x) * (dp.y) * v[7];
  return mk3(dx, dy, dz);
}
/* step (BVH/BVH2Common.cpp:689-694) */
static float step01(float e0, float e1, float x) { return clampf_((x - e0) / (e1 - e0), 0.0f, 1.0f); }

/* NORMAL_MODE_SDF_SMOOTHED for the ID32F_IRGB32F_IN layout (BVH/BVH2Common.cpp:838-905):
 * the normals of the 8 voxels around the hit, read across brick borders through the
 * 27-neighbour table, blended with weights that switch over +-beta of the voxel centre */
static void smooth_normal(const orc_scene *s, uint32_t node_id, f3 voxelPos, f3 start_q, float fnear, float d,
                          f3 ray_dir, uint32_t v_size, float sz_inv, orc_hit *hit) {
  const orc_sbs_header *h = &s->sbs_hdr;
  const float beta = 0.5f;
  const f3 dp = add3(start_q, scl3((hit->t - fnear) / d, ray_dir));
  f3 normals[8];
  float values_n[8];
  for (int i = 0; i < 8; i++) normals[i] = mk3(0, 0, 0);
  const f3 nmq = mk3(dp.x < 0.5f ? step01(-beta, beta, dp.x) : step01(-beta, beta, dp.x - 1.0f),
                     dp.y < 0.5f ? step01(-beta, beta, dp.y) : step01(-beta, beta, dp.y - 1.0f),
                     dp.z < 0.5f ? step01(-beta, beta, dp.z) : step01(-beta, beta, dp.z - 1.0f));
  const int v0[3] = {(int)(dp.x < 0.5f ? voxelPos.x - 1 : voxelPos.x), (int)(dp.y < 0.5f ? voxelPos.y - 1 : voxelPos.y),
                     (int)(dp.z < 0.5f ? voxelPos.z - 1 : voxelPos.z)};
  const int bsz = (int)h->brick_size;
  for (int i = 0; i < 8; i++) {
    const int vi[3] = {v0[0] + ((i & 4) >> 2), v0[1] + ((i & 2) >> 1), v0[2] + (i & 1)};
    int bp[3];
    for (int a = 0; a < 3; a++) bp[a] = vi[a] >= 0 ? (vi[a] < bsz ? 0 : 1) : -1;
    const uint32_t nb = (uint32_t)(9 * (bp[0] + 1) + 3 * (bp[1] + 1) + (bp[2] + 1));
    const f3 dvox = sub3(mk3((float)vi[0], (float)vi[1], (float)vi[2]), voxelPos);
    uint32_t nid;
    f3 nvp;
    if (nb == 9 + 3 + 1) {
      nid = node_id;
      nvp = mk3((float)vi[0], (float)vi[1], (float)vi[2]);
    } else {
      const uint32_t v_off = s->sbs_nodes[node_id].data_offset;
      nid = s->sbs_values[v_off + v_size * v_size * v_size + 8 + nb];
      const float b = (float)h->brick_size;
      nvp = sub3(mk3((float)vi[0], (float)vi[1], (float)vi[2]), mk3(b * (float)bp[0], b * (float)bp[1], b * (float)bp[2]));
    }
    if (nid != 0x80000000u) {
      load_distance_values(s, nid, nvp, v_size, sz_inv, values_n);
      normals[i] = normalize3(tri_diff(values_n, sub3(dp, dvox)));
    }
  }
  const float w[8] = {(1 - nmq.x) * (1 - nmq.y) * (1 - nmq.z), (1 - nmq.x) * (1 - nmq.y) * (nmq.z),
                      (1 - nmq.x) * (nmq.y) * (1 - nmq.z),     (1 - nmq.x) * (nmq.y) * (nmq.z),
                      (nmq.x) * (1 - nmq.y) * (1 - nmq.z),     (nmq.x) * (1 - nmq.y) * (nmq.z),
                      (nmq.x) * (nmq.y) * (1 - nmq.z),         (nmq.x) * (nmq.y) * (nmq.z)};
  f3 sm = scl3(w[0], normals[0]);
  for (int i = 1; i < 8; i++) sm = add3(sm, scl3(w[i], normals[i]));
  const f2 en = encode_normal(normalize3(sm));
  hit->coords[2] = en.x;
  hit->coords[3] = en.y;
}

/* OctreeBrickIntersect, BVH/BVH2Common.cpp:764-984 (trilinear; COL-layout colour) */
static void brick_intersect(const orc_scene *s, uint32_t type, f3 ray_pos, f3 ray_dir, float tNear,
                            uint32_t geom_id, uint32_t bvh_node_id, orc_hit *hit, orc_counters *cnt) {
  const orc_sbs_header *h = &s->sbs_hdr;
  float values[8];
  uint32_t prim_id = bvh_node_id;
  uint32_t node_id = prim_id;                        /* + m_SdfSBSRoots[sdfId] (single SBS) */
  uint32_t v_size = h->brick_size + 2 * h->brick_pad + 1;
  const orc_sbs_node *nd = &s->sbs_nodes[node_id];
  float px = (float)(nd->pos_xy >> 16), py = (float)(nd->pos_xy & 0x0000FFFF);
  float pz = (float)(nd->pos_z_lod_size >> 16), sz = (float)(nd->pos_z_lod_size & 0x0000FFFF);
  float sz_inv = 2.0f / sz;
  float bs = (float)h->brick_size;
  float d = 2.0f / (sz * bs);
  f3 brick_min = add3(mk3(-1, -1, -1), scl3(sz_inv, mk3(px, py, pz)));
  f3 brick_max = add3(brick_min, scl3(sz_inv, mk3(1, 1, 1)));
  f3 inv = safe_inverse(ray_dir);
  f2 bnf = ray_box2(ray_pos, inv, brick_min, brick_max);
  float old_t = hit->t;
  const float scale = 0.5f * sz * bs;
  if (cnt) cnt->n_leaf++;
  /* the reference loop is unbounded: a ray crosses at most 3*brick_size voxels,
   * but a grazing ray whose position rounds back into the voxel it left advances
   * by only +1e-6 a step (at least 7.6e-7 once rounded, for t < 32; nothing
   * beyond).  8*brick_size+16 steps plus 1.5e6 per unit of segment length cover
   * every walk the reference finishes (orc_walk_step_bound, the engine's bound) */
  const uint32_t max_steps = orc_walk_step_bound(h->brick_size, bnf.y - bnf.x);
  for (uint32_t step = 0; bnf.x < bnf.y && hit->t == old_t && step < max_steps; step++) {
    f3 hit_pos = add3(ray_pos, scl3(bnf.x, ray_dir));
    f3 local_pos = mul3s(sub3(hit_pos, brick_min), scale);
    f3 voxelPos = mk3(floorf(clampf_(local_pos.x, 1e-6f, bs - 1e-6f)),
                      floorf(clampf_(local_pos.y, 1e-6f, bs - 1e-6f)),
                      floorf(clampf_(local_pos.z, 1e-6f, bs - 1e-6f)));
    f3 min_pos = add3(brick_min, scl3(d, voxelPos));
    f3 max_pos = add3(min_pos, scl3(d, mk3(1, 1, 1)));
    float vmin = load_distance_values(s, node_id, voxelPos, v_size, sz_inv, values);
    if (cnt) cnt->n_vox++;
    f2 fnf = ray_box2(ray_pos, inv, min_pos, max_pos);
    if (tNear < fnf.x && vmin <= 0.0f) {
      f3 start_pos = add3(ray_pos, scl3(fnf.x, ray_dir));
      f3 start_q = mul3s(sub3(start_pos, min_pos), scale);
      float qFar = (fnf.y - fnf.x) * scale;
      local_surface_intersection(s, type, ray_dir, geom_id, values, prim_id, d, 0.0f, qFar, fnf, start_q, hit, cnt);
      if (h->aux_data == (5u << 24) && s->preset.normal_mode == 2 && need_normal(&s->preset) && hit->t != old_t)
        smooth_normal(s, node_id, voxelPos, start_q, fnf.x, d, ray_dir, v_size, sz_inv, hit);
    }
    bnf.x += fmaxf_(0.0f, fnf.y - bnf.x) + 1e-6f;
  }
  if (hit->t < old_t) {                                                  /* colour, :912-982 */
    const uint32_t layout = h->aux_data & 0xFF000000u;
    if (layout == (4u << 24) || layout == (5u << 24)) {
      f3 pos = add3(ray_pos, scl3(hit->t, ray_dir));
      f3 dp = mul3s(sub3(pos, brick_min), 0.5f * sz);
      uint32_t t_off = nd->data_offset + v_size * v_size * v_size;
      float w[8] = {(1 - dp.x) * (1 - dp.y) * (1 - dp.z), (1 - dp.x) * (1 - dp.y) * (dp.z),
                    (1 - dp.x) * (dp.y) * (1 - dp.z), (1 - dp.x) * (dp.y) * (dp.z),
                    (dp.x) * (1 - dp.y) * (1 - dp.z), (dp.x) * (1 - dp.y) * (dp.z),
                    (dp.x) * (dp.y) * (1 - dp.z), (dp.x) * (dp.y) * (dp.z)};
      f3 col = mk3(0, 0, 0);
      for (int i = 0; i < 8; i++) {
        const float *c = &s->sbs_values_f[s->sbs_values[t_off + i]];
        f3 ci = mk3(w[i] * c[0], w[i] * c[1], w[i] * c[2]);
        col = i == 0 ? ci : add3(col, ci);
      }
      col = mk3(clampf_(floorf(255.0f * col.x + 0.5f), 0.0f, 255.0f),
                clampf_(floorf(255.0f * col.y + 0.5f), 0.0f, 255.0f),
                clampf_(floorf(255.0f * col.z + 0.5f), 0.0f, 255.0f));
      hit->coords[0] = col.x + col.y / 256.0f;
      hit->coords[1] = col.z;
    } else if (layout == (2u << 24) || layout == (3u << 24)) {   /* DX_UV16 / DX_RGB8: 8 words after the distances */
      f3 pos = add3(ray_pos, scl3(hit->t, ray_dir));
      f3 dp = mul3s(sub3(pos, brick_min), 0.5f * sz);
      const uint32_t vpi = 4 / h->bytes_per_value;
      const uint32_t *tw = s->sbs_values + nd->data_offset + (v_size * v_size * v_size + vpi - 1) / vpi;
      float w[8] = {(1 - dp.x) * (1 - dp.y) * (1 - dp.z), (1 - dp.x) * (1 - dp.y) * (dp.z),
                    (1 - dp.x) * (dp.y) * (1 - dp.z), (1 - dp.x) * (dp.y) * (dp.z),
                    (dp.x) * (1 - dp.y) * (1 - dp.z), (dp.x) * (1 - dp.y) * (dp.z),
                    (dp.x) * (dp.y) * (1 - dp.z), (dp.x) * (dp.y) * (dp.z)};
      if (layout == (2u << 24)) {   /* texture coordinates, 16 bits each */
        float u = 0, v = 0;
        for (int i = 0; i < 8; i++) {
          const float ui = w[i] * (1.5259022e-5f * (float)(tw[i] >> 16));
          const float vi = w[i] * (1.5259022e-5f * (float)(tw[i] & 0xFFFF));
          u = i == 0 ? ui : u + ui;
          v = i == 0 ? vi : v + vi;
        }
        hit->coords[0] = u;
        hit->coords[1] = v;
      } else {                      /* RGB8 colours */
        f3 col = mk3(0, 0, 0);
        for (int i = 0; i < 8; i++) {
          f3 ci = mk3(w[i] * (float)((tw[i] >> 0) & 0xFF), w[i] * (float)((tw[i] >> 8) & 0xFF),
                      w[i] * (float)((tw[i] >> 16) & 0xFF));
          col = i == 0 ? ci : add3(col, ci);
        }
        col = mk3(clampf_(floorf(col.x + 0.5f), 0.0f, 255.0f), clampf_(floorf(col.y + 0.5f), 0.0f, 255.0f),
                  clampf_(floorf(col.z + 0.5f), 0.0f, 255.0f));
        hit->coords[0] = col.x + col.y / 256.0f;
        hit->coords[1] = col.z;
      }
    }
  }
}

/* OctreeNodeIntersect (SVS branch), BVH/BVH2Common.cpp:633-655 with
 * RayNodeIntersection :126-153 */
static void svs_node_intersect(const orc_scene *s, f3 ray_pos, f3 ray_dir, float tNear,
                               uint32_t geom_id, uint32_t bvh_node_id, orc_hit *hit, orc_counters *cnt) {
  float values[8];
  uint32_t prim_id = bvh_node_id, node_id = prim_id;
  const orc_svs_node *nd = &s->svs_nodes[node_id];
  float px = (float)(nd->pos_xy >> 16), py = (float)(nd->pos_xy & 0x0000FFFF);
  float pz = (float)(nd->pos_z_lod_size >> 16), sz = (float)(nd->pos_z_lod_size & 0x0000FFFF);
  float d_max = 2 * 1.73205081f / sz;
  f3 min_pos = add3(mk3(-1, -1, -1), mk3(2.0f * px / sz, 2.0f * py / sz, 2.0f * pz / sz));
  f3 max_pos = add3(min_pos, mk3(2.0f * 1 / sz, 2.0f * 1 / sz, 2.0f * 1 / sz));
  f3 size = sub3(max_pos, min_pos);
  for (int i = 0; i < 8; i++) {
    /* -d_max + 2*d_max*(1.0/255.0f)*q : the double literal promotes the product to double */
    double q = (double)((nd->values[i / 4] >> (8 * (i % 4))) & 0xFF);
    values[i] = (float)(-d_max + 2 * d_max * (1.0 / 255.0f) * q);
  }
  f2 fnf = ray_box2(ray_pos, safe_inverse(ray_dir), min_pos, max_pos);
  f3 start_pos = add3(ray_pos, scl3(fnf.x, ray_dir));
  float d = fmaxf_(size.x, fmaxf_(size.y, size.z));
  f3 start_q = mk3((start_pos.x - min_pos.x) / d, (start_pos.y - min_pos.y) / d, (start_pos.z - min_pos.z) / d);
  float qFar = (fnf.y - fnf.x) / d;
  float qNear = tNear > fnf.x ? (tNear - fnf.x) / d : 0.0f;
  if (cnt) { cnt->n_leaf++; cnt->n_vox++; }
  if (qNear > 0.0f) return;
  local_surface_intersection(s, ORC_TYPE_SDF_SVS, ray_dir, geom_id, values, prim_id, d, qNear, qFar, fnf, start_q, hit, cnt);
}

/* IntersectAllTrianglesInLeaf, BVH/BVH2Common.cpp:2776-2840 (geometry normal) */
static void triangles_in_leaf(const orc_scene *s, f3 ray_pos, f3 ray_dir, float tNear, uint32_t geom_id,
                              uint32_t a_start, uint32_t a_count, orc_hit *hit, orc_counters *cnt) {
  for (uint32_t tri = a_start; tri < a_start + a_count; tri++) {
    const uint32_t A = s->tri_indices[tri * 3 + 0], B = s->tri_indices[tri * 3 + 1], C = s->tri_indices[tri * 3 + 2];
    const float *pa = s->vert_pos4 + 4 * A, *pb = s->vert_pos4 + 4 * B, *pc = s->vert_pos4 + 4 * C;
    const f3 A_pos = mk3(pa[0], pa[1], pa[2]), B_pos = mk3(pb[0], pb[1], pb[2]), C_pos = mk3(pc[0], pc[1], pc[2]);
    const f3 edge1 = sub3(B_pos, A_pos), edge2 = sub3(C_pos, A_pos);
    const f3 pvec = cross3(ray_dir, edge2);
    const f3 tvec = sub3(ray_pos, A_pos);
    const f3 qvec = cross3(tvec, edge1);
    const float invDet = 1.0f / dot3(edge1, pvec);
    const float v = dot3(tvec, pvec) * invDet;
    const float u = dot3(qvec, ray_dir) * invDet;
    const float t = dot3(edge2, qvec) * invDet;
    if (cnt) cnt->n_tri++;
    if (v >= -1e-6f && u >= -1e-6f && (u + v <= 1.0f + 1e-6f) && t > tNear && t < hit->t) {
      hit->t = t;
      hit->prim_id = tri;
      hit->inst_id = 0;
      hit->geom_id = geom_id | (ORC_TYPE_MESH_TRIANGLE << 24);
      hit->coords[0] = u;
      hit->coords[1] = v;
      if (need_normal(&s->preset)) {
        f3 n = cross3(edge1, edge2);
        n = normalize3(matmul4x3(s->inst_inv_t, n));
        f2 en = encode_normal(n);
        hit->coords[2] = en.x; hit->coords[3] = en.y;
      } else {
        hit->coords[2] = 0; hit->coords[3] = 0;
      }
    }
  }
}

/* GeomData*::Intersect dispatch, BVH/BVH2Common.h:525-618; returns nonzero tag on hit. */
static uint32_t leaf_intersect(const orc_scene *s, f3 ray_pos, f3 ray_dir, float tNear,
                               uint32_t aabb_id, orc_hit *hit, orc_counters *cnt) {
  const float tPrev = hit->t;
  const uint32_t geom_id = 0;
  if (s->type == ORC_TYPE_MESH_TRIANGLE) {
    uint32_t sc = s->leaf_start_count[aabb_id];
    triangles_in_leaf(s, ray_pos, ray_dir, tNear, geom_id, extract_start(sc), extract_count(sc), hit, cnt);
    return hit->t >= tPrev ? 0 : 1;   /* TAG_TRIANGLE */
  } else if (s->type == ORC_TYPE_SDF_SVS) {
    svs_node_intersect(s, ray_pos, ray_dir, tNear, geom_id, extract_start(aabb_id), hit, cnt);
    return hit->t >= tPrev ? 0 : 3;   /* TAG_SDF_NODE */
  } else {
    brick_intersect(s, s->type, ray_pos, ray_dir, tNear, geom_id, extract_start(aabb_id), hit, cnt);
    return hit->t >= tPrev ? 0 : 4;   /* TAG_SDF_BRICK */
  }
}

/* BVH2TraverseF32, BVH/BVH2Common.cpp:3407-3488.  closest_hit=0 keeps the
 * reference's early-out after the first SDF hit (:3402-3405, :3478). */
static void bvh2_traverse(const orc_scene *s, f3 ray_pos, f3 ray_dir, float tNear, int stopOnFirstHit,
                          orc_hit *hit, orc_counters *cnt) {
  uint32_t stack[80];
  int top = 0;
  uint32_t leftNodeOffset = 0;
  int hitFound = 0;
  const f3 inv = safe_inverse(ray_dir);
  while (top >= 0 && !hitFound) {
    while (top >= 0 && ((leftNodeOffset & LEAF_BIT) == 0)) {
      const orc_bvh_pair *fat = &s->pairs[leftNodeOffset];
      if (cnt) cnt->n_fat++;
      const uint32_t n0 = fat->l.left_offset, n1 = fat->r.left_offset;
      const f2 tm0 = ray_box2(ray_pos, inv, mk3(fat->l.bmin[0], fat->l.bmin[1], fat->l.bmin[2]),
                              mk3(fat->l.bmax[0], fat->l.bmax[1], fat->l.bmax[2]));
      const f2 tm1 = ray_box2(ray_pos, inv, mk3(fat->r.bmin[0], fat->r.bmin[1], fat->r.bmin[2]),
                              mk3(fat->r.bmax[0], fat->r.bmax[1], fat->r.bmax[2]));
      const int hit0 = (tm0.x <= tm0.y) && (tm0.y >= tNear) && (tm0.x <= hit->t);
      const int hit1 = (tm1.x <= tm1.y) && (tm1.y >= tNear) && (tm1.x <= hit->t);
      leftNodeOffset = hit0 ? n0 : n1;
      if (hit0 && hit1) {
        leftNodeOffset = (tm0.x <= tm1.x) ? n0 : n1;
        stack[top] = (tm0.x <= tm1.x) ? n1 : n0;
        top++;
      }
      if (!hit0 && !hit1) {
        top--;
        leftNodeOffset = stack[top > 0 ? top : 0];
      }
    }
    if (top >= 0 && leftNodeOffset != 0xFFFFFFFFu) {
      /* the SDF bias is passed to every leaf type (:3472-3476) */
      const float tNearSdf = fmaxf_(tNear, 0.1f);
      uint32_t tag = leaf_intersect(s, ray_pos, ray_dir, tNearSdf, extract_start(leftNodeOffset), hit, cnt);
      hitFound = (tag != 0) && ((tag != 1 && !s->closest_hit) || stopOnFirstHit);
    }
    top--;
    leftNodeOffset = stack[top > 0 ? top : 0];
  }
}

/* RayQuery_NearestHit, BVH/BVH2Common.cpp:3490-3559 (single instance: the TLAS is
 * one leaf node, BVH/BVH2Common_host.cpp:1430-1437). */
orc_hit orc_ray_query_nearest(const orc_scene *s, const float pos_near[4], const float dir_far[4],
                              orc_counters *cnt) {
  float far_ = dir_far[3];
  int stopOnFirstHit = (far_ <= 0.0f);
  if (stopOnFirstHit) far_ *= -1.0f;
  orc_hit hit;
  hit.t = far_;
  hit.prim_id = 0xFFFFFFFFu; hit.inst_id = 0xFFFFFFFFu; hit.geom_id = 0xFFFFFFFFu;
  hit.coords[0] = 1.0f; hit.coords[1] = 0.0f; hit.coords[2] = 0.0f; hit.coords[3] = 0.0f;
  const f3 p = mk3(pos_near[0], pos_near[1], pos_near[2]);
  const f3 dd = mk3(dir_far[0], dir_far[1], dir_far[2]);
  /* TLAS: a single leaf node holding the instance box (:3508-3529) */
  {
    const f3 inv = safe_inverse(dd);
    const f2 bh = ray_box2(p, inv, mk3(s->inst_bmin[0], s->inst_bmin[1], s->inst_bmin[2]),
                           mk3(s->inst_bmax[0], s->inst_bmax[1], s->inst_bmax[2]));
    const int intersects = (bh.x <= bh.y) && (bh.y > pos_near[3]) && (bh.x < hit.t);
    if (!intersects) return hit;
  }
  const f3 ray_pos = matmul4x3(s->inst_inv, p);
  const f3 ray_dir = matmul3x3(s->inst_inv, dd);
  bvh2_traverse(s, ray_pos, ray_dir, pos_near[3], stopOnFirstHit, &hit, cnt);
  if (hit.geom_id != 0xFFFFFFFFu && (hit.geom_id >> 24) == ORC_TYPE_MESH_TRIANGLE)
    hit.prim_id = s->prim_indices[hit.prim_id];                    /* :3550-3556 */
  return hit;
}

/* ---------------- Renderer ---------------- */
static void mat_vec4(const float m[16], const float v[4], float r[4]) {
  for (int i = 0; i < 4; i++) r[i] = m[i * 4 + 0] * v[0] + m[i * 4 + 1] * v[1] + m[i * 4 + 2] * v[2] + m[i * 4 + 3] * v[3];
}

void orc_eye_ray(uint32_t x, uint32_t y, uint32_t w, uint32_t h, float dx, float dy,
                 const float proj_inv[16], const float wv_inv[16], float pos_near[4], float dir_far[4]) {
  /* EyeRayDirNormalized, render_common.h:25-31 */
  float fx = ((float)x + dx) / (float)w, fy = ((float)y + dy) / (float)h;
  float v[4] = {2.0f * fx - 1.0f, -2.0f * fy + 1.0f, 1.0f, 1.0f}, r[4];
  mat_vec4(proj_inv, v, r);
  const float ww = r[3];
  f3 dir = normalize3(mk3(r[0] / ww, r[1] / ww, r[2] / ww));
  /* transform_ray3f, render_common.h:45-55 */
  f3 pos = mk3(0, 0, 0);
  f3 p0 = matmul4x3(wv_inv, pos);
  f3 p2 = matmul4x3(wv_inv, add3(pos, scl3(100.0f, dir)));
  f3 diff = sub3(p2, p0);
  dir = normalize3(diff);
  pos_near[0] = p0.x; pos_near[1] = p0.y; pos_near[2] = p0.z; pos_near[3] = 0.0f;
  dir_far[0] = dir.x; dir_far[1] = dir.y; dir_far[2] = dir.z; dir_far[3] = 1e9f;
}

/* decode_normal, Renderer/eye_ray.cpp:22-33 */
static f3 decode_normal(float ex, float ey) {
  f3 v = mk3(ex, ey, 1.0f - fabsf(ex) - fabsf(ey));
  if (v.z < 0) {
    float vx = v.x;
    v.x = (1.0f - fabsf(v.y)) * ((v.x >= 0.0) ? +1.0f : -1.0f);
    v.y = (1.0f - fabsf(vx)) * ((v.y >= 0.0) ? +1.0f : -1.0f);
  }
  return normalize3(v);
}

/* MultiRenderer::m_palette (Renderer/eye_ray.h:235-241) and decode_RGBA8
 * (Renderer/eye_ray.cpp:15-19) */
static const uint32_t orc_palette[20] = {0xffe6194bu, 0xff3cb44bu, 0xffffe119u, 0xff0082c8u, 0xfff58231u,
                                         0xff911eb4u, 0xff46f0f0u, 0xfff032e6u, 0xffd2f53cu, 0xfffabebeu,
                                         0xff008080u, 0xffe6beffu, 0xffaa6e28u, 0xfffffac8u, 0xff800000u,
                                         0xffaaffc3u, 0xff808000u, 0xffffd8b1u, 0xff000080u, 0xff808080u};
static void decode_rgba8(uint32_t c, float out[4]) {
  out[0] = (float)(c & 0xFF) * (1.0f / 255.0f);
  out[1] = (float)((c >> 8) & 0xFF) * (1.0f / 255.0f);
  out[2] = (float)((c >> 16) & 0xFF) * (1.0f / 255.0f);
  out[3] = (float)((c >> 24) & 0xFF) * (1.0f / 255.0f);
}

void orc_shade(const orc_scene *s, const orc_hit *hit, const float pos_near[4], const float dir_far[4], float out[4]) {
  /* kernel_RayTrace, Renderer/eye_ray.cpp:162-489 */
  if (hit->prim_id == 0xFFFFFFFFu) { out[0] = 0; out[1] = 0; out[2] = 0; out[3] = 1; return; }
  float z = hit->t, z_near = 0.1f, z_far = 10;
  uint32_t type = hit->geom_id >> 24;
  f3 norm;
  if (type == ORC_TYPE_MESH_TRIANGLE) {
    /* geometry normal from the original triangle (Renderer/eye_ray.cpp:187-207) */
    const uint32_t *ix = s->tri_indices_orig + 3 * hit->prim_id;
    const float *pa = s->vert_pos4 + 4 * ix[0], *pb = s->vert_pos4 + 4 * ix[1], *pc = s->vert_pos4 + 4 * ix[2];
    const f3 e1 = mk3(pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]);
    const f3 e2 = mk3(pc[0] - pa[0], pc[1] - pa[1], pc[2] - pa[2]);
    norm = normalize3(matmul4x3(s->inst_inv_t, cross3(e1, e2)));
  } else {
    norm = decode_normal(hit->coords[2], hit->coords[3]);
  }
  f3 rd = mk3(dir_far[0], dir_far[1], dir_far[2]);
  float ns = signf_(dot3(scl3(-1.0f, rd), norm));
  norm = scl3(ns, norm);   /* norm * norm_sign */
  switch (s->preset.render_mode) {
    case 0: out[0] = out[1] = out[2] = out[3] = 1; break;                               /* MASK */
    case 2: { float d = (1 / z - 1 / z_near) / (1 / z_far - 1 / z_near); out[0] = out[1] = out[2] = d; out[3] = 1; } break;
    case 3: { float d = ((z - z_near) / (z_far - z_near)); out[0] = out[1] = out[2] = d; out[3] = 1; } break;
    case 4: { float d = 1 - ((z - z_near) / (z_far - z_near)); out[0] = out[1] = out[2] = d; out[3] = 1; } break;
    case 8: out[0] = fabsf(norm.x); out[1] = fabsf(norm.y); out[2] = fabsf(norm.z); out[3] = 1; break;
    case 1: case 17: {
      /* LAMBERT_NO_TEX: white; LAMBERT: the brick colour, else the default textured
       * material's constant texel (0, 1, 1) (Renderer/eye_ray_host.cpp:30-33) */
      f3 color = s->preset.render_mode == 17 ? mk3(0, 1, 1) : mk3(1, 1, 1);
      if (s->preset.render_mode == 17 && type == ORC_TYPE_SDF_SBS_COL) {
        color.x = roundf(hit->coords[0]) / 255.0f;
        color.y = hit->coords[0] - floorf(hit->coords[0]);
        color.z = roundf(hit->coords[1]) / 255.0f;
      }
      /* default lights, Renderer/eye_ray_host.cpp:40 */
      const f3 ldir = normalize3(mk3(1, 1, 1));
      const float lc = 2.0f / 3.0f;
      f3 fc = mk3(0, 0, 0);
      float q = fmaxf_(0.0f, dot3(norm, ldir));
      fc = add3(fc, scl3(q, mul3(mk3(lc, lc, lc), color)));
      fc = add3(fc, mul3(mk3(0.25f, 0.25f, 0.25f), color));
      out[0] = fc.x; out[1] = fc.y; out[2] = fc.z; out[3] = 1;
    } break;
    case 5: decode_rgba8(orc_palette[hit->prim_id % 20u], out); break;               /* PRIMITIVE */
    case 6: decode_rgba8(orc_palette[type % 20u], out); break;                        /* TYPE */
    case 7: decode_rgba8(orc_palette[(hit->geom_id & 0x00FFFFFFu) % 20u], out); break; /* GEOM */
    case 9:                                                                           /* BARYCENTRIC */
      out[0] = hit->coords[0]; out[1] = hit->coords[1]; out[2] = 1 - hit->coords[0] - hit->coords[1]; out[3] = 1;
      break;
    case 10: {                                                                        /* ST_ITERATIONS */
      const uint32_t it = hit->prim_id;
      if (it == 0) { out[0] = out[1] = out[2] = 0.5f; out[3] = 1; }
      else if (it <= 64) {
        float q = (float)it / 64; q = q < 0.0f ? 0.0f : (q > 1.0f ? 1.0f : q);
        const float r = 1 - q;
        out[0] = q * 0.0f + r * 0.0f; out[1] = q * 0.0f + r * 1.0f; out[2] = q * 1.0f + r * 0.0f; out[3] = q * 1.0f + r * 1.0f;
      } else {
        float q = (float)(it - 64) / (256 - 64); q = q < 0.0f ? 0.0f : (q > 1.0f ? 1.0f : q);
        const float r = 1 - q;
        out[0] = q * 1.0f + r * 0.0f; out[1] = q * 0.0f + r * 0.0f; out[2] = q * 0.0f + r * 1.0f; out[3] = q * 1.0f + r * 1.0f;
      }
    } break;
    case 16: {                                                                        /* DIFFUSE */
      f3 color = mk3(0, 1, 1);
      if (type == ORC_TYPE_SDF_SBS_COL) {
        color.x = roundf(hit->coords[0]) / 255.0f;
        color.y = hit->coords[0] - floorf(hit->coords[0]);
        color.z = roundf(hit->coords[1]) / 255.0f;
      }
      out[0] = color.x; out[1] = color.y; out[2] = color.z; out[3] = 1;
    } break;
    case 12: case 18: {                                                               /* PHONG(_NO_TEX) */
      /* Renderer/eye_ray.cpp:420-483 with the default lights: the direct light adds an
       * unshadowed Lambert term and a shadowed Phong term; the shadow ray is a nearest-hit
       * query from just before the hit point towards the light */
      const float Kd = 0.25f, Ks = 0.25f, BIAS = 1e-6f;
      f3 color = s->preset.render_mode == 12 ? mk3(1, 1, 1) : mk3(0, 1, 1);
      if (s->preset.render_mode == 18 && type == ORC_TYPE_SDF_SBS_COL) {
        color.x = roundf(hit->coords[0]) / 255.0f;
        color.y = hit->coords[0] - floorf(hit->coords[0]);
        color.z = roundf(hit->coords[1]) / 255.0f;
      }
      f3 fc = mk3(0, 0, 0);
      {
        const f3 ld = normalize3(mk3(1, 1, 1));
        const float l = 2.0f / 3.0f;
        const f3 lc = mk3(l, l, l);
        const f3 surf = add3(mk3(pos_near[0], pos_near[1], pos_near[2]), scl3(hit->t - BIAS, rd));
        const float q = fmaxf_(0.0f, dot3(norm, ld));
        fc = add3(fc, scl3(q, mul3(lc, color)));
        const float sp[4] = {surf.x, surf.y, surf.z, pos_near[3]}, sd[4] = {ld.x, ld.y, ld.z, dir_far[3]};
        orc_counters cc;
        memset(&cc, 0, sizeof(cc));
        const orc_hit sh = orc_ray_query_nearest(s, sp, sd, &cc);
        const float shade = (sh.prim_id == 0xFFFFFFFFu) ? 1.0f : 0.0f;
        const f3 refl = add3(scl3(-1.0f, ld), scl3(2.0f * dot3(norm, ld), norm));
        const float inner = Kd * fmaxf_(0.0f, dot3(norm, ld)) + Ks * powf(fmaxf_(0.0f, dot3(norm, refl)), 32.0f);
        fc = add3(fc, mul3(scl3(inner, scl3(shade, lc)), color));
      }
      fc = add3(fc, mul3(mk3(0.25f, 0.25f, 0.25f), color));   /* ambient */
      out[0] = fc.x; out[1] = fc.y; out[2] = fc.z; out[3] = 1;
    } break;
    case 19: {                                                                        /* HSV_DEPTH */
      const float iz = pos_near[2] + z * dir_far[2];
      float zt = (iz + 1.f) * 2.f;
      zt = zt - (float)(int)zt;
      if (zt < 0.f) zt = 1.f + zt;
      float c[4] = {1.0f, 1.0f, 1.0f, 1.0f};
      const float vmin = (1.f - 1.f) * 1.0f;
      float hi;
      const float a = (1.0f - vmin) * modff(zt * 6.f, &hi);
      uint32_t h = (uint32_t)hi;
      h = h <= 5u ? h : 5u;
      c[(2u + (h >> 1)) % 3u] = vmin;
      if ((h & 1u) != 0u) c[h >> 1] = 1.0f - a;
      else c[(1u + (h >> 1)) % 3u] = vmin + a;
      out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = 1.f;
    } break;
    default: out[0] = 1; out[1] = 0; out[2] = 1; out[3] = 1; break;
  }
}

/* rand3 / rand2, Renderer/eye_ray.cpp:53-80 */
void orc_rand2(uint32_t x, uint32_t y, uint32_t iter, uint32_t seed, float *rx, float *ry) {
  x = x + 1233u * (iter + seed) % 171u;
  y = y + 453u * (iter + seed) % 765u;
  uint32_t v0 = x, v1 = y, v2 = x ^ y;
  v0 = v0 * 1664525u + 1013904223u; v1 = v1 * 1664525u + 1013904223u; v2 = v2 * 1664525u + 1013904223u;
  v0 += v1 * v2; v1 += v2 * v0; v2 += v0 * v1;
  v0 ^= v0 >> 16u; v1 ^= v1 >> 16u; v2 ^= v2 >> 16u;
  v0 += v1 * v2; v1 += v2 * v0; v2 += v0 * v1;
  const float k = 1.0f / (float)0xffffffffu;
  *rx = (float)v0 * k;
  *ry = (float)v1 * k;
}

static orc_counters render_impl(const orc_scene *s, uint32_t w, uint32_t h, const float proj_inv[16],
                                const float wv_inv[16], const uint32_t *pix, uint32_t n_pix,
                                orc_hit *hits, float *rgba, int threads) {
  orc_counters tot; memset(&tot, 0, sizeof(tot));
  const long n = pix ? (long)n_pix : (long)w * (long)h;
  const uint32_t spp = s->preset.spp ? s->preset.spp : 1;
  const uint32_t spp_sqrt = (uint32_t)sqrt((double)spp);
  const float i_spp_sqrt = 1.0f / (float)spp_sqrt;
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#else
  (void)threads;
#endif
  uint64_t a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) reduction(+ : a0, a1, a2, a3, a4, a5)
  for (long i = 0; i < n; i++) {
    uint32_t pidx = pix ? pix[i] : (uint32_t)i;
    uint32_t x = pidx % w, y = pidx / w;
    orc_counters c; memset(&c, 0, sizeof(c));
    float acc[4] = {0, 0, 0, 0};
    orc_hit first;
    for (uint32_t sidx = 0; sidx < spp; sidx++) {
      /* CastRaySingle's sub-pixel offset, Renderer/eye_ray.cpp:100-107 */
      float dx = i_spp_sqrt * (float)(sidx / spp_sqrt + 0.5), dy = i_spp_sqrt * (float)(sidx % spp_sqrt + 0.5);
      if (s->preset.ray_gen_mode == 1) orc_rand2(x, y, sidx + s->seed % 2u, s->seed, &dx, &dy);
      float pn[4], df[4], col[4];
      orc_eye_ray(x, y, w, h, dx, dy, proj_inv, wv_inv, pn, df);
      orc_hit hh = orc_ray_query_nearest(s, pn, df, &c);
      if (sidx == 0) first = hh;
      if (rgba) { orc_shade(s, &hh, pn, df, col); for (int k = 0; k < 4; k++) acc[k] += col[k]; }
    }
    if (hits) hits[i] = first;
    if (rgba) for (int k = 0; k < 4; k++) rgba[4 * i + k] = acc[k] / (float)spp;
    a0 += c.n_fat; a1 += c.n_leaf; a2 += c.n_vox; a3 += c.n_vox_loaded; a4 += c.n_finder; a5 += c.n_tri;
  }
  tot.n_fat = a0; tot.n_leaf = a1; tot.n_vox = a2; tot.n_vox_loaded = a3; tot.n_finder = a4; tot.n_tri = a5;
  return tot;
}

orc_counters orc_render(const orc_scene *s, uint32_t w, uint32_t h, const float proj_inv[16],
                        const float wv_inv[16], orc_hit *hits, float *rgba, int threads) {
  return render_impl(s, w, h, proj_inv, wv_inv, NULL, 0, hits, rgba, threads);
}

orc_counters orc_render_pixels(const orc_scene *s, uint32_t w, uint32_t h, const float proj_inv[16],
                               const float wv_inv[16], const uint32_t *pix, uint32_t n_pix,
                               orc_hit *hits, int threads) {
  return render_impl(s, w, h, proj_inv, wv_inv, pix, n_pix, hits, NULL, threads);
}

void orc_eye_rays(uint32_t w, uint32_t h, const float proj_inv[16], const float wv_inv[16], const uint32_t *pix,
                  uint32_t n, float dx, float dy, float *pos_near, float *dir_far) {
  for (uint32_t i = 0; i < n; i++)
    orc_eye_ray(pix[i] % w, pix[i] / w, w, h, dx, dy, proj_inv, wv_inv, pos_near + 4 * i, dir_far + 4 * i);
}

void orc_query_rays(const orc_scene *s, const float *pos_near, const float *dir_far, uint32_t n, orc_hit *out,
                    int threads) {
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#else
  (void)threads;
#endif
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
  for (long i = 0; i < (long)n; i++) out[i] = orc_ray_query_nearest(s, pos_near + 4 * i, dir_far + 4 * i, NULL);
}

void orc_free(void *p) { free(p); }
