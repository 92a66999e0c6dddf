/*
 * CPU oracle for the differentiable SDF render — TEST INFRASTRUCTURE ONLY
 * (see lrt_oracle_dr.h).  Compiled with -ffp-contract=off.
 */
#include "lrt_oracle_dr.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* float instantiation: the oracle proper */
#define R float
#define SFX(n) n##_f
#define RSQRT(x) sqrtf(x)
#define RABS(x) fabsf(x)
#define RFLOOR(x) floorf(x)
#define NEWTON_EPS 1e-7f
#define NEWTON_ITERS 10
#include "lrt_oracle_dr_core.h"
#undef R
#undef SFX
#undef RSQRT
#undef RABS
#undef RFLOOR
#undef NEWTON_EPS
#undef NEWTON_ITERS

/* double instantiation: forward only, for central finite differences */
#define R double
#define SFX(n) n##_d
#define RSQRT(x) sqrt(x)
#define RABS(x) fabs(x)
#define RFLOOR(x) floor(x)
#define NEWTON_EPS 1e-13
#define NEWTON_ITERS 60
#include "lrt_oracle_dr_core.h"
#undef R
#undef SFX
#undef RSQRT
#undef RABS
#undef RFLOOR
#undef NEWTON_EPS
#undef NEWTON_ITERS

typedef v3_f f3v;

static void put_hit(uint32_t *o, const hitdr_f *h) {
  memcpy(o + 0, &h->t, 4);
  o[1] = h->primId; o[2] = h->instId; o[3] = h->geomId;
  memcpy(o + 4, &h->color.x, 4); memcpy(o + 5, &h->color.y, 4); memcpy(o + 6, &h->color.z, 4);
  memcpy(o + 7, &h->sdf, 4);
  memcpy(o + 8, &h->normal.x, 4); memcpy(o + 9, &h->normal.y, 4); memcpy(o + 10, &h->normal.z, 4);
  o[11] = h->check_vox_border;
}

void orc_dr_query(const orc_dr_scene *s, const float *params, uint32_t flags, const float *pos_near,
                  const float *dir_far, uint32_t n, uint32_t *out) {
  ctx_f cx = {s, params};
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < (int64_t)n; i++) {
    payload_f pl;
    hitdr_f h = query_f(&cx, flags, pos_near + 4 * i, dir_far + 4 * i, &pl);
    uint32_t *o = out + 576 * i;
    memset(o, 0, 576 * 4);
    put_hit(o, &h);
    put_hit(o + 14, &pl.missed_hit);
    for (int k = 0; k < 8; k++) {
      o[28 + k] = pl.missed_indices[k];
      memcpy(o + 36 + k, &pl.missed_dSDF_dtheta[k], 4);
      o[44 + 2 * k] = pl.dc_index[k];
      memcpy(o + 45 + 2 * k, &pl.dc_value[k], 4);
    }
    for (int k = 0; k < 64; k++) {
      uint32_t *q = o + 60 + 8 * k;
      memcpy(q + 0, &pl.dd_diffuse[k].x, 4); memcpy(q + 1, &pl.dd_diffuse[k].y, 4); memcpy(q + 2, &pl.dd_diffuse[k].z, 4);
      q[3] = pl.dd_index[k];
      memcpy(q + 4, &pl.dd_norm[k].x, 4); memcpy(q + 5, &pl.dd_norm[k].y, 4); memcpy(q + 6, &pl.dd_norm[k].z, 4);
      memcpy(q + 7, &pl.dd_dist[k], 4);
    }
  }
}

/* ---------------- pixel glue, diff_render/MultiRendererDR.cpp ---------------- */

/* rand3 / rand2, Renderer/eye_ray.cpp:53-80 (lrt_oracle.c) */
static void rand2(uint32_t x, uint32_t y, uint32_t iter, uint32_t seed, float *rx, float *ry) {
  orc_rand2(x, y, iter, seed, rx, ry);
}

static const float Z_NEAR = 0.1f, Z_FAR = 10.0f;   /* diff_render/MultiRendererDR.cpp:25-26 */
static inline float lin_depth(float z) { return (z - Z_NEAR) / (Z_FAR - Z_NEAR); }

/* ray flags of CastRayWithGrad (:1113-1140) */
static uint32_t pixel_flags(const orc_dr_preset *p) {
  if (p->input_type == 1) return ORC_DR_RAY_FLAG_DDIST_DPOS;
  uint32_t f = 0;
  if (p->reconstruction_flags & ORC_DR_RECON_COLOR) f |= ORC_DR_RAY_FLAG_DDIFFUSE_DCOLOR;
  if (p->reconstruction_flags & ORC_DR_RECON_GEOMETRY) {
    if (p->render_mode == ORC_DR_RENDER_DIFFUSE) f |= ORC_DR_RAY_FLAG_DDIFFUSE_DPOS;
    else if (p->render_mode == ORC_DR_RENDER_LAMBERT) f |= ORC_DR_RAY_FLAG_DDIFFUSE_DPOS | ORC_DR_RAY_FLAG_DNORM_DPOS;
    else if (p->render_mode == ORC_DR_RENDER_NORMAL) f |= ORC_DR_RAY_FLAG_DNORM_DPOS;
  }
  return f;
}

/* CalculateColorWithGrad (:902-979); dC_dD / dC_dN hold the caller's initial
 * identity / zero for the modes that leave them untouched. */
static f3v color_grad(const orc_dr_preset *p, const hitdr_f *h, m3_f *dC_dD, m3_f *dC_dN) {
  f3v c = mk_f(1, 0, 1);
  const f3v z = mk_f(0, 0, 0);
  switch (p->render_mode) {
    case ORC_DR_RENDER_DIFFUSE:
      c = h->color;
      *dC_dD = rows_f(mk_f(1, 0, 0), mk_f(0, 1, 0), mk_f(0, 0, 1));
      *dC_dN = rows_f(z, z, z);
      break;
    case ORC_DR_RENDER_LAMBERT:
      c = z;
      *dC_dD = rows_f(z, z, z);
      *dC_dN = rows_f(z, z, z);
      for (uint32_t i = 0; i < p->n_lights; i++) {
        const orc_dr_light *L = &p->lights[i];
        f3v lc = mk_f(L->color[0], L->color[1], L->color[2]);
        if (L->type == 0) {
          f3v sp = mk_f(L->dir[0], L->dir[1], L->dir[2]);
          float q = mx_f(0.0f, dot_f(h->normal, sp));
          c = add_f(c, muls_f(mul_f(lc, h->color), q));
          if (q > 0.0f) {
            m3_f a = rows_f(mk_f(lc.x * q, 0, 0), mk_f(0, lc.y * q, 0), mk_f(0, 0, lc.z * q));
            m3_f b = rows_f(scl_f(lc.x * h->color.x, sp), scl_f(lc.y * h->color.y, sp), scl_f(lc.z * h->color.z, sp));
            for (int r = 0; r < 3; r++) { dC_dD->row[r] = add_f(dC_dD->row[r], a.row[r]); dC_dN->row[r] = add_f(dC_dN->row[r], b.row[r]); }
          }
        } else {
          c = add_f(c, mul_f(lc, h->color));
          m3_f a = rows_f(mk_f(lc.x, 0, 0), mk_f(0, lc.y, 0), mk_f(0, 0, lc.z));
          for (int r = 0; r < 3; r++) dC_dD->row[r] = add_f(dC_dD->row[r], a.row[r]);
        }
      }
      break;
    case ORC_DR_RENDER_MASK:
      c = mk_f(1, 1, 1);
      *dC_dD = rows_f(z, z, z);
      *dC_dN = rows_f(z, z, z);
      break;
    case ORC_DR_RENDER_LINEAR_DEPTH: {
      float d = lin_depth(h->t);
      c = mk_f(d, d, d);
    } break;
    case ORC_DR_RENDER_NORMAL:
      c = h->normal;
      *dC_dD = rows_f(z, z, z);
      *dC_dN = rows_f(mk_f(1, 0, 0), mk_f(0, 1, 0), mk_f(0, 0, 1));
      break;
    default: break;
  }
  return c;
}

/* CalculateColor (:855-900) */
static f3v color_plain(const orc_dr_preset *p, const hitdr_f *h) {
  m3_f a, b;
  return color_grad(p, h, &a, &b);
}

/* Loss / LossGrad (:51-96), float4 as 4 floats */
static float loss4(uint32_t fn, const float c[4], const float r[4]) {
  if (fn == 0) {
    float d0 = c[0] - r[0], d1 = c[1] - r[1], d2 = c[2] - r[2], d3 = c[3] - r[3];
    return d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
  }
  return fabsf(c[0] - r[0]) + fabsf(c[1] - r[1]) + fabsf(c[2] - r[2]) + fabsf(c[3] - r[3]);
}
static void loss_grad4(uint32_t fn, const float c[4], const float r[4], float g[4]) {
  for (int i = 0; i < 4; i++) {
    float d = c[i] - r[i];
    g[i] = fn == 0 ? 2.0f * d : (d < 0 ? -1.0f : 1.0f);
  }
}

/* t_samples_to_threshold (:995-1061) */
static float t_threshold(const float *samples, unsigned count, float default_value, unsigned default_count) {
  enum { G = 10, GAP = 4 };
  float dmin = samples[0], dmax = samples[0];
  for (unsigned i = 1; i < count; i++) { dmin = mn_f(dmin, samples[i]); dmax = mx_f(dmax, samples[i]); }
  if (default_count > 0) { dmin = mn_f(dmin, default_value); dmax = mx_f(dmax, default_value); }
  float diff = mx_f(1e-9f, dmax - dmin);
  unsigned g[G] = {0};
  for (unsigned i = 0; i < count; i++) {
    float d = (samples[i] - dmin) / diff;
    float b = d * G;
    int bi = b >= (float)(G - 1) ? G - 1 : (b <= 0.0f ? 0 : (int)b);
    g[bi]++;
  }
  {
    float dd = (default_value - dmin) / diff;
    float b = dd * G;
    int bi = b >= (float)(G - 1) ? G - 1 : (b <= 0.0f ? 0 : (int)b);
    g[bi] += default_count;
  }
  int max_len = 0, max_start = -1, start = -1;
  for (int i = 1; i < G; i++) {
    if (start != -1) {
      if (g[i] != 0) {
        int len = i - start;
        if (len > max_len) { max_len = len; max_start = start; }
        start = -1;
      }
    } else if (g[i] == 0) {
      start = i;
    }
  }
  if (max_len > GAP) return dmin + diff * (max_start + 0.5f * max_len) / G;
  return 0.0f;
}

static void mat4_mul(const float *a, const float *b, float *r) {   /* LiteMath float4x4 product */
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++)
      r[i * 4 + j] = a[i * 4 + 0] * b[0 * 4 + j] + a[i * 4 + 1] * b[1 * 4 + j] + a[i * 4 + 2] * b[2 * 4 + j] +
                     a[i * 4 + 3] * b[3 * 4 + j];
}

/* TransformWorldToScreenSpace (:1296-1301) with m_proj * m_worldView precomputed */
static void w2s(const float pv[16], f3v p, float *sx, float *sy) {
  float r[4];
  for (int i = 0; i < 4; i++) r[i] = pv[i * 4] * p.x + pv[i * 4 + 1] * p.y + pv[i * 4 + 2] * p.z + pv[i * 4 + 3] * 1.0f;
  float w = r[3];
  *sx = 0.5f * (r[0] / w + 1.0f);
  *sy = 1.0f - 0.5f * (r[1] / w + 1.0f);
}

typedef struct {
  const orc_dr_scene *s; const float *P; const orc_dr_preset *p; const orc_dr_view *v;
  const float *ref; float *img; float *depth; float pv[16];
} rctx;

/* CastRayWithGrad (:1084-1294); returns the pixel loss */
static float cast_ray_grad(const rctx *r, uint32_t x, uint32_t y, float *g) {
  const orc_dr_preset *p = r->p;
  const uint32_t W = r->v->width, spp = p->spp;
  uint8_t *mask = p->raycasting_mask ? r->v->cast_mask : NULL;
  if (mask && !mask[(size_t)y * W + x]) return 0.0f;   /* masked pixel: not cast (:1097-1100) */
  ctx_f cx = {r->s, r->P};
  const uint32_t flags = pixel_flags(p);
  f3v res = mk_f(0, 0, 0);
  int hit_count = 0;
  float *samples = (float *)malloc(sizeof(float) * (spp ? spp : 1));
  /* per hit sample: 8 colour PDs (index, dFinalColor) and 64 distance PDs */
  uint32_t *ci = (uint32_t *)malloc(sizeof(uint32_t) * 8 * spp), *di = (uint32_t *)malloc(sizeof(uint32_t) * 64 * spp);
  f3v *cv = (f3v *)malloc(sizeof(f3v) * 8 * spp), *dv = (f3v *)malloc(sizeof(f3v) * 64 * spp);
  payload_f *pl = (payload_f *)malloc(sizeof(payload_f));
  for (uint32_t i = 0; i < spp; i++) {
    float dx, dy, pos[4], dir[4];
    rand2(x, y, i, p->seed, &dx, &dy);
    orc_eye_ray(x, y, r->v->width, r->v->height, dx, dy, r->v->proj_inv, r->v->wv_inv, pos, dir);
    m3_f dCdD = rows_f(mk_f(1, 0, 0), mk_f(0, 1, 0), mk_f(0, 0, 1));
    m3_f dCdN = rows_f(mk_f(0, 0, 0), mk_f(0, 0, 0), mk_f(0, 0, 0));
    hitdr_f h = query_f(&cx, flags, pos, dir, pl);
    if (h.primId == 0xFFFFFFFFu) continue;
    f3v c = color_grad(p, &h, &dCdD, &dCdN);
    res = add_f(res, divs_f(c, (float)spp));
    if (flags & ORC_DR_RAY_FLAG_DDIFFUSE_DCOLOR)
      for (int k = 0; k < 8; k++) {
        float val = pl->dc_value[k];
        ci[8 * hit_count + k] = pl->dc_index[k];
        cv[8 * hit_count + k] = mv_f(dCdD, mk_f(val, val, val));
      }
    if (flags & (ORC_DR_RAY_FLAG_DDIFFUSE_DPOS | ORC_DR_RAY_FLAG_DNORM_DPOS)) {
      for (int k = 0; k < 64; k++) {
        di[64 * hit_count + k] = pl->dd_index[k];
        dv[64 * hit_count + k] = add_f(mv_f(dCdD, pl->dd_diffuse[k]), mv_f(dCdN, pl->dd_norm[k]));
      }
    } else if (flags & ORC_DR_RAY_FLAG_DDIST_DPOS) {
      for (int k = 0; k < 64; k++) {
        di[64 * hit_count + k] = pl->dd_index[k];
        float q = pl->dd_dist[k];
        dv[64 * hit_count + k] = divs_f(mk_f(q, q, q), Z_FAR - Z_NEAR);
      }
    }
    samples[hit_count] = h.t;
    hit_count++;
  }
  const size_t px = (size_t)y * W + x;
  if (mask) mask[px] = hit_count > 0 ? 1 : 0;           /* process_mask, copied to masks[image] (:443-448, :1164-1167) */
  float cm[4] = {res.x, res.y, res.z, (float)hit_count / (float)spp};
  memcpy(r->img + 4 * px, cm, 16);
  r->depth[px] = hit_count == 0 ? 0.0f : t_threshold(samples, hit_count, 1e9f, spp - hit_count);
  const float *rf = r->ref + 4 * px;
  float loss = loss4(p->loss_function, cm, rf);
  float lg[4];
  loss_grad4(p->loss_function, cm, rf, lg);
  f3v dL = mk_f(lg[0], lg[1], lg[2]);
  dL = divs_f(muls_f(dL, 1.0f), (float)spp);
  if (flags & ORC_DR_RAY_FLAG_DDIFFUSE_DCOLOR)
    for (int k = 0; k < 8 * hit_count; k++) {
      if (ci[k] == 0xFFFFFFFFu) continue;
      f3v d = mul_f(dL, cv[k]);
      g[ci[k] + 0] += d.x; g[ci[k] + 1] += d.y; g[ci[k] + 2] += d.z;
    }
  if (flags & (ORC_DR_RAY_FLAG_DDIFFUSE_DPOS | ORC_DR_RAY_FLAG_DNORM_DPOS | ORC_DR_RAY_FLAG_DDIST_DPOS))
    for (int k = 0; k < 64 * hit_count; k++) {
      if (di[k] == 0xFFFFFFFFu) continue;
      g[di[k]] += dot_f(dL, dv[k]);
    }
  free(samples); free(ci); free(di); free(cv); free(dv); free(pl);
  return loss;
}

/* CalculateBorderRayDerivatives (:1319-1375) */
static void border_ray_derivs(const rctx *r, float pdf, const payload_f *pl, const hitdr_f *h, const float pos[4],
                              const float dir[4], float *g) {
  const orc_dr_preset *p = r->p;
  const uint32_t W = r->v->width, H = r->v->height;
  const float eps = p->border_relax_eps;
  const int miss = h->primId == 0xFFFFFFFFu;
  float cd[4] = {0, 0, 0, 0};
  if (p->input_type == 0) {
    f3v fin = color_plain(p, &pl->missed_hit);
    f3v fout = miss ? mk_f(0, 0, 0) : color_plain(p, h);
    f3v dd = sub_f(fin, fout);
    cd[0] = dd.x; cd[1] = dd.y; cd[2] = dd.z; cd[3] = miss ? 1.0f : 0.0f;
  } else {
    float din = lin_depth(pl->missed_hit.t), dout = miss ? 0.0f : lin_depth(h->t);
    cd[0] = cd[1] = cd[2] = din - dout; cd[3] = miss ? 1.0f : 0.0f;
  }
  for (int j = 0; j < 8; j++) {
    if (pl->missed_indices[j] == 0xFFFFFFFFu) continue;
    float bd = mx_f(0.0f, pl->missed_hit.sdf);
    f3v ys = add_f(mk_f(pos[0], pos[1], pos[2]), scl_f(pl->missed_hit.t, mk_f(dir[0], dir[1], dir[2])));
    f3v xs = sub_f(ys, scl_f(bd, pl->missed_hit.normal));
    float sx, sy;
    w2s(r->pv, xs, &sx, &sy);
    /* the reference converts to unsigned without a range check; out-of-image
     * projections (which read outside its image there) are skipped here */
    float fx = sx * (float)W, fy = sy * (float)H;
    if (!(fx >= 0.0f && fx < (float)W && fy >= 0.0f && fy < (float)H)) continue;
    uint32_t xp = (uint32_t)fx, yp = (uint32_t)fy;
    if (xp >= W || yp >= H) continue;
    float lg[4];
    loss_grad4(p->loss_function, r->img + 4 * ((size_t)yp * W + xp), r->ref + 4 * ((size_t)yp * W + xp), lg);
    float dt = lg[0] * cd[0] + lg[1] * cd[1] + lg[2] * cd[2] + lg[3] * cd[3];
    float diff = pdf * (1.0f / eps) * dt * pl->missed_dSDF_dtheta[j];
    g[pl->missed_indices[j]] += diff;
  }
}

/* CastBorderRay (:1377-1499), random sampling */
static void cast_border_ray(const rctx *r, uint32_t x, uint32_t y, float *g) {
  const orc_dr_preset *p = r->p;
  ctx_f cx = {r->s, r->P};
  payload_f *pl = (payload_f *)malloc(sizeof(payload_f));
  for (uint32_t sid = 0; sid < p->border_spp; sid++) {
    float dx, dy, pos[4], dir[4];
    rand2(x, y, sid, p->seed, &dx, &dy);
    orc_eye_ray(x, y, r->v->width, r->v->height, dx, dy, r->v->proj_inv, r->v->wv_inv, pos, dir);
    hitdr_f h = query_f(&cx, ORC_DR_RAY_FLAG_BORDER, pos, dir, pl);
    if (pl->missed_hit.sdf < p->border_relax_eps)
      border_ray_derivs(r, 1.0f / (float)p->border_spp, pl, &h, pos, dir, g);
  }
  free(pl);
}

/* ---- SVM border sampling, CastBorderRaySVM (:1651-1931) ---- */
void orc_dr_svm_fit(float *X, uint32_t N, float W[4]) {   /* SVM_fit (:1518-1546) */
  const float etha = 0.01f, alpha = 0.1f;
  const int epochs = 200;
  for (uint32_t i = 0; i < 3 * N; i++) X[i] = X[i] * etha;
  uint32_t errors = N;
  float w0 = -1.0f, w1 = 1.0f, w2 = 0.0f;
  const float mult = 1.0f - etha * alpha / (float)epochs;
  for (int e = 0; e < epochs && errors > 0; e++) {
    errors = 0;
    for (uint32_t j = 0; j < N; j++) {
      const float margin = w0 * X[3 * j] + w1 * X[3 * j + 1] + w2 * X[3 * j + 2];
      w0 = w0 * mult; w1 = w1 * mult; w2 = w2 * mult;
      if (margin < 0) {
        w0 = w0 + X[3 * j]; w1 = w1 + X[3 * j + 1]; w2 = w2 + X[3 * j + 2];
        errors++;
      }
    }
  }
  W[0] = w0; W[1] = w1; W[2] = w2; W[3] = (float)errors / (float)N;
}

static uint32_t out_code(float x, float y) {   /* ComputeOutCode (:1552-1578), window [0,1]^2 */
  uint32_t c = 0;
  if (x < 0.0f) c |= 1u; else if (x > 1.0f) c |= 2u;
  if (y < 0.0f) c |= 4u; else if (y > 1.0f) c |= 8u;
  return c;
}

/* CohenSutherlandLineClip (:1580-1649).  Each pass moves one end onto a window
 * edge; four passes settle a segment, and the loop is bounded at eight (a
 * segment still unsettled then is rejected; the GPU kernel uses the same bound). */
int orc_dr_line_clip(float *x0, float *y0, float *x1, float *y1) {
  uint32_t c0 = out_code(*x0, *y0), c1 = out_code(*x1, *y1);
  for (int it = 0; it < 8; it++) {
    if (!(c0 | c1)) return 1;
    if (c0 & c1) return 0;
    float x = -1, y = -1;
    const uint32_t co = c1 > c0 ? c1 : c0;
    if (co & 8u) { x = *x0 + (*x1 - *x0) * (1.0f - *y0) / (*y1 - *y0); y = 1.0f; }
    else if (co & 4u) { x = *x0 + (*x1 - *x0) * (0.0f - *y0) / (*y1 - *y0); y = 0.0f; }
    else if (co & 2u) { y = *y0 + (*y1 - *y0) * (1.0f - *x0) / (*x1 - *x0); x = 1.0f; }
    else if (co & 1u) { y = *y0 + (*y1 - *y0) * (0.0f - *x0) / (*x1 - *x0); x = 0.0f; }
    if (co == c0) { *x0 = x; *y0 = y; c0 = out_code(*x0, *y0); }
    else { *x1 = x; *y1 = y; c1 = out_code(*x1, *y1); }
  }
  return 0;
}

/* The SVM stage of CastBorderRaySVM for one border pixel: the sampling line, or
 * count 0 when the pixel has no border to integrate.  The reference draws the
 * stripe positions from the process-wide rand() (urand, :36-39), whose sequence
 * depends on OpenMP scheduling; here both uniforms come from rand2 of the sample
 * index, so every implementation draws the same stripe points. */
void orc_dr_svm_line(const orc_dr_scene *s, const float *params, const orc_dr_preset *p, const orc_dr_view *v,
                     uint32_t x, uint32_t y, orc_dr_svm_line_t *L) {
  const float min_sample_radius = 0.15f, sample_radius_mult = 2.0f, max_error_rate = 0.05f;
  const float min_stripe_area = 0.005f, svm_samples_budget = 0.25f;
  const float relax_eps = p->border_relax_eps;
  memset(L, 0, sizeof(*L));
  unsigned svm_spp = (unsigned)(svm_samples_budget * (float)p->border_spp);
  if (svm_spp < 1u) svm_spp = 1u;
  const uint32_t sq = (uint32_t)sqrt((double)svm_spp);
  const float isq = 1.0f / (float)sq;
  svm_spp = sq * sq;
  L->svm_spp = svm_spp;
  ctx_f cx = {s, params};
  payload_f *pl = (payload_f *)malloc(sizeof(payload_f));
  float *X = (float *)malloc(sizeof(float) * 3 * svm_spp), *ts = (float *)malloc(sizeof(float) * svm_spp);
  f3v closest = mk_f(1e6f, 1e6f, 1e6f);
  float closest_t = 1e6f;
  for (uint32_t k = 0; k < svm_spp; k++) {
    float rx, ry, pos[4], dir[4];
    rand2(x, y, k, p->seed, &rx, &ry);
    const float dx = isq * ((float)(k / sq) + rx), dy = isq * ((float)(k % sq) + ry);
    orc_eye_ray(x, y, v->width, v->height, dx, dy, v->proj_inv, v->wv_inv, pos, dir);
    hitdr_f h = query_f(&cx, 0u, pos, dir, pl);
    X[3 * k] = dx; X[3 * k + 1] = dy; X[3 * k + 2] = 1.0f;
    ts[k] = h.t;
    if (h.t < closest_t) {
      closest_t = h.t;
      closest = add_f(mk_f(pos[0], pos[1], pos[2]), scl_f(h.t, mk_f(dir[0], dir[1], dir[2])));
    }
  }
  const float thr = t_threshold(ts, svm_spp, 0.0f, 0u);
  unsigned type0 = 0;
  for (uint32_t k = 0; k < svm_spp; k++) {
    const float lab = ts[k] <= thr ? -1.0f : 1.0f;
    type0 += ts[k] <= thr ? 1u : 0u;
    X[3 * k] *= lab; X[3 * k + 1] *= lab; X[3 * k + 2] *= lab;
  }
  if (type0 == svm_spp || type0 == 0) goto done;
  {
    float W[4];
    orc_dr_svm_fit(X, svm_spp, W);
    const float err = W[3];
    const float f0 = (float)type0 / (float)svm_spp;
    const float rare = mn_f(f0, 1.0f - f0);
    float p0x = 0, p0y = 0, p1x = 0, p1y = 0, rx = 0, ry = 0, nx = 0, ny = 0, radius = 0, area = 0;
    int force = 0;
    if (err > max_error_rate || 2 * err > rare) {
      force = 1;
      area = 1.0f;
    } else {
      if (fabsf(W[1]) > 1e-6f && fabsf(W[0]) > 1e-6f) {
        p0x = 0.0f; p0y = -W[2] / W[1];
        p1x = 1.0f; p1y = (-W[2] - W[0]) / W[1];
        const float rY = p1y - p0y;
        if (p0y < -1e-6f || p0y > 1 + 1e-6f) {
          const float k1 = -p0y / rY, k2 = (1 - p0y) / rY, k = (fabsf(k1) < fabsf(k2)) ? k1 : k2;
          p0x = p0x + k * 1.0f; p0y = p0y + k * rY;
        }
        if (p1y < -1e-6f || p1y > 1 + 1e-6f) {
          const float k1 = -p1y / rY, k2 = (1 - p1y) / rY, k = (fabsf(k1) < fabsf(k2)) ? k1 : k2;
          p1x = p1x + k * 1.0f; p1y = p1y + k * rY;
        }
      } else if (fabsf(W[0]) > 1e-6f) {
        p0x = -W[2] / W[0]; p0y = 0.0f;
        p1x = -W[2] / W[0]; p1y = 1.0f;
      } else {
        force = 1;
      }
      if (!orc_dr_line_clip(&p0x, &p0y, &p1x, &p1y)) goto done;
      float thick;
      {
        const f3v up = mk_f(v->world_view[4], v->world_view[5], v->world_view[6]);
        float ax, ay, bx, by;
        float pv[16];
        mat4_mul(v->proj, v->world_view, pv);
        w2s(pv, closest, &ax, &ay);
        w2s(pv, add_f(closest, scl_f(relax_eps, up)), &bx, &by);
        const float ddx = bx - ax, ddy = by - ay;
        thick = sqrtf(ddx * ddx + ddy * ddy) * (float)(v->width > v->height ? v->width : v->height);
      }
      radius = mx_f(min_sample_radius, thick) + sample_radius_mult * err;
      rx = p1x - p0x; ry = p1y - p0y;
      float l = sqrtf(rx * rx + ry * ry);
      const float ux = rx / l, uy = ry / l;
      p0x = p0x - radius * ux; p0y = p0y - radius * uy;
      p1x = p1x + radius * ux; p1y = p1y + radius * uy;
      rx = p1x - p0x; ry = p1y - p0y;
      l = sqrtf(ry * ry + rx * rx);
      nx = -ry / l; ny = rx / l;
      area = 2 * radius * sqrtf(rx * rx + ry * ry);
      if (!force && area < min_stripe_area) goto done;
    }
    const float area_mult = mn_f(1.0f, 0.05f + 2.0f * area);
    unsigned cnt = (unsigned)(area_mult * (float)(p->border_spp - svm_spp));
    if (cnt < 1u) cnt = 1u;
    L->count = cnt;
    L->force = (uint32_t)force;
    L->p0[0] = p0x; L->p0[1] = p0y; L->r[0] = rx; L->r[1] = ry; L->n[0] = nx; L->n[1] = ny;
    L->radius = radius;
    L->pdf = force ? 1.0f / (float)cnt : area / (float)cnt;
  }
done:
  free(pl); free(X); free(ts);
}

/* The sub-pixel position of border sample j (sample index svm_spp + j) of a line. */
void orc_dr_svm_sample(const orc_dr_svm_line_t *L, uint32_t x, uint32_t y, uint32_t seed, uint32_t j, float d[2]) {
  float u, w;
  rand2(x, y, L->svm_spp + j, seed, &u, &w);
  if (L->force) { d[0] = u; d[1] = w; return; }
  const float a = u, b = w * 2.0f - 1.0f;         /* urand(0, 1), urand(-1, 1) */
  const float br = b * L->radius;
  d[0] = (L->p0[0] + a * L->r[0]) + br * L->n[0];
  d[1] = (L->p0[1] + a * L->r[1]) + br * L->n[1];
}

/* CastBorderRaySVM (:1651-1931) */
static void cast_border_ray_svm(const rctx *r, uint32_t x, uint32_t y, float *g) {
  const orc_dr_preset *p = r->p;
  orc_dr_svm_line_t L;
  orc_dr_svm_line(r->s, r->P, p, r->v, x, y, &L);
  if (L.count == 0) return;
  ctx_f cx = {r->s, r->P};
  payload_f *pl = (payload_f *)malloc(sizeof(payload_f));
  for (uint32_t j = 0; j < L.count; j++) {
    float d[2], pos[4], dir[4];
    orc_dr_svm_sample(&L, x, y, p->seed, j, d);
    if (!(d[0] > 0 && d[0] < 1 && d[1] > 0 && d[1] < 1)) continue;
    orc_eye_ray(x, y, r->v->width, r->v->height, d[0], d[1], r->v->proj_inv, r->v->wv_inv, pos, dir);
    hitdr_f h = query_f(&cx, ORC_DR_RAY_FLAG_BORDER, pos, dir, pl);
    if (pl->missed_hit.sdf < p->border_relax_eps) border_ray_derivs(r, L.pdf, pl, &h, pos, dir, g);
  }
  free(pl);
}

static int nthreads(int threads) {
#ifdef _OPENMP
  return threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
  return 1;
#endif
}

/* The reference's pixel order: SuperBlockIndex2DOpt / kernel_PackXY
 * (Renderer/eye_ray.cpp:524-570) over the size padded to PACK_XY_BLOCK_SIZE (8):
 * 4x4 blocks inside 2x2 super-blocks.  RenderDR walks tidX = 0, 1, ... through
 * this table; out[] receives the row-major indices of the in-image entries in
 * that order (all W*H pixels; the reference's loop bound W*H leaves some out
 * when W or H is not a multiple of 8, which is rendered fully here). */
static uint32_t packed_order(uint32_t W, uint32_t H, uint32_t *out) {
  const uint32_t W8 = 8 * ((W + 7) / 8), H8 = 8 * ((H + 7) / 8);
  uint32_t *tab = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)W8 * H8);
  for (uint32_t y = 0; y < H8; y++)
    for (uint32_t x = 0; x < W8; x++) {
      const uint32_t inBlockIdX = x & 3u, inBlockIdY = y & 3u, localIndex = inBlockIdY * 4 + inBlockIdX;
      const uint32_t wBlocks = W8 >> 2, blockX = x >> 2, blockY = y >> 2;
      const uint32_t inHBlockIdX = blockX & 1u, inHBlockIdY = blockY & 1u, localIndexH = inHBlockIdY * 2 + inHBlockIdX;
      const uint32_t wBlocksH = wBlocks >> 1, blockHX = blockX >> 1, blockHY = blockY >> 1;
      tab[(blockHX + blockHY * wBlocksH) * 64 + localIndexH * 16 + localIndex] = (y << 16) | x;
    }
  uint32_t n = 0;
  for (uint32_t i = 0; i < W8 * H8; i++) {
    const uint32_t x = tab[i] & 0xFFFFu, y = tab[i] >> 16;
    if (x < W && y < H) out[n++] = y * W + x;
  }
  free(tab);
  return n;
}

double orc_dr_render(const orc_dr_scene *s, const float *params, const orc_dr_preset *p, const orc_dr_view *v,
                     const float *image_ref, float *out_image, float *out_depth, float *grad,
                     uint8_t *border_mask, int threads) {
  const int T = nthreads(threads);
  const uint32_t W = v->width, H = v->height, N = W * H, np = s->n_params;
  rctx r;
  r.s = s; r.P = params; r.p = p; r.v = v; r.ref = image_ref; r.img = out_image; r.depth = out_depth;
  mat4_mul(v->proj, v->world_view, r.pv);
  float *slices = (float *)calloc((size_t)np * T, sizeof(float));
  double *lv = (double *)calloc(T, sizeof(double));
  const uint32_t steps = (N + T - 1) / T;
  uint32_t *order = (uint32_t *)malloc(sizeof(uint32_t) * N);
  packed_order(W, H, order);
  /* I: pixels in the packed order, split into T contiguous ranges (:596-607) */
#pragma omp parallel for num_threads(T) schedule(static, 1)
  for (int t = 0; t < T; t++) {
    uint32_t b = t * steps, e = (t + 1) * steps < N ? (t + 1) * steps : N;
    for (uint32_t k = b; k < e; k++) {
      const uint32_t i = order[k];
      lv[t] += cast_ray_grad(&r, i % W, i / W, slices + (size_t)np * t);
    }
  }
  /* II: border pixels, listed in the packed order (:609-685) */
  uint32_t *border = (uint32_t *)malloc(sizeof(uint32_t) * N);
  uint32_t nb = 0;
  for (uint32_t k = 0; k < N; k++) {
    const uint32_t i = order[k];
    uint32_t x = i % W, y = i / W;
    float d0 = out_image[4 * (size_t)i + 3], max_diff = 0, max_thr = 0;
    if (x >= 1 && x < W - 1 && y >= 1 && y < H - 1)
      for (int ddx = -1; ddx <= 1; ddx++)
        for (int ddy = -1; ddy <= 1; ddy++) {
          size_t q = (size_t)(y + ddy) * W + x + ddx;
          max_diff = mx_f(max_diff, fabsf(d0 - out_image[4 * q + 3]));
          max_thr = mx_f(max_thr, out_depth[q]);
        }
    int is_border = p->render_mode == ORC_DR_RENDER_MASK ? max_diff > 0 : (max_diff > 0 || max_thr > 0);
    if (border_mask) border_mask[i] = (uint8_t)is_border;
    if (is_border) border[nb++] = i;
  }
  /* III: border integral (:690-731) */
  if (nb > 0 && (p->reconstruction_flags & ORC_DR_RECON_GEOMETRY)) {
    const uint32_t bsteps = (nb + T - 1) / T;
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; t++) {
      uint32_t b = t * bsteps, e = (t + 1) * bsteps < nb ? (t + 1) * bsteps : nb;
      for (uint32_t i = b; i < e; i++) {
        if (p->border_sampling == 1) cast_border_ray_svm(&r, border[i] % W, border[i] / W, slices + (size_t)np * t);
        else cast_border_ray(&r, border[i] % W, border[i] / W, slices + (size_t)np * t);
      }
    }
  }
  /* IV: getBaseGradientMult (:140-145), applied to every slice; slices summed in order */
  const float gm = (float)(pow(np + 1.0, 2.0 / 3.0) / ((double)W * (double)H));
  for (size_t i = 0; i < (size_t)np * T; i++) slices[i] *= gm;
  for (uint32_t j = 0; j < np; j++) {
    float a = slices[j];
    for (int t = 1; t < T; t++) a += slices[j + (size_t)np * t];
    grad[j] = a;
  }
  double loss = 0;
  for (int t = 0; t < T; t++) loss += lv[t];
  free(slices); free(lv); free(border); free(order);
  return loss / (double)N;
}

void orc_dr_adam(uint32_t iter, const float *g, float *x, float *state, uint32_t n, float lr, float b1, float b2,
                 float eps) {
  float *V = state, *S = state + n;
  const double c1 = 1.0 - pow((double)b1, (double)(iter + 1)), c2 = 1.0 - pow((double)b2, (double)(iter + 1));
  for (uint32_t i = 0; i < n; i++) {
    float gi = g[i];
    V[i] = b1 * V[i] + (1 - b1) * gi;
    float Vh = (float)((double)V[i] / c1);
    S[i] = b2 * S[i] + (1 - b2) * gi * gi;
    float Sh = (float)((double)S[i] / c2);
    float nx = x[i] - lr * Vh / (sqrtf(Sh) + eps);
    x[i] = clampr_f(nx, -1000.0f, 1000.0f);
  }
}

void orc_dr_step(const orc_dr_scene *s, float *params, const orc_dr_preset *p, const orc_dr_view *views,
                 const float *images, uint32_t n_images, uint32_t iter, float *adam_state, float *grad_out,
                 double *losses, float *images_out, int threads) {
  const uint32_t np = s->n_params;
  float *acc = (float *)calloc(np, sizeof(float)), *g = (float *)malloc(sizeof(float) * np);
  size_t off = 0;
  for (uint32_t k = 0; k < n_images; k++) {
    const orc_dr_view *v = &views[k];
    const size_t n = (size_t)v->width * v->height;
    /* zeroed: a pixel outside the ray-casting mask is not rendered and keeps what the
     * reference's image held there, the miss (0, 0, 0, 0) of its last cast */
    float *img = (float *)calloc(4 * n, sizeof(float)), *dep = (float *)calloc(n, sizeof(float));
    double l = orc_dr_render(s, params, p, v, images + 4 * off, img, dep, g, NULL, threads);
    if (losses) losses[k] = l;
    if (images_out) memcpy(images_out + 4 * off, img, 16 * n);
    if (p->accumulate_batch) for (uint32_t j = 0; j < np; j++) acc[j] += g[j];
    else memcpy(acc, g, sizeof(float) * np);     /* the reference refills its buffer per image */
    free(img); free(dep);
    off += n;
  }
  if (p->reg_function != 0) orc_dr_regularize(s, params, p, acc);               /* :453-456 */
  if (p->redistancing_enable && p->redistancing_interval && iter % p->redistancing_interval == 0) {   /* :459-466 */
    const uint32_t bc = (uint32_t)cbrt((double)s->n_nodes);
    const uint32_t pc = bc * s->hdr.brick_size + 1;
    orc_dr_redistance(params, pc, 2.f / pc, pc);
  }
  for (uint32_t j = 0; j < np; j++) acc[j] /= (float)n_images;
  if (grad_out) memcpy(grad_out, acc, sizeof(float) * np);
  orc_dr_adam(iter, acc, params, adam_state, np, p->lr, p->beta1, p->beta2, p->eps);
  free(acc); free(g);
}

/* double-precision interior loss (forward part of CastRayWithGrad) */
double orc_dr_loss_f64(const orc_dr_scene *s, const double *params, const orc_dr_preset *p,
                       const orc_dr_view *v, const float *image_ref, uint8_t *hit_count) {
  const uint32_t W = v->width, H = v->height, N = W * H;
  ctx_d cx = {s, params};
  double total = 0;
#pragma omp parallel for reduction(+ : total) schedule(dynamic, 16)
  for (int64_t i = 0; i < (int64_t)N; i++) {
    const uint32_t x = (uint32_t)(i % W), y = (uint32_t)(i / W);
    payload_d *pl = (payload_d *)malloc(sizeof(payload_d));
    v3_d res = mk_d(0, 0, 0);
    int hc = 0;
    for (uint32_t k = 0; k < p->spp; k++) {
      float dx, dy, pos[4], dir[4];
      rand2(x, y, k, p->seed, &dx, &dy);
      orc_eye_ray(x, y, W, H, dx, dy, v->proj_inv, v->wv_inv, pos, dir);
      hitdr_d h = query_d(&cx, 0, pos, dir, pl);
      if (h.primId == 0xFFFFFFFFu) continue;
      v3_d c = mk_d(1, 0, 1);
      switch (p->render_mode) {
        case ORC_DR_RENDER_DIFFUSE: c = h.color; break;
        case ORC_DR_RENDER_LAMBERT:
          c = mk_d(0, 0, 0);
          for (uint32_t li = 0; li < p->n_lights; li++) {
            const orc_dr_light *L = &p->lights[li];
            v3_d lc = mk_d(L->color[0], L->color[1], L->color[2]);
            if (L->type == 0) {
              double q = mx_d(0.0, dot_d(h.normal, mk_d(L->dir[0], L->dir[1], L->dir[2])));
              c = add_d(c, muls_d(mul_d(lc, h.color), q));
            } else {
              c = add_d(c, mul_d(lc, h.color));
            }
          }
          break;
        case ORC_DR_RENDER_MASK: c = mk_d(1, 1, 1); break;
        case ORC_DR_RENDER_LINEAR_DEPTH: { double d = (h.t - Z_NEAR) / (Z_FAR - Z_NEAR); c = mk_d(d, d, d); } break;
        case ORC_DR_RENDER_NORMAL: c = h.normal; break;
        default: break;
      }
      res = add_d(res, divs_d(c, (double)p->spp));
      hc++;
    }
    free(pl);
    const float *rf = image_ref + 4 * i;
    double cm[4] = {res.x, res.y, res.z, (double)hc / p->spp};
    double l = 0;
    for (int k = 0; k < 4; k++) {
      double d = cm[k] - rf[k];
      l += p->loss_function == 0 ? d * d : fabs(d);
    }
    total += l;
    if (hit_count) hit_count[i] = (uint8_t)hc;
  }
  return total / (double)N;
}

/* ---------------- create_grid_sbs + neighbours ---------------- */
uint32_t orc_dr_grid_sbs(uint32_t bc, uint32_t bs, const orc_sdf *f, const float *color3, orc_sbs_header *hdr,
                         orc_sbs_node **nodes_out, uint32_t **values_out, uint32_t *n_values, float **params_out,
                         uint32_t *n_params) {
  const uint32_t v = bs + 1, dist_per_node = v * v * v, pc = bc * bs + 1u, cc = bc + 1u;
  const uint32_t c_off = pc * pc * pc, nn = bc * bc * bc;
  const uint32_t per_old = dist_per_node + 8, per_new = dist_per_node + 8 + 27;
  hdr->brick_size = bs; hdr->brick_pad = 0; hdr->bytes_per_value = 4; hdr->aux_data = ORC_SBS_LAYOUT_ID32F_IRGB32F_IN;
  const uint32_t np = pc * pc * pc + 3 * cc * cc * cc;
  float *P = (float *)malloc(sizeof(float) * np);
  const float gdiv = (float)(bc * bs);
  for (uint32_t x = 0; x < pc; x++)
    for (uint32_t y = 0; y < pc; y++)
      for (uint32_t z = 0; z < pc; z++) {
        float px = 2.0f * ((float)x / gdiv) - 1.0f, py = 2.0f * ((float)y / gdiv) - 1.0f, pz = 2.0f * ((float)z / gdiv) - 1.0f;
        P[x * pc * pc + y * pc + z] = orc_sdf_eval(f, px, py, pz);
      }
  const float cdiv = (float)bc;
  for (uint32_t x = 0; x < cc; x++)
    for (uint32_t y = 0; y < cc; y++)
      for (uint32_t z = 0; z < cc; z++) {
        uint32_t idx = x * cc * cc + y * cc + z;
        float dx = (float)x / cdiv, dy = (float)y / cdiv, dz = (float)z / cdiv;
        float c[3];
        if (color3) { c[0] = color3[0]; c[1] = color3[1]; c[2] = color3[2]; }
        else {
          float qx = 2.0f * dx - 1.0f, qy = 2.0f * dy - 1.0f, qz = 2.0f * dz - 1.0f;
          c[0] = 0.5f + 0.5f * qx; c[1] = 0.5f + 0.5f * qy; c[2] = 0.5f + 0.5f * qz;
        }
        P[c_off + 3 * idx + 0] = c[0]; P[c_off + 3 * idx + 1] = c[1]; P[c_off + 3 * idx + 2] = c[2];
      }
  orc_sbs_node *nodes = (orc_sbs_node *)calloc(nn, sizeof(orc_sbs_node));
  uint32_t *vals = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)nn * per_new);
  for (uint32_t bx = 0; bx < bc; bx++)
    for (uint32_t by = 0; by < bc; by++)
      for (uint32_t bz = 0; bz < bc; bz++) {
        uint32_t n = bx * bc * bc + by * bc + bz, off = n * per_new;
        nodes[n].pos_xy = (bx << 16) | by;
        nodes[n].pos_z_lod_size = (bz << 16) | bc;
        nodes[n].data_offset = off;
        for (uint32_t x = 0; x < v; x++)
          for (uint32_t y = 0; y < v; y++)
            for (uint32_t z = 0; z < v; z++)
              vals[off + x * v * v + y * v + z] = (bx * bs + x) * pc * pc + (by * bs + y) * pc + (bz * bs + z);
        for (uint32_t x = 0; x < 2; x++)
          for (uint32_t y = 0; y < 2; y++)
            for (uint32_t z = 0; z < 2; z++)
              vals[off + dist_per_node + x * 4 + y * 2 + z] = c_off + 3 * ((bx + x) * cc * cc + (by + y) * cc + (bz + z));
        for (int i = 0; i < 27; i++) vals[off + per_old + i] = ORC_INVALID_IDX;
      }
  /* neighbours through shared corners (utils/sparse_octree_builder.cpp:2802-2850) */
  uint32_t *adj = (uint32_t *)malloc(sizeof(uint32_t) * 9 * (size_t)np);   /* count + 8 node ids per value */
  for (size_t i = 0; i < (size_t)np; i++) { adj[9 * i] = 0; for (int k = 1; k < 9; k++) adj[9 * i + k] = ORC_INVALID_IDX; }
  for (uint32_t n = 0; n < nn; n++)
    for (int r = 0; r < 8; r++) {
      uint32_t ix = (v - 1) * ((r & 4) >> 2), iy = (v - 1) * ((r & 2) >> 1), iz = (v - 1) * (r & 1);
      uint32_t corner = vals[nodes[n].data_offset + ix * v * v + iy * v + iz];
      adj[9 * (size_t)corner + 1 + r] = n;
      adj[9 * (size_t)corner]++;
    }
  for (size_t i = 0; i < (size_t)np; i++) {
    if (adj[9 * i] <= 1) continue;
    for (int r1 = 0; r1 < 8; r1++) {
      if (adj[9 * i + 1 + r1] == ORC_INVALID_IDX) continue;
      for (int r2 = 0; r2 < 8; r2++) {
        if (adj[9 * i + 1 + r2] == ORC_INVALID_IDX || r1 == r2) continue;
        /* (the reference compares nodes[r1] and nodes[r2] sizes, equal on a grid) */
        int dx = ((r2 & 4) >> 2) - ((r1 & 4) >> 2) + 1, dy = ((r2 & 2) >> 1) - ((r1 & 2) >> 1) + 1, dz = (r2 & 1) - (r1 & 1) + 1;
        uint32_t nb = 9 * dx + 3 * dy + dz;
        uint32_t node_id = adj[9 * i + 1 + r2], nbr = adj[9 * i + 1 + r1];
        vals[nodes[node_id].data_offset + per_old + nb] = nbr;
      }
    }
  }
  free(adj);
  *nodes_out = nodes; *values_out = vals; *n_values = nn * per_new; *params_out = P; *n_params = np;
  return nn;
}


/* Regularization, diff_render/MultiRendererDR.cpp:1933-2055 (the reference sums
 * per-thread slices afterwards; here one pass in node order) */
void orc_dr_regularize(const orc_dr_scene *s, const float *params, const orc_dr_preset *p, float *grad) {
  const uint32_t v = s->hdr.brick_size + 1;
  const float power = p->reg_power, lambda = p->reg_lambda;
  for (uint32_t node = 0; node < s->n_nodes; node++) {
    const uint32_t off = s->nodes[node].data_offset;
    for (uint32_t i0 = 0; i0 < v; i0++)
      for (uint32_t j0 = 0; j0 < v; j0++)
        for (uint32_t k0 = 0; k0 < v; k0++) {
          const uint32_t idx = off + i0 * v * v + j0 * v + k0;
          const int has[6] = {i0 > 0, i0 < v - 1, j0 > 0, j0 < v - 1, k0 > 0, k0 < v - 1};
          const int64_t step[6] = {-(int64_t)(v * v), (int64_t)(v * v), -(int64_t)v, (int64_t)v, -1, 1};
          for (int n = 0; n < 6; n++) {
            if (!has[n]) continue;
            float d = params[s->values[idx]] - params[s->values[(int64_t)idx + step[n]]];
            const float sgn_d = d > 0.0f ? 1.0f : -1.0f;
            d = fabsf(d);
            grad[s->values[idx]] += lambda * power * sgn_d * powf(d, power - 1);
          }
        }
  }
}

/* SolveEikonal, :2058-2120 (f = 1) */
static float solve_eikonal(float m0, float m1, float m2, float h) {
  float m[3] = {m0, m1, m2}, t;
  if (m[0] > m[1]) { t = m[0]; m[0] = m[1]; m[1] = t; }
  if (m[0] > m[2]) { t = m[0]; m[0] = m[2]; m[2] = t; }
  if (m[1] > m[2]) { t = m[1]; m[1] = m[2]; m[2] = t; }
  float dist_new = m[0] + h;
  if (dist_new > m[1]) {
    const float h_2 = h * h;
    float m_sum = m[0] + m[1], c_2 = (m[0] - m[1]) * (m[0] - m[1]);
    float x2 = (m_sum + sqrtf(2 * h_2 - c_2)) * 0.5f;
    dist_new = x2;
    if (dist_new > m[2]) {
      const float one_third = 1.f / 3;
      m_sum += m[2];
      c_2 = 3.f * (m[0] * m[0] + m[1] * m[1] + m[2] * m[2] - h_2);
      x2 = (m_sum + sqrtf(m_sum * m_sum - c_2)) * one_third;
      dist_new = x2;
    }
  }
  return dist_new;
}

/* Redistance, :2122-2330.  Every update of an iteration reads the previous
 * iteration's array, so the reference's 8 sweep orderings all compute the same
 * values: one Jacobi update per iteration. */
void orc_dr_redistance(float *dist, uint32_t n, float h, uint32_t n_iters) {
  const size_t N = (size_t)n * n * n;
  const int64_t off[3] = {(int64_t)n * n, (int64_t)n, 1};
  const float big = 99999.f;
  float *b[2] = {(float *)malloc(4 * N), (float *)malloc(4 * N)};
  uint8_t *frozen = (uint8_t *)malloc(N);
  for (size_t li = 0; li < N; li++) {
    const int ix[3] = {(int)(li / ((size_t)n * n)), (int)((li / n) % n), (int)(li % n)};
    frozen[li] = 0;
    b[0][li] = b[1][li] = big;
    const float dv = dist[li];
    if (dv == 0.f) { frozen[li] = 1; b[0][li] = b[1][li] = 0.f; }
    if (!frozen[li])
      for (int dim = 0; dim < 3; dim++)
        for (int sg = -1; sg < 2; sg += 2) {
          const int q = ix[dim] + sg;
          if (q >= 0 && q < (int)n) {
            const float nv = dist[(int64_t)li + sg * off[dim]];
            if (nv * dv < 0) { b[0][li] = b[1][li] = dv; frozen[li] = 1; }
          }
        }
  }
  int cur = 0;
  for (uint32_t it = 0; it < n_iters; it++) {
    const float *old = b[1 - cur];
    float *nw = b[cur];
    for (size_t li = 0; li < N; li++) {
      nw[li] = old[li];
      if (frozen[li]) continue;
      const int ix[3] = {(int)(li / ((size_t)n * n)), (int)((li / n) % n), (int)(li % n)};
      float am[3] = {big, big, big};
      for (int dim = 0; dim < 3; dim++) {
        if (ix[dim] > 0 && ix[dim] < (int)n - 1) {
          am[dim] = old[(int64_t)li - off[dim]];
          const float tmp = old[(int64_t)li + off[dim]];
          if (fabsf(tmp) < fabsf(am[dim])) am[dim] = tmp;
        } else if (ix[dim] > 0 && ix[dim] == (int)n - 1) {
          am[dim] = old[(int64_t)li - off[dim]];
        } else if (ix[dim] == 0 && ix[dim] < (int)n - 1) {
          am[dim] = old[(int64_t)li + off[dim]];
        }
      }
      if (am[0] < big || am[1] < big || am[2] < big) {
        const int pos_part = am[0] >= 0.f && am[1] >= 0.f && am[2] >= 0.f;
        if (pos_part) {
          const float e = solve_eikonal(am[0], am[1], am[2], h);
          nw[li] = e < old[li] ? e : old[li];                          /* std::min */
        } else {
          for (int k = 0; k < 3; k++) if (am[k] < 0.f) am[k] = -am[k];
          const float e = -solve_eikonal(am[0], am[1], am[2], h), o = -fabsf(old[li]);
          nw[li] = e < o ? o : e;                                      /* std::max */
        }
      }
    }
    cur = 1 - cur;
  }
  memcpy(dist, b[1 - cur], 4 * N);
  free(b[0]); free(b[1]); free(frozen);
}

/* ---- OptimizeGrid's grids (diff_render/MultiRendererDR.cpp:228-276) ---- */
static void gradient_color_f(float px, float py, float pz, float *c) {   /* DR_common.cpp:25-35 */
  const float w[8] = {(1 - px) * (1 - py) * (1 - pz), (1 - px) * (1 - py) * (pz), (1 - px) * (py) * (1 - pz),
                      (1 - px) * (py) * (pz),         (px) * (1 - py) * (1 - pz), (px) * (1 - py) * (pz),
                      (px) * (py) * (1 - pz),         (px) * (py) * (pz)};
  static const float col[8][3] = {{1, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 1, 0}, {1, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 1, 0}};
  for (int k = 0; k < 3; k++) {
    float a = w[0] * col[0][k];
    for (int i = 1; i < 8; i++) a = a + w[i] * col[i][k];
    c[k] = a;
  }
}

static float grid_sampler_f(const float *d, uint32_t gs, uint32_t bs, const float p[3]) {   /* :242-262 */
  const uint32_t pc = gs * bs + 1u;
  float f[3], dp[3];
  uint32_t i[3];
  for (int k = 0; k < 3; k++) {
    float c = 0.5f * (p[k] + 1.0f);
    c = mn_f(mx_f(c, 0.0f), 1.0f + 1e-6f);
    f[k] = (c * (float)gs) * (float)bs;
    i[k] = (uint32_t)(f[k] + 1e-6f);
    dp[k] = f[k] - (float)i[k];
  }
#define AT(a, b, c) d[(a) * pc * pc + (b) * pc + (c)]
  if (i[0] < pc - 1 && i[1] < pc - 1 && i[2] < pc - 1) {
    const float x = dp[0], y = dp[1], z = dp[2];
    return (1 - x) * (1 - y) * (1 - z) * AT(i[0], i[1], i[2]) + (1 - x) * (1 - y) * z * AT(i[0], i[1], i[2] + 1) +
           (1 - x) * y * (1 - z) * AT(i[0], i[1] + 1, i[2]) + (1 - x) * y * z * AT(i[0], i[1] + 1, i[2] + 1) +
           x * (1 - y) * (1 - z) * AT(i[0] + 1, i[1], i[2]) + x * (1 - y) * z * AT(i[0] + 1, i[1], i[2] + 1) +
           x * y * (1 - z) * AT(i[0] + 1, i[1] + 1, i[2]) + x * y * z * AT(i[0] + 1, i[1] + 1, i[2] + 1);
  }
  return AT(i[0], i[1], i[2]);
#undef AT
}

void orc_dr_grid_resample(uint32_t gs, uint32_t bs, const float *old_params, uint32_t old_bs, float *out) {
  const uint32_t pc = gs * bs + 1u, cc = gs + 1u, c_off = pc * pc * pc;
  const float gdiv = (float)(gs * bs), cdiv = (float)gs;
  for (uint32_t x = 0; x < pc; x++)
    for (uint32_t y = 0; y < pc; y++)
      for (uint32_t z = 0; z < pc; z++) {
        const float p[3] = {2.0f * ((float)x / gdiv) - 1.0f, 2.0f * ((float)y / gdiv) - 1.0f,
                            2.0f * ((float)z / gdiv) - 1.0f};
        float v;
        if (old_params) {
          v = grid_sampler_f(old_params, gs, old_bs, p);
        } else {   /* circle_sdf(float3(0, -0.15, 0), 0.7, p), DR_common.cpp:16-19 */
          const float dx = p[0] - 0.0f, dy = p[1] - (-0.15f), dz = p[2] - 0.0f;
          v = sqrtf(dx * dx + dy * dy + dz * dz) - 0.7f;
        }
        out[x * pc * pc + y * pc + z] = v;
      }
  for (uint32_t x = 0; x < cc; x++)
    for (uint32_t y = 0; y < cc; y++)
      for (uint32_t z = 0; z < cc; z++) {
        const uint32_t idx = x * cc * cc + y * cc + z;
        gradient_color_f(2.0f * ((float)x / cdiv) - 1.0f, 2.0f * ((float)y / cdiv) - 1.0f,
                         2.0f * ((float)z / cdiv) - 1.0f, out + c_off + 3 * idx);
      }
}
