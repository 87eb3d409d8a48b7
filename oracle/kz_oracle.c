/*
 * kz_oracle.c - CPU oracle for the kazan draw path.  TEST INFRASTRUCTURE ONLY (see kz_oracle.h).
 * PARITY UNPINNED: no reference rasteriser exists (vulkan-driver/src/api_impl.rs:4632-4653 are stubs);
 * the rules restated here are the Vulkan specification's "Rasterization" and "Fragment operations"
 * chapters with the open choices fixed as listed in kz_oracle.h.
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared -pthread (see oracle/Makefile).
 */
#include "kz_oracle.h"
#include "../kazan_gb300/csrc/kz_srgb_table.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define KZO_MAXK 4        /* varyings per vertex for the two shaders (rgba or normal xyz) */
#define KZO_G 4.0f        /* guard band factor */
#define KZO_MAXPOLY 9

/* Vulkan enumerant values used below (from the specification) */
enum { CMP_NEVER, CMP_LESS, CMP_EQUAL, CMP_LEQUAL, CMP_GREATER, CMP_NOTEQUAL, CMP_GEQUAL, CMP_ALWAYS };
enum {
  BF_ZERO, BF_ONE, BF_SRC_COLOR, BF_ONE_MINUS_SRC_COLOR, BF_DST_COLOR, BF_ONE_MINUS_DST_COLOR, BF_SRC_ALPHA,
  BF_ONE_MINUS_SRC_ALPHA, BF_DST_ALPHA, BF_ONE_MINUS_DST_ALPHA, BF_CONSTANT_COLOR, BF_ONE_MINUS_CONSTANT_COLOR,
  BF_CONSTANT_ALPHA, BF_ONE_MINUS_CONSTANT_ALPHA, BF_SRC_ALPHA_SATURATE
};
enum { BO_ADD, BO_SUBTRACT, BO_REVERSE_SUBTRACT, BO_MIN, BO_MAX };

uint8_t kzo_unorm8(float v) {
  float c = fminf(fmaxf(v, 0.0f), 1.0f);
  return (uint8_t)(int)rintf(c * 255.0f);
}

static float u8_to_f32(uint8_t u) { return (float)u / 255.0f; }

/* ---- shaders (the SPIR-V semantics the PTX backend implements, restated in C) ---- */

typedef struct {
  float c[4 + KZO_MAXK]; /* clip position x,y,z,w then varyings */
} cvert;

static int shader_varyings(const kzo_draw* d) {
  return d->shader == KZO_SHADER_COLOR ? 4 : d->shader == KZO_SHADER_TEXTURED ? 2 : 3;
}

/* ---- texture sampling (kz_pipeline.cu kz_tex2d restated) ---- */

static int32_t tex_wrap(int32_t i, int32_t size, uint32_t mode) {
  switch (mode) {
    case 0: { /* REPEAT */
      int32_t m = i % size;
      return m < 0 ? m + size : m;
    }
    case 1: { /* MIRRORED_REPEAT */
      int32_t m = i % (2 * size);
      if (m < 0) m += 2 * size;
      m -= size;
      return size - 1 - (m >= 0 ? m : -(1 + m));
    }
    case 3: /* CLAMP_TO_BORDER */
      return i < 0 || i >= size ? -1 : i;
    case 4: { /* MIRROR_CLAMP_TO_EDGE */
      int32_t mir = i >= 0 ? i : -(1 + i);
      return mir < size ? mir : size - 1;
    }
    default: /* CLAMP_TO_EDGE */
      return i < 0 ? 0 : (i >= size ? size - 1 : i);
  }
}

static int32_t tex_int(float x) { return (int32_t)fminf(fmaxf(x, -1.0e9f), 1.0e9f); }

static void tex_texel(const kzo_texture* t, int32_t i, int32_t j, float out[4]) {
  if (i < 0 || j < 0) {
    uint32_t b = (t->sampler >> 12) & 3u;
    float c = b == 2 ? 1.0f : 0.0f;
    out[0] = out[1] = out[2] = c;
    out[3] = b == 0 ? 0.0f : 1.0f;
    return;
  }
  const uint8_t* p = t->texels + (size_t)j * t->pitch + (size_t)i * 4;
  float c[4];
  for (int k = 0; k < 4; k++) c[k] = (float)p[k] / 255.0f;
  if (t->format == 2) {
    out[0] = c[2];
    out[1] = c[1];
    out[2] = c[0];
  } else {
    out[0] = c[0];
    out[1] = c[1];
    out[2] = c[2];
  }
  out[3] = c[3];
}

static float tex_lerp(float a, float b, float f) { return a + f * (b - a); }

void kzo_tex2d(const kzo_texture* t, float s, float tc, float out[4]) {
  const int32_t w = (int32_t)t->width, h = (int32_t)t->height;
  const uint32_t mu = (t->sampler >> 4) & 7u, mv = (t->sampler >> 8) & 7u;
  float u = s, v = tc;
  if (!(t->sampler & 2u)) {
    u = s * (float)w;
    v = tc * (float)h;
  }
  if (!(t->sampler & 1u)) {
    tex_texel(t, tex_wrap(tex_int(floorf(u)), w, mu), tex_wrap(tex_int(floorf(v)), h, mv), out);
    return;
  }
  float u0 = u - 0.5f, v0 = v - 0.5f;
  float fi = floorf(u0), fj = floorf(v0);
  float a = fminf(fmaxf(u0 - fi, 0.0f), 1.0f), b = fminf(fmaxf(v0 - fj, 0.0f), 1.0f);
  int32_t i0 = tex_int(fi), j0 = tex_int(fj);
  int32_t x0 = tex_wrap(i0, w, mu), x1 = tex_wrap(i0 + 1, w, mu);
  int32_t y0 = tex_wrap(j0, h, mv), y1 = tex_wrap(j0 + 1, h, mv);
  float t00[4], t10[4], t01[4], t11[4];
  tex_texel(t, x0, y0, t00);
  tex_texel(t, x1, y0, t10);
  tex_texel(t, x0, y1, t01);
  tex_texel(t, x1, y1, t11);
  for (int k = 0; k < 4; k++) out[k] = tex_lerp(tex_lerp(t00[k], t10[k], a), tex_lerp(t01[k], t11[k], a), b);
}

/* vertex shader: COLOR is gl_Position = in0, out0 = in1; LAMBERT is gl_Position = mvp * vec4(in0, 1),
 * out0 = in1.  OpMatrixTimesVector is r_i = fma(m3i, v3, fma(m2i, v2, fma(m1i, v1, m0i * v0))). */
static void run_vs(const kzo_draw* d, uint32_t vid, cvert* out) {
  if (d->shader == KZO_SHADER_COLOR) {
    const float* v = d->vertices + (size_t)vid * 8;
    for (int i = 0; i < 8; i++) out->c[i] = v[i];
  } else if (d->shader == KZO_SHADER_TEXTURED) {
    const float* v = d->vertices + (size_t)vid * 6;
    for (int i = 0; i < 6; i++) out->c[i] = v[i];
    out->c[6] = out->c[7] = 0.0f;
  } else {
    const float* v = d->vertices + (size_t)vid * 6;
    const float* m = d->mvp;
    float in[4] = {v[0], v[1], v[2], 1.0f};
    for (int i = 0; i < 4; i++) {
      float t = m[0 * 4 + i] * in[0];
      t = fmaf(m[1 * 4 + i], in[1], t);
      t = fmaf(m[2 * 4 + i], in[2], t);
      t = fmaf(m[3 * 4 + i], in[3], t);
      out->c[i] = t;
    }
    out->c[4] = v[3];
    out->c[5] = v[4];
    out->c[6] = v[5];
    out->c[7] = 0.0f;
  }
}

/* fragment shader: COLOR writes the varying; LAMBERT writes
 * vec4(albedo * max(dot(normalize(n), L), 0), 1) with
 * dot(a, b) = fma(a2, b2, fma(a1, b1, a0 * b0)) and normalize(x) = x * (1 / sqrt(dot(x, x))). */
static void run_fs(const kzo_draw* d, const float* var, float out[4]) {
  if (d->shader == KZO_SHADER_COLOR) {
    for (int i = 0; i < 4; i++) out[i] = var[i];
  } else if (d->shader == KZO_SHADER_TEXTURED) {
    kzo_tex2d(&d->tex, var[0], var[1], out);
  } else {
    float n0 = var[0], n1 = var[1], n2 = var[2];
    float dd = fmaf(n2, n2, fmaf(n1, n1, n0 * n0));
    float len = sqrtf(dd);
    float inv = 1.0f / len;
    float m0 = n0 * inv, m1 = n1 * inv, m2 = n2 * inv;
    float dl = fmaf(m2, d->light[2], fmaf(m1, d->light[1], m0 * d->light[0]));
    dl = fmaxf(dl, 0.0f);
    out[0] = d->albedo[0] * dl;
    out[1] = d->albedo[1] * dl;
    out[2] = d->albedo[2] * dl;
    out[3] = 1.0f;
  }
}

/* ---- clipping ---- */

static float plane_dist(const float* p, int plane) {
  switch (plane) {
    case 0: return p[2];                  /* z >= 0 */
    case 1: return p[3] - p[2];           /* z <= w */
    case 2: return p[0] + KZO_G * p[3];   /* x >= -4w */
    case 3: return KZO_G * p[3] - p[0];   /* x <= 4w */
    case 4: return p[1] + KZO_G * p[3];   /* y >= -4w */
    default: return KZO_G * p[3] - p[1];  /* y <= 4w */
  }
}

/* returns the number of polygon vertices (0 = rejected) */
static int clip_polygon(const cvert in[3], int nc, cvert poly[KZO_MAXPOLY]) {
  cvert a[KZO_MAXPOLY], b[KZO_MAXPOLY];
  int n = 3;
  for (int i = 0; i < 3; i++) a[i] = in[i];
  cvert* cur = a;
  cvert* nxt = b;
  for (int plane = 0; plane < 6; plane++) {
    int any_out = 0;
    for (int i = 0; i < n; i++)
      if (plane_dist(cur[i].c, plane) < 0.0f) any_out = 1;
    if (!any_out) continue;
    int m = 0;
    for (int i = 0; i < n; i++) {
      const cvert* p = &cur[i];
      const cvert* q = &cur[(i + 1) % n];
      float dp = plane_dist(p->c, plane), dq = plane_dist(q->c, plane);
      int pin = dp >= 0.0f, qin = dq >= 0.0f;
      if (pin) nxt[m++] = *p;
      if (pin != qin) {
        const cvert* vi = pin ? p : q;
        const cvert* vo = pin ? q : p;
        float di = pin ? dp : dq, dout = pin ? dq : dp;
        float t = di / (di - dout);
        cvert c;
        for (int k = 0; k < 4 + nc; k++) c.c[k] = fmaf(t, vo->c[k] - vi->c[k], vi->c[k]);
        nxt[m++] = c;
      }
    }
    n = m;
    cvert* tmp = cur;
    cur = nxt;
    nxt = tmp;
    if (n < 3) return 0;
  }
  for (int i = 0; i < n; i++) {
    if (!(cur[i].c[3] > 0.0f)) return 0;
    poly[i] = cur[i];
  }
  return n;
}

/* ---- prepared (sub-)triangle ---- */

typedef struct {
  int32_t X[3], Y[3];
  int64_t S;
  float inv_s;
  float z0, dz1, dz2;
  float iw[3];
  float a[3][KZO_MAXK]; /* varying * (1/w) */
  int tl[3];
  int32_t bx0, by0, bx1, by1; /* inclusive pixel box */
  int front;
  uint32_t draw;
} prep;

typedef struct {
  prep* v;
  size_t n, cap;
  kzo_stats st;
} prep_list;

static void push_prep(prep_list* l, const prep* p) {
  if (l->n == l->cap) {
    l->cap = l->cap ? l->cap * 2 : 1024;
    l->v = (prep*)realloc(l->v, l->cap * sizeof(prep));
  }
  l->v[l->n++] = *p;
}

static int64_t floordiv256(int64_t a) { return a >= 0 ? a / 256 : -((-a + 255) / 256); }

void kzo_draw_rect(uint32_t width, uint32_t height, const int32_t area[4], const kzo_draw* d, int32_t out[4]) {
  int32_t x0 = 0, y0 = 0, x1 = (int32_t)width, y1 = (int32_t)height;
  if (area[0] > x0) x0 = area[0];
  if (area[1] > y0) y0 = area[1];
  if (area[2] < x1) x1 = area[2];
  if (area[3] < y1) y1 = area[3];
  if (d->scissor[0] > x0) x0 = d->scissor[0];
  if (d->scissor[1] > y0) y0 = d->scissor[1];
  if (d->scissor[0] + d->scissor[2] < x1) x1 = d->scissor[0] + d->scissor[2];
  if (d->scissor[1] + d->scissor[3] < y1) y1 = d->scissor[1] + d->scissor[3];
  /* pixel x is inside the viewport iff x + 0.5 lies in [vx, vx + vw) */
  float vx = d->viewport[0], vy = d->viewport[1], vw = d->viewport[2], vh = d->viewport[3];
  float ylo = vh >= 0.0f ? vy : vy + vh, yhi = vh >= 0.0f ? vy + vh : vy;
  int32_t px0 = (int32_t)ceilf(vx - 0.5f), px1 = (int32_t)ceilf(vx + vw - 0.5f);
  int32_t py0 = (int32_t)ceilf(ylo - 0.5f), py1 = (int32_t)ceilf(yhi - 0.5f);
  if (px0 > x0) x0 = px0;
  if (py0 > y0) y0 = py0;
  if (px1 < x1) x1 = px1;
  if (py1 < y1) y1 = py1;
  out[0] = x0;
  out[1] = y0;
  out[2] = x1;
  out[3] = y1;
}

/* project + snap + cull + orient one (sub-)triangle; appends to the list if it can produce fragments */
static void setup_tri(const kzo_draw* d, uint32_t di, const int32_t rect[4], const cvert v[3], int nc,
                      prep_list* out) {
  float hx = 0.5f * d->viewport[2], ox = d->viewport[0] + hx;
  float hy = 0.5f * d->viewport[3], oy = d->viewport[1] + hy;
  float pz = d->viewport[5] - d->viewport[4], oz = d->viewport[4];
  prep p;
  float zf[3];
  memset(&p, 0, sizeof(p));
  for (int i = 0; i < 3; i++) {
    float iw = 1.0f / v[i].c[3];
    float xd = v[i].c[0] * iw, yd = v[i].c[1] * iw, zd = v[i].c[2] * iw;
    float xf = fmaf(xd, hx, ox), yf = fmaf(yd, hy, oy);
    zf[i] = fmaf(zd, pz, oz);
    p.X[i] = (int32_t)rintf(xf * 256.0f);
    p.Y[i] = (int32_t)rintf(yf * 256.0f);
    p.iw[i] = iw;
    for (int k = 0; k < nc; k++) p.a[i][k] = v[i].c[4 + k] * iw;
  }
  int64_t S = (int64_t)(p.X[1] - p.X[0]) * (p.Y[2] - p.Y[0]) - (int64_t)(p.X[2] - p.X[0]) * (p.Y[1] - p.Y[0]);
  if (S == 0) {
    out->st.rejected++;
    return;
  }
  int front = d->front_ccw ? (S < 0) : (S > 0);
  if (((d->cull_mode & 2u) && !front) || ((d->cull_mode & 1u) && front)) {
    out->st.rejected++;
    return;
  }
  if (S < 0) {
    int32_t t;
    float f;
    t = p.X[1]; p.X[1] = p.X[2]; p.X[2] = t;
    t = p.Y[1]; p.Y[1] = p.Y[2]; p.Y[2] = t;
    f = zf[1]; zf[1] = zf[2]; zf[2] = f;
    f = p.iw[1]; p.iw[1] = p.iw[2]; p.iw[2] = f;
    for (int k = 0; k < nc; k++) {
      f = p.a[1][k];
      p.a[1][k] = p.a[2][k];
      p.a[2][k] = f;
    }
    S = -S;
  }
  int32_t minx = p.X[0], maxx = p.X[0], miny = p.Y[0], maxy = p.Y[0];
  for (int i = 1; i < 3; i++) {
    if (p.X[i] < minx) minx = p.X[i];
    if (p.X[i] > maxx) maxx = p.X[i];
    if (p.Y[i] < miny) miny = p.Y[i];
    if (p.Y[i] > maxy) maxy = p.Y[i];
  }
  /* pixels with a sample point (offset 128, or 32..224 for 4 samples) in [min, max] */
  const int64_t lo = d->samples == 4 ? 32 : 128, hi = d->samples == 4 ? 224 : 128;
  int64_t bx0 = -floordiv256(-((int64_t)minx - hi)); /* ceil((minx - hi) / 256) */
  int64_t by0 = -floordiv256(-((int64_t)miny - hi));
  int64_t bx1 = floordiv256((int64_t)maxx - lo);
  int64_t by1 = floordiv256((int64_t)maxy - lo);
  if (bx0 < rect[0]) bx0 = rect[0];
  if (by0 < rect[1]) by0 = rect[1];
  if (bx1 > rect[2] - 1) bx1 = rect[2] - 1;
  if (by1 > rect[3] - 1) by1 = rect[3] - 1;
  if (bx0 > bx1 || by0 > by1) {
    out->st.rejected++;
    return;
  }
  p.bx0 = (int32_t)bx0;
  p.by0 = (int32_t)by0;
  p.bx1 = (int32_t)bx1;
  p.by1 = (int32_t)by1;
  for (int e = 0; e < 3; e++) {
    int a = (e + 1) % 3, b = (e + 2) % 3; /* edge e is opposite vertex e: v(e+1) -> v(e+2) */
    int32_t dx = p.X[b] - p.X[a], dy = p.Y[b] - p.Y[a];
    p.tl[e] = (dy < 0) || (dy == 0 && dx > 0);
  }
  p.S = S;
  p.inv_s = 1.0f / (float)S;
  p.z0 = zf[0];
  p.dz1 = zf[1] - zf[0];
  p.dz2 = zf[2] - zf[0];
  p.front = front;
  p.draw = di;
  out->st.subtris++;
  push_prep(out, &p);
}

static void process_triangle(const kzo_draw* d, uint32_t di, const int32_t rect[4], uint32_t t, prep_list* out) {
  uint32_t vid[3];
  for (int j = 0; j < 3; j++) {
    if (d->indices)
      vid[j] = (uint32_t)((int64_t)d->indices[d->first + 3 * t + j] + d->vertex_offset);
    else
      vid[j] = d->first + 3 * t + (uint32_t)j;
  }
  int nc = shader_varyings(d);
  cvert v[3];
  for (int j = 0; j < 3; j++) run_vs(d, vid[j], &v[j]);
  out->st.tris++;
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 4; k++)
      if (!isfinite(v[j].c[k])) {
        out->st.rejected++;
        return;
      }
  /* trivial reject against the view volume -w <= x,y <= w, 0 <= z <= w */
  int all[6] = {1, 1, 1, 1, 1, 1};
  for (int j = 0; j < 3; j++) {
    const float* c = v[j].c;
    all[0] &= c[0] > c[3];
    all[1] &= c[0] < -c[3];
    all[2] &= c[1] > c[3];
    all[3] &= c[1] < -c[3];
    all[4] &= c[2] < 0.0f;
    all[5] &= c[2] > c[3];
  }
  if (all[0] | all[1] | all[2] | all[3] | all[4] | all[5]) {
    out->st.rejected++;
    return;
  }
  int need = 0;
  for (int j = 0; j < 3; j++)
    for (int plane = 0; plane < 6; plane++)
      if (plane_dist(v[j].c, plane) < 0.0f) need = 1;
  if (!need) {
    setup_tri(d, di, rect, v, nc, out);
    return;
  }
  out->st.clipped++;
  cvert poly[KZO_MAXPOLY];
  int n = clip_polygon(v, nc, poly);
  if (n == 0) {
    out->st.rejected++;
    return;
  }
  for (int i = 1; i + 1 < n; i++) {
    cvert tri[3] = {poly[0], poly[i], poly[i + 1]};
    setup_tri(d, di, rect, tri, nc, out);
  }
}

static int depth_cmp(uint32_t op, float z, float d) {
  switch (op) {
    case CMP_NEVER: return 0;
    case CMP_LESS: return z < d;
    case CMP_EQUAL: return z == d;
    case CMP_LEQUAL: return z <= d;
    case CMP_GREATER: return z > d;
    case CMP_NOTEQUAL: return z != d;
    case CMP_GEQUAL: return z >= d;
    default: return 1;
  }
}

float kzo_depth_value(float z, uint32_t depth_format) {
  if (depth_format == KZO_DEPTH_D16) return rintf(z * 65535.0f);
  if (depth_format == KZO_DEPTH_D24S8) return rintf(z * 16777215.0f);
  return z;
}

/* VkStencilOp applied to the stored value s, through the write mask */
static uint8_t stencil_apply(uint32_t op, uint8_t s, const kzo_stencil* so) {
  uint32_t v;
  switch (op) {
    case 1: v = 0; break;                                  /* ZERO */
    case 2: v = so->reference & 0xFFu; break;              /* REPLACE */
    case 3: v = s < 255 ? s + 1u : 255u; break;            /* INCREMENT_AND_CLAMP */
    case 4: v = s > 0 ? s - 1u : 0u; break;                /* DECREMENT_AND_CLAMP */
    case 5: v = ~(uint32_t)s & 0xFFu; break;               /* INVERT */
    case 6: v = (s + 1u) & 0xFFu; break;                   /* INCREMENT_AND_WRAP */
    case 7: v = (s - 1u) & 0xFFu; break;                   /* DECREMENT_AND_WRAP */
    default: v = s; break;                                 /* KEEP */
  }
  uint32_t wm = so->write_mask & 0xFFu;
  return (uint8_t)((s & ~wm) | (v & wm));
}

/* the stencil comparison: reference OP stored, both under the compare mask */
static int stencil_cmp(uint32_t op, uint32_t ref, uint32_t val) {
  switch (op) {
    case CMP_NEVER: return 0;
    case CMP_LESS: return ref < val;
    case CMP_EQUAL: return ref == val;
    case CMP_LEQUAL: return ref <= val;
    case CMP_GREATER: return ref > val;
    case CMP_NOTEQUAL: return ref != val;
    case CMP_GEQUAL: return ref >= val;
    default: return 1;
  }
}

static float blend_factor(uint32_t f, int c, const float s[4], const float dst[4], const float k[4]) {
  switch (f) {
    case BF_ZERO: return 0.0f;
    case BF_ONE: return 1.0f;
    case BF_SRC_COLOR: return s[c];
    case BF_ONE_MINUS_SRC_COLOR: return 1.0f - s[c];
    case BF_DST_COLOR: return dst[c];
    case BF_ONE_MINUS_DST_COLOR: return 1.0f - dst[c];
    case BF_SRC_ALPHA: return s[3];
    case BF_ONE_MINUS_SRC_ALPHA: return 1.0f - s[3];
    case BF_DST_ALPHA: return dst[3];
    case BF_ONE_MINUS_DST_ALPHA: return 1.0f - dst[3];
    case BF_CONSTANT_COLOR: return k[c];
    case BF_ONE_MINUS_CONSTANT_COLOR: return 1.0f - k[c];
    case BF_CONSTANT_ALPHA: return k[3];
    case BF_ONE_MINUS_CONSTANT_ALPHA: return 1.0f - k[3];
    case BF_SRC_ALPHA_SATURATE: return c < 3 ? fminf(s[3], 1.0f - dst[3]) : 1.0f;
    default: return 0.0f;
  }
}

static float blend_op(uint32_t op, float s, float sf, float d, float df) {
  switch (op) {
    case BO_ADD: return fmaf(s, sf, d * df);
    case BO_SUBTRACT: return fmaf(s, sf, -(d * df));
    case BO_REVERSE_SUBTRACT: return fmaf(d, df, -(s * sf));
    case BO_MIN: return fminf(s, d);
    default: return fmaxf(s, d);
  }
}

/* 8-bit sRGB: the encode steps (threshold k - 1 is the smallest float with code k) and the decode values
 * of the sRGB transfer function, exact to the float (generated in 60-digit arithmetic) */
static const float srgb_thr[255] = KZ_SRGB_THRESHOLDS;
static const float srgb_dec[256] = KZ_SRGB_DECODE;

uint8_t kzo_srgb8(float v) {
  if (!(v > 0.0f)) return 0;
  if (v >= 1.0f) return 255;
  int n = 0;
  while (n < 255 && srgb_thr[n] <= v) n++; /* the steps at or below v */
  return (uint8_t)n;
}

/* one channel of a fragment output stored into the colour texel */
static uint8_t store_channel(const kzo_draw* d, int i, float v) {
  return d->srgb && i < 3 ? kzo_srgb8(v) : kzo_unorm8(v);
}

/* colour write or blend of one fragment output into the RGBA8 texel c.  The attachment is unsigned
 * normalized, so source, destination and the blend constants are clamped to [0, 1] before blending
 * (Vulkan specification, "Blend Operations"). */
static void write_color(const kzo_draw* d, uint8_t* c, const float out[4]) {
  if (d->blend_enable) {
    float s[4], dst[4], k[4];
    for (int i = 0; i < 4; i++) {
      s[i] = fminf(fmaxf(out[i], 0.0f), 1.0f);
      dst[i] = d->srgb && i < 3 ? srgb_dec[c[i]] : u8_to_f32(c[i]);
      k[i] = fminf(fmaxf(d->blend_const[i], 0.0f), 1.0f);
    }
    for (int i = 0; i < 4; i++) {
      if (!(d->write_mask & (1u << i))) continue;
      float r;
      if (i < 3)
        r = blend_op(d->color_op, s[i], blend_factor(d->src_color, i, s, dst, k), dst[i],
                     blend_factor(d->dst_color, i, s, dst, k));
      else
        r = blend_op(d->alpha_op, s[3], blend_factor(d->src_alpha, 3, s, dst, k), dst[3],
                     blend_factor(d->dst_alpha, 3, s, dst, k));
      c[i] = store_channel(d, i, r);
    }
  } else {
    for (int i = 0; i < 4; i++)
      if (d->write_mask & (1u << i)) c[i] = store_channel(d, i, out[i]);
  }
}

static const int32_t ms_dx[4] = {96, 224, 32, 160}, ms_dy[4] = {32, 96, 160, 224};

/* one pixel of a 4x multisampled draw (kzo_draw::samples) */
static void raster_pixel_ms(const kzo_draw* d, const prep* p, int nc, int32_t x, int32_t y, size_t pix, uint8_t* color,
                            float* depth, float zmin, float zmax, kzo_stats* st) {
  int64_t Es[4][3];
  unsigned cover = 0;
  for (int s = 0; s < 4; s++) {
    int64_t px = (int64_t)x * 256 + ms_dx[s], py = (int64_t)y * 256 + ms_dy[s];
    int inside = 1;
    for (int e = 0; e < 3; e++) {
      int a = (e + 1) % 3, b = (e + 2) % 3;
      Es[s][e] = (int64_t)(p->X[b] - p->X[a]) * (py - p->Y[a]) - (int64_t)(p->Y[b] - p->Y[a]) * (px - p->X[a]);
      if (!(Es[s][e] > 0 || (Es[s][e] == 0 && p->tl[e]))) inside = 0;
    }
    if (inside) cover |= 1u << s;
  }
  if (!cover) return;
  st->fragments++;
  float zs[4];
  unsigned pass = 0;
  for (int s = 0; s < 4; s++) {
    if (!((cover >> s) & 1u)) continue;
    float l1 = (float)Es[s][1] * p->inv_s, l2 = (float)Es[s][2] * p->inv_s;
    float z = fmaf(l2, p->dz2, fmaf(l1, p->dz1, p->z0));
    zs[s] = fminf(fmaxf(z, zmin), zmax) + 0.0f;
    if (!(d->depth_test && depth) || depth_cmp(d->depth_compare, zs[s], depth[pix * 4 + (size_t)s])) pass |= 1u << s;
  }
  if (!pass) return;
  st->depth_pass++;
  /* the fragment shader at the pixel centre */
  int64_t px = (int64_t)x * 256 + 128, py = (int64_t)y * 256 + 128;
  int64_t E[3];
  for (int e = 0; e < 3; e++) {
    int a = (e + 1) % 3, b = (e + 2) % 3;
    E[e] = (int64_t)(p->X[b] - p->X[a]) * (py - p->Y[a]) - (int64_t)(p->Y[b] - p->Y[a]) * (px - p->X[a]);
  }
  float l0 = (float)E[0] * p->inv_s, l1 = (float)E[1] * p->inv_s, l2 = (float)E[2] * p->inv_s;
  float q = fmaf(l2, p->iw[2], fmaf(l1, p->iw[1], l0 * p->iw[0]));
  float rq = 1.0f / q;
  float var[KZO_MAXK];
  for (int k = 0; k < nc; k++) var[k] = fmaf(l2, p->a[2][k], fmaf(l1, p->a[1][k], l0 * p->a[0][k])) * rq;
  float out[4];
  run_fs(d, var, out);
  for (int s = 0; s < 4; s++) {
    if (!((pass >> s) & 1u)) continue;
    if (d->depth_test && d->depth_write && depth) depth[pix * 4 + (size_t)s] = zs[s];
    write_color(d, color + (pix * 4 + (size_t)s) * 4, out);
  }
}

void kzo_resolve(uint32_t width, uint32_t height, const uint8_t* color4, uint8_t* color) {
  for (size_t pix = 0; pix < (size_t)width * height; pix++)
    for (int c = 0; c < 4; c++) {
      unsigned sum = 2;
      for (int s = 0; s < 4; s++) sum += color4[(pix * 4 + (size_t)s) * 4 + (size_t)c];
      color[pix * 4 + (size_t)c] = (uint8_t)(sum / 4);
    }
}

/* rasterise one prepared triangle over rows [ylo, yhi) */
static void raster_prep(const kzo_draw* draws, const prep* p, uint32_t width, uint8_t* color, float* depth,
                        uint8_t* stencil, uint32_t depth_format, int32_t ylo, int32_t yhi, kzo_stats* st) {
  const kzo_draw* d = &draws[p->draw];
  int nc = shader_varyings(d);
  int32_t y0 = p->by0 > ylo ? p->by0 : ylo, y1 = p->by1 < yhi - 1 ? p->by1 : yhi - 1;
  float zmin = fminf(d->viewport[4], d->viewport[5]), zmax = fmaxf(d->viewport[4], d->viewport[5]);
  for (int32_t y = y0; y <= y1; y++) {
    int64_t py = (int64_t)y * 256 + 128;
    for (int32_t x = p->bx0; x <= p->bx1; x++) {
      if (d->samples == 4) {
        raster_pixel_ms(d, p, nc, x, y, (size_t)y * width + (size_t)x, color, depth, zmin, zmax, st);
        continue;
      }
      int64_t px = (int64_t)x * 256 + 128;
      int64_t E[3];
      int inside = 1;
      for (int e = 0; e < 3; e++) {
        int a = (e + 1) % 3, b = (e + 2) % 3;
        E[e] = (int64_t)(p->X[b] - p->X[a]) * (py - p->Y[a]) - (int64_t)(p->Y[b] - p->Y[a]) * (px - p->X[a]);
        if (!(E[e] > 0 || (E[e] == 0 && p->tl[e]))) inside = 0;
      }
      if (!inside) continue;
      st->fragments++;
      float l0 = (float)E[0] * p->inv_s, l1 = (float)E[1] * p->inv_s, l2 = (float)E[2] * p->inv_s;
      float z = fmaf(l2, p->dz2, fmaf(l1, p->dz1, p->z0));
      z = fminf(fmaxf(z, zmin), zmax);
      z = z + 0.0f;
      size_t pix = (size_t)y * width + (size_t)x;
      const float zc = kzo_depth_value(z, depth_format);
      const int dpass = !(d->depth_test && depth) || depth_cmp(d->depth_compare, zc, depth[pix]);
      if (d->stencil_test && stencil) {
        const kzo_stencil* so = p->front ? &d->front : &d->back;
        uint8_t sv = stencil[pix];
        if (!stencil_cmp(so->compare_op, so->reference & so->compare_mask & 0xFFu, sv & so->compare_mask)) {
          stencil[pix] = stencil_apply(so->fail_op, sv, so);
          continue;
        }
        stencil[pix] = stencil_apply(dpass ? so->pass_op : so->depth_fail_op, sv, so);
      }
      if (!dpass) continue;
      st->depth_pass++;
      float q = fmaf(l2, p->iw[2], fmaf(l1, p->iw[1], l0 * p->iw[0]));
      float rq = 1.0f / q;
      float var[KZO_MAXK];
      for (int k = 0; k < nc; k++) {
        float num = fmaf(l2, p->a[2][k], fmaf(l1, p->a[1][k], l0 * p->a[0][k]));
        var[k] = num * rq;
      }
      float out[4];
      run_fs(d, var, out);
      if (d->depth_test && d->depth_write && depth) depth[pix] = zc;
      write_color(d, color + pix * 4, out);
    }
  }
}

/* ---- drivers: sequential and banded-parallel ---- */

typedef struct {
  const kzo_draw* draws;
  uint32_t num_draws;
  const int32_t (*rects)[4];
  const uint64_t* tri_base; /* prefix sums of triangle counts */
  uint64_t t0, t1;
  prep_list list;
} setup_job;

static void* setup_worker(void* arg) {
  setup_job* j = (setup_job*)arg;
  uint32_t di = 0;
  for (uint64_t g = j->t0; g < j->t1; g++) {
    while (g >= j->tri_base[di + 1]) di++;
    process_triangle(&j->draws[di], di, j->rects[di], (uint32_t)(g - j->tri_base[di]), &j->list);
  }
  return NULL;
}

typedef struct {
  const kzo_draw* draws;
  setup_job* jobs;
  int njobs;
  uint32_t width;
  uint8_t* color;
  float* depth;
  uint8_t* stencil;
  uint32_t depth_format;
  int32_t ylo, yhi;
  kzo_stats st;
} raster_job;

static void* raster_worker(void* arg) {
  raster_job* r = (raster_job*)arg;
  for (int j = 0; j < r->njobs; j++) {
    const prep_list* l = &r->jobs[j].list;
    for (size_t i = 0; i < l->n; i++) {
      const prep* p = &l->v[i];
      if (p->by1 < r->ylo || p->by0 >= r->yhi) continue;
      raster_prep(r->draws, p, r->width, r->color, r->depth, r->stencil, r->depth_format, r->ylo, r->yhi, &r->st);
    }
  }
  return NULL;
}

int kzo_render(uint32_t width, uint32_t height, uint8_t* color, float* depth, const int32_t render_area[4],
               uint32_t num_draws, const kzo_draw* draws, int nthreads, kzo_stats* stats) {
  return kzo_render_ds(width, height, color, depth, NULL, KZO_DEPTH_D32, render_area, num_draws, draws, nthreads,
                       stats);
}

int kzo_render_ds(uint32_t width, uint32_t height, uint8_t* color, float* depth, uint8_t* stencil,
                  uint32_t depth_format, const int32_t render_area[4], uint32_t num_draws, const kzo_draw* draws,
                  int nthreads, kzo_stats* stats) {
  if (nthreads < 1) nthreads = 1;
  uint64_t* base = (uint64_t*)calloc(num_draws + 1, sizeof(uint64_t));
  int32_t(*rects)[4] = (int32_t(*)[4])calloc(num_draws ? num_draws : 1, sizeof(int32_t[4]));
  if (!base || !rects) return -1;
  for (uint32_t i = 0; i < num_draws; i++) {
    base[i + 1] = base[i] + draws[i].tri_count;
    kzo_draw_rect(width, height, render_area, &draws[i], rects[i]);
  }
  uint64_t total = base[num_draws];
  int nsetup = nthreads;
  if ((uint64_t)nsetup > total) nsetup = total ? (int)total : 1;
  setup_job* jobs = (setup_job*)calloc((size_t)nsetup, sizeof(setup_job));
  pthread_t* th = (pthread_t*)calloc((size_t)(nthreads > nsetup ? nthreads : nsetup), sizeof(pthread_t));
  for (int j = 0; j < nsetup; j++) {
    jobs[j].draws = draws;
    jobs[j].num_draws = num_draws;
    jobs[j].rects = (const int32_t(*)[4])rects;
    jobs[j].tri_base = base;
    jobs[j].t0 = total * (uint64_t)j / (uint64_t)nsetup;
    jobs[j].t1 = total * (uint64_t)(j + 1) / (uint64_t)nsetup;
  }
  if (nsetup == 1) {
    setup_worker(&jobs[0]);
  } else {
    for (int j = 0; j < nsetup; j++) pthread_create(&th[j], NULL, setup_worker, &jobs[j]);
    for (int j = 0; j < nsetup; j++) pthread_join(th[j], NULL);
  }
  int nbands = nthreads;
  if ((uint32_t)nbands > height) nbands = height ? (int)height : 1;
  raster_job* rj = (raster_job*)calloc((size_t)nbands, sizeof(raster_job));
  for (int b = 0; b < nbands; b++) {
    rj[b].draws = draws;
    rj[b].jobs = jobs;
    rj[b].njobs = nsetup;
    rj[b].width = width;
    rj[b].color = color;
    rj[b].depth = depth;
    rj[b].stencil = stencil;
    rj[b].depth_format = depth_format;
    rj[b].ylo = (int32_t)((uint64_t)height * (uint64_t)b / (uint64_t)nbands);
    rj[b].yhi = (int32_t)((uint64_t)height * (uint64_t)(b + 1) / (uint64_t)nbands);
  }
  if (nbands == 1) {
    raster_worker(&rj[0]);
  } else {
    for (int b = 0; b < nbands; b++) pthread_create(&th[b], NULL, raster_worker, &rj[b]);
    for (int b = 0; b < nbands; b++) pthread_join(th[b], NULL);
  }
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    for (int j = 0; j < nsetup; j++) {
      stats->tris += jobs[j].list.st.tris;
      stats->rejected += jobs[j].list.st.rejected;
      stats->clipped += jobs[j].list.st.clipped;
      stats->subtris += jobs[j].list.st.subtris;
    }
    for (int b = 0; b < nbands; b++) {
      stats->fragments += rj[b].st.fragments;
      stats->depth_pass += rj[b].st.depth_pass;
    }
  }
  for (int j = 0; j < nsetup; j++) free(jobs[j].list.v);
  free(jobs);
  free(rj);
  free(th);
  free(base);
  free(rects);
  return 0;
}

void kzo_clear_color_srgb(uint32_t width, uint8_t* color, const int32_t rect[4], const float rgba[4]) {
  uint8_t px[4] = {kzo_srgb8(rgba[0]), kzo_srgb8(rgba[1]), kzo_srgb8(rgba[2]), kzo_unorm8(rgba[3])};
  for (int32_t y = rect[1]; y < rect[3]; y++)
    for (int32_t x = rect[0]; x < rect[2]; x++) memcpy(color + ((size_t)y * width + (size_t)x) * 4, px, 4);
}

void kzo_clear_color(uint32_t width, uint8_t* color, const int32_t rect[4], const float rgba[4]) {
  uint8_t px[4];
  for (int i = 0; i < 4; i++) px[i] = kzo_unorm8(rgba[i]);
  for (int32_t y = rect[1]; y < rect[3]; y++)
    for (int32_t x = rect[0]; x < rect[2]; x++) memcpy(color + ((size_t)y * width + (size_t)x) * 4, px, 4);
}

void kzo_clear_depth(uint32_t width, float* depth, const int32_t rect[4], float value) {
  for (int32_t y = rect[1]; y < rect[3]; y++)
    for (int32_t x = rect[0]; x < rect[2]; x++) depth[(size_t)y * width + (size_t)x] = value;
}
