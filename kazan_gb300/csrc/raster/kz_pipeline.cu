/*
 * kz_pipeline.cu - sm_103a pipeline kernels of the kazan draw path.
 *
 * Compiled once (nvcc -rdc=true -cubin) into a relocatable device object.  The shader stages are not
 * part of it: kz_vs / kz_vs_pos / kz_fs are resolved when a pipeline set is JIT-linked with the PTX
 * that the shader backend emits from SPIR-V (see shader/kz_ptx_backend.cpp).  The reference has no
 * counterpart for any kernel here (vulkan-driver/src/api_impl.rs:4632-4653 are `unimplemented!()`).
 *
 * Phases of one raster segment (see kz_raster_abi.h):
 *   visibility mode (opaque segments: no blending, a depth rule a minimum can express)
 *     vis_init      per pixel: the 64-bit key (depth, primitive) of the cleared or loaded depth
 *     vis_geometry  per 32-triangle group, one warp: index fetch, position-only vertex shader, clip codes,
 *                   projection, 16.8 snap, cull, setup; the warp rasterises the small triangles itself
 *                   (64-bit atomicMin into the keys) and turns the large ones into 8x8-block jobs
 *     vis_large     per job, one warp: the job's blocks
 *     vis_resolve   per 32-pixel row run, one warp: the winning primitive's setup again, one fragment-shader
 *                   call per pixel, colour and depth stored
 *   ordered mode (blending, discard, stencil, other compare ops, D16 / D24S8, multisampling)
 *     geometry      per triangle: as above, plus the record's shading setup -> KzTriRecord, tile counts
 *     scan          per tile: exclusive prefix of the counts -> bin offsets; capacity checks; the tiles'
 *                   raster order (largest bins first)
 *     bin           per record: its index into each overlapped tile's bin
 *     raster        per tile, taken from a counter in that order: bin sorted by primitive in shared
 *                   memory, each pixel run through it in API order (coverage, depth / stencil, fragment
 *                   shader, blend); the common case stages the tile's colour and depth through TMA
 *   Both run as separate kernels (chained by programmatic dependent launch) or inside one persistent
 *   cooperative kernel with bounded grid barriers between the phases.
 *
 * Arithmetic follows the rules the CPU oracle restates (every float op an explicit IEEE single op;
 * the file is built with -fmad=false and uses the __f*_rn intrinsics), so coverage, depth and colour
 * are bit-identical to it.
 */
#include <stdint.h>

#include "../kz_raster_abi.h"
#include "../kz_srgb_table.h"
#include "kz_exact.h"

/* vertex shader functions fetch their own attributes from the draw's vertex buffers */
extern "C" __device__ void kz_vs(uint32_t pipe, const KzDraw* draw, uint32_t vid, uint32_t iid, const uint8_t* push,
                                 KzVsOut* out);
extern "C" __device__ float4 kz_vs_pos(uint32_t pipe, const KzDraw* draw, uint32_t vid, uint32_t iid,
                                       const uint8_t* push);
extern "C" __device__ uint32_t kz_fs(uint32_t pipe, const KzFsIn* in, const uint8_t* push, float* color);
/* the fragment shader with inputs and outputs in registers, for interfaces of at most 8 varyings: varyings
 * v0..v7, gl_FragCoord, gl_FrontFacing in; colour and the discard flag out (float bits in 32-bit words) */
struct __align__(16) KzFsResult {
  float c[4];
  uint32_t discard;
  uint32_t pad[3];
};
extern "C" __device__ KzFsResult kz_fs_r8(uint32_t pipe, const uint8_t* push, uint32_t v0, uint32_t v1, uint32_t v2,
                                          uint32_t v3, uint32_t v4, uint32_t v5, uint32_t v6, uint32_t v7,
                                          uint32_t fc0, uint32_t fc1, uint32_t fc2, uint32_t fc3, uint32_t front);

/* gl_Position of the three vertices of one triangle in one call (push constants read once) */
struct KzPos3 {
  float4 p[3];
};
extern "C" __device__ KzPos3 kz_vs_pos3(uint32_t pipe, const KzDraw* draw, uint32_t vid0, uint32_t vid1, uint32_t vid2,
                                        uint32_t iid, const uint8_t* push);

#define KZ_THREADS 256
#define KZ_SORT_CAP 4096          /* ordered mode: largest bin sorted in shared memory */
#define KZ_BATCH 32               /* ordered mode: triangles set up per batch */

/* texture sampling (kz_tex2d, kz_tex_fetch) lives in kz_tex.cu, a separate object linked with the shaders */

namespace {

/* ---------------- exact arithmetic ---------------- */

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

__device__ __forceinline__ uint8_t unorm8(float v) {
  float c = fminf(fmaxf(v, 0.0f), 1.0f);
  return (uint8_t)__float2int_rn(fmul(c, 255.0f));
}
__device__ __forceinline__ float u8f(uint32_t u) { return fdiv(__uint2float_rn(u), 255.0f); }

/* the 8-bit sRGB formats (red, green and blue as sRGB codes, alpha linear): the exact encode steps and
 * decode values of kz_srgb_table.h, here for kernels without their own shared copy */
__device__ const float kz_srgb_thr_g[256] = KZ_SRGB_THRESHOLDS; /* 255 steps; the last entry is padding */
__device__ const float kz_srgb_dec_g[256] = KZ_SRGB_DECODE;

__device__ __forceinline__ bool cf_srgb(uint32_t fmt) { return fmt == KZ_CF_RGBA8_SRGB || fmt == KZ_CF_BGRA8_SRGB; }
__device__ __forceinline__ bool cf_bgra(uint32_t fmt) { return fmt == KZ_CF_BGRA8 || fmt == KZ_CF_BGRA8_SRGB; }

/* the 8-bit sRGB code of linear v: the number of encode steps thr[0..254] (ascending) at or below v, by
 * binary search; 0 for v <= 0 or NaN, 255 for v >= 1 */
__device__ __forceinline__ uint32_t srgb8(float v, const float* thr) {
  if (!(v > 0.0f)) return 0u;
  if (v >= 1.0f) return 255u;
  uint32_t n = 0;
#pragma unroll
  for (uint32_t step = 128; step > 0; step >>= 1)
    if (n + step <= 255u && thr[n + step - 1] <= v) n += step;
  return n;
}

/* shared-memory table of the raster kernels: u8f(k) for k = 0..255 (the sRGB tables stay in global
 * memory: with them the persistent kernel's static and dynamic shared memory would pass 48 KB) */
#define KZ_CTAB_FLOATS 256
__device__ __forceinline__ void fill_color_tabs(float* t) {
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) t[i] = u8f(i);
}


/* ---------------- frame access ---------------- */

struct Ctx {
  const KzFrame* f;
  const KzSegment* seg;
  KzSegCounters* cnt;
  KzStatus* st;
  const KzDraw* draws;
  const KzPipe* pipes;
};

__device__ __forceinline__ Ctx make_ctx(const KzFrame& f, uint32_t s) {
  Ctx c;
  c.f = &f;
  c.seg = reinterpret_cast<const KzSegment*>(f.segments) + s;
  c.cnt = reinterpret_cast<KzSegCounters*>(c.seg->counters);
  c.st = reinterpret_cast<KzStatus*>(f.status);
  c.draws = reinterpret_cast<const KzDraw*>(f.draws);
  c.pipes = reinterpret_cast<const KzPipe*>(f.pipes);
  return c;
}

__device__ __forceinline__ const uint8_t* push_ptr(const KzFrame& f, const KzDraw& d) {
  return reinterpret_cast<const uint8_t*>(f.push) + (size_t)d.push_index * KZ_PUSH_BYTES;
}

/* last draw of the segment whose prim_base <= g */
__device__ uint32_t find_draw(const KzDraw* draws, uint32_t first, uint32_t count, uint32_t g) {
  uint32_t lo = first, hi = first + count;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (draws[mid].prim_base <= g) lo = mid;
    else hi = mid;
  }
  return lo;
}

/* the last draw of [first, first + count) whose chunk_base <= k (draws without triangles share the
 * chunk_base of the next draw, so they are never chosen) */
__device__ __forceinline__ uint32_t draw_of_chunk(const KzDraw* draws, uint32_t first, uint32_t count, uint32_t k) {
  uint32_t lo = first, hi = first + count;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (draws[mid].chunk_base <= k) lo = mid;
    else hi = mid;
  }
  return lo;
}

/* chunk k of a segment: a table entry; for indirect segments, the draw from the chunk table built on the
 * device, or from a search when the table was too small */
__device__ __forceinline__ KzChunk chunk_at(const Ctx& c, uint32_t k) {
  const KzSegment& seg = *c.seg;
  if (!seg.indirect) return reinterpret_cast<const KzChunk*>(c.f->chunks)[seg.first_chunk + k];
  if (seg.num_chunks <= seg.chunk_cap) return reinterpret_cast<const KzChunk*>(seg.chunk_table)[k];
  const uint32_t lo = draw_of_chunk(c.draws, seg.first_draw, seg.num_draws, k);
  const KzDraw& d = c.draws[lo];
  KzChunk ch;
  ch.draw = lo;
  ch.first = (k - d.chunk_base) * KZ_CHUNK;
  ch.count = min((uint32_t)KZ_CHUNK, d.tri_count * d.instance_count - ch.first);
  ch.pad = 0;
  return ch;
}

__device__ void tri_vertices(const KzDraw& d, uint32_t local, uint32_t vid[3], uint32_t& iid) {
  /* one instance (the common case, warp-uniform): no division */
  const uint32_t inst = d.instance_count == 1 ? 0u : local / d.tri_count;
  const uint32_t t = local - inst * d.tri_count;
  iid = d.first_instance + inst;
  if (d.indexed == 1) {
    const uint32_t* ib = reinterpret_cast<const uint32_t*>(d.ib) + (size_t)3 * t;
    for (int j = 0; j < 3; j++) vid[j] = __ldg(ib + j) + (uint32_t)d.vertex_offset;
  } else if (d.indexed == 2) {
    const uint16_t* ib = reinterpret_cast<const uint16_t*>(d.ib) + (size_t)3 * t;
    for (int j = 0; j < 3; j++) vid[j] = (uint32_t)__ldg(ib + j) + (uint32_t)d.vertex_offset;
  } else {
    for (int j = 0; j < 3; j++) vid[j] = (uint32_t)d.vertex_offset + 3u * t + (uint32_t)j;
  }
}

/* ---------------- clipping ---------------- */

__device__ __forceinline__ float plane_dist(const float* p, int plane) {
  switch (plane) {
    case 0: return p[2];
    case 1: return fsub(p[3], p[2]);
    case 2: return fadd(p[0], fmul(KZ_GUARD_BAND, p[3]));
    case 3: return fsub(fmul(KZ_GUARD_BAND, p[3]), p[0]);
    case 4: return fadd(p[1], fmul(KZ_GUARD_BAND, p[3]));
    default: return fsub(fmul(KZ_GUARD_BAND, p[3]), p[1]);
  }
}

/* 0: reject, 1: inside the guard band, 2: needs clipping */
__device__ int classify(const float pos[3][4]) {
  bool all[6] = {true, true, true, true, true, true};
#pragma unroll
  for (int j = 0; j < 3; j++) {
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (!isfinite(pos[j][k])) return 0;
    const float* c = pos[j];
    all[0] &= c[0] > c[3];
    all[1] &= c[0] < -c[3];
    all[2] &= c[1] > c[3];
    all[3] &= c[1] < -c[3];
    all[4] &= c[2] < 0.0f;
    all[5] &= c[2] > c[3];
  }
  if (all[0] | all[1] | all[2] | all[3] | all[4] | all[5]) return 0;
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int plane = 0; plane < 6; plane++)
      if (plane_dist(pos[j], plane) < 0.0f) return 2;
  return 1;
}

struct ClipV {
  float c[4 + KZ_MAX_VARYINGS];
};

/* Sutherland-Hodgman against z>=0, z<=w, |x|,|y|<=4w; nc varyings ride along.  Returns the polygon
 * size (0 = rejected). */
__device__ __noinline__ int clip_polygon(ClipV* a, int nc) {
  ClipV b[KZ_MAX_CLIP_VERTS];
  int n = 3;
  ClipV* cur = a;
  ClipV* nxt = b;
  for (int plane = 0; plane < 6; plane++) {
    bool any_out = false;
    for (int i = 0; i < n; i++)
      if (plane_dist(cur[i].c, plane) < 0.0f) any_out = true;
    if (!any_out) continue;
    int m = 0;
    for (int i = 0; i < n; i++) {
      const ClipV& p = cur[i];
      const ClipV& q = cur[(i + 1) % n];
      float dp = plane_dist(p.c, plane), dq = plane_dist(q.c, plane);
      bool pin = dp >= 0.0f, qin = dq >= 0.0f;
      if (pin) nxt[m++] = p;
      if (pin != qin) {
        const ClipV& vi = pin ? p : q;
        const ClipV& vo = pin ? q : p;
        float di = pin ? dp : dq, dout = pin ? dq : dp;
        float t = fdiv(di, fsub(di, dout));
        ClipV c;
        for (int k = 0; k < 4 + nc; k++) c.c[k] = ffma(t, fsub(vo.c[k], vi.c[k]), vi.c[k]);
        nxt[m++] = c;
      }
    }
    n = m;
    ClipV* tmp = cur;
    cur = nxt;
    nxt = tmp;
    if (n < 3) return 0;
  }
  for (int i = 0; i < n; i++) {
    if (!(cur[i].c[3] > 0.0f)) return 0;
    if (cur != a) a[i] = cur[i];
  }
  return n;
}

/* ---------------- triangle setup ---------------- */

struct Proj {
  int32_t X, Y;
  float z, iw;
};

__device__ __forceinline__ Proj project(const KzDraw& d, const float* c) {
  Proj p;
  float iw = fdiv(1.0f, c[3]);
  float xd = fmul(c[0], iw), yd = fmul(c[1], iw), zd = fmul(c[2], iw);
  float xf = ffma(xd, d.hx, d.ox), yf = ffma(yd, d.hy, d.oy);
  p.z = ffma(zd, d.pz, d.oz);
  p.X = __float2int_rn(fmul(xf, 256.0f));
  p.Y = __float2int_rn(fmul(yf, 256.0f));
  p.iw = iw;
  return p;
}

/* Fills the coverage/depth record from three projected vertices; returns false when the triangle can
 * produce no fragment (degenerate, culled, or no pixel centre in its box). */
__device__ __forceinline__ bool make_record(const KzDraw& d, const KzPipe& pp, Proj v[3], KzTriRecord& r, bool& swapped) {
  int64_t S = (int64_t)(v[1].X - v[0].X) * (v[2].Y - v[0].Y) - (int64_t)(v[2].X - v[0].X) * (v[1].Y - v[0].Y);
  if (S == 0) return false;
  bool front = pp.front_ccw ? (S < 0) : (S > 0);
  if (((pp.cull_mode & 2u) && !front) || ((pp.cull_mode & 1u) && front)) return false;
  swapped = S < 0;
  if (swapped) {
    Proj t = v[1];
    v[1] = v[2];
    v[2] = t;
    S = -S;
  }
  int32_t minx = min(v[0].X, min(v[1].X, v[2].X)), maxx = max(v[0].X, max(v[1].X, v[2].X));
  int32_t miny = min(v[0].Y, min(v[1].Y, v[2].Y)), maxy = max(v[0].Y, max(v[1].Y, v[2].Y));
  /* pixels with a sample point (p * 256 + o, o = 128, or KZ_MS_LO..KZ_MS_HI when multisampled) in
   * [min, max]: ceil((min - hi) / 256) .. floor((max - lo) / 256); snapped coordinates stay within the
   * guard band (|X| < 2^23), so 32-bit arithmetic shifts are exact */
  const int32_t lo = d.samples > 1 ? KZ_MS_LO : 128, hi = d.samples > 1 ? KZ_MS_HI : 128;
  int32_t bx0 = (minx - hi + 255) >> 8;
  int32_t by0 = (miny - hi + 255) >> 8;
  int32_t bx1 = (maxx - lo) >> 8;
  int32_t by1 = (maxy - lo) >> 8;
  if (bx0 < d.rect[0]) bx0 = d.rect[0];
  if (by0 < d.rect[1]) by0 = d.rect[1];
  if (bx1 > d.rect[2] - 1) bx1 = d.rect[2] - 1;
  if (by1 > d.rect[3] - 1) by1 = d.rect[3] - 1;
  if (bx0 > bx1 || by0 > by1) return false;
  uint32_t info = 0;
#pragma unroll
  for (int e = 0; e < 3; e++) {
    int a = (e + 1) % 3, b = (e + 2) % 3;
    int32_t dx = v[b].X - v[a].X, dy = v[b].Y - v[a].Y;
    if ((dy < 0) || (dy == 0 && dx > 0)) info |= 1u << e;
  }
  if (swapped) info |= 8u;
  if (front) info |= 256u;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    r.x[i] = v[i].X;
    r.y[i] = v[i].Y;
  }
  r.z0 = v[0].z;
  r.dz1 = fsub(v[1].z, v[0].z);
  r.dz2 = fsub(v[2].z, v[0].z);
  r.inv_s = fdiv(1.0f, kz_i64_to_f32(S));
  r.info = info;
  r.bb0 = (uint32_t)bx0 | ((uint32_t)by0 << 16);
  r.bb1 = (uint32_t)bx1 | ((uint32_t)by1 << 16);
  return true;
}

/* edge e of a record is v(e+1) -> v(e+2); E_e(p) = dx (py - ya) - dy (px - xa) */
struct Edges {
  int32_t dx[3], dy[3], xa[3], ya[3];
  int64_t thr[3];
};

__device__ __forceinline__ void edges_of(const KzTriRecord& r, Edges& e) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    int a = (k + 1) % 3, b = (k + 2) % 3;
    e.dx[k] = r.x[b] - r.x[a];
    e.dy[k] = r.y[b] - r.y[a];
    e.xa[k] = r.x[a];
    e.ya[k] = r.y[a];
    e.thr[k] = ((r.info >> k) & 1u) ? 0 : 1;
  }
}

__device__ __forceinline__ int64_t edge_at(const Edges& e, int k, int64_t px, int64_t py) {
  return (int64_t)e.dx[k] * (py - e.ya[k]) - (int64_t)e.dy[k] * (px - e.xa[k]);
}

/* ---------------- full setup for shading ---------------- */

struct Shade {
  KzTriRecord r;      /* coverage + depth */
  float iw[3];
  float a[3][KZ_MAX_VARYINGS];
  uint32_t pipe;
  uint32_t draw;
  uint32_t ok;
};

__device__ __forceinline__ void vs_full(const Ctx& c, const KzDraw& d, const KzPipe&, uint32_t vid, uint32_t iid,
                                        KzVsOut& o) {
  kz_vs(d.pipe, &d, vid, iid, push_ptr(*c.f, d), &o);
}

/* Build the shading setup of a (sub-)triangle from three full vertices (clip position + varyings). */
__device__ bool shade_from_vertices(const KzDraw& d, const KzPipe& p, const ClipV* v, int nc, Shade& s) {
  Proj pr[3];
  for (int i = 0; i < 3; i++) pr[i] = project(d, v[i].c);
  bool swapped = false;
  if (!make_record(d, p, pr, s.r, swapped)) return false;
  int order[3] = {0, swapped ? 2 : 1, swapped ? 1 : 2};
  for (int i = 0; i < 3; i++) {
    const ClipV& src = v[order[i]];
    float iw = fdiv(1.0f, src.c[3]);
    s.iw[i] = iw;
    for (int k = 0; k < nc; k++) {
      float val = src.c[4 + k];
      bool flat = (p.flat_mask >> k) & 1u;
      if (flat) val = v[0].c[4 + k];
      s.a[i][k] = (flat || ((p.noperspective_mask >> k) & 1u)) ? val : fmul(val, iw);
    }
  }
  return true;
}

/* True if pixel (x, y) is covered by the record. */
__device__ __forceinline__ bool covers(const KzTriRecord& r, int32_t x, int32_t y, int64_t E[3]) {
  Edges e;
  edges_of(r, e);
  int64_t px = (int64_t)x * 256 + 128, py = (int64_t)y * 256 + 128;
  bool in = true;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    E[k] = edge_at(e, k, px, py);
    in &= E[k] >= e.thr[k];
  }
  return in;
}

/* clipped primitive: redo the clip with varyings and pick the sub-triangle (by index, or by coverage
 * of pixel (x, y) when sub == 0) */
__device__ __noinline__ bool shade_clipped(const KzDraw& d, const KzPipe& p, const KzVsOut* o, int nc, int32_t x,
                                           int32_t y, uint32_t sub, Shade& s) {
  ClipV v[KZ_MAX_CLIP_VERTS];
  for (int j = 0; j < 3; j++) {
    for (int k = 0; k < 4; k++) v[j].c[k] = o[j].pos[k];
    for (int k = 0; k < nc; k++) v[j].c[4 + k] = o[j].var[k];
  }
  ClipV v0 = v[0];
  int n = clip_polygon(v, nc);
  for (int i = 0; i < n; i++)
    for (int k = 0; k < nc; k++)
      if ((p.flat_mask >> k) & 1u) v[i].c[4 + k] = v0.c[4 + k];
  for (int i = 1; i + 1 < n; i++) {
    if (sub != 0 && (uint32_t)i != sub) continue;
    ClipV tri[3] = {v[0], v[i], v[i + 1]};
    if (!shade_from_vertices(d, p, tri, nc, s)) continue;
    if (sub != 0) return true;
    int64_t E[3];
    if (covers(s.r, x, y, E)) return true;
  }
  return false;
}

/* setup of an unclipped triangle straight from the vertex-shader outputs */
__device__ __forceinline__ bool shade_direct(const KzDraw& d, const KzPipe& p, const KzVsOut* o, int nc, Shade& s) {
  Proj pr[3];
  for (int i = 0; i < 3; i++) pr[i] = project(d, o[i].pos);
  bool swapped = false;
  if (!make_record(d, p, pr, s.r, swapped)) return false;
  int order[3] = {0, swapped ? 2 : 1, swapped ? 1 : 2};
  for (int i = 0; i < 3; i++) {
    const KzVsOut& src = o[order[i]];
    float iw = fdiv(1.0f, src.pos[3]);
    s.iw[i] = iw;
    for (int k = 0; k < nc; k++) {
      bool flat = (p.flat_mask >> k) & 1u;
      float val = flat ? o[0].var[k] : src.var[k];
      s.a[i][k] = (flat || ((p.noperspective_mask >> k) & 1u)) ? val : fmul(val, iw);
    }
  }
  return true;
}

/* Recompute primitive g of the segment for shading at pixel (x, y) (sub-triangle chosen by coverage
 * when the primitive was clipped, or by `sub` when it is known: sub = clip sub-index, 0 = any). */
__device__ bool shade_setup(const Ctx& c, uint32_t g, int32_t x, int32_t y, uint32_t sub, Shade& s) {
  const KzSegment& seg = *c.seg;
  uint32_t di;
  if (seg.draw_lut) {
    /* the draw holding primitive 256 (g / 256), then forward to the draw holding g */
    di = __ldg(reinterpret_cast<const uint32_t*>(seg.draw_lut) + (g >> 8));
    while (di + 1 < seg.first_draw + seg.num_draws && c.draws[di + 1].prim_base <= g) di++;
  } else {
    di = find_draw(c.draws, seg.first_draw, seg.num_draws, g);
  }
  const KzDraw& d = c.draws[di];
  const KzPipe& p = c.pipes[d.pipe];
  uint32_t vid[3], iid;
  tri_vertices(d, g - d.prim_base, vid, iid);
  int nc = (int)p.num_varyings;
  KzVsOut o[3];
  for (int j = 0; j < 3; j++) vs_full(c, d, p, vid[j], iid, o[j]);
  s.pipe = d.pipe;
  s.draw = di;
  float pos[3][4];
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 4; k++) pos[j][k] = o[j].pos[k];
  int cls = classify(pos);
  if (cls == 0) return false;
  if (cls == 1) return shade_direct(d, p, o, nc, s);
  return shade_clipped(d, p, o, nc, x, y, sub, s);
}

/* interpolate varyings and run the fragment shader.  REGS: pass the inputs in registers (kz_fs_r8) when
 * the interface has at most 8 varyings; otherwise through a KzFsIn in local memory (kz_fs), which costs
 * fewer registers in kernels that are already at their register limit.  CALLS false: the caller knows that
 * every pipeline of the segment has no fragment shader or one that only copies varyings 0..3 to the colour,
 * so no shader function is called (and none of the call's register saving is compiled in). */
template <bool REGS, bool CALLS = true>
__device__ __forceinline__ uint32_t shade_pixel(const Ctx& c, const Shade& s, int32_t x, int32_t y, const int64_t E[3],
                                                float z, float col[4]) {
  const KzPipe& p = c.pipes[s.pipe];
  const KzDraw& d = c.draws[s.draw];
  float l0 = fmul(kz_i64_to_f32(E[0]), s.r.inv_s);
  float l1 = fmul(kz_i64_to_f32(E[1]), s.r.inv_s);
  float l2 = fmul(kz_i64_to_f32(E[2]), s.r.inv_s);
  float q = ffma(l2, s.iw[2], ffma(l1, s.iw[1], fmul(l0, s.iw[0])));
  float rq = fdiv(1.0f, q);
  const int nc = (int)p.num_varyings;
  const float fx = fadd((float)x, 0.5f), fy = fadd((float)y, 0.5f);
  const uint32_t front = (s.r.info >> 8) & 1u;
  if (!p.has_fs) {
    col[0] = col[1] = col[2] = col[3] = 0.0f;
    return 0;
  }
  if (!CALLS || p.fs_passthrough) {
    /* the shader only copies varyings 0..3 to the colour: the same values without the call */
#pragma unroll
    for (int k = 0; k < 4; k++) {
      float num = ffma(l2, s.a[2][k], ffma(l1, s.a[1][k], fmul(l0, s.a[0][k])));
      const bool flat = (p.flat_mask >> k) & 1u;
      float val = ((p.noperspective_mask >> k) & 1u) || flat ? num : fmul(num, rq);
      if (flat) val = s.a[0][k];
      col[k] = val;
    }
    return 0;
  }
  if (REGS && nc <= 8) {
    uint32_t v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      float val = 0.0f;
      if (k < nc) {
        float num = ffma(l2, s.a[2][k], ffma(l1, s.a[1][k], fmul(l0, s.a[0][k])));
        const bool flat = (p.flat_mask >> k) & 1u;
        val = ((p.noperspective_mask >> k) & 1u) || flat ? num : fmul(num, rq);
        if (flat) val = s.a[0][k];
      }
      v[k] = __float_as_uint(val);
    }
    const KzFsResult rr = kz_fs_r8(s.pipe, push_ptr(*c.f, d), v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7],
                                   __float_as_uint(fx), __float_as_uint(fy), __float_as_uint(z), __float_as_uint(q),
                                   front);
    col[0] = rr.c[0];
    col[1] = rr.c[1];
    col[2] = rr.c[2];
    col[3] = rr.c[3];
    return rr.discard;
  }
  KzFsIn in;
  for (int k = 0; k < nc; k++) {
    float num = ffma(l2, s.a[2][k], ffma(l1, s.a[1][k], fmul(l0, s.a[0][k])));
    in.var[k] = ((p.noperspective_mask >> k) & 1u) || ((p.flat_mask >> k) & 1u) ? num : fmul(num, rq);
    if ((p.flat_mask >> k) & 1u) in.var[k] = s.a[0][k];
  }
  in.frag_coord[0] = fx;
  in.frag_coord[1] = fy;
  in.frag_coord[2] = z;
  in.frag_coord[3] = q;
  in.front_facing = front;
  return kz_fs(s.pipe, &in, push_ptr(*c.f, d), col);
}

/* ---------------- fragment operations ---------------- */

__device__ __forceinline__ bool depth_cmp(uint32_t op, float z, float d) {
  switch (op) {
    case 0: return false;
    case 1: return z < d;
    case 2: return z == d;
    case 3: return z <= d;
    case 4: return z > d;
    case 5: return z != d;
    case 6: return z >= d;
    default: return true;
  }
}

__device__ float blend_factor(uint32_t f, int ch, const float s[4], const float dst[4], const float k[4]) {
  switch (f) {
    case 0: return 0.0f;
    case 1: return 1.0f;
    case 2: return s[ch];
    case 3: return fsub(1.0f, s[ch]);
    case 4: return dst[ch];
    case 5: return fsub(1.0f, dst[ch]);
    case 6: return s[3];
    case 7: return fsub(1.0f, s[3]);
    case 8: return dst[3];
    case 9: return fsub(1.0f, dst[3]);
    case 10: return k[ch];
    case 11: return fsub(1.0f, k[ch]);
    case 12: return k[3];
    case 13: return fsub(1.0f, k[3]);
    case 14: return ch < 3 ? fminf(s[3], fsub(1.0f, dst[3])) : 1.0f;
    default: return 0.0f;
  }
}

__device__ __forceinline__ float blend_op(uint32_t op, float s, float sf, float d, float df) {
  switch (op) {
    case 0: return ffma(s, sf, fmul(d, df));
    case 1: return ffma(s, sf, -fmul(d, df));
    case 2: return ffma(d, df, -fmul(s, sf));
    case 3: return fminf(s, d);
    default: return fmaxf(s, d);
  }
}

/* colour in attachment byte order -> RGBA channel order */
__device__ __forceinline__ uint32_t to_rgba(uint32_t px, uint32_t fmt) {
  if (cf_bgra(fmt)) return (px & 0xFF00FF00u) | ((px >> 16) & 0xFFu) | ((px & 0xFFu) << 16);
  return px;
}
__device__ __forceinline__ uint32_t from_rgba(uint32_t px, uint32_t fmt) { return to_rgba(px, fmt); }

/* apply blend + write mask; dst/out packed RGBA (R in the low byte).  `k`: the draw's blend constants
 * (clamped to [0, 1] at recording).  `u8tab`, when given, holds u8f(k) for k = 0..255 (the same quotients,
 * read instead of divided); `srgb`: the attachment is 8-bit sRGB. */
__device__ uint32_t color_write(const KzPipe& p, const float* k, uint32_t dst, const float col[4],
                                const float* u8tab = nullptr, bool srgb = false) {
  /* sRGB attachments: red, green and blue are decoded to linear before blending and encoded after */
  const float* thr = kz_srgb_thr_g;
  uint32_t out = dst;
  if (p.blend_enable) {
    const float* dec = kz_srgb_dec_g;
    float s[4], dd[4];
    for (int i = 0; i < 4; i++) {
      s[i] = fminf(fmaxf(col[i], 0.0f), 1.0f);
      uint32_t u = (dst >> (8 * i)) & 0xFFu;
      dd[i] = srgb && i < 3 ? dec[u] : (u8tab ? u8tab[u] : u8f(u));
    }
    for (int i = 0; i < 4; i++) {
      if (!((p.write_mask >> i) & 1u)) continue;
      float r;
      if (i < 3)
        r = blend_op(p.color_op, s[i], blend_factor(p.src_color, i, s, dd, k), dd[i],
                     blend_factor(p.dst_color, i, s, dd, k));
      else
        r = blend_op(p.alpha_op, s[3], blend_factor(p.src_alpha, 3, s, dd, k), dd[3],
                     blend_factor(p.dst_alpha, 3, s, dd, k));
      uint32_t b = srgb && i < 3 ? srgb8(r, thr) : (uint32_t)unorm8(r);
      out = (out & ~(0xFFu << (8 * i))) | (b << (8 * i));
    }
  } else {
    for (int i = 0; i < 4; i++) {
      if (!((p.write_mask >> i) & 1u)) continue;
      uint32_t b = srgb && i < 3 ? srgb8(col[i], thr) : (uint32_t)unorm8(col[i]);
      out = (out & ~(0xFFu << (8 * i))) | (b << (8 * i));
    }
  }
  return out;
}

/* ---------------- visibility keys ---------------- */

__device__ __forceinline__ unsigned long long vis_key(uint32_t mode, float z, uint32_t g) {
  uint32_t zb = __float_as_uint(z);
  switch (mode) {
    case KZ_VIS_LESS: return ((unsigned long long)zb << 32) | (g + 1u);
    case KZ_VIS_LEQUAL: return ((unsigned long long)zb << 32) | (0xFFFFFFFEu - g);
    case KZ_VIS_GREATER: return ((unsigned long long)(~zb) << 32) | (g + 1u);
    case KZ_VIS_GEQUAL: return ((unsigned long long)(~zb) << 32) | (0xFFFFFFFEu - g);
    default: return (unsigned long long)(0xFFFFFFFEu - g);
  }
}
__device__ __forceinline__ unsigned long long vis_init(uint32_t mode, float d) {
  uint32_t db = __float_as_uint(d);
  switch (mode) {
    case KZ_VIS_LESS: return (unsigned long long)db << 32;
    case KZ_VIS_LEQUAL: return ((unsigned long long)db << 32) | 0xFFFFFFFFull;
    case KZ_VIS_GREATER: return (unsigned long long)(~db) << 32;
    case KZ_VIS_GEQUAL: return ((unsigned long long)(~db) << 32) | 0xFFFFFFFFull;
    default: return 0xFFFFFFFFull;
  }
}
/* returns true and the primitive when the key holds a fragment */
__device__ __forceinline__ bool vis_decode(uint32_t mode, unsigned long long k, uint32_t& g, float& z) {
  uint32_t lo = (uint32_t)k, hi = (uint32_t)(k >> 32);
  bool frag;
  if (mode == KZ_VIS_LESS || mode == KZ_VIS_GREATER) {
    frag = lo != 0;
    g = lo - 1u;
  } else {
    frag = lo != 0xFFFFFFFFu;
    g = 0xFFFFFFFEu - lo;
  }
  z = (mode == KZ_VIS_GREATER || mode == KZ_VIS_GEQUAL) ? __uint_as_float(~hi) : __uint_as_float(hi);
  return frag;
}

/* ---------------- status ---------------- */

__device__ __forceinline__ uint32_t status_flags(const KzStatus* st) {
  return *reinterpret_cast<const volatile uint32_t*>(&st->flags);
}
/* Whether segment s must be skipped (a barrier gave up, or an earlier or this segment overflowed its
 * scratch).  Called by every thread of the block at once; the answer is the same for all of them: other
 * blocks may set the flags while this block reads them, and a block whose threads disagreed would leave some
 * of them waiting at a later __syncthreads for threads that have left. */
__device__ __forceinline__ bool segment_blocked(const Ctx& c, uint32_t s) {
  uint32_t f = status_flags(c.st);
  bool blocked = false;
  if (f & KZ_STATUS_BARRIER_TIMEOUT) blocked = true;
  else if (f & (KZ_STATUS_RECORD_OVERFLOW | KZ_STATUS_PAIR_OVERFLOW))
    blocked = *reinterpret_cast<const volatile uint32_t*>(&c.st->failed_segment) <= s;
  return __syncthreads_or(blocked ? 1 : 0) != 0;
}
__device__ void mark_failed(KzStatus* st, uint32_t bits, uint32_t s) {
  atomicMin(&st->failed_segment, s);
  atomicOr(&st->flags, bits);
}

/* ---------------- phase: geometry ---------------- */

__device__ __forceinline__ void tile_range(const KzSegment& seg, const KzTriRecord& r, int& tx0, int& ty0, int& tx1,
                                           int& ty1) {
  int T = (int)seg.tile;
  tx0 = (int)(r.bb0 & 0xFFFFu) / T;
  ty0 = (int)(r.bb0 >> 16) / T;
  tx1 = (int)(r.bb1 & 0xFFFFu) / T;
  ty1 = (int)(r.bb1 >> 16) / T;
}

/* Conservative test: can any sample point of tile (tx, ty) (pixel centres, or the 4x sample positions of
 * a multisampled pass) be inside the record's three edges? */
__device__ __forceinline__ bool tile_overlaps(const KzSegment& seg, const Edges& e, int tx, int ty) {
  int T = (int)seg.tile;
  const int64_t lo = seg.samples > 1 ? KZ_MS_LO : 128, hi = seg.samples > 1 ? KZ_MS_HI : 128;
  int64_t x0 = (int64_t)(tx * T) * 256 + lo, x1 = (int64_t)(tx * T + T - 1) * 256 + hi;
  int64_t y0 = (int64_t)(ty * T) * 256 + lo, y1 = (int64_t)(ty * T + T - 1) * 256 + hi;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    int64_t px = e.dy[k] < 0 ? x1 : x0; /* maximise -dy*px */
    int64_t py = e.dx[k] > 0 ? y1 : y0; /* maximise dx*py */
    if (edge_at(e, k, px, py) < e.thr[k]) return false;
  }
  return true;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

/* tile counts of a record; single-tile records (the common case) are aggregated per warp */
__device__ void count_tiles(const Ctx& c, const KzTriRecord& r, bool active) {
  const KzSegment& seg = *c.seg;
  int tx0 = 0, ty0 = 0, tx1 = -1, ty1 = -1;
  if (active) tile_range(seg, r, tx0, ty0, tx1, ty1);
  bool single = active && tx0 == tx1 && ty0 == ty1;
  uint32_t* tc = reinterpret_cast<uint32_t*>(seg.tile_count);
  uint32_t t = single ? (uint32_t)(ty0 * (int)seg.tiles_x + tx0) : 0xFFFFFFFFu;
  uint32_t peers = __match_any_sync(0xFFFFFFFFu, t);
  if (single && (__ffs(peers) - 1) == (int)(threadIdx.x & 31)) atomicAdd(&tc[t], (uint32_t)__popc(peers));
  if (!active || single) return;
  Edges e;
  edges_of(r, e);
  for (int ty = ty0; ty <= ty1; ty++)
    for (int tx = tx0; tx <= tx1; tx++)
      if (tile_overlaps(seg, e, tx, ty)) atomicAdd(&tc[ty * seg.tiles_x + tx], 1u);
}

__device__ void store_record(const Ctx& c, uint32_t idx, const KzTriRecord& r) {
  if (idx < c.seg->rec_cap) {
    KzTriRecord* dst = reinterpret_cast<KzTriRecord*>(c.seg->records) + idx;
    const uint4* s4 = reinterpret_cast<const uint4*>(&r);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    d4[0] = s4[0];
    d4[1] = s4[1];
    d4[2] = s4[2];
    d4[3] = s4[3];
  }
}

/* slow path (clipped primitives): one record at a time.  Its tile counts follow the rule bin_record places
 * the record by: a record whose box lies in one tile is counted there without the overlap test (as
 * count_tiles counts it); a count that missed a record its bin receives would spill into the next tile's bin */
__device__ void emit_record(const Ctx& c, KzTriRecord& r) {
  uint32_t idx = atomicAdd(&c.cnt->rec_count, 1u);
  store_record(c, idx, r);
  const KzSegment& seg = *c.seg;
  int tx0, ty0, tx1, ty1;
  tile_range(seg, r, tx0, ty0, tx1, ty1);
  uint32_t* tc = reinterpret_cast<uint32_t*>(seg.tile_count);
  if (tx0 == tx1 && ty0 == ty1) {
    atomicAdd(&tc[ty0 * seg.tiles_x + tx0], 1u);
    return;
  }
  Edges e;
  edges_of(r, e);
  for (int ty = ty0; ty <= ty1; ty++)
    for (int tx = tx0; tx <= tx1; tx++)
      if (tile_overlaps(seg, e, tx, ty)) atomicAdd(&tc[ty * seg.tiles_x + tx], 1u);
}

__device__ __noinline__ void geometry_clipped(const Ctx& c, const KzDraw& d, const KzPipe& p, float pos[3][4],
                                              uint32_t g, uint32_t di) {
  ClipV v[KZ_MAX_CLIP_VERTS];
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 4; k++) v[j].c[k] = pos[j][k];
  int n = clip_polygon(v, 0);
  for (int i = 1; i + 1 < n; i++) {
    Proj pr[3] = {project(d, v[0].c), project(d, v[i].c), project(d, v[i + 1].c)};
    KzTriRecord r;
    bool sw;
    if (!make_record(d, p, pr, r, sw)) continue;
    r.g = g;
    r.draw = di;
    r.pad = 0;
    r.info |= (uint32_t)i << 4;
    emit_record(c, r);
  }
}

/* returns true with the record of an unclipped visible triangle (and its vertex indices, instance and
 * whether setup swapped vertices 1 and 2); clipped triangles are emitted here */
__device__ bool geometry_triangle(const Ctx& c, uint32_t di, uint32_t local, KzTriRecord& r, uint32_t vid[3],
                                  uint32_t& iid, bool& sw) {
  const KzDraw& d = c.draws[di];
  const KzPipe& p = c.pipes[d.pipe];
  tri_vertices(d, local, vid, iid);
  float pos[3][4];
  const uint8_t* push = push_ptr(*c.f, d);
  for (int j = 0; j < 3; j++) {
    float4 q = kz_vs_pos(d.pipe, &d, vid[j], iid, push);
    pos[j][0] = q.x;
    pos[j][1] = q.y;
    pos[j][2] = q.z;
    pos[j][3] = q.w;
  }
  uint32_t g = d.prim_base + local;
  int cls = classify(pos);
  if (cls == 0) return false;
  if (cls == 2) {
    geometry_clipped(c, d, p, pos, g, di);
    return false;
  }
  Proj pr[3] = {project(d, pos[0]), project(d, pos[1]), project(d, pos[2])};
  if (!make_record(d, p, pr, r, sw)) return false;
  r.g = g;
  r.draw = di;
  r.pad = 0;
  return true;
}

/* the shading setup of an unclipped record, stored beside it once so that the tiles it overlaps do not
 * recompute it: full vertex shader of its three vertices, then what shade_direct computes */
__device__ void write_shade(const Ctx& c, uint32_t idx, uint32_t di, const uint32_t vid[3], uint32_t iid, bool swapped) {
  const KzSegment& seg = *c.seg;
  if (idx >= seg.rec_cap || !seg.shades) return;
  const KzDraw& d = c.draws[di];
  const KzPipe& p = c.pipes[d.pipe];
  KzVsOut o[3];
  for (int j = 0; j < 3; j++) vs_full(c, d, p, vid[j], iid, o[j]);
  float* dst = reinterpret_cast<float*>(seg.shades + (size_t)idx * seg.shade_stride);
  const int nc = (int)p.num_varyings;
  const int order[3] = {0, swapped ? 2 : 1, swapped ? 1 : 2};
  for (int i = 0; i < 3; i++) {
    const KzVsOut& src = o[order[i]];
    float iw = fdiv(1.0f, src.pos[3]);
    dst[i] = iw;
    for (int k = 0; k < nc; k++) {
      bool flat = (p.flat_mask >> k) & 1u;
      float val = flat ? o[0].var[k] : src.var[k];
      dst[4 + i * nc + k] = (flat || ((p.noperspective_mask >> k) & 1u)) ? val : fmul(val, iw);
    }
  }
}

/* one chunk per block: records are allocated with one atomic per block */
__device__ void geometry_chunk(const Ctx& c, uint32_t chunk, uint32_t* sh) {
  const KzChunk ch = chunk_at(c, chunk);
  KzTriRecord r;
  bool have = false, sw = false;
  uint32_t vid[3] = {0, 0, 0}, iid = 0;
  if (threadIdx.x < ch.count) have = geometry_triangle(c, ch.draw, ch.first + threadIdx.x, r, vid, iid, sw);
  uint32_t ballot = __ballot_sync(0xFFFFFFFFu, have);
  uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[warp] = (uint32_t)__popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (uint32_t w = 0; w < (blockDim.x >> 5); w++) {
      uint32_t v = sh[w];
      sh[w] = run;
      run += v;
    }
    sh[32] = run ? atomicAdd(&c.cnt->rec_count, run) : 0u;
  }
  __syncthreads();
  uint32_t idx = sh[32] + sh[warp] + (uint32_t)__popc(ballot & lanemask_lt());
  if (have) {
    store_record(c, idx, r);
    write_shade(c, idx, ch.draw, vid, iid, sw);
  }
  count_tiles(c, r, have);
  __syncthreads();
}

/* ---------------- phase: scan (one block) ---------------- */

__device__ void scan_tiles(const Ctx& c, uint32_t s, uint32_t* sh) {
  const KzSegment& seg = *c.seg;
  uint32_t n = seg.tiles_x * seg.tiles_y;
  const uint32_t* tc = reinterpret_cast<const uint32_t*>(seg.tile_count);
  uint32_t* to = reinterpret_cast<uint32_t*>(seg.tile_offset);
  uint32_t* cur = reinterpret_cast<uint32_t*>(seg.tile_cursor);
  uint32_t* order = reinterpret_cast<uint32_t*>(seg.tile_order);
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  /* sh: [0, 32) per-warp sums, [32, 65) the order's buckets (floor(log2(bin size)) + 1, empty bins 0),
   * [blockDim.x] the running total */
  uint32_t* wsum = sh;
  uint32_t* hist = sh + 32;
  if (threadIdx.x <= 32) hist[threadIdx.x] = 0;
  if (threadIdx.x == 0) sh[blockDim.x] = 0;
  __syncthreads();
  /* exclusive prefix of the counts, blockDim.x tiles at a time (coalesced), with a warp-shuffle scan */
  uint32_t mx = 0;
  for (uint32_t base = 0; base < n; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < n ? tc[i] : 0u;
    mx = max(mx, v);
    if (i < n && order) atomicAdd(&hist[32 - __clz(v)], 1u);
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      uint32_t w = lane < nw ? wsum[lane] : 0u, wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
        if (lane >= (uint32_t)o) wi += t;
      }
      if (lane < nw) wsum[lane] = wi - w; /* exclusive per warp */
    }
    __syncthreads();
    const uint32_t carry = sh[blockDim.x];
    if (i < n) {
      to[i] = carry + wsum[wid] + incl - v;
      cur[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) sh[blockDim.x] = carry + wsum[wid] + incl;
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
  if (lane == 0) atomicMax(&c.cnt->max_bin, mx);
  /* the raster's tile order: by decreasing bucket, empty bins last, so that the largest bins start first
   * and the raster kernel's tail is made of small ones */
  if (order) {
    if (threadIdx.x == 0) {
      uint32_t at = 0;
      for (int k = 32; k >= 0; k--) {
        const uint32_t v = hist[k];
        hist[k] = at;
        at += v;
      }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) order[atomicAdd(&hist[32 - __clz(tc[i])], 1u)] = i;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t pairs = sh[blockDim.x];
    to[n] = pairs;
    c.cnt->pair_count = pairs;
    uint32_t recs = c.cnt->rec_count;
    uint32_t bits = 0;
    if (recs > seg.rec_cap) bits |= KZ_STATUS_RECORD_OVERFLOW;
    if (pairs > seg.pair_cap) bits |= KZ_STATUS_PAIR_OVERFLOW;
    atomicMax(&c.st->need_records, recs);
    atomicMax(&c.st->need_pairs, pairs);
    if (bits) mark_failed(c.st, bits, s);
    __threadfence();
  }
  __syncthreads();
}

/* ---------------- phase: bin ---------------- */

__device__ void bin_record(const Ctx& c, uint32_t ri, bool active) {
  const KzSegment& seg = *c.seg;
  KzTriRecord r;
  int tx0 = 0, ty0 = 0, tx1 = -1, ty1 = -1;
  if (active) {
    r = reinterpret_cast<const KzTriRecord*>(seg.records)[ri];
    tile_range(seg, r, tx0, ty0, tx1, ty1);
  }
  const uint32_t* to = reinterpret_cast<const uint32_t*>(seg.tile_offset);
  uint32_t* cur = reinterpret_cast<uint32_t*>(seg.tile_cursor);
  uint32_t* bins = reinterpret_cast<uint32_t*>(seg.bins);
  bool single = active && tx0 == tx1 && ty0 == ty1;
  uint32_t t = single ? (uint32_t)(ty0 * (int)seg.tiles_x + tx0) : 0xFFFFFFFFu;
  uint32_t peers = __match_any_sync(0xFFFFFFFFu, t);
  int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (single && leader == (int)(threadIdx.x & 31)) base = to[t] + atomicAdd(&cur[t], (uint32_t)__popc(peers));
  base = __shfl_sync(0xFFFFFFFFu, base, leader);
  /* every write stays inside its tile's bin [to[t], to[t + 1]) (the counts and this placement follow one rule,
   * so none is dropped; the bound keeps a miscount from reaching another tile's bin or past the buffer) */
  if (single) {
    const uint32_t pos = base + (uint32_t)__popc(peers & lanemask_lt());
    if (pos < to[t + 1]) bins[pos] = ri;
  }
  if (!active || single) return;
  Edges e;
  edges_of(r, e);
  for (int ty = ty0; ty <= ty1; ty++)
    for (int tx = tx0; tx <= tx1; tx++)
      if (tile_overlaps(seg, e, tx, ty)) {
        uint32_t tt = ty * seg.tiles_x + tx;
        const uint32_t pos = to[tt] + atomicAdd(&cur[tt], 1u);
        if (pos < to[tt + 1]) bins[pos] = ri;
      }
}

/* ---------------- phase: raster ---------------- */

__device__ __forceinline__ KzTriRecord load_record(const KzSegment& seg, uint32_t ri) {
  const uint4* src = reinterpret_cast<const uint4*>(reinterpret_cast<const KzTriRecord*>(seg.records) + ri);
  KzTriRecord r;
  uint4* d = reinterpret_cast<uint4*>(&r);
  d[0] = __ldg(src);
  d[1] = __ldg(src + 1);
  d[2] = __ldg(src + 2);
  d[3] = __ldg(src + 3);
  return r;
}

struct TileInfo {
  int32_t x0, y0, x1, y1; /* inclusive pixel bounds of the tile inside the framebuffer and render area */
  int32_t ox, oy;         /* tile origin */
  uint32_t n, base;
};

__device__ __forceinline__ bool tile_info(const KzSegment& seg, uint32_t t, TileInfo& ti) {
  int T = (int)seg.tile;
  ti.ox = (int32_t)(t % seg.tiles_x) * T;
  ti.oy = (int32_t)(t / seg.tiles_x) * T;
  ti.x0 = max(ti.ox, seg.area[0]);
  ti.y0 = max(ti.oy, seg.area[1]);
  ti.x1 = min(ti.ox + T, min((int32_t)seg.width, seg.area[2])) - 1;
  ti.y1 = min(ti.oy + T, min((int32_t)seg.height, seg.area[3])) - 1;
  ti.n = reinterpret_cast<const uint32_t*>(seg.tile_count)[t];
  ti.base = reinterpret_cast<const uint32_t*>(seg.tile_offset)[t];
  return ti.x0 <= ti.x1 && ti.y0 <= ti.y1;
}

__device__ __forceinline__ uint32_t* color_px(const KzSegment& seg, int32_t x, int32_t y) {
  return reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(seg.color) + (size_t)y * seg.color_pitch) + x;
}
__device__ __forceinline__ float* depth_px(const KzSegment& seg, int32_t x, int32_t y) {
  return reinterpret_cast<float*>(reinterpret_cast<char*>(seg.depth) + (size_t)y * seg.depth_pitch) + x;
}

/* the depth texel at (x, y) as the depth test compares it (D32: the float; D16 / D24: the integer in a
 * float), and the stencil value of a D24S8 texel */
__device__ __forceinline__ float load_depth(const KzSegment& seg, int32_t x, int32_t y, uint32_t& stencil) {
  const char* row = reinterpret_cast<const char*>(seg.depth) + (size_t)y * seg.depth_pitch;
  stencil = 0;
  if (seg.depth_format == KZ_DF_D16) return (float)reinterpret_cast<const uint16_t*>(row)[x];
  if (seg.depth_format == KZ_DF_D24S8) {
    uint32_t w = reinterpret_cast<const uint32_t*>(row)[x];
    stencil = w >> 24;
    return (float)(w & 0xFFFFFFu);
  }
  return reinterpret_cast<const float*>(row)[x];
}

__device__ __forceinline__ void store_depth(const KzSegment& seg, int32_t x, int32_t y, float d, uint32_t stencil) {
  char* row = reinterpret_cast<char*>(seg.depth) + (size_t)y * seg.depth_pitch;
  if (seg.depth_format == KZ_DF_D16) reinterpret_cast<uint16_t*>(row)[x] = (uint16_t)d;
  else if (seg.depth_format == KZ_DF_D24S8) reinterpret_cast<uint32_t*>(row)[x] = (uint32_t)d | (stencil << 24);
  else reinterpret_cast<float*>(row)[x] = d;
}

/* a fragment depth z in [0, 1] as the depth format compares and stores it: rint(z * (2^bits - 1)) for
 * D16 / D24 (the product a correctly rounded single), z itself for D32 */
__device__ __forceinline__ float depth_value(float z, uint32_t format) {
  if (format == KZ_DF_D16) return rintf(fmul(z, 65535.0f));
  if (format == KZ_DF_D24S8) return rintf(fmul(z, 16777215.0f));
  return z;
}

/* the stencil test: reference OP stored, both under the compare mask (VkCompareOp) */
__device__ __forceinline__ bool stencil_cmp(uint32_t op, uint32_t ref, uint32_t val) {
  switch (op) {
    case 0: return false;
    case 1: return ref < val;
    case 2: return ref == val;
    case 3: return ref <= val;
    case 4: return ref > val;
    case 5: return ref != val;
    case 6: return ref >= val;
    default: return true;
  }
}

/* VkStencilOp `op` on stored value s through the write mask; w1 = compareMask | writeMask << 8 |
 * reference << 16 */
__device__ __forceinline__ uint32_t stencil_apply(uint32_t op, uint32_t s, uint32_t w1) {
  uint32_t v;
  switch (op) {
    case 1: v = 0; break;
    case 2: v = (w1 >> 16) & 0xFFu; break;
    case 3: v = s < 255u ? s + 1u : 255u; break;
    case 4: v = s > 0u ? s - 1u : 0u; break;
    case 5: v = ~s & 0xFFu; break;
    case 6: v = (s + 1u) & 0xFFu; break;
    case 7: v = (s - 1u) & 0xFFu; break;
    default: v = s; break;
  }
  uint32_t wm = (w1 >> 8) & 0xFFu;
  return (s & ~wm) | (v & wm);
}

/* ================= visibility-buffer path (opaque segments) ================= */

#define KZ_SMALL_PX 32      /* clipped sub-triangles with boxes of at most this many pixels are rasterised by
                               their geometry thread */
/* KzFrame::warp_px: unclipped triangles with boxes of at most this many pixels are rasterised by their
 * geometry warp (vis_warp_raster), larger ones become jobs of KzFrame::job_blocks 8x8 blocks (1..32: one lane
 * per block); both are set per command buffer (the autotuner's knobs) */
__device__ __forceinline__ uint32_t job_blocks(const Ctx& c) { return min(max(c.f->job_blocks, 1u), 32u); }

__device__ __forceinline__ unsigned long long* vis_px(const KzSegment& seg, int32_t x, int32_t y) {
  return reinterpret_cast<unsigned long long*>(seg.vis) + (size_t)y * seg.width + x;
}

/* keep the smaller key: a fire-and-forget 64-bit min reduction at L2 (the result is unused, so the
 * issuing thread never waits for it) */
__device__ __forceinline__ void vis_store(const KzSegment& seg, unsigned long long k, int32_t x, int32_t y) {
  atomicMin(vis_px(seg, x, y), k);
}

__device__ __forceinline__ unsigned long long frag_key(const KzSegment& seg, const KzTriRecord& r, float zmin,
                                                       float zmax, float fE1, float fE2) {
  float l1 = fmul(fE1, r.inv_s), l2 = fmul(fE2, r.inv_s);
  float z = ffma(l2, r.dz2, ffma(l1, r.dz1, r.z0));
  z = fadd(fminf(fmaxf(z, zmin), zmax), 0.0f);
  return vis_key(seg.vis_key, z, r.g);
}

/* rasterise a small record (box of at most KZ_SMALL_PX pixels) into the keys, one thread */
__device__ uint32_t vis_small(const KzSegment& seg, const KzTriRecord& r, float zmin, float zmax) {
  int32_t bx0 = (int32_t)(r.bb0 & 0xFFFFu), by0 = (int32_t)(r.bb0 >> 16);
  int32_t bx1 = (int32_t)(r.bb1 & 0xFFFFu), by1 = (int32_t)(r.bb1 >> 16);
  int32_t ox = bx0 * 256 + 128, oy = by0 * 256 + 128;
  int32_t xr[3], yr[3];
  bool near = true;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    xr[i] = r.x[i] - ox;
    yr[i] = r.y[i] - oy;
    near &= (xr[i] > -8192 && xr[i] < 8192 && yr[i] > -8192 && yr[i] < 8192);
  }
  uint32_t frags = 0;
  if (near) {
    /* every vertex and pixel centre lies within 32 pixels of the box origin: each product of the edge
     * function is below 2^28, so 32-bit arithmetic is exact (same integers as the 64-bit form) */
    int32_t dx[3], dy[3], xa[3], ya[3], thr[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      int a = (k + 1) % 3, b = (k + 2) % 3;
      dx[k] = xr[b] - xr[a];
      dy[k] = yr[b] - yr[a];
      xa[k] = xr[a];
      ya[k] = yr[a];
      thr[k] = ((r.info >> k) & 1u) ? 0 : 1;
    }
    for (int32_t y = by0; y <= by1; y++) {
      int32_t py = (y - by0) * 256;
      int32_t E0 = dx[0] * (py - ya[0]) + dy[0] * xa[0];
      int32_t E1 = dx[1] * (py - ya[1]) + dy[1] * xa[1];
      int32_t E2 = dx[2] * (py - ya[2]) + dy[2] * xa[2];
      for (int32_t x = bx0; x <= bx1; x++) {
        if (E0 >= thr[0] && E1 >= thr[1] && E2 >= thr[2]) {
          frags++;
          vis_store(seg, frag_key(seg, r, zmin, zmax, __int2float_rn(E1), __int2float_rn(E2)), x, y);
        }
        E0 -= dy[0] * 256;
        E1 -= dy[1] * 256;
        E2 -= dy[2] * 256;
      }
    }
    return frags;
  }
  Edges e;
  edges_of(r, e);
  int64_t px0 = (int64_t)bx0 * 256 + 128;
  for (int32_t y = by0; y <= by1; y++) {
    int64_t py = (int64_t)y * 256 + 128;
    int64_t E0 = edge_at(e, 0, px0, py), E1 = edge_at(e, 1, px0, py), E2 = edge_at(e, 2, px0, py);
    for (int32_t x = bx0; x <= bx1; x++) {
      if (E0 >= e.thr[0] && E1 >= e.thr[1] && E2 >= e.thr[2]) {
        frags++;
        vis_store(seg, frag_key(seg, r, zmin, zmax, kz_i64_to_f32(E1), kz_i64_to_f32(E2)), x, y);
      }
      E0 -= (int64_t)e.dy[0] * 256;
      E1 -= (int64_t)e.dy[1] * 256;
      E2 -= (int64_t)e.dy[2] * 256;
    }
  }
  return frags;
}

__device__ __forceinline__ uint32_t box_area(const KzTriRecord& r) {
  return ((r.bb1 & 0xFFFFu) - (r.bb0 & 0xFFFFu) + 1) * ((r.bb1 >> 16) - (r.bb0 >> 16) + 1);
}

__device__ __forceinline__ uint32_t box_blocks(const KzTriRecord& r, uint32_t& nbx) {
  nbx = ((r.bb1 & 0xFFFFu) - (r.bb0 & 0xFFFFu) + 8) / 8;
  uint32_t nby = ((r.bb1 >> 16) - (r.bb0 >> 16) + 8) / 8;
  return nbx * nby;
}

/* emit a large record and its jobs (job = record index, first block) */
__device__ void vis_emit_large(const Ctx& c, const KzTriRecord& r) {
  uint32_t idx = atomicAdd(&c.cnt->rec_count, 1u);
  store_record(c, idx, r);
  uint32_t nbx, nb = box_blocks(r, nbx);
  const uint32_t jb = job_blocks(c);
  uint32_t njobs = (nb + jb - 1) / jb;
  uint32_t j0 = atomicAdd(&c.cnt->pair_count, njobs);
  uint32_t cap = c.seg->pair_cap / 2;
  if (idx >= c.seg->rec_cap) return;
  uint2* jobs = reinterpret_cast<uint2*>(c.seg->bins);
  for (uint32_t j = 0; j < njobs && j0 + j < cap; j++) jobs[j0 + j] = make_uint2(idx, j * jb);
}

/* emit the records of the lanes where `large` holds (their boxes exceed warp_px pixels) with one
 * record and one job reservation for the whole warp (all lanes call it) */
__device__ __forceinline__ void vis_emit_large_warp(const Ctx& c, const KzTriRecord& r, bool large) {
  const uint32_t m = __ballot_sync(0xFFFFFFFFu, large);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const uint32_t jb = job_blocks(c);
  uint32_t nbx = 0, njobs = 0;
  if (large) njobs = (box_blocks(r, nbx) + jb - 1) / jb;
  uint32_t jincl = njobs;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xFFFFFFFFu, jincl, o);
    if (lane >= o) jincl += t;
  }
  const uint32_t jtotal = __shfl_sync(0xFFFFFFFFu, jincl, 31);
  const int leader = __ffs(m) - 1;
  uint32_t rbase = 0, jbase = 0;
  if (lane == leader) {
    rbase = atomicAdd(&c.cnt->rec_count, (uint32_t)__popc(m));
    jbase = atomicAdd(&c.cnt->pair_count, jtotal);
  }
  rbase = __shfl_sync(0xFFFFFFFFu, rbase, leader);
  jbase = __shfl_sync(0xFFFFFFFFu, jbase, leader);
  if (!large) return;
  uint32_t idx = rbase + (uint32_t)__popc(m & lanemask_lt());
  store_record(c, idx, r);
  if (idx >= c.seg->rec_cap) return;
  uint32_t j0 = jbase + jincl - njobs, cap = c.seg->pair_cap / 2;
  uint2* jobs = reinterpret_cast<uint2*>(c.seg->bins);
  for (uint32_t j = 0; j < njobs && j0 + j < cap; j++) jobs[j0 + j] = make_uint2(idx, j * jb);
}

/* one record: small -> rasterise now, large -> jobs */
__device__ uint32_t vis_record(const Ctx& c, const KzTriRecord& r) {
  const KzDraw& d = c.draws[r.draw];
  if (box_area(r) <= KZ_SMALL_PX) return vis_small(*c.seg, r, d.zmin, d.zmax);
  vis_emit_large(c, r);
  return 0;
}

__device__ __noinline__ uint32_t vis_clipped(const Ctx& c, const KzDraw& d, const KzPipe& p, float pos[3][4],
                                             uint32_t g, uint32_t di) {
  ClipV v[KZ_MAX_CLIP_VERTS];
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 4; k++) v[j].c[k] = pos[j][k];
  int n = clip_polygon(v, 0);
  uint32_t frags = 0;
  for (int i = 1; i + 1 < n; i++) {
    Proj pr[3] = {project(d, v[0].c), project(d, v[i].c), project(d, v[i + 1].c)};
    KzTriRecord r;
    bool sw;
    if (!make_record(d, p, pr, r, sw)) continue;
    r.g = g;
    r.draw = di;
    r.pad = 0;
    r.info |= (uint32_t)i << 4;
    frags += vis_record(c, r);
  }
  return frags;
}

/* a shaded vertex as the triangles of a chunk need it: clip position, clip outcode and (when inside
 * the guard band) its projected 16.8 position and depth */
struct VEntry {
  float4 clip;
  int32_t X, Y;
  float z;
  uint32_t code; /* bits 0-5 outside the view volume (x>w, x<-w, y>w, y<-w, z<0, z>w); bits 6-11 outside
                    a clip plane (near, far, guard band); bit 12 non-finite */
};

/* the clip position and clip outcode of a shaded vertex (its projection follows in vertex_project) */
__device__ __forceinline__ VEntry vertex_code(float4 clip) {
  VEntry e;
  e.clip = clip;
  const float c[4] = {clip.x, clip.y, clip.z, clip.w};
  uint32_t code = 0;
  if (!(isfinite(c[0]) && isfinite(c[1]) && isfinite(c[2]) && isfinite(c[3]))) {
    code = 1u << 12;
  } else {
    code |= (c[0] > c[3]) ? 1u : 0u;
    code |= (c[0] < -c[3]) ? 2u : 0u;
    code |= (c[1] > c[3]) ? 4u : 0u;
    code |= (c[1] < -c[3]) ? 8u : 0u;
    code |= (c[2] < 0.0f) ? 16u : 0u;
    code |= (c[2] > c[3]) ? 32u : 0u;
    /* outside a clip plane: plane_dist(c, p) < 0 for near, far and the four guard-band planes.  The
     * signs of those float sums equal these comparisons (4w is an exact scaling, and a rounded sum of two
     * floats has the sign of the exact sum), so the codes are the same */
    const float gw = fmul(KZ_GUARD_BAND, c[3]);
    code |= (code & 48u) << 2;
    code |= (c[0] < -gw) ? 256u : 0u;
    code |= (c[0] > gw) ? 512u : 0u;
    code |= (c[1] < -gw) ? 1024u : 0u;
    code |= (c[1] > gw) ? 2048u : 0u;
  }
  e.X = e.Y = 0;
  e.z = 0.0f;
  e.code = code;
  return e;
}

/* the projected 16.8 position and depth of a vertex with a clip position inside every clip plane */
__device__ __forceinline__ void vertex_project(const KzDraw& d, VEntry& e) {
  if (!(e.code & ((63u << 6) | (1u << 12)))) {
    const float c[4] = {e.clip.x, e.clip.y, e.clip.z, e.clip.w};
    Proj p = project(d, c);
    e.X = p.X;
    e.Y = p.Y;
    e.z = p.z;
  }
}

/* set up the triangle of three shaded vertices.  Returns 1 with `out` set when the triangle's box holds
 * at most warp_px pixels (the warp rasterises it, vis_warp_raster), 2 with `out` set when it is larger
 * (jobs, vis_emit_large_warp), 0 otherwise; clipped triangles are rasterised here (their fragments are
 * added to `frags`). */
__device__ __forceinline__ int vis_triangle(const Ctx& c, const KzDraw& d, const KzPipe& p, uint32_t di, uint32_t g,
                             const VEntry (&v)[3], KzTriRecord& out, uint32_t& frags) {
  uint32_t any = v[0].code | v[1].code | v[2].code;
  if (any & (1u << 12)) return 0;
  if (v[0].code & v[1].code & v[2].code & 63u) return 0; /* outside one view-volume plane */
  if (any & (63u << 6)) {
    float pos[3][4];
    for (int j = 0; j < 3; j++) {
      pos[j][0] = v[j].clip.x;
      pos[j][1] = v[j].clip.y;
      pos[j][2] = v[j].clip.z;
      pos[j][3] = v[j].clip.w;
    }
    frags += vis_clipped(c, d, p, pos, g, di);
    return 0;
  }
  Proj pr[3];
  for (int j = 0; j < 3; j++) {
    pr[j].X = v[j].X;
    pr[j].Y = v[j].Y;
    pr[j].z = v[j].z;
    pr[j].iw = 0.0f;
  }
  bool sw;
  if (!make_record(d, p, pr, out, sw)) return 0;
  out.g = g;
  out.draw = di;
  out.pad = 0;
  return box_area(out) <= c.f->warp_px ? 1 : 2;
}

#define KZ_GEO_SMEM (KZ_THREADS * (96 + 1))
/* the divisor table's range: the pixel quads per row, ceil(w / 4), of every warp-rasterised box of width up
 * to 512 (wider ones compute their divisor) */
#define KZ_MAGIC_MAX 128

/* table[pw] = floor((2^32 - 1) / pw) + 1 for pw in [2, KZ_MAGIC_MAX] (0 for 0 and 1), filled by the block */
__device__ __forceinline__ void fill_magic(uint32_t* table) {
  for (uint32_t i = threadIdx.x; i <= KZ_MAGIC_MAX; i += blockDim.x) table[i] = i > 1 ? 0xFFFFFFFFu / i + 1u : 0u;
}

/* what the warp raster keeps of a record, in shared memory (one slot per lane) */
struct WarpTri {
  int64_t e[3];       /* edge functions at the centre of the box's first pixel, minus the edge's threshold
                         (1 unless top-left): covered iff all three are >= 0 */
  int32_t ex[3];      /* edge function step per pixel in x (-dy * 256) */
  int32_t ey[3];      /* ... and in y (dx * 256) */
  int32_t ox, oy;     /* first pixel of the box */
  uint32_t pw, magic; /* pixel quads per box row, ceil(w / 4); umulhi(i, magic) = i / pw for i < 2^16 */
  uint32_t start, w;  /* number of the box's first quad in the warp's list; box width */
  float z0, dz1, dz2, inv_s;
  uint32_t g, thr;    /* primitive number; bit k: edge k's threshold is 1; bit 3: every edge value over the
                         box fits in 32 bits */
};                    /* 96 bytes */
static_assert(sizeof(WarpTri) == 96, "WarpTri layout");

/* one covered pixel of a warp-rasterised triangle: its depth key into the visibility buffer */
__device__ __forceinline__ void warp_fragment(const KzSegment& seg, const WarpTri& t, int64_t e1, int64_t e2, float zmin,
                                              float zmax, int32_t x, int32_t y) {
  uint32_t thr = t.thr;
  float l1 = fmul(kz_i64_to_f32(e1 + (int64_t)((thr >> 1) & 1u)), t.inv_s);
  float l2 = fmul(kz_i64_to_f32(e2 + (int64_t)((thr >> 2) & 1u)), t.inv_s);
  float z = ffma(l2, t.dz2, ffma(l1, t.dz1, t.z0));
  z = fadd(fminf(fmaxf(z, zmin), zmax), 0.0f);
  vis_store(seg, vis_key(seg.vis_key, z, t.g), x, y);
}

/* the same for edge values known to fit in 32 bits (E1, E2 with their thresholds added back) */
__device__ __forceinline__ void warp_fragment32(const KzSegment& seg, const WarpTri& t, int32_t e1, int32_t e2,
                                                float zmin, float zmax, int32_t x, int32_t y) {
  float l1 = fmul(__int2float_rn(e1), t.inv_s);
  float l2 = fmul(__int2float_rn(e2), t.inv_s);
  float z = ffma(l2, t.dz2, ffma(l1, t.dz1, t.z0));
  z = fadd(fminf(fmaxf(z, zmin), zmax), 0.0f);
  vis_store(seg, vis_key(seg.vis_key, z, t.g), x, y);
}

/* rasterise every lane's record (valid where `have`) into the keys with the whole warp.  Each box row is
 * cut into quads of four horizontally adjacent pixels (the last one of a row may be shorter); the quads of
 * all lanes' boxes are numbered consecutively and the warp takes 32 consecutive quads per step, so lanes stay
 * busy however unequal the boxes are and neighbouring lanes write neighbouring keys (four pixels a lane: 1 %
 * less kernel time than two on the 4,096-draw frame).  In a step, each triangle whose quads meet the step's
 * window writes its lane into `owner` at the window position of its first quad there; lane l's triangle is the
 * one marked at the highest position <= l.  `slots`: this warp's 32 WarpTri, `owner`: its 32-entry table,
 * both in shared memory. */
__device__ __forceinline__ uint32_t vis_warp_raster(const KzSegment& seg, const KzTriRecord& r, bool have, float zmin,
                                                    float zmax, WarpTri* slots, uint8_t* owner,
                                                    const uint32_t* magic_tab) {
  const int lane = threadIdx.x & 31;
  uint32_t n = 0;
  if (have) {
    uint32_t w = (r.bb1 & 0xFFFFu) - (r.bb0 & 0xFFFFu) + 1;
    n = ((r.bb1 >> 16) - (r.bb0 >> 16) + 1) * ((w + 3) >> 2);
  }
  uint32_t incl = n;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += t;
  }
  const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  if (total == 0) return 0;
  const uint32_t start = incl - n;
  if (have) {
    WarpTri& t = slots[lane];
    Edges e;
    edges_of(r, e);
    t.ox = (int32_t)(r.bb0 & 0xFFFFu);
    t.oy = (int32_t)(r.bb0 >> 16);
    t.w = (r.bb1 & 0xFFFFu) - (r.bb0 & 0xFFFFu) + 1;
    t.pw = (t.w + 3) >> 2;
    /* floor((2^32 - 1) / pw) + 1: the rounded-up reciprocal for every pw > 1 (exact when pw is a power of 2);
     * from the block's table for the widths warp-rasterised boxes have */
    t.magic = t.pw <= KZ_MAGIC_MAX ? magic_tab[t.pw] : 0xFFFFFFFFu / t.pw + 1u;
    t.start = start;
    uint32_t thr = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      t.ex[k] = -e.dy[k] * 256;
      t.ey[k] = e.dx[k] * 256;
      thr |= (uint32_t)e.thr[k] << k;
    }
    bool fits = true;
    const int32_t xlo = min(r.x[0], min(r.x[1], r.x[2])), xhi = max(r.x[0], max(r.x[1], r.x[2]));
    const int32_t ylo = min(r.y[0], min(r.y[1], r.y[2])), yhi = max(r.y[0], max(r.y[1], r.y[2]));
    if (xhi - xlo < (1 << 14) && yhi - ylo < (1 << 14)) {
      /* vertices within 64 px of each other: every edge vector component and every offset from a vertex to a
       * pixel centre of the box (the one-sample box of centres lies inside the vertices' extent) is below 2^14
       * in magnitude, so each product is below 2^28 and every edge value over the box below 2^29: exact in
       * 32 bits */
      const int32_t px = t.ox * 256 + 128, py = t.oy * 256 + 128;
#pragma unroll
      for (int k = 0; k < 3; k++) t.e[k] = e.dx[k] * (py - e.ya[k]) - e.dy[k] * (px - e.xa[k]) - e.thr[k];
    } else {
      const int64_t px = (int64_t)t.ox * 256 + 128, py = (int64_t)t.oy * 256 + 128;
      const int64_t h1 = (int64_t)((r.bb1 >> 16) - (r.bb0 >> 16)), w1 = (int64_t)t.w - 1;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        t.e[k] = edge_at(e, k, px, py) - e.thr[k];
        /* largest |value| the edge takes over the box (with margin: three steps past its last column) */
        int64_t ae = t.e[k] < 0 ? -t.e[k] : t.e[k];
        int64_t bound = ae + (int64_t)abs(t.ex[k]) * (w1 + 3) + (int64_t)abs(t.ey[k]) * h1 + 1;
        fits = fits && bound < 0x7FFFFFFFll;
      }
    }
    t.thr = thr | (fits ? 8u : 0u);
    t.z0 = r.z0;
    t.dz1 = r.dz1;
    t.dz2 = r.dz2;
    t.inv_s = r.inv_s;
    t.g = r.g;
  }
  uint32_t frags = 0;
  const uint32_t upto = 0xFFFFFFFFu >> (31 - lane); /* window positions 0..lane */
  for (uint32_t base = 0; base < total; base += 32) {
    bool meets = n != 0 && start < base + 32 && start + n > base;
    uint32_t pos = start > base ? start - base : 0u;
    if (meets) owner[pos] = (uint8_t)lane;
    uint32_t marks = __reduce_or_sync(0xFFFFFFFFu, meets ? 1u << pos : 0u);
    __syncwarp();
    uint32_t o = owner[31 - __clz(marks & upto)];
    __syncwarp();
    uint32_t idx = base + (uint32_t)lane;
    if (idx >= total) continue;
    const WarpTri& t = slots[o];
    uint32_t local = idx - t.start;
    uint32_t pw = t.pw;
    uint32_t y = pw > 1 ? __umulhi(local, t.magic) : local;
    int32_t x = (int32_t)(local - y * pw) * 4;
    int32_t sx0 = t.ex[0], sx1 = t.ex[1], sx2 = t.ex[2];
    int32_t px = t.ox + x, py = t.oy + (int32_t)y;
    const uint32_t tthr = t.thr;
    if (tthr & 8u) {
      /* every edge value of this box fits in 32 bits: the same integers in 32-bit arithmetic */
      int32_t e0 = (int32_t)t.e[0] + sx0 * x + t.ey[0] * (int32_t)y;
      int32_t e1 = (int32_t)t.e[1] + sx1 * x + t.ey[1] * (int32_t)y;
      int32_t e2 = (int32_t)t.e[2] + sx2 * x + t.ey[2] * (int32_t)y;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (k > 0) {
          if ((uint32_t)x + k >= t.w) break;
          e0 += sx0;
          e1 += sx1;
          e2 += sx2;
        }
        if ((e0 | e1 | e2) >= 0) {
          frags++;
          warp_fragment32(seg, t, e1 + (int32_t)((tthr >> 1) & 1u), e2 + (int32_t)((tthr >> 2) & 1u), zmin, zmax, px + k, py);
        }
      }
      continue;
    }
    int64_t e0 = t.e[0] + (int64_t)sx0 * x + (int64_t)t.ey[0] * (int32_t)y;
    int64_t e1 = t.e[1] + (int64_t)sx1 * x + (int64_t)t.ey[1] * (int32_t)y;
    int64_t e2 = t.e[2] + (int64_t)sx2 * x + (int64_t)t.ey[2] * (int32_t)y;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (k > 0) {
        if ((uint32_t)x + k >= t.w) break;
        e0 += sx0;
        e1 += sx1;
        e2 += sx2;
      }
      if ((e0 | e1 | e2) >= 0) {
        frags++;
        warp_fragment(seg, t, e1, e2, zmin, zmax, px + k, py);
      }
    }
  }
  __syncwarp();
  return frags;
}

/* geometry of the 32 triangles [32 sub, 32 sub + 32) of one chunk, one warp, one lane per triangle: the
 * lane shades its three vertices (position-only vertex shader), clips, projects and sets up its triangle;
 * the warp then emits its large triangles together and rasterises the small and medium ones together
 * (vis_warp_raster).  Returns the lane's fragment count. */
__device__ __forceinline__ uint32_t vis_geometry_warp(const Ctx& c, uint32_t chunk, uint32_t sub, WarpTri* slots,
                                                      uint8_t* owner, const uint32_t* magic_tab) {
  const KzChunk ch = chunk_at(c, chunk);
  if (sub * 32 >= ch.count) return 0;
  const KzDraw& d = c.draws[ch.draw];
  const KzPipe& p = c.pipes[d.pipe];
  const uint8_t* push = push_ptr(*c.f, d);
  uint32_t off = sub * 32 + (threadIdx.x & 31);
  uint32_t local = ch.first + off;
  uint32_t frags = 0;
  KzTriRecord r;
  int kind = 0;
  if (off < ch.count) {
    uint32_t vid[3], iid;
    tri_vertices(d, local, vid, iid);
    const KzPos3 q = kz_vs_pos3(d.pipe, &d, vid[0], vid[1], vid[2], iid, push);
    VEntry e[3];
#pragma unroll
    for (int j = 0; j < 3; j++) e[j] = vertex_code(q.p[j]);
    /* project only triangles that are not trivially outside the view volume (whole off-screen meshes skip
     * the divisions); vis_triangle rejects the others on the same codes */
    const uint32_t any = e[0].code | e[1].code | e[2].code;
    if (!(any & (1u << 12)) && !(e[0].code & e[1].code & e[2].code & 63u)) {
#pragma unroll
      for (int j = 0; j < 3; j++) vertex_project(d, e[j]);
    }
    kind = vis_triangle(c, d, p, ch.draw, d.prim_base + local, e, r, frags);
  }
  vis_emit_large_warp(c, r, kind == 2);
  frags += vis_warp_raster(*c.seg, r, kind == 1, d.zmin, d.zmax, slots, owner, magic_tab);
  return frags;
}

/* the geometry of a segment by warps: warp w of `warps` takes the 32-triangle groups w, w + warps, ...
 * (8 groups per chunk) of the launch's chunks [chunk_begin, chunk_end), then adds its fragment count to the
 * statistics.  `smem`: 8 warps x 32 WarpTri,
 * then 8 warps x 32 owner bytes (KZ_GEO_SMEM bytes). */
__device__ void vis_geometry_warps(const Ctx& c, unsigned char* smem, const uint32_t* magic_tab, uint32_t w,
                                   uint32_t warps) {
  const uint32_t wib = threadIdx.x >> 5;
  WarpTri* slots = reinterpret_cast<WarpTri*>(smem) + wib * 32;
  uint8_t* owner = smem + KZ_THREADS * sizeof(WarpTri) + wib * 32;
  const uint32_t cb = c.f->chunk_begin, ce = min(c.f->chunk_end, c.seg->num_chunks);
  const uint32_t groups = cb < ce ? (ce - cb) * 8 : 0u;
  uint32_t frags = 0;
  for (uint32_t i = w; i < groups; i += warps)
    frags += vis_geometry_warp(c, cb + i / 8, i % 8, slots, owner, magic_tab);
  for (int o = 16; o > 0; o >>= 1) frags += __shfl_xor_sync(0xFFFFFFFFu, frags, o);
  if ((threadIdx.x & 31) == 0 && frags) {
    atomicAdd(&c.cnt->fragments, frags);
    atomicAdd(&c.st->fragments_lo, frags);
  }
}

/* one large-triangle job, one warp: up to job_blocks 8x8 blocks of the record's box.
 * Lane b < job_blocks first evaluates the three edge functions at block b's first pixel centre and
 * drops the block when, for some edge, even the block's largest value (at the corner the edge's
 * gradient points to) is below the threshold.  The warp then walks the remaining blocks: each lane adds
 * its fixed offset within the block to the block's edge values (the same integers as evaluating the edge
 * functions at the pixel directly; in 32-bit arithmetic when every value over the box fits). */
__device__ uint32_t vis_large_job(const Ctx& c, uint2 job, int lane) {
  const KzSegment& seg = *c.seg;
  const KzTriRecord r = load_record(seg, job.x);
  const KzDraw& d = c.draws[r.draw];
  float zmin = d.zmin, zmax = d.zmax;
  Edges e;
  edges_of(r, e);
  int32_t bx0 = (int32_t)(r.bb0 & 0xFFFFu), by0 = (int32_t)(r.bb0 >> 16);
  int32_t bx1 = (int32_t)(r.bb1 & 0xFFFFu), by1 = (int32_t)(r.bb1 >> 16);
  uint32_t nbx, nb = box_blocks(r, nbx);
  /* block test, one block per lane; E* hold the edge values minus their thresholds (covered iff all >= 0) */
  uint32_t b = job.y + (uint32_t)lane;
  bool live = (uint32_t)lane < job_blocks(c) && b < nb;
  int32_t ox = 0, oy = 0;
  int64_t E0 = 0, E1 = 0, E2 = 0;
  if (live) {
    uint32_t row = b / nbx;
    ox = bx0 + (int32_t)(b - row * nbx) * 8;
    oy = by0 + (int32_t)row * 8;
    int64_t px = (int64_t)ox * 256 + 128, py = (int64_t)oy * 256 + 128;
    E0 = edge_at(e, 0, px, py) - e.thr[0];
    E1 = edge_at(e, 1, px, py) - e.thr[1];
    E2 = edge_at(e, 2, px, py) - e.thr[2];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      int64_t ek = k == 0 ? E0 : (k == 1 ? E1 : E2);
      int64_t mx = ek + (e.dy[k] < 0 ? -(int64_t)e.dy[k] * (7 * 256) : 0) + (e.dx[k] > 0 ? (int64_t)e.dx[k] * (7 * 256) : 0);
      live = live && mx >= 0;
    }
  }
  uint32_t mask = __ballot_sync(0xFFFFFFFFu, live);
  /* every edge value over the box (blocks reach 7 pixels past its last row and column) fits in 32 bits? */
  bool fits = true;
  {
    const int64_t wx = (int64_t)(bx1 - bx0) + 8, wy = (int64_t)(by1 - by0) + 8;
    const int64_t px = (int64_t)bx0 * 256 + 128, py = (int64_t)by0 * 256 + 128;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      int64_t ek = edge_at(e, k, px, py);
      int64_t ae = ek < 0 ? -ek : ek;
      fits = fits && ae + (int64_t)abs(e.dy[k]) * 256 * wx + (int64_t)abs(e.dx[k]) * 256 * wy + 2 < 0x7FFFFFFFll;
    }
  }
  /* this lane's offset inside a block: column lx, rows ly and ly + 4 */
  const int lx = lane & 7, ly = lane >> 3;
  uint32_t frags = 0;
  if (fits) {
    int32_t inc[3], half[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      inc[k] = e.dx[k] * (ly * 256) - e.dy[k] * (lx * 256);
      half[k] = e.dx[k] * (4 * 256);
    }
    const int32_t th1 = (int32_t)e.thr[1], th2 = (int32_t)e.thr[2];
    while (mask) {
      int src = __ffs(mask) - 1;
      mask &= mask - 1;
      int32_t bxo = __shfl_sync(0xFFFFFFFFu, ox, src), byo = __shfl_sync(0xFFFFFFFFu, oy, src);
      int32_t e0 = __shfl_sync(0xFFFFFFFFu, (int32_t)E0, src) + inc[0];
      int32_t e1 = __shfl_sync(0xFFFFFFFFu, (int32_t)E1, src) + inc[1];
      int32_t e2 = __shfl_sync(0xFFFFFFFFu, (int32_t)E2, src) + inc[2];
      int32_t x = bxo + lx;
      if (x > bx1) continue;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        int32_t y = byo + ly + 4 * h;
        if (y <= by1 && (e0 | e1 | e2) >= 0) {
          frags++;
          float l1 = fmul(__int2float_rn(e1 + th1), r.inv_s), l2 = fmul(__int2float_rn(e2 + th2), r.inv_s);
          float z = ffma(l2, r.dz2, ffma(l1, r.dz1, r.z0));
          z = fadd(fminf(fmaxf(z, zmin), zmax), 0.0f);
          vis_store(seg, vis_key(seg.vis_key, z, r.g), x, y);
        }
        e0 += half[0];
        e1 += half[1];
        e2 += half[2];
      }
    }
    return frags;
  }
  int64_t inc[3], half[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    inc[k] = (int64_t)e.dx[k] * (ly * 256) - (int64_t)e.dy[k] * (lx * 256);
    half[k] = (int64_t)e.dx[k] * (4 * 256);
  }
  while (mask) {
    int src = __ffs(mask) - 1;
    mask &= mask - 1;
    int32_t bxo = __shfl_sync(0xFFFFFFFFu, ox, src), byo = __shfl_sync(0xFFFFFFFFu, oy, src);
    int64_t e0 = __shfl_sync(0xFFFFFFFFu, E0, src) + inc[0];
    int64_t e1 = __shfl_sync(0xFFFFFFFFu, E1, src) + inc[1];
    int64_t e2 = __shfl_sync(0xFFFFFFFFu, E2, src) + inc[2];
    int32_t x = bxo + lx;
    if (x > bx1) continue;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      int32_t y = byo + ly + 4 * h;
      if (y <= by1 && (e0 | e1 | e2) >= 0) {
        frags++;
        float l1 = fmul(kz_i64_to_f32(e1 + e.thr[1]), r.inv_s), l2 = fmul(kz_i64_to_f32(e2 + e.thr[2]), r.inv_s);
        float z = ffma(l2, r.dz2, ffma(l1, r.dz1, r.z0));
        z = fadd(fminf(fmaxf(z, zmin), zmax), 0.0f);
        vis_store(seg, vis_key(seg.vis_key, z, r.g), x, y);
      }
      e0 += half[0];
      e1 += half[1];
      e2 += half[2];
    }
  }
  return frags;
}

__device__ void vis_init_range(const KzSegment& seg, size_t i0, size_t stride) {
  size_t n = (size_t)seg.width * seg.height;
  bool clear_d = seg.depth_load == KZ_LOAD_CLEAR;
  for (size_t i = i0; i < n; i += stride) {
    int32_t x = (int32_t)(i % seg.width), y = (int32_t)(i / seg.width);
    float dv = 1.0f;
    if (seg.depth) dv = clear_d ? seg.clear_depth : *depth_px(seg, x, y);
    reinterpret_cast<unsigned long long*>(seg.vis)[i] = vis_init(seg.vis_key, dv);
  }
}

/* resolve 32 consecutive pixels of one row, one warp */
__device__ void vis_resolve_run(const Ctx& c, uint32_t item) {
  const KzSegment& seg = *c.seg;
  uint32_t runs = (seg.width + 31) / 32;
  int32_t y = (int32_t)(item / runs), x = (int32_t)(item % runs) * 32 + (int32_t)(threadIdx.x & 31);
  if (x >= (int32_t)seg.width || x < seg.area[0] || x >= seg.area[2] || y < seg.area[1] || y >= seg.area[3]) return;
  bool clear_c = seg.color_load == KZ_LOAD_CLEAR, clear_d = seg.depth_load == KZ_LOAD_CLEAR;
  const bool has_color = seg.color != 0, has_depth = seg.depth != 0;
  uint32_t g;
  float z;
  if (vis_decode(seg.vis_key, *vis_px(seg, x, y), g, z)) {
    Shade s;
    if (shade_setup(c, g, x, y, 0, s)) {
      int64_t E[3];
      covers(s.r, x, y, E);
      float col[4];
      shade_pixel<true>(c, s, x, y, E, z, col);
      const KzPipe& p = c.pipes[s.pipe];
      if (has_color) {
        uint32_t dst = clear_c ? seg.clear_color : *color_px(seg, x, y);
        *color_px(seg, x, y) = from_rgba(color_write(p, c.draws[s.draw].blend_const, to_rgba(dst, seg.color_format),
                                                     col, nullptr, cf_srgb(seg.color_format)),
                                         seg.color_format);
      }
      if (has_depth && p.depth_test && p.depth_write) *depth_px(seg, x, y) = z;
      else if (has_depth && clear_d) *depth_px(seg, x, y) = seg.clear_depth;
      return;
    }
  }
  if (has_color && clear_c) *color_px(seg, x, y) = seg.clear_color;
  if (has_depth && clear_d) *depth_px(seg, x, y) = seg.clear_depth;
}

/* the large-triangle jobs [j0, njobs) of a segment, warp w of `warps` taking jobs j0 + w, j0 + w + warps, ...;
 * adds the fragments to the statistics */
__device__ __forceinline__ void vis_large_phase(const Ctx& c, uint32_t j0, uint32_t njobs, uint32_t w,
                                                uint32_t warps) {
  const uint2* jobs = reinterpret_cast<const uint2*>(c.seg->bins);
  const int lane = threadIdx.x & 31;
  uint32_t frags = 0;
  for (uint32_t j = j0 + w; j < njobs; j += warps) frags += vis_large_job(c, jobs[j], lane);
  for (int o = 16; o > 0; o >>= 1) frags += __shfl_xor_sync(0xFFFFFFFFu, frags, o);
  if (lane == 0 && frags) {
    atomicAdd(&c.cnt->fragments, frags);
    atomicAdd(&c.st->fragments_lo, frags);
  }
}

/* the resolve of a segment's 32-pixel row runs, warp w of `warps` taking runs w, w + warps, ... */
__device__ __forceinline__ void vis_resolve_phase(const Ctx& c, uint32_t w, uint32_t warps) {
  const uint32_t items = ((c.seg->width + 31) / 32) * c.seg->height;
  for (uint32_t i = w; i < items; i += warps) vis_resolve_run(c, i);
}

/* after geometry: large-triangle scratch overflow check (every block reads the same final counts) */
__device__ bool vis_check(const Ctx& c, uint32_t s) {
  uint32_t recs = *reinterpret_cast<volatile uint32_t*>(&c.cnt->rec_count);
  uint32_t jobs = *reinterpret_cast<volatile uint32_t*>(&c.cnt->pair_count);
  uint32_t bits = 0;
  if (recs > c.seg->rec_cap) bits |= KZ_STATUS_RECORD_OVERFLOW;
  if (jobs > c.seg->pair_cap / 2) bits |= KZ_STATUS_PAIR_OVERFLOW;
  if (bits && threadIdx.x == 0 && blockIdx.x == 0) {
    atomicMax(&c.st->need_records, recs);
    atomicMax(&c.st->need_pairs, jobs * 2);
    mark_failed(c.st, bits, s);
  }
  return bits == 0;
}

/* ordered mode: per-pixel in-order processing of the tile's bin, sorted by primitive */
/* one triangle of an ordered tile's batch, as the pixel loop reads it from shared memory */
struct BatchEntry {
  Shade s;                 /* record, 1/w and varyings, pipeline and draw */
  int64_t e[3];            /* edge functions at the centre of the tile's first pixel, minus their thresholds */
  int32_t ex[3], ey[3];    /* edge steps per pixel in x (-dy * 256) and y (dx * 256) */
  float zmin, zmax;
  uint32_t valid;          /* bit 0: the entry has a fragment setup; bit 1: `rect` cuts the tile */
  int8_t rect[4];          /* the draw's rectangle (first and last pixel column and row) relative to the tile,
                              clamped to [-1, 64] */
  uint32_t fits;           /* every edge value over the tile fits in 32 bits */
  uint32_t depth;          /* bit 0 test, bit 1 write, bits 2.. compare op */
  uint32_t blend;          /* 0 none, 1 straight alpha (SRC_ALPHA, ONE_MINUS_SRC_ALPHA, ADD), 2 any other */
  uint32_t write_mask;
  uint32_t thr;            /* bit k: edge k's threshold is 1 */
  uint32_t stencil;        /* bit 0 stencil test, bit 1 the fragment shader runs before the tests (it may
                              discard, and a discarded fragment leaves the stencil alone) */
  uint32_t st[4];          /* KzPipe::stencil, front then back */
};
static_assert(KZ_SORT_CAP * 8 + KZ_BATCH * sizeof(BatchEntry) <= KZ_DYN_SMEM,
              "ordered tile raster: sort keys and batch fit the dynamic shared memory");

/* blend with SRC_ALPHA / ONE_MINUS_SRC_ALPHA and ADD for colour and alpha: the same operations as
 * color_write's general path for these factors */
__device__ __forceinline__ uint32_t blend_straight_alpha(uint32_t dst, const float col[4], const float* u8tab,
                                                         uint32_t wm) {
  float a = fminf(fmaxf(col[3], 0.0f), 1.0f);
  float ia = fsub(1.0f, a);
  uint32_t out = dst;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (!((wm >> i) & 1u)) continue;
    float sv = i == 3 ? a : fminf(fmaxf(col[i], 0.0f), 1.0f);
    float d = u8tab[(dst >> (8 * i)) & 0xFFu];
    float r = ffma(sv, a, fmul(d, ia));
    out = (out & ~(0xFFu << (8 * i))) | ((uint32_t)unorm8(r) << (8 * i));
  }
  return out;
}

/* PER: pixels per thread (1 for tiles up to 16x16, 4 for 32x32), a compile-time constant so that the
 * tile's colour and depth stay in registers; the call handles the tile's pixels [base, base + PER *
 * blockDim.x) (64x64 tiles take four calls).  The bin is sorted by primitive number; each batch of
 * KZ_BATCH triangles is set up in shared memory, then every thread runs its pixels through the batch in
 * order: coverage, depth test, fragment shader, depth write, blend.  `u8tab`: u8f(k) for k = 0..255. */
/* sample s of a 4x multisampled pixel, relative to the pixel centre in 1/256 pixel */
__device__ __constant__ int32_t kz_ms_dx[KZ_MS_SAMPLES] = {-32, 96, -96, 32};
__device__ __constant__ int32_t kz_ms_dy[KZ_MS_SAMPLES] = {-96, -32, 32, 96};

__device__ __forceinline__ uint32_t* color_sample(const KzSegment& seg, int32_t x, int32_t y, int s) {
  return reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(seg.color) + (size_t)y * seg.color_pitch) + 4 * x + s;
}
__device__ __forceinline__ float* depth_sample(const KzSegment& seg, int32_t x, int32_t y, int s) {
  return reinterpret_cast<float*>(reinterpret_cast<char*>(seg.depth) + (size_t)y * seg.depth_pitch) + 4 * x + s;
}

/* ---------------- TMA staging of a tile's framebuffer block (kz_k_raster_direct) ---------------- */

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

/* the shared-memory copy of one tile's colour and depth texels (row-major, tile x tile) and the mbarrier its
 * tensor loads complete on */
struct TileStage {
  uint32_t* color;
  float* depth;
  uint64_t* mbar;
  uint32_t phase; /* parity of the mbarrier phase the next load completes */
};

#define KZ_TMA_WAIT_NS 100000000ull /* a tile's tensor loads complete within microseconds; give up after 100 ms */

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

/* one 2-D tensor load of the box at texel (x, y) into shared memory, completing its bytes on the mbarrier */
__device__ __forceinline__ void tma_load_2d(void* dst, uint64_t tmap, int32_t x, int32_t y, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_addr(dst)), "l"(tmap), "r"(x), "r"(y), "r"(smem_addr(mbar))
      : "memory");
}

__device__ __forceinline__ void tma_store_2d(uint64_t tmap, int32_t x, int32_t y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
               ::"l"(tmap), "r"(x), "r"(y), "r"(smem_addr(src))
               : "memory");
}

/* wait until the mbarrier completes the phase of parity `parity`; false after KZ_TMA_WAIT_NS */
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity) {
  const uint32_t a = smem_addr(mbar);
  unsigned long long t0 = 0;
  for (uint32_t i = 0;; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (i == 0) t0 = globaltimer();
    else if (globaltimer() - t0 > KZ_TMA_WAIT_NS) return false;
  }
}

/* MS: a 4x multisampled pass (PER 1, D32): coverage, depth test, depth write and colour per sample; the
 * fragment shader runs once per pixel, at the pixel centre, when some covered sample passes the depth
 * test */
/* CALLS: see shade_pixel.  TMA (PER 1, one sample, D32): `ts` holds the tile's colour and depth in shared
 * memory for the attachments that have a tensor map: thread 0 starts their tensor loads before the bin is
 * sorted, every thread waits for them before reading its pixels, and after the raster thread 0 writes the
 * block back with tensor stores (pixels outside the framebuffer are neither read nor written; pixels of the
 * tile outside the render area are written back unchanged).  Returns false when a load did not complete
 * (KZ_STATUS_TMA_TIMEOUT). */
template <int PER, bool DS, bool MS, bool CALLS, bool TMA = false>
__device__ bool raster_tile_ordered(const Ctx& c, uint32_t t, unsigned char* smem, const float* u8tab, int base,
                                    TileStage* ts = nullptr) {
  static_assert(!TMA || (PER == 1 && !DS && !MS), "TMA staging: one pixel per thread, one sample, D32");
  const KzSegment& seg = *c.seg;
  TileInfo ti;
  if (!tile_info(seg, t, ti)) return true;
  bool clear_c = seg.color_load == KZ_LOAD_CLEAR, clear_d = seg.depth_load == KZ_LOAD_CLEAR;
  /* DS: a D16 / D24S8 attachment (integer depths, stencil); otherwise D32 without stencil */
  const bool has_st = DS && seg.depth_format == KZ_DF_D24S8, clear_s = has_st && seg.stencil_load == KZ_LOAD_CLEAR;
  const bool srgb = cf_srgb(seg.color_format);
  if (ti.n == 0 && !clear_c && !clear_d && !clear_s) return true;
  if (ti.n > KZ_SORT_CAP) {
    if (threadIdx.x == 0) atomicOr(&c.st->flags, KZ_STATUS_BIN_TOO_LARGE);
    return true;
  }
  const int T = (int)seg.tile;
  const bool tma_c = TMA && seg.tmap_color && seg.color, tma_d = TMA && seg.tmap_depth && seg.depth;
  if (TMA && (tma_c || tma_d) && threadIdx.x == 0) {
    const uint32_t bytes = (uint32_t)(T * T * 4) * ((tma_c ? 1u : 0u) + (tma_d ? 1u : 0u));
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(ts->mbar)), "r"(bytes)
                 : "memory");
    if (tma_c) tma_load_2d(ts->color, seg.tmap_color, ti.ox, ti.oy, ts->mbar);
    if (tma_d) tma_load_2d(ts->depth, seg.tmap_depth, ti.ox, ti.oy, ts->mbar);
  }
  unsigned long long* sk = reinterpret_cast<unsigned long long*>(smem);
  BatchEntry* batch = reinterpret_cast<BatchEntry*>(smem + KZ_SORT_CAP * 8);
  const KzTriRecord* recs = reinterpret_cast<const KzTriRecord*>(seg.records);
  const uint32_t* bins = reinterpret_cast<const uint32_t*>(seg.bins) + ti.base;
  uint32_t m = 1;
  while (m < ti.n) m <<= 1;
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
    if (i < ti.n) {
      uint32_t ri = bins[i];
      sk[i] = ((unsigned long long)recs[ri].g << 32) | ri;
    } else {
      sk[i] = ~0ull;
    }
  }
  __syncthreads();
  for (uint32_t k = 2; k <= m; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        uint32_t l = i ^ j;
        if (l > i) {
          unsigned long long a = sk[i], b = sk[l];
          bool up = (i & k) == 0;
          if ((a > b) == up) {
            sk[i] = b;
            sk[l] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  if (TMA && (tma_c || tma_d)) {
    /* the tile's texels in shared memory before any thread reads them */
    bool ok = __syncthreads_and(mbar_wait(ts->mbar, ts->phase) ? 1 : 0) != 0;
    if (!ok) { /* give up: flag it, wait once more (bounded) for the copies in flight, and end the kernel */
      if (threadIdx.x == 0) atomicOr(&c.st->flags, KZ_STATUS_TMA_TIMEOUT);
      __syncthreads_and(mbar_wait(ts->mbar, ts->phase) ? 1 : 0);
      return false;
    }
    ts->phase ^= 1u;
  }
  /* this thread's pixels: offsets in the tile and whether they lie in the framebuffer and render area */
  const bool has_color = seg.color != 0, has_depth = seg.depth != 0;
  int lx[PER], ly[PER];
  bool in[PER];
  uint32_t colv[PER];
  float depv[PER];
  uint32_t stv[PER];
  constexpr int NS = MS ? KZ_MS_SAMPLES : 1;
  uint32_t colm[NS];
  float depm[NS];
#pragma unroll
  for (int q = 0; q < PER; q++) {
    int i = base + (int)threadIdx.x + q * (int)blockDim.x;
    lx[q] = i % T;
    ly[q] = i / T;
    int32_t x = ti.ox + lx[q], y = ti.oy + ly[q];
    in[q] = i < T * T && x >= ti.x0 && x <= ti.x1 && y >= ti.y0 && y <= ti.y1;
    colv[q] = 0;
    depv[q] = 1.0f;
    stv[q] = 0;
    if (!in[q]) continue;
    if constexpr (MS) {
#pragma unroll
      for (int s = 0; s < NS; s++) {
        colm[s] = has_color ? to_rgba(clear_c ? seg.clear_color : *color_sample(seg, x, y, s), seg.color_format) : 0u;
        depm[s] = has_depth ? (clear_d ? seg.clear_depth : *depth_sample(seg, x, y, s)) : 1.0f;
      }
      continue;
    }
    if (TMA && tma_c) colv[q] = to_rgba(clear_c ? seg.clear_color : ts->color[ly[q] * T + lx[q]], seg.color_format);
    else if (has_color) colv[q] = to_rgba(clear_c ? seg.clear_color : *color_px(seg, x, y), seg.color_format);
    if (TMA && tma_d) {
      depv[q] = clear_d ? seg.clear_depth : ts->depth[ly[q] * T + lx[q]];
    } else if (has_depth && DS) {
      uint32_t s0 = 0;
      float d0 = clear_d && (clear_s || !has_st) ? 0.0f : load_depth(seg, x, y, s0);
      depv[q] = clear_d ? seg.clear_depth : d0;
      stv[q] = clear_s ? seg.clear_stencil : s0;
    } else if (has_depth) {
      depv[q] = clear_d ? seg.clear_depth : *depth_px(seg, x, y);
    }
  }
  const int64_t tpx = (int64_t)ti.ox * 256 + 128, tpy = (int64_t)ti.oy * 256 + 128;
  uint32_t frags = 0;
  for (uint32_t b0 = 0; b0 < ti.n; b0 += KZ_BATCH) {
    uint32_t nb = min((uint32_t)KZ_BATCH, ti.n - b0);
    __syncthreads();
    if (threadIdx.x < nb) {
      unsigned long long key = sk[b0 + threadIdx.x];
      uint32_t ri = (uint32_t)key;
      const KzTriRecord r = recs[ri];
      BatchEntry& be = batch[threadIdx.x];
      uint32_t sub = (r.info >> 4) & 15u;
      if (sub == 0 && seg.shades) {
        /* unclipped: the setup the geometry phase stored beside the record */
        be.s.r = r;
        be.s.draw = r.draw;
        be.s.pipe = c.draws[r.draw].pipe;
        const int nc = (int)c.pipes[be.s.pipe].num_varyings;
        const float* src = reinterpret_cast<const float*>(seg.shades + (size_t)ri * seg.shade_stride);
        for (int i = 0; i < 3; i++) {
          be.s.iw[i] = __ldg(src + i);
          for (int k = 0; k < nc; k++) be.s.a[i][k] = __ldg(src + 4 + i * nc + k);
        }
        be.valid = 1u;
      } else {
        be.valid = shade_setup(c, r.g, 0, 0, sub, be.s) ? 1u : 0u;
      }
      const KzDraw& bd = c.draws[r.draw];
      const KzPipe& bp = c.pipes[bd.pipe];
      if (bd.rect[0] > ti.x0 || bd.rect[1] > ti.y0 || bd.rect[2] - 1 < ti.x1 || bd.rect[3] - 1 < ti.y1) {
        be.valid |= be.valid << 1;
        be.rect[0] = (int8_t)min(max(bd.rect[0] - ti.ox, -1), 64);
        be.rect[1] = (int8_t)min(max(bd.rect[1] - ti.oy, -1), 64);
        be.rect[2] = (int8_t)min(max(bd.rect[2] - 1 - ti.ox, -1), 64);
        be.rect[3] = (int8_t)min(max(bd.rect[3] - 1 - ti.oy, -1), 64);
      }
      be.zmin = bd.zmin;
      be.zmax = bd.zmax;
      be.depth = (bp.depth_test ? 1u : 0u) | (bp.depth_write ? 2u : 0u) | (bp.depth_compare << 2);
      bool straight = bp.src_color == 6 && bp.dst_color == 7 && bp.color_op == 0 && bp.src_alpha == 6 &&
                      bp.dst_alpha == 7 && bp.alpha_op == 0;
      be.blend = bp.blend_enable ? (straight && !srgb ? 1u : 2u) : 0u;
      be.write_mask = bp.write_mask;
      be.stencil = bp.stencil_test && has_st ? (1u | (bp.fs_discards ? 2u : 0u)) : 0u;
#pragma unroll
      for (int k = 0; k < 4; k++) be.st[k] = bd.stencil[k];
      /* edge values at the tile's first pixel centre, from the record that shading uses */
      Edges ed;
      edges_of(be.s.r, ed);
      bool fits = true;
      uint32_t thr = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        be.e[k] = edge_at(ed, k, tpx, tpy) - ed.thr[k];
        be.ex[k] = -ed.dy[k] * 256;
        be.ey[k] = ed.dx[k] * 256;
        thr |= (uint32_t)ed.thr[k] << k;
        int64_t ae = be.e[k] < 0 ? -be.e[k] : be.e[k];
        fits = fits && ae + ((int64_t)abs(be.ex[k]) + (int64_t)abs(be.ey[k])) * (T - 1) + 1 < 0x7FFFFFFFll;
      }
      be.thr = thr;
      be.fits = fits ? 1u : 0u;
    }
    __syncthreads();
    for (uint32_t j = 0; j < nb; j++) {
      const BatchEntry& be = batch[j];
      if (!be.valid) continue;
      /* bit 1: the draw's viewport and scissor rectangle cuts this tile, so pixels outside it are skipped
       * (bins hold every tile the clamped box meets; inside the tile the edges alone would also cover pixels
       * beyond the rectangle) */
      const bool cut = (be.valid & 2u) != 0;
#pragma unroll
      for (int q = 0; q < PER; q++) {
        if (!in[q]) continue;
        if (cut && (lx[q] < be.rect[0] || lx[q] > be.rect[2] || ly[q] < be.rect[1] || ly[q] > be.rect[3])) continue;
        int64_t E[3];
        if constexpr (MS) {
          /* edge values at the pixel centre, then at each sample (the steps per 1/256 pixel are ex / 256 and
           * ey / 256, exact) */
          int64_t ec[3];
#pragma unroll
          for (int k = 0; k < 3; k++) ec[k] = be.e[k] + (int64_t)be.ex[k] * lx[q] + (int64_t)be.ey[k] * ly[q];
          int64_t es[NS][3];
          uint32_t cover = 0;
#pragma unroll
          for (int s = 0; s < NS; s++) {
#pragma unroll
            for (int k = 0; k < 3; k++)
              es[s][k] = ec[k] + (int64_t)kz_ms_dx[s] * (be.ex[k] / 256) + (int64_t)kz_ms_dy[s] * (be.ey[k] / 256);
            if ((es[s][0] | es[s][1] | es[s][2]) >= 0) cover |= 1u << s;
          }
          if (!cover) continue;
          frags++;
          const KzTriRecord& r = be.s.r;
          const bool dtest = (be.depth & 1u) && has_depth;
          float zs[NS];
          uint32_t pass = 0;
#pragma unroll
          for (int s = 0; s < NS; s++) {
            if (!((cover >> s) & 1u)) continue;
            float l1 = fmul(kz_i64_to_f32(es[s][1] + (int64_t)((be.thr >> 1) & 1u)), r.inv_s);
            float l2 = fmul(kz_i64_to_f32(es[s][2] + (int64_t)(be.thr >> 2)), r.inv_s);
            float z = ffma(l2, r.dz2, ffma(l1, r.dz1, r.z0));
            zs[s] = fadd(fminf(fmaxf(z, be.zmin), be.zmax), 0.0f);
            if (!dtest || depth_cmp(be.depth >> 2, zs[s], depm[s])) pass |= 1u << s;
          }
          if (!pass) continue;
          E[0] = ec[0] + (int64_t)(be.thr & 1u);
          E[1] = ec[1] + (int64_t)((be.thr >> 1) & 1u);
          E[2] = ec[2] + (int64_t)(be.thr >> 2);
          float l1 = fmul(kz_i64_to_f32(E[1]), r.inv_s), l2 = fmul(kz_i64_to_f32(E[2]), r.inv_s);
          float zc = fadd(fminf(fmaxf(ffma(l2, r.dz2, ffma(l1, r.dz1, r.z0)), be.zmin), be.zmax), 0.0f);
          int32_t x = ti.ox + lx[q], y = ti.oy + ly[q];
          float col[4];
          if (shade_pixel<false, CALLS>(c, be.s, x, y, E, zc, col)) continue;
#pragma unroll
          for (int s = 0; s < NS; s++) {
            if (!((pass >> s) & 1u)) continue;
            if (dtest && (be.depth & 2u)) depm[s] = zs[s];
            if (!has_color) continue;
            if (be.blend == 1u) colm[s] = blend_straight_alpha(colm[s], col, u8tab, be.write_mask);
            else colm[s] = color_write(c.pipes[be.s.pipe], c.draws[be.s.draw].blend_const, colm[s], col, u8tab, srgb);
          }
          continue;
        }
        if (be.fits) {
          /* the same integers in 32-bit arithmetic (bounded over the tile) */
          int32_t e0 = (int32_t)be.e[0] + be.ex[0] * lx[q] + be.ey[0] * ly[q];
          int32_t e1 = (int32_t)be.e[1] + be.ex[1] * lx[q] + be.ey[1] * ly[q];
          int32_t e2 = (int32_t)be.e[2] + be.ex[2] * lx[q] + be.ey[2] * ly[q];
          if ((e0 | e1 | e2) < 0) continue;
          E[0] = e0;
          E[1] = e1;
          E[2] = e2;
        } else {
          int64_t e0 = be.e[0] + (int64_t)be.ex[0] * lx[q] + (int64_t)be.ey[0] * ly[q];
          int64_t e1 = be.e[1] + (int64_t)be.ex[1] * lx[q] + (int64_t)be.ey[1] * ly[q];
          int64_t e2 = be.e[2] + (int64_t)be.ex[2] * lx[q] + (int64_t)be.ey[2] * ly[q];
          if ((e0 | e1 | e2) < 0) continue;
          E[0] = e0;
          E[1] = e1;
          E[2] = e2;
        }
        E[0] += (int64_t)(be.thr & 1u);
        E[1] += (int64_t)((be.thr >> 1) & 1u);
        E[2] += (int64_t)(be.thr >> 2);
        frags++;
        const KzTriRecord& r = be.s.r;
        float l1 = fmul(kz_i64_to_f32(E[1]), r.inv_s), l2 = fmul(kz_i64_to_f32(E[2]), r.inv_s);
        float z = ffma(l2, r.dz2, ffma(l1, r.dz1, r.z0));
        z = fadd(fminf(fmaxf(z, be.zmin), be.zmax), 0.0f);
        const bool dtest = (be.depth & 1u) && has_depth;
        const float zq = DS ? depth_value(z, seg.depth_format) : z;
        int32_t x = ti.ox + lx[q], y = ti.oy + ly[q];
        float col[4];
        if (DS && be.stencil) {
          /* late tests when the shader may discard: a discarded fragment changes nothing */
          if ((be.stencil & 2u) && shade_pixel<false, CALLS>(c, be.s, x, y, E, z, col)) continue;
          const bool dpass = !dtest || depth_cmp(be.depth >> 2, zq, depv[q]);
          const bool front = (be.s.r.info >> 8) & 1u;
          const uint32_t w0 = front ? be.st[0] : be.st[2], w1 = front ? be.st[1] : be.st[3];
          const uint32_t cm = w1 & 0xFFu, sv = stv[q];
          if (!stencil_cmp((w0 >> 9) & 7u, (w1 >> 16) & cm, sv & cm)) {
            stv[q] = stencil_apply(w0 & 7u, sv, w1);
            continue;
          }
          stv[q] = stencil_apply(dpass ? (w0 >> 3) & 7u : (w0 >> 6) & 7u, sv, w1);
          if (!dpass) continue;
          if (!(be.stencil & 2u) && shade_pixel<false, CALLS>(c, be.s, x, y, E, z, col)) continue;
        } else {
          if (dtest && !depth_cmp(be.depth >> 2, zq, depv[q])) continue;
          if (shade_pixel<false, CALLS>(c, be.s, x, y, E, z, col)) continue;
        }
        if (dtest && (be.depth & 2u)) depv[q] = zq;
        if (!has_color) continue;
        if (be.blend == 1u) colv[q] = blend_straight_alpha(colv[q], col, u8tab, be.write_mask);
        else colv[q] = color_write(c.pipes[be.s.pipe], c.draws[be.s.draw].blend_const, colv[q], col, u8tab, srgb);
      }
    }
  }
  if (frags) {
    atomicAdd(&c.cnt->fragments, frags);
    atomicAdd(&c.st->fragments_lo, frags);
  }
#pragma unroll
  for (int q = 0; q < PER; q++) {
    if (!in[q]) continue;
    int32_t x = ti.ox + lx[q], y = ti.oy + ly[q];
    if constexpr (MS) {
#pragma unroll
      for (int s = 0; s < NS; s++) {
        if (has_color) *color_sample(seg, x, y, s) = from_rgba(colm[s], seg.color_format);
        if (has_depth) *depth_sample(seg, x, y, s) = depm[s];
      }
      continue;
    }
    if (TMA && tma_c) ts->color[ly[q] * T + lx[q]] = from_rgba(colv[q], seg.color_format);
    else if (has_color) *color_px(seg, x, y) = from_rgba(colv[q], seg.color_format);
    if (TMA && tma_d) ts->depth[ly[q] * T + lx[q]] = depv[q];
    else if (has_depth && DS) store_depth(seg, x, y, depv[q], stv[q]);
    else if (has_depth) *depth_px(seg, x, y) = depv[q];
  }
  if (TMA && (tma_c || tma_d)) {
    /* the block back to the attachments: the shared-memory writes made visible to the tensor stores, then
     * thread 0 stores and waits until the stores have read shared memory (the next tile reuses it) */
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      if (tma_c) tma_store_2d(seg.tmap_color, ti.ox, ti.oy, ts->color);
      if (tma_d) tma_store_2d(seg.tmap_depth, ti.ox, ti.oy, ts->depth);
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    }
    __syncthreads();
  }
  return true;
}

__device__ void raster_tile(const Ctx& c, uint32_t t, unsigned char* smem, const float* u8tab) {
  const uint32_t T = c.seg->tile;
  const bool ds = c.seg->depth_format != KZ_DF_D32;
  if (c.seg->samples > 1) { /* tiles of at most 16 x 16 */
    raster_tile_ordered<1, false, true, true>(c, t, smem, u8tab, 0);
  } else if (T <= 16) {
    if (ds) raster_tile_ordered<1, true, false, true>(c, t, smem, u8tab, 0);
    else raster_tile_ordered<1, false, false, true>(c, t, smem, u8tab, 0);
  } else {
    for (int base = 0; base < (int)(T * T); base += 4 * KZ_THREADS) {
      __syncthreads();
      if (ds) raster_tile_ordered<4, true, false, true>(c, t, smem, u8tab, base);
      else raster_tile_ordered<4, false, false, true>(c, t, smem, u8tab, base);
    }
  }
  __syncthreads();
  /* leave the tile counts at zero for the next segment */
  if (threadIdx.x == 0) reinterpret_cast<uint32_t*>(c.seg->tile_count)[t] = 0;
}

/* ---------------- grid barrier (persistent kernel) ---------------- */

/* Every block arrives once per call.  A block that has waited `limit_ns` nanoseconds (KzFrame::barrier_ns;
 * 0: it gives up at its first check) flags KZ_STATUS_BARRIER_TIMEOUT, and every block that sees the flag
 * leaves the kernel instead of spinning.  No block passes a barrier before all blocks have arrived at it. */
__device__ bool grid_barrier(KzStatus* st, uint32_t limit_ns) {
  __syncthreads();
  __shared__ uint32_t ok;
  if (threadIdx.x == 0) {
    volatile uint32_t* genp = &st->barrier_gen;
    uint32_t gen = *genp;
    __threadfence();
    uint32_t arrived = atomicAdd(&st->barrier_arrive, 1u) + 1u;
    ok = 1;
    if (arrived == gridDim.x) {
      atomicExch(&st->barrier_arrive, 0u);
      __threadfence();
      atomicAdd(&st->barrier_gen, 1u);
    } else {
      unsigned long long t0 = globaltimer();
      while (*genp == gen) {
        if (status_flags(st) & KZ_STATUS_BARRIER_TIMEOUT) {
          ok = 0;
          break;
        }
        if (globaltimer() - t0 >= (unsigned long long)limit_ns) {
          atomicOr(&st->flags, KZ_STATUS_BARRIER_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(200);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ uint32_t grab(uint32_t* counter, uint32_t* sh) {
  __syncthreads();
  if (threadIdx.x == 0) *sh = atomicAdd(counter, 1u);
  __syncthreads();
  return *sh;
}

}  // namespace

/* ================= kernels ================= */

/* Programmatic dependent launch: the driver may launch a kernel before the kernel ahead of it in the
 * stream has completed (cudaLaunchAttributeProgrammaticStreamSerialization), so the launch overlaps the
 * predecessor's completion.  Every kernel first waits until its predecessor has completed and that grid's
 * writes are visible (a no-op when it was launched the ordinary way).  No kernel triggers its successor
 * early (griddepcontrol.launch_dependents): successor blocks scheduled while the predecessor still ran
 * made every workload slower (0.2295 -> 0.242 ms on a 1M-triangle draw), so a successor starts once its
 * predecessor's blocks have all exited. */
__device__ __forceinline__ void kz_pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

extern "C" __global__ void __launch_bounds__(KZ_THREADS) kz_k_geometry(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  __shared__ uint32_t sh[40];
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  const uint32_t ce = min(f.chunk_end, c.seg->num_chunks);
  for (uint32_t k = f.chunk_begin + blockIdx.x; k < ce; k += gridDim.x) geometry_chunk(c, k, sh);
}

#define KZ_IND_THREADS 1024
#define KZ_IND_ITEMS 4

/* one indirect command as read: VkDrawIndirectCommand {vertexCount, instanceCount, firstVertex,
 * firstInstance} or VkDrawIndexedIndirectCommand {indexCount, instanceCount, firstIndex, vertexOffset,
 * firstInstance}, with the draw's limits */
struct IndirectCmd {
  uint32_t tri, inst, first, first_inst;
  int32_t voff;
  uint32_t indexed;
  unsigned long long ib_base;
};

/* loads only (read-only path), so that the loads of several commands overlap; a command at or past the
 * count of a vkCmdDraw*IndirectCount call draws nothing; a command whose vertices, indices or instances lie
 * past the bound buffers gets no instances (`bad` set when it would have drawn) */
__device__ __forceinline__ IndirectCmd load_indirect(const KzDraw& d, bool& bad) {
  IndirectCmd c;
  const uint32_t* cmd = reinterpret_cast<const uint32_t*>(__ldg(&d.indirect));
  c.indexed = __ldg(&d.indexed);
  c.tri = __ldg(cmd) / 3;
  c.inst = __ldg(cmd + 1);
  c.first = __ldg(cmd + 2);
  if (c.indexed) {
    c.voff = (int32_t)__ldg(cmd + 3);
    c.first_inst = __ldg(cmd + 4);
  } else {
    c.voff = (int32_t)c.first;
    c.first_inst = __ldg(cmd + 3);
  }
  c.ib_base = __ldg(&d.ib_base);
  const uint32_t* count = reinterpret_cast<const uint32_t*>(__ldg(&d.count_addr));
  if (count && __ldg(&d.call_index) >= __ldg(count)) c.tri = c.inst = 0;
  bool ok = (unsigned long long)c.first + 3ull * c.tri <= __ldg(&d.elem_limit) &&
            (unsigned long long)c.first_inst + c.inst <= __ldg(&d.instance_limit);
  if (!ok) {
    bad |= c.tri != 0 && c.inst != 0;
    c.inst = 0;
  }
  return c;
}

/* the indirect draws of segment s (one block, before the segment's other kernels): each thread reads
 * KZ_IND_ITEMS consecutive commands (load_indirect), the block scans their triangle and chunk counts, then
 * each thread writes its draws' counts and index address, and prim_base and chunk_base as exclusive prefix
 * sums over the segment in draw order (a chunk never spans two draws, as in the chunk table of direct
 * draws); finally the segment's num_prims, num_chunks and draw lookup pointer. */
extern "C" __global__ void __launch_bounds__(KZ_IND_THREADS) kz_k_indirect(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  __shared__ unsigned long long warp_p[KZ_IND_THREADS / 32], warp_c[KZ_IND_THREADS / 32];
  KzSegment* seg = reinterpret_cast<KzSegment*>(f.segments) + s;
  KzDraw* draws = reinterpret_cast<KzDraw*>(f.draws) + seg->first_draw;
  KzStatus* st = reinterpret_cast<KzStatus*>(f.status);
  const uint32_t n = seg->num_draws, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long prim_run = 0, chunk_run = 0;
  bool bad = false;
  for (uint32_t base = 0; base < n; base += KZ_IND_THREADS * KZ_IND_ITEMS) {
    const uint32_t i0 = base + threadIdx.x * KZ_IND_ITEMS;
    IndirectCmd cmd[KZ_IND_ITEMS];
#pragma unroll
    for (int j = 0; j < KZ_IND_ITEMS; j++) {
      if (i0 + j < n) cmd[j] = load_indirect(draws[i0 + j], bad);
      else cmd[j].tri = cmd[j].inst = 0;
    }
    unsigned long long tp = 0, tc = 0;
#pragma unroll
    for (int j = 0; j < KZ_IND_ITEMS; j++) {
      unsigned long long p = (unsigned long long)cmd[j].tri * cmd[j].inst;
      tp += p;
      tc += (p + KZ_CHUNK - 1) / KZ_CHUNK;
    }
    unsigned long long ip = tp, ic = tc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long a = __shfl_up_sync(0xFFFFFFFFu, ip, o), b = __shfl_up_sync(0xFFFFFFFFu, ic, o);
      if (lane >= (uint32_t)o) {
        ip += a;
        ic += b;
      }
    }
    if (lane == 31) {
      warp_p[warp] = ip;
      warp_c[warp] = ic;
    }
    __syncthreads();
    unsigned long long wp = 0, wc = 0, bp = 0, bc = 0;
    for (uint32_t w = 0; w < KZ_IND_THREADS / 32; w++) {
      if (w < warp) {
        wp += warp_p[w];
        wc += warp_c[w];
      }
      bp += warp_p[w];
      bc += warp_c[w];
    }
    unsigned long long pb = prim_run + wp + ip - tp, cb = chunk_run + wc + ic - tc;
#pragma unroll
    for (int j = 0; j < KZ_IND_ITEMS; j++) {
      if (i0 + j >= n) break;
      KzDraw& d = draws[i0 + j];
      const IndirectCmd& c = cmd[j];
      unsigned long long p = (unsigned long long)c.tri * c.inst;
      d.tri_count = c.tri;
      d.instance_count = c.inst;
      d.vertex_offset = c.voff;
      d.first_instance = c.first_inst;
      if (c.indexed) d.ib = c.ib_base + (unsigned long long)c.first * (c.indexed == 1 ? 4u : 2u);
      d.prim_base = (uint32_t)min(pb, 0xFFFFFFFFull);
      d.chunk_base = (uint32_t)min(cb, 0xFFFFFFFFull);
      pb += p;
      cb += (p + KZ_CHUNK - 1) / KZ_CHUNK;
    }
    prim_run += bp;
    chunk_run += bc;
    __syncthreads();
  }
  bad = __syncthreads_or(bad) != 0;
  if (threadIdx.x == 0) {
    if (prim_run >= 0xFFFFFFF0ull) {
      prim_run = chunk_run = 0;
      atomicOr(&st->flags, (uint32_t)KZ_STATUS_INDIRECT_LIMIT);
    }
    seg->num_prims = (uint32_t)prim_run;
    seg->num_chunks = (uint32_t)chunk_run;
    seg->draw_lut = (prim_run + 255) / 256 <= seg->lut_cap ? seg->lut_table : 0ull;
    if (bad) atomicOr(&st->flags, (uint32_t)KZ_STATUS_INDIRECT_RANGE);
  }
}

/* after kz_k_indirect, every thread of the grid: the chunk table (KzChunk per chunk, as for direct draws)
 * and the draw lookup (draw holding primitive 256 i) of an indirect segment, where they fit their room */
extern "C" __global__ void __launch_bounds__(KZ_THREADS) kz_k_indirect_tables(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  const KzSegment& seg = reinterpret_cast<const KzSegment*>(f.segments)[s];
  const KzDraw* draws = reinterpret_cast<const KzDraw*>(f.draws);
  const uint32_t nc = seg.num_chunks <= seg.chunk_cap ? seg.num_chunks : 0u;
  const uint32_t nl = seg.draw_lut ? (seg.num_prims + 255) / 256 : 0u;
  KzChunk* chunk_table = reinterpret_cast<KzChunk*>(seg.chunk_table);
  uint32_t* lut = reinterpret_cast<uint32_t*>(seg.draw_lut);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < max(nc, nl); k += gridDim.x * blockDim.x) {
    if (k < nc) {
      const uint32_t di = draw_of_chunk(draws, seg.first_draw, seg.num_draws, k);
      const KzDraw& d = draws[di];
      KzChunk ch;
      ch.draw = di;
      ch.first = (k - d.chunk_base) * KZ_CHUNK;
      ch.count = min((uint32_t)KZ_CHUNK, d.tri_count * d.instance_count - ch.first);
      ch.pad = 0;
      chunk_table[k] = ch;
    }
    if (k < nl) lut[k] = find_draw(draws, seg.first_draw, seg.num_draws, k * 256u);
  }
}

extern "C" __global__ void __launch_bounds__(KZ_THREADS) kz_k_scan(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  __shared__ uint32_t sh[KZ_THREADS + 1];
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  scan_tiles(c, s, sh);
}

extern "C" __global__ void __launch_bounds__(KZ_THREADS) kz_k_bin(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  uint32_t n = min(c.cnt->rec_count, c.seg->rec_cap);
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
    uint32_t i = i0 + threadIdx.x;
    bin_record(c, i, i < n);
  }
}

/* 4 blocks per SM (at most 64 registers, some spilled): measured on the ordered blend workload at 2.90 ms
 * against 3.44 (3 blocks, 85 registers), 3.78 (2 blocks, 128 registers) and 3.06 (5 blocks) */
/* the next tile for this block of a tile-raster kernel: the segment's tile cursor indexes the tile order the
 * scan wrote (largest bins first), so blocks that finish early take more tiles and the tail is made of small
 * bins (bins differ by tens of times in size); `slot` is a shared word of the block */
__device__ __forceinline__ uint32_t next_tile(const Ctx& c, uint32_t& slot) {
  if (threadIdx.x == 0) {
    const uint32_t k = atomicAdd(&c.cnt->tile_next, 1u), n = c.seg->tiles_x * c.seg->tiles_y;
    slot = k < n && c.seg->tile_order ? reinterpret_cast<const uint32_t*>(c.seg->tile_order)[k] : k;
  }
  __syncthreads();
  const uint32_t t = slot;
  __syncthreads();
  return t;
}

extern "C" __global__ void __launch_bounds__(KZ_THREADS, 4) kz_k_raster(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float u8tab[KZ_CTAB_FLOATS];
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  fill_color_tabs(u8tab);
  uint32_t ntiles = c.seg->tiles_x * c.seg->tiles_y;
  __shared__ uint32_t tnext;
  for (;;) {
    const uint32_t t = next_tile(c, tnext);
    if (t >= ntiles) break;
    raster_tile(c, t, smem, u8tab);
  }
}

/* kz_k_raster for the common ordered segment -- one sample per pixel, D32 depth, tiles of at most 16x16, and
 * pipelines that call no fragment-shader function (none, or one that only copies the interpolated colour):
 * a kernel with only that instance of the tile raster, so that its register allocation serves it alone;
 * each tile's colour and depth are staged in shared memory by TMA tensor copies where the segment has
 * tensor maps */
/* the ordered tile raster of one segment kind as a kernel of its own, so that its registers serve that
 * instance alone: DS, a D16 / D24S8 attachment with one sample per pixel (tiles of at most 16 x 16); MS, four
 * samples per pixel */
template <bool DS, bool MS>
__device__ __forceinline__ void raster_tiles_of(const KzFrame& f, uint32_t s, unsigned char* smem, float* u8tab) {
  kz_pdl_enter();
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  fill_color_tabs(u8tab);
  uint32_t ntiles = c.seg->tiles_x * c.seg->tiles_y;
  __shared__ uint32_t tnext;
  for (;;) {
    const uint32_t t = next_tile(c, tnext);
    if (t >= ntiles) break;
    raster_tile_ordered<1, DS, MS, true>(c, t, smem, u8tab, 0);
    __syncthreads();
    if (threadIdx.x == 0) reinterpret_cast<uint32_t*>(c.seg->tile_count)[t] = 0; /* as raster_tile leaves it */
  }
}
extern "C" __global__ void __launch_bounds__(KZ_THREADS, 4) kz_k_raster_ds(KzFrame f, uint32_t s) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float u8tab[KZ_CTAB_FLOATS];
  raster_tiles_of<true, false>(f, s, smem, u8tab);
}
extern "C" __global__ void __launch_bounds__(KZ_THREADS, 4) kz_k_raster_ms(KzFrame f, uint32_t s) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float u8tab[KZ_CTAB_FLOATS];
  raster_tiles_of<false, true>(f, s, smem, u8tab);
}
extern "C" __global__ void __launch_bounds__(KZ_THREADS, 4) kz_k_raster_direct(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float u8tab[KZ_CTAB_FLOATS];
  /* the tile's framebuffer block (tiles of at most 16 x 16 texels) */
  __shared__ __align__(128) uint32_t tile_color[16 * 16];
  __shared__ __align__(128) float tile_depth[16 * 16];
  __shared__ __align__(8) uint64_t tile_mbar;
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  fill_color_tabs(u8tab);
  if (threadIdx.x == 0) mbar_init(&tile_mbar, 1);
  __syncthreads();
  TileStage ts;
  ts.color = tile_color;
  ts.depth = tile_depth;
  ts.mbar = &tile_mbar;
  ts.phase = 0;
  uint32_t ntiles = c.seg->tiles_x * c.seg->tiles_y;
  __shared__ uint32_t tnext;
  for (;;) {
    const uint32_t t = next_tile(c, tnext);
    if (t >= ntiles) break;
    if (!raster_tile_ordered<1, false, false, false, true>(c, t, smem, u8tab, 0, &ts)) return;
    __syncthreads();
    if (threadIdx.x == 0) reinterpret_cast<uint32_t*>(c.seg->tile_count)[t] = 0; /* as raster_tile leaves it */
  }
}

extern "C" __global__ void __launch_bounds__(KZ_THREADS) kz_k_vis_init(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  vis_init_range(*c.seg, (size_t)blockIdx.x * blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}

extern "C" __global__ void __launch_bounds__(KZ_THREADS, 4) kz_k_vis_geometry(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  __shared__ __align__(16) unsigned char slots[KZ_GEO_SMEM];
  __shared__ uint32_t magic_tab[KZ_MAGIC_MAX + 1];
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  fill_magic(magic_tab);
  __syncthreads();
  vis_geometry_warps(c, slots, magic_tab, blockIdx.x * (KZ_THREADS / 32) + (threadIdx.x >> 5),
                     gridDim.x * (KZ_THREADS / 32));
}

/* 4 blocks per SM: 0.313 ms on the 4,096-draw workload against 0.357 (3 blocks) and 0.341 (5 blocks) */
/* With f.jobs_incremental (the per-draw launch form: one launch after each draw's geometry), a launch takes
 * the jobs [large_done, pair_count) and its last block to finish moves large_done to pair_count for the next
 * launch; otherwise it takes all of the segment's jobs. */
extern "C" __global__ void __launch_bounds__(KZ_THREADS, 4) kz_k_vis_large(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s) || !vis_check(c, s)) return;
  const uint32_t njobs = c.cnt->pair_count;
  const uint32_t j0 = f.jobs_incremental ? *reinterpret_cast<volatile uint32_t*>(&c.cnt->large_done) : 0u;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5), w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  vis_large_phase(c, j0, njobs, w, warps);
  if (f.jobs_incremental) {
    __syncthreads();
    if (threadIdx.x == 0 && atomicAdd(&c.cnt->large_blocks, 1u) == gridDim.x - 1) {
      c.cnt->large_done = njobs;
      c.cnt->large_blocks = 0;
    }
  }
}

/* 4 blocks per SM (64 registers, the most its fragment-shader callee allows at 5 is 51): 0.155 ms against
 * 0.162 at 3 resident blocks */
extern "C" __global__ void __launch_bounds__(KZ_THREADS, 4) kz_k_vis_resolve(KzFrame f, uint32_t s) {
  kz_pdl_enter();
  Ctx c = make_ctx(f, s);
  if (segment_blocked(c, s)) return;
  vis_resolve_phase(c, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), gridDim.x * (blockDim.x >> 5));
}

/* The phases of visibility segment s inside a persistent kernel: key init, geometry, large-triangle jobs
 * and resolve, separated by grid barriers.  Pixels, 32-triangle groups, jobs and row runs are strided
 * statically over the grid's warps, as the separate kernels stride them.  Returns 0 to go on with the next
 * segment, 1 when the segment's scratch overflowed (every block stops at the same segment, the host replays
 * from it), 2 when a barrier gave up (the kernel ends).  `last`: no barrier after the resolve. */
__device__ int persistent_vis_segment(const KzFrame& f, uint32_t s, unsigned char* geo_smem,
                                      const uint32_t* magic_tab, bool last) {
  Ctx c = make_ctx(f, s);
  KzStatus* st = c.st;
  const uint32_t warps = gridDim.x * (KZ_THREADS / 32), w = blockIdx.x * (KZ_THREADS / 32) + (threadIdx.x >> 5);
  vis_init_range(*c.seg, (size_t)blockIdx.x * blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
  if (!grid_barrier(st, f.barrier_ns)) return 2;
  vis_geometry_warps(c, geo_smem, magic_tab, w, warps);
  if (!grid_barrier(st, f.barrier_ns)) return 2;
  if (!vis_check(c, s)) return 1;
  vis_large_phase(c, 0, c.cnt->pair_count, w, warps);
  if (!grid_barrier(st, f.barrier_ns)) return 2;
  vis_resolve_phase(c, w, warps);
  if (!last && !grid_barrier(st, f.barrier_ns)) return 2;
  return 0;
}

/* the whole command buffer in one cooperative launch: phases separated by bounded grid barriers; ordered
 * segments take their chunks, records and tiles from per-segment work-stealing counters */
extern "C" __global__ void __launch_bounds__(KZ_THREADS, 3) kz_k_persistent(KzFrame f) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t item;
  __shared__ uint32_t scan_sh[KZ_THREADS + 1];
  __shared__ uint32_t geo_sh[40];
  __shared__ float u8tab[KZ_CTAB_FLOATS];
  __shared__ uint32_t magic_tab[KZ_MAGIC_MAX + 1];
  fill_color_tabs(u8tab);
  fill_magic(magic_tab);
  KzStatus* st = reinterpret_cast<KzStatus*>(f.status);
  for (uint32_t s = f.first_segment; s < f.num_segments; s++) {
    Ctx c = make_ctx(f, s);
    if (segment_blocked(c, s)) break;
    if (c.seg->mode == KZ_MODE_VISIBILITY) {
      __syncthreads();
      const int r = persistent_vis_segment(f, s, smem, magic_tab, false);
      if (r == 2) return;
      if (r == 1) break;
      continue;
    }
    for (;;) {
      uint32_t k = grab(&c.cnt->geom_next, &item);
      if (k >= c.seg->num_chunks) break;
      geometry_chunk(c, k, geo_sh);
    }
    if (!grid_barrier(st, f.barrier_ns)) return;
    if (blockIdx.x == 0) scan_tiles(c, s, scan_sh);
    if (!grid_barrier(st, f.barrier_ns)) return;
    if (segment_blocked(c, s)) break;
    uint32_t n = min(c.cnt->rec_count, c.seg->rec_cap);
    for (;;) {
      uint32_t k = grab(&c.cnt->bin_next, &item);
      uint32_t i = k * blockDim.x + threadIdx.x;
      if (k * blockDim.x >= n) break;
      bin_record(c, i, i < n);
    }
    if (!grid_barrier(st, f.barrier_ns)) return;
    uint32_t ntiles = c.seg->tiles_x * c.seg->tiles_y;
    for (;;) {
      uint32_t t = next_tile(c, item);
      if (t >= ntiles) break;
      raster_tile(c, t, smem, u8tab);
    }
    if (!grid_barrier(st, f.barrier_ns)) return;
  }
}

/* the persistent form of passes whose segments are all opaque (visibility mode): only the visibility
 * phases, so the kernel keeps the 64-register budget and the 4 resident blocks per SM of the separate
 * kernels; the last segment ends without a barrier */
extern "C" __global__ void __launch_bounds__(KZ_THREADS, 4) kz_k_persistent_vis(KzFrame f) {
  __shared__ __align__(16) unsigned char slots[KZ_GEO_SMEM];
  __shared__ uint32_t magic_tab[KZ_MAGIC_MAX + 1];
  fill_magic(magic_tab);
  __syncthreads();
  for (uint32_t s = f.first_segment; s < f.num_segments; s++) {
    Ctx c = make_ctx(f, s);
    if (segment_blocked(c, s)) break;
    if (persistent_vis_segment(f, s, slots, magic_tab, s + 1 == f.num_segments) != 0) return;
  }
}

/* vkCmdClearColorImage / vkCmdClearDepthStencilImage / render-pass clears outside the raster:
 * fill rows [y0, y1) x [x0, x1) of a 4-byte-per-pixel image with `value` (16-byte stores where the
 * row segment is aligned) */
/* multisample resolve of a w x h rectangle: per pixel and byte, (sum of the KZ_MS_SAMPLES samples + 2) / 4 */
extern "C" __global__ void __launch_bounds__(KZ_THREADS) kz_k_resolve(uint64_t src, uint32_t spitch, int32_t sx,
                                                                      int32_t sy, uint64_t dst, uint32_t dpitch,
                                                                      int32_t dx, int32_t dy, int32_t w, int32_t h) {
  kz_pdl_enter();
  const long long total = (long long)w * h;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    int32_t x = (int32_t)(i % w), y = (int32_t)(i / w);
    /* four 32-bit loads: an image bound at any 4-byte memory offset keeps them aligned */
    const uint32_t* p = reinterpret_cast<const uint32_t*>(reinterpret_cast<const char*>(src) + (size_t)(sy + y) * spitch +
                                                          (size_t)(sx + x) * 16u);
    const uint4 s = make_uint4(p[0], p[1], p[2], p[3]);
    uint32_t out = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      uint32_t sum = 2u + ((s.x >> (8 * c)) & 0xFFu) + ((s.y >> (8 * c)) & 0xFFu) + ((s.z >> (8 * c)) & 0xFFu) +
                     ((s.w >> (8 * c)) & 0xFFu);
      out |= (sum >> 2) << (8 * c);
    }
    *reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(dst) + (size_t)(dy + y) * dpitch + (size_t)(dx + x) * 4u) = out;
  }
}

extern "C" __global__ void __launch_bounds__(KZ_THREADS) kz_k_clear(uint64_t base, uint32_t pitch, int32_t x0,
                                                                    int32_t y0, int32_t x1, int32_t y1,
                                                                    uint32_t value) {
  kz_pdl_enter();
  int32_t w = x1 - x0, h = y1 - y0;
  if (w <= 0 || h <= 0) return;
  int32_t lead = (int32_t)((4 - (x0 & 3)) & 3);
  if (lead > w) lead = w;
  int32_t body = (w - lead) / 4;
  int32_t tail = w - lead - body * 4;
  int32_t per_row = lead + body + tail;
  long long total = (long long)per_row * h;
  uint4 v4 = make_uint4(value, value, value, value);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    int32_t y = y0 + (int32_t)(i / per_row);
    int32_t k = (int32_t)(i % per_row);
    uint32_t* row = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(base) + (size_t)y * pitch);
    if (k < lead) {
      row[x0 + k] = value;
    } else if (k < lead + body) {
      int32_t x = x0 + lead + (k - lead) * 4;
      if ((reinterpret_cast<uintptr_t>(row + x) & 15u) == 0) {
        *reinterpret_cast<uint4*>(row + x) = v4;
      } else {
        row[x] = value; row[x + 1] = value; row[x + 2] = value; row[x + 3] = value;
      }
    } else {
      row[x0 + lead + body * 4 + (k - lead - body)] = value;
    }
  }
}
