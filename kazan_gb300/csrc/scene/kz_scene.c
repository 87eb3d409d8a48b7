/*
 * kz_scene.c - seeded synthetic scenes for the draw-path workloads.
 *
 * The reference publishes no benchmark scenes (its draw path is unimplemented,
 * vulkan-driver/src/api_impl.rs:4632-4653), so the workloads are synthetic and fully determined by a
 * seed.  Random numbers: splitmix64 (Steele, Lea, Flood 2014) expands the seed into the state and
 * stream of a PCG32 generator (O'Neill 2014, XSH-RR output); a float is (u32 >> 8) * 2^-24 in [0, 1).
 *
 *   small soup   : n triangles, clip-space x,y in [-1,1], z in [0,1], w = 1, RGBA in [0,1]
 *                  (8 floats per vertex: position then colour)
 *   blend soup   : n triangles with log-uniform pixel area, random centroid, alpha 0.5
 *   sphere mesh  : jittered latitude/longitude grid on the unit sphere, random unit normals
 *                  (6 floats per vertex: position then normal), u32 triangle-list indices
 *   cameras      : perspective (Vulkan clip space: y down, depth 0..1) model-view-projection matrices
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define KZ_EXPORT __attribute__((visibility("default")))

typedef struct {
  uint64_t state, inc;
} kz_pcg32;

static uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint32_t pcg_next(kz_pcg32* r) {
  uint64_t old = r->state;
  r->state = old * 6364136223846793005ull + r->inc;
  uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return (xorshifted >> rot) | (xorshifted << ((-rot) & 31u));
}

static void pcg_seed(kz_pcg32* r, uint64_t seed) {
  uint64_t s = seed;
  uint64_t init_state = splitmix64(&s);
  uint64_t init_seq = splitmix64(&s);
  r->state = 0;
  r->inc = (init_seq << 1u) | 1u;
  pcg_next(r);
  r->state += init_state;
  pcg_next(r);
}

static float pcg_float(kz_pcg32* r) { return (float)(pcg_next(r) >> 8) * (1.0f / 16777216.0f); }

KZ_EXPORT uint32_t kz_rng_first(uint64_t seed) {
  kz_pcg32 r;
  pcg_seed(&r, seed);
  return pcg_next(&r);
}

KZ_EXPORT void kz_rng_floats(uint64_t seed, uint32_t n, float* out) {
  kz_pcg32 r;
  pcg_seed(&r, seed);
  for (uint32_t i = 0; i < n; i++) out[i] = pcg_float(&r);
}

/* small soup: 3n vertices, 8 floats each */
KZ_EXPORT void kz_scene_soup(uint64_t seed, uint32_t n, float* out) {
  kz_pcg32 r;
  pcg_seed(&r, seed);
  for (uint32_t v = 0; v < 3 * n; v++) {
    float* o = out + (size_t)v * 8;
    o[0] = pcg_float(&r) * 2.0f - 1.0f;
    o[1] = pcg_float(&r) * 2.0f - 1.0f;
    o[2] = pcg_float(&r);
    o[3] = 1.0f;
    for (int k = 0; k < 4; k++) o[4 + k] = pcg_float(&r);
  }
}

/* blend soup: 3n vertices, 8 floats each; pixel area log-uniform in [amin, amax] */
KZ_EXPORT void kz_scene_blend(uint64_t seed, uint32_t n, uint32_t width, uint32_t height, float amin, float amax,
                              float alpha, float* out) {
  kz_pcg32 r;
  pcg_seed(&r, seed);
  const double two_pi = 6.283185307179586;
  double la = log((double)amin), lb = log((double)amax);
  for (uint32_t t = 0; t < n; t++) {
    double area = exp(la + (lb - la) * pcg_float(&r));
    double cx = (double)width * pcg_float(&r), cy = (double)height * pcg_float(&r);
    double base = two_pi * pcg_float(&r);
    double px[3], py[3];
    for (int k = 0; k < 3; k++) {
      double ang = base + two_pi * k / 3.0 + (pcg_float(&r) - 0.5) * 1.2;
      double rad = 0.5 + 0.5 * pcg_float(&r);
      px[k] = rad * cos(ang);
      py[k] = rad * sin(ang);
    }
    double a0 = 0.5 * fabs((px[1] - px[0]) * (py[2] - py[0]) - (px[2] - px[0]) * (py[1] - py[0]));
    double s = a0 > 1e-9 ? sqrt(area / a0) : 0.0;
    for (int k = 0; k < 3; k++) {
      float* o = out + ((size_t)t * 3 + (size_t)k) * 8;
      double fx = cx + s * px[k], fy = cy + s * py[k];
      o[0] = (float)(2.0 * fx / (double)width - 1.0);
      o[1] = (float)(2.0 * fy / (double)height - 1.0);
      o[2] = pcg_float(&r);
      o[3] = 1.0f;
      o[4] = pcg_float(&r);
      o[5] = pcg_float(&r);
      o[6] = pcg_float(&r);
      o[7] = alpha;
    }
  }
}

/* sphere mesh dimensions for at least `tris` triangles: rows x cols cells, 2 triangles per cell */
KZ_EXPORT void kz_mesh_dims(uint32_t tris, uint32_t* rows, uint32_t* cols) {
  uint64_t cells = ((uint64_t)tris + 1) / 2;
  if (cells == 0) cells = 1;
  uint32_t rr = (uint32_t)floor(sqrt((double)cells / 2.0) + 0.5);
  if (rr < 1) rr = 1;
  uint32_t cc = (uint32_t)((cells + rr - 1) / rr);
  if (cc < 3) cc = 3;
  *rows = rr;
  *cols = cc;
}

KZ_EXPORT uint32_t kz_mesh_vertex_count(uint32_t tris) {
  uint32_t rr, cc;
  kz_mesh_dims(tris, &rr, &cc);
  return (rr + 1) * (cc + 1);
}

/* jittered lat/long grid on the unit sphere; polar caps of 0.04*pi left open.  Triangles wind so that
 * the outside is front-facing for VK_FRONT_FACE_COUNTER_CLOCKWISE under the cameras below. */
KZ_EXPORT void kz_mesh_sphere(uint64_t seed, uint32_t tris, float* verts, uint32_t* idx) {
  kz_pcg32 r;
  pcg_seed(&r, seed);
  uint32_t rows, cols;
  kz_mesh_dims(tris, &rows, &cols);
  const double pi = 3.141592653589793;
  const double th0 = 0.04 * pi, th1 = pi - 0.04 * pi;
  for (uint32_t i = 0; i <= rows; i++) {
    for (uint32_t j = 0; j <= cols; j++) {
      double ji = (double)(j % cols), ii = (double)i;
      float jx = pcg_float(&r), jy = pcg_float(&r);
      if (i > 0 && i < rows) ii += 0.35 * ((double)jy - 0.5);
      if (j > 0 && j < cols) ji += 0.35 * ((double)jx - 0.5);
      double th = th0 + (th1 - th0) * ii / (double)rows;
      double ph = 2.0 * pi * ji / (double)cols;
      float* o = verts + ((size_t)i * (cols + 1) + j) * 6;
      o[0] = (float)(sin(th) * cos(ph));
      o[1] = (float)(cos(th));
      o[2] = (float)(sin(th) * sin(ph));
      double nz = 2.0 * pcg_float(&r) - 1.0, nph = 2.0 * pi * pcg_float(&r);
      double s = sqrt(fmax(0.0, 1.0 - nz * nz));
      o[3] = (float)(s * cos(nph));
      o[4] = (float)(s * sin(nph));
      o[5] = (float)nz;
    }
  }
  uint32_t t = 0;
  for (uint32_t i = 0; i < rows && t < tris; i++) {
    for (uint32_t j = 0; j < cols && t < tris; j++) {
      uint32_t a = i * (cols + 1) + j, b = a + 1, c = a + (cols + 1), d = c + 1;
      idx[3 * t + 0] = a;
      idx[3 * t + 1] = b;
      idx[3 * t + 2] = c;
      t++;
      if (t >= tris) break;
      idx[3 * t + 0] = b;
      idx[3 * t + 1] = d;
      idx[3 * t + 2] = c;
      t++;
    }
  }
}

/* column-major 4x4 helpers in double */
static void mat_mul(const double* a, const double* b, double* out) {
  double t[16];
  for (int c = 0; c < 4; c++)
    for (int rr = 0; rr < 4; rr++) {
      double s = 0.0;
      for (int k = 0; k < 4; k++) s += a[k * 4 + rr] * b[c * 4 + k];
      t[c * 4 + rr] = s;
    }
  memcpy(out, t, sizeof(t));
}

/* Vulkan-style perspective: right-handed view space looking down -z, clip y down, depth 0..1 */
static void perspective(double fovy, double aspect, double zn, double zf, double* m) {
  double f = 1.0 / tan(fovy * 0.5);
  memset(m, 0, 16 * sizeof(double));
  m[0] = f / aspect;
  m[5] = -f;
  m[10] = zf / (zn - zf);
  m[11] = -1.0;
  m[14] = zn * zf / (zn - zf);
}

static void translate(double x, double y, double z, double* m) {
  memset(m, 0, 16 * sizeof(double));
  m[0] = m[5] = m[10] = m[15] = 1.0;
  m[12] = x;
  m[13] = y;
  m[14] = z;
}

static void to_f32(const double* m, float* out) {
  for (int i = 0; i < 16; i++) out[i] = (float)m[i];
}

/* single large draw: sphere at the origin, camera on +z at `dist`, fov 60 degrees, near 0.1, far 100 */
KZ_EXPORT void kz_mvp_single(uint32_t width, uint32_t height, double dist, float* out) {
  double p[16], v[16], m[16];
  perspective(60.0 * 3.141592653589793 / 180.0, (double)width / (double)height, 0.1, 100.0, p);
  translate(0.0, 0.0, -dist, v);
  mat_mul(p, v, m);
  to_f32(m, out);
}

/* batched draws: per draw a uniform random rotation (Shoemake) and translation in [-5,5]^3; camera on
 * +z at distance 20; seed ^ draw selects the stream */
KZ_EXPORT void kz_mvp_batched(uint64_t seed, uint32_t draw, uint32_t width, uint32_t height, float* out) {
  kz_pcg32 r;
  pcg_seed(&r, seed ^ ((uint64_t)draw * 0x9E3779B97F4A7C15ull + 1));
  const double pi = 3.141592653589793;
  double u1 = pcg_float(&r), u2 = pcg_float(&r), u3 = pcg_float(&r);
  double a = sqrt(1.0 - u1), b = sqrt(u1);
  double qx = a * sin(2 * pi * u2), qy = a * cos(2 * pi * u2), qz = b * sin(2 * pi * u3), qw = b * cos(2 * pi * u3);
  double rot[16] = {1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy + qz * qw), 2 * (qx * qz - qy * qw), 0,
                    2 * (qx * qy - qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz + qx * qw), 0,
                    2 * (qx * qz + qy * qw), 2 * (qy * qz - qx * qw), 1 - 2 * (qx * qx + qy * qy), 0,
                    0, 0, 0, 1};
  double tx = 10.0 * pcg_float(&r) - 5.0, ty = 10.0 * pcg_float(&r) - 5.0, tz = 10.0 * pcg_float(&r) - 5.0;
  double t[16], model[16], p[16], v[16], pv[16], m[16];
  translate(tx, ty, tz, t);
  mat_mul(t, rot, model);
  perspective(60.0 * pi / 180.0, (double)width / (double)height, 0.1, 100.0, p);
  translate(0.0, 0.0, -20.0, v);
  mat_mul(p, v, pv);
  mat_mul(pv, model, m);
  to_f32(m, out);
}

/* per-draw triangle counts floor(exp(U[ln lo, ln hi])) */
KZ_EXPORT uint64_t kz_batched_counts(uint64_t seed, uint32_t ndraws, uint32_t lo, uint32_t hi, uint32_t* counts) {
  kz_pcg32 r;
  pcg_seed(&r, seed);
  double la = log((double)lo), lb = log((double)hi);
  uint64_t total = 0;
  for (uint32_t i = 0; i < ndraws; i++) {
    uint32_t c = (uint32_t)floor(exp(la + (lb - la) * pcg_float(&r)));
    if (c < lo) c = lo;
    if (c > hi) c = hi;
    counts[i] = c;
    total += c;
  }
  return total;
}
