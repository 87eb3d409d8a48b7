/*
 * kz_oracle.h - CPU oracle for the kazan draw path.  TEST INFRASTRUCTURE ONLY.
 *
 * This is the checker the GPU path is compared against; it is never linked into, called by or
 * shipped with the driver.  Only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.
 *
 * PARITY UNPINNED: the reference driver has no rasteriser.  vkCmdDraw, vkCmdDrawIndexed and
 * vkCmdClearColorImage are `unimplemented!()` (vulkan-driver/src/api_impl.rs:4632-4653,4780-4790),
 * no reference test renders anything (vulkan-driver/src/lib.rs:134-135 is an empty test module), and
 * the reference cannot be built here (no Rust toolchain).  This oracle therefore restates the
 * rasterisation rules of the Vulkan specification, with the choices the specification leaves open
 * fixed as follows (the GPU kernels make the same choices):
 *   - viewport transform xf = fma(x/w, w/2, x0 + w/2) in f32, with x/w computed as x * (1/w);
 *   - 8 sub-pixel bits: X = rint(xf * 256) (round to nearest even), int32;
 *   - samples at pixel centres (x*256+128, y*256+128); exact int64 edge functions;
 *   - top-left fill rule in framebuffer space (y down): an edge a->b of a triangle with positive
 *     signed area S is "top-left" iff dy < 0, or dy == 0 and dx > 0;
 *   - facing per Vulkan: area a = -S/2; VK_FRONT_FACE_COUNTER_CLOCKWISE means a > 0 is front;
 *   - clipping against z >= 0, z <= w and a guard band |x|,|y| <= 4w (Sutherland-Hodgman, planes in
 *     that order, new vertices interpolated from the inside vertex towards the outside one);
 *   - screen-space barycentrics l_i = (float)E_i * (1/(float)S); depth z0 + l1 dz1 + l2 dz2 by fma,
 *     clamped to the viewport depth range; perspective-correct varyings divided by the interpolated 1/w;
 *   - UNORM8 stores rint(clamp(c, 0, 1) * 255); blending in f32 with dst = u8 / 255;
 *   - 8-bit sRGB attachments store the sRGB transfer function's code of red, green and blue and blend
 *     with their decoded values, both from kazan_gb300/csrc/kz_srgb_table.h (generated in 60-digit
 *     decimal arithmetic; tests/test_srgb.py checks it against the transfer function in float64).
 * Every float operation is an explicit IEEE single operation (built with -ffp-contract=off and fmaf
 * where the GPU fuses), so results are bit-identical to the kernels.
 */
#ifndef KZ_ORACLE_H
#define KZ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { KZO_SHADER_COLOR = 0, KZO_SHADER_LAMBERT = 1, KZO_SHADER_TEXTURED = 2 };

/* depth attachment formats: the depth plane holds what the depth test compares, D32 the float depth,
 * D16 / D24 the integer rint(z * (2^bits - 1)) (exact in a float) */
enum { KZO_DEPTH_D32 = 0, KZO_DEPTH_D16 = 1, KZO_DEPTH_D24S8 = 2 };

/* VkStencilOpState */
typedef struct kzo_stencil {
  uint32_t fail_op, pass_op, depth_fail_op, compare_op;
  uint32_t compare_mask, write_mask, reference;
} kzo_stencil;

/* a combined image sampler of one mip level (the GPU's KzDescriptor): RGBA8 or BGRA8 UNORM texels */
typedef struct kzo_texture {
  const uint8_t* texels;    /* texel (0, 0) */
  uint32_t width, height;
  uint32_t pitch;           /* bytes per row */
  uint32_t format;          /* 1: RGBA8, 2: BGRA8 */
  uint32_t sampler;         /* bit 0 LINEAR, bit 1 unnormalized coordinates, bits 4..6 / 8..10 address mode u / v
                               (VkSamplerAddressMode), bits 12..13 border (0 transparent black, 1 opaque
                               black, 2 opaque white) */
} kzo_texture;

typedef struct kzo_draw {
  uint32_t shader;          /* KZO_SHADER_COLOR: pos f32x4 + rgba f32x4 (8 floats per vertex);
                               KZO_SHADER_LAMBERT: pos f32x3 + normal f32x3 (6 floats per vertex);
                               KZO_SHADER_TEXTURED: pos f32x4 + uv f32x2 (6 floats per vertex) */
  const float* vertices;
  const uint32_t* indices;  /* NULL for vkCmdDraw */
  uint32_t first;           /* firstVertex (vkCmdDraw) or firstIndex (vkCmdDrawIndexed) */
  int32_t vertex_offset;    /* vkCmdDrawIndexed vertexOffset */
  uint32_t tri_count;
  float mvp[16];            /* column-major, LAMBERT vertex shader */
  float albedo[3];          /* LAMBERT fragment shader constants */
  float light[3];
  uint32_t cull_mode;       /* VkCullModeFlags */
  uint32_t front_ccw;
  uint32_t depth_test, depth_write, depth_compare; /* VkCompareOp */
  uint32_t blend_enable;
  uint32_t src_color, dst_color, color_op, src_alpha, dst_alpha, alpha_op;
  uint32_t write_mask;
  float blend_const[4];
  float viewport[6];        /* x, y, width, height, minDepth, maxDepth */
  int32_t scissor[4];       /* x, y, width, height */
  kzo_texture tex;          /* TEXTURED fragment shader: colour = texture(tex, uv) */
  uint32_t stencil_test;    /* stencil test against the stencil plane (D24S8 targets) */
  kzo_stencil front, back;
  uint32_t samples;         /* 0 or 1: one sample at the pixel centre; 4: the standard 4x positions (96, 32),
                               (224, 96), (32, 160), (160, 224) in 1/256 pixel, colour and depth planes holding
                               4 samples per pixel (sample s of pixel p at p * 4 + s), coverage, depth and
                               colour per sample, the fragment shader once per pixel at its centre (only D32,
                               no stencil) */
  uint32_t srgb;            /* 1: the colour attachment is 8-bit sRGB: red, green and blue are stored as sRGB
                               codes (the Vulkan specification's sRGB transfer function, rounded to nearest)
                               and decoded to linear before blending; alpha stays linear */
} kzo_draw;

typedef struct kzo_stats {
  uint64_t tris;            /* triangles submitted */
  uint64_t rejected;        /* trivially rejected, culled, degenerate or empty */
  uint64_t clipped;         /* triangles that needed clipping */
  uint64_t subtris;         /* (sub-)triangles rasterised */
  uint64_t fragments;       /* covered samples inside the pixel rectangle, before the depth test */
  uint64_t depth_pass;      /* fragments that passed the depth test */
} kzo_stats;

/* Render draws in order into an RGBA8 colour image (width*height*4 bytes, row-major) and an optional
 * D32 depth image.  render_area = x0, y0, x1, y1 (exclusive).  nthreads <= 1 runs the plain in-order
 * loop; nthreads > 1 runs setup in parallel over triangles and rasterises horizontal bands in parallel
 * (each band walks the triangles in API order, so the result is identical). */
int kzo_render(uint32_t width, uint32_t height, uint8_t* color, float* depth, const int32_t render_area[4],
               uint32_t num_draws, const kzo_draw* draws, int nthreads, kzo_stats* stats);

/* kzo_render with a depth plane in `depth_format` and an optional 8-bit stencil plane (width * height).
 * Per fragment, in order: stencil test (reference & compare mask against stored & compare mask; on
 * failure failOp and the fragment ends), depth test (on failure depthFailOp and the fragment ends),
 * passOp, fragment shader, depth write, colour; ops write through the write mask. */
int kzo_render_ds(uint32_t width, uint32_t height, uint8_t* color, float* depth, uint8_t* stencil,
                  uint32_t depth_format, const int32_t render_area[4], uint32_t num_draws, const kzo_draw* draws,
                  int nthreads, kzo_stats* stats);

/* the multisample resolve: per pixel and byte, (sum of the 4 samples + 2) / 4 */
void kzo_resolve(uint32_t width, uint32_t height, const uint8_t* color4, uint8_t* color);

/* the value a depth of z is compared and stored as in `depth_format` */
float kzo_depth_value(float z, uint32_t depth_format);

/* vkCmdClearColorImage / vkCmdClearDepthStencilImage restated for a rectangle */
void kzo_clear_color(uint32_t width, uint8_t* color, const int32_t rect[4], const float rgba[4]);

/* the 8-bit sRGB code of linear v, and the clear of an sRGB colour image (sRGB red, green, blue; linear
 * alpha) */
uint8_t kzo_srgb8(float v);
void kzo_clear_color_srgb(uint32_t width, uint8_t* color, const int32_t rect[4], const float rgba[4]);
void kzo_clear_depth(uint32_t width, float* depth, const int32_t rect[4], float value);

/* f32 -> UNORM8 as the driver stores it */
uint8_t kzo_unorm8(float v);

/* OpImageSample* on `t` at (s, t): NEAREST texel (floor u, floor v), or LINEAR
 * lerp(lerp(t00, t10, a), lerp(t01, t11, a), b) around (u - 0.5, v - 0.5) with lerp(x, y, f) = x + f * (y - x),
 * each operation rounded separately; u = s * width unless unnormalized; texels c / 255; the Vulkan
 * specification's wrapping operation per address mode */
void kzo_tex2d(const kzo_texture* t, float s, float tc, float out[4]);

/* pixel rectangle of a draw: framebuffer & render area & scissor & viewport (x0, y0, x1, y1 exclusive) */
void kzo_draw_rect(uint32_t width, uint32_t height, const int32_t render_area[4], const kzo_draw* d,
                   int32_t out[4]);

#ifdef __cplusplus
}
#endif

#endif
