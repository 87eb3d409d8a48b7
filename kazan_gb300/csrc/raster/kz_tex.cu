/*
 * kz_tex.cu - texture sampling functions the JIT-linked fragment and vertex shaders call (OpImageSample*,
 * OpImageFetch): kz_tex2d and kz_tex_fetch.
 *
 * A separate relocatable object from the pipeline kernels (kz_pipeline.cu), compiled with -maxrregcount=64:
 * the linker rejects a callee that needs more registers than its calling kernel allows, and the ordered
 * tile raster runs 4 blocks of 256 threads per SM (at most 64 registers).  The kernels do not call these
 * functions themselves; nvJitLink links both objects with each pipeline set's shader PTX.
 *
 * Arithmetic: every float operation an explicit IEEE single operation (built with -fmad=false and the
 * __f*_rn intrinsics), the rule the CPU oracle's kzo_tex2d restates.
 */
#include <stdint.h>

#include "../kz_raster_abi.h"

/* ---------------- texture sampling (called by the JIT-linked shaders) ---------------- */

/* texel index after the sampler's address mode (the Vulkan specification's wrapping operation); -1 when
 * the index falls on the border (CLAMP_TO_BORDER) */
__device__ __forceinline__ int32_t kz_tex_wrap(int32_t i, int32_t size, uint32_t mode) {
  switch (mode) {
    case 0: { /* REPEAT */
      int32_t m = i % size;
      return m < 0 ? m + size : m;
    }
    case 1: { /* MIRRORED_REPEAT: (size - 1) - mirror((i mod 2 size) - size) */
      int32_t m = i % (2 * size);
      if (m < 0) m += 2 * size;
      m -= size;
      int32_t mir = m >= 0 ? m : -(1 + m);
      return size - 1 - mir;
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

/* a floored coordinate as an integer, NaN and values beyond +-1e9 clamped (fmaxf/fminf return the other
 * operand of a NaN) */
__device__ __forceinline__ int32_t kz_tex_int(float x) { return (int32_t)fminf(fmaxf(x, -1.0e9f), 1.0e9f); }

/* the 32-bit texel word at (i, j), or the border colour as a word (transparent black 0, opaque black
 * 0xFF000000, opaque white 0xFFFFFFFF: its bytes convert to exactly 0.0 and 1.0, the same in either
 * byte order) */
__device__ __forceinline__ uint32_t kz_tex_word(const KzDescriptor& d, int32_t i, int32_t j) {
  if (i < 0 || j < 0) {
    uint32_t b = (d.sampler >> KZ_SAMP_BORDER_SHIFT) & 3u;
    return b == 0 ? 0u : (b == 1 ? 0xFF000000u : 0xFFFFFFFFu);
  }
  return __ldg(reinterpret_cast<const uint32_t*>(d.addr + (uint64_t)j * d.pitch + (uint64_t)i * 4u));
}

/* channel k (0 r, 1 g, 2 b, 3 a) of a texel word as c / 255 (IEEE division) */
__device__ __forceinline__ float kz_tex_channel(uint32_t w, uint32_t format, int k) {
  int byte = (format == KZ_CF_BGRA8 && k < 3) ? 2 - k : k;
  return __fdiv_rn((float)((w >> (8 * byte)) & 0xFFu), 255.0f);
}

__device__ __forceinline__ float kz_tex_lerp(float a, float b, float t) {
  return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a)));
}

/* OpImageFetch (texelFetch) of texel (i, j); outside the image (0, 0, 0, 0), as robust image access
 * returns */
extern "C" __device__ __noinline__ float4 kz_tex_fetch(const KzDescriptor* desc, int32_t i, int32_t j) {
  const KzDescriptor d = *desc;
  if (i < 0 || j < 0 || i >= (int32_t)d.width || j >= (int32_t)d.height) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  uint32_t w = kz_tex_word(d, i, j);
  return make_float4(kz_tex_channel(w, d.format, 0), kz_tex_channel(w, d.format, 1), kz_tex_channel(w, d.format, 2),
                     kz_tex_channel(w, d.format, 3));
}

/* OpImageSample* on a combined image sampler of one mip level: coordinates scaled by the image size
 * (unless unnormalized); NEAREST takes texel (floor u, floor v); LINEAR takes the four texels around
 * (u - 0.5, v - 0.5) and blends them with the fractions a, b as lerp(lerp(t00, t10, a), lerp(t01, t11, a), b),
 * every operation a separately rounded IEEE single operation (the CPU oracle's kzo_tex2d is the same). */
extern "C" __device__ __noinline__ float4 kz_tex2d(const KzDescriptor* desc, float s, float t) {
  const KzDescriptor d = *desc;
  const int32_t w = (int32_t)d.width, h = (int32_t)d.height;
  const uint32_t mu = (d.sampler >> KZ_SAMP_ADDR_U_SHIFT) & 7u, mv = (d.sampler >> KZ_SAMP_ADDR_V_SHIFT) & 7u;
  float u = s, v = t;
  if (!(d.sampler & KZ_SAMP_UNNORMALIZED)) {
    u = __fmul_rn(s, (float)w);
    v = __fmul_rn(t, (float)h);
  }
  float c[4];
  if (!(d.sampler & KZ_SAMP_LINEAR)) {
    uint32_t t0 = kz_tex_word(d, kz_tex_wrap(kz_tex_int(floorf(u)), w, mu), kz_tex_wrap(kz_tex_int(floorf(v)), h, mv));
#pragma unroll
    for (int k = 0; k < 4; k++) c[k] = kz_tex_channel(t0, d.format, k);
    return make_float4(c[0], c[1], c[2], c[3]);
  }
  float u0 = __fsub_rn(u, 0.5f), v0 = __fsub_rn(v, 0.5f);
  float fi = floorf(u0), fj = floorf(v0);
  float a = fminf(fmaxf(__fsub_rn(u0, fi), 0.0f), 1.0f), b = fminf(fmaxf(__fsub_rn(v0, fj), 0.0f), 1.0f);
  int32_t i0 = kz_tex_int(fi), j0 = kz_tex_int(fj);
  int32_t x0 = kz_tex_wrap(i0, w, mu), x1 = kz_tex_wrap(i0 + 1, w, mu);
  int32_t y0 = kz_tex_wrap(j0, h, mv), y1 = kz_tex_wrap(j0 + 1, h, mv);
  uint32_t t00 = kz_tex_word(d, x0, y0), t10 = kz_tex_word(d, x1, y0);
  uint32_t t01 = kz_tex_word(d, x0, y1), t11 = kz_tex_word(d, x1, y1);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float top = kz_tex_lerp(kz_tex_channel(t00, d.format, k), kz_tex_channel(t10, d.format, k), a);
    float bot = kz_tex_lerp(kz_tex_channel(t01, d.format, k), kz_tex_channel(t11, d.format, k), a);
    c[k] = kz_tex_lerp(top, bot, b);
  }
  return make_float4(c[0], c[1], c[2], c[3]);
}

