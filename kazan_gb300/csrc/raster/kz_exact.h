/*
 * kz_exact.h - exact integer helpers shared by the pipeline kernels and their CPU test (tests/test_exact.py).
 *
 * kz_i64_to_f32: round-to-nearest-even conversion of a 64-bit integer to binary32, computed with integer
 * operations only.  It returns the same bits as the IEEE conversion (C's (float)x under the default
 * rounding mode, CUDA's __ll2float_rn); on sm_103a the hardware 64-bit integer conversion issues on the
 * FP64 pipe, which this avoids.
 */
#ifndef KZ_EXACT_H
#define KZ_EXACT_H

#include <stdint.h>

#if defined(__CUDACC__)
#define KZ_HD __host__ __device__ __forceinline__
#else
#define KZ_HD static inline
#endif

KZ_HD int kz_clz64(uint64_t a) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)a);
#else
  return a ? __builtin_clzll(a) : 64;
#endif
}

KZ_HD uint32_t kz_i64_to_f32_bits(int64_t v) {
  if (v == 0) return 0;
  uint32_t sign = v < 0 ? 0x80000000u : 0u;
  uint64_t a = v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
  int msb = 63 - kz_clz64(a);
  uint64_t m;
  if (msb <= 23) {
    m = a << (23 - msb);
  } else {
    int shift = msb - 23;
    m = a >> shift;
    uint64_t rem = a & ((1ull << shift) - 1ull);
    uint64_t half = 1ull << (shift - 1);
    if (rem > half || (rem == half && (m & 1ull))) m++;
    if (m == (1ull << 24)) {
      m >>= 1;
      msb++;
    }
  }
  return sign | ((uint32_t)(msb + 127) << 23) | ((uint32_t)m & 0x7FFFFFu);
}

#if defined(__CUDACC__)
__device__ __forceinline__ float kz_i64_to_f32(int64_t v) {
  /* values that fit in 32 bits use the native conversion (same rounding) */
  if (v == (int64_t)(int32_t)v) return __int2float_rn((int32_t)v);
  return __uint_as_float(kz_i64_to_f32_bits(v));
}
#endif

#endif
