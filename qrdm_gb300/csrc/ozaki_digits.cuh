// ozaki_digits.cuh -- the digit split shared by the Ozaki-scheme kernels:
// FP64 -> fixed point at a power-of-two scale, balanced base-256 digits
// exact in BF16, and the scalar helpers of the recombination.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace qrdm {

// round(x * 2^sh) as int64 (|result| < 2^62 by the caller's choice of sh)
__device__ __forceinline__ long long fixed_point(double x, int sh) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int E = (int)((b >> 52) & 0x7FF);
  long long M = (long long)(b & 0xFFFFFFFFFFFFFull);
  int e2;
  if (E == 0) {
    e2 = -1074 + sh;
  } else {
    M |= (1ll << 52);
    e2 = E - 1075 + sh;
  }
  long long F;
  if (e2 >= 0) {
    F = M << (e2 > 62 ? 62 : e2);
  } else if (e2 < -60) {
    F = 0;
  } else {
    F = (M + (1ll << (-e2 - 1))) >> (-e2);
  }
  return (b >> 63) ? -F : F;
}

// S balanced base-256 digits of F (d[0] most significant; the lower ones in
// [-128, 127]).  Adding 128 at every lower digit position makes those digits
// plain bytes of G = F + bias (no carries), so each is one byte extract:
// d = byte - 128; the top digit is G >> 8 (S - 1).
template <int S>
__device__ __forceinline__ void balanced_digits(long long F, int* d) {
  const long long G = F + (long long)(0x8080808080808080ull >> (8 * (9 - S)));
  const uint32_t lo = (uint32_t)G, hi = (uint32_t)((unsigned long long)G >> 32);
#pragma unroll
  for (int b = 0; b < S - 1; ++b) {  // byte b from the bottom = digit S-1-b
    const uint32_t word = b < 4 ? lo : hi;
    d[S - 1 - b] = (int)((word >> (8 * (b & 3))) & 255u) - 128;
  }
  d[0] = (int)(G >> (8 * (S - 1)));
}

// |d| <= 256 integer -> FP32 exactly via the 1.5 * 2^23 shifter (one integer
// add, one FP32 add), whose upper 16 bits are its exact BF16 encoding.
__device__ __forceinline__ uint32_t digit_f32_bits(int d) {
  return __float_as_uint(__int_as_float(0x4B400000 + d) - 12582912.0f);
}
__device__ __forceinline__ uint32_t pack2_bf16(int lo, int hi) {
  return (digit_f32_bits(lo) >> 16) | (digit_f32_bits(hi) & 0xFFFF0000u);
}
__device__ __forceinline__ unsigned short bf16_bits(int d) {
  return (unsigned short)(digit_f32_bits(d) >> 16);
}
// exact FP32 integer (|x| < 2^31) -> int32
__device__ __forceinline__ int f32_to_int(float x) { return __float2int_rn(x); }

// 2^e as a double (normal range), built from its bit pattern
__device__ __forceinline__ double pow2d(int e) {
  e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
  return __longlong_as_double((long long)(e + 1023) << 52);
}

__device__ __forceinline__ int scale_exp_of(double bound) {
  if (!(bound > 0.0) || !(bound < 1.7976931348623157e308)) return 0;
  int e;
  frexp(bound, &e);
  return e + 1;  // |x| <= bound < 2^e  ->  |x| / 2^(e+1) < 1/2
}

}  // namespace qrdm
