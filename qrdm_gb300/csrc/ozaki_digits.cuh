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
// FP16 digits (the single-problem Ozaki kernels; A and B of one MMA share
// the type).  |d| <= 512 integer pair -> two FP16, exactly: 1536 + d lies in
// [1024, 2048), where FP16's spacing is 1, so its bits are 0x6600 + d, and
// one packed half-precision subtraction of 1536 leaves d.
__device__ __forceinline__ uint32_t pack2_f16(int lo, int hi) {
  const uint32_t w = ((uint32_t)(0x6600 + lo) & 0xFFFFu) | ((uint32_t)(0x6600 + hi) << 16);
  uint32_t r;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(w), "r"(0x66006600u));
  return r;
}
// Lower balanced digits of two entries from their biased fixed-point words:
// byte b (0..3) of w0 and of w1 is digit + 128.  One byte permute places
// them in the low bytes of the two halves, one logic op makes the halves
// 1024 + byte (bits 0x6400 | byte) and one packed subtraction of 1152 leaves
// byte - 128: three instructions per digit pair.
__device__ __forceinline__ uint32_t digit_pair_f16(uint32_t w0, uint32_t w1, int b) {
  const uint32_t sel = (uint32_t)b | ((uint32_t)b << 4) | ((uint32_t)(b + 4) << 8) | ((uint32_t)(b + 4) << 12);
  const uint32_t t = (__byte_perm(w0, w1, sel) & 0x00FF00FFu) | 0x64006400u;
  uint32_t r;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(t), "r"(0x64806480u));
  return r;
}
// S FP16 digit pairs of two entries (x in the low halves) at scale 2^sh:
// out[p] for digit p (most significant first), the balanced digits of
// balanced_digits<S>.
template <int S>
__device__ __forceinline__ void digits2_f16(double x, double y, int sh, uint32_t* out) {
  const long long bias = (long long)(0x8080808080808080ull >> (8 * (9 - S)));
  const long long G0 = fixed_point(x, sh) + bias, G1 = fixed_point(y, sh) + bias;
  out[0] = pack2_f16((int)(G0 >> (8 * (S - 1))), (int)(G1 >> (8 * (S - 1))));
#pragma unroll
  for (int b = 0; b < S - 1; ++b) {  // byte b from the bottom = digit S-1-b
    const uint32_t w0 = b < 4 ? (uint32_t)G0 : (uint32_t)((unsigned long long)G0 >> 32);
    const uint32_t w1 = b < 4 ? (uint32_t)G1 : (uint32_t)((unsigned long long)G1 >> 32);
    out[S - 1 - b] = digit_pair_f16(w0, w1, b & 3);
  }
}

// exact FP32 integer (|x| < 2^31) -> int32
__device__ __forceinline__ int f32_to_int(float x) { return __float2int_rn(x); }

// 2^e as a double (normal range), built from its bit pattern
__device__ __forceinline__ double pow2d(int e) {
  e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// |x| <= bound < 2^e  ->  returns e + 1, so |x| / 2^(e+1) < 1/2; 0 for a
// bound that is not positive and finite.  Read off the exponent field with
// integer instructions (frexp and FP64 compares would take the FP64 pipe).
__device__ __forceinline__ int scale_exp_of(double bound) {
  const long long b = __double_as_longlong(bound);
  if (b <= 0) return 0;  // negative, zero, or NaN with the sign bit set
  const int E = (int)(b >> 52);
  if (E == 0x7FF || b == 0x7FEFFFFFFFFFFFFFll) return 0;  // infinity, NaN, DBL_MAX (no 2^(e+1) above it)
  if (E == 0) {              // subnormal
    int e;
    frexp(bound, &e);
    return e + 1;
  }
  return E - 1021;  // bound in [2^(E-1023), 2^(E-1022))
}

// v 2^e rounded to nearest (ties to even), |v| < 2^62, built with integer
// instructions (a 64-bit integer conversion runs on the FP64 pipe, the
// scarce unit of the Ozaki epilogues); scales whose result would leave the
// normal range take the conversion.
__device__ __forceinline__ double oz_i64_scaled(long long v, int e) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)v & 0x8000000000000000ull;
  unsigned long long m = (unsigned long long)(v < 0 ? -v : v);
  const int lz = __clzll((long long)m);
  const int ex = 1023 + 63 - lz + e;
  if (ex <= 0 || ex >= 2046) return (double)v * pow2d(e);
  m <<= lz;  // leading one at bit 63
  const unsigned long long rest = m & 0x7FFull;
  unsigned long long mant = m >> 11;  // 53 bits
  mant += (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
  // mant = 2^53 after rounding carries into the exponent field
  return __longlong_as_double((long long)(sgn | (((unsigned long long)ex << 52) + mant - (1ull << 52))));
}

// f 2^e exactly as a double, built from the FP32 bit pattern with integer
// instructions; zero, subnormal or out-of-range inputs give 0 (the callers'
// values there are far below the result's rounding).
__device__ __forceinline__ double oz_f32_scaled(float f, int e) {
  const unsigned u = __float_as_uint(f);
  const int E8 = (int)((u >> 23) & 0xFF);
  const int ex = E8 - 127 + 1023 + e;
  if (E8 == 0 || E8 == 0xFF || ex <= 0 || ex >= 2047) return 0.0;
  const unsigned long long bits = ((unsigned long long)(u >> 31) << 63) | ((unsigned long long)ex << 52) |
                                  ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)bits);
}

}  // namespace qrdm
