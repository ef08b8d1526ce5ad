// bitconv.cuh -- FP32 <-> FP64 conversions by integer operations, for host
// and device.
//
// On this GPU the conversion instructions run on the FP64 pipe (1/64 of the
// FP32 rate), beside the FP64 arithmetic of the kernels that need them; the
// same results built from the operand's bits use the integer pipe.  Normal
// numbers and zeros take the integer path; subnormals, infinities, NaNs and
// (for FP64 -> FP32) values outside the float range take the hardware
// conversion.  Both return exactly what the C cast returns (FP32 -> FP64 is
// exact, FP64 -> FP32 rounds to nearest, ties to even), checked on the host
// against numpy on random bit patterns of every exponent, on rounding ties
// and on the special values.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FG_HD __host__ __device__ __forceinline__
#else
#define FG_HD inline
#endif

namespace fg {

FG_HD double bits_to_double(uint64_t u) {
  double d;
  memcpy(&d, &u, sizeof(d));
  return d;
}
FG_HD uint64_t double_bits(double d) {
  uint64_t u;
  memcpy(&u, &d, sizeof(u));
  return u;
}
FG_HD float bits_to_float(uint32_t u) {
  float f;
  memcpy(&f, &u, sizeof(f));
  return f;
}
FG_HD uint32_t float_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, sizeof(u));
  return u;
}

// (double)f: the exponent rebased by 1023 - 127 = 896, the 23-bit mantissa
// shifted into the top of the 52-bit one
FG_HD double f2d_bits(float f) {
  const uint32_t u = float_bits(f), a = u & 0x7FFFFFFFu;
  if (a - 0x00800000u >= 0x7F000000u)  // signed zero from its bits; subnormal, infinity, NaN: the cast
    return a == 0u ? bits_to_double((uint64_t)(u & 0x80000000u) << 32) : (double)f;
  const uint64_t hi = (uint64_t)(((a >> 3) + (896u << 20)) | (u & 0x80000000u));
  return bits_to_double((hi << 32) | (uint64_t)(uint32_t)(u << 29));
}

// (float)d: the exponent rebased by -896, the top 23 of the 52 mantissa bits
// kept and the 29 dropped ones rounded to nearest, ties to even (a carry out
// of the mantissa moves into the exponent, as the rounding must); biased
// exponents 897 .. 1150 give normal floats (or infinity after rounding up
// the largest), everything else takes the cast -- in a function of its own
// on the device, so that the compiler does not evaluate the cast for every
// element and select (the cast is the FP64-pipe instruction this avoids).
#ifdef __CUDACC__
static __host__ __device__ __noinline__ float d2f_cast(double d) { return (float)d; }
#else
inline float d2f_cast(double d) { return (float)d; }
#endif
FG_HD float d2f_bits(double d) {
  const uint64_t u = double_bits(d);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7FFu;
  if (e < 897u || e > 1150u) return d2f_cast(d);
  const uint64_t m = u & 0xFFFFFFFFFFFFFull;
  const uint32_t keep = (uint32_t)(m >> 29), rest = (uint32_t)(m & 0x1FFFFFFFull);
  uint32_t r = ((e - 896u) << 23) | keep;
  if (rest > 0x10000000u || (rest == 0x10000000u && (keep & 1u))) r += 1u;
  return bits_to_float(r | ((uint32_t)(u >> 32) & 0x80000000u));
}

}  // namespace fg
