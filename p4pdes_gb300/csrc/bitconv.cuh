// bitconv.cuh -- the exact FP32 -> FP64 conversion by integer operations,
// for host and device.
//
// On this GPU the conversion instructions run on the FP64 pipe (1/64 of the
// FP32 rate), beside the FP64 arithmetic of the kernels that need them; the
// same result built from the operand's bits uses the integer pipe.  Normal
// numbers and zeros take the integer path; subnormals, infinities and NaNs
// take the hardware conversion.  It returns exactly what the C cast returns (the
// conversion is exact), checked on the host against numpy on random bit
// patterns of every exponent and on the special values.
// (The other direction, rounded to nearest even from the bits, measured no
// faster in the inner solves' set-up kernel, whose time the FP64 scaling
// multiply and the memory traffic set.)
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

}  // namespace fg
