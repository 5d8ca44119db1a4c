// rk_bits.cuh -- FP64 <-> FP32 conversions on the integer pipe.
//
// On GB300 a hardware F2F conversion to or from FP64 issues at about the
// rate of an FP64 add (two per SM and clock), so a mixed-precision kernel
// that converts its operands would spend as much on conversions as on the
// FP64 arithmetic it saves.  These conversions work on the IEEE-754 bit
// fields with integer shifts, adds and selects (several per clock):
//   d2f: round to nearest, ties away from zero; magnitudes below the
//        smallest normal float become a signed zero, above the largest float
//        an infinity; NaN stays NaN.
//   f2d: exact for normal floats; subnormal floats become a signed zero.
// Neither is bit-compatible with the hardware conversion in every case
// (ties, subnormals); the mixed form needs only the relative error 2^-24.
// The functions also compile for the host (tests check them there).
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define RK_BITS_FN __host__ __device__ __forceinline__
#else
#define RK_BITS_FN inline
#endif

namespace rk {

RK_BITS_FN uint64_t bits_of(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
#endif
}
RK_BITS_FN double double_of(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  std::memcpy(&d, &u, 8);
  return d;
#endif
}
RK_BITS_FN uint32_t bits_of(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
RK_BITS_FN float float_of(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

RK_BITS_FN float d2f(double d) {
  const uint64_t u = bits_of(d);
  const uint64_t m = u & 0x7fffffffffffffffull;
  const uint32_t s = (uint32_t)(u >> 32) & 0x80000000u;
  const uint64_t a = m + (1ull << 28);  // half an FP32 unit in the last place
  const int e = (int)(a >> 52) - (1023 - 127);
  uint32_t r = s | ((uint32_t)e << 23) | ((uint32_t)(a >> 29) & 0x7fffffu);
  r = e <= 0 ? s : r;
  r = e >= 255 ? (s | 0x7f800000u) : r;
  r = m > 0x7ff0000000000000ull ? (s | 0x7fc00000u) : r;  // NaN
  return float_of(r);
}

RK_BITS_FN double f2d(float f) {
  const uint32_t u = bits_of(f);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint64_t s = (uint64_t)(u & 0x80000000u) << 32;
  const uint64_t mant = (uint64_t)(u & 0x7fffffu) << 29;
  uint64_t r = s | ((uint64_t)(e + (1023 - 127)) << 52) | mant;
  r = e == 0 ? s : r;
  r = e == 255 ? (s | 0x7ff0000000000000ull | mant) : r;
  return double_of(r);
}

}  // namespace rk
