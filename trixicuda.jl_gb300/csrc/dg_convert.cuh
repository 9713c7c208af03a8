// dg_convert.cuh -- float <-> double conversions on the integer pipe.
//
// GB300 executes FP64 arithmetic *and* 64-bit floating-point conversions
// (F2F) on its FP64 units, which retire about 2 operations per clock per SM
// (measured: 1.26 TFLOP/s FP64 FMA vs 78.6 TFLOP/s FP32).  The mixed-precision
// kernels convert every loaded and stored value, so these conversions are
// done with 32-bit integer operations instead.  Both are exact re-encodings
// of IEEE-754 binary64/binary32 (double -> float rounds to nearest, ties to
// even); zeros are handled inline, and subnormal, infinite and NaN inputs
// fall back to the hardware conversion.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace trixi {

// double -> float, round to nearest even.
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu);
  // results that are normal floats: unbiased exponent in [-126, 127]
  if (e < 1023 - 126 || e > 1023 + 127) {
    if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(sign);
    return (float)x;
  }
  const uint32_t m = ((hi & 0x000fffffu) << 3) | (lo >> 29);  // top 23 mantissa bits
  const uint32_t rest = lo & 0x1fffffffu;                     // 29 discarded bits
  uint32_t r = sign | ((uint32_t)(e - 1023 + 127) << 23) | m;
  // ties to even; a carry out of the mantissa increments the exponent
  if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) r += 1u;
  return __uint_as_float(r);
}

// float -> double, exact.
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) {
    if ((b & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((unsigned long long)(b >> 31) << 63));
    return (double)f;
  }
  const uint32_t hi = (b & 0x80000000u) | ((e + (1023u - 127u)) << 20) | ((b & 0x007fffffu) >> 3);
  const uint32_t lo = (b & 0x7u) << 29;
  return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}

// Conversions used by the kernels: exact identity for double, integer-pipe
// conversions for float.
template <typename R>
__device__ __forceinline__ R from_double(double x);
template <>
__device__ __forceinline__ double from_double<double>(double x) { return x; }
template <>
__device__ __forceinline__ float from_double<float>(double x) { return d2f_rn(x); }

__device__ __forceinline__ double to_double(double x) { return x; }
__device__ __forceinline__ double to_double(float x) { return f2d_exact(x); }

}  // namespace trixi
