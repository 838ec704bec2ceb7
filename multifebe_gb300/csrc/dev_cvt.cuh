// Exact binary32 -> binary64 conversion formed with integer instructions.
// GB300 runs about two binary64 operations per cycle per SM, and the hardware
// conversion occupies that pipe too; this builds the same bit pattern on the
// integer pipe, for kernels whose binary64 work is a few additions per result.
#pragma once
#include <cstdint>

namespace mfb {

// binary32 -> binary64, exact for every finite input (subnormals included);
// inf / NaN through the hardware conversion
__device__ __forceinline__ double f32_to_f64_exact(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned ex = (u >> 23) & 0xFFu;
  const unsigned long long sg = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned mt = u & 0x7FFFFFu;
  if (ex == 0xFFu) return (double)x;
  if (ex == 0u) {
    if (mt == 0u) return __longlong_as_double((long long)sg);
    const int p = 31 - __clz((int)mt);  // leading bit of the subnormal's mantissa, value mt 2^-149
    return __longlong_as_double((long long)(sg | ((unsigned long long)(p - 149 + 1023) << 52) |
                                            (((unsigned long long)mt << (52 - p)) & 0xFFFFFFFFFFFFFULL)));
  }
  return __longlong_as_double((long long)(sg | ((unsigned long long)(ex + 896u) << 52) | ((unsigned long long)mt << 29)));
}

}  // namespace mfb
