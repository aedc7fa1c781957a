// Exact integer -> nearest double conversion with integer instructions only (the FP64
// pipe of this GPU runs at about 1/64 of the FP32 rate), shared by the split-precision GEMM
// epilogue and the double-float helpers.
#pragma once

#include <cstdint>
#include <cstring>

namespace qltg {

// z 2^e (negated when neg) rounded to the nearest double (ties to even), with integer
// operations only: the FP64 pipe of this GPU is slow, and no path here touches it.
__host__ __device__ __forceinline__ double scaled_i64(long long z, int e, bool neg) {
  if (z == 0) return 0.0;
  const unsigned long long a = z < 0 ? 0ull - (unsigned long long)z : (unsigned long long)z;
  const unsigned long long sgn = ((z < 0) != neg) ? 0x8000000000000000ull : 0ull;
#ifdef __CUDA_ARCH__
  const int lz = __clzll((long long)a);
#else
  const int lz = __builtin_clzll(a);
#endif
  const int be = 1023 + 63 - lz + e;                    // biased exponent of the leading bit
  unsigned long long bits;
  if (be >= 1) {
    const unsigned long long m = a << lz;               // leading one at bit 63
    unsigned long long mant = m >> 11;                  // 53 bits, leading one at bit 52
    const unsigned long long rem = m & 0x7FFull;
    mant += (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
    // (be - 1) << 52 plus the mantissa with its leading one adds the exponent; a rounding
    // carry to 2^53 moves into the exponent by itself, and past 2046 it reaches infinity
    bits = be < 2047 ? ((unsigned long long)(be - 1) << 52) + mant : 0x7FF0000000000000ull;
    if (bits > 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
  } else {
    // subnormal result: a 2^(e + 1074) in units of 2^-1074, rounded to nearest-even
    const int sh = -(e + 1074);                         // > 0 here unless a is large
    if (sh <= 0) {
      bits = a << (-sh);                                // cannot overflow: be < 1
    } else if (sh >= 64) {
      bits = (sh == 64 && a > 0x8000000000000000ull) ? 1ull : 0ull;
    } else {
      const unsigned long long q = a >> sh, r = a - (q << sh), half = 1ull << (sh - 1);
      bits = q + ((r > half || (r == half && (q & 1ull))) ? 1ull : 0ull);
    }
  }
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)(sgn | bits));
#else
  double r;
  const unsigned long long rb = sgn | bits;
  memcpy(&r, &rb, sizeof r);
  return r;
#endif
}

}  // namespace qltg
