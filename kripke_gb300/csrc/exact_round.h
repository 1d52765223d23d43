// exact_round.h -- correctly rounded double of an exact integer combination,
// in integer arithmetic only.
//
// The tensor-core digit products end with v = h * 2^32 + l, an exact integer
// (|h| < 2^41, |l| < 2^49), to be scaled by a power of two and rounded once to
// the nearest double (ties to even).  Splitting v into two exact doubles and
// adding them rounds correctly too, but costs an FP64 add per output, which
// GB300 issues at 1/64 of its integer rate; here v is normalised and rounded
// with one 64-bit and one 32-bit word.  Host and device
// compile the same code, so the CPU tests compare it bit for bit with the
// two-double sum.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define KGB_HD __host__ __device__ __forceinline__
#else
#define KGB_HD inline
#endif

namespace kgb {

KGB_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

KGB_HD double bitsToDouble(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

KGB_HD int clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __clz((int)x);
#else
  return __builtin_clz(x);
#endif
}

// (h * 2^32 + l) * 2^scale rounded to nearest, ties to even, for |h| < 2^52
// and |l| < 2^62.  `ok` is cleared (and 0 returned) when the result is not a
// normal double; the caller then takes a slower path.
//
// With l = lh * 2^32 + ll (ll the unsigned low word), v = H * 2^32 + ll for
// H = h + lh, and |v| = A * 2^32 + B with A = |H| (less one when v < 0 and
// ll != 0) and B < 2^32, so only A needs 64 bits: the 53-bit significand is
// (A << (32 - sh)) | (B >> sh) for a shift sh <= 32 and the rounding looks
// at B alone.
KGB_HD double roundScaled32(int64_t h, int64_t l, int scale, bool &ok) {
  const int64_t H = h + (l >> 32);
  const uint32_t ll = (uint32_t)l;
  if (H == 0 && ll == 0) return 0.0;
  const bool neg = H < 0;
  const uint64_t A = neg ? (uint64_t)(-H) - (ll != 0 ? 1u : 0u) : (uint64_t)H;
  const uint32_t B = neg ? 0u - ll : ll;
  int p;  // leading bit of |v|
  uint64_t mant;
  if (A != 0) {
    p = 95 - clz64(A);
    if (p <= 52) {
      mant = ((A << 32) | B) << (52 - p);
    } else {
      const int sh = p - 52;  // 1 .. 32, since A < 2^53
      if (sh < 32) {
        mant = (A << (32 - sh)) | (B >> sh);
        const uint32_t rem = B & ((1u << sh) - 1u), half = 1u << (sh - 1);
        if (rem > half || (rem == half && (mant & 1u))) ++mant;
      } else {  // A is the significand, B the remainder against half = 2^31
        mant = A;
        if (B > 0x80000000u || (B == 0x80000000u && (mant & 1u))) ++mant;
      }
      if (mant >> 53) {
        mant >>= 1;
        ++p;
      }
    }
  } else {
    p = 31 - clz32(B);
    mant = (uint64_t)B << (52 - p);
  }
  const int e = p + scale + 1023;
  if (e < 1 || e > 2046) {
    ok = false;
    return 0.0;
  }
  return bitsToDouble((neg ? (1ull << 63) : 0u) | ((uint64_t)e << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

}  // namespace kgb
