// exact_round.h -- correctly rounded double of an exact integer combination,
// in integer arithmetic only.
//
// The tensor-core digit products end with v = h * 2^32 + l, an exact integer
// (|h| < 2^41, |l| < 2^49), to be scaled by a power of two and rounded once to
// the nearest double (ties to even).  Splitting v into two exact doubles and
// adding them rounds correctly too, but costs an FP64 add per output, which
// GB300 issues at 1/64 of its integer rate; here the 128-bit value is
// normalised and rounded with 64-bit integer operations.  Host and device
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

// (h * 2^SHIFT + l) * 2^scale rounded to nearest, ties to even, for
// |h| < 2^(63 - SHIFT), |l| < 2^62.  `ok` is cleared (and 0 returned) when the
// result is not a normal double; the caller then takes a slower path.
template <int SHIFT>
KGB_HD double roundScaled(int64_t h, int64_t l, int scale, bool &ok) {
  static_assert(SHIFT > 0 && SHIFT < 64, "shift of the high part");
  // v as a 128-bit two's-complement pair (hi, lo)
  const uint64_t hl = (uint64_t)h << SHIFT;
  uint64_t lo = hl + (uint64_t)l;
  int64_t hi = (h >> (64 - SHIFT)) + (l >> 63) + (lo < hl ? 1 : 0);
  if (hi == 0 && lo == 0) return 0.0;
  const bool neg = hi < 0;
  if (neg) {  // magnitude
    lo = ~lo + 1u;
    hi = ~hi + (lo == 0 ? 1 : 0);
  }
  const uint64_t uh = (uint64_t)hi;
  int p = uh ? 127 - clz64(uh) : 63 - clz64(lo);  // leading bit
  uint64_t mant;
  if (p <= 52) {
    mant = lo << (52 - p);
  } else {
    const int sh = p - 52;  // below 64 for the stated ranges
    mant = (lo >> sh) | (sh == 0 ? 0u : uh << (64 - sh));
    const uint64_t rem = lo & ((1ull << sh) - 1u), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (mant & 1u))) ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++p;
    }
  }
  const int e = p + scale + 1023;
  if (e < 1 || e > 2046) {
    ok = false;
    return 0.0;
  }
  return bitsToDouble((neg ? (1ull << 63) : 0u) | ((uint64_t)e << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

}  // namespace kgb
