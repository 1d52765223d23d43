// exact_round.h -- correctly rounded double of an exact integer combination,
// in integer arithmetic only.
//
// The tensor-core digit products end with v = h * 2^32 + l, an exact integer
// (|h| < 2^38, |l| < 2^48), to be scaled by a power of two and rounded once to
// the nearest double (ties to even).  Splitting v into two exact doubles and
// adding them rounds correctly too, but costs FP64 conversions and an FP64 add
// per output, which GB300 issues at 1/64 of its integer rate; here v is
// normalised and rounded in one 64-bit word.  Host and device compile the
// same code, so the CPU tests compare it bit for bit with the two-double sum.
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

// (h * 2^32 + l) * 2^scale rounded to nearest, ties to even, for |h| < 2^38
// and |l| < 2^56.  `ok` is cleared (and 0 returned) when the result is not a
// normal double; the caller then takes a slower path.
//
// When |v| < 2^63, v itself is formed in 64 bits.  Otherwise q = floor(v / 2^8)
// with its last bit set when v is not a multiple of 2^8 -- v rounded to odd at
// unit 2^8 -- has at least 56 significant bits, and rounding it to 53 bits
// gives the double that rounding v gives (round-to-odd with two or more extra
// bits: Boldo and Melquiond, "Emulation of FMA and correctly rounded sums:
// proved algorithms using rounding to odd", IEEE Trans. Computers 57(4), 2008).
// The magnitude is then normalised with one count of leading zeros and one
// shift, and the round-half-even increment is added below the exponent field,
// so a carry out of the significand raises the exponent.  No branch depends on
// the data except the rare out-of-range exit.
KGB_HD double roundScaledOdd(int64_t h, int64_t l, int scale, bool &ok) {
  const int64_t q = (int64_t)((uint64_t)h << 24) + (l >> 8);
  const bool big = (uint64_t)(q + ((int64_t)1 << 55)) >= (1ull << 56);  // q outside [-2^55, 2^55)
  const int64_t v = big ? (q | (int64_t)((l & 0xFF) != 0)) : (int64_t)(((uint64_t)h << 32) + (uint64_t)l);
  if (v == 0) return 0.0;
  const uint64_t s = (uint64_t)(v >> 63);  // all ones when negative
  const uint64_t m = ((uint64_t)v ^ s) - s;
  const int lz = clz64(m);
  const uint64_t n = m << lz;  // leading bit at 63
  const uint64_t mant = n >> 11;
  const uint64_t inc = ((n & 0x7FFu) + 0x3FFu + (mant & 1u)) >> 11;  // round half to even
  const int e = 1086 - lz + scale + (big ? 8 : 0);                     // biased exponent of m * 2^scale
  if (e < 1 || e > 2045) {
    ok = false;
    return 0.0;
  }
  return bitsToDouble((s << 63) | (((uint64_t)(e - 1) << 52) + mant + inc));
}

}  // namespace kgb
