// Conversions between float and double on the integer pipe.
//
// GB300 issues float<->double conversions on its FP64 pipe, at the FP64 FMA
// rate (measured about 1.9 per clock per SM either way, against integer
// operations at many times that).  The mixed-precision kernels convert
// between their FP32 and FP64 parts a dozen or more times per cell, so they
// use these instead: the same IEEE results (exact widening; narrowing
// rounded to nearest, ties to even), formed from the bit patterns.  Zero
// takes a short path; subnormal, out-of-range, infinite and NaN operands
// take the hardware conversion.  Plain C++ on the host, so the test suite
// checks them against the host's conversions (every float; many doubles).
#pragma once
#include <string.h>

#if defined(__CUDACC__)
#define HG_CONV_FN __host__ __device__ __forceinline__
#else
#define HG_CONV_FN static inline
#endif

HG_CONV_FN double f2d(float f) {
  unsigned u;
  memcpy(&u, &f, 4);
  const unsigned e = (u >> 23) & 0xffu;
  unsigned long long b;
  if (e - 1u < 254u) {
    // normal: rebias the exponent (127 -> 1023), widen the fraction
    b = ((unsigned long long)(u & 0x80000000u) << 32) |
        ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
  } else if ((u & 0x7fffffffu) == 0u) {
    b = (unsigned long long)(u & 0x80000000u) << 32;
  } else {
    return (double)f;
  }
  double d;
  memcpy(&d, &b, 8);
  return d;
}

HG_CONV_FN float d2f(double d) {
  unsigned long long b;
  memcpy(&b, &d, 8);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  const unsigned s = (unsigned)(b >> 32) & 0x80000000u;
  unsigned r;
  if (e - 897u < 254u) {
    // float exponent 1..254 before rounding: keep 23 of the 52 fraction bits
    // and round the 29 dropped ones to nearest, ties to even; a carry out of
    // the fraction raises the exponent (254 -> 255 is the overflow to
    // infinity that rounding to nearest gives)
    const unsigned long long m = b & 0xfffffffffffffULL;
    unsigned v = ((e - 896u) << 23) | (unsigned)(m >> 29);
    const unsigned long long rem = m & 0x1fffffffULL;
    v += (rem > 0x10000000ULL || (rem == 0x10000000ULL && (v & 1u))) ? 1u : 0u;
    r = s | v;
  } else if ((b & 0x7fffffffffffffffULL) == 0ULL) {
    r = s;
  } else {
    return (float)d;
  }
  float f;
  memcpy(&f, &r, 4);
  return f;
}
