// Checks the integer-pipe float<->double conversions of fpconv.h against
// the host's IEEE conversions: every float widened, and narrowed doubles
// drawn at random, at the midpoints between neighbouring floats (exact
// ties and one double ulp either side) and with every exponent at the
// edges of the float range.  Prints "ok <checked>" or the first mismatches.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <initializer_list>

#include "fpconv.h"

static uint64_t state = 88172645463325252ULL;
static uint64_t next() {
  state ^= state << 13;
  state ^= state >> 7;
  state ^= state << 17;
  return state;
}
static unsigned long long bad = 0, checked = 0;
static bool same_f(float a, float b) { return memcmp(&a, &b, 4) == 0 || (a != a && b != b); }
static bool same_d(double a, double b) { return memcmp(&a, &b, 8) == 0 || (a != a && b != b); }
static void narrow(double d) {
  ++checked;
  const float a = d2f(d), b = (float)d;
  if (!same_f(a, b) && bad++ < 5) printf("d2f %a -> %a, expected %a\n", d, a, b);
}

int main(int argc, char** argv) {
  const bool all_floats = argc < 2 || argv[1][0] != 's';
  const uint64_t nf = all_floats ? 0x100000000ULL : 0x1000000ULL;
  for (uint64_t i = 0; i < nf; ++i) {
    const uint32_t u = all_floats ? (uint32_t)i : (uint32_t)next();
    float f;
    memcpy(&f, &u, 4);
    ++checked;
    if (!same_d(f2d(f), (double)f) && bad++ < 5) printf("f2d %a wrong\n", (double)f);
  }
  for (int i = 0; i < 20000000; ++i) {
    const uint64_t b = next();
    double d;
    memcpy(&d, &b, 8);
    narrow(d);
  }
  for (int i = 0; i < 5000000; ++i) {
    const uint32_t u = (uint32_t)next();
    float f;
    memcpy(&f, &u, 4);
    if (!std::isfinite(f)) continue;
    const float g = nextafterf(f, INFINITY);
    if (!std::isfinite(g)) continue;
    const double mid = ((double)f + (double)g) * 0.5;
    narrow(mid);
    narrow(nextafter(mid, INFINITY));
    narrow(nextafter(mid, -INFINITY));
  }
  for (unsigned e : {0u, 1u, 895u, 896u, 897u, 898u, 1149u, 1150u, 1151u, 1152u, 2046u, 2047u})
    for (int i = 0; i < 500000; ++i) {
      const uint64_t b = ((next() & 1ULL) << 63) | ((uint64_t)e << 52) | (next() & 0xfffffffffffffULL);
      const uint64_t vs[3] = {b, (b & ~(uint64_t)0x1fffffff) | (uint64_t)0x10000000,
                              b | (uint64_t)0x1fffffff};
      for (uint64_t v : vs) {
        double d;
        memcpy(&d, &v, 8);
        narrow(d);
      }
    }
  for (double d : {0.0, -0.0, (double)INFINITY, -(double)INFINITY, (double)NAN,
                   3.4028235677973366e38, 3.4028235677973362e38, 1.1754942807573643e-38})
    narrow(d);
  if (bad) {
    printf("FAILED %llu of %llu\n", bad, checked);
    return 1;
  }
  printf("ok %llu\n", checked);
  return 0;
}
