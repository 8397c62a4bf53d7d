// Checks sd::div and sd::scale of swfd_sdiv.cuh against the host's IEEE
// binary64 division and scaling
// (x86-64 SSE2 or AArch64, round to nearest, ties to even) on random and
// edge-case operands.  Prints the number of mismatching bit patterns.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swfd_sdiv.cuh"

static uint64_t st = 0x9e3779b97f4a7c15ull;
static uint64_t rnd() {
  st ^= st << 13;
  st ^= st >> 7;
  st ^= st << 17;
  return st;
}
static double from_bits(uint64_t b) {
  double x;
  memcpy(&x, &b, 8);
  return x;
}
static bool same(double a, double b) {
  if (a != a && b != b) return true;
  return memcmp(&a, &b, 8) == 0;
}
static double pick(int mode) {
  switch (mode) {
    case 0:  // any bit pattern (NaN, inf, subnormal included)
      return from_bits(rnd());
    case 1:  // magnitudes near 1
      return ldexp((double)(rnd() >> 11) / 9007199254740992.0 + 0.5, (int)(rnd() % 41) - 20) *
             ((rnd() & 1) ? -1 : 1);
    case 2: {  // significands with long runs of ones or zeros
      const uint64_t run = (rnd() & 1) ? 0xfffffffffffffull : 0;
      const uint64_t m = run ^ (rnd() >> (12 + rnd() % 52));
      const uint64_t ex = 1023 - 30 + rnd() % 61;
      return from_bits((ex << 52) | (m & 0xfffffffffffffull));
    }
    default: {  // near the exponent limits
      const uint64_t ex = (rnd() & 1) ? rnd() % 8 : 2039 + rnd() % 9;
      return from_bits(((rnd() & 1) << 63) | (ex << 52) | (rnd() >> 12));
    }
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  long bad = 0, fast = 0, bads = 0;
  for (long i = 0; i < n; ++i) {
    const double a = pick(i % 4), b = pick((i / 4) % 4);
    if (!same(swfd::sd::div(a, b), a / b)) {
      if (bad < 5) printf("mismatch %a / %a: %a vs %a\n", a, b, swfd::sd::div(a, b), a / b);
      bad++;
    }
    // quotients with exact and tie-adjacent values: a = q * b for a 53-bit q
    const double q = pick(1), c = pick(1);
    const double p = q * c;
    if (!same(swfd::sd::div(p, c), p / c)) bad++;
    if (!same(swfd::sd::scale<1>(a), a * 2.0) || !same(swfd::sd::scale<2>(a), a * 4.0) ||
        !same(swfd::sd::scale<-1>(a), a * 0.5) || !same(swfd::sd::scale<-2>(a), a * 0.25))
      bads++;
    {  // the branch-free form: equal wherever it does not flag
      int bad_nf = 0;
      const double r = swfd::sd::div_nf(a, b, bad_nf);
      if (!bad_nf && !same(r, a / b)) bad++;
      int bad_q = 0;
      if (!same(swfd::sd::div_nf(p, c, bad_q), p / c) && !bad_q) bad++;
    }
    const uint32_t ea = (uint32_t)(swfd::sd::dbits(a) >> 52) & 0x7ff;
    fast += ea != 0 && ea != 0x7ff;
  }
  const double edge[] = {1.0, -1.0, 3.0, 0.1, 0.3, 0.6, 1e-12, 1e300, 1e-300, 0.0, -0.0,
                         4.9e-324, 2.2250738585072014e-308, 1.7976931348623157e308, INFINITY,
                         -INFINITY, NAN, 1.0000000000000002, 0.9999999999999999};
  const int ne = sizeof(edge) / sizeof(edge[0]);
  for (int i = 0; i < ne; ++i)
    for (int j = 0; j < ne; ++j)
    {
      if (!same(swfd::sd::div(edge[i], edge[j]), edge[i] / edge[j])) {
        printf("edge mismatch %a / %a\n", edge[i], edge[j]);
        bad++;
      }
    }
  for (int i = 0; i < ne; ++i)
    if (!same(swfd::sd::scale<-1>(edge[i]), edge[i] * 0.5) ||
        !same(swfd::sd::scale<1>(edge[i]), edge[i] * 2.0))
      bads++;
  printf("div %ld scale %ld (of %ld, %ld with a normal first operand)\n", bad, bads,
         2 * n + ne * ne, fast);
  return (bad || bads) ? 1 : 0;
}
