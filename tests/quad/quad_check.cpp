// Checks the software binary128 arithmetic of swfd_quad.cuh against GCC's
// _Float128 (IEEE binary128, round to nearest even) on random and edge-case
// binary64 operands.  Prints the number of mismatches per operation.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swfd_quad.cuh"

using namespace swfd::qd;
typedef _Float128 F;

static uint64_t st = 0x243f6a8885a308d3ull;
static uint64_t rnd() {
  st ^= st << 13;
  st ^= st >> 7;
  st ^= st << 17;
  return st;
}
static double rdouble(int mode) {
  double x;
  if (mode == 0) {  // any finite bit pattern
    uint64_t b;
    do {
      b = rnd();
    } while (((b >> 52) & 0x7ff) == 0x7ff);
    memcpy(&x, &b, 8);
  } else {  // magnitudes near 1 with varied exponents
    x = ((double)(rnd() >> 11) / 9007199254740992.0 + 0.5) * ldexp(1.0, (int)(rnd() % 81) - 40);
    if (rnd() & 1) x = -x;
  }
  return x;
}
// the binary128 value of a q128 as _Float128
static F toF(const q128& a) {
  if (a.nf) return (F)a.d;
  if ((a.hi | a.lo) == 0) return a.s ? -(F)0 : (F)0;
  F m = (F)a.hi * (F)18446744073709551616.0 + (F)a.lo;  // exact: < 2^113
  F r = ldexpf128(m, a.e - 112);
  return a.s ? -r : r;
}
static bool same(F a, F b) {
  if (a != a && b != b) return true;
  return memcmp(&a, &b, sizeof(F)) == 0;
}
static bool same_d(double a, double b) {
  if (a != a && b != b) return true;
  return memcmp(&a, &b, 8) == 0;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 200000;
  long bad[11] = {0};
  const char* names[11] = {"from/to", "add", "sub", "mul", "div", "chain", "to_double", "neg0", "div113",
                           "ln2", "exp"};
  for (long i = 0; i < n; ++i) {
    const int mode = i & 1;
    double x = rdouble(mode), y = rdouble(mode);
    if (i % 97 == 0) y = -x;                 // exact cancellation
    if (i % 89 == 0) y = x * (1 + 0x1p-52);  // near cancellation
    if (i % 83 == 0) y = 0.0;
    const q128 qx = from_double(x), qy = from_double(y);
    if (!same_d(to_double(qx), x)) bad[0]++;
    const F fx = (F)x, fy = (F)y;
    if (!same(toF(add(qx, qy)), fx + fy)) bad[1]++;
    if (!same(toF(sub(qx, qy)), fx - fy)) bad[2]++;
    if (!same(toF(mul(qx, qy)), fx * fy)) bad[3]++;
    if (y != 0 && !same(toF(div(qx, qy)), fx / fy)) bad[4]++;
    // a chain like the WENO smoothness indicator, all in binary128, then rounded
    const double z = rdouble(1);
    const q128 c1312 = div(from_double(13), from_double(12));
    const q128 s = add(sub(qx, mul(from_double(2), qy)), from_double(z));
    const q128 r = add(mul(c1312, mul(s, s)), mul(from_double(0.25), mul(qy, qy)));
    const F fs = fx - (F)2 * fy + (F)z;
    const F fr = (F)13 / (F)12 * (fs * fs) + (F)0.25 * (fy * fy);
    if (!same(toF(r), fr)) bad[5]++;
    if (!same_d(to_double(r), (double)fr)) bad[6]++;
    // division of operands with full 113-bit significands
    const double w = rdouble(mode);
    const q128 qn = add(mul(qx, from_double(z)), from_double(w)), qd = mul(qy, add(from_double(z), qx));
    const F fn = fx * (F)z + (F)w, fd = fy * ((F)z + fx);
    if (fd != 0 && !same(toF(div(qn, qd)), fn / fd)) bad[8]++;
    // divisors and dividends whose significands are long runs of ones
    const double h = ldexp(1.0, -(int)(rnd() % 60) - 53), g = ldexp(1.0, -(int)(rnd() % 60) - 53);
    const q128 q1 = sub(from_double(1.0), from_double(h)), q2 = sub(from_double(x), from_double(x * g));
    const F f1 = (F)1 - (F)h, f2 = (F)x - (F)(x * g);
    if (x != 0 && !same(toF(div(q2, q1)), f2 / f1)) bad[8]++;
    if (x != 0 && !same(toF(div(q1, q2)), f1 / f2)) bad[8]++;
  }
  // to_double on values near the subnormal range and at rounding ties
  for (long i = 0; i < n / 4; ++i) {
    const double x = ldexp((double)(rnd() >> 11), -(int)(rnd() % 60) - 1040);
    const double y = ldexp((double)(rnd() >> 11), -(int)(rnd() % 30) - 30);
    const q128 q = mul(from_double(x), from_double(y));
    const F f = (F)x * (F)y;
    if (!same_d(to_double(q), (double)f)) bad[6]++;
  }
  if (!same_d(to_double(add(from_double(-0.0), from_double(-0.0))), -0.0)) bad[7]++;
  if (!same_d(to_double(add(from_double(1.5), from_double(-1.5))), 0.0)) bad[7]++;
  // exp_rd against the same algorithm in _Float128 (the oracle's oracle_exp)
  {
    const F ln2f = ((F)0x1.62e42fefa39efp-1 + (F)0x1.abc9e3b39803fp-56) + (F)0x1.7b57a079a1934p-111;
    if (!same(toF(ln2_q()), ln2f) || !same(ln2f, (F)0.693147180559945309417232121458176568f128))
      bad[9]++;
    q128 qc[EXP_N + 1];
    F fc[EXP_N + 1];
    exp_coefs(qc);
    fc[0] = 1;
    for (int k = 1; k <= EXP_N; ++k) fc[k] = fc[k - 1] / (F)k;
    for (int k = 0; k <= EXP_N; ++k)
      if (!same(toF(qc[k]), fc[k])) bad[10]++;
    for (long i = 0; i < n / 2; ++i) {
      const double x = (i % 3 == 0) ? -746. * (double)(rnd() >> 11) / 9007199254740992.0
                                    : ((double)(rnd() >> 11) / 9007199254740992.0 - 0.5) * 200.;
      const double kd = rint(x * 1.4426950408889634);
      const F r = (F)x - (F)kd * ln2f;
      F p = fc[EXP_N];
      for (int k = EXP_N - 1; k >= 0; --k) p = p * r + fc[k];
      uint64_t bits[2] = {0, (uint64_t)((int)kd + 16383) << 48};
      F two_k;
      memcpy(&two_k, bits, sizeof(two_k));
      if (!same_d(exp_rd(x, qc), (double)(p * two_k))) bad[10]++;
    }
  }
  long total = 0;
  for (int k = 0; k < 11; ++k) {
    printf("%s %ld\n", names[k], bad[k]);
    total += bad[k];
  }
  return total ? 1 : 0;
}
