// swfd_quad.cuh -- IEEE binary128 arithmetic in software (host and device).
//
// The reference is compiled with -fdefault-real-8 only, under which gfortran
// promotes double-kind literals (1d-6, 13d0/12d0, 0.75d0, 2d0, 3d0, 1d-15)
// to REAL(16): every subexpression that holds one is evaluated in binary128
// and rounded to binary64 once, where it is assigned.  The literals =
// SWFD_LITERALS_QUAD mode evaluates those subexpressions with this code, so
// that the rounded results are those of the reference build.
//
// A value is kept unpacked: (-1)^s * m * 2^(e - 112) with the 113-bit
// significand m in [2^112, 2^113) held in two 64-bit words (hi < 2^49), or
// zero.  add, sub, mul and div round to nearest, ties to even, as IEEE
// binary128 does; from_double is exact; to_double rounds to nearest, ties to
// even (subnormal results included).  Operands that are not finite are
// carried as a binary64 value and combined in binary64 (inf and NaN behave
// as in binary128 for every operation used here).  Exponents stay far from
// the binary128 limits for operands that come from binary64, so binary128
// overflow, underflow and subnormals do not arise.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define SWFD_QD __host__ __device__ __forceinline__
// the division (a loop of eight quotient digits) is kept out of line
#define SWFD_QD_CALL static __host__ __device__ __noinline__
#else
#define SWFD_QD static inline
#define SWFD_QD_CALL static
#endif

namespace swfd {
namespace qd {

struct q128 {
  uint64_t hi, lo;  // significand (hi < 2^49); both 0 for zero
  int32_t e;        // unbiased exponent of the leading bit
  uint32_t s;       // sign
  uint32_t nf;      // 1: not finite, value in `d`
  double d;
};

// ---- 128-bit helpers on (hi, lo) pairs -------------------------------------
SWFD_QD void mul64(uint64_t a, uint64_t b, uint64_t& hi, uint64_t& lo) {
#ifdef __CUDA_ARCH__
  lo = a * b;
  hi = __umul64hi(a, b);
#else
  const unsigned __int128 p = (unsigned __int128)a * b;
  lo = (uint64_t)p;
  hi = (uint64_t)(p >> 64);
#endif
}
SWFD_QD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}
SWFD_QD int clz128(uint64_t hi, uint64_t lo) { return hi ? clz64(hi) : 64 + clz64(lo); }
// (hi:lo) >> n for 0 <= n < 128; *sticky |= (bits shifted out != 0)
SWFD_QD void shr128(uint64_t& hi, uint64_t& lo, int n, uint32_t* sticky) {
  if (n <= 0) return;
  if (n >= 128) {
    if (sticky) *sticky |= (hi | lo) != 0;
    hi = lo = 0;
    return;
  }
  if (n >= 64) {
    const int k = n - 64;
    if (sticky) *sticky |= (lo != 0) || (k && (hi << (64 - k)) != 0);
    lo = k ? hi >> k : hi;
    hi = 0;
    return;
  }
  if (sticky) *sticky |= (lo << (64 - n)) != 0;
  lo = (lo >> n) | (hi << (64 - n));
  hi >>= n;
}
SWFD_QD void shl128(uint64_t& hi, uint64_t& lo, int n) {
  if (n <= 0) return;
  if (n >= 64) {
    hi = lo << (n - 64);
    lo = 0;
    return;
  }
  hi = (hi << n) | (lo >> (64 - n));
  lo <<= n;
}
SWFD_QD bool ge128(uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl) {
  return ah > bh || (ah == bh && al >= bl);
}
SWFD_QD void sub128(uint64_t& ah, uint64_t& al, uint64_t bh, uint64_t bl) {
  const uint64_t l = al - bl;
  ah = ah - bh - (al < bl);
  al = l;
}
SWFD_QD void add128(uint64_t& ah, uint64_t& al, uint64_t bh, uint64_t bl) {
  const uint64_t l = al + bl;
  ah = ah + bh + (l < al);
  al = l;
}

SWFD_QD q128 make_zero(uint32_t s) {
  q128 r;
  r.hi = r.lo = 0;
  r.e = 0;
  r.s = s;
  r.nf = 0;
  r.d = 0;
  return r;
}
SWFD_QD q128 make_nf(double v) {
  q128 r = make_zero(0);
  r.nf = 1;
  r.d = v;
  return r;
}
SWFD_QD bool is_zero(const q128& a) { return !a.nf && (a.hi | a.lo) == 0; }

// round (hi:lo), a significand of 113 + 3 bits (guard, round, sticky in the
// low three bits, further sticky in `st`), to 113 bits; exponent e of the
// leading bit
SWFD_QD q128 round_pack(uint32_t s, int32_t e, uint64_t hi, uint64_t lo, uint32_t st) {
  // normalize so that the leading bit is bit 115 of the 116-bit field
  const int lz = clz128(hi, lo);
  const int want = 128 - 116;  // leading zeros of a normalized 116-bit field
  if (lz > want) {
    shl128(hi, lo, lz - want);
    e -= lz - want;
  } else if (lz < want) {
    shr128(hi, lo, want - lz, &st);
    e += want - lz;
  }
  const uint32_t grs = (uint32_t)(lo & 7) | (st ? 1u : 0u);
  shr128(hi, lo, 3, nullptr);
  // grs: bit 2 guard, bits 1..0 round/sticky
  const bool up = (grs > 4) || (grs == 4 && (lo & 1));
  if (up) {
    add128(hi, lo, 0, 1);
    if (hi >> 49) {  // 2^113: renormalize
      shr128(hi, lo, 1, nullptr);
      e += 1;
    }
  }
  q128 r;
  r.hi = hi;
  r.lo = lo;
  r.e = e;
  r.s = s;
  r.nf = 0;
  r.d = 0;
  return r;
}

SWFD_QD q128 from_double(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  const uint32_t s = (uint32_t)(b >> 63);
  const int be = (int)((b >> 52) & 0x7ff);
  uint64_t m = b & 0x000fffffffffffffull;
  if (be == 0x7ff) return make_nf(x);
  if (be == 0 && m == 0) return make_zero(s);
  int32_t e;
  if (be == 0) {  // subnormal: normalize
    const int lz = clz64(m) - 11;  // leading bit to position 52
    m <<= lz;
    e = -1022 - lz;
  } else {
    m |= 1ull << 52;
    e = be - 1023;
  }
  // 53-bit significand to 113 bits: shift left by 60
  q128 r;
  r.hi = m >> 4;
  r.lo = m << 60;
  r.e = e;
  r.s = s;
  r.nf = 0;
  r.d = 0;
  return r;
}

SWFD_QD double to_double(const q128& a) {
  if (a.nf) return a.d;
  if ((a.hi | a.lo) == 0) return a.s ? -0.0 : 0.0;
  int32_t e = a.e;
  // low bits to drop: 60 of the 113 for a normal result, more below 2^-1022
  int drop = 60;
  if (e < -1022) drop += -1022 - e;
  uint64_t bits;
  if (drop > 113) {  // below 2^-1075, or exactly its tie: rounds to zero
    bits = 0;
  } else {
    uint64_t hi = a.hi, lo = a.lo;
    uint32_t st = 0;
    shr128(hi, lo, drop - 1, &st);
    const uint32_t guard = (uint32_t)(lo & 1);
    shr128(hi, lo, 1, nullptr);
    uint64_t m = lo;
    if (guard && (st || (m & 1))) m += 1;
    if (e < -1022) {
      bits = m;  // subnormal; a carry to 2^52 is the smallest normal
    } else {
      if (m >> 53) {  // the rounding carried to 2^53
        m >>= 1;
        e += 1;
      }
      bits = e > 1023 ? 0x7ff0000000000000ull
                      : ((uint64_t)(e + 1023) << 52) | (m & 0x000fffffffffffffull);
    }
  }
  bits |= (uint64_t)a.s << 63;
  double r;
  memcpy(&r, &bits, 8);
  return r;
}

SWFD_QD q128 neg(q128 a) {
  if (a.nf) return make_nf(-a.d);
  a.s ^= 1u;
  return a;
}

SWFD_QD q128 add(q128 a, q128 b) {
  if (a.nf || b.nf) return make_nf(to_double(a) + to_double(b));
  if (is_zero(a)) {
    if (is_zero(b)) return make_zero(a.s & b.s);
    return b;
  }
  if (is_zero(b)) return a;
  // |a| >= |b|
  const bool swap = (b.e > a.e) || (b.e == a.e && ge128(b.hi, b.lo, a.hi, a.lo) &&
                                    !(b.hi == a.hi && b.lo == a.lo));
  if (swap) {
    const q128 t = a;
    a = b;
    b = t;
  }
  uint64_t ah = a.hi, al = a.lo, bh = b.hi, bl = b.lo;
  shl128(ah, al, 3);  // guard, round, sticky positions
  shl128(bh, bl, 3);
  uint32_t st = 0;
  shr128(bh, bl, a.e - b.e, &st);
  if (st) bl |= 1;  // sticky into the low bit
  if (a.s == b.s) {
    add128(ah, al, bh, bl);
  } else {
    sub128(ah, al, bh, bl);
    if ((ah | al) == 0) return make_zero(0);  // exact cancellation: +0
  }
  return round_pack(a.s, a.e, ah, al, 0);
}

SWFD_QD q128 sub(q128 a, q128 b) { return add(a, neg(b)); }

// a * 2^k, exact
SWFD_QD q128 scale2(q128 a, int k) {
  if (a.nf) {
    a.d = a.d * (k >= 0 ? (double)(1ull << k) : 1.0 / (double)(1ull << -k));
    return a;
  }
  if ((a.hi | a.lo) != 0) a.e += k;
  return a;
}

SWFD_QD q128 mul(const q128& a, const q128& b) {
  if (a.nf || b.nf) return make_nf(to_double(a) * to_double(b));
  if (is_zero(a) || is_zero(b)) return make_zero(a.s ^ b.s);
  // 226-bit product of the two 113-bit significands
  uint64_t p00h, p00l, p01h, p01l, p10h, p10l, p11h, p11l;
  mul64(a.lo, b.lo, p00h, p00l);
  mul64(a.lo, b.hi, p01h, p01l);
  mul64(a.hi, b.lo, p10h, p10l);
  mul64(a.hi, b.hi, p11h, p11l);
  // words w0..w3 of the product
  uint64_t w0 = p00l, w1 = p00h, w2 = p11l, w3 = p11h;
  uint64_t c;
  w1 += p01l;
  c = w1 < p01l;
  w2 += c;
  w3 += (w2 < c);
  w1 += p10l;
  c = w1 < p10l;
  w2 += c;
  w3 += (w2 < c);
  w2 += p01h;
  w3 += (w2 < p01h);
  w2 += p10h;
  w3 += (w2 < p10h);
  // product in [2^224, 2^226): its leading bit is bit 224 or 225 of w3:w2:w1:w0
  const int top = (w3 >> 33) ? 225 : 224;
  int32_t e = a.e + b.e + (top - 224);
  // keep bits top..top-115 (116 bits) in hi:lo, the rest into sticky
  // the 116 bits top..top-115 into hi:lo, the bits below into the sticky
  const int k = top - 115 - 64;  // 45 or 46
  const uint32_t st = (w0 != 0) || ((w1 << (64 - k)) != 0);
  const uint64_t lo = (w1 >> k) | (w2 << (64 - k));
  const uint64_t hi = (w2 >> k) | (w3 << (64 - k));
  return round_pack(a.s ^ b.s, e, hi, lo, st);
}

// Division: the quotient of the significands in digits of 15 bits.  Each
// digit is estimated in binary32 from the top 32 bits of the partial
// remainder and a reciprocal of the divisor's top 32 bits (absolute error
// below 0.01, so the estimate is the digit or one off), then corrected
// against the exact 128-bit remainder, which stays below the divisor.  The
// leading quotient bit and 8 digits give 121 bits; with the remainder's
// sticky bit that rounds correctly to binary128.  No binary64 arithmetic:
// the FP64 pipe is the scarce one.
SWFD_QD_CALL q128 div(const q128& a, const q128& b) {
  if (a.nf || b.nf || is_zero(b)) return make_nf(to_double(a) / to_double(b));
  if (is_zero(a)) return make_zero(a.s ^ b.s);
  uint64_t rh = a.hi, rl = a.lo;
  int32_t e = a.e - b.e;
  if (!ge128(rh, rl, b.hi, b.lo)) {  // ma < mb: scale so that mb <= ma < 2 mb
    shl128(rh, rl, 1);
    e -= 1;
  }
  sub128(rh, rl, b.hi, b.lo);  // the leading quotient bit is 1
  uint64_t qh = 0, ql = 1;
  // mb in [2^112, 2^113): mb ~ mt * 2^81, so 2^96 / mb ~ 2^15 / mt
  const uint32_t mt = (uint32_t)(b.hi >> 17);
  const float rcp = 32768.0f / (float)mt;
  const uint32_t b0 = (uint32_t)b.lo, b1 = (uint32_t)(b.lo >> 32);
#pragma unroll 1
  for (int k = 0; k < 8; ++k) {
    shl128(rh, rl, 15);  // remainder * 2^15 < mb * 2^15 < 2^128
    const float est = (float)(uint32_t)(rh >> 32) * rcp;
    const uint32_t d32 = est >= 32767.0f ? 32767u : (uint32_t)est;
    uint64_t dg = d32;
    // dg * mb (< 2^128) from 32-bit limbs of mb's low word
    const uint64_t l0 = (uint64_t)b0 * d32, l1 = (uint64_t)b1 * d32;
    uint64_t pl = l0 + (l1 << 32);
    uint64_t ph = (l1 >> 32) + (pl < l0 ? 1 : 0) + b.hi * dg;
    for (int t = 0; t < 3 && !ge128(rh, rl, ph, pl); ++t) {  // estimate too large
      sub128(ph, pl, b.hi, b.lo);
      --dg;
    }
    sub128(rh, rl, ph, pl);
    for (int t = 0; t < 3 && ge128(rh, rl, b.hi, b.lo); ++t) {  // too small
      sub128(rh, rl, b.hi, b.lo);
      ++dg;
    }
    shl128(qh, ql, 15);
    ql |= dg;
  }
  // the quotient's leading bit is bit 120; round_pack's e refers to bit 115
  return round_pack(a.s ^ b.s, e - 5, qh, ql, (rh | rl) != 0);
}

// comparisons of finite values
SWFD_QD int cmp_abs(const q128& a, const q128& b) {
  const bool za = is_zero(a), zb = is_zero(b);
  if (za || zb) return za && zb ? 0 : (za ? -1 : 1);
  if (a.e != b.e) return a.e < b.e ? -1 : 1;
  if (a.hi != b.hi) return a.hi < b.hi ? -1 : 1;
  if (a.lo != b.lo) return a.lo < b.lo ? -1 : 1;
  return 0;
}
SWFD_QD double sqd(double x) { return x * x; }

// the binary64 neighbours of a finite binary128 value: the largest binary64
// <= a (rd) and the smallest >= a (ru)
SWFD_QD double rd(const q128& a) {
  const double d = to_double(a);
  const q128 diff = sub(from_double(d), a);
  if (is_zero(diff) || diff.s) return d;
  return nextafter(d, -1.0 / 0.0);
}
SWFD_QD double ru(const q128& a) {
  const double d = to_double(a);
  const q128 diff = sub(from_double(d), a);
  if (is_zero(diff) || !diff.s) return d;
  return nextafter(d, 1.0 / 0.0);
}

// ---- exp for the detonation's chemistry source -----------------------------
// exp(x) evaluated in binary128 and rounded once to binary64: x = k*ln2 + r,
// k the nearest integer to x*(1/ln2) in binary64, r = x - k*ln2 in binary128
// (ln2 the binary128 sum of a triple-double split, 113 bits), exp(r) by Horner
// on the Taylor coefficients 1/n!, n <= EXP_N (each the binary128 quotient of
// the previous by n; exp_coefs), times 2^k exactly.  The truncation and the
// roundings stay near 2^-105 relative, so the binary64 result is the
// correctly rounded exp except where exp(x) lies within that of a rounding
// boundary.
constexpr int EXP_N = 24;
SWFD_QD q128 ln2_q() {
  return add(add(from_double(0x1.62e42fefa39efp-1), from_double(0x1.abc9e3b39803fp-56)),
             from_double(0x1.7b57a079a1934p-111));
}
SWFD_QD_CALL void exp_coefs(q128* c) {
  c[0] = from_double(1.0);
  for (int n = 1; n <= EXP_N; ++n) c[n] = div(c[n - 1], from_double((double)n));
}
SWFD_QD_CALL double exp_rd(double x, const q128* c) {
  if (x != x) return x;
  if (x > 710.) return INFINITY;
  if (x < -746.) return 0.;
  const double kd = rint(x * 1.4426950408889634);
  const q128 r = sub(from_double(x), mul(from_double(kd), ln2_q()));
  q128 p = c[EXP_N];
#pragma unroll 1
  for (int n = EXP_N - 1; n >= 0; --n) p = add(mul(p, r), c[n]);
  return to_double(scale2(p, (int)kd));
}

}  // namespace qd
}  // namespace swfd
