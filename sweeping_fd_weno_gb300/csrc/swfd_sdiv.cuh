// swfd_sdiv.cuh -- IEEE binary64 division and scaling by powers of two on the
// integer and FP32 pipes (host and device).
//
// A GB300 SM retires two FP64 operations per clock against 128 integer or
// FP32 ones, and an IEEE binary64 division costs a sequence of FP64
// operations.  sd::div returns the correctly rounded quotient (round to
// nearest, ties to even) -- the same bits as the hardware division -- from
// integer arithmetic on the significands: the leading quotient bit and five
// digits of 11 bits, each estimated in binary32 and corrected exactly, then
// rounded with the remainder as sticky bit (schoolbook division with
// estimated quotient digits: Knuth, TAOCP vol. 2, 4.3.1, Algorithm D).  Operands that are zero,
// subnormal, infinite or NaN, and quotients whose exponent is within a
// binade of the binary64 limits, take the hardware division, so the result
// equals a / b for every input.  sd::scale<K> (x * 2^K: an addition to the
// exponent field) falls back in the same way and equals x * 2^K for every
// input.  (A software product -- 106-bit integer product, rounded -- measured
// slower than the hardware DMUL in the flux kernel: its dependent integer
// chain outweighs the FP64 issue it saves.)
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define SWFD_SD __host__ __device__ __forceinline__
// the hardware fallbacks are calls, so that the compiler cannot if-convert
// them into FP64 instructions that every call would execute
#define SWFD_SD_SLOW static __host__ __device__ __noinline__
#else
#define SWFD_SD static inline
#define SWFD_SD_SLOW static
#endif

namespace swfd {
namespace sd {

SWFD_SD uint64_t dbits(double x) {
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
}
SWFD_SD double dfrom(uint64_t u) {
  double x;
  memcpy(&x, &u, 8);
  return x;
}
SWFD_SD uint32_t fbits(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
}
SWFD_SD float ffrom(uint32_t u) {
  float x;
  memcpy(&x, &u, 4);
  return x;
}
SWFD_SD_SLOW double div_hw(double a, double b) { return a / b; }
SWFD_SD_SLOW double mul_hw(double a, double b) { return a * b; }

// correctly rounded binary32 reciprocal (only an estimate is needed)
SWFD_SD float rcp32(float x) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}

SWFD_SD double div(double a, double b) {
  const uint64_t ua = dbits(a), ub = dbits(b);
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  // biased exponent of the quotient when ma >= mb; the result's is e or e - 1
  // before rounding and at most one more after it
  int32_t e = (int32_t)ea - (int32_t)eb + 1023;
  if (ea - 1u >= 2046u || eb - 1u >= 2046u || e < 2 || e > 2045) {
    // a zero dividend over a normal divisor: a zero with the sign of the
    // quotient (IEEE 754), without the fallback call -- flux differences of
    // a uniform state at rest are exact zeros.  Tested inside the range
    // branch, so the normal operands' path has no extra instruction.
    if ((ua << 1) == 0 && eb - 1u < 2046u) return dfrom((ua ^ ub) & 0x8000000000000000ull);
    return div_hw(a, b);
  }
  const uint64_t frac = 0xfffffffffffffull;
  const uint64_t B = (ub & frac) | (1ull << 52);
  uint64_t A = (ua & frac) | (1ull << 52);
  if (A < B) {  // scale so that B <= A < 2B
    A <<= 1;
    e -= 1;
  }
  A -= B;  // the leading quotient bit is 1
  uint64_t q = 1;
  // 2^41 / B from B's top 32 bits (relative error near 2^-23)
  const float rcp = 1048576.0f * rcp32((float)(uint32_t)(B >> 21));
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    A <<= 11;  // A < B * 2^11 < 2^64
    // A >> 41 (< 2^23) as a float without a conversion instruction
    const float n = ffrom(0x4b000000u | (uint32_t)(A >> 41)) - 8388608.0f;
    // the nearest integer to the estimate of A / B (absolute error below
    // 0.001: truncation of A 2^-11, of B and the float roundings 2^11 * 2^-22),
    // so it is the digit d = floor(A / B) or d + 1
    const uint32_t dg = fbits(n * rcp + 8388608.0f) & 0x7fffffu;
    uint64_t P = B * dg;  // <= B * 2^11 < 2^64
    uint64_t d = dg;
    if (P > A) {
      P -= B;
      d -= 1;
    }
    A -= P;  // now A < B
    q = (q << 11) | d;
  }
  // q holds 56 bits; round to 53 with A != 0 as sticky
  const uint32_t low = (uint32_t)q & 7u;
  q >>= 3;
  if (low > 4u || (low == 4u && (A != 0 || (q & 1)))) q += 1;
  if (q >> 53) {  // rounded up to 2^53
    q >>= 1;
    e += 1;
  }
  return dfrom(((ua ^ ub) & 0x8000000000000000ull) | ((uint64_t)e << 52) | (q & frac));
}

// a / b by the same steps as div, without the fallback: for operands or
// quotients outside the range div computes itself it sets `bad` and returns an
// unspecified value.  No branch: a caller that divides many times checks
// `bad` once and redoes the work with div.
SWFD_SD double div_nf(double a, double b, int& bad) {
  const uint64_t ua = dbits(a), ub = dbits(b);
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  int32_t e = (int32_t)ea - (int32_t)eb + 1023;
  bad |= (ea - 1u >= 2046u) | (eb - 1u >= 2046u) | (e < 2) | (e > 2045);
  const uint64_t frac = 0xfffffffffffffull;
  const uint64_t B = (ub & frac) | (1ull << 52);
  uint64_t A = (ua & frac) | (1ull << 52);
  const bool lt = A < B;
  A = lt ? A << 1 : A;
  e -= lt ? 1 : 0;
  A -= B;
  uint64_t q = 1;
  const float rcp = 1048576.0f * rcp32((float)(uint32_t)(B >> 21));
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    A <<= 11;
    const float n = ffrom(0x4b000000u | (uint32_t)(A >> 41)) - 8388608.0f;
    const uint32_t dg = fbits(n * rcp + 8388608.0f) & 0x7fffffu;
    uint64_t P = B * dg;
    const bool over = P > A;
    P -= over ? B : 0;
    A -= P;
    q = (q << 11) | (uint64_t)(dg - (over ? 1u : 0u));
  }
  const uint32_t low = (uint32_t)q & 7u;
  q >>= 3;
  q += (low > 4u || (low == 4u && (A != 0 || (q & 1)))) ? 1 : 0;
  const bool carry = (q >> 53) != 0;
  q = carry ? q >> 1 : q;
  e += carry ? 1 : 0;
  return dfrom(((ua ^ ub) & 0x8000000000000000ull) | ((uint64_t)(uint32_t)e << 52) | (q & frac));
}

// x * 2^K: only the exponent field changes while x and the result are normal
template <int K>
SWFD_SD double scale(double x) {
  constexpr uint32_t lo = K < 0 ? 1 - K : 1, hi = K > 0 ? 2046 - K : 2046;
  constexpr double f = K >= 0 ? (double)(1ull << (K >= 0 ? K : 0)) : 1.0 / (double)(1ull << (K < 0 ? -K : 0));
  const uint64_t u = dbits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  if (e - lo > hi - lo) return (u << 1) == 0 ? x : mul_hw(x, f);  // +-0 * 2^K = +-0
  return dfrom(u + ((uint64_t)(int64_t)K << 52));
}

}  // namespace sd
}  // namespace swfd
