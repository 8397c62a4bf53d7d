// swfd_device.cuh -- device arithmetic shared by the kernels.
//
// Every expression keeps the reference's Fortran operation order in FP64.
// The FP32-bulk instantiations (T = float) are not bit-exact by design and
// use single-precision math throughout, with reciprocals where several
// divisions share a denominator.  The
// library is compiled with -fmad=false so that no multiply-add is contracted
// (the x86-64 reference build has no FMA).  Terms the reference multiplies by
// the constants 0 or 1 inside the eigenvector products are left out: x*1 is
// exact and adding an exact zero does not change a nonzero sum, so the
// values are identical (only the sign of an exactly-zero result may differ).
//
// The bulk arithmetic is templated on its scalar type T: T = double is the
// FP64 path (value-for-value the reference), T = float the FP32-bulk path.
// Constants are written T(c) so that a float instantiation stays in float.
#pragma once

#include "swfd_internal.h"
#include "swfd_sdiv.cuh"

namespace swfd {

// c(-1:2,0:2) of MODULE weno5 (ex3_vortex_accuracy_2d/weno5.f90:3-15)
#define SWFD_C13 0.333333333333333333333333333333333
#define SWFD_C56 0.833333333333333333333333333333333
#define SWFD_CM16 (-0.166666666666666666666666666666667)
#define SWFD_C116 1.83333333333333333333333333333333
#define SWFD_CM76 (-1.16666666666666666666666666666667)

template <class T>
__device__ __forceinline__ T tsq(T a) { return a * a; }
// single-precision math stays single precision (no promotion to double)
__device__ __forceinline__ double tsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float tsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double tabs(double a) { return fabs(a); }
__device__ __forceinline__ float tabs(float a) { return fabsf(a); }
// -a (IEEE negation: the sign bit flipped).  Binary64 on the integer pipe, so
// a negated value that is selected at run time, not folded into its
// product, costs no FP64 instruction.
__device__ __forceinline__ double tneg(double a) {
  return __hiloint2double(__double2hiint(a) ^ (int)0x80000000, __double2loint(a));
}
__device__ __forceinline__ float tneg(float a) { return -a; }
__device__ __forceinline__ double dsq(double a) { return a * a; }
// a / b.  Binary64: sd::div, the correctly rounded quotient (the bits of the
// hardware division) from integer and FP32 arithmetic, which leaves the FP64
// pipe -- the bound of the flux kernels -- to the additions and products.
// Binary32: the hardware division.
__device__ __forceinline__ double tdiv(double a, double b) { return sd::div(a, b); }
__device__ __forceinline__ float tdiv(float a, float b) { return a / b; }
// Division policies of the WENO reconstructions: DivHw is tdiv (the exact
// quotient, with its out-of-range fallback); DivFlag the same quotient without
// the fallback branch, raising *bad where the fallback would be needed, so a
// caller computes many quotients in straight-line code and redoes the work
// with DivHw in the rare flagged case.
struct DivHw {
  template <class T>
  __device__ __forceinline__ T operator()(T a, T b) const { return tdiv(a, b); }
};
struct DivFlag {
  int* bad;
  __device__ __forceinline__ double operator()(double a, double b) const {
    return sd::div_nf(a, b, *bad);
  }
};
// a / b with tdiv's bits and no branch for the common operands: a zero
// dividend over a normal divisor gives the signed zero inline (the state at
// rest has zero momenta); other operands or quotients outside sd::div_nf's
// range set bad, and the caller redoes its divisions with tdiv.  Independent
// divisions in straight-line code interleave, where tdiv's fallback branch
// would run them one after another.
__device__ __forceinline__ double div_nfz(double a, double b, int& bad) {
  int out = 0;
  const double q = sd::div_nf(a, b, out);
  const uint64_t ua = sd::dbits(a), ub = sd::dbits(b);
  const bool z = (ua << 1) == 0 && ((uint32_t)(ub >> 52) & 0x7ffu) - 1u < 2046u;
  bad |= z ? 0 : out;
  return z ? sd::dfrom((ua ^ ub) & 0x8000000000000000ull) : q;
}

// x * 2^K.  Binary64: sd::scale, an addition to the exponent field (the bits
// of the hardware product).  Binary32: the product.
template <int K>
__device__ __forceinline__ double tscale(double x) { return sd::scale<K>(x); }
template <int K>
__device__ __forceinline__ float tscale(float x) {
  constexpr float f = K >= 0 ? float(1u << (K >= 0 ? K : 0)) : 1.0f / float(1u << (K < 0 ? -K : 0));
  return x * f;
}

// 1/x for the FP32-bulk form: the correctly rounded reciprocal from sd::div
// (integer and FP32 pipes; a Newton refinement of an FP32 seed cost four
// DFMAs and two conversions on the FP64 pipe)
__device__ __forceinline__ double rcp_bulk(double x) { return sd::div(1.0, x); }

// binary64 <-> binary32 conversions on the integer pipes, the bits of the
// hardware conversions (round to nearest even): GB300 runs conversions to
// and from 64-bit types at the FP64 rate.  Zeros keep their sign inline
// (tested in the out-of-range branch only); subnormal, infinite, NaN and
// out-of-range values take the hardware conversion (out of line).
static __device__ __noinline__ float d2f_hw(double x) { return (float)x; }
static __device__ __noinline__ double f2d_hw(float x) { return (double)x; }
__device__ __forceinline__ float d2f(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((u >> 52) & 0x7ff) - 1023 + 127;
  if ((unsigned)(e - 1) >= 254u)  // +-0 inline, the rest out of line
    return (u << 1) == 0 ? __uint_as_float((unsigned)(u >> 32)) : d2f_hw(x);
  const unsigned long long m = u & 0xfffffffffffffull;
  unsigned r = (unsigned)(m >> 29);
  const unsigned rem = (unsigned)m & 0x1fffffffu;
  r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;
  // a rounding carry moves into the exponent (up to infinity, as RNE does)
  return __uint_as_float(((unsigned)(u >> 32) & 0x80000000u) | (((unsigned)e << 23) + r));
}
__device__ __forceinline__ double f2d(float x) {
  const unsigned b = __float_as_uint(x);
  const unsigned e = (b >> 23) & 0xffu;
  if (e - 1u >= 254u)  // +-0 inline, the rest out of line
    return (b << 1) == 0u ? __longlong_as_double((long long)((unsigned long long)b << 32))
                          : f2d_hw(x);
  return __longlong_as_double((long long)(((unsigned long long)(b & 0x80000000u) << 32) |
                                          ((unsigned long long)(e + 896u) << 52) |
                                          ((unsigned long long)(b & 0x7fffffu) << 29)));
}
__device__ __forceinline__ double tod(double x) { return x; }
__device__ __forceinline__ double tod(float x) { return f2d(x); }

// beta(1:3) (weno5.f90:100-102); am2..ap2 = average(-2..2)
template <class T>
__device__ __forceinline__ void weno_beta(T am2, T am1, T a0, T ap1, T ap2, T& b1, T& b2, T& b3) {
  const T c1312 = T(13.0 / 12.0);
  // 2d0*, 4d0* and 0.25d0* as exponent shifts (tscale): the same values
  T s1 = a0 - tscale<1>(ap1) + ap2, t1 = T(3.0) * a0 - tscale<2>(ap1) + ap2;
  T s2 = am1 - tscale<1>(a0) + ap1, t2 = am1 - ap1;
  T s3 = am2 - tscale<1>(am1) + a0, t3 = am2 - tscale<2>(am1) + T(3.0) * a0;
  b1 = c1312 * tsq(s1) + tscale<-2>(tsq(t1));
  b2 = c1312 * tsq(s2) + tscale<-2>(tsq(t2));
  b3 = c1312 * tsq(s3) + tscale<-2>(tsq(t3));
}

// literals = QUAD (the reference build): the smoothness indicators and the
// alphas of the nonlinear weights in binary128, as gfortran evaluates
// 13d0/12d0*(..)**2 + 0.25d0*(..)**2 and 0.3/(1d-6+beta)**2 under
// -fdefault-real-8, each rounded to binary64 once (weno5.f90:100-106,
// 134-140); the candidate values and the weights stay binary64
struct QuadWeno {
  qd::q128 c1312, eps;  // 13d0/12d0 and the epsilon in binary128
};
static __device__ __noinline__ void weno_beta_qd(double am2, double am1, double a0, double ap1,
                                             double ap2, const QuadWeno& qw, double& b1,
                                             double& b2, double& b3) {
  using namespace qd;
  const q128 m2 = from_double(am2), m1 = from_double(am1), z = from_double(a0);
  const q128 p1 = from_double(ap1), p2 = from_double(ap2), three = from_double(3.0);
  q128 s = add(sub(z, scale2(p1, 1)), p2);
  q128 t = add(sub(mul(three, z), scale2(p1, 2)), p2);
  b1 = to_double(add(mul(qw.c1312, mul(s, s)), scale2(mul(t, t), -2)));
  s = add(sub(m1, scale2(z, 1)), p1);
  b2 = to_double(add(mul(qw.c1312, mul(s, s)), scale2(from_double(dsq(am1 - ap1)), -2)));
  s = add(sub(m2, scale2(m1, 1)), z);
  t = add(sub(m2, scale2(m1, 2)), mul(three, z));
  b3 = to_double(add(mul(qw.c1312, mul(s, s)), scale2(mul(t, t), -2)));
}
__device__ __forceinline__ double weno_alpha_qd(double lin, double beta, const QuadWeno& qw) {
  using namespace qd;
  const q128 s = add(qw.eps, from_double(beta));
  return to_double(div(from_double(lin), mul(s, s)));
}
static __device__ __noinline__ double weno_right_qd(double am2, double am1, double a0, double ap1,
                                                double ap2, const QuadWeno& qw) {
  const double um1 = SWFD_C13 * am2 + SWFD_CM76 * am1 + SWFD_C116 * a0;
  const double um2 = SWFD_CM16 * am1 + SWFD_C56 * a0 + SWFD_C13 * ap1;
  const double um3 = SWFD_C13 * a0 + SWFD_C56 * ap1 + SWFD_CM16 * ap2;
  double b1, b2, b3;
  weno_beta_qd(am2, am1, a0, ap1, ap2, qw, b1, b2, b3);
  const double a1 = weno_alpha_qd(0.3, b1, qw), a2 = weno_alpha_qd(0.6, b2, qw),
               a3 = weno_alpha_qd(0.1, b3, qw);
  const double s = a1 + a2 + a3;
  return sd::div(a1, s) * um3 + sd::div(a2, s) * um2 + sd::div(a3, s) * um1;
}
static __device__ __noinline__ double weno_left_qd(double am2, double am1, double a0, double ap1,
                                               double ap2, const QuadWeno& qw) {
  const double up1 = SWFD_CM16 * am2 + SWFD_C56 * am1 + SWFD_C13 * a0;
  const double up2 = SWFD_C13 * am1 + SWFD_C56 * a0 + SWFD_CM16 * ap1;
  const double up3 = SWFD_C116 * a0 + SWFD_CM76 * ap1 + SWFD_C13 * ap2;
  double b1, b2, b3;
  weno_beta_qd(am2, am1, a0, ap1, ap2, qw, b1, b2, b3);
  const double a1 = weno_alpha_qd(0.1, b1, qw), a2 = weno_alpha_qd(0.6, b2, qw),
               a3 = weno_alpha_qd(0.3, b3, qw);
  const double s = a1 + a2 + a3;
  return sd::div(a1, s) * up3 + sd::div(a2, s) * up2 + sd::div(a3, s) * up1;
}

// weno_right (weno5.f90:120-146)
template <class T, class D = DivHw>
__device__ __forceinline__ T weno_right(T am2, T am1, T a0, T ap1, T ap2, T eps, D div = D()) {
  T um1 = T(SWFD_C13) * am2 + T(SWFD_CM76) * am1 + T(SWFD_C116) * a0;
  T um2 = T(SWFD_CM16) * am1 + T(SWFD_C56) * a0 + T(SWFD_C13) * ap1;
  T um3 = T(SWFD_C13) * a0 + T(SWFD_C56) * ap1 + T(SWFD_CM16) * ap2;
  T b1, b2, b3;
  weno_beta(am2, am1, a0, ap1, ap2, b1, b2, b3);
  T a1 = div(T(0.3), tsq(eps + b1));
  T a2 = div(T(0.6), tsq(eps + b2));
  T a3 = div(T(0.1), tsq(eps + b3));
  T s = a1 + a2 + a3;
  T w1, w2, w3;
  if constexpr (sizeof(T) == 4) {  // FP32-bulk: one reciprocal for the three weights
    const T rs = T(1.) / s;
    w1 = a1 * rs, w2 = a2 * rs, w3 = a3 * rs;
  } else {  // the reference's three divisions (weno5.f90:134-140)
    w1 = div(a1, s), w2 = div(a2, s), w3 = div(a3, s);
  }
  return w1 * um3 + w2 * um2 + w3 * um1;
}

// weno_left (weno5.f90:86-113)
template <class T, class D = DivHw>
__device__ __forceinline__ T weno_left(T am2, T am1, T a0, T ap1, T ap2, T eps, D div = D()) {
  T up1 = T(SWFD_CM16) * am2 + T(SWFD_C56) * am1 + T(SWFD_C13) * a0;
  T up2 = T(SWFD_C13) * am1 + T(SWFD_C56) * a0 + T(SWFD_CM16) * ap1;
  T up3 = T(SWFD_C116) * a0 + T(SWFD_CM76) * ap1 + T(SWFD_C13) * ap2;
  T b1, b2, b3;
  weno_beta(am2, am1, a0, ap1, ap2, b1, b2, b3);
  T a1 = div(T(0.1), tsq(eps + b1));
  T a2 = div(T(0.6), tsq(eps + b2));
  T a3 = div(T(0.3), tsq(eps + b3));
  T s = a1 + a2 + a3;
  T w1, w2, w3;
  if constexpr (sizeof(T) == 4) {
    const T rs = T(1.) / s;
    w1 = a1 * rs, w2 = a2 * rs, w3 = a3 * rs;
  } else {  // weno5.f90:104-110
    w1 = div(a1, s), w2 = div(a2, s), w3 = div(a3, s);
  }
  return w1 * up3 + w2 * up2 + w3 * up1;
}

// Roe-averaged eigenvectors of one interface, in terms of the velocity normal
// (vn) and tangential (vt) to the interface
// (x pass ex3_vortex_accuracy_2d/main.f90:153-199, y pass :354-400).
template <class T>
struct Eigen2D {
  T vn, vt, cm, qm, e_nm, e_np, e_hm, e_hp;  // evr entries
  T l1_0, l1_n, l1_t, l1_3;                  // evl row 1
  T l3_0, l3_n, l3_t, l3_3;                  // evl row 3
  T l4_0, l4_n, l4_t, l4_3;                  // evl row 4 (row 2 is [-vt, 0, 1, 0])
};

// qreg (QD, ex4 and ex6 of the QUAD build only): the 1d-15 regularisers in
// binary128 (ex4_sedov_2d/main.f90:199-210)
template <class T, bool QD = false>
__device__ __forceinline__ void roe_eigen2d(T g1, int ydir, T wl, T wr, T vxl, T vxr, T vyl,
                                            T vyr, T hl, T hr, Eigen2D<T>& E,
                                            const qd::q128* qreg = nullptr) {
  T t0;
  if constexpr (QD) {
    if (qreg)
      t0 = qd::to_double(qd::div(qd::from_double(wl), qd::add(qd::from_double(wl + wr), *qreg)));
    else
      t0 = tdiv(wl, wl + wr + T(1.e-15));
  } else {
    t0 = tdiv(wl, wl + wr + T(1.e-15));
  }
  T t1 = T(1.) - t0;
  T vxm = t0 * vxl + t1 * vxr;
  T vym = t0 * vyl + t1 * vyr;
  T hm = t0 * hl + t1 * hr;
  T qm = tscale<-1>(vxm * vxm + vym * vym);
  T cm;
  if constexpr (QD) {
    if (qreg)
      cm = qd::to_double(qd::add(qd::from_double(tsqrt(tabs(g1 * (hm - qm)))), *qreg));
    else
      cm = tsqrt(tabs(g1 * (hm - qm))) + T(1.e-15);
  } else {
    cm = tsqrt(tabs(g1 * (hm - qm))) + T(1.e-15);
  }
  T vn = ydir ? vym : vxm;
  T vt = ydir ? vxm : vym;
  t0 = vn * cm;
  E.vn = vn;
  E.vt = vt;
  E.cm = cm;
  E.qm = qm;
  E.e_nm = vn - cm;
  E.e_np = vn + cm;
  E.e_hm = hm - t0;
  E.e_hp = hm + t0;
  T rcm = tdiv(T(1.), cm);
  T b1 = g1 * rcm * rcm;
  T b2 = qm * b1;
  t0 = vn * rcm;
  t1 = b1 * vn;
  T t2 = tscale<-1>(b1);
  T t3 = b1 * vt;
  E.l1_0 = tscale<-1>(b2 + t0);
  E.l1_n = tneg(tscale<-1>(t1 + rcm));  // (-0.5)*x == -(0.5*x)
  E.l1_t = tneg(tscale<-1>(t3));
  E.l1_3 = t2;
  E.l3_0 = T(1.) - b2;
  E.l3_n = t1;
  E.l3_t = t3;
  E.l3_3 = tneg(b1);
  E.l4_0 = tscale<-1>(b2 - t0);
  E.l4_n = tneg(tscale<-1>(t1 - rcm));
  E.l4_t = E.l1_t;
  E.l4_3 = t2;
}

// One reconstruction for lane side s as a single instruction stream for both
// sides: weno_right (s = 0) and weno_left (s = 1) of stencil v0..v4 have the
// same shape -- three candidates k1*v_a + k2*v_b + k3*v_c over the same
// positions, the same smoothness indicators, the weights d/(eps+beta)^2
// normalised by three divisions, and w1*A + w2*B + w3*C -- and differ only in
// the constants, which each lane selects; so a warp whose lanes take both
// sides does not diverge, and each side's operations, operands and their
// order are the reference's (weno5.f90:86-146).
template <class D>
__device__ __forceinline__ double weno_side(double v0, double v1, double v2, double v3, double v4,
                                            int side, double eps, D div) {
  // weno_right: A = um3 = c13 v2 + c56 v3 + cm16 v4,  B = um2 = cm16 v1 + c56 v2 + c13 v3,
  //             C = um1 = c13 v0 + cm76 v1 + c116 v2, weights d = 0.3, 0.6, 0.1
  // weno_left:  A = up3 = c116 v2 + cm76 v3 + c13 v4, B = up2 = c13 v1 + c56 v2 + cm16 v3,
  //             C = up1 = cm16 v0 + c56 v1 + c13 v2,  weights d = 0.1, 0.6, 0.3
  const bool l = side != 0;
  const double a1 = l ? SWFD_C116 : SWFD_C13, a2 = l ? SWFD_CM76 : SWFD_C56,
               a3 = l ? SWFD_C13 : SWFD_CM16;
  const double b1 = l ? SWFD_C13 : SWFD_CM16, b3 = l ? SWFD_CM16 : SWFD_C13;
  const double c1 = l ? SWFD_CM16 : SWFD_C13, c2 = l ? SWFD_C56 : SWFD_CM76,
               c3 = l ? SWFD_C13 : SWFD_C116;
  const double d1 = l ? 0.1 : 0.3, d3 = l ? 0.3 : 0.1;
  const double A = a1 * v2 + a2 * v3 + a3 * v4;
  const double B = b1 * v1 + SWFD_C56 * v2 + b3 * v3;
  const double C = c1 * v0 + c2 * v1 + c3 * v2;
  double be1, be2, be3;
  weno_beta(v0, v1, v2, v3, v4, be1, be2, be3);
  const double w1 = div(d1, tsq(eps + be1));
  const double w2 = div(0.6, tsq(eps + be2));
  const double w3 = div(d3, tsq(eps + be3));
  const double sum = w1 + w2 + w3;
  return div(w1, sum) * A + div(w2, sum) * B + div(w3, sum) * C;
}

// FP32-bulk reconstructions: weno5's expressions (weno5.f90:86-146) in
// binary32 with fused multiply-adds and reciprocal-estimate weights
// (__fdividef: CUDA's fast approximate division, within 2 ulp).  The
// FP32-bulk form is accepted by its error against the FP64 form, not bit for
// bit; every FP32 path (one instance, fused stage, batch) calls these, so
// they agree with each other bit for bit.
__device__ __forceinline__ void weno_beta_f32(float am2, float am1, float a0, float ap1, float ap2,
                                              float& b1, float& b2, float& b3) {
  const float c1312 = 13.f / 12.f;
  const float s1 = fmaf(-2.f, ap1, a0) + ap2, t1 = fmaf(3.f, a0, fmaf(-4.f, ap1, ap2));
  const float s2 = fmaf(-2.f, a0, am1) + ap1, t2 = am1 - ap1;
  const float s3 = fmaf(-2.f, am1, am2) + a0, t3 = fmaf(3.f, a0, fmaf(-4.f, am1, am2));
  b1 = fmaf(c1312, s1 * s1, 0.25f * (t1 * t1));
  b2 = fmaf(c1312, s2 * s2, 0.25f * (t2 * t2));
  b3 = fmaf(c1312, s3 * s3, 0.25f * (t3 * t3));
}
// the three nonlinear weights of linear weights d1, d2, d3 applied to the
// candidates c1, c2, c3
__device__ __forceinline__ float weno_combine_f32(float b1, float b2, float b3, float d1, float d2,
                                                  float d3, float c1, float c2, float c3,
                                                  float eps) {
  const float e1 = eps + b1, e2 = eps + b2, e3 = eps + b3;
  const float a1 = __fdividef(d1, e1 * e1), a2 = __fdividef(d2, e2 * e2),
              a3 = __fdividef(d3, e3 * e3);
  const float rs = __fdividef(1.f, a1 + a2 + a3);
  return fmaf(a1 * rs, c1, fmaf(a2 * rs, c2, (a3 * rs) * c3));
}
__device__ __forceinline__ float weno_right(float am2, float am1, float a0, float ap1, float ap2,
                                            float eps) {
  const float um1 = fmaf(float(SWFD_C116), a0, fmaf(float(SWFD_CM76), am1, float(SWFD_C13) * am2));
  const float um2 = fmaf(float(SWFD_C13), ap1, fmaf(float(SWFD_C56), a0, float(SWFD_CM16) * am1));
  const float um3 = fmaf(float(SWFD_CM16), ap2, fmaf(float(SWFD_C56), ap1, float(SWFD_C13) * a0));
  float b1, b2, b3;
  weno_beta_f32(am2, am1, a0, ap1, ap2, b1, b2, b3);
  return weno_combine_f32(b1, b2, b3, 0.3f, 0.6f, 0.1f, um3, um2, um1, eps);
}
__device__ __forceinline__ float weno_left(float am2, float am1, float a0, float ap1, float ap2,
                                           float eps) {
  const float up1 = fmaf(float(SWFD_C13), a0, fmaf(float(SWFD_C56), am1, float(SWFD_CM16) * am2));
  const float up2 = fmaf(float(SWFD_CM16), ap1, fmaf(float(SWFD_C56), a0, float(SWFD_C13) * am1));
  const float up3 = fmaf(float(SWFD_C13), ap2, fmaf(float(SWFD_CM76), ap1, float(SWFD_C116) * a0));
  float b1, b2, b3;
  weno_beta_f32(am2, am1, a0, ap1, ap2, b1, b2, b3);
  return weno_combine_f32(b1, b2, b3, 0.1f, 0.6f, 0.3f, up3, up2, up1, eps);
}

// evl(k,:) . f with f in component order (rho, m_x, m_y, E), summed left to
// right over the component index as the reference does (main.f90:212-213).
// FP32-bulk: the same sums with fused multiply-adds.
template <int YDIR, class T>
__device__ __forceinline__ T proj_row(T l0, T ln, T lt, T l3, T f0, T f1, T f2, T f3) {
  if constexpr (sizeof(T) == 4) {
    if (!YDIR) return fmaf(l3, f3, fmaf(lt, f2, fmaf(ln, f1, l0 * f0)));
    return fmaf(l3, f3, fmaf(ln, f2, fmaf(lt, f1, l0 * f0)));
  }
  if (!YDIR) return l0 * f0 + ln * f1 + lt * f2 + l3 * f3;
  return l0 * f0 + lt * f1 + ln * f2 + l3 * f3;
}
// evl row 2: x pass [-vym, 0, 1, 0] -> f2 - vym*f0; y pass [-vxm, 1, 0, 0] -> f1 - vxm*f0
template <int YDIR, class T>
__device__ __forceinline__ T proj_row2(T vt, T f0, T f1, T f2) {
  if constexpr (sizeof(T) == 4) return fmaf(-vt, f0, YDIR ? f1 : f2);
  if (!YDIR) return -vt * f0 + f2;
  return -vt * f0 + f1;
}

}  // namespace swfd
