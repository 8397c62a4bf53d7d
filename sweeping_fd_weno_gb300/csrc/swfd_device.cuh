// swfd_device.cuh -- device arithmetic shared by the kernels.
//
// Every expression keeps the reference's Fortran operation order.  The
// library is compiled with -fmad=false so that no multiply-add is contracted
// (the x86-64 reference build has no FMA).  Terms the reference multiplies by
// the constants 0 or 1 inside the eigenvector products are left out: x*1 is
// exact and adding an exact zero does not change a nonzero sum, so the
// values are identical (only the sign of an exactly-zero result may differ).
#pragma once

#include "swfd_internal.h"

namespace swfd {

// c(-1:2,0:2) of MODULE weno5 (ex3_vortex_accuracy_2d/weno5.f90:3-15)
#define SWFD_C13 0.333333333333333333333333333333333
#define SWFD_C56 0.833333333333333333333333333333333
#define SWFD_CM16 (-0.166666666666666666666666666666667)
#define SWFD_C116 1.83333333333333333333333333333333
#define SWFD_CM76 (-1.16666666666666666666666666666667)

__device__ __forceinline__ double dsq(double a) { return a * a; }

// beta(1:3) (weno5.f90:100-102); am2..ap2 = average(-2..2)
__device__ __forceinline__ void weno_beta(double am2, double am1, double a0, double ap1, double ap2,
                                          double& b1, double& b2, double& b3) {
  const double c1312 = 13.0 / 12.0;
  b1 = c1312 * dsq(a0 - 2.0 * ap1 + ap2) + 0.25 * dsq(3.0 * a0 - 4.0 * ap1 + ap2);
  b2 = c1312 * dsq(am1 - 2.0 * a0 + ap1) + 0.25 * dsq(am1 - ap1);
  b3 = c1312 * dsq(am2 - 2.0 * am1 + a0) + 0.25 * dsq(am2 - 4.0 * am1 + 3.0 * a0);
}

// weno_right (weno5.f90:120-146)
__device__ __forceinline__ double weno_right(double am2, double am1, double a0, double ap1,
                                             double ap2, double eps) {
  double um1 = SWFD_C13 * am2 + SWFD_CM76 * am1 + SWFD_C116 * a0;
  double um2 = SWFD_CM16 * am1 + SWFD_C56 * a0 + SWFD_C13 * ap1;
  double um3 = SWFD_C13 * a0 + SWFD_C56 * ap1 + SWFD_CM16 * ap2;
  double b1, b2, b3;
  weno_beta(am2, am1, a0, ap1, ap2, b1, b2, b3);
  double a1 = 0.3 / dsq(eps + b1);
  double a2 = 0.6 / dsq(eps + b2);
  double a3 = 0.1 / dsq(eps + b3);
  double s = a1 + a2 + a3;
  double w1 = a1 / s, w2 = a2 / s, w3 = a3 / s;
  return w1 * um3 + w2 * um2 + w3 * um1;
}

// weno_left (weno5.f90:86-113)
__device__ __forceinline__ double weno_left(double am2, double am1, double a0, double ap1,
                                            double ap2, double eps) {
  double up1 = SWFD_CM16 * am2 + SWFD_C56 * am1 + SWFD_C13 * a0;
  double up2 = SWFD_C13 * am1 + SWFD_C56 * a0 + SWFD_CM16 * ap1;
  double up3 = SWFD_C116 * a0 + SWFD_CM76 * ap1 + SWFD_C13 * ap2;
  double b1, b2, b3;
  weno_beta(am2, am1, a0, ap1, ap2, b1, b2, b3);
  double a1 = 0.1 / dsq(eps + b1);
  double a2 = 0.6 / dsq(eps + b2);
  double a3 = 0.3 / dsq(eps + b3);
  double s = a1 + a2 + a3;
  double w1 = a1 / s, w2 = a2 / s, w3 = a3 / s;
  return w1 * up3 + w2 * up2 + w3 * up1;
}

// Roe-averaged eigenvectors of one interface, in terms of the velocity normal
// (vn) and tangential (vt) to the interface
// (x pass ex3_vortex_accuracy_2d/main.f90:153-199, y pass :354-400).
struct Eigen2D {
  double vn, vt, cm, qm, e_nm, e_np, e_hm, e_hp;  // evr entries
  double l1_0, l1_n, l1_t, l1_3;                  // evl row 1
  double l3_0, l3_n, l3_t, l3_3;                  // evl row 3
  double l4_0, l4_n, l4_t, l4_3;                  // evl row 4 (row 2 is [-vt, 0, 1, 0])
};

__device__ __forceinline__ void roe_eigen2d(double g1, int ydir, double wl, double wr, double vxl,
                                            double vxr, double vyl, double vyr, double hl, double hr,
                                            Eigen2D& E) {
  double t0 = wl / (wl + wr + 1.e-15);
  double t1 = 1. - t0;
  double vxm = t0 * vxl + t1 * vxr;
  double vym = t0 * vyl + t1 * vyr;
  double hm = t0 * hl + t1 * hr;
  double qm = 0.5 * (vxm * vxm + vym * vym);
  double cm = sqrt(fabs(g1 * (hm - qm))) + 1.e-15;
  double vn = ydir ? vym : vxm;
  double vt = ydir ? vxm : vym;
  t0 = vn * cm;
  E.vn = vn;
  E.vt = vt;
  E.cm = cm;
  E.qm = qm;
  E.e_nm = vn - cm;
  E.e_np = vn + cm;
  E.e_hm = hm - t0;
  E.e_hp = hm + t0;
  double rcm = 1. / cm;
  double b1 = g1 * rcm * rcm;
  double b2 = qm * b1;
  t0 = vn * rcm;
  t1 = b1 * vn;
  double t2 = 0.5 * b1;
  double t3 = b1 * vt;
  E.l1_0 = 0.5 * (b2 + t0);
  E.l1_n = -0.5 * (t1 + rcm);
  E.l1_t = -0.5 * t3;
  E.l1_3 = t2;
  E.l3_0 = 1. - b2;
  E.l3_n = t1;
  E.l3_t = t3;
  E.l3_3 = -b1;
  E.l4_0 = 0.5 * (b2 - t0);
  E.l4_n = -0.5 * (t1 - rcm);
  E.l4_t = -0.5 * t3;
  E.l4_3 = t2;
}

// evl(k,:) . f with f in component order (rho, m_x, m_y, E), summed left to
// right over the component index as the reference does (main.f90:212-213).
template <int YDIR>
__device__ __forceinline__ double proj_row(double l0, double ln, double lt, double l3, double f0,
                                           double f1, double f2, double f3) {
  if (!YDIR) return l0 * f0 + ln * f1 + lt * f2 + l3 * f3;
  return l0 * f0 + lt * f1 + ln * f2 + l3 * f3;
}
// evl row 2: x pass [-vym, 0, 1, 0] -> f2 - vym*f0; y pass [-vxm, 1, 0, 0] -> f1 - vxm*f0
template <int YDIR>
__device__ __forceinline__ double proj_row2(double vt, double f0, double f1, double f2) {
  if (!YDIR) return -vt * f0 + f2;
  return -vt * f0 + f1;
}

}  // namespace swfd
