// swfd_1d.cuh -- the per-cell expressions of the 1D point-energy solver
// (ex2_sedov_1d/main.f90): findalpha of a cell, fflux and the Lax-Friedrichs
// split, the cell-centred eigenvectors, one lane's reconstruction and the
// back projection, the scheme's RHS, the RK combination and
// checkpositivity.  The separate stage kernels (swfd_kernels.cu) and the
// persistent solve kernel (swfd_solve1d.cu) both call these, so that every
// value is computed by the same code in both.
#pragma once

#include "swfd_device.cuh"

namespace swfd {


// findalpha of one cell (ex2_sedov_1d/main.f90:278-283); the caller takes
// max(0, .) over the cells
__device__ __forceinline__ double alpha1d(const Params& p, double u1, double u2, double u3) {
  const double g1 = p.gamma1, gamma = p.gamma;
  int bad = 0;
  double k2 = div_nfz(u2 * u2, u1, bad), v = div_nfz(u2, u1, bad);
  if (bad) k2 = tdiv(u2 * u2, u1), v = tdiv(u2, u1);
  double pres = g1 * (u3 - tscale<-1>(k2));
  double sound = sqrt(tdiv(gamma * pres, u1));
  return fabs(v) + sound;
}

// fflux (ex2_sedov_1d/main.f90:57-73) of one cell
__device__ __forceinline__ void fflux1d(const Params& p, double rho, double mx, double e,
                                        double f[3]) {
  const double g1 = p.gamma1;
  double vx = 0.;
  if (rho > p.lim8_gt) vx = tdiv(mx, rho);
  if (rho <= p.lim8_le) vx = 0.;
  double pres = g1 * (e - 0.5 * rho * (vx * vx));
  f[0] = mx;
  f[1] = rho * (vx * vx) + pres;
  f[2] = (e + pres) * vx;
}

// the split of one cell from its state a and fflux f:
// fp = 0.5 (u + f/alphamax), fn = 0.5 (u - f/alphamax)  (:82-85); the
// divisions are tdiv's correctly rounded quotients (the hardware's bits)
template <class T>
__device__ __forceinline__ void split1d_f(const double a[3], const double f[3], double amd,
                                          T sp[3], T sn[3]) {
  const T am = T(amd);
  T q[3];
  if constexpr (sizeof(T) == 8) {
    int bad = 0;
    for (int c = 0; c < 3; ++c) q[c] = div_nfz(f[c], amd, bad);
    if (bad)
      for (int c = 0; c < 3; ++c) q[c] = tdiv(f[c], amd);
  } else {
    for (int c = 0; c < 3; ++c) q[c] = tdiv(T(f[c]), am);
  }
  for (int c = 0; c < 3; ++c) {  // 0.5d0* as an exponent shift (tscale): the same values
    sp[c] = tscale<-1>(T(a[c]) + q[c]);
    sn[c] = tscale<-1>(T(a[c]) - q[c]);
  }
}

// one component of split1d_f (binary64): the same values, one division
__device__ __forceinline__ void split1d_one(double u, double f, double amd, double& sp,
                                            double& sn) {
  int bad = 0;
  double q = div_nfz(f, amd, bad);
  if (bad) q = tdiv(f, amd);
  sp = tscale<-1>(u + q);
  sn = tscale<-1>(u - q);
}

template <class T>
__device__ __forceinline__ void split1d(const Params& p, double rho, double mx, double e,
                                        double amd, T sp[3], T sn[3]) {
  const double a[3] = {rho, mx, e};
  double f[3];
  fflux1d(p, rho, mx, e, f);
  split1d_f<T>(a, f, amd, sp, sn);
}

// eigenvectors at cell m (ex2_sedov_1d/main.f90:103-133): vxm and hm come
// from the FP64 state (pressure recovery), the rest is in T
template <class T>
struct Eigen1D {
  T vxm, qm, r10, r12, r20, r22;  // evr rows 2 and 3 (row 1 is ones)
  T L[3][3];                      // evl
};
template <class T>
__device__ __forceinline__ void eigen1d(double g1d, double u1, double u2, double u3,
                                        Eigen1D<T>& E) {
  int bad = 0;
  double vxd = div_nfz(u2, u1, bad), k2 = div_nfz(tscale<-1>(u2 * u2), u1, bad);
  if (bad) vxd = tdiv(u2, u1), k2 = tdiv(tscale<-1>(u2 * u2), u1);
  double hmd = tdiv(g1d * (u3 - k2) + u3, u1);
  const T g1 = T(g1d), vxm = T(vxd), hm = T(hmd);
  T qm = tscale<-1>(vxm) * vxm;
  T cm = sqrt(g1 * (hm - qm));
  T t0 = vxm * cm;
  E.vxm = vxm;
  E.qm = qm;
  E.r10 = vxm - cm, E.r12 = vxm + cm, E.r20 = hm - t0, E.r22 = hm + t0;
  T rcm = tdiv(T(1.), cm);
  T b1 = g1 * rcm * rcm;
  T b2 = qm * b1;
  t0 = vxm * rcm;
  T t1 = b1 * vxm;
  T t2 = tscale<-1>(b1);
  // (-0.5)*x == -(0.5*x); the negations as sign flips (tneg)
  E.L[0][0] = tscale<-1>(b2 + t0), E.L[0][1] = tneg(tscale<-1>(t1 + rcm)), E.L[0][2] = t2;
  E.L[1][0] = T(1.) - b2, E.L[1][1] = t1, E.L[1][2] = tneg(b1);
  E.L[2][0] = tscale<-1>(b2 - t0), E.L[2][1] = tneg(tscale<-1>(t1 - rcm)), E.L[2][2] = t2;
}

static __device__ __noinline__ double weno_side_hw(double v0, double v1, double v2, double v3,
                                                   double v4, int side, double eps) {
  return weno_side(v0, v1, v2, v3, v4, side, eps, DivHw());
}

// One lane of a cell's group of eight: lane sub 0..5 reconstructs field
// k = sub/2 of side sub%2 (0: weno_right of the positive split flux, 1:
// weno_left of the negative one); lanes 6 and 7 repeat lane 0's work.
// sp(side, c, jj): split component c of the side at cell m + jj - 2.
template <class T, bool QD, class SP>
__device__ __forceinline__ T recon1d(const Params& p, const Eigen1D<T>& E, int sub, SP sp) {
  const T weps = T(p.weno_eps);
  const int k = sub < 6 ? sub >> 1 : 0, side = sub & 1;
  // row k of evl, selected in registers
  const T l0 = k == 0 ? E.L[0][0] : k == 1 ? E.L[1][0] : E.L[2][0];
  const T l1 = k == 0 ? E.L[0][1] : k == 1 ? E.L[1][1] : E.L[2][1];
  const T l2 = k == 0 ? E.L[0][2] : k == 1 ? E.L[1][2] : E.L[2][2];
  T cs[5];
#pragma unroll
  for (int jj = 0; jj < 5; ++jj)
    cs[jj] = l0 * sp(side, 0, jj) + l1 * sp(side, 1, jj) + l2 * sp(side, 2, jj);
  T v;
  if constexpr (QD) {
    const QuadWeno qw{p.q_c1312, p.q_weno_eps};
    v = side ? weno_left_qd(cs[0], cs[1], cs[2], cs[3], cs[4], qw)
             : weno_right_qd(cs[0], cs[1], cs[2], cs[3], cs[4], qw);
  } else if constexpr (sizeof(T) == 8) {
    // weno_right and weno_left as one instruction stream (the lanes of a
    // group take both sides without diverging), its divisions straight-line
    int bad = 0;
    v = weno_side(cs[0], cs[1], cs[2], cs[3], cs[4], side, weps, DivFlag{&bad});
    if (bad) v = weno_side_hw(cs[0], cs[1], cs[2], cs[3], cs[4], side, weps);
  } else {
    v = side ? weno_left(cs[0], cs[1], cs[2], cs[3], cs[4], weps)
             : weno_right(cs[0], cs[1], cs[2], cs[3], cs[4], weps);
  }
  return v;
}

// output component sub (0..5) of a cell's interface fluxes from its six
// reconstructions: 0..2 the positive flux evr . ur, 3..5 the negative one
// evr . ul (:152-157); lanes 6 and 7 get a value nobody stores
template <class T>
__device__ __forceinline__ T back1d_combine(const Eigen1D<T>& E, T ur0, T ul0, T ur1, T ul1, T ur2,
                                            T ul2, int sub) {
  // one instruction stream for the six lanes (a warp pays for every FP64
  // instruction of every branch its lanes take): the lane's row of evr and
  // side selected in registers; row 1 is ones, and 1*x is x exactly
  const int row = sub % 3;
  const bool neg = sub >= 3;
  const T a0 = neg ? ul0 : ur0, a1 = neg ? ul1 : ur1, a2 = neg ? ul2 : ur2;
  const T e0 = row == 0 ? T(1) : row == 1 ? E.r10 : E.r20;
  const T e1 = row == 0 ? T(1) : row == 1 ? E.vxm : E.qm;
  const T e2 = row == 0 ? T(1) : row == 1 ? E.r12 : E.r22;
  return e0 * a0 + e1 * a1 + e2 * a2;
}

// The group of G (8 or 16) aligned lanes exchanges its six reconstructions
// by warp shuffles (every lane of the warp takes part): reconstruction m
// (field m/2, side m%2) is on lane m * G/8 of the group, and lane sub 0..5
// returns output component sub
template <class T, int G = 8>
__device__ __forceinline__ T back1d(const Eigen1D<T>& E, T v, int sub) {
  static_assert(G == 8 || G == 16, "groups of eight or sixteen lanes");
  constexpr int S = G / 8;
  const int base = threadIdx.x & ~(G - 1) & 31;
  const T ur0 = __shfl_sync(0xffffffffu, v, base + 0 * S);
  const T ul0 = __shfl_sync(0xffffffffu, v, base + 1 * S);
  const T ur1 = __shfl_sync(0xffffffffu, v, base + 2 * S);
  const T ul1 = __shfl_sync(0xffffffffu, v, base + 3 * S);
  const T ur2 = __shfl_sync(0xffffffffu, v, base + 4 * S);
  const T ul2 = __shfl_sync(0xffffffffu, v, base + 5 * S);
  return back1d_combine(E, ur0, ul0, ur1, ul1, ur2, ul2, sub);
}

// The persistent solve's reconstruction: sixteen lanes per flux cell, two
// per reconstruction.  The pair u = sub/2 (u < 6) reconstructs field u/2 of
// side u%2 as recon1d's lane u does (pairs 6 and 7 repeat pairs 0 and 1);
// each lane of the pair takes part of weno_side's operations, so the warp
// issues ~50 FP64 instructions for a reconstruction instead of ~80.  Lane 0
// of the pair projects the stencil values v2..v4 and forms the candidate of
// v2..v4 with its smoothness indicator and weight; lane 1 projects v0..v2
// and does the same for the candidate of v0..v2; both form the middle
// candidate and weight from v1..v3 (one value from the partner), the sum of
// the weights and the normalised terms; lane 0 adds the partner's term and
// returns the reconstruction.  Every operation, operand and order is
// weno_side's (weno5.f90:86-146), so the value equals recon1d's.
template <class SP>
__device__ __forceinline__ double recon1d_pair(const Params& p, const Eigen1D<double>& E, int sub,
                                               SP sp) {
  const double eps = p.weno_eps;
  const int u = sub >> 1, h = sub & 1;
  const int k = u < 6 ? u >> 1 : 0, side = u & 1;
  const double l0 = k == 0 ? E.L[0][0] : k == 1 ? E.L[1][0] : E.L[2][0];
  const double l1 = k == 0 ? E.L[0][1] : k == 1 ? E.L[1][1] : E.L[2][1];
  const double l2 = k == 0 ? E.L[0][2] : k == 1 ? E.L[1][2] : E.L[2][2];
  const int j0 = h ? 0 : 2;
  double c[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    c[i] = l0 * sp(side, 0, j0 + i) + l1 * sp(side, 1, j0 + i) + l2 * sp(side, 2, j0 + i);
  // the partner's middle value: v1 on lane 0, v3 on lane 1
  const double o = __shfl_xor_sync(0xffffffffu, c[1], 1);
  const double v1 = h ? c[1] : o, v2 = h ? c[2] : c[0], v3 = h ? o : c[1];
  const bool l = side != 0;
  // the lane's own candidate: A = a1 v2 + a2 v3 + a3 v4 (lane 0) or
  // C = c1 v0 + c2 v1 + c3 v2 (lane 1), weno_side's constants
  const double k1 = h ? (l ? SWFD_CM16 : SWFD_C13) : (l ? SWFD_C116 : SWFD_C13);
  const double k2 = h ? (l ? SWFD_C56 : SWFD_CM76) : (l ? SWFD_CM76 : SWFD_C56);
  const double k3 = h ? (l ? SWFD_C13 : SWFD_C116) : (l ? SWFD_C13 : SWFD_CM16);
  const double P = k1 * c[0] + k2 * c[1] + k3 * c[2];
  // its smoothness indicator (weno_beta): beta1 of v2..v4 on lane 0, beta3
  // of v0..v2 on lane 1; s is the same form, t1 = 3 v2 - 4 v3 + v4 and
  // t3 = v0 - 4 v1 + 3 v2
  const double c1312 = 13.0 / 12.0;
  const double s = c[0] - tscale<1>(c[1]) + c[2];
  const double m3 = 3.0 * (h ? c[2] : c[0]);
  const double t = (h ? c[0] : m3) - tscale<2>(c[1]) + (h ? m3 : c[2]);
  const double bP = c1312 * tsq(s) + tscale<-2>(tsq(t));
  // the middle candidate B and beta2 of v1..v3, on both lanes
  const double b1 = l ? SWFD_C13 : SWFD_CM16, b3 = l ? SWFD_CM16 : SWFD_C13;
  const double B = b1 * v1 + SWFD_C56 * v2 + b3 * v3;
  const double s2 = v1 - tscale<1>(v2) + v3, t2 = v1 - v3;
  const double bB = c1312 * tsq(s2) + tscale<-2>(tsq(t2));
  int bad = 0;
  const DivFlag dv{&bad};
  const double dP = h ? (l ? 0.3 : 0.1) : (l ? 0.1 : 0.3);
  const double wP = dv(dP, tsq(eps + bP));
  const double w2 = dv(0.6, tsq(eps + bB));
  const double ow = __shfl_xor_sync(0xffffffffu, wP, 1);
  const double w1 = h ? ow : wP, w3 = h ? wP : ow;
  const double sum = w1 + w2 + w3;
  const double tP = dv(wP, sum) * P;
  const double s12 = tP + dv(w2, sum) * B;  // lane 0: w1/sum * A + w2/sum * B
  const double oP = __shfl_xor_sync(0xffffffffu, tP, 1);
  double v = s12 + oP;  // lane 0: + w3/sum * C
  if (__any_sync(0xffffffffu, bad)) {  // a quotient outside sd::div's range: hardware division
    const double y0 = __shfl_xor_sync(0xffffffffu, c[0], 1);
    if (h == 0) v = weno_side_hw(y0, v1, c[0], c[1], c[2], side, eps);
  }
  return v;
}

// use_limiter = 1 (ex2_sedov_1d/main.f90:159-245): the positivity limiter
// of one split flux of cell m.  ave: the split flux at cell m (hp(:, m) or
// hn(:, m)), out: its reconstructed flux (hp_flux(:, m) or hn_flux(:, m)),
// limited in place; nd, np count the density and pressure limitings.
template <class T>
__device__ __forceinline__ void zs_limit1d(const Params& p, const T ave[3], T out[3], int& nd,
                                           int& np) {
  const T g1 = T(p.gamma1);
  const T d_ave = ave[0], m_ave = ave[1], e_ave = ave[2];
  const T p_ave = g1 * (e_ave - T(0.5) * (m_ave * m_ave) / d_ave);
  T pt[2][3];
  for (int c = 0; c < 3; ++c) {
    pt[0][c] = out[c];
    pt[1][c] = (ave[c] - out[c] / T(12.)) / T(11. / 12.);
  }
  T theta = T(1.);
  for (int ig = 0; ig < 2; ++ig) {
    const T d_l = pt[ig][0];
    if (d_l < T(0.)) theta = fmin(theta, fabs(d_ave - T(0.)) / fabs(d_ave - d_l));
  }
  if (theta < T(1.)) {
    out[0] = theta * out[0] + (T(1.) - theta) * d_ave;
    ++nd;
  }
  theta = T(1.);
  pt[0][0] = out[0];
  pt[1][0] = (ave[0] - out[0] / T(12.)) / T(11. / 12.);
  for (int ig = 0; ig < 2; ++ig) {
    const T d_l = pt[ig][0], m_l = pt[ig][1], e_l = pt[ig][2];
    const T p_l = g1 * (e_l - (m_l * m_l) / d_l / T(2.));
    if (p_l < T(0.)) theta = fmin(theta, fabs(p_ave - T(0.)) / fabs(p_ave - p_l));
  }
  if (theta < T(1.)) {
    ++np;
    for (int c = 0; c < 3; ++c) out[c] = theta * out[c] + (T(1.) - theta) * ave[c];
  }
}

// the limitings into den_count and pre_count (cnt[0], cnt[1])
__device__ __forceinline__ void count_limited(unsigned long long* cnt, int nd, int np) {
  if (nd) atomicAdd(cnt, (unsigned long long)nd);
  if (np) atomicAdd(cnt + 1, (unsigned long long)np);
}

// The limiter on a cell's two reconstructed split fluxes, after back1d (a
// group of G lanes): lane 0 of the group limits hp_flux (its three components from lanes 0..2),
// lane 3 hn_flux (lanes 3..5); ave(side, c) is the split value at cell m.
// Every lane of the warp takes part; lanes 0 and 3 return true with w, the
// side's limited components, and add their limitings to nd, np.
template <class T, int G = 8, class AV>
__device__ __forceinline__ bool limit1d_group(const Params& p, T r, int sub, AV ave, T w[3],
                                              int& nd, int& np) {
  const int base = (threadIdx.x & ~(G - 1) & 31) + (sub >= 3 ? 3 : 0);
#pragma unroll
  for (int c = 0; c < 3; ++c) w[c] = __shfl_sync(0xffffffffu, r, base + c);
  if (sub != 0 && sub != 3) return false;
  const int side = sub == 3;
  const T a[3] = {ave(side, 0), ave(side, 1), ave(side, 2)};
  zs_limit1d<T>(p, a, w, nd, np);
  return true;
}

// scheme of one component of an interior cell (ex2_sedov_1d/main.f90:252-271):
// flus(i) = alphamax*(hp(i-1) - hn(i)), RHS = -(flus(i+1) - flus(i))/dx, from
// hp(i-1), hn(i), hp(i), hn(i+1)
template <class T>
__device__ __forceinline__ T rhs1d_value(const Params& p, double amd, T hp_m, T hn_0, T hp_0,
                                         T hn_p) {
  const T am = T(amd);
  T fl_i = am * (hp_m - hn_0);
  T fl_ip1 = am * (hp_0 - hn_p);
  return -tdiv(fl_ip1 - fl_i, T(p.dx));
}

// u = 0.75d0*u0 + 0.25d0*v and u = (u0 + 2d0*v)/3d0 (ex2_sedov_1d/main.f90:310,321;
// ex3_vortex_accuracy_2d/main.f90:604,621); in binary128 for the QUAD build
// (0.75*u0 and 0.25*v are exact there).  u0 may alias the stage's output
// (stage 3 writes the step-start buffer): each element of u0 is read only by
// the thread that then writes it.
__device__ __forceinline__ double rk_combine(const Params& p, int stage, double u0, double v) {
  if (p.quad) {
    using namespace qd;
    if (stage == 2)
      return to_double(add(mul(from_double(0.75), from_double(u0)), scale2(from_double(v), -2)));
    return to_double(div(add(from_double(u0), scale2(from_double(v), 1)), from_double(3.0)));
  }
  if (stage == 2) return 0.75 * u0 + tscale<-2>(v);
  return tdiv(u0 + tscale<1>(v), 3.0);
}

// one component's RK stage value from its state u, RHS r and (stages 2 and
// 3) u0 at *u0p; FP32-bulk accumulates in FP64 with fused multiply-adds
template <class T>
__device__ __forceinline__ double rk1d_value(const Params& p, int stage, double dt, double r,
                                             double u, const double* u0p) {
  double v;
  if (sizeof(T) == 4) {
    v = fma(dt, r, u);
    if (stage == 2) v = fma(0.75, *u0p, 0.25 * v);
    else if (stage == 3) v = fma(2.0, v, *u0p) * (1.0 / 3.0);
  } else {
    v = u + dt * r;
    if (stage >= 2) v = rk_combine(p, stage, *u0p, v);
  }
  return v;
}

// checkpositivity of one cell (ex2_sedov_1d/main.f90:381-387)
template <class T>
__device__ __forceinline__ int pos1d_bad(const Params& p, double n0, double n1, double n2) {
  double pe;
  if (sizeof(T) == 4) pe = fma(n1 * n1, -0.5 * rcp_bulk(n0), n2);
  else pe = n2 - tscale<-1>(tdiv(n1 * n1, n0));
  if (p.pos_strict) return (n0 < p.eps) || (pe < p.eps);
  return (n0 <= p.eps) || (pe <= p.eps);
}

}  // namespace swfd
