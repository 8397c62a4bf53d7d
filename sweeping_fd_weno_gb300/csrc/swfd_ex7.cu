// swfd_ex7.cu -- the reactive Euler detonation of ex7_detonation/main.f90.
//
// Five components (rho, m_x, m_y, E, rho*Y), the equation of state
// p = g1*(E - kinetic - q*rho*Y) (:168-174), the chemistry source
// -k*rho*Y*exp(-t*rho/p) on the fifth component (:752-771), 5x5 Roe
// eigenvectors (:241-308, :524-584).  The reference runs on cut_x x cut_y MPI
// ranks, and its arithmetic depends on that layout (per-rank-row and
// per-rank-column Lax-Friedrichs alpha, a wall mirror applied to the local
// arrays of the ranks on the left edge, fluxes at rank boundaries computed by
// both neighbours), so the ranks are kept: every rank's local grid
// u(5,-2:nxl+3,-2:nyl+3) with its own ghost layers is a slice of one device
// buffer, and each kernel runs over all ranks at once.  Exchanges copy ghost
// layers between slices in the reference's order; the sweep works on the
// gathered interior as rank 0 does.
//
// Arithmetic: binary64 in the reference's operation order (the library is
// built with -fmad=false), divisions and power-of-two products through
// tdiv/tscale (the same bits as the hardware operations), exp through
// qd::exp_rd (binary128, rounded once), which the oracle evaluates with the
// same binary128 operations.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "swfd_device.cuh"
#include "swfd_ex7.h"
#include "swfd_graph.h"

namespace swfd {

namespace {

constexpr int E7_BLOCK = 256;

// ordered key of a binary64 value for atomicMin (NaN values are skipped by the callers)
__device__ __forceinline__ unsigned long long e7_key(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double e7_unkey(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  memcpy(&d, &b, 8);
  return d;
}

// the slice of rank r: component c, local cell (i, j), i and j from -2
__device__ __forceinline__ int64_t e7_at(const Ex7View& e, int r, int c, int i, int j) {
  return ((int64_t)(r * 5 + c) * e.LJ + (j + 2)) * e.LI + (i + 2);
}
__device__ __forceinline__ int64_t e7_cell(const Ex7View& e, int r, int i, int j) {
  return ((int64_t)r * e.LJ + (j + 2)) * e.LI + (i + 2);
}

// eos (:168-174): g1*(e - 0.5*rho*vx**2 - 0.5*rho*vy**2 - q*y)
__device__ __forceinline__ double e7_eos(const Ex7View& e, double rho, double vx, double vy,
                                         double en, double y) {
  const double hr = tscale<-1>(rho);
  return e.g1 * (en - hr * (vx * vx) - hr * (vy * vy) - e.q * y);
}

// fflux / gflux (:110-166)
__device__ __forceinline__ void e7_flux(const Ex7View& e, const double* a, double* f, int gdir) {
  const double rho = a[0], mx = a[1], my = a[2], en = a[3], y = a[4];
  double vx = tdiv(mx, rho), vy = tdiv(my, rho);
  if (rho < e.eps2) vx = 0.;
  if (rho < e.eps2) vy = 0.;
  const double pres = e7_eos(e, rho, vx, vy, en, y);
  if (!gdir) {
    f[0] = mx;
    f[1] = rho * (vx * vx) + pres;
    f[2] = rho * vx * vy;
    f[3] = (en + pres) * vx;
    f[4] = y * vx;
  } else {
    f[0] = my;
    f[1] = rho * vx * vy;
    f[2] = rho * (vy * vy) + pres;
    f[3] = (en + pres) * vy;
    f[4] = y * vy;
  }
}

// per-line Roe preparation (:200-215, :474-489): {w, vx, vy, ratio, h}
__device__ __forceinline__ void e7_prep(const Ex7View& e, const double* a, double* out) {
  const double den = a[0], xmt = a[1], ymt = a[2], eng = a[3], yrho = a[4];
  const double t0 = tdiv(1., den), vex = xmt * t0, vey = ymt * t0;
  const double pre = e.g1 * (eng - tscale<-1>(xmt * vex + ymt * vey) - e.q * yrho);
  out[0] = sqrt(fabs(den));
  out[1] = vex;
  out[2] = vey;
  out[3] = yrho * t0;
  out[4] = (pre + eng) * t0;
}

// chemsource (:752-771): -k*y*exp(-t*rho/p)
__device__ __forceinline__ double e7_chem(const Ex7View& e, const double* a) {
  const double rho = a[0], mx = a[1], my = a[2], en = a[3], y = a[4];
  double vx = tdiv(mx, rho), vy = tdiv(my, rho);
  if (rho < e.lim8_lt) vx = 0.;  // rho < 1d-8
  if (rho < e.lim8_lt) vy = 0.;
  const double pres = e7_eos(e, rho, vx, vy, en, y);
  return -(e.kc * y * qd::exp_rd(-tdiv(e.tc * rho, pres), e.expc));
}

// ---------------------------------------------------------------------------
// findalpha (:774-808): per-cell alpha of every rank's local cells (ghosts
// included) and the global maximum (NaN values skipped, as MAX does)
// ---------------------------------------------------------------------------
__global__ void k7_alpha(Ex7View e) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)e.R * e.LI * e.LJ;
  double v = 0.;
  if (t < n) {
    const int r = (int)(t / ((int64_t)e.LI * e.LJ));
    const int cell = (int)(t % ((int64_t)e.LI * e.LJ));
    const int i = cell % e.LI - 2, j = cell / e.LI - 2;
    const double u1 = e.u[e7_at(e, r, 0, i, j)], u2 = e.u[e7_at(e, r, 1, i, j)],
                 u3 = e.u[e7_at(e, r, 2, i, j)], u4 = e.u[e7_at(e, r, 3, i, j)],
                 u5 = e.u[e7_at(e, r, 4, i, j)];
    const double den = u1;
    double vx, vy;
    if (den >= e.eps2) {
      vx = tdiv(u2, den);
      vy = tdiv(u3, den);
    } else {
      vx = 0.;
      vy = 0.;
    }
    const double hd = tscale<-1>(den);
    const double pres = e.g1 * (u4 - hd * (vx * vx) - hd * (vy * vy) - u5 * e.q);
    const double sound = sqrt(tdiv(e.gamma * pres, den));
    const double a = fmax(fabs(tdiv(u2, u1)) + sound, fabs(tdiv(u3, u1)) + sound);
    e.alpha[e7_cell(e, r, i, j)] = a;
    v = a > 0. ? a : 0.;
  }
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v > 0.)
    atomicMax(&e.sc->am_bits, (unsigned long long)__double_as_longlong(v));
}

// stage 1: dt = min(dx*cfl/alphamax, dy*cfl/alphamax, T - time) (:814-819)
__global__ void k7_dt(Ex7View e) {
  const double am = __longlong_as_double((long long)e.sc->am_bits);
  e.sc->alphamax = am;
  const double dtx = tdiv(e.dx * e.cfl, am), dty = tdiv(e.dy * e.cfl, am);
  const double dt = fmin(fmin(dtx, dty), e.T - e.sc->time);
  e.sc->dt = dt;
  if (!isfinite(am) || !(am > 0.) || !isfinite(dt)) e.sc->err |= E7_ERR_NONFINITE;
}
__global__ void k7_alphamax(Ex7View e) {
  e.sc->alphamax = __longlong_as_double((long long)e.sc->am_bits);
}

// wall mirror of the x pass (:186-197): on the ranks of the left edge, local
// columns total, total-1, total-2 of the rows j (0..nyl+1) at or below global
// row step*total take columns total+1..total+3, x momentum negated
__global__ void k7_mirror_x(Ex7View e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int rows = e.nyl + 2;
  if (t >= e.cut_y * rows * 3) return;
  const int py = t / (rows * 3), rem = t % (rows * 3), j = rem / 3, i = rem % 3;
  const int r = e.cut_x * py;  // px == 0
  if (py * e.nyl + j > e.wall) return;
  for (int c = 0; c < 5; ++c)
    e.u[e7_at(e, r, c, e.total - i, j)] = e.u[e7_at(e, r, c, e.total + 1 + i, j)];
  e.u[e7_at(e, r, 1, e.total - i, j)] = -e.u[e7_at(e, r, 1, e.total + 1 + i, j)];
}

// wall mirror of the y pass (:456-470): on the ranks of the left edge whose
// local row j is global row step*total, rows j, j-1, j-2 of columns
// 1..total take rows j+1..j+3, y momentum negated
__global__ void k7_mirror_y(Ex7View e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.cut_y * 3 * e.total) return;
  const int py = t / (3 * e.total), rem = t % (3 * e.total), i = rem / e.total,
            k = rem % e.total + 1;
  const int j = e.wall - py * e.nyl;
  if (j < -2 || j > e.nyl + 3) return;
  const int r = e.cut_x * py;
  for (int c = 0; c < 5; ++c) e.u[e7_at(e, r, c, k, j - i)] = e.u[e7_at(e, r, c, k, j + 1 + i)];
  e.u[e7_at(e, r, 2, k, j - i)] = -e.u[e7_at(e, r, 2, k, j + 1 + i)];
}

// alpha of a rank's local row (ydir 0: max over i = -2..nxl+3, :217-223) or
// column (ydir 1: max over j = -2..nyl+3, :492-497), one warp per line;
// MAX starting from 0 skips NaN values
__global__ void k7_line_alpha(Ex7View e, int ydir) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int lines = ydir ? e.LI : e.LJ, len = ydir ? e.LJ : e.LI;
  if (warp >= e.R * lines) return;
  const int r = warp / lines, l = warp % lines - 2;
  double v = 0.;
  for (int m = lane; m < len; m += 32) {
    const double a = ydir ? e.alpha[e7_cell(e, r, l, m - 2)] : e.alpha[e7_cell(e, r, m - 2, l)];
    v = fmax(v, a);
  }
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) e.lal[(int64_t)r * e.LL + (l + 2)] = v;
}

// LF splitting of a rank's line (:224-227 x pass for local columns
// -2..nxl+3 of rows 0..nyl+1; :498-501 y pass for rows -2..nyl+3 of columns
// 0..nxl+1) with the line's alpha, and the Roe line data of the cells the
// interfaces read (x: columns 0..nxl+2; y: rows 0..nyl+2)
__global__ void k7_split(Ex7View e, int ydir) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int ni = ydir ? e.nxl + 2 : e.LI, nj = ydir ? e.LJ : e.nyl + 2;
  if (t >= (int64_t)e.R * ni * nj) return;
  const int r = (int)(t / ((int64_t)ni * nj)), cell = (int)(t % ((int64_t)ni * nj));
  const int i = cell % ni + (ydir ? 0 : -2), j = cell / ni + (ydir ? -2 : 0);
  double a[5], f[5];
  for (int c = 0; c < 5; ++c) a[c] = e.u[e7_at(e, r, c, i, j)];
  e7_flux(e, a, f, ydir);
  const double al = e.lal[(int64_t)r * e.LL + (ydir ? i : j) + 2];
  for (int c = 0; c < 5; ++c) {
    const double fa = tdiv(f[c], al);
    e.sp[e7_at(e, r, c, i, j)] = tscale<-1>(a[c] + fa);
    e.sn[e7_at(e, r, c, i, j)] = tscale<-1>(a[c] - fa);
  }
  const int m = ydir ? j : i, mmax = ydir ? e.nyl + 2 : e.nxl + 2;
  if (m >= 0 && m <= mmax) {
    double pr[5];
    e7_prep(e, a, pr);
    for (int c = 0; c < 5; ++c) e.roe[e7_at(e, r, c, i, j)] = pr[c];
  }
}

// one interface (x pass :228-334, y pass :506-600): Roe average, 5x5
// eigenvectors, projections of the five stencil points, ten WENO5
// reconstructions, back projection; every product of the eigenvector sums is
// formed, zeros and ones included, in the reference's order
template <bool QD>
__device__ __forceinline__ void e7_eigen(const Ex7View& e, int ydir, const double* L,
                                         const double* Rr, double (*evl)[5], double (*evr)[5]) {
  const double g1 = e.g1, q = e.q;
  double t0 = QD ? qd::to_double(qd::div(qd::from_double(L[0]),
                                         qd::add(qd::from_double(L[0] + Rr[0]), e.q_1em15)))
                 : tdiv(L[0], L[0] + Rr[0] + 1e-15);
  double t1 = 1. - t0;
  const double vxm = t0 * L[1] + t1 * Rr[1];
  const double vym = t0 * L[2] + t1 * Rr[2];
  const double ym = t0 * L[3] + t1 * Rr[3];
  const double hm = t0 * L[4] + t1 * Rr[4];
  const double qm = tscale<-1>(vxm * vxm + vym * vym);
  const double cm = QD ? qd::to_double(qd::add(qd::from_double(sqrt(fabs(g1 * (hm - qm - q * ym)))),
                                               e.q_1em15))
                       : sqrt(fabs(g1 * (hm - qm - q * ym))) + 1e-15;
  const double rcm = tdiv(1., cm);
  const double b1 = g1 * rcm * rcm;
  const double b2 = qm * b1;
  if (!ydir) {
    t0 = vxm * cm;
    const double er[5][5] = {{1.0, 1.0, 0.0, 0.0, 1.0},
                             {vxm - cm, vxm, 0., 0., vxm + cm},
                             {vym, vym, -1., 0., vym},
                             {hm - t0, qm, -vym, q, hm + t0},
                             {ym, 0., 0., 1., ym}};
    t0 = vxm * rcm;
    t1 = b1 * vxm;
    const double t2 = tscale<-1>(b1), t3 = b1 * vym;
    const double el[5][5] = {
        {tscale<-1>(b2 + t0), -tscale<-1>(t1 + rcm), -tscale<-1>(t3), t2, -(t2 * q)},
        {1. - b2, t1, t3, -b1, b1 * q},
        {vym, 0.0, -1.0, 0.0, 0.0},
        {-(b2 * ym), t1 * ym, t3 * ym, -(b1 * ym), 1. + q * ym * b1},
        {tscale<-1>(b2 - t0), -tscale<-1>(t1 - rcm), -tscale<-1>(t3), t2, -(t2 * q)}};
    for (int k = 0; k < 5; ++k)
      for (int m = 0; m < 5; ++m) {
        evr[k][m] = er[k][m];
        evl[k][m] = el[k][m];
      }
  } else {
    t0 = vym * cm;
    const double er[5][5] = {{1.0, 1.0, 0.0, 0.0, 1.0},
                             {vxm, vxm, 1.0, 0., vxm},
                             {vym - cm, vym, 0., 0., vym + cm},
                             {hm - t0, qm, vxm, q, hm + t0},
                             {ym, 0., 0., 1., ym}};
    t0 = vym * rcm;
    t1 = b1 * vym;
    const double t2 = tscale<-1>(b1), t3 = b1 * vxm;
    const double el[5][5] = {
        {tscale<-1>(b2 + t0), -tscale<-1>(t3), -tscale<-1>(t1 + rcm), t2, -(q * t2)},
        {1. - b2, t3, t1, -b1, b1 * q},
        {-vxm, 1.0, 0.0, 0.0, 0.0},
        {-(ym * b2), ym * t3, ym * t1, -(ym * b1), 1. + ym * b1 * q},
        {tscale<-1>(b2 - t0), -tscale<-1>(t3), -tscale<-1>(t1 - rcm), t2, -(q * t2)}};
    for (int k = 0; k < 5; ++k)
      for (int m = 0; m < 5; ++m) {
        evr[k][m] = er[k][m];
        evl[k][m] = el[k][m];
      }
  }
}

template <bool QD>
__device__ __forceinline__ void e7_interface(const Ex7View& e, int ydir, const double* L,
                                             const double* Rr, const double (*sp)[5],
                                             const double (*sn)[5], double* outp, double* outn) {
  double evr[5][5], evl[5][5];
  e7_eigen<QD>(e, ydir, L, Rr, evl, evr);
  double ur[5], ul[5];
  for (int k = 0; k < 5; ++k) {
    double cp[5], cn[5];
    for (int ig = 0; ig < 5; ++ig) {
      cp[ig] = evl[k][0] * sp[ig][0] + evl[k][1] * sp[ig][1] + evl[k][2] * sp[ig][2] +
               evl[k][3] * sp[ig][3] + evl[k][4] * sp[ig][4];
      cn[ig] = evl[k][0] * sn[ig][0] + evl[k][1] * sn[ig][1] + evl[k][2] * sn[ig][2] +
               evl[k][3] * sn[ig][3] + evl[k][4] * sn[ig][4];
    }
    if constexpr (QD) {
      const QuadWeno qw{e.q_c1312, e.q_eps};
      ur[k] = weno_right_qd(cp[0], cp[1], cp[2], cp[3], cp[4], qw);
      ul[k] = weno_left_qd(cn[0], cn[1], cn[2], cn[3], cn[4], qw);
    } else {
      ur[k] = weno_right<double>(cp[0], cp[1], cp[2], cp[3], cp[4], e.weno_eps);
      ul[k] = weno_left<double>(cn[0], cn[1], cn[2], cn[3], cn[4], e.weno_eps);
    }
  }
  for (int k = 0; k < 5; ++k) {
    outp[k] = evr[k][0] * ur[0] + evr[k][1] * ur[1] + evr[k][2] * ur[2] + evr[k][3] * ur[3] +
              evr[k][4] * ur[4];
    outn[k] = evr[k][0] * ul[0] + evr[k][1] * ul[1] + evr[k][2] * ul[2] + evr[k][3] * ul[3] +
              evr[k][4] * ul[4];
  }
}

// use_limiter = 1: the positivity limiter of one split flux (:336-440), five
// components and q*Y in both pressures, theta clamped at 0; returns the
// density (bit 0) and pressure (bit 1) limitings
__device__ int e7_zs_limit(const Ex7View& e, const double* ave, double* out) {
  const double g1 = e.g1, q = e.q;
  const double d_ave = ave[0], m_ave = ave[1], n_ave = ave[2], e_ave = ave[3], y_ave = ave[4];
  const double p_ave = g1 * (e_ave - tdiv(tscale<-1>(m_ave * m_ave), d_ave) -
                             tdiv(tscale<-1>(n_ave * n_ave), d_ave) - q * y_ave);
  double p1[5];
  for (int c = 0; c < 5; ++c) p1[c] = tdiv(ave[c] - tdiv(out[c], 12.), 11. / 12.);
  int lim = 0;
  double theta = 1.0;
  if (out[0] < 0.) theta = fmin(theta, tdiv(fabs(d_ave - 0.), fabs(d_ave - out[0])));
  if (p1[0] < 0.) theta = fmin(theta, tdiv(fabs(d_ave - 0.), fabs(d_ave - p1[0])));
  theta = fmax(theta, 0.);
  if (theta < 1.) {
    out[0] = theta * out[0] + (1. - theta) * d_ave;
    lim |= 1;
  }
  theta = 1.;
  p1[0] = tdiv(ave[0] - tdiv(out[0], 12.), 11. / 12.);
  for (int ig = 0; ig < 2; ++ig) {
    const double* pt = ig == 0 ? out : p1;
    const double d_l = pt[0];
    const double p_l = g1 * (pt[3] - tscale<-1>(tdiv(pt[1] * pt[1], d_l)) -
                             tscale<-1>(tdiv(pt[2] * pt[2], d_l)) - q * pt[4]);
    if (p_l < 0.) theta = fmin(theta, tdiv(fabs(p_ave - 0.), fabs(p_ave - p_l)));
  }
  theta = fmax(theta, 0.);
  if (theta < 1.) {
    for (int c = 0; c < 5; ++c) out[c] = theta * out[c] + (1. - theta) * ave[c];
    lim |= 2;
  }
  return lim;
}

// interfaces of every rank (x: i+1/2 for local i = 0..nxl+1 on rows
// 0..nyl+1; y: j+1/2 for j = 0..nyl+1 on columns 0..nxl+1), scaled by the
// line's alpha (:444-445, :728-729)
template <bool QD, bool LIM>
__global__ void __launch_bounds__(128) k7_flux(Ex7View e, int ydir) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int ni = e.nxl + 2, nj = e.nyl + 2;
  if (t >= (int64_t)e.R * ni * nj) return;
  const int r = (int)(t / ((int64_t)ni * nj)), cell = (int)(t % ((int64_t)ni * nj));
  const int i = cell % ni, j = cell / ni;
  const int di = ydir ? 0 : 1, dj = ydir ? 1 : 0;
  double L[5], Rr[5], sp[5][5], sn[5][5], op[5], on[5];
  for (int c = 0; c < 5; ++c) {
    L[c] = e.roe[e7_at(e, r, c, i, j)];
    Rr[c] = e.roe[e7_at(e, r, c, i + di, j + dj)];
  }
  for (int ig = 0; ig < 5; ++ig)
    for (int c = 0; c < 5; ++c) {
      const int64_t o = e7_at(e, r, c, i + di * (ig - 2), j + dj * (ig - 2));
      sp[ig][c] = e.sp[o];
      sn[ig][c] = e.sn[o];
    }
  e7_interface<QD>(e, ydir, L, Rr, sp, sn, op, on);
  if constexpr (LIM) {
    const int lp = e7_zs_limit(e, sp[2], op), ln = e7_zs_limit(e, sn[2], on);
    const int den = (lp & 1) + (ln & 1), pre = (lp >> 1) + (ln >> 1);
    if (den) atomicAdd((unsigned long long*)&e.sc->lim_den, (unsigned long long)den);
    if (pre) atomicAdd((unsigned long long*)&e.sc->lim_pre, (unsigned long long)pre);
  }
  const double al = e.lal[(int64_t)r * e.LL + (ydir ? i : j) + 2];
  double* fp = ydir ? e.gpf : e.fpf;
  double* fn = ydir ? e.gnf : e.fnf;
  for (int c = 0; c < 5; ++c) {
    fp[e7_at(e, r, c, i, j)] = al * op[c];
    fn[e7_at(e, r, c, i, j)] = al * on[c];
  }
}

// scheme (:738-750) + the RK combination (:824,846,867) over every local cell
// (the RHS is zero outside the interior) + checkpositivity (:890-913)
template <bool QD>
__global__ void k7_rk(Ex7View e, int stage) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int bad = 0;
  if (t < (int64_t)e.R * e.LI * e.LJ) {
    const int r = (int)(t / ((int64_t)e.LI * e.LJ)), cell = (int)(t % ((int64_t)e.LI * e.LJ));
    const int i = cell % e.LI - 2, j = cell / e.LI - 2;
    const bool interior = i >= 1 && i <= e.nxl && j >= 1 && j <= e.nyl;
    const double dt = e.sc->dt;
    double a[5], nv[5];
    for (int c = 0; c < 5; ++c) a[c] = e.u[e7_at(e, r, c, i, j)];
    for (int c = 0; c < 5; ++c) {
      double rhs = 0.;
      if (interior) {
        const double A = (e.fpf[e7_at(e, r, c, i, j)] - e.fnf[e7_at(e, r, c, i + 1, j)]) -
                         (e.fpf[e7_at(e, r, c, i - 1, j)] - e.fnf[e7_at(e, r, c, i, j)]);
        const double B = (e.gpf[e7_at(e, r, c, i, j)] - e.gnf[e7_at(e, r, c, i, j + 1)]) -
                         (e.gpf[e7_at(e, r, c, i, j - 1)] - e.gnf[e7_at(e, r, c, i, j)]);
        rhs = -tdiv(A, e.dx) - tdiv(B, e.dy);
        if (c == 4) rhs = rhs + e7_chem(e, a);
      }
      const int64_t o = e7_at(e, r, c, i, j);
      double v = a[c] + dt * rhs;
      if (QD && stage >= 2) {  // 0.75d0*u0 + 0.25d0*(..), (u0 + 2d0*(..))/3d0 in binary128
        using namespace qd;
        v = stage == 2 ? to_double(add(mul(from_double(0.75), from_double(e.u0[o])),
                                       scale2(from_double(v), -2)))
                       : to_double(div(add(from_double(e.u0[o]), scale2(from_double(v), 1)),
                                       from_double(3.0)));
      } else if (stage == 2) {
        v = 0.75 * e.u0[o] + tscale<-2>(v);
      } else if (stage == 3) {
        v = tdiv(e.u0[o] + tscale<1>(v), 3.0);
      }
      nv[c] = v;
      e.u[o] = v;
    }
    if (interior) {
      if (nv[0] <= e.eps) bad = 1;
      const double pe = nv[3] - tscale<-1>(tdiv(nv[2] * nv[2], nv[0])) -
                        tscale<-1>(tdiv(nv[1] * nv[1], nv[0])) - e.q * nv[4];
      if (pe <= e.eps) bad = 1;
    }
  }
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0 && bad) atomicOr(&e.sc->postag, 1);
}

// exchange_x (:1073-1133): ghost columns from the x neighbours (periodic in
// the rank grid); reads interior columns only, so one pass is the exchange
__global__ void k7_exchange_x(Ex7View e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.R * e.LJ * 3) return;
  const int r = t / (e.LJ * 3), rem = t % (e.LJ * 3), j = rem / 3 - 2, m = rem % 3 + 1;
  const int px = r % e.cut_x, py = r / e.cut_x;
  const int right = (px + 1) % e.cut_x + e.cut_x * py;
  const int left = (px + e.cut_x - 1) % e.cut_x + e.cut_x * py;
  for (int c = 0; c < 5; ++c) {
    e.u[e7_at(e, r, c, e.nxl + m, j)] = e.u[e7_at(e, right, c, m, j)];
    e.u[e7_at(e, r, c, 1 - m, j)] = e.u[e7_at(e, left, c, e.nxl + 1 - m, j)];
  }
}

// exchange_y (:1135-1194): ghost rows (all local columns) from the y neighbours
__global__ void k7_exchange_y(Ex7View e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.R * e.LI * 3) return;
  const int r = t / (e.LI * 3), rem = t % (e.LI * 3), i = rem / 3 - 2, m = rem % 3 + 1;
  const int px = r % e.cut_x, py = r / e.cut_x;
  const int up = px + e.cut_x * ((py + 1) % e.cut_y);
  const int down = px + e.cut_x * ((py + e.cut_y - 1) % e.cut_y);
  for (int c = 0; c < 5; ++c) {
    e.u[e7_at(e, r, c, i, e.nyl + m)] = e.u[e7_at(e, up, c, i, m)];
    e.u[e7_at(e, r, c, i, 1 - m)] = e.u[e7_at(e, down, c, i, e.nyl + 1 - m)];
  }
}

__device__ __forceinline__ void e7_set(const Ex7View& e, int r, int i, int j, double a, double b,
                                       double c, double d, double f) {
  e.u[e7_at(e, r, 0, i, j)] = a;
  e.u[e7_at(e, r, 1, i, j)] = b;
  e.u[e7_at(e, r, 2, i, j)] = c;
  e.u[e7_at(e, r, 3, i, j)] = d;
  e.u[e7_at(e, r, 4, i, j)] = f;
}

// the boundary rules of bc (:1000-1069), in the reference's order: 0 the
// quiescent bottom and right ghosts, 1 the reflecting top, 2 the inflow left,
// 3 the quiescent solid block (global i < total, j < step*total, ghosts
// included)
__global__ void k7_bc_rule(Ex7View e, int which) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)e.R * e.LI * e.LJ) return;
  const int r = (int)(t / ((int64_t)e.LI * e.LJ)), cell = (int)(t % ((int64_t)e.LI * e.LJ));
  const int i = cell % e.LI - 2, j = cell / e.LI - 2;
  const int px = r % e.cut_x, py = r / e.cut_x;
  if (which == 0) {
    if ((py == 0 && j <= 0) || (px == e.cut_x - 1 && i >= e.nxl + 1))
      e7_set(e, r, i, j, 1., 0., 0., 55., 1.);
  } else if (which == 1) {
    if (py == e.cut_y - 1 && j >= e.nyl + 1) {
      for (int c = 0; c < 5; ++c) e.u[e7_at(e, r, c, i, j)] = e.u[e7_at(e, r, c, i, e.nyl)];
      e.u[e7_at(e, r, 2, i, j)] = -e.u[e7_at(e, r, 2, i, e.nyl)];
    }
  } else if (which == 2) {
    if (px == 0 && i <= 0) e7_set(e, r, i, j, 11., 11. * 6.18, 0., 970., 11.);
  } else {
    if (i + px * e.nxl < e.total && j + py * e.nyl < e.wall)
      e7_set(e, r, i, j, 1., 0., 0., 55., 1.);
  }
}

// gather_to_root / scatter_from_root (:1864-1986): the ranks' interiors <->
// the global interior, compact (i fastest) for the sweep
__global__ void k7_gather(Ex7View e, int to_global) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = (int64_t)e.nx * e.ny;
  if (t >= N) return;
  const int I = (int)(t % e.nx) + 1, J = (int)(t / e.nx) + 1;
  const int px = (I - 1) / e.nxl, py = (J - 1) / e.nyl, r = px + e.cut_x * py;
  const int i = I - px * e.nxl, j = J - py * e.nyl;
  for (int c = 0; c < 5; ++c) {
    if (to_global) e.ug[c * N + t] = e.u[e7_at(e, r, c, i, j)];
    else e.u[e7_at(e, r, c, i, j)] = e.ug[c * N + t];
  }
}

// the global view u(5,-2:nx+3,-2:ny+3) <-> the ranks: interior cells from
// their owners, ghost cells from the edge ranks (to_view); every local cell
// of every rank from the view (from the view)
__global__ void k7_view(Ex7View e, int to_view) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int GI = e.nx + 6, GJ = e.ny + 6;
  if (to_view) {
    if (t >= (int64_t)GI * GJ) return;
    const int I = (int)(t % GI) - 2, J = (int)(t / GI) - 2;
    const int px = I <= 0 ? 0 : min((I - 1) / e.nxl, e.cut_x - 1);
    const int py = J <= 0 ? 0 : min((J - 1) / e.nyl, e.cut_y - 1);
    const int r = px + e.cut_x * py, i = I - px * e.nxl, j = J - py * e.nyl;
    for (int c = 0; c < 5; ++c) e.gview[c + 5 * t] = e.u[e7_at(e, r, c, i, j)];
  } else {
    if (t >= (int64_t)e.R * e.LI * e.LJ) return;
    const int r = (int)(t / ((int64_t)e.LI * e.LJ)), cell = (int)(t % ((int64_t)e.LI * e.LJ));
    const int i = cell % e.LI - 2, j = cell / e.LI - 2;
    const int I = (r % e.cut_x) * e.nxl + i, J = (r / e.cut_x) * e.nyl + j;
    const int64_t g = (int64_t)(I + 2) + (int64_t)GI * (J + 2);
    for (int c = 0; c < 5; ++c) e.u[e7_at(e, r, c, i, j)] = e.gview[c + 5 * g];
  }
}

// ---------------------------------------------------------------------------
// sweep_lim (:1433-1737) on the gathered interior.  Orderings (:1808-1862):
// I column by column (k = (j-1)*nx + ..., i up on odd j, down on even j),
// II row by row.  A pass step at position k may change its cell and the next
// one, and only the previous step's writes can change whether step k adjusts
// (the ordering-II mixing of component 5 included), so a pass is: flag the
// positions that adjust on the pass-start state, compact them in order, and
// walk them in one thread, continuing each chain of adjusted steps.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int e7_pos(const Ex7View& e, int ord, int k) {
  if (ord == 0) {
    const int j = k / e.nx + 1, m = k % e.nx;
    const int i = (j % 2 == 1) ? m + 1 : e.nx - m;
    return (j - 1) * e.nx + (i - 1);
  }
  const int i = k / e.ny + 1, m = k % e.ny;
  const int j = (i % 2 == 1) ? m + 1 : e.ny - m;
  return (j - 1) * e.nx + (i - 1);
}

// g1*(v4 - 0.5*v2*v2/v1 - 0.5*v3**2/v1 - q*v5) (form 0: :1503) or
// g1*(v4 - 0.5*v2**2/v1 - 0.5*v3**2/v1 - q*v5) (form 1: :1405,1533)
__device__ __forceinline__ double e7_psweep(const Ex7View& e, const double* v, int form) {
  const double a = form == 0 ? tdiv(tscale<-1>(v[1]) * v[1], v[0]) : tdiv(tscale<-1>(v[1] * v[1]), v[0]);
  return e.g1 * (v[3] - a - tdiv(tscale<-1>(v[2] * v[2]), v[0]) - e.q * v[4]);
}

__global__ void k7_min(Ex7View e) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t N = (int64_t)e.nx * e.ny;
  unsigned long long kp = ~0ull, kr = ~0ull;
  if (t < N) {
    const double u1 = e.ug[t], u2 = e.ug[N + t], u3 = e.ug[2 * N + t], u4 = e.ug[3 * N + t];
    const double p = e.g1 * (u4 - tdiv(tscale<-1>(u2 * u2 + u3 * u3), u1));
    if (p == p) kp = e7_key(p);
    if (u1 == u1) kr = e7_key(u1);
  }
  for (int o = 16; o > 0; o >>= 1) {
    kp = min(kp, (unsigned long long)__shfl_xor_sync(0xffffffffu, kp, o));
    kr = min(kr, (unsigned long long)__shfl_xor_sync(0xffffffffu, kr, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&e.sc->p_min_key, kp);
    atomicMin(&e.sc->rho_min_key, kr);
  }
}

// scalar_sweep (:1740-1806): the density passes along ordering I (delta =
// 1d-12, equal weights); rare, so one thread
__global__ void k7_density(Ex7View e) {
  const int N = e.nx * e.ny;
  const double delta = 1e-12, w = 1. / ((double)e.nx * (double)e.ny);
  double* rho = e.ug;
  for (int k = 0; k < N - 1; ++k) {
    const int a = e7_pos(e, 0, k), b = e7_pos(e, 0, k + 1);
    const double v_i = rho[a], v_n = rho[b];
    if (v_i < delta) {
      rho[b] = v_n + tdiv(w, w) * (v_i - delta);
      rho[a] = delta;
    }
  }
  for (int k = N - 1; k >= 1; --k) {
    const int a = e7_pos(e, 0, k), b = e7_pos(e, 0, k - 1);
    const double v_i = rho[a], v_n = rho[b];
    if (v_i < delta) {
      rho[b] = v_n + tdiv(w, w) * (v_i - delta);
      rho[a] = delta;
    }
  }
  e.sc->den_count++;
}

// v_i of step k: components 1-4 at ordering `ord`, component 5 at ordering I
__device__ __forceinline__ void e7_vi(const Ex7View& e, int ord, int k, double* v) {
  const int64_t N = (int64_t)e.nx * e.ny;
  const int a = e7_pos(e, ord, k), b = e7_pos(e, 0, k);
  for (int c = 0; c < 4; ++c) v[c] = e.ug[c * N + a];
  v[4] = e.ug[4 * N + b];
}
__device__ __forceinline__ bool e7_bad(const Ex7View& e, const double* v) {
  return e7_psweep(e, v, 0) <= e.eps || v[0] <= e.eps;
}

// ordering of pass pair q: I for odd q, II for even (:1490-1493); ord < 0
// takes it from the device's q
__device__ __forceinline__ int e7_ord(const Ex7View& e, int ord) {
  return ord >= 0 ? ord : ((e.sc->q % 2 == 1) ? 0 : 1);
}

__global__ void k7_flag(Ex7View e, int ord, int fwd) {
  ord = e7_ord(e, ord);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int N = e.nx * e.ny;
  if (k >= N) return;
  int f = 0;
  if (fwd ? k <= N - 2 : k >= 1) {
    double v[5];
    e7_vi(e, ord, k, v);
    f = e7_bad(e, v) ? 1 : 0;
  }
  e.flag[k] = f;
}

// ordered compaction of the flags into list[0..nflag), one block
__global__ void __launch_bounds__(1024) k7_compact(Ex7View e) {
  __shared__ int warp_cnt[32];
  __shared__ int base_sh;
  const int N = e.nx * e.ny, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) base_sh = 0;
  __syncthreads();
  for (int start = 0; start < N; start += 1024) {
    const int k = start + tid;
    const int f = k < N ? e.flag[k] : 0;
    const unsigned m = __ballot_sync(0xffffffffu, f);
    if (lane == 0) warp_cnt[wid] = __popc(m);
    __syncthreads();
    int off = base_sh;
    for (int w = 0; w < wid; ++w) off += warp_cnt[w];
    if (f) e.list[off + __popc(m & ((1u << lane) - 1u))] = k;
    __syncthreads();
    if (tid == 0) {
      int s = 0;
      for (int w = 0; w < 32; ++w) s += warp_cnt[w];
      base_sh += s;
    }
    __syncthreads();
  }
  if (tid == 0) e.sc->nflag = base_sh;
}

// nod_lim (:1399-1429)
__device__ void e7_nod_lim(const Ex7View& e, const double* v1, const double* v2,
                           const double* vb, double* out) {
  const double eps = e.eps;
  const double p1 = e7_psweep(e, v1, 1), p2 = e7_psweep(e, v2, 1);
  double t;
  if (p2 > eps) {
    t = tdiv(p1 - eps, p1 - p2);
    e.sc->t_pos++;
  } else {
    const double pb = e7_psweep(e, vb, 1);
    const double t_1 = tdiv(p1 - eps, p1 - pb);
    double s12 = 0., s1b = 0.;
    for (int c = 4; c >= 0; --c) {
      const double d2 = v2[c] - v1[c], db = vb[c] - v1[c];
      s12 = c == 4 ? d2 * d2 : s12 + d2 * d2;
      s1b = c == 4 ? db * db : s1b + db * db;
    }
    t = fmin(tdiv(t_1 * sqrt(s1b), sqrt(s12)), 0.25);
    e.sc->t_neg++;
  }
  for (int c = 0; c < 5; ++c) out[c] = (1 - t) * v1[c] + t * v2[c];
}

// one step of a pass at position k (:1497-1548 ordering I, :1611-1658
// ordering II); returns whether it adjusted
__device__ bool e7_step(const Ex7View& e, int ord, int fwd, int k) {
  const int64_t N = (int64_t)e.nx * e.ny;
  const double w = 1. / ((double)e.nx * (double)e.ny);
  double vi[5], vp[5], vit[5], vpt[5];
  e7_vi(e, ord, k, vi);
  const double pres_v_i = e7_psweep(e, vi, 0);
  if (!(pres_v_i <= e.eps || vi[0] <= e.eps)) return false;
  const int kn = fwd ? k + 1 : k - 1;
  const int k5 = ord ? k - 1 : kn;
  if (k5 < 0) {  // the reference would read sweepI(0)
    e.sc->err |= E7_ERR_SWEEP_INDEX;
    return false;
  }
  const int a = e7_pos(e, ord, k), b = e7_pos(e, 0, k);
  const int cc = e7_pos(e, ord, kn), d = e7_pos(e, 0, k5);
  for (int c = 0; c < 4; ++c) vp[c] = e.ug[c * N + cc];
  vp[4] = e.ug[4 * N + d];
  e7_nod_lim(e, vi, vp, e.sc->ubar, vit);
  for (int c = 0; c < 5; ++c) vpt[c] = vp[c] + tdiv(w, w) * (vi[c] - vit[c]);
  for (int c = 0; c < 4; ++c) e.ug[c * N + a] = vit[c];
  e.ug[4 * N + b] = vit[4];
  for (int c = 0; c < 4; ++c) e.ug[c * N + cc] = vpt[c];
  e.ug[4 * N + d] = vpt[4];
  if (ord == 0) {  // stop "total pressure increased" (:1537-1546), ordering I only
    const double pres_v_p = e7_psweep(e, vp, 0);
    const double pres_v_i_t = e7_psweep(e, vit, 1);
    const double pres_v_p_t = e7_psweep(e, vpt, 1);
    if (pres_v_i + pres_v_p > pres_v_i_t + pres_v_p_t + e.eps) e.sc->err |= E7_ERR_SWEEP_CHECK;
  }
  return true;
}

__global__ void k7_walk(Ex7View e, int ord, int fwd) {
  ord = e7_ord(e, ord);
  const int N = e.nx * e.ny, nf = e.sc->nflag;
  const int dk = fwd ? 1 : -1, kend = fwd ? N - 1 : 0;
  int li = fwd ? 0 : nf - 1;
  int k = nf > 0 ? e.list[li] : -1;
  while (k >= 0) {
    while (fwd ? (li < nf && e.list[li] <= k) : (li >= 0 && e.list[li] >= k)) li += dk;
    const bool active = e7_step(e, ord, fwd, k);
    if (e.sc->err) return;
    const int nk = k + dk;
    if (active && nk != kend) k = nk;
    else k = (fwd ? li < nf : li >= 0) ? e.list[li] : -1;
  }
}

// ---------------------------------------------------------------------------
// the sweep's and the stages' decisions on the device (graph conditions; in
// the eager launch mode the condition word sc->cond)
// ---------------------------------------------------------------------------
// the sweep after checkpositivity (:858-863), unless alpha or dt went bad
__global__ void k7_cond_postag(cudaGraphConditionalHandle h, Ex7View e) {
  set_cond(h, &e.sc->cond, (e.sc->postag && !(e.sc->err & E7_ERR_NONFINITE)) ? 1u : 0u);
}
// scalar_sweep only when min rho < 1d-12 (:1748-1755)
__global__ void k7_cond_density(cudaGraphConditionalHandle h, Ex7View e) {
  set_cond(h, &e.sc->cond, e7_unkey(e.sc->rho_min_key) < 1e-12 ? 1u : 0u);
}
// after u_bar: the stop on P(u_bar) <= 0 (:1495-1499), the sweep's count and
// track entries, then the pass pairs from q = 1
__global__ void k7_sweep_begin(cudaGraphConditionalHandle h, Ex7View e, int swp_num) {
  Ex7Scalars* sc = e.sc;
  const double* ub = sc->ubar;
  if (e.g1 * (ub[3] - 0.5 * (ub[1] * ub[1]) / ub[0] - 0.5 * (ub[2] * ub[2]) / ub[0] -
              e.q * ub[4]) <= 0.) {
    sc->err |= E7_ERR_PUBAR;
    set_cond(h, &sc->cond, 0u);
    return;
  }
  const long long n = sc->sweep_count++;
  if (n < sc->track_cap)
    sc->tracks[n] = sc->tracks[sc->track_cap + n] = sc->tracks[2 * sc->track_cap + n] = 0;
  sc->t_pos = sc->t_neg = 0;
  sc->q = 1;
  if (swp_num < 1) {
    sc->fail_count++;
    sc->err |= E7_ERR_NOCONV;
  }
  set_cond(h, &sc->cond, swp_num >= 1 ? 1u : 0u);
}
// after a pass pair and the minima: the stops (total pressure increased,
// sweepI(0)), the exit test p_min > eps and rho_min > eps with its track
// entries (:1660-1672), or the next q up to swp_num
__global__ void k7_q_end(cudaGraphConditionalHandle h, Ex7View e, int swp_num) {
  Ex7Scalars* sc = e.sc;
  if (sc->err & (E7_ERR_SWEEP_CHECK | E7_ERR_SWEEP_INDEX)) {
    set_cond(h, &sc->cond, 0u);
    return;
  }
  sc->pre_count++;
  if (e7_unkey(sc->p_min_key) > e.eps && e7_unkey(sc->rho_min_key) > e.eps) {
    const long long n = sc->sweep_count - 1, c = sc->track_cap;
    if (n < c) {
      sc->tracks[n] = sc->q;
      sc->tracks[c + n] = (int)sc->t_neg;
      sc->tracks[2 * c + n] = (int)sc->t_pos;
    }
    set_cond(h, &sc->cond, 0u);
    return;
  }
  if (++sc->q > swp_num) {
    sc->fail_count++;
    sc->err |= E7_ERR_NOCONV;
    set_cond(h, &sc->cond, 0u);
    return;
  }
  set_cond(h, &sc->cond, 1u);
}
// time = time + dt (:97-99)
__global__ void k7_time_advance(Ex7View e) { e.sc->time = e.sc->time + e.sc->dt; }

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

unsigned e7_grid(int64_t n, int b = E7_BLOCK) { return (unsigned)((n + b - 1) / b); }

swfd_status e7_fail(swfd_handle* h, swfd_status st, const std::string& m) {
  if (h) h->last_error = m;
  set_last_error(m);
  return st;
}
#define E7CU(h, call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return e7_fail((h), e_ == cudaErrorMemoryAllocation ? SWFD_ERR_OOM : SWFD_ERR_CUDA, \
                     std::string("detonation: ") + cudaGetErrorString(e_));             \
  } while (0)
#define ST(call)                  \
  do {                            \
    swfd_status s_ = (call);      \
    if (s_ != SWFD_OK) return s_; \
  } while (0)
#define E7K(h, launch)             \
  do {                             \
    launch;                        \
    E7CU(h, cudaGetLastError());   \
    (h)->ex7->launches++;          \
  } while (0)

swfd_status e7_sync_scalars(swfd_handle* h) {
  Ex7* x = h->ex7;
  E7CU(h, cudaMemcpyAsync(x->hs, x->v.sc, sizeof(Ex7Scalars), cudaMemcpyDeviceToHost, h->stream));
  E7CU(h, cudaStreamSynchronize(h->stream));
  return SWFD_OK;
}

// a launch recorded into the builder (a capture, or eager on the stream)
#define E7B(b, launch)          \
  do {                          \
    launch;                     \
    (b).ok(cudaGetLastError()); \
    (b).k(1);                   \
  } while (0)

// the interface kernel specialised on the literal form and the limiter
void e7_emit_flux(Builder& b, const Ex7View& v, int64_t faces, int ydir, cudaStream_t s) {
  const unsigned g = e7_grid(faces, 128);
  const bool lim = v.use_limiter == 1;
  if (v.quad) {
    if (lim) E7B(b, (k7_flux<true, true><<<g, 128, 0, s>>>(v, ydir)));
    else E7B(b, (k7_flux<true, false><<<g, 128, 0, s>>>(v, ydir)));
  } else {
    if (lim) E7B(b, (k7_flux<false, true><<<g, 128, 0, s>>>(v, ydir)));
    else E7B(b, (k7_flux<false, false><<<g, 128, 0, s>>>(v, ydir)));
  }
}

void e7_emit_bc(Builder& b, const Ex7View& v, cudaStream_t s) {
  for (int rep = 0; rep < 2; ++rep) {  // twice, for the corners (:943-959)
    E7B(b, (k7_exchange_x<<<e7_grid((int64_t)v.R * v.LJ * 3), E7_BLOCK, 0, s>>>(v)));
    E7B(b, (k7_exchange_y<<<e7_grid((int64_t)v.R * v.LI * 3), E7_BLOCK, 0, s>>>(v)));
  }
  const unsigned g = e7_grid((int64_t)v.R * v.LI * v.LJ);
  for (int which = 0; which < 4; ++which) E7B(b, (k7_bc_rule<<<g, E7_BLOCK, 0, s>>>(v, which)));
}

// plain stream launches (initdata's bc)
swfd_status e7_bc(swfd_handle* h) {
  Builder b;
  b.h = h;
  b.eager = true;
  b.launched = &h->ex7->launches;
  e7_emit_bc(b, h->ex7->v, h->stream);
  if (b.err != cudaSuccess)
    return e7_fail(h, SWFD_ERR_CUDA, std::string("detonation: ") + cudaGetErrorString(b.err));
  return SWFD_OK;
}

// sweep_lim on the gathered interior (:1435-1680): gather, [scalar_sweep],
// u_bar, then WHILE the pass pairs run { ordering I or II forward and
// backward, the minima, the exit test }, scatter.  Every decision is a
// device kernel's (k7_cond_density, k7_sweep_begin, k7_q_end).
void e7_emit_sweep(Builder& b, Ex7* x, cudaStream_t s) {
  const Ex7View& v = x->v;
  const int64_t N = (int64_t)v.nx * v.ny;
  Ex7Scalars* sc = v.sc;
  int* saved = b.count;
  x->k_sweep = x->k_q = 0;  // every stage emits the same sweep: count it once
  b.count = &x->k_sweep;
  E7B(b, (k7_gather<<<e7_grid(N), E7_BLOCK, 0, s>>>(v, 1)));
  B_OK(b, cudaMemsetAsync(&sc->rho_min_key, 0xff, 2 * sizeof(unsigned long long), s));
  E7B(b, (k7_min<<<e7_grid(N), E7_BLOCK, 0, s>>>(v)));
  const cudaGraphConditionalHandle hd = b.handle();
  E7B(b, (k7_cond_density<<<1, 1, 0, s>>>(hd, v)));
  b.cond(s, cudaGraphCondTypeIf, hd, [&](cudaStream_t sd) {
    b.count = nullptr;  // counted through den_count
    E7B(b, (k7_density<<<1, 1, 0, sd>>>(v)));
    b.count = &x->k_sweep;
  });
  // u_bar: five sequential sums, j outer (:1464-1485)
  const double w = 1. / ((double)v.nx * (double)v.ny);
  for (int c = 0; c < 5; ++c) {
    B_OK(b, launch_seq_sum(v.ug + c * N, N, w, &sc->ubar[c], x->sum_scratch, s));
    b.k(3);
  }
  const cudaGraphConditionalHandle hw = b.handle();
  E7B(b, (k7_sweep_begin<<<1, 1, 0, s>>>(hw, v, x->swp_num)));
  b.cond(s, cudaGraphCondTypeWhile, hw, [&](cudaStream_t sq) {
    b.count = &x->k_q;
    for (int fwd = 1; fwd >= 0; --fwd) {
      E7B(b, (k7_flag<<<e7_grid(N), E7_BLOCK, 0, sq>>>(v, -1, fwd)));
      E7B(b, (k7_compact<<<1, 1024, 0, sq>>>(v)));
      E7B(b, (k7_walk<<<1, 1, 0, sq>>>(v, -1, fwd)));
    }
    B_OK(b, cudaMemsetAsync(&sc->rho_min_key, 0xff, 2 * sizeof(unsigned long long), sq));
    E7B(b, (k7_min<<<e7_grid(N), E7_BLOCK, 0, sq>>>(v)));
    E7B(b, (k7_q_end<<<1, 1, 0, sq>>>(hw, v, x->swp_num)));
    b.count = &x->k_sweep;
  });
  E7B(b, (k7_gather<<<e7_grid(N), E7_BLOCK, 0, s>>>(v, 0)));
  b.count = saved;
}

// rk (:810-888): three stages of wenofd, scheme, the RK combination,
// checkpositivity, IF (postag) the sweep, bc; then the time advance
void e7_emit_step(Builder& b, Ex7* x, cudaStream_t s) {
  const Ex7View& v = x->v;
  const int64_t cells = (int64_t)v.R * v.LI * v.LJ;
  const int64_t faces = (int64_t)v.R * (v.nxl + 2) * (v.nyl + 2);
  x->k_step = 0;
  b.count = &x->k_step;
  for (int stage = 1; stage <= 3; ++stage) {
    B_OK(b, cudaMemsetAsync(&v.sc->am_bits, 0, sizeof(unsigned long long), s));
    E7B(b, (k7_alpha<<<e7_grid(cells), E7_BLOCK, 0, s>>>(v)));
    if (stage == 1) E7B(b, (k7_dt<<<1, 1, 0, s>>>(v)));
    else E7B(b, (k7_alphamax<<<1, 1, 0, s>>>(v)));
    // wenofd: x pass then y pass, each after its wall mirror
    E7B(b, (k7_mirror_x<<<e7_grid((int64_t)v.cut_y * (v.nyl + 2) * 3), E7_BLOCK, 0, s>>>(v)));
    E7B(b, (k7_line_alpha<<<e7_grid((int64_t)v.R * v.LJ * 32), E7_BLOCK, 0, s>>>(v, 0)));
    E7B(b, (k7_split<<<e7_grid((int64_t)v.R * v.LI * (v.nyl + 2)), E7_BLOCK, 0, s>>>(v, 0)));
    e7_emit_flux(b, v, faces, 0, s);
    E7B(b, (k7_mirror_y<<<e7_grid((int64_t)v.cut_y * 3 * v.total), E7_BLOCK, 0, s>>>(v)));
    E7B(b, (k7_line_alpha<<<e7_grid((int64_t)v.R * v.LI * 32), E7_BLOCK, 0, s>>>(v, 1)));
    E7B(b, (k7_split<<<e7_grid((int64_t)v.R * (v.nxl + 2) * v.LJ), E7_BLOCK, 0, s>>>(v, 1)));
    e7_emit_flux(b, v, faces, 1, s);
    // u0 = u after wenofd, whose wall mirrors rewrite cells of u (:822)
    if (stage == 1)
      B_OK(b, cudaMemcpyAsync(v.u0, v.u, 5 * cells * sizeof(double), cudaMemcpyDeviceToDevice, s));
    B_OK(b, cudaMemsetAsync(&v.sc->postag, 0, sizeof(int), s));
    if (v.quad) E7B(b, (k7_rk<true><<<e7_grid(cells), E7_BLOCK, 0, s>>>(v, stage)));
    else E7B(b, (k7_rk<false><<<e7_grid(cells), E7_BLOCK, 0, s>>>(v, stage)));
    if (x->use_limiter == 2) {
      const cudaGraphConditionalHandle hs = b.handle();
      E7B(b, (k7_cond_postag<<<1, 1, 0, s>>>(hs, v)));
      b.cond(s, cudaGraphCondTypeIf, hs, [&](cudaStream_t sw) { e7_emit_sweep(b, x, sw); });
      b.count = &x->k_step;
    }
    e7_emit_bc(b, v, s);
  }
  E7B(b, (k7_time_advance<<<1, 1, 0, s>>>(v)));
}

// the step graph, captured once
swfd_status e7_build_step(swfd_handle* h) {
  Ex7* x = h->ex7;
  if (x->g_step || h->eager) return SWFD_OK;
  Builder b;
  b.h = h;
  b.cap = h->cap;
  b.max_depth = SWFD_CAP_DEPTH - 1;
  cudaStream_t s = h->cap[0];
  E7CU(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  cudaStreamCaptureStatus cs;
  b.ok(cudaStreamGetCaptureInfo(s, &cs, nullptr, &b.root, nullptr, nullptr, nullptr));
  e7_emit_step(b, x, s);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (b.err != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return e7_fail(h, SWFD_ERR_CUDA, std::string("detonation graph capture: ") +
                                         cudaGetErrorString(b.err != cudaSuccess ? b.err : e2));
  }
  cudaError_t e3 = cudaGraphInstantiate(&x->g_step, g, 0);
  cudaGraphDestroy(g);
  if (e3 != cudaSuccess)
    return e7_fail(h, SWFD_ERR_CUDA,
                   std::string("detonation graph instantiate: ") + cudaGetErrorString(e3));
  return SWFD_OK;
}

// the device's view of the track buffer (after a reset of the scalars too)
swfd_status e7_publish_tracks(swfd_handle* h) {
  Ex7* x = h->ex7;
  const long long lc = x->track_cap;
  E7CU(h, cudaMemcpyAsync(&x->v.sc->tracks, &x->tracks, sizeof(int*), cudaMemcpyHostToDevice,
                          h->stream));
  E7CU(h, cudaMemcpyAsync(&x->v.sc->track_cap, &lc, sizeof(long long), cudaMemcpyHostToDevice,
                          h->stream));
  E7CU(h, cudaStreamSynchronize(h->stream));
  return SWFD_OK;
}

// room on the device for `extra` more sweeps' track entries (the host
// mirror holds the count after the last step)
swfd_status e7_ensure_tracks(swfd_handle* h, int64_t extra) {
  Ex7* x = h->ex7;
  const int64_t need = x->hs->sweep_count + extra;
  if (need <= x->track_cap) return SWFD_OK;
  const int64_t cap = std::max<int64_t>(need, 2 * x->track_cap + 1024);
  int* nt = nullptr;
  E7CU(h, cudaMalloc(&nt, 3 * cap * sizeof(int)));
  E7CU(h, cudaMemsetAsync(nt, 0, 3 * cap * sizeof(int), h->stream));
  for (int c = 0; c < 3 && x->tracks; ++c)
    E7CU(h, cudaMemcpyAsync(nt + c * cap, x->tracks + c * x->track_cap,
                            x->track_cap * sizeof(int), cudaMemcpyDeviceToDevice, h->stream));
  E7CU(h, cudaStreamSynchronize(h->stream));
  cudaFree(x->tracks);
  x->tracks = nt;
  x->track_cap = cap;
  return e7_publish_tracks(h);
}

}  // namespace

swfd_status ex7_check(const swfd_config& c, std::string& err) {
  if (c.total <= 0 || c.cut_x <= 0 || c.cut_y <= 0) {
    err = "detonation: total, cut_x and cut_y must be positive";
    return SWFD_ERR_INVALID;
  }
  const int nxl = 5 * c.total / c.cut_x, nyl = 5 * c.total / c.cut_y;
  if (c.nx != c.cut_x * nxl || c.ny != c.cut_y * nyl) {
    err = "detonation: nx must be cut_x*(5*total/cut_x) and ny cut_y*(5*total/cut_y)";
    return SWFD_ERR_INVALID;
  }
  if (nxl < 3 || nyl < 3 || c.total > nxl) {
    err = "detonation: the local grid must hold 3 ghost layers and the wall columns total..total+3";
    return SWFD_ERR_INVALID;
  }
  // the y-pass wall mirror writes rows j-2..j and reads j+1..j+3 of the local
  // row j that is global row 2*total; outside 0..nyl the reference indexes
  // past its arrays
  for (int py = 0; py < c.cut_y; ++py) {
    const int j = 2 * c.total - py * nyl;
    if (j >= -2 && j <= nyl + 3 && (j < 0 || j > nyl)) {
      err = "detonation: the wall row falls on a ghost row of a rank (the reference would index "
            "outside its arrays); choose another total or rank grid";
      return SWFD_ERR_UNSUPPORTED;
    }
  }
  if (c.precision != SWFD_PRECISION_FP64 || (c.rk_choice != 0 && c.rk_choice != 1)) {
    err = "detonation: precision FP64 and rk_choice 1 only";
    return SWFD_ERR_UNSUPPORTED;
  }
  if (c.swp_num <= 0 && c.use_limiter == 2) {
    err = "detonation: swp_num must be positive";
    return SWFD_ERR_INVALID;
  }
  return SWFD_OK;
}

swfd_status ex7_create(swfd_handle* h, std::string& err) {
  const swfd_config& c = h->cfg;
  Ex7* x = new Ex7();
  h->ex7 = x;
  x->use_limiter = c.use_limiter;
  x->swp_num = c.swp_num;
  Ex7View& v = x->v;
  v.cut_x = c.cut_x;
  v.cut_y = c.cut_y;
  v.R = c.cut_x * c.cut_y;
  v.nxl = 5 * c.total / c.cut_x;
  v.nyl = 5 * c.total / c.cut_y;
  v.LI = v.nxl + 6;
  v.LJ = v.nyl + 6;
  v.LL = std::max(v.LI, v.LJ);
  v.total = c.total;
  v.wall = 2 * c.total;  // step = 2 (:12)
  v.nx = c.nx;
  v.ny = c.ny;
  // xleft = 5./cut_x*position_x, dx = (xright - xleft)/nx (:1224-1231): rank
  // (0,0)'s; every rank's must agree for one dt
  v.dx = (5. / c.cut_x * (0 + 1) - 5. / c.cut_x * 0) / v.nxl;
  v.dy = (5. / c.cut_y * (0 + 1) - 5. / c.cut_y * 0) / v.nyl;
  for (int p = 0; p < c.cut_x; ++p)
    if ((5. / c.cut_x * (p + 1) - 5. / c.cut_x * p) / v.nxl != v.dx) {
      err = "detonation: the ranks' dx differ (the reference's ranks would take different dt)";
      return SWFD_ERR_UNSUPPORTED;
    }
  for (int p = 0; p < c.cut_y; ++p)
    if ((5. / c.cut_y * (p + 1) - 5. / c.cut_y * p) / v.nyl != v.dy) {
      err = "detonation: the ranks' dy differ (the reference's ranks would take different dt)";
      return SWFD_ERR_UNSUPPORTED;
    }
  v.gamma = c.gamma;
  v.g1 = c.gamma - 1.;
  v.cfl = c.cfl;
  v.T = c.time_terminal;
  v.eps = 1e-13;
  v.eps2 = 1e-8;
  v.weno_eps = 1e-12;
  v.q = 50.;
  v.tc = 50.;
  v.kc = 2566.4;
  v.use_limiter = c.use_limiter;
  v.lim8_lt = 1e-8;
  x->t_loop = c.time_terminal - 1e-10;
  if (c.literals == SWFD_LITERALS_QUAD) {  // the constants of the 4-component path
    using namespace qd;
    const q128 one = from_double(1.0);
    v.quad = 1;
    v.q_c1312 = div(from_double(13.0), from_double(12.0));
    v.q_eps = div(one, from_double(1e12));
    v.q_1em15 = div(one, from_double(1e15));
    v.lim8_lt = ru(div(one, from_double(1e8)));  // rho < 1d-8 <=> rho < ru(1d-8)
    x->t_loop = rd(sub(from_double(c.time_terminal), div(one, from_double(1e10))));
  }
  // one device block: 9 rank buffers of 5 planes, alpha, line alphas, the
  // gathered interior, the global view, exp coefficients, scalars, flags
  const int64_t rp = (int64_t)v.R * v.LI * v.LJ, N = (int64_t)v.nx * v.ny;
  const int64_t gv = (int64_t)5 * (v.nx + 6) * (v.ny + 6);
  const int64_t ndbl = 9 * 5 * rp + rp + (int64_t)v.R * v.LL + 5 * N + gv;
  const size_t qbytes = sizeof(qd::q128) * (qd::EXP_N + 1);
  const size_t bytes = ndbl * sizeof(double) + qbytes + sizeof(Ex7Scalars) + 2 * N * sizeof(int) + 256;
  cudaError_t e = cudaMalloc(&x->block, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&x->sum_scratch, seq_sum_scratch_bytes(N));
  if (e != cudaSuccess) {
    err = std::string("detonation: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SWFD_ERR_OOM : SWFD_ERR_CUDA;
  }
  double* d = (double*)x->block;
  double** bufs[] = {&v.u, &v.u0, &v.sp, &v.sn, &v.fpf, &v.fnf, &v.gpf, &v.gnf, &v.roe};
  for (double** b : bufs) {
    *b = d;
    d += 5 * rp;
  }
  v.alpha = d;
  d += rp;
  v.lal = d;
  d += (int64_t)v.R * v.LL;
  v.ug = d;
  d += 5 * N;
  v.gview = d;
  d += gv;
  v.expc = (const qd::q128*)d;
  char* p = (char*)d + qbytes;
  p = (char*)(((uintptr_t)p + 15) & ~(uintptr_t)15);
  v.sc = (Ex7Scalars*)p;
  p += sizeof(Ex7Scalars);
  v.flag = (int*)p;
  v.list = v.flag + N;
  if ((e = cudaMallocHost(&x->hs, sizeof(Ex7Scalars))) != cudaSuccess) {
    err = std::string("detonation: ") + cudaGetErrorString(e);
    return SWFD_ERR_CUDA;
  }
  qd::q128 coef[qd::EXP_N + 1];
  qd::exp_coefs(coef);
  if ((e = cudaMemsetAsync(x->block, 0, bytes, h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync((void*)v.expc, coef, qbytes, cudaMemcpyHostToDevice, h->stream)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(h->stream)) != cudaSuccess) {
    err = std::string("detonation: ") + cudaGetErrorString(e);
    return SWFD_ERR_CUDA;
  }
  return SWFD_OK;
}

void ex7_destroy(Ex7* x) {
  if (!x) return;
  if (x->g_step) cudaGraphExecDestroy(x->g_step);
  cudaFree(x->tracks);
  cudaFree(x->block);
  cudaFree(x->sum_scratch);
  if (x->hs) cudaFreeHost(x->hs);
  delete x;
}

// initdata (:1196-1260): zero, then the post-detonation state where x < 0.5
// and the quiescent state elsewhere on local cells 0..nxl+1 x 0..nyl+1 of every
// rank; then bc (:1259)
swfd_status ex7_init(swfd_handle* h) {
  Ex7* x = h->ex7;
  const Ex7View& v = x->v;
  std::vector<double> u((size_t)5 * v.R * v.LI * v.LJ, 0.0);
  for (int r = 0; r < v.R; ++r) {
    const int px = r % v.cut_x;
    const double xleft = 5. / v.cut_x * px;
    const double dx = (5. / v.cut_x * (px + 1) - xleft) / v.nxl;
    for (int j = 0; j <= v.nyl + 1; ++j)
      for (int i = 0; i <= v.nxl + 1; ++i) {
        const double xc = xleft + i * dx - dx / 2.;
        const double s[5] = {11., 11. * 6.18, 0., 970., 11.}, q[5] = {1., 0., 0., 55., 1.};
        for (int c = 0; c < 5; ++c)
          u[(((size_t)r * 5 + c) * v.LJ + (j + 2)) * v.LI + (i + 2)] = xc < 0.5 ? s[c] : q[c];
      }
  }
  E7CU(h, cudaMemcpyAsync(v.u, u.data(), u.size() * sizeof(double), cudaMemcpyHostToDevice,
                          h->stream));
  ST(e7_bc(h));
  E7CU(h, cudaMemsetAsync(v.sc, 0, sizeof(Ex7Scalars), h->stream));
  h->time = 0.;
  ST(e7_publish_tracks(h));  // the reset cleared the scalars' track buffer
  return e7_sync_scalars(h);
}

swfd_status ex7_upload(swfd_handle* h, const double* u) {
  const Ex7View& v = h->ex7->v;
  const int64_t gv = (int64_t)5 * (v.nx + 6) * (v.ny + 6);
  E7CU(h, cudaMemcpyAsync(v.gview, u, gv * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  E7K(h, (k7_view<<<e7_grid((int64_t)v.R * v.LI * v.LJ), E7_BLOCK, 0, h->stream>>>(v, 0)));
  E7CU(h, cudaStreamSynchronize(h->stream));
  return SWFD_OK;
}

swfd_status ex7_download(swfd_handle* h, double* u) {
  const Ex7View& v = h->ex7->v;
  const int64_t gv = (int64_t)5 * (v.nx + 6) * (v.ny + 6);
  E7K(h, (k7_view<<<e7_grid(gv / 5), E7_BLOCK, 0, h->stream>>>(v, 1)));
  E7CU(h, cudaMemcpyAsync(u, v.gview, gv * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  E7CU(h, cudaStreamSynchronize(h->stream));
  return SWFD_OK;
}

swfd_status ex7_set_time(swfd_handle* h, double t) {
  h->time = t;
  E7CU(h, cudaMemcpyAsync(&h->ex7->v.sc->time, &h->time, sizeof(double), cudaMemcpyHostToDevice,
                          h->stream));
  E7CU(h, cudaStreamSynchronize(h->stream));
  return SWFD_OK;
}

swfd_status ex7_find_alpha(swfd_handle* h, double* alphamax) {
  Ex7* x = h->ex7;
  const Ex7View& v = x->v;
  E7CU(h, cudaMemsetAsync(&v.sc->am_bits, 0, sizeof(unsigned long long), h->stream));
  E7K(h, (k7_alpha<<<e7_grid((int64_t)v.R * v.LI * v.LJ), E7_BLOCK, 0, h->stream>>>(v)));
  E7K(h, (k7_alphamax<<<1, 1, 0, h->stream>>>(v)));
  ST(e7_sync_scalars(h));
  *alphamax = x->hs->alphamax;
  return SWFD_OK;
}

// One step (:810-888) as one graph launch (SWFD_LAUNCH=eager: the same
// kernels on the stream, the conditions read back), then one read-back of
// the scalars: the device's errors become the step's status, its time the
// host's.
swfd_status ex7_step(swfd_handle* h, double* dt_out) {
  Ex7* x = h->ex7;
  ST(e7_ensure_tracks(h, 3));
  const Ex7Scalars before = *x->hs;
  if (h->eager) {
    Builder b;
    b.h = h;
    b.eager = true;
    b.cond_word = &x->v.sc->cond;
    b.launched = &x->launches;
    e7_emit_step(b, x, h->stream);
    if (b.err != cudaSuccess)
      return e7_fail(h, SWFD_ERR_CUDA, std::string("detonation: ") + cudaGetErrorString(b.err));
  } else {
    ST(e7_build_step(h));
    E7CU(h, cudaGraphLaunch(x->g_step, h->stream));
  }
  ST(e7_sync_scalars(h));
  const Ex7Scalars& a = *x->hs;
  if (!h->eager)  // kernels run: the step's, each sweep's fixed part, densities, pass pairs
    x->launches += x->k_step + (a.sweep_count - before.sweep_count) * x->k_sweep +
                   (a.den_count - before.den_count) + (a.pre_count - before.pre_count) * x->k_q;
  if (a.err & E7_ERR_NONFINITE)
    return e7_fail(h, SWFD_ERR_NONFINITE, "detonation: non-finite alpha or dt");
  if (a.err & E7_ERR_PUBAR)
    return e7_fail(h, SWFD_ERR_PUBAR_NONPOS, "detonation sweep: P(u_bar) <= 0");
  if (a.err & E7_ERR_SWEEP_CHECK)
    return e7_fail(h, SWFD_ERR_SWEEP_CHECK, "detonation sweep: total pressure increased");
  if (a.err & E7_ERR_SWEEP_INDEX)
    return e7_fail(h, SWFD_ERR_UNSUPPORTED,
                   "detonation sweep: the first ordering-II step adjusts, where the "
                   "reference reads sweepI(0)");
  if (a.err & E7_ERR_NOCONV)
    return e7_fail(h, SWFD_ERR_SWEEP_NOCONV, "detonation sweep: swp_num reached");
  h->time = a.time;
  if (dt_out) *dt_out = a.dt;
  return SWFD_OK;
}

// the device's tracks of the sweeps so far (n entries each)
swfd_status e7_read_tracks(swfd_handle* h, std::vector<int32_t>& t, int64_t& n) {
  Ex7* x = h->ex7;
  ST(e7_sync_scalars(h));
  n = std::min<int64_t>(x->hs->sweep_count, x->track_cap);
  t.assign(3 * (size_t)n, 0);
  for (int c = 0; c < 3 && n > 0; ++c)
    E7CU(h, cudaMemcpy(t.data() + c * n, x->tracks + c * x->track_cap, n * sizeof(int32_t),
                       cudaMemcpyDeviceToHost));
  return SWFD_OK;
}

swfd_status ex7_stats(swfd_handle* h, swfd_sweep_stats* st) {
  const Ex7* x = h->ex7;
  std::vector<int32_t> t;
  int64_t n = 0;
  ST(e7_read_tracks(h, t, n));
  memset(st, 0, sizeof(*st));
  st->sweep_count = x->hs->sweep_count;
  for (int64_t k = 0; k < n; ++k) {
    st->total_sweep += t[k];
    st->max_sweep = std::max<int64_t>(st->max_sweep, t[k]);
    st->total_neg += t[n + k];
    st->max_neg = std::max<int64_t>(st->max_neg, t[n + k]);
    st->total_pos += t[2 * n + k];
    st->max_pos = std::max<int64_t>(st->max_pos, t[2 * n + k]);
  }
  st->den_count = x->hs->den_count + x->hs->lim_den;  // the ranks' limiter counts, summed
  st->pre_count = x->hs->pre_count + x->hs->lim_pre;
  st->sweep_fail_count = x->hs->fail_count;
  return SWFD_OK;
}

int64_t ex7_tracks(swfd_handle* h, int32_t* sweep, int32_t* neg, int32_t* pos, int64_t cap) {
  std::vector<int32_t> t;
  int64_t n = 0;
  if (e7_read_tracks(h, t, n) != SWFD_OK) return -1;
  const int64_t m = std::min<int64_t>(n, cap);
  for (int64_t k = 0; k < m; ++k) {
    if (sweep) sweep[k] = t[k];
    if (neg) neg[k] = t[n + k];
    if (pos) pos[k] = t[2 * n + k];
  }
  return n;
}

int64_t ex7_launches(swfd_handle* h) { return h->ex7->launches; }
double ex7_t_loop(swfd_handle* h) { return h->ex7->t_loop; }

}  // namespace swfd
