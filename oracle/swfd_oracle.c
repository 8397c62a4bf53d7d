/*
 * swfd_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, single-threaded restatement of the reference's sweeping
 * FD-WENO Euler time step (dcgriffi/Sweeping_FD_WENO, Fortran).  It is the
 * parity oracle for the CUDA library and the timed CPU baseline.  Only the
 * tests, __graft_entry__.smoke() and bench.py (CPU-baseline leg) may load
 * it; the product never calls, links or falls back to it.
 *
 * Parity pinning: the reference ships no tests and no golden outputs, and no
 * Fortran compiler exists in this container, so the reference cannot be run
 * here.  The restatement is pinned by known-answer properties of the
 * reference's own algorithm (5th-order vortex convergence,
 * ex3_vortex_accuracy_2d/main.f90:725-777; exact conservation of the sweeps;
 * positivity after a converged sweep; WENO5 reproduction of quadratics),
 * checked in tests/test_oracle.py.
 *
 * Faithfulness rules followed throughout:
 *  - operation order is the Fortran left-to-right order of each statement;
 *    x**2 is x*x; no reassociation, no reciprocal-multiply for a division;
 *    compiled with -ffp-contract=off so no FMA is formed;
 *  - gfortran -fdefault-real-8 (the reference Makefiles, e.g.
 *    ex3_vortex_accuracy_2d/Makefile:15) promotes double-kind literals
 *    (1d-6, 13d0/12d0, 0.75d0, 1d-15 ...) to REAL(16); every subexpression
 *    that contains one is evaluated in _Float128 when cfg.literals ==
 *    SWFD_LITERALS_QUAD and rounded to double once on assignment, exactly as
 *    a mixed REAL(8)/REAL(16) Fortran expression is;
 *  - MIN/MAX are fmin/fmax.
 *
 * Memory layout: u(ncomp, -2:nx+3, -2:ny+3) in Fortran column-major order,
 * the layout of the reference arrays (ex3_vortex_accuracy_2d/main.f90:8).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/swfd.h"

typedef _Float128 Q;

#define MAXC 4

typedef struct oracle {
  swfd_config cfg;
  int ndim, nc, nx, ny, LI, LJ;
  int quad;
  double gamma, gamma1, eps, eps2, weno_eps, dx, dy;
  Q weno_eps_q;
  /* per-example switches (the variant matrix of the reference) */
  int problem;
  double *u, *u0, *rhs, *fp, *fn, *gp, *gn, *fpf, *fnf, *gpf, *gnf;
  double *x, *y;
  double *wk_w, *wk_vx, *wk_vy, *wk_h; /* per-line Roe prep, 0:max(nx,ny)+2 */
  double *rho_t;                        /* sweep scratch */
  int *sI_i, *sI_j, *sII_i, *sII_j;     /* snake orderings, 1-based cells */
  double weight;                        /* all weights are equal */
  double alphamax, dt, time;
  int postag;
  /* statistics (ex3_vortex_accuracy_2d/main.f90:14,24-31) */
  int64_t sweep_count, den_count, pre_count, fail_count;
  int64_t t_pos_count, t_neg_count;
  int64_t restarts;       /* restart RK: dt halvings of all steps */
  int32_t *sweep_track, *neg_track, *pos_track;
  int64_t track_cap;
  int status;
  /* ex6 (shock diffraction): the reference's cut_x x cut_y MPI ranks, each a
   * local grid nxl x nyl with its own ghost layers (`rk`), the per-cell alpha
   * of each rank, and the inflow state */
  int ex4like; /* ex4 and ex6: eps2 flux guard, 1d-15 Roe regularisers */
  int total, cut_x, cut_y, nxl, nyl, px, py;
  struct oracle** rk;
  double* alpha;
  double dle, ule, ple;
  /* ex7 (detonation): q_const, t_const, k_const (ex7_detonation/main.f90:18),
   * the wall's top row step*total (:12,188) and the per-line Roe Y ratio */
  double qc, tc, kc;
  int wall_rows;
  double* wk_ratio;
  int ranks_stale; /* the global state was set from outside: rebuild the ranks */
} oracle;

/* ------------------------------------------------------------------ */
/* indexing                                                            */
/* ------------------------------------------------------------------ */
static inline size_t IX(const oracle* o, int c, int i, int j) {
  return (size_t)c + (size_t)o->nc * ((size_t)(i + 2) + (size_t)o->LI * (size_t)(j + 2));
}
#define U(a, c, i, j) ((a)[IX(o, (c), (i), (j))])

static inline double sq(double a) { return a * a; }
static inline Q sqq(Q a) { return a * a; }

/* ------------------------------------------------------------------ */
/* WENO5 (ex3_vortex_accuracy_2d/weno5.f90:3-15, 86-146)               */
/* ------------------------------------------------------------------ */
/* c(-1:2,0:2), reshaped column-major from weno5.f90:3-15 */
static const double WC[4][3] = {
    /* c(-1,:) */ {1.83333333333333333333333333333333, -1.16666666666666666666666666666667,
                   0.333333333333333333333333333333333},
    /* c( 0,:) */ {0.333333333333333333333333333333333, 0.833333333333333333333333333333333,
                   -0.166666666666666666666666666666667},
    /* c( 1,:) */ {-0.166666666666666666666666666666667, 0.833333333333333333333333333333333,
                   0.333333333333333333333333333333333},
    /* c( 2,:) */ {0.333333333333333333333333333333333, -1.16666666666666666666666666666667,
                   1.83333333333333333333333333333333}};
#define CW(r, i) WC[(r) + 1][(i)]

/* smoothness indicators beta(1:3), weno5.f90:100-102 (a[0..4] = average(-2..2)) */
static void weno_beta(int quad, const double* a, double* b) {
  const double am2 = a[0], am1 = a[1], a0 = a[2], ap1 = a[3], ap2 = a[4];
  if (quad) {
    const Q c1312 = (Q)13 / (Q)12, two = 2, three = 3, four = 4, qrt = 0.25;
    Q s, t;
    s = (Q)a0 - two * (Q)ap1 + (Q)ap2;
    t = three * (Q)a0 - four * (Q)ap1 + (Q)ap2;
    b[0] = (double)(c1312 * sqq(s) + qrt * sqq(t));
    s = (Q)am1 - two * (Q)a0 + (Q)ap1;
    /* (average(-1)-average(1))**2 has only REAL(8) operands */
    b[1] = (double)(c1312 * sqq(s) + qrt * (Q)sq(am1 - ap1));
    s = (Q)am2 - two * (Q)am1 + (Q)a0;
    t = (Q)am2 - four * (Q)am1 + three * (Q)a0;
    b[2] = (double)(c1312 * sqq(s) + qrt * sqq(t));
  } else {
    const double c1312 = 13.0 / 12.0;
    b[0] = c1312 * sq(a0 - 2.0 * ap1 + ap2) + 0.25 * sq(3.0 * a0 - 4.0 * ap1 + ap2);
    b[1] = c1312 * sq(am1 - 2.0 * a0 + ap1) + 0.25 * sq(am1 - ap1);
    b[2] = c1312 * sq(am2 - 2.0 * am1 + a0) + 0.25 * sq(am2 - 4.0 * am1 + 3.0 * a0);
  }
}

/* alpha = lin/(eps+beta)**2, weno5.f90:104-106,138-140 */
static double weno_alpha(const oracle* o, double lin, double beta) {
  if (o->quad) {
    Q s = o->weno_eps_q + (Q)beta;
    return (double)((Q)lin / (s * s));
  }
  double s = o->weno_eps + beta;
  return lin / (s * s);
}

/* weno_left (weno5.f90:86-113) */
double oracle_weno_left_impl(const oracle* o, const double* a) {
  double up[3], beta[3], al[3], ww[3];
  for (int k = 1; k <= 3; ++k) {
    int is = k - 3;
    double s = 0.0;
    for (int i = 0; i <= 2; ++i) s = s + CW(-is - 1, i) * a[is + i + 2];
    up[k - 1] = s;
  }
  weno_beta(o->quad, a, beta);
  al[0] = weno_alpha(o, 0.1, beta[0]);
  al[1] = weno_alpha(o, 0.6, beta[1]);
  al[2] = weno_alpha(o, 0.3, beta[2]);
  ww[0] = al[0] / (al[0] + al[1] + al[2]);
  ww[1] = al[1] / (al[0] + al[1] + al[2]);
  ww[2] = al[2] / (al[0] + al[1] + al[2]);
  return ww[0] * up[2] + ww[1] * up[1] + ww[2] * up[0];
}

/* weno_right (weno5.f90:120-146) */
double oracle_weno_right_impl(const oracle* o, const double* a) {
  double um[3], beta[3], al[3], ww[3];
  for (int k = 1; k <= 3; ++k) {
    int is = k - 3;
    double s = 0.0;
    for (int i = 0; i <= 2; ++i) s = s + CW(-is, i) * a[is + i + 2];
    um[k - 1] = s;
  }
  weno_beta(o->quad, a, beta);
  al[0] = weno_alpha(o, 0.3, beta[0]);
  al[1] = weno_alpha(o, 0.6, beta[1]);
  al[2] = weno_alpha(o, 0.1, beta[2]);
  ww[0] = al[0] / (al[0] + al[1] + al[2]);
  ww[1] = al[1] / (al[0] + al[1] + al[2]);
  ww[2] = al[2] / (al[0] + al[1] + al[2]);
  return ww[0] * um[2] + ww[1] * um[1] + ww[2] * um[0];
}

/* ------------------------------------------------------------------ */
/* literal-sensitive comparisons and RK combinations                    */
/* ------------------------------------------------------------------ */
/* rho < 1d-8 with a double-kind literal (ex3_vortex_accuracy_2d/main.f90:75) */
static int lt_lit_1em8(const oracle* o, double rho) {
  if (o->quad) return (Q)rho < (Q)1e-8f128;
  return rho < 1e-8;
}
static int gt_lit_1em8(const oracle* o, double rho) {
  if (o->quad) return (Q)rho > (Q)1e-8f128;
  return rho > 1e-8;
}
static int le_lit_1em8(const oracle* o, double rho) {
  if (o->quad) return (Q)rho <= (Q)1e-8f128;
  return rho <= 1e-8;
}
/* u = 0.75d0*u0 + 0.25d0*(u + dt*RHS)  (ex3_vortex_accuracy_2d/main.f90:604) */
static inline double rk2(const oracle* o, double u0, double v) {
  if (o->quad) return (double)((Q)0.75 * (Q)u0 + (Q)0.25 * (Q)v);
  return 0.75 * u0 + 0.25 * v;
}
/* u = (u0 + 2d0*(u + dt*RHS))/3d0  (ex3_vortex_accuracy_2d/main.f90:621) */
static inline double rk3(const oracle* o, double u0, double v) {
  if (o->quad) return (double)(((Q)u0 + (Q)2 * (Q)v) / (Q)3);
  return (u0 + 2.0 * v) / 3.0;
}

/* ------------------------------------------------------------------ */
/* 2D: fluxes (ex3_vortex_accuracy_2d/main.f90:61-113,                  */
/*             ex4_sedov_2d/main.f90:125-177)                           */
/* ------------------------------------------------------------------ */
static void fflux2d(const oracle* o, const double* a, double* f, int gdir) {
  double rho = a[0], mx = a[1], my = a[2], e = a[3];
  double vx = mx / rho, vy = my / rho;
  int guard = o->ex4like ? (rho < o->eps2) : lt_lit_1em8(o, rho);
  if (guard) vx = 0.0;
  if (guard) vy = 0.0;
  double pres = o->gamma1 * (e - 0.5 * rho * (vx * vx) - 0.5 * rho * (vy * vy));
  if (!gdir) {
    f[0] = mx;
    f[1] = rho * (vx * vx) + pres;
    f[2] = rho * vx * vy;
    f[3] = (e + pres) * vx;
  } else {
    f[0] = my;
    f[1] = rho * vx * vy;
    f[2] = rho * (vy * vy) + pres;
    f[3] = (e + pres) * vy;
  }
}

/* findalpha (ex3_vortex_accuracy_2d/main.f90:549-562;
 *            eps2-guarded form ex5_mach2000_jet/main.f90:553-589,
 *            ex4_sedov_2d/main.f90:652-683) */
static void findalpha2d(oracle* o) {
  double am = 0.0;
  for (int i = -2; i <= o->nx + 3; ++i)
    for (int j = -2; j <= o->ny + 3; ++j) {
      double u1 = U(o->u, 0, i, j), u2 = U(o->u, 1, i, j), u3 = U(o->u, 2, i, j),
             u4 = U(o->u, 3, i, j);
      double den = u1;
      if (o->problem == SWFD_PROBLEM_VORTEX_2D) {
        double pres = o->gamma1 * (u4 - u2 * u2 / u1 / 2.0 - u3 * u3 / u1 / 2.0);
        double sound = sqrt(o->gamma * pres / den);
        am = fmax(fmax(am, fabs(u2 / u1) + sound), fabs(u3 / u1) + sound);
      } else {
        double vx, vy;
        if (den >= o->eps2) {
          vx = u2 / den;
          vy = u3 / den;
        } else {
          vx = 0.0;
          vy = 0.0;
        }
        double pres = o->gamma1 * (u4 - 0.5 * den * (vx * vx) - 0.5 * den * (vy * vy));
        double sound = sqrt(o->gamma * pres / den);
        double a = fmax(fabs(u2 / u1) + sound, fabs(u3 / u1) + sound);
        am = fmax(am, a);
      }
    }
  o->alphamax = am;
}

/* Roe average + eigenvectors + characteristic WENO for one interface of one
 * line (x pass ex3_vortex_accuracy_2d/main.f90:148-229, y pass :349-431;
 * ex4 regularisers ex4_sedov_2d/main.f90:234,240,455). s[m][c] holds the
 * split fluxes of stencil cells m = 0..4 (offsets -2..2).  ydir swaps the
 * roles of the two momentum components. */
static void interface2d(const oracle* o, int ydir, double wl, double wr, double vxl, double vxr,
                        double vyl, double vyr, double hl, double hr, const double sp[5][4],
                        const double sn[5][4], double* outp, double* outn) {
  double evr[4][4], evl[4][4], cu_p[4][5], cu_n[4][5], ur[4], ul[4];
  const double g1 = o->gamma1;
  double t0, t1, t2, t3;
  if (o->ex4like && o->quad)
    t0 = (double)((Q)wl / ((Q)(wl + wr) + (Q)1e-15f128));
  else
    t0 = wl / (wl + wr + 1.e-15);
  t1 = 1. - t0;
  double vxm = t0 * vxl + t1 * vxr;
  double vym = t0 * vyl + t1 * vyr;
  double hm = t0 * hl + t1 * hr;
  double qm = 0.5 * (vxm * vxm + vym * vym);
  double cm;
  if (o->ex4like && o->quad)
    cm = (double)((Q)sqrt(fabs(g1 * (hm - qm))) + (Q)1e-15f128);
  else if (o->ex4like)
    cm = sqrt(fabs(g1 * (hm - qm))) + 1e-15;
  else
    cm = sqrt(fabs(g1 * (hm - qm))) + 1.e-15;
  double vn = ydir ? vym : vxm; /* velocity normal to the interface */
  double vt = ydir ? vxm : vym; /* tangential velocity */
  t0 = vn * cm;
  /* evr rows: 1 = density, 2 = x-momentum, 3 = y-momentum, 4 = energy */
  evr[0][0] = 1.0; evr[0][1] = 0.0; evr[0][2] = 1.0; evr[0][3] = 1.0;
  if (!ydir) {
    evr[1][0] = vxm - cm; evr[1][1] = 0.0; evr[1][2] = vxm; evr[1][3] = vxm + cm;
    evr[2][0] = vym;      evr[2][1] = 1.0; evr[2][2] = vym; evr[2][3] = vym;
  } else {
    evr[1][0] = vxm;      evr[1][1] = 1.0; evr[1][2] = vxm; evr[1][3] = vxm;
    evr[2][0] = vym - cm; evr[2][1] = 0.0; evr[2][2] = vym; evr[2][3] = vym + cm;
  }
  evr[3][0] = hm - t0; evr[3][1] = vt; evr[3][2] = qm; evr[3][3] = hm + t0;
  double rcm = 1. / cm;
  double b1 = g1 * rcm * rcm;
  double b2 = qm * b1;
  t0 = vn * rcm;
  t1 = b1 * vn;
  t2 = 0.5 * b1;
  t3 = b1 * vt;
  if (!ydir) {
    evl[0][0] = 0.5 * (b2 + t0); evl[0][1] = -0.5 * (t1 + rcm); evl[0][2] = -0.5 * t3; evl[0][3] = t2;
    evl[1][0] = -vym;            evl[1][1] = 0.0;               evl[1][2] = 1.0;        evl[1][3] = 0.0;
    evl[2][0] = 1. - b2;         evl[2][1] = t1;                evl[2][2] = t3;         evl[2][3] = -b1;
    evl[3][0] = 0.5 * (b2 - t0); evl[3][1] = -0.5 * (t1 - rcm); evl[3][2] = -0.5 * t3; evl[3][3] = t2;
  } else {
    evl[0][0] = 0.5 * (b2 + t0); evl[0][1] = -0.5 * t3; evl[0][2] = -0.5 * (t1 + rcm); evl[0][3] = t2;
    evl[1][0] = -vxm;            evl[1][1] = 1.0;       evl[1][2] = 0.0;               evl[1][3] = 0.0;
    evl[2][0] = 1. - b2;         evl[2][1] = t3;        evl[2][2] = t1;                evl[2][3] = -b1;
    evl[3][0] = 0.5 * (b2 - t0); evl[3][1] = -0.5 * t3; evl[3][2] = -0.5 * (t1 - rcm); evl[3][3] = t2;
  }
  for (int ig = 0; ig < 5; ++ig)
    for (int k = 0; k < 4; ++k) {
      cu_p[k][ig] = evl[k][0] * sp[ig][0] + evl[k][1] * sp[ig][1] + evl[k][2] * sp[ig][2] +
                    evl[k][3] * sp[ig][3];
      cu_n[k][ig] = evl[k][0] * sn[ig][0] + evl[k][1] * sn[ig][1] + evl[k][2] * sn[ig][2] +
                    evl[k][3] * sn[ig][3];
    }
  for (int kk = 0; kk < 4; ++kk) {
    ur[kk] = oracle_weno_right_impl(o, cu_p[kk]);
    ul[kk] = oracle_weno_left_impl(o, cu_n[kk]);
  }
  for (int k = 0; k < 4; ++k) {
    outp[k] = evr[k][0] * ur[0] + evr[k][1] * ur[1] + evr[k][2] * ur[2] + evr[k][3] * ur[3];
    outn[k] = evr[k][0] * ul[0] + evr[k][1] * ul[1] + evr[k][2] * ul[2] + evr[k][3] * ul[3];
  }
}

/* cell preparation of one line (x pass ex3_vortex_accuracy_2d/main.f90:134-147,
 * y pass :335-348; ex4 y pass uses 1./(den+1d-15), ex4_sedov_2d/main.f90:426) */
static void prep_cell(const oracle* o, int ydir, const double* a, double* w, double* vx,
                      double* vy, double* h) {
  double den = a[0], xmt = a[1], ymt = a[2], eng = a[3];
  double t0;
  if (ydir && o->ex4like) {
    if (o->quad)
      t0 = (double)((Q)1 / ((Q)den + (Q)1e-15f128));
    else
      t0 = 1. / (den + 1e-15);
  } else {
    t0 = 1. / den;
  }
  double vex = xmt * t0, vey = ymt * t0;
  double pre = o->gamma1 * (eng - 0.5 * (xmt * vex + ymt * vey));
  *w = sqrt(fabs(den));
  *vx = vex;
  *vy = vey;
  *h = (pre + eng) * t0;
}

/* use_limiter = 1: positivity limiter of one split flux (ex3_vortex_accuracy_2d/main.f90:241-329,
 * y pass :444-530; ex6 clamps theta at 0, ex6_shock_diffraction/main.f90:330,351,379,398).
 * ave: the split flux of the interface's left cell; out: its reconstructed flux. */
static void zs_limit(oracle* o, const double* ave, double* out) {
  const double g1 = o->gamma1;
  const int clamp = o->problem == SWFD_PROBLEM_SHOCK_DIFFRACTION;
  const double d_ave = ave[0], m_ave = ave[1], n_ave = ave[2], e_ave = ave[3];
  const double p_ave = g1 * (e_ave - 0.5 * (m_ave * m_ave) / d_ave - 0.5 * (n_ave * n_ave) / d_ave);
  double point[2][4];
  double theta = 1.0;
  for (int c = 0; c < 4; ++c) {
    point[0][c] = out[c];
    point[1][c] = (ave[c] - out[c] / 12.) / (11. / 12.);
  }
  for (int ig = 0; ig < 2; ++ig) {
    double d_l = point[ig][0];
    if (d_l < 0.) theta = fmin(theta, fabs(d_ave - 0.) / fabs(d_ave - d_l));
  }
  if (clamp) theta = fmax(theta, 0.);
  if (theta < 1.) {
    out[0] = theta * out[0] + (1. - theta) * d_ave;
    o->den_count++;
  }
  theta = 1.;
  point[0][0] = out[0];
  point[1][0] = (ave[0] - out[0] / 12.) / (11. / 12.);
  for (int ig = 0; ig < 2; ++ig) {
    double d_l = point[ig][0], m_l = point[ig][1], n_l = point[ig][2], e_l = point[ig][3];
    double p_l = g1 * (e_l - (m_l * m_l) / d_l / 2. - (n_l * n_l) / d_l / 2.);
    if (p_l < 0.) theta = fmin(theta, fabs(p_ave - 0.) / fabs(p_ave - p_l));
  }
  if (clamp) theta = fmax(theta, 0.);
  if (theta < 1.) {
    o->pre_count++;
    for (int c = 0; c < 4; ++c) out[c] = theta * out[c] + (1. - theta) * ave[c];
  }
}

/* the limiter on both split fluxes of an interface whose left cell is (i, j) */
static void limit_interface(oracle* o, const double* pos, const double* neg, int i, int j,
                            double* op, double* on) {
  if (o->cfg.use_limiter != 1) return;
  double a[4], b[4];
  for (int c = 0; c < 4; ++c) {
    a[c] = pos[IX(o, c, i, j)];
    b[c] = neg[IX(o, c, i, j)];
  }
  zs_limit(o, a, op);
  zs_limit(o, b, on);
}

/* wenofd (ex3_vortex_accuracy_2d/main.f90:115-534; ex4_sedov_2d/main.f90:179-637) */
static void wenofd2d(oracle* o) {
  const int nx = o->nx, ny = o->ny;
  findalpha2d(o);
  const double am = o->alphamax;
  for (int i = -2; i <= nx + 3; ++i)
    for (int j = -2; j <= ny + 3; ++j) {
      double a[4], f[4], g[4];
      for (int c = 0; c < 4; ++c) a[c] = U(o->u, c, i, j);
      fflux2d(o, a, f, 0);
      fflux2d(o, a, g, 1);
      for (int c = 0; c < 4; ++c) {
        U(o->fp, c, i, j) = 0.5 * (a[c] + f[c] / am);
        U(o->fn, c, i, j) = 0.5 * (a[c] - f[c] / am);
        U(o->gp, c, i, j) = 0.5 * (a[c] + g[c] / am);
        U(o->gn, c, i, j) = 0.5 * (a[c] - g[c] / am);
      }
    }
  const int premul = (o->problem == SWFD_PROBLEM_SEDOV_2D);
  /* x pass */
  for (int j = 0; j <= ny + 1; ++j) {
    for (int i = 0; i <= nx + 2; ++i) {
      double a[4];
      for (int c = 0; c < 4; ++c) a[c] = U(o->u, c, i, j);
      prep_cell(o, 0, a, &o->wk_w[i], &o->wk_vx[i], &o->wk_vy[i], &o->wk_h[i]);
    }
    for (int i = 0; i <= nx + 1; ++i) {
      double sp[5][4], sn[5][4], op[4], on[4];
      for (int ig = 0; ig < 5; ++ig)
        for (int c = 0; c < 4; ++c) {
          sp[ig][c] = U(o->fp, c, i + ig - 2, j);
          sn[ig][c] = U(o->fn, c, i + ig - 2, j);
        }
      interface2d(o, 0, o->wk_w[i], o->wk_w[i + 1], o->wk_vx[i], o->wk_vx[i + 1], o->wk_vy[i],
                  o->wk_vy[i + 1], o->wk_h[i], o->wk_h[i + 1], (const double(*)[4])sp,
                  (const double(*)[4])sn, op, on);
      limit_interface(o, o->fp, o->fn, i, j, op, on);
      for (int c = 0; c < 4; ++c) {
        U(o->fpf, c, i, j) = premul ? am * op[c] : op[c];
        U(o->fnf, c, i, j) = premul ? am * on[c] : on[c];
      }
    }
  }
  /* y pass */
  for (int i = 0; i <= nx + 1; ++i) {
    for (int j = 0; j <= ny + 2; ++j) {
      double a[4];
      for (int c = 0; c < 4; ++c) a[c] = U(o->u, c, i, j);
      prep_cell(o, 1, a, &o->wk_w[j], &o->wk_vx[j], &o->wk_vy[j], &o->wk_h[j]);
    }
    for (int j = 0; j <= ny + 1; ++j) {
      double sp[5][4], sn[5][4], op[4], on[4];
      for (int ig = 0; ig < 5; ++ig)
        for (int c = 0; c < 4; ++c) {
          sp[ig][c] = U(o->gp, c, i, j + ig - 2);
          sn[ig][c] = U(o->gn, c, i, j + ig - 2);
        }
      interface2d(o, 1, o->wk_w[j], o->wk_w[j + 1], o->wk_vx[j], o->wk_vx[j + 1], o->wk_vy[j],
                  o->wk_vy[j + 1], o->wk_h[j], o->wk_h[j + 1], (const double(*)[4])sp,
                  (const double(*)[4])sn, op, on);
      limit_interface(o, o->gp, o->gn, i, j, op, on);
      for (int c = 0; c < 4; ++c) {
        U(o->gpf, c, i, j) = premul ? am * op[c] : op[c];
        U(o->gnf, c, i, j) = premul ? am * on[c] : on[c];
      }
    }
  }
}

/* scheme (ex3_vortex_accuracy_2d/main.f90:536-547; ex4_sedov_2d/main.f90:639-650) */
static void scheme2d(oracle* o) {
  const size_t n = (size_t)o->nc * o->LI * o->LJ;
  memset(o->rhs, 0, n * sizeof(double));
  const double am = o->alphamax, dx = o->dx, dy = o->dy;
  const int premul = o->ex4like;
  for (int i = 1; i <= o->nx; ++i)
    for (int j = 1; j <= o->ny; ++j)
      for (int c = 0; c < 4; ++c) {
        double A = (U(o->fpf, c, i, j) - U(o->fnf, c, i + 1, j)) -
                   (U(o->fpf, c, i - 1, j) - U(o->fnf, c, i, j));
        double B = (U(o->gpf, c, i, j) - U(o->gnf, c, i, j + 1)) -
                   (U(o->gpf, c, i, j - 1) - U(o->gnf, c, i, j));
        if (premul)
          U(o->rhs, c, i, j) = -A / dx - B / dy;
        else
          U(o->rhs, c, i, j) = -(am * A) / dx - (am * B) / dy;
      }
}

/* checkpositivity (ex3_vortex_accuracy_2d/main.f90:634-651; `<` in
 * ex4_sedov_2d/main.f90:779-801 and ex5_mach2000_jet/main.f90:667-684) */
static int checkpositivity2d(const oracle* o) {
  const int strict = (o->problem == SWFD_PROBLEM_SEDOV_2D || o->problem == SWFD_PROBLEM_JET_2D);
  int postag = 0;
  for (int i = 1; i <= o->nx; ++i)
    for (int j = 1; j <= o->ny; ++j) {
      double u1 = U(o->u, 0, i, j), u2 = U(o->u, 1, i, j), u3 = U(o->u, 2, i, j),
             u4 = U(o->u, 3, i, j);
      double pe = u4 - u3 * u3 / u1 / 2. - u2 * u2 / u1 / 2.;
      if (strict) {
        if (u1 < o->eps) postag = 1;
        if (pe < o->eps) postag = 1;
      } else {
        if (u1 <= o->eps) postag = 1;
        if (pe <= o->eps) postag = 1;
      }
    }
  return postag;
}

/* bc (ex3_vortex_accuracy_2d/main.f90:653-669 periodic;
 *     ex4_sedov_2d/main.f90:922-994 reflect x=0,y=0 + outflow;
 *     ex5_mach2000_jet/main.f90:686-742 jet inflow + reflect y=0 + outflow) */
static void bc2d(oracle* o) {
  const int nx = o->nx, ny = o->ny;
  double* u = o->u;
  if (o->problem == SWFD_PROBLEM_VORTEX_2D) {
    for (int j = -2; j <= ny + 3; ++j)
      for (int i = 1; i <= 3; ++i)
        for (int c = 0; c < 4; ++c) {
          U(u, c, 1 - i, j) = U(u, c, nx + 1 - i, j);
          U(u, c, nx + i, j) = U(u, c, i, j);
        }
    for (int j = 1; j <= 3; ++j)
      for (int i = -2; i <= nx + 3; ++i)
        for (int c = 0; c < 4; ++c) {
          U(u, c, i, 1 - j) = U(u, c, i, ny + 1 - j);
          U(u, c, i, ny + j) = U(u, c, i, j);
        }
  } else if (o->problem == SWFD_PROBLEM_SEDOV_2D) {
    for (int j = -2; j <= ny + 3; ++j)
      for (int i = 1; i <= 3; ++i) {
        U(u, 0, 1 - i, j) = U(u, 0, i, j);
        U(u, 1, 1 - i, j) = -U(u, 1, i, j);
        U(u, 2, 1 - i, j) = U(u, 2, i, j);
        U(u, 3, 1 - i, j) = U(u, 3, i, j);
      }
    for (int j = 1; j <= 3; ++j)
      for (int i = -2; i <= nx + 3; ++i) {
        U(u, 0, i, 1 - j) = U(u, 0, i, j);
        U(u, 1, i, 1 - j) = U(u, 1, i, j);
        U(u, 2, i, 1 - j) = -U(u, 2, i, j);
        U(u, 3, i, 1 - j) = U(u, 3, i, j);
      }
    /* x(nx+1) > xm and y(ny+1) > ym always hold on the single block */
    for (int ig = 1; ig <= 3; ++ig)
      for (int j = -2; j <= ny + 3; ++j)
        for (int c = 0; c < 4; ++c) U(u, c, nx + ig, j) = U(u, c, nx, j);
    for (int ig = 1; ig <= 3; ++ig)
      for (int i = -2; i <= nx + 3; ++i)
        for (int c = 0; c < 4; ++c) U(u, c, i, ny + ig) = U(u, c, i, ny);
  } else if (o->problem == SWFD_PROBLEM_JET_2D) {
    /* variant 1: the full domain [0,1]x[-0.25,0.25] of the jet (inflow for
     * |y| <= 0.05, outflow at the bottom in place of the y = 0 symmetry
     * plane); the loops and their order are the half domain's */
    const int full = o->cfg.variant == 1;
    const double ujet = 800.;
    for (int j = -2; j <= ny + 3; ++j) {
      if (full ? fabs(o->y[j + 2]) <= 0.05 : o->y[j + 2] <= 0.05) {
        for (int i = 1; i <= 3; ++i) {
          U(u, 0, 1 - i, j) = 5.;
          U(u, 1, 1 - i, j) = 5. * ujet;
          U(u, 2, 1 - i, j) = 0.;
          U(u, 3, 1 - i, j) =
              0.4127 / o->gamma1 + 0.5 * (U(u, 1, 1 - i, j) * U(u, 1, 1 - i, j)) / U(u, 0, 1 - i, j);
        }
      } else {
        for (int i = 1; i <= 3; ++i) {
          U(u, 0, 1 - i, j) = 0.5;
          U(u, 1, 1 - i, j) = 0.;
          U(u, 2, 1 - i, j) = 0.;
          U(u, 3, 1 - i, j) = 0.4127 / o->gamma1;
        }
      }
    }
    if (full) {
      for (int ig = 1; ig <= 3; ++ig)
        for (int i = -2; i <= nx + 3; ++i)
          for (int c = 0; c < 4; ++c) U(u, c, i, 1 - ig) = U(u, c, i, 1);
    } else {
      for (int j = 1; j <= 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) {
          for (int c = 0; c < 4; ++c) U(u, c, i, 1 - j) = U(u, c, i, j);
          U(u, 2, i, 1 - j) = -U(u, 2, i, j);
        }
    }
    for (int ig = 1; ig <= 3; ++ig)
      for (int j = -2; j <= ny + 3; ++j)
        for (int c = 0; c < 4; ++c) U(u, c, nx + ig, j) = U(u, c, nx, j);
    for (int ig = 1; ig <= 3; ++ig)
      for (int i = -2; i <= nx + 3; ++i)
        for (int c = 0; c < 4; ++c) U(u, c, i, ny + ig) = U(u, c, i, ny);
  }
}

/* ------------------------------------------------------------------ */
/* 2D sweeping post-process                                             */
/* ------------------------------------------------------------------ */
/* sweeping_order (ex3_vortex_accuracy_2d/main.f90:1211-1270) */
static void sweeping_order(oracle* o) {
  const int nx = o->nx, ny = o->ny;
  int k = 0;
  for (int j = 1; j <= ny; ++j) {
    if (j % 2 == 1)
      for (int i = 1; i <= nx; ++i) { o->sI_i[k] = i; o->sI_j[k] = j; ++k; }
    else
      for (int i = nx; i >= 1; --i) { o->sI_i[k] = i; o->sI_j[k] = j; ++k; }
  }
  k = 0;
  for (int i = 1; i <= nx; ++i) {
    if (i % 2 == 1)
      for (int j = 1; j <= ny; ++j) { o->sII_i[k] = i; o->sII_j[k] = j; ++k; }
    else
      for (int j = ny; j >= 1; --j) { o->sII_i[k] = i; o->sII_j[k] = j; ++k; }
  }
}

static inline double pres2d_sweep(double g1, const double* v) {
  return g1 * (v[3] - 0.5 * (v[1] * v[1] + v[2] * v[2]) / (v[0]));
}

/* nod_lim (ex3_vortex_accuracy_2d/main.f90:846-884) */
static void nod_lim2d(oracle* o, const double* v1, const double* v2, const double* vb,
                      double* out) {
  const double g1 = o->gamma1, eps = o->eps;
  double p1 = g1 * (v1[3] - 0.5 * (v1[1] * v1[1] + v1[2] * v1[2]) / v1[0]);
  double p2 = g1 * (v2[3] - 0.5 * (v2[1] * v2[1] + v2[2] * v2[2]) / v2[0]);
  double t;
  if (p2 > eps) {
    t = (p1 - eps) / (p1 - p2);
    o->t_pos_count++;
  } else {
    double pb = g1 * (vb[3] - 0.5 * (vb[1] * vb[1] + vb[2] * vb[2]) / vb[0]);
    double t_1 = (p1 - eps) / (p1 - pb);
    double d12 = sqrt(sq(v2[3] - v1[3]) + sq(v2[2] - v1[2]) + sq(v2[1] - v1[1]) + sq(v2[0] - v1[0]));
    double d1b = sqrt(sq(vb[3] - v1[3]) + sq(vb[2] - v1[2]) + sq(vb[1] - v1[1]) + sq(vb[0] - v1[0]));
    t = fmin(t_1 * d1b / d12, 0.25);
    o->t_neg_count++;
  }
  for (int c = 0; c < 4; ++c) out[c] = (1 - t) * v1[c] + t * v2[c];
}

static void track_push(oracle* o) {
  if (o->sweep_count > o->track_cap) {
    int64_t cap = o->track_cap ? 2 * o->track_cap : 1024;
    o->sweep_track = realloc(o->sweep_track, cap * sizeof(int32_t));
    o->neg_track = realloc(o->neg_track, cap * sizeof(int32_t));
    o->pos_track = realloc(o->pos_track, cap * sizeof(int32_t));
    for (int64_t k = o->track_cap; k < cap; ++k)
      o->sweep_track[k] = o->neg_track[k] = o->pos_track[k] = 0;
    o->track_cap = cap;
  }
}

/* scalar_sweep (ex3_vortex_accuracy_2d/main.f90:1140-1209) */
static void scalar_sweep2d(oracle* o) {
  const int nx = o->nx, ny = o->ny, N = nx * ny;
  double rho_min = 1e20;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) rho_min = fmin(U(o->u, 0, i, j), rho_min);
  const double delta = 1e-12;
  if (rho_min < delta) {
    double* rt = o->rho_t; /* rho_t(i,j), i fastest */
#define RT(i, j) rt[(size_t)((i)-1) + (size_t)nx * (size_t)((j)-1)]
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) RT(i, j) = U(o->u, 0, i, j);
    const double w = o->weight;
    for (int k = 0; k < N - 1; ++k) {
      double v_i = RT(o->sI_i[k], o->sI_j[k]);
      double v_ip1 = RT(o->sI_i[k + 1], o->sI_j[k + 1]);
      if (v_i < delta) {
        RT(o->sI_i[k + 1], o->sI_j[k + 1]) = v_ip1 + (w / w) * (v_i - delta);
        RT(o->sI_i[k], o->sI_j[k]) = delta;
      }
    }
    for (int k = N - 1; k >= 1; --k) {
      double v_i = RT(o->sI_i[k], o->sI_j[k]);
      double v_im1 = RT(o->sI_i[k - 1], o->sI_j[k - 1]);
      if (v_i < delta) {
        RT(o->sI_i[k - 1], o->sI_j[k - 1]) = v_im1 + (w / w) * (v_i - delta);
        RT(o->sI_i[k], o->sI_j[k]) = delta;
      }
    }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) U(o->u, 0, i, j) = RT(i, j);
#undef RT
    o->den_count++;
  }
}

/* one forward or backward pass along an ordering
 * (ex3_vortex_accuracy_2d/main.f90:939-1016 ordering I, :1023-1104 ordering II) */
static int pressure_pass2d(oracle* o, const int* oi, const int* oj, int N, int forward,
                           const double* ubar, int check) {
  const double g1 = o->gamma1, eps = o->eps, w = o->weight;
  int k0 = forward ? 0 : N - 1, k1 = forward ? N - 1 : 0, dk = forward ? 1 : -1;
  for (int k = k0; k != k1; k += dk) {
    double vi[4], vp[4], vit[4], d[4], vpt[4];
    for (int c = 0; c < 4; ++c) vi[c] = U(o->u, c, oi[k], oj[k]);
    double pres_v_i = pres2d_sweep(g1, vi);
    if (pres_v_i <= eps || vi[0] <= eps) {
      for (int c = 0; c < 4; ++c) vp[c] = U(o->u, c, oi[k + dk], oj[k + dk]);
      nod_lim2d(o, vi, vp, ubar, vit);
      for (int c = 0; c < 4; ++c) d[c] = vi[c] - vit[c];
      for (int c = 0; c < 4; ++c) {
        vpt[c] = vp[c] + (w / w) * (d[c]);
        U(o->u, c, oi[k], oj[k]) = vit[c];
        U(o->u, c, oi[k + dk], oj[k + dk]) = vpt[c];
      }
      /* ex6: total pressure must not increase (ex6_shock_diffraction/main.f90:1413-1423,
       * active in the ordering-I passes) */
      if (check) {
        double pres_v_p = pres2d_sweep(g1, vp);
        double pres_v_i_t = pres2d_sweep(g1, vit);
        double pres_v_p_t = pres2d_sweep(g1, vpt);
        if (pres_v_i + pres_v_p > pres_v_i_t + pres_v_p_t + eps) return SWFD_ERR_SWEEP_CHECK;
      }
    }
  }
  return SWFD_OK;
}

/* sweep_lim (ex3_vortex_accuracy_2d/main.f90:888-1137; P(u_bar) check and
 * stop-on-failure of ex4_sedov_2d/main.f90:1447-1454,1747-1752; `>=` exit
 * test of ex5_mach2000_jet/main.f90:1162) */
static int sweep_lim2d(oracle* o) {
  const int nx = o->nx, ny = o->ny, N = nx * ny;
  scalar_sweep2d(o);
  double ra = 0.0, m1a = 0.0, m2a = 0.0, ea = 0.0;
  const double w = o->weight;
  if (o->cfg.ubar_mode == SWFD_UBAR_TREE) {
    /* not used by the oracle: the oracle is always sequential */
  }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      ra = ra + w * U(o->u, 0, i, j);
      m1a = m1a + w * U(o->u, 1, i, j);
      m2a = m2a + w * U(o->u, 2, i, j);
      ea = ea + w * U(o->u, 3, i, j);
    }
  double ubar[4] = {ra, m1a, m2a, ea};
  if (o->ex4like) {
    if (o->gamma1 * (ubar[3] - 0.5 * (ubar[1] * ubar[1] + ubar[2] * ubar[2]) / ubar[0]) <= 0.)
      return SWFD_ERR_PUBAR_NONPOS;
  }
  o->sweep_count++;
  track_push(o);
  o->t_pos_count = 0;
  o->t_neg_count = 0;
  const int ge = (o->problem == SWFD_PROBLEM_JET_2D);
  for (int q = 1; q <= o->cfg.swp_num; ++q) {
    const int* oi = (q % 2 == 1) ? o->sI_i : o->sII_i;
    const int* oj = (q % 2 == 1) ? o->sI_j : o->sII_j;
    const int check = o->problem == SWFD_PROBLEM_SHOCK_DIFFRACTION && (q % 2 == 1);
    int st = pressure_pass2d(o, oi, oj, N, 1, ubar, check);
    if (st == SWFD_OK) st = pressure_pass2d(o, oi, oj, N, 0, ubar, check);
    if (st != SWFD_OK) return st;
    double rho_min = 1e20, p_min = 1e20;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double v[4];
        for (int c = 0; c < 4; ++c) v[c] = U(o->u, c, i, j);
        p_min = fmin(o->gamma1 * (v[3] - 0.5 * (v[1] * v[1] + v[2] * v[2]) / v[0]), p_min);
        rho_min = fmin(v[0], rho_min);
      }
    o->pre_count++;
    int ok = ge ? (p_min >= o->eps && rho_min >= o->eps) : (p_min > o->eps && rho_min > o->eps);
    if (ok) {
      o->sweep_track[o->sweep_count - 1] = q;
      o->neg_track[o->sweep_count - 1] = (int32_t)o->t_neg_count;
      o->pos_track[o->sweep_count - 1] = (int32_t)o->t_pos_count;
      break;
    }
    if (q == o->cfg.swp_num) {
      o->fail_count++;
      if (o->ex4like) return SWFD_ERR_SWEEP_NOCONV;
    }
  }
  return SWFD_OK;
}

/* ------------------------------------------------------------------ */
/* 1D (ex2_sedov_1d/main.f90, built with -fdefault-real-8)              */
/* ------------------------------------------------------------------ */
#define U1(a, c, i) ((a)[(size_t)(c) + 3 * (size_t)((i) + 2)])

/* fflux (ex2_sedov_1d/main.f90:57-73) */
static void fflux1d(const oracle* o, double rho, double mx, double e, double* f) {
  double vx = 0.0; /* the reference leaves vx undefined only for NaN rho */
  if (gt_lit_1em8(o, rho)) vx = mx / rho;
  if (le_lit_1em8(o, rho)) vx = 0.;
  double pres = o->gamma1 * (e - 0.5 * rho * (vx * vx));
  f[0] = mx;
  f[1] = rho * (vx * vx) + pres;
  f[2] = (e + pres) * vx;
}

/* findalpha (ex2_sedov_1d/main.f90:273-285) */
static void findalpha1d(oracle* o) {
  double am = 0.0;
  for (int i = -2; i <= o->nx + 3; ++i) {
    double den = U1(o->u, 0, i);
    double pres = o->gamma1 * (U1(o->u, 2, i) - U1(o->u, 1, i) * U1(o->u, 1, i) / U1(o->u, 0, i) / 2.);
    double sound = sqrt(o->gamma * pres / den);
    am = fmax(am, fabs(U1(o->u, 1, i) / U1(o->u, 0, i)) + sound);
  }
  o->alphamax = am;
}

/* use_limiter = 1 in ex2 (ex2_sedov_1d/main.f90:159-245): the positivity
 * limiter of one split flux of cell m, with three components.  ave: the split
 * flux at cell m (hp(:, m) or hn(:, m)); out: its reconstructed flux
 * (hp_flux(:, m) or hn_flux(:, m)), limited in place. */
static void zs_limit1d(oracle* o, const double* ave, double* out) {
  const double g1 = o->gamma1;
  const double d_ave = ave[0], m_ave = ave[1], e_ave = ave[2];
  const double p_ave = g1 * (e_ave - 0.5 * (m_ave * m_ave) / d_ave);
  double point[2][3];
  double theta = 1.0;
  for (int c = 0; c < 3; ++c) {
    point[0][c] = out[c];
    point[1][c] = (ave[c] - out[c] / 12.) / (11. / 12.);
  }
  for (int ig = 0; ig < 2; ++ig) {
    double d_l = point[ig][0];
    if (d_l < 0.) theta = fmin(theta, fabs(d_ave - 0.) / fabs(d_ave - d_l));
  }
  if (theta < 1.) {
    out[0] = theta * out[0] + (1. - theta) * d_ave;
    o->den_count++;
  }
  theta = 1.;
  point[0][0] = out[0];
  point[1][0] = (ave[0] - out[0] / 12.) / (11. / 12.);
  for (int ig = 0; ig < 2; ++ig) {
    double d_l = point[ig][0], m_l = point[ig][1], e_l = point[ig][2];
    double p_l = g1 * (e_l - (m_l * m_l) / d_l / 2.);
    if (p_l < 0.) theta = fmin(theta, fabs(p_ave - 0.) / fabs(p_ave - p_l));
  }
  if (theta < 1.) {
    o->pre_count++;
    for (int c = 0; c < 3; ++c) out[c] = theta * out[c] + (1. - theta) * ave[c];
  }
}

/* wenofd (ex2_sedov_1d/main.f90:75-250): eigenvectors at cell m */
static void wenofd1d(oracle* o) {
  const int n = o->nx;
  findalpha1d(o);
  const double am = o->alphamax, g1 = o->gamma1;
  for (int i = -2; i <= n + 3; ++i) {
    double f[3];
    fflux1d(o, U1(o->u, 0, i), U1(o->u, 1, i), U1(o->u, 2, i), f);
    for (int c = 0; c < 3; ++c) {
      U1(o->fp, c, i) = 0.5 * (U1(o->u, c, i) + f[c] / am);
      U1(o->fn, c, i) = 0.5 * (U1(o->u, c, i) - f[c] / am);
    }
  }
  for (int m = 0; m <= n + 1; ++m) {
    double evr[3][3], evl[3][3], cu_p[3][5], cu_n[3][5], ur[3], ul[3];
    double u1 = U1(o->u, 0, m), u2 = U1(o->u, 1, m), u3 = U1(o->u, 2, m);
    double vxm = u2 / u1;
    double hm = (g1 * (u3 - 0.5 * (u2 * u2) / u1) + u3) / u1;
    double qm = 0.5 * vxm * vxm;
    double cm = sqrt(g1 * (hm - qm));
    double t0 = vxm * cm;
    evr[0][0] = 1.0; evr[0][1] = 1.0; evr[0][2] = 1.0;
    evr[1][0] = vxm - cm; evr[1][1] = vxm; evr[1][2] = vxm + cm;
    evr[2][0] = hm - t0; evr[2][1] = qm; evr[2][2] = hm + t0;
    double rcm = 1. / cm;
    double b1 = g1 * rcm * rcm;
    double b2 = qm * b1;
    t0 = vxm * rcm;
    double t1 = b1 * vxm;
    double t2 = 0.5 * b1;
    evl[0][0] = 0.5 * (b2 + t0); evl[0][1] = -0.5 * (t1 + rcm); evl[0][2] = t2;
    evl[1][0] = 1. - b2;         evl[1][1] = t1;                evl[1][2] = -b1;
    evl[2][0] = 0.5 * (b2 - t0); evl[2][1] = -0.5 * (t1 - rcm); evl[2][2] = t2;
    for (int jj = 0; jj < 5; ++jj)
      for (int k = 0; k < 3; ++k) {
        int mm = m + jj - 2;
        cu_p[k][jj] = evl[k][0] * U1(o->fp, 0, mm) + evl[k][1] * U1(o->fp, 1, mm) +
                      evl[k][2] * U1(o->fp, 2, mm);
        cu_n[k][jj] = evl[k][0] * U1(o->fn, 0, mm) + evl[k][1] * U1(o->fn, 1, mm) +
                      evl[k][2] * U1(o->fn, 2, mm);
      }
    for (int kk = 0; kk < 3; ++kk) {
      ur[kk] = oracle_weno_right_impl(o, cu_p[kk]);
      ul[kk] = oracle_weno_left_impl(o, cu_n[kk]);
    }
    for (int k = 0; k < 3; ++k) {
      U1(o->fpf, k, m) = evr[k][0] * ur[0] + evr[k][1] * ur[1] + evr[k][2] * ur[2];
      U1(o->fnf, k, m) = evr[k][0] * ul[0] + evr[k][1] * ul[1] + evr[k][2] * ul[2];
    }
    if (o->cfg.use_limiter == 1) { /* :159-245, hp_flux then hn_flux */
      double a[3], b[3], op[3], on[3];
      for (int c = 0; c < 3; ++c) {
        a[c] = U1(o->fp, c, m);
        b[c] = U1(o->fn, c, m);
        op[c] = U1(o->fpf, c, m);
        on[c] = U1(o->fnf, c, m);
      }
      zs_limit1d(o, a, op);
      zs_limit1d(o, b, on);
      for (int c = 0; c < 3; ++c) {
        U1(o->fpf, c, m) = op[c];
        U1(o->fnf, c, m) = on[c];
      }
    }
  }
}

/* scheme (ex2_sedov_1d/main.f90:252-271) */
static void scheme1d(oracle* o) {
  const int n = o->nx;
  memset(o->rhs, 0, (size_t)3 * o->LI * sizeof(double));
  double* flus = o->gp; /* scratch: flus(:, 1:n+1) */
  for (int i = 1; i <= n + 1; ++i)
    for (int c = 0; c < 3; ++c)
      U1(flus, c, i) = o->alphamax * (U1(o->fpf, c, i - 1) - U1(o->fnf, c, i));
  for (int i = 1; i <= n; ++i)
    for (int c = 0; c < 3; ++c) U1(o->rhs, c, i) = -(U1(flus, c, i + 1) - U1(flus, c, i)) / o->dx;
}

/* checkpositivity (ex2_sedov_1d/main.f90:376-392) */
static int checkpositivity1d(const oracle* o) {
  int postag = 0;
  for (int m = 1; m <= o->nx; ++m) {
    if (U1(o->u, 0, m) <= o->eps) postag = 1;
    if (U1(o->u, 2, m) - U1(o->u, 1, m) * U1(o->u, 1, m) / U1(o->u, 0, m) / 2. <= o->eps) postag = 1;
  }
  return postag;
}

/* nod_lim (ex2_sedov_1d/main.f90:517-560) */
static void nod_lim1d(oracle* o, const double* v1, const double* v2, const double* vb,
                      double* out) {
  const double g1 = o->gamma1, eps = o->eps;
  double p1 = g1 * (v1[2] - 0.5 * (v1[1] * v1[1] / v1[0]));
  double p2 = g1 * (v2[2] - 0.5 * (v2[1] * v2[1] / v2[0]));
  double t;
  if (p2 > eps) {
    t = (p1 - eps) / (p1 - p2);
    o->t_pos_count++;
  } else {
    double pb = g1 * (vb[2] - 0.5 * (vb[1] * vb[1] / vb[0]));
    double t_1 = (p1 - eps) / (p1 - pb);
    double d12 = sqrt(sq(v2[2] - v1[2]) + sq(v2[1] - v1[1]) + sq(v2[0] - v1[0]));
    double d1b = sqrt(sq(vb[2] - v1[2]) + sq(vb[1] - v1[1]) + sq(vb[0] - v1[0]));
    t = fmin(t_1 * d1b / d12, 0.25);
    o->t_neg_count++;
  }
  for (int c = 0; c < 3; ++c) out[c] = (1 - t) * v1[c] + t * v2[c];
}

/* scalar_sweep (ex2_sedov_1d/main.f90:729-790): always, over -2..n+3 */
static void scalar_sweep1d(oracle* o) {
  const int n = o->nx;
  const double delta = 1e-13, w = o->weight;
  double* rt = o->rho_t; /* rho_t(-2:n+3) */
  for (int j = -2; j <= n + 3; ++j) rt[j + 2] = U1(o->u, 0, j);
  for (int j = -2; j <= n + 2; ++j) {
    double v_j = rt[j + 2], v_jp1 = rt[j + 3];
    if (v_j < delta) {
      rt[j + 3] = v_jp1 + (w / w) * (v_j - delta);
      rt[j + 2] = delta;
    }
  }
  for (int j = n + 3; j >= -1; --j) {
    double v_j = rt[j + 2], v_jm1 = rt[j + 1];
    if (v_j < delta) {
      rt[j + 1] = v_jm1 + (w / w) * (v_j - delta);
      rt[j + 2] = delta;
    }
  }
  for (int j = -2; j <= n + 3; ++j) U1(o->u, 0, j) = rt[j + 2];
  o->den_count++;
}

/* sweep_lim (ex2_sedov_1d/main.f90:564-726) */
static int sweep_lim1d(oracle* o) {
  const int n = o->nx;
  const double g1 = o->gamma1, eps = o->eps, w = o->weight;
  scalar_sweep1d(o);
  double ra = 0.0, ma = 0.0, ea = 0.0; /* dot_product(., weights), in index order */
  for (int i = -2; i <= n + 3; ++i) ra = ra + U1(o->u, 0, i) * w;
  for (int i = -2; i <= n + 3; ++i) ma = ma + U1(o->u, 1, i) * w;
  for (int i = -2; i <= n + 3; ++i) ea = ea + U1(o->u, 2, i) * w;
  double ubar[3] = {ra, ma, ea};
  o->sweep_count++;
  track_push(o);
  o->t_pos_count = 0;
  o->t_neg_count = 0;
  for (int q = 1; q <= o->cfg.swp_num; ++q) {
    for (int j = -2; j <= n + 2; ++j) {
      double vj[3], vp[3], vjt[3];
      for (int c = 0; c < 3; ++c) vj[c] = U1(o->u, c, j);
      double pres_v_j = g1 * (vj[2] - 0.5 * (vj[1] * vj[1]) / vj[0]);
      if (pres_v_j <= eps || vj[0] <= eps) {
        for (int c = 0; c < 3; ++c) vp[c] = U1(o->u, c, j + 1);
        nod_lim1d(o, vj, vp, ubar, vjt);
        for (int c = 0; c < 3; ++c) {
          double d = vj[c] - vjt[c];
          U1(o->u, c, j) = vjt[c];
          U1(o->u, c, j + 1) = vp[c] + (w / w) * (d);
        }
      }
    }
    for (int j = n + 3; j >= -1; --j) {
      double vj[3], vp[3], vjt[3];
      for (int c = 0; c < 3; ++c) vj[c] = U1(o->u, c, j);
      double pres_v_j = g1 * (vj[2] - 0.5 * (vj[1] * vj[1]) / vj[0]);
      if (pres_v_j <= eps || vj[0] <= eps) {
        for (int c = 0; c < 3; ++c) vp[c] = U1(o->u, c, j - 1);
        nod_lim1d(o, vj, vp, ubar, vjt);
        for (int c = 0; c < 3; ++c) {
          double d = vj[c] - vjt[c];
          U1(o->u, c, j) = vjt[c];
          U1(o->u, c, j - 1) = vp[c] + (w / w) * (d);
        }
      }
    }
    double rho_min = 1e20, p_min = 1e20;
    for (int i = -2; i <= n + 3; ++i) {
      double u1 = U1(o->u, 0, i), u2 = U1(o->u, 1, i), u3 = U1(o->u, 2, i);
      p_min = fmin(g1 * (u3 - 0.5 * (u2 * u2) / u1), p_min);
      rho_min = fmin(u1, rho_min);
    }
    o->pre_count++;
    if (p_min > eps && rho_min > eps) {
      o->sweep_track[o->sweep_count - 1] = q;
      o->neg_track[o->sweep_count - 1] = (int32_t)o->t_neg_count;
      o->pos_track[o->sweep_count - 1] = (int32_t)o->t_pos_count;
      break;
    }
    if (q == o->cfg.swp_num) o->fail_count++; /* ex2 records nothing */
  }
  return SWFD_OK;
}

/* ------------------------------------------------------------------ */
/* ex1: the MATLAB script ex1_double_rarefaction_1d/FD_WENO_Application.m */
/* with its helpers (get_variables.m, get_pressure_data.m, scalar_pos.m, */
/* apply_sweep.m, swp_alg_triag_nxt.m, node_adj_scale_lim_triag.m).     */
/* MATLAB evaluates its operators left to right with the precedence of  */
/* its documentation (unary minus before * and /); x.^2 is taken as x*x, */
/* a row times a column (the weighted means) as a left-to-right sum and  */
/* a 3x3 matrix times a vector row by row left to right.  MATLAB itself  */
/* is not available, so these choices are not pinned against its output. */
/* The script keeps no ghost cells: o->u's interior 1..n is its u(:,1:n) */
/* and the ghosts hold the padding FD_WENO_Step would build from it.     */
/* ------------------------------------------------------------------ */
static int ex1_periodic(const oracle* o) {
  const int pr = o->cfg.variant; /* FD_WENO_Application.m:27-150 */
  return pr == 1 || pr == 2 || pr == 6;
}

/* the padding of FD_WENO_Step (:394-411): wrap or constant extension */
static void ex1_pad(const oracle* o, const double* u, double* pad, int ldp) {
  const int n = o->nx, per = ex1_periodic(o);
  for (int J = 1; J <= n + 6; ++J) {
    int i;
    if (J <= 3) i = per ? n - 3 + J : 1;
    else if (J > n + 3) i = per ? J - n - 3 : n;
    else i = J - 3;
    for (int c = 0; c < 3; ++c) pad[c * ldp + J] = u[c + 3 * (i + 2)];
  }
}

/* scalarWeno (:588-629): out[0] the value at the right face from the left
 * (umOut), out[1] the value at the left face of cell 4 from the right (upOut) */
static void ex1_scalar_weno(const double* s, double* um_out, double* up_out) {
  const double umm = s[0], um = s[1], u = s[2], up = s[3], upp = s[4], uppp = s[5];
  const double c13 = 1. / 3., c76 = 7. / 6., c116 = 11. / 6., c16 = 1. / 6., c56 = 5. / 6.;
  const double c1312 = 13. / 12., c14 = 1. / 4., eps = 10e-6;
  const double cw1 = 1. / 10., cw2 = 3. / 5., cw3 = 3. / 10.;
  double um1 = c13 * umm - c76 * um + c116 * u;
  double um2 = -c16 * um + c56 * u + c13 * up;
  double um3 = c13 * u + c56 * up - c16 * upp;
  double b1 = c1312 * sq(umm - 2 * um + u) + c14 * sq(umm - 4 * um + 3 * u);
  double b2 = c1312 * sq(um - 2 * u + up) + c14 * sq(um - up);
  double b3 = c1312 * sq(u - 2 * up + upp) + c14 * sq(3 * u - 4 * up + upp);
  double w1 = cw1 / sq(b1 + eps), w2 = cw2 / sq(b2 + eps), w3 = cw3 / sq(b3 + eps);
  double sw = w1 + w2 + w3;
  *um_out = w1 / sw * um1 + w2 / sw * um2 + w3 / sw * um3;
  double up1 = c116 * up - c76 * upp + c13 * uppp;
  double up2 = c13 * u + c56 * up - c16 * upp;
  double up3 = -c16 * um + c56 * u + c13 * up;
  b1 = c1312 * sq(uppp - 2 * upp + up) + c14 * sq(uppp - 4 * upp + 3 * up);
  b2 = c1312 * sq(upp - 2 * up + u) + c14 * sq(upp - u);
  b3 = c1312 * sq(up - 2 * u + um) + c14 * sq(3 * up - 4 * u + um);
  w1 = cw1 / sq(b1 + eps), w2 = cw2 / sq(b2 + eps), w3 = cw3 / sq(b3 + eps);
  sw = w1 + w2 + w3;
  *up_out = w1 / sw * up1 + w2 / sw * up2 + w3 / sw * up3;
}

/* FD_WENO_Step (:392-585): fP(:,k) the flux at the right face of cell k,
 * fM(:,k) at its left face; u is the interior state (3 x n, ghosts unused) */
static void ex1_fluxes(const oracle* o, const double* u, double* fP, double* fM) {
  const int n = o->nx, N = n + 6, L = N + 1, per = ex1_periodic(o);
  const double g1 = o->gamma - 1;
  double* pad = malloc(3 * L * sizeof(double));
  double* ar = malloc(12 * L * sizeof(double));
  double *ro = ar, *m = ar + L, *E = ar + 2 * L, *v = ar + 3 * L, *p = ar + 4 * L,
         *H1 = ar + 5 * L, *vxm = ar + 6 * L, *hxm = ar + 7 * L, *qm = ar + 8 * L,
         *cm = ar + 9 * L, *t2 = ar + 10 * L, *sr = ar + 11 * L;
  /* get_variables (get_variables.m), then the padding */
  double* iv = malloc(5 * L * sizeof(double));
  for (int i = 1; i <= n; ++i) {
    const double r = u[0 + 3 * (i + 2)], mm = u[1 + 3 * (i + 2)], e = u[2 + 3 * (i + 2)];
    iv[i] = r, iv[L + i] = mm, iv[2 * L + i] = e;
    iv[3 * L + i] = mm / r;
    iv[4 * L + i] = g1 * (e - 1. / 2. * (mm * mm) / r);
  }
  for (int J = 1; J <= N; ++J) {
    int i;
    if (J <= 3) i = per ? n - 3 + J : 1;
    else if (J > n + 3) i = per ? J - n - 3 : n;
    else i = J - 3;
    ro[J] = iv[i], m[J] = iv[L + i], E[J] = iv[2 * L + i], v[J] = iv[3 * L + i];
    p[J] = iv[4 * L + i];
  }
  free(iv);
  for (int J = 1; J <= N; ++J) {
    sr[J] = sqrt(ro[J]);
    H1[J] = (p[J] + E[J]) / ro[J];
  }
  /* Roe averages at J+1/2 (circshift wraps the last), per-field alpha */
  double a1 = 0, a2 = 0, a3 = 0;
  for (int J = 1; J <= N; ++J) {
    const int Jn = J == N ? 1 : J + 1;
    const double t0 = sr[J] / (sr[J] + sr[Jn]);
    const double t1 = 1 - t0;
    vxm[J] = t0 * v[J] + t1 * v[Jn];
    hxm[J] = t0 * H1[J] + t1 * H1[Jn];
    qm[J] = 0.5 * (vxm[J] * vxm[J]);
    cm[J] = sqrt(g1 * (hxm[J] - qm[J]));
    t2[J] = vxm[J] * cm[J];
    const double l1 = fabs(vxm[J] - cm[J]), l2 = fabs(vxm[J]), l3 = fabs(vxm[J] + cm[J]);
    if (J == 1) a1 = l1, a2 = l2, a3 = l3;
    else a1 = fmax(a1, l1), a2 = fmax(a2, l2), a3 = fmax(a3, l3);
  }
  const double al[3] = {a1, a2, a3};
  /* the flux at interface J+1/2 from cells J-2..J+3 (:445-517) */
  for (int kk = 0; kk <= n; ++kk) {
    const int J = kk + 3;
    if (kk == 0 && per) continue;
    const double V = vxm[J], H = hxm[J], q = qm[J], c = cm[J], T2 = t2[J];
    const double rcm = 1 / c;
    const double b1 = g1 * (rcm * rcm), b2 = q * b1, t0h = V * rcm, t1h = b1 * V, t2h = 0.5 * b1;
    const double Lm[3][3] = {{0.5 * (b2 + t0h), -0.5 * (t1h + rcm), t2h},
                             {1 - b2, t1h, -b1},
                             {0.5 * (b2 - t0h), -0.5 * (t1h - rcm), t2h}};
    double gp[3][6], gm[3][6];
    for (int idx = 0; idx < 6; ++idx) {
      const int i = J - 2 + idx;
      const double uu[3] = {ro[i], m[i], E[i]};
      const double fu[3] = {m[i], ro[i] * (v[i] * v[i]) + p[i], v[i] * (E[i] + p[i])};
      for (int r = 0; r < 3; ++r) {
        const double w = Lm[r][0] * uu[0] + Lm[r][1] * uu[1] + Lm[r][2] * uu[2];
        const double g = Lm[r][0] * fu[0] + Lm[r][1] * fu[1] + Lm[r][2] * fu[2];
        gp[r][idx] = 1. / 2. * (g + al[r] * w);
        gm[r][idx] = 1. / 2. * (g - al[r] * w);
      }
    }
    double gh[3];
    for (int r = 0; r < 3; ++r) {
      double um_p, up_p, um_m, up_m;
      ex1_scalar_weno(gm[r], &um_m, &up_m);
      ex1_scalar_weno(gp[r], &um_p, &up_p);
      gh[r] = up_m + um_p;
    }
    double f[3];
    f[0] = 1 * gh[0] + 1 * gh[1] + 1 * gh[2];
    f[1] = (V - c) * gh[0] + V * gh[1] + (V + c) * gh[2];
    f[2] = (H - T2) * gh[0] + q * gh[1] + (H + T2) * gh[2];
    for (int r = 0; r < 3; ++r) {
      if (kk >= 1) fP[r + 3 * (kk - 1)] = f[r];
      if (kk == 0) fM[r] = f[r];
    }
  }
  for (int k = 1; k <= n; ++k)
    for (int r = 0; r < 3; ++r) {
      if (k >= 2) fM[r + 3 * (k - 1)] = fP[r + 3 * (k - 2)];
      else if (per) fM[r] = fP[r + 3 * (n - 1)];
    }
  free(pad);
  free(ar);
}

/* get_pressure_data.m: min of P = E - m^2/rho/2 and P of the weighted mean */
static void ex1_pressure_data(const oracle* o, const double* u, double* pmin, double* pu_avg) {
  const int n = o->nx;
  const double w = o->weight;
  double ra = 0, ma = 0, ea = 0, mn = 0;
  for (int i = 1; i <= n; ++i) {
    const double* x = u + 3 * (i + 2);
    const double P = x[2] - 1. / 2. * ((x[1] * x[1]) / x[0]);
    mn = (i == 1) ? P : fmin(mn, P);
    ra = ra + x[0] * w, ma = ma + x[1] * w, ea = ea + x[2] * w;
  }
  *pmin = mn;
  *pu_avg = ea - 1. / 2. * ((ma * ma) / ra);
}

/* scalar_pos.m: the density sweep, forward then backward, floor m = 1e-16 */
static void ex1_scalar_pos(oracle* o, double* u) {
  const int n = o->nx;
  const double m = 1e-16, w = o->weight;
  for (int j = 1; j <= n - 1; ++j) {
    const double vj = u[3 * (j + 2)], vp = u[3 * (j + 3)];
    if (vj < m) {
      u[3 * (j + 3)] = vp + (w / w) * (vj - m);
      u[3 * (j + 2)] = m;
    }
  }
  for (int j = n; j >= 2; --j) {
    const double vj = u[3 * (j + 2)], vp = u[3 * (j + 1)];
    if (vj < m) {
      u[3 * (j + 1)] = vp + (w / w) * (vj - m);
      u[3 * (j + 2)] = m;
    }
  }
  o->den_count++;
}

/* the pressure of the sweep functions, with their own gamma = 1.4 */
static double ex1_P14(const double* x) { return (1.4 - 1) * (x[2] - 1. / 2. * ((x[1] * x[1]) / x[0])); }

/* node_adj_scale_lim_triag.m */
static void ex1_node_adj(oracle* o, const double* v1, const double* v2, const double* vb,
                         double* out) {
  const double epsi = 1e-13;
  double t;
  if (ex1_P14(v2) > epsi) {
    t = (ex1_P14(v1) - epsi) / (ex1_P14(v1) - ex1_P14(v2));
    o->t_pos_count++;
  } else {
    const double t1 = (ex1_P14(v1) - epsi) / (ex1_P14(v1) - ex1_P14(vb));
    const double d1 = sqrt(sq(vb[2] - v1[2]) + sq(vb[1] - v1[1]) + sq(vb[0] - v1[0]));
    const double d2 = sqrt(sq(v2[2] - v1[2]) + sq(v2[1] - v1[1]) + sq(v2[0] - v1[0]));
    t = fmin(t1 * d1 / d2, 0.25);
    o->t_neg_count++;
  }
  for (int c = 0; c < 3; ++c) out[c] = (1 - t) * v1[c] + t * v2[c];
}

/* swp_alg_triag_nxt.m */
static void ex1_swp_alg(oracle* o, double* u) {
  const int n = o->nx;
  const double w = o->weight, epsi = 1e-12;
  double ub[3] = {0, 0, 0};
  for (int c = 0; c < 3; ++c)
    for (int i = 1; i <= n; ++i) ub[c] = ub[c] + u[c + 3 * (i + 2)] * w;
  o->sweep_count++;
  track_push(o);
  o->t_pos_count = o->t_neg_count = 0;
  int q;
  for (q = 1; q <= o->cfg.swp_num; ++q) {
    for (int pass = 0; pass < 2; ++pass)
      for (int s = 1; s <= n - 1; ++s) {
        const int j = pass == 0 ? s : n - s + 1, jp = pass == 0 ? j + 1 : j - 1;
        double* vj = u + 3 * (j + 2);
        double* vp = u + 3 * (jp + 2);
        if (ex1_P14(vj) <= epsi || vj[0] < 0) {
          double vjt[3], a[3], b[3];
          for (int c = 0; c < 3; ++c) a[c] = vj[c], b[c] = vp[c];
          ex1_node_adj(o, a, b, ub, vjt);
          for (int c = 0; c < 3; ++c) {
            const double d = a[c] - vjt[c];
            vj[c] = vjt[c];
            vp[c] = b[c] + (w / w) * d;
          }
        }
      }
    o->pre_count++;
    double pmin, pu;
    ex1_pressure_data(o, u, &pmin, &pu);
    double rmin = 0;
    for (int i = 1; i <= n; ++i) rmin = (i == 1) ? u[3 * (i + 2)] : fmin(rmin, u[3 * (i + 2)]);
    if (pmin > epsi && rmin > epsi) break;
  }
  if (q > o->cfg.swp_num) {
    q = o->cfg.swp_num;
    o->fail_count++;
  }
  o->sweep_track[o->sweep_count - 1] = q;
  o->neg_track[o->sweep_count - 1] = (int32_t)o->t_neg_count;
  o->pos_track[o->sweep_count - 1] = (int32_t)o->t_pos_count;
}

/* apply_sweep.m */
static void ex1_apply_sweep(oracle* o, double* u) {
  const int n = o->nx;
  double rmin = 0;
  for (int i = 1; i <= n; ++i) rmin = (i == 1) ? u[3 * (i + 2)] : fmin(rmin, u[3 * (i + 2)]);
  if (rmin <= 1e-13) ex1_scalar_pos(o, u);
  double pmin, pu;
  ex1_pressure_data(o, u, &pmin, &pu);
  if (pmin <= 1e-13 && pu > 0) {
    ex1_scalar_pos(o, u);
    ex1_pressure_data(o, u, &pmin, &pu);
    if (pu > 1e-13) ex1_swp_alg(o, u);
  }
}

/* one pass of the script's time loop (:212-289) */
static int ex1_step(oracle* o) {
  const int n = o->nx, ln = 3 * (n + 6);
  const double g = o->gamma, g1 = g - 1, h = o->dx;
  double* u = o->u;
  /* eigenvalues of the cell states and the time step (:217-252) */
  double a1 = 0, a2 = 0, a3 = 0;
  for (int i = 1; i <= n; ++i) {
    const double ro = u[3 * (i + 2)], m = u[1 + 3 * (i + 2)], E = u[2 + 3 * (i + 2)];
    const double v = m / ro;
    const double p = E * g1 - 1. / 2. * ro * (v * v) * g1;
    const double c = sqrt((g * p) / ro);
    const double l1 = fabs(v - c), l2 = fabs(v), l3 = fabs(v + c);
    if (i == 1) a1 = l1, a2 = l2, a3 = l3;
    else a1 = fmax(a1, l1), a2 = fmax(a2, l2), a3 = fmax(a3, l3);
  }
  const double alpha = fmax(fmax(a1, a2), a3);
  o->alphamax = alpha;
  double k = o->cfg.cfl * h / alpha;
  if (o->cfg.time_terminal - o->time < k) k = o->cfg.time_terminal - o->time;
  const double l = k / h;
  o->dt = k;
  double* uh = calloc(ln, sizeof(double));
  double* fP = calloc(3 * n, sizeof(double));
  double* fM = calloc(3 * n, sizeof(double));
  const int sweeping = o->cfg.use_limiter == 2;
  for (int stage = 1; stage <= 3; ++stage) {
    ex1_fluxes(o, stage == 1 ? u : uh, fP, fM);
    for (int i = 1; i <= n; ++i)
      for (int c = 0; c < 3; ++c) {
        const size_t a = c + 3 * (size_t)(i + 2);
        const double d = l * (fP[c + 3 * (i - 1)] - fM[c + 3 * (i - 1)]);
        if (stage == 1) uh[a] = u[a] - d;
        else if (stage == 2) uh[a] = 3. / 4. * u[a] + 1. / 4. * (uh[a] - d);
        else uh[a] = 1. / 3. * u[a] + 2. / 3. * (uh[a] - d);
      }
    if (sweeping) ex1_apply_sweep(o, uh);
  }
  memcpy(u, uh, ln * sizeof(double));
  double* pad = malloc(3 * (n + 7) * sizeof(double));
  ex1_pad(o, u, pad, n + 7);
  for (int J = 1; J <= 3; ++J)
    for (int c = 0; c < 3; ++c) {
      u[c + 3 * (J - 1)] = pad[c * (n + 7) + J];                   /* cells -2..0 */
      u[c + 3 * (n + 2 + J)] = pad[c * (n + 7) + n + 3 + J];       /* cells n+1..n+3 */
    }
  free(pad);
  free(uh);
  free(fP);
  free(fM);
  o->time = o->time + k;
  return SWFD_OK;
}

/* initial data of the script's problems (:27-150, :188-205) on the cell
 * midpoints of xL:h:xR; MATLAB's colon builds the second half of its nodes
 * from the right end (a + n*d) */
static void ex1_init(oracle* o) {
  const int n = o->nx, pr = o->cfg.variant;
  const double g = o->gamma, pi = 3.141592653589793;
  double xl = 0, xr = 2 * pi;
  if (pr == 3) xl = -1, xr = 1;
  else if (pr == 4) xl = -5, xr = 5;
  else if (pr == 5) xl = -0.5, xr = 0.5;
  else if (pr == 6) xl = -3, xr = 3;
  else if (pr == 7) xl = -0.05, xr = 0.05;
  const double h = (xr - xl) / n;
  o->dx = h;
  const double hi = xl + n * h;
  for (int i = 1; i <= n; ++i) {
    const int k0 = i - 1, k1 = i;
    const double x0 = (2 * k0 <= n) ? xl + k0 * h : hi - (n - k0) * h;
    const double x1 = (2 * k1 <= n) ? xl + k1 * h : hi - (n - k1) * h;
    const double x = (x0 + x1) / 2;
    o->x[i + 2] = x;
    double ro = 0, v = 0, p = 0;
    const int i1 = x <= 0, i2 = x > 0;
    switch (pr) {
      case 1: ro = 1 + 0.2 * sin(x), v = 1, p = 1; break;
      case 2: ro = 1 + 1. / 2. * sin(x), v = 1. / 2. * sin(x), p = pow(1 + 1. / 2. * sin(x), g); break;
      case 3: ro = 0 + 1 * i1 + 0.125 * i2, v = 0, p = 0 + 1 * i1 + 0.1 * i2; break;
      case 4: ro = 0 + 0.445 * i1 + 0.5 * i2, v = 0 + 0.698 * i1 + 0 * i2,
              p = 0 + 3.528 * i1 + 0.571 * i2; break;
      case 5: ro = 0 + 7 * i1 + 7 * i2, v = 0 + -1 * i1 + 1 * i2, p = 0 + 0.2 * i1 + 0.2 * i2; break;
      case 6: {
        const int j1 = x >= (-2. / 402.), j2 = x > (2. / 402.);
        const double E0 = 0 + (3200000. * 201.) * j1 - (3200000. * 201.) * j2 + 1e-12 * 1;
        ro = 1, v = 0;
        p = (g - 1) * (E0 - 1. / 2. * ro * (v * v));
        break;
      }
      default: ro = 5, v = 0, p = 0.4127; break;
    }
    const double m = v * ro;
    const double E = p / (g - 1) + 1. / 2. * ro * (v * v);
    U1(o->u, 0, i) = ro, U1(o->u, 1, i) = m, U1(o->u, 2, i) = E;
  }
  o->weight = 1. * 1. / n; /* ones(1,nSteps)*1/nSteps */
  double* pad = malloc(3 * (n + 7) * sizeof(double));
  ex1_pad(o, o->u, pad, n + 7);
  for (int J = 1; J <= 3; ++J)
    for (int c = 0; c < 3; ++c) {
      o->u[c + 3 * (J - 1)] = pad[c * (n + 7) + J];
      o->u[c + 3 * (n + 2 + J)] = pad[c * (n + 7) + n + 3 + J];
    }
  free(pad);
}

/* ------------------------------------------------------------------ */
/* stage / step / loop                                                 */
/* ------------------------------------------------------------------ */
static void wenofd_any(oracle* o) {
  if (o->ndim == 1) wenofd1d(o); else wenofd2d(o);
}
static void scheme_any(oracle* o) {
  if (o->ndim == 1) scheme1d(o); else scheme2d(o);
}
static int check_any(oracle* o) { return o->ndim == 1 ? checkpositivity1d(o) : checkpositivity2d(o); }
static int sweep_any(oracle* o) { return o->ndim == 1 ? sweep_lim1d(o) : sweep_lim2d(o); }
static void bc_any(oracle* o) {
  if (o->ndim == 2) bc2d(o); /* ex2's bc is empty (ex2_sedov_1d/main.f90:394-403) */
}

static size_t state_len(const oracle* o) { return (size_t)o->nc * o->LI * o->LJ; }

/* dt rule of the problem, evaluated right after the stage-1 wenofd
 * (ex2_sedov_1d/main.f90:293; ex3_vortex_accuracy_2d/main.f90:570-572;
 *  ex4_sedov_2d/main.f90:696-700; ex5_mach2000_jet/main.f90:597-605) */
static void compute_dt(oracle* o) {
  const double cfl = o->cfg.cfl, am = o->alphamax;
  switch (o->problem) {
    case SWFD_PROBLEM_SEDOV_1D: o->dt = o->dx * cfl / am; break;
    case SWFD_PROBLEM_VORTEX_2D: o->dt = pow(o->dx, 5. / 3.) * cfl / am; break;
    default: {
      double dtx = o->dx * cfl / am, dty = o->dy * cfl / am;
      double dtc = fmin(dtx, dty);
      o->dt = fmin(dtc, o->cfg.time_terminal - o->time);
    }
  }
}


/* ------------------------------------------------------------------ */
/* ex6: Mach 5.09 shock diffraction (ex6_shock_diffraction/main.f90).  */
/* The reference runs on cut_x x cut_y MPI ranks and its arithmetic    */
/* depends on that layout, so the oracle keeps one local grid per rank  */
/* (u(4,-2:nxl+3,-2:nyl+3) with its own ghost layers), exchanges ghosts */
/* as exchange_x/exchange_y do, gathers the interior for the sweep and  */
/* scatters it back.  o->u is the assembled global view.               */
/* ------------------------------------------------------------------ */
static oracle* ex6_rank_create(const oracle* g, int px, int py) {
  oracle* r = calloc(1, sizeof(oracle));
  r->cfg = g->cfg;
  r->problem = g->problem;
  r->quad = g->quad;
  r->ndim = 2;
  r->nc = g->nc;
  r->nx = g->nxl;
  r->ny = g->nyl;
  r->LI = r->nx + 6;
  r->LJ = r->ny + 6;
  r->gamma = g->gamma;
  r->gamma1 = g->gamma1;
  r->eps = g->eps;
  r->eps2 = g->eps2;
  r->weno_eps = g->weno_eps;
  r->weno_eps_q = g->weno_eps_q;
  r->ex4like = 1;
  r->px = px;
  r->py = py;
  r->total = g->total;
  r->dx = g->dx;
  r->dy = g->dy;
  const size_t n = state_len(r);
  double** arrs[] = {&r->u, &r->u0, &r->rhs, &r->fp, &r->fn, &r->gp,
                     &r->gn, &r->fpf, &r->fnf, &r->gpf, &r->gnf};
  for (size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); ++k) *arrs[k] = calloc(n, sizeof(double));
  r->alpha = calloc((size_t)r->LI * r->LJ, sizeof(double));
  int mx = (r->nx > r->ny ? r->nx : r->ny) + 3;
  r->wk_w = calloc(mx, sizeof(double));
  r->wk_vx = calloc(mx, sizeof(double));
  r->wk_vy = calloc(mx, sizeof(double));
  r->wk_h = calloc(mx, sizeof(double));
  r->wk_ratio = calloc(mx, sizeof(double));
  r->qc = g->qc;
  r->tc = g->tc;
  r->kc = g->kc;
  r->wall_rows = g->wall_rows;
  return r;
}

static void ex6_rank_destroy(oracle* r) {
  double* arrs[] = {r->u, r->u0, r->rhs, r->fp, r->fn, r->gp, r->gn, r->fpf, r->fnf, r->gpf, r->gnf,
                    r->alpha, r->wk_w, r->wk_vx, r->wk_vy, r->wk_h, r->wk_ratio};
  for (size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); ++k) free(arrs[k]);
  free(r);
}

#define UR(r, a, c, i, j) ((a)[IX((r), (c), (i), (j))])
#define ALPHA(r, i, j) ((r)->alpha[(size_t)((i) + 2) + (size_t)(r)->LI * (size_t)((j) + 2)])

/* the rank owning global cell (I, J); ghost cells belong to the edge ranks */
static int ex6_owner_x(const oracle* o, int I) {
  int px = I <= 0 ? 0 : (I - 1) / o->nxl;
  return px >= o->cut_x ? o->cut_x - 1 : px;
}
static int ex6_owner_y(const oracle* o, int J) {
  int py = J <= 0 ? 0 : (J - 1) / o->nyl;
  return py >= o->cut_y ? o->cut_y - 1 : py;
}

/* global view <- ranks: interior from the owners, ghosts from the edge ranks */
static void ex6_assemble(oracle* o) {
  for (int J = -2; J <= o->ny + 3; ++J)
    for (int I = -2; I <= o->nx + 3; ++I) {
      int px = ex6_owner_x(o, I), py = ex6_owner_y(o, J);
      const oracle* r = o->rk[px + o->cut_x * py];
      int i = I - px * o->nxl, j = J - py * o->nyl;
      for (int c = 0; c < o->nc; ++c) o->u[IX(o, c, I, J)] = r->u[IX(r, c, i, j)];
    }
}

/* ranks <- global view, every local cell including ghosts */
static void ex6_distribute(oracle* o) {
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    oracle* r = o->rk[k];
    for (int j = -2; j <= r->ny + 3; ++j)
      for (int i = -2; i <= r->nx + 3; ++i) {
        int I = r->px * o->nxl + i, J = r->py * o->nyl + j;
        for (int c = 0; c < o->nc; ++c) r->u[IX(r, c, i, j)] = o->u[IX(o, c, I, J)];
      }
  }
  o->ranks_stale = 0;
}

/* findalpha of one rank (ex6_shock_diffraction/main.f90:662-691): per-cell
 * alpha over the local cells including ghosts; returns the local max */
static double ex6_findalpha(oracle* r) {
  double am = 0.;
  for (int i = -2; i <= r->nx + 3; ++i)
    for (int j = -2; j <= r->ny + 3; ++j) {
      double u1 = UR(r, r->u, 0, i, j), u2 = UR(r, r->u, 1, i, j), u3 = UR(r, r->u, 2, i, j),
             u4 = UR(r, r->u, 3, i, j);
      double den = u1, vx, vy;
      if (den >= r->eps2) {
        vx = u2 / den;
        vy = u3 / den;
      } else {
        vx = 0.;
        vy = 0.;
      }
      double pres = r->gamma1 * (u4 - 0.5 * den * (vx * vx) - 0.5 * den * (vy * vy));
      double sound = sqrt(r->gamma * pres / den);
      double a = fmax(fabs(u2 / u1) + sound, fabs(u3 / u1) + sound);
      ALPHA(r, i, j) = a;
      am = fmax(am, a);
    }
  return am;
}

/* wenofd of one rank (ex6_shock_diffraction/main.f90:170-647): wall mirror
 * at column total for global rows <= 6*total (:191-201), per-row alpha over
 * the rank's local row (:218-224), fluxes scaled by it (:411-412); wall
 * mirror at row 6*total over columns 1..total (:416-430); per-column alpha
 * (:450-456) and scaling (:641-642) in the y pass */
static void ex6_wenofd(oracle* r) {
  const int nx = r->nx, ny = r->ny, total = r->total;
  for (int j = 0; j <= ny + 1; ++j) {
    if (r->px == 0 && r->py * ny + j <= total * 6)
      for (int i = 0; i <= 2; ++i) {
        for (int c = 0; c < 4; ++c) UR(r, r->u, c, total - i, j) = UR(r, r->u, c, total + 1 + i, j);
        UR(r, r->u, 1, total - i, j) = -UR(r, r->u, 1, total + 1 + i, j);
      }
    for (int i = 0; i <= nx + 2; ++i) {
      double a[4];
      for (int c = 0; c < 4; ++c) a[c] = UR(r, r->u, c, i, j);
      prep_cell(r, 0, a, &r->wk_w[i], &r->wk_vx[i], &r->wk_vy[i], &r->wk_h[i]);
    }
    double al = 0.;
    for (int i = -2; i <= nx + 3; ++i) al = fmax(al, ALPHA(r, i, j));
    for (int i = -2; i <= nx + 3; ++i) {
      double a[4], f[4];
      for (int c = 0; c < 4; ++c) a[c] = UR(r, r->u, c, i, j);
      fflux2d(r, a, f, 0);
      for (int c = 0; c < 4; ++c) {
        UR(r, r->fp, c, i, j) = 0.5 * (a[c] + f[c] / al);
        UR(r, r->fn, c, i, j) = 0.5 * (a[c] - f[c] / al);
      }
    }
    for (int i = 0; i <= nx + 1; ++i) {
      double sp[5][4], sn[5][4], op[4], on[4];
      for (int ig = 0; ig < 5; ++ig)
        for (int c = 0; c < 4; ++c) {
          sp[ig][c] = UR(r, r->fp, c, i + ig - 2, j);
          sn[ig][c] = UR(r, r->fn, c, i + ig - 2, j);
        }
      interface2d(r, 0, r->wk_w[i], r->wk_w[i + 1], r->wk_vx[i], r->wk_vx[i + 1], r->wk_vy[i],
                  r->wk_vy[i + 1], r->wk_h[i], r->wk_h[i + 1], (const double(*)[4])sp,
                  (const double(*)[4])sn, op, on);
      limit_interface(r, r->fp, r->fn, i, j, op, on);
      for (int c = 0; c < 4; ++c) {
        UR(r, r->fpf, c, i, j) = al * op[c];
        UR(r, r->fnf, c, i, j) = al * on[c];
      }
    }
  }
  if (r->px == 0)
    for (int j = -2; j <= ny + 3; ++j)
      if (r->py * ny + j == total * 6)
        for (int i = 0; i <= 2; ++i)
          for (int k = 1; k <= total; ++k) {
            for (int c = 0; c < 4; ++c) UR(r, r->u, c, k, j - i) = UR(r, r->u, c, k, j + 1 + i);
            UR(r, r->u, 2, k, j - i) = -UR(r, r->u, 2, k, j + 1 + i);
          }
  for (int i = 0; i <= nx + 1; ++i) {
    for (int j = 0; j <= ny + 2; ++j) {
      double a[4];
      for (int c = 0; c < 4; ++c) a[c] = UR(r, r->u, c, i, j);
      prep_cell(r, 1, a, &r->wk_w[j], &r->wk_vx[j], &r->wk_vy[j], &r->wk_h[j]);
    }
    double al = 0.;
    for (int j = -2; j <= ny + 3; ++j) al = fmax(al, ALPHA(r, i, j));
    for (int j = -2; j <= ny + 3; ++j) {
      double a[4], g[4];
      for (int c = 0; c < 4; ++c) a[c] = UR(r, r->u, c, i, j);
      fflux2d(r, a, g, 1);
      for (int c = 0; c < 4; ++c) {
        UR(r, r->gp, c, i, j) = 0.5 * (a[c] + g[c] / al);
        UR(r, r->gn, c, i, j) = 0.5 * (a[c] - g[c] / al);
      }
    }
    for (int j = 0; j <= ny + 1; ++j) {
      double sp[5][4], sn[5][4], op[4], on[4];
      for (int ig = 0; ig < 5; ++ig)
        for (int c = 0; c < 4; ++c) {
          sp[ig][c] = UR(r, r->gp, c, i, j + ig - 2);
          sn[ig][c] = UR(r, r->gn, c, i, j + ig - 2);
        }
      interface2d(r, 1, r->wk_w[j], r->wk_w[j + 1], r->wk_vx[j], r->wk_vx[j + 1], r->wk_vy[j],
                  r->wk_vy[j + 1], r->wk_h[j], r->wk_h[j + 1], (const double(*)[4])sp,
                  (const double(*)[4])sn, op, on);
      limit_interface(r, r->gp, r->gn, i, j, op, on);
      for (int c = 0; c < 4; ++c) {
        UR(r, r->gpf, c, i, j) = al * op[c];
        UR(r, r->gnf, c, i, j) = al * on[c];
      }
    }
  }
}

/* exchange_x (:946-1006): ghost columns from the x neighbours (periodic) */
static void ex6_exchange_x(oracle* o) {
  const int n = o->cut_x * o->cut_y;
  double** snap = malloc(n * sizeof(double*));
  for (int k = 0; k < n; ++k) {
    snap[k] = malloc(state_len(o->rk[k]) * sizeof(double));
    memcpy(snap[k], o->rk[k]->u, state_len(o->rk[k]) * sizeof(double));
  }
  for (int k = 0; k < n; ++k) {
    oracle* r = o->rk[k];
    int left = (r->px + o->cut_x - 1) % o->cut_x + o->cut_x * r->py;
    int right = (r->px + 1) % o->cut_x + o->cut_x * r->py;
    const oracle* rl = o->rk[left];
    const oracle* rr = o->rk[right];
    for (int j = -2; j <= r->ny + 3; ++j)
      for (int m = 1; m <= 3; ++m)
        for (int c = 0; c < o->nc; ++c) {
          r->u[IX(r, c, r->nx + m, j)] = snap[right][IX(rr, c, m, j)];
          r->u[IX(r, c, 1 - m, j)] = snap[left][IX(rl, c, rl->nx + 1 - m, j)];
        }
  }
  for (int k = 0; k < n; ++k) free(snap[k]);
  free(snap);
}

/* exchange_y (:1008-1067): ghost rows from the y neighbours (periodic) */
static void ex6_exchange_y(oracle* o) {
  const int n = o->cut_x * o->cut_y;
  double** snap = malloc(n * sizeof(double*));
  for (int k = 0; k < n; ++k) {
    snap[k] = malloc(state_len(o->rk[k]) * sizeof(double));
    memcpy(snap[k], o->rk[k]->u, state_len(o->rk[k]) * sizeof(double));
  }
  for (int k = 0; k < n; ++k) {
    oracle* r = o->rk[k];
    int down = r->px + o->cut_x * ((r->py + o->cut_y - 1) % o->cut_y);
    int up = r->px + o->cut_x * ((r->py + 1) % o->cut_y);
    const oracle* rd = o->rk[down];
    const oracle* ru = o->rk[up];
    for (int m = 1; m <= 3; ++m)
      for (int i = -2; i <= r->nx + 3; ++i)
        for (int c = 0; c < o->nc; ++c) {
          r->u[IX(r, c, i, r->ny + m)] = snap[up][IX(ru, c, i, m)];
          r->u[IX(r, c, i, 1 - m)] = snap[down][IX(rd, c, i, rd->ny + 1 - m)];
        }
  }
  for (int k = 0; k < n; ++k) free(snap[k]);
  free(snap);
}

/* bc (:797-944): exchanges twice, then fixed bottom, fixed right, copied
 * top, inflow left and the quiescent column i = 1 (the loop index after
 * `do i = -2, 0`) below row 6*total */
static void ex6_bc(oracle* o) {
  ex6_exchange_x(o);
  ex6_exchange_y(o);
  ex6_exchange_x(o);
  ex6_exchange_y(o);
  const double g = o->gamma, g1 = o->gamma1;
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    oracle* r = o->rk[k];
    const int nx = r->nx, ny = r->ny;
    if (r->py == 0)
      for (int jj = -2; jj <= 0; ++jj)
        for (int i = -2; i <= nx + 3; ++i) {
          UR(r, r->u, 0, i, jj) = g;
          UR(r, r->u, 1, i, jj) = 0.;
          UR(r, r->u, 2, i, jj) = 0.;
          UR(r, r->u, 3, i, jj) = 1. / g1;
        }
    if (r->px == o->cut_x - 1)
      for (int ii = 1; ii <= 3; ++ii)
        for (int j = -2; j <= ny + 3; ++j) {
          UR(r, r->u, 0, nx + ii, j) = g;
          UR(r, r->u, 1, nx + ii, j) = 0.;
          UR(r, r->u, 2, nx + ii, j) = 0.;
          UR(r, r->u, 3, nx + ii, j) = 1. / g1;
        }
    if (r->py == o->cut_y - 1)
      for (int ii = 1; ii <= 3; ++ii)
        for (int i = -2; i <= nx + 3; ++i)
          for (int c = 0; c < 4; ++c) UR(r, r->u, c, i, ny + ii) = UR(r, r->u, c, i, ny);
    if (r->px == 0) {
      for (int ii = -2; ii <= 0; ++ii)
        for (int j = -2; j <= ny + 3; ++j) {
          UR(r, r->u, 0, ii, j) = o->dle;
          UR(r, r->u, 1, ii, j) = o->ule * o->dle;
          UR(r, r->u, 2, ii, j) = 0.;
          UR(r, r->u, 3, ii, j) = o->ple / g1 + 0.5 * o->dle * (o->ule * o->ule);
        }
      const int i = 1; /* the DO variable after `do i = -2, 0` */
      for (int j = -2; j <= ny + 3; ++j)
        if (i + r->px * nx < o->total && j + r->py * ny < 6 * o->total) {
          UR(r, r->u, 0, i, j) = 1.;
          UR(r, r->u, 1, i, j) = 0.;
          UR(r, r->u, 2, i, j) = 0.;
          UR(r, r->u, 3, i, j) = 1. / g1;
        }
    }
  }
}

/* checkpositivity over every rank's interior (`<=`, :773-795) */
static int ex6_checkpositivity(oracle* o) {
  int postag = 0;
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) postag |= checkpositivity2d(o->rk[k]);
  return postag;
}

/* gather_to_root / scatter_from_root: the global interior <-> the ranks */
static void ex6_gather(oracle* o) {
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    const oracle* r = o->rk[k];
    for (int j = 1; j <= r->ny; ++j)
      for (int i = 1; i <= r->nx; ++i)
        for (int c = 0; c < o->nc; ++c)
          o->u[IX(o, c, r->px * o->nxl + i, r->py * o->nyl + j)] = r->u[IX(r, c, i, j)];
  }
}
static void ex6_scatter(oracle* o) {
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    oracle* r = o->rk[k];
    for (int j = 1; j <= r->ny; ++j)
      for (int i = 1; i <= r->nx; ++i)
        for (int c = 0; c < o->nc; ++c)
          r->u[IX(r, c, i, j)] = o->u[IX(o, c, r->px * o->nxl + i, r->py * o->nyl + j)];
  }
}

/* wenofd + scheme on every rank; returns the global alphamax */
static double ex6_flux_divergence(oracle* o) {
  double am = 0.;
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) am = fmax(am, ex6_findalpha(o->rk[k]));
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    ex6_wenofd(o->rk[k]);
    scheme2d(o->rk[k]);
  }
  return am;
}

/* rk (:693-771) */
static int ex6_step(oracle* o) {
  if (o->ranks_stale) ex6_distribute(o);
  const int n = o->cut_x * o->cut_y;
  for (int stage = 1; stage <= 3; ++stage) {
    double am = ex6_flux_divergence(o);
    o->alphamax = am;
    if (stage == 1) {
      compute_dt(o);
      for (int k = 0; k < n; ++k)
        memcpy(o->rk[k]->u0, o->rk[k]->u, state_len(o->rk[k]) * sizeof(double));
    }
    const double dt = o->dt;
    for (int k = 0; k < n; ++k) {
      oracle* r = o->rk[k];
      const size_t len = state_len(r);
      for (size_t m = 0; m < len; ++m) {
        double v = r->u[m] + dt * r->rhs[m];
        if (stage == 1) r->u[m] = v;
        else if (stage == 2) r->u[m] = rk2(o, r->u0[m], v);
        else r->u[m] = rk3(o, r->u0[m], v);
      }
    }
    o->postag = ex6_checkpositivity(o);
    ex6_gather(o);
    if (o->cfg.use_limiter == 2 && o->postag == 1) {
      int st = sweep_lim2d(o);
      o->postag = 0;
      if (st != SWFD_OK) {
        ex6_assemble(o);
        return o->status = st;
      }
    }
    ex6_scatter(o);
    ex6_bc(o);
  }
  o->time = o->time + o->dt;
  ex6_assemble(o);
  return SWFD_OK;
}

/* initdata (:1069-1150): post-shock state for i <= total/2 above row 6*total
 * on the ranks of column 0, pre-shock state elsewhere, ghosts included */
static void ex6_init(oracle* o) {
  const double g = o->gamma, g1 = o->gamma1;
  const double xm1 = 5.09, ss = xm1;
  const double dri = g, pri = 1.;
  const double ach2 = ((0.0 - ss) * (0.0 - ss)) / g / pri * dri;
  o->ple = pri * (g * ach2 / (g + 1.) * 2. - (g - 1.) / (g + 1.));
  o->dle = dri * (g + 1.) / 2. * ach2 / ((g - 1.) / 2. * ach2 + 1.);
  o->ule = (0.0 - ss) / o->dle * dri + ss;
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    oracle* r = o->rk[k];
    for (int j = -2; j <= r->ny + 3; ++j)
      for (int i = -2; i <= r->nx + 3; ++i) {
        if (r->px == 0 && i <= o->total / 2 && r->py * r->ny + j >= o->total * 6) {
          UR(r, r->u, 0, i, j) = o->dle;
          UR(r, r->u, 1, i, j) = o->ule * o->dle;
          UR(r, r->u, 2, i, j) = 0.;
          UR(r, r->u, 3, i, j) = o->ple / g1 + 0.5 * o->dle * (o->ule * o->ule);
        } else {
          UR(r, r->u, 0, i, j) = dri;
          UR(r, r->u, 1, i, j) = 0.;
          UR(r, r->u, 2, i, j) = 0.;
          UR(r, r->u, 3, i, j) = pri / g1;
        }
      }
  }
  o->ranks_stale = 0;
  ex6_assemble(o);
}

/* ------------------------------------------------------------------ */
/* ex7: reactive Euler detonation (ex7_detonation/main.f90).  Five      */
/* components (rho, m_x, m_y, E, rho*Y), eos p = g1*(E - kinetic - q*Y),*/
/* the chemistry source -k*Y*exp(-t*rho/p) on the fifth.  The rank      */
/* layout, exchanges, gather and scatter are ex6's (5 components).      */
/* ------------------------------------------------------------------ */

/* exp(x) evaluated in binary128 and rounded once to binary64: x = k*ln2 + r
 * with k the nearest integer to x*(1/ln2) (binary64), r = x - k*ln2 in
 * binary128, exp(r) by Horner on the Taylor coefficients 1/n! (n <= 24, each
 * the binary128 quotient of the previous by n), times 2^k exactly.  The
 * library evaluates the same sequence of binary128 operations (qd::exp_rd),
 * so the two agree bit for bit.  The result is the correctly rounded exp
 * wherever the binary128 evaluation decides the rounding; the host libm's
 * exp differs from it by one ulp on a small fraction of arguments. */
#define EXP7_N 24
static Q exp7_coef[EXP7_N + 1];
static int exp7_ready;
double oracle_exp(double x) {
  if (x != x) return x;
  if (x > 710.) return INFINITY;
  if (x < -746.) return 0.;
  if (!exp7_ready) {
    exp7_coef[0] = 1;
    for (int n = 1; n <= EXP7_N; ++n) exp7_coef[n] = exp7_coef[n - 1] / (Q)n;
    exp7_ready = 1;
  }
  const double kd = rint(x * 1.4426950408889634);
  /* ln2 as the binary128 sum of a triple-double split (113 bits) */
  const Q ln2 = ((Q)0x1.62e42fefa39efp-1 + (Q)0x1.abc9e3b39803fp-56) + (Q)0x1.7b57a079a1934p-111;
  const Q r = (Q)x - (Q)kd * ln2;
  Q p = exp7_coef[EXP7_N];
  for (int n = EXP7_N - 1; n >= 0; --n) p = p * r + exp7_coef[n];
  /* 2^k as binary128 bits (exponent field k + 16383, zero fraction): exact */
  const uint64_t bits[2] = {0, (uint64_t)((int)kd + 16383) << 48};
  Q two_k;
  memcpy(&two_k, bits, sizeof(two_k));
  return (double)(p * two_k);
}

/* eos (:168-174) */
static inline double ex7_eos(const oracle* r, double rho, double vx, double vy, double e,
                             double y) {
  return r->gamma1 * (e - 0.5 * rho * (vx * vx) - 0.5 * rho * (vy * vy) - r->qc * y);
}

/* fflux / gflux (:110-166) */
static void ex7_flux(const oracle* r, const double* a, double* f, int gdir) {
  const double rho = a[0], mx = a[1], my = a[2], e = a[3], y = a[4];
  double vx = mx / rho, vy = my / rho;
  if (rho < r->eps2) vx = 0.;
  if (rho < r->eps2) vy = 0.;
  const double pres = ex7_eos(r, rho, vx, vy, e, y);
  if (!gdir) {
    f[0] = mx;
    f[1] = rho * (vx * vx) + pres;
    f[2] = rho * vx * vy;
    f[3] = (e + pres) * vx;
    f[4] = y * vx;
  } else {
    f[0] = my;
    f[1] = rho * vx * vy;
    f[2] = rho * (vy * vy) + pres;
    f[3] = (e + pres) * vy;
    f[4] = y * vy;
  }
}

/* per-line Roe preparation (x pass :200-215, y pass :474-489):
 * out = {w, vx, vy, ratio, h} */
static void ex7_prep(const oracle* r, const double* a, double* out) {
  const double den = a[0], xmt = a[1], ymt = a[2], eng = a[3], yrho = a[4];
  const double t0 = 1. / den, vex = xmt * t0, vey = ymt * t0;
  const double pre = r->gamma1 * (eng - 0.5 * (xmt * vex + ymt * vey) - r->qc * yrho);
  out[0] = sqrt(fabs(den));
  out[1] = vex;
  out[2] = vey;
  out[3] = yrho * t0;
  out[4] = (pre + eng) * t0;
}

/* chemsource (:752-771) */
static double ex7_chemsource(const oracle* r, const double* a) {
  const double rho = a[0], mx = a[1], my = a[2], e = a[3], y = a[4];
  double vx = mx / rho, vy = my / rho;
  if (lt_lit_1em8(r, rho)) vx = 0.;
  if (lt_lit_1em8(r, rho)) vy = 0.;
  const double pres = ex7_eos(r, rho, vx, vy, e, y);
  return -(r->kc * y * oracle_exp(-(r->tc * rho / pres)));
}

/* one interface: Roe average, 5x5 eigenvectors, projections, ten WENO5
 * reconstructions, back projection (x pass :228-334, y pass :506-600);
 * L, R = {w, vx, vy, ratio, h} of the two cells; every product of the
 * eigenvector sums is formed, zeros and ones included, in the reference's order */
static void ex7_interface(const oracle* r, int ydir, const double* L, const double* R,
                          const double sp[5][5], const double sn[5][5], double* outp,
                          double* outn) {
  const double g1 = r->gamma1, q = r->qc;
  double evr[5][5], evl[5][5], cu_p[5][5], cu_n[5][5], ur[5], ul[5];
  /* w/(w+w1+1d-15) and sqrt(..)+1d-15 with the literal in binary128 under
   * the reference build (:234,240) */
  double t0 = r->quad ? (double)((Q)L[0] / ((Q)(L[0] + R[0]) + 1e-15f128))
                      : L[0] / (L[0] + R[0] + 1e-15);
  double t1 = 1. - t0;
  const double vxm = t0 * L[1] + t1 * R[1];
  const double vym = t0 * L[2] + t1 * R[2];
  const double ym = t0 * L[3] + t1 * R[3];
  const double hm = t0 * L[4] + t1 * R[4];
  const double qm = 0.5 * (vxm * vxm + vym * vym);
  const double cm = r->quad ? (double)((Q)sqrt(fabs(g1 * (hm - qm - q * ym))) + 1e-15f128)
                            : sqrt(fabs(g1 * (hm - qm - q * ym))) + 1e-15;
  const double rcm = 1. / cm;
  const double b1 = g1 * rcm * rcm;
  const double b2 = qm * b1;
  double t2, t3;
  if (!ydir) {
    t0 = vxm * cm;
    const double er[5][5] = {{1.0, 1.0, 0.0, 0.0, 1.0},
                             {vxm - cm, vxm, 0., 0., vxm + cm},
                             {vym, vym, -1., 0., vym},
                             {hm - t0, qm, -vym, q, hm + t0},
                             {ym, 0., 0., 1., ym}};
    memcpy(evr, er, sizeof(er));
    t0 = vxm * rcm;
    t1 = b1 * vxm;
    t2 = 0.5 * b1;
    t3 = b1 * vym;
    const double el[5][5] = {{0.5 * (b2 + t0), -0.5 * (t1 + rcm), -0.5 * t3, t2, -t2 * q},
                             {1. - b2, t1, t3, -b1, b1 * q},
                             {vym, 0.0, -1.0, 0.0, 0.0},
                             {-b2 * ym, t1 * ym, t3 * ym, -b1 * ym, 1. + q * ym * b1},
                             {0.5 * (b2 - t0), -0.5 * (t1 - rcm), -0.5 * t3, t2, -t2 * q}};
    memcpy(evl, el, sizeof(el));
  } else {
    t0 = vym * cm;
    const double er[5][5] = {{1.0, 1.0, 0.0, 0.0, 1.0},
                             {vxm, vxm, 1.0, 0., vxm},
                             {vym - cm, vym, 0., 0., vym + cm},
                             {hm - t0, qm, vxm, q, hm + t0},
                             {ym, 0., 0., 1., ym}};
    memcpy(evr, er, sizeof(er));
    t0 = vym * rcm;
    t1 = b1 * vym;
    t2 = 0.5 * b1;
    t3 = b1 * vxm;
    const double el[5][5] = {{0.5 * (b2 + t0), -0.5 * t3, -0.5 * (t1 + rcm), t2, -q * t2},
                             {1. - b2, t3, t1, -b1, b1 * q},
                             {-vxm, 1.0, 0.0, 0.0, 0.0},
                             {-ym * b2, ym * t3, ym * t1, -ym * b1, 1. + ym * b1 * q},
                             {0.5 * (b2 - t0), -0.5 * t3, -0.5 * (t1 - rcm), t2, -q * t2}};
    memcpy(evl, el, sizeof(el));
  }
  for (int ig = 0; ig < 5; ++ig)
    for (int k = 0; k < 5; ++k) {
      cu_p[k][ig] = evl[k][0] * sp[ig][0] + evl[k][1] * sp[ig][1] + evl[k][2] * sp[ig][2] +
                    evl[k][3] * sp[ig][3] + evl[k][4] * sp[ig][4];
      cu_n[k][ig] = evl[k][0] * sn[ig][0] + evl[k][1] * sn[ig][1] + evl[k][2] * sn[ig][2] +
                    evl[k][3] * sn[ig][3] + evl[k][4] * sn[ig][4];
    }
  for (int kk = 0; kk < 5; ++kk) {
    ur[kk] = oracle_weno_right_impl(r, cu_p[kk]);
    ul[kk] = oracle_weno_left_impl(r, cu_n[kk]);
  }
  for (int k = 0; k < 5; ++k) {
    outp[k] = evr[k][0] * ur[0] + evr[k][1] * ur[1] + evr[k][2] * ur[2] + evr[k][3] * ur[3] +
              evr[k][4] * ur[4];
    outn[k] = evr[k][0] * ul[0] + evr[k][1] * ul[1] + evr[k][2] * ul[2] + evr[k][3] * ul[3] +
              evr[k][4] * ul[4];
  }
}

/* use_limiter = 1: the positivity limiter of one split flux (:336-440), five
 * components and q*Y in both pressures, theta clamped at 0 */
static void ex7_zs_limit(oracle* r, const double* ave, double* out) {
  const double g1 = r->gamma1, q = r->qc;
  const double d_ave = ave[0], m_ave = ave[1], n_ave = ave[2], e_ave = ave[3], y_ave = ave[4];
  const double p_ave =
      g1 * (e_ave - 0.5 * (m_ave * m_ave) / d_ave - 0.5 * (n_ave * n_ave) / d_ave - q * y_ave);
  double point[2][5];
  double theta = 1.0;
  for (int c = 0; c < 5; ++c) {
    point[0][c] = out[c];
    point[1][c] = (ave[c] - out[c] / 12.) / (11. / 12.);
  }
  for (int ig = 0; ig < 2; ++ig) {
    const double d_l = point[ig][0];
    if (d_l < 0.) theta = fmin(theta, fabs(d_ave - 0.) / fabs(d_ave - d_l));
  }
  theta = fmax(theta, 0.);
  if (theta < 1.) {
    out[0] = theta * out[0] + (1. - theta) * d_ave;
    r->den_count++;
  }
  theta = 1.;
  point[0][0] = out[0];
  point[1][0] = (ave[0] - out[0] / 12.) / (11. / 12.);
  for (int ig = 0; ig < 2; ++ig) {
    const double d_l = point[ig][0], m_l = point[ig][1], n_l = point[ig][2], e_l = point[ig][3],
                 y_l = point[ig][4];
    const double p_l = g1 * (e_l - (m_l * m_l) / d_l / 2. - (n_l * n_l) / d_l / 2. - q * y_l);
    if (p_l < 0.) theta = fmin(theta, fabs(p_ave - 0.) / fabs(p_ave - p_l));
  }
  theta = fmax(theta, 0.);
  if (theta < 1.) {
    r->pre_count++;
    for (int c = 0; c < 5; ++c) out[c] = theta * out[c] + (1. - theta) * ave[c];
  }
}

/* findalpha of one rank (:774-808; source_alpha is computed there but never
 * used, so it is left out) */
static double ex7_findalpha(oracle* r) {
  double am = 0.;
  for (int i = -2; i <= r->nx + 3; ++i)
    for (int j = -2; j <= r->ny + 3; ++j) {
      const double u1 = UR(r, r->u, 0, i, j), u2 = UR(r, r->u, 1, i, j),
                   u3 = UR(r, r->u, 2, i, j), u4 = UR(r, r->u, 3, i, j),
                   u5 = UR(r, r->u, 4, i, j);
      const double den = u1;
      double vx, vy;
      if (den >= r->eps2) {
        vx = u2 / den;
        vy = u3 / den;
      } else {
        vx = 0.;
        vy = 0.;
      }
      const double pres =
          r->gamma1 * (u4 - 0.5 * den * (vx * vx) - 0.5 * den * (vy * vy) - u5 * r->qc);
      const double sound = sqrt(r->gamma * pres / den);
      const double a = fmax(fabs(u2 / u1) + sound, fabs(u3 / u1) + sound);
      ALPHA(r, i, j) = a;
      am = fmax(am, a);
    }
  return am;
}

/* wenofd of one rank (:176-736): wall mirror at column total for global rows
 * <= step*total (:186-197), per-row alpha over the rank's local row
 * (:217-223), fluxes scaled by it (:444-445); wall mirror at row step*total
 * over columns 1..total (:456-470); per-column alpha (:492-497) and scaling
 * (:728-729) in the y pass */
static void ex7_wenofd(oracle* r) {
  const int nx = r->nx, ny = r->ny, total = r->total;
  double pr[5], sp[5][5], sn[5][5], op[5], on[5], a[5], f[5];
  for (int j = 0; j <= ny + 1; ++j) {
    if (r->px == 0 && r->py * ny + j <= r->wall_rows)
      for (int i = 0; i <= 2; ++i) {
        for (int c = 0; c < 5; ++c) UR(r, r->u, c, total - i, j) = UR(r, r->u, c, total + 1 + i, j);
        UR(r, r->u, 1, total - i, j) = -UR(r, r->u, 1, total + 1 + i, j);
      }
    for (int i = 0; i <= nx + 2; ++i) {
      for (int c = 0; c < 5; ++c) a[c] = UR(r, r->u, c, i, j);
      ex7_prep(r, a, pr);
      r->wk_w[i] = pr[0];
      r->wk_vx[i] = pr[1];
      r->wk_vy[i] = pr[2];
      r->wk_ratio[i] = pr[3];
      r->wk_h[i] = pr[4];
    }
    double al = 0.;
    for (int i = -2; i <= nx + 3; ++i) al = fmax(al, ALPHA(r, i, j));
    for (int i = -2; i <= nx + 3; ++i) {
      for (int c = 0; c < 5; ++c) a[c] = UR(r, r->u, c, i, j);
      ex7_flux(r, a, f, 0);
      for (int c = 0; c < 5; ++c) {
        UR(r, r->fp, c, i, j) = 0.5 * (a[c] + f[c] / al);
        UR(r, r->fn, c, i, j) = 0.5 * (a[c] - f[c] / al);
      }
    }
    for (int i = 0; i <= nx + 1; ++i) {
      for (int ig = 0; ig < 5; ++ig)
        for (int c = 0; c < 5; ++c) {
          sp[ig][c] = UR(r, r->fp, c, i + ig - 2, j);
          sn[ig][c] = UR(r, r->fn, c, i + ig - 2, j);
        }
      const double L[5] = {r->wk_w[i], r->wk_vx[i], r->wk_vy[i], r->wk_ratio[i], r->wk_h[i]};
      const double R[5] = {r->wk_w[i + 1], r->wk_vx[i + 1], r->wk_vy[i + 1], r->wk_ratio[i + 1],
                           r->wk_h[i + 1]};
      ex7_interface(r, 0, L, R, (const double(*)[5])sp, (const double(*)[5])sn, op, on);
      if (r->cfg.use_limiter == 1) {
        ex7_zs_limit(r, sp[2], op);
        ex7_zs_limit(r, sn[2], on);
      }
      for (int c = 0; c < 5; ++c) {
        UR(r, r->fpf, c, i, j) = al * op[c];
        UR(r, r->fnf, c, i, j) = al * on[c];
      }
    }
  }
  if (r->px == 0)
    for (int j = -2; j <= ny + 3; ++j)
      if (r->py * ny + j == r->wall_rows)
        for (int i = 0; i <= 2; ++i)
          for (int k = 1; k <= total; ++k) {
            for (int c = 0; c < 5; ++c) UR(r, r->u, c, k, j - i) = UR(r, r->u, c, k, j + 1 + i);
            UR(r, r->u, 2, k, j - i) = -UR(r, r->u, 2, k, j + 1 + i);
          }
  for (int i = 0; i <= nx + 1; ++i) {
    for (int j = 0; j <= ny + 2; ++j) {
      for (int c = 0; c < 5; ++c) a[c] = UR(r, r->u, c, i, j);
      ex7_prep(r, a, pr);
      r->wk_w[j] = pr[0];
      r->wk_vx[j] = pr[1];
      r->wk_vy[j] = pr[2];
      r->wk_ratio[j] = pr[3];
      r->wk_h[j] = pr[4];
    }
    double al = 0.;
    for (int j = -2; j <= ny + 3; ++j) al = fmax(al, ALPHA(r, i, j));
    for (int j = -2; j <= ny + 3; ++j) {
      for (int c = 0; c < 5; ++c) a[c] = UR(r, r->u, c, i, j);
      ex7_flux(r, a, f, 1);
      for (int c = 0; c < 5; ++c) {
        UR(r, r->gp, c, i, j) = 0.5 * (a[c] + f[c] / al);
        UR(r, r->gn, c, i, j) = 0.5 * (a[c] - f[c] / al);
      }
    }
    for (int j = 0; j <= ny + 1; ++j) {
      for (int ig = 0; ig < 5; ++ig)
        for (int c = 0; c < 5; ++c) {
          sp[ig][c] = UR(r, r->gp, c, i, j + ig - 2);
          sn[ig][c] = UR(r, r->gn, c, i, j + ig - 2);
        }
      const double L[5] = {r->wk_w[j], r->wk_vx[j], r->wk_vy[j], r->wk_ratio[j], r->wk_h[j]};
      const double R[5] = {r->wk_w[j + 1], r->wk_vx[j + 1], r->wk_vy[j + 1], r->wk_ratio[j + 1],
                           r->wk_h[j + 1]};
      ex7_interface(r, 1, L, R, (const double(*)[5])sp, (const double(*)[5])sn, op, on);
      if (r->cfg.use_limiter == 1) {
        ex7_zs_limit(r, sp[2], op);
        ex7_zs_limit(r, sn[2], on);
      }
      for (int c = 0; c < 5; ++c) {
        UR(r, r->gpf, c, i, j) = al * op[c];
        UR(r, r->gnf, c, i, j) = al * on[c];
      }
    }
  }
}

/* scheme (:738-750): flux differences of the alpha-scaled fluxes plus the
 * chemistry source on the fifth component */
static void ex7_scheme(oracle* r) {
  for (int i = 1; i <= r->nx; ++i)
    for (int j = 1; j <= r->ny; ++j) {
      for (int c = 0; c < 5; ++c)
        UR(r, r->rhs, c, i, j) =
            -((UR(r, r->fpf, c, i, j) - UR(r, r->fnf, c, i + 1, j)) -
              (UR(r, r->fpf, c, i - 1, j) - UR(r, r->fnf, c, i, j))) / r->dx -
            ((UR(r, r->gpf, c, i, j) - UR(r, r->gnf, c, i, j + 1)) -
             (UR(r, r->gpf, c, i, j - 1) - UR(r, r->gnf, c, i, j))) / r->dy;
      double a[5];
      for (int c = 0; c < 5; ++c) a[c] = UR(r, r->u, c, i, j);
      UR(r, r->rhs, 4, i, j) = UR(r, r->rhs, 4, i, j) + ex7_chemsource(r, a);
    }
}

/* checkpositivity over every rank's interior (:890-913) */
static int ex7_checkpositivity(oracle* o) {
  int postag = 0;
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    const oracle* r = o->rk[k];
    for (int i = 1; i <= r->nx; ++i)
      for (int j = 1; j <= r->ny; ++j) {
        const double u1 = UR(r, r->u, 0, i, j), u2 = UR(r, r->u, 1, i, j),
                     u3 = UR(r, r->u, 2, i, j), u4 = UR(r, r->u, 3, i, j),
                     u5 = UR(r, r->u, 4, i, j);
        if (u1 <= r->eps) postag = 1;
        if (u4 - u3 * u3 / u1 / 2. - u2 * u2 / u1 / 2. - r->qc * u5 <= r->eps) postag = 1;
      }
  }
  return postag;
}

static inline void ex7_set(oracle* r, int i, int j, double a, double b, double c, double d,
                           double e) {
  UR(r, r->u, 0, i, j) = a;
  UR(r, r->u, 1, i, j) = b;
  UR(r, r->u, 2, i, j) = c;
  UR(r, r->u, 3, i, j) = d;
  UR(r, r->u, 4, i, j) = e;
}

/* bc (:915-1071): exchanges twice, then the quiescent bottom and right, the
 * reflecting top, the inflow left and the quiescent solid block (global
 * i < total, j < step*total), ghosts included */
static void ex7_bc(oracle* o) {
  ex6_exchange_x(o);
  ex6_exchange_y(o);
  ex6_exchange_x(o);
  ex6_exchange_y(o);
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    oracle* r = o->rk[k];
    const int nx = r->nx, ny = r->ny;
    if (r->py == 0)
      for (int jj = -2; jj <= 0; ++jj)
        for (int i = -2; i <= nx + 3; ++i) ex7_set(r, i, jj, 1., 0., 0., 55., 1.);
    if (r->px == o->cut_x - 1)
      for (int ii = 1; ii <= 3; ++ii)
        for (int j = -2; j <= ny + 3; ++j) ex7_set(r, nx + ii, j, 1., 0., 0., 55., 1.);
    if (r->py == o->cut_y - 1)
      for (int ii = 1; ii <= 3; ++ii)
        for (int i = -2; i <= nx + 3; ++i) {
          for (int c = 0; c < 5; ++c) UR(r, r->u, c, i, ny + ii) = UR(r, r->u, c, i, ny);
          UR(r, r->u, 2, i, ny + ii) = -UR(r, r->u, 2, i, ny);
        }
    if (r->px == 0)
      for (int ii = -2; ii <= 0; ++ii)
        for (int j = -2; j <= ny + 3; ++j) ex7_set(r, ii, j, 11., 11. * 6.18, 0., 970., 11.);
    for (int i = -2; i <= nx + 3; ++i)
      for (int j = -2; j <= ny + 3; ++j)
        if (i + r->px * nx < o->total && j + r->py * ny < o->wall_rows)
          ex7_set(r, i, j, 1., 0., 0., 55., 1.);
  }
}

/* initdata (:1196-1260): the post-detonation state where x < 0.5, the
 * quiescent state elsewhere, on local cells 0..nx+1 x 0..ny+1 of every rank;
 * then bc */
static void ex7_init(oracle* o) {
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    oracle* r = o->rk[k];
    memset(r->u, 0, state_len(r) * sizeof(double));
    const double xleft = 5. / o->cut_x * r->px;
    for (int i = 0; i <= r->nx + 1; ++i)
      for (int j = 0; j <= r->ny + 1; ++j) {
        const double x = xleft + i * r->dx - r->dx / 2.;
        if (x < 0.5) ex7_set(r, i, j, 11., 11. * 6.18, 0., 970., 11.);
        else ex7_set(r, i, j, 1., 0., 0., 55., 1.);
      }
  }
  ex7_bc(o);
  o->ranks_stale = 0;
  ex6_assemble(o);
}

/* pressure of a sweep vector: `form` 0 is g1*(v4 - 0.5*v2*v2/v1 -
 * 0.5*v3**2/v1 - q*v5) (the unadjusted v_i and v_p, :1503,1532), 1 the
 * all-squared g1*(v4 - 0.5*v2**2/v1 - 0.5*v3**2/v1 - q*v5) (nod_lim, the
 * adjusted vectors and u_bar, :1405-1406,1533-1535) */
static inline double ex7_psweep(const oracle* o, const double* v, int form) {
  if (form == 0)
    return o->gamma1 * (v[3] - 0.5 * v[1] * v[1] / v[0] - 0.5 * (v[2] * v[2]) / v[0] - o->qc * v[4]);
  return o->gamma1 * (v[3] - 0.5 * (v[1] * v[1]) / v[0] - 0.5 * (v[2] * v[2]) / v[0] - o->qc * v[4]);
}

/* nod_lim (:1399-1429) */
static void ex7_nod_lim(oracle* o, const double* v1, const double* v2, const double* vb,
                        double* out) {
  const double eps = o->eps;
  const double p1 = ex7_psweep(o, v1, 1), p2 = ex7_psweep(o, v2, 1);
  double t;
  if (p2 > eps) {
    t = (p1 - eps) / (p1 - p2);
    o->t_pos_count++;
  } else {
    const double pb = ex7_psweep(o, vb, 1);
    const double t_1 = (p1 - eps) / (p1 - pb);
    const double d12 = sqrt(sq(v2[4] - v1[4]) + sq(v2[3] - v1[3]) + sq(v2[2] - v1[2]) +
                            sq(v2[1] - v1[1]) + sq(v2[0] - v1[0]));
    const double d1b = sqrt(sq(vb[4] - v1[4]) + sq(vb[3] - v1[3]) + sq(vb[2] - v1[2]) +
                            sq(vb[1] - v1[1]) + sq(vb[0] - v1[0]));
    t = fmin(t_1 * d1b / d12, 0.25);
    o->t_neg_count++;
  }
  for (int c = 0; c < 5; ++c) out[c] = (1 - t) * v1[c] + t * v2[c];
}

/* One pass (:1481-1704).  Ordering I (ord 0): every component at sweepI(k).
 * Ordering II (ord 1) keeps the reference's indexing: components 1-4 at
 * sweepII(k) and sweepII(k+-1), component 5 at sweepI(k) and, for the
 * neighbour, sweepI(k-1) in both directions.  The total-pressure check
 * stops the run in the ordering-I passes only. */
static int ex7_pass(oracle* o, int ord, int forward, const double* ubar) {
  const int N = o->nx * o->ny;
  const double eps = o->eps, w = o->weight;
  const int *Ii = o->sI_i, *Ij = o->sI_j;
  const int *Ai = ord ? o->sII_i : o->sI_i, *Aj = ord ? o->sII_j : o->sI_j;
  const int k0 = forward ? 0 : N - 1, k1 = forward ? N - 1 : 0, dk = forward ? 1 : -1;
  for (int k = k0; k != k1; k += dk) {
    double vi[5], vp[5], vit[5], d[5], vpt[5];
    /* cells of v_i (components 1-4, component 5) and of v_p */
    const int ai = Ai[k], aj = Aj[k], bi = Ii[k], bj = Ij[k];
    for (int c = 0; c < 4; ++c) vi[c] = U(o->u, c, ai, aj);
    vi[4] = U(o->u, 4, bi, bj);
    const double pres_v_i = ex7_psweep(o, vi, 0);
    if (pres_v_i <= eps || vi[0] <= eps) {
      const int kn = k + dk;            /* v_p's components 1-4 */
      const int k5 = ord ? k - 1 : kn;  /* v_p's component 5 */
      if (k5 < 0) return SWFD_ERR_UNSUPPORTED; /* the reference reads sweepI(0) */
      const int ci = Ai[kn], cj = Aj[kn], di = Ii[k5], dj = Ij[k5];
      for (int c = 0; c < 4; ++c) vp[c] = U(o->u, c, ci, cj);
      vp[4] = U(o->u, 4, di, dj);
      ex7_nod_lim(o, vi, vp, ubar, vit);
      for (int c = 0; c < 5; ++c) d[c] = vi[c] - vit[c];
      for (int c = 0; c < 5; ++c) vpt[c] = vp[c] + (w / w) * (d[c]);
      for (int c = 0; c < 4; ++c) U(o->u, c, ai, aj) = vit[c];
      U(o->u, 4, bi, bj) = vit[4];
      for (int c = 0; c < 4; ++c) U(o->u, c, ci, cj) = vpt[c];
      U(o->u, 4, di, dj) = vpt[4];
      if (ord == 0) {
        const double pres_v_p = ex7_psweep(o, vp, 0);
        const double pres_v_i_t = ex7_psweep(o, vit, 1);
        const double pres_v_p_t = ex7_psweep(o, vpt, 1);
        if (pres_v_i + pres_v_p > pres_v_i_t + pres_v_p_t + eps) return SWFD_ERR_SWEEP_CHECK;
      }
    }
  }
  return SWFD_OK;
}

/* sweep_lim (:1433-1737) on the gathered interior: the density sweep, u_bar
 * (sequential, j outer), the P(u_bar) stop, alternating I/II pass pairs and
 * the exit test on g1*(E - 0.5*(m_x^2+m_y^2)/rho) and rho (no q*Y term) */
static int ex7_sweep_lim(oracle* o) {
  const int nx = o->nx, ny = o->ny;
  scalar_sweep2d(o);
  double ra = 0.0, m1a = 0.0, m2a = 0.0, ea = 0.0, ya = 0.0;
  const double w = o->weight;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      ra = ra + w * U(o->u, 0, i, j);
      m1a = m1a + w * U(o->u, 1, i, j);
      m2a = m2a + w * U(o->u, 2, i, j);
      ea = ea + w * U(o->u, 3, i, j);
      ya = ya + w * U(o->u, 4, i, j);
    }
  const double ubar[5] = {ra, m1a, m2a, ea, ya};
  if (o->gamma1 * (ea - 0.5 * (m1a * m1a) / ra - 0.5 * (m2a * m2a) / ra - o->qc * ya) <= 0.)
    return SWFD_ERR_PUBAR_NONPOS;
  o->sweep_count++;
  track_push(o);
  o->t_pos_count = 0;
  o->t_neg_count = 0;
  for (int q = 1; q <= o->cfg.swp_num; ++q) {
    const int ord = (q % 2 == 1) ? 0 : 1;
    int st = ex7_pass(o, ord, 1, ubar);
    if (st == SWFD_OK) st = ex7_pass(o, ord, 0, ubar);
    if (st != SWFD_OK) return st;
    double rho_min = 1e20, p_min = 1e20;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const double u1 = U(o->u, 0, i, j), u2 = U(o->u, 1, i, j), u3 = U(o->u, 2, i, j),
                     u4 = U(o->u, 3, i, j);
        p_min = fmin(o->gamma1 * (u4 - 0.5 * (u2 * u2 + u3 * u3) / u1), p_min);
        rho_min = fmin(u1, rho_min);
      }
    o->pre_count++;
    if (p_min > o->eps && rho_min > o->eps) {
      o->sweep_track[o->sweep_count - 1] = q;
      o->neg_track[o->sweep_count - 1] = (int32_t)o->t_neg_count;
      o->pos_track[o->sweep_count - 1] = (int32_t)o->t_pos_count;
      break;
    }
    if (q == o->cfg.swp_num) {
      o->fail_count++;
      return SWFD_ERR_SWEEP_NOCONV;
    }
  }
  return SWFD_OK;
}

/* wenofd + scheme on every rank; returns the global alphamax */
static double ex7_flux_divergence(oracle* o) {
  double am = 0.;
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) am = fmax(am, ex7_findalpha(o->rk[k]));
  for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
    ex7_wenofd(o->rk[k]);
    ex7_scheme(o->rk[k]);
  }
  return am;
}

/* rk (:810-888): dt = min(dx*cfl/alphamax, dy*cfl/alphamax, T - time) */
static int ex7_step(oracle* o) {
  if (o->ranks_stale) ex6_distribute(o);
  const int n = o->cut_x * o->cut_y;
  for (int stage = 1; stage <= 3; ++stage) {
    const double am = ex7_flux_divergence(o);
    o->alphamax = am;
    if (stage == 1) {
      const double dtx = o->dx * o->cfg.cfl / am, dty = o->dy * o->cfg.cfl / am;
      o->dt = fmin(fmin(dtx, dty), o->cfg.time_terminal - o->time);
      for (int k = 0; k < n; ++k)
        memcpy(o->rk[k]->u0, o->rk[k]->u, state_len(o->rk[k]) * sizeof(double));
    }
    const double dt = o->dt;
    for (int k = 0; k < n; ++k) {
      oracle* r = o->rk[k];
      const size_t len = state_len(r);
      for (size_t m = 0; m < len; ++m) {
        const double v = r->u[m] + dt * r->rhs[m];
        if (stage == 1) r->u[m] = v;
        else if (stage == 2) r->u[m] = rk2(o, r->u0[m], v);
        else r->u[m] = rk3(o, r->u0[m], v);
      }
    }
    o->postag = ex7_checkpositivity(o);
    ex6_gather(o);
    if (o->cfg.use_limiter == 2 && o->postag == 1) {
      const int st = ex7_sweep_lim(o);
      o->postag = 0;
      if (st != SWFD_OK) {
        ex6_assemble(o);
        return o->status = st;
      }
    }
    ex6_scatter(o);
    ex7_bc(o);
  }
  o->time = o->time + o->dt;
  ex6_assemble(o);
  return SWFD_OK;
}

/* rk / rk3 (ex3_vortex_accuracy_2d/main.f90:564-632; ex2_sedov_1d/main.f90:287-328) */
/* The dt-halving restart RK of ex2 (RK_choice /= 1, ex2_sedov_1d/main.f90:
 * 330-374).  A stage whose result fails checkpositivity sends the step back to
 * label 110: u = u0, dt = dt/2, alphamax = alphatemp, and stage 1 is redone
 * with the fluxes of the last wenofd (the reference does not call wenofd
 * again there).  No sweeps; ex2's bc is empty.  The reference loops without
 * bound; here SWFD_RESTART_LIMIT halvings end the step with an error. */
static int step_restart1d(oracle* o) {
  const size_t n = state_len(o);
  double* u = o->u;
  wenofd_any(o);
  compute_dt(o);
  const double alphatemp = o->alphamax;
  int postag = 0, restarts = 0;
  for (;;) {
    if (postag == 1) {
      if (restarts >= SWFD_RESTART_LIMIT) return o->status = SWFD_ERR_RESTART_LIMIT;
      ++restarts;
      memcpy(u, o->u0, n * sizeof(double));
      o->dt = o->dt / 2.;
      o->alphamax = alphatemp;
    }
    memcpy(o->u0, u, n * sizeof(double));
    int stage;
    for (stage = 1; stage <= 3; ++stage) {
      if (stage > 1) wenofd_any(o);
      scheme_any(o);
      const double dt = o->dt;
      for (size_t k = 0; k < n; ++k) {
        double v = u[k] + dt * o->rhs[k];
        if (stage == 1) u[k] = v;
        else if (stage == 2) u[k] = rk2(o, o->u0[k], v);
        else u[k] = rk3(o, o->u0[k], v);
      }
      postag = check_any(o);
      if (postag == 1) break;
    }
    if (stage > 3) break;
  }
  o->restarts += restarts;
  o->postag = 0;
  o->time = o->time + o->dt;
  return SWFD_OK;
}

int oracle_step(oracle* o) {
  if (o->problem == SWFD_PROBLEM_SHOCK_DIFFRACTION) return ex6_step(o);
  if (o->problem == SWFD_PROBLEM_DETONATION) return ex7_step(o);
  if (o->problem == SWFD_PROBLEM_MATLAB_1D) return ex1_step(o);
  if (o->cfg.rk_choice == 2) return step_restart1d(o);
  const size_t n = state_len(o);
  double* u = o->u;
  int st;
  for (int stage = 1; stage <= 3; ++stage) {
    wenofd_any(o);
    if (stage == 1) {
      compute_dt(o);
      memcpy(o->u0, u, n * sizeof(double));
    }
    scheme_any(o);
    const double dt = o->dt;
    for (size_t k = 0; k < n; ++k) {
      double v = u[k] + dt * o->rhs[k];
      if (stage == 1) u[k] = v;
      else if (stage == 2) u[k] = rk2(o, o->u0[k], v);
      else u[k] = rk3(o, o->u0[k], v);
    }
    o->postag = check_any(o);
    if (o->cfg.use_limiter == 2 && o->postag == 1) {
      st = sweep_any(o);
      o->postag = 0;
      if (st != SWFD_OK) return o->status = st;
    }
    bc_any(o);
  }
  o->time = o->time + o->dt;
  return SWFD_OK;
}

/* time <= time_terminal - 1d-10 (ex3_vortex_accuracy_2d/main.f90:51) */
int oracle_time_loop_continue(const oracle* o) {
  if (o->problem == SWFD_PROBLEM_MATLAB_1D) return o->time < o->cfg.time_terminal; /* :212 */
  if (o->quad) return (Q)o->time <= (Q)o->cfg.time_terminal - (Q)1e-10f128;
  return o->time <= o->cfg.time_terminal - 1e-10;
}

int64_t oracle_run(oracle* o, int64_t max_steps) {
  int64_t k = 0;
  while (oracle_time_loop_continue(o)) {
    if (max_steps > 0 && k >= max_steps) break;
    int st = oracle_step(o);
    ++k;
    if (st != SWFD_OK) return -1;
  }
  return k;
}

/* ------------------------------------------------------------------ */
/* initial data (host side of each example)                             */
/* ------------------------------------------------------------------ */
/* exact (ex3_vortex_accuracy_2d/main.f90:699-718) */
static void vortex_exact(const oracle* o, double x, double y, double t, double* e) {
  const double pi = 3.14159265358979323846264338327950, g1 = o->gamma1, gamma = o->gamma;
  double r = sqrt(sq(x - 5. - t) + sq(y - 5. - t));
  double mag = 10.0828;
  e[0] = pow(1 - g1 * (mag * mag) / 8. / gamma / (pi * pi) * exp(1. - r * r), 1. / g1);
  e[1] = e[0] * (1. - mag / 2. / pi * exp((1. - r * r) / 2.) * (y - 5.));
  e[2] = e[0] * (1. + mag / 2. / pi * exp((1. - r * r) / 2.) * (x - 5.));
  e[3] = pow(e[0], gamma) / g1 + 0.5 * (e[1] * e[1]) / e[0] + 0.5 * (e[2] * e[2]) / e[0];
}

void oracle_init(oracle* o) {
  const int nx = o->nx, ny = o->ny;
  memset(o->u, 0, state_len(o) * sizeof(double));
  o->time = 0.0;
  o->sweep_count = o->den_count = o->pre_count = o->fail_count = 0;
  o->status = 0;
  switch (o->problem) {
    case SWFD_PROBLEM_MATLAB_1D:
      ex1_init(o);
      break;
    case SWFD_PROBLEM_SEDOV_1D: { /* ex2_sedov_1d/main.f90:405-428 */
      double xleft = -2., xright = 2.;
      o->dx = (xright - xleft) / nx;
      for (int i = -2; i <= nx + 3; ++i) o->x[i + 2] = xleft + i * o->dx - o->dx / 2.;
      for (int i = -2; i <= nx + 3; ++i) {
        U1(o->u, 0, i) = 1.;
        U1(o->u, 1, i) = 0.;
        U1(o->u, 2, i) = o->cfg.e_background;
      }
      U1(o->u, 2, nx / 2 + 1) = o->cfg.e_blast / o->dx;
      break;
    }
    case SWFD_PROBLEM_VORTEX_2D: { /* ex3_vortex_accuracy_2d/main.f90:671-697 */
      double xleft = 0., xright = 10., yleft = 0., yright = 10.;
      o->dx = (xright - xleft) / nx;
      o->dy = (yright - yleft) / ny;
      for (int i = -2; i <= nx + 3; ++i) o->x[i + 2] = xleft + i * o->dx - o->dx / 2.;
      for (int i = -2; i <= ny + 3; ++i) o->y[i + 2] = yleft + i * o->dy - o->dy / 2.;
      for (int j = -2; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) {
          double e[4];
          vortex_exact(o, o->x[i + 2], o->y[j + 2], 0., e);
          for (int c = 0; c < 4; ++c) U(o->u, c, i, j) = e[c];
        }
      bc2d(o);
      break;
    }
    case SWFD_PROBLEM_SEDOV_2D: { /* ex4_sedov_2d/main.f90:1121-1189, one block */
      const double xm = 1.3, ym = 1.3;
      double xleft = xm / 1 * 0, xright = xm / 1 * (0 + 1);
      double yleft = ym / 1 * 0, yright = ym / 1 * (0 + 1);
      o->dx = (xright - xleft) / nx;
      o->dy = (yright - yleft) / ny;
      for (int i = -2; i <= nx + 3; ++i) o->x[i + 2] = xleft + i * o->dx - o->dx / 2.;
      for (int i = -2; i <= ny + 3; ++i) o->y[i + 2] = yleft + i * o->dy - o->dy / 2.;
      for (int j = -2; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) {
          U(o->u, 0, i, j) = 1;
          U(o->u, 3, i, j) = o->cfg.e_background;
        }
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double gx = xleft + o->dx * (i - 0.5), gy = yleft + o->dy * (j - 0.5);
          if (fabs(gx - 0.0) <= o->dx / 2.0 && fabs(gy - 0.0) <= o->dy / 2.0)
            U(o->u, 3, i, j) = o->cfg.e_blast / (o->dx * o->dy);
        }
      bc2d(o);
      break;
    }
    case SWFD_PROBLEM_SHOCK_DIFFRACTION:
      ex6_init(o);
      break;
    case SWFD_PROBLEM_DETONATION:
      ex7_init(o);
      break;
    case SWFD_PROBLEM_JET_2D: { /* ex5_mach2000_jet/main.f90:744-768; variant 1 the full
                                   domain y in [-0.25, 0.25] */
      double xleft = 0., xright = 1., yleft = o->cfg.variant == 1 ? -0.25 : 0., yright = 0.25;
      o->dx = (xright - xleft) / nx;
      o->dy = (yright - yleft) / ny;
      for (int i = -2; i <= nx + 3; ++i) o->x[i + 2] = xleft + i * o->dx - o->dx / 2.;
      for (int i = -2; i <= ny + 3; ++i) o->y[i + 2] = yleft + i * o->dy - o->dy / 2.;
      for (int j = -2; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) {
          U(o->u, 0, i, j) = 0.5;
          U(o->u, 3, i, j) = 0.4127 / o->gamma1;
        }
      bc2d(o);
      break;
    }
  }
}

/* ------------------------------------------------------------------ */
/* lifetime + accessors (ctypes surface of the oracle)                  */
/* ------------------------------------------------------------------ */
oracle* oracle_create(const swfd_config* cfg) {
  oracle* o = calloc(1, sizeof(oracle));
  o->cfg = *cfg;
  o->problem = cfg->problem;
  o->quad = cfg->literals == SWFD_LITERALS_QUAD;
  o->ndim = (cfg->problem == SWFD_PROBLEM_SEDOV_1D || cfg->problem == SWFD_PROBLEM_MATLAB_1D) ? 1 : 2;
  o->nc = o->ndim == 1 ? 3 : 4;
  o->nx = cfg->nx;
  o->ny = o->ndim == 1 ? 1 : cfg->ny;
  o->LI = o->nx + 6;
  o->LJ = o->ndim == 1 ? 1 : o->ny + 6;
  o->gamma = cfg->gamma;
  o->gamma1 = cfg->gamma - 1.;
  o->eps = 1e-13;
  o->eps2 = 1e-8;
  o->weno_eps = 1e-6;
  o->weno_eps_q = 1e-6f128;
  o->ex4like = (cfg->problem == SWFD_PROBLEM_SEDOV_2D || cfg->problem == SWFD_PROBLEM_SHOCK_DIFFRACTION);
  if (cfg->problem == SWFD_PROBLEM_DETONATION) {
    /* u(5,...), q_const = 50, t_const = 50, k_const = 2566.4, step = 2
     * (ex7_detonation/main.f90:11-19); ex6's WENO epsilon (weno5.f90:104-106) */
    o->nc = 5;
    o->qc = 50.;
    o->tc = 50.;
    o->kc = 2566.4;
    o->wall_rows = 2 * cfg->total;
  }
  if (cfg->problem == SWFD_PROBLEM_SHOCK_DIFFRACTION || cfg->problem == SWFD_PROBLEM_DETONATION) {
    /* alpha(k)=lin(k)/(1d-12+beta(k))**2 (ex6_shock_diffraction/weno5.f90:104-106,138-140) */
    o->weno_eps = 1e-12;
    o->weno_eps_q = 1e-12f128;
    o->total = cfg->total;
    o->cut_x = cfg->cut_x;
    o->cut_y = cfg->cut_y;
    o->nxl = cfg->nx / cfg->cut_x;
    o->nyl = cfg->ny / cfg->cut_y;
  }
  const size_t n = state_len(o);
  double** arrs[] = {&o->u, &o->u0, &o->rhs, &o->fp, &o->fn, &o->gp,
                     &o->gn, &o->fpf, &o->fnf, &o->gpf, &o->gnf};
  for (size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); ++k) *arrs[k] = calloc(n, sizeof(double));
  o->x = calloc(o->nx + 6, sizeof(double));
  o->y = calloc(o->ny + 6, sizeof(double));
  int mx = (o->nx > o->ny ? o->nx : o->ny) + 3;
  o->wk_w = calloc(mx, sizeof(double));
  o->wk_vx = calloc(mx, sizeof(double));
  o->wk_vy = calloc(mx, sizeof(double));
  o->wk_h = calloc(mx, sizeof(double));
  if (o->ndim == 2) {
    size_t N = (size_t)o->nx * o->ny;
    o->rho_t = calloc(N, sizeof(double));
    o->sI_i = calloc(N, sizeof(int));
    o->sI_j = calloc(N, sizeof(int));
    o->sII_i = calloc(N, sizeof(int));
    o->sII_j = calloc(N, sizeof(int));
    sweeping_order(o);
    /* weights(i,j) = 1./(nSteps_x*nSteps_y) (ex3_vortex_accuracy_2d/main.f90:44) */
    o->weight = 1. / ((double)o->nx * (double)o->ny);
    if (o->problem == SWFD_PROBLEM_DETONATION) {
      /* xleft = 5./cut_x*position_x, dx = (xright - xleft)/nx per rank
       * (ex7_detonation/main.f90:1224-1231); rank (0,0)'s for the time step */
      o->dx = (5. / o->cut_x * (0 + 1) - 5. / o->cut_x * 0) / o->nxl;
      o->dy = (5. / o->cut_y * (0 + 1) - 5. / o->cut_y * 0) / o->nyl;
      o->rk = calloc((size_t)o->cut_x * o->cut_y, sizeof(oracle*));
      for (int py = 0; py < o->cut_y; ++py)
        for (int px = 0; px < o->cut_x; ++px) {
          oracle* r = ex6_rank_create(o, px, py);
          r->dx = (5. / o->cut_x * (px + 1) - 5. / o->cut_x * px) / o->nxl;
          r->dy = (5. / o->cut_y * (py + 1) - 5. / o->cut_y * py) / o->nyl;
          o->rk[px + o->cut_x * py] = r;
        }
    } else if (o->problem == SWFD_PROBLEM_SHOCK_DIFFRACTION) {
      /* xlen = xright - xleft, dx = xlen/nx per rank (:1097-1104); rank (0,0)'s
       * for the time step, every rank's own for its flux differences */
      o->dx = (13. / o->cut_x * (0 + 1) - 13. / o->cut_x * 0) / o->nxl;
      o->dy = (11. / o->cut_y * (0 + 1) - 11. / o->cut_y * 0) / o->nyl;
      o->rk = calloc((size_t)o->cut_x * o->cut_y, sizeof(oracle*));
      for (int py = 0; py < o->cut_y; ++py)
        for (int px = 0; px < o->cut_x; ++px) {
          oracle* r = ex6_rank_create(o, px, py);
          r->dx = (13. / o->cut_x * (px + 1) - 13. / o->cut_x * px) / o->nxl;
          r->dy = (11. / o->cut_y * (py + 1) - 11. / o->cut_y * py) / o->nyl;
          o->rk[px + o->cut_x * py] = r;
        }
    }
  } else {
    o->rho_t = calloc(o->nx + 6, sizeof(double));
    /* weights(i) = 1/(nSteps + 6) (ex2_sedov_1d/main.f90:31) */
    o->weight = 1 / ((double)o->nx + 6);
  }
  return o;
}

void oracle_destroy(oracle* o) {
  if (!o) return;
  double* arrs[] = {o->u, o->u0, o->rhs, o->fp, o->fn, o->gp, o->gn, o->fpf, o->fnf, o->gpf, o->gnf,
                    o->x, o->y, o->wk_w, o->wk_vx, o->wk_vy, o->wk_h, o->rho_t};
  for (size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); ++k) free(arrs[k]);
  free(o->sI_i); free(o->sI_j); free(o->sII_i); free(o->sII_j);
  free(o->sweep_track); free(o->neg_track); free(o->pos_track);
  if (o->rk) {
    for (int k = 0; k < o->cut_x * o->cut_y; ++k) ex6_rank_destroy(o->rk[k]);
    free(o->rk);
  }
  free(o);
}

int64_t oracle_state_len(const oracle* o) { return (int64_t)state_len(o); }
void oracle_get_state(const oracle* o, double* out) { memcpy(out, o->u, state_len(o) * sizeof(double)); }
void oracle_set_state(oracle* o, const double* in) {
  memcpy(o->u, in, state_len(o) * sizeof(double));
  if (o->rk) o->ranks_stale = 1;
}
double oracle_get_time(const oracle* o) { return o->time; }
void oracle_set_time(oracle* o, double t) { o->time = t; }
double oracle_get_dt(const oracle* o) { return o->dt; }
int64_t oracle_get_restarts(const oracle* o) { return o->restarts; }
double oracle_get_alphamax(const oracle* o) { return o->alphamax; }
double oracle_get_dx(const oracle* o) { return o->dx; }
double oracle_get_dy(const oracle* o) { return o->dy; }
int oracle_get_status(const oracle* o) { return o->status; }

/* findalpha of the current state */
double oracle_find_alpha(oracle* o) {
  if (o->rk) {
    if (o->ranks_stale) ex6_distribute(o);
    double am = 0.;
    for (int k = 0; k < o->cut_x * o->cut_y; ++k)
      am = fmax(am, o->problem == SWFD_PROBLEM_DETONATION ? ex7_findalpha(o->rk[k])
                                                          : ex6_findalpha(o->rk[k]));
    return o->alphamax = am;
  }
  if (o->ndim == 1) findalpha1d(o); else findalpha2d(o);
  return o->alphamax;
}

/* wenofd + scheme of the current state; rhs in the state layout */
void oracle_flux_divergence(oracle* o, double* rhs) {
  if (o->rk) {
    if (o->ranks_stale) ex6_distribute(o);
    o->alphamax = o->problem == SWFD_PROBLEM_DETONATION ? ex7_flux_divergence(o)
                                                        : ex6_flux_divergence(o);
    memset(rhs, 0, state_len(o) * sizeof(double));
    for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
      const oracle* r = o->rk[k];
      for (int j = 1; j <= r->ny; ++j)
        for (int i = 1; i <= r->nx; ++i)
          for (int c = 0; c < o->nc; ++c)
            rhs[IX(o, c, r->px * o->nxl + i, r->py * o->nyl + j)] = r->rhs[IX(r, c, i, j)];
    }
    ex6_assemble(o); /* the wall mirrors change the state, as in the reference */
    return;
  }
  wenofd_any(o);
  scheme_any(o);
  memcpy(rhs, o->rhs, state_len(o) * sizeof(double));
}

int oracle_check_positivity(oracle* o) {
  if (o->rk) {
    if (o->ranks_stale) ex6_distribute(o);
    return o->problem == SWFD_PROBLEM_DETONATION ? ex7_checkpositivity(o)
                                                 : ex6_checkpositivity(o);
  }
  return check_any(o);
}

/* sweep_lim on the current state */
int oracle_sweep(oracle* o) {
  if (o->rk) {
    if (o->ranks_stale) ex6_distribute(o);
    ex6_gather(o);
    int st = o->problem == SWFD_PROBLEM_DETONATION ? ex7_sweep_lim(o) : sweep_lim2d(o);
    ex6_scatter(o);
    return st;
  }
  return sweep_any(o);
}

/* bc on the current state */
void oracle_bc(oracle* o) {
  if (o->rk) {
    if (o->ranks_stale) ex6_distribute(o);
    if (o->problem == SWFD_PROBLEM_DETONATION) ex7_bc(o);
    else ex6_bc(o);
    ex6_assemble(o);
    return;
  }
  bc_any(o);
}

/* stats: out[0..9] in swfd_sweep_stats order */
void oracle_get_stats(const oracle* o, int64_t* out) {
  int64_t tot = 0, mx = 0, tn = 0, mn = 0, tp = 0, mp = 0;
  for (int64_t k = 0; k < o->sweep_count; ++k) {
    tot += o->sweep_track[k];
    if (k == 0 || o->sweep_track[k] > mx) mx = o->sweep_track[k];
    tn += o->neg_track[k];
    if (k == 0 || o->neg_track[k] > mn) mn = o->neg_track[k];
    tp += o->pos_track[k];
    if (k == 0 || o->pos_track[k] > mp) mp = o->pos_track[k];
  }
  out[0] = o->sweep_count; out[1] = tot; out[2] = mx; out[3] = tn; out[4] = mn;
  int64_t den = o->den_count, pre = o->pre_count;
  if (o->rk) /* the ranks' limiter counts, summed (ex6_shock_diffraction/main.f90:1167-1173) */
    for (int k = 0; k < o->cut_x * o->cut_y; ++k) {
      den += o->rk[k]->den_count;
      pre += o->rk[k]->pre_count;
    }
  out[5] = tp; out[6] = mp; out[7] = den; out[8] = pre; out[9] = o->fail_count;
}

int64_t oracle_get_tracks(const oracle* o, int32_t* sweep, int32_t* neg, int32_t* pos, int64_t cap) {
  int64_t n = o->sweep_count < cap ? o->sweep_count : cap;
  for (int64_t k = 0; k < n; ++k) {
    if (sweep) sweep[k] = o->sweep_track[k];
    if (neg) neg[k] = o->neg_track[k];
    if (pos) pos[k] = o->pos_track[k];
  }
  return o->sweep_count;
}

/* scalar WENO entry points (weno5.f90:86-146) */
void oracle_weno5(const double* stencils, int64_t n, double weno_eps, int literals, double* uleft,
                  double* uright) {
  oracle o;
  memset(&o, 0, sizeof(o));
  o.quad = literals == SWFD_LITERALS_QUAD;
  o.weno_eps = weno_eps;
  o.weno_eps_q = (weno_eps == 1e-12) ? 1e-12f128 : 1e-6f128;
  for (int64_t k = 0; k < n; ++k) {
    if (uleft) uleft[k] = oracle_weno_left_impl(&o, stencils + 5 * k);
    if (uright) uright[k] = oracle_weno_right_impl(&o, stencils + 5 * k);
  }
}
