// swfd_api.cu -- the C ABI: handle lifetime, problem set-up, the SSP-RK3
// step/stage orchestration, the sweep driver and the statistics.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "swfd_control.h"
#include "swfd_graph.h"
#include "swfd_internal.h"
#include "swfd_ex7.h"

using namespace swfd;

namespace swfd {

// Derive the per-example switches (the reference's variant matrix) and the
// grid spacing exactly as each initdata computes it.
// Options the library implements; everything else is rejected before any
// CUDA call.
// the MATLAB script's domain and boundary treatment per `problem`
// (ex1_double_rarefaction_1d/FD_WENO_Application.m:27-150)
void matlab_domain(int variant, double* xl, double* xr) {
  const double pi = 3.141592653589793;
  *xl = 0, *xr = 2 * pi;
  if (variant == 3) *xl = -1, *xr = 1;
  else if (variant == 4) *xl = -5, *xr = 5;
  else if (variant == 5) *xl = -0.5, *xr = 0.5;
  else if (variant == 6) *xl = -3, *xr = 3;
  else if (variant == 7) *xl = -0.05, *xr = 0.05;
}
int matlab_periodic(int variant) { return variant == 1 || variant == 2 || variant == 6; }

swfd_status check_config(const swfd_config& c, std::string& err) {
  auto bad = [&](swfd_status st, const char* m) {
    err = m;
    return st;
  };
  if (c.abi_version != SWFD_ABI_VERSION) return bad(SWFD_ERR_INVALID, "abi_version mismatch");
  if (c.literals != SWFD_LITERALS_DOUBLE && c.literals != SWFD_LITERALS_QUAD)
    return bad(SWFD_ERR_INVALID, "unknown literals mode");
  if (c.literals == SWFD_LITERALS_QUAD &&
      (c.precision != SWFD_PRECISION_FP64 || c.problem == SWFD_PROBLEM_MATLAB_1D))
    return bad(SWFD_ERR_UNSUPPORTED,
               "literals QUAD: the FP64 form of the Fortran examples only");
  if (c.precision != SWFD_PRECISION_FP64 && c.precision != SWFD_PRECISION_FP32_BULK)
    return bad(SWFD_ERR_INVALID, "unknown precision");
  if (c.use_limiter != 0 && c.use_limiter != 1 && c.use_limiter != 2)
    return bad(SWFD_ERR_INVALID, "use_limiter must be 0, 1 or 2");
  if (c.ubar_mode != SWFD_UBAR_SEQUENTIAL)
    return bad(SWFD_ERR_UNSUPPORTED, "ubar_mode: only sequential is built");
  if (c.swp_num < 1) return bad(SWFD_ERR_INVALID, "swp_num must be >= 1");
  if (c.sweep_mode != SWFD_SWEEP_PARALLEL && c.sweep_mode != SWFD_SWEEP_SEQUENTIAL)
    return bad(SWFD_ERR_INVALID, "unknown sweep_mode");
  if (!(c.gamma > 1.0)) return bad(SWFD_ERR_INVALID, "gamma must be > 1");
  if (c.rk_choice < 0 || c.rk_choice > 2) return bad(SWFD_ERR_INVALID, "rk_choice must be 0, 1 or 2");
  if (c.problem == SWFD_PROBLEM_MATLAB_1D) {
    if (c.variant < 1 || c.variant > 7) return bad(SWFD_ERR_INVALID, "variant: the script's problem 1..7");
    if (c.use_limiter == 1)
      return bad(SWFD_ERR_UNSUPPORTED, "the MATLAB script has no flux limiter (use_limiter 0 or 2)");
    if (c.precision != SWFD_PRECISION_FP64)
      return bad(SWFD_ERR_UNSUPPORTED, "the MATLAB script's scheme runs in FP64 only");
    if (c.rk_choice == 2) return bad(SWFD_ERR_INVALID, "rk_choice 2 (the restart RK) exists only in ex2");
  }
  if (c.problem == SWFD_PROBLEM_JET_2D && c.variant != 0 && c.variant != 1)
    return bad(SWFD_ERR_INVALID, "variant: 0 (the reference's half domain) or 1 (full domain)");
  if (c.rk_choice == 2 && c.problem != SWFD_PROBLEM_SEDOV_1D)
    return bad(SWFD_ERR_INVALID, "rk_choice 2 (the dt-halving restart RK) exists only in ex2");
  if (c.problem == SWFD_PROBLEM_DETONATION) return ex7_check(c, err);
  if (c.problem == SWFD_PROBLEM_SHOCK_DIFFRACTION) {
    // ex6_shock_diffraction/main.f90:16-18: nx = 13*total/cut_x per rank,
    // ny = 11*total/cut_y per rank
    auto pow2 = [](int v) { return v >= 1 && (v & (v - 1)) == 0; };
    if (!pow2(c.cut_x) || !pow2(c.cut_y))
      return bad(SWFD_ERR_UNSUPPORTED, "cut_x and cut_y must be powers of two (exact rank widths)");
    if (c.total < 4) return bad(SWFD_ERR_INVALID, "total must be >= 4");
    const int nxl = 13 * c.total / c.cut_x, nyl = 11 * c.total / c.cut_y;
    if (c.nx != c.cut_x * nxl || c.ny != c.cut_y * nyl)
      return bad(SWFD_ERR_INVALID, "nx, ny must be cut_x*(13*total/cut_x), cut_y*(11*total/cut_y)");
    // the walls must lie inside single ranks, away from their ghost layers,
    // so that every rank that touches them sees the same cells
    // (the y mirror's rows 6*total-2..6*total must also stay out of the rank
    // below's ghost rows: local row >= 6)
    const int j0 = 6 * c.total - (6 * c.total - 1) / nyl * nyl;
    if (c.total > nxl - 6 || j0 < 6 || j0 > nyl - 3 || 6 * c.total >= c.ny)
      return bad(SWFD_ERR_UNSUPPORTED, "step walls too close to a rank boundary for this rank grid");
  }
  return SWFD_OK;
}

swfd_status make_params(const swfd_config& c, Params& p, std::string& err) {
  Geom& g = p.g;
  p.problem = c.problem;
  p.literals = c.literals;
  p.precision = c.precision;
  p.gamma = c.gamma;
  p.gamma1 = c.gamma - 1.;
  p.eps = 1e-13;
  p.eps2 = 1e-8;
  p.weno_eps = 1e-6;
  p.time_terminal = c.time_terminal;
  if (c.nx < 8) {
    err = "nx must be >= 8";
    return SWFD_ERR_INVALID;
  }
  switch (c.problem) {
    case SWFD_PROBLEM_MATLAB_1D: {  // FD_WENO_Application.m:170-175: h = (xR-xL)/nSteps
      g.ndim = 1;
      g.nc = 3;
      g.nx = c.nx;
      g.ny = 1;
      g.LI = c.nx + 6;
      g.LJ = 1;
      double xl, xr;
      matlab_domain(c.variant, &xl, &xr);
      p.dx = (xr - xl) / c.nx;
      p.dy = 0;
      break;
    }
    case SWFD_PROBLEM_SEDOV_1D: {
      g.ndim = 1;
      g.nc = 3;
      g.nx = c.nx;
      g.ny = 1;
      g.LI = c.nx + 6;
      g.LJ = 1;
      double xleft = -2., xright = 2.;  // ex2_sedov_1d/main.f90:408-410
      p.dx = (xright - xleft) / c.nx;
      p.dy = 0;
      p.dt_rule = 1;
      p.dt_num_x = p.dx * c.cfl;  // dt = dx*cfl/alphamax (:293)
      break;
    }
    case SWFD_PROBLEM_VORTEX_2D:
    case SWFD_PROBLEM_SEDOV_2D:
    case SWFD_PROBLEM_JET_2D:
    case SWFD_PROBLEM_SHOCK_DIFFRACTION: {
      if (c.ny < 8) {
        err = "ny must be >= 8";
        return SWFD_ERR_INVALID;
      }
      g.ndim = 2;
      g.nc = 4;
      g.nx = c.nx;
      g.ny = c.ny;
      g.LI = c.nx + 6;
      g.LJ = c.ny + 6;
      if (c.problem == SWFD_PROBLEM_VORTEX_2D) {
        p.dx = (10. - 0.) / c.nx;  // ex3_vortex_accuracy_2d/main.f90:675-681
        p.dy = (10. - 0.) / c.ny;
        p.dt_rule = 3;
        p.dt_num_x = pow(p.dx, 5. / 3.) * c.cfl;  // :572
      } else if (c.problem == SWFD_PROBLEM_SEDOV_2D) {
        const double xm = 1.3, ym = 1.3;  // ex4_sedov_2d/main.f90:20,1154-1161 (one block)
        double xleft = xm / 1 * 0, xright = xm / 1 * (0 + 1);
        double yleft = ym / 1 * 0, yright = ym / 1 * (0 + 1);
        p.dx = (xright - xleft) / c.nx;
        p.dy = (yright - yleft) / c.ny;
        p.dt_rule = 4;
        p.alpha_guarded = 1;
        p.flux_guard_eps2 = 1;
        p.roe_reg_ex4 = 1;
        p.alpha_premul = 1;
        p.pos_strict = 1;
      } else if (c.problem == SWFD_PROBLEM_SHOCK_DIFFRACTION) {
        p.cut_x = c.cut_x;
        p.cut_y = c.cut_y;
        p.nxl = c.nx / c.cut_x;
        p.nyl = c.ny / c.cut_y;
        p.total = c.total;
        // xlen = 13./cut_x*(px+1) - 13./cut_x*px, dx = xlen/nx (:1097-1104);
        // the same for every rank when cut_x, cut_y are powers of two
        p.dx = (13. / c.cut_x * (0 + 1) - 13. / c.cut_x * 0) / p.nxl;
        p.dy = (11. / c.cut_y * (0 + 1) - 11. / c.cut_y * 0) / p.nyl;
        p.dt_rule = 4;
        p.alpha_guarded = 1;
        p.flux_guard_eps2 = 1;
        p.roe_reg_ex4 = 1;
        p.alpha_premul = 1;
        p.seg_alpha = 1;
        p.sweep_check = 1;
        p.weno_eps = 1e-12;  // ex6_shock_diffraction/weno5.f90:104-106,138-140
        // Mach 5.09 post-shock state (:1113-1129)
        const double gm = c.gamma, xm1 = 5.09, ss = xm1, dri = gm, pri = 1.;
        const double ach2 = ((0.0 - ss) * (0.0 - ss)) / gm / pri * dri;
        const double ple = pri * (gm * ach2 / (gm + 1.) * 2. - (gm - 1.) / (gm + 1.));
        const double dle = dri * (gm + 1.) / 2. * ach2 / ((gm - 1.) / 2. * ach2 + 1.);
        const double ule = (0.0 - ss) / dle * dri + ss;
        p.inflow[0] = dle;
        p.inflow[1] = ule * dle;
        p.inflow[2] = 0.;
        p.inflow[3] = ple / p.gamma1 + 0.5 * dle * (ule * ule);
      } else {
        // variant 1: the full domain y in [-0.25, 0.25] (inflow for
        // |y| <= 0.05, outflow at the bottom) in place of the reference's
        // upper half with its y = 0 symmetry plane
        const double yleft = c.variant == 1 ? -0.25 : 0.;
        p.jet_full = c.variant == 1;
        p.dx = (1. - 0.) / c.nx;  // ex5_mach2000_jet/main.f90:748-754
        p.dy = (0.25 - yleft) / c.ny;
        p.dt_rule = 4;
        p.alpha_guarded = 1;
        p.pos_strict = 1;
        p.exit_ge = 1;
        // inflow rows: y(j) = yleft + j*dy - dy/2 <= 0.05 (:703); full
        // domain |y(j)| <= 0.05.  Rows jet_jmin..jet_jmax.
        p.jet_jmin = c.ny + 4;
        p.jet_jmax = -3;
        for (int j = -2; j <= c.ny + 3; ++j) {
          const double y = yleft + j * p.dy - p.dy / 2.;
          if (p.jet_full ? fabs(y) <= 0.05 : y <= 0.05) {
            p.jet_jmin = std::min(p.jet_jmin, j);
            p.jet_jmax = j;
          }
        }
        const double ujet = 800.;
        p.jet_in[0] = 5.;
        p.jet_in[1] = 5. * ujet;
        p.jet_in[2] = 0.;
        p.jet_in[3] = 0.4127 / p.gamma1 + 0.5 * (p.jet_in[1] * p.jet_in[1]) / p.jet_in[0];
        p.jet_amb[0] = 0.5;
        p.jet_amb[1] = 0.;
        p.jet_amb[2] = 0.;
        p.jet_amb[3] = 0.4127 / p.gamma1;
      }
      if (p.dt_rule == 4) {
        p.dt_num_x = p.dx * c.cfl;
        p.dt_num_y = p.dy * c.cfl;
      }
      break;
    }
    default:
      err = "unknown problem";
      return SWFD_ERR_INVALID;
  }
  g.pitch = ((g.LI + 31) / 32) * 32;
  g.plane = (int64_t)g.pitch * g.LJ;
  // cell and face indices are decomposed in 32-bit arithmetic on the device
  if ((int64_t)(g.LI + 6 * 64) * (g.LJ + 6 * 64) >= (int64_t)1 << 31) {
    err = "grid too large (cells and faces are indexed in 32 bits)";
    return SWFD_ERR_INVALID;
  }
  p.fdx_inv = (float)(1.0 / p.dx);
  p.fdy_inv = g.ndim == 2 ? (float)(1.0 / p.dy) : 0.f;
  p.stop_sweep = c.problem == SWFD_PROBLEM_SEDOV_2D || c.problem == SWFD_PROBLEM_SHOCK_DIFFRACTION;
  // the positivity limiter of the split fluxes (use_limiter 1; 1D:
  // ex2_sedov_1d/main.f90:159-245)
  p.limiter = c.use_limiter == 1;
  p.limiter_clamp = c.problem == SWFD_PROBLEM_SHOCK_DIFFRACTION;
  if (!p.seg_alpha) {
    p.cut_x = p.cut_y = 1;
    p.nxl = g.nx;
    p.nyl = g.ny;
  }
  // split / flux planes: one copy per rank segment (6 more columns per x
  // segment, 6 more rows per y segment)
  p.sg = g;
  if (g.ndim == 2) {
    p.sg.LI = g.LI + 6 * (p.cut_x - 1);
    p.sg.LJ = g.LJ + 6 * (p.cut_y - 1);
    p.sg.pitch = ((p.sg.LI + 31) / 32) * 32;
    p.sg.plane = (int64_t)p.sg.pitch * p.sg.LJ;
  }
  // DO WHILE (time <= time_terminal - 1d-10), and the literal-dependent
  // constants of the reference's -fdefault-real-8 build (1d-6, 1d-12, 1d-15,
  // 1d-8, 1d-10 and 13d0/12d0 as binary128, each the nearest binary128 to the
  // decimal value: a correctly rounded quotient of exact binary64 integers)
  p.t_loop = c.time_terminal - 1e-10;
  if (c.literals == SWFD_LITERALS_QUAD) {
    using namespace qd;
    const q128 one = from_double(1.0);
    p.quad = 1;
    p.q_c1312 = div(from_double(13.0), from_double(12.0));
    p.q_weno_eps = div(one, from_double(p.weno_eps == 1e-12 ? 1e12 : 1e6));
    p.q_1em15 = div(one, from_double(1e15));
    const q128 c8 = div(one, from_double(1e8));
    p.lim8_lt = ru(c8);  // rho < c  <=>  rho < ru(c)
    p.lim8_gt = rd(c8);  // rho > c  <=>  rho > rd(c)
    p.lim8_le = rd(c8);  // rho <= c <=>  rho <= rd(c)
    p.t_loop = rd(sub(from_double(c.time_terminal), div(one, from_double(1e10))));
  }
  return SWFD_OK;
}

// ---------------------------------------------------------------------------
// initial data on the host (same libm as the reference's gfortran runtime)
// ---------------------------------------------------------------------------
inline double sqd(double a) { return a * a; }

// exact (ex3_vortex_accuracy_2d/main.f90:699-718)
void vortex_exact(double g1, double gamma, double x, double y, double t, double* e) {
  const double pi = 3.14159265358979323846264338327950;
  double r = sqrt(sqd(x - 5. - t) + sqd(y - 5. - t));
  double mag = 10.0828;
  e[0] = pow(1 - g1 * (mag * mag) / 8. / gamma / (pi * pi) * exp(1. - r * r), 1. / g1);
  e[1] = e[0] * (1. - mag / 2. / pi * exp((1. - r * r) / 2.) * (y - 5.));
  e[2] = e[0] * (1. + mag / 2. / pi * exp((1. - r * r) / 2.) * (x - 5.));
  e[3] = pow(e[0], gamma) / g1 + 0.5 * (e[1] * e[1]) / e[0] + 0.5 * (e[2] * e[2]) / e[0];
}

// Fortran-layout initial state, ghosts included (bc is applied on the device)
void init_host_state(const Params& p, const swfd_config& cfg, double* u) {
  const Geom& g = p.g;
  const int nx = g.nx, ny = g.ny, nc = g.nc, LI = g.LI;
  auto U = [&](int c, int i, int j) -> double& {
    return u[(size_t)c + (size_t)nc * ((size_t)(i + 2) + (size_t)LI * (size_t)(j + 2))];
  };
  std::fill(u, u + (size_t)g.nc * g.LI * g.LJ, 0.0);
  switch (p.problem) {
    case SWFD_PROBLEM_MATLAB_1D: {
      // FD_WENO_Application.m:27-150,170-205: cell midpoints of xL:h:xR
      // (MATLAB's colon builds its second half from the right end a + n*d),
      // rho, v, p of the problem, then m = v*rho, E = p/(gamma-1) + rho v^2/2
      double xl, xr;
      matlab_domain(cfg.variant, &xl, &xr);
      const double h = p.dx, hi = xl + nx * h, gm = p.gamma;
      for (int i = 1; i <= nx; ++i) {
        const int k0 = i - 1, k1 = i;
        const double x0 = (2 * k0 <= nx) ? xl + k0 * h : hi - (nx - k0) * h;
        const double x1 = (2 * k1 <= nx) ? xl + k1 * h : hi - (nx - k1) * h;
        const double x = (x0 + x1) / 2;
        const int i1 = x <= 0, i2 = x > 0;
        double ro = 0, v = 0, pr = 0;
        switch (cfg.variant) {
          case 1: ro = 1 + 0.2 * sin(x), v = 1, pr = 1; break;
          case 2:
            ro = 1 + 1. / 2. * sin(x), v = 1. / 2. * sin(x), pr = pow(1 + 1. / 2. * sin(x), gm);
            break;
          case 3: ro = 0 + 1 * i1 + 0.125 * i2, v = 0, pr = 0 + 1 * i1 + 0.1 * i2; break;
          case 4:
            ro = 0 + 0.445 * i1 + 0.5 * i2, v = 0 + 0.698 * i1 + 0 * i2;
            pr = 0 + 3.528 * i1 + 0.571 * i2;
            break;
          case 5:
            ro = 0 + 7 * i1 + 7 * i2, v = 0 + -1 * i1 + 1 * i2, pr = 0 + 0.2 * i1 + 0.2 * i2;
            break;
          case 6: {
            const int j1 = x >= (-2. / 402.), j2 = x > (2. / 402.);
            const double e0 = 0 + (3200000. * 201.) * j1 - (3200000. * 201.) * j2 + 1e-12 * 1;
            ro = 1, v = 0;
            pr = (gm - 1) * (e0 - 1. / 2. * ro * (v * v));
            break;
          }
          default: ro = 5, v = 0, pr = 0.4127; break;
        }
        U(0, i, -2) = ro;
        U(1, i, -2) = v * ro;
        U(2, i, -2) = pr / (gm - 1) + 1. / 2. * ro * (v * v);
      }
      // the ghosts hold FD_WENO_Step's padding (wrap or constant extension)
      const int per = matlab_periodic(cfg.variant);
      for (int k = 1; k <= 3; ++k)
        for (int c = 0; c < 3; ++c) {
          U(c, k - 3, -2) = U(c, per ? nx - 3 + k : 1, -2);
          U(c, nx + k, -2) = U(c, per ? k : nx, -2);
        }
      break;
    }
    case SWFD_PROBLEM_SEDOV_1D:  // ex2_sedov_1d/main.f90:405-428
      for (int i = -2; i <= nx + 3; ++i) {
        U(0, i, -2) = 1.;
        U(1, i, -2) = 0.;
        U(2, i, -2) = cfg.e_background;
      }
      U(2, nx / 2 + 1, -2) = cfg.e_blast / p.dx;
      break;
    case SWFD_PROBLEM_VORTEX_2D:  // ex3_vortex_accuracy_2d/main.f90:683-694
      for (int j = -2; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) {
          double x = 0. + i * p.dx - p.dx / 2., y = 0. + j * p.dy - p.dy / 2., e[4];
          vortex_exact(p.gamma1, p.gamma, x, y, 0., e);
          for (int c = 0; c < 4; ++c) U(c, i, j) = e[c];
        }
      break;
    case SWFD_PROBLEM_SEDOV_2D:  // ex4_sedov_2d/main.f90:1170-1186
      for (int j = -2; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) {
          U(0, i, j) = 1;
          U(3, i, j) = cfg.e_background;
        }
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double gx = 0. + p.dx * (i - 0.5), gy = 0. + p.dy * (j - 0.5);
          if (fabs(gx - 0.0) <= p.dx / 2.0 && fabs(gy - 0.0) <= p.dy / 2.0)
            U(3, i, j) = cfg.e_blast / (p.dx * p.dy);
        }
      break;
    case SWFD_PROBLEM_JET_2D:  // ex5_mach2000_jet/main.f90:763-765
      for (int j = -2; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) {
          U(0, i, j) = 0.5;
          U(3, i, j) = 0.4127 / p.gamma1;
        }
      break;
    case SWFD_PROBLEM_SHOCK_DIFFRACTION:  // ex6_shock_diffraction/main.f90:1132-1148
      // post-shock state for i <= total/2 at or above row 6*total (on the
      // ranks of column 0), pre-shock state elsewhere; ghosts included, no bc
      for (int j = -2; j <= ny + 3; ++j)
        for (int i = -2; i <= nx + 3; ++i) {
          const bool post = i <= p.total / 2 && j >= p.total * 6;
          for (int c = 0; c < 4; ++c)
            U(c, i, j) = post ? p.inflow[c] : (c == 0 ? p.gamma : (c == 3 ? 1. / p.gamma1 : 0.));
        }
      break;
  }
}

}  // namespace swfd

namespace {
thread_local std::string g_last_error;
}  // namespace

void swfd::set_last_error(const std::string& m) { g_last_error = m; }

namespace {

swfd_status fail(swfd_handle* h, swfd_status st, const std::string& msg) {
  if (h) h->last_error = msg;
  g_last_error = msg;
  return st;
}

#define CU(h, call)                                                                 \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail((h), e_ == cudaErrorMemoryAllocation ? SWFD_ERR_OOM : SWFD_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(e_));              \
  } while (0)

// launch `call`, which issues n kernels of this library, and count them
#define LAUNCH(h, n, call)            \
  do {                                \
    CU((h), (call));                  \
    (h)->prof.kernel_launches += (n); \
  } while (0)

#define ST(call)                          \
  do {                                    \
    swfd_status s_ = (call);              \
    if (s_ != SWFD_OK) return s_;         \
  } while (0)

int64_t host_len(const Params& p) { return (int64_t)p.g.nc * p.g.LI * p.g.LJ; }

// ---------------------------------------------------------------------------
// initial data on the host (same libm as the reference's gfortran runtime)
// ---------------------------------------------------------------------------

// Fortran-layout initial state of the handle's problem
void init_host(const swfd_handle* h, double* u) { swfd::init_host_state(h->p, h->cfg, u); }

double* cur_state(swfd_handle* h) { return h->st[h->cur]; }

swfd_status sync_scalars(swfd_handle* h) {
  CU(h, cudaMemcpyAsync(h->hsc, h->dsc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  h->time = h->hsc->time;
  return SWFD_OK;
}

// report (and clear) the error bits the device set during the last launch
swfd_status check_device_error(swfd_handle* h) {
  ST(sync_scalars(h));
  int e = h->hsc->error;
  if (!e) return SWFD_OK;
  CU(h, cudaMemsetAsync(&h->dsc->error, 0, sizeof(int), h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  h->hsc->error = 0;
  if (e & ERR_BIT_TIMEOUT)
    return fail(h, SWFD_ERR_TIMEOUT, "device-side wait timed out (persistent 1D solve barrier)");
  if (e & ERR_BIT_RESTART)
    return fail(h, SWFD_ERR_RESTART_LIMIT, "restart RK: no positive state within "
                                           "SWFD_RESTART_LIMIT dt halvings");
  if (e & ERR_BIT_CHECK)
    return fail(h, SWFD_ERR_SWEEP_CHECK,
                "Sweep check failed: total pressure increased after adjustment");
  if (e & ERR_BIT_PUBAR) return fail(h, SWFD_ERR_PUBAR_NONPOS, "P(u_bar) <= 0");
  if (e & ERR_BIT_NOCONV) return fail(h, SWFD_ERR_SWEEP_NOCONV, "SWEEP FAIL: swp_num reached");
  return fail(h, SWFD_ERR_NONFINITE,
              std::string("non-finite ") + ((e & ERR_BIT_ALPHA) ? "alphamax" : "dt") + " on the device");
}

swfd_status finish_pending(swfd_handle* h);

// a call that reads or writes the handle's state first finishes the steps
// swfd_step_async enqueued (their status is reported here)
#define SETTLE(h)                               \
  do {                                          \
    if ((h)->pending) ST(finish_pending(h));    \
  } while (0)

// the device track arrays must hold sweep_count + extra entries
swfd_status ensure_tracks(swfd_handle* h, int64_t extra) {
  ST(sync_scalars(h));
  int64_t need = h->hsc->sweep_count + extra;
  if (need <= h->track_cap) return SWFD_OK;
  int64_t cap = std::max<int64_t>(need, 2 * h->track_cap + 1024);
  int* nt = nullptr;
  CU(h, cudaMalloc(&nt, 3 * cap * sizeof(int)));
  CU(h, cudaMemsetAsync(nt, 0, 3 * cap * sizeof(int), h->stream));
  if (h->d_tracks)
    for (int k = 0; k < 3; ++k)
      CU(h, cudaMemcpyAsync(nt + k * cap, h->d_tracks + k * h->track_cap,
                            h->track_cap * sizeof(int), cudaMemcpyDeviceToDevice, h->stream));
  CU(h, cudaMemcpyAsync(&h->dsc->tracks, &nt, sizeof(int*), cudaMemcpyHostToDevice, h->stream));
  long long c = cap;
  CU(h, cudaMemcpyAsync(&h->dsc->track_cap, &c, sizeof(long long), cudaMemcpyHostToDevice,
                        h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  cudaFree(h->d_tracks);
  h->d_tracks = nt;
  h->track_cap = cap;
  return SWFD_OK;
}

// sweep_lim (ex3_vortex_accuracy_2d/main.f90:888-1137; 1D ex2_sedov_1d/main.f90:564-726;
// ex4 P(u_bar) check :1447-1454 and stop :1747-1752; ex5 `>=` exit :1162)
void emit_sweep(Builder& b, cudaStream_t s, double* u) {
  swfd_handle* h = b.h;
  const Params& p = h->p;
  const bool seq = h->cfg.sweep_mode == SWFD_SWEEP_SEQUENTIAL;
  int* saved = b.count;
  h->k_density = 0;
  h->k_q = 0;
  auto density = [&](cudaStream_t sd) {
    b.count = &h->k_density;
    if (seq) {
      B_OK(b, launch_density_sweep(p, u, sd));
      b.k(1);
    } else {
      int n = 0;
      B_OK(b, launch_density_sweep_par(p, u, h->sweep_scratch, h->sweep_cluster, sd, &n));
      b.k(n);
    }
    if (p.g.ndim == 1) {
      B_OK(b, launch_count_density(h->dsc, sd));
      b.k(1);
    }
    b.count = saved;
  };
  if (p.g.ndim == 1) {
    density(s);
  } else {
    B_OK(b, launch_rho_min(p, u, h->dsc, s));
    cudaGraphConditionalHandle hd = b.handle();
    B_OK(b, launch_cond_density(hd, h->dsc, s));
    b.k(2);
    b.cond(s, cudaGraphCondTypeIf, hd, density);
  }
  B_OK(b, launch_ubar(p, u, h->dsc, h->ubar_scratch, s));
  cudaGraphConditionalHandle hw = b.handle();
  B_OK(b, launch_sweep_begin(hw, p, h->dsc, p.stop_sweep, h->cfg.swp_num, s));
  B_OK(b, cudaMemsetAsync(&h->dsc->t_pos, 0, 2 * sizeof(long long), s));
  b.k(4);  // u_bar's three kernels and sweep_begin
  b.cond(s, cudaGraphCondTypeWhile, hw, [&](cudaStream_t sq) {
    b.count = &h->k_q;
    B_OK(b, launch_q_begin(p, h->dsc, sq));
    b.k(1);
    if (seq) {
      B_OK(b, launch_pressure_pass(p, u, -1, 1, h->dsc, sq));
      B_OK(b, launch_pressure_pass(p, u, -1, 0, h->dsc, sq));
      b.k(2);
    } else {
      int n = 0;
      B_OK(b, launch_pressure_pass_par(p, u, -1, 1, h->sweep_scratch, h->sweep_cluster, h->dsc,
                                       sq, &n));
      B_OK(b, launch_pressure_pass_par(p, u, -1, 0, h->sweep_scratch, h->sweep_cluster, h->dsc,
                                       sq, &n));
      b.k(n);
    }
    B_OK(b, launch_exit_count(p, u, h->dsc, sq));
    B_OK(b, launch_q_end(hw, h->dsc, h->cfg.swp_num, p.stop_sweep, sq));
    b.k(2);
    b.count = saved;
  });
}

// one RK stage: findalpha, [dt], LF split, WENO fluxes, RHS + RK combination +
// checkpositivity, [sweep], bc  (ex3_vortex_accuracy_2d/main.f90:564-632)
// the bc of stages 1 and 2 carries the next stage's findalpha (2D problems
// without rank segments); stage 1's findalpha, which also sets dt, stays apart
bool fused_alpha(const Params& p) { return p.g.ndim == 2 && !p.seg_alpha; }

// The FP32-bulk fused stage: findalpha + terms (stage 1, with dt), the
// stage kernel, [sweep], bc + the next stage's findalpha + terms (stages 1
// and 2) or the bc alone (stage 3).  The split planes hold the terms.
void emit_stage32(Builder& b, cudaStream_t s, int k, double* in, double* u0, double* out,
                  bool events) {
  swfd_handle* h = b.h;
  const Params& p = h->p;
  if (k == 1) {
    B_OK(b, launch_alpha_terms32(p, in, h->dsc, s, false, true, h->split, h->roe));
    b.k(1);
  }
  if (events)
    B_OK(b, b.eager ? cudaEventRecord(h->ev[2 * (k - 1)], s)
                    : cudaEventRecordWithFlags(h->ev[2 * (k - 1)], s, cudaEventRecordExternal));
  const bool sweeps = h->cfg.use_limiter == 2;
  const cudaGraphConditionalHandle hs = sweeps ? b.handle() : 0;
  B_OK(b, launch_stage32(p, h->stage32, k, in, u0, h->split, h->roe, h->dsc, out, s, hs,
                         sweeps ? 1 : 0));
  b.k(1);
  if (events)
    B_OK(b, b.eager ? cudaEventRecord(h->ev[2 * (k - 1) + 1], s)
                    : cudaEventRecordWithFlags(h->ev[2 * (k - 1) + 1], s,
                                               cudaEventRecordExternal));
  if (sweeps) {
    int* saved = b.count;
    h->k_sweep_fixed = 0;
    b.count = &h->k_sweep_fixed;
    b.cond(s, cudaGraphCondTypeIf, hs, [&](cudaStream_t sw) { emit_sweep(b, sw, out); });
    b.count = saved;
  }
  if (k < 3) B_OK(b, launch_alpha_terms32(p, out, h->dsc, s, true, false, h->split, h->roe));
  else B_OK(b, launch_bc(p, out, s));
  b.k(1);
}

void emit_stage(Builder& b, cudaStream_t s, int k, double* in, double* u0, double* out,
                bool events) {
  swfd_handle* h = b.h;
  const Params& p = h->p;
  if (h->stage32) return emit_stage32(b, s, k, in, u0, out, events);
  if (k == 1 || !fused_alpha(p)) {
    B_OK(b, launch_alpha(p, in, h->dsc, s, k == 1));
    b.k(1);
  }
  {
    int nk = 0;
    B_OK(b, launch_split(p, in, h->dsc, h->split, h->roe, s, &nk));
    b.k(nk);
  }
  // external event-record nodes (a plain record on a capturing stream would
  // only be a capture dependency)
  if (events)
    B_OK(b, b.eager ? cudaEventRecord(h->ev[2 * (k - 1)], s)
                    : cudaEventRecordWithFlags(h->ev[2 * (k - 1)], s, cudaEventRecordExternal));
  B_OK(b, launch_flux(p, h->split, p.g.ndim == 1 ? in : h->roe, h->dsc, h->flux, &h->dsc->flux_work, s));
  b.k(1);
  if (events)
    B_OK(b, b.eager ? cudaEventRecord(h->ev[2 * (k - 1) + 1], s)
                    : cudaEventRecordWithFlags(h->ev[2 * (k - 1) + 1], s,
                                               cudaEventRecordExternal));
  const bool sweeps = h->cfg.use_limiter == 2;
  const cudaGraphConditionalHandle hs = sweeps ? b.handle() : 0;
  B_OK(b, launch_rk(p, k, in, u0, h->flux, h->dsc, out, s, hs, sweeps ? 1 : 0));
  b.k(1);
  if (sweeps) {
    int* saved = b.count;
    h->k_sweep_fixed = 0;  // every stage emits the same sweep: count it once
    b.count = &h->k_sweep_fixed;
    b.cond(s, cudaGraphCondTypeIf, hs, [&](cudaStream_t sw) { emit_sweep(b, sw, out); });
    b.count = saved;
  }
  if (p.g.ndim == 2) {
    if (k < 3 && fused_alpha(p)) B_OK(b, launch_bc_alpha(p, out, h->dsc, s));
    else B_OK(b, launch_bc(p, out, s));
    b.k(1);
  }
}

// The dt-halving restart RK of ex2 (rk_choice 2, ex2_sedov_1d/main.f90:330-374):
//   wenofd(X); dt; alphatemp = alphamax
//   WHILE (restart) { [dt = dt/2, alphamax = alphatemp]; stage 1: X -> Y;
//     IF (positive) { wenofd(Y); stage 2: Y, X -> Z;
//       IF (positive) { wenofd(Z); stage 3: Z, X -> Y } }
//     restart = !positive }
//   X = Y
// The loop never overwrites u0 = X (stage 3 writes Y), so the reference's
// `u = u0` needs no copy, and a restarted stage 1 uses the fluxes of the
// last wenofd, as the reference's does.  ex2's bc is a no-op; no sweeps.
void emit_step_restart(Builder& b, cudaStream_t s) {
  swfd_handle* h = b.h;
  const Params& p = h->p;
  double* X = h->st[h->cur];
  double* Y = h->st[(h->cur + 1) % 3];
  double* Z = h->st[(h->cur + 2) % 3];
  int* saved = b.count;
  auto wenofd = [&](cudaStream_t sx, double* in, bool with_dt) {
    B_OK(b, launch_alpha(p, in, h->dsc, sx, with_dt));
    int nk = 0;
    B_OK(b, launch_split(p, in, h->dsc, h->split, h->roe, sx, &nk));
    B_OK(b, launch_flux(p, h->split, p.g.ndim == 1 ? in : h->roe, h->dsc, h->flux,
                        &h->dsc->flux_work, sx));
    b.k(2 + nk);
  };
  h->k_rs_fixed = 0;
  b.count = &h->k_rs_fixed;
  wenofd(s, X, true);
  const cudaGraphConditionalHandle hw = b.handle();
  B_OK(b, launch_restart_init(hw, h->dsc, s));
  b.k(1);
  b.cond(s, cudaGraphCondTypeWhile, hw, [&](cudaStream_t sl) {
    h->k_rs_iter = 0;
    b.count = &h->k_rs_iter;
    B_OK(b, launch_restart_begin(h->dsc, sl));
    const cudaGraphConditionalHandle h2 = b.handle();
    B_OK(b, launch_rk(p, 1, X, X, h->flux, h->dsc, Y, sl, h2, 2));
    b.k(2);
    b.cond(sl, cudaGraphCondTypeIf, h2, [&](cudaStream_t s2) {
      h->k_rs_s2 = 0;
      b.count = &h->k_rs_s2;
      wenofd(s2, Y, false);
      const cudaGraphConditionalHandle h3 = b.handle();
      B_OK(b, launch_rk(p, 2, Y, X, h->flux, h->dsc, Z, s2, h3, 2));
      b.k(1);
      b.cond(s2, cudaGraphCondTypeIf, h3, [&](cudaStream_t s3) {
        h->k_rs_s3 = 0;
        b.count = &h->k_rs_s3;
        wenofd(s3, Z, false);
        B_OK(b, launch_rk(p, 3, Z, X, h->flux, h->dsc, Y, s3, 0, 0));
        b.k(1);
      });
    });
    b.count = &h->k_rs_iter;
    B_OK(b, launch_restart_end(hw, h->dsc, sl));
    b.k(1);
  });
  b.count = &h->k_rs_fixed;
  B_OK(b, launch_restart_commit(p, Y, X, h->dsc, s));
  b.k(1);
  b.count = saved;
}

void emit_step(Builder& b, cudaStream_t s, bool events) {
  swfd_handle* h = b.h;
  if (h->cfg.rk_choice == 2) {
    emit_step_restart(b, s);
    return;
  }
  double* X = h->st[h->cur];
  double* Y = h->st[(h->cur + 1) % 3];
  double* Z = h->st[(h->cur + 2) % 3];
  int* saved = b.count;
  h->k_stage = 0;
  b.count = &h->k_stage;  // the three stages, sweeps counted apart
  emit_stage(b, s, 1, X, X, Y, events);
  emit_stage(b, s, 2, Y, X, Z, events);
  emit_stage(b, s, 3, Z, X, X, events);
  b.count = saved;
}

enum { GRAPH_STEP = 0, GRAPH_SOLVE = 1, GRAPH_SWEEP = 2 };

// the work of one graph kind, emitted into a capture or launched eagerly
void emit_kind(Builder& b, cudaStream_t s, int kind) {
  swfd_handle* h = b.h;
  if (kind == GRAPH_STEP) {
    emit_step(b, s, h->prof_on != 0);  // the flux events only when profiling
    B_OK(b, launch_time_advance(h->dsc, s));
    b.k(1);
  } else if (kind == GRAPH_SOLVE) {
    B_OK(b, cudaMemsetAsync(&h->dsc->steps, 0, sizeof(long long), s));
    cudaGraphConditionalHandle hr = b.handle();
    B_OK(b, launch_run_cond(hr, h->dsc, h->p.t_loop, s));
    b.k(1);
    b.cond(s, cudaGraphCondTypeWhile, hr, [&](cudaStream_t sb) {
      emit_step(b, sb, false);
      B_OK(b, launch_time_advance_cond(hr, h->dsc, h->p.t_loop, sb));
      b.k(1);
    });
  } else {
    h->k_sweep_fixed = 0;
    b.count = &h->k_sweep_fixed;
    emit_sweep(b, s, h->st[h->cur]);
  }
}

swfd_status build_graph(swfd_handle* h, int kind, cudaGraphExec_t* out) {
  if (*out || h->eager) return SWFD_OK;
  Builder b;
  b.h = h;
  b.cap = h->cap;
  b.max_depth = SWFD_CAP_DEPTH - 1;
  cudaStream_t s = h->cap[0];
  CU(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  cudaStreamCaptureStatus cs;
  b.ok(cudaStreamGetCaptureInfo(s, &cs, nullptr, &b.root, nullptr, nullptr, nullptr));
  emit_kind(b, s, kind);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (b.err != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(h, SWFD_ERR_CUDA,
                std::string("graph capture: ") +
                    cudaGetErrorString(b.err != cudaSuccess ? b.err : e2));
  }
  cudaError_t e3 = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e3 != cudaSuccess)
    return fail(h, SWFD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
  return SWFD_OK;
}

// run one graph kind: launch its graph, or (eager mode) its kernels directly
swfd_status launch_kind(swfd_handle* h, int kind, cudaGraphExec_t g) {
  if (!h->eager) {
    CU(h, cudaGraphLaunch(g, h->stream));
    return SWFD_OK;
  }
  Builder b;
  b.h = h;
  b.eager = true;
  b.cond_word = &h->dsc->cond;
  b.launched = &h->eager_launches;
  emit_kind(b, h->stream, kind);
  if (b.err != cudaSuccess)
    return fail(h, SWFD_ERR_CUDA, std::string("eager launch: ") + cudaGetErrorString(b.err));
  return SWFD_OK;
}

// kernels run by a launch, from the counters' increments (a step: its three
// stages and the time advance; a sweep: its fixed part, the density sweep if
// it ran, and one body per iteration q)
void account(swfd_handle* h, const DevScalars& before, const DevScalars& after, int64_t steps,
             int64_t extra) {
  int64_t sweeps = after.sweep_count - before.sweep_count;
  int64_t dens = after.den_count - before.den_count;
  int64_t qs = after.pre_count - before.pre_count;
  if (h->eager) {  // counted as launched
    h->prof.kernel_launches += h->eager_launches;
    h->eager_launches = 0;
  } else if (h->cfg.rk_choice == 2) {
    const int64_t it = after.rk_runs[1] - before.rk_runs[1];
    const int64_t s2 = after.rk_runs[2] - before.rk_runs[2];
    const int64_t s3 = after.rk_runs[3] - before.rk_runs[3];
    h->prof.kernel_launches += steps * (h->k_rs_fixed + 1) + it * h->k_rs_iter +
                               s2 * h->k_rs_s2 + s3 * h->k_rs_s3 + extra;
  } else {
    h->prof.kernel_launches += steps * (h->k_stage + 1) + sweeps * h->k_sweep_fixed +
                               dens * h->k_density + qs * h->k_q + extra;
  }
  h->prof.stages += 3 * steps;
  h->prof.sweep_invocations += sweeps;
}

// write the host-held parts of the device scalars (tracks) after a reset
swfd_status reset_scalars(swfd_handle* h) {
  memset(h->hsc, 0, sizeof(DevScalars));
  h->hsc->tracks = h->d_tracks;
  h->hsc->track_cap = h->track_cap;
  CU(h, cudaMemcpyAsync(h->dsc, h->hsc, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream));
  if (h->d_tracks)
    CU(h, cudaMemsetAsync(h->d_tracks, 0, 3 * h->track_cap * sizeof(int), h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  h->time = 0;
  return SWFD_OK;
}

swfd_status finish_pending(swfd_handle* h) {
  const int64_t n = h->pending;
  h->pending = 0;
  swfd_status st = check_device_error(h);
  account(h, h->pending_before, *h->hsc, n, 0);
  if (h->prof_on && h->cfg.rk_choice != 2) {  // the last step's flux launches
    for (int k = 0; k < 3; ++k) {
      float ms = 0.f;
      CU(h, cudaEventElapsedTime(&ms, h->ev[2 * k], h->ev[2 * k + 1]));
      h->prof.flux_ms += ms;
      h->prof.flux_launches += 1;
    }
  }
  return st;
}

// The 1D solve as persistent launches (swfd_solve1d.cu): one cooperative
// launch runs the time loop on the device; a stage whose checkpositivity
// fails ends it, sweep_lim runs on that stage's output as plain launches
// (the conditions read on the host) and the next launch resumes at the
// following stage.  SWFD_SOLVE1D=graph keeps the graph kernels.
bool use_solve1d(swfd_handle* h, Solve1dShape* sh) {
  if (h->cfg.rk_choice == 2 || h->s1_refused) return false;
  const char* env = getenv("SWFD_SOLVE1D");
  if (env && strcmp(env, "graph") == 0) return false;
  return solve1d_shape(h->p, sh);
}

swfd_status run_solve1d(swfd_handle* h, const Solve1dShape& sh, int64_t max_steps,
                        int64_t* nsteps_out) {
  const size_t pre_bytes = 2 * (size_t)h->p.g.LI * SWFD_SOLVE1D_PRE * sizeof(double);
  // the reduction words (three per block) and the ready flags (one per
  // block), at most one block per cell
  const size_t LI = (size_t)h->p.g.LI;
  if (!h->s1_scratch)
    CU(h, cudaMalloc(&h->s1_scratch,
                     pre_bytes + 3 * LI * SWFD_SOLVE1D_WSTRIDE * sizeof(unsigned long long) +
                         LI * sizeof(unsigned)));
  Solve1dArgs a;
  for (int k = 0; k < 3; ++k) a.st[k] = h->st[(h->cur + k) % 3];
  a.pre = (double*)h->s1_scratch;
  a.red = (unsigned long long*)((char*)h->s1_scratch + pre_bytes);
  a.ready = (unsigned*)(a.red + 3 * LI * SWFD_SOLVE1D_WSTRIDE);
  a.cells = sh.cells;
  a.sweeps = h->cfg.use_limiter == 2;
  int64_t done = 0;
  const int64_t chunk = 4096;  // steps per launch sequence (bounds the track growth)
  swfd_status st = SWFD_OK;
  while (h->time <= h->p.t_loop) {
    if (max_steps > 0 && done >= max_steps) {
      st = SWFD_ERR_MAX_STEPS;
      break;
    }
    long long lim = (long long)(max_steps > 0 ? std::min<int64_t>(chunk, max_steps - done) : chunk);
    ST(ensure_tracks(h, 3 * lim));
    const DevScalars before = *h->hsc;
    CU(h, cudaMemcpyAsync(&h->dsc->steps_limit, &lim, sizeof(long long), cudaMemcpyHostToDevice,
                          h->stream));
    CU(h, cudaMemsetAsync(&h->dsc->steps, 0, sizeof(long long), h->stream));
    a.resume = 1;
    for (;;) {
      const cudaError_t le = launch_solve1d(h->p, sh, a, h->dsc, h->stream);
      if (le == cudaErrorCooperativeLaunchTooLarge && done == 0 && a.resume == 1) {
        // the grid cannot be resident at once here (another context holds
        // SMs): nothing ran; the caller takes the graph kernels
        cudaGetLastError();
        h->s1_refused = 1;
        if (nsteps_out) *nsteps_out = 0;
        return SWFD_OK;
      }
      CU(h, le);
      h->prof.kernel_launches += 1;
      st = check_device_error(h);
      const int pause = h->hsc->solve_pause;
      if (st != SWFD_OK || !pause) break;
      // sweep_lim on the output of stage `pause`
      Builder b;
      b.h = h;
      b.eager = true;
      b.cond_word = &h->dsc->cond;
      b.launched = &h->eager_launches;
      emit_sweep(b, h->stream, a.st[pause % 3]);
      if (b.err != cudaSuccess)
        return fail(h, SWFD_ERR_CUDA, std::string("1D sweep: ") + cudaGetErrorString(b.err));
      h->prof.kernel_launches += h->eager_launches;
      h->eager_launches = 0;
      st = check_device_error(h);
      if (st != SWFD_OK) break;
      a.resume = pause + 1;
    }
    const int64_t steps = h->hsc->steps;
    h->prof.stages += 3 * steps;
    h->prof.sweep_invocations += h->hsc->sweep_count - before.sweep_count;
    done += steps;
    if (st != SWFD_OK) break;
    if (steps < lim) break;  // the time test ended the loop
  }
  if (nsteps_out) *nsteps_out = done;
  return st;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* swfd_status_string(swfd_status s) {
  switch (s) {
    case SWFD_OK: return "ok";
    case SWFD_ERR_INVALID: return "invalid argument";
    case SWFD_ERR_CUDA: return "CUDA error";
    case SWFD_ERR_SWEEP_NOCONV: return "sweep did not converge within swp_num";
    case SWFD_ERR_PUBAR_NONPOS: return "P(u_bar) <= 0";
    case SWFD_ERR_NONFINITE: return "non-finite alpha or dt";
    case SWFD_ERR_OOM: return "device allocation failed";
    case SWFD_ERR_TIMEOUT: return "device-side wait timed out";
    case SWFD_ERR_UNSUPPORTED: return "unsupported option";
    case SWFD_ERR_MAX_STEPS: return "step limit reached";
    case SWFD_ERR_SWEEP_CHECK: return "sweep check failed: total pressure increased";
    case SWFD_ERR_RESTART_LIMIT: return "restart RK: dt-halving limit reached";
    default: return "unknown status";
  }
}

swfd_status swfd_config_default(swfd_config* cfg, int32_t problem) {
  if (!cfg) return fail(nullptr, SWFD_ERR_INVALID, "cfg is NULL");
  memset(cfg, 0, sizeof(*cfg));
  cfg->abi_version = SWFD_ABI_VERSION;
  cfg->problem = problem;
  cfg->use_limiter = 2;
  cfg->swp_num = 20000;
  cfg->literals = SWFD_LITERALS_DOUBLE;
  cfg->precision = SWFD_PRECISION_FP64;
  cfg->ubar_mode = SWFD_UBAR_SEQUENTIAL;
  cfg->device = 0;
  cfg->gamma = 1.4;
  cfg->rk_choice = 1;
  switch (problem) {
    case SWFD_PROBLEM_SEDOV_1D:  // ex2_sedov_1d/main.f90:4-7,423-425
      cfg->nx = 800;
      cfg->ny = 1;
      cfg->swp_num = 50;
      cfg->cfl = 1.2;
      cfg->time_terminal = 0.001;
      cfg->e_background = 1e-9 / (1.4 - 1.);
      cfg->e_blast = 3200000.0;
      break;
    case SWFD_PROBLEM_VORTEX_2D:  // ex3_vortex_accuracy_2d/main.f90:5-7,570
      cfg->nx = cfg->ny = 180;
      cfg->cfl = 0.5;
      cfg->time_terminal = 0.01;
      break;
    case SWFD_PROBLEM_SEDOV_2D:  // ex4_sedov_2d/main.f90:18-20,687,1172,1182
      cfg->nx = cfg->ny = 640;
      cfg->cfl = 0.5;
      cfg->time_terminal = 1;
      cfg->e_background = 1e-12;
      cfg->e_blast = 0.244816;
      break;
    case SWFD_PROBLEM_JET_2D:  // ex5_mach2000_jet/main.f90:4-6,597
      cfg->nx = 800;
      cfg->ny = 200;
      cfg->cfl = 1. / 4.;
      cfg->time_terminal = 0.001;
      cfg->gamma = 5. / 3.;
      break;
    case SWFD_PROBLEM_MATLAB_1D:  // FD_WENO_Application.m:10,95-110,158-165 (problem = 5)
      cfg->variant = 5;
      cfg->nx = 200;
      cfg->ny = 1;
      cfg->swp_num = 200000;
      cfg->cfl = 0.85;
      cfg->time_terminal = 0.3;
      break;
    case SWFD_PROBLEM_SHOCK_DIFFRACTION:  // ex6_shock_diffraction/main.f90:16-20,695
      cfg->total = 80;
      cfg->cut_x = 4;
      cfg->cut_y = 8;
      cfg->nx = 4 * (13 * 80 / 4);
      cfg->ny = 8 * (11 * 80 / 8);
      cfg->cfl = 0.9;
      cfg->time_terminal = 2.3;
      break;
    case SWFD_PROBLEM_DETONATION:  // ex7_detonation/main.f90:11-19,43,812
      cfg->total = 80;
      cfg->cut_x = 4;
      cfg->cut_y = 8;
      cfg->nx = 4 * (5 * 80 / 4);
      cfg->ny = 8 * (5 * 80 / 8);
      cfg->cfl = 0.88;
      cfg->time_terminal = 0.6;
      cfg->gamma = 1.2;
      break;
    default:
      return fail(nullptr, SWFD_ERR_INVALID, "unknown problem");
  }
  return SWFD_OK;
}

swfd_status swfd_create(const swfd_config* cfg, swfd_handle** out) {
  if (!cfg || !out) return fail(nullptr, SWFD_ERR_INVALID, "NULL argument");
  *out = nullptr;
  std::string err;
  swfd_status st = check_config(*cfg, err);
  if (st != SWFD_OK) return fail(nullptr, st, err);
  if (cfg->problem == SWFD_PROBLEM_DETONATION) {  // its own rank-sliced engine
    swfd_handle* h = new swfd_handle();
    h->cfg = *cfg;
    h->device = cfg->device;
    const char* lm = getenv("SWFD_LAUNCH");  // eager: plain launches (for profilers)
    h->eager = lm && strcmp(lm, "eager") == 0;
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    for (int k = 0; k < SWFD_CAP_DEPTH && e == cudaSuccess; ++k)  // graph capture streams
      e = cudaStreamCreateWithFlags(&h->cap[k], cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      swfd_destroy(h);
      return fail(nullptr, SWFD_ERR_CUDA, std::string("swfd_create: ") + cudaGetErrorString(e));
    }
    st = ex7_create(h, err);
    if (st != SWFD_OK) {
      swfd_destroy(h);
      return fail(nullptr, st, err);
    }
    *out = h;
    return SWFD_OK;
  }
  swfd_handle* h = new swfd_handle();
  h->cfg = *cfg;
  st = make_params(*cfg, h->p, err);
  if (st != SWFD_OK) {
    delete h;
    return fail(nullptr, st, err);
  }
  h->device = cfg->device;
  {  // SWFD_LAUNCH=eager: plain stream launches instead of graphs (for profilers)
    const char* lm = getenv("SWFD_LAUNCH");
    h->eager = lm && strcmp(lm, "eager") == 0;
  }
  if (const char* hb = getenv("SWFD_HEAVY_BLOCK")) {  // 32..1024: the splitting's and RK's block
    const int v = atoi(hb);
    if (v >= 32 && v <= 1024 && (v & (v - 1)) == 0) h->p.heavy_block = v;
  }
  {  // the fused FP32-bulk stage where it applies (SWFD_FP32_STAGE=split: the
     // separate splitting, flux and RK kernels, the same bits)
    const Params& q = h->p;
    const char* fs = getenv("SWFD_FP32_STAGE");
    const bool on = q.precision == SWFD_PRECISION_FP32_BULK && q.g.ndim == 2 && !q.seg_alpha &&
                    !q.limiter && !q.quad && cfg->rk_choice != 2 &&
                    !(fs && strcmp(fs, "split") == 0);
    // SWFD_STAGE32_SHAPE pins the stage kernel's launch shape (1..5)
    const char* sh = getenv("SWFD_STAGE32_SHAPE");
    const int shape = sh ? atoi(sh) : 0;
    h->stage32 = on ? ((shape >= 1 && shape <= 5) ? shape : 4) : 0;
  }
  const Geom& g = h->p.g;
  auto cleanup_fail = [&](cudaError_t e) {
    std::string m = std::string("swfd_create: ") + cudaGetErrorString(e);
    swfd_destroy(h);
    return fail(nullptr, e == cudaErrorMemoryAllocation ? SWFD_ERR_OOM : SWFD_ERR_CUDA, m);
  };
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cleanup_fail(e);
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return cleanup_fail(e);
  if (h->stage32 && (e = stage32_setup()) != cudaSuccess) return cleanup_fail(e);
  const size_t pb = (size_t)g.plane * sizeof(double);
  for (int k = 0; k < 3; ++k)
    if ((e = cudaMalloc(&h->st[k], g.nc * pb)) != cudaSuccess) return cleanup_fail(e);
  // split and flux planes: one copy per rank segment (sg; sg == g except ex6)
  const size_t sb = (size_t)h->p.sg.plane * sizeof(double);
  if ((e = cudaMalloc(&h->split, 4 * g.nc * sb)) != cudaSuccess) return cleanup_fail(e);
  if ((e = cudaMalloc(&h->roe, 8 * pb)) != cudaSuccess) return cleanup_fail(e);
  if ((e = cudaMalloc(&h->flux, 4 * g.nc * sb)) != cudaSuccess) return cleanup_fail(e);
  if (h->p.seg_alpha) {  // per-cell alpha, alpha per rank row and per rank column
    const size_t n = (size_t)g.plane + (size_t)g.LJ * h->p.cut_x + (size_t)g.LI * h->p.cut_y +
                     (size_t)12 * (6 * h->p.total + 2);
    if ((e = cudaMalloc(&h->seg_buf, n * sizeof(double))) != cudaSuccess) return cleanup_fail(e);
    h->p.alpha_plane = h->seg_buf;
    h->p.seg_ax = h->seg_buf + g.plane;
    h->p.seg_ay = h->p.seg_ax + (size_t)g.LJ * h->p.cut_x;
    h->p.wall_save = h->p.seg_ay + (size_t)g.LI * h->p.cut_y;
  }
  if ((e = cudaMalloc(&h->rhs_tmp, g.nc * pb)) != cudaSuccess) return cleanup_fail(e);
  if (cfg->problem == SWFD_PROBLEM_MATLAB_1D &&
      (e = cudaMalloc(&h->m1_wk, matlab1d_workspace(g.nx) * sizeof(double))) != cudaSuccess)
    return cleanup_fail(e);
  if ((e = cudaMalloc(&h->dsc, sizeof(DevScalars))) != cudaSuccess) return cleanup_fail(e);
  if ((e = cudaMallocHost(&h->hsc, sizeof(DevScalars))) != cudaSuccess) return cleanup_fail(e);
  const size_t hb = (size_t)host_len(h->p) * sizeof(double);
  if ((e = cudaMalloc(&h->d_stage, hb)) != cudaSuccess) return cleanup_fail(e);
  if ((e = cudaMalloc(&h->sweep_scratch, sweep_scratch_bytes(h->p))) != cudaSuccess)
    return cleanup_fail(e);
  if (h->p.problem != SWFD_PROBLEM_MATLAB_1D &&
      ((e = cudaMalloc(&h->sweep_cluster, sweep_cluster_bytes(h->p))) != cudaSuccess ||
       (e = cudaMalloc(&h->ubar_scratch, ubar_scratch_bytes(h->p))) != cudaSuccess))
    return cleanup_fail(e);
  for (int k = 0; k < 8; ++k)
    if ((e = cudaEventCreate(&h->ev[k])) != cudaSuccess) return cleanup_fail(e);
  for (int k = 0; k < SWFD_CAP_DEPTH; ++k)
    if ((e = cudaStreamCreateWithFlags(&h->cap[k], cudaStreamNonBlocking)) != cudaSuccess)
      return cleanup_fail(e);
  h->track_cap = 1024;
  if ((e = cudaMalloc(&h->d_tracks, 3 * h->track_cap * sizeof(int))) != cudaSuccess)
    return cleanup_fail(e);
  for (int k = 0; k < 3; ++k)
    if ((e = cudaMemsetAsync(h->st[k], 0, g.nc * pb, h->stream)) != cudaSuccess)
      return cleanup_fail(e);
  if ((e = cudaMemsetAsync(h->split, 0, 4 * g.nc * sb, h->stream)) != cudaSuccess) return cleanup_fail(e);
  if ((e = cudaMemsetAsync(h->roe, 0, 8 * pb, h->stream)) != cudaSuccess) return cleanup_fail(e);
  if ((e = cudaMemsetAsync(h->flux, 0, 4 * g.nc * sb, h->stream)) != cudaSuccess) return cleanup_fail(e);
  if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cleanup_fail(e);
  if (reset_scalars(h) != SWFD_OK) {
    std::string m = h->last_error;
    swfd_destroy(h);
    return fail(nullptr, SWFD_ERR_CUDA, m);
  }
  *out = h;
  return SWFD_OK;
}

swfd_status swfd_destroy(swfd_handle* h) {
  if (!h) return SWFD_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  ex7_destroy(h->ex7);
  for (int k = 0; k < 3; ++k) cudaFree(h->st[k]);
  cudaFree(h->split);
  cudaFree(h->roe);
  cudaFree(h->flux);
  cudaFree(h->seg_buf);
  cudaFree(h->rhs_tmp);
  cudaFree(h->m1_wk);
  cudaFree(h->s1_scratch);
  cudaFree(h->dsc);
  cudaFree(h->d_stage);
  cudaFree(h->sweep_scratch);
  cudaFree(h->sweep_cluster);
  cudaFree(h->ubar_scratch);
  if (h->hsc) cudaFreeHost(h->hsc);
  for (int k = 0; k < 8; ++k)
    if (h->ev[k]) cudaEventDestroy(h->ev[k]);
  if (h->g_step) cudaGraphExecDestroy(h->g_step);
  if (h->g_solve) cudaGraphExecDestroy(h->g_solve);
  if (h->g_sweep) cudaGraphExecDestroy(h->g_sweep);
  for (int k = 0; k < SWFD_CAP_DEPTH; ++k)
    if (h->cap[k]) cudaStreamDestroy(h->cap[k]);
  cudaFree(h->d_tracks);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return SWFD_OK;
}

swfd_status swfd_upload_state(swfd_handle* h, const double* u) {
  if (!h || !u) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  if (h->ex7) return ex7_upload(h, u);
  CU(h, cudaSetDevice(h->device));
  const size_t hb = (size_t)host_len(h->p) * sizeof(double);
  CU(h, cudaMemcpyAsync(h->d_stage, u, hb, cudaMemcpyHostToDevice, h->stream));
  CU(h, launch_fortran_to_soa(h->p, h->d_stage, cur_state(h), h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  return SWFD_OK;
}

swfd_status swfd_download_state(swfd_handle* h, double* u) {
  if (!h || !u) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  if (h->ex7) return ex7_download(h, u);
  CU(h, cudaSetDevice(h->device));
  const size_t hb = (size_t)host_len(h->p) * sizeof(double);
  CU(h, launch_soa_to_fortran(h->p, cur_state(h), h->d_stage, h->stream));
  CU(h, cudaMemcpyAsync(u, h->d_stage, hb, cudaMemcpyDeviceToHost, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  return SWFD_OK;
}

swfd_status swfd_init_problem(swfd_handle* h) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  SETTLE(h);
  if (h->ex7) return ex7_init(h);
  std::vector<double> u((size_t)host_len(h->p));
  init_host(h, u.data());
  ST(swfd_upload_state(h, u.data()));
  // the reference applies bc after initdata except ex6, whose time loop starts
  // from initdata directly (ex6_shock_diffraction/main.f90:97-103)
  if (h->p.g.ndim == 2 && h->p.problem != SWFD_PROBLEM_SHOCK_DIFFRACTION)
    LAUNCH(h, 1, launch_bc(h->p, cur_state(h), h->stream));
  ST(reset_scalars(h));
  return SWFD_OK;
}

swfd_status swfd_get_time(swfd_handle* h, double* t) {
  if (!h || !t) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  *t = h->time;
  return SWFD_OK;
}

swfd_status swfd_set_time(swfd_handle* h, double t) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  SETTLE(h);
  if (h->ex7) return ex7_set_time(h, t);
  CU(h, cudaSetDevice(h->device));
  h->time = t;
  CU(h, cudaMemcpyAsync(&h->dsc->time, &h->time, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CU(h, cudaStreamSynchronize(h->stream));
  return SWFD_OK;
}

// the MATLAB script's scheme: up to max_steps steps in one launch
swfd_status matlab1d_steps(swfd_handle* h, long long max_steps, int64_t* steps_out) {
  ST(ensure_tracks(h, 3 * max_steps));
  DevScalars before = *h->hsc;
  CU(h, cudaMemsetAsync(&h->dsc->steps, 0, sizeof(long long), h->stream));
  CU(h, launch_matlab1d(h->p, cur_state(h), h->m1_wk, h->dsc, max_steps,
                        matlab_periodic(h->cfg.variant), h->cfg.use_limiter == 2, h->cfg.swp_num,
                        h->cfg.cfl, h->stream));
  swfd_status st = check_device_error(h);
  if (steps_out) *steps_out = h->hsc->steps;
  h->prof.kernel_launches += 1;
  h->prof.stages += 3 * h->hsc->steps;
  h->prof.sweep_invocations += h->hsc->sweep_count - before.sweep_count;
  return st;
}

// after a step's graph: the one synchronisation (scalars and device
// errors), launch accounting, the flux timings with profiling on, dt
swfd_status step_done(swfd_handle* h, const DevScalars& before, double* dt_out) {
  swfd_status st = check_device_error(h);
  account(h, before, *h->hsc, 1, 0);
  if (h->prof_on && h->cfg.rk_choice != 2) {  // the restart RK records no flux events
    for (int k = 0; k < 3; ++k) {
      float ms = 0.f;
      CU(h, cudaEventElapsedTime(&ms, h->ev[2 * k], h->ev[2 * k + 1]));
      h->prof.flux_ms += ms;
      h->prof.flux_launches += 1;
    }
  }
  if (dt_out) *dt_out = h->hsc->dt;
  return st;
}

// the step graph, with the flux event nodes exactly when profiling is on
// (each node is a dependency hop inside the step)
swfd_status step_graph(swfd_handle* h) {
  if (h->g_step && h->g_step_events != h->prof_on) {
    cudaGraphExecDestroy(h->g_step);
    h->g_step = nullptr;
  }
  ST(build_graph(h, GRAPH_STEP, &h->g_step));
  h->g_step_events = h->prof_on;
  return SWFD_OK;
}

swfd_status swfd_step(swfd_handle* h, double* dt_out) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  SETTLE(h);
  if (h->ex7) return ex7_step(h, dt_out);
  CU(h, cudaSetDevice(h->device));
  if (h->cfg.problem == SWFD_PROBLEM_MATLAB_1D) {
    swfd_status st = matlab1d_steps(h, 1, nullptr);
    if (dt_out) *dt_out = h->hsc->dt;
    return st;
  }
  ST(step_graph(h));
  // the host mirror holds the scalars of the last step (no step is pending):
  // the track arrays grow, with a synchronisation, only when a step's three
  // sweeps could overflow them
  if (h->hsc->sweep_count + 3 > h->track_cap) ST(ensure_tracks(h, 3));
  DevScalars before = *h->hsc;
  ST(launch_kind(h, GRAPH_STEP, h->g_step));
  return step_done(h, before, dt_out);
}

/* One step from a host state to a host state: the upload, the step graph and
 * the download on the handle's stream with one synchronisation at the end
 * (what swfd_upload_state, swfd_step and swfd_download_state do with three). */
swfd_status swfd_step_host(swfd_handle* h, const double* u_in, double* u_out, double* dt_out) {
  if (!h || !u_in || !u_out) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  if (h->ex7 || h->eager || h->cfg.problem == SWFD_PROBLEM_MATLAB_1D) {
    ST(swfd_upload_state(h, u_in));
    ST(swfd_step(h, dt_out));
    return swfd_download_state(h, u_out);
  }
  CU(h, cudaSetDevice(h->device));
  ST(step_graph(h));
  if (h->hsc->sweep_count + 3 > h->track_cap) ST(ensure_tracks(h, 3));
  const size_t hb = (size_t)host_len(h->p) * sizeof(double);
  CU(h, cudaMemcpyAsync(h->d_stage, u_in, hb, cudaMemcpyHostToDevice, h->stream));
  CU(h, launch_fortran_to_soa(h->p, h->d_stage, cur_state(h), h->stream));
  DevScalars before = *h->hsc;
  CU(h, cudaGraphLaunch(h->g_step, h->stream));
  CU(h, launch_soa_to_fortran(h->p, cur_state(h), h->d_stage, h->stream));
  CU(h, cudaMemcpyAsync(u_out, h->d_stage, hb, cudaMemcpyDeviceToHost, h->stream));
  return step_done(h, before, dt_out);
}

swfd_status swfd_step_async(swfd_handle* h) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  if (h->eager || h->cfg.problem == SWFD_PROBLEM_MATLAB_1D || h->ex7)
    return swfd_step(h, nullptr);  // eager sections read conditions on the host
  CU(h, cudaSetDevice(h->device));
  ST(step_graph(h));
  // a step records at most three sweeps: grow the track arrays (after
  // finishing what is enqueued) before the pending steps could overflow them
  if (h->hsc->sweep_count + 3 * (h->pending + 1) > h->track_cap) {
    SETTLE(h);
    ST(ensure_tracks(h, 3));
  }
  if (h->pending == 0) h->pending_before = *h->hsc;
  CU(h, cudaGraphLaunch(h->g_step, h->stream));
  h->pending++;
  return SWFD_OK;
}

swfd_status swfd_autotune(swfd_handle* h, int32_t* flux_min_blocks) {
  if (!h || !flux_min_blocks) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  if (h->ex7) {  // one launch shape
    *flux_min_blocks = 0;
    return SWFD_OK;
  }
  SETTLE(h);
  CU(h, cudaSetDevice(h->device));
  *flux_min_blocks = 0;
  Params& p = h->p;
  // the fused FP32-bulk stage has one launch shape
  if (p.g.ndim != 2 || p.seg_alpha || p.limiter || h->stage32) return SWFD_OK;
  // the flux kernel's inputs for the current state (findalpha and the
  // splitting only rewrite per-stage scratch: alphamax, split and Roe planes)
  double* u = cur_state(h);
  CU(h, launch_alpha(p, u, h->dsc, h->stream));
  int nk = 0;
  CU(h, launch_split(p, u, h->dsc, h->split, h->roe, h->stream, &nk));
  int cand[16];
  const int nc = flux_min_blocks_candidates(p.precision == SWFD_PRECISION_FP32_BULK, cand);
  const int saved = p.flux_minb;
  float best = 0.f;
  int pick = cand[0];
  // SWFD_FLUX_MIN_BLOCKS pins one of the candidates (reproducible profiles)
  int pinned = 0;
  if (const char* env = getenv("SWFD_FLUX_MIN_BLOCKS"))
    for (int k = 0; k < nc; ++k)
      if (atoi(env) == cand[k]) pinned = cand[k];
  for (int k = 0; k < nc && !pinned; ++k) {
    p.flux_minb = cand[k];
    CU(h, launch_flux(p, h->split, h->roe, h->dsc, h->flux, &h->dsc->flux_work, h->stream));
    CU(h, cudaEventRecord(h->ev[0], h->stream));
    for (int r = 0; r < 5; ++r)
      CU(h, launch_flux(p, h->split, h->roe, h->dsc, h->flux, &h->dsc->flux_work, h->stream));
    CU(h, cudaEventRecord(h->ev[1], h->stream));
    CU(h, cudaEventSynchronize(h->ev[1]));
    float ms = 0.f;
    CU(h, cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
    if (k == 0 || ms < best) best = ms, pick = cand[k];
  }
  if (pinned) pick = pinned;
  p.flux_minb = pick;
  if (pick != saved) {  // the graphs hold the parameters by value: capture them again
    if (h->g_step) cudaGraphExecDestroy(h->g_step);
    if (h->g_solve) cudaGraphExecDestroy(h->g_solve);
    if (h->g_sweep) cudaGraphExecDestroy(h->g_sweep);
    h->g_step = h->g_solve = h->g_sweep = nullptr;
  }
  ST(check_device_error(h));
  *flux_min_blocks = pick;
  return SWFD_OK;
}

swfd_status swfd_finish(swfd_handle* h) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  CU(h, cudaSetDevice(h->device));
  if (!h->pending) return SWFD_OK;
  return finish_pending(h);
}

swfd_status swfd_run(swfd_handle* h, int64_t max_steps, int64_t* nsteps_out) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  SETTLE(h);
  if (h->ex7) {  // DO WHILE (time <= time_terminal - 1d-10) (ex7_detonation/main.f90:97)
    int64_t done = 0;
    swfd_status st = SWFD_OK;
    while (h->time <= ex7_t_loop(h)) {
      if (max_steps > 0 && done >= max_steps) {
        st = SWFD_ERR_MAX_STEPS;
        break;
      }
      st = ex7_step(h, nullptr);
      ++done;
      if (st != SWFD_OK) break;
    }
    if (nsteps_out) *nsteps_out = done;
    return st;
  }
  CU(h, cudaSetDevice(h->device));
  if (h->cfg.problem == SWFD_PROBLEM_MATLAB_1D) {
    // while t < tFinal (FD_WENO_Application.m:212), tested on the device
    int64_t done = 0;
    swfd_status st = SWFD_OK;
    const int64_t chunk = 4096;
    while (h->time < h->cfg.time_terminal) {
      if (max_steps > 0 && done >= max_steps) {
        st = SWFD_ERR_MAX_STEPS;
        break;
      }
      const long long lim =
          (long long)(max_steps > 0 ? std::min<int64_t>(chunk, max_steps - done) : chunk);
      int64_t steps = 0;
      const double t_before = h->time;
      st = matlab1d_steps(h, lim, &steps);
      done += steps;
      if (st != SWFD_OK || steps < lim) break;
      if (!(h->time > t_before)) {  // k = 0 (an infinite alpha): the script would loop forever
        st = fail(h, SWFD_ERR_NONFINITE, "the time step is 0: the time loop does not advance");
        break;
      }
    }
    if (nsteps_out) *nsteps_out = done;
    return st;
  }
  {
    Solve1dShape sh;
    if (use_solve1d(h, &sh)) {
      const swfd_status s1 = run_solve1d(h, sh, max_steps, nsteps_out);
      if (!h->s1_refused) return s1;
    }
  }
  ST(build_graph(h, GRAPH_SOLVE, &h->g_solve));
  int64_t done = 0;
  const int64_t chunk = 4096;  // steps per graph launch (bounds the track growth)
  swfd_status st = SWFD_OK;
  // DO WHILE (time <= time_terminal - 1d-10)  (ex3_vortex_accuracy_2d/main.f90:51),
  // evaluated on the device after every step
  while (h->time <= h->p.t_loop) {
    if (max_steps > 0 && done >= max_steps) {
      st = SWFD_ERR_MAX_STEPS;
      break;
    }
    long long lim = (long long)(max_steps > 0 ? std::min<int64_t>(chunk, max_steps - done) : chunk);
    ST(ensure_tracks(h, 3 * lim));
    DevScalars before = *h->hsc;
    CU(h, cudaMemcpyAsync(&h->dsc->steps_limit, &lim, sizeof(long long), cudaMemcpyHostToDevice,
                          h->stream));
    ST(launch_kind(h, GRAPH_SOLVE, h->g_solve));
    st = check_device_error(h);
    int64_t steps = h->hsc->steps;
    account(h, before, *h->hsc, steps, 2);
    done += steps;
    if (st != SWFD_OK) break;
    if (steps < lim) break;  // the time test ended the loop
  }
  if (nsteps_out) *nsteps_out = done;
  return st;
}

swfd_status swfd_flux_divergence(swfd_handle* h, double* rhs) {
  if (!h || !rhs) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  if (h->ex7)
    return fail(h, SWFD_ERR_UNSUPPORTED, "the detonation runs whole steps, find_alpha and state I/O");
  if (h->cfg.problem == SWFD_PROBLEM_MATLAB_1D)
    return fail(h, SWFD_ERR_UNSUPPORTED, "the MATLAB script's scheme runs whole steps only");
  CU(h, cudaSetDevice(h->device));
  const Params& p = h->p;
  double* u = cur_state(h);
  CU(h, launch_alpha(p, u, h->dsc, h->stream));
  int nk = 0;
  CU(h, launch_split(p, u, h->dsc, h->split, h->roe, h->stream, &nk));
  CU(h, launch_flux(p, h->split, p.g.ndim == 1 ? u : h->roe, h->dsc, h->flux, &h->dsc->flux_work, h->stream));
  CU(h, launch_rhs(p, h->flux, h->dsc, h->rhs_tmp, h->stream));
  const size_t hb = (size_t)host_len(p) * sizeof(double);
  CU(h, launch_soa_to_fortran(p, h->rhs_tmp, h->d_stage, h->stream));
  CU(h, cudaMemcpyAsync(rhs, h->d_stage, hb, cudaMemcpyDeviceToHost, h->stream));
  ST(check_device_error(h));
  return SWFD_OK;
}

swfd_status swfd_sweep(swfd_handle* h) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  SETTLE(h);
  if (h->ex7)
    return fail(h, SWFD_ERR_UNSUPPORTED, "the detonation runs whole steps, find_alpha and state I/O");
  if (h->cfg.problem == SWFD_PROBLEM_MATLAB_1D)
    return fail(h, SWFD_ERR_UNSUPPORTED, "the MATLAB script's scheme runs whole steps only");
  CU(h, cudaSetDevice(h->device));
  ST(build_graph(h, GRAPH_SWEEP, &h->g_sweep));
  ST(ensure_tracks(h, 1));
  DevScalars before = *h->hsc;
  ST(launch_kind(h, GRAPH_SWEEP, h->g_sweep));
  swfd_status st = check_device_error(h);
  account(h, before, *h->hsc, 0, 0);
  return st;
}

swfd_status swfd_check_positivity(swfd_handle* h, int32_t* postag) {
  if (!h || !postag) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  if (h->ex7)
    return fail(h, SWFD_ERR_UNSUPPORTED, "the detonation runs whole steps, find_alpha and state I/O");
  if (h->cfg.problem == SWFD_PROBLEM_MATLAB_1D)
    return fail(h, SWFD_ERR_UNSUPPORTED, "the MATLAB script's scheme runs whole steps only");
  CU(h, cudaSetDevice(h->device));
  CU(h, launch_positivity(h->p, cur_state(h), h->dsc, h->stream));
  ST(sync_scalars(h));
  *postag = h->hsc->postag;
  return SWFD_OK;
}

swfd_status swfd_find_alpha(swfd_handle* h, double* alphamax) {
  if (!h || !alphamax) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  if (h->ex7) return ex7_find_alpha(h, alphamax);
  if (h->cfg.problem == SWFD_PROBLEM_MATLAB_1D)
    return fail(h, SWFD_ERR_UNSUPPORTED, "the MATLAB script's scheme runs whole steps only");
  CU(h, cudaSetDevice(h->device));
  CU(h, launch_alpha(h->p, cur_state(h), h->dsc, h->stream));
  ST(sync_scalars(h));
  *alphamax = h->hsc->alphamax;
  return SWFD_OK;
}

namespace {
swfd_status fetch_tracks(swfd_handle* h, std::vector<int32_t>& tr, int64_t& n) {
  ST(sync_scalars(h));
  n = std::min<int64_t>(h->hsc->sweep_count, h->track_cap);
  tr.assign(3 * (size_t)n, 0);
  for (int k = 0; k < 3 && n > 0; ++k)
    CU(h, cudaMemcpy(tr.data() + k * n, h->d_tracks + k * h->track_cap, n * sizeof(int32_t),
                     cudaMemcpyDeviceToHost));
  return SWFD_OK;
}
}  // namespace

swfd_status swfd_get_restarts(swfd_handle* h, int64_t* restarts) {
  if (!h || !restarts) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  if (h->ex7) {
    *restarts = 0;
    return SWFD_OK;
  }
  CU(h, cudaSetDevice(h->device));
  ST(sync_scalars(h));
  *restarts = h->hsc->restart_total;
  return SWFD_OK;
}

swfd_status swfd_get_sweep_stats(swfd_handle* h, swfd_sweep_stats* s) {
  if (!h || !s) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  if (h->ex7) return ex7_stats(h, s);
  CU(h, cudaSetDevice(h->device));
  std::vector<int32_t> tr;
  int64_t n = 0;
  ST(fetch_tracks(h, tr, n));
  memset(s, 0, sizeof(*s));
  s->sweep_count = h->hsc->sweep_count;
  for (int64_t k = 0; k < n; ++k) {
    int32_t sw = tr[k], ng = tr[n + k], ps = tr[2 * n + k];
    s->total_sweep += sw;
    s->total_neg += ng;
    s->total_pos += ps;
    if (k == 0 || sw > s->max_sweep) s->max_sweep = sw;
    if (k == 0 || ng > s->max_neg) s->max_neg = ng;
    if (k == 0 || ps > s->max_pos) s->max_pos = ps;
  }
  s->den_count = h->hsc->den_count;
  s->pre_count = h->hsc->pre_count;
  s->sweep_fail_count = h->hsc->fail_count;
  return SWFD_OK;
}

swfd_status swfd_get_sweep_tracks(swfd_handle* h, int32_t* sweep, int32_t* neg, int32_t* pos,
                                  int64_t cap, int64_t* count) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  SETTLE(h);
  if (h->ex7) {
    const int64_t n = ex7_tracks(h, sweep, neg, pos, std::max<int64_t>(cap, 0));
    if (count) *count = n;
    return SWFD_OK;
  }
  CU(h, cudaSetDevice(h->device));
  std::vector<int32_t> tr;
  int64_t n = 0;
  ST(fetch_tracks(h, tr, n));
  int64_t m = std::min<int64_t>(n, std::max<int64_t>(cap, 0));
  for (int64_t k = 0; k < m; ++k) {
    if (sweep) sweep[k] = tr[k];
    if (neg) neg[k] = tr[n + k];
    if (pos) pos[k] = tr[2 * n + k];
  }
  if (count) *count = n;
  return SWFD_OK;
}

swfd_status swfd_weno5_batch(const double* stencils, int64_t n, double weno_eps, int32_t literals,
                             int32_t device, double* uleft, double* uright) {
  if (n < 0 || (n > 0 && !stencils)) return fail(nullptr, SWFD_ERR_INVALID, "bad arguments");
  if (literals != SWFD_LITERALS_DOUBLE && literals != SWFD_LITERALS_QUAD)
    return fail(nullptr, SWFD_ERR_INVALID, "unknown literals mode");
  if (literals == SWFD_LITERALS_QUAD && weno_eps != 1e-6 && weno_eps != 1e-12)
    return fail(nullptr, SWFD_ERR_INVALID, "literals QUAD: the reference's epsilons 1e-6, 1e-12");
  if (n == 0) return SWFD_OK;
  CU(nullptr, cudaSetDevice(device));
  double *ds = nullptr, *dl = nullptr, *dr = nullptr;
  cudaStream_t s = nullptr;
  auto done = [&](swfd_status st) {
    if (s) cudaStreamSynchronize(s);
    cudaFree(ds);
    cudaFree(dl);
    cudaFree(dr);
    if (s) cudaStreamDestroy(s);
    return st;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc(&ds, 5 * n * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&dl, n * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&dr, n * sizeof(double))) != cudaSuccess ||
      (e = cudaMemcpyAsync(ds, stencils, 5 * n * sizeof(double), cudaMemcpyHostToDevice, s)) !=
          cudaSuccess ||
      (e = launch_weno_batch(ds, n, weno_eps, literals == SWFD_LITERALS_QUAD, dl, dr, s)) !=
          cudaSuccess ||
      (uleft && (e = cudaMemcpyAsync(uleft, dl, n * sizeof(double), cudaMemcpyDeviceToHost, s)) !=
                    cudaSuccess) ||
      (uright && (e = cudaMemcpyAsync(uright, dr, n * sizeof(double), cudaMemcpyDeviceToHost, s)) !=
                     cudaSuccess) ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return done(fail(nullptr, SWFD_ERR_CUDA, std::string("swfd_weno5_batch: ") + cudaGetErrorString(e)));
  return done(SWFD_OK);
}

swfd_status swfd_sequential_sum(const double* x, int64_t n, double w, int32_t device,
                                double* out) {
  if (n < 0 || n > INT32_MAX || (n > 0 && !x) || !out)
    return fail(nullptr, SWFD_ERR_INVALID, "bad arguments");
  CU(nullptr, cudaSetDevice(device));
  double *dx = nullptr, *ds = nullptr;
  void* scratch = nullptr;
  cudaStream_t s = nullptr;
  auto done = [&](swfd_status st) {
    if (s) cudaStreamSynchronize(s);
    cudaFree(dx);
    cudaFree(ds);
    cudaFree(scratch);
    if (s) cudaStreamDestroy(s);
    return st;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc(&dx, (n > 0 ? n : 1) * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&ds, sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&scratch, seq_sum_scratch_bytes(n > 0 ? n : 1))) != cudaSuccess ||
      (n > 0 && (e = cudaMemcpyAsync(dx, x, n * sizeof(double), cudaMemcpyHostToDevice, s)) !=
                    cudaSuccess) ||
      (e = launch_seq_sum(dx, n, w, ds, scratch, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(out, ds, sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return done(
        fail(nullptr, SWFD_ERR_CUDA, std::string("swfd_sequential_sum: ") + cudaGetErrorString(e)));
  return done(SWFD_OK);
}

swfd_status swfd_get_stream(swfd_handle* h, void** stream) {
  if (!h || !stream) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  *stream = (void*)h->stream;
  return SWFD_OK;
}

swfd_status swfd_set_profiling(swfd_handle* h, int32_t on) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  SETTLE(h);  // enqueued steps report with the setting they ran under
  h->prof_on = on ? 1 : 0;
  return SWFD_OK;
}

swfd_status swfd_get_profile(swfd_handle* h, swfd_profile* prof) {
  if (!h || !prof) return fail(h, SWFD_ERR_INVALID, "NULL argument");
  SETTLE(h);
  *prof = h->prof;
  if (h->ex7) prof->kernel_launches = ex7_launches(h);
  return SWFD_OK;
}

swfd_status swfd_reset_profile(swfd_handle* h) {
  if (!h) return fail(h, SWFD_ERR_INVALID, "NULL handle");
  h->prof = swfd_profile{};
  return SWFD_OK;
}

swfd_status swfd_last_error(swfd_handle* h, char* buf, size_t len) {
  if (!buf || len == 0) return SWFD_ERR_INVALID;
  const std::string& m = h ? h->last_error : g_last_error;
  snprintf(buf, len, "%s", m.c_str());
  return SWFD_OK;
}

}  // extern "C"
