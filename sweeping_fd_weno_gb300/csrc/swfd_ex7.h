// swfd_ex7.h -- the detonation engine (ex7_detonation/main.f90): device view,
// device scalars and the entry points the C-ABI routes to.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "swfd_internal.h"

namespace swfd {

// device error bits
constexpr int E7_ERR_NONFINITE = 1;     // alpha or dt not finite
constexpr int E7_ERR_SWEEP_CHECK = 2;   // a nodal adjustment raised the pair's total pressure
constexpr int E7_ERR_SWEEP_INDEX = 4;   // the ordering-II pass needed sweepI(0)
constexpr int E7_ERR_PUBAR = 8;         // the sweep's P(u_bar) <= 0
constexpr int E7_ERR_NOCONV = 16;       // the sweep reached swp_num

struct Ex7Scalars {
  unsigned long long am_bits;  // alphamax as bits (non-negative values)
  double alphamax, dt, time;
  int postag, err;
  unsigned long long rho_min_key, p_min_key;  // ordered keys of the exit-test minima
  long long t_pos, t_neg;                     // nod_lim branch counts of the current sweep
  int nflag, pad;
  double ubar[5];
  long long lim_den, lim_pre;  // use_limiter = 1: density and pressure limitings
  // the sweep's control on the device: its pass pair q, the condition word of
  // the eager launch mode, the statistics and the tracks (sweep, neg, pos;
  // 3 x track_cap, grown by the host between steps)
  int q, cond;
  long long sweep_count, den_count, pre_count, fail_count;
  int* tracks;
  long long track_cap;
};

// everything a kernel needs, passed by value
struct Ex7View {
  int R, cut_x, cut_y, nxl, nyl, LI, LJ, LL, total, wall, nx, ny;
  double dx, dy, gamma, g1, cfl, T, eps, eps2, weno_eps, q, tc, kc;
  // per-rank slices (R x 5 planes of LI x LJ): state, step-start state,
  // split fluxes (x pass, then y pass), interface fluxes, Roe line data
  double *u, *u0, *sp, *sn, *fpf, *fnf, *gpf, *gnf, *roe;
  double* alpha;  // R planes of LI x LJ
  double* lal;    // per rank: alpha of each local row (x pass) or column (y pass), LL entries
  double* ug;     // gathered interior for the sweep: 5 planes of nx*ny, i fastest
  double* gview;  // the global view u(5,-2:nx+3,-2:ny+3) for upload and download
  const qd::q128* expc;  // Taylor coefficients of exp (qd::exp_coefs)
  // literals QUAD (the reference's -fdefault-real-8 build): 13d0/12d0, 1d-12
  // and 1d-15 in binary128, and rho < 1d-8 as rho < lim8_lt
  int quad, use_limiter;
  double lim8_lt;
  qd::q128 q_c1312, q_eps, q_1em15;
  Ex7Scalars* sc;
  int* flag;  // sweep: per position, 1 if the step is active on the pass-start state
  int* list;  // sweep: the flagged positions in increasing order
};

struct Ex7 {
  Ex7View v{};
  Ex7Scalars* hs = nullptr;  // pinned mirror of v.sc
  void* block = nullptr;     // one device allocation holding every buffer
  void* sum_scratch = nullptr;  // the u_bar sums' terms and chunk summaries
  int use_limiter = 2, swp_num = 0;
  double t_loop = 0.;  // DO WHILE (time <= time_terminal - 1d-10), literal-exact
  int* tracks = nullptr;  // device sweep tracks (3 x track_cap)
  int64_t track_cap = 0;
  // one step as a CUDA graph: three stages, each with an IF around the sweep
  // (whose pass pairs are a WHILE) -- no host synchronisation inside a step
  cudaGraphExec_t g_step = nullptr;
  // kernels per graph section (launch accounting): the step without sweeps,
  // a sweep's fixed part, one pass pair
  int k_step = 0, k_sweep = 0, k_q = 0;
  long long launches = 0;
};

// configuration check (total, rank grid, wall mirrors inside the local arrays)
swfd_status ex7_check(const swfd_config& c, std::string& err);
swfd_status ex7_create(swfd_handle* h, std::string& err);
void ex7_destroy(Ex7* x);
swfd_status ex7_init(swfd_handle* h);
swfd_status ex7_upload(swfd_handle* h, const double* u);
swfd_status ex7_download(swfd_handle* h, double* u);
swfd_status ex7_step(swfd_handle* h, double* dt_out);
swfd_status ex7_set_time(swfd_handle* h, double t);
swfd_status ex7_find_alpha(swfd_handle* h, double* alphamax);
swfd_status ex7_stats(swfd_handle* h, swfd_sweep_stats* s);
int64_t ex7_tracks(swfd_handle* h, int32_t* sweep, int32_t* neg, int32_t* pos, int64_t cap);
int64_t ex7_launches(swfd_handle* h);
double ex7_t_loop(swfd_handle* h);

}  // namespace swfd
