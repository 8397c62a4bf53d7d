// swfd_internal.h -- shared declarations of the CUDA library (not installed).
#pragma once

#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/swfd.h"
#include "swfd_quad.cuh"

namespace swfd {

// Device layout: structure-of-arrays planes.  Plane c holds component c of
// every cell (i, j), i in [-2, nx+3], j in [-2, ny+3], at offset
// (i + 2) + pitch * (j + 2).  pitch is nx + 6 rounded up to 32 doubles so
// that every row starts on a 256-byte boundary.  1D problems use one row.
struct Geom {
  int ndim = 2;
  int nc = 4;      // conserved components
  int nx = 0, ny = 1;
  int LI = 0, LJ = 0;  // nx + 6, ny + 6 (1 in 1D)
  int pitch = 0;
  int64_t plane = 0;   // doubles per plane
  __host__ __device__ int64_t at(int i, int j) const {
    return (int64_t)(i + 2) + (int64_t)pitch * (int64_t)(j + 2);
  }
};

// Per-problem switches of the reference's variant matrix, resolved on the
// host once and passed to every kernel by value.
struct Params {
  Geom g;
  int problem = 0;
  int literals = 0;
  int precision = 0;     // SWFD_PRECISION_*
  int pos_strict = 0;    // checkpositivity uses `<` (ex4, ex5)
  int exit_ge = 0;       // sweep exit test uses `>=` (ex5)
  int alpha_guarded = 0; // findalpha with the eps2 velocity guard (ex4, ex5)
  int flux_guard_eps2 = 0;  // fflux guard `rho < eps2` (ex4) instead of 1d-8
  int roe_reg_ex4 = 0;   // 1d-15 Roe regularisers and y-pass 1/(den+1d-15)
  int alpha_premul = 0;  // fluxes scaled by alpha inside wenofd (ex4)
  int dt_rule = 0;       // 1: dx*cfl/a; 3: dx**(5/3)*cfl/a; 4: min(dx,dy)*cfl/a clamped
  double gamma = 1.4, gamma1 = 0.4, eps = 1e-13, eps2 = 1e-8, weno_eps = 1e-6;
  double dx = 0, dy = 0;
  float fdx_inv = 0.f, fdy_inv = 0.f;  // FP32-bulk flux differences: 1/dx, 1/dy
  // literals = SWFD_LITERALS_QUAD (the reference's -fdefault-real-8 build):
  // the subexpressions with a double-kind literal in binary128
  int quad = 0;
  qd::q128 q_c1312, q_weno_eps, q_1em15;  // 13d0/12d0, the WENO epsilon, 1d-15
  // rho < 1d-8, rho > 1d-8, rho <= 1d-8 as binary64 comparisons with these
  // bounds: the literal itself, or the binary64 neighbours of its binary128
  // value (no binary64 lies between them)
  double lim8_lt = 1e-8, lim8_gt = 1e-8, lim8_le = 1e-8;
  double t_loop = 0;  // the time loop test time <= T - 1d-10, as time <= t_loop
  double dt_num_x = 0;   // dx*cfl   (or dx**(5/3)*cfl for dt_rule 3)
  double dt_num_y = 0;   // dy*cfl
  double time_terminal = 0;
  // jet inflow (ex5_mach2000_jet/main.f90:702-719)
  int jet_jmax = 0;      // y(j) <= 0.05  <=>  j <= jet_jmax (half domain)
  int jet_jmin = -2;     // full domain: |y(j)| <= 0.05  <=>  jet_jmin <= j <= jet_jmax
  int jet_full = 0;      // variant 1: full domain, outflow at the bottom
  double jet_in[4] = {0, 0, 0, 0};
  double jet_amb[4] = {0, 0, 0, 0};
  int stop_sweep = 0;    // P(u_bar) <= 0 and swp_num exhaustion stop the run (ex4, ex6)
  int limiter = 0;       // use_limiter = 1: the positivity flux limiter in wenofd
  int limiter_clamp = 0; // ex6 clamps its theta at 0 (theta = max(theta, 0.))
  int flux_minb = 0;     // flux kernel launch shape chosen by swfd_autotune (0: default)
  // largest block of the splitting and RK kernels (~70 registers a thread):
  // 128 puts a 360^2 grid's cells in one wave of resident blocks
  int heavy_block = 128;
  // Shock diffraction (ex6_shock_diffraction/main.f90).  The reference's
  // rank grid cut_x x cut_y (ranks of nxl x nyl cells) is part of its
  // arithmetic: the x pass of row j uses the max alpha over the cells of
  // its rank's local row (ghosts included), the y pass likewise per local
  // column, and a flux at a rank boundary is computed by both ranks, each
  // with its own alpha.  The split and flux planes therefore hold one copy
  // per rank segment: x-direction copies shifted by 6 columns per segment,
  // y-direction copies by 6 rows (geometry sg; sg == g when cut_x = cut_y = 1).
  int seg_alpha = 0;     // LF alpha per rank row / column instead of alphamax
  int cut_x = 1, cut_y = 1, nxl = 0, nyl = 0;
  int total = 0;         // step width in cells; the step top is row 6*total
  int sweep_check = 0;   // pressure-increase check in ordering-I passes
  double inflow[4] = {0, 0, 0, 0};  // left inflow state (post-shock)
  Geom sg;               // geometry of the split and flux planes
  double* alpha_plane = nullptr;    // per-cell alpha (g geometry)
  double* seg_ax = nullptr;         // alpha of (row j, x segment s): [(j+2)*cut_x + s]
  double* seg_ay = nullptr;         // alpha of (column i, y segment t): [(i+2)*cut_y + t]
  // ex6: the x wall mirror runs over each rank's local rows 0..nyl+1 only, so
  // a rank's outer ghost rows (local -2, -1, nyl+2, nyl+3) keep the
  // pre-mirror values of the wall columns, and its y pass reads those.  The
  // mirror saves them here: [((j * 3) + k) * 4 + c], column total - k, row j.
  double* wall_save = nullptr;
};

// ex6: does y segment t see cell (i, j) as it was before the x wall mirror?
__host__ __device__ __forceinline__ bool seg_sees_premirror(const Params& p, int i, int j, int t) {
  if (i < p.total - 2 || i > p.total || j < 0 || j > 6 * p.total || j > p.g.ny + 1) return false;
  const int l = j - t * p.nyl;
  return l == -2 || l == -1 || l == p.nyl + 2 || l == p.nyl + 3;
}

// offsets of the segment copies in the split / flux planes
__host__ __device__ __forceinline__ int64_t seg_x_off(const Params& p, int i, int j, int s) {
  return (int64_t)(i + 2 + 6 * s) + (int64_t)p.sg.pitch * (int64_t)(j + 2);
}
__host__ __device__ __forceinline__ int64_t seg_y_off(const Params& p, int i, int j, int t) {
  return (int64_t)(i + 2) + (int64_t)p.sg.pitch * (int64_t)(j + 2 + 6 * t);
}

// interfaces of one stage: x faces of rows 1..ny, per rank segment its
// local faces 0..nxl+1 (without segments: 0..nx+1); y faces of columns
// 1..nx, per segment its local faces 0..nyl+1.  With the limiter every face
// the reference computes is computed, because the limiter counts events on
// all of them: the x pass of each rank runs over its local rows 0..nyl+1 and
// the y pass over its local columns 0..nxl+1 (rows and columns where ranks
// overlap are computed, and counted, by both).
__host__ __device__ __forceinline__ int64_t flux_rows_x(const Params& p, bool lim) {
  return lim ? (int64_t)p.cut_y * (p.nyl + 2) : (int64_t)p.g.ny;
}
__host__ __device__ __forceinline__ int64_t flux_cols_y(const Params& p, bool lim) {
  return lim ? (int64_t)p.cut_x * (p.nxl + 2) : (int64_t)p.g.nx;
}
__host__ __device__ __forceinline__ int64_t flux_faces_x(const Params& p, bool lim = false) {
  return (int64_t)p.cut_x * (p.nxl + 2) * flux_rows_x(p, lim);
}
__host__ __device__ __forceinline__ int64_t flux_faces_y(const Params& p, bool lim = false) {
  return flux_cols_y(p, lim) * p.cut_y * (p.nyl + 2);
}


// Device scalars of one handle, in one small allocation.  The sweep
// statistics and the per-sweep tracks live here so that a whole step (and a
// whole solve) runs on the device without host round trips.
enum : int {
  ERR_BIT_ALPHA = 1,     // alphamax not finite or not positive
  ERR_BIT_DT = 2,        // dt not finite
  ERR_BIT_PUBAR = 4,     // P(u_bar) <= 0 (ex4 stop)
  ERR_BIT_NOCONV = 8,    // sweep reached swp_num (ex4 stop)
  ERR_BIT_CHECK = 16,    // nodal adjustment raised the total pressure (ex6 stop)
  ERR_BIT_RESTART = 32,  // restart RK: SWFD_RESTART_LIMIT dt halvings without a positive state
  ERR_BIT_TIMEOUT = 64   // a bounded device-side wait (a grid barrier) ran out
};

// conditional nesting depth of the graphs: solve WHILE > restart WHILE > IF > IF
#define SWFD_CAP_DEPTH 6

struct DevScalars {
  double alphamax;
  double dt;
  double time;
  double ubar[4];
  unsigned long long alpha_bits;
  unsigned long long rho_min_key;
  int postag;
  int bad_count;         // cells failing the sweep exit test
  int error;             // ERR_BIT_*
  int q;                 // current sweep iteration (1-based)
  int ordering;          // ordering of the current pass (0: 1D, 1: I, 2: II)
  int flux_work;         // chunk counter of the persistent flux kernel
  int flux_done;         // its warps that found the chunks exhausted (follows flux_work)
  long long t_pos, t_neg;
  long long sweep_count, den_count, pre_count, fail_count;
  long long steps;        // steps taken by the current solve launch
  long long steps_limit;  // bound of the current solve launch
  int* tracks;            // sweep_track, neg_track, pos_track: 3 x track_cap
  long long track_cap;
  // batched engine only
  int sweeping;           // this instance is inside its sweep q loop
  int dens_active;        // this instance runs the density sweep of this stage
  double t_end;           // time_terminal of the instance
  int cond;               // eager launch mode: value of the last conditional decision
  int alpha_done;         // findalpha blocks finished (the last one re-arms it)
  int rk_done;            // RK-stage blocks finished (the last one re-arms it)
  int restarts;           // restart RK: dt halvings of the current step
  double alphatemp;       // restart RK: alphamax of the step's first findalpha
  long long restart_total;  // restart RK: dt halvings of all steps
  long long rk_runs[4];   // RK stages run, by stage (1..3)
  int solve_pause;        // persistent 1D solve: the stage whose sweep is pending (0: none)
};

// The value of a conditional node: set on the graph's handle, or written to
// a condition word when the section runs as plain launches (handle 0).
__device__ __forceinline__ void set_cond(cudaGraphConditionalHandle h, int* word, unsigned v) {
  if (h) cudaGraphSetConditional(h, v);
  else *word = (int)v;
}

// One instance of the batched engine, as the batched kernels see it.
struct BatchSlot {
  Params p;
  double* st[3];          // X (step start / u0), Y, Z
  void* split;
  void* roe;
  void* flux;
  void* sweep_scratch;
  DevScalars* dsc;
  long long ncell;        // LI * LJ
  long long chunk_begin;  // first flux chunk of this slot in the batch's chunk space
  long long chunks_x;     // x-direction flux chunks
  long long chunks;       // all flux chunks
  int active;             // 1 while the instance is being advanced
  int use_limiter;
  int swp_num;
  int stop_on_fail;       // ex4: a sweep that reaches swp_num stops the instance
};

// Device scalars of the batch.
struct BatchCtl {
  int any_postag;         // some active slot flagged a cell this stage
  int n_sweeping;         // slots still inside their sweep q loop
  int flux_work;          // chunk counter of the persistent flux kernel
  int n_active;           // slots still being advanced
  long long total_chunks;
  long long total_tiles;  // cell tiles of the running slots (tile_cells cells each)
  int tile_cells;         // cells per tile of the per-cell batched kernels
  long long steps;        // steps taken by the current launch
  long long steps_limit;
  long long total_s32;    // fused FP32-bulk stage: tiles and ghost chunks of the running slots
  int cond;               // eager launch mode: value of the last conditional decision
};

// What a batched launch needs (host side).
struct BatchLaunch {
  BatchSlot* tab;           // device slot table
  BatchCtl* ctl;            // device batch scalars
  const long long* prefix;  // device flux-chunk prefix (n_slots + 1)
  const long long* tprefix; // device cell-tile prefix (n_slots + 1)
  const long long* s32prefix; // device prefix of the fused stage's tiles and ghost chunks
  int n_slots;
  long long max_cell;       // largest slot (LI*LJ)
  int fp32;
  int ubar_tree;
  int segmented;            // slots may hold rank-segmented problems (ex6)
};

}  // namespace swfd

namespace swfd {
struct Ex7;  // the detonation engine (swfd_ex7.h)
}

namespace swfd {
// The persistent 1D solve (swfd_solve1d.cu): one block per SM, each owning
// `cells` consecutive cells, the whole time loop in one cooperative launch.
#define SWFD_SOLVE1D_MAX_BLOCK 512
#define SWFD_SOLVE1D_MIN_CELLS 6
#define SWFD_SOLVE1D_MAX_CELLS 62
// per cell and stage parity: fflux (3 doubles) and the eigenvectors (15)
#define SWFD_SOLVE1D_PRE 18
// grid reductions: three sets of one word per block, each word on a
// 128-byte line of its own (the launcher fills them with ones); a block
// polls at most SWFD_SOLVE1D_POLL words per thread
#define SWFD_SOLVE1D_POLL 4
#define SWFD_SOLVE1D_WSTRIDE 16
struct Solve1dArgs {
  double* st[3];            // X (the step's start and u0), Y, Z
  double* pre;              // 2 x LI x SWFD_SOLVE1D_PRE
  unsigned long long* red;  // 3 x grid x SWFD_SOLVE1D_WSTRIDE: a block's maximum alpha bits
                            // and positivity flag
  unsigned* ready;          // per block: the epoch of its published terms (zeroed by the launcher)
  int cells;                // cells per block
  int resume;               // 1: stage 1; 2, 3: that stage after the previous stage's
                            // sweep; 4: the time advance after a stage-3 sweep
  int sweeps;               // use_limiter == 2: a failed checkpositivity pauses for sweep_lim
};
// A block's ranges in the persistent 1D solve (cells at offsets 0..LI-1,
// cell i at i + 2): owned cells [a0, a1), interface-flux cells [f0, f1]
// within 2..nx+3 (the reference's m = 0..nx+1), split cells [s0, s0 + ns) =
// [f0 - 2, f1 + 2], of which nhl cells below a0 and nhr from a1 up are the
// halo.  The kernel and its layout probe both call this.
struct Solve1dLayout {
  int a0, a1, nown, f0, f1, nf, s0, ns, nhl, nhr;
};
__host__ __device__ __forceinline__ Solve1dLayout solve1d_layout(int b, int cells, int LI,
                                                                 int nx) {
  Solve1dLayout L;
  L.a0 = b * cells;
  L.a1 = min(LI, L.a0 + cells);
  L.nown = L.a1 - L.a0;
  L.f0 = max(L.a0 - 1, 2);
  L.f1 = min(L.a1, nx + 3);
  L.nf = L.f1 - L.f0 + 1;
  L.s0 = L.f0 - 2;
  L.ns = L.nf + 4;
  L.nhl = L.a0 - L.s0;
  L.nhr = max(0, L.f1 + 3 - L.a1);
  return L;
}
struct Solve1dShape {
  int grid, block, cells;
  size_t smem;
};
}  // namespace swfd

struct swfd_handle {
  swfd_config cfg;
  swfd::Params p;
  int device = 0;
  cudaStream_t stream = nullptr;
  // state buffers (3 rotating states of nc planes each)
  double* st[3] = {nullptr, nullptr, nullptr};
  int cur = 0;  // index of the current state buffer
  // scratch planes
  double* split = nullptr;  // fp, fn (x) and gp, gn (y): 4*nc planes
  double* roe = nullptr;    // w, vx, vy, h for x (4 planes) and y (4 planes)
  double* flux = nullptr;   // fp_flux, fn_flux, gp_flux, gn_flux: 4*nc planes
  double* seg_buf = nullptr;  // ex6: per-cell alpha and alpha per rank row / column
  double* rhs_tmp = nullptr;  // nc planes (flux_divergence output)
  void* sweep_scratch = nullptr;  // flag bits, flagged list, chain results
  void* sweep_cluster = nullptr;  // cluster walks: pass-start values, carries, backup
  void* ubar_scratch = nullptr;   // u_bar: the terms and the chunks' summaries
  swfd::DevScalars* dsc = nullptr;   // device scalars
  swfd::DevScalars* hsc = nullptr;   // pinned host mirror
  // host-side run state
  double time = 0;
  std::string last_error;
  // instrumentation
  int prof_on = 0;
  cudaEvent_t ev[8] = {};
  swfd_profile prof = {};
  // CUDA graphs, built on first use: one SSP-RK3 step (with flux events),
  // a solve (WHILE time <= T - 1d-10 over the step), and sweep_lim alone
  cudaGraphExec_t g_step = nullptr, g_solve = nullptr, g_sweep = nullptr;
  int g_step_events = 0;  // g_step records the flux events (built with profiling on)
  cudaStream_t cap[SWFD_CAP_DEPTH] = {};  // capture streams, one per conditional nesting depth
  int* d_tracks = nullptr;   // device sweep tracks (3 x track_cap)
  int64_t track_cap = 0;
  // kernels per graph section, for launch accounting
  int k_stage = 0, k_sweep_fixed = 0, k_density = 0, k_q = 0, k_step = 0;
  // restart RK: kernels per step outside the loop, per loop iteration, per
  // stage 2 and per stage 3 run
  int k_rs_fixed = 0, k_rs_iter = 0, k_rs_s2 = 0, k_rs_s3 = 0;
  // steps enqueued by swfd_step_async and not yet finished, and the scalars
  // before the first of them
  int64_t pending = 0;
  swfd::DevScalars pending_before{};
  double* m1_wk = nullptr;  // the MATLAB 1D scheme's workspace
  // eager launch mode (SWFD_LAUNCH=eager): the graph sections run as plain
  // stream launches and the conditions are read back on the host; for
  // profilers that do not look inside graphs with conditional nodes
  int eager = 0;
  long long eager_launches = 0;
  // FP32-bulk 2D stages as two kernels (k_alpha_terms32, k_stage32): the
  // stage kernel's launch shape (launch_stage32), 0 = the separate kernels
  // (rank segments, the limiter, SWFD_FP32_STAGE=split)
  int stage32 = 0;
  // host staging for layout conversion
  double* h_stage = nullptr;  // pinned, nc * LI * LJ doubles
  double* d_stage = nullptr;  // device, nc * LI * LJ doubles
  // the detonation (ex7) keeps its own rank-sliced state; set only for that problem
  swfd::Ex7* ex7 = nullptr;
  // the persistent 1D solve's scratch, allocated on its first run: the
  // cells' precomputed terms, then the three reduction slots and the
  // grid-barrier counter
  void* s1_scratch = nullptr;
  int s1_refused = 0;  // the device refused the cooperative grid: graph kernels from then on
};

namespace swfd {

// api.cu
swfd_status check_config(const swfd_config& c, std::string& err);
swfd_status make_params(const swfd_config& c, Params& p, std::string& err);
void set_last_error(const std::string& m);  // the process-wide message of swfd_last_error
// initdata of the problem (ghosts included) in the layout u(nc,-2:nx+3,-2:ny+3)
void init_host_state(const Params& p, const swfd_config& cfg, double* u);

// kernels.cu
cudaError_t launch_bc(const Params& p, double* u, cudaStream_t s);
// 2D bc fused with the next stage's findalpha (no dt); not for rank segments
cudaError_t launch_bc_alpha(const Params& p, double* u, DevScalars* dsc, cudaStream_t s);
// findalpha into dsc->alphamax; with_dt: the dt rule follows (stage 1).
// dsc's alpha_bits and alpha_done are zero between launches.
cudaError_t launch_alpha(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s,
                         bool with_dt = false);
// FP32-bulk fused stage (2D, no rank segments, no limiter): [bc,] findalpha
// [and dt] with the nine splitting terms and the Roe planes of every cell
// (terms: 9 float planes of the state's pitch; roe: the splitting's Roe
// planes), then one kernel for the split fluxes, interface fluxes, RHS, RK
// combination and checkpositivity of a stage.  stage32_setup sets the
// kernel's dynamic shared memory limit (once per process and device).
cudaError_t launch_alpha_terms32(const Params& p, double* u, DevScalars* dsc, cudaStream_t s,
                                 bool bc, bool with_dt, void* terms, void* roe);
// shape: 1 = 256 threads per tile, 2 tiles per SM; 2 = 320 x 2; 3 = 256 x 3;
// 4 = 256 x 4 (default); 5 = 320 x 3
cudaError_t launch_stage32(const Params& p, int shape, int stage, const double* u,
                           const double* u0, const void* terms, const void* roe, DevScalars* dsc,
                           double* out, cudaStream_t s, cudaGraphConditionalHandle hs,
                           int decide);
cudaError_t stage32_setup();
size_t stage32_smem_bytes();
// split, roe and flux planes hold doubles (FP64) or floats (FP32 bulk)
cudaError_t launch_prep(const Params& p, const double* u, const DevScalars* dsc, void* split,
                        void* roe, cudaStream_t s, int which = 3);
cudaError_t launch_split(const Params& p, double* u, const DevScalars* dsc, void* split, void* roe,
                         cudaStream_t s, int* nk);
// work: two device ints, zero between launches (the chunk counter of the 2D
// kernel and its count of finished warps; the kernel leaves them zero)
cudaError_t launch_flux(const Params& p, const void* split, const void* roe,
                        const DevScalars* dsc, void* flux, int* work, cudaStream_t s);
// the MATLAB script's scheme (swfd_matlab1d.cu): up to max_steps steps of
// `while t < tFinal` in one single-block launch; wk holds
// matlab1d_workspace(nx) doubles
int64_t matlab1d_workspace(int n);
cudaError_t launch_matlab1d(const Params& p, double* u, double* wk, DevScalars* d,
                            long long max_steps, int periodic, int sweeping, int swp_num,
                            double cfl, cudaStream_t s);
// decide 1 / 2: set the IF condition hs (0: the condition word) to postag / !postag
cudaError_t launch_rk(const Params& p, int stage, const double* u, const double* u0,
                      const void* flux, const DevScalars* dsc, double* out, cudaStream_t s,
                      cudaGraphConditionalHandle hs, int decide);
cudaError_t launch_rhs(const Params& p, const void* flux, const DevScalars* dsc, double* rhs,
                       cudaStream_t s);
cudaError_t launch_positivity(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s);
cudaError_t launch_time_advance(DevScalars* dsc, cudaStream_t s);

// solve1d.cu: the launch shape of the persistent 1D solve (FP64, binary64
// literals); false when the problem or the device does not take it (the
// solve then runs as graph kernels)
bool solve1d_shape(const Params& p, Solve1dShape* sh);
// one cooperative launch: stages from a.resume while time <= t_loop and
// dsc->steps < dsc->steps_limit; it stops early at a stage whose
// checkpositivity failed (dsc->solve_pause = the stage) when a.sweeps
cudaError_t launch_solve1d(const Params& p, const Solve1dShape& sh, const Solve1dArgs& a,
                           DevScalars* dsc, cudaStream_t s);
cudaError_t launch_fortran_to_soa(const Params& p, const double* src, double* dst, cudaStream_t s);
cudaError_t launch_soa_to_fortran(const Params& p, const double* src, double* dst, cudaStream_t s);
// quad: the reference build's binary128 smoothness indicators and alphas
// (eps 1d-6 or 1d-12)
cudaError_t launch_weno_batch(const double* st, int64_t n, double eps, int quad, double* ul,
                              double* ur,
                              cudaStream_t s);

cudaError_t launch_batch_stage(const BatchLaunch& b, int stage, int in, int out,
                               cudaGraphConditionalHandle h_sweep, cudaStream_t s);
cudaError_t launch_batch_bc(const BatchLaunch& b, int out, cudaStream_t s);
// findalpha over the running slots' state `in` (the batch autotuner's probe)
cudaError_t launch_batch_alpha(const BatchLaunch& b, int in, cudaStream_t s);
// the FP32-bulk fused stage over the batch (every running slot 2D without
// rank segments or limiter): stage reset, findalpha with the splitting terms,
// the per-slot alphamax [and dt], the stage kernel over all slots' tiles and
// ghost chunks (stage32_items each, s32prefix), the sweep condition
cudaError_t launch_batch_stage32(const BatchLaunch& b, int stage, int in, int out,
                                 cudaGraphConditionalHandle h_sweep, cudaStream_t s);
long long stage32_items(const Params& p);
// launch-shape candidates of the flux kernel (resident blocks per SM; FP64
// values SWFD_FLUX_PAIR + b and SWFD_FLUX_LOOP + b select the lane-pair
// kernels with b blocks per SM); returns their number, the default first
#define SWFD_FLUX_PAIR 10
// SWFD_FLUX_LOOP + b: the lane-pair kernel's short form (one code path for both
// directions, the characteristic fields in a loop)
#define SWFD_FLUX_LOOP 20
// SWFD_FLUX_SHARE + b: the short form with each interface's eigenvectors
// formed once, by one lane, and shared through shared memory
#define SWFD_FLUX_SHARE 40
// the FP64 flux kernel's default shape: the short lane-pair kernel with
// shared eigenvectors, 5 blocks per SM
#define SWFD_FLUX_DEFAULT64 (SWFD_FLUX_SHARE + 5)
int flux_min_blocks_candidates(bool f32, int* out);
cudaError_t launch_batch_time_advance(const BatchLaunch& b, cudaStream_t s);
cudaError_t launch_batch_run_cond(cudaGraphConditionalHandle h, const BatchLaunch& b, int advance,
                                  cudaStream_t s);

cudaError_t launch_batch_sweep_head(const BatchLaunch& b, int out, cudaStream_t s);
cudaError_t launch_batch_sweep_iter(const BatchLaunch& b, int out, cudaGraphConditionalHandle h,
                                    cudaStream_t s);
cudaError_t launch_batch_sweep_cond(const BatchLaunch& b, cudaGraphConditionalHandle h,
                                    cudaStream_t s);

// sweep.cu
cudaError_t launch_rho_min(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s);
cudaError_t launch_density_sweep(const Params& p, double* u, cudaStream_t s);
// ubar.cu: u_bar into dsc->ubar (three kernels over the whole GPU, exact)
size_t ubar_scratch_bytes(const Params& p);
cudaError_t launch_ubar(const Params& p, const double* u, DevScalars* dsc, void* scratch,
                        cudaStream_t s);
// s = 0; s = s + w*x(m) for m = 0..n-1 in that order, into *out (device)
size_t seq_sum_scratch_bytes(int64_t n);
cudaError_t launch_seq_sum(const double* x, int64_t n, double w, double* out, void* scratch,
                           cudaStream_t s);
// ordering < 0: the pass reads its ordering from dsc->ordering
cudaError_t launch_pressure_pass(const Params& p, double* u, int ordering, int forward,
                                 DevScalars* dsc, cudaStream_t s);
cudaError_t launch_exit_count(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s);
size_t sweep_scratch_bytes(const Params& p);
size_t sweep_cluster_bytes(const Params& p);  // the cluster-parallel passes' scratch
cudaError_t launch_pressure_pass_par(const Params& p, double* u, int ordering, int forward,
                                     void* scratch, void* cluster, DevScalars* dsc,
                                     cudaStream_t s, int* nlaunch);
cudaError_t launch_density_sweep_par(const Params& p, double* u, void* scratch, void* cluster,
                                     cudaStream_t s, int* nlaunch);

}  // namespace swfd
