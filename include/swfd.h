/*
 * swfd.h -- C ABI of the GB300-native sweeping positivity-preserving
 * FD-WENO Euler time step.
 *
 * The reference (dcgriffi/Sweeping_FD_WENO) has no library interface: each
 * example is one Fortran PROGRAM whose internal procedures are called by host
 * association.  Every entry point below replaces one of those procedures (or
 * a group of them) and names it, as path:line inside the reference project.
 * A Fortran host binds them with iso_c_binding (fortran/swfd_mod.f90).
 *
 * Conventions
 *  - Every call returns swfd_status: 0 on success, a negative value on error.
 *    Nothing in the library calls exit(); the reference's `stop` paths map to
 *    status codes and the host decides whether to stop.
 *  - State arrays crossing the ABI use the reference's own layout
 *    u(ncomp, -2:nx+3, -2:ny+3), Fortran column-major (component fastest,
 *    then x index, then y index), double precision, ghost layers included.
 *    1D problems use u(3, -2:nx+3).
 *  - The handle owns all device memory.  Host arrays are only borrowed for the
 *    duration of the call that receives them.
 *  - One handle per host thread.  Each handle owns one CUDA stream.
 */
#ifndef SWFD_H
#define SWFD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWFD_ABI_VERSION 2

typedef int32_t swfd_status;
enum {
  SWFD_OK = 0,
  SWFD_ERR_INVALID = -1,        /* bad argument or configuration */
  SWFD_ERR_CUDA = -2,           /* a CUDA runtime call failed */
  SWFD_ERR_SWEEP_NOCONV = -3,   /* sweep hit swp_num without P,rho > eps
                                   (ex4_sedov_2d/main.f90:1747-1752 `stop`) */
  SWFD_ERR_PUBAR_NONPOS = -4,   /* P(u_bar) <= 0 before the pressure sweep
                                   (ex4_sedov_2d/main.f90:1447-1454 `stop`) */
  SWFD_ERR_NONFINITE = -5,      /* alpha or dt is not finite */
  SWFD_ERR_OOM = -6,            /* device allocation refused */
  SWFD_ERR_TIMEOUT = -7,        /* a bounded device-side wait expired */
  SWFD_ERR_UNSUPPORTED = -8,    /* option recognised but not implemented */
  SWFD_ERR_MAX_STEPS = -9,      /* run_to stopped at its step limit */
  SWFD_ERR_SWEEP_CHECK = -10,   /* a nodal adjustment raised the pair's total
                                   pressure (ex6_shock_diffraction/main.f90:1413-1423,
                                   1472-1482 `stop`) */
  SWFD_ERR_RESTART_LIMIT = -11  /* the dt-halving restart RK (rk_choice 2) found no
                                   positive state within SWFD_RESTART_LIMIT halvings;
                                   the reference would loop on (ex2_sedov_1d/main.f90:
                                   340-348 `goto 110`) */
};

/* Bound on the dt halvings of one restart-RK step (dt/2^1100 is 0). */
#define SWFD_RESTART_LIMIT 1100

/* Problem = one reference example, with all of its per-example switches
 * (operation order, epsilons, comparison operators, boundary conditions). */
enum {
  SWFD_PROBLEM_MATLAB_1D = 1,  /* ex1_double_rarefaction_1d/FD_WENO_Application.m: the
                                  MATLAB script's own 1D scheme (per-field Lax-Friedrichs
                                  alpha, WENO eps 1e-5, sweep after every stage); its
                                  `problem` number is config.variant (5 as shipped) */
  SWFD_PROBLEM_SEDOV_1D = 2,   /* ex2_sedov_1d/main.f90 */
  SWFD_PROBLEM_VORTEX_2D = 3,  /* ex3_vortex_accuracy_2d/main.f90 */
  SWFD_PROBLEM_SEDOV_2D = 4,   /* ex4_sedov_2d/main.f90 on one 1x1 block */
  SWFD_PROBLEM_JET_2D = 5,     /* ex5_mach2000_jet/main.f90 */
  SWFD_PROBLEM_SHOCK_DIFFRACTION = 6  /* ex6_shock_diffraction/main.f90: the
                                   reference's cut_x x cut_y MPI decomposition is
                                   part of its arithmetic (per-rank-row and
                                   per-rank-column Lax-Friedrichs alpha, fluxes at
                                   rank boundaries computed by both ranks) and is
                                   reproduced on one grid */,
  SWFD_PROBLEM_DETONATION = 7  /* ex7_detonation/main.f90: reactive Euler, five
                                  components (rho, m_x, m_y, E, rho*Y; the state
                                  is u(5,-2:nx+3,-2:ny+3)), the chemistry source
                                  on the fifth; ex6's rank decomposition with
                                  nx = cut_x*(5*total/cut_x), ny = cut_y*(5*total/cut_y),
                                  the wall's top row 2*total */
};

/* How the reference's double-kind literals (1d-6, 13d0/12d0, 0.75d0, ...)
 * are evaluated.  The reference Makefiles build with -fdefault-real-8 only,
 * under which gfortran promotes those literals (and the subexpressions that
 * contain them) to REAL(16).  SWFD_LITERALS_DOUBLE evaluates everything in
 * binary64 (the -fdefault-double-8 build). */
enum { SWFD_LITERALS_DOUBLE = 0, SWFD_LITERALS_QUAD = 1 };

/* Arithmetic of the WENO flux and the RK update.  Pressure recovery, the
 * positivity test, the sweeps and the conservation sums are always FP64. */
enum { SWFD_PRECISION_FP64 = 0, SWFD_PRECISION_FP32_BULK = 1 };

/* u_bar of the pressure sweep: the reference's sequential weighted sum
 * (ex3_vortex_accuracy_2d/main.f90:913-920), or a deterministic tree sum. */
enum { SWFD_UBAR_SEQUENTIAL = 0, SWFD_UBAR_TREE = 1 };

/* How a sweep pass walks its ordering.  Both give the reference's values and
 * counts: PARALLEL runs the independent chains of nodal adjustments
 * concurrently and follows only chains that reach the next flagged cell in
 * sequence; SEQUENTIAL walks every cell in one GPU thread. */
enum { SWFD_SWEEP_PARALLEL = 0, SWFD_SWEEP_SEQUENTIAL = 1 };

typedef struct swfd_config {
  int32_t abi_version;   /* must be SWFD_ABI_VERSION */
  int32_t problem;       /* SWFD_PROBLEM_* */
  int32_t nx, ny;        /* interior cells; ny is ignored in 1D */
  int32_t use_limiter;   /* 2 = sweeping (reference default), 0 = none,
                            1 = Zhang-Shu positivity-preserving flux limiter */
  int32_t swp_num;       /* max forward/backward sweep pairs per RK stage */
  int32_t literals;      /* SWFD_LITERALS_* */
  int32_t precision;     /* SWFD_PRECISION_* */
  int32_t ubar_mode;     /* SWFD_UBAR_* */
  int32_t device;        /* CUDA device ordinal */
  double cfl;            /* CFL number of the problem's dt rule */
  double time_terminal;  /* final time T */
  double gamma;          /* ratio of specific heats */
  double e_background;   /* point-energy problems: background total energy */
  double e_blast;        /* point-energy problems: blast energy numerator
                            (1D: E = e_blast/dx, 2D: E = e_blast/(dx*dy)) */
  int32_t sweep_mode;    /* SWFD_SWEEP_PARALLEL (default) or SWFD_SWEEP_SEQUENTIAL */
  int32_t total;         /* shock diffraction and detonation: the reference's `total`
                            (step width in cells; the step top is row 6*total,
                            detonation 2*total); 0 otherwise */
  int32_t cut_x, cut_y;  /* shock diffraction and detonation: the reference's rank
                            grid (4 x 8); shock diffraction nx = cut_x*(13*total/cut_x),
                            ny = cut_y*(11*total/cut_y) */
  int32_t rk_choice;     /* the reference's RK_choice: 1 (or 0) = SSP-RK3 with the
                            sweeping post-process (rk3); 2 = the dt-halving
                            restart RK of ex2 (`rk`, ex2_sedov_1d/main.f90:330-374:
                            a stage that fails checkpositivity restarts the step
                            from u0 with dt/2; no sweeps).  2 is 1D only. */
  int32_t variant;       /* SWFD_PROBLEM_MATLAB_1D: the script's `problem` (1 linear
                            advection, 2 nonlinear, 3 Sod, 4 Lax, 5 double rarefaction,
                            6 point energy, 7 jet ambient state);
                            SWFD_PROBLEM_JET_2D: 0 the reference's upper half domain
                            [0,1]x[0,0.25] with its y = 0 symmetry plane, 1 the full
                            domain [0,1]x[-0.25,0.25] (inflow for |y| <= 0.05, outflow
                            at the bottom; ny counts the whole height); 0 otherwise */
  int32_t reserved[2];   /* zero */
} swfd_config;

/* Sweep statistics exactly as the reference counts them
 * (ex3_vortex_accuracy_2d/main.f90:815-840; counters :14, :24-31). */
typedef struct swfd_sweep_stats {
  int64_t sweep_count;      /* sweep_lim invocations */
  int64_t total_sweep;      /* sum of sweep_track(1:sweep_count) */
  int64_t max_sweep;        /* maxval(sweep_track(1:sweep_count)) */
  int64_t total_neg;        /* negative-pair nodal adjustments */
  int64_t max_neg;
  int64_t total_pos;        /* positive-neighbour nodal adjustments */
  int64_t max_pos;
  int64_t den_count;        /* density sweeps performed */
  int64_t pre_count;        /* forward/backward sweep pairs performed */
  int64_t sweep_fail_count; /* sweeps that hit swp_num ("SWEEP FAIL") */
} swfd_sweep_stats;

typedef struct swfd_handle swfd_handle;

/* Fill cfg with the reference example's compile-time PARAMETERs
 * (ex2_sedov_1d/main.f90:4-7, ex3_vortex_accuracy_2d/main.f90:5-7,
 *  ex4_sedov_2d/main.f90:15-20,50, ex5_mach2000_jet/main.f90:4-6). */
swfd_status swfd_config_default(swfd_config* cfg, int32_t problem);

/* Allocate device state for one problem instance.  Replaces the module-level
 * arrays of each PROGRAM (ex3_vortex_accuracy_2d/main.f90:8-37) and
 * sweeping_order (:1211-1270). */
swfd_status swfd_create(const swfd_config* cfg, swfd_handle** out);
swfd_status swfd_destroy(swfd_handle* h);

/* Initial data + bc: initdata (ex3_vortex_accuracy_2d/main.f90:671-697,
 * ex2_sedov_1d/main.f90:405-428, ex4_sedov_2d/main.f90:1121-1189,
 * ex5_mach2000_jet/main.f90:744-768).  Sets time to 0, clears statistics. */
swfd_status swfd_init_problem(swfd_handle* h);

/* Copy a host state u(ncomp,-2:nx+3,-2:ny+3) in / out. */
swfd_status swfd_upload_state(swfd_handle* h, const double* u);
swfd_status swfd_download_state(swfd_handle* h, double* u);

/* wenofd + scheme (ex3_vortex_accuracy_2d/main.f90:115-547): alpha of the
 * current state, then RHS(ncomp,-2:nx+3,-2:ny+3) (zero in the ghosts). */
swfd_status swfd_flux_divergence(swfd_handle* h, double* rhs);

/* One SSP-RK3 step: rk (ex3_vortex_accuracy_2d/main.f90:564-632) followed by
 * `time = time + dt` (:53).  dt_out may be NULL. */
swfd_status swfd_step(swfd_handle* h, double* dt_out);

/* One step from a host state to a host state (a host that keeps its state
 * u(ncomp,-2:nx+3,-2:ny+3) between steps, as the reference's time loop
 * does, ex3_vortex_accuracy_2d/main.f90:51-56): upload u_in, swfd_step,
 * download into u_out, with one synchronisation at the end.  u_in may equal
 * u_out.  dt_out may be NULL. */
swfd_status swfd_step_host(swfd_handle* h, const double* u_in, double* u_out, double* dt_out);

/* The time loop DO WHILE (time <= time_terminal - 1d-10)
 * (ex3_vortex_accuracy_2d/main.f90:51-56), bounded by max_steps (<= 0: none).
 * nsteps_out may be NULL. */
swfd_status swfd_run(swfd_handle* h, int64_t max_steps, int64_t* nsteps_out);

/* swfd_step without waiting: enqueue one step on the handle's stream
 * (swfd_get_stream) and return.  swfd_finish waits for the enqueued steps and
 * reports their status; every other call on the handle finishes them first
 * (the device state is stream-ordered either way).  With profiling on,
 * swfd_finish adds the flux timings of the last enqueued step. */
swfd_status swfd_step_async(swfd_handle* h);

/* Autotuner.  swfd_autotune times the launch shapes of the flux kernel
 * (resident blocks per SM against registers per thread) on the handle's
 * current state and keeps the fastest for the handle's later steps; results
 * do not change.  Problems with rank segments or the flux limiter keep the
 * default shape (*flux_min_blocks = 0).  swfd_batch_autotune times the cell-tile
 * size of the batch's per-cell kernels on the running instances and keeps
 * the fastest. */
swfd_status swfd_autotune(swfd_handle* h, int32_t* flux_min_blocks);
swfd_status swfd_finish(swfd_handle* h);

/* Restart RK (rk_choice 2): dt halvings over all steps so far (the
 * `goto 110` restarts of ex2_sedov_1d/main.f90:350,360,370); 0 otherwise. */
swfd_status swfd_get_restarts(swfd_handle* h, int64_t* restarts);

/* sweep_lim on the current state, as called after an RK stage whose
 * checkpositivity flagged a cell (ex3_vortex_accuracy_2d/main.f90:888-1137). */
swfd_status swfd_sweep(swfd_handle* h);

/* checkpositivity (ex3_vortex_accuracy_2d/main.f90:634-651): *postag = 1 if
 * an interior cell fails the problem's positivity test. */
swfd_status swfd_check_positivity(swfd_handle* h, int32_t* postag);

/* findalpha (ex3_vortex_accuracy_2d/main.f90:549-562) of the current state. */
swfd_status swfd_find_alpha(swfd_handle* h, double* alphamax);

swfd_status swfd_get_time(swfd_handle* h, double* t);
swfd_status swfd_set_time(swfd_handle* h, double t);

/* Statistics printed by output (ex3_vortex_accuracy_2d/main.f90:815-840). */
swfd_status swfd_get_sweep_stats(swfd_handle* h, swfd_sweep_stats* s);
/* Per-sweep tracks sweep_track/neg_track/pos_track(1:sweep_count); any of
 * the output pointers may be NULL; writes min(cap, sweep_count) entries. */
swfd_status swfd_get_sweep_tracks(swfd_handle* h, int32_t* sweep, int32_t* neg,
                                  int32_t* pos, int64_t cap, int64_t* count);

/* The scalar WENO5 reconstructions of MODULE weno5, weno_left/weno_right
 * (ex3_vortex_accuracy_2d/weno5.f90:86-146), evaluated on the GPU for n
 * stencils average(-2:2) stored contiguously (5 doubles each). */
swfd_status swfd_weno5_batch(const double* stencils, int64_t n, double weno_eps,
                             int32_t literals, int32_t device, double* uleft,
                             double* uright);

/* The u_bar summation of sweep_lim (ex3_vortex_accuracy_2d/main.f90:913-920)
 * over a flat array: s = 0; DO m = 1, n: s = s + w*x(m), rounded step by step
 * in that order, evaluated on the GPU by the kernel the sweep uses
 * (a unit-test entry point; n < 2^31). */
swfd_status swfd_sequential_sum(const double* x, int64_t n, double w, int32_t device,
                                double* out);

/* ---------------------------------------------------------------------------
 * Batched engine and serving.  No counterpart in the reference, which runs one
 * problem per program (the MPI examples spread one grid over 32 ranks).  Many
 * independent 2D instances stay resident on one GPU and advance together: each
 * stage is one launch per kernel over all instances and a run is one CUDA
 * graph.  Instances are admitted and retired between runs (continuous
 * batching); each keeps its own alpha, dt, time, sweeps and statistics and
 * stops at its own time_terminal.
 * ------------------------------------------------------------------------- */
typedef struct swfd_batch swfd_batch;
typedef struct swfd_batch_config {
  int32_t max_slots;     /* instances resident at once */
  int32_t max_nx, max_ny;/* largest grid a slot accepts */
  int32_t precision;     /* SWFD_PRECISION_*, one precision for the whole batch */
  int32_t ubar_mode;     /* SWFD_UBAR_* */
  int32_t device;
  int64_t pool_bytes;    /* HBM budget for instance state; 0 = 80% of free memory */
  int32_t reserved[8];
} swfd_batch_config;

swfd_status swfd_batch_config_default(swfd_batch_config* cfg);
swfd_status swfd_batch_create(const swfd_batch_config* cfg, swfd_batch** out);
swfd_status swfd_batch_destroy(swfd_batch* b);
/* Admit one instance: initdata of cfg->problem (the batch's precision is
 * used).  SWFD_ERR_OOM when no slot or not enough of the HBM budget is free. */
swfd_status swfd_batch_admit(swfd_batch* b, const swfd_config* cfg, int64_t request_id);
/* Advance every running instance by up to max_steps SSP-RK3 steps; an
 * instance stops at its own T (DO WHILE time <= T - 1d-10) or on an error. */
swfd_status swfd_batch_run(swfd_batch* b, int64_t max_steps, int64_t* steps_out);
/* Instances that finished since the last poll, with their status. */
swfd_status swfd_batch_poll(swfd_batch* b, int64_t* ids, int32_t* status, int32_t cap,
                            int32_t* n_out);
/* State u(4,-2:nx+3,-2:ny+3) and time of an admitted instance. */
swfd_status swfd_batch_download(swfd_batch* b, int64_t request_id, double* u, double* time_out);
swfd_status swfd_batch_stats(swfd_batch* b, int64_t request_id, swfd_sweep_stats* s);
/* Free the instance's slot and memory. */
swfd_status swfd_batch_release(swfd_batch* b, int64_t request_id);
swfd_status swfd_batch_info(swfd_batch* b, int32_t* running, int32_t* free_slots,
                            int64_t* free_bytes);
/* Progress of one request: simulated time and SSP-RK3 steps taken so far
 * (from the last run; no device synchronisation beyond that). */
swfd_status swfd_batch_progress(swfd_batch* b, int64_t request_id, double* time_out,
                                int64_t* steps_out);
/* The CUDA stream (cudaStream_t) the batch's graph runs on. */
swfd_status swfd_batch_get_stream(swfd_batch* b, void** stream);
swfd_status swfd_batch_autotune(swfd_batch* b, int32_t* tile_cells);

/* Instrumentation (no counterpart in the reference, which only prints a
 * wall-clock "CPU Time", ex4_sedov_2d/main.f90:111,118-119). */
typedef struct swfd_profile {
  int64_t kernel_launches;  /* kernels this handle launched since the reset */
  int64_t stages;           /* RK stages executed */
  int64_t flux_launches;    /* WENO flux kernel launches timed with events */
  double flux_ms;           /* summed event time of those launches */
  int64_t sweep_invocations;
  double sweep_ms;          /* summed event time of sweep_lim work */
} swfd_profile;

/* The CUDA stream (cudaStream_t) every kernel of this handle runs on. */
swfd_status swfd_get_stream(swfd_handle* h, void** stream);
/* on != 0: bracket the flux kernels and the sweep with CUDA events. */
swfd_status swfd_set_profiling(swfd_handle* h, int32_t on);
swfd_status swfd_get_profile(swfd_handle* h, swfd_profile* prof);
swfd_status swfd_reset_profile(swfd_handle* h);

/* swfd_flux_divergence without any allocation.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc, such as code
 * running under an allocator that owns all device memory (a framework's
 * caching allocator or a memory pool that forbids other allocations),
 * real-time loops where an allocation may block, or callers that only hold
 * device pointers they were handed.
 *
 * u and rhs are DEVICE arrays in the layout u(ncomp,-2:nx+3,-2:ny+3) of the
 * current ABI (rhs is zero in the ghosts); the work is queued on `stream`
 * (a cudaStream_t; NULL = the legacy default stream) and the call returns
 * without waiting.  cfg selects the problem and device as for swfd_create.
 * Every intermediate lives in one file-scope device array of 8 MiB that each
 * GPU loading the library holds until the process exits; grids that do not
 * fit (beyond about 130 x 130 cells in 2D, 27000 cells in 1D) are rejected
 * with SWFD_ERR_INVALID and a message in swfd_last_error(NULL, ...).
 * All calls share that array and it keeps the last call's contents: calls
 * whose work overlaps on the GPU race and corrupt each other, so order them
 * on one stream.  The first call on a device looks up the array's address
 * with that device current; make it before any stream capture.  Calls on a
 * stream that is not capturing look the address up again (a cudaDeviceReset
 * followed by a new context is followed); calls during capture reuse it. */
swfd_status swfd_flux_divergence_static(const swfd_config* cfg, const double* u, double* rhs,
                                        void* stream);

/* Last error message of the handle (or of the process when h is NULL). */
swfd_status swfd_last_error(swfd_handle* h, char* buf, size_t len);
const char* swfd_status_string(swfd_status s);

#ifdef __cplusplus
}
#endif
#endif /* SWFD_H */
