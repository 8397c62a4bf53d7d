! swfd_mod.f90 -- iso_c_binding interface of libswfd (include/swfd.h) for the
! reference's Fortran hosts.
!
! The reference examples are single PROGRAMs whose procedures share state by
! host association (ex3_vortex_accuracy_2d/main.f90:1-57).  A host that adds
! `use swfd_mod` replaces its CALL rk loop (:51-56) with swfd_step / swfd_run
! on a handle, keeps its own PARAMETERs (use_limiter, swp_num, cfl, grid,
! time_terminal) in a swfd_config, passes its state array
! u(ncomp,-2:nx+3,-2:ny+3) as it is (the library uses the same column-major
! layout, ghosts included) and prints its statistics block from
! swfd_sweep_stats.  Every function returns a status: 0 on success, negative
! on error (the reference's `stop`s become SWFD_ERR_*).
!
! No Fortran compiler exists in the build image, so this file is checked as
! text: tests/test_fortran_binding.py compares every interface below with the
! prototypes of include/swfd.h and the ctypes prototypes of the package.
module swfd_mod
  use iso_c_binding
  implicit none

  integer(c_int32_t), parameter :: SWFD_ABI_VERSION = 2

  ! status codes
  integer(c_int32_t), parameter :: SWFD_OK = 0
  integer(c_int32_t), parameter :: SWFD_ERR_INVALID = -1
  integer(c_int32_t), parameter :: SWFD_ERR_CUDA = -2
  integer(c_int32_t), parameter :: SWFD_ERR_SWEEP_NOCONV = -3   ! "SWEEP FAIL" stop
  integer(c_int32_t), parameter :: SWFD_ERR_PUBAR_NONPOS = -4   ! P(u_bar) <= 0 stop
  integer(c_int32_t), parameter :: SWFD_ERR_NONFINITE = -5
  integer(c_int32_t), parameter :: SWFD_ERR_OOM = -6
  integer(c_int32_t), parameter :: SWFD_ERR_TIMEOUT = -7
  integer(c_int32_t), parameter :: SWFD_ERR_UNSUPPORTED = -8
  integer(c_int32_t), parameter :: SWFD_ERR_MAX_STEPS = -9
  integer(c_int32_t), parameter :: SWFD_ERR_SWEEP_CHECK = -10   ! ex6 "Sweep check failed"
  integer(c_int32_t), parameter :: SWFD_ERR_RESTART_LIMIT = -11

  ! problems: one per reference example
  integer(c_int32_t), parameter :: SWFD_PROBLEM_MATLAB_1D = 1
  integer(c_int32_t), parameter :: SWFD_PROBLEM_SEDOV_1D = 2
  integer(c_int32_t), parameter :: SWFD_PROBLEM_VORTEX_2D = 3
  integer(c_int32_t), parameter :: SWFD_PROBLEM_SEDOV_2D = 4
  integer(c_int32_t), parameter :: SWFD_PROBLEM_JET_2D = 5
  integer(c_int32_t), parameter :: SWFD_PROBLEM_SHOCK_DIFFRACTION = 6
  integer(c_int32_t), parameter :: SWFD_PROBLEM_DETONATION = 7

  ! evaluation of the double-kind literals: binary64, or binary128 as the
  ! -fdefault-real-8 build of the reference evaluates them
  integer(c_int32_t), parameter :: SWFD_LITERALS_DOUBLE = 0
  integer(c_int32_t), parameter :: SWFD_LITERALS_QUAD = 1
  integer(c_int32_t), parameter :: SWFD_PRECISION_FP64 = 0
  integer(c_int32_t), parameter :: SWFD_PRECISION_FP32_BULK = 1
  integer(c_int32_t), parameter :: SWFD_UBAR_SEQUENTIAL = 0
  integer(c_int32_t), parameter :: SWFD_UBAR_TREE = 1
  integer(c_int32_t), parameter :: SWFD_SWEEP_PARALLEL = 0
  integer(c_int32_t), parameter :: SWFD_SWEEP_SEQUENTIAL = 1

  ! the PARAMETERs of one example (swfd_config_default fills the reference's)
  type, bind(C) :: swfd_config
    integer(c_int32_t) :: abi_version
    integer(c_int32_t) :: problem
    integer(c_int32_t) :: nx
    integer(c_int32_t) :: ny
    integer(c_int32_t) :: use_limiter   ! 2 sweeping, 1 flux limiter, 0 none
    integer(c_int32_t) :: swp_num
    integer(c_int32_t) :: literals
    integer(c_int32_t) :: precision
    integer(c_int32_t) :: ubar_mode
    integer(c_int32_t) :: device
    real(c_double) :: cfl
    real(c_double) :: time_terminal
    real(c_double) :: gamma
    real(c_double) :: e_background
    real(c_double) :: e_blast
    integer(c_int32_t) :: sweep_mode
    integer(c_int32_t) :: total         ! ex6 / ex7 PARAMETER total
    integer(c_int32_t) :: cut_x         ! ex6 / ex7 rank grid
    integer(c_int32_t) :: cut_y
    integer(c_int32_t) :: rk_choice     ! ex2 PARAMETER RK_choice
    integer(c_int32_t) :: variant       ! ex1: the MATLAB script's `problem`
    integer(c_int32_t) :: reserved(2)
  end type swfd_config

  ! the statistics block of `output` (ex3_vortex_accuracy_2d/main.f90:815-840)
  type, bind(C) :: swfd_sweep_stats
    integer(c_int64_t) :: sweep_count
    integer(c_int64_t) :: total_sweep
    integer(c_int64_t) :: max_sweep
    integer(c_int64_t) :: total_neg
    integer(c_int64_t) :: max_neg
    integer(c_int64_t) :: total_pos
    integer(c_int64_t) :: max_pos
    integer(c_int64_t) :: den_count
    integer(c_int64_t) :: pre_count
    integer(c_int64_t) :: sweep_fail_count
  end type swfd_sweep_stats

  type, bind(C) :: swfd_profile
    integer(c_int64_t) :: kernel_launches
    integer(c_int64_t) :: stages
    integer(c_int64_t) :: flux_launches
    real(c_double) :: flux_ms
    integer(c_int64_t) :: sweep_invocations
    real(c_double) :: sweep_ms
  end type swfd_profile

  type, bind(C) :: swfd_batch_config
    integer(c_int32_t) :: max_slots
    integer(c_int32_t) :: max_nx
    integer(c_int32_t) :: max_ny
    integer(c_int32_t) :: precision
    integer(c_int32_t) :: ubar_mode
    integer(c_int32_t) :: device
    integer(c_int64_t) :: pool_bytes
    integer(c_int32_t) :: reserved(8)
  end type swfd_batch_config

  interface
    ! ---- one problem instance ------------------------------------------
    integer(c_int32_t) function swfd_config_default(cfg, problem) &
        bind(C, name="swfd_config_default")
      import :: c_int32_t, swfd_config
      type(swfd_config) :: cfg
      integer(c_int32_t), value :: problem
    end function

    integer(c_int32_t) function swfd_create(cfg, h) bind(C, name="swfd_create")
      import :: c_int32_t, c_ptr, swfd_config
      type(swfd_config) :: cfg
      type(c_ptr) :: h
    end function

    integer(c_int32_t) function swfd_destroy(h) bind(C, name="swfd_destroy")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
    end function

    ! initdata + bc
    integer(c_int32_t) function swfd_init_problem(h) bind(C, name="swfd_init_problem")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int32_t) function swfd_upload_state(h, u) bind(C, name="swfd_upload_state")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: u(*)
    end function

    integer(c_int32_t) function swfd_download_state(h, u) bind(C, name="swfd_download_state")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: u(*)
    end function

    ! wenofd + scheme
    integer(c_int32_t) function swfd_flux_divergence(h, rhs) &
        bind(C, name="swfd_flux_divergence")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: rhs(*)
    end function

    ! CALL rk; time = time + dt
    integer(c_int32_t) function swfd_step(h, dt) bind(C, name="swfd_step")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: dt
    end function

    ! CALL rk on the host's own u, in and out, with one synchronisation
    integer(c_int32_t) function swfd_step_host(h, u_in, u_out, dt) &
        bind(C, name="swfd_step_host")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: u_in(*)
      real(c_double) :: u_out(*)
      real(c_double) :: dt
    end function

    ! DO WHILE (time <= time_terminal - 1d-10)
    integer(c_int32_t) function swfd_run(h, max_steps, nsteps) bind(C, name="swfd_run")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: h
      integer(c_int64_t), value :: max_steps
      integer(c_int64_t) :: nsteps
    end function

    integer(c_int32_t) function swfd_step_async(h) bind(C, name="swfd_step_async")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int32_t) function swfd_autotune(h, flux_min_blocks) bind(C, name="swfd_autotune")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
      integer(c_int32_t) :: flux_min_blocks
    end function

    integer(c_int32_t) function swfd_finish(h) bind(C, name="swfd_finish")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int32_t) function swfd_get_restarts(h, restarts) bind(C, name="swfd_get_restarts")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: h
      integer(c_int64_t) :: restarts
    end function

    ! sweep_lim
    integer(c_int32_t) function swfd_sweep(h) bind(C, name="swfd_sweep")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
    end function

    ! checkpositivity
    integer(c_int32_t) function swfd_check_positivity(h, postag) &
        bind(C, name="swfd_check_positivity")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
      integer(c_int32_t) :: postag
    end function

    ! findalpha
    integer(c_int32_t) function swfd_find_alpha(h, alphamax) bind(C, name="swfd_find_alpha")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: alphamax
    end function

    integer(c_int32_t) function swfd_get_time(h, t) bind(C, name="swfd_get_time")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: t
    end function

    integer(c_int32_t) function swfd_set_time(h, t) bind(C, name="swfd_set_time")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), value :: t
    end function

    integer(c_int32_t) function swfd_get_sweep_stats(h, s) bind(C, name="swfd_get_sweep_stats")
      import :: c_int32_t, c_ptr, swfd_sweep_stats
      type(c_ptr), value :: h
      type(swfd_sweep_stats) :: s
    end function

    ! sweep_track, neg_track, pos_track (1:sweep_count)
    integer(c_int32_t) function swfd_get_sweep_tracks(h, sweep, neg, pos, cap, count) &
        bind(C, name="swfd_get_sweep_tracks")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: h
      integer(c_int32_t) :: sweep(*)
      integer(c_int32_t) :: neg(*)
      integer(c_int32_t) :: pos(*)
      integer(c_int64_t), value :: cap
      integer(c_int64_t) :: count
    end function

    ! MODULE weno5: weno_left / weno_right on n stencils average(-2:2)
    integer(c_int32_t) function swfd_weno5_batch(stencils, n, weno_eps, literals, device, &
                                                 uleft, uright) bind(C, name="swfd_weno5_batch")
      import :: c_int32_t, c_int64_t, c_double
      real(c_double) :: stencils(*)
      integer(c_int64_t), value :: n
      real(c_double), value :: weno_eps
      integer(c_int32_t), value :: literals
      integer(c_int32_t), value :: device
      real(c_double) :: uleft(*)
      real(c_double) :: uright(*)
    end function

    integer(c_int32_t) function swfd_sequential_sum(x, n, w, device, out) &
        bind(C, name="swfd_sequential_sum")
      import :: c_int32_t, c_int64_t, c_double
      real(c_double) :: x(*)
      integer(c_int64_t), value :: n
      real(c_double), value :: w
      integer(c_int32_t), value :: device
      real(c_double) :: out
    end function

    ! ---- batched engine and serving ------------------------------------
    integer(c_int32_t) function swfd_batch_config_default(cfg) &
        bind(C, name="swfd_batch_config_default")
      import :: c_int32_t, swfd_batch_config
      type(swfd_batch_config) :: cfg
    end function

    integer(c_int32_t) function swfd_batch_create(cfg, b) bind(C, name="swfd_batch_create")
      import :: c_int32_t, c_ptr, swfd_batch_config
      type(swfd_batch_config) :: cfg
      type(c_ptr) :: b
    end function

    integer(c_int32_t) function swfd_batch_destroy(b) bind(C, name="swfd_batch_destroy")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: b
    end function

    integer(c_int32_t) function swfd_batch_admit(b, cfg, request_id) &
        bind(C, name="swfd_batch_admit")
      import :: c_int32_t, c_int64_t, c_ptr, swfd_config
      type(c_ptr), value :: b
      type(swfd_config) :: cfg
      integer(c_int64_t), value :: request_id
    end function

    integer(c_int32_t) function swfd_batch_run(b, max_steps, steps) bind(C, name="swfd_batch_run")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: b
      integer(c_int64_t), value :: max_steps
      integer(c_int64_t) :: steps
    end function

    integer(c_int32_t) function swfd_batch_poll(b, ids, status, cap, n) &
        bind(C, name="swfd_batch_poll")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: b
      integer(c_int64_t) :: ids(*)
      integer(c_int32_t) :: status(*)
      integer(c_int32_t), value :: cap
      integer(c_int32_t) :: n
    end function

    integer(c_int32_t) function swfd_batch_download(b, request_id, u, time) &
        bind(C, name="swfd_batch_download")
      import :: c_int32_t, c_int64_t, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int64_t), value :: request_id
      real(c_double) :: u(*)
      real(c_double) :: time
    end function

    integer(c_int32_t) function swfd_batch_stats(b, request_id, s) bind(C, name="swfd_batch_stats")
      import :: c_int32_t, c_int64_t, c_ptr, swfd_sweep_stats
      type(c_ptr), value :: b
      integer(c_int64_t), value :: request_id
      type(swfd_sweep_stats) :: s
    end function

    integer(c_int32_t) function swfd_batch_release(b, request_id) &
        bind(C, name="swfd_batch_release")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: b
      integer(c_int64_t), value :: request_id
    end function

    integer(c_int32_t) function swfd_batch_info(b, running, free_slots, free_bytes) &
        bind(C, name="swfd_batch_info")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: b
      integer(c_int32_t) :: running
      integer(c_int32_t) :: free_slots
      integer(c_int64_t) :: free_bytes
    end function

    integer(c_int32_t) function swfd_batch_progress(b, request_id, time, steps) &
        bind(C, name="swfd_batch_progress")
      import :: c_int32_t, c_int64_t, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int64_t), value :: request_id
      real(c_double) :: time
      integer(c_int64_t) :: steps
    end function

    integer(c_int32_t) function swfd_batch_get_stream(b, stream) &
        bind(C, name="swfd_batch_get_stream")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: b
      type(c_ptr) :: stream
    end function

    integer(c_int32_t) function swfd_batch_autotune(b, tile_cells) &
        bind(C, name="swfd_batch_autotune")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: b
      integer(c_int32_t) :: tile_cells
    end function

    ! ---- instrumentation -----------------------------------------------
    integer(c_int32_t) function swfd_get_stream(h, stream) bind(C, name="swfd_get_stream")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
      type(c_ptr) :: stream
    end function

    integer(c_int32_t) function swfd_set_profiling(h, on) bind(C, name="swfd_set_profiling")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
      integer(c_int32_t), value :: on
    end function

    integer(c_int32_t) function swfd_get_profile(h, prof) bind(C, name="swfd_get_profile")
      import :: c_int32_t, c_ptr, swfd_profile
      type(c_ptr), value :: h
      type(swfd_profile) :: prof
    end function

    integer(c_int32_t) function swfd_reset_profile(h) bind(C, name="swfd_reset_profile")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: h
    end function

    ! wenofd + scheme on device arrays, with no allocation (u and rhs are
    ! device addresses, stream a cudaStream_t)
    integer(c_int32_t) function swfd_flux_divergence_static(cfg, u, rhs, stream) &
        bind(C, name="swfd_flux_divergence_static")
      import :: c_int32_t, c_ptr, swfd_config
      type(swfd_config) :: cfg
      type(c_ptr), value :: u
      type(c_ptr), value :: rhs
      type(c_ptr), value :: stream
    end function

    ! ---- errors --------------------------------------------------------
    integer(c_int32_t) function swfd_last_error(h, buf, len) bind(C, name="swfd_last_error")
      import :: c_int32_t, c_ptr, c_char, c_size_t
      type(c_ptr), value :: h
      character(kind=c_char) :: buf(*)
      integer(c_size_t), value :: len
    end function

    ! returns a C string (const char*)
    type(c_ptr) function swfd_status_string(s) bind(C, name="swfd_status_string")
      import :: c_ptr, c_int32_t
      integer(c_int32_t), value :: s
    end function
  end interface
end module swfd_mod
