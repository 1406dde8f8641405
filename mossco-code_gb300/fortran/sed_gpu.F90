!> @file sed_gpu.F90
!! @brief ISO_C_BINDING interface to the GB300 sediment-column solver.
!!
!! Binds the C ABI of include/mossco_sed.h for MOSSCO's Fortran host.  The
!! module mirrors the reference's call `call ode_solver(sed, dt, method)`
!! (src/utilities/solver_library.F90:80) with `call sed_gpu_ode_solver(gpu,
!! sed, dt, method, rc)`, which advances sed%conc in place and applies the
!! component's NaN check and clamp (src/components/fabm_sediment_component.F90
!! :1715-1732) on the device.  Arrays are passed in their Fortran layout:
!! conc(i,j,k,n), bdys(i,j,n+1), fluxes(i,j,n) are exactly the C ABI's
!! [ntr][kmax][ncol], [ntr+1][ncol], [ntr][ncol] with col = i + inum*(j-1).
module sed_gpu

  use iso_c_binding
  implicit none
  private

  integer, parameter, public :: SED_NTR = 11
  integer, parameter, public :: SED_NBGC = 17
  integer, parameter, public :: SED_HIST_BINS = 16, SED_KMAX_LIMIT = 127
  integer, parameter, public :: SED_OK = 0, SED_E_ARG = -1, SED_E_NAN = -2
  integer, parameter, public :: SED_E_SUBSTEP_CAP = -3, SED_E_CUDA = -4
  integer, parameter, public :: SED_E_STATE = -5, SED_E_NOMEM = -6
  integer, parameter, public :: SED_E_NODEVICE = -7
  integer, parameter, public :: SED_FP32 = 0, SED_FP64 = 1
  integer, parameter, public :: SED_CUT_PER_COLUMN = 0, SED_CUT_GLOBAL = 1
  !> ode_solver methods (solver_library.F90:32-35)
  integer, parameter, public :: SED_EULER = 0, SED_RUNGE_KUTTA_4 = 1, &
                                SED_ADAPTIVE_EULER = 2, SED_RUNGE_KUTTA_4_38 = 3

  !> sed_params of mossco_sed.h (same member order and kinds)
  type, bind(C), public :: sed_params_t
    real(c_double)  :: diffusivity, bioturbation
    integer(c_int)  :: bcup_dissolved, bcup_particulate, mol_diff_mode
    real(c_double)  :: mol_diff_d0
    real(c_double)  :: dt_min, relative_change_min, atol
    integer(c_int)  :: max_attempts, cut_scope
    real(c_double)  :: rLabile, rSemilabile, NCrLdet, NCrSdet, PAds, PAdsODU, &
                       NH3Ads, CprodMax, rnit, ksO2nitri, rODUox, ksO2oduox, &
                       ksO2oxic, ksNO3denit, kinO2denit, kinNO3anox, kinO2anox
    integer(c_int)  :: epilogue
    real(c_double)  :: minimum(SED_NTR)
    integer(c_int)  :: precision, budgets, device
    !> bioturbation_profile 3: Zhang & Wirtz factor from the TOC profile
    integer(c_int)  :: bioturbation_profile
    real(c_double)  :: bioturb_k_l, bioturb_L1, bioturb_L2, bioturb_beta, &
                       bioturb_b, bioturb_dry_density
    !> > 0: microbial rates times exp(-temp_activation (1/(T+273) - 1/288))
    real(c_double)  :: temp_activation
    !> type_rhs_driver's adaptive_solver_diagnostics (grid-wide cut)
    integer(c_int)  :: adaptive_solver_diagnostics
  end type

  type, bind(C), public :: sed_stats_t
    integer(c_long_long) :: attempts, accepted, column_steps
    integer(c_int)       :: max_col_attempts, capped_columns, nan_cells, &
                            gpu_launches
    real(c_double)       :: min_dt, device_ms
    integer(c_long_long) :: surrogate_columns
  end type

  !> sed_tuning of mossco_sed.h: launch choices per depth class (1: up to
  !! 32 layers, 2: 33..64), sed_ode_solver's pipeline depth, substep cap
  type, bind(C), public :: sed_tuning_t
    integer(c_int) :: tile_columns(2), threads(2), blocks_per_sm(2)
    integer(c_int) :: pipeline_chunks, segments, max_attempts
    real(c_float)  :: step_ms, ode_solver_ms
    integer(c_int) :: trials
  end type
  integer, parameter, public :: SED_TUNE_PIPELINE = 1, SED_TUNE_CAP = 2
  integer, parameter, public :: SED_SPINUP_COLUMN = 0, SED_SPINUP_ALL = 1

  !> a solver handle
  type, public :: sed_gpu_t
    type(c_ptr) :: h = c_null_ptr
  end type

  interface
    integer(c_int) function sed_default_params(p) bind(C, name='sed_default_params')
      import :: c_int, sed_params_t
      type(sed_params_t), intent(out) :: p
    end function
    integer(c_int) function sed_create(p, inum, jnum, kmax, ntr, h) bind(C, name='sed_create')
      import :: c_int, c_ptr, sed_params_t
      type(sed_params_t), intent(in) :: p
      integer(c_int), value :: inum, jnum, kmax, ntr
      type(c_ptr), intent(out) :: h
    end function
    integer(c_int) function sed_set_grid(h, dz, dzc, phi, phi_i, biofac, flux_cap, kact, mask) &
        bind(C, name='sed_set_grid')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, dz, dzc, phi, phi_i, biofac, flux_cap, kact, mask
    end function
    integer(c_int) function sed_ode_solver(h, conc, bdys, fluxes, dt, method, st) &
        bind(C, name='sed_ode_solver')
      import :: c_int, c_ptr, c_double, sed_stats_t
      type(c_ptr), value :: h, conc, bdys, fluxes
      real(c_double), value :: dt
      integer(c_int), value :: method
      type(sed_stats_t), intent(out) :: st
    end function
    !> an OMEXDIA+P parameter set per column, params(i,j,1:SED_NBGC) in
    !! sed_params_t's order (c_null_ptr: the handle's set)
    integer(c_int) function sed_set_column_bgc(h, params) bind(C, name='sed_set_column_bgc')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, params
    end function
    integer(c_int) function sed_get_rhs(h, conc, rhs, fluxes) bind(C, name='sed_get_rhs')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, conc, rhs, fluxes
    end function
    integer(c_int) function sed_set_forcing(h, bdys, fluxes) bind(C, name='sed_set_forcing')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, bdys, fluxes
    end function
    !> device-resident state for many coupling steps (a coupled run keeps
    !! conc on the device between sed_step calls)
    integer(c_int) function sed_set_state(h, conc) bind(C, name='sed_set_state')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, conc
    end function
    integer(c_int) function sed_get_state(h, conc) bind(C, name='sed_get_state')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, conc
    end function
    integer(c_int) function sed_step(h, dt, method, nsteps, st) bind(C, name='sed_step')
      import :: c_int, c_ptr, c_double, sed_stats_t
      type(c_ptr), value :: h
      real(c_double), value :: dt
      integer(c_int), value :: method, nsteps
      type(sed_stats_t), intent(out) :: st
    end function
    integer(c_int) function sed_spinup(h, mode, column, bdys1, fluxes1, dt, method, nsteps, st) &
        bind(C, name='sed_spinup')
      import :: c_int, c_ptr, c_double, c_long_long, sed_stats_t
      type(c_ptr), value :: h, bdys1, fluxes1
      integer(c_int), value :: mode, column, method
      real(c_double), value :: dt
      integer(c_long_long), value :: nsteps
      type(sed_stats_t), intent(out) :: st
    end function
    integer(c_int) function sed_set_boundary(h, temperature, surface, velocity, present) &
        bind(C, name='sed_set_boundary')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, temperature, surface, velocity, present
    end function
    integer(c_int) function sed_get_min_dt(h, min_dt) bind(C, name='sed_get_min_dt')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, min_dt
    end function
    integer(c_int) function sed_get_min_dt_grid_cell(h, last_min_dt, cell) &
        bind(C, name='sed_get_min_dt_grid_cell')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, last_min_dt, cell
    end function
    integer(c_int) function sed_get_boundary(h, bdys, fluxes) bind(C, name='sed_get_boundary')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, bdys, fluxes
    end function
    integer(c_int) function sed_host_register(ptr, bytes) bind(C, name='sed_host_register')
      import :: c_int, c_ptr, c_size_t
      type(c_ptr), value :: ptr
      integer(c_size_t), value :: bytes
    end function
    integer(c_int) function sed_get_tuning(h, t) bind(C, name='sed_get_tuning')
      import :: c_int, c_ptr, sed_tuning_t
      type(c_ptr), value :: h
      type(sed_tuning_t), intent(out) :: t
    end function
    integer(c_int) function sed_set_tuning(h, t) bind(C, name='sed_set_tuning')
      import :: c_int, c_ptr, sed_tuning_t
      type(c_ptr), value :: h
      type(sed_tuning_t), intent(in) :: t
    end function
    integer(c_int) function sed_autotune(h, dt, method, flags, t) bind(C, name='sed_autotune')
      import :: c_int, c_ptr, c_double, sed_tuning_t
      type(c_ptr), value :: h
      real(c_double), value :: dt
      integer(c_int), value :: method, flags
      type(sed_tuning_t), intent(out) :: t
    end function
    subroutine sed_destroy(h) bind(C, name='sed_destroy')
      import :: c_ptr
      type(c_ptr), value :: h
    end subroutine
    !> diagnostics of the last step: surface fluxes [SED_NTR][ncol] (get_rhs
    !! :692), attempts [ncol], FP64 budgets [4][ncol]
    integer(c_int) function sed_get_fluxes(h, fluxes) bind(C, name='sed_get_fluxes')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, fluxes
    end function
    integer(c_int) function sed_get_attempts(h, attempts) bind(C, name='sed_get_attempts')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, attempts
    end function
    !> substep histogram of the last step: counts(SED_HIST_BINS), bin 0 no
    !! attempt, bin b attempts in [2**(b-1), 2**b), the last bin all above
    integer(c_int) function sed_get_attempt_histogram(h, counts) &
        bind(C, name='sed_get_attempt_histogram')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: h
      integer(c_long_long), intent(out) :: counts(*)
    end function
    integer(c_int) function sed_get_budgets(h, budgets) bind(C, name='sed_get_budgets')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, budgets
    end function
    !> the handle's work on a caller's cudaStream_t (c_ptr)
    integer(c_int) function sed_set_stream(h, stream) bind(C, name='sed_set_stream')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, stream
    end function
    integer(c_int) function sed_host_unregister(ptr) bind(C, name='sed_host_unregister')
      import :: c_int, c_ptr
      type(c_ptr), value :: ptr
    end function
    !> pinned host memory for the state, bdys and fluxes arrays (c_f_pointer
    !! gives the Fortran array); freed by sed_host_free
    integer(c_int) function sed_host_alloc(bytes, ptr) bind(C, name='sed_host_alloc')
      import :: c_int, c_ptr, c_size_t
      integer(c_size_t), value :: bytes
      type(c_ptr), intent(out) :: ptr
    end function
    integer(c_int) function sed_host_free(ptr) bind(C, name='sed_host_free')
      import :: c_int, c_ptr
      type(c_ptr), value :: ptr
    end function
    !> one drop-in coupling step without a handle and without allocation
    integer(c_int) function sed_ode_solver_noalloc(p, inum, jnum, kmax, dz, dzc, phi, phi_i, &
        biofac, flux_cap, kact, conc, bdys, fluxes, dt, method, st) &
        bind(C, name='sed_ode_solver_noalloc')
      import :: c_int, c_ptr, c_double, sed_params_t, sed_stats_t
      type(sed_params_t), intent(in) :: p
      integer(c_int), value :: inum, jnum, kmax
      type(c_ptr), value :: dz, dzc, phi, phi_i, biofac, flux_cap, kact, conc, bdys, fluxes
      real(c_double), value :: dt
      integer(c_int), value :: method
      type(sed_stats_t), intent(out) :: st
    end function
    !> Column-increment surrogate (no counterpart in the reference): an MLP
    !! whose trained state a Fortran component loads from arrays (state of
    !! sed_sur_state_size floats, norm of 11 + 2 nin + 2 nout floats, both as
    !! the Python side's Surrogate.checkpoint() gives them) and then steps
    !! with sed_step_surrogate or sed_ode_solver_surrogate.  Arrays are
    !! c_loc of real(c_float) / real(c_double) arrays; s is the surrogate's
    !! handle (type(c_ptr)).
    integer(c_int) function sed_sur_create(nin, nout, hidden, nhidden, max_batch, seed, &
        device, s) bind(C, name='sed_sur_create')
      import :: c_int, c_ptr, c_long_long
      integer(c_int), value :: nin, nout, hidden, nhidden, max_batch
      integer(c_long_long), value :: seed
      integer(c_int), value :: device
      type(c_ptr), intent(out) :: s
    end function
    integer(c_int) function sed_sur_num_params(s) bind(C, name='sed_sur_num_params')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function sed_sur_set_weights(s, params) bind(C, name='sed_sur_set_weights')
      import :: c_int, c_ptr
      type(c_ptr), value :: s, params
    end function
    integer(c_int) function sed_sur_get_weights(s, params) bind(C, name='sed_sur_get_weights')
      import :: c_int, c_ptr
      type(c_ptr), value :: s, params
    end function
    integer(c_int) function sed_sur_state_size(s) bind(C, name='sed_sur_state_size')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function sed_sur_get_state(s, state, step) bind(C, name='sed_sur_get_state')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: s, state
      integer(c_long_long), intent(out) :: step
    end function
    integer(c_int) function sed_sur_set_state(s, state, step) bind(C, name='sed_sur_set_state')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: s, state
      integer(c_long_long), value :: step
    end function
    integer(c_int) function sed_sur_set_norm(s, norm, n) bind(C, name='sed_sur_set_norm')
      import :: c_int, c_ptr
      type(c_ptr), value :: s, norm
      integer(c_int), value :: n
    end function
    !> host rows x(nin, m) -> y(nout, m) (the C rows [m][nin], [m][nout])
    integer(c_int) function sed_sur_forward(s, x, y, m) bind(C, name='sed_sur_forward')
      import :: c_int, c_ptr
      type(c_ptr), value :: s, x, y
      integer(c_int), value :: m
    end function
    !> device rows (device addresses as c_ptr), m a multiple of 128
    integer(c_int) function sed_sur_forward_device(s, x_dev, y_dev, m) &
        bind(C, name='sed_sur_forward_device')
      import :: c_int, c_ptr
      type(c_ptr), value :: s, x_dev, y_dev
      integer(c_int), value :: m
    end function
    !> one Adam step on a device batch; loss: c_loc of a real(c_float), or
    !! c_null_ptr
    integer(c_int) function sed_sur_train_step(s, x_dev, y_dev, m, lr, loss) &
        bind(C, name='sed_sur_train_step')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: s, x_dev, y_dev
      integer(c_int), value :: m
      real(c_float), value :: lr
      type(c_ptr), value :: loss
    end function
    integer(c_int) function sed_sur_grads(s, x, y, m, grads, loss) bind(C, name='sed_sur_grads')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: s, x, y
      integer(c_int), value :: m
      type(c_ptr), value :: grads
      real(c_float), intent(out) :: loss
    end function
    integer(c_int) function sed_sur_set_tensor_cores(s, on) bind(C, name='sed_sur_set_tensor_cores')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
      integer(c_int), value :: on
    end function
    integer(c_int) function sed_sur_set_stream(s, stream) bind(C, name='sed_sur_set_stream')
      import :: c_int, c_ptr
      type(c_ptr), value :: s, stream
    end function
    type(c_ptr) function sed_sur_last_error(s) bind(C, name='sed_sur_last_error')
      import :: c_ptr
      type(c_ptr), value :: s
    end function
    !> nsteps gated surrogate coupling steps of the handle's device state
    integer(c_int) function sed_step_surrogate(h, s, dt, nsteps, tol, res_atol, st) &
        bind(C, name='sed_step_surrogate')
      import :: c_int, c_ptr, c_double, sed_stats_t
      type(c_ptr), value :: h, s
      real(c_double), value :: dt
      integer(c_int), value :: nsteps
      real(c_double), value :: tol, res_atol
      type(sed_stats_t), intent(out) :: st
    end function
    !> the drop-in call with the surrogate: sed_ode_solver's host arrays
    integer(c_int) function sed_ode_solver_surrogate(h, s, conc, bdys, fluxes, dt, tol, &
        res_atol, st) bind(C, name='sed_ode_solver_surrogate')
      import :: c_int, c_ptr, c_double, sed_stats_t
      type(c_ptr), value :: h, s, conc, bdys, fluxes
      real(c_double), value :: dt, tol, res_atol
      type(sed_stats_t), intent(out) :: st
    end function
    !> training rows of one plain step into device arrays (c_ptr)
    integer(c_int) function sed_sur_collect(h, c0, dt, x_dev, y_dev, pitch_x, pitch_y, &
        capacity, count, st) bind(C, name='sed_sur_collect')
      import :: c_int, c_ptr, c_double, c_long_long, sed_stats_t
      type(c_ptr), value :: h, c0
      real(c_double), value :: dt
      type(c_ptr), value :: x_dev, y_dev
      integer(c_int), value :: pitch_x, pitch_y
      integer(c_long_long), value :: capacity
      integer(c_long_long), intent(inout) :: count
      type(sed_stats_t), intent(out) :: st
    end function
    subroutine sed_sur_destroy(s) bind(C, name='sed_sur_destroy')
      import :: c_ptr
      type(c_ptr), value :: s
    end subroutine
    !> C strings (const char*), read with sed_c_string
    type(c_ptr) function sed_error_string(code) bind(C, name='sed_error_string')
      import :: c_ptr, c_int
      integer(c_int), value :: code
    end function
    type(c_ptr) function sed_last_error(h) bind(C, name='sed_last_error')
      import :: c_ptr
      type(c_ptr), value :: h
    end function
    type(c_ptr) function sed_tracer_name(n) bind(C, name='sed_tracer_name')
      import :: c_ptr, c_int
      integer(c_int), value :: n
    end function
    integer(c_int) function sed_tracer_is_particulate(n) bind(C, name='sed_tracer_is_particulate')
      import :: c_int
      integer(c_int), value :: n
    end function
    function c_strlen(s) bind(C, name='strlen')
      import :: c_ptr, c_size_t
      type(c_ptr), value :: s
      integer(c_size_t) :: c_strlen
    end function
  end interface

  public :: sed_default_params, sed_gpu_init, sed_gpu_ode_solver, &
            sed_gpu_get_rhs, sed_gpu_finalize, sed_get_tuning, sed_set_tuning, &
            sed_autotune, sed_set_boundary, sed_get_boundary, sed_spinup, &
            sed_get_min_dt, sed_get_min_dt_grid_cell, sed_set_column_bgc, sed_set_state, sed_get_state, &
            sed_step, sed_get_fluxes, sed_get_attempts, sed_get_budgets, sed_set_stream, &
            sed_host_register, sed_host_unregister, sed_host_alloc, sed_host_free, &
            sed_get_attempt_histogram, &
            sed_ode_solver_noalloc, &
            sed_sur_create, sed_sur_num_params, sed_sur_set_weights, sed_sur_get_weights, &
            sed_sur_state_size, sed_sur_get_state, sed_sur_set_state, sed_sur_set_norm, &
            sed_sur_forward, sed_sur_forward_device, sed_sur_train_step, sed_sur_grads, &
            sed_sur_set_tensor_cores, sed_sur_set_stream, sed_sur_last_error, &
            sed_step_surrogate, sed_ode_solver_surrogate, sed_sur_collect, sed_sur_destroy, &
            sed_error_string, sed_last_error, sed_tracer_name, sed_tracer_is_particulate, &
            sed_c_string

contains

  !> Create a handle for the driver's grid (after type_sed%initialize):
  !! grid%dz, grid%dzc, porosity, intf_porosity, bioturbation_factor,
  !! flux_cap and mask (masked columns, or masked bottom layers only).  ntr
  !! is the driver's nvar, the tracer planes of its conc array
  !! (fabm_sediment_driver.F90:353); the library refuses any count but
  !! SED_NTR with SED_E_ARG, so it never reads past the caller's arrays.
  subroutine sed_gpu_init(gpu, p, inum, jnum, knum, ntr, dz, dzc, porosity, &
                          intf_porosity, bioturbation_factor, flux_cap, mask, rc)
    type(sed_gpu_t), intent(out) :: gpu
    type(sed_params_t), intent(in) :: p
    integer, intent(in) :: inum, jnum, knum, ntr
    real(c_double), dimension(:,:,:), intent(in), target, contiguous :: &
      dz, dzc, porosity, intf_porosity, bioturbation_factor, flux_cap
    integer(c_int), dimension(:,:,:), intent(in), target, contiguous :: mask
    integer, intent(out) :: rc
    rc = sed_create(p, int(inum, c_int), int(jnum, c_int), int(knum, c_int), &
                    int(ntr, c_int), gpu%h)
    if (rc /= SED_OK) return
    rc = sed_set_grid(gpu%h, c_loc(dz), c_loc(dzc), c_loc(porosity), &
                      c_loc(intf_porosity), c_loc(bioturbation_factor), &
                      c_loc(flux_cap), c_null_ptr, c_loc(mask))
  end subroutine

  !> Drop-in for `call ode_solver(sed, dt, ode_method)` plus the component
  !! epilogue: conc advanced in place, dissolved rows of fluxes set to the
  !! surface fluxes of the last right-hand side (get_rhs :692).
  subroutine sed_gpu_ode_solver(gpu, conc, bdys, fluxes, dt, method, rc, stats)
    type(sed_gpu_t), intent(in) :: gpu
    real(c_double), dimension(:,:,:,:), intent(inout), target, contiguous :: conc
    real(c_double), dimension(:,:,:), intent(in), target, contiguous :: bdys
    real(c_double), dimension(:,:,:), intent(inout), target, contiguous :: fluxes
    real(c_double), intent(in) :: dt
    integer, intent(in) :: method
    integer, intent(out) :: rc
    type(sed_stats_t), intent(out), optional :: stats
    type(sed_stats_t) :: st
    rc = sed_ode_solver(gpu%h, c_loc(conc), c_loc(bdys), c_loc(fluxes), dt, &
                        int(method, c_int), st)
    if (present(stats)) stats = st
  end subroutine

  !> Drop-in for type_sed%get_rhs (fabm_sediment_driver.F90:575-717).
  subroutine sed_gpu_get_rhs(gpu, conc, bdys, fluxes, rhs, rc)
    type(sed_gpu_t), intent(in) :: gpu
    real(c_double), dimension(:,:,:,:), intent(in), target, contiguous :: conc
    real(c_double), dimension(:,:,:), intent(in), target, contiguous :: bdys
    real(c_double), dimension(:,:,:), intent(inout), target, contiguous :: fluxes
    real(c_double), dimension(:,:,:,:), intent(out), target, contiguous :: rhs
    integer, intent(out) :: rc
    rc = sed_set_forcing(gpu%h, c_loc(bdys), c_loc(fluxes))
    if (rc /= SED_OK) return
    rc = sed_get_rhs(gpu%h, c_loc(conc), c_loc(rhs), c_loc(fluxes))
  end subroutine

  !> A C string of the library (sed_error_string, sed_last_error,
  !! sed_tracer_name, pel_last_error) as a Fortran string.
  function sed_c_string(p) result(str)
    type(c_ptr), intent(in) :: p
    character(len=:), allocatable :: str
    character(kind=c_char), pointer :: chars(:)
    integer :: i, n
    if (.not. c_associated(p)) then
      str = ''
      return
    end if
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: str)
    do i = 1, n
      str(i:i) = chars(i)
    end do
  end function

  subroutine sed_gpu_finalize(gpu)
    type(sed_gpu_t), intent(inout) :: gpu
    call sed_destroy(gpu%h)
    gpu%h = c_null_ptr
  end subroutine

end module sed_gpu
