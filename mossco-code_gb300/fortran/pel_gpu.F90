!> @file pel_gpu.F90
!! @brief ISO_C_BINDING interface to the GB300 pelagic-driver solver.
!!
!! Binds the C ABI of include/mossco_pel.h for MOSSCO's Fortran host.  The
!! component's Run loop (src/components/fabm_pelagic_component.F90:1931,
!! 2061-2240: light, then per internal step ode_solver, the soil-surface
!! fluxes, the external flux fields and clip_below_minimum) becomes
!! `call pel_gpu_run(gpu, pel%conc, t_couple, dt, ode_method, rc)`; the
!! driver's `call ode_solver(pel, dt, method)` becomes pel_gpu_ode_solver.
!! Arrays keep their Fortran layout: conc(i,j,k,n) is the C ABI's
!! [ntr][knum][ncol] with col = i + inum*(j-1), k = 1 the bottom layer.
module pel_gpu

  use iso_c_binding
  implicit none
  private

  integer, parameter, public :: PEL_NTR = 4
  integer, parameter, public :: PEL_CUT_PER_CELL = 0, PEL_CUT_GLOBAL = 1

  !> pel_params of mossco_pel.h (same member order and kinds)
  type, bind(C), public :: pel_params_t
    real(c_double) :: p0, z0, kc, I_min, rmax, gmax, Iv, alpha, &
                      rpn, rzn, rdn, rpdu, rpdl, rzd
    real(c_double) :: dt_min, relative_change_min, background_extinction, atol
    integer(c_int) :: max_attempts, cut_scope
    real(c_double) :: minimum(PEL_NTR)
    integer(c_int) :: precision, device
  end type

  type, bind(C), public :: pel_stats_t
    integer(c_long_long) :: attempts, accepted, column_steps
    integer(c_int)       :: max_cell_attempts, capped_cells, nan_cells, gpu_launches
    real(c_double)       :: min_dt, device_ms
  end type

  type, public :: pel_gpu_t
    type(c_ptr) :: h = c_null_ptr
  end type

  interface
    !> the handle's last error message (a C string: read it with sed_c_string)
    type(c_ptr) function pel_last_error(h) bind(C, name='pel_last_error')
      import :: c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function pel_default_params(p) bind(C, name='pel_default_params')
      import :: c_int, pel_params_t
      type(pel_params_t), intent(out) :: p
    end function
    integer(c_int) function pel_create(p, inum, jnum, knum, ntr, h) bind(C, name='pel_create')
      import :: c_int, c_ptr, pel_params_t
      type(pel_params_t), intent(in) :: p
      integer(c_int), value :: inum, jnum, knum, ntr
      type(c_ptr), intent(out) :: h
    end function
    subroutine pel_destroy(h) bind(C, name='pel_destroy')
      import :: c_ptr
      type(c_ptr), value :: h
    end subroutine
    integer(c_int) function pel_set_grid(h, layer_height, mask) bind(C, name='pel_set_grid')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, layer_height, mask
    end function
    integer(c_int) function pel_set_forcing(h, I_0, albedo, bottom_flux, surface_flux, &
                                            soil_flux) bind(C, name='pel_set_forcing')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, I_0, albedo, bottom_flux, surface_flux, soil_flux
    end function
    integer(c_int) function pel_set_open_boundary(h, open_boundary, boundary_value, &
                                                  has_value) bind(C, name='pel_set_open_boundary')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, open_boundary, boundary_value, has_value
    end function
    integer(c_int) function pel_set_state(h, conc) bind(C, name='pel_set_state')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, conc
    end function
    integer(c_int) function pel_get_state(h, conc) bind(C, name='pel_get_state')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, conc
    end function
    integer(c_int) function pel_light(h, conc, par) bind(C, name='pel_light')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, conc, par
    end function
    integer(c_int) function pel_get_rhs(h, conc, rhs) bind(C, name='pel_get_rhs')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, conc, rhs
    end function
    integer(c_int) function pel_ode_solver(h, conc, dt, method, st) bind(C, name='pel_ode_solver')
      import :: c_int, c_ptr, c_double, pel_stats_t
      type(c_ptr), value :: h, conc
      real(c_double), value :: dt
      integer(c_int), value :: method
      type(pel_stats_t), intent(out) :: st
    end function
    integer(c_int) function pel_run(h, conc, t_couple, dt, method, st) bind(C, name='pel_run')
      import :: c_int, c_ptr, c_double, pel_stats_t
      type(c_ptr), value :: h, conc
      real(c_double), value :: t_couple, dt
      integer(c_int), value :: method
      type(pel_stats_t), intent(out) :: st
    end function
    integer(c_int) function pel_step(h, t_couple, dt, method, nruns, st) bind(C, name='pel_step')
      import :: c_int, c_ptr, c_double, pel_stats_t
      type(c_ptr), value :: h
      real(c_double), value :: t_couple, dt
      integer(c_int), value :: method, nruns
      type(pel_stats_t), intent(out) :: st
    end function
  end interface

  public :: pel_default_params, pel_create, pel_destroy, pel_set_grid, pel_set_forcing, &
            pel_set_open_boundary, pel_set_state, pel_get_state, pel_light, pel_get_rhs, pel_ode_solver, &
            pel_run, pel_step, pel_last_error
  public :: pel_gpu_init, pel_gpu_forcing, pel_gpu_run, pel_gpu_ode_solver, pel_gpu_finalize

contains

  !> initialize_domain + update_grid (fabm_pelagic_driver.F90:215-293,362-378)
  subroutine pel_gpu_init(gpu, p, inum, jnum, knum, layer_height, mask, rc)
    type(pel_gpu_t), intent(out) :: gpu
    type(pel_params_t), intent(in) :: p
    integer, intent(in) :: inum, jnum, knum
    real(c_double), dimension(:,:,:), intent(in), target, contiguous :: layer_height
    integer(c_int), dimension(:,:,:), intent(in), target, contiguous :: mask
    integer, intent(out) :: rc
    rc = pel_create(p, int(inum, c_int), int(jnum, c_int), int(knum, c_int), &
                    int(PEL_NTR, c_int), gpu%h)
    if (rc /= 0) return
    rc = pel_set_grid(gpu%h, c_loc(layer_height), c_loc(mask))
  end subroutine

  !> I_0, albedo and the bfl(n)%p soil-surface upward fluxes of the Run
  subroutine pel_gpu_forcing(gpu, I_0, albedo, bottom_flux, rc)
    type(pel_gpu_t), intent(in) :: gpu
    real(c_double), dimension(:,:), intent(in), target, contiguous :: I_0, albedo
    real(c_double), dimension(:,:,:), intent(in), target, contiguous :: bottom_flux
    integer, intent(out) :: rc
    rc = pel_set_forcing(gpu%h, c_loc(I_0), c_loc(albedo), c_loc(bottom_flux), &
                         c_null_ptr, c_null_ptr)
  end subroutine

  !> The component's Run over one coupling interval on pel%conc, in place.
  subroutine pel_gpu_run(gpu, conc, t_couple, dt, method, rc, stats)
    type(pel_gpu_t), intent(in) :: gpu
    real(c_double), dimension(:,:,:,:), intent(inout), target, contiguous :: conc
    real(c_double), intent(in) :: t_couple, dt
    integer, intent(in) :: method
    integer, intent(out) :: rc
    type(pel_stats_t), intent(out), optional :: stats
    type(pel_stats_t) :: st
    rc = pel_run(gpu%h, c_loc(conc), real(t_couple, c_double), real(dt, c_double), &
                 int(method, c_int), st)
    if (present(stats)) stats = st
  end subroutine

  !> Drop-in for `call ode_solver(pel, dt, method)` with the PAR of the last
  !! pel_light call.
  subroutine pel_gpu_ode_solver(gpu, conc, dt, method, rc)
    type(pel_gpu_t), intent(in) :: gpu
    real(c_double), dimension(:,:,:,:), intent(inout), target, contiguous :: conc
    real(c_double), intent(in) :: dt
    integer, intent(in) :: method
    integer, intent(out) :: rc
    type(pel_stats_t) :: st
    rc = pel_ode_solver(gpu%h, c_loc(conc), real(dt, c_double), int(method, c_int), st)
  end subroutine

  subroutine pel_gpu_finalize(gpu)
    type(pel_gpu_t), intent(inout) :: gpu
    call pel_destroy(gpu%h)
    gpu%h = c_null_ptr
  end subroutine

end module pel_gpu
