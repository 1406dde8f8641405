!> @file type_sed_gpu.F90
!! @brief The sediment driver type with its step on the GPU.
!!
!! type_sed_gpu extends the reference's type_sed
!! (src/drivers/fabm_sediment_driver.F90:69-113) by a handle of the GB300
!! library (include/mossco_sed.h, bound in sed_gpu.F90).  gpu_init builds
!! the device grid from the driver's own arrays after type_sed%initialize
!! and init_concentrations; gpu_ode_solver replaces
!! `call ode_solver(sed, dt, method)` (src/utilities/solver_library.F90:80)
!! plus the component's NaN check and clamp
!! (src/components/fabm_sediment_component.F90:1715-1732) on sed%conc,
!! sed%bdys and sed%fluxes in place.  Compiled with the reference's modules
!! (fabm_sediment_driver, fabm) on the module path.
module sediment_driver_gpu

  use iso_c_binding
  use fabm_sediment_driver, only: type_sed
  use sed_gpu
  implicit none
  private

  type, extends(type_sed), public :: type_sed_gpu
    type(sed_gpu_t) :: gpu
    logical :: gpu_ready = .false.
  contains
    procedure :: gpu_init
    procedure :: gpu_ode_solver
    procedure :: gpu_finalize
  end type

contains

  !> The device grid and parameters from the driver's state.  precision is
  !! SED_FP64 (bit-identical to the CPU path's arithmetic) or SED_FP32.
  subroutine gpu_init(self, precision, cut_scope, rc)
    class(type_sed_gpu), intent(inout) :: self
    integer, intent(in) :: precision, cut_scope
    integer, intent(out) :: rc
    type(sed_params_t) :: p
    integer(c_int), allocatable, target :: mask(:,:,:)
    integer :: n
    rc = sed_default_params(p)
    if (rc /= SED_OK) return
    p%diffusivity = self%diffusivity
    p%bioturbation = self%bioturbation
    p%bcup_dissolved = self%bcup_dissolved_variables
    p%bcup_particulate = self%bcup_particulate_variables
    p%dt_min = self%dt_min
    p%relative_change_min = self%relative_change_min
    p%precision = precision
    p%cut_scope = cut_scope
    p%bioturbation_profile = self%bioturbation_profile
    p%bioturb_k_l = self%k_l
    p%bioturb_L1 = self%L1
    p%bioturb_L2 = self%L2
    p%bioturb_beta = self%beta
    p%bioturb_b = self%b
    do n = 1, self%nvar
      p%minimum(n) = self%model%state_variables(n)%minimum
    end do
    allocate(mask(self%inum, self%jnum, self%knum))
    mask = merge(1_c_int, 0_c_int, self%mask)
    call sed_gpu_init(self%gpu, p, self%inum, self%jnum, self%knum, self%grid%dz, &
                      self%grid%dzc, self%porosity, self%intf_porosity, &
                      self%bioturbation_factor, self%flux_cap, mask, rc)
    self%gpu_ready = rc == SED_OK
  end subroutine

  !> `call ode_solver(self, dt, method)` and the component's epilogue on the
  !! GPU: self%conc advanced in place, the dissolved rows of self%fluxes set
  !! to the surface fluxes as get_rhs sets them (:692).
  subroutine gpu_ode_solver(self, dt, method, rc)
    class(type_sed_gpu), intent(inout) :: self
    real(c_double), intent(in) :: dt
    integer, intent(in) :: method
    integer, intent(out) :: rc
    if (.not. self%gpu_ready) then
      rc = SED_E_STATE
      return
    end if
    call sed_gpu_ode_solver(self%gpu, self%conc, self%bdys, self%fluxes, dt, method, rc)
  end subroutine

  subroutine gpu_finalize(self)
    class(type_sed_gpu), intent(inout) :: self
    if (self%gpu_ready) call sed_gpu_finalize(self%gpu)
    self%gpu_ready = .false.
  end subroutine

end module sediment_driver_gpu
