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
!!
!! Tracers.  The driver's state has nvar = size(model%state_variables)
!! tracers in FABM's order (fabm_sediment_driver.F90:353), linked by name
!! (:457,609).  The library holds the eleven OMEXDIA+P tracers of
!! sed_tracer_name() in its own order, so gpu_init matches FABM's state
!! variable names against them (the part of the name after the model
!! instance: ldetC, sdetC, ldetN, sdetN, ldetP or detP, adsP, oxy, no3, nh3,
!! odu, po4, the names of the reference's hzg_omexdia_cnp and hzg_omexdia_p
!! namelists, examples/standalone/omexdia_p/fabm_sed.nml:18-77).  A model
!! with another tracer count, or without one of the eleven, is refused with
!! SED_E_ARG before anything is allocated: the reference's hzg_omexdia_p
!! (8 states) and hzg_omexdia_cnp (10, no adsorbed P) are refused.  When the
!! order differs, gpu_ode_solver gathers the state into the library's order
!! and scatters it back.
!!
!! Rate constants.  FABM reads the model's parameters from its namelist
!! (fabm_sed.nml, &hzg_omexdia_cnp or &hzg_omexdia_p, :18-77); gpu_init reads
!! the same group from the same file, so the device rates use the user's
!! values.
module sediment_driver_gpu

  use iso_c_binding
  use fabm_sediment_driver, only: type_sed
  use sed_gpu
  implicit none
  private

  !> FABM state-variable name endings of the library's tracers, in
  !! sed_tracer_name() order (two spellings of labile detritus P)
  character(len=5), parameter :: tracer_keys(SED_NTR) = [character(len=5) :: &
    'ldetC', 'sdetC', 'ldetN', 'sdetN', 'ldetP', 'adsP', 'oxy', 'no3', 'nh3', 'odu', 'po4']
  character(len=5), parameter :: tracer_alias(SED_NTR) = [character(len=5) :: &
    '', '', '', '', 'detP', '', '', '', '', '', '']

  type, extends(type_sed), public :: type_sed_gpu
    type(sed_gpu_t) :: gpu
    logical :: gpu_ready = .false.
    !> perm(n): FABM state index of the library's tracer n
    integer :: perm(SED_NTR) = 0
    logical :: identity = .true.
    !> the state, boundary and flux arrays in the library's tracer order
    !! (used when the orders differ)
    real(c_double), allocatable :: lconc(:,:,:,:), lbdys(:,:,:), lfluxes(:,:,:)
    character(len=256) :: gpu_message = ''
  contains
    procedure :: gpu_init
    procedure :: gpu_ode_solver
    procedure :: gpu_finalize
  end type

contains

  !> lower-case copy of a string
  pure function lower(s) result(t)
    character(len=*), intent(in) :: s
    character(len=len(s)) :: t
    integer :: i, c
    t = s
    do i = 1, len(s)
      c = iachar(s(i:i))
      if (c >= iachar('A') .and. c <= iachar('Z')) t(i:i) = achar(c + 32)
    end do
  end function

  !> does name end with '_' // key (case-insensitive)?
  pure logical function ends_with_key(name, key)
    character(len=*), intent(in) :: name, key
    character(len=:), allocatable :: n, k
    n = lower(trim(name))
    k = '_' // lower(trim(key))
    ends_with_key = len_trim(key) > 0 .and. len(n) >= len(k)
    if (ends_with_key) ends_with_key = n(len(n) - len(k) + 1:) == k
  end function

  !> The library's tracer order from FABM's state names; rc = SED_E_ARG
  !! with self%gpu_message naming the problem.
  subroutine gpu_tracer_map(self, rc)
    class(type_sed_gpu), intent(inout) :: self
    integer, intent(out) :: rc
    integer :: n, m
    rc = SED_OK
    if (self%nvar /= SED_NTR) then
      write(self%gpu_message, '(A,I0,A,I0,A)') 'the FABM model has ', self%nvar, &
        ' state variables; the GPU library holds the ', SED_NTR, ' OMEXDIA+P tracers'
      rc = SED_E_ARG
      return
    end if
    self%perm = 0
    do n = 1, SED_NTR
      do m = 1, self%nvar
        if (ends_with_key(self%model%state_variables(m)%name, tracer_keys(n)) .or. &
            ends_with_key(self%model%state_variables(m)%name, tracer_alias(n))) then
          self%perm(n) = m
          exit
        end if
      end do
      if (self%perm(n) == 0) then
        write(self%gpu_message, '(A,A,A)') 'no FABM state variable for the tracer ', &
          trim(sed_c_string(sed_tracer_name(int(n - 1, c_int)))), &
          ' (name ending _' // trim(tracer_keys(n)) // ')'
        rc = SED_E_ARG
        return
      end if
    end do
    self%identity = all(self%perm == [(n, n = 1, SED_NTR)])
  end subroutine

  !> The OMEXDIA+P rate constants of the FABM namelist file (the group
  !! &hzg_omexdia_cnp, else &hzg_omexdia_p), per day as the file gives them.
  subroutine gpu_read_bgc(p, nmlfile, rc)
    type(sed_params_t), intent(inout) :: p
    character(len=*), intent(in) :: nmlfile
    integer, intent(out) :: rc
    real(c_double) :: rLabile, rSemilabile, NCrLdet, NCrSdet, PAds, PAdsODU, NH3Ads, &
                      CprodMax, rnit, ksO2nitri, rODUox, ksO2oduox, ksO2oxic, ksNO3denit, &
                      kinO2denit, kinNO3anox, kinO2anox
    real(c_double) :: ldetC_init, sdetC_init, ldetN_init, sdetN_init, ldetP_init, &
                      detP_init, no3_init, nh3_init, po4_init, oxy_init, odu_init
    namelist /hzg_omexdia_cnp/ rLabile, rSemilabile, NCrLdet, NCrSdet, PAds, PAdsODU, &
      NH3Ads, CprodMax, rnit, ksO2nitri, rODUox, ksO2oduox, ksO2oxic, ksNO3denit, &
      kinO2denit, kinNO3anox, kinO2anox, ldetC_init, sdetC_init, ldetN_init, sdetN_init, &
      ldetP_init, no3_init, nh3_init, po4_init, oxy_init, odu_init
    namelist /hzg_omexdia_p/ rLabile, rSemilabile, NCrLdet, NCrSdet, PAds, PAdsODU, &
      NH3Ads, CprodMax, rnit, ksO2nitri, rODUox, ksO2oduox, ksO2oxic, ksNO3denit, &
      kinO2denit, kinNO3anox, kinO2anox, ldetC_init, sdetC_init, oxy_init, odu_init, &
      no3_init, nh3_init, detP_init, po4_init
    integer :: unit, ios
    ! the library's defaults stand for entries the group leaves out
    rLabile = p%rLabile; rSemilabile = p%rSemilabile; NCrLdet = p%NCrLdet
    NCrSdet = p%NCrSdet; PAds = p%PAds; PAdsODU = p%PAdsODU; NH3Ads = p%NH3Ads
    CprodMax = p%CprodMax; rnit = p%rnit; ksO2nitri = p%ksO2nitri; rODUox = p%rODUox
    ksO2oduox = p%ksO2oduox; ksO2oxic = p%ksO2oxic; ksNO3denit = p%ksNO3denit
    kinO2denit = p%kinO2denit; kinNO3anox = p%kinNO3anox; kinO2anox = p%kinO2anox
    open(newunit=unit, file=nmlfile, status='old', action='read', iostat=ios)
    if (ios /= 0) then
      rc = SED_E_ARG
      return
    end if
    read(unit, nml=hzg_omexdia_cnp, iostat=ios)
    if (ios /= 0) then
      rewind(unit)
      read(unit, nml=hzg_omexdia_p, iostat=ios)
    end if
    close(unit)
    if (ios /= 0) then
      rc = SED_E_ARG
      return
    end if
    p%rLabile = rLabile; p%rSemilabile = rSemilabile; p%NCrLdet = NCrLdet
    p%NCrSdet = NCrSdet; p%PAds = PAds; p%PAdsODU = PAdsODU; p%NH3Ads = NH3Ads
    p%CprodMax = CprodMax; p%rnit = rnit; p%ksO2nitri = ksO2nitri; p%rODUox = rODUox
    p%ksO2oduox = ksO2oduox; p%ksO2oxic = ksO2oxic; p%ksNO3denit = ksNO3denit
    p%kinO2denit = kinO2denit; p%kinNO3anox = kinNO3anox; p%kinO2anox = kinO2anox
    rc = SED_OK
  end subroutine

  !> The device grid and parameters from the driver's state.  precision is
  !! SED_FP64 (bit-identical to the CPU path's arithmetic) or SED_FP32;
  !! nmlfile is FABM's namelist file (the reference's default fabm_sed.nml).
  subroutine gpu_init(self, precision, cut_scope, rc, nmlfile)
    class(type_sed_gpu), intent(inout) :: self
    integer, intent(in) :: precision, cut_scope
    integer, intent(out) :: rc
    character(len=*), intent(in), optional :: nmlfile
    type(sed_params_t) :: p
    integer(c_int), allocatable, target :: mask(:,:,:)
    integer :: n
    call gpu_tracer_map(self, rc)
    if (rc /= SED_OK) return
    rc = sed_default_params(p)
    if (rc /= SED_OK) return
    if (present(nmlfile)) then
      call gpu_read_bgc(p, nmlfile, rc)
    else
      call gpu_read_bgc(p, 'fabm_sed.nml', rc)
    end if
    if (rc /= SED_OK) then
      self%gpu_message = 'no &hzg_omexdia_cnp or &hzg_omexdia_p group in the FABM namelist'
      return
    end if
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
    do n = 1, SED_NTR
      p%minimum(n) = self%model%state_variables(self%perm(n))%minimum
    end do
    if (.not. self%identity) then
      allocate(self%lconc(self%inum, self%jnum, self%knum, SED_NTR))
      allocate(self%lbdys(self%inum, self%jnum, SED_NTR + 1))
      allocate(self%lfluxes(self%inum, self%jnum, SED_NTR))
    end if
    allocate(mask(self%inum, self%jnum, self%knum))
    mask = merge(1_c_int, 0_c_int, self%mask)
    call sed_gpu_init(self%gpu, p, self%inum, self%jnum, self%knum, self%nvar, self%grid%dz, &
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
    integer :: n
    if (.not. self%gpu_ready) then
      rc = SED_E_STATE
      return
    end if
    if (self%identity) then
      call sed_gpu_ode_solver(self%gpu, self%conc, self%bdys, self%fluxes, dt, method, rc)
      return
    end if
    ! FABM's order -> the library's
    self%lbdys(:,:,1) = self%bdys(:,:,1)
    do n = 1, SED_NTR
      self%lconc(:,:,:,n) = self%conc(:,:,:,self%perm(n))
      self%lbdys(:,:,n + 1) = self%bdys(:,:,self%perm(n) + 1)
      self%lfluxes(:,:,n) = self%fluxes(:,:,self%perm(n))
    end do
    call sed_gpu_ode_solver(self%gpu, self%lconc, self%lbdys, self%lfluxes, dt, method, rc)
    if (rc /= SED_OK) return
    do n = 1, SED_NTR
      self%conc(:,:,:,self%perm(n)) = self%lconc(:,:,:,n)
      self%fluxes(:,:,self%perm(n)) = self%lfluxes(:,:,n)
    end do
  end subroutine

  subroutine gpu_finalize(self)
    class(type_sed_gpu), intent(inout) :: self
    if (self%gpu_ready) call sed_gpu_finalize(self%gpu)
    self%gpu_ready = .false.
    if (allocated(self%lconc)) deallocate(self%lconc, self%lbdys, self%lfluxes)
  end subroutine

end module sediment_driver_gpu
