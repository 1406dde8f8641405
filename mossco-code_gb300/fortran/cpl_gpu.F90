!> @file cpl_gpu.F90
!! @brief ISO_C_BINDING interface to the GB300 pelagic -> soil coupling.
!!
!! Binds include/mossco_cpl.h.  In a coupled MOSSCO set-up the
!! pelagic_soil_connector's Run (src/mediators/pelagic_soil_connector.F90
!! :176-2122) and the sediment component's get_boundary_conditions
!! (src/components/fabm_sediment_component.F90:1865-2030) become one call,
!! `call cpl_gpu_pelagic_soil(pgpu, sgpu, p, f, temperature, rc)`, from the
!! pelagic handle's device state into the sediment handle's boundary; the
!! soil_pelagic_connector's Run (src/mediators/soil_pelagic_connector.F90
!! :179-965) becomes `rc = cpl_soil_pelagic(sgpu%h, pgpu%h, sp, f, c_null_ptr,
!! c_null_ptr, c_null_ptr)`, from the soil's fluxes into the pelagic handle's
!! bottom fluxes.  The
!! 2-D fields keep their Fortran layout: temperature(i,j) is the C ABI's
!! [ncol] with col = i + inum*(j-1).
module cpl_gpu

  use iso_c_binding
  use sed_gpu, only: sed_gpu_t
  use pel_gpu, only: pel_gpu_t
  implicit none
  private

  integer, parameter, public :: CPL_AS_RUN = 0, CPL_AS_NAMED = 1

  !> cpl_params of mossco_cpl.h: the &pelagic_soil_connector namelist
  type, bind(C), public :: cpl_params_t
    real(c_double) :: sinking_factor, sinking_factor_min, NC_ldet, NC_sdet, &
                      convertN, convertP, half_sedimentation_depth, &
                      half_sedimentation_tke, critical_detritus
    integer(c_int) :: mode
  end type

  !> cpl_fields of mossco_cpl.h: 0-based pelagic tracer index, or -1
  type, bind(C), public :: cpl_fields_t
    integer(c_int) :: detN, detC, detP, din, nitrate, ammonium, oxygen, odu, dip
  end type

  !> cpl_soil_params of mossco_cpl.h: the &soil_pelagic_connector namelist
  type, bind(C), public :: cpl_soil_params_t
    real(c_double) :: dinflux_const, dipflux_const, NC_ldet, NC_sdet, convertN, convertP
  end type

  !> cpl_stats of mossco_cpl.h
  type, bind(C), public :: cpl_stats_t
    integer(c_int)       :: gpu_launches
    integer(c_long_long) :: columns
    real(c_double)       :: kernel_ms, device_ms
  end type

  interface
    integer(c_int) function cpl_default_params(p) bind(C, name='cpl_default_params')
      import :: c_int, cpl_params_t
      type(cpl_params_t), intent(out) :: p
    end function
    integer(c_int) function cpl_npzd_fields(f) bind(C, name='cpl_npzd_fields')
      import :: c_int, cpl_fields_t
      type(cpl_fields_t), intent(out) :: f
    end function
    integer(c_int) function cpl_pelagic_soil(pel, sed, p, f, temperature, water_depth, &
        tke, velocity_in, surface_out, velocity_out, present_out, stats) &
        bind(C, name='cpl_pelagic_soil')
      import :: c_int, c_ptr, cpl_params_t, cpl_fields_t
      type(c_ptr), value :: pel, sed
      type(cpl_params_t), intent(in) :: p
      type(cpl_fields_t), intent(in) :: f
      type(c_ptr), value :: temperature, water_depth, tke, velocity_in, &
                            surface_out, velocity_out, present_out, stats
    end function
    integer(c_int) function cpl_soil_default_params(p) bind(C, name='cpl_soil_default_params')
      import :: c_int, cpl_soil_params_t
      type(cpl_soil_params_t), intent(out) :: p
    end function
    !> soil_pelagic_connector's Run: the soil handle's fluxes after its step
    !! into the pelagic handle's bottom fluxes, on the device
    integer(c_int) function cpl_soil_pelagic(sed, pel, p, f, bottom_flux_out, present_out, &
        stats) bind(C, name='cpl_soil_pelagic')
      import :: c_int, c_ptr, cpl_soil_params_t, cpl_fields_t
      type(c_ptr), value :: sed, pel
      type(cpl_soil_params_t), intent(in) :: p
      type(cpl_fields_t), intent(in) :: f
      type(c_ptr), value :: bottom_flux_out, present_out, stats
    end function
  end interface

  public :: cpl_default_params, cpl_npzd_fields, cpl_pelagic_soil, cpl_gpu_pelagic_soil, &
            cpl_soil_default_params, cpl_soil_pelagic

contains

  !> One connector Run and boundary assembly on the device.  water_depth and
  !! tke (water_depth_ and turbulent_kinetic_energy_at_soil_surface) are
  !! optional, as the connector finds them or not in its export state.
  subroutine cpl_gpu_pelagic_soil(pgpu, sgpu, p, f, temperature, rc, water_depth, tke)
    type(pel_gpu_t), intent(in) :: pgpu
    type(sed_gpu_t), intent(in) :: sgpu
    type(cpl_params_t), intent(in) :: p
    type(cpl_fields_t), intent(in) :: f
    real(c_double), dimension(:,:), intent(in), target, contiguous :: temperature
    integer, intent(out) :: rc
    real(c_double), dimension(:,:), intent(in), target, contiguous, optional :: &
      water_depth, tke
    type(c_ptr) :: d, t
    d = c_null_ptr
    t = c_null_ptr
    if (present(water_depth)) d = c_loc(water_depth)
    if (present(tke)) t = c_loc(tke)
    rc = cpl_pelagic_soil(pgpu%h, sgpu%h, p, f, c_loc(temperature), d, t, c_null_ptr, &
                          c_null_ptr, c_null_ptr, c_null_ptr, c_null_ptr)
  end subroutine

end module cpl_gpu
