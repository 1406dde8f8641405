/*
 * mossco_cpl.h -- C ABI of the pelagic -> soil coupling on the device.
 *
 * Replaces the Run of MOSSCO's pelagic_soil_connector
 * (src/mediators/pelagic_soil_connector.F90:176-2122) between a pelagic
 * handle (mossco_pel.h) and a sediment handle (mossco_sed.h) on the same
 * inum x jnum grid.  The pelagic state's bottom layer (k = 0, the
 * connector's lbnd(3)) becomes the sediment's "_at_soil_surface" fields,
 * and these become the sediment handle's bdys / fluxes exactly as
 * sed_set_boundary makes them (get_boundary_conditions,
 * src/components/fabm_sediment_component.F90:1865-2030).  Both stay on the
 * device: the call reads the pelagic handle's device state and writes the
 * sediment handle's device boundary, ordered after the pelagic handle's
 * stream by an event.  Every call returns SED_OK or a negative SED_E_* code.
 *
 * The ESMF field lookup by name (the connector's includeList searches)
 * becomes a table of pelagic tracer indices, cpl_fields.  The per-column
 * arithmetic is the connector's, in FP64, whatever the handles' precision.
 */
#ifndef MOSSCO_CPL_H
#define MOSSCO_CPL_H

#include "mossco_pel.h"
#include "mossco_sed.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Which export field each detritus formula ends up in.
 * CPL_AS_RUN: as the connector's Run writes them.  For labile and
 *   semilabile carbon and nitrogen it looks up the concentration and the
 *   z-velocity field together and writes the velocity formula into
 *   fieldList(1) again (:1287-1296 and the three blocks after it); with
 *   exact-name matching that is the concentration field in both ESMF item
 *   orders, so these concentrations carry sinking_factor*fac_env*detN and
 *   their velocities keep what the fields held (velocity_in, or 0 as the
 *   sediment component initialises them, fabm_sediment_component.F90:1180).
 *   Likewise the nitrate block (:1863-1935) looks the nitrate field up but
 *   writes through the ammonium field's pointer, so ammonium takes the
 *   nitrate value and the nitrate field is not written: its row keeps the
 *   sediment handle's previous boundary (present_out[7] = 0).
 * CPL_AS_NAMED: each formula into the field its comment names: the C:N
 *   split into the concentrations, sinking_factor*fac_env*detN into the
 *   z-velocities, ammonium and nitrate into their own fields. */
#define CPL_AS_RUN 0
#define CPL_AS_NAMED 1

/* &pelagic_soil_connector (pelagic_soil_connector.F90:38-45,146-148) */
typedef struct cpl_params {
  double sinking_factor;           /* 0.3 */
  double sinking_factor_min;       /* 0.02 (a default-real literal: 0.0199999995529651) */
  double NC_ldet, NC_sdet;         /* 0.23, 0.01 */
  double convertN, convertP;       /* 1, 1 */
  double half_sedimentation_depth; /* m, 0.1 (default-real literal) */
  double half_sedimentation_tke;   /* m2/s2, 1000 */
  double critical_detritus;        /* mmolC/m3, 60 */
  int mode;                        /* CPL_AS_RUN (default) or CPL_AS_NAMED */
} cpl_params;

/* Pelagic tracer index (0 .. PEL_NTR-1) of each field the connector looks
 * up, or -1 when the pelagic model has no such field. */
typedef struct cpl_fields {
  int detN;     /* detritus_in_water, detN_in_water, ... (:923-930) */
  int detC;     /* Detritus_Carbon_detC_in_water (:1027-1028) */
  int detP;     /* detP_in_water (:1530-1531) */
  int din;      /* nutrients_in_water, DIN_in_water, ... */
  int nitrate;  /* nitrate_in_water */
  int ammonium; /* ammonium_in_water, dissolved_ammonium_nh3_in_water */
  int oxygen;   /* dissolved_oxygen_in_water, ... (:652-656) */
  int odu;      /* dissolved_reduced_substances_odu_in_water (:697-698) */
  int dip;      /* DIP_in_water, phosphate_in_water, ...: written by the
                   reverse connector only (the forward Run overwrites it and
                   never reads it, :2080-2094) */
} cpl_fields;

/* what one cpl_pelagic_soil call did on the device */
typedef struct cpl_stats {
  int gpu_launches;      /* kernels this library launched for the call */
  long long columns;     /* columns mapped */
  double kernel_ms;      /* k_pelagic_soil alone (CUDA events) */
  double device_ms;      /* the call's device span: copies, mapping and the
                            sediment's boundary assembly (CUDA events) */
} cpl_stats;

int cpl_default_params(cpl_params *p);
/* gotm_npzd's fields: detN = detritus (3), din = nutrients (0), others -1
 * (its bottom fluxes: nutrients_ and detritus_upward_flux_at_soil_surface) */
int cpl_npzd_fields(cpl_fields *f);

/* &soil_pelagic_connector (src/mediators/soil_pelagic_connector.F90:36-41,
 * 140); NC_ldet and NC_sdet are read by the namelist and unused by the Run */
typedef struct cpl_soil_params {
  double dinflux_const;  /* mmol/m2/yr added to the DIN flux, 0 */
  double dipflux_const;  /* mmol/m2/yr added to the phosphate flux, -1 */
  double NC_ldet, NC_sdet; /* 0.2, 0.04 */
  double convertN, convertP; /* 1, 1 */
} cpl_soil_params;

int cpl_soil_default_params(cpl_soil_params *p);

/* One connector Run followed by the sediment's boundary assembly.
 *   temperature  [ncol] temperature_at_soil_surface (required; the pelagic
 *                handle carries no temperature)
 *   water_depth  [ncol] water_depth_at_soil_surface, or NULL (absent)
 *   tke          [ncol] the first of turbulent_diffusivity_of_momentum_ and
 *                turbulent_kinetic_energy_at_soil_surface that the
 *                connector's lookup returns (:1164-1195), or NULL
 *   velocity_in  [SED_NTR][ncol] the z-velocity fields' contents before the
 *                call, or NULL (zeros); only particulate rows are read
 *   surface_out, velocity_out  [SED_NTR][ncol] the export fields after the
 *                call (host copies for inspection), or NULL; surface rows
 *                the Run does not write read 0, velocity rows velocity_in's
 *                (non-particulate rows 0)
 *   present_out  [SED_NTR] 1 where the connector wrote the tracer's
 *                concentration field, or NULL
 *   stats        or NULL
 * The pelagic handle needs its state (pel_set_state or a step), the
 * sediment handle its grid, and with bcup_dissolved = 1 its state.  No
 * nitrate, ammonium or DIN field: SED_E_ARG (the Run returns
 * ESMF_RC_NOT_FOUND, :1806,1855).  Both handles on one device. */
int cpl_pelagic_soil(pel_handle *pel, sed_handle *sed, const cpl_params *p,
                     const cpl_fields *f, const double *temperature,
                     const double *water_depth, const double *tke,
                     const double *velocity_in, double *surface_out,
                     double *velocity_out, int *present_out, cpl_stats *stats);

/* The reverse direction: one Run of soil_pelagic_connector
 * (src/mediators/soil_pelagic_connector.F90:179-965).  The sediment
 * component exports every tracer's upward flux at the soil surface as
 * -fluxes(:,:,n) (fabm_sediment_component.F90:1808-1815); the connector maps
 * them to the pelagic fields' <name>_upward_flux_at_soil_surface, which the
 * pelagic Run applies to its bottom layer (bfl, fabm_pelagic_component.F90
 * :2093-2105).  This call reads the sediment handle's device fluxes after its
 * last step and writes the pelagic handle's bottom-flux rows (as
 * pel_set_forcing's bottom_flux) on the device; rows of fields the connector
 * does not write keep their values (zeros if the handle had none).
 *   bottom_flux_out  [PEL_NTR][ncol] the pelagic bottom fluxes after the
 *                    call (host copy), or NULL
 *   present_out      [PEL_NTR] 1 where the connector wrote the row, or NULL
 * The sediment handle needs its forcing (a step's fluxes), the pelagic
 * handle its grid. */
int cpl_soil_pelagic(sed_handle *sed, pel_handle *pel, const cpl_soil_params *p,
                     const cpl_fields *f, double *bottom_flux_out, int *present_out,
                     cpl_stats *stats);

#ifdef __cplusplus
}
#endif

#endif
