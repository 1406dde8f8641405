/*
 * cpl_oracle.h -- FP64 CPU oracle of MOSSCO's pelagic_soil_connector Run.
 *
 * TEST INFRASTRUCTURE ONLY (see cpl_oracle.c).
 */
#ifndef CPL_ORACLE_H
#define CPL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* &pelagic_soil_connector (pelagic_soil_connector.F90:38-45,146-148) */
typedef struct {
  double sinking_factor, sinking_factor_min, NC_ldet, NC_sdet, convertN, convertP,
      half_sedimentation_depth, half_sedimentation_tke, critical_detritus;
  int as_named; /* 0: fields as the Run writes them; 1: as the comments name them */
} orc_cpl;

/* pelagic tracer index of each field, -1 = absent */
typedef struct {
  int detN, detC, detP, din, nitrate, ammonium, oxygen, odu;
} orc_cpl_fields;

/* The connector's defaults, with its default-real literals */
void orc_cpl_defaults(orc_cpl *p);

/* conc [ntr][knum][ncol] pelagic state (k = 0 bottom); depth, tke [ncol] or
 * NULL.  surface [11][ncol] and velocity [11][ncol] hold the soil fields'
 * contents before the Run and are updated as the Run writes them; present
 * [11] is set to 1 for every concentration field the Run writes.  Returns 0,
 * or -1 when no nitrate, ammonium or DIN field exists (ESMF_RC_NOT_FOUND). */
int orc_cpl_run(const orc_cpl *p, const orc_cpl_fields *f, const double *conc,
                int ncol, int knum, const double *depth, const double *tke,
                double *surface, double *velocity, int *present);

/* &soil_pelagic_connector (soil_pelagic_connector.F90:36-41) */
typedef struct {
  double dinflux_const, dipflux_const, NC_ldet, NC_sdet, convertN, convertP;
} orc_cpl_soil;

/* pelagic tracer row of each field the reverse Run writes, -1 = absent */
typedef struct {
  int nitrate, ammonium, din, dip, oxygen, odu, detN, detC, detP;
} orc_cpl_soil_fields;

void orc_cpl_soil_defaults(orc_cpl_soil *p);

/* One soil_pelagic_connector Run: fluxes [11][ncol] are the sediment's
 * (downward positive); bfl [ntr][ncol] holds the pelagic bottom fluxes
 * before the Run and is updated where the Run writes; present [ntr] is set
 * to 1 for every row written. */
void orc_cpl_soil_run(const orc_cpl_soil *p, const orc_cpl_soil_fields *f,
                      const double *fluxes, int ncol, int ntr, double *bfl, int *present);

#ifdef __cplusplus
}
#endif
#endif
