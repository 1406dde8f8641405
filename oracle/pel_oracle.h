/*
 * pel_oracle.h -- FP64 CPU oracle for the MOSSCO pelagic driver path.
 *
 * TEST INFRASTRUCTURE ONLY (see pel_oracle.c).
 *
 * Layout as the library's: conc[n][k][col] is the reference's
 * conc(i,j,k,n) with col = i + inum*(j-1); k = 0 is the bottom layer and
 * k = knum-1 the surface layer (GETM/GOTM order, fabm_pelagic_driver.F90:
 * set_surface_index(knum)).
 */
#ifndef PEL_ORACLE_H
#define PEL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_PEL_NTR 4 /* gotm_npzd: nutrient, phytoplankton, zooplankton, detritus */

/* gotm_npzd parameters with rates per second (the namelist's per-day
 * values divided by 86400) */
typedef struct {
  double p0, z0, kc, I_min, rmax, gmax, Iv, alpha;
  double rpn, rzn, rdn, rpdu, rpdl, rzd;
} orc_npzd;

typedef struct {
  int ncol, knum;
  const double *layer_height;   /* [knum][ncol] */
  const unsigned char *mask;    /* [knum][ncol], nonzero = masked; or NULL */
  const double *I_0;            /* [ncol] surface PAR, W/m2 */
  const double *albedo;         /* [ncol] or NULL (0) */
  const double *bottom_flux;    /* [ntr][ncol] upward flux at the soil surface, /m2/s, or NULL */
  const double *surface_flux;   /* [ntr][ncol] *_flux_at_surface, /m2/s, or NULL */
  const double *soil_flux;      /* [ntr][ncol] *_flux_at_soil_surface, /m2/s, or NULL */
  const double *minimum;        /* [ntr] clip floor */
  double background_extinction; /* 1/m */
  double dt_min, relative_change_min, atol;
  long max_attempts;
  int cut_scope;                /* 0 per cell, 1 the reference's grid-wide any() */
  orc_npzd bgc;
  /* open boundaries (fabm_pelagic_component.F90:2115-2155): columns with
   * open_boundary[col] set take boundary_value[n][col] in every layer, for
   * each tracer n with has_boundary_value[n], after the bottom fluxes of
   * every internal step; NULL = none */
  const unsigned char *open_boundary;   /* [ncol] */
  const double *boundary_value;         /* [ntr][ncol] */
  const int *has_boundary_value;        /* [ntr] */
} orc_pel;

typedef struct {
  long attempts, accepted, max_cell_attempts;
  double min_dt;
  int capped, nan_cells;
} orc_pel_stats;

/* the exponential both this oracle and the FP64 device path use */
double orc_pel_exp(double x);
void orc_npzd_rates(const orc_npzd *m, const double *c, double par, double iopt,
                    double *r);
void orc_pel_light(const orc_pel *m, const double *conc, double *par);
void orc_pel_get_rhs(const orc_pel *m, const double *conc, const double *par,
                     double *rhs);
int orc_pel_ode_solver(const orc_pel *m, double *conc, const double *par,
                       double dt, int method, orc_pel_stats *st);
int orc_pel_run(const orc_pel *m, double *conc, double t_couple, double dt,
                int method, orc_pel_stats *st, double *par_out, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
