/*
 * sed_oracle.h -- FP64 CPU oracle for the MOSSCO sediment-column hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm, which tests/ and __graft_entry__.smoke() compare against and
 * bench.py's CPU-baseline leg times.  The product path (the CUDA library) never
 * links, loads or calls it.
 *
 * Parity status: the ODE stepper and the transport stencil follow the
 * reference source line by line and are pinned by known-answer tests built
 * from the reference's own solver test; the OMEXDIA+P reaction rates live in
 * the external FABM library (model hzg_omexdia_p, unpinned version) and are a
 * restatement of the published model -- parity for the rates is UNPINNED.
 *
 * Layout: every per-cell array is Fortran conc(i,j,k,n) order, i.e. element
 * (n,k,col) sits at [(n*kmax + k)*ncol + col] with col = i + inum*j
 * (src/components/fabm_sediment_component.F90:521).  Per-column arrays
 * (bdys, fluxes) are [field][ncol].
 */
#ifndef SED_ORACLE_H
#define SED_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NTR 11

/* OMEXDIA+P parameters, per-day units as in
 * examples/standalone/omexdia_p/fabm_sed.nml:51-77 and :18-46. */
typedef struct {
  double rLabile, rSemilabile, NCrLdet, NCrSdet, PAds, PAdsODU, NH3Ads,
      CprodMax, rnit, ksO2nitri, rODUox, ksO2oduox, ksO2oxic, ksNO3denit,
      kinO2denit, kinNO3anox, kinO2anox;
} orc_bgc;

/* Driver + solver state that get_rhs / ode_solver read.  Mirrors the fields
 * of type_sed (src/drivers/fabm_sediment_driver.F90:69-113) and
 * type_rhs_driver (src/utilities/solver_library.F90:37-49). */
typedef struct {
  int ncol;  /* inum*jnum */
  int kmax;  /* knum */
  int ntr;   /* nvar, must be ORC_NTR */
  const int *kact;        /* [ncol] active layers per column, 0 = land */
  const double *dz;       /* [kmax][ncol] layer height (m) */
  const double *dzc;      /* [kmax-1][ncol] centre distance (m) */
  const double *phi;      /* [kmax][ncol] porosity at centres */
  const double *phi_i;    /* [kmax][ncol] porosity at upper interfaces */
  const double *biofac;   /* [kmax][ncol] bioturbation_factor */
  const double *flux_cap; /* [kmax][ncol] only read for bcup 4 */
  const unsigned char *particulate; /* [ntr] */
  const double *minimum;  /* [ntr] clamp value of the component epilogue */
  double diffusivity;     /* cm2/d */
  double bioturbation;    /* cm2/d */
  int bcup_dissolved;     /* 1 flux, 2 concentration, 3 zero-gradient */
  int bcup_particulate;   /* 1 flux, 4 capped flux cascade */
  int mol_diff_mode;      /* 0 reference (diffusivity+0.035T), 1 tortuosity */
  double mol_diff_d0;     /* m2/s, mode 1 free-solution diffusivity */
  double dt_min;
  double relative_change_min;
  double atol;            /* absolute tolerance of the positivity test:
                             reject if c1 - (1+rcm) c < -atol (0 = reference) */
  long max_attempts;      /* guard on the adaptive loop (reference has none) */
  orc_bgc bgc;
  /* bioturbation_profile 3 (Zhang & Wirtz 2017, get_rhs :618-645): the
   * bioturbation factor follows an infauna biomass estimated from the TOC
   * profile at every get_rhs, replacing biofac, with bioturbation * f_T = 1.
   * Namelist constants bioturb_* (fabm_sediment_driver.F90:208,226-231). */
  int bioturbation_profile;
  double bioturb_k_l, bioturb_L1, bioturb_L2, bioturb_beta, bioturb_b,
      bioturb_dry_density;
  /* [ncol] a parameter set per column (an ensemble), or NULL for bgc */
  const orc_bgc *bgc_col;
  /* > 0: rLabile, rSemilabile, CprodMax, rnit and rODUox multiplied by
   * exp(-temp_activation (1/(T+273) - 1/288)), T the column's temperature
   * (the Arrhenius form of f_T, fabm_sediment_driver.F90:648); 0: none */
  double temp_activation;
} orc_model;

typedef struct {
  long attempts;      /* get_rhs-equivalent evaluations of the adaptive loop */
  long accepted;      /* accepted substeps */
  long rejected;      /* step cuts */
  long max_col_attempts;
  double min_dt;      /* smallest accepted dt_red */
  int capped;         /* columns that hit max_attempts */
  int nan_cells;
} orc_stats;

/* a5: fabm_sed_grid%init_grid (fabm_sediment_driver.F90:127-177). */
void orc_init_grid_linear(int kmax, double dzmin, double *dz, double *zc,
                          double *zi, double *dzc);

/* a6/a7: porosity, bioturbation factor, flux cap and interface porosity as
 * in initialize (fabm_sediment_driver.F90:278-304) and update_porosity
 * (:430-435), for one column profile. */
void orc_init_profiles(int kmax, const double *zc, const double *zi,
                       const double *dz, double porosity_max,
                       double porosity_fac, int bioturbation_profile,
                       double bioturbation, double bioturbation_depth,
                       double bioturbation_min, double pom_flux_max,
                       double *phi, double *phi_i, double *biofac,
                       double *flux_cap);

/* Interface porosity only (update_porosity :434-435). */
void orc_interface_porosity(int kmax, const double *phi, double *phi_i);

/* a11: OMEXDIA+P local rates for one cell, per second; fr multiplies the
 * microbial rate constants (the temperature factor; 1 for none). */
void orc_omexdia_p(const orc_bgc *p, double fr, const double *c, double *r,
                   double *denit);

/* a10: diff3d for one column (fabm_sediment_driver.F90:739-825); all
 * arrays contiguous over the column's K layers, Flux has K+1 entries. */
void orc_diff3d(int K, const double *C, double Cup, double Cdown,
                double fluxup, double fluxdown, int bcup, int bcdown,
                const double *D, const double *VF, const double *dz,
                const double *dzc, const double *flux_cap, double *Flux,
                double *dC);

/* a9: get_rhs over the whole grid (fabm_sediment_driver.F90:575-717).
 * fluxes is read (flux boundaries) and written (dissolved surface flux). */
void orc_get_rhs(const orc_model *m, const double *conc, const double *bdys,
                 double *fluxes, double *rhs, double *denit);

/* a2-a4: ode_solver (solver_library.F90:80-189) over the whole grid: the
 * adaptive cut is decided by any() across all columns.  Returns 0, or -3 if
 * max_attempts was hit. */
int orc_ode_solver(const orc_model *m, double *conc, const double *bdys,
                   double *fluxes, double dt, int method, orc_stats *st);

/* type_rhs_driver's diagnostics of the adaptive method
 * (solver_library.F90:43-45): the smallest accepted substep so far and the
 * (i,j,k,n) cell (1-based) of the smallest relative change (c1-c)/c at the
 * substep that set it.  They persist across calls, as on the driver. */
typedef struct {
  double last_min_dt;
  int last_min_dt_grid_cell[4];
  int inum;               /* grid columns along i (col = i + inum*j) */
} orc_diag;

void orc_diag_init(orc_diag *d, int inum);

/* ADAPTIVE_EULER over the whole grid with adaptive_solver_diagnostics on
 * (:129-136), updating d. */
int orc_ode_solver_diag(const orc_model *m, double *conc, const double *bdys,
                        double *fluxes, double dt, orc_diag *d, orc_stats *st);

/* Same stepper applied to every column as its own 1-column grid (the
 * per-column refinement the reference's TODO at solver_library.F90:113-116
 * asks for).  OpenMP over columns with nthreads threads (<=0: default). */
int orc_ode_solver_percol(const orc_model *m, double *conc, const double *bdys,
                          double *fluxes, double dt, int method, int nthreads,
                          orc_stats *st);

/* a12: component epilogue (fabm_sediment_component.F90:1718-1732): count
 * NaN cells (check_NaN :2377-2421) then clamp to the per-tracer minimum. */
int orc_epilogue(const orc_model *m, double *conc);

/* A coupling-step loop: nsteps x (ode_solver + epilogue), per-column or
 * global.  Returns the first non-zero status. */
int orc_run(const orc_model *m, double *conc, const double *bdys,
            double *fluxes, double dt, int method, int percol, int nsteps,
            int nthreads, orc_stats *st);

/* a13: dissolved flux estimate of get_boundary_conditions
 * (fabm_sediment_component.F90:2012-2014) for bcup_dissolved = 1. */
void orc_bc_flux_estimate(const orc_model *m, const double *conc,
                          const double *bdys, double *fluxes);

/* a13: get_boundary_conditions (fabm_sediment_component.F90:1865-2030) for
 * every column: temperature -> bdys[0]; for each tracer n with present[n]
 * (the import state holds it): particulate fluxes[n] = -surface[n] *
 * velocity[n] (downward positive, :1978,1986); dissolved bdys[n+1] =
 * surface[n] and fluxes[n] = the diffusive estimate of :2012-2014 for
 * bcup_dissolved 1 (from conc's first layer; 0 for land columns), else 0.
 * Absent tracers keep their bdys/fluxes. */
void orc_assemble_bc(const orc_model *m, const double *conc, const double *temperature,
                     const double *surface, const double *velocity,
                     const int *present, double *bdys, double *fluxes);

/* FP64 column inventories sum_k phi dz C for every tracer: [ntr][ncol]. */
void orc_inventory(const orc_model *m, const double *conc, double *inv);

#ifdef __cplusplus
}
#endif
#endif
