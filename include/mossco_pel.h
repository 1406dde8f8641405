/*
 * mossco_pel.h -- C ABI of the GB300 pelagic-driver solver.
 *
 * The second driver behind the same ABI shape as mossco_sed.h: MOSSCO's
 * fabm_pelagic driver right-hand side (local FABM rates, here the GOTM NPZD
 * model that the reference's pelagic set-ups select) integrated by the
 * solver_library ODE stepper over every water cell, with the pelagic
 * component's Run around it.  Plain pointers and sizes only; every call
 * returns SED_OK (0) or a negative SED_E_* code of mossco_sed.h.  A handle
 * owns one CUDA stream and its device buffers; calls on one handle are not
 * thread safe.
 *
 * Layout (the reference's Fortran order read backwards, C order):
 *   per cell   [ntr][knum][ncol]  == conc(i,j,k,n), col = i + inum*j
 *   per layer  [knum][ncol]       == layer_height(i,j,k), par(i,j,k)
 *   per column [ncol]             == I_0(i,j), albedo(i,j)
 *   fluxes     [ntr][ncol]        == bfl(n)%p(i,j) and the flux fields
 * k = 0 is the bottom layer and k = knum-1 the surface layer, as the
 * driver's set_bottom_index(1) / set_surface_index(knum).
 *
 * Reference interfaces replaced (paths inside platipodium/mossco-code):
 *   ode_solver(rhs_driver, dt, method)   src/utilities/solver_library.F90:80-90
 *   get_rhs(rhs_driver, rhs)             src/drivers/fabm_pelagic_driver.F90:380-417
 *   light(pf)                            src/drivers/fabm_pelagic_driver.F90:774-814
 *   clip_below_minimum(pf)               src/drivers/fabm_pelagic_driver.F90:910-927
 *   Run loop (light, internal steps, soil-surface fluxes, external flux
 *   fields, clip)                        src/components/fabm_pelagic_component.F90:1931,2061-2240
 */
#ifndef MOSSCO_PEL_H
#define MOSSCO_PEL_H

#include "mossco_sed.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PEL_NTR 4          /* gotm_npzd: nutrient, phytoplankton,
                              zooplankton, detritus (mmol N/m3) */
#define PEL_KMAX_LIMIT 4096

/* step-cut scope of the adaptive method */
#define PEL_CUT_PER_CELL 0 /* each water cell cuts its own substep (the
                              rhs is local to the cell) */
#define PEL_CUT_GLOBAL 1   /* one cut for the whole grid, as on one PET */

typedef struct pel_params {
  /* gotm_npzd (&gotm_npzd of examples/fabmsed_fabm0d/fabm.nml:57-79);
   * rates per day, converted to per second inside */
  double p0, z0;       /* mmol/m3 background phytoplankton / zooplankton */
  double kc;           /* m2/mmol self-shading */
  double I_min;        /* W/m2 minimum optimal PAR */
  double rmax, gmax;   /* 1/d nutrient uptake, grazing */
  double Iv;           /* m3/mmol Ivlev constant */
  double alpha;        /* mmol/m3 half saturation */
  double rpn, rzn, rdn, rpdu, rpdl, rzd; /* 1/d */
  /* fabm_pelagic namelist (fabm_pelagic_component.F90:47,393) */
  double dt_min;              /* s */
  double relative_change_min; /* e.g. -0.9 */
  double background_extinction; /* 1/m, fabm_pelagic_driver.F90:65 */
  double atol;                /* absolute floor of the positivity test
                                 (0: the reference's test) */
  int max_attempts;           /* adaptive attempts per cell (or grid) and
                                 internal step */
  int cut_scope;              /* PEL_CUT_PER_CELL or PEL_CUT_GLOBAL */
  double minimum[PEL_NTR];    /* clip_below_minimum floor per tracer */
  int precision;              /* SED_FP32 (default) or SED_FP64 */
  int device;                 /* CUDA ordinal */
} pel_params;

typedef struct pel_stats {
  long long attempts;     /* adaptive attempts, summed over cells */
  long long accepted;     /* accepted substeps */
  long long column_steps; /* water columns x Runs */
  int max_cell_attempts;  /* max attempts of one cell in one internal step */
  int capped_cells;       /* cell-steps that hit max_attempts */
  int nan_cells;          /* NaN cells seen after ode_solver */
  int gpu_launches;       /* kernels this library launched for the call */
  double min_dt;          /* smallest accepted substep (s) */
  double device_ms;       /* device time of the call (CUDA events) */
} pel_stats;

typedef struct pel_handle pel_handle;

/* gotm_npzd namelist values of fabm.nml, dt_min 1e-8 and
 * relative_change_min -0.9 of the component, background extinction 1/7.9
 * (Jerlov 6), clip at 0, FP32, per-cell cuts. */
int pel_default_params(pel_params *p);

/* Create a solver for an inum x jnum grid of knum layers and ntr tracers
 * (must be PEL_NTR): fabm_pelagic_driver.F90:215-293 initialize_domain. */
int pel_create(const pel_params *p, int inum, int jnum, int knum, int ntr,
               pel_handle **out);
void pel_destroy(pel_handle *h);
const char *pel_last_error(const pel_handle *h);

/* Layer heights [knum][ncol] (m; update_grid :362-378) and the mask
 * [knum][ncol] (> 0 masked, any pattern; NULL: none).  Masked cells are
 * never read or written and add no optical depth. */
int pel_set_grid(pel_handle *h, const double *layer_height, const int *mask);

/* Forcing of a Run: surface PAR I_0 [ncol] (W/m2), albedo [ncol] (NULL: 0),
 * bottom_flux [ntr][ncol] (`<name>_upward_flux_at_soil_surface`, /m2/s,
 * :2100-2105), surface_flux [ntr][ncol] (`_flux_at_surface` fields,
 * :2193-2194) and soil_flux [ntr][ncol] (`_flux_at_soil_surface` fields,
 * added unless the bottom cell would go negative, :2196-2203); each flux may
 * be NULL (none). */
int pel_set_forcing(pel_handle *h, const double *I_0, const double *albedo,
                    const double *bottom_flux, const double *surface_flux,
                    const double *soil_flux);

/* Vertically homogeneous open-boundary values of the Run
 * (fabm_pelagic_component.F90:2115-2155, `<name>_boundary_value_hz`
 * fields): after every internal step's bottom fluxes, every water cell of a
 * column with open_boundary[col] != 0 takes boundary_value[n][col] for each
 * tracer n with has_value[n] != 0 (a field present in the import state).
 * open_boundary [ncol] (NULL: no open boundary from now on),
 * boundary_value [ntr][ncol], has_value [ntr]. */
int pel_set_open_boundary(pel_handle *h, const int *open_boundary,
                          const double *boundary_value, const int *has_value);

int pel_set_state(pel_handle *h, const double *conc);
int pel_get_state(pel_handle *h, double *conc);

/* light (:774-814): PAR [knum][ncol] of conc (host, NULL: the device
 * state), kept in the handle for pel_get_rhs / pel_ode_solver and copied to
 * par when it is not NULL. */
int pel_light(pel_handle *h, const double *conc, double *par);

/* Drop-in for get_rhs (:380-417) of conc with the handle's PAR. */
int pel_get_rhs(pel_handle *h, const double *conc, double *rhs);

/* Drop-in for `call ode_solver(pel, dt, method)` on the caller's host conc
 * (updated in place) with the handle's PAR; no epilogue. */
int pel_ode_solver(pel_handle *h, double *conc, double dt, int method,
                   pel_stats *stats);

/* One Run of the component over a coupling interval t_couple: light once
 * (:1931), then internal steps of dt, the last one shortened to end on
 * t_couple (:2061-2070), each ode_solver followed by the NaN count, the
 * soil-surface fluxes, the external flux fields and clip_below_minimum.
 * conc is the caller's host array (updated in place) or NULL for the
 * device-resident state. */
int pel_run(pel_handle *h, double *conc, double t_couple, double dt,
            int method, pel_stats *stats);

/* nruns Runs on the device-resident state, forcing as last set. */
int pel_step(pel_handle *h, double t_couple, double dt, int method, int nruns,
             pel_stats *stats);

#ifdef __cplusplus
}
#endif
#endif
