/*
 * pel_oracle.c -- FP64 CPU oracle for the MOSSCO pelagic driver path.
 *
 * TEST INFRASTRUCTURE ONLY: the values the tests compare the CUDA pelagic
 * library with, and the timed CPU baseline of its bench line.  Nothing in the product path links
 * or calls this file.
 *
 * Restates, in the reference's operation order:
 *   src/utilities/solver_library.F90:80-189      ode_solver (4 methods)
 *   src/drivers/fabm_pelagic_driver.F90:380-417  get_rhs (rhs = 0, local rates)
 *   src/drivers/fabm_pelagic_driver.F90:774-814  light (PAR from the surface down)
 *   src/drivers/fabm_pelagic_driver.F90:910-927  clip_below_minimum
 *   src/components/fabm_pelagic_component.F90:2061-2240  Run: light once
 *     (:1931), then per internal step ode_solver (:2081), the soil-surface
 *     upward fluxes (:2093-2105), the external surface and soil fluxes
 *     (:2188-2203) and the clip (:2238); NaN checks count cells here.
 * and the FABM model gotm_npzd that the reference's pelagic set-ups select
 * (examples/fabmsed_fabm0d/fabm.nml:8, parameters :57-79).  FABM is not in
 * the reference tree; the rates follow the published GOTM NPZD model
 * (Burchard, Bolding, Kuehn, Meister, Neumann and Umlauf 2006, J. Mar. Syst.
 * 61:180-211): Steele light limitation with iopt = max(I_0/4, I_min),
 * Monod nutrient uptake, squared-Ivlev grazing, linear exudation,
 * excretion, mortality and remineralisation; self-shading kc (p0 + p + d).
 * Parity of the rates is UNPINNED: no reference test or output fixes them.
 *
 * Build with -ffp-contract=off so that x86 and aarch64 give the same bits.
 */
#include "pel_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NTR ORC_PEL_NTR
#define AT(n, k, col, K, ncol) (((size_t)(n) * (K) + (k)) * (ncol) + (col))

/* exp(x) by Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2 (W. J. Cody
 * and W. Waite, Software Manual for the Elementary Functions, 1980), and the
 * Taylor series of exp(r) to degree 13 (truncation below 2^-56 relative) in
 * Horner form with fused multiply-adds.  ln2 is split into the double
 * nearest to it and the remainder.  Every step is an IEEE operation with one
 * rounding (rint, fma, ldexp), so the FP64 device path computes the same
 * bits.  Results below 2^-1020 flush to 0 and above 2^1023.9 go to inf. */
double orc_pel_exp(double x) {
  const double inv_ln2 = 1.4426950408889634;       /* 1/ln 2 */
  const double ln2_hi = 0.6931471805599453;        /* nearest double to ln 2 */
  const double ln2_lo = 2.3190468138462996e-17;    /* ln 2 - ln2_hi */
  if (x != x) return x;
  if (x < -707.0) return 0.0;
  if (x > 709.7) return HUGE_VAL;
  const double k = rint(x * inv_ln2);
  double r = fma(-k, ln2_hi, x);
  r = fma(-k, ln2_lo, r);
  double s = 1.0 / 6227020800.0;                   /* 1/13! */
  s = fma(s, r, 1.0 / 479001600.0);
  s = fma(s, r, 1.0 / 39916800.0);
  s = fma(s, r, 1.0 / 3628800.0);
  s = fma(s, r, 1.0 / 362880.0);
  s = fma(s, r, 1.0 / 40320.0);
  s = fma(s, r, 1.0 / 5040.0);
  s = fma(s, r, 1.0 / 720.0);
  s = fma(s, r, 1.0 / 120.0);
  s = fma(s, r, 1.0 / 24.0);
  s = fma(s, r, 1.0 / 6.0);
  s = fma(s, r, 0.5);
  s = fma(s, r, 1.0);
  s = fma(s, r, 1.0);
  return ldexp(s, (int)k);
}

/* gotm_npzd local rates of one cell, c = (n, p, z, d); each expression
 * evaluated left to right as the Fortran statements of the model would be. */
void orc_npzd_rates(const orc_npzd *m, const double *c, double par, double iopt,
                    double *r) {
  const double n = c[0], p = c[1], z = c[2], d = c[3];
  const double rpd = par >= m->I_min ? m->rpdu : m->rpdl;
  /* primary production: rmax * par/iopt * exp(1 - par/iopt) * n/(alpha+n) * (p+p0) */
  const double x = par / iopt;
  const double fnp = m->rmax * par / iopt * orc_pel_exp(1.0 - x) * n /
                     (m->alpha + n) * (p + m->p0);
  /* grazing: gmax * (1 - exp(-Iv^2 p^2)) * (z+z0) */
  const double fpz = m->gmax * (1.0 - orc_pel_exp(-(m->Iv * m->Iv * (p * p)))) *
                     (z + m->z0);
  r[0] = -fnp + m->rpn * p + m->rzn * z + m->rdn * d;
  r[1] = fnp - fpz - m->rpn * p - rpd * p;
  r[2] = fpz - m->rzn * z - m->rzd * z;
  r[3] = rpd * p + m->rzd * z - m->rdn * d;
}

static int masked(const orc_pel *m, int k, int col) {
  return m->mask && m->mask[(size_t)k * m->ncol + col];
}

/* light (fabm_pelagic_driver.F90:774-814) of one column: optical depth at
 * each layer centre accumulated from the surface in half layers,
 * PAR = I_0 (1 - albedo) exp(-bioext).  A masked cell adds no optical depth. */
static void light_column(const orc_pel *m, const double *conc, int col,
                         double *par) {
  const int K = m->knum, nc = m->ncol;
  const double I0 = m->I_0[col];
  const double alb = m->albedo ? m->albedo[col] : 0.0;
  const double localpar = I0 * (1.0 - alb);
  double prev = 0.0;
  for (int k = K - 1; k >= 0; k--) {
    double b = prev;
    if (!masked(m, k, col)) {
      const double p = conc[AT(1, k, col, K, nc)], d = conc[AT(3, k, col, K, nc)];
      const double ext = m->bgc.kc * (m->bgc.p0 + p + d);
      const double t = (ext + m->background_extinction) * 0.5 *
                       m->layer_height[(size_t)k * nc + col];
      b = prev + t;      /* :789 first half of layer k */
      prev = b + t;      /* :792 second half, carried to layer k-1 */
    }
    par[(size_t)k * nc + col] = localpar * orc_pel_exp(-b);
  }
}

void orc_pel_light(const orc_pel *m, const double *conc, double *par) {
  for (int col = 0; col < m->ncol; col++) light_column(m, conc, col, par);
}

static double iopt_of(const orc_pel *m, int col) {
  const double a = 0.25 * m->I_0[col];
  return a > m->bgc.I_min ? a : m->bgc.I_min;
}

/* get_rhs (:380-417): rhs = 0 (masked cells stay 0), then the local rates.
 * gotm_npzd has no surface exchange, so fabm_do_surface adds nothing. */
void orc_pel_get_rhs(const orc_pel *m, const double *conc, const double *par,
                     double *rhs) {
  const int K = m->knum, nc = m->ncol;
  for (int col = 0; col < nc; col++) {
    const double iopt = iopt_of(m, col);
    for (int k = 0; k < K; k++) {
      double c[NTR], r[NTR] = {0, 0, 0, 0};
      if (!masked(m, k, col)) {
        for (int n = 0; n < NTR; n++) c[n] = conc[AT(n, k, col, K, nc)];
        orc_npzd_rates(&m->bgc, c, par[(size_t)k * nc + col], iopt, r);
      }
      for (int n = 0; n < NTR; n++) rhs[AT(n, k, col, K, nc)] = r[n];
    }
  }
}

/* ode_solver of one cell (solver_library.F90:97-186).  The pelagic rhs is
 * local, so a cell's stages see only the cell: this equals the whole-grid
 * form for the fixed methods and for the adaptive one with a per-cell cut. */
static void cell_fixed(const orc_pel *m, double *c, double par, double iopt,
                       double dt, int method) {
  const orc_npzd *b = &m->bgc;
  const double third = 1.0 / 3.0;
  double r0[NTR], r1[NTR], r2[NTR], r3[NTR], c1[NTR];
  if (method == 0) { /* :99-102 */
    orc_npzd_rates(b, c, par, iopt, r0);
    for (int n = 0; n < NTR; n++) c[n] = c[n] + dt * r0[n];
  } else if (method == 1) { /* :142-163 */
    orc_npzd_rates(b, c, par, iopt, r0);
    for (int n = 0; n < NTR; n++) c1[n] = c[n] + 0.5 * dt * r0[n];
    orc_npzd_rates(b, c1, par, iopt, r1);
    for (int n = 0; n < NTR; n++) c1[n] = c[n] + 0.5 * dt * r1[n];
    orc_npzd_rates(b, c1, par, iopt, r2);
    for (int n = 0; n < NTR; n++) c1[n] = c[n] + dt * r2[n];
    orc_npzd_rates(b, c1, par, iopt, r3);
    for (int n = 0; n < NTR; n++)
      c[n] = c[n] + dt * third * (0.5 * r0[n] + r1[n] + r2[n] + 0.5 * r3[n]);
  } else { /* :164-185 */
    orc_npzd_rates(b, c, par, iopt, r0);
    for (int n = 0; n < NTR; n++) c1[n] = c[n] + third * dt * r0[n];
    orc_npzd_rates(b, c1, par, iopt, r1);
    for (int n = 0; n < NTR; n++) c1[n] = c[n] + dt * (r1[n] - third * r0[n]);
    orc_npzd_rates(b, c1, par, iopt, r2);
    for (int n = 0; n < NTR; n++) c1[n] = c[n] + dt * (r0[n] - r1[n] + r2[n]);
    orc_npzd_rates(b, c1, par, iopt, r3);
    for (int n = 0; n < NTR; n++)
      c[n] = c[n] + dt * 1.0 / 8.0 * (r0[n] + 3.0 * r1[n] + 3.0 * r2[n] + r3[n]);
  }
}

/* positivity test of solver_library.F90:121 (AVOID_DIVISION), with the
 * absolute floor atol (0 = the reference's test) */
static int below(const orc_pel *m, double c1, double c) {
  return c1 - (1.0 + m->relative_change_min) * c < -m->atol;
}

/* ADAPTIVE_EULER (:104-140) for one cell; a rejected attempt leaves the
 * state unchanged, so its rhs is reused. */
static int cell_adaptive(const orc_pel *m, double *c, double par, double iopt,
                         double dt, long *attempts, long *accepted,
                         double *min_dt) {
  double r[NTR];
  double dt_int = 0.0, dt_red = dt;
  long att = 0;
  orc_npzd_rates(&m->bgc, c, par, iopt, r);
  while (dt_int < dt) {
    if (att >= m->max_attempts) { *attempts += att; return 1; }
    att++;
    int bad = 0;
    for (int n = 0; n < NTR; n++) bad |= below(m, c[n] + dt_red * r[n], c[n]);
    if (bad && dt_red > m->dt_min) {
      dt_red = dt_red * 0.25;
    } else {
      for (int n = 0; n < NTR; n++) c[n] = c[n] + dt_red * r[n];
      dt_int = dt_int + dt_red;
      (*accepted)++;
      if (dt_red < *min_dt) *min_dt = dt_red;
      if (dt_int < dt) orc_npzd_rates(&m->bgc, c, par, iopt, r);
    }
  }
  *attempts += att;
  return 0;
}

/* ADAPTIVE_EULER with the reference's grid-wide any() (:119-121). */
static int grid_adaptive(const orc_pel *m, double *conc, const double *par,
                         double dt, orc_pel_stats *st) {
  const int K = m->knum, nc = m->ncol;
  const size_t cells = (size_t)K * nc;
  double *rhs = malloc(NTR * cells * sizeof(double));
  if (!rhs) return -1;
  double dt_int = 0.0, dt_red = dt;
  long att = 0;
  int rc = 0;
  orc_pel_get_rhs(m, conc, par, rhs);
  while (dt_int < dt) {
    if (att >= m->max_attempts) { st->capped = 1; rc = 1; break; }
    att++;
    int bad = 0;
    for (size_t i = 0; i < NTR * cells && !bad; i++) {
      const size_t cell = i % cells;
      if (m->mask && m->mask[cell]) continue;
      bad |= below(m, conc[i] + dt_red * rhs[i], conc[i]);
    }
    if (bad && dt_red > m->dt_min) {
      dt_red = dt_red * 0.25;
    } else {
      for (size_t i = 0; i < NTR * cells; i++) {
        if (m->mask && m->mask[i % cells]) continue;
        conc[i] = conc[i] + dt_red * rhs[i];
      }
      dt_int = dt_int + dt_red;
      st->accepted++;
      if (dt_red < st->min_dt) st->min_dt = dt_red;
      if (dt_int < dt) orc_pel_get_rhs(m, conc, par, rhs);
    }
  }
  st->attempts += att;
  if (att > st->max_cell_attempts) st->max_cell_attempts = att;
  free(rhs);
  return rc;
}

static void stats_init(orc_pel_stats *st) {
  memset(st, 0, sizeof *st);
  st->min_dt = HUGE_VAL;
}

/* ode_solver over the grid with the handle's PAR; returns 0, or 1 when a
 * cell (or the grid) reached max_attempts. */
int orc_pel_ode_solver(const orc_pel *m, double *conc, const double *par,
                       double dt, int method, orc_pel_stats *st) {
  const int K = m->knum, nc = m->ncol;
  if (method == 2 && m->cut_scope == 1) return grid_adaptive(m, conc, par, dt, st);
  int rc = 0;
  for (int col = 0; col < nc; col++) {
    const double iopt = iopt_of(m, col);
    for (int k = 0; k < K; k++) {
      if (masked(m, k, col)) continue;
      double c[NTR];
      for (int n = 0; n < NTR; n++) c[n] = conc[AT(n, k, col, K, nc)];
      const double par_k = par[(size_t)k * nc + col];
      if (method == 2) {
        long a0 = st->attempts;
        if (cell_adaptive(m, c, par_k, iopt, dt, &st->attempts, &st->accepted,
                          &st->min_dt)) {
          st->capped = 1;
          rc = 1;
        }
        if (st->attempts - a0 > st->max_cell_attempts)
          st->max_cell_attempts = st->attempts - a0;
      } else {
        cell_fixed(m, c, par_k, iopt, dt, method);
        st->attempts++;
        st->accepted++;
        if (dt < st->min_dt) st->min_dt = dt;
        if (st->max_cell_attempts < 1) st->max_cell_attempts = 1;
      }
      for (int n = 0; n < NTR; n++) conc[AT(n, k, col, K, nc)] = c[n];
    }
  }
  return rc;
}

/* The component's per-step epilogue on one column (:2093-2105, :2188-2203,
 * :2238): bottom upward fluxes where the bottom layer has a height,
 * open-boundary values (:2115-2155), external surface fluxes into the top
 * layer, soil-surface fluxes into the
 * bottom layer unless they would make it negative, then the clip.  Returns
 * the NaN cells seen after ode_solver. */
static int epilogue_column(const orc_pel *m, double *conc, int col, double dt) {
  const int K = m->knum, nc = m->ncol;
  int nan = 0;
  for (int k = 0; k < K; k++) {
    if (masked(m, k, col)) continue;
    for (int n = 0; n < NTR; n++) {
      const double v = conc[AT(n, k, col, K, nc)];
      if (v != v) { nan++; break; }
    }
  }
  const double hb = m->layer_height[col];
  const double ht = m->layer_height[(size_t)(K - 1) * nc + col];
  if (!masked(m, 0, col) && m->bottom_flux && hb > 0.0)
    for (int n = 0; n < NTR; n++) {
      double *c = &conc[AT(n, 0, col, K, nc)];
      *c = *c + m->bottom_flux[(size_t)n * nc + col] * dt / hb;
    }
  /* vertically homogeneous boundary values (:2115-2155); masked cells are
   * not written, as everywhere in this restatement */
  if (m->open_boundary && m->open_boundary[col])
    for (int n = 0; n < NTR; n++) {
      if (!m->has_boundary_value[n]) continue;
      for (int k = 0; k < K; k++)
        if (!masked(m, k, col))
          conc[AT(n, k, col, K, nc)] = m->boundary_value[(size_t)n * nc + col];
    }
  if (!masked(m, K - 1, col) && m->surface_flux)
    for (int n = 0; n < NTR; n++) {
      double *c = &conc[AT(n, K - 1, col, K, nc)];
      *c = *c + m->surface_flux[(size_t)n * nc + col] * dt / ht;
    }
  if (!masked(m, 0, col) && m->soil_flux)
    for (int n = 0; n < NTR; n++) {
      double *c = &conc[AT(n, 0, col, K, nc)];
      const double inc = m->soil_flux[(size_t)n * nc + col] * dt / hb;
      if (*c + inc > 0.0) *c = *c + inc;
    }
  for (int k = 0; k < K; k++) {
    if (masked(m, k, col)) continue;
    for (int n = 0; n < NTR; n++) {
      double *c = &conc[AT(n, k, col, K, nc)];
      if (*c < m->minimum[n]) *c = m->minimum[n];
    }
  }
  return nan;
}

/* One column through one Run with a per-cell cut (or a fixed method). */
static int run_column(const orc_pel *m, double *conc, int col, double t_couple,
                      double dt, int method, orc_pel_stats *st, double *par) {
  const int K = m->knum, nc = m->ncol;
  const double iopt = iopt_of(m, col);
  int rc = 0;
  light_column(m, conc, col, par);
  double t = 0.0;
  while (t < t_couple) {
    const double h = t + dt > t_couple ? t_couple - t : dt;
    for (int k = 0; k < K; k++) {
      if (masked(m, k, col)) continue;
      double c[NTR];
      for (int n = 0; n < NTR; n++) c[n] = conc[AT(n, k, col, K, nc)];
      const double par_k = par[(size_t)k * nc + col];
      if (method == 2) {
        const long a0 = st->attempts;
        if (cell_adaptive(m, c, par_k, iopt, h, &st->attempts, &st->accepted,
                          &st->min_dt)) {
          st->capped = 1;
          rc = 1;
        }
        if (st->attempts - a0 > st->max_cell_attempts)
          st->max_cell_attempts = st->attempts - a0;
      } else {
        cell_fixed(m, c, par_k, iopt, h, method);
        st->attempts++;
        st->accepted++;
        if (h < st->min_dt) st->min_dt = h;
        if (st->max_cell_attempts < 1) st->max_cell_attempts = 1;
      }
      for (int n = 0; n < NTR; n++) conc[AT(n, k, col, K, nc)] = c[n];
    }
    st->nan_cells += epilogue_column(m, conc, col, h);
    t = t + h;
  }
  return rc;
}

/* One Run of the pelagic component over a coupling interval t_couple:
 * light once (:1931), then internal steps of dt, the last one shortened to
 * end on t_couple (:2061-2070), each followed by the epilogue.  Cells are
 * independent under a per-cell cut, so columns run in parallel (nthreads,
 * 0 = OpenMP default).  Returns 0, 1 (substep cap) or 2 (NaN). */
int orc_pel_run(const orc_pel *m, double *conc, double t_couple, double dt,
                int method, orc_pel_stats *st, double *par_out, int nthreads) {
  const size_t cells = (size_t)m->knum * m->ncol;
  stats_init(st);
  double *par = par_out ? par_out : malloc(cells * sizeof(double));
  if (!par) return -1;
  int rc = 0;
  if (method == 2 && m->cut_scope == 1) {
    orc_pel_light(m, conc, par);
    double t = 0.0;
    while (t < t_couple) {
      const double h = t + dt > t_couple ? t_couple - t : dt;
      if (grid_adaptive(m, conc, par, h, st)) rc = 1;
      for (int col = 0; col < m->ncol; col++) st->nan_cells += epilogue_column(m, conc, col, h);
      t = t + h;
    }
  } else {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    long attempts = 0, accepted = 0, maxatt = 0;
    double mindt = HUGE_VAL;
    int capped = 0, nan = 0, rcs = 0;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64) \
    reduction(+ : attempts, accepted, nan) reduction(max : maxatt, capped, rcs) \
    reduction(min : mindt)
    for (int col = 0; col < m->ncol; col++) {
      orc_pel_stats cs;
      stats_init(&cs);
      const int r = run_column(m, conc, col, t_couple, dt, method, &cs, par);
      attempts += cs.attempts;
      accepted += cs.accepted;
      nan += cs.nan_cells;
      if (cs.max_cell_attempts > maxatt) maxatt = cs.max_cell_attempts;
      if (cs.capped > capped) capped = cs.capped;
      if (r > rcs) rcs = r;
      if (cs.min_dt < mindt) mindt = cs.min_dt;
    }
    st->attempts = attempts;
    st->accepted = accepted;
    st->max_cell_attempts = maxatt;
    st->min_dt = mindt;
    st->capped = capped;
    st->nan_cells = nan;
    rc = rcs;
  }
  if (!par_out) free(par);
  if (st->nan_cells && rc == 0) rc = 2;
  return rc;
}
