/*
 * sed_oracle.c -- FP64 CPU oracle for the MOSSCO sediment-column hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the values the tests compare the CUDA library
 * with, and the timed CPU baseline.  Nothing in the product path links or calls this file.
 *
 * Restates, in the reference's own operation order:
 *   src/utilities/solver_library.F90:80-189      ode_solver (4 methods)
 *   src/drivers/fabm_sediment_driver.F90:127-177 init_grid
 *   src/drivers/fabm_sediment_driver.F90:278-304 porosity / bioturbation
 *   src/drivers/fabm_sediment_driver.F90:430-435 interface porosity
 *   src/drivers/fabm_sediment_driver.F90:575-717 get_rhs
 *   src/drivers/fabm_sediment_driver.F90:739-825 diff3d
 *   src/components/fabm_sediment_component.F90:1715-1732 NaN check + clamp
 * and the OMEXDIA+P rates (external FABM model hzg_omexdia_p, not in the
 * reference tree) from the published OMEXDIA model (Soetaert, Herman and
 * Middelburg 1996, Geochim. Cosmochim. Acta 60:1019) with the parameter
 * names of examples/standalone/omexdia_p/fabm_sed.nml.  Parity of the rates
 * is UNPINNED: no reference test or output fixes them.
 *
 * Build with -ffp-contract=off so that x86 and aarch64 give the same bits.
 */
#include "sed_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(n, k, col, kmax, ncol) (((size_t)(n) * (kmax) + (k)) * (ncol) + (col))

/* ------------------------------------------------------------------------ */
/* a5: linear grid of fabm_sediment_driver.F90:147-168 (one column).         */
void orc_init_grid_linear(int kmax, double dzmin, double *dz, double *zc,
                          double *zi, double *dzc) {
  /* :147 self_fac = 0.18/((knum+1)/2 * dzmin) - 1 */
  double fac = 0.18 / ((kmax + 1) / 2.0 * dzmin) - 1.0;
  zi[0] = 0.0;
  for (int k = 1; k <= kmax; k++) {
    /* :161 dz = (1 + (fac-1)*(k-1)/(knum-1)) * dzmin, integer (k-1) times a
     * real then divided by an integer, left to right */
    double w = (fac - 1.0) * (k - 1) / (kmax - 1);
    dz[k - 1] = (1.0 + w) * dzmin;
    zc[k - 1] = zi[k - 1] + 0.5 * dz[k - 1];
    zi[k] = zi[k - 1] + dz[k - 1];
  }
  for (int k = 0; k < kmax - 1; k++) dzc[k] = zc[k + 1] - zc[k];
}

/* a7: update_porosity :434-435 */
void orc_interface_porosity(int kmax, const double *phi, double *phi_i) {
  phi_i[0] = phi[0];
  for (int k = 1; k < kmax; k++) phi_i[k] = 0.5 * (phi[k - 1] + phi[k]);
}

/* a6: initialize :278-304 for one column. */
void orc_init_profiles(int kmax, const double *zc, const double *zi,
                       const double *dz, double porosity_max,
                       double porosity_fac, int bioturbation_profile,
                       double bioturbation, double bioturbation_depth,
                       double bioturbation_min, double pom_flux_max,
                       double *phi, double *phi_i, double *biofac,
                       double *flux_cap) {
  for (int k = 0; k < kmax; k++) {
    /* :280 porosity = porosity_max * (1 - porosity_fac * zc) */
    phi[k] = porosity_max * (1.0 - porosity_fac * zc[k]);
    /* :284-291 flux cap, non-increasing from layer 3 on */
    flux_cap[k] = pom_flux_max / 86400.0 * (1.0 - phi[k]) * dz[k];
    if (k > 1 && flux_cap[k] > flux_cap[k - 1]) flux_cap[k] = flux_cap[k - 1];
    /* :294-303 bioturbation factor at interfaces (default stays 1.0) */
    double b = 1.0;
    if (bioturbation_profile == 1) {
      double lin = bioturbation_depth - 100.0 * zi[k];
      if (lin < 0.0) lin = 0.0;
      lin = lin / bioturbation_depth;
      double lo = bioturbation_min / bioturbation;
      b = lo > lin ? lo : lin;
    } else if (bioturbation_profile == 2) {
      b = exp(-100.0 * zi[k] / bioturbation_depth);
    }
    biofac[k] = b;
  }
  orc_interface_porosity(kmax, phi, phi_i);
}

/* ------------------------------------------------------------------------ */
/* a11: OMEXDIA+P rates (per second) for one cell.  Tracer order:
 *  0 fdetC 1 sdetC 2 fdetN 3 sdetN 4 fdetP 5 adsP (particulate)
 *  6 O2 7 NO3 8 NH4 9 ODU 10 PO4 (dissolved)
 * Published OMEXDIA: first-order decay of two detritus classes, carbon
 * mineralisation split into oxic / denitrification / anoxic pathways by
 * Monod limitation and inhibition terms rescaled to sum to one,
 * nitrification and ODU re-oxidation with O2 Monod terms, NO3 use of 0.8 mol
 * per mol C in denitrification, NH3 adsorption factor 1/(1+NH3Ads).  The P
 * extension: detritus P mineralises with the labile rate, and PO4 exchanges
 * with an explicit adsorbed-P pool at rate PAds, the sorbing share being
 * PAdsODU/(PAdsODU+ODU) (iron-bound P released as reduced substances
 * accumulate).  CprodMax caps total carbon mineralisation (per day). */
void orc_omexdia_p(const orc_bgc *p, double fr, const double *c, double *r,
                   double *denit) {
  const double spd = 86400.0;
  double fdetC = c[0], sdetC = c[1], fdetN = c[2], sdetN = c[3], fdetP = c[4];
  double adsP = c[5], O2 = c[6], NO3 = c[7], NH4 = c[8], ODU = c[9];
  double PO4 = c[10];
  /* fr: the temperature factor of the microbial rates (1 without) */
  double rF = p->rLabile / spd * fr;
  double rS = p->rSemilabile / spd * fr;
  double CprodF = rF * fdetC;
  double CprodS = rS * sdetC;
  double NprodF = rF * fdetN;
  double NprodS = rS * sdetN;
  double Pprod = rF * fdetP;
  double Cprod = CprodF + CprodS;
  double cmax = p->CprodMax / spd * fr;
  double lim = 1.0;
  if (Cprod > cmax) lim = cmax / Cprod;
  double oxlim = O2 / (O2 + p->ksO2oxic);
  double dnlim = (1.0 - O2 / (O2 + p->kinO2denit)) * (NO3 / (NO3 + p->ksNO3denit));
  double anlim = (1.0 - O2 / (O2 + p->kinO2anox)) * (1.0 - NO3 / (NO3 + p->kinNO3anox));
  double rescale = 1.0 / (oxlim + dnlim + anlim);
  double Cmin = lim * Cprod;
  double OxicMin = Cmin * oxlim * rescale;
  double Denit = Cmin * dnlim * rescale;
  double AnoxicMin = Cmin * anlim * rescale;
  double rnit = p->rnit / spd * fr;
  double rodu = p->rODUox / spd * fr;
  double Nitri = rnit * NH4 * (O2 / (O2 + p->ksO2nitri));
  double OduOx = rodu * ODU * (O2 / (O2 + p->ksO2oduox));
  double fox = p->PAdsODU / (p->PAdsODU + ODU);
  double Rads = p->PAds / spd * (fox * PO4 - (1.0 - fox) * adsP);
  r[0] = -(lim * CprodF);
  r[1] = -(lim * CprodS);
  r[2] = -(lim * NprodF);
  r[3] = -(lim * NprodS);
  r[4] = -(lim * Pprod);
  r[5] = Rads;
  r[6] = -OxicMin - 2.0 * Nitri - OduOx;
  r[7] = -0.8 * Denit + Nitri;
  r[8] = (lim * (NprodF + NprodS) - Nitri) / (1.0 + p->NH3Ads);
  r[9] = AnoxicMin - OduOx;
  r[10] = lim * Pprod - Rads;
  if (denit) *denit = Denit;
}

/* ------------------------------------------------------------------------ */
/* a10: diff3d :769-820, one column, 0-based layers. */
void orc_diff3d(int K, const double *C, double Cup, double Cdown,
                double fluxup, double fluxdown, int bcup, int bcdown,
                const double *D, const double *VF, const double *dz,
                const double *dzc, const double *flux_cap, double *Flux,
                double *dC) {
  for (int k = 0; k < K; k++) dC[k] = 0.0;
  /* :776-778 interior interfaces, positive flux downward */
  for (int k = 1; k < K; k++) Flux[k] = -D[k] * (C[k] - C[k - 1]) / dzc[k - 1];
  /* :782-803 upper boundary */
  if (bcup == 1) {
    Flux[0] = fluxup;
  } else if (bcup == 2) {
    Flux[0] = -D[0] * (C[0] - Cup) / dz[0];
  } else if (bcup == 4) {
    Flux[0] = fluxup;
    int k = 1;
    double rest = Flux[0] - flux_cap[0];
    while (rest > 0.0 && k <= K - 1) {
      Flux[k] = Flux[k] + rest;
      rest = rest - flux_cap[k];
      k++;
    }
    if (k > K - 1) Flux[K - 1] = Flux[K - 1] + rest;
  } else {
    /* 3, and the undefined 0 of the namelist, as a zero flux */
    Flux[0] = 0.0;
  }
  /* :806-816 lower boundary */
  if (bcdown == 1) {
    Flux[K] = fluxdown;
  } else if (bcdown == 2) {
    Flux[K] = -D[K - 1] * (Cdown - C[K - 1]) / dz[K - 1];
  } else {
    Flux[K] = 0.0;
  }
  /* :818-820 */
  for (int k = 0; k < K; k++) dC[k] = (Flux[k] - Flux[k + 1]) / (VF[k] * dz[k]);
}

/* ------------------------------------------------------------------------ */
typedef struct {
  double *dz, *dzc, *phi, *phi_i, *bf, *cap; /* column copies */
  double *diff, *cin, *vf, *flux, *dC, *tr, *cell, *rate, *wt;
} rhs_ws;

static void rhs_ws_alloc(rhs_ws *w, int kmax, int ntr) {
  size_t K = (size_t)kmax;
  w->dz = calloc(K, sizeof(double));
  w->dzc = calloc(K, sizeof(double));
  w->phi = calloc(K, sizeof(double));
  w->phi_i = calloc(K, sizeof(double));
  w->bf = calloc(K, sizeof(double));
  w->cap = calloc(K, sizeof(double));
  w->diff = calloc(K, sizeof(double));
  w->cin = calloc(K, sizeof(double));
  w->vf = calloc(K, sizeof(double));
  w->flux = calloc(K + 1, sizeof(double));
  w->dC = calloc(K, sizeof(double));
  w->tr = calloc(K * ntr, sizeof(double));
  w->cell = calloc(ntr, sizeof(double));
  w->rate = calloc(ntr, sizeof(double));
  w->wt = calloc(K, sizeof(double));
}

static void rhs_ws_free(rhs_ws *w) {
  free(w->dz); free(w->dzc); free(w->phi); free(w->phi_i); free(w->bf);
  free(w->cap); free(w->diff); free(w->cin); free(w->vf); free(w->flux);
  free(w->dC); free(w->tr); free(w->cell); free(w->rate); free(w->wt);
}

/* bioturbation_profile 3 (get_rhs :618-645) for one column of K layers:
 * weighted TOC [mg C / g dry mass] from the two carbon detritus pools (POC
 * class factors of initialize :380-386), its dz-weighted column sum divided
 * by cumdepth -- the depth of the last layer's upper interface, the value the
 * environment loop :593-605 leaves behind -- the infauna biomass and the
 * factor beta biomass^b / TOC, in the reference's operation order.  zc is
 * formed from dz as init_grid does (:150-152). */
static void zhang_wirtz_factor(const orc_model *m, int K, const double *dz,
                               const double *phi, const double *C0,
                               const double *C1, double *wt, double *bf) {
  const double f1 = 1.0 / 1.2 * 12.01 / m->bioturb_dry_density / 1000.0;
  const double f2 = 1.0 / 6.0 * 12.01 / m->bioturb_dry_density / 1000.0;
  for (int k = 0; k < K; k++) {
    wt[k] = 0.0;
    wt[k] = wt[k] + f1 * phi[k] / (1.0 - phi[k]) * C0[k];
    wt[k] = wt[k] + f2 * phi[k] / (1.0 - phi[k]) * C1[k];
  }
  double cum = 0.0;
  for (int k = 0; k < K - 1; k++) cum = cum + dz[k];
  double sum = 0.0;
  for (int k = 0; k < K; k++) sum = sum + dz[k] * wt[k];
  const double avg = sum / cum;
  double zi = 0.0;
  for (int k = 0; k < K; k++) {
    const double zc = zi + 0.5 * dz[k];
    zi = zi + dz[k];
    const double biomass = wt[k] * exp(zc * 100.0 * m->bioturb_k_l) * avg /
                           (m->bioturb_L1 + m->bioturb_L2 * exp(zc * 200.0 * m->bioturb_k_l));
    bf[k] = m->bioturb_beta * pow(biomass, m->bioturb_b) / wt[k];
  }
}

/* get_rhs for one column `col` of model m (arrays of stride m->ncol). */
static void get_rhs_col(const orc_model *m, int col, const double *conc,
                        const double *bdys, double *fluxes, double *rhs,
                        double *denit, rhs_ws *w) {
  const int KM = m->kmax, N = m->ntr;
  const long nc = m->ncol;
  const int K = m->kact[col];
  for (int n = 0; n < N; n++)
    for (int k = 0; k < KM; k++) rhs[IDX(n, k, col, KM, nc)] = 0.0;
  if (denit)
    for (int k = 0; k < KM; k++) denit[(size_t)k * nc + col] = 0.0;
  if (K <= 0) return; /* masked column: rhs = transport = 0 (:703-708) */

  for (int k = 0; k < K; k++) {
    w->dz[k] = m->dz[(size_t)k * nc + col];
    w->phi[k] = m->phi[(size_t)k * nc + col];
    w->phi_i[k] = m->phi_i[(size_t)k * nc + col];
    w->bf[k] = m->biofac[(size_t)k * nc + col];
    w->cap[k] = m->flux_cap ? m->flux_cap[(size_t)k * nc + col] : 0.0;
    if (k < K - 1) w->dzc[k] = m->dzc[(size_t)k * nc + col];
  }
  /* :593-605 temperature of the column = bottom-water temperature */
  const double T = bdys[col];
  /* :648 f_T; with profile 3, f_T = 1 and bioturbation = 1 (:622-623) and
   * the factor is recomputed from the state */
  double f_T = 1.0 * exp(-4500.0 * (1.0 / (T + 273.0) - (1.0 / 288.0)));
  double bioturbation = m->bioturbation;
  /* temperature factor of the microbial rates (sed_params.temp_activation):
   * the same Arrhenius form and 288 K reference as f_T */
  const double fr = m->temp_activation > 0.0
                        ? exp(-m->temp_activation * (1.0 / (T + 273.0) - (1.0 / 288.0)))
                        : 1.0;
  if (m->bioturbation_profile == 3) {
    for (int k = 0; k < K; k++) {
      w->cin[k] = conc[IDX(0, k, col, KM, nc)];
      w->vf[k] = conc[IDX(1, k, col, KM, nc)];
    }
    zhang_wirtz_factor(m, K, w->dz, w->phi, w->cin, w->vf, w->wt, w->bf);
    f_T = 1.0;
    bioturbation = 1.0;
  }

  for (int n = 0; n < N; n++) {
    /* :652-653 */
    for (int k = 0; k < K; k++)
      w->diff[k] = bioturbation * f_T / 86400.0 / 10000.0 *
                   (1.0 - w->phi_i[k]) * w->bf[k];
    const double cup = bdys[(size_t)(n + 1) * nc + col];
    const double fup = fluxes[(size_t)n * nc + col];
    double *trn = w->tr + (size_t)n * K;
    if (m->particulate[n]) {
      /* :658-678 bulk concentration mixed, volume fraction 1-phi */
      for (int k = 0; k < K; k++) {
        w->cin[k] = conc[IDX(n, k, col, KM, nc)] * w->phi[k];
        w->vf[k] = 1.0 - w->phi[k];
      }
      orc_diff3d(K, w->cin, cup, 0.0, fup, 0.0, m->bcup_particulate, 3,
                 w->diff, w->vf, w->dz, w->dzc, w->cap, w->flux, w->dC);
      for (int k = 0; k < K; k++)
        trn[k] = w->dC[k] * (1.0 - w->phi[k]) / w->phi[k];
    } else {
      /* :682-693 molecular diffusion added for dissolved tracers */
      for (int k = 0; k < K; k++) {
        double mol;
        if (m->mol_diff_mode == 1)
          mol = m->mol_diff_d0 * w->phi_i[k] / (1.0 - 2.0 * log(w->phi_i[k]));
        else
          mol = (m->diffusivity + T * 0.035) * w->phi_i[k] / 86400.0 / 10000.0;
        w->diff[k] = w->diff[k] + mol;
        w->cin[k] = conc[IDX(n, k, col, KM, nc)];
      }
      orc_diff3d(K, w->cin, cup, 0.0, fup, 0.0, m->bcup_dissolved, 3, w->diff,
                 w->phi, w->dz, w->dzc, w->cap, w->flux, w->dC);
      for (int k = 0; k < K; k++) trn[k] = w->dC[k];
      fluxes[(size_t)n * nc + col] = w->flux[0];
    }
  }
  /* :696-715 local rates plus transport */
  for (int k = 0; k < K; k++) {
    for (int n = 0; n < N; n++) w->cell[n] = conc[IDX(n, k, col, KM, nc)];
    double dn = 0.0;
    orc_omexdia_p(m->bgc_col ? &m->bgc_col[col] : &m->bgc, fr, w->cell, w->rate, &dn);
    for (int n = 0; n < N; n++)
      rhs[IDX(n, k, col, KM, nc)] = w->rate[n] + w->tr[(size_t)n * K + k];
    if (denit) denit[(size_t)k * nc + col] = dn;
  }
}

void orc_get_rhs(const orc_model *m, const double *conc, const double *bdys,
                 double *fluxes, double *rhs, double *denit) {
  rhs_ws w;
  rhs_ws_alloc(&w, m->kmax, m->ntr);
  for (int col = 0; col < m->ncol; col++)
    get_rhs_col(m, col, conc, bdys, fluxes, rhs, denit, &w);
  rhs_ws_free(&w);
}

/* ------------------------------------------------------------------------ */
typedef struct {
  double *rhs0, *rhs1, *rhs2, *rhs3, *c1;
  rhs_ws rw;
} ode_ws;

static void ode_ws_alloc(ode_ws *w, const orc_model *m) {
  size_t n = (size_t)m->ntr * m->kmax * m->ncol;
  w->rhs0 = calloc(n, sizeof(double));
  w->rhs1 = calloc(n, sizeof(double));
  w->rhs2 = calloc(n, sizeof(double));
  w->rhs3 = calloc(n, sizeof(double));
  w->c1 = calloc(n, sizeof(double));
  rhs_ws_alloc(&w->rw, m->kmax, m->ntr);
}

static void ode_ws_free(ode_ws *w) {
  free(w->rhs0); free(w->rhs1); free(w->rhs2); free(w->rhs3); free(w->c1);
  rhs_ws_free(&w->rw);
}

static void rhs_all(const orc_model *m, const double *conc, const double *bdys,
                    double *fluxes, double *rhs, ode_ws *w) {
  for (int col = 0; col < m->ncol; col++)
    get_rhs_col(m, col, conc, bdys, fluxes, rhs, NULL, &w->rw);
}

/* Visits every active cell (n,k,col) of the model. */
#define FOR_ACTIVE(m, body)                                                  \
  for (int n_ = 0; n_ < (m)->ntr; n_++)                                      \
    for (int col_ = 0; col_ < (m)->ncol; col_++)                             \
      for (int k_ = 0; k_ < (m)->kact[col_]; k_++) {                         \
        size_t i_ = IDX(n_, k_, col_, (m)->kmax, (m)->ncol);                 \
        body;                                                                \
      }

/* minloc((c1 - c)/c) over the grid's whole (i,j,k,n) array in Fortran
 * element order (i fastest), the diagnostic of solver_library.F90:133-134.
 * Cells the solver does not step (land, masked tails) keep c1 = c, as the
 * reference's rhs = 0 there leaves them.  NaN quotients (c = 0) are skipped,
 * as gfortran's MINLOC skips them; with no other value the first element is
 * returned.  Indices are 1-based. */
static void minloc_relative_change(const orc_model *m, const double *conc,
                                   const double *c1, int inum, int cell[4]) {
  const int KM = m->kmax, nc = m->ncol;
  int found = 0;
  double best = 0.0;
  size_t pos = 0, idx = 0;
  for (int n = 0; n < m->ntr; n++)
    for (int k = 0; k < KM; k++)
      for (int col = 0; col < nc; col++, idx++) {
        const size_t i = IDX(n, k, col, KM, nc);
        const double c = conc[i];
        const double v = (k < m->kact[col] ? c1[i] - c : c - c) / c;
        if (v != v) continue;
        if (!found || v < best) {
          found = 1;
          best = v;
          pos = idx;
        }
      }
  const size_t col = pos % (size_t)nc, kn = pos / (size_t)nc;
  cell[0] = (int)(col % (size_t)inum) + 1;
  cell[1] = (int)(col / (size_t)inum) + 1;
  cell[2] = (int)(kn % (size_t)KM) + 1;
  cell[3] = (int)(kn / (size_t)KM) + 1;
}

static int ode_solver_ws(const orc_model *m, double *conc, const double *bdys,
                         double *fluxes, double dt, int method, orc_stats *st,
                         ode_ws *w, orc_diag *diag) {
  const double third = 1.0 / 3.0;
  double *c1 = w->c1;
  switch (method) {
  case 0: /* EULER :99-102 */
    rhs_all(m, conc, bdys, fluxes, w->rhs0, w);
    FOR_ACTIVE(m, conc[i_] = conc[i_] + dt * w->rhs0[i_]);
    if (st) { st->attempts++; st->accepted++; }
    return 0;
  case 2: { /* ADAPTIVE_EULER :104-140 */
    double dt_int = 0.0, dt_red = dt;
    const double keep = 1.0 + m->relative_change_min;
    long att = 0;
    int rc = 0;
    while (dt_int < dt) {
      if (m->max_attempts > 0 && att >= m->max_attempts) { rc = -3; break; }
      att++;
      rhs_all(m, conc, bdys, fluxes, w->rhs0, w);
      int reject = 0;
      FOR_ACTIVE(m, {
        c1[i_] = conc[i_] + dt_red * w->rhs0[i_];
        if (c1[i_] - keep * conc[i_] < -m->atol) reject = 1;
      });
      if (reject && dt_red > m->dt_min) {
        dt_red = dt_red * 0.25;
        if (st) st->rejected++;
      } else {
        /* adaptive_solver_diagnostics (:129-136), before conc = c1 */
        if (diag && dt_red < diag->last_min_dt) {
          diag->last_min_dt = dt_red;
          minloc_relative_change(m, conc, c1, diag->inum, diag->last_min_dt_grid_cell);
        }
        FOR_ACTIVE(m, conc[i_] = c1[i_]);
        dt_int = dt_int + dt_red;
        if (st) {
          st->accepted++;
          if (dt_red < st->min_dt) st->min_dt = dt_red;
        }
      }
    }
    if (st) {
      st->attempts += att;
      if (att > st->max_col_attempts) st->max_col_attempts = att;
      if (rc) st->capped++;
    }
    return rc;
  }
  case 1: /* RUNGE_KUTTA_4 :142-163 */
    rhs_all(m, conc, bdys, fluxes, w->rhs0, w);
    FOR_ACTIVE(m, c1[i_] = conc[i_] + 0.5 * dt * w->rhs0[i_]);
    rhs_all(m, c1, bdys, fluxes, w->rhs1, w);
    FOR_ACTIVE(m, c1[i_] = conc[i_] + 0.5 * dt * w->rhs1[i_]);
    rhs_all(m, c1, bdys, fluxes, w->rhs2, w);
    FOR_ACTIVE(m, c1[i_] = conc[i_] + dt * w->rhs2[i_]);
    rhs_all(m, c1, bdys, fluxes, w->rhs3, w);
    FOR_ACTIVE(m, conc[i_] = conc[i_] + dt * third *
                                           (0.5 * w->rhs0[i_] + w->rhs1[i_] +
                                            w->rhs2[i_] + 0.5 * w->rhs3[i_]));
    if (st) { st->attempts += 4; st->accepted++; }
    return 0;
  case 3: /* RUNGE_KUTTA_4_38 :164-185 */
    rhs_all(m, conc, bdys, fluxes, w->rhs0, w);
    FOR_ACTIVE(m, c1[i_] = conc[i_] + third * dt * w->rhs0[i_]);
    rhs_all(m, c1, bdys, fluxes, w->rhs1, w);
    FOR_ACTIVE(m, c1[i_] = conc[i_] + dt * (w->rhs1[i_] - third * w->rhs0[i_]));
    rhs_all(m, c1, bdys, fluxes, w->rhs2, w);
    FOR_ACTIVE(m, c1[i_] = conc[i_] + dt * (w->rhs0[i_] - w->rhs1[i_] + w->rhs2[i_]));
    rhs_all(m, c1, bdys, fluxes, w->rhs3, w);
    FOR_ACTIVE(m, conc[i_] = conc[i_] + dt * 1.0 / 8.0 *
                                           (w->rhs0[i_] + 3.0 * w->rhs1[i_] +
                                            3.0 * w->rhs2[i_] + w->rhs3[i_]));
    if (st) { st->attempts += 4; st->accepted++; }
    return 0;
  default:
    return -1;
  }
}

int orc_ode_solver(const orc_model *m, double *conc, const double *bdys,
                   double *fluxes, double dt, int method, orc_stats *st) {
  ode_ws w;
  ode_ws_alloc(&w, m);
  int rc = ode_solver_ws(m, conc, bdys, fluxes, dt, method, st, &w, NULL);
  ode_ws_free(&w);
  return rc;
}

void orc_diag_init(orc_diag *d, int inum) {
  d->last_min_dt = (double)1.e20f;  /* solver_library.F90:44: a default-real
                                       literal widened to the driver's kind */
  for (int i = 0; i < 4; i++) d->last_min_dt_grid_cell[i] = -99;  /* :45 */
  d->inum = inum;
}

int orc_ode_solver_diag(const orc_model *m, double *conc, const double *bdys,
                        double *fluxes, double dt, orc_diag *d, orc_stats *st) {
  ode_ws w;
  ode_ws_alloc(&w, m);
  int rc = ode_solver_ws(m, conc, bdys, fluxes, dt, 2, st, &w, d);
  ode_ws_free(&w);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Per-column mode: each column is copied into a 1-column model and stepped
 * alone, so its cut sequence depends only on its own cells. */
typedef struct {
  orc_model m1;
  int kact;
  double *dz, *dzc, *phi, *phi_i, *bf, *cap, *conc, *bdys, *fluxes;
  ode_ws w;
} col_ctx;

static void col_ctx_init(col_ctx *c, const orc_model *m) {
  c->m1 = *m;
  c->m1.ncol = 1;
  size_t K = (size_t)m->kmax, N = (size_t)m->ntr;
  c->dz = calloc(K, sizeof(double));
  c->dzc = calloc(K, sizeof(double));
  c->phi = calloc(K, sizeof(double));
  c->phi_i = calloc(K, sizeof(double));
  c->bf = calloc(K, sizeof(double));
  c->cap = calloc(K, sizeof(double));
  c->conc = calloc(N * K, sizeof(double));
  c->bdys = calloc(N + 1, sizeof(double));
  c->fluxes = calloc(N, sizeof(double));
  c->m1.kact = &c->kact;
  c->m1.dz = c->dz;
  c->m1.dzc = c->dzc;
  c->m1.phi = c->phi;
  c->m1.phi_i = c->phi_i;
  c->m1.biofac = c->bf;
  c->m1.flux_cap = c->cap;
  ode_ws_alloc(&c->w, &c->m1);
}

static void col_ctx_free(col_ctx *c) {
  free(c->dz); free(c->dzc); free(c->phi); free(c->phi_i); free(c->bf);
  free(c->cap); free(c->conc); free(c->bdys); free(c->fluxes);
  ode_ws_free(&c->w);
}

static int step_one_column(const orc_model *m, col_ctx *c, int col,
                           double *conc, const double *bdys, double *fluxes,
                           double dt, int method, orc_stats *st) {
  const size_t nc = (size_t)m->ncol;
  const int KM = m->kmax, N = m->ntr, K = m->kact[col];
  if (K <= 0) return 0;
  c->kact = K;
  c->m1.bgc_col = m->bgc_col ? &m->bgc_col[col] : NULL;  /* the column's set */
  for (int k = 0; k < KM; k++) {
    c->dz[k] = m->dz[k * nc + col];
    c->phi[k] = m->phi[k * nc + col];
    c->phi_i[k] = m->phi_i[k * nc + col];
    c->bf[k] = m->biofac[k * nc + col];
    c->cap[k] = m->flux_cap ? m->flux_cap[k * nc + col] : 0.0;
    if (k < KM - 1) c->dzc[k] = m->dzc[k * nc + col];
  }
  for (int n = 0; n < N; n++)
    for (int k = 0; k < KM; k++) c->conc[n * KM + k] = conc[IDX(n, k, col, KM, nc)];
  for (int f = 0; f <= N; f++) c->bdys[f] = bdys[f * nc + col];
  for (int n = 0; n < N; n++) c->fluxes[n] = fluxes[n * nc + col];
  int rc = ode_solver_ws(&c->m1, c->conc, c->bdys, c->fluxes, dt, method, st, &c->w, NULL);
  for (int n = 0; n < N; n++)
    for (int k = 0; k < KM; k++) conc[IDX(n, k, col, KM, nc)] = c->conc[n * KM + k];
  for (int n = 0; n < N; n++) fluxes[n * nc + col] = c->fluxes[n];
  return rc;
}

static void stats_init(orc_stats *s) {
  memset(s, 0, sizeof(*s));
  s->min_dt = 1e300;
}

static void stats_merge(orc_stats *a, const orc_stats *b) {
  a->attempts += b->attempts;
  a->accepted += b->accepted;
  a->rejected += b->rejected;
  if (b->max_col_attempts > a->max_col_attempts) a->max_col_attempts = b->max_col_attempts;
  if (b->min_dt < a->min_dt) a->min_dt = b->min_dt;
  a->capped += b->capped;
  a->nan_cells += b->nan_cells;
}

static int run_percol(const orc_model *m, double *conc, const double *bdys,
                      double *fluxes, double dt, int method, int nsteps,
                      int nthreads, orc_stats *st) {
  int rc_all = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    col_ctx c;
    col_ctx_init(&c, m);
    orc_stats loc;
    stats_init(&loc);
    int rc_loc = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
    for (int col = 0; col < m->ncol; col++) {
      for (int s = 0; s < nsteps; s++) {
        orc_stats cs;
        stats_init(&cs);
        int rc = step_one_column(m, &c, col, conc, bdys, fluxes, dt, method, &cs);
        /* component epilogue on this column (:1718-1732) */
        const size_t nc = (size_t)m->ncol;
        for (int n = 0; n < m->ntr; n++)
          for (int k = 0; k < m->kact[col]; k++) {
            double *v = &conc[IDX(n, k, col, m->kmax, nc)];
            if (*v != *v) cs.nan_cells++;
            else if (m->minimum && *v < m->minimum[n]) *v = m->minimum[n];
          }
        stats_merge(&loc, &cs);
        if (rc && !rc_loc) rc_loc = rc;
        if (rc) break;
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      if (st) stats_merge(st, &loc);
      if (rc_loc && !rc_all) rc_all = rc_loc;
    }
    col_ctx_free(&c);
  }
  return rc_all;
}

int orc_ode_solver_percol(const orc_model *m, double *conc, const double *bdys,
                          double *fluxes, double dt, int method, int nthreads,
                          orc_stats *st) {
  /* one coupling step without the epilogue */
  int rc_all = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    col_ctx c;
    col_ctx_init(&c, m);
    orc_stats loc;
    stats_init(&loc);
    int rc_loc = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
    for (int col = 0; col < m->ncol; col++) {
      int rc = step_one_column(m, &c, col, conc, bdys, fluxes, dt, method, &loc);
      if (rc && !rc_loc) rc_loc = rc;
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      if (st) stats_merge(st, &loc);
      if (rc_loc && !rc_all) rc_all = rc_loc;
    }
    col_ctx_free(&c);
  }
  return rc_all;
}

/* ------------------------------------------------------------------------ */
int orc_epilogue(const orc_model *m, double *conc) {
  int nan = 0;
  FOR_ACTIVE(m, {
    if (conc[i_] != conc[i_]) nan++;
    else if (m->minimum && conc[i_] < m->minimum[n_]) conc[i_] = m->minimum[n_];
  });
  return nan;
}

int orc_run(const orc_model *m, double *conc, const double *bdys,
            double *fluxes, double dt, int method, int percol, int nsteps,
            int nthreads, orc_stats *st) {
  if (st) stats_init(st);
  if (percol) return run_percol(m, conc, bdys, fluxes, dt, method, nsteps, nthreads, st);
  ode_ws w;
  ode_ws_alloc(&w, m);
  int rc = 0;
  for (int s = 0; s < nsteps && rc == 0; s++) {
    rc = ode_solver_ws(m, conc, bdys, fluxes, dt, method, st, &w, NULL);
    int nan = orc_epilogue(m, conc);
    if (st) st->nan_cells += nan;
    if (nan && rc == 0) rc = -2;
  }
  ode_ws_free(&w);
  return rc;
}

/* ------------------------------------------------------------------------ */
void orc_bc_flux_estimate(const orc_model *m, const double *conc,
                          const double *bdys, double *fluxes) {
  const size_t nc = (size_t)m->ncol;
  for (int n = 0; n < m->ntr; n++) {
    if (m->particulate[n]) continue;
    for (size_t col = 0; col < nc; col++) {
      if (m->kact[col] <= 0) continue;
      double T = bdys[col];
      double c0 = conc[IDX(n, 0, col, m->kmax, nc)];
      double cb = bdys[(size_t)(n + 1) * nc + col];
      fluxes[(size_t)n * nc + col] =
          -(c0 - cb) / m->dz[col] *
          (m->bioturbation + m->diffusivity + T * 0.035) * m->phi[col] /
          86400.0 / 10000.0;
    }
  }
}

void orc_assemble_bc(const orc_model *m, const double *conc, const double *temperature,
                     const double *surface, const double *velocity,
                     const int *present, double *bdys, double *fluxes) {
  const size_t nc = (size_t)m->ncol;
  for (size_t col = 0; col < nc; col++) bdys[col] = temperature[col];
  for (int n = 0; n < m->ntr; n++) {
    if (present && !present[n]) continue;
    for (size_t col = 0; col < nc; col++) {
      const size_t i = (size_t)n * nc + col;
      if (m->particulate[n]) {
        fluxes[i] = -surface[i] * velocity[i];
        continue;
      }
      bdys[(size_t)(n + 1) * nc + col] = surface[i];
      if (m->bcup_dissolved == 1 && m->kact[col] > 0) {
        const double T = bdys[col];
        fluxes[i] = -(conc[IDX(n, 0, col, m->kmax, nc)] - bdys[(size_t)(n + 1) * nc + col]) /
                    m->dz[col] * (m->bioturbation + m->diffusivity + T * 0.035) *
                    m->phi[col] / 86400.0 / 10000.0;
      } else {
        fluxes[i] = 0.0;
      }
    }
  }
}

void orc_inventory(const orc_model *m, const double *conc, double *inv) {
  const size_t nc = (size_t)m->ncol;
  for (int n = 0; n < m->ntr; n++)
    for (size_t col = 0; col < nc; col++) {
      double s = 0.0;
      for (int k = 0; k < m->kact[col]; k++)
        s += m->phi[k * nc + col] * m->dz[k * nc + col] *
             conc[IDX(n, k, col, m->kmax, nc)];
      inv[(size_t)n * nc + col] = s;
    }
}
