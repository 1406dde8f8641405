/*
 * cpl_oracle.c -- FP64 CPU oracle of MOSSCO's pelagic_soil_connector Run.
 *
 * TEST INFRASTRUCTURE ONLY.  Imported by tests/ (through pel_oracle.py) to
 * check the device coupling; the product never links it.
 *
 * Restates src/mediators/pelagic_soil_connector.F90 Run (:176-2122) for 3-D
 * pelagic fields and 2-D soil fields, statement by statement and in the
 * Run's order: each whole-array Fortran assignment is one loop over the
 * columns, and a field the Run writes twice is written twice here.  The ESMF
 * lookups by name become the pelagic tracer indices of orc_cpl_fields; the
 * bottom layer is k = 0 (the Run's lbnd(3)).  Literals without a kind
 * suffix are default (single-precision) reals in the reference and appear
 * here as float constants widened to double.
 *
 * Soil tracer rows (the sediment's OMEXDIA+P order): 0 labile C, 1
 * semilabile C, 2 labile N, 3 semilabile N, 4 labile P, 5 adsorbed P, 6 O2,
 * 7 NO3, 8 NH4, 9 ODU, 10 PO4.
 *
 * Parity: PINNED only to the reference's source text; the connector has no
 * test and no example output in the reference tree.
 */
#include "cpl_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { LC = 0, SC = 1, LN = 2, SN = 3, LP = 4, OX = 6, NI = 7, AM = 8, OD = 9, PH = 10 };

/* Every column is independent: large grids split each whole-array loop over
 * the host threads (elementwise, so the result does not depend on them). */
#ifdef _OPENMP
#define PFOR _Pragma("omp parallel for schedule(static) if(ncol > 65536)")
#else
#define PFOR
#endif

void orc_cpl_defaults(orc_cpl *p) {
  /* :38-45 */
  p->sinking_factor = 0.3;
  p->NC_ldet = 0.23;
  p->NC_sdet = 0.01;
  p->convertN = 1.0;
  p->convertP = 1.0;
  p->sinking_factor_min = (double)0.02f;
  p->half_sedimentation_depth = (double)0.1f;
  p->half_sedimentation_tke = 1.0e3;
  p->critical_detritus = 60.0;
  p->as_named = 0;
}

/* bottom-layer value of pelagic tracer n in column i */
static double bot(const double *conc, int n, int ncol, int knum, int i) {
  return conc[(size_t)n * knum * ncol + i];
}

int orc_cpl_run(const orc_cpl *p, const orc_cpl_fields *f, const double *conc,
                int ncol, int knum, const double *depth, const double *tke,
                double *surface, double *velocity, int *present) {
  const double one_e5 = (double)1e-5f, one_e3 = (double)1e-3f, nine_e9 = (double)9e9f;
  double *CN = malloc(sizeof(double) * ncol), *fl = malloc(sizeof(double) * ncol),
         *rl = malloc(sizeof(double) * ncol), *fs = malloc(sizeof(double) * ncol),
         *rs = malloc(sizeof(double) * ncol), *fe = malloc(sizeof(double) * ncol),
         *din = malloc(sizeof(double) * ncol);
  int i, n;
  for (n = 0; n < 11; n++) present[n] = 0;
#define ROW(a, r) ((a) + (size_t)(r) * ncol)
#define B(fld) bot(conc, (fld), ncol, knum, i)

  /* oxygen and its deficit, :801-866 (both found / deficit only / oxygen
   * only; the oxygen-only branch of the reference reads the deficit's
   * pointers, which are not associated then: here oxygen alone is copied) */
  if (f->oxygen >= 0 && f->odu >= 0) {
    PFOR
    for (i = 0; i < ncol; i++) ROW(surface, OX)[i] = B(f->oxygen);
    PFOR
    for (i = 0; i < ncol; i++) ROW(surface, OD)[i] = B(f->odu);
    present[OX] = present[OD] = 1;
  } else if (f->odu >= 0) {
    PFOR
    for (i = 0; i < ncol; i++) {
      const double x = -B(f->odu);
      ROW(surface, OX)[i] = x > 0.0 ? x : 0.0;
    }
    PFOR
    for (i = 0; i < ncol; i++) {
      const double x = B(f->odu);
      ROW(surface, OD)[i] = x > 0.0 ? x : 0.0;
    }
    present[OX] = present[OD] = 1;
  } else if (f->oxygen >= 0) {
    PFOR
    for (i = 0; i < ncol; i++) ROW(surface, OX)[i] = B(f->oxygen);
    present[OX] = 1;
  }

  /* C:N of the detritus, :1018-1072 */
  PFOR
  for (i = 0; i < ncol; i++) CN[i] = 106.0 / 16.0;
  if (f->detN >= 0 && f->detC >= 0)
    PFOR
    for (i = 0; i < ncol; i++) CN[i] = B(f->detC) / (one_e5 + B(f->detN));

  /* labile / semilabile factors, :1074-1121 */
  PFOR
  for (i = 0; i < ncol; i++) fl[i] = (1.0 - p->NC_sdet * CN[i]) / (p->NC_ldet - p->NC_sdet);
  PFOR
  for (i = 0; i < ncol; i++) rl[i] = fl[i] * p->NC_ldet;
  PFOR
  for (i = 0; i < ncol; i++)
    if (fl[i] > CN[i]) { fl[i] = CN[i]; rl[i] = 1.0; }
  PFOR
  for (i = 0; i < ncol; i++)
    if (fl[i] < 0.0) { fl[i] = 0.0; rl[i] = 0.0; }
  PFOR
  for (i = 0; i < ncol; i++) fs[i] = CN[i] - fl[i];
  PFOR
  for (i = 0; i < ncol; i++) rs[i] = 1.0 - rl[i];
  PFOR
  for (i = 0; i < ncol; i++) fe[i] = 1.0;

  /* water depth, :1126-1160 */
  if (depth && p->half_sedimentation_depth > one_e3)
    PFOR
    for (i = 0; i < ncol; i++)
      fe[i] = fe[i] * (depth[i] * depth[i]) /
              (depth[i] * depth[i] + p->half_sedimentation_depth * p->half_sedimentation_depth);
  /* turbulence, :1164-1198 */
  if (tke && p->half_sedimentation_tke < nine_e9)
    PFOR
    for (i = 0; i < ncol; i++)
      fe[i] = fe[i] * p->half_sedimentation_tke / (tke[i] + p->half_sedimentation_tke);
  /* minimum sedimentation, :1202-1210 */
  PFOR
  for (i = 0; i < ncol; i++) fe[i] = fe[i] + p->sinking_factor_min / p->sinking_factor;
  /* detritus carbon above critical_detritus, :1213-1236 */
  if (f->detC >= 0 && p->critical_detritus > one_e3 && p->critical_detritus < nine_e9)
    PFOR
    for (i = 0; i < ncol; i++) {
      const double x = B(f->detC) / p->critical_detritus;
      const double x2 = x * x;
      fe[i] = fe[i] * 1.0 / (1.0 + x2 * x2);
    }

  /* labile carbon, semilabile carbon, labile nitrogen, semilabile nitrogen,
   * :1243-1490: the concentration, then the velocity formula into
   * fieldList(1) again (the concentration: the Run as written) or into the
   * z-velocity field (as_named) */
  if (f->detN >= 0) {
    const double *fac[4] = {fl, fs, rl, rs};
    const int row[4] = {LC, SC, LN, SN};
    int b;
    for (b = 0; b < 4; b++) {
      double *dst = ROW(surface, row[b]);
      PFOR
      for (i = 0; i < ncol; i++) dst[i] = fac[b][i] * p->convertN * B(f->detN);
      dst = p->as_named ? ROW(velocity, row[b]) : ROW(surface, row[b]);
      PFOR
      for (i = 0; i < ncol; i++) dst[i] = p->sinking_factor * fe[i] * B(f->detN);
      present[row[b]] = 1;
    }
  }
  /* phosphorus, :1492-1646 */
  if (f->detN >= 0) {
    PFOR
    for (i = 0; i < ncol; i++) ROW(surface, LP)[i] = 1.0 / 16.0 * p->convertN * B(f->detN);
    present[LP] = 1;
  }
  if (f->detP >= 0) {
    PFOR
    for (i = 0; i < ncol; i++) ROW(surface, LP)[i] = B(f->detP);
    present[LP] = 1;
  }
  if (f->detN >= 0)
    PFOR
    for (i = 0; i < ncol; i++)
      ROW(velocity, LP)[i] = p->sinking_factor * fe[i] * B(f->detN);

  /* ammonium, :1685-1860 */
  {
    const int hN = f->nitrate >= 0, hA = f->ammonium >= 0, hD = f->din >= 0;
    if (!hN && !hA && !hD) {
      free(CN); free(fl); free(rl); free(fs); free(rs); free(fe); free(din);
      return -1;
    }
    PFOR
    for (i = 0; i < ncol; i++) {
      double v;
      if (hA) v = p->convertN * B(f->ammonium);
      else if (hD && hN) v = p->convertN * (B(f->din) - B(f->nitrate));
      else if (hD) v = p->convertN * 0.5 * B(f->din);
      else v = p->convertN * B(f->nitrate);
      ROW(surface, AM)[i] = v;
    }
    /* nitrate, :1863-1935: the block looks the nitrate field up (:1863)
     * but writes through fieldList(1) (rank 1, :1872) or farrayPtr2 (rank
     * 2, :1924), both still the ammonium field of :1766-1806; so the Run
     * as written overwrites ammonium and leaves the nitrate field alone */
    {
      double *dst = p->as_named ? ROW(surface, NI) : ROW(surface, AM);
      PFOR
      for (i = 0; i < ncol; i++) {
        double v;
        if (hN) v = p->convertN * B(f->nitrate);
        else if (hA && hD) v = p->convertN * (B(f->din) - B(f->ammonium));
        else if (hD) v = p->convertN * 0.5 * B(f->din);
        else v = p->convertN * B(f->ammonium);
        dst[i] = v;
      }
    }
    /* phosphate from DIN (a DIP field is overwritten, not read), :1988-2110 */
    PFOR
    for (i = 0; i < ncol; i++) {
      if (hD) din[i] = B(f->din);
      else if (hA && hN) din[i] = B(f->nitrate) + B(f->ammonium);
      else if (hA) din[i] = 2 * B(f->ammonium);
      else din[i] = 2 * B(f->nitrate);
    }
    PFOR
    for (i = 0; i < ncol; i++) {
      const double dip = 1.0 / 16.0 * p->convertN * din[i];
      ROW(surface, PH)[i] = p->convertP * dip;
    }
    present[AM] = present[PH] = 1;
    if (p->as_named) present[NI] = 1;
  }
#undef B
#undef ROW
  free(CN); free(fl); free(rl); free(fs); free(rs); free(fe); free(din);
  return 0;
}

/* ---- soil_pelagic_connector (src/mediators/soil_pelagic_connector.F90) */

void orc_cpl_soil_defaults(orc_cpl_soil *p) {
  /* :36-41; 0.0 and -1. are default-real literals */
  p->dinflux_const = (double)0.0f;
  p->dipflux_const = (double)-1.0f;
  p->NC_ldet = 0.20;
  p->NC_sdet = 0.04;
  p->convertP = 1.0;
  p->convertN = 1.0;
}

/* the soil's export names (the pelagic_soil_connector's own searches use
 * them: :1243-1493, :1768, :1864, :2088, :740, :768) */
static const char *const soil_names[11] = {
    "detritus_labile_carbon",        "detritus_semilabile_carbon",
    "detritus_labile_nitrogen",      "detritus_semilabile_nitrogen",
    "detritus_labile_phosphorus",    "adsorbed_phosphorus",
    "dissolved_oxygen",              "mole_concentration_of_nitrate",
    "mole_concentration_of_ammonium", "dissolved_reduced_substances",
    "mole_concentration_of_phosphate"};

/* MOSSCO_StringMatchPattern (mossco_strings.F90:331-396) for a pattern
 * with one inner asterisk: only the part after the asterisk is compared,
 * as the end of the item */
static int match_after_star(const char *item, const char *pattern) {
  const char *star = strchr(pattern, '*');
  size_t li = strlen(item), ls;
  if (!star) return strcmp(item, pattern) == 0;
  star++;
  ls = strlen(star);
  return li >= ls && strcmp(item + li - ls, star) == 0;
}

static int by_name(const void *a, const void *b) {
  return strcmp(soil_names[*(const int *)a], soil_names[*(const int *)b]);
}

/* zero, then += every soil upward flux whose name the pattern matches, in
 * ESMF's alphabetical item order (:776-805, :846-875, :915-944) */
static void detritus_sum(const char *pattern, const double *fluxes, int ncol, double *dst) {
  int order[11], i, n;
  char item[96];
  for (n = 0; n < 11; n++) order[n] = n;
  qsort(order, 11, sizeof(int), by_name);
  PFOR
  for (i = 0; i < ncol; i++) dst[i] = 0.0;
  for (n = 0; n < 11; n++) {
    snprintf(item, sizeof item, "%s_upward_flux_at_soil_surface", soil_names[order[n]]);
    if (!match_after_star(item, pattern)) continue;
    PFOR
    for (i = 0; i < ncol; i++) dst[i] = dst[i] + -fluxes[(size_t)order[n] * ncol + i];
  }
}

void orc_cpl_soil_run(const orc_cpl_soil *p, const orc_cpl_soil_fields *f,
                      const double *fluxes, int ncol, int ntr, double *bfl, int *present) {
  /* the soil's export: upward flux = -fluxes(:,:,n) (fabm_sediment_component
   * .F90:1808-1815) */
  double *up = malloc(sizeof(double) * 11 * (size_t)ncol);
  const double year = (double)(86400.0f * 365.0f);
  int i, n;
  for (n = 0; n < 11 * ncol; n++) up[n] = -fluxes[n];
  for (n = 0; n < ntr; n++) present[n] = 0;
#define UP(r) (up + (size_t)(r) * ncol)
#define ROW(r) (bfl + (size_t)(r) * ncol)
  if (f->nitrate >= 0) {  /* :352-356 */
    PFOR
    for (i = 0; i < ncol; i++) ROW(f->nitrate)[i] = UP(NI)[i];
    present[f->nitrate] = 1;
  }
  if (f->ammonium >= 0) {  /* :408-412 */
    PFOR
    for (i = 0; i < ncol; i++) ROW(f->ammonium)[i] = p->convertN * UP(AM)[i];
    present[f->ammonium] = 1;
  }
  if (f->din >= 0) {  /* :467-473 */
    PFOR
    for (i = 0; i < ncol; i++)
      ROW(f->din)[i] = (UP(AM)[i] + UP(NI)[i] + p->dinflux_const / year) * p->convertN;
    present[f->din] = 1;
  }
  if (f->dip >= 0) {  /* :528-534 */
    PFOR
    for (i = 0; i < ncol; i++)
      ROW(f->dip)[i] = p->convertP * (UP(PH)[i] + p->dipflux_const / year);
    present[f->dip] = 1;
  }
  if (f->odu >= 0 && f->oxygen >= 0) {  /* :643-667 */
    PFOR
    for (i = 0; i < ncol; i++) ROW(f->odu)[i] = UP(OD)[i];
    PFOR
    for (i = 0; i < ncol; i++) ROW(f->oxygen)[i] = UP(OX)[i];
    present[f->odu] = present[f->oxygen] = 1;
  } else if (f->odu >= 0) {
    PFOR
    for (i = 0; i < ncol; i++) ROW(f->odu)[i] = UP(OD)[i] - UP(OX)[i];
    present[f->odu] = 1;
  } else if (f->oxygen >= 0) {
    PFOR
    for (i = 0; i < ncol; i++) ROW(f->oxygen)[i] = UP(OX)[i] - UP(OD)[i];
    present[f->oxygen] = 1;
  }
  if (f->detN >= 0) {
    detritus_sum("detritus*nitrogen_upward_flux_at_soil_surface", fluxes, ncol, ROW(f->detN));
    present[f->detN] = 1;
  }
  if (f->detC >= 0) {
    detritus_sum("detritus*carbon_upward_flux_at_soil_surface", fluxes, ncol, ROW(f->detC));
    present[f->detC] = 1;
  }
  if (f->detP >= 0) {
    detritus_sum("detritus*phosphorous_upward_flux_at_soil_surface", fluxes, ncol, ROW(f->detP));
    present[f->detP] = 1;
  }
#undef UP
#undef ROW
  free(up);
}
