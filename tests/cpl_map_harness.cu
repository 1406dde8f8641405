// cpl_map_harness.cu -- runs the coupling kernels' per-column arithmetic
// (mossco-code_gb300/csrc/cpl_map.cuh, the source the kernels call) on the
// host, so that tests/test_coupling.py can check it bit for bit against the
// connector oracles without a GPU.  Built by that test with nvcc; reads its
// cases from stdin and writes hex floats to stdout.
//
// Forward case:  F, then the nine cpl_params doubles and the mode, the nine
// cpl_fields ints, has_depth has_tke ncol, then per column the four
// bottom-layer values, the depth and the turbulence.  Output per column:
// the eleven surface values, the rows written, the velocity value and its
// rows.
// Reverse case:  R, then the six cpl_soil_params doubles, the nine
// cpl_fields ints, ncol, then per column the eleven sediment fluxes and
// the four bottom fluxes before the Run.  Output per column: the four
// bottom fluxes after it.
#include <cstdio>

#include "cpl_map.cuh"

using namespace cplmap;

struct Bottom {
  const double* b;
  CPL_HD double operator()(int n) const { return b[n]; }
};
struct Up {
  const double* fl;
  CPL_HD double operator()(int n) const { return -fl[n]; }
};
struct Put {
  double* out;
  CPL_HD void operator()(int row, double v) const { out[row] = v; }
};

static int read_fields(cpl_fields* f) {
  return scanf("%d %d %d %d %d %d %d %d %d", &f->detN, &f->detC, &f->detP, &f->din,
               &f->nitrate, &f->ammonium, &f->oxygen, &f->odu, &f->dip) == 9;
}

static int forward() {
  cpl_params p;
  cpl_fields f;
  int hd, ht, ncol;
  if (scanf("%lf %lf %lf %lf %lf %lf %lf %lf %lf %d", &p.sinking_factor,
            &p.sinking_factor_min, &p.NC_ldet, &p.NC_sdet, &p.convertN, &p.convertP,
            &p.half_sedimentation_depth, &p.half_sedimentation_tke, &p.critical_detritus,
            &p.mode) != 10 || !read_fields(&f) || scanf("%d %d %d", &hd, &ht, &ncol) != 3)
    return 1;
  const Forward a = make_forward(&p, &f, hd != 0, ht != 0);
  for (int c = 0; c < ncol; c++) {
    double b[4], depth, tke;
    if (scanf("%lf %lf %lf %lf %lf %lf", &b[0], &b[1], &b[2], &b[3], &depth, &tke) != 6)
      return 1;
    const ForwardOut o = pelagic_soil_column(a, Bottom{b}, depth, tke);
    for (int n = 0; n < NTR; n++) printf("%a ", o.S[n]);
    printf("%u %a %u\n", o.srows, o.w, o.vrows);
  }
  return 0;
}

static int reverse() {
  cpl_soil_params p;
  cpl_fields f;
  int ncol;
  if (scanf("%lf %lf %lf %lf %lf %lf", &p.dinflux_const, &p.dipflux_const, &p.NC_ldet,
            &p.NC_sdet, &p.convertN, &p.convertP) != 6 || !read_fields(&f) ||
      scanf("%d", &ncol) != 1)
    return 1;
  const Reverse a = make_reverse(&p, &f);
  for (int c = 0; c < ncol; c++) {
    double fl[NTR], out[PEL_NTR];
    for (int n = 0; n < NTR; n++)
      if (scanf("%lf", &fl[n]) != 1) return 1;
    for (int n = 0; n < PEL_NTR; n++)
      if (scanf("%lf", &out[n]) != 1) return 1;
    soil_pelagic_column(a, Up{fl}, Put{out});
    for (int n = 0; n < PEL_NTR; n++) printf("%a ", out[n]);
    printf("\n");
  }
  return 0;
}

int main() {
  char kind[4];
  int rc = 0;
  while (rc == 0 && scanf("%3s", kind) == 1) rc = kind[0] == 'F' ? forward() : reverse();
  return rc;
}
