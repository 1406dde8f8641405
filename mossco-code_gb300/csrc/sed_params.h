// sed_params.h -- conversion of the C ABI's sed_params into the kernels'
// Params (rates per second, precision-specific constants) and the cut-level
// clock of the adaptive loop for a given coupling step.
#pragma once

#include <cmath>

#include "../../include/mossco_sed.h"
#include "sed_device.cuh"

namespace sed {

template <typename real>
inline Params<real> make_params(const sed_params& s) {
  Params<real> p{};
  const double spd = 86400.0;
  p.rF = (real)(s.rLabile / spd);
  p.rS = (real)(s.rSemilabile / spd);
  p.cmax = (real)(s.CprodMax / spd);
  p.rnit = (real)(s.rnit / spd);
  p.rodu = (real)(s.rODUox / spd);
  p.pads = (real)(s.PAds / spd);
  p.ksO2oxic = (real)s.ksO2oxic;
  p.kinO2denit = (real)s.kinO2denit;
  p.ksNO3denit = (real)s.ksNO3denit;
  p.kinO2anox = (real)s.kinO2anox;
  p.kinNO3anox = (real)s.kinNO3anox;
  p.ksO2nitri = (real)s.ksO2nitri;
  p.ksO2oduox = (real)s.ksO2oduox;
  p.PAdsODU = (real)s.PAdsODU;
  p.nh3fac = (real)(1.0 / (1.0 + s.NH3Ads));
  p.nh3den = (real)(1.0 + s.NH3Ads);
  p.mol_mode = s.mol_diff_mode;
  p.keep = (real)(1.0 + s.relative_change_min);
  p.natol = (real)(-s.atol);
  for (int n = 0; n < NTR; n++) p.minimum[n] = (real)s.minimum[n];
  p.dt_min = s.dt_min;
  p.bcup_d = s.bcup_dissolved;
  p.max_attempts = s.max_attempts;
  p.epilogue = s.epilogue;
  p.budgets = s.budgets;
  p.bio3 = s.bioturbation_profile == 3;
  p.toc_f1 = (real)(1.0 / 1.2 * 12.01 / s.bioturb_dry_density / 1000.0);
  p.toc_f2 = (real)(1.0 / 6.0 * 12.01 / s.bioturb_dry_density / 1000.0);
  p.bio_beta = (real)s.bioturb_beta;
  p.bio_b = (real)s.bioturb_b;
  p.bio_L1 = (real)s.bioturb_L1;
  p.bio_L2 = (real)s.bioturb_L2;
  return p;
}

// Cut levels of the adaptive loop for a coupling step dt: mstop is the
// first m with dt/4^m <= dt_min (cuts stop there, solver_library.F90:126).
// The partial sums dt_int = sum dt/4^m are then multiples of dt/4^mstop; if
// dt's significand has b bits and b + 2 mstop <= 53 every one of them is
// exact in FP64, so integer ticks take the reference's decisions exactly.
template <typename real>
inline void set_clock(Params<real>& p, double dt, double dt_min) {
  int mstop = 0;
  double d = dt;
  while (!(d <= dt_min) && mstop < 64) { d *= 0.25; mstop++; }
  int e = 0;
  const double mant = std::frexp(dt, &e);
  unsigned long long sig = (unsigned long long)std::ldexp(mant, 53);
  int tz = 0;
  while (sig && !(sig & 1ull)) { sig >>= 1; tz++; }
  const int bits = 53 - tz;
  p.mstop = mstop;
  p.ticks = (mstop <= 31 && bits + 2 * mstop <= 53) ? 1 : 0;
}

}  // namespace sed
