// cpl_map.cuh -- the per-column arithmetic of the two MOSSCO connectors,
// shared by the coupling kernels (cpl_capi.cu) and a host-compiled check of
// the same source.  Host and device evaluate it in IEEE double without
// contraction (-fmad=false on the device, -ffp-contract=off on the host), so
// both give the same bits.
#pragma once

#include "../../include/mossco_cpl.h"

#ifdef __CUDACC__
#define CPL_HD __host__ __device__
#else
#define CPL_HD
#endif

namespace cplmap {

constexpr int NTR = SED_NTR;
constexpr int NPART = 6;  // particulate tracers lead the sediment's order
// sediment tracer rows (sed_tracer_name)
constexpr int kLabC = 0, kSemC = 1, kLabN = 2, kSemN = 3, kLabP = 4, kOxy = 6, kNit = 7,
              kAmm = 8, kOdu = 9, kPho = 10;

// pelagic_soil_connector: per-launch constants formed on the host in IEEE
// double with the operations and rounding the Fortran expressions give them
struct Forward {
  int detN, detC, detP, din, nit, amm, oxy, odu;
  double sf, ncl, ncs, cN, cP, htke, crit;
  double hsd2;      // half_sedimentation_depth**2
  double sfmin_sf;  // sinking_factor_min/sinking_factor
  double c16N;      // 1.0d0/16.0d0 * convertN
  double c05N;      // convertN*0.5d0
  int as_named;
  int crit_on;      // detC present and 1e-3 < critical_detritus < 9e9
  int use_depth;    // water depth given and half_sedimentation_depth > 1e-3
  int use_tke;      // turbulence given and half_sedimentation_tke < 9e9
};

inline Forward make_forward(const cpl_params* p, const cpl_fields* f, bool depth, bool tke) {
  Forward a{};
  a.detN = f->detN; a.detC = f->detC; a.detP = f->detP; a.din = f->din;
  a.nit = f->nitrate; a.amm = f->ammonium; a.oxy = f->oxygen; a.odu = f->odu;
  a.sf = p->sinking_factor;
  a.ncl = p->NC_ldet; a.ncs = p->NC_sdet; a.cN = p->convertN; a.cP = p->convertP;
  a.htke = p->half_sedimentation_tke;
  a.crit = p->critical_detritus;
  a.hsd2 = p->half_sedimentation_depth * p->half_sedimentation_depth;
  a.sfmin_sf = p->sinking_factor_min / p->sinking_factor;
  a.c16N = 1.0 / 16.0 * p->convertN;
  a.c05N = p->convertN * 0.5;
  a.as_named = p->mode == CPL_AS_NAMED;
  // the Run's guards on the namelist values (:1150, :1181, :1215), with its
  // default-real literals
  a.crit_on = f->detC >= 0 && p->critical_detritus > (double)1e-3f &&
              p->critical_detritus < (double)9e9f;
  a.use_depth = depth && p->half_sedimentation_depth > (double)1e-3f;
  a.use_tke = tke && p->half_sedimentation_tke < (double)9e9f;
  return a;
}

// rows of the soil's fields one column's Run writes
struct ForwardOut {
  double S[NTR];     // *_at_soil_surface; rows the Run does not write are 0
  unsigned srows;    // the rows of S the Run writes
  double w;          // the velocity value written
  unsigned vrows;    // *_z_velocity_at_soil_surface rows that take w
};

// Fortran max(0.0, x) of the connector's oxygen split (:823-844)
CPL_HD inline double pos(double x) { return x > 0.0 ? x : 0.0; }

// One column of pelagic_soil_connector's Run (:648-2110; 3-D pelagic, 2-D
// soil fields).  B(n) is the bottom-layer value of pelagic tracer n.
template <class Bottom>
CPL_HD inline ForwardOut pelagic_soil_column(const Forward& a, Bottom B, double depth,
                                             double tke) {
  ForwardOut o;
  for (int n = 0; n < NTR; n++) o.S[n] = 0.0;
  o.srows = 0u;
  o.w = 0.0;
  o.vrows = 0u;
  // ---- detritus (:1018-1236 factors, :1243-1646 fields)
  if (a.detN >= 0 || a.detP >= 0) {
    double fenv = 1.0;
    if (a.use_depth) {  // 1.0 * d**2 is d**2 exactly
      const double d2 = depth * depth;
      fenv = d2 / (d2 + a.hsd2);
    }
    if (a.use_tke) fenv = fenv * a.htke / (tke + a.htke);
    fenv = fenv + a.sfmin_sf;
    if (a.crit_on) {
      const double t = B(a.detC) / a.crit;
      const double t2 = t * t;
      fenv = fenv * 1.0 / (1.0 + t2 * t2);
    }
    const double w = a.sf * fenv;
    if (a.detN >= 0) {
      const double N = B(a.detN);
      o.w = w * N;
      if (a.as_named) {
        double CN = 106.0 / 16.0;
        if (a.detC >= 0) CN = B(a.detC) / ((double)1e-5f + N);
        double fl = (1.0 - a.ncs * CN) / (a.ncl - a.ncs);
        double rl = fl * a.ncl;
        if (fl > CN) { fl = CN; rl = 1.0; }
        if (fl < 0.0) { fl = 0.0; rl = 0.0; }
        const double fs = CN - fl;
        const double rs = 1.0 - rl;
        o.S[kLabC] = fl * a.cN * N;
        o.S[kSemC] = fs * a.cN * N;
        o.S[kLabN] = rl * a.cN * N;
        o.S[kSemN] = rs * a.cN * N;
        o.vrows = (1u << kLabC) | (1u << kSemC) | (1u << kLabN) | (1u << kSemN);
      } else {
        // the velocity formula written into fieldList(1) again: the
        // concentration fields (:1264-1273 and the blocks after it)
        for (int n = kLabC; n <= kSemN; n++) o.S[n] = o.w;
      }
      o.S[kLabP] = a.c16N * N;
      o.vrows |= 1u << kLabP;
      o.srows |= (1u << kLabC) | (1u << kSemC) | (1u << kLabN) | (1u << kSemN) | (1u << kLabP);
    }
    if (a.detP >= 0) {
      o.S[kLabP] = B(a.detP);
      o.srows |= 1u << kLabP;
    }
  }
  // ---- oxygen and its deficit (:801-866)
  if (a.oxy >= 0 && a.odu >= 0) {
    o.S[kOxy] = B(a.oxy);
    o.S[kOdu] = B(a.odu);
    o.srows |= (1u << kOxy) | (1u << kOdu);
  } else if (a.odu >= 0) {
    const double x = B(a.odu);
    o.S[kOxy] = pos(-x);
    o.S[kOdu] = pos(x);
    o.srows |= (1u << kOxy) | (1u << kOdu);
  } else if (a.oxy >= 0) {  // the reference's branch reads unassociated pointers
    o.S[kOxy] = B(a.oxy);
    o.srows |= 1u << kOxy;
  }
  // ---- dissolved nitrogen (:1743-1935) and phosphate (:1988-2110)
  const bool hN = a.nit >= 0, hA = a.amm >= 0, hD = a.din >= 0;
  const double Nt = hN ? B(a.nit) : 0.0;
  const double A = hA ? B(a.amm) : 0.0;
  const double D = hD ? B(a.din) : 0.0;
  const double amm = hA ? a.cN * A
                   : (hD && hN) ? a.cN * (D - Nt)
                   : hD ? a.c05N * D
                   : a.cN * Nt;
  const double nit = hN ? a.cN * Nt
                   : (hA && hD) ? a.cN * (D - A)
                   : hD ? a.c05N * D
                   : a.cN * A;
  if (a.as_named) {
    o.S[kAmm] = amm;
    o.S[kNit] = nit;
    o.srows |= (1u << kAmm) | (1u << kNit);
  } else {
    // the nitrate block writes through the ammonium field's pointer
    // (fieldList(1) / farrayPtr2 of :1766-1806, :1872, :1924): ammonium
    // ends up with the nitrate value and the nitrate field is not written
    o.S[kAmm] = nit;
    o.srows |= 1u << kAmm;
  }
  const double din = hD ? D : (hA && hN) ? Nt + A : hA ? 2 * A : 2 * Nt;
  o.S[kPho] = a.cP * (a.c16N * din);
  o.srows |= 1u << kPho;
  return o;
}

// The rows the forward Run writes: the same in every column, read from one
// column of ones.
struct Ones {
  CPL_HD double operator()(int) const { return 1.0; }
};
inline unsigned forward_rows(const Forward& a) {
  return pelagic_soil_column(a, Ones{}, 1.0, 1.0).srows;
}

// soil_pelagic_connector (:179-965): per-launch constants and the rows of
// the pelagic bottom fluxes it writes
struct Reverse {
  int nit, amm, din, dip, oxy, odu, detN, detC, detP;  // pelagic rows, -1 absent
  double cN, cP;
  double dinc, dipc;  // dinflux_const/(86400.0*365.0), dipflux_const/(...)
};

inline Reverse make_reverse(const cpl_soil_params* p, const cpl_fields* f) {
  Reverse a{};
  a.nit = f->nitrate; a.amm = f->ammonium; a.din = f->din; a.dip = f->dip;
  a.oxy = f->oxygen; a.odu = f->odu; a.detN = f->detN; a.detC = f->detC; a.detP = f->detP;
  a.cN = p->convertN;
  a.cP = p->convertP;
  // (86400.0*365.0) is a default-real product, 31536000 exactly
  const double year = (double)(86400.0f * 365.0f);
  a.dinc = p->dinflux_const / year;
  a.dipc = p->dipflux_const / year;
  return a;
}

// One column of the reverse Run.  U(n) is the soil's upward flux of its
// tracer n, -fluxes(:,:,n) (fabm_sediment_component.F90:1808-1815); W(row,
// v) writes the pelagic bottom-flux row.  Each flux is read only when a
// field that needs it is present.
template <class Up, class Write>
CPL_HD inline void soil_pelagic_column(const Reverse& a, Up U, Write W) {
  if (a.nit >= 0) W(a.nit, U(kNit));                               // :352-356
  if (a.amm >= 0) W(a.amm, a.cN * U(kAmm));                        // :408-412
  if (a.din >= 0) W(a.din, (U(kAmm) + U(kNit) + a.dinc) * a.cN);   // :467-473
  if (a.dip >= 0) W(a.dip, a.cP * (U(kPho) + a.dipc));             // :528-534
  if (a.odu >= 0 && a.oxy >= 0) {                                  // :643-667
    W(a.odu, U(kOdu));
    W(a.oxy, U(kOxy));
  } else if (a.odu >= 0) {
    W(a.odu, U(kOdu) - U(kOxy));
  } else if (a.oxy >= 0) {
    W(a.oxy, U(kOxy) - U(kOdu));
  }
  // detritus: zero, then every soil flux the Run's pattern matches, in
  // ESMF's alphabetical item order (:734-960); 'detritus*phosphorous'
  // matches none of the soil's names
  if (a.detN >= 0) W(a.detN, 0.0 + U(kLabN) + U(kSemN));
  if (a.detC >= 0) W(a.detC, 0.0 + U(kLabC) + U(kSemC));
  if (a.detP >= 0) W(a.detP, 0.0);
}

}  // namespace cplmap
