// sed_device.cuh -- device-side building blocks of the sediment-column solver.
//
// One warp owns one sediment column: lane l holds layers l and (for LPL=2)
// l+32 of all 11 tracers in registers, so a right-hand side evaluation is
// local arithmetic plus two warp shuffles per tracer for the interface
// fluxes, and the adaptive step decision is one warp vote.
//
// Reference semantics followed here (paths inside platipodium/mossco-code):
//   get_rhs   src/drivers/fabm_sediment_driver.F90:575-717
//   diff3d    src/drivers/fabm_sediment_driver.F90:739-825
//   ode_solver src/utilities/solver_library.F90:80-189
//   epilogue  src/components/fabm_sediment_component.F90:1715-1732
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace sed {

constexpr int NTR = 11;    // tracers
constexpr int NPART = 6;   // tracers 0..5 are particulate
constexpr int NDISS = 5;   // tracers 6..10 are dissolved
constexpr int NCOEF = 4;   // FP32 per-layer coefficient rows: phi, vol, gb, gm
constexpr int NCOEF64 = 6; // FP64 rows: phi, phi_i, biofac, dz, len, mol
constexpr int NFORCE = 13; // per-column forcing rows: bioT, dmul, bnd[11]
constexpr int SURF_ROW = 12; // premultiplied surface row: NTR reals, padded to 8 bytes
constexpr unsigned FULL = 0xffffffffu;

enum : int { ST_NAN = 1, ST_CAP = 2, ST_ARG = 4 };

// Tracer indices
enum : int {
  T_FDETC = 0, T_SDETC, T_FDETN, T_SDETN, T_FDETP, T_ADSP,
  T_O2, T_NO3, T_NH4, T_ODU, T_PO4
};

// Coefficient rows staged per layer: the FP32 kernels use folded
// conductances, the FP64 kernels the reference's own per-cell arrays so
// that they evaluate get_rhs in its exact operation order.
// Bioturbation profile 3 adds rows: FP32 the depth term and the averaging
// weight (the bioturbation row then holds the conductance per unit factor);
// FP64 exp(zc 100 k_l), exp(zc 200 k_l) and the column's cumdepth.
constexpr int NCOEF_BIO3 = NCOEF + 2;
constexpr int NCOEF64_BIO3 = NCOEF64 + 3;
template <typename real>
__host__ __device__ constexpr int coef_rows(bool bio3) {
  return sizeof(real) == 8 ? (bio3 ? NCOEF64_BIO3 : NCOEF64) : (bio3 ? NCOEF_BIO3 : NCOEF);
}

// Reaction and solver constants in kernel units (rates per second).
template <typename real>
struct Params {
  real rF, rS, cmax, rnit, rodu, pads;
  real ksO2oxic, kinO2denit, ksNO3denit, kinO2anox, kinNO3anox, ksO2nitri,
      ksO2oduox, PAdsODU, nh3fac, nh3den;
  real keep;          // 1 + relative_change_min
  real natol;         // -atol: reject if c1 - keep c < natol
  real minimum[NTR];  // clamp of the component epilogue
  double dt_min;
  int mstop;          // first cut level m with dt/4^m <= dt_min
  int ticks;          // 1: integer time ticks reproduce the FP64 sums
  int bcup_d;         // 1 flux, 2 concentration, 3 zero
  int mol_mode;       // 0 (diffusivity + 0.035 T) phi_i, 1 tortuosity
  int max_attempts;
  int epilogue;
  int budgets;
  // bioturbation profile 3 (get_rhs :618-645): POC-class factors to mg C per
  // g dry mass (initialize :383,386), beta and the exponent b
  int bio3;
  real toc_f1, toc_f2, bio_beta, bio_b, bio_L1, bio_L2;
};

// The rate parameters of Params that a per-column parameter set replaces,
// in the order of the per-slot table; the first NRATE_TEMP of them (rF, rS,
// cmax, rnit, rodu) are the microbial rates that temperature scales.
constexpr int NBGC_DEV = 16;
constexpr int NRATE_TEMP = 5;

// Temperature factor of the microbial rates at T degC for activation
// temperature Ta (K): the Arrhenius form and 288 K reference the driver
// applies to bioturbation (fabm_sediment_driver.F90:648).
__host__ __device__ inline double rate_factor(double Ta, double T) {
  return exp(-Ta * (1.0 / (T + 273.0) - (1.0 / 288.0)));
}

template <typename real>
__host__ __device__ __forceinline__ real* bgc_field(Params<real>& p, int i) {
  real* f[NBGC_DEV] = {&p.rF, &p.rS, &p.cmax, &p.rnit, &p.rodu, &p.pads, &p.ksO2oxic,
                       &p.kinO2denit, &p.ksNO3denit, &p.kinO2anox, &p.kinNO3anox,
                       &p.ksO2nitri, &p.ksO2oduox, &p.PAdsODU, &p.nh3fac, &p.nh3den};
  return f[i];
}

// The column's parameter set from the per-slot table (warp-uniform loads).
template <typename real>
__device__ __forceinline__ void load_bgc(Params<real>& p, const real* __restrict__ tab,
                                         size_t ns, int slot) {
  p.rF = tab[0 * ns + slot];
  p.rS = tab[1 * ns + slot];
  p.cmax = tab[2 * ns + slot];
  p.rnit = tab[3 * ns + slot];
  p.rodu = tab[4 * ns + slot];
  p.pads = tab[5 * ns + slot];
  p.ksO2oxic = tab[6 * ns + slot];
  p.kinO2denit = tab[7 * ns + slot];
  p.ksNO3denit = tab[8 * ns + slot];
  p.kinO2anox = tab[9 * ns + slot];
  p.kinNO3anox = tab[10 * ns + slot];
  p.ksO2nitri = tab[11 * ns + slot];
  p.ksO2oduox = tab[12 * ns + slot];
  p.PAdsODU = tab[13 * ns + slot];
  p.nh3fac = tab[14 * ns + slot];
  p.nh3den = tab[15 * ns + slot];
}

struct DevStats {
  unsigned long long surrogate;    // columns whose surrogate step was accepted
  unsigned long long attempts;
  unsigned long long accepted;
  unsigned long long column_steps;
  unsigned long long min_dt_bits;  // bit pattern of a positive double
  int max_col_attempts;
  int capped;
  int nan_cells;
  int status;
};

// ---------------------------------------------------------------------------
// division helpers: fast reciprocal in FP32, IEEE division in FP64
// a/b as a times the hardware's approximate reciprocal of b (the
// denominators here are Monod sums and positive rates, far from the range
// where that loses accuracy)
__device__ __forceinline__ float sdiv(float a, float b) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return a * r;
}
__device__ __forceinline__ double sdiv(double a, double b) { return a / b; }
// Explicit fused multiply-add.  The kernels are compiled without automatic
// contraction, so every FP32 rounding is the one written here, and results
// do not depend on which kernel (tile or warp-direct, any tuning) inlines
// the code.
__device__ __forceinline__ float fm(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fm(double a, double b, double c) { return fma(a, b, c); }

// ---------------------------------------------------------------------------
// OMEXDIA+P local rates of one cell (per second).  Published OMEXDIA
// (Soetaert, Herman, Middelburg 1996): two detritus classes with first-order
// decay; carbon mineralisation split into oxic / denitrification / anoxic
// pathways by Monod limitation and inhibition terms rescaled to sum to one;
// nitrification and ODU oxidation with O2 Monod terms; 0.8 mol NO3 per mol C
// denitrified; NH4 adsorption factor 1/(1+NH3Ads).  P extension: detrital P
// mineralises at the labile rate and PO4 exchanges with an adsorbed-P pool at
// rate PAds, the sorbing share being PAdsODU/(PAdsODU+ODU).
template <typename real>
__device__ __forceinline__ void omexdia_p(const Params<real>& p,
                                          const real (&c)[NTR],
                                          real (&r)[NTR], real& denit) {
  const real fdetC = c[T_FDETC], sdetC = c[T_SDETC], fdetN = c[T_FDETN];
  const real sdetN = c[T_SDETN], fdetP = c[T_FDETP], adsP = c[T_ADSP];
  const real O2 = c[T_O2], NO3 = c[T_NO3], NH4 = c[T_NH4], ODU = c[T_ODU];
  const real PO4 = c[T_PO4];
  // independent products and Monod denominators in FP32x2 pairs (each
  // component rounds as the scalar operation would)
  const float2 CprodFS = __fmul2_rn(make_float2(p.rF, p.rS), make_float2(fdetC, sdetC));
  const float2 NprodFS = __fmul2_rn(make_float2(p.rF, p.rS), make_float2(fdetN, sdetN));
  const float2 d01 = __fadd2_rn(make_float2(O2, O2), make_float2(p.ksO2oxic, p.kinO2denit));
  const float2 d23 = __fadd2_rn(make_float2(O2, O2), make_float2(p.kinO2anox, p.ksO2nitri));
  const float2 d45 = __fadd2_rn(make_float2(O2, NO3), make_float2(p.ksO2oduox, p.ksNO3denit));
  const float2 d67 = __fadd2_rn(make_float2(NO3, p.PAdsODU), make_float2(p.kinNO3anox, ODU));
  const real CprodF = CprodFS.x, CprodS = CprodFS.y;
  const real Cprod = CprodF + CprodS;
  const real lim = Cprod > p.cmax ? sdiv(p.cmax, Cprod) : real(1);
  const real oxlim = sdiv(O2, d01.x);
  const real dnlim = sdiv(p.kinO2denit, d01.y) * sdiv(NO3, d45.y);
  const real anlim = sdiv(p.kinO2anox, d23.x) * sdiv(p.kinNO3anox, d67.x);
  const real Cmin = sdiv(lim * Cprod, oxlim + dnlim + anlim);
  const float2 OxDn = __fmul2_rn(make_float2(Cmin, Cmin), make_float2(oxlim, dnlim));
  const real OxicMin = OxDn.x;
  const real Denit = OxDn.y;
  const real AnoxicMin = Cmin * anlim;
  const float2 NO = __fmul2_rn(__fmul2_rn(make_float2(p.rnit, p.rodu), make_float2(NH4, ODU)),
                               make_float2(sdiv(O2, d23.y), sdiv(O2, d45.x)));
  const real Nitri = NO.x;
  const real OduOx = NO.y;
  const real Rads = sdiv(p.pads * fm(p.PAdsODU, PO4, -(ODU * adsP)), d67.y);
  const real NprodF = NprodFS.x, NprodS = NprodFS.y;
  const real Pprod = p.rF * fdetP;
  // detritus decay -(lim prod) as (-lim) prod: the same values, one sign
  // flip instead of one per packed component
  const real nlim = -lim;
  const float2 rC = __fmul2_rn(make_float2(nlim, nlim), CprodFS);
  const float2 rN = __fmul2_rn(make_float2(nlim, nlim), NprodFS);
  r[T_FDETC] = rC.x;
  r[T_SDETC] = rC.y;
  r[T_FDETN] = rN.x;
  r[T_SDETN] = rN.y;
  r[T_FDETP] = -(lim * Pprod);
  r[T_ADSP] = Rads;
  r[T_O2] = fm(real(-2), Nitri, -OxicMin) - OduOx;
  r[T_NO3] = fm(real(-0.8), Denit, Nitri);
  r[T_NH4] = fm(lim, NprodF + NprodS, -Nitri) * p.nh3fac;
  r[T_ODU] = AnoxicMin - OduOx;
  r[T_PO4] = fm(lim, Pprod, -Rads);
  denit = Denit;
}

// ---------------------------------------------------------------------------
// Neighbour exchange along the column.  Layer L = s*32 + lane.
template <typename real, int LPL>
__device__ __forceinline__ void from_above(const real (&v)[LPL], real (&out)[LPL],
                                           int lane) {
#pragma unroll
  for (int s = 0; s < LPL; s++) out[s] = __shfl_up_sync(FULL, v[s], 1);
  if (LPL > 1) {
#pragma unroll
    for (int s = 1; s < LPL; s++) {
      real t = __shfl_sync(FULL, v[s - 1], 31);
      if (lane == 0) out[s] = t;
    }
  }
}

template <typename real, int LPL>
__device__ __forceinline__ void from_below(const real (&v)[LPL], real (&out)[LPL],
                                           int lane) {
#pragma unroll
  for (int s = 0; s < LPL; s++) out[s] = __shfl_down_sync(FULL, v[s], 1);
  if (LPL > 1) {
#pragma unroll
    for (int s = 0; s + 1 < LPL; s++) {
      real t = __shfl_sync(FULL, v[s + 1], 0);
      if (lane == 31) out[s] = t;
    }
  }
}

// Per-lane coefficients of one column for one coupling step.
template <typename real, int LPL, bool BC4>
struct Lane {
  real phi[LPL];   // porosity at the layer centre
  real ivol[LPL];  // 1 / (phi dz)
  real ad[LPL];    // dissolved interface conductance D/len (upper interface)
  real ap[LPL];    // particulate interface conductance
  real vol[LPL];   // phi dz (budgets)
  // per tracer: bottom-water value or downward surface flux, read from the
  // shared-memory forcing rows (only lane 0 uses them)
  const real* bnd_s;
  int bnd_stride;
  __device__ __forceinline__ real bnd(int n) const { return bnd_s[n * bnd_stride]; }
  real src[BC4 ? LPL : 1][BC4 ? NPART : 1];  // capped-flux cascade sources
  // FP32 form: the surface interface (upper interface of layer 0) carries
  // no conductance; its flux is alpha b - beta C0 with b the tracer's
  // surface value, alpha and beta zero on every lane but lane 0.  There:
  // particulates (a flux condition) alpha_p = 1; dissolved tracers
  // alpha_d = beta = ad0 (concentration condition, ad0 the dissolved
  // surface conductance), alpha_d = 1, beta = 0 (flux), or both 0 (none)
  real alpha_p, alpha_d, beta;
  // FP32 form: alpha b of every tracer, multiplied once per column and
  // read by the right-hand sides from shared memory (a 32-bit shared
  // address): lane 0 reads its warp's row (SURF_ROW floats, 8-byte aligned,
  // so a tracer pair is one 64-bit load), every other lane a row of zeros
  unsigned ab_sa;
  __device__ __forceinline__ float ab(int n) const {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(ab_sa + 4u * n));
    return v;
  }
  __device__ __forceinline__ float2 ab2(int n) const {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(ab_sa + 4u * n));
    return v;
  }
  // FP64 reference-order path (diff3d's own operands)
  real dz[LPL], len[LPL], Dp[LPL], Dd[LPL];
  real ext_a[BC4 ? LPL : 1][BC4 ? NPART : 1];  // cascade additions in the loop
  real ext_b[BC4 ? LPL : 1][BC4 ? NPART : 1];  // and the final one (:800-802)
  // bioturbation profile 3.  FP32: TOC weight phi/(1-phi), averaging weight
  // dz/cumdepth, depth term exp(a z)/(L1 + L2 exp(2 a z)), the bioturbation
  // conductance per unit factor and the molecular conductance.  FP64: the
  // reference's exp(zc 100 k_l), exp(zc 200 k_l), cumdepth, the prefix
  // bioturbation f_T / 86400 / 1e4 (1 - phi_i) and the molecular part.
  real wc[LPL], hw[LPL], gz[LPL], gb3[LPL], dm[LPL];
  real e1[LPL], e2[LPL], pre[LPL], mol[LPL];
  real cum;
};

// Profile-3 conductances of one right-hand side, FP32 (get_rhs :624-644):
// weighted TOC per layer, its dz-weighted column mean (a warp sum), infauna
// biomass and the factor beta biomass^b / TOC, folded into the particulate
// (ap) and dissolved (ad) interface conductances.  Lanes past the column
// get zero conductances.
//
// As in the static form, the surface interface carries no conductance: its
// dissolved value (lane 0) is returned in ad_top.
template <typename real, int LPL, bool BC4>
__device__ __forceinline__ void bio3_conductances(const Params<real>& p,
                                                  const Lane<real, LPL, BC4>& lc,
                                                  int lane, int K,
                                                  const real (&C)[LPL][NTR],
                                                  real (&ap)[LPL], real (&ad)[LPL],
                                                  real& ad_top) {
  real wt[LPL];
  real part = real(0);
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    wt[s] = lc.wc[s] * fm(p.toc_f1, C[s][T_FDETC], p.toc_f2 * C[s][T_SDETC]);
    part = fm(lc.hw[s], wt[s], part);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(FULL, part, o);
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const real biomass = wt[s] * lc.gz[s] * part;
    const real fac = sdiv(p.bio_beta * __powf(biomass, p.bio_b), wt[s]);
    const int L = s * 32 + lane;
    const bool inner = L < K && L != 0;
    const real a = lc.gb3[s] * fac;
    const real d = a + lc.dm[s];
    ap[s] = inner ? a : real(0);
    ad[s] = inner ? d : real(0);
    if (s == 0) ad_top = L == 0 ? d : real(0);
  }
}

// diff3d transport of tracer n added to R (FP32 folded form): interface
// fluxes F = a (C_above - C), the surface interface's flux alpha b - beta C
// on lane 0 (a = 0 there), then dC = (F - F_below) / (phi dz).  Branch- and
// select-free: lanes past the column hold zero state and conductances; the
// no-flux bottom drops F_below at K-1 by the zero conductance below it.
// PRE: alpha b is read from the column's premultiplied surface row; else it
// is formed from alpha and the boundary value (alpha varies per rhs).
template <int LPL, bool BC4, bool PART, bool PRE>
__device__ __forceinline__ void transport_one(const Lane<float, LPL, BC4>& lc, int n,
                                              const float (&a)[LPL], float alpha, float beta,
                                              int lane, const float (&C)[LPL][NTR],
                                              float (&R)[LPL][NTR], float (&ftop)[NTR]) {
  float v[LPL], vm[LPL], F[LPL], Fb[LPL];
#pragma unroll
  for (int s = 0; s < LPL; s++) v[s] = PART ? lc.phi[s] * C[s][n] : C[s][n];
  from_above<float, LPL>(v, vm, lane);
  const float ab = PRE ? lc.ab(n) : alpha * lc.bnd(n);
  const float top = PART ? ab : fm(-beta, v[0], ab);
#pragma unroll
  for (int s = 0; s < LPL; s++) F[s] = s == 0 ? fm(a[s], vm[s] - v[s], top) : a[s] * (vm[s] - v[s]);
  ftop[n] = F[0];
  from_below<float, LPL>(F, Fb, lane);
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const float div = F[s] - Fb[s];
    if (BC4 && PART)
      R[s][n] = R[s][n] + fm(div, lc.ivol[s], lc.src[BC4 ? s : 0][BC4 ? n : 0]);
    else
      R[s][n] = fm(div, lc.ivol[s], R[s][n]);
  }
}

__device__ __forceinline__ float2 splat(float a) { return make_float2(a, a); }
// a - b per component as one packed FMA, b (-1) + a: the product is exact,
// so each component rounds once, exactly as the subtraction does (signed
// zeros included), and no separate sign flip of b is issued.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}

// transport_one for tracers n and n+1 of one class at once: the same
// operations in packed FP32x2 arithmetic (each component rounds as the
// scalar operation does), halving the arithmetic instructions.
template <int LPL, bool BC4, bool PART, bool PRE>
__device__ __forceinline__ void transport_pair(const Lane<float, LPL, BC4>& lc, int n,
                                               const float (&a)[LPL], float alpha, float beta,
                                               int lane, const float (&C)[LPL][NTR],
                                               float (&R)[LPL][NTR], float (&ftop)[NTR]) {
  float vx[LPL], vy[LPL], mx[LPL], my[LPL];
  float2 v[LPL], F[LPL];
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const float2 c = make_float2(C[s][n], C[s][n + 1]);
    v[s] = PART ? __fmul2_rn(splat(lc.phi[s]), c) : c;
    vx[s] = v[s].x;
    vy[s] = v[s].y;
  }
  from_above<float, LPL>(vx, mx, lane);
  from_above<float, LPL>(vy, my, lane);
  // alpha b: the column's premultiplied pair (n even: one 64-bit load), or
  // formed here when alpha changes between right-hand sides
  const float2 ab = PRE ? lc.ab2(n)
                        : __fmul2_rn(splat(alpha), make_float2(lc.bnd(n), lc.bnd(n + 1)));
  const float2 top = PART ? ab : __ffma2_rn(splat(-beta), v[0], ab);
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const float2 d = sub2(make_float2(mx[s], my[s]), v[s]);
    F[s] = s == 0 ? __ffma2_rn(splat(a[s]), d, top) : __fmul2_rn(splat(a[s]), d);
  }
  ftop[n] = F[0].x;
  ftop[n + 1] = F[0].y;
  float fx[LPL], fy[LPL], bx[LPL], by[LPL];
#pragma unroll
  for (int s = 0; s < LPL; s++) { fx[s] = F[s].x; fy[s] = F[s].y; }
  from_below<float, LPL>(fx, bx, lane);
  from_below<float, LPL>(fy, by, lane);
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const float2 div = sub2(F[s], make_float2(bx[s], by[s]));
    float2 r = make_float2(R[s][n], R[s][n + 1]);
    if (BC4 && PART)
      r = __fadd2_rn(r, __ffma2_rn(div, splat(lc.ivol[s]),
                                   make_float2(lc.src[BC4 ? s : 0][BC4 ? n : 0],
                                               lc.src[BC4 ? s : 0][BC4 ? n + 1 : 0])));
    else
      r = __ffma2_rn(div, splat(lc.ivol[s]), r);
    R[s][n] = r.x;
    R[s][n + 1] = r.y;
  }
}

// Right-hand side of one column (FP32 form): OMEXDIA+P rates plus diff3d
// transport.  ftop receives the flux through the sediment surface (lane 0
// only).  Branch-free: lanes beyond the column's K layers hold zero state
// and zero conductances, so their rates and fluxes vanish by construction;
// the surface boundary enters through the lane coefficients ab / beta, the
// no-flux bottom by the zero conductance below layer K-1.
template <typename real, int LPL, bool BC4, bool BIO3>
__device__ __forceinline__ void column_rhs(const Params<real>& p,
                                           const Lane<real, LPL, BC4>& lc,
                                           int lane, int K,
                                           const real (&C)[LPL][NTR],
                                           real (&R)[LPL][NTR],
                                           real (&ftop)[NTR],
                                           real (&dn)[LPL]) {
  static_assert(std::is_same<real, float>::value, "FP32 form");
  real apv[LPL], adv[LPL];
  real alpha_d = lc.alpha_d, beta = lc.beta;
  if constexpr (BIO3) {
    real ad_top;
    bio3_conductances<real, LPL, BC4>(p, lc, lane, K, C, apv, adv, ad_top);
    if (p.bcup_d == 2) {  // concentration condition, this rhs's conductance
      alpha_d = ad_top;
      beta = ad_top;
    }
  } else {
#pragma unroll
    for (int s = 0; s < LPL; s++) { apv[s] = lc.ap[s]; adv[s] = lc.ad[s]; }
  }
#pragma unroll
  for (int s = 0; s < LPL; s++) omexdia_p<real>(p, C[s], R[s], dn[s]);
  // tracer pairs of one class in packed FP32x2 arithmetic, tracer 10 alone
  // alpha b from the column's premultiplied row, except for dissolved
  // tracers under profile 3, whose alpha may follow this rhs's conductance
  const real alpha_p = lc.alpha_p;
  constexpr bool PRE_D = !BIO3;
  transport_pair<LPL, BC4, true, true>(lc, 0, apv, alpha_p, 0.0f, lane, C, R, ftop);
  transport_pair<LPL, BC4, true, true>(lc, 2, apv, alpha_p, 0.0f, lane, C, R, ftop);
  transport_pair<LPL, BC4, true, true>(lc, 4, apv, alpha_p, 0.0f, lane, C, R, ftop);
  transport_pair<LPL, BC4, false, PRE_D>(lc, 6, adv, alpha_d, beta, lane, C, R, ftop);
  transport_pair<LPL, BC4, false, PRE_D>(lc, 8, adv, alpha_d, beta, lane, C, R, ftop);
  transport_one<LPL, BC4, false, PRE_D>(lc, NTR - 1, adv, alpha_d, beta, lane, C, R, ftop);
}

// ---------------------------------------------------------------------------
// FP64 warp sum (budgets)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

template <typename real>
__device__ __forceinline__ real warp_incl_scan(real v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    real t = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Sources of the BcUp=4 capped-flux cascade (diff3d :791-802): the surface
// flux beyond each layer's cap is passed down, and what reaches the bottom
// is added to the last interior interface.  The cascade is constant during
// a coupling step, so it enters as a fixed source per layer.
template <typename real, int LPL, bool BC4>
__device__ __forceinline__ void cascade_sources(Lane<real, LPL, BC4>& lc,
                                                const real (&cap)[LPL],
                                                int lane, int K) {
  if (!BC4) return;
  // inclusive prefix of caps over layers
  real pre[LPL];
  real carry = real(0);
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    pre[s] = warp_incl_scan<real>(cap[s], lane) + carry;
    carry = __shfl_sync(FULL, pre[s], 31);
  }
#pragma unroll
  for (int n = 0; n < NPART; n++) {
    const real fup = lc.bnd(n);
    real rest[LPL];  // rest after layer L: fup - sum_{j<=L} cap_j
#pragma unroll
    for (int s = 0; s < LPL; s++) rest[s] = fup - pre[s];
    real ra[LPL];    // rest after the layer above (rest_{L-1})
    from_above<real, LPL>(rest, ra, lane);
    real extra[LPL];
#pragma unroll
    for (int s = 0; s < LPL; s++) {
      const int L = s * 32 + lane;
      real e = real(0);
      if (L >= 1 && L <= K - 1 && ra[s] > real(0)) e = ra[s];
      extra[s] = e;
    }
    // what is left after the last layer goes to interface K-1
#pragma unroll
    for (int s = 0; s < LPL; s++) {
      const int L = s * 32 + lane;
      if (L == K - 1) {
        if (K == 1) extra[s] += rest[s];
        else if (ra[s] > real(0)) extra[s] += rest[s];
      }
    }
    real eb[LPL];
    from_below<real, LPL>(extra, eb, lane);
#pragma unroll
    for (int s = 0; s < LPL; s++) {
      const int L = s * 32 + lane;
      const real below = (L >= K - 1) ? real(0) : eb[s];
      lc.src[s][n] = (L < K) ? (extra[s] - below) * lc.ivol[s] : real(0);
    }
  }
}


// ---------------------------------------------------------------------------
// FP64 reference-order path.  The same OMEXDIA+P rates and diff3d transport
// written operation for operation as the FP64 CPU restatement evaluates them
// (compiled without FMA contraction), so that FP64 device results equal the
// restatement bit for bit and the decisions of the adaptive loop coincide.
__device__ __forceinline__ void omexdia_p_ref(const Params<double>& p,
                                              const double (&c)[NTR],
                                              double (&r)[NTR], double& denit) {
  const double fdetC = c[T_FDETC], sdetC = c[T_SDETC], fdetN = c[T_FDETN];
  const double sdetN = c[T_SDETN], fdetP = c[T_FDETP], adsP = c[T_ADSP];
  const double O2 = c[T_O2], NO3 = c[T_NO3], NH4 = c[T_NH4], ODU = c[T_ODU];
  const double PO4 = c[T_PO4];
  const double CprodF = p.rF * fdetC;
  const double CprodS = p.rS * sdetC;
  const double NprodF = p.rF * fdetN;
  const double NprodS = p.rS * sdetN;
  const double Pprod = p.rF * fdetP;
  const double Cprod = CprodF + CprodS;
  double lim = 1.0;
  if (Cprod > p.cmax) lim = p.cmax / Cprod;
  const double oxlim = O2 / (O2 + p.ksO2oxic);
  const double dnlim = (1.0 - O2 / (O2 + p.kinO2denit)) * (NO3 / (NO3 + p.ksNO3denit));
  const double anlim = (1.0 - O2 / (O2 + p.kinO2anox)) * (1.0 - NO3 / (NO3 + p.kinNO3anox));
  const double rescale = 1.0 / (oxlim + dnlim + anlim);
  const double Cmin = lim * Cprod;
  const double OxicMin = Cmin * oxlim * rescale;
  const double Denit = Cmin * dnlim * rescale;
  const double AnoxicMin = Cmin * anlim * rescale;
  const double Nitri = p.rnit * NH4 * (O2 / (O2 + p.ksO2nitri));
  const double OduOx = p.rodu * ODU * (O2 / (O2 + p.ksO2oduox));
  const double fox = p.PAdsODU / (p.PAdsODU + ODU);
  const double Rads = p.pads * (fox * PO4 - (1.0 - fox) * adsP);
  r[T_FDETC] = -(lim * CprodF);
  r[T_SDETC] = -(lim * CprodS);
  r[T_FDETN] = -(lim * NprodF);
  r[T_SDETN] = -(lim * NprodS);
  r[T_FDETP] = -(lim * Pprod);
  r[T_ADSP] = Rads;
  r[T_O2] = -OxicMin - 2.0 * Nitri - OduOx;
  r[T_NO3] = -0.8 * Denit + Nitri;
  r[T_NH4] = (lim * (NprodF + NprodS) - Nitri) / p.nh3den;
  r[T_ODU] = AnoxicMin - OduOx;
  r[T_PO4] = lim * Pprod - Rads;
  denit = Denit;
}

// Profile-3 diffusivities of one right-hand side in the reference's
// operation order (get_rhs :624-644, :652-653, :682-683): the column sum of
// dz * TOC runs layer by layer as the Fortran sum does.  pow is CUDA's, so
// the result can differ from the CPU restatement in the last bit.
template <int LPL, bool BC4>
__device__ __forceinline__ void bio3_diffusivities(const Params<double>& p,
                                                   const Lane<double, LPL, BC4>& lc,
                                                   int lane, int K,
                                                   const double (&C)[LPL][NTR],
                                                   double (&Dp)[LPL], double (&Dd)[LPL]) {
  double wt[LPL], v[LPL];
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const bool act = s * 32 + lane < K;
    double w = 0.0;
    w = w + p.toc_f1 * lc.phi[s] / (1.0 - lc.phi[s]) * C[s][T_FDETC];
    w = w + p.toc_f2 * lc.phi[s] / (1.0 - lc.phi[s]) * C[s][T_SDETC];
    wt[s] = act ? w : 1.0;
    v[s] = act ? lc.dz[s] * w : 0.0;
  }
  double sum = 0.0;
  for (int L = 0; L < K; L++) {
    double t = 0.0;
#pragma unroll
    for (int s = 0; s < LPL; s++) {
      const double u = __shfl_sync(FULL, v[s], L & 31);
      if (s == (L >> 5)) t = u;
    }
    sum = sum + t;
  }
  const double avg = sum / lc.cum;
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const bool act = s * 32 + lane < K;
    const double biomass = wt[s] * lc.e1[s] * avg / (p.bio_L1 + p.bio_L2 * lc.e2[s]);
    const double fac = p.bio_beta * pow(biomass, p.bio_b) / wt[s];
    const double diff = lc.pre[s] * fac;
    Dp[s] = act ? diff : 0.0;
    Dd[s] = act ? diff + lc.mol[s] : 0.0;
  }
}

template <int LPL, bool BC4, bool BIO3>
__device__ __forceinline__ void column_rhs_ref(const Params<double>& p,
                                               const Lane<double, LPL, BC4>& lc,
                                               int lane, int K,
                                               const double (&C)[LPL][NTR],
                                               double (&R)[LPL][NTR],
                                               double (&ftop)[NTR],
                                               double (&dn)[LPL]) {
  double Dpv[LPL], Ddv[LPL];
  if constexpr (BIO3) {
    bio3_diffusivities<LPL, BC4>(p, lc, lane, K, C, Dpv, Ddv);
  } else {
#pragma unroll
    for (int s = 0; s < LPL; s++) { Dpv[s] = lc.Dp[s]; Ddv[s] = lc.Dd[s]; }
  }
#pragma unroll
  for (int s = 0; s < LPL; s++) omexdia_p_ref(p, C[s], R[s], dn[s]);
#pragma unroll
  for (int n = 0; n < NTR; n++) {
    const bool part = n < NPART;
    double v[LPL], vm[LPL], F[LPL], Fb[LPL];
#pragma unroll
    for (int s = 0; s < LPL; s++) v[s] = part ? C[s][n] * lc.phi[s] : C[s][n];
    from_above<double, LPL>(v, vm, lane);
    // diff3d :776-778, interior interfaces
#pragma unroll
    for (int s = 0; s < LPL; s++) {
      const double D = part ? Dpv[s] : Ddv[s];
      F[s] = -D * (v[s] - vm[s]) / lc.len[s];
    }
    // :782-803 upper boundary
    if (lane == 0) {
      double f0;
      if (part) f0 = lc.bnd(n);
      else if (p.bcup_d == 2) f0 = -Ddv[0] * (v[0] - lc.bnd(n)) / lc.dz[0];
      else if (p.bcup_d == 1) f0 = lc.bnd(n);
      else f0 = 0.0;
      F[0] = f0;
    }
    if (BC4 && part) {
#pragma unroll
      for (int s = 0; s < LPL; s++) {
        F[s] = F[s] + lc.ext_a[BC4 ? s : 0][BC4 ? n : 0];
        F[s] = F[s] + lc.ext_b[BC4 ? s : 0][BC4 ? n : 0];
      }
    }
    if (lane == 0) ftop[n] = F[0];
    from_below<double, LPL>(F, Fb, lane);
    // :818-820 divergence; particulates scaled back to pore water (:677-678)
#pragma unroll
    for (int s = 0; s < LPL; s++) {
      const int L = s * 32 + lane;
      const double below = (L >= K - 1) ? 0.0 : Fb[s];
      double t;
      if (part) {
        const double dC = (F[s] - below) / ((1.0 - lc.phi[s]) * lc.dz[s]);
        t = dC * (1.0 - lc.phi[s]) / lc.phi[s];
      } else {
        t = (F[s] - below) / (lc.phi[s] * lc.dz[s]);
      }
      R[s][n] = (L < K) ? R[s][n] + t : 0.0;
    }
  }
}

// BcUp=4 cascade in the reference's serial order (diff3d :791-802): the
// running rest is broadcast layer by layer so every addition rounds as in
// the CPU loop.
template <int LPL, bool BC4>
__device__ __forceinline__ void cascade_ref(Lane<double, LPL, BC4>& lc,
                                            const double (&cap)[LPL],
                                            int lane, int K) {
  if (!BC4) return;
#pragma unroll
  for (int n = 0; n < NPART; n++) {
#pragma unroll
    for (int s = 0; s < LPL; s++) {
      lc.ext_a[BC4 ? s : 0][BC4 ? n : 0] = 0.0;
      lc.ext_b[BC4 ? s : 0][BC4 ? n : 0] = 0.0;
    }
    const double fup = lc.bnd(n);
    double rest = fup - __shfl_sync(FULL, cap[0], 0);
    int k = 1;
    while (rest > 0.0 && k <= K - 1) {
      const int ks = k >> 5, kl = k & 31;
#pragma unroll
      for (int s = 0; s < LPL; s++)
        if (s == ks && lane == kl) lc.ext_a[BC4 ? s : 0][BC4 ? n : 0] = rest;
      double ck = 0.0;
#pragma unroll
      for (int s = 0; s < LPL; s++) {
        const double t = __shfl_sync(FULL, cap[s], kl);
        if (s == ks) ck = t;
      }
      rest = rest - ck;
      k++;
    }
    if (k > K - 1) {
      const int L = K - 1, ks = L >> 5, kl = L & 31;
#pragma unroll
      for (int s = 0; s < LPL; s++)
        if (s == ks && lane == kl) lc.ext_b[BC4 ? s : 0][BC4 ? n : 0] = rest;
    }
  }
}

}  // namespace sed
