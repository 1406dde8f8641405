// pel_capi.cu -- the pelagic driver's step on the GPU and its C ABI
// (include/mossco_pel.h).
//
// MOSSCO's fabm_pelagic driver has a purely local right-hand side
// (src/drivers/fabm_pelagic_driver.F90:380-417: rhs = 0, then FABM's rates
// cell by cell); the only vertical coupling is light (:774-814), computed
// once per Run of the component (fabm_pelagic_component.F90:1931) from the
// surface down.  So one thread owns one water column and walks it from the
// surface layer to the bottom layer: it accumulates the optical depth,
// forms the cell's PAR, integrates the cell over the whole Run (every
// internal step with its epilogue) in registers, and writes it back.  Each
// value of the state is read and written once per Run, and consecutive
// threads touch consecutive columns of each [k][col] row.
//
// With the reference's grid-wide cut (PEL_CUT_GLOBAL) the adaptive method
// needs one decision per attempt over the whole grid; that path runs as
// separate light / rhs / test / accept / epilogue kernels with the decision
// read back on the host, as the parity mode.
#include "mossco_pel.h"
#include "cpl_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

namespace {

constexpr int NTR = PEL_NTR;
constexpr unsigned FULL = 0xffffffffu;
constexpr int kThreads = 128;

struct DevStats {
  unsigned long long attempts, accepted, capped, nan;
  unsigned long long min_dt_bits;  // host side of the grid-wide path: bits
                                   // of the smallest accepted substep
  int max_att;
  int mcut_full, mcut_last;        // most cuts of an accepted substep in a
                                   // full / the last internal step, -1 none
  int flag;                        // grid-wide test: any cell rejected
};

template <typename real>
struct Npzd {
  real p0, z0, kc, I_min, rmax, gmax, Iv2, alpha, rpn, rzn, rdn, rpdu, rpdl, rzd;
  real nIv2L;  // -Iv^2 log2(e): the FP32 grazing exponent as a power of two
};

template <typename real>
struct Args {
  const real* h;              // [K][ncol] layer heights
  const unsigned char* mask;  // [K][ncol] or null
  const real* I0;             // [ncol]
  const real* alb;            // [ncol] or null
  const real* bfl;            // [NTR][ncol] or null
  const real* sfl;
  const real* soil;
  // open boundaries (fabm_pelagic_component.F90:2115-2155): columns with
  // ob[col] set take bv[n][col] in every layer for each tracer n of bvmask
  const unsigned char* ob;    // [ncol] or null
  const real* bv;             // [NTR][ncol]
  unsigned bvmask;
  real* par;                  // [K][ncol]
  const int* wcols;           // [nwater] columns with a water cell, ascending
  int nwater;
  Npzd<real> m;
  real minimum[NTR];
  real bg, keep, natol;
  // The Run's internal steps (fabm_pelagic_component.F90:2061-2070),
  // scheduled once on the host by the reference's loop: nfull steps of
  // h_full, then one of h_last if has_last.  mstop: cuts allowed before
  // dt_red <= dt_min; ticks: the adaptive bookkeeping in integer ticks of
  // h / 4^mstop is exact (every partial sum of the reference's FP64 dt_int
  // is representable), so the FP32 kernels need no FP64 arithmetic.
  double h_full, h_last, dt_min;
  real hr_full, hr_last;
  int nfull, has_last, mstop_full, mstop_last, ticks;
  int ncol, K, max_attempts;
  DevStats* stats;
};

// exp of the FP64 path: Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2
// (Cody and Waite, Software Manual for the Elementary Functions, 1980), the
// Taylor series of exp(r) to degree 13 in Horner form with fused
// multiply-adds, and the scaling by 2^k.  Each step is an IEEE operation
// with one rounding, so the oracle's C function of the same steps gives the
// same bits.  Results below 2^-1020 flush to 0, above 2^1023.9 go to inf.
__device__ __forceinline__ double pexp(double x) {
  const double inv_ln2 = 1.4426950408889634;
  const double ln2_hi = 0.6931471805599453;
  const double ln2_lo = 2.3190468138462996e-17;
  if (x != x) return x;
  if (x < -707.0) return 0.0;
  if (x > 709.7) return HUGE_VAL;
  const double k = rint(x * inv_ln2);
  double r = fma(-k, ln2_hi, x);
  r = fma(-k, ln2_lo, r);
  double s = 1.0 / 6227020800.0;
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
__device__ __forceinline__ float pexp(float x) { return __expf(x); }
// 2^x and 1/x by the hardware's approximate instructions (FP32 path)
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ double pdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float pdiv(float a, float b) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return a * r;
}
// a*b + c: one fused multiply-add in FP32; in FP64 a product and a sum
// rounded separately, as the oracle's left-to-right statements are (the
// unit is compiled without automatic contraction)
__device__ __forceinline__ double fm(double a, double b, double c) { return a * b + c; }
__device__ __forceinline__ float fm(float a, float b, float c) { return fmaf(a, b, c); }

// The light-dependent factors of gotm_npzd, fixed for a cell during a Run
// (PAR is computed once per Run): the mortality switch and
// L = rmax * par / iopt * exp(1 - par/iopt), the Steele light limitation
// times the maximum rate, evaluated left to right.
template <typename real>
__device__ __forceinline__ void light_terms(const Npzd<real>& m, real par, real iopt,
                                            real& L, real& rpd) {
  rpd = par >= m.I_min ? m.rpdu : m.rpdl;
  const real x = pdiv(par, iopt);
  L = pdiv(m.rmax * par, iopt) * pexp(real(1) - x);
}

// gotm_npzd local rates of a cell c = (n, p, z, d): primary production
// L n/(alpha+n) (p+p0), grazing gmax (1 - exp(-Iv^2 p^2)) (z+z0), linear
// exudation, excretion, mortality and remineralisation (Burchard et al.
// 2006, J. Mar. Syst. 61:180-211).  The four rates sum to zero.
template <typename real>
__device__ __forceinline__ void rates(const Npzd<real>& m, const real (&c)[NTR], real L,
                                      real rpd, real (&r)[NTR]) {
  const real n = c[0], p = c[1], z = c[2], d = c[3];
  real fnp, fpz;
  if constexpr (std::is_same<real, float>::value) {
    // exp(-Iv^2 p^2) = 2^(-Iv^2 log2(e) p^2); n/(alpha+n) by a reciprocal
    fnp = L * n * rcp_approx(m.alpha + n) * (p + m.p0);
    fpz = m.gmax * (1.0f - ex2_approx(m.nIv2L * (p * p))) * (z + m.z0);
  } else {
    fnp = pdiv(L * n, m.alpha + n) * (p + m.p0);
    fpz = m.gmax * (real(1) - pexp(-(m.Iv2 * (p * p)))) * (z + m.z0);
  }
  // each sum left to right: ((-fnp + rpn p) + rzn z) + rdn d, ...
  r[0] = fm(m.rdn, d, fm(m.rzn, z, fm(m.rpn, p, -fnp)));
  r[1] = fm(-rpd, p, fm(-m.rpn, p, fnp - fpz));
  r[2] = fm(-m.rzd, z, fm(-m.rzn, z, fpz));
  r[3] = fm(-m.rdn, d, fm(m.rzd, z, rpd * p));
}

struct CellStats {
  unsigned long long att = 0, acc = 0, capped = 0, nan = 0;
  int maxatt = 0;
  int mfull = -1, mlast = -1;  // most cuts of an accepted substep
};

// ode_solver (src/utilities/solver_library.F90:97-186) on one cell.  The
// rhs is local, so this equals the whole-grid statements for the fixed
// methods and for the adaptive one with a per-cell cut; each stage is
// combined in the reference's operation order.
template <typename real, int METHOD>
__device__ __forceinline__ void step_cell(const Args<real>& a, real (&c)[NTR], real L, real rpd,
                                          bool last, CellStats& s) {
  const real hr = last ? a.hr_last : a.hr_full;
  if (METHOD == SED_ADAPTIVE_EULER) {  // :104-140, a rejection reuses the rhs
    real r[NTR];
    real dtr = hr;
    int att = 0, m = 0, macc = -1;
    rates(a.m, c, L, rpd, r);
    if (sizeof(real) == 4 && a.ticks) {
      const int mstop = last ? a.mstop_last : a.mstop_full;
      const unsigned long long T = 1ull << (2 * mstop);
      unsigned long long t = 0, inc = T;
      while (t < T) {
        if (att >= a.max_attempts) { s.capped++; break; }
        att++;
        bool bad = false;
#pragma unroll
        for (int n = 0; n < NTR; n++) bad |= fm(-a.keep, c[n], fm(dtr, r[n], c[n])) < a.natol;
        if (bad && m < mstop) {
          m++;
          dtr = dtr * real(0.25);
          inc >>= 2;
        } else {
#pragma unroll
          for (int n = 0; n < NTR; n++) c[n] = fm(dtr, r[n], c[n]);
          t += inc;
          s.acc++;
          macc = m;
          if (t < T) rates(a.m, c, L, rpd, r);
        }
      }
    } else {
      const double hs = last ? a.h_last : a.h_full;
      double dt_int = 0.0, dt_red = hs;
      while (dt_int < hs) {
        if (att >= a.max_attempts) { s.capped++; break; }
        att++;
        bool bad = false;
#pragma unroll
        for (int n = 0; n < NTR; n++) bad |= fm(-a.keep, c[n], fm(dtr, r[n], c[n])) < a.natol;
        if (bad && dt_red > a.dt_min) {
          m++;
          dt_red = dt_red * 0.25;
          dtr = dtr * real(0.25);
        } else {
#pragma unroll
          for (int n = 0; n < NTR; n++) c[n] = fm(dtr, r[n], c[n]);
          dt_int = dt_int + dt_red;
          s.acc++;
          macc = m;
          if (dt_int < hs) rates(a.m, c, L, rpd, r);
        }
      }
    }
    s.att += att;
    s.maxatt = att > s.maxatt ? att : s.maxatt;
    if (last) s.mlast = macc > s.mlast ? macc : s.mlast;
    else s.mfull = macc > s.mfull ? macc : s.mfull;
    return;
  }
  const real dt = hr;
  const real third = real(1.0 / 3.0);
  const real half = real(0.5);
  real r0[NTR], r1[NTR], r2[NTR], r3[NTR], c1[NTR];
  if (METHOD == SED_EULER) {  // :99-102
    rates(a.m, c, L, rpd, r0);
#pragma unroll
    for (int n = 0; n < NTR; n++) c[n] = fm(dt, r0[n], c[n]);
  } else if (METHOD == SED_RUNGE_KUTTA_4) {  // :142-163
    const real hdt = half * dt, dt3 = dt * third;
    rates(a.m, c, L, rpd, r0);
#pragma unroll
    for (int n = 0; n < NTR; n++) c1[n] = fm(hdt, r0[n], c[n]);
    rates(a.m, c1, L, rpd, r1);
#pragma unroll
    for (int n = 0; n < NTR; n++) c1[n] = fm(hdt, r1[n], c[n]);
    rates(a.m, c1, L, rpd, r2);
#pragma unroll
    for (int n = 0; n < NTR; n++) c1[n] = fm(dt, r2[n], c[n]);
    rates(a.m, c1, L, rpd, r3);
#pragma unroll
    for (int n = 0; n < NTR; n++)  // c + dt/3 (((r0/2 + r1) + r2) + r3/2)
      c[n] = fm(dt3, fm(half, r3[n], fm(half, r0[n], r1[n]) + r2[n]), c[n]);
  } else {  // RUNGE_KUTTA_4_38, :164-185
    const real dt3 = third * dt, dt8 = dt * real(1) / real(8);
    rates(a.m, c, L, rpd, r0);
#pragma unroll
    for (int n = 0; n < NTR; n++) c1[n] = fm(dt3, r0[n], c[n]);
    rates(a.m, c1, L, rpd, r1);
#pragma unroll
    for (int n = 0; n < NTR; n++) c1[n] = fm(dt, fm(-third, r0[n], r1[n]), c[n]);
    rates(a.m, c1, L, rpd, r2);
#pragma unroll
    for (int n = 0; n < NTR; n++) c1[n] = fm(dt, r0[n] - r1[n] + r2[n], c[n]);
    rates(a.m, c1, L, rpd, r3);
#pragma unroll
    for (int n = 0; n < NTR; n++)  // c + dt/8 (((r0 + 3 r1) + 3 r2) + r3)
      c[n] = fm(dt8, fm(real(3), r2[n], fm(real(3), r1[n], r0[n])) + r3[n], c[n]);
  }
  s.att++;
  s.acc++;
  s.maxatt = s.maxatt > 1 ? s.maxatt : 1;
  if (last) s.mlast = 0 > s.mlast ? 0 : s.mlast;
  else s.mfull = 0 > s.mfull ? 0 : s.mfull;
}

// The Run's per-step epilogue on one cell (fabm_pelagic_component.F90):
// NaN count after ode_solver (:2084), the soil-surface upward fluxes where
// the bottom layer has a height (:2100-2105), the vertically homogeneous
// open-boundary values (:2115-2155), the external surface fluxes into the
// top layer (:2193-2194), the soil-surface flux fields unless the bottom
// cell would go negative (:2196-2203), then clip_below_minimum
// (fabm_pelagic_driver.F90:910-927).
template <typename real>
__device__ __forceinline__ void epilogue_cell(const Args<real>& a, real (&c)[NTR], int k, int col,
                                              real hk, real dt, CellStats& s) {
  // a NaN in any tracer makes the sum NaN (one compare per cell)
  const real sum = (c[0] + c[1]) + (c[2] + c[3]);
  s.nan += sum != sum;
  if (k == 0 && a.bfl && hk > real(0)) {
#pragma unroll
    for (int n = 0; n < NTR; n++) c[n] = c[n] + a.bfl[(size_t)n * a.ncol + col] * dt / hk;
  }
  if (a.ob && a.ob[col]) {
#pragma unroll
    for (int n = 0; n < NTR; n++)
      if ((a.bvmask >> n) & 1u) c[n] = a.bv[(size_t)n * a.ncol + col];
  }
  if (k == a.K - 1 && a.sfl) {
#pragma unroll
    for (int n = 0; n < NTR; n++) c[n] = c[n] + a.sfl[(size_t)n * a.ncol + col] * dt / hk;
  }
  if (k == 0 && a.soil) {
#pragma unroll
    for (int n = 0; n < NTR; n++) {
      const real inc = a.soil[(size_t)n * a.ncol + col] * dt / hk;
      if (c[n] + inc > real(0)) c[n] = c[n] + inc;
    }
  }
#pragma unroll
  for (int n = 0; n < NTR; n++)
    if (c[n] < a.minimum[n]) c[n] = a.minimum[n];
}

template <typename real>
__device__ __forceinline__ real iopt_of(const Args<real>& a, real I0) {
  const real q = real(0.25) * I0;  // iopt = max(I_0/4, I_min)
  return q > a.m.I_min ? q : a.m.I_min;
}

__device__ __forceinline__ void flush_stats(DevStats* st, CellStats s) {
  for (int o = 16; o > 0; o >>= 1) {
    s.att += __shfl_down_sync(FULL, s.att, o);
    s.acc += __shfl_down_sync(FULL, s.acc, o);
    s.capped += __shfl_down_sync(FULL, s.capped, o);
    s.nan += __shfl_down_sync(FULL, s.nan, o);
    const int ma = __shfl_down_sync(FULL, s.maxatt, o);
    s.maxatt = ma > s.maxatt ? ma : s.maxatt;
    const int mf = __shfl_down_sync(FULL, s.mfull, o);
    s.mfull = mf > s.mfull ? mf : s.mfull;
    const int ml = __shfl_down_sync(FULL, s.mlast, o);
    s.mlast = ml > s.mlast ? ml : s.mlast;
  }
  if ((threadIdx.x & 31) == 0) {
    if (s.att) atomicAdd(&st->attempts, s.att);
    if (s.acc) atomicAdd(&st->accepted, s.acc);
    if (s.capped) atomicAdd(&st->capped, s.capped);
    if (s.nan) atomicAdd(&st->nan, s.nan);
    if (s.maxatt) atomicMax(&st->max_att, s.maxatt);
    if (s.mfull >= 0) atomicMax(&st->mcut_full, s.mfull);
    if (s.mlast >= 0) atomicMax(&st->mcut_last, s.mlast);
  }
}

// One Run (LIGHT && EPI) or one ode_solver call with the handle's PAR
// (neither) for every water column: thread = column, layers from the
// surface down.
// The next layer's values are loaded before the current cell is integrated,
// so each thread keeps a load in flight while it computes.
template <typename real, typename store, int METHOD, bool LIGHT, bool EPI>
__global__ void __launch_bounds__(kThreads, 8) k_pel_run(Args<real> a, store* __restrict__ conc) {
  // threads take the water columns in order: no lane idles on land, and
  // neighbouring lanes still read neighbouring addresses
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  CellStats s;
  if (t < a.nwater) {
    const int col = a.wcols[t];
    const size_t plane = (size_t)a.K * a.ncol;
    const real I0 = a.I0[col];
    const real localpar = I0 * (real(1) - (a.alb ? a.alb[col] : real(0)));
    const real iopt = iopt_of(a, I0);
    real prev = real(0);
    // layer K-1 (the surface layer) first
    size_t i = (size_t)(a.K - 1) * a.ncol + col;
    bool nmsk = a.mask && a.mask[i];
    real cn[NTR], hn = a.h[i];
#pragma unroll
    for (int n = 0; n < NTR; n++) cn[n] = nmsk ? real(0) : (real)conc[n * plane + i];
    for (int k = a.K - 1; k >= 0; k--) {
      const bool msk = nmsk;
      const real hk = hn;
      real c[NTR];
#pragma unroll
      for (int n = 0; n < NTR; n++) c[n] = cn[n];
      const size_t ik = i;
      if (k > 0) {  // prefetch layer k-1
        i -= a.ncol;
        nmsk = a.mask && a.mask[i];
        hn = a.h[i];
#pragma unroll
        for (int n = 0; n < NTR; n++) cn[n] = nmsk ? real(0) : (real)conc[n * plane + i];
      }
      real par;
      if (LIGHT) {  // fabm_pelagic_driver.F90:786-799, half layers from the top
        real b = prev;
        if (!msk) {
          const real ext = a.m.kc * (a.m.p0 + c[1] + c[3]);
          const real t = (ext + a.bg) * real(0.5) * hk;
          b = prev + t;
          prev = b + t;
        }
        par = localpar * pexp(-b);
        if (a.par) a.par[ik] = par;
      } else {
        par = msk ? real(0) : a.par[ik];
      }
      if (msk) continue;
      real L, rpd;
      light_terms(a.m, par, iopt, L, rpd);
      const int nsteps = a.nfull + a.has_last;
      for (int st = 0; st < nsteps; st++) {  // :2061-2070
        const bool last = st == a.nfull;
        step_cell<real, METHOD>(a, c, L, rpd, last, s);
        if (EPI) epilogue_cell(a, c, k, col, hk, last ? a.hr_last : a.hr_full, s);
      }
#pragma unroll
      for (int n = 0; n < NTR; n++) conc[n * plane + ik] = (store)c[n];
    }
  }
  flush_stats(a.stats, s);
}

// ---- grid-wide cut (the reference's any() over the PET) -------------------

template <typename real, typename store>
__global__ void __launch_bounds__(kThreads) k_pel_light(Args<real> a, const store* __restrict__ conc) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= a.ncol) return;
  const size_t plane = (size_t)a.K * a.ncol;
  const real I0 = a.I0[col];
  const real localpar = I0 * (real(1) - (a.alb ? a.alb[col] : real(0)));
  real prev = real(0);
  for (int k = a.K - 1; k >= 0; k--) {
    const size_t i = (size_t)k * a.ncol + col;
    real b = prev;
    if (!(a.mask && a.mask[i])) {
      const real p = (real)conc[plane + i], d = (real)conc[3 * plane + i];
      const real ext = a.m.kc * (a.m.p0 + p + d);
      const real t = (ext + a.bg) * real(0.5) * a.h[i];
      b = prev + t;
      prev = b + t;
    }
    a.par[i] = localpar * pexp(-b);
  }
}

// get_rhs (fabm_pelagic_driver.F90:380-417): rhs = 0, then the local rates.
template <typename real, typename store>
__global__ void __launch_bounds__(kThreads) k_pel_rhs(Args<real> a, const store* __restrict__ conc,
                                                      store* __restrict__ rhs) {
  const size_t plane = (size_t)a.K * a.ncol;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane;
       i += (size_t)gridDim.x * blockDim.x) {
    real r[NTR] = {real(0), real(0), real(0), real(0)};
    if (!(a.mask && a.mask[i])) {
      const int col = (int)(i % a.ncol);
      real c[NTR];
#pragma unroll
      for (int n = 0; n < NTR; n++) c[n] = (real)conc[n * plane + i];
      real L, rpd;
      light_terms(a.m, a.par[i], iopt_of(a, a.I0[col]), L, rpd);
      rates(a.m, c, L, rpd, r);
    }
#pragma unroll
    for (int n = 0; n < NTR; n++) rhs[n * plane + i] = (store)r[n];
  }
}

// positivity test of solver_library.F90:121 over every water cell
template <typename real>
__global__ void __launch_bounds__(kThreads) k_pel_test(Args<real> a, const real* __restrict__ conc,
                                                       const real* __restrict__ rhs, real dtr) {
  const size_t plane = (size_t)a.K * a.ncol;
  bool bad = false;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane;
       i += (size_t)gridDim.x * blockDim.x) {
    if (a.mask && a.mask[i]) continue;
#pragma unroll
    for (int n = 0; n < NTR; n++) {
      const real c = conc[n * plane + i];
      bad |= (c + dtr * rhs[n * plane + i]) - a.keep * c < a.natol;
    }
  }
  if (__any_sync(FULL, bad) && (threadIdx.x & 31) == 0) atomicOr(&a.stats->flag, 1);
}

template <typename real>
__global__ void __launch_bounds__(kThreads) k_pel_accept(Args<real> a, real* __restrict__ conc,
                                                         const real* __restrict__ rhs, real dtr) {
  const size_t plane = (size_t)a.K * a.ncol;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane;
       i += (size_t)gridDim.x * blockDim.x) {
    if (a.mask && a.mask[i]) continue;
#pragma unroll
    for (int n = 0; n < NTR; n++) conc[n * plane + i] = conc[n * plane + i] + dtr * rhs[n * plane + i];
  }
}

template <typename real>
__global__ void __launch_bounds__(kThreads) k_pel_epilogue(Args<real> a, real* __restrict__ conc,
                                                           real hr) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  CellStats s;
  if (col < a.ncol) {
    const size_t plane = (size_t)a.K * a.ncol;
    for (int k = 0; k < a.K; k++) {
      const size_t i = (size_t)k * a.ncol + col;
      if (a.mask && a.mask[i]) continue;
      real c[NTR];
#pragma unroll
      for (int n = 0; n < NTR; n++) c[n] = conc[n * plane + i];
      epilogue_cell(a, c, k, col, a.h[i], hr, s);
#pragma unroll
      for (int n = 0; n < NTR; n++) conc[n * plane + i] = c[n];
    }
  }
  flush_stats(a.stats, s);
}

template <typename src, typename dst>
__global__ void k_pel_convert(const src* __restrict__ in, dst* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (dst)in[i];
}

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t b) {
    if (p && bytes >= b) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, b ? b : 16);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

struct Schedule {
  double t_couple = -1.0, dt = -1.0;
  int nfull = 0, has_last = 0;
  double h_full = 0.0, h_last = 0.0;
  int mstop_full = 0, mstop_last = 0;
  bool ticks = false;
};

struct pel_handle {
  pel_params prm{};
  Schedule sched;
  int inum = 0, jnum = 0, ncol = 0, K = 0, device = 0, sms = 0;
  int water_cols = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  bool have_grid = false, have_forcing = false, have_state = false, have_par = false;
  bool has_mask = false, has_alb = false, has_bfl = false, has_sfl = false, has_soil = false;
  unsigned bvmask = 0;  // tracers with open-boundary values (0: none)
  DevBuf d_h, d_mask, d_I0, d_alb, d_bfl, d_sfl, d_soil, d_par, d_state, d_stage, d_rhs,
      d_work, d_stats, d_wcols, d_ob, d_bv;
  DevStats* h_stats = nullptr;  // pinned
  long long launches = 0;
  std::vector<int> wcols;       // host copy of d_wcols
  // pipelined host calls: copy-in, per-chunk step and copy-out streams
  cudaStream_t s_in = nullptr, s_out = nullptr, s_cmp[8] = {};
  cudaEvent_t e_start = nullptr, e_done = nullptr, e_in[8] = {}, e_cmp[8] = {};

  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(SED_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
  bool fp64() const { return prm.precision == SED_FP64; }
  size_t rsize() const { return fp64() ? sizeof(double) : sizeof(float); }
  size_t cells() const { return (size_t)K * ncol; }
  ~pel_handle() {
    if (stream) cudaStreamSynchronize(stream);
    for (cudaStream_t st : {s_in, s_out})
      if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
    for (cudaStream_t st : s_cmp)
      if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
    for (cudaEvent_t ev : {e_start, e_done})
      if (ev) cudaEventDestroy(ev);
    for (int c = 0; c < 8; c++) {
      if (e_in[c]) cudaEventDestroy(e_in[c]);
      if (e_cmp[c]) cudaEventDestroy(e_cmp[c]);
    }
    if (h_stats) cudaFreeHost(h_stats);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
};

#define PK(expr, what)                                    \
  do {                                                    \
    cudaError_t e_ = (expr);                              \
    if (e_ != cudaSuccess) return h->cuda_fail(e_, what); \
  } while (0)

namespace {

int check_params(pel_handle* h, const pel_params& p) {
  const double nonneg[] = {p.p0, p.z0, p.kc, p.rmax, p.gmax, p.Iv, p.alpha, p.rpn,
                           p.rzn, p.rdn, p.rpdu, p.rpdl, p.rzd, p.background_extinction,
                           p.atol, p.dt_min};
  for (double v : nonneg)
    if (!(v >= 0.0) || !std::isfinite(v)) return h->fail(SED_E_ARG, "negative or non-finite parameter");
  if (!(p.I_min > 0.0)) return h->fail(SED_E_ARG, "I_min must be > 0");
  if (!(p.relative_change_min > -1.0 && p.relative_change_min <= 0.0))
    return h->fail(SED_E_ARG, "relative_change_min must lie in (-1, 0]");
  if (p.max_attempts <= 0) return h->fail(SED_E_ARG, "max_attempts must be > 0");
  if (p.cut_scope != PEL_CUT_PER_CELL && p.cut_scope != PEL_CUT_GLOBAL)
    return h->fail(SED_E_ARG, "cut_scope must be PEL_CUT_PER_CELL or PEL_CUT_GLOBAL");
  if (p.precision != SED_FP32 && p.precision != SED_FP64)
    return h->fail(SED_E_ARG, "precision must be SED_FP32 or SED_FP64");
  for (int n = 0; n < NTR; n++)
    if (std::isnan(p.minimum[n])) return h->fail(SED_E_ARG, "minimum is NaN");
  return SED_OK;
}

// Significant bits of x's significand (x > 0, finite).
int sig_bits(double x) {
  int e;
  const double m = std::frexp(x, &e);
  unsigned long long mant = (unsigned long long)std::ldexp(m, 53);
  int tz = 0;
  while (mant && !(mant & 1ull)) {
    mant >>= 1;
    tz++;
  }
  return 53 - tz;
}

// Cuts by 1/4 the adaptive method may take from h: the first m with
// h 4^-m <= dt_min (solver_library.F90:126-127).
int cuts_allowed(double h, double dt_min) {
  int m = 0;
  for (double d = h; d > dt_min && m < 1100; d *= 0.25) m++;
  return m;
}

// The internal steps of a Run by the reference's loop in FP64
// (fabm_pelagic_component.F90:2061-2070): steps of dt, the last one
// shortened to end on t_couple.
Schedule make_schedule(double t_couple, double dt, double dt_min) {
  Schedule s;
  s.t_couple = t_couple;
  s.dt = dt;
  s.h_full = dt;
  double t = 0.0;
  while (t < t_couple) {
    if (t + dt > t_couple) {
      s.has_last = 1;
      s.h_last = t_couple - t;
      t = t + s.h_last;
    } else {
      s.nfull++;
      t = t + dt;
    }
  }
  s.mstop_full = cuts_allowed(s.h_full, dt_min);
  s.mstop_last = s.has_last ? cuts_allowed(s.h_last, dt_min) : 0;
  auto exact = [](double h, int mstop) { return mstop <= 26 && sig_bits(h) + 2 * mstop <= 53; };
  s.ticks = (s.nfull == 0 || exact(s.h_full, s.mstop_full)) &&
            (!s.has_last || exact(s.h_last, s.mstop_last));
  return s;
}

template <typename real>
Args<real> make_args(pel_handle* h, double t_couple, double dt) {
  const pel_params& p = h->prm;
  const double day = 86400.0;  // per-day namelist rates to per second
  Args<real> a{};
  a.h = h->d_h.as<real>();
  a.mask = h->has_mask ? h->d_mask.as<unsigned char>() : nullptr;
  a.I0 = h->d_I0.as<real>();
  a.alb = h->has_alb ? h->d_alb.as<real>() : nullptr;
  a.bfl = h->has_bfl ? h->d_bfl.as<real>() : nullptr;
  a.sfl = h->has_sfl ? h->d_sfl.as<real>() : nullptr;
  a.soil = h->has_soil ? h->d_soil.as<real>() : nullptr;
  a.ob = h->bvmask ? h->d_ob.as<unsigned char>() : nullptr;
  a.bv = h->bvmask ? h->d_bv.as<real>() : nullptr;
  a.bvmask = h->bvmask;
  a.par = h->d_par.as<real>();
  a.wcols = h->d_wcols.as<int>();
  a.nwater = h->water_cols;
  a.m.p0 = (real)p.p0;
  a.m.z0 = (real)p.z0;
  a.m.kc = (real)p.kc;
  a.m.I_min = (real)p.I_min;
  a.m.rmax = (real)(p.rmax / day);
  a.m.gmax = (real)(p.gmax / day);
  a.m.Iv2 = (real)(p.Iv * p.Iv);
  a.m.nIv2L = (real)(-(p.Iv * p.Iv) * 1.4426950408889634);
  a.m.alpha = (real)p.alpha;
  a.m.rpn = (real)(p.rpn / day);
  a.m.rzn = (real)(p.rzn / day);
  a.m.rdn = (real)(p.rdn / day);
  a.m.rpdu = (real)(p.rpdu / day);
  a.m.rpdl = (real)(p.rpdl / day);
  a.m.rzd = (real)(p.rzd / day);
  for (int n = 0; n < NTR; n++) a.minimum[n] = (real)p.minimum[n];
  a.bg = (real)p.background_extinction;
  a.keep = (real)(1.0 + p.relative_change_min);
  a.natol = (real)(-p.atol);
  a.dt_min = p.dt_min;
  if (h->sched.t_couple != t_couple || h->sched.dt != dt)
    h->sched = make_schedule(t_couple, dt, p.dt_min);
  const Schedule& sc = h->sched;
  a.h_full = sc.h_full;
  a.h_last = sc.h_last;
  a.hr_full = (real)sc.h_full;
  a.hr_last = (real)sc.h_last;
  a.nfull = sc.nfull;
  a.has_last = sc.has_last;
  a.mstop_full = sc.mstop_full;
  a.mstop_last = sc.mstop_last;
  a.ticks = sc.ticks;
  a.ncol = h->ncol;
  a.K = h->K;
  a.max_attempts = p.max_attempts;
  a.stats = h->d_stats.as<DevStats>();
  return a;
}

int col_blocks(const pel_handle* h) { return (h->ncol + kThreads - 1) / kThreads; }
int cell_blocks(const pel_handle* h) {
  const size_t b = (h->cells() + kThreads - 1) / kThreads;
  const size_t cap = (size_t)h->sms * 16;
  return (int)(b < cap ? b : cap);
}

int reset_stats(pel_handle* h) {
  memset(h->h_stats, 0, sizeof(DevStats));
  double big = 1e300;
  memcpy(&h->h_stats->min_dt_bits, &big, sizeof big);
  h->h_stats->mcut_full = h->h_stats->mcut_last = -1;
  PK(cudaMemcpyAsync(h->d_stats.p, h->h_stats, sizeof(DevStats), cudaMemcpyHostToDevice,
                     h->stream),
     "stats reset");
  return SED_OK;
}

// one thread per water column of a.wcols[0 .. a.nwater)
template <typename real, typename store, bool LIGHT, bool EPI>
void launch_run(pel_handle* h, const Args<real>& a, store* conc, int method, cudaStream_t st) {
  const dim3 g(a.nwater > 0 ? (a.nwater + kThreads - 1) / kThreads : 1), b(kThreads);
  switch (method) {
    case SED_EULER: k_pel_run<real, store, SED_EULER, LIGHT, EPI><<<g, b, 0, st>>>(a, conc); break;
    case SED_RUNGE_KUTTA_4:
      k_pel_run<real, store, SED_RUNGE_KUTTA_4, LIGHT, EPI><<<g, b, 0, st>>>(a, conc);
      break;
    case SED_ADAPTIVE_EULER:
      k_pel_run<real, store, SED_ADAPTIVE_EULER, LIGHT, EPI><<<g, b, 0, st>>>(a, conc);
      break;
    default:
      k_pel_run<real, store, SED_RUNGE_KUTTA_4_38, LIGHT, EPI><<<g, b, 0, st>>>(a, conc);
      break;
  }
  h->launches++;
}

template <typename src, typename dst>
void convert(pel_handle* h, const void* in, void* out, size_t n) {
  k_pel_convert<src, dst><<<cell_blocks(h), kThreads, 0, h->stream>>>(
      static_cast<const src*>(in), static_cast<dst*>(out), n);
  h->launches++;
}

// The grid-wide adaptive ode_solver on the device state (real) with the
// handle's PAR: rhs, then attempts whose decision is read back.
template <typename real>
int grid_adaptive(pel_handle* h, real* conc, double hs, long long& attempts) {
  Args<real> a = make_args<real>(h, hs, hs);
  PK(h->d_rhs.alloc(NTR * h->cells() * sizeof(real)), "rhs buffer");  // grid path only
  real* rhs = h->d_rhs.as<real>();
  const int cb = cell_blocks(h);
  double dt_int = 0.0, dt_red = hs;
  real dtr = (real)hs;
  int att = 0;
  k_pel_rhs<real, real><<<cb, kThreads, 0, h->stream>>>(a, conc, rhs);
  h->launches++;
  while (dt_int < hs) {
    if (att >= h->prm.max_attempts) {
      h->h_stats->capped++;
      break;
    }
    att++;
    PK(cudaMemsetAsync(&a.stats->flag, 0, sizeof(int), h->stream), "flag reset");
    k_pel_test<real><<<cb, kThreads, 0, h->stream>>>(a, conc, rhs, dtr);
    h->launches++;
    int flag = 0;
    PK(cudaMemcpyAsync(&h->h_stats->flag, &a.stats->flag, sizeof(int), cudaMemcpyDeviceToHost,
                       h->stream),
       "flag read");
    PK(cudaStreamSynchronize(h->stream), "grid test");
    flag = h->h_stats->flag;
    if (flag && dt_red > h->prm.dt_min) {
      dt_red = dt_red * 0.25;
      dtr = dtr * real(0.25);
    } else {
      k_pel_accept<real><<<cb, kThreads, 0, h->stream>>>(a, conc, rhs, dtr);
      h->launches++;
      dt_int = dt_int + dt_red;
      h->h_stats->accepted++;
      double md;
      memcpy(&md, &h->h_stats->min_dt_bits, sizeof md);
      if (dt_red < md) memcpy(&h->h_stats->min_dt_bits, &dt_red, sizeof md);
      if (dt_int < hs) {
        k_pel_rhs<real, real><<<cb, kThreads, 0, h->stream>>>(a, conc, rhs);
        h->launches++;
      }
    }
  }
  attempts += att;
  if (att > h->h_stats->max_att) h->h_stats->max_att = att;
  PK(cudaGetLastError(), "grid adaptive");
  return SED_OK;
}

int need(pel_handle* h, bool grid, bool forcing, bool state, bool par) {
  if (grid && !h->have_grid) return h->fail(SED_E_STATE, "pel_set_grid not called");
  if (forcing && !h->have_forcing) return h->fail(SED_E_STATE, "pel_set_forcing not called");
  if (state && !h->have_state) return h->fail(SED_E_STATE, "no state: call pel_set_state");
  if (par && !h->have_par) return h->fail(SED_E_STATE, "no PAR: call pel_light first");
  return SED_OK;
}

template <typename real>
int upload_real(pel_handle* h, DevBuf& buf, const double* src, size_t n, const char* what) {
  std::vector<real> tmp(n);
  for (size_t i = 0; i < n; i++) tmp[i] = (real)src[i];
  PK(buf.alloc(n * sizeof(real)), what);
  PK(cudaMemcpyAsync(buf.p, tmp.data(), n * sizeof(real), cudaMemcpyHostToDevice, h->stream),
     what);
  PK(cudaStreamSynchronize(h->stream), what);  // tmp goes out of scope
  return SED_OK;
}

int upload(pel_handle* h, DevBuf& buf, const double* src, size_t n, const char* what) {
  return h->fp64() ? upload_real<double>(h, buf, src, n, what)
                   : upload_real<float>(h, buf, src, n, what);
}

// Collect the device statistics of a call (after its work on the stream).
int finish_stats(pel_handle* h, pel_stats* st, long long host_attempts, long long launches0,
                 int runs) {
  DevStats ds;
  memcpy(&ds, h->h_stats, sizeof ds);  // host-side counters of the grid path
  PK(cudaMemcpyAsync(h->h_stats, h->d_stats.p, sizeof(DevStats), cudaMemcpyDeviceToHost,
                     h->stream),
     "stats read");
  PK(cudaEventRecord(h->ev1, h->stream), "event");
  PK(cudaStreamSynchronize(h->stream), "step");
  const DevStats& dv = *h->h_stats;
  if (st) {
    memset(st, 0, sizeof *st);
    st->attempts = (long long)dv.attempts + host_attempts;
    st->accepted = (long long)dv.accepted + (long long)ds.accepted;
    st->column_steps = (long long)h->water_cols * runs;
    st->max_cell_attempts = dv.max_att > ds.max_att ? dv.max_att : ds.max_att;
    st->capped_cells = (int)(dv.capped + ds.capped);
    st->nan_cells = (int)dv.nan;
    st->gpu_launches = (int)(h->launches - launches0);
    double md;
    memcpy(&md, &ds.min_dt_bits, sizeof md);  // grid-wide path (host side)
    if (dv.mcut_full >= 0) md = std::fmin(md, std::ldexp(h->sched.h_full, -2 * dv.mcut_full));
    if (dv.mcut_last >= 0) md = std::fmin(md, std::ldexp(h->sched.h_last, -2 * dv.mcut_last));
    st->min_dt = md < 1e300 ? md : 0.0;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    st->device_ms = ms;
  }
  if (dv.nan) return h->fail(SED_E_NAN, "%llu NaN cells after ode_solver", dv.nan);
  if (dv.capped + ds.capped)
    return h->fail(SED_E_SUBSTEP_CAP, "%llu cell-steps reached max_attempts",
                   (unsigned long long)(dv.capped + ds.capped));
  return SED_OK;
}

// One Run or ode_solver call on `conc` (store: double for host-array calls,
// real for the device state).  The grid-wide adaptive path works on the
// device state, converting a double array in and out.
template <typename real, typename store>
int run_on(pel_handle* h, store* conc, double t_couple, double dt, int method, bool light,
           bool epi, long long& host_attempts) {
  if (method == SED_ADAPTIVE_EULER && h->prm.cut_scope == PEL_CUT_GLOBAL) {
    // works on a real array: the device state itself, or a scratch copy of
    // a host call's double array (the resident state is left alone)
    const bool same = (void*)conc == h->d_state.p;
    if (!same) PK(h->d_work.alloc(NTR * h->cells() * sizeof(real)), "work");
    real* st = same ? h->d_state.as<real>() : h->d_work.as<real>();
    if (!same) convert<store, real>(h, conc, st, NTR * h->cells());
    Args<real> a = make_args<real>(h, t_couple, dt);
    if (light) {
      k_pel_light<real, real><<<col_blocks(h), kThreads, 0, h->stream>>>(a, st);
      h->launches++;
      h->have_par = true;
    }
    double t = 0.0;
    while (t < t_couple) {
      const double hs = t + dt > t_couple ? t_couple - t : dt;
      int rc = grid_adaptive<real>(h, st, hs, host_attempts);
      if (rc) return rc;
      if (epi) {
        k_pel_epilogue<real><<<col_blocks(h), kThreads, 0, h->stream>>>(a, st, (real)hs);
        h->launches++;
      }
      t = t + hs;
    }
    if (!same) convert<real, store>(h, st, conc, NTR * h->cells());
  } else {
    Args<real> a = make_args<real>(h, t_couple, dt);
    if (light && epi) launch_run<real, store, true, true>(h, a, conc, method, h->stream);
    else launch_run<real, store, false, false>(h, a, conc, method, h->stream);
    if (light) h->have_par = true;
  }
  PK(cudaGetLastError(), "pelagic kernels");
  return SED_OK;
}

int check_method(pel_handle* h, int method, double t_couple, double dt) {
  if (method < SED_EULER || method > SED_RUNGE_KUTTA_4_38)
    return h->fail(SED_E_ARG, "method must be 0..3");
  if (!(dt > 0.0) || !(t_couple > 0.0) || !std::isfinite(dt) || !std::isfinite(t_couple))
    return h->fail(SED_E_ARG, "time steps must be positive and finite");
  if (t_couple / dt > 1e7) return h->fail(SED_E_ARG, "too many internal steps per Run");
  return SED_OK;
}

int ensure_pipeline(pel_handle* h) {
  if (h->s_in) return SED_OK;
  PK(cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking), "stream");
  PK(cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking), "stream");
  for (auto& st : h->s_cmp) PK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
  PK(cudaEventCreateWithFlags(&h->e_start, cudaEventDisableTiming), "event");
  PK(cudaEventCreateWithFlags(&h->e_done, cudaEventDisableTiming), "event");
  for (int c = 0; c < 8; c++) {
    PK(cudaEventCreateWithFlags(&h->e_in[c], cudaEventDisableTiming), "event");
    PK(cudaEventCreateWithFlags(&h->e_cmp[c], cudaEventDisableTiming), "event");
  }
  return SED_OK;
}

// A Run or ode_solver call on the caller's host array with the copies in
// flight: the grid is cut into 8 column ranges; range c's host->device copy
// (one 2-D copy of its columns in every [tracer][layer] row), its step (on
// its own stream) and its device->host copy are ordered by events, so one
// range arrives while another is stepped and a third leaves.  The ranges
// are disjoint in the staging array, in conc and in the water-column list.
template <typename real>
int host_pipelined(pel_handle* h, double* conc, double t_couple, double dt, int method,
                   bool light, bool epi) {
  int rc = ensure_pipeline(h);
  if (rc) return rc;
  const int nch = 8;
  const size_t pitch = (size_t)h->ncol * sizeof(double), rows = (size_t)NTR * h->K;
  double* stage = h->d_stage.as<double>();
  PK(cudaEventRecord(h->e_start, h->stream), "event");
  PK(cudaStreamWaitEvent(h->s_in, h->e_start, 0), "wait");
  for (int c = 0; c < nch; c++) {
    const int col0 = (int)((long long)h->ncol * c / nch);
    const int col1 = (int)((long long)h->ncol * (c + 1) / nch);
    const size_t width = (size_t)(col1 - col0) * sizeof(double);
    if (width)
      PK(cudaMemcpy2DAsync(stage + col0, pitch, conc + col0, pitch, width, rows,
                           cudaMemcpyHostToDevice, h->s_in),
         "conc range in");
    PK(cudaEventRecord(h->e_in[c], h->s_in), "event");
    PK(cudaStreamWaitEvent(h->s_cmp[c], h->e_in[c], 0), "wait");
    const int w0 = (int)(std::lower_bound(h->wcols.begin(), h->wcols.end(), col0) - h->wcols.begin());
    const int w1 = (int)(std::lower_bound(h->wcols.begin(), h->wcols.end(), col1) - h->wcols.begin());
    if (w1 > w0) {
      Args<real> a = make_args<real>(h, t_couple, dt);
      a.wcols += w0;
      a.nwater = w1 - w0;
      if (light && epi) launch_run<real, double, true, true>(h, a, stage, method, h->s_cmp[c]);
      else launch_run<real, double, false, false>(h, a, stage, method, h->s_cmp[c]);
    }
    PK(cudaEventRecord(h->e_cmp[c], h->s_cmp[c]), "event");
    PK(cudaStreamWaitEvent(h->s_out, h->e_cmp[c], 0), "wait");
    if (width)
      PK(cudaMemcpy2DAsync(conc + col0, pitch, stage + col0, pitch, width, rows,
                           cudaMemcpyDeviceToHost, h->s_out),
         "conc range out");
  }
  PK(cudaEventRecord(h->e_done, h->s_out), "event");
  PK(cudaStreamWaitEvent(h->stream, h->e_done, 0), "wait");
  PK(cudaGetLastError(), "pelagic kernels");
  if (light) h->have_par = true;
  return SED_OK;
}

// A call on the caller's host array conc: copy in, work, copy out (in
// flight for the per-cell steppers, in turn for the grid-wide cut).
template <typename real>
int host_call(pel_handle* h, double* conc, double t_couple, double dt, int method, bool light,
              bool epi, pel_stats* st) {
  const size_t bytes = NTR * h->cells() * sizeof(double);
  PK(h->d_stage.alloc(bytes), "stage");
  int rc = reset_stats(h);
  if (rc) return rc;
  const long long l0 = h->launches;
  long long host_att = 0;
  PK(cudaEventRecord(h->ev0, h->stream), "event");
  if (!(method == SED_ADAPTIVE_EULER && h->prm.cut_scope == PEL_CUT_GLOBAL) && h->ncol >= 8) {
    rc = host_pipelined<real>(h, conc, t_couple, dt, method, light, epi);
    if (rc) return rc;
    return finish_stats(h, st, host_att, l0, 1);
  }
  PK(cudaMemcpyAsync(h->d_stage.p, conc, bytes, cudaMemcpyHostToDevice, h->stream), "conc in");
  rc = run_on<real, double>(h, h->d_stage.as<double>(), t_couple, dt, method, light, epi,
                            host_att);
  if (rc) return rc;
  PK(cudaMemcpyAsync(conc, h->d_stage.p, bytes, cudaMemcpyDeviceToHost, h->stream), "conc out");
  return finish_stats(h, st, host_att, l0, 1);
}

template <typename real>
int device_runs(pel_handle* h, double t_couple, double dt, int method, int nruns, pel_stats* st) {
  int rc = reset_stats(h);
  if (rc) return rc;
  const long long l0 = h->launches;
  long long host_att = 0;
  PK(cudaEventRecord(h->ev0, h->stream), "event");
  for (int r = 0; r < nruns; r++) {
    rc = run_on<real, real>(h, h->d_state.as<real>(), t_couple, dt, method, true, true, host_att);
    if (rc) return rc;
  }
  return finish_stats(h, st, host_att, l0, nruns);
}

}  // namespace

extern "C" {

int pel_default_params(pel_params* p) {
  if (!p) return SED_E_ARG;
  memset(p, 0, sizeof *p);
  // &gotm_npzd, examples/fabmsed_fabm0d/fabm.nml:57-79
  p->p0 = 0.0225;
  p->z0 = 0.0225;
  p->kc = 0.03;
  p->I_min = 25.0;
  p->rmax = 1.0;
  p->gmax = 0.2;
  p->Iv = 1.1;
  p->alpha = 1.35;
  p->rpn = 0.01;
  p->rzn = 0.01;
  p->rdn = 0.01;
  p->rpdu = 0.02;
  p->rpdl = 0.1;
  p->rzd = 0.02;
  // fabm_pelagic_component.F90:47, fabm_pelagic_driver.F90:65
  p->dt_min = 1.0e-8;
  p->relative_change_min = -0.9;
  p->background_extinction = 1.0 / 7.9;
  p->atol = 0.0;
  p->max_attempts = 4096;
  p->cut_scope = PEL_CUT_PER_CELL;
  p->precision = SED_FP32;
  p->device = 0;
  return SED_OK;
}

int pel_create(const pel_params* p, int inum, int jnum, int knum, int ntr, pel_handle** out) {
  if (!p || !out) return SED_E_ARG;
  *out = nullptr;
  if (inum < 1 || jnum < 1 || knum < 1 || knum > PEL_KMAX_LIMIT || ntr != NTR ||
      (long long)inum * jnum > (1ll << 30))
    return SED_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SED_E_NODEVICE;
  if (p->device < 0 || p->device >= ndev) return SED_E_ARG;
  pel_handle* h = new pel_handle();
  h->prm = *p;
  if (check_params(h, *p)) {
    delete h;
    return SED_E_ARG;
  }
  h->inum = inum;
  h->jnum = jnum;
  h->ncol = inum * jnum;
  h->K = knum;
  h->device = p->device;
  auto bad = [&](cudaError_t e) {
    if (e == cudaSuccess) return false;
    delete h;
    return true;
  };
  if (bad(cudaSetDevice(h->device))) return SED_E_CUDA;
  if (bad(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device)))
    return SED_E_CUDA;
  if (bad(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking))) return SED_E_CUDA;
  if (bad(cudaEventCreate(&h->ev0)) || bad(cudaEventCreate(&h->ev1))) return SED_E_CUDA;
  if (bad(cudaHostAlloc((void**)&h->h_stats, sizeof(DevStats), cudaHostAllocDefault)))
    return SED_E_NOMEM;
  const size_t cells = h->cells();
  if (h->d_stats.alloc(sizeof(DevStats)) != cudaSuccess ||
      h->d_par.alloc(cells * h->rsize()) != cudaSuccess ||
      h->d_state.alloc(NTR * cells * h->rsize()) != cudaSuccess) {
    delete h;
    return SED_E_NOMEM;
  }
  *out = h;
  return SED_OK;
}

void pel_destroy(pel_handle* h) { delete h; }

const char* pel_last_error(const pel_handle* h) { return h ? h->err.c_str() : "null handle"; }

int pel_set_grid(pel_handle* h, const double* layer_height, const int* mask) {
  if (!h) return SED_E_ARG;
  if (!layer_height) return h->fail(SED_E_ARG, "layer_height is NULL");
  const size_t cells = h->cells();
  std::vector<unsigned char> m(cells, 0);
  if (mask)
    for (size_t i = 0; i < cells; i++) m[i] = mask[i] > 0;
  for (size_t i = 0; i < cells; i++)
    if (!m[i] && !(layer_height[i] > 0.0 && std::isfinite(layer_height[i])))
      return h->fail(SED_E_ARG, "layer height of water cell %zu is not positive", i);
  cudaSetDevice(h->device);
  int rc = upload(h, h->d_h, layer_height, cells, "layer heights");
  if (rc) return rc;
  h->has_mask = mask != nullptr;
  if (mask) {
    PK(h->d_mask.alloc(cells), "mask");
    PK(cudaMemcpyAsync(h->d_mask.p, m.data(), cells, cudaMemcpyHostToDevice, h->stream), "mask");
    PK(cudaStreamSynchronize(h->stream), "mask");
  }
  std::vector<int> wcols;
  for (int c = 0; c < h->ncol; c++) {
    bool wet = false;
    for (int k = 0; k < h->K && !wet; k++) wet = !m[(size_t)k * h->ncol + c];
    if (wet) wcols.push_back(c);
  }
  h->water_cols = (int)wcols.size();
  h->wcols = wcols;
  PK(h->d_wcols.alloc((wcols.size() + 1) * sizeof(int)), "water columns");
  if (!wcols.empty()) {
    PK(cudaMemcpyAsync(h->d_wcols.p, wcols.data(), wcols.size() * sizeof(int),
                       cudaMemcpyHostToDevice, h->stream),
       "water columns");
    PK(cudaStreamSynchronize(h->stream), "water columns");
  }
  h->have_grid = true;
  h->have_par = false;
  return SED_OK;
}

int pel_set_forcing(pel_handle* h, const double* I_0, const double* albedo,
                    const double* bottom_flux, const double* surface_flux,
                    const double* soil_flux) {
  if (!h) return SED_E_ARG;
  if (!I_0) return h->fail(SED_E_ARG, "I_0 is NULL");
  cudaSetDevice(h->device);
  const size_t nc = h->ncol;
  for (size_t i = 0; i < nc; i++)
    if (!(I_0[i] >= 0.0) || !std::isfinite(I_0[i])) return h->fail(SED_E_ARG, "I_0 must be >= 0");
  int rc = upload(h, h->d_I0, I_0, nc, "I_0");
  if (!rc && albedo) rc = upload(h, h->d_alb, albedo, nc, "albedo");
  if (!rc && bottom_flux) rc = upload(h, h->d_bfl, bottom_flux, NTR * nc, "bottom flux");
  if (!rc && surface_flux) rc = upload(h, h->d_sfl, surface_flux, NTR * nc, "surface flux");
  if (!rc && soil_flux) rc = upload(h, h->d_soil, soil_flux, NTR * nc, "soil flux");
  if (rc) return rc;
  h->has_alb = albedo != nullptr;
  h->has_bfl = bottom_flux != nullptr;
  h->has_sfl = surface_flux != nullptr;
  h->has_soil = soil_flux != nullptr;
  h->have_forcing = true;
  h->have_par = false;
  return SED_OK;
}

int pel_set_open_boundary(pel_handle* h, const int* open_boundary,
                          const double* boundary_value, const int* has_value) {
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "pel_set_grid has not been called");
  cudaSetDevice(h->device);
  if (!open_boundary) {
    h->bvmask = 0;
    return SED_OK;
  }
  if (!boundary_value || !has_value)
    return h->fail(SED_E_ARG, "boundary_value and has_value are required");
  const size_t nc = h->ncol;
  unsigned mask = 0;
  for (int n = 0; n < NTR; n++)
    if (has_value[n]) mask |= 1u << n;
  std::vector<unsigned char> ob(nc);
  for (size_t c = 0; c < nc; c++) ob[c] = open_boundary[c] != 0;
  for (int n = 0; n < NTR; n++) {
    if (!(mask >> n & 1u)) continue;
    for (size_t c = 0; c < nc; c++)
      if (ob[c] && !std::isfinite(boundary_value[(size_t)n * nc + c]))
        return h->fail(SED_E_ARG, "boundary value %d of open column %zu is not finite", n, c);
  }
  PK(h->d_ob.alloc(nc), "open boundary");
  PK(cudaMemcpyAsync(h->d_ob.p, ob.data(), nc, cudaMemcpyHostToDevice, h->stream),
     "open boundary");
  PK(cudaStreamSynchronize(h->stream), "open boundary");  // ob goes out of scope
  int rc = upload(h, h->d_bv, boundary_value, NTR * nc, "boundary values");
  if (rc) return rc;
  h->bvmask = mask;
  return SED_OK;
}

int pel_set_state(pel_handle* h, const double* conc) {
  if (!h || !conc) return h ? h->fail(SED_E_ARG, "conc is NULL") : SED_E_ARG;
  cudaSetDevice(h->device);
  const size_t n = NTR * h->cells();
  if (h->fp64()) {
    PK(cudaMemcpyAsync(h->d_state.p, conc, n * sizeof(double), cudaMemcpyHostToDevice,
                       h->stream),
       "state in");
  } else {
    PK(h->d_stage.alloc(n * sizeof(double)), "stage");
    PK(cudaMemcpyAsync(h->d_stage.p, conc, n * sizeof(double), cudaMemcpyHostToDevice,
                       h->stream),
       "state in");
    convert<double, float>(h, h->d_stage.p, h->d_state.p, n);
  }
  PK(cudaStreamSynchronize(h->stream), "state in");
  h->have_state = true;
  return SED_OK;
}

int pel_get_state(pel_handle* h, double* conc) {
  if (!h || !conc) return h ? h->fail(SED_E_ARG, "conc is NULL") : SED_E_ARG;
  if (int rc = need(h, false, false, true, false)) return rc;
  cudaSetDevice(h->device);
  const size_t n = NTR * h->cells();
  if (h->fp64()) {
    PK(cudaMemcpyAsync(conc, h->d_state.p, n * sizeof(double), cudaMemcpyDeviceToHost,
                       h->stream),
       "state out");
  } else {
    PK(h->d_stage.alloc(n * sizeof(double)), "stage");
    convert<float, double>(h, h->d_state.p, h->d_stage.p, n);
    PK(cudaMemcpyAsync(conc, h->d_stage.p, n * sizeof(double), cudaMemcpyDeviceToHost,
                       h->stream),
       "state out");
  }
  PK(cudaStreamSynchronize(h->stream), "state out");
  return SED_OK;
}

int pel_light(pel_handle* h, const double* conc, double* par) {
  if (!h) return SED_E_ARG;
  if (int rc = need(h, true, true, conc == nullptr, false)) return rc;
  cudaSetDevice(h->device);
  const size_t cells = h->cells();
  if (h->fp64()) {
    Args<double> a = make_args<double>(h, 1.0, 1.0);
    const double* src = h->d_state.as<double>();
    if (conc) {
      PK(h->d_stage.alloc(NTR * cells * sizeof(double)), "stage");
      PK(cudaMemcpyAsync(h->d_stage.p, conc, NTR * cells * sizeof(double),
                         cudaMemcpyHostToDevice, h->stream),
         "conc in");
      src = h->d_stage.as<double>();
    }
    k_pel_light<double, double><<<col_blocks(h), kThreads, 0, h->stream>>>(a, src);
  } else {
    Args<float> a = make_args<float>(h, 1.0, 1.0);
    if (conc) {
      PK(h->d_stage.alloc(NTR * cells * sizeof(double)), "stage");
      PK(cudaMemcpyAsync(h->d_stage.p, conc, NTR * cells * sizeof(double),
                         cudaMemcpyHostToDevice, h->stream),
         "conc in");
      k_pel_light<float, double><<<col_blocks(h), kThreads, 0, h->stream>>>(
          a, h->d_stage.as<double>());
    } else {
      k_pel_light<float, float><<<col_blocks(h), kThreads, 0, h->stream>>>(
          a, h->d_state.as<float>());
    }
  }
  h->launches++;
  PK(cudaGetLastError(), "light");
  if (par) {
    if (h->fp64()) {
      PK(cudaMemcpyAsync(par, h->d_par.p, cells * sizeof(double), cudaMemcpyDeviceToHost,
                         h->stream),
         "par out");
    } else {
      std::vector<float> tmp(cells);
      PK(cudaMemcpyAsync(tmp.data(), h->d_par.p, cells * sizeof(float), cudaMemcpyDeviceToHost,
                         h->stream),
         "par out");
      PK(cudaStreamSynchronize(h->stream), "light");
      for (size_t i = 0; i < cells; i++) par[i] = tmp[i];
    }
  }
  PK(cudaStreamSynchronize(h->stream), "light");
  h->have_par = true;
  return SED_OK;
}

int pel_get_rhs(pel_handle* h, const double* conc, double* rhs) {
  if (!h || !conc || !rhs) return h ? h->fail(SED_E_ARG, "NULL array") : SED_E_ARG;
  if (int rc = need(h, true, true, false, true)) return rc;
  cudaSetDevice(h->device);
  const size_t n = NTR * h->cells();
  PK(h->d_stage.alloc(2 * n * sizeof(double)), "stage");
  double* in = h->d_stage.as<double>();
  double* out = in + n;
  PK(cudaMemcpyAsync(in, conc, n * sizeof(double), cudaMemcpyHostToDevice, h->stream), "conc in");
  if (h->fp64()) {
    k_pel_rhs<double, double><<<cell_blocks(h), kThreads, 0, h->stream>>>(
        make_args<double>(h, 1.0, 1.0), in, out);
  } else {
    k_pel_rhs<float, double><<<cell_blocks(h), kThreads, 0, h->stream>>>(
        make_args<float>(h, 1.0, 1.0), in, out);
  }
  h->launches++;
  PK(cudaGetLastError(), "rhs");
  PK(cudaMemcpyAsync(rhs, out, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "rhs out");
  PK(cudaStreamSynchronize(h->stream), "rhs");
  return SED_OK;
}

int pel_ode_solver(pel_handle* h, double* conc, double dt, int method, pel_stats* stats) {
  if (!h || !conc) return h ? h->fail(SED_E_ARG, "conc is NULL") : SED_E_ARG;
  if (int rc = check_method(h, method, dt, dt)) return rc;
  if (int rc = need(h, true, true, false, true)) return rc;
  cudaSetDevice(h->device);
  return h->fp64() ? host_call<double>(h, conc, dt, dt, method, false, false, stats)
                   : host_call<float>(h, conc, dt, dt, method, false, false, stats);
}

int pel_run(pel_handle* h, double* conc, double t_couple, double dt, int method,
            pel_stats* stats) {
  if (!h) return SED_E_ARG;
  if (int rc = check_method(h, method, t_couple, dt)) return rc;
  if (int rc = need(h, true, true, conc == nullptr, false)) return rc;
  cudaSetDevice(h->device);
  if (!conc)
    return h->fp64() ? device_runs<double>(h, t_couple, dt, method, 1, stats)
                     : device_runs<float>(h, t_couple, dt, method, 1, stats);
  return h->fp64() ? host_call<double>(h, conc, t_couple, dt, method, true, true, stats)
                   : host_call<float>(h, conc, t_couple, dt, method, true, true, stats);
}

int pel_step(pel_handle* h, double t_couple, double dt, int method, int nruns,
             pel_stats* stats) {
  if (!h) return SED_E_ARG;
  if (nruns < 1) return h->fail(SED_E_ARG, "nruns must be >= 1");
  if (int rc = check_method(h, method, t_couple, dt)) return rc;
  if (int rc = need(h, true, true, true, false)) return rc;
  cudaSetDevice(h->device);
  return h->fp64() ? device_runs<double>(h, t_couple, dt, method, nruns, stats)
                   : device_runs<float>(h, t_couple, dt, method, nruns, stats);
}

}  // extern "C"

int cpl::pel_view(pel_handle* h, PelView* v, bool need_state) {
  if (!h || !v) return SED_E_ARG;
  if (int rc = need(h, true, false, need_state, false)) return rc;
  v->state = h->have_state ? h->d_state.p : nullptr;
  v->fp64 = h->fp64();
  v->ncol = h->ncol;
  v->K = h->K;
  v->device = h->device;
  v->stream = h->stream;
  return SED_OK;
}

int cpl::pel_bottom_flux(pel_handle* h, void** bfl) {
  if (!h || !bfl) return SED_E_ARG;
  if (int rc = need(h, true, false, false, false)) return rc;
  if (!h->has_bfl) {
    const size_t bytes = NTR * (size_t)h->ncol * h->rsize();
    PK(h->d_bfl.alloc(bytes), "bottom flux");
    PK(cudaMemsetAsync(h->d_bfl.p, 0, bytes, h->stream), "bottom flux");
    PK(cudaStreamSynchronize(h->stream), "bottom flux");
    h->has_bfl = true;
  }
  *bfl = h->d_bfl.p;
  return SED_OK;
}
