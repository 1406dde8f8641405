// sed_kernels.cuh -- sm_103a kernels of the sediment-column solver
// (templates; sed_kernels_f32.cu and sed_kernels_f64.cu instantiate them).
//
// k_column_step: persistent kernel, one coupling step for every column.
//   Blocks pull tiles of TC consecutive column slots from a device work
//   counter (atomicAdd, no waits), stage the tile's state, coefficients and
//   forcing into shared memory with coalesced 16-byte loads, then each warp
//   pulls columns of the tile (shared-memory counter) and integrates one
//   column entirely in registers: per-column adaptive Euler (or Euler / RK4
//   / RK4 3/8), FP64 step bookkeeping, fused NaN check + clamp, FP64
//   budgets.  The tile is written back with coalesced stores.
// k_column_rhs:   the same staging, one right-hand side (get_rhs mirror and
//                 the grid-wide adaptive mode).
// k_trial / k_accept / k_epilogue: elementwise steps of the grid-wide cut.
// k_gather_* / k_scatter_* / k_prep_*: layout and precision conversion
//   between the reference's FP64 host arrays and the device layout.
#pragma once
#include "sed_device.cuh"
#include "sed_launch.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

namespace sed {

// ---------------------------------------------------------------------------
// shared-memory tile layout
template <typename real>
struct TileLayout {
  int tcp, kt;
  size_t conc, coef, cap, force, sflux, bud, nsub, total;
  __host__ __device__ TileLayout(int tc, int kt_, bool bc4, int ncoef) : kt(kt_) {
    tcp = tc + 16 / (int)sizeof(real);  // row pad keeps 16-byte alignment
    size_t r = sizeof(real);
    conc = 0;
    coef = conc + (size_t)NTR * kt * tcp * r;
    cap = coef + (size_t)ncoef * kt * tcp * r;
    force = cap + (bc4 ? (size_t)kt * tcp * r : 0);
    sflux = force + (size_t)NFORCE * tcp * r;
    bud = sflux + (size_t)NDISS * tcp * r;
    bud = (bud + 15) & ~(size_t)15;
    nsub = bud + (size_t)4 * tc * sizeof(double);
    total = nsub + (size_t)tc * sizeof(int);
    total = (total + 15) & ~(size_t)15;
  }
};

template <typename real>
size_t tile_smem_bytes(int tc, int lpl, bool bc4, int kind, bool bio3) {
  (void)kind;
  return TileLayout<real>(tc, 32 * lpl, bc4, coef_rows<real>(bio3)).total;
}

// 16-byte global -> shared copy in flight (cp.async, L2 only): a thread
// issues all its pieces of a tile before waiting once, instead of one
// load-to-use latency per piece.  Both addresses are 16-byte aligned: tiles
// start at multiples of 8 slots, rows are padded to 16 bytes.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Row walk of a staging copy: the 16-byte pieces of rows [0, rows) of tc
// reals, nthreads threads.  When the pieces per row (vpr) are a power of two
// dividing nthreads (every tile width and block size the launches use), a
// thread keeps its piece index v and steps its row by nthreads / vpr, so the
// per-piece index arithmetic is a few adds; otherwise each piece index is
// divided out.  f(row, v) copies one piece.
template <typename F>
__device__ __forceinline__ void walk_pieces(int rows, int vpr, int tid, int nthreads, F f) {
  if ((vpr & (vpr - 1)) == 0 && nthreads % vpr == 0) {
    const int sh = __ffs(vpr) - 1;
    const int v = tid & (vpr - 1);
    const int rstep = nthreads >> sh;
    for (int row = tid >> sh; row < rows; row += rstep) f(row, v);
  } else {
    for (int i = tid; i < rows * vpr; i += nthreads) {
      const int row = i / vpr;
      f(row, i - row * vpr);
    }
  }
}

// Copy `rows` rows of tc reals between global (row stride gstride, first
// element at gbase + row_index*gstride) and shared memory (row stride tcp).
// To shared memory the copies are asynchronous: cp_async_wait_all before
// the block barrier that publishes them.
template <typename real, bool TO_SHARED>
__device__ __forceinline__ void copy_rows(real* sm, real* gbase, size_t gstride,
                                          int rows, int tc, int tcp,
                                          int row_step_global, int tid,
                                          int nthreads) {
  constexpr int EPV = 16 / sizeof(real);  // elements per 16-byte vector
  walk_pieces(rows, tc / EPV, tid, nthreads, [&](int row, int v) {
    real* g = gbase + (size_t)row * row_step_global * gstride + v * EPV;
    real* s = sm + (size_t)row * tcp + v * EPV;
    if (TO_SHARED)
      cp_async16(s, g);
    else
      *reinterpret_cast<uint4*>(g) = *reinterpret_cast<const uint4*>(s);
  });
}

// rows of a [nrow_groups][kmax][nslot] array restricted to k < kt:
// copies group g, layer k for all g < ngroups, k < kt.  The (g, k) of a
// row follows the row walk incrementally.
template <typename real, bool TO_SHARED>
__device__ __forceinline__ void copy_grouped(real* sm, real* g0, int ngroups,
                                             int kt, int KT, int kmax,
                                             size_t nslot, int tc, int tcp,
                                             int tid, int nthreads) {
  constexpr int EPV = 16 / sizeof(real);
  int g = 0, k = 0, at = 0;  // the row (g, k) = g kt + k last visited
  walk_pieces(ngroups * kt, tc / EPV, tid, nthreads, [&](int row, int v) {
    k += row - at;
    at = row;
    if (k >= kt) {
      const int q = k < 2 * kt ? 1 : k / kt;
      g += q;
      k -= q * kt;
    }
    real* gp = g0 + ((size_t)g * kmax + k) * nslot + v * EPV;
    real* sp = sm + ((size_t)g * KT + k) * tcp + v * EPV;
    if (TO_SHARED)
      cp_async16(sp, gp);
    else
      *reinterpret_cast<uint4*>(gp) = *reinterpret_cast<const uint4*>(sp);
  });
}

// ---------------------------------------------------------------------------
template <typename real, int LPL, bool BC4, bool BIO3>
__device__ __forceinline__ void load_lane(Lane<real, LPL, BC4>& lc,
                                          real (&C)[LPL][NTR],
                                          const real* s_conc,
                                          const real* s_coef,
                                          const real* s_cap,
                                          const real* s_force, int j, int KT,
                                          int tcp, int lane, int K,
                                          int mol_mode, int bcup_d) {
  const real bioT = s_force[0 * tcp + j];
  const real dmul = s_force[1 * tcp + j];
#pragma unroll
  for (int n = 0; n < 1; n++) {
    lc.bnd_s = s_force + 2 * tcp + j;
    lc.bnd_stride = tcp;
  }
  real cap[LPL];
  real ad0 = real(0);  // the dissolved surface conductance (FP32 form, lane 0)
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const int L = s * 32 + lane;
    const bool act = L < K;
    const int Lc = act ? L : 0;
    auto row = [&](int r) { return s_coef[(r * KT + Lc) * tcp + j]; };
    if constexpr (std::is_same<real, double>::value) {
      // the reference's operands: get_rhs :652-653 and :682-683
      const double phi = row(0), phi_i = row(1), bf = row(2), dz = row(3);
      const double len = row(4), mol1 = row(5);
      const double pre = bioT / 86400.0 / 10000.0 * (1.0 - phi_i);
      const double diff = pre * bf;
      const double mol = mol_mode == 1 ? mol1 : dmul * phi_i / 86400.0 / 10000.0;
      if constexpr (BIO3) {
        lc.e1[s] = act ? row(NCOEF64) : 1.0;
        lc.e2[s] = act ? row(NCOEF64 + 1) : 1.0;
        lc.pre[s] = act ? pre : 0.0;
        lc.mol[s] = act ? mol : 0.0;
        if (s == 0) lc.cum = s_coef[((NCOEF64 + 2) * KT + 0) * tcp + j];
      }
      lc.phi[s] = act ? phi : 1.0;
      lc.dz[s] = act ? dz : 1.0;
      lc.len[s] = act ? len : 1.0;
      lc.Dp[s] = act ? diff : 0.0;
      lc.Dd[s] = act ? diff + mol : 0.0;
      lc.vol[s] = act ? phi * dz : 0.0;
      lc.ivol[s] = 0.0;
      lc.ad[s] = 0.0;
      lc.ap[s] = 0.0;
    } else {
      const real phi = row(0), vol = row(1), gb = row(2), gm = row(3);
      // the surface interface (L = 0) carries no conductance: its flux is
      // the lane's ab - beta C (below)
      const bool inner = act && L != 0;
      const real d = fm(bioT, gb, dmul * gm);
      lc.phi[s] = act ? phi : real(0);
      lc.vol[s] = act ? vol : real(0);
      lc.ivol[s] = act ? real(1) / vol : real(0);
      lc.ap[s] = inner ? bioT * gb : real(0);
      lc.ad[s] = inner ? d : real(0);
      if (s == 0 && L == 0) ad0 = d;
      if constexpr (BIO3) {
        lc.wc[s] = act ? phi / (real(1) - phi) : real(0);
        lc.gz[s] = act ? row(NCOEF) : real(0);
        lc.hw[s] = act ? row(NCOEF + 1) : real(0);
        lc.gb3[s] = act ? gb : real(0);
        lc.dm[s] = act ? dmul * gm : real(0);
      }
    }
    cap[s] = (BC4 && act) ? s_cap[Lc * tcp + j] : real(0);
#pragma unroll
    for (int n = 0; n < NTR; n++)
      C[s][n] = act ? s_conc[(n * KT + Lc) * tcp + j] : real(0);
  }
  if constexpr (std::is_same<real, double>::value) {
    cascade_ref<LPL, BC4>(lc, cap, lane, K);
  } else {
    cascade_sources<real, LPL, BC4>(lc, cap, lane, K);
    // surface fluxes: particulates and BcUp 1 the given flux, BcUp 2 the
    // conductance times (bottom water - C0), BcUp 3 none
    const bool top = lane == 0;
    lc.alpha_p = top ? real(1) : real(0);
    lc.alpha_d = !top ? real(0) : (bcup_d == 2 ? ad0 : (bcup_d == 1 ? real(1) : real(0)));
    lc.beta = (top && bcup_d == 2) ? ad0 : real(0);
  }
}

// A block's surface rows (FP32 form): warp w's alpha b row at w SURF_ROW,
// the zero row at SURF_ZERO.  The zero row starts in bank 2 of 32, so a
// load of one tracer pair by lane 0 (its warp's row) and by the other lanes
// (the zero row) touches disjoint banks for every warp of a 256-thread block.
constexpr int SURF_ZERO = 8 * SURF_ROW + 2;
constexpr int SURF_FLOATS = SURF_ZERO + SURF_ROW;

// The column's alpha b row, formed once per column by lane 0 with the same
// rounding as the product it replaces, and read by every right-hand side.
template <typename real, int LPL, bool BC4>
__device__ __forceinline__ void set_surface_row(Lane<real, LPL, BC4>& lc, float* s_surf,
                                                int warp, int lane) {
  if constexpr (std::is_same<real, float>::value) {
    float* row = s_surf + warp * SURF_ROW;
    __syncwarp();  // the previous column's right-hand sides are done with the row
    if (lane == 0) {
#pragma unroll
      for (int n = 0; n < NTR; n++) row[n] = (n < NPART ? lc.alpha_p : lc.alpha_d) * lc.bnd(n);
    }
    __syncwarp();
    lc.ab_sa = (unsigned)__cvta_generic_to_shared(lane == 0 ? row : s_surf + SURF_ZERO);
  }
}

// The right-hand side used by the steppers: folded FP32 form, or the
// reference-order FP64 form.
template <typename real, int LPL, bool BC4, bool BIO3>
__device__ __forceinline__ void rhs_any(const Params<real>& p,
                                        const Lane<real, LPL, BC4>& lc, int lane,
                                        int K, const real (&C)[LPL][NTR],
                                        real (&R)[LPL][NTR], real (&ftop)[NTR],
                                        real (&dn)[LPL]) {
  if constexpr (std::is_same<real, double>::value)
    column_rhs_ref<LPL, BC4, BIO3>(p, lc, lane, K, C, R, ftop, dn);
  else
    column_rhs<real, LPL, BC4, BIO3>(p, lc, lane, K, C, R, ftop, dn);
}

// c + dt r (one rounding in FP32 via FMA; the reference's multiply then add
// in FP64) and the sign of c1 - keep c (:121).
__device__ __forceinline__ float upd(float c, float dt, float r) { return fmaf(dt, r, c); }
__device__ __forceinline__ double upd(double c, double dt, double r) { return c + dt * r; }
__device__ __forceinline__ bool below_keep(float c1, float keep, float c, float natol) {
  return fmaf(-keep, c, c1) < natol;
}
__device__ __forceinline__ bool below_keep(double c1, double keep, double c, double natol) {
  return c1 - keep * c < natol;
}

// FP64 column inventories of the P and N pools (warp-reduced).
template <int LPL, bool BC4>
__device__ __forceinline__ void inventories(const Lane<double, LPL, BC4>& lc,
                                            const double (&C)[LPL][NTR],
                                            double& invP, double& invN) {
  double p = 0.0, nn = 0.0;
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const double v = lc.vol[s];
    p += v * (C[s][T_FDETP] + C[s][T_ADSP] + C[s][T_PO4]);
    nn += v * (C[s][T_FDETN] + C[s][T_SDETN] + C[s][T_NO3] + C[s][T_NH4]);
  }
  invP = warp_sum(p);
  invN = warp_sum(nn);
}

// Double-word (hi + lo) FP32 arithmetic: error-free TwoSum / TwoProduct
// (Knuth, Dekker) keep ~48 significant bits, so the FP32 kernels carry their
// budget reductions at about FP64 accuracy without the FP64 pipe (GB300
// issues FP64 at a small fraction of its FP32 rate).
struct DW {
  float hi, lo;
};
__device__ __forceinline__ DW dw_add(DW x, DW y) {
  const float s = x.hi + y.hi;
  const float bp = s - x.hi;
  const float e = (x.hi - (s - bp)) + (y.hi - bp) + (x.lo + y.lo);
  const float hi = s + e;
  return DW{hi, e - (hi - s)};
}
__device__ __forceinline__ DW dw_prod(float a, float b) {
  const float p = a * b;
  return DW{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ DW dw_from(float a) { return DW{a, 0.0f}; }
__device__ __forceinline__ DW dw_warp_sum(DW x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DW y{__shfl_xor_sync(FULL, x.hi, o), __shfl_xor_sync(FULL, x.lo, o)};
    x = dw_add(x, y);
  }
  return x;
}
__device__ __forceinline__ double dw_value(DW x) { return (double)x.hi + (double)x.lo; }

// sum_k vol_k * (sum of the pool's tracers), double-word, warp-reduced
template <int LPL, bool BC4, int NP>
__device__ __forceinline__ DW dw_inventory(const Lane<float, LPL, BC4>& lc,
                                           const float (&C)[LPL][NTR],
                                           const int (&idx)[NP]) {
  DW acc = dw_from(0.0f);
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    DW pool = dw_from(C[s][idx[0]]);
#pragma unroll
    for (int q = 1; q < NP; q++) pool = dw_add(pool, dw_from(C[s][idx[q]]));
    DW prod = dw_prod(lc.vol[s], pool.hi);
    prod.lo = fmaf(lc.vol[s], pool.lo, prod.lo);
    acc = dw_add(acc, prod);
  }
  return dw_warp_sum(acc);
}

struct ColResult {
  int attempts;
  int accepted;
  int capped;
  int nan;
  double min_dt;
};

// Two compensated running sums (Knuth's TwoSum: t = s + x, bp = t - s,
// c += (s - (t - bp)) + (x - bp), s = t) in packed FP32x2 arithmetic, each
// component rounding as the scalar operation would: the per-substep
// surface-flux integrals of the P and N pools carry their rounding error
// along without FP64 arithmetic inside the substep loop.
struct CompSum2 {
  float2 s, c;
  __device__ __forceinline__ void zero() { s = make_float2(0.0f, 0.0f); c = s; }
  __device__ __forceinline__ void add(float2 x) {
    const float2 t = __fadd2_rn(s, x);
    const float2 bp = sub2(t, s);
    const float2 tb = sub2(t, bp);
    const float2 e = __fadd2_rn(sub2(s, tb), sub2(x, bp));
    c = __fadd2_rn(c, e);
    s = t;
  }
  __device__ __forceinline__ double value_x() const { return (double)s.x + (double)c.x; }
  __device__ __forceinline__ double value_y() const { return (double)s.y + (double)c.y; }
};

// Budget bookkeeping of one column over one coupling step: column
// inventories of the P and N pools at the start and end of the step (warp
// reductions), the surface inflow of both pools and the N lost to
// denitrification (0.8 mol N per mol C) accumulated per substep.  FP64
// state: FP64 throughout.  FP32 state: double-word FP32 sums, converted to
// FP64 once per column-step.
template <typename real, int LPL, bool BC4>
struct Budget;

template <int LPL, bool BC4>
struct Budget<double, LPL, BC4> {
  double inv0P, inv0N, inP, inN;
  double n2[LPL];
  __device__ __forceinline__ void start(const Params<double>& p,
                                        const Lane<double, LPL, BC4>& lc,
                                        const double (&C)[LPL][NTR]) {
    inP = 0.0; inN = 0.0; inv0P = 0.0; inv0N = 0.0;
#pragma unroll
    for (int s = 0; s < LPL; s++) n2[s] = 0.0;
    if (p.budgets) inventories<LPL, BC4>(lc, C, inv0P, inv0N);
  }
  __device__ __forceinline__ void account(const Params<double>& p, double w,
                                          const double (&ftop)[NTR],
                                          const double (&dn)[LPL]) {
    if (!p.budgets) return;
    inP += w * (ftop[T_FDETP] + ftop[T_ADSP] + ftop[T_PO4]);
    inN += w * (ftop[T_FDETN] + ftop[T_SDETN] + ftop[T_NO3] + ftop[T_NH4]);
#pragma unroll
    for (int s = 0; s < LPL; s++) n2[s] += w * 0.8 * dn[s];
  }
  __device__ __forceinline__ void finish(const Params<double>& p,
                                         const Lane<double, LPL, BC4>& lc,
                                         const double (&C)[LPL][NTR],
                                         double (&bud)[4], int lane) {
    if (!p.budgets) return;
    double inv1P, inv1N;
    inventories<LPL, BC4>(lc, C, inv1P, inv1N);
    double loss = 0.0;
#pragma unroll
    for (int s = 0; s < LPL; s++) loss += lc.vol[s] * n2[s];
    loss = warp_sum(loss);
    const double fP = __shfl_sync(FULL, inP, 0);
    const double fN = __shfl_sync(FULL, inN, 0);
    bud[0] = inv1P;
    bud[1] = inv1P - inv0P - fP;
    bud[2] = inv1N;
    bud[3] = inv1N - inv0N - fN + loss;
  }
};

template <int LPL, bool BC4>
struct Budget<float, LPL, BC4> {
  DW inv0P, inv0N;
  CompSum2 inPN;  // surface inflow of the P (x) and N (y) pools
  float n2[LPL];
  __device__ __forceinline__ void start(const Params<float>& p,
                                        const Lane<float, LPL, BC4>& lc,
                                        const float (&C)[LPL][NTR]) {
    inPN.zero();
#pragma unroll
    for (int s = 0; s < LPL; s++) n2[s] = 0.0f;
    if (p.budgets) {
      constexpr int iP[3] = {T_FDETP, T_ADSP, T_PO4};
      constexpr int iN[4] = {T_FDETN, T_SDETN, T_NO3, T_NH4};
      inv0P = dw_inventory<LPL, BC4, 3>(lc, C, iP);
      inv0N = dw_inventory<LPL, BC4, 4>(lc, C, iN);
    }
  }
  __device__ __forceinline__ void account(const Params<float>& p, float w,
                                          const float (&ftop)[NTR],
                                          const float (&dn)[LPL]) {
    if (!p.budgets) return;
    // P: (FDETP + ADSP) + PO4, N: ((FDETN + SDETN) + NO3) + NH4, in pairs
    const float2 a = __fadd2_rn(make_float2(ftop[T_FDETP], ftop[T_FDETN]),
                                make_float2(ftop[T_ADSP], ftop[T_SDETN]));
    const float2 b = __fadd2_rn(a, make_float2(ftop[T_PO4], ftop[T_NO3]));
    inPN.add(__fmul2_rn(make_float2(w, w), make_float2(b.x, b.y + ftop[T_NH4])));
#pragma unroll
    for (int s = 0; s < LPL; s++) n2[s] = fmaf(w * 0.8f, dn[s], n2[s]);
  }
  __device__ __forceinline__ void finish(const Params<float>& p,
                                         const Lane<float, LPL, BC4>& lc,
                                         const float (&C)[LPL][NTR],
                                         double (&bud)[4], int lane) {
    if (!p.budgets) return;
    constexpr int iP[3] = {T_FDETP, T_ADSP, T_PO4};
    constexpr int iN[4] = {T_FDETN, T_SDETN, T_NO3, T_NH4};
    const DW inv1P = dw_inventory<LPL, BC4, 3>(lc, C, iP);
    const DW inv1N = dw_inventory<LPL, BC4, 4>(lc, C, iN);
    DW loss = dw_from(0.0f);
#pragma unroll
    for (int s = 0; s < LPL; s++) loss = dw_add(loss, dw_prod(lc.vol[s], n2[s]));
    loss = dw_warp_sum(loss);
    if (lane == 0) {  // lane 0 holds the surface inflow sums
      const double v1P = dw_value(inv1P), v1N = dw_value(inv1N);
      bud[0] = v1P;
      bud[1] = v1P - dw_value(inv0P) - inPN.value_x();
      bud[2] = v1N;
      bud[3] = v1N - dw_value(inv0N) - inPN.value_y() + dw_value(loss);
    }
  }
};

// Component epilogue: NaN check (:1718-1723) and clamp (:1726-1732).
template <typename real, int LPL>
__device__ __forceinline__ int epilogue(const Params<real>& p, int lane, int K,
                                        real (&C)[LPL][NTR]) {
  if (!p.epilogue) return 0;
  int nan = 0;
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    const bool act = s * 32 + lane < K;
#pragma unroll
    for (int n = 0; n < NTR; n++) {
      const real v = C[s][n];
      if (act && v != v) nan++;
      else if (act && v < p.minimum[n]) C[s][n] = p.minimum[n];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nan += __shfl_xor_sync(FULL, nan, o);
  return nan;
}

// One attempt of the adaptive Euler step at substep dtr: whether any of
// the lane's cells fails the positivity test c1 - (1+rcm) c < -atol with
// c1 = c + dtr r (:117-121).  Lanes past the column hold zeros: c1 = 0
// never falls below -atol.
template <typename real, int LPL>
__device__ __forceinline__ bool attempt_fails(const Params<real>& p, const real (&C)[LPL][NTR],
                                              const real (&R)[LPL][NTR], real dtr) {
  bool bad = false;
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    if constexpr (std::is_same<real, float>::value) {
      // tracer pairs in packed FP32x2 FMAs (per component the scalar's
      // rounding), tracer 10 alone
#pragma unroll
      for (int n = 0; n + 1 < NTR; n += 2) {
        const float2 c = make_float2(C[s][n], C[s][n + 1]);
        const float2 c1 = __ffma2_rn(make_float2(dtr, dtr),
                                     make_float2(R[s][n], R[s][n + 1]), c);
        const float2 t = __ffma2_rn(make_float2(-p.keep, -p.keep), c, c1);
        bad |= (t.x < p.natol) | (t.y < p.natol);
      }
      bad |= below_keep(upd(C[s][NTR - 1], dtr, R[s][NTR - 1]), p.keep, C[s][NTR - 1],
                        p.natol);
    } else {
#pragma unroll
      for (int n = 0; n < NTR; n++) {
        const real c1 = upd(C[s][n], dtr, R[s][n]);
        // sign of c1 - (1+rcm) c; in FP32 exact for the operands (one FMA)
        bad |= below_keep(c1, p.keep, C[s][n], p.natol);
      }
    }
  }
  return bad;
}

// The accepted attempt: C = C + dtr R (:137), the same roundings as the test.
template <typename real, int LPL>
__device__ __forceinline__ void attempt_apply(real (&C)[LPL][NTR], const real (&R)[LPL][NTR],
                                              real dtr) {
#pragma unroll
  for (int s = 0; s < LPL; s++) {
    if constexpr (std::is_same<real, float>::value) {
#pragma unroll
      for (int n = 0; n + 1 < NTR; n += 2) {
        const float2 c1 = __ffma2_rn(make_float2(dtr, dtr), make_float2(R[s][n], R[s][n + 1]),
                                     make_float2(C[s][n], C[s][n + 1]));
        C[s][n] = c1.x;
        C[s][n + 1] = c1.y;
      }
      C[s][NTR - 1] = upd(C[s][NTR - 1], dtr, R[s][NTR - 1]);
    } else {
#pragma unroll
      for (int n = 0; n < NTR; n++) C[s][n] = upd(C[s][n], dtr, R[s][n]);
    }
  }
}

// ADAPTIVE_EULER (solver_library.F90:104-140) on one column, cut decided by
// the column's own cells.  A rejected attempt re-evaluates get_rhs at the
// same state in the reference, which yields the same rhs, so it is reused.
//
// Time bookkeeping: the reference sums dt_int += dt_red in FP64 with
// dt_red = dt/4^m.  When the host has shown that every such partial sum is
// exact in FP64 (p.ticks), the same decisions are taken with integer ticks
// of dt/4^mstop (mstop = first level with dt/4^m <= dt_min), which keeps the
// loop off the FP64 pipe; otherwise the FP64 sums are kept.
template <typename real, int LPL, bool BC4, bool BIO3, bool TICKS>
__device__ __forceinline__ ColResult solve_adaptive(
    const Params<real>& p, const Lane<real, LPL, BC4>& lc, int lane, int K,
    real (&C)[LPL][NTR], real (&ftop)[NTR], double dt, double (&bud)[4]) {
  real R[LPL][NTR];
  real dn[LPL];
  ColResult res{0, 0, 0, 0, 1e300};
  Budget<real, LPL, BC4> B;
  B.start(p, lc, C);
  unsigned long long t = 0, T = 0, inc = 0;
  double dt_int = 0.0, dt_red = dt;
  if (TICKS) { T = 1ull << (2 * p.mstop); inc = T; }
  int m = 0, mmax = -1;
  real dtr = (real)dt;
  rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, C, R, ftop, dn);
  while (TICKS ? (t < T) : (dt_int < dt)) {
    if (res.attempts >= p.max_attempts) { res.capped = 1; break; }
    res.attempts++;
    const bool reject = __any_sync(FULL, attempt_fails<real, LPL>(p, C, R, dtr));
    const bool can_cut = TICKS ? (m < p.mstop) : (dt_red > p.dt_min);
    if (reject && can_cut) {
      m++;
      dtr = dtr * real(0.25);
      if (TICKS) inc >>= 2;
      else dt_red = dt_red * 0.25;
    } else {
      B.account(p, dtr, ftop, dn);
      attempt_apply<real, LPL>(C, R, dtr);
      if (TICKS) t += inc;
      else dt_int = dt_int + dt_red;
      res.accepted++;
      mmax = m > mmax ? m : mmax;
      if (TICKS ? (t < T) : (dt_int < dt))
        rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, C, R, ftop, dn);
    }
  }
  if (mmax >= 0) res.min_dt = ldexp(dt, -2 * mmax);
  B.finish(p, lc, C, bud, lane);
  res.nan = epilogue<real, LPL>(p, lane, K, C);
  return res;
}

// The gate of the surrogate step: the adaptive Euler step's first attempt,
// the whole coupling step dt at once.  If it is accepted (or no cut is
// allowed) the column is finished exactly as solve_adaptive finishes it
// after that one attempt; otherwise the result has attempts = -1, the state
// C untouched and no budget or epilogue work.
template <typename real, int LPL, bool BC4, bool BIO3>
__device__ __forceinline__ ColResult probe_column(
    const Params<real>& p, const Lane<real, LPL, BC4>& lc, int lane, int K,
    real (&C)[LPL][NTR], real (&ftop)[NTR], double dt, double (&bud)[4]) {
  real R[LPL][NTR];
  real dn[LPL];
  ColResult res{-1, 0, 0, 0, 1e300};
  const real dtr = (real)dt;
  rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, C, R, ftop, dn);
  const bool reject = __any_sync(FULL, attempt_fails<real, LPL>(p, C, R, dtr));
  // a cut is allowed at the first attempt (m = 0 < mstop, or dt > dt_min)
  const bool can_cut = p.ticks ? (0 < p.mstop) : (dt > p.dt_min);
  if (reject && can_cut) return res;
  Budget<real, LPL, BC4> B;
  B.start(p, lc, C);
  B.account(p, dtr, ftop, dn);
  attempt_apply<real, LPL>(C, R, dtr);
  res.attempts = 1;
  res.accepted = 1;
  res.min_dt = dt;
  B.finish(p, lc, C, bud, lane);
  res.nan = epilogue<real, LPL>(p, lane, K, C);
  return res;
}

// EULER (:99-102), RUNGE_KUTTA_4 (:142-163), RUNGE_KUTTA_4_38 (:164-185),
// each stage combined in the reference's operation order.
template <typename real, int LPL, bool BC4, bool BIO3>
__device__ __forceinline__ ColResult solve_fixed(
    const Params<real>& p, const Lane<real, LPL, BC4>& lc, int lane, int K,
    real (&C)[LPL][NTR], real (&ftop)[NTR], double dt, int method,
    double (&bud)[4]) {
  real R[LPL][NTR];
  real dn[LPL];
  ColResult res{1, 1, 0, 0, dt};
  Budget<real, LPL, BC4> B;
  B.start(p, lc, C);
  const real dtr = (real)dt;
  if (method == 0) {
    rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, C, R, ftop, dn);
    B.account(p, dtr, ftop, dn);
#pragma unroll
    for (int s = 0; s < LPL; s++)
#pragma unroll
      for (int n = 0; n < NTR; n++) C[s][n] = upd(C[s][n], dtr, R[s][n]);
  } else {
    const bool rk38 = method == 3;
    const real third = real(1.0 / 3.0);
    real Cs[LPL][NTR], R0[LPL][NTR], R1[LPL][NTR], R2[LPL][NTR];
    // stage 1: rhs0 at conc
    rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, C, R0, ftop, dn);
    B.account(p, (real)(rk38 ? dt / 8.0 : dt / 6.0), ftop, dn);
#pragma unroll
    for (int s = 0; s < LPL; s++)
#pragma unroll
      for (int n = 0; n < NTR; n++)
        Cs[s][n] = rk38 ? C[s][n] + third * dtr * R0[s][n]
                        : C[s][n] + real(0.5) * dtr * R0[s][n];
    // stage 2: rhs1 at c1
    rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, Cs, R1, ftop, dn);
    B.account(p, (real)(rk38 ? 3.0 * dt / 8.0 : dt / 3.0), ftop, dn);
#pragma unroll
    for (int s = 0; s < LPL; s++)
#pragma unroll
      for (int n = 0; n < NTR; n++)
        Cs[s][n] = rk38 ? C[s][n] + dtr * (R1[s][n] - third * R0[s][n])
                        : C[s][n] + real(0.5) * dtr * R1[s][n];
    // stage 3: rhs2
    rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, Cs, R2, ftop, dn);
    B.account(p, (real)(rk38 ? 3.0 * dt / 8.0 : dt / 3.0), ftop, dn);
#pragma unroll
    for (int s = 0; s < LPL; s++)
#pragma unroll
      for (int n = 0; n < NTR; n++)
        Cs[s][n] = rk38 ? C[s][n] + dtr * (R0[s][n] - R1[s][n] + R2[s][n])
                        : C[s][n] + dtr * R2[s][n];
    // stage 4: rhs3 and the combination
    rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, Cs, R, ftop, dn);
    B.account(p, (real)(rk38 ? dt / 8.0 : dt / 6.0), ftop, dn);
#pragma unroll
    for (int s = 0; s < LPL; s++)
#pragma unroll
      for (int n = 0; n < NTR; n++) {
        if (rk38)
          C[s][n] = C[s][n] + dtr * real(1) / real(8) *
                                  (R0[s][n] + real(3) * R1[s][n] +
                                   real(3) * R2[s][n] + R[s][n]);
        else
          C[s][n] = C[s][n] + dtr * third *
                                  (real(0.5) * R0[s][n] + R1[s][n] + R2[s][n] +
                                   real(0.5) * R[s][n]);
      }
  }
  B.finish(p, lc, C, bud, lane);
  res.nan = epilogue<real, LPL>(p, lane, K, C);
  return res;
}

// ---------------------------------------------------------------------------
// KIND_ADAPT / KIND_FIXED: one coupling step; KIND_RHS: one right-hand side
// written to a.out.
// Resident blocks per SM the register allocation is sized for: three
// 256-thread blocks for FP32 one-layer-per-lane columns (80 registers), two
// for two layers per lane, one for the FP64 path.
template <typename real, int LPL>
struct MinBlocks {
  static constexpr int value = sizeof(real) == 4 ? (LPL == 1 ? 3 : LPL == 2 ? 2 : 1) : 1;
};

template <typename real, int LPL, bool BC4, bool BIO3, int KIND>
__global__ void __launch_bounds__(256, (MinBlocks<real, LPL>::value))
k_column(ColumnArgs<real> a, Params<real> p) {
  constexpr int mode = KIND == KIND_RHS ? 1 : 0;
  constexpr int NCO = coef_rows<real>(BIO3);
  extern __shared__ __align__(16) unsigned char smem[];
  const int tc = a.tc;
  constexpr int KT = 32 * LPL;
  TileLayout<real> L(tc, KT, BC4, NCO);
  const int tcp = L.tcp;
  real* s_conc = reinterpret_cast<real*>(smem + L.conc);
  real* s_coef = reinterpret_cast<real*>(smem + L.coef);
  real* s_cap = reinterpret_cast<real*>(smem + L.cap);
  real* s_force = reinterpret_cast<real*>(smem + L.force);
  real* s_sflux = reinterpret_cast<real*>(smem + L.sflux);
  double* s_bud = reinterpret_cast<double*>(smem + L.bud);
  int* s_nsub = reinterpret_cast<int*>(smem + L.nsub);
  __shared__ int s_tile, s_next;
  __shared__ int s_heavy[64];  // KIND_PROBE: the tile's columns the gate rejects
  __shared__ int s_hcol[64], s_hn;  // KIND_PROBE: their tile columns, in order
  __shared__ unsigned s_hat;        // and their first list entry
  __shared__ unsigned long long b_att, b_acc, b_cols, b_mindt;
  __shared__ int b_maxatt, b_cap, b_nan;
  __shared__ __align__(16) float s_surf[SURF_FLOATS];

  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31;
  if (tid == 0) {
    b_att = 0; b_acc = 0; b_cols = 0; b_mindt = 0x7FF0000000000000ull;
    b_maxatt = 0; b_cap = 0; b_nan = 0;
  }
  if (tid < SURF_ROW) s_surf[SURF_ZERO + tid] = 0.0f;
  const size_t ns = (size_t)a.nslot;

  for (;;) {
    if (tid == 0) { s_tile = (int)atomicAdd(a.queue, 1u); s_next = 0; }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= a.ntiles) break;
    const int slot0 = a.slot0 + tile * tc;
    const int kt = a.tile_k ? a.tile_k[a.tile0 + tile] : (a.kmax < KT ? a.kmax : KT);
    copy_grouped<real, true>(s_conc, a.conc + slot0, NTR, kt, KT, a.kmax, ns, tc, tcp, tid,
                             nthr);
    copy_grouped<real, true>(s_coef, const_cast<real*>(a.coef) + slot0, NCO, kt, KT,
                             a.kmax, ns, tc, tcp, tid, nthr);
    if (BC4)
      copy_grouped<real, true>(s_cap, const_cast<real*>(a.cap) + slot0, 1, kt,
                               KT, a.kmax, ns, tc, tcp, tid, nthr);
    copy_rows<real, true>(s_force, const_cast<real*>(a.force) + slot0, ns,
                          NFORCE, tc, tcp, 1, tid, nthr);
    cp_async_wait_all();
    __syncthreads();

    for (;;) {
      int j = 0;
      if (lane == 0) j = atomicAdd(&s_next, 1);
      j = __shfl_sync(FULL, j, 0);
      if (j >= tc) break;
      const int K = a.kact[slot0 + j];
      if (KIND == KIND_PROBE && lane == 0) s_heavy[j] = 0;
      if (K <= 0) {
        if (lane == 0) {
          s_nsub[j] = 0;
          if (mode == 0 && a.mindt) a.mindt[slot0 + j] = 0.0;
#pragma unroll
          for (int d = 0; d < NDISS; d++) s_sflux[d * tcp + j] = real(0);
          for (int b = 0; b < 4; b++) s_bud[b * tc + j] = 0.0;
        }
        continue;
      }
      Lane<real, LPL, BC4> lc;
      real C[LPL][NTR];
      load_lane<real, LPL, BC4, BIO3>(lc, C, s_conc, s_coef, s_cap, s_force, j, KT,
                                      tcp, lane, K, p.mol_mode, p.bcup_d);
      set_surface_row(lc, s_surf, tid >> 5, lane);
      real ftop[NTR];
#pragma unroll
      for (int n = 0; n < NTR; n++) ftop[n] = real(0);
      if (KIND == KIND_RHS) {
        real R[LPL][NTR];
        real dn[LPL];
        rhs_any<real, LPL, BC4, BIO3>(p, lc, lane, K, C, R, ftop, dn);
#pragma unroll
        for (int s = 0; s < LPL; s++) {
          const int Ll = s * 32 + lane;
          if (Ll < K)
#pragma unroll
            for (int n = 0; n < NTR; n++) s_conc[(n * KT + Ll) * tcp + j] = R[s][n];
        }
        if (lane == 0) {
#pragma unroll
          for (int d = 0; d < NDISS; d++) s_sflux[d * tcp + j] = ftop[NPART + d];
          s_nsub[j] = 1;
        }
        continue;
      }
      double bud[4] = {0.0, 0.0, 0.0, 0.0};
      ColResult r;
      constexpr bool PROBE = KIND == KIND_PROBE;
      if (PROBE)
        r = probe_column<real, LPL, BC4, BIO3>(p, lc, lane, K, C, ftop, a.dt, bud);
      else if (KIND == KIND_ADAPT)
        r = p.ticks ? solve_adaptive<real, LPL, BC4, BIO3, true>(p, lc, lane, K, C, ftop, a.dt,
                                                                bud)
                    : solve_adaptive<real, LPL, BC4, BIO3, false>(p, lc, lane, K, C, ftop, a.dt,
                                                                 bud);
      else
        r = solve_fixed<real, LPL, BC4, BIO3>(p, lc, lane, K, C, ftop, a.dt, a.method,
                                              bud);
      if (PROBE && r.attempts < 0) {
        // the gate rejects the column: its staged state goes back as it was
        if (lane == 0) {
          s_heavy[j] = 1;
          s_nsub[j] = 0;
#pragma unroll
          for (int d = 0; d < NDISS; d++) s_sflux[d * tcp + j] = real(0);
          for (int b = 0; b < 4; b++) s_bud[b * tc + j] = 0.0;
        }
        continue;
      }
#pragma unroll
      for (int s = 0; s < LPL; s++) {
        const int Ll = s * 32 + lane;
        if (Ll < K)
#pragma unroll
          for (int n = 0; n < NTR; n++) s_conc[(n * KT + Ll) * tcp + j] = C[s][n];
      }
      if (lane == 0) {
#pragma unroll
        for (int d = 0; d < NDISS; d++) s_sflux[d * tcp + j] = ftop[NPART + d];
        for (int b = 0; b < 4; b++) s_bud[b * tc + j] = bud[b];
        s_nsub[j] = r.attempts;
        if (a.mindt) a.mindt[slot0 + j] = r.accepted > 0 ? r.min_dt : 0.0;
        atomicAdd(&b_att, (unsigned long long)r.attempts);
        atomicAdd(&b_acc, (unsigned long long)r.accepted);
        atomicAdd(&b_cols, 1ull);
        atomicMax(&b_maxatt, r.attempts);
        if (r.capped) atomicAdd(&b_cap, 1);
        if (r.nan) atomicAdd(&b_nan, r.nan);
        if (r.accepted > 0)
          atomicMin(&b_mindt, (unsigned long long)__double_as_longlong(r.min_dt));
      }
    }
    __syncthreads();
    if (KIND == KIND_PROBE) {
      if (tid < 32) {
        // the tile's rejected columns into the list in tile order, one
        // reservation per tile: warp 0 ranks them by ballot (tiles of up to
        // 64 columns, two halves)
        const unsigned lo = __ballot_sync(FULL, lane < tc && s_heavy[lane]);
        const unsigned hi = __ballot_sync(FULL, lane + 32 < tc && s_heavy[lane + 32]);
        const int nlo = __popc(lo), n = nlo + __popc(hi);
        unsigned at = 0;
        if (lane == 0 && n > 0) at = atomicAdd(a.nheavy, (unsigned)n);
        at = __shfl_sync(FULL, at, 0);
        const unsigned below = (1u << lane) - 1u;
        if ((lo >> lane) & 1u) {
          const int r = __popc(lo & below);
          s_hcol[r] = lane;
          a.heavy[at + r] = slot0 + lane;
        }
        if ((hi >> lane) & 1u) {
          const int r = nlo + __popc(hi & below);
          s_hcol[r] = lane + 32;
          a.heavy[at + r] = slot0 + lane + 32;
        }
        if (lane == 0) {
          s_hn = n;
          s_hat = at;
        }
      }
      if (a.xfeat) {
        // their network input rows, from the staged (unchanged) state and
        // forcing: a thread owns features f, tid + nthr, ... and writes them
        // for every listed column of the tile (consecutive threads,
        // consecutive features of a row); the full-accuracy FP32 logarithm
        // and the IEEE quotient, so a row rounds to BF16 as the host's FP64
        // features of the same state almost always do
        __syncthreads();
        const int n = s_hn, pin = a.pin, nin = a.nin, K = a.kmax;
        const int nstate = NTR * K;
        const float* c0 = a.norm;
        const float* mu = c0 + NTR;
        const float* sd = mu + nin;
        unsigned short* x = a.xfeat + (size_t)s_hat * pin;
        for (int f = tid; f < pin; f += nthr) {
          const real* src = nullptr;
          float add = 0.0f, m = 0.0f, sdf = 1.0f;
          bool state = false;
          if (f < nstate) {
            const int tr = f / K, k = f - tr * K;
            src = s_conc + (tr * KT + k) * tcp;
            add = c0[tr];
            state = true;
          } else if (f < nin) {
            src = s_force + (f - nstate) * tcp;
          }
          if (src) {
            m = mu[f];
            sdf = sd[f];
          }
          for (int r = 0; r < n; r++) {
            float v = 0.0f;
            if (src) {
              const float c = (float)src[s_hcol[r]];
              v = __fdiv_rn((state ? logf(fmaxf(c, 0.0f) + add) : c) - m, sdf);
            }
            x[(size_t)r * pin + f] = __bfloat16_as_ushort(__float2bfloat16(v));
          }
        }
      }
    }
    // stage out
    real* dst = (mode == 1) ? a.out : a.conc;
    copy_grouped<real, false>(s_conc, dst + slot0, NTR, kt, KT, a.kmax, ns, tc,
                              tcp, tid, nthr);
    copy_rows<real, false>(s_sflux, a.sflux + slot0, ns, NDISS, tc, tcp, 1,
                           tid, nthr);
    for (int i = tid; i < tc; i += nthr) {
      a.nsub[slot0 + i] = s_nsub[i];
      if (a.budget)
        for (int b = 0; b < 4; b++) a.budget[(size_t)b * ns + slot0 + i] = s_bud[b * tc + i];
    }
  }
  __syncthreads();
  if (tid == 0 && mode == 0) {
    atomicAdd(&a.stats->attempts, b_att);
    atomicAdd(&a.stats->accepted, b_acc);
    atomicAdd(&a.stats->column_steps, b_cols);
    atomicMin(&a.stats->min_dt_bits, b_mindt);
    atomicMax(&a.stats->max_col_attempts, b_maxatt);
    if (b_cap) { atomicAdd(&a.stats->capped, b_cap); atomicOr(&a.stats->status, ST_CAP); }
    if (b_nan) { atomicAdd(&a.stats->nan_cells, b_nan); atomicOr(&a.stats->status, ST_NAN); }
  }
}

// ---------------------------------------------------------------------------
// Warp-direct form of the stepping kinds (KIND_ADAPT / KIND_FIXED).  The tile
// kernel makes a block's warps wait at every tile boundary for the tile's
// slowest column; once the column profiles develop, substep counts per
// column spread over two orders of magnitude and those waits dominate.  Here
// each warp pulls one column at a time from the work counter, loads it
// straight from global memory (lane = layer; neighbouring warps share the L2
// sectors of neighbouring slots), steps it and writes it back.  The only
// shared memory is the warp's copy of its column's 11 surface values; the
// only block barriers are at entry and exit.
// ENS: every column takes its own OMEXDIA+P parameter set from a.bgc.
template <typename real, int LPL, bool BC4, bool BIO3, int KIND, bool MULTI, bool ENS>
__global__ void __launch_bounds__(256, (MinBlocks<real, LPL>::value))
k_column_warp(ColumnArgs<real> a, Params<real> p) {
  __shared__ real s_bnd[8][NFORCE];
  __shared__ __align__(16) float s_surf[SURF_FLOATS];
  __shared__ unsigned long long b_att, b_acc, b_cols, b_mindt, b_sur;
  __shared__ int b_maxatt, b_cap, b_nan;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    b_att = 0; b_acc = 0; b_cols = 0; b_sur = 0; b_mindt = 0x7FF0000000000000ull;
    b_maxatt = 0; b_cap = 0; b_nan = 0;
  }
  if (tid < SURF_ROW) s_surf[SURF_ZERO + tid] = 0.0f;
  __syncthreads();
  const size_t ns = (size_t)a.nslot;
  real* sb = s_bnd[warp];
  int ncols = a.ntiles;
  if (a.list && a.nlist) {
    const int n = (int)*a.nlist;
    ncols = n < ncols ? n : ncols;
  }
  for (;;) {
    int j = 0;
    if (lane == 0) j = (int)atomicAdd(a.queue, 1u);
    j = __shfl_sync(FULL, j, 0);
    if (j >= ncols) break;
    // the launch's j-th column: of a slot list (the surrogate step's heavy
    // columns), or of the slot range
    const int slot = a.list ? a.list[j] : a.slot0 + j;
    const int K = a.kact[slot];
    if (K <= 0) {
      // land or padding: zero outputs
      if (lane == 0) {
        a.nsub[slot] = 0;
        if (a.mindt) a.mindt[slot] = 0.0;
        for (int d = 0; d < NDISS; d++) a.sflux[d * ns + slot] = real(0);
        if (a.budget)
          for (int b = 0; b < 4; b++) a.budget[b * ns + slot] = 0.0;
      }
      continue;
    }
    if (lane < NFORCE) sb[lane] = a.force[lane * ns + slot];
    __syncwarp();
    Lane<real, LPL, BC4> lc;
    real C[LPL][NTR];
    // global arrays in load_lane's (row, column) form: rows of kmax layers
    // per tracer / coefficient, columns of stride nslot; then the surface
    // values the substeps read come from the warp's shared copy
    load_lane<real, LPL, BC4, BIO3>(lc, C, a.conc, a.coef, a.cap, a.force, slot, a.kmax,
                                    (int)ns, lane, K, p.mol_mode, p.bcup_d);
    lc.bnd_s = sb + 2;
    lc.bnd_stride = 1;
    set_surface_row(lc, s_surf, warp, lane);
    Params<real> pc = p;
    if (ENS) load_bgc(pc, a.bgc, ns, slot);
    real ftop[NTR];
    if constexpr (KIND == KIND_SUR) {
      // The network's proposal P from the state C and prediction row j:
      // P = max(exp(log(max(C, 0) + c0) + mu_d + sd_d y) - c0, 0), cell
      // (n, k) at feature n K + k (every column has K = kmax layers here).
      // C stays the start state for the fallback.
      real P[LPL][NTR];
      {
        const float* yr = a.yhat + (size_t)j * a.ldy;
        const float* c0 = a.norm;
        const float* mud = a.norm + NTR + 2 * a.nin;
        const float* sdd = mud + a.nout;
#pragma unroll
        for (int s = 0; s < LPL; s++) {
          const int L = s * 32 + lane;
#pragma unroll
          for (int n = 0; n < NTR; n++) {
            P[s][n] = C[s][n];  // lanes past the column: zero
            if (L < K) {
              const int f = n * K + L;
              const float u = logf(fmaxf((float)C[s][n], 0.0f) + c0[n]) + mud[f] + sdd[f] * yr[f];
              P[s][n] = (real)fmaxf(expf(u) - c0[n], 0.0f);
            }
          }
        }
      }
      // Quasi-steady test of P: the plain right-hand side at P may change no
      // cell by more than res_tol of its value over one step,
      // dt |f(P)| <= res_tol (|P| + res_atol) in every active cell.  At the
      // end of a column's heavy steps the plain solver's own states change
      // by about 1 % per step this way; a proposal off the slow manifold of
      // the stiff cells fails by orders of magnitude.  NaN fails.
      epilogue<real, LPL>(pc, lane, K, P);
      bool pass;
      {
        real R[LPL][NTR];
        real dn[LPL];
#pragma unroll
        for (int n = 0; n < NTR; n++) ftop[n] = real(0);
        rhs_any<real, LPL, BC4, BIO3>(pc, lc, lane, K, P, R, ftop, dn);
        const real dtr = (real)a.dt, at = (real)a.res_atol, tol = (real)a.res_tol;
        bool ok = true;
#pragma unroll
        for (int s = 0; s < LPL; s++) {
          const int L = s * 32 + lane;
          if (L < K)
#pragma unroll
            for (int n = 0; n < NTR; n++)
              ok = ok && (dtr * fabs(R[s][n]) <= tol * (fabs(P[s][n]) + at));
        }
        pass = __all_sync(FULL, ok);
      }
      if (pass) {
#pragma unroll
        for (int s = 0; s < LPL; s++) {
          const int L = s * 32 + lane;
          if (L < K)
#pragma unroll
            for (int n = 0; n < NTR; n++) a.conc[((size_t)n * a.kmax + L) * ns + slot] = P[s][n];
        }
        if (lane == 0) {
#pragma unroll
          for (int d = 0; d < NDISS; d++) a.sflux[d * ns + slot] = ftop[NPART + d];
          a.nsub[slot] = 0;
          if (a.mindt) a.mindt[slot] = 0.0;
          if (a.budget)
            for (int b = 0; b < 4; b++) a.budget[b * ns + slot] = 0.0;
          atomicAdd(&b_sur, 1ull);
          atomicAdd(&b_cols, 1ull);
        }
        __syncwarp();
        continue;
      }
      // failed: the plain adaptive step from C, below
    }
    double bud[4];
    ColResult r;
    // MULTI: a.nrepeat steps in a row (the loop costs registers, so the
    // single-step kernel has none)
    const int nrep = MULTI ? (a.nrepeat > 1 ? a.nrepeat : 1) : 1;
    for (int rep = 0; rep < nrep; rep++) {
#pragma unroll
      for (int n = 0; n < NTR; n++) ftop[n] = real(0);
      for (int b = 0; b < 4; b++) bud[b] = 0.0;
      if (KIND == KIND_ADAPT || KIND == KIND_SUR)
        r = pc.ticks
                ? solve_adaptive<real, LPL, BC4, BIO3, true>(pc, lc, lane, K, C, ftop, a.dt, bud)
                : solve_adaptive<real, LPL, BC4, BIO3, false>(pc, lc, lane, K, C, ftop, a.dt, bud);
      else
        r = solve_fixed<real, LPL, BC4, BIO3>(pc, lc, lane, K, C, ftop, a.dt, a.method, bud);
      if (lane == 0) {
        atomicAdd(&b_att, (unsigned long long)r.attempts);
        atomicAdd(&b_acc, (unsigned long long)r.accepted);
        atomicAdd(&b_cols, 1ull);
        atomicMax(&b_maxatt, r.attempts);
        if (r.capped) atomicAdd(&b_cap, 1);
        if (r.nan) atomicAdd(&b_nan, r.nan);
        if (r.accepted > 0)
          atomicMin(&b_mindt, (unsigned long long)__double_as_longlong(r.min_dt));
      }
    }
#pragma unroll
    for (int s = 0; s < LPL; s++) {
      const int L = s * 32 + lane;
      if (L < K)
#pragma unroll
        for (int n = 0; n < NTR; n++) a.conc[((size_t)n * a.kmax + L) * ns + slot] = C[s][n];
    }
    if (lane == 0) {
#pragma unroll
      for (int d = 0; d < NDISS; d++) a.sflux[d * ns + slot] = ftop[NPART + d];
      a.nsub[slot] = r.attempts;
      if (a.mindt) a.mindt[slot] = r.accepted > 0 ? r.min_dt : 0.0;
      if (a.budget)
        for (int b = 0; b < 4; b++) a.budget[b * ns + slot] = bud[b];
    }
    __syncwarp();
  }
  __syncthreads();
  if (tid == 0) {
    if (b_sur) atomicAdd(&a.stats->surrogate, b_sur);
    atomicAdd(&a.stats->attempts, b_att);
    atomicAdd(&a.stats->accepted, b_acc);
    atomicAdd(&a.stats->column_steps, b_cols);
    atomicMin(&a.stats->min_dt_bits, b_mindt);
    atomicMax(&a.stats->max_col_attempts, b_maxatt);
    if (b_cap) { atomicAdd(&a.stats->capped, b_cap); atomicOr(&a.stats->status, ST_CAP); }
    if (b_nan) { atomicAdd(&a.stats->nan_cells, b_nan); atomicOr(&a.stats->status, ST_NAN); }
  }
}

// Spin-up broadcast (fabm_sediment_component.F90:616-624): the profile of slot
// src into every other active slot, first min(K, K_src) layers.
template <typename real>
__global__ void k_broadcast(real* __restrict__ conc, const int* __restrict__ kact, int src,
                            int nslot, int kmax) {
  const int ks = kact[src];
  const size_t total = (size_t)NTR * kmax * nslot;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const size_t nk = i / nslot;
    const int k = (int)(nk % kmax);
    if (slot == src || k >= kact[slot] || k >= ks) continue;
    conc[i] = conc[nk * nslot + src];
  }
}

// ---------------------------------------------------------------------------
// Grid-wide adaptive cut (the reference's any() over the whole local grid).
template <typename real>
__global__ void k_trial(const real* __restrict__ conc, const real* __restrict__ rhs,
                        const int* __restrict__ kact, int nslot, int kmax,
                        real dtr, real keep, real natol, int* flag) {
  const size_t total = (size_t)NTR * kmax * nslot;
  bool bad = false;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const int k = (int)((i / nslot) % kmax);
    if (k >= kact[slot]) continue;
    const real c = conc[i];
    const real c1 = upd(c, dtr, rhs[i]);
    bad |= below_keep(c1, keep, c, natol);
  }
  if (__any_sync(FULL, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

template <typename real>
__global__ void k_accept(real* __restrict__ conc, const real* __restrict__ rhs,
                         const int* __restrict__ kact, int nslot, int kmax,
                         real dtr) {
  const size_t total = (size_t)NTR * kmax * nslot;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const int k = (int)((i / nslot) % kmax);
    if (k >= kact[slot]) continue;
    conc[i] = upd(conc[i], dtr, rhs[i]);
  }
}

// adaptive_solver_diagnostics (solver_library.F90:133-134): the smallest
// relative change (c1 - c) / c of the substep about to be accepted, over the
// active cells, in FP64 (NaN quotients skipped).  Pass 1: the minimum as an
// order-preserving key of its bits; pass 2: the smallest Fortran element
// index, col + ncol (k + kmax n), among the cells equal to it.
__device__ __forceinline__ unsigned long long order_key(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_value(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

template <typename real>
__device__ __forceinline__ double rel_change(real c, real dtr, real r) {
  const real c1 = upd(c, dtr, r);
  return ((double)c1 - (double)c) / (double)c;
}

template <typename real>
__global__ void k_minloc_value(const real* __restrict__ conc, const real* __restrict__ rhs,
                               const int* __restrict__ kact, int nslot, int kmax, real dtr,
                               unsigned long long* key) {
  const size_t total = (size_t)NTR * kmax * nslot;
  unsigned long long best = ~0ull;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const int k = (int)((i / nslot) % kmax);
    if (k >= kact[slot]) continue;
    const double v = rel_change(conc[i], dtr, rhs[i]);
    if (v != v) continue;
    const unsigned long long kv = order_key(v);
    best = kv < best ? kv : best;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(FULL, best, o);
    best = t < best ? t : best;
  }
  if ((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(key, best);
}

template <typename real>
__global__ void k_minloc_index(const real* __restrict__ conc, const real* __restrict__ rhs,
                               const int* __restrict__ kact, const int* __restrict__ slot_col,
                               int nslot, int kmax, int ncol, real dtr,
                               const unsigned long long* key, unsigned long long* index) {
  const unsigned long long kmin = *key;
  if (kmin == ~0ull) return;  // no valid quotient
  const double vmin = key_value(kmin);
  const size_t total = (size_t)NTR * kmax * nslot;
  unsigned long long best = ~0ull;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const size_t nk = i / nslot;
    const int k = (int)(nk % kmax);
    if (k >= kact[slot]) continue;
    const double v = rel_change(conc[i], dtr, rhs[i]);
    if (!(v == vmin)) continue;
    const int n = (int)(nk / kmax);
    const unsigned long long f =
        (unsigned long long)slot_col[slot] + (unsigned long long)ncol * (k + (size_t)kmax * n);
    best = f < best ? f : best;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(FULL, best, o);
    best = t < best ? t : best;
  }
  if ((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(index, best);
}

template <typename real>
__global__ void k_epilogue(real* __restrict__ conc, const int* __restrict__ kact,
                           int nslot, int kmax, Params<real> p, DevStats* st) {
  const size_t total = (size_t)NTR * kmax * nslot;
  int nan = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const int k = (int)((i / nslot) % kmax);
    const int n = (int)(i / ((size_t)nslot * kmax));
    if (k >= kact[slot]) continue;
    const real v = conc[i];
    if (v != v) nan++;
    else if (v < p.minimum[n]) conc[i] = p.minimum[n];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nan += __shfl_xor_sync(FULL, nan, o);
  if ((threadIdx.x & 31) == 0 && nan) {
    atomicAdd(&st->nan_cells, nan);
    atomicOr(&st->status, ST_NAN);
  }
}

// ---------------------------------------------------------------------------
// Layout / precision conversion.  host layout [g][kmax][ncol] (FP64),
// device layout [g][kmax][nslot] (real), slot_col maps slot -> column (-1 pad)
template <typename real>
__global__ void k_gather(const double* __restrict__ src, real* __restrict__ dst,
                         const int* __restrict__ slot_col, int ngroups, int kmax,
                         int ncol, int nslot, int slot0, int nseg) {
  const size_t total = (size_t)ngroups * kmax * nseg;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = slot0 + (int)(i % nseg);
    const size_t gk = i / nseg;
    const int col = slot_col[slot];
    dst[gk * nslot + slot] = col >= 0 ? (real)src[gk * ncol + col] : real(0);
  }
}

template <typename real>
__global__ void k_scatter(const real* __restrict__ src, double* __restrict__ dst,
                          const int* __restrict__ slot_col,
                          const int* __restrict__ kact, int ngroups, int kmax,
                          int ncol, int nslot, int slot0, int nseg) {
  const size_t total = (size_t)ngroups * kmax * nseg;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = slot0 + (int)(i % nseg);
    const size_t gk = i / nseg;
    const int k = (int)(gk % kmax);
    const int col = slot_col[slot];
    if (col >= 0 && k < kact[slot]) dst[gk * ncol + col] = (double)src[gk * nslot + slot];
  }
}

// dissolved surface fluxes [NDISS][nslot] -> rows NPART.. of fluxes[NTR][ncol]
template <typename real>
__global__ void k_scatter_flux(const real* __restrict__ sflux,
                               double* __restrict__ fluxes,
                               const int* __restrict__ slot_col,
                               const int* __restrict__ kact, int ncol,
                               int nslot) {
  const size_t total = (size_t)NDISS * nslot;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const int d = (int)(i / nslot);
    const int col = slot_col[slot];
    if (col >= 0 && kact[slot] > 0)
      fluxes[(size_t)(NPART + d) * ncol + col] = (double)sflux[i];
  }
}

// Per-layer coefficients of the transport, from the reference's arrays:
//   phi, vol = phi dz, gb = (1-phi_i) biofac / len / 8.64e8,
//   gm = phi_i / len / 8.64e8 (mode 0) or d0 phi_i / (1 - 2 ln phi_i) / len,
// len = dz for the surface interface, dzc below (diff3d :777,786) and
// 8.64e8 = 86400 s * 1e4 cm2/m2 (get_rhs :652,683).
// The FP64 variant stores the reference's per-cell operands instead:
//   phi, phi_i, biofac, dz, len, mol (mol = d0 phi_i/(1-2 ln phi_i) computed
//   on the host for mode 1, so both sides use the same logarithm).
template <typename real>
__global__ void k_prep_grid(const double* __restrict__ dz,
                            const double* __restrict__ dzc,
                            const double* __restrict__ phi,
                            const double* __restrict__ phi_i,
                            const double* __restrict__ biofac,
                            const double* __restrict__ cap,
                            const double* __restrict__ mol,
                            const int* __restrict__ slot_col,
                            real* __restrict__ coef, real* __restrict__ capd,
                            int kmax, int ncol, int nslot, int mode, double d0) {
  if constexpr (std::is_same<real, double>::value) {
    const size_t total = (size_t)kmax * nslot;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
      const int slot = (int)(i % nslot);
      const int k = (int)(i / nslot);
      const int col = slot_col[slot];
      double v[NCOEF64] = {1.0, 1.0, 0.0, 1.0, 1.0, 0.0};
      double v_cap = 0.0;
      if (col >= 0) {
        const size_t c = (size_t)k * ncol + col;
        v[0] = phi[c];
        v[1] = phi_i[c];
        v[2] = biofac[c];
        v[3] = dz[c];
        v[4] = (k == 0) ? dz[c] : dzc[(size_t)(k - 1) * ncol + col];
        v[5] = mol ? mol[c] : 0.0;
        if (cap) v_cap = cap[c];
      }
      for (int r = 0; r < NCOEF64; r++) coef[((size_t)r * kmax + k) * nslot + slot] = v[r];
      if (capd) capd[i] = v_cap;
    }
    return;
  }
  const size_t total = (size_t)kmax * nslot;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const int k = (int)(i / nslot);
    const int col = slot_col[slot];
    double v_phi = 1.0, v_vol = 1.0, v_gb = 0.0, v_gm = 0.0, v_cap = 0.0;
    if (col >= 0) {
      const size_t c = (size_t)k * ncol + col;
      const double ph = phi[c], pi = phi_i[c];
      const double len = (k == 0) ? dz[c] : dzc[(size_t)(k - 1) * ncol + col];
      v_phi = ph;
      v_vol = ph * dz[c];
      v_gb = (1.0 - pi) * biofac[c] / len / 8.64e8;
      if (mode == 1)
        v_gm = (mol ? mol[c] : d0 * pi / (1.0 - 2.0 * log(pi))) / len;
      else
        v_gm = pi / len / 8.64e8;
      if (cap) v_cap = cap[c];
    }
    coef[(0 * (size_t)kmax + k) * nslot + slot] = (real)v_phi;
    coef[(1 * (size_t)kmax + k) * nslot + slot] = (real)v_vol;
    coef[(2 * (size_t)kmax + k) * nslot + slot] = (real)v_gb;
    coef[(3 * (size_t)kmax + k) * nslot + slot] = (real)v_gm;
    if (capd) capd[i] = (real)v_cap;
  }
}

// get_boundary_conditions (fabm_sediment_component.F90:1865-2030) on the
// device, per column: temperature -> bdys[0]; for every tracer in
// present_mask, particulate fluxes[n] = -surface * velocity (downward
// positive, :1978,1986), dissolved bdys[n+1] = surface and fluxes[n] = the
// diffusive estimate of :2012-2014 (bcup_dissolved 1, from the state's first
// layer; 0 for land) or 0.  top = [dz(1)][porosity(1)] per column (FP64).
template <typename real>
__global__ void k_assemble_bc(const double* __restrict__ temperature,
                              const double* __restrict__ surface,
                              const double* __restrict__ velocity, unsigned present_mask,
                              const real* __restrict__ conc, const int* __restrict__ col_slot,
                              const double* __restrict__ top, double* __restrict__ bdys,
                              double* __restrict__ fluxes, int ncol, int nslot, int kmax,
                              int bcup_d, double bioturbation, double diffusivity) {
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    const double T = temperature[col];
    bdys[col] = T;
    const int slot = col_slot[col];
    for (int n = 0; n < NTR; n++) {
      if (!((present_mask >> n) & 1u)) continue;
      const size_t i = (size_t)n * ncol + col;
      if (n < NPART) {
        fluxes[i] = -surface[i] * velocity[i];
        continue;
      }
      const double cb = surface[i];
      bdys[(size_t)(n + 1) * ncol + col] = cb;
      double f = 0.0;
      if (bcup_d == 1 && slot >= 0) {
        const double c0 = (double)conc[(size_t)n * kmax * nslot + slot];
        f = -(c0 - cb) / top[col] * (bioturbation + diffusivity + T * 0.035) *
            top[(size_t)ncol + col] / 86400.0 / 10000.0;
      }
      fluxes[i] = f;
    }
  }
}

// Per-column forcing of one coupling step: bioturbation x f_T (get_rhs :648,
// :652), the molecular multiplier, and the surface value of every tracer
// (bottom-water concentration or downward flux, diff3d's Cup / fluxup).
template <typename real>
__global__ void k_prep_force(const double* __restrict__ bdys,
                             const double* __restrict__ fluxes,
                             const int* __restrict__ slot_col,
                             real* __restrict__ force, int ncol, int nslot,
                             double bio, double diffusivity, int mode,
                             int bcup_d, int bio3) {
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < nslot;
       slot += gridDim.x * blockDim.x) {
    const int col = slot_col[slot];
    double f[NFORCE];
    for (int i = 0; i < NFORCE; i++) f[i] = 0.0;
    if (col >= 0) {
      const double T = bdys[col];
      const double fT = 1.0 * exp(-4500.0 * (1.0 / (T + 273.0) - (1.0 / 288.0)));
      f[0] = bio3 ? 1.0 : bio * fT;  // profile 3: bioturbation = f_T = 1 (:622-623)
      f[1] = (mode == 1) ? 1.0 : (diffusivity + T * 0.035);
      for (int n = 0; n < NTR; n++) {
        const bool part = n < NPART;
        const double fl = fluxes[(size_t)n * ncol + col];
        const double cb = bdys[(size_t)(n + 1) * ncol + col];
        f[2 + n] = part ? fl : (bcup_d == 1 ? fl : cb);
      }
    }
    for (int i = 0; i < NFORCE; i++) force[(size_t)i * nslot + slot] = (real)f[i];
  }
}

// Temperature-dependent rates: the per-slot parameter table from its base,
// the microbial rate constants (rows 0-4 of the table: rF, rS, cmax, rnit,
// rodu) multiplied by the column's factor -- fac[col] when given (formed on
// the host), else rate_factor of the column's temperature bdys[col].  Land
// slots keep the base.
template <typename real>
__global__ void k_rate_temperature(const real* __restrict__ base, real* __restrict__ tab,
                                   const int* __restrict__ slot_col,
                                   const double* __restrict__ bdys,
                                   const double* __restrict__ fac, double Ta, int nslot) {
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < nslot;
       slot += gridDim.x * blockDim.x) {
    const int col = slot_col[slot];
    const double f = col < 0 ? 1.0 : (fac ? fac[col] : rate_factor(Ta, bdys[col]));
#pragma unroll
    for (int i = 0; i < NBGC_DEV; i++) {
      const real b = base[(size_t)i * nslot + slot];
      tab[(size_t)i * nslot + slot] = i < NRATE_TEMP ? (real)((double)b * f) : b;
    }
  }
}

// ---------------------------------------------------------------------------
// launchers
static int grid_for(size_t total, int block, int sms) {
  size_t g = (total + block - 1) / block;
  size_t cap = (size_t)sms * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// Coefficient rows of bioturbation profile 3 from the host's per-cell
// exp(zc 100 k_l), exp(zc 200 k_l) and per-column cumdepth (the depth of
// the last layer's upper interface).  FP32: row 2 becomes the bioturbation
// conductance per unit factor (1 - phi_i) / len / 8.64e8, row NCOEF the
// depth term e1 / (L1 + L2 e2) and row NCOEF+1 the averaging weight
// dz / cumdepth.  FP64: rows NCOEF64.. hold e1, e2 and cumdepth.
template <typename real>
__global__ void k_prep_bio3(const double* __restrict__ dz, const double* __restrict__ dzc,
                            const double* __restrict__ phi_i, const double* __restrict__ e1,
                            const double* __restrict__ e2, const double* __restrict__ cum,
                            const int* __restrict__ slot_col, real* __restrict__ coef,
                            int kmax, int ncol, int nslot, double L1, double L2) {
  const size_t total = (size_t)kmax * nslot;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i % nslot);
    const int k = (int)(i / nslot);
    const int col = slot_col[slot];
    auto at = [&](int r) -> real& { return coef[((size_t)r * kmax + k) * nslot + slot]; };
    if constexpr (std::is_same<real, double>::value) {
      double v0 = 1.0, v1 = 1.0, v2 = 1.0;
      if (col >= 0) {
        const size_t c = (size_t)k * ncol + col;
        v0 = e1[c];
        v1 = e2[c];
        v2 = cum[col];
      }
      at(NCOEF64) = v0;
      at(NCOEF64 + 1) = v1;
      at(NCOEF64 + 2) = v2;
    } else {
      double gb = 0.0, g = 0.0, hw = 0.0;
      if (col >= 0) {
        const size_t c = (size_t)k * ncol + col;
        const double len = (k == 0) ? dz[c] : dzc[(size_t)(k - 1) * ncol + col];
        gb = (1.0 - phi_i[c]) / len / 8.64e8;
        g = e1[c] / (L1 + L2 * e2[c]);
        hw = dz[c] / cum[col];
      }
      at(2) = (real)gb;
      at(NCOEF) = (real)g;
      at(NCOEF + 1) = (real)hw;
    }
  }
}

template <typename real>
cudaError_t launch_assemble_bc(const double* temperature, const double* surface,
                               const double* velocity, unsigned present_mask, const real* conc,
                               const int* col_slot, const double* top, double* bdys,
                               double* fluxes, int ncol, int nslot, int kmax, int bcup_d,
                               double bioturbation, double diffusivity, int sms,
                               cudaStream_t st) {
  k_assemble_bc<real><<<grid_for(ncol, 128, sms), 128, 0, st>>>(
      temperature, surface, velocity, present_mask, conc, col_slot, top, bdys, fluxes, ncol,
      nslot, kmax, bcup_d, bioturbation, diffusivity);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_prep_bio3(const double* dz, const double* dzc, const double* phi_i,
                             const double* e1, const double* e2, const double* cum,
                             const int* slot_col, real* coef, int kmax, int ncol, int nslot,
                             double L1, double L2, int sms, cudaStream_t st) {
  const size_t total = (size_t)kmax * nslot;
  k_prep_bio3<real><<<grid_for(total, 256, sms), 256, 0, st>>>(
      dz, dzc, phi_i, e1, e2, cum, slot_col, coef, kmax, ncol, nslot, L1, L2);
  return cudaGetLastError();
}

template <typename real, int LPL, bool BC4, bool BIO3, int KIND>
static cudaError_t launch_column_t(const ColumnArgs<real>& a, const Params<real>& p,
                                   int blocks, int threads, cudaStream_t st) {
  // the shared-memory limit was raised by column_blocks_per_sm at set-up, so
  // this launch makes no attribute call and can be stream-captured
  const size_t smem = tile_smem_bytes<real>(a.tc, LPL, BC4, KIND, BIO3);
  k_column<real, LPL, BC4, BIO3, KIND><<<blocks, threads, smem, st>>>(a, p);
  return cudaGetLastError();
}

template <typename real, int LPL, bool BC4, bool BIO3>
cudaError_t launch_column_k(const ColumnArgs<real>& a, const Params<real>& p,
                                   int kind, int blocks, int threads,
                                   cudaStream_t st) {
  if (kind == KIND_ADAPT)
    return launch_column_t<real, LPL, BC4, BIO3, KIND_ADAPT>(a, p, blocks, threads, st);
  if (kind == KIND_FIXED)
    return launch_column_t<real, LPL, BC4, BIO3, KIND_FIXED>(a, p, blocks, threads, st);
  if (kind == KIND_PROBE) {
    // the surrogate's gate: FP32 state of at most 63 layers
    if constexpr (std::is_same<real, float>::value && LPL <= 2)
      return launch_column_t<real, LPL, BC4, BIO3, KIND_PROBE>(a, p, blocks, threads, st);
    return cudaErrorInvalidValue;
  }
  return launch_column_t<real, LPL, BC4, BIO3, KIND_RHS>(a, p, blocks, threads, st);
}

template <typename real, int LPL, bool BC4>
static cudaError_t launch_column_b(const ColumnArgs<real>& a, const Params<real>& p,
                                   int kind, int blocks, int threads, cudaStream_t st) {
  return p.bio3 ? launch_column_k<real, LPL, BC4, true>(a, p, kind, blocks, threads, st)
                : launch_column_k<real, LPL, BC4, false>(a, p, kind, blocks, threads, st);
}

template <typename real>
cudaError_t launch_column(const ColumnArgs<real>& a, const Params<real>& p,
                          int lpl, bool bc4, int kind, int blocks, int threads,
                          cudaStream_t st) {
  if (lpl == 1)
    return bc4 ? launch_column_b<real, 1, true>(a, p, kind, blocks, threads, st)
               : launch_column_b<real, 1, false>(a, p, kind, blocks, threads, st);
  if (lpl == 4)
    return bc4 ? launch_column_b<real, 4, true>(a, p, kind, blocks, threads, st)
               : launch_column_b<real, 4, false>(a, p, kind, blocks, threads, st);
  return bc4 ? launch_column_b<real, 2, true>(a, p, kind, blocks, threads, st)
             : launch_column_b<real, 2, false>(a, p, kind, blocks, threads, st);
}

template <typename real, int LPL, bool BC4, bool BIO3, int KIND>
static int occupancy_t(int tc, int threads) {
  const size_t smem = tile_smem_bytes<real>(tc, LPL, BC4, KIND, BIO3);
  auto fn = k_column<real, LPL, BC4, BIO3, KIND>;
  // the limit is raised to the device maximum (never lowered), so handles
  // with different tile widths can share the kernel
  // (the opt-in maximum less the kernel's static shared variables)
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) return 0;
  const int dyn_max = optin - (int)fa.sharedSizeBytes;
  if (dyn_max < (int)smem) return 0;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max) !=
      cudaSuccess)
    return 0;
  cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                       cudaSharedmemCarveoutMaxShared);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess)
    return 0;
  return nb;
}

template <typename real, int LPL, bool BC4, bool BIO3>
int occupancy_k(int tc, int kind, int threads) {
  if (kind == KIND_ADAPT) return occupancy_t<real, LPL, BC4, BIO3, KIND_ADAPT>(tc, threads);
  if (kind == KIND_FIXED) return occupancy_t<real, LPL, BC4, BIO3, KIND_FIXED>(tc, threads);
  if (kind == KIND_PROBE) {
    if constexpr (std::is_same<real, float>::value && LPL <= 2)
      return occupancy_t<real, LPL, BC4, BIO3, KIND_PROBE>(tc, threads);
    return 0;
  }
  return occupancy_t<real, LPL, BC4, BIO3, KIND_RHS>(tc, threads);
}

template <typename real, int LPL, bool BC4>
static int occupancy_b(int tc, int kind, int threads, bool bio3) {
  return bio3 ? occupancy_k<real, LPL, BC4, true>(tc, kind, threads)
              : occupancy_k<real, LPL, BC4, false>(tc, kind, threads);
}

template <typename real>
int column_blocks_per_sm(int tc, int lpl, bool bc4, int kind, int threads, bool bio3) {
  if (lpl == 1)
    return bc4 ? occupancy_b<real, 1, true>(tc, kind, threads, bio3)
               : occupancy_b<real, 1, false>(tc, kind, threads, bio3);
  if (lpl == 4)
    return bc4 ? occupancy_b<real, 4, true>(tc, kind, threads, bio3)
               : occupancy_b<real, 4, false>(tc, kind, threads, bio3);
  return bc4 ? occupancy_b<real, 2, true>(tc, kind, threads, bio3)
             : occupancy_b<real, 2, false>(tc, kind, threads, bio3);
}

template <typename real, int LPL, bool BC4, bool BIO3, int KIND, bool MULTI, bool ENS>
static cudaError_t launch_warp_t(const ColumnArgs<real>& a, const Params<real>& p, int blocks,
                                 int threads, cudaStream_t st) {
  k_column_warp<real, LPL, BC4, BIO3, KIND, MULTI, ENS><<<blocks, threads, 0, st>>>(a, p);
  return cudaGetLastError();
}

// several steps per launch (a.nrepeat > 1) exist for the adaptive method;
// ENS: the per-column parameter-set variants (compiled in their own units)
template <typename real, int LPL, bool BC4, bool BIO3, bool ENS>
cudaError_t launch_warp_e(const ColumnArgs<real>& a, const Params<real>& p, int kind,
                          int blocks, int threads, cudaStream_t st) {
  if (kind == KIND_SUR) {
    // the surrogate step's residual test and fallback: FP32 state, one
    // parameter set
    if constexpr (std::is_same<real, float>::value && !ENS && LPL <= 2) {
      if (a.nrepeat > 1) return cudaErrorInvalidValue;
      return launch_warp_t<real, LPL, BC4, BIO3, KIND_SUR, false, ENS>(a, p, blocks, threads, st);
    }
    return cudaErrorInvalidValue;
  }
  if (kind == KIND_FIXED) {
    if (a.nrepeat > 1) return cudaErrorInvalidValue;
    return launch_warp_t<real, LPL, BC4, BIO3, KIND_FIXED, false, ENS>(a, p, blocks, threads, st);
  }
  return a.nrepeat > 1
             ? launch_warp_t<real, LPL, BC4, BIO3, KIND_ADAPT, true, ENS>(a, p, blocks, threads, st)
             : launch_warp_t<real, LPL, BC4, BIO3, KIND_ADAPT, false, ENS>(a, p, blocks, threads, st);
}

template <typename real, int LPL, bool BC4, bool BIO3>
cudaError_t launch_warp_k(const ColumnArgs<real>& a, const Params<real>& p, int kind,
                          int blocks, int threads, cudaStream_t st) {
  return launch_warp_e<real, LPL, BC4, BIO3, false>(a, p, kind, blocks, threads, st);
}
template <typename real, int LPL, bool BC4, bool BIO3>
cudaError_t launch_warp_ens(const ColumnArgs<real>& a, const Params<real>& p, int kind,
                            int blocks, int threads, cudaStream_t st) {
  return launch_warp_e<real, LPL, BC4, BIO3, true>(a, p, kind, blocks, threads, st);
}

template <typename real, int LPL, bool BC4, bool BIO3, int KIND, bool MULTI>
static int warp_occupancy_t(int threads) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &nb, k_column_warp<real, LPL, BC4, BIO3, KIND, MULTI, false>, threads, 0) !=
      cudaSuccess)
    return 0;
  return nb;
}

template <typename real, int LPL, bool BC4, bool BIO3>
int warp_occupancy_k(int kind, int threads) {
  if (kind == KIND_FIXED) return warp_occupancy_t<real, LPL, BC4, BIO3, KIND_FIXED, false>(threads);
  if (kind == KIND_SUR) {
    if constexpr (std::is_same<real, float>::value && LPL <= 2)
      return warp_occupancy_t<real, LPL, BC4, BIO3, KIND_SUR, false>(threads);
    return 0;
  }
  return std::min(warp_occupancy_t<real, LPL, BC4, BIO3, KIND_ADAPT, false>(threads),
                  warp_occupancy_t<real, LPL, BC4, BIO3, KIND_ADAPT, true>(threads));
}

template <typename real, int LPL, bool BC4, bool BIO3>
static cudaError_t launch_warp_any(const ColumnArgs<real>& a, const Params<real>& p, int kind,
                                   int blocks, int threads, cudaStream_t st) {
  // per-column parameter sets: columns of at most 63 layers
  if constexpr (LPL > 2) {
    if (a.bgc) return cudaErrorInvalidValue;
    return launch_warp_k<real, LPL, BC4, BIO3>(a, p, kind, blocks, threads, st);
  } else {
    return a.bgc ? launch_warp_ens<real, LPL, BC4, BIO3>(a, p, kind, blocks, threads, st)
                 : launch_warp_k<real, LPL, BC4, BIO3>(a, p, kind, blocks, threads, st);
  }
}

template <typename real>
cudaError_t launch_column_warp(const ColumnArgs<real>& a, const Params<real>& p, int lpl,
                               bool bc4, int kind, int blocks, int threads, cudaStream_t st) {
  const bool b3 = p.bio3 != 0;
  if (lpl == 1) {
    if (bc4) return b3 ? launch_warp_any<real, 1, true, true>(a, p, kind, blocks, threads, st)
                       : launch_warp_any<real, 1, true, false>(a, p, kind, blocks, threads, st);
    return b3 ? launch_warp_any<real, 1, false, true>(a, p, kind, blocks, threads, st)
              : launch_warp_any<real, 1, false, false>(a, p, kind, blocks, threads, st);
  }
  if (lpl == 4) {
    if (bc4) return b3 ? launch_warp_any<real, 4, true, true>(a, p, kind, blocks, threads, st)
                       : launch_warp_any<real, 4, true, false>(a, p, kind, blocks, threads, st);
    return b3 ? launch_warp_any<real, 4, false, true>(a, p, kind, blocks, threads, st)
              : launch_warp_any<real, 4, false, false>(a, p, kind, blocks, threads, st);
  }
  if (bc4) return b3 ? launch_warp_any<real, 2, true, true>(a, p, kind, blocks, threads, st)
                     : launch_warp_any<real, 2, true, false>(a, p, kind, blocks, threads, st);
  return b3 ? launch_warp_any<real, 2, false, true>(a, p, kind, blocks, threads, st)
            : launch_warp_any<real, 2, false, false>(a, p, kind, blocks, threads, st);
}

template <typename real>
int column_warp_blocks_per_sm(int lpl, bool bc4, int kind, int threads, bool bio3) {
  if (lpl == 1) {
    if (bc4) return bio3 ? warp_occupancy_k<real, 1, true, true>(kind, threads)
                         : warp_occupancy_k<real, 1, true, false>(kind, threads);
    return bio3 ? warp_occupancy_k<real, 1, false, true>(kind, threads)
                : warp_occupancy_k<real, 1, false, false>(kind, threads);
  }
  if (lpl == 4) {
    if (bc4) return bio3 ? warp_occupancy_k<real, 4, true, true>(kind, threads)
                         : warp_occupancy_k<real, 4, true, false>(kind, threads);
    return bio3 ? warp_occupancy_k<real, 4, false, true>(kind, threads)
                : warp_occupancy_k<real, 4, false, false>(kind, threads);
  }
  if (bc4) return bio3 ? warp_occupancy_k<real, 2, true, true>(kind, threads)
                       : warp_occupancy_k<real, 2, true, false>(kind, threads);
  return bio3 ? warp_occupancy_k<real, 2, false, true>(kind, threads)
              : warp_occupancy_k<real, 2, false, false>(kind, threads);
}

template <typename real>
cudaError_t launch_broadcast(real* conc, const int* kact, int src, int nslot, int kmax, int sms,
                             cudaStream_t st) {
  const size_t total = (size_t)NTR * kmax * nslot;
  k_broadcast<real><<<grid_for(total, 256, sms), 256, 0, st>>>(conc, kact, src, nslot, kmax);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_minloc(const real* conc, const real* rhs, const int* kact, const int* slot_col,
                          int nslot, int kmax, int ncol, real dtr, unsigned long long* out,
                          int sms, cudaStream_t st) {
  const size_t total = (size_t)NTR * kmax * nslot;
  cudaError_t e = cudaMemsetAsync(out, 0xFF, 2 * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  k_minloc_value<real><<<grid_for(total, 256, sms), 256, 0, st>>>(conc, rhs, kact, nslot, kmax,
                                                                  dtr, out);
  k_minloc_index<real><<<grid_for(total, 256, sms), 256, 0, st>>>(
      conc, rhs, kact, slot_col, nslot, kmax, ncol, dtr, out, out + 1);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_trial(const real* conc, const real* rhs, const int* kact,
                         int nslot, int kmax, real dtr, real keep, real natol,
                         int* flag, int sms, cudaStream_t st) {
  const size_t total = (size_t)NTR * kmax * nslot;
  k_trial<real><<<grid_for(total, 256, sms), 256, 0, st>>>(conc, rhs, kact, nslot,
                                                          kmax, dtr, keep, natol, flag);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_accept(real* conc, const real* rhs, const int* kact, int nslot,
                          int kmax, real dtr, int sms, cudaStream_t st) {
  const size_t total = (size_t)NTR * kmax * nslot;
  k_accept<real><<<grid_for(total, 256, sms), 256, 0, st>>>(conc, rhs, kact, nslot,
                                                           kmax, dtr);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_epilogue(real* conc, const int* kact, int nslot, int kmax,
                            const Params<real>& p, DevStats* stats, int sms,
                            cudaStream_t st) {
  const size_t total = (size_t)NTR * kmax * nslot;
  k_epilogue<real><<<grid_for(total, 256, sms), 256, 0, st>>>(conc, kact, nslot,
                                                             kmax, p, stats);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_gather_range(const double* src, real* dst, const int* slot_col,
                                int ngroups, int kmax, int ncol, int nslot, int slot0,
                                int nseg, int sms, cudaStream_t st) {
  if (nseg <= 0) return cudaSuccess;
  const size_t total = (size_t)ngroups * kmax * nseg;
  k_gather<real><<<grid_for(total, 256, sms), 256, 0, st>>>(src, dst, slot_col, ngroups,
                                                           kmax, ncol, nslot, slot0, nseg);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_gather(const double* src, real* dst, const int* slot_col,
                          int ngroups, int kmax, int ncol, int nslot, int sms,
                          cudaStream_t st) {
  return launch_gather_range<real>(src, dst, slot_col, ngroups, kmax, ncol, nslot, 0,
                                   nslot, sms, st);
}

template <typename real>
cudaError_t launch_scatter_range(const real* src, double* dst, const int* slot_col,
                                 const int* kact, int ngroups, int kmax, int ncol,
                                 int nslot, int slot0, int nseg, int sms,
                                 cudaStream_t st) {
  if (nseg <= 0) return cudaSuccess;
  const size_t total = (size_t)ngroups * kmax * nseg;
  k_scatter<real><<<grid_for(total, 256, sms), 256, 0, st>>>(
      src, dst, slot_col, kact, ngroups, kmax, ncol, nslot, slot0, nseg);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_scatter(const real* src, double* dst, const int* slot_col,
                           const int* kact, int ngroups, int kmax, int ncol,
                           int nslot, int sms, cudaStream_t st) {
  return launch_scatter_range<real>(src, dst, slot_col, kact, ngroups, kmax, ncol, nslot,
                                    0, nslot, sms, st);
}

template <typename real>
cudaError_t launch_scatter_flux(const real* sflux, double* fluxes,
                                const int* slot_col, const int* kact, int ncol,
                                int nslot, int sms, cudaStream_t st) {
  const size_t total = (size_t)NDISS * nslot;
  k_scatter_flux<real><<<grid_for(total, 256, sms), 256, 0, st>>>(
      sflux, fluxes, slot_col, kact, ncol, nslot);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_prep_grid(const double* dz, const double* dzc,
                             const double* phi, const double* phi_i,
                             const double* biofac, const double* cap,
                             const double* mol, const int* slot_col, real* coef,
                             real* capd, int kmax, int ncol, int nslot, int mode,
                             double d0, int sms, cudaStream_t st) {
  const size_t total = (size_t)kmax * nslot;
  k_prep_grid<real><<<grid_for(total, 256, sms), 256, 0, st>>>(
      dz, dzc, phi, phi_i, biofac, cap, mol, slot_col, coef, capd, kmax, ncol,
      nslot, mode, d0);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_prep_force(const double* bdys, const double* fluxes,
                              const int* slot_col, real* force, int ncol,
                              int nslot, double bio, double diffusivity,
                              int mode, int bcup_d, int bio3, int sms, cudaStream_t st) {
  k_prep_force<real><<<grid_for(nslot, 128, sms), 128, 0, st>>>(
      bdys, fluxes, slot_col, force, ncol, nslot, bio, diffusivity, mode, bcup_d, bio3);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_rate_temperature(const real* base, real* tab, const int* slot_col,
                                    const double* bdys, const double* fac, double Ta,
                                    int nslot, int sms, cudaStream_t st) {
  k_rate_temperature<real><<<grid_for(nslot, 256, sms), 256, 0, st>>>(base, tab, slot_col,
                                                                     bdys, fac, Ta, nslot);
  return cudaGetLastError();
}

// The kernels of one profile-3 setting for every layers-per-lane / BcUp-4
// combination: the BIO3 = true set is compiled in its own translation unit
// (declared extern where the dispatchers are instantiated).
#define SED_VARIANT(prefix, real, BIO3)                                         \
  prefix template cudaError_t launch_column_k<real, 1, false, BIO3>(            \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_column_k<real, 1, true, BIO3>(             \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_column_k<real, 2, false, BIO3>(            \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_column_k<real, 2, true, BIO3>(             \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template int occupancy_k<real, 1, false, BIO3>(int, int, int);         \
  prefix template int occupancy_k<real, 1, true, BIO3>(int, int, int);          \
  prefix template int occupancy_k<real, 2, false, BIO3>(int, int, int);         \
  prefix template int occupancy_k<real, 2, true, BIO3>(int, int, int);

// The warp-direct kernels of one profile-3 setting.
#define SED_WARP_VARIANT(prefix, real, BIO3)                                    \
  prefix template cudaError_t launch_warp_k<real, 1, false, BIO3>(              \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_warp_k<real, 1, true, BIO3>(               \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_warp_k<real, 2, false, BIO3>(              \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_warp_k<real, 2, true, BIO3>(               \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template int warp_occupancy_k<real, 1, false, BIO3>(int, int);         \
  prefix template int warp_occupancy_k<real, 1, true, BIO3>(int, int);          \
  prefix template int warp_occupancy_k<real, 2, false, BIO3>(int, int);         \
  prefix template int warp_occupancy_k<real, 2, true, BIO3>(int, int);

// The kernels of the deepest class (64..127 layers, four per lane), one
// parameter set, compiled in their own translation units: the tile kernels
// and the warp-direct ones.
#define SED_DEEP_TILE_VARIANT(prefix, real, BIO3)                               \
  prefix template cudaError_t launch_column_k<real, 4, false, BIO3>(            \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_column_k<real, 4, true, BIO3>(             \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template int occupancy_k<real, 4, false, BIO3>(int, int, int);         \
  prefix template int occupancy_k<real, 4, true, BIO3>(int, int, int);
#define SED_DEEP_WARP_VARIANT(prefix, real, BIO3)                               \
  prefix template cudaError_t launch_warp_k<real, 4, false, BIO3>(              \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_warp_k<real, 4, true, BIO3>(               \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template int warp_occupancy_k<real, 4, false, BIO3>(int, int);         \
  prefix template int warp_occupancy_k<real, 4, true, BIO3>(int, int);
#define SED_DEEP_VARIANT(prefix, real, BIO3)                                    \
  SED_DEEP_TILE_VARIANT(prefix, real, BIO3)                                     \
  SED_DEEP_WARP_VARIANT(prefix, real, BIO3)

// The warp-direct kernels with a parameter set per column.
#define SED_WARP_ENS_VARIANT(prefix, real, BIO3)                                \
  prefix template cudaError_t launch_warp_ens<real, 1, false, BIO3>(            \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_warp_ens<real, 1, true, BIO3>(             \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_warp_ens<real, 2, false, BIO3>(            \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t); \
  prefix template cudaError_t launch_warp_ens<real, 2, true, BIO3>(             \
      const ColumnArgs<real>&, const Params<real>&, int, int, int, cudaStream_t);

#define SED_INSTANTIATE(real)                                                   \
  template size_t tile_smem_bytes<real>(int, int, bool, int, bool);             \
  template cudaError_t launch_column<real>(const ColumnArgs<real>&,             \
                                           const Params<real>&, int, bool, int, \
                                           int, int, cudaStream_t);             \
  template int column_blocks_per_sm<real>(int, int, bool, int, int, bool);      \
  template cudaError_t launch_minloc<real>(const real*, const real*, const int*, \
                                           const int*, int, int, int, real,     \
                                           unsigned long long*, int, cudaStream_t); \
  template cudaError_t launch_trial<real>(const real*, const real*, const int*, \
                                          int, int, real, real, real, int*,     \
                                          int, cudaStream_t);                   \
  template cudaError_t launch_accept<real>(real*, const real*, const int*, int, \
                                           int, real, int, cudaStream_t);       \
  template cudaError_t launch_epilogue<real>(real*, const int*, int, int,       \
                                             const Params<real>&, DevStats*,    \
                                             int, cudaStream_t);                \
  template cudaError_t launch_gather<real>(const double*, real*, const int*,    \
                                           int, int, int, int, int,             \
                                           cudaStream_t);                       \
  template cudaError_t launch_scatter<real>(const real*, double*, const int*,   \
                                            const int*, int, int, int, int,     \
                                            int, cudaStream_t);                 \
  template cudaError_t launch_gather_range<real>(const double*, real*,          \
                                                 const int*, int, int, int, int, \
                                                 int, int, int, cudaStream_t);  \
  template cudaError_t launch_scatter_range<real>(const real*, double*,         \
                                                  const int*, const int*, int,  \
                                                  int, int, int, int, int, int, \
                                                  cudaStream_t);                \
  template cudaError_t launch_scatter_flux<real>(const real*, double*,          \
                                                 const int*, const int*, int,   \
                                                 int, int, cudaStream_t);       \
  template cudaError_t launch_prep_grid<real>(                                  \
      const double*, const double*, const double*, const double*,               \
      const double*, const double*, const double*, const int*, real*, real*,    \
      int, int, int, int, double, int, cudaStream_t);                           \
  template cudaError_t launch_prep_force<real>(const double*, const double*,    \
                                               const int*, real*, int, int,     \
                                               double, double, int, int, int,   \
                                               int, cudaStream_t);              \
  template cudaError_t launch_rate_temperature<real>(                           \
      const real*, real*, const int*, const double*, const double*, double,     \
      int, int, cudaStream_t);                                                  \
  template cudaError_t launch_assemble_bc<real>(                                \
      const double*, const double*, const double*, unsigned, const real*,       \
      const int*, const double*, double*, double*, int, int, int, int, double,  \
      double, int, cudaStream_t);                                               \
  template cudaError_t launch_column_warp<real>(const ColumnArgs<real>&,       \
                                                const Params<real>&, int, bool, \
                                                int, int, int, cudaStream_t);   \
  template int column_warp_blocks_per_sm<real>(int, bool, int, int, bool);      \
  template cudaError_t launch_broadcast<real>(real*, const int*, int, int, int, \
                                              int, cudaStream_t);               \
  template cudaError_t launch_prep_bio3<real>(                                  \
      const double*, const double*, const double*, const double*,               \
      const double*, const double*, const int*, real*, int, int, int, double,   \
      double, int, cudaStream_t);

}  // namespace sed
