// sed_launch.h -- host-visible kernel arguments and launchers.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "sed_device.cuh"

namespace sed {

// KIND_PROBE and KIND_SUR are the surrogate step's gate (tile kernel) and
// its residual test with the plain fallback (warp-direct kernel), FP32 state
enum : int { KIND_ADAPT = 0, KIND_FIXED = 1, KIND_RHS = 2, KIND_SUR = 3, KIND_PROBE = 4 };

// Arguments of the tile kernel.  Device layouts (slot = compacted column):
//   conc  [NTR][kmax][nslot]     coef  [coef_rows][kmax][nslot]
//   cap   [kmax][nslot] (BcUp 4) force [NFORCE][nslot]
//   sflux [NDISS][nslot]         budget[4][nslot] (FP64)
template <typename real>
struct ColumnArgs {
  real* conc;
  real* out;          // KIND_RHS destination
  const real* coef;
  const real* cap;
  const real* force;
  const int* kact;    // [nslot]
  const int* tile_k;  // layers to stage per tile, tile_k[tile0 + tile]; null:
                      // stage min(kmax, 32 x layers per lane) layers
  real* sflux;
  double* budget;     // may be null
  int* nsub;          // [nslot] attempts of the last step
  double* mindt;      // [nslot] smallest accepted substep of the last step
                      // (0: no substep); may be null
  unsigned* queue;    // tile counter, zero before the launch
  DevStats* stats;
  // the launch covers slots [slot0, slot0 + ntiles * tc); tile0 indexes tile_k
  int nslot, kmax, tc, slot0, tile0, ntiles;
  double dt;
  int method;
  // surrogate coupling step (KIND_SUR): the tolerances of the residual test;
  // a proposal that passes is written into conc, a column whose proposal
  // fails takes the plain adaptive step
  double res_tol, res_atol;
  // warp-direct kernel: the launch's columns are list[0 .. ntiles) (slots)
  // instead of the slot range.  KIND_PROBE (tile kernel) appends the slot of
  // every column whose first attempt was rejected to heavy[], reserving each
  // tile's entries with one atomicAdd on *nheavy
  const int* list;
  int* heavy;
  unsigned* nheavy;
  // warp-direct kernel with a list: when set, the list's length on the
  // device (the gate's count); the launch covers min(ntiles, *nlist) columns
  const unsigned* nlist;
  // KIND_SUR: the network's prediction rows (row j for the list's j-th
  // column, pitch ldy) and its normalisation c0[11] | mu_x[nin] | sd_x[nin] |
  // mu_d[nout] | sd_d[nout]
  const float* yhat;
  const float* norm;
  int ldy, nin, nout;
  // KIND_PROBE: the network's input rows of the rejected columns, BF16 bits
  // [row][pin], row i for heavy[i]: the standardised log(max(C, 0) + c0)
  // of the 11 K state values (tracer-major) and the 13 forcing rows, zero
  // up to pin (normalisation in norm, nin = 11 K + 13); null: none
  unsigned short* xfeat;
  int pin;
  // warp-direct kernel: coupling steps per launch with constant forcing
  // (0 or 1: one); each warp keeps its column in registers between them
  int nrepeat;
  // warp-direct kernel: per-slot OMEXDIA+P rate parameters [NBGC_DEV][nslot]
  // (an ensemble of parameter sets), or null for the Params set
  const real* bgc;
};

template <typename real>
size_t tile_smem_bytes(int tc, int lpl, bool bc4, int kind, bool bio3);

template <typename real>
cudaError_t launch_column(const ColumnArgs<real>& a, const Params<real>& p,
                          int lpl, bool bc4, int kind, int blocks, int threads,
                          cudaStream_t st);

template <typename real>
int column_blocks_per_sm(int tc, int lpl, bool bc4, int kind, int threads, bool bio3);

// Warp-direct column kernel (tile width 0 in the tuning; the stepping
// kinds): every warp pulls single columns from the work counter and
// reads and writes them in global memory, with no shared tiles and no block
// barriers.  a.ntiles counts the range's slots.
template <typename real>
cudaError_t launch_column_warp(const ColumnArgs<real>& a, const Params<real>& p, int lpl,
                               bool bc4, int kind, int blocks, int threads, cudaStream_t st);
template <typename real>
int column_warp_blocks_per_sm(int lpl, bool bc4, int kind, int threads, bool bio3);

// adaptive_solver_diagnostics: out[0] = order key of the smallest relative
// change (c1 - c) / c over the active cells of the substep dtr, out[1] =
// the smallest Fortran element index holding it (all ones: none)
template <typename real>
cudaError_t launch_minloc(const real* conc, const real* rhs, const int* kact, const int* slot_col,
                          int nslot, int kmax, int ncol, real dtr, unsigned long long* out,
                          int sms, cudaStream_t st);

template <typename real>
cudaError_t launch_trial(const real* conc, const real* rhs, const int* kact,
                         int nslot, int kmax, real dtr, real keep, real natol,
                         int* flag, int sms, cudaStream_t st);

template <typename real>
cudaError_t launch_accept(real* conc, const real* rhs, const int* kact,
                          int nslot, int kmax, real dtr, int sms,
                          cudaStream_t st);

template <typename real>
cudaError_t launch_epilogue(real* conc, const int* kact, int nslot, int kmax,
                            const Params<real>& p, DevStats* stats, int sms,
                            cudaStream_t st);

template <typename real>
cudaError_t launch_gather(const double* src, real* dst, const int* slot_col,
                          int ngroups, int kmax, int ncol, int nslot, int sms,
                          cudaStream_t st);

// the same restricted to slots [slot0, slot0 + nseg) of [ngroups][kmax][nslot]
template <typename real>
cudaError_t launch_gather_range(const double* src, real* dst, const int* slot_col,
                                int ngroups, int kmax, int ncol, int nslot, int slot0,
                                int nseg, int sms, cudaStream_t st);

template <typename real>
cudaError_t launch_scatter(const real* src, double* dst, const int* slot_col,
                           const int* kact, int ngroups, int kmax, int ncol,
                           int nslot, int sms, cudaStream_t st);

template <typename real>
cudaError_t launch_scatter_range(const real* src, double* dst, const int* slot_col,
                                 const int* kact, int ngroups, int kmax, int ncol,
                                 int nslot, int slot0, int nseg, int sms,
                                 cudaStream_t st);

template <typename real>
cudaError_t launch_scatter_flux(const real* sflux, double* fluxes,
                                const int* slot_col, const int* kact, int ncol,
                                int nslot, int sms, cudaStream_t st);

template <typename real>
cudaError_t launch_prep_grid(const double* dz, const double* dzc,
                             const double* phi, const double* phi_i,
                             const double* biofac, const double* cap,
                             const double* mol, const int* slot_col, real* coef,
                             real* capd, int kmax, int ncol, int nslot, int mode,
                             double d0, int sms, cudaStream_t st);

template <typename real>
cudaError_t launch_prep_force(const double* bdys, const double* fluxes,
                              const int* slot_col, real* force, int ncol,
                              int nslot, double bio, double diffusivity,
                              int mode, int bcup_d, int bio3, int sms, cudaStream_t st);

// temperature-dependent rates: tab = base with the microbial rate rows
// scaled by each column's factor (fac[ncol] from the host, or NULL to form
// it from the temperature row bdys[0][ncol])
template <typename real>
cudaError_t launch_rate_temperature(const real* base, real* tab, const int* slot_col,
                                    const double* bdys, const double* fac, double Ta,
                                    int nslot, int sms, cudaStream_t st);

// spin-up: the profile of slot src into every other active slot
template <typename real>
cudaError_t launch_broadcast(real* conc, const int* kact, int src, int nslot, int kmax, int sms,
                             cudaStream_t st);

// boundary conditions from the pelagic fields at the soil surface
template <typename real>
cudaError_t launch_assemble_bc(const double* temperature, const double* surface,
                               const double* velocity, unsigned present_mask, const real* conc,
                               const int* col_slot, const double* top, double* bdys,
                               double* fluxes, int ncol, int nslot, int kmax, int bcup_d,
                               double bioturbation, double diffusivity, int sms,
                               cudaStream_t st);

// coefficient rows of bioturbation profile 3 (after launch_prep_grid)
template <typename real>
cudaError_t launch_prep_bio3(const double* dz, const double* dzc, const double* phi_i,
                             const double* e1, const double* e2, const double* cum,
                             const int* slot_col, real* coef, int kmax, int ncol, int nslot,
                             double L1, double L2, int sms, cudaStream_t st);

}  // namespace sed
