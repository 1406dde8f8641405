/*
 * mossco_sed.h -- C ABI of the GB300 sediment-column solver.
 *
 * A drop-in for MOSSCO's sediment-column hot path: the fabm_sediment
 * driver's right-hand side integrated by the solver_library ODE stepper
 * over every column of the grid.  Plain pointers and sizes only; every call
 * returns SED_OK (0) or a negative SED_E_* code.  A handle owns one CUDA
 * stream and its device buffers; calls on one handle are not thread safe.
 *
 * Array layout is the reference's Fortran order read backwards (C order):
 *   per cell      [ntr][kmax][ncol]  == conc(i,j,k,n), i fastest, col=i+inum*j
 *   per layer     [kmax][ncol]       == dz(i,j,k), porosity(i,j,k), ...
 *   dzc           [kmax-1][ncol]     == grid%dzc(i,j,k)
 *   bdys          [ntr+1][ncol]      == bdys(i,j,1:nvar+1), temperature first
 *   fluxes        [ntr][ncol]        == fluxes(i,j,1:nvar)
 * (src/components/fabm_sediment_component.F90:521,538-541).
 *
 * Reference interfaces replaced (paths inside platipodium/mossco-code):
 *   ode_solver(rhs_driver, dt, method)  src/utilities/solver_library.F90:80-90
 *   type_sed%get_rhs(rhs)               src/drivers/fabm_sediment_driver.F90:575-582
 *   Run-loop epilogue (NaN, clamp)      src/components/fabm_sediment_component.F90:1715-1732
 */
#ifndef MOSSCO_SED_H
#define MOSSCO_SED_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SED_NTR 11        /* OMEXDIA+P tracers, order in sed_tracer_name() */
#define SED_KMAX_LIMIT 127 /* layers per column the kernels hold on chip
                              (one, two or four per lane of a warp, the last
                              lane free) */

/* return codes */
#define SED_OK 0
#define SED_E_ARG (-1)          /* bad size, pointer or option */
#define SED_E_NAN (-2)          /* NaN in the state after a step */
#define SED_E_SUBSTEP_CAP (-3)  /* adaptive loop hit max_attempts */
#define SED_E_CUDA (-4)         /* CUDA runtime error */
#define SED_E_STATE (-5)        /* call order: grid / forcing / state missing */
#define SED_E_NOMEM (-6)        /* device or pinned allocation failed */
#define SED_E_NODEVICE (-7)     /* no CUDA device */
#define SED_E_TOO_LARGE (-9)    /* grid exceeds the no-allocation scratch */

/* Size of the device array behind sed_ode_solver_noalloc (64 MiB). */
#define SED_NOALLOC_SCRATCH_BYTES (64u << 20)

/* ode_solver methods (solver_library.F90:32-35) */
#define SED_EULER 0
#define SED_RUNGE_KUTTA_4 1
#define SED_ADAPTIVE_EULER 2
#define SED_RUNGE_KUTTA_4_38 3

/* step-cut scope of the adaptive method */
#define SED_CUT_PER_COLUMN 0 /* each column cuts its own substep */
#define SED_CUT_GLOBAL 1     /* one cut for the whole grid, as on one PET */

/* state precision on the device */
#define SED_FP32 0
#define SED_FP64 1

typedef struct sed_params {
  /* type_sed scalars (fabm_sediment_driver.F90:72-80, sed_nml :211-231) */
  double diffusivity;         /* cm2/d, molecular part for mol_diff_mode 0 */
  double bioturbation;        /* cm2/d */
  int bcup_dissolved;         /* 1 flux, 2 concentration, 3 zero flux */
  int bcup_particulate;       /* 1 flux, 4 capped flux cascade */
  int mol_diff_mode;          /* 0 (diffusivity+0.035 T) phi_i,
                                 1 mol_diff_d0 phi_i / (1 - 2 ln phi_i) */
  double mol_diff_d0;         /* m2/s */
  /* type_rhs_driver scalars (solver_library.F90:40-41) */
  double dt_min;              /* s */
  double relative_change_min; /* e.g. -0.9 */
  double atol;                /* absolute tolerance of the positivity test:
                                 a substep is rejected if c1 - (1+rcm) c <
                                 -atol in any cell (0: the reference's test,
                                 solver_library.F90:121) */
  int max_attempts;           /* adaptive attempts per column-step, > 0 */
  int cut_scope;              /* SED_CUT_PER_COLUMN or SED_CUT_GLOBAL */
  /* OMEXDIA+P, per-day units (examples/standalone/omexdia_p/fabm_sed.nml) */
  double rLabile, rSemilabile, NCrLdet, NCrSdet, PAds, PAdsODU, NH3Ads,
      CprodMax, rnit, ksO2nitri, rODUox, ksO2oduox, ksO2oxic, ksNO3denit,
      kinO2denit, kinNO3anox, kinO2anox;
  /* component epilogue (fabm_sediment_component.F90:1718-1732) */
  int epilogue;               /* 1: NaN check + clamp after each step */
  double minimum[SED_NTR];    /* clamp value per tracer */
  /* device options */
  int precision;              /* SED_FP32 (default) or SED_FP64 */
  int budgets;                /* 1: FP64 P and N budgets per column-step */
  int device;                 /* CUDA ordinal */
  /* bioturbation_profile (fabm_sediment_driver.F90:73,204): 3 recomputes the
   * bioturbation factor from the TOC profile at every right-hand side
   * (Zhang & Wirtz 2017, get_rhs :618-645; biofac of sed_set_grid and the
   * temperature factor are then unused); any other value uses biofac.  The
   * constants are sed_nml's bioturb_* (:226-231). */
  int bioturbation_profile;
  double bioturb_k_l, bioturb_L1, bioturb_L2, bioturb_beta, bioturb_b,
      bioturb_dry_density;
  /* Temperature dependence of the microbial rates (K).  The reference hands
   * the column temperature to the reaction model at every right-hand side
   * (fabm_sediment_driver.F90:613); with temp_activation > 0, rLabile,
   * rSemilabile, CprodMax, rnit and rODUox are multiplied in each column by
   * exp(-temp_activation (1/(T+273) - 1/288)), T = bdys[0] in degC: the
   * Arrhenius form and reference temperature the driver applies to
   * bioturbation (:648, with 4500 K).  0 (default): rates independent of
   * temperature.  > 0 steps with per-column cuts and the warp-direct
   * kernels, as per-column parameter sets do; the surrogate, training rows,
   * sed_get_rhs and sed_ode_solver_noalloc refuse it. */
  double temp_activation;
  /* type_rhs_driver's adaptive_solver_diagnostics (solver_library.F90:43,
   * :129-136): with SED_CUT_GLOBAL, every accepted adaptive substep smaller
   * than the smallest so far records its size and the grid cell of the
   * smallest relative change (c1 - c) / c; see sed_get_min_dt_grid_cell. */
  int adaptive_solver_diagnostics;
} sed_params;

typedef struct sed_stats {
  long long attempts;     /* adaptive attempts, summed over columns */
  long long accepted;     /* accepted substeps */
  long long column_steps; /* active columns x coupling steps */
  int max_col_attempts;   /* max attempts of one column in one step */
  int capped_columns;     /* column-steps that hit max_attempts */
  int nan_cells;          /* NaN cells found by the epilogue */
  int gpu_launches;       /* kernels this library launched for the call */
  double min_dt;          /* smallest accepted substep (s) */
  double device_ms;       /* device time of the call's steps (CUDA events
                             on the handle's stream) */
  long long surrogate_columns; /* column-steps taken by the surrogate */
} sed_stats;

typedef struct sed_handle sed_handle;

/* Reference defaults: sed_nml defaults, BcUp 2/1, dt_min 1e-9, -0.9,
 * hzg_omexdia_p parameters of fabm_sed.nml:51-77, clamp at 0, FP32. */
int sed_default_params(sed_params *p);

/* Create a solver for an inum x jnum grid of kmax layers (kmax <=
 * SED_KMAX_LIMIT) and ntr tracers (must be SED_NTR).  Replaces the
 * allocations of fabm_sediment_component.F90:521-541 and
 * type_sed%initialize. */
int sed_create(const sed_params *p, int inum, int jnum, int kmax, int ntr,
               sed_handle **out);

/* Grid and porosity (fabm_sediment_driver.F90:127-177, :278-304, :430-435).
 * flux_cap may be NULL unless bcup_particulate == 4.  kact[ncol] gives the
 * active layers per column (0 = land); when NULL, mask[kmax][ncol] (the
 * reference's mask, > 0 masked, whole columns or a masked tail only) is
 * used; when both are NULL every column is active with kmax layers. */
int sed_set_grid(sed_handle *h, const double *dz, const double *dzc,
                 const double *phi, const double *phi_i, const double *biofac,
                 const double *flux_cap, const int *kact, const int *mask);

/* Boundary conditions of get_boundary_conditions
 * (fabm_sediment_component.F90:1865-2030): bdys[0] is temperature. */
int sed_set_forcing(sed_handle *h, const double *bdys, const double *fluxes);

/* Boundary conditions assembled on the device from the pelagic fields at the
 * soil surface, as get_boundary_conditions does each coupling step
 * (fabm_sediment_component.F90:1865-2030), so a device-resident state needs
 * no host round trip:
 *   temperature[ncol]    -> bdys[0]
 *   surface[ntr][ncol]   pelagic concentration of each tracer at the soil
 *                        surface (`<name>_at_soil_surface`)
 *   velocity[ntr][ncol]  its vertical velocity, m/s, negative downward
 *                        (`<name>_z_velocity_at_soil_surface`); read for
 *                        particulate tracers only, may be NULL if none is
 *                        present
 *   present[ntr]         nonzero where the import state holds the tracer
 *                        (NULL: all); absent tracers keep their values
 * Particulate: fluxes[n] = -surface * velocity (:1978,1986).  Dissolved:
 * bdys[n+1] = surface, fluxes[n] = the diffusive estimate of :2012-2014 from
 * the state's first layer when bcup_dissolved is 1 (needs the state; 0 for
 * land columns), else 0.  Then the step's forcing rows are formed, as
 * sed_set_forcing does. */
int sed_set_boundary(sed_handle *h, const double *temperature,
                     const double *surface, const double *velocity,
                     const int *present);
/* The handle's current bdys [ntr+1][ncol] and fluxes [ntr][ncol] (either
 * may be NULL).  After a step the dissolved rows of fluxes hold that step's
 * surface fluxes, as get_rhs writes them (:692). */
int sed_get_boundary(sed_handle *h, double *bdys, double *fluxes);

int sed_set_state(sed_handle *h, const double *conc);
int sed_get_state(sed_handle *h, double *conc);

/* nsteps coupling steps of length dt on the device-resident state (each a
 * captured CUDA graph); forcing stays as last set. */
int sed_step(sed_handle *h, double dt, int method, int nsteps,
             sed_stats *stats);

/* Spin-up before the run (fabm_sediment_component.F90:557-632: presimulation
 * years of hourly ode_solver calls on a 1-column model, whose profile is then
 * copied into every unmasked column).  nsteps coupling steps of dt with
 * constant forcing, each warp keeping its column in registers for up to 24
 * steps per launch.  Needs the initial state (sed_set_state).
 *   SED_SPINUP_COLUMN: the reference's scheme.  Column `column` of the grid
 *     (-1: the first column with the most active layers) is integrated alone
 *     with bdys1[ntr+1] / fluxes1[ntr] (the namelist's bottom water and
 *     deposition fluxes), then its profile is copied into every other active
 *     column (their first min(K, K_column) layers).  The handle's own forcing
 *     is left as it was.
 *   SED_SPINUP_ALL: every active column is integrated with its own forcing
 *     (sed_set_forcing / sed_set_boundary); bdys1 and fluxes1 are unused.
 *     On the GPU this costs about as much as one column.
 * The caller sets bcup_dissolved and bioturbation_profile as the reference
 * does for its sed1d (:598-600). */
#define SED_SPINUP_COLUMN 0
#define SED_SPINUP_ALL 1
int sed_spinup(sed_handle *h, int mode, int column, const double *bdys1,
               const double *fluxes1, double dt, int method, long long nsteps,
               sed_stats *stats);

/* Drop-in for `call ode_solver(sed, dt, method)` followed by the component
 * epilogue: conc is the caller's host array, updated in place; fluxes is
 * read (flux boundaries) and its dissolved rows are overwritten with the
 * surface flux of the last right-hand side, as get_rhs does (:692). */
int sed_ode_solver(sed_handle *h, double *conc, const double *bdys,
                   double *fluxes, double dt, int method, sed_stats *stats);

/* Drop-in for type_sed%get_rhs (fabm_sediment_driver.F90:575-717): rhs of
 * conc with the current forcing; fluxes as in sed_ode_solver. */
int sed_get_rhs(sed_handle *h, const double *conc, double *rhs,
                double *fluxes);

/* Surface fluxes [ntr][ncol] after the last step (dissolved rows). */
int sed_get_fluxes(sed_handle *h, double *fluxes);

/* Per column of the last step: attempts [ncol] (0 on land). */
int sed_get_attempts(sed_handle *h, int *attempts);

/* Substep histogram of the last step (no counterpart in the reference,
 * whose solver logs each cut): counts[SED_HIST_BINS] over the active
 * columns, bin 0 the columns without an attempt (taken by the surrogate),
 * bin b >= 1 those with 2^(b-1) <= attempts < 2^b, the last bin every
 * count above.  Formed on the device from the per-column attempt counters. */
#define SED_HIST_BINS 16
int sed_get_attempt_histogram(sed_handle *h, long long *counts);

/* Smallest accepted substep of every column in the last step, [ncol] (s;
 * 0 for land columns and columns without one): the per-column form of
 * type_rhs_driver's last_min_dt (solver_library.F90:130-136); the grid's
 * minimum and its column are the minimum and argmin of this array. */
int sed_get_min_dt(sed_handle *h, double *min_dt);

/* Ensembles (no counterpart in the reference, whose rates take the one
 * parameter set of fabm_sed.nml): an OMEXDIA+P parameter set per column,
 * params[SED_NBGC][ncol] in sed_params' order and units (rLabile ...
 * kinO2anox, per day), so that many parameter sets -- a calibration, a
 * sensitivity study, an ensemble spin-up with SED_SPINUP_ALL -- run as the
 * columns of one grid in one launch.  NULL returns every column to the
 * handle's set.  With per-column sets the handle steps with the
 * warp-direct kernels (tile width 0; sed_set_tuning refuses others) and
 * per-column cuts; sed_get_rhs and the surrogate step answer SED_E_STATE.
 * A column whose set equals the handle's gives the same bits as without. */
#define SED_NBGC 17
int sed_set_column_bgc(sed_handle *h, const double *params);

/* type_rhs_driver's last_min_dt and last_min_dt_grid_cell
 * (solver_library.F90:44-45, :129-136), kept across calls since sed_create:
 * 1e20 (as a default real) and -99 until a recording substep.  cell[4] =
 * (i, j, k, n), 1-based, of the smallest relative change in the substep
 * that set last_min_dt; NaN quotients are skipped (gfortran's MINLOC), and
 * cells the solver does not step count with relative change 0.  Recorded by
 * the grid-wide cut (SED_CUT_GLOBAL) with adaptive_solver_diagnostics set;
 * SED_E_STATE otherwise. */
int sed_get_min_dt_grid_cell(sed_handle *h, double *last_min_dt, int *cell);

/* FP64 budgets of the last step, [4][ncol]: P inventory, P residual,
 * N inventory, N residual (mmol/m2).  Requires params.budgets. */
int sed_get_budgets(sed_handle *h, double *budgets);

/* Run the handle's work on a caller's CUDA stream (a cudaStream_t passed
 * as void*; NULL restores the handle's own stream).  The stream must not be
 * the legacy default stream, because a step is captured as a CUDA graph. */
int sed_set_stream(sed_handle *h, void *stream);

/* Pin (or unpin) a caller's host array so copies run at full speed. */
int sed_host_register(void *ptr, size_t bytes);
int sed_host_unregister(void *ptr);
/* Pinned host memory from the CUDA allocator (no counterpart in the
 * reference): a caller that allocates its state, bdys and fluxes arrays
 * here gets the drop-in calls' column-chunk copies at the link's rate.  On
 * the Grace hosts measured, the same copies from malloc'd memory pinned
 * with sed_host_register ran 8-10x slower for multi-GB arrays.  *ptr is
 * NULL on failure; free with sed_host_free. */
int sed_host_alloc(size_t bytes, void **ptr);
int sed_host_free(void *ptr);

/* ------------------------------------------------------------------------
 * Launch tuning (no counterpart in the reference, whose solver has no
 * launch parameters).  Index [0] of the per-class fields is the class of
 * columns with up to 31 active layers (one layer per lane), [1] the class
 * with 32..63 (two layers per lane); the class with 64..127 (four layers
 * per lane) keeps the defaults.  sed_set_grid lays the active columns
 * out once (depth class, then `segments` contiguous column ranges balanced
 * by active layers, each padded to 64 slots), so every tuning below is a
 * pure launch choice: results are bit-identical under any of them.  The
 * defaults are the warp-direct kernel with 128 threads for FP32 state and
 * tiles of 32 / 16 columns with 256 threads for FP64. */
typedef struct sed_tuning {
  int tile_columns[2];  /* columns staged per tile: 8, 16, 32 or 64; 0 = the
                           warp-direct kernel: every warp steps one column
                           at a time in global memory, no tiles */
  int threads[2];       /* threads per block: 64, 128, 192 or 256 */
  int blocks_per_sm[2]; /* resident blocks per SM of the persistent grid;
                           0 = as many as fit */
  int pipeline_chunks;  /* sed_ode_solver: column ranges whose host->device
                           copy, step and device->host copy run in flight
                           (1 = copy all, step, copy back); divides segments */
  int segments;         /* column ranges of the layout (read-only) */
  int max_attempts;     /* substep cap per column-step (= sed_params one) */
  float step_ms;        /* sed_autotune: one coupling step, tuned */
  float ode_solver_ms;  /* sed_autotune with SED_TUNE_PIPELINE: one
                           sed_ode_solver call, tuned */
  int trials;           /* sed_autotune: candidate launches timed */
} sed_tuning;

#define SED_TUNE_PIPELINE 1 /* also time sed_ode_solver's pipeline depth
                               (pinned host scratch of one FP64 state) */
#define SED_TUNE_CAP 2      /* also set max_attempts to 4x the largest
                               per-column attempt count seen (>= 64) */

int sed_get_tuning(const sed_handle *h, sed_tuning *t);
/* Validates every field (SED_E_ARG) and that each class's tile fits the
 * device (SED_E_CUDA); the output-only fields are ignored. */
int sed_set_tuning(sed_handle *h, const sed_tuning *t);
/* Times candidate tile widths and block sizes per depth class (and, with
 * flags, the pipeline depth and the substep cap) on the handle's current
 * state and forcing, keeps the fastest, and restores the state, surface
 * fluxes and diagnostics it found.  Needs sed_set_state (or a previous
 * sed_ode_solver) and sed_set_forcing.  out may be NULL. */
int sed_autotune(sed_handle *h, double dt, int method, int flags,
                 sed_tuning *out);

/* One coupling step of the drop-in above for callers that cannot allocate
 * device memory (no counterpart in the reference).  Some callers cannot
 * call cudaMalloc: a component whose framework owns the GPU's memory pool
 * and forbids other allocators, or a call site that cannot keep a solver
 * handle (and the buffers sed_create allocates) alive between calls.  This
 * call creates no handle and allocates nothing: every device buffer of the
 * step lives in one static device array of SED_NOALLOC_SCRATCH_BYTES, which
 * each GPU that loads the library holds until the process exits.  The
 * arguments are the host arrays of sed_set_grid and sed_ode_solver (conc
 * and fluxes updated in place); p must ask for SED_FP32 state and
 * per-column cuts, and budgets are not computed.  A grid whose buffers do
 * not fit the array (about 4.7 KB per column at 30 layers, so ~14 000
 * columns) is rejected with SED_E_TOO_LARGE.  The call runs the tile form
 * of the column kernel on the array; its results equal sed_ode_solver's bit
 * for bit.  Every call looks up the array's device address in the current
 * context of p->device (the first call in a context loads the module; make
 * that first call before any stream capture), so a cudaDeviceReset by the
 * caller between calls is harmless.  All calls share the array, so calls
 * that overlap on the GPU (from several host threads of one process) race.
 * The work runs on the calling thread's per-thread default stream
 * (cudaStreamPerThread), so it does not wait for other streams of the
 * device, and the call returns when it is done.  After an error return the
 * caller's conc and fluxes are unchanged. */
int sed_ode_solver_noalloc(const sed_params *p, int inum, int jnum, int kmax,
                           const double *dz, const double *dzc,
                           const double *phi, const double *phi_i,
                           const double *biofac, const double *flux_cap,
                           const int *kact, double *conc, const double *bdys,
                           double *fluxes, double dt, int method,
                           sed_stats *stats);

/* ------------------------------------------------------------------------
 * Column-increment surrogate (no counterpart in the reference): an MLP
 * nin -> hidden (x nhidden, GELU) -> nout with BF16 tensor-core products,
 * FP32 accumulation and FP32 master weights trained with Adam.  Parameters
 * are exchanged unpadded, layer by layer: W[out][in] then b[out]. */
typedef struct sed_surrogate sed_surrogate;
int sed_sur_create(int nin, int nout, int hidden, int nhidden, int max_batch,
                   unsigned long long seed, int device, sed_surrogate **out);
int sed_sur_num_params(const sed_surrogate *s);
int sed_sur_set_weights(sed_surrogate *s, const float *params);
int sed_sur_get_weights(sed_surrogate *s, float *params);
/* Checkpoint of the training state: state[sed_sur_state_size(s)] holds the
 * parameters, then Adam's first and second moments (each in the layout of
 * sed_sur_get_weights), and *step Adam's step count.  Training resumed from
 * a checkpoint on the same batches gives the same parameters, bit for bit,
 * as training without the interruption. */
int sed_sur_state_size(const sed_surrogate *s);
int sed_sur_get_state(sed_surrogate *s, float *state, long long *step);
int sed_sur_set_state(sed_surrogate *s, const float *state, long long step);
/* host rows x[m][nin] -> y[m][nout] */
int sed_sur_forward(sed_surrogate *s, const float *x, float *y, int m);
/* device rows: x BF16 [m][pad128(nin)] -> y FP32 [m][pad128(nout)],
 * m a multiple of 128, both arrays 16-byte aligned (else SED_E_ARG) */
int sed_sur_forward_device(sed_surrogate *s, const void *x_dev, void *y_dev,
                           int m);
/* one Adam step on a device batch (x BF16 [m][pad128(nin)], y BF16
 * [m][pad128(nout)], m a multiple of 128, <= max_batch); loss may be NULL */
int sed_sur_train_step(sed_surrogate *s, const void *x_dev, const void *y_dev,
                       int m, float lr, float *loss);
/* MSE loss and its parameter gradients for host rows (no update) */
int sed_sur_grads(sed_surrogate *s, const float *x, const float *y, int m,
                  float *grads, float *loss);
/* Tensor-core engine (no counterpart in the reference).  On (the default):
 * the network's inference -- sed_sur_forward_device and the surrogate step
 * -- runs as one fused kernel on the tcgen05 tensor cores (accumulators in
 * tensor memory, operands staged by TMA) when the shape fits (input width
 * up to 384, hidden width 256, output width up to 512), and the training
 * products (sed_sur_train_step, sed_sur_grads, sed_sur_forward: forward
 * with kept pre-activations, input and weight gradients) run as tcgen05
 * GEMMs.  Off: every product runs as an mma.sync GEMM.  Returns 1 when the
 * fused inference kernel is in use, 0 when not, < 0 on error. */
int sed_sur_set_tensor_cores(sed_surrogate *s, int on);
/* Run the surrogate's work on a caller's CUDA stream (a cudaStream_t as
 * void*; NULL restores its own stream). */
int sed_sur_set_stream(sed_surrogate *s, void *stream);
const char *sed_sur_last_error(const sed_surrogate *s);
/* Normalisation of the column surrogate, n = 11 + 2 nin + 2 nout floats:
 * c0[11] | mu_x[nin] | sd_x[nin] | mu_d[nout] | sd_d[nout], with nin =
 * 11 K + 13 and nout = 11 K for a grid of K layers. */
int sed_sur_set_norm(sed_surrogate *s, const float *norm, int n);
/* nsteps coupling steps of the handle's device state with the surrogate
 * (FP32 state, per-column cuts, every active column at kmax <= 63 layers).
 * Each
 * step runs:
 *   1. the gate: every column's first adaptive attempt, the whole step at
 *      once.  A column whose attempt is accepted is done, with exactly the
 *      plain step's result (most columns, most steps); the others -- whose
 *      plain step would take many substeps -- are listed;
 *   2. the network's proposal for the listed columns;
 *   3. the residual test of each proposal P with the plain right-hand side:
 *      P is taken when dt |f(P)| <= tol (|P| + res_atol) in every cell (a
 *      state the plain dynamics would move by at most tol of its value over
 *      a step); NaN fails;
 *   4. the plain adaptive solver on the listed columns whose proposal failed.
 * With tol = 0 nothing is taken and the result equals sed_step's bit for
 * bit.  stats.surrogate_columns counts the column-steps taken from the
 * network; their attempts count 0 and their budgets are zero. */
int sed_step_surrogate(sed_handle *h, sed_surrogate *s, double dt, int nsteps,
                       double tol, double res_atol, sed_stats *stats);
/* The drop-in call with the surrogate: sed_ode_solver's arguments (host
 * arrays conc [ntr][kmax][ncol] in and out, bdys, fluxes in and out) and one
 * gated surrogate coupling step as sed_step_surrogate takes it, with the
 * state's host<->device copies pipelined over the column segments: each
 * segment is gated as it arrives, and copied back as soon as its columns are
 * done.  Results equal sed_set_state + sed_step_surrogate + sed_get_state,
 * bit for bit. */
int sed_ode_solver_surrogate(sed_handle *h, sed_surrogate *s, double *conc,
                             const double *bdys, double *fluxes, double dt,
                             double tol, double res_atol, sed_stats *stats);

/* Training rows from the plain solver: one plain adaptive coupling step of
 * the handle's device state (FP32, per-column cuts, every active column at
 * kmax layers), then a row for every column whose step took more than one
 * attempt -- the columns step 1 of sed_step_surrogate hands to the network.
 * Rows go to caller device arrays (FP32), starting at row *count:
 *   x[row][0 .. 11 K)        log(max(C, 0) + c0[n]) before the step,
 *                            tracer-major (n K + k)
 *   x[row][11 K .. 11 K+13)  the column's 13 forcing rows
 *   y[row][0 .. 11 K)        log(max(C', 0) + c0[n]) - the same before
 * with row pitches pitch_x, pitch_y (floats).  Rows past capacity are
 * dropped; *count returns min(rows so far, capacity). */
int sed_sur_collect(sed_handle *h, const float *c0, double dt, float *x_dev,
                    float *y_dev, int pitch_x, int pitch_y,
                    long long capacity, long long *count, sed_stats *stats);
void sed_sur_destroy(sed_surrogate *s);

const char *sed_error_string(int code);
const char *sed_last_error(const sed_handle *h);
const char *sed_tracer_name(int n);
int sed_tracer_is_particulate(int n);

void sed_destroy(sed_handle *h);

#ifdef __cplusplus
}
#endif
#endif
