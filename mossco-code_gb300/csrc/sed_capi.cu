// sed_capi.cu -- host side of the C ABI declared in include/mossco_sed.h.
//
// A handle owns one CUDA stream, the device-resident column state and the
// per-layer coefficients.  Active columns are compacted into "slots" (land
// columns are never touched on the device): depth class, then column
// segment, then active-layer count.  Columns of up to 31 layers run one
// layer per lane, deeper ones (to 63) two.  Each class is stepped by the
// tile kernel (tiles of tc slots) or the warp-direct kernel, as tuned.  A
// coupling step is a captured CUDA graph (queue reset + one persistent
// kernel per depth class), replayed for every step.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mossco_sed.h"
#include "cpl_internal.h"
#include "sed_launch.h"
#include "sed_params.h"
#include "sur_internal.h"
#include "sur_loop.h"

// A named NVTX range over the rest of the enclosing scope: profilers (nsys,
// ncu --nvtx) show every entry point's span on the timeline.  Without a
// profiler attached the push and pop are a check of a function pointer.
struct NvtxScope {
  explicit NvtxScope(const char* name) { nvtxRangePushA(name); }
  ~NvtxScope() { nvtxRangePop(); }
  NvtxScope(const NvtxScope&) = delete;
  NvtxScope& operator=(const NvtxScope&) = delete;
};

using namespace sed;

namespace {

const char* kTracerNames[SED_NTR] = {
    "detritus_labile_carbon",       "detritus_semilabile_carbon",
    "detritus_labile_nitrogen",     "detritus_semilabile_nitrogen",
    "detritus_labile_phosphorus",   "adsorbed_phosphorus",
    "dissolved_oxygen",             "dissolved_nitrate",
    "dissolved_ammonium",           "dissolved_reduced_substances",
    "dissolved_phosphate"};

// Column ranges of the layout, and work counters: 2 for whole-class
// launches, 2 per pipeline chunk and class.
constexpr int kMaxSeg = 8;
// depth classes: up to 31 active layers (one per lane of a warp), 32..63
// (two), 64..127 (four); the first two are the tunable ones of sed_tuning
constexpr int kBins = 3;
constexpr int kTunedBins = 2;
constexpr int kQueues = kBins + kBins * kMaxSeg;
inline int depth_class(int k) { return k <= 31 ? 0 : (k <= 63 ? 1 : 2); }
constexpr int kSlotPad = 64;  // every segment is a multiple of every tile width

// One depth class: its slots, split into the segments of the column ranges,
// and its launch tuning.
struct Bin {
  int lpl = 1;
  int slot0 = 0, nslots = 0;       // slot range of the class
  int segb[kMaxSeg + 1] = {};      // segment s = slots [segb[s], segb[s+1])
  int tc = 32, threads = 256;      // tile width (0: warp-direct), threads per block
  int bps = 0;                     // blocks per SM asked for (0 = all that fit)
  int occ = 0;                     // blocks per SM that fit at (tc, threads)
  int tc_fb = 32, occ_tile = 0;    // warp-direct classes: the tile kernel
                                   // (widest of 32/16/8 that fits) serving
                                   // the other kinds
  int tk0 = 0;                     // first tile of the class in tile_k
  int blocks(int sms, int ntiles) const {
    const int per = (bps > 0 && bps < occ) ? bps : occ;
    return std::max(1, std::min(ntiles, per * sms));
  }
};

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
    if (p) { cudaFree(p); p = nullptr; bytes = 0; }
    cudaError_t e = cudaMalloc(&p, b ? b : 16);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

struct sed_handle {
  sed_params prm{};
  int inum = 0, jnum = 0, ncol = 0, kmax = 0;
  int device = 0, sms = 0;
  cudaStream_t stream = nullptr;      // stream in use
  cudaStream_t own_stream = nullptr;  // stream created by the handle
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  bool have_grid = false, have_forcing = false, have_state = false;
  // per-column OMEXDIA+P parameter sets (sed_set_column_bgc), [SED_NBGC][ncol]
  bool has_bgc = false;
  // temperature-dependent rates: the per-slot table is d_bgc_base scaled by
  // each column's factor whenever the forcing changes; rfac_host: d_rfac
  // holds the factors of the current forcing formed on the host (FP64)
  bool rfac_host = false;
  std::vector<double> bgc_cols;
  // slots: depth class, then column segment, then active layers
  int nslot = 0, nactive = 0;
  std::vector<int> slot_col, slot_k;
  // adaptive_solver_diagnostics (grid-wide cut): last_min_dt and its cell
  // (1-based i, j, k, n), kept across calls; still_zero: the first Fortran
  // element of a cell the solver does not step that has a valid quotient
  // (c - c) / c = 0 (a nonzero finite value), from the last host state
  // (-1: none)
  double last_min_dt = (double)1e20f;
  int last_cell[4] = {-99, -99, -99, -99};
  long long still_zero = -1;
  DevBuf d_minloc;
  Bin bins[kBins];
  int nseg = 1;                 // column ranges of the layout
  std::vector<int> seg_col;     // [nseg + 1] column bounds
  int pipe = 1;                 // sed_ode_solver pipeline chunks
  // pipelined sed_ode_solver: copy-in, two step, copy-out streams
  cudaStream_t s_in = nullptr, s_out = nullptr, s_cmp[kMaxSeg] = {};
  cudaEvent_t pe_start = nullptr, pe_done = nullptr;
  cudaEvent_t pe_in[kMaxSeg] = {}, pe_cmp[kMaxSeg] = {}, pe_cnt[kMaxSeg] = {};
  // device buffers
  DevBuf d_bgc;  // [NBGC_DEV][nslot] derived per-slot rate parameters
  DevBuf d_bgc_base, d_rfac;  // its unscaled form; [ncol] rate factors
  DevBuf d_slot_col, d_kact, d_tile_k, d_conc, d_coef, d_cap, d_force, d_sflux,
      d_budget, d_nsub, d_queue, d_stats, d_flag, d_stage, d_bdys, d_fluxes,
      d_rhs, d_rhs_stage, d_grid, d_force64, d_xfeat, d_yhat, d_backup,
      d_col_slot, d_top, d_bcin, d_mindt;
  // surrogate step: heavy-column slot list, its counter, hidden activations
  DevBuf d_list, d_gate, d_act;
  DevBuf d_hist;  // [SED_HIST_BINS] attempts histogram
  std::vector<double> force64;  // host forcing rows (FP64 state)
  std::vector<double> rfac64;   // host rate factors (FP64 state)
  DevStats* h_stats = nullptr;  // pinned
  int* h_flag = nullptr;        // pinned
  unsigned long long* h_count = nullptr;  // pinned, kMaxSeg counters
  // graph of one coupling step
  cudaGraphExec_t graph = nullptr;
  double graph_dt = -1.0;
  int graph_method = -1;
  int graph_launches = 0;
  long long launches = 0;

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
  bool temp_rates() const { return prm.temp_activation > 0.0; }
  // the kernels read a per-slot parameter table
  bool table() const { return has_bgc || temp_rates(); }
  size_t rsize() const { return fp64() ? sizeof(double) : sizeof(float); }
  ~sed_handle();
};

#define CK(expr, what)                                      \
  do {                                                      \
    cudaError_t e_ = (expr);                                \
    if (e_ != cudaSuccess) return h->cuda_fail(e_, what);   \
  } while (0)

namespace {

int check_params(sed_handle* h, const sed_params& p) {
  if (p.bcup_dissolved < 1 || p.bcup_dissolved > 3)
    return h->fail(SED_E_ARG, "bcup_dissolved must be 1, 2 or 3 (got %d)", p.bcup_dissolved);
  if (p.bcup_particulate != 1 && p.bcup_particulate != 4)
    return h->fail(SED_E_ARG, "bcup_particulate must be 1 or 4 (got %d)", p.bcup_particulate);
  if (p.mol_diff_mode != 0 && p.mol_diff_mode != 1)
    return h->fail(SED_E_ARG, "mol_diff_mode must be 0 or 1");
  if (p.max_attempts <= 0) return h->fail(SED_E_ARG, "max_attempts must be > 0");
  if (!(p.atol >= 0.0)) return h->fail(SED_E_ARG, "atol must be >= 0");
  if (p.precision != SED_FP32 && p.precision != SED_FP64)
    return h->fail(SED_E_ARG, "precision must be SED_FP32 or SED_FP64");
  if (p.cut_scope != SED_CUT_PER_COLUMN && p.cut_scope != SED_CUT_GLOBAL)
    return h->fail(SED_E_ARG, "cut_scope must be per-column or global");
  if (p.bioturbation_profile == 3 &&
      !(p.bioturb_dry_density > 0.0 && p.bioturb_b > 0.0 && p.bioturb_L1 + p.bioturb_L2 > 0.0))
    return h->fail(SED_E_ARG, "bioturbation profile 3 needs dry density > 0, b > 0, L1+L2 > 0");
  if (!(p.temp_activation >= 0.0) || !std::isfinite(p.temp_activation))
    return h->fail(SED_E_ARG, "temp_activation must be >= 0 and finite");
  if (p.temp_activation > 0.0 && p.cut_scope == SED_CUT_GLOBAL)
    return h->fail(SED_E_ARG, "temperature-dependent rates need per-column cuts");
  return SED_OK;
}

void reset_graph(sed_handle* h) {
  if (h->graph) cudaGraphExecDestroy(h->graph);
  h->graph = nullptr;
  h->graph_dt = -1.0;
  h->graph_method = -1;
}

template <typename real>
ColumnArgs<real> column_args(sed_handle* h, const Bin& b, int bin_index,
                             double dt, int method) {
  ColumnArgs<real> a{};
  a.conc = h->d_conc.as<real>();
  a.out = h->d_rhs.as<real>();
  a.coef = h->d_coef.as<real>();
  a.cap = h->prm.bcup_particulate == 4 ? h->d_cap.as<real>() : nullptr;
  a.force = h->d_force.as<real>();
  a.kact = h->d_kact.as<int>();
  a.tile_k = h->d_tile_k.as<int>();
  a.sflux = h->d_sflux.as<real>();
  a.budget = h->prm.budgets ? h->d_budget.as<double>() : nullptr;
  a.nsub = h->d_nsub.as<int>();
  a.mindt = h->d_mindt.as<double>();
  a.queue = h->d_queue.as<unsigned>() + bin_index;
  a.stats = h->d_stats.as<DevStats>();
  a.nslot = h->nslot;
  a.kmax = h->kmax;
  a.tc = b.tc;
  a.slot0 = b.slot0;
  a.tile0 = b.tk0;
  a.ntiles = b.tc ? b.nslots / b.tc : b.nslots;
  a.dt = dt;
  a.method = method;
  a.bgc = h->table() ? h->d_bgc.as<real>() : nullptr;
  return a;
}

// restrict a class launch to its slots [s0, s1) (segment bounds)
template <typename real>
void restrict_args(ColumnArgs<real>& a, const Bin& b, int s0, int s1, unsigned* queue) {
  a.slot0 = s0;
  a.tile0 = b.tc ? b.tk0 + (s0 - b.slot0) / b.tc : 0;
  a.ntiles = b.tc ? (s1 - s0) / b.tc : s1 - s0;
  a.queue = queue;
}

// Launch one class's kernel over a's slot range.  Warp-direct classes (tc 0)
// step with k_column_warp; their other kinds (rhs, residual) use the tile
// kernel (the widest of 32/16/8 columns that fits) staging every layer.
template <typename real>
cudaError_t launch_bin(sed_handle* h, ColumnArgs<real> a, const Params<real>& p,
                       const Bin& bin, int kind, cudaStream_t st) {
  const bool bc4 = h->prm.bcup_particulate == 4;
  if (bin.tc == 0) {
    if (kind == KIND_ADAPT || kind == KIND_FIXED)
      return launch_column_warp<real>(a, p, bin.lpl, bc4, kind, bin.blocks(h->sms, a.ntiles),
                                      bin.threads, st);
    a.tc = bin.tc_fb;
    a.tile_k = nullptr;
    a.tile0 = 0;
    a.ntiles /= bin.tc_fb;
    const int blocks = std::max(1, std::min(a.ntiles, bin.occ_tile * h->sms));
    return launch_column<real>(a, p, bin.lpl, bc4, kind, blocks, bin.threads, st);
  }
  return launch_column<real>(a, p, bin.lpl, bc4, kind, bin.blocks(h->sms, a.ntiles),
                             bin.threads, st);
}

// Enqueue the tile kernels of every depth class (one coupling step, or one
// right-hand side for KIND_RHS).
template <typename real>
int enqueue_columns(sed_handle* h, double dt, int method, int kind) {
  Params<real> p = make_params<real>(h->prm);
  set_clock(p, dt, h->prm.dt_min);
  CK(cudaMemsetAsync(h->d_queue.p, 0, kBins * sizeof(unsigned), h->stream), "queue reset");
  for (int b = 0; b < kBins; b++) {
    const Bin& bin = h->bins[b];
    if (bin.nslots == 0) continue;
    ColumnArgs<real> a = column_args<real>(h, bin, b, dt, method);
    CK(launch_bin<real>(h, a, p, bin, kind, h->stream), "column kernel launch");
    h->launches++;
  }
  return SED_OK;
}

int stats_reset(sed_handle* h) {
  DevStats z{};
  z.min_dt_bits = 0x7FF0000000000000ull;  // +inf
  *h->h_stats = z;
  CK(cudaMemcpyAsync(h->d_stats.p, h->h_stats, sizeof(DevStats),
                     cudaMemcpyHostToDevice, h->stream), "stats reset");
  return SED_OK;
}

int stats_fetch(sed_handle* h, sed_stats* out, long long launches0,
                bool timed = false) {
  CK(cudaMemcpyAsync(h->h_stats, h->d_stats.p, sizeof(DevStats),
                     cudaMemcpyDeviceToHost, h->stream), "stats fetch");
  CK(cudaStreamSynchronize(h->stream), "step");
  const DevStats& s = *h->h_stats;
  float ms = 0.0f;
  if (timed) CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1), "event time");
  if (out) {
    out->device_ms = ms;
    out->surrogate_columns = (long long)s.surrogate;
    out->attempts = (long long)s.attempts;
    out->accepted = (long long)s.accepted;
    out->column_steps = (long long)s.column_steps;
    out->max_col_attempts = s.max_col_attempts;
    out->capped_columns = s.capped;
    out->nan_cells = s.nan_cells;
    out->gpu_launches = (int)(h->launches - launches0);
    double md;
    unsigned long long bits = s.min_dt_bits;
    memcpy(&md, &bits, sizeof md);
    out->min_dt = md;
  }
  if (s.status & ST_NAN)
    return h->fail(SED_E_NAN, "NaN in %d cells after the step", s.nan_cells);
  if (s.status & ST_CAP)
    return h->fail(SED_E_SUBSTEP_CAP, "%d column-steps hit max_attempts=%d", s.capped,
                   h->prm.max_attempts);
  return SED_OK;
}

// One coupling step of every column, per-column cut (graph replay).
template <typename real>
int step_percol(sed_handle* h, double dt, int method) {
  const int kind = method == SED_ADAPTIVE_EULER ? KIND_ADAPT : KIND_FIXED;
  if (!h->graph || h->graph_dt != dt || h->graph_method != method) {
    reset_graph(h);
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    const long long l0 = h->launches;
    int rc = enqueue_columns<real>(h, dt, method, kind);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc != SED_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return h->cuda_fail(e, "end capture");
    h->graph_launches = (int)(h->launches - l0);
    h->launches = l0;
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { h->graph = nullptr; return h->cuda_fail(e, "graph instantiate"); }
    h->graph_dt = dt;
    h->graph_method = method;
  }
  CK(cudaGraphLaunch(h->graph, h->stream), "graph launch");
  h->launches += h->graph_launches;
  return SED_OK;
}

// One coupling step with the reference's grid-wide cut: any() over every
// active cell of the grid decides the substep (solver_library.F90:121).
// adaptive_solver_diagnostics (solver_library.F90:129-136) at an accepted
// substep dt_red smaller than last_min_dt: the substep and the cell of the
// smallest relative change, as gfortran's MINLOC takes it over the whole
// grid -- first in element order, NaN skipped; cells the solver does not
// step have quotient 0 where their value is nonzero and finite; with no
// valid quotient at all, the first element.
template <typename real>
int record_min_dt(sed_handle* h, double dt_red) {
  CK(h->d_minloc.alloc(2 * sizeof(unsigned long long)), "diagnostics");
  CK(launch_minloc<real>(h->d_conc.as<real>(), h->d_rhs.as<real>(), h->d_kact.as<int>(),
                         h->d_slot_col.as<int>(), h->nslot, h->kmax, h->ncol, (real)dt_red,
                         h->d_minloc.as<unsigned long long>(), h->sms, h->stream),
     "diagnostics launch");
  h->launches += 2;
  unsigned long long r[2];
  CK(cudaMemcpyAsync(r, h->d_minloc.p, sizeof r, cudaMemcpyDeviceToHost, h->stream),
     "diagnostics copy");
  CK(cudaStreamSynchronize(h->stream), "diagnostics");
  const bool active = r[0] != ~0ull;
  double vmin = 0.0;
  if (active) {  // the key's double
    const unsigned long long b = (r[0] >> 63) ? (r[0] & 0x7FFFFFFFFFFFFFFFull) : ~r[0];
    memcpy(&vmin, &b, sizeof vmin);
  }
  const long long still = h->still_zero;
  long long pos;
  if (!active) pos = still >= 0 ? still : 0;
  else if (vmin < 0.0 || still < 0) pos = (long long)r[1];
  else if (vmin == 0.0) pos = std::min((long long)r[1], still);
  else pos = still;
  const long long nc = h->ncol, col = pos % nc, kn = pos / nc;
  h->last_min_dt = dt_red;
  h->last_cell[0] = (int)(col % h->inum) + 1;
  h->last_cell[1] = (int)(col / h->inum) + 1;
  h->last_cell[2] = (int)(kn % h->kmax) + 1;
  h->last_cell[3] = (int)(kn / h->kmax) + 1;
  return SED_OK;
}

template <typename real>
int step_global(sed_handle* h, double dt) {
  const Params<real> p = make_params<real>(h->prm);
  const size_t n = (size_t)NTR * h->kmax * h->nslot;
  CK(h->d_rhs.alloc(n * sizeof(real)), "rhs buffer");
  double dt_int = 0.0, dt_red = dt;
  bool need_rhs = true;
  long long att = 0, acc = 0;
  double min_dt = 1e300;
  bool capped = false;
  while (dt_int < dt) {
    if (att >= h->prm.max_attempts) {
      capped = true;
      break;
    }
    att++;
    if (need_rhs) {
      int rc = enqueue_columns<real>(h, dt, 0, KIND_RHS);
      if (rc) return rc;
      need_rhs = false;
    }
    CK(cudaMemsetAsync(h->d_flag.p, 0, sizeof(int), h->stream), "flag reset");
    CK(launch_trial<real>(h->d_conc.as<real>(), h->d_rhs.as<real>(), h->d_kact.as<int>(),
                          h->nslot, h->kmax, (real)dt_red, p.keep, p.natol,
                          h->d_flag.as<int>(), h->sms, h->stream), "trial launch");
    h->launches++;
    CK(cudaMemcpyAsync(h->h_flag, h->d_flag.p, sizeof(int), cudaMemcpyDeviceToHost,
                       h->stream), "flag fetch");
    CK(cudaStreamSynchronize(h->stream), "trial");
    if (*h->h_flag && dt_red > h->prm.dt_min) {
      dt_red = dt_red * 0.25;
    } else {
      if (h->prm.adaptive_solver_diagnostics && dt_red < h->last_min_dt) {
        int rc = record_min_dt<real>(h, dt_red);
        if (rc) return rc;
      }
      CK(launch_accept<real>(h->d_conc.as<real>(), h->d_rhs.as<real>(), h->d_kact.as<int>(),
                             h->nslot, h->kmax, (real)dt_red, h->sms, h->stream),
         "accept launch");
      h->launches++;
      dt_int = dt_int + dt_red;
      acc++;
      if (dt_red < min_dt) min_dt = dt_red;
      need_rhs = true;
    }
  }
  if (h->prm.epilogue) {
    CK(launch_epilogue<real>(h->d_conc.as<real>(), h->d_kact.as<int>(), h->nslot,
                             h->kmax, p, h->d_stats.as<DevStats>(), h->sms, h->stream),
       "epilogue launch");
    h->launches++;
  }
  // host-side counters merged into the device stats record
  DevStats tmp;
  CK(cudaMemcpyAsync(&tmp, h->d_stats.p, sizeof tmp, cudaMemcpyDeviceToHost, h->stream),
     "stats");
  CK(cudaStreamSynchronize(h->stream), "global step");
  tmp.attempts += (unsigned long long)(att * h->nactive);
  tmp.accepted += (unsigned long long)(acc * h->nactive);
  tmp.column_steps += (unsigned long long)h->nactive;
  tmp.max_col_attempts = std::max(tmp.max_col_attempts, (int)att);
  if (capped) { tmp.status |= ST_CAP; tmp.capped += h->nactive; }
  {
    // one dt sequence for the whole grid: every active column's smallest
    std::vector<double> md(h->nslot, 0.0);
    for (int i = 0; i < h->nslot; i++)
      if (h->slot_col[i] >= 0 && acc > 0) md[i] = min_dt;
    CK(cudaMemcpyAsync(h->d_mindt.p, md.data(), md.size() * sizeof(double),
                       cudaMemcpyHostToDevice, h->stream), "smallest substeps");
    CK(cudaStreamSynchronize(h->stream), "global step");
  }
  unsigned long long bits;
  memcpy(&bits, &min_dt, sizeof bits);
  if (acc > 0 && bits < tmp.min_dt_bits) tmp.min_dt_bits = bits;
  CK(cudaMemcpyAsync(h->d_stats.p, &tmp, sizeof tmp, cudaMemcpyHostToDevice, h->stream),
     "stats");
  CK(cudaStreamSynchronize(h->stream), "global step");
  return SED_OK;
}

template <typename real>
int step_any(sed_handle* h, double dt, int method) {
  if (method == SED_ADAPTIVE_EULER && h->prm.cut_scope == SED_CUT_GLOBAL) {
    if (h->table())
      return h->fail(SED_E_STATE,
                     "per-column parameter sets and temperature-dependent rates need "
                     "per-column cuts");
    return step_global<real>(h, dt);
  }
  return step_percol<real>(h, dt, method);
}

int dispatch_step(sed_handle* h, double dt, int method) {
  return h->fp64() ? step_any<double>(h, dt, method) : step_any<float>(h, dt, method);
}

template <typename real>
int gather_state(sed_handle* h) {
  CK(launch_gather<real>(h->d_stage.as<double>(), h->d_conc.as<real>(),
                         h->d_slot_col.as<int>(), NTR, h->kmax, h->ncol, h->nslot,
                         h->sms, h->stream), "gather launch");
  h->launches++;
  return SED_OK;
}

template <typename real>
int scatter_state(sed_handle* h, const real* src, double* dst) {
  CK(launch_scatter<real>(src, dst, h->d_slot_col.as<int>(),
                          h->d_kact.as<int>(), NTR, h->kmax, h->ncol, h->nslot,
                          h->sms, h->stream), "scatter launch");
  h->launches++;
  return SED_OK;
}

template <typename real>
int scatter_fluxes(sed_handle* h) {
  CK(launch_scatter_flux<real>(h->d_sflux.as<real>(), h->d_fluxes.as<double>(),
                               h->d_slot_col.as<int>(), h->d_kact.as<int>(), h->ncol,
                               h->nslot, h->sms, h->stream), "flux scatter launch");
  h->launches++;
  return SED_OK;
}

// Temperature-dependent rates: the per-slot table from its base, the
// microbial rate constants scaled by the column's factor (the host's, in
// d_rfac, when rfac_host; else formed on the device from bdys[0]).
template <typename real>
int rate_table(sed_handle* h) {
  CK(launch_rate_temperature<real>(h->d_bgc_base.as<real>(), h->d_bgc.as<real>(),
                                   h->d_slot_col.as<int>(), h->d_bdys.as<double>(),
                                   h->rfac_host ? h->d_rfac.as<double>() : nullptr,
                                   h->prm.temp_activation, h->nslot, h->sms, h->stream),
     "rate factor launch");
  h->launches++;
  return SED_OK;
}

template <typename real>
int prep_force(sed_handle* h) {
  CK(launch_prep_force<real>(h->d_bdys.as<double>(), h->d_fluxes.as<double>(),
                             h->d_slot_col.as<int>(), h->d_force.as<real>(), h->ncol,
                             h->nslot, h->prm.bioturbation, h->prm.diffusivity,
                             h->prm.mol_diff_mode, h->prm.bcup_dissolved,
                             h->prm.bioturbation_profile == 3 ? 1 : 0, h->sms, h->stream),
     "forcing launch");
  h->launches++;
  h->rfac_host = false;
  return h->temp_rates() ? rate_table<real>(h) : SED_OK;
}

// FP64 state: the per-column forcing rows are formed on the host with the
// host's exp, exactly as get_rhs forms them (:648, :652, :682), then
// gathered into slot order, so FP64 device results match the CPU
// restatement bit for bit.
int prep_force_host64(sed_handle* h, const double* bdys, const double* fluxes) {
  const int ncol = h->ncol;
  h->force64.assign((size_t)NFORCE * ncol, 0.0);
  double* f = h->force64.data();
  for (int c = 0; c < ncol; c++) {
    const double T = bdys[c];
    const double f_T = 1.0 * std::exp(-4500.0 * (1.0 / (T + 273.0) - (1.0 / 288.0)));
    // profile 3: bioturbation = f_T = 1 (get_rhs :622-623)
    f[c] = h->prm.bioturbation_profile == 3 ? 1.0 : h->prm.bioturbation * f_T;
    f[(size_t)ncol + c] = h->prm.mol_diff_mode == 1 ? 1.0 : (h->prm.diffusivity + T * 0.035);
    for (int n = 0; n < NTR; n++) {
      const double fl = fluxes[(size_t)n * ncol + c];
      const double cb = bdys[(size_t)(n + 1) * ncol + c];
      f[(size_t)(2 + n) * ncol + c] =
          n < NPART ? fl : (h->prm.bcup_dissolved == 1 ? fl : cb);
    }
  }
  CK(h->d_force64.alloc(h->force64.size() * sizeof(double)), "forcing staging");
  CK(cudaMemcpyAsync(h->d_force64.p, f, h->force64.size() * sizeof(double),
                     cudaMemcpyHostToDevice, h->stream), "forcing copy");
  CK(launch_gather<double>(h->d_force64.as<double>(), h->d_force.as<double>(),
                           h->d_slot_col.as<int>(), NFORCE, 1, ncol, h->nslot, h->sms,
                           h->stream), "forcing gather");
  h->launches++;
  h->rfac_host = false;
  if (!h->temp_rates()) return SED_OK;
  // the rate factors with the host's exp, as the CPU restatement forms them
  std::vector<double>& fr = h->rfac64;
  fr.resize(ncol);
  for (int c = 0; c < ncol; c++) fr[c] = rate_factor(h->prm.temp_activation, bdys[c]);
  CK(h->d_rfac.alloc((size_t)ncol * sizeof(double)), "rate factors");
  CK(cudaMemcpyAsync(h->d_rfac.p, fr.data(), (size_t)ncol * sizeof(double),
                     cudaMemcpyHostToDevice, h->stream), "rate factors copy");
  h->rfac_host = true;
  return rate_table<double>(h);
}

int upload_forcing(sed_handle* h, const double* bdys, const double* fluxes) {
  const size_t nb = (size_t)(NTR + 1) * h->ncol * sizeof(double);
  const size_t nf = (size_t)NTR * h->ncol * sizeof(double);
  CK(cudaMemcpyAsync(h->d_bdys.p, bdys, nb, cudaMemcpyHostToDevice, h->stream), "bdys copy");
  CK(cudaMemcpyAsync(h->d_fluxes.p, fluxes, nf, cudaMemcpyHostToDevice, h->stream), "fluxes copy");
  int rc = h->fp64() ? prep_force_host64(h, bdys, fluxes) : prep_force<float>(h);
  if (rc) return rc;
  h->have_forcing = true;
  return SED_OK;
}

// The first Fortran element (n, k, col order) of a cell the solver does not
// step -- a land column or a masked tail -- with a nonzero finite value.
long long first_still_cell(const sed_handle* h, const double* conc) {
  const int nc = h->ncol, km = h->kmax;
  std::vector<int> kcol(nc, 0);
  for (int s = 0; s < h->nslot; s++)
    if (h->slot_col[s] >= 0) kcol[h->slot_col[s]] = h->slot_k[s];
  std::vector<int> still;
  for (int c = 0; c < nc; c++)
    if (kcol[c] < km) still.push_back(c);
  if (still.empty()) return -1;
  for (int n = 0; n < NTR; n++)
    for (int k = 0; k < km; k++)
      for (int c : still) {
        if (k < kcol[c]) continue;
        const double v = conc[((size_t)n * km + k) * nc + c];
        if (v != 0.0 && std::isfinite(v)) return (long long)c + (long long)nc * (k + (long long)km * n);
      }
  return -1;
}

int upload_state(sed_handle* h, const double* conc) {
  if (h->prm.adaptive_solver_diagnostics) h->still_zero = first_still_cell(h, conc);
  const size_t bytes = (size_t)NTR * h->kmax * h->ncol * sizeof(double);
  CK(cudaMemcpyAsync(h->d_stage.p, conc, bytes, cudaMemcpyHostToDevice, h->stream), "conc copy");
  int rc = h->fp64() ? gather_state<double>(h) : gather_state<float>(h);
  if (rc) return rc;
  h->have_state = true;
  return SED_OK;
}

int download_state(sed_handle* h, double* conc) {
  const size_t bytes = (size_t)NTR * h->kmax * h->ncol * sizeof(double);
  int rc = h->fp64() ? scatter_state<double>(h, h->d_conc.as<double>(), h->d_stage.as<double>())
                     : scatter_state<float>(h, h->d_conc.as<float>(), h->d_stage.as<double>());
  if (rc) return rc;
  CK(cudaMemcpyAsync(conc, h->d_stage.p, bytes, cudaMemcpyDeviceToHost, h->stream), "conc copy back");
  return SED_OK;
}

// Blocks per SM of a class's tile at its (tc, threads) for every kernel
// kind the handle launches; 0 when the tile does not fit.
int class_occupancy(sed_handle* h, const Bin& b, int tc, int threads) {
  const bool bc4 = h->prm.bcup_particulate == 4;
  int occ = 1 << 30;
  for (int kd : {KIND_ADAPT, KIND_FIXED, KIND_RHS}) {
    const bool bio3 = h->prm.bioturbation_profile == 3;
    const int o = h->fp64() ? column_blocks_per_sm<double>(tc, b.lpl, bc4, kd, threads, bio3)
                            : column_blocks_per_sm<float>(tc, b.lpl, bc4, kd, threads, bio3);
    occ = std::min(occ, o);
  }
  return occ;
}

// Occupancy and per-tile layer counts of the current tuning; raises the
// kernels' shared-memory limit before any capture and drops the step graph.
// The per-slot table of derived rate parameters: each column's sed_params
// set (its own with sed_set_column_bgc, else the handle's) through
// make_params, so a column with the handle's own set gets the bits of the
// uniform path.  With temperature-dependent rates this is the unscaled
// base, scaled by rate_table once the forcing is known.
template <typename real>
int upload_bgc(sed_handle* h) {
  const int ns = h->nslot, nc = h->ncol;
  std::vector<real> tab((size_t)NBGC_DEV * ns);
  Params<real> base = make_params<real>(h->prm);
  for (int s = 0; s < ns; s++) {
    const int c = h->slot_col[s];
    Params<real> q = base;
    if (c >= 0 && h->has_bgc) {
      sed_params sp = h->prm;
      double* f[SED_NBGC] = {&sp.rLabile, &sp.rSemilabile, &sp.NCrLdet, &sp.NCrSdet,
                             &sp.PAds, &sp.PAdsODU, &sp.NH3Ads, &sp.CprodMax, &sp.rnit,
                             &sp.ksO2nitri, &sp.rODUox, &sp.ksO2oduox, &sp.ksO2oxic,
                             &sp.ksNO3denit, &sp.kinO2denit, &sp.kinNO3anox, &sp.kinO2anox};
      for (int i = 0; i < SED_NBGC; i++) *f[i] = h->bgc_cols[(size_t)i * nc + c];
      q = make_params<real>(sp);
    }
    for (int i = 0; i < NBGC_DEV; i++) tab[(size_t)i * ns + s] = *bgc_field(q, i);
  }
  DevBuf& dst = h->temp_rates() ? h->d_bgc_base : h->d_bgc;
  CK(h->d_bgc.alloc(tab.size() * sizeof(real)), "parameter sets");
  CK(dst.alloc(tab.size() * sizeof(real)), "parameter sets");
  CK(cudaMemcpyAsync(dst.p, tab.data(), tab.size() * sizeof(real), cudaMemcpyHostToDevice,
                     h->stream),
     "parameter sets copy");
  CK(cudaStreamSynchronize(h->stream), "parameter sets copy");
  if (h->temp_rates() && h->have_forcing) return rate_table<real>(h);
  return SED_OK;
}

int apply_tuning(sed_handle* h) {
  std::vector<int> tile_k;
  for (int b = 0; b < kBins; b++) {
    Bin& bin = h->bins[b];
    bin.tk0 = (int)tile_k.size();
    bin.occ = 0;
    if (bin.nslots == 0) continue;
    if (bin.tc == 0) {
      const bool bc4 = h->prm.bcup_particulate == 4, bio3 = h->prm.bioturbation_profile == 3;
      auto occ = [&](int kind) {
        return h->fp64() ? column_warp_blocks_per_sm<double>(bin.lpl, bc4, kind, bin.threads, bio3)
                         : column_warp_blocks_per_sm<float>(bin.lpl, bc4, kind, bin.threads, bio3);
      };
      bin.occ = std::min(occ(KIND_ADAPT), occ(KIND_FIXED));
      bin.occ_tile = 0;
      for (bin.tc_fb = 32; bin.tc_fb >= 8; bin.tc_fb /= 2)
        if ((bin.occ_tile = class_occupancy(h, bin, bin.tc_fb, bin.threads)) > 0) break;
      if (bin.occ <= 0 || bin.occ_tile <= 0)
        return h->fail(SED_E_CUDA, "warp-direct kernel of %d threads does not fit", bin.threads);
      continue;
    }
    bin.occ = class_occupancy(h, bin, bin.tc, bin.threads);
    if (bin.occ <= 0)
      return h->fail(SED_E_CUDA, "tile of %d columns x %d layers does not fit on the device",
                     bin.tc, 32 * bin.lpl);
    for (int t = 0; t < bin.nslots / bin.tc; t++) {
      int m = 1;
      for (int j = 0; j < bin.tc; j++) m = std::max(m, h->slot_k[bin.slot0 + t * bin.tc + j]);
      tile_k.push_back(m);
    }
  }
  if (tile_k.empty()) tile_k.push_back(1);
  CK(h->d_tile_k.alloc(tile_k.size() * sizeof(int)), "tile_k");
  CK(cudaMemcpyAsync(h->d_tile_k.p, tile_k.data(), tile_k.size() * sizeof(int),
                     cudaMemcpyHostToDevice, h->stream), "tile_k copy");
  CK(cudaStreamSynchronize(h->stream), "tile_k copy");
  reset_graph(h);
  return SED_OK;
}

int ready(sed_handle* h) {
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  if (!h->have_forcing) return h->fail(SED_E_STATE, "sed_set_forcing has not been called");
  return SED_OK;
}

int ensure_pipeline(sed_handle* h) {
  if (h->s_in) return SED_OK;
  CK(cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking), "stream");
  CK(cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking), "stream");
  // chunk c's step stream has a higher priority than chunk c+1's (as far
  // as the device's priority range goes): the block scheduler then finishes
  // the chunks in order, so each chunk's copy back overlaps the steps of
  // the later ones, which fill only the SMs the earlier chunks leave free
  int least = 0, greatest = 0;
  CK(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
  for (int c = 0; c < kMaxSeg; c++)
    CK(cudaStreamCreateWithPriority(&h->s_cmp[c], cudaStreamNonBlocking,
                                    std::min(least, greatest + c)),
       "stream");
  CK(cudaEventCreateWithFlags(&h->pe_start, cudaEventDisableTiming), "event");
  CK(cudaEventCreateWithFlags(&h->pe_done, cudaEventDisableTiming), "event");
  for (int c = 0; c < kMaxSeg; c++) {
    CK(cudaEventCreateWithFlags(&h->pe_in[c], cudaEventDisableTiming), "event");
    CK(cudaEventCreateWithFlags(&h->pe_cmp[c], cudaEventDisableTiming), "event");
    CK(cudaEventCreateWithFlags(&h->pe_cnt[c], cudaEventDisableTiming), "event");
  }
  return SED_OK;
}

// sed_ode_solver with the copies in flight: the columns are cut into
// h->pipe chunks of whole segments.  Chunk c's host->device copy (one 2-D
// copy of its column range in every [tracer][layer] row), its gather, step
// and scatter (on its own step stream, so the steps of several chunks
// overlap and a chunk's tail of slow columns shares the GPU with the next
// chunk's step), and its
// device->host copy are ordered by events, so chunk c+1 arrives while c is
// stepped and c-1 leaves.  Each chunk writes a disjoint column range of the
// staging array and of conc, and its own slots.
template <typename real>
int ode_solver_pipelined(sed_handle* h, double* conc, double dt, int method) {
  int rc = ensure_pipeline(h);
  if (rc) return rc;
  Params<real> p = make_params<real>(h->prm);
  set_clock(p, dt, h->prm.dt_min);
  const int kind = method == SED_ADAPTIVE_EULER ? KIND_ADAPT : KIND_FIXED;
  const size_t pitch = (size_t)h->ncol * sizeof(double);
  const size_t rows = (size_t)NTR * h->kmax;
  double* stage = h->d_stage.as<double>();
  unsigned* q = h->d_queue.as<unsigned>();
  CK(cudaMemsetAsync(q, 0, kQueues * sizeof(unsigned), h->stream), "queue reset");
  const int per = h->nseg / h->pipe;
  CK(cudaEventRecord(h->pe_start, h->stream), "event");
  CK(cudaStreamWaitEvent(h->s_in, h->pe_start, 0), "wait");
  for (int c = 0; c < h->pipe; c++) {
    const int g0 = c * per, g1 = g0 + per;
    const int col0 = h->seg_col[g0], col1 = h->seg_col[g1];
    const size_t width = (size_t)(col1 - col0) * sizeof(double);
    if (width)
      CK(cudaMemcpy2DAsync(stage + col0, pitch, conc + col0, pitch, width, rows,
                           cudaMemcpyHostToDevice, h->s_in), "conc chunk copy");
    CK(cudaEventRecord(h->pe_in[c], h->s_in), "event");
    cudaStream_t cs = h->s_cmp[c];
    CK(cudaStreamWaitEvent(cs, h->pe_in[c], 0), "wait");
    for (int b = 0; b < kBins; b++) {
      const Bin& bin = h->bins[b];
      const int sl0 = bin.segb[g0], sl1 = bin.segb[g1];
      if (sl1 == sl0) continue;
      CK(launch_gather_range<real>(stage, h->d_conc.as<real>(), h->d_slot_col.as<int>(), NTR,
                                   h->kmax, h->ncol, h->nslot, sl0, sl1 - sl0, h->sms, cs),
         "gather launch");
      ColumnArgs<real> a = column_args<real>(h, bin, b, dt, method);
      restrict_args(a, bin, sl0, sl1, q + kBins + kBins * c + b);
      CK(launch_bin<real>(h, a, p, bin, kind, cs), "column kernel launch");
      CK(launch_scatter_range<real>(h->d_conc.as<real>(), stage, h->d_slot_col.as<int>(),
                                    h->d_kact.as<int>(), NTR, h->kmax, h->ncol, h->nslot,
                                    sl0, sl1 - sl0, h->sms, cs), "scatter launch");
      h->launches += 3;
    }
    CK(cudaEventRecord(h->pe_cmp[c], cs), "event");
    CK(cudaStreamWaitEvent(h->s_out, h->pe_cmp[c], 0), "wait");
    if (width)
      CK(cudaMemcpy2DAsync(conc + col0, pitch, stage + col0, pitch, width, rows,
                           cudaMemcpyDeviceToHost, h->s_out), "conc chunk copy back");
  }
  // s_out has waited for every chunk's step: the surface fluxes are final
  CK(launch_scatter_flux<real>(h->d_sflux.as<real>(), h->d_fluxes.as<double>(),
                               h->d_slot_col.as<int>(), h->d_kact.as<int>(), h->ncol,
                               h->nslot, h->sms, h->s_out), "flux scatter launch");
  h->launches++;
  CK(cudaEventRecord(h->pe_done, h->s_out), "event");
  CK(cudaStreamWaitEvent(h->stream, h->pe_done, 0), "wait");
  return SED_OK;
}

// The drop-in step on host arrays (sed_ode_solver without the statistics).
int ode_solver_impl(sed_handle* h, double* conc, const double* bdys, double* fluxes,
                    double dt, int method) {
  int rc;
  if ((rc = upload_forcing(h, bdys, fluxes))) return rc;
  const bool pipelined = h->pipe > 1 && !(method == SED_ADAPTIVE_EULER &&
                                          h->prm.cut_scope == SED_CUT_GLOBAL);
  if (pipelined) {
    rc = h->fp64() ? ode_solver_pipelined<double>(h, conc, dt, method)
                   : ode_solver_pipelined<float>(h, conc, dt, method);
    if (rc) return rc;
    h->have_state = true;
  } else {
    if ((rc = upload_state(h, conc))) return rc;
    if ((rc = dispatch_step(h, dt, method))) return rc;
    if ((rc = download_state(h, conc))) return rc;
    rc = h->fp64() ? scatter_fluxes<double>(h) : scatter_fluxes<float>(h);
    if (rc) return rc;
  }
  CK(cudaMemcpyAsync(fluxes, h->d_fluxes.p, (size_t)NTR * h->ncol * sizeof(double),
                     cudaMemcpyDeviceToHost, h->stream), "fluxes copy back");
  return SED_OK;
}

// ---------------------------------------------------------------------------
// autotuner

// device buffers a trial step changes, saved once and put back before every
// trial and at the end
struct Saved {
  DevBuf* buf;
  size_t bytes;
};

std::vector<Saved> trial_buffers(sed_handle* h) {
  const size_t ns = h->nslot, rs = h->rsize();
  std::vector<Saved> v = {{&h->d_conc, (size_t)NTR * h->kmax * ns * rs},
                          {&h->d_sflux, (size_t)NDISS * ns * rs},
                          {&h->d_nsub, ns * sizeof(int)},
                          {&h->d_force, (size_t)NFORCE * ns * rs},
                          {&h->d_fluxes, (size_t)NTR * h->ncol * sizeof(double)},
                          {&h->d_bdys, (size_t)(NTR + 1) * h->ncol * sizeof(double)}};
  if (h->prm.budgets) v.push_back({&h->d_budget, 4 * ns * sizeof(double)});
  return v;
}

int save_state(sed_handle* h, bool restore) {
  size_t off = 0, total = 0;
  auto bufs = trial_buffers(h);
  for (auto& b : bufs) total += (b.bytes + 255) & ~(size_t)255;
  if (!restore) CK(h->d_backup.alloc(total), "autotune backup");
  for (auto& b : bufs) {
    char* bk = h->d_backup.as<char>() + off;
    CK(cudaMemcpyAsync(restore ? b.buf->p : bk, restore ? bk : b.buf->p, b.bytes,
                       cudaMemcpyDeviceToDevice, h->stream), "autotune backup copy");
    off += (b.bytes + 255) & ~(size_t)255;
  }
  return SED_OK;
}

// time of one class's step kernel (b >= 0) or of a whole coupling step
// (b < 0), from the saved state, best of `reps`
template <typename real>
int time_step(sed_handle* h, int b, double dt, int method, int reps, float* best) {
  *best = 1e30f;
  const int kind = method == SED_ADAPTIVE_EULER ? KIND_ADAPT : KIND_FIXED;
  Params<real> p = make_params<real>(h->prm);
  set_clock(p, dt, h->prm.dt_min);
  for (int r = 0; r <= reps; r++) {  // r = 0 warms up
    int rc = save_state(h, true);
    if (rc) return rc;
    CK(cudaEventRecord(h->ev0, h->stream), "event");
    if (b >= 0) {
      const Bin& bin = h->bins[b];
      CK(cudaMemsetAsync(h->d_queue.p, 0, kBins * sizeof(unsigned), h->stream), "queue reset");
      ColumnArgs<real> a = column_args<real>(h, bin, b, dt, method);
      CK(launch_bin<real>(h, a, p, bin, kind, h->stream), "autotune launch");
    } else {
      rc = step_any<real>(h, dt, method);
      if (rc) return rc;
    }
    CK(cudaEventRecord(h->ev1, h->stream), "event");
    CK(cudaEventSynchronize(h->ev1), "autotune step");
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1), "event time");
    if (r > 0) *best = std::min(*best, ms);
  }
  return SED_OK;
}

template <typename real>
int autotune_t(sed_handle* h, double dt, int method, int flags, sed_tuning* out) {
  int rc = save_state(h, false);
  if (rc) return rc;
  int trials = 0;
  const int tcs[] = {0, 8, 16, 32, 64};
  const int thr[] = {64, 128, 256};
  for (int b = 0; b < kTunedBins; b++) {
    Bin& bin = h->bins[b];
    if (bin.nslots == 0) continue;
    int best_tc = bin.tc, best_thr = bin.threads;
    float best_ms = 1e30f;
    for (int tc : tcs)
      for (int th : thr) {
        if (tc > 0 && h->table()) continue;  // per-slot tables step warp-direct only
        if (tc > 0) {
          const int occ = class_occupancy(h, bin, tc, th);
          if (occ <= 0 || bin.nslots < tc) continue;
        }
        bin.tc = tc;
        bin.threads = th;
        bin.bps = 0;
        if ((rc = apply_tuning(h))) return rc;
        float ms;
        if ((rc = time_step<real>(h, b, dt, method, 2, &ms))) return rc;
        trials++;
        if (ms < best_ms) { best_ms = ms; best_tc = tc; best_thr = th; }
      }
    bin.tc = best_tc;
    bin.threads = best_thr;
    if ((rc = apply_tuning(h))) return rc;
  }
  float step_ms;
  if ((rc = time_step<real>(h, -1, dt, method, 2, &step_ms))) return rc;
  if (flags & SED_TUNE_CAP) {
    // attempts of the last timed step (the stats record of the trials)
    DevStats z{};
    z.min_dt_bits = 0x7FF0000000000000ull;
    CK(cudaMemcpyAsync(h->d_stats.p, &z, sizeof z, cudaMemcpyHostToDevice, h->stream), "stats");
    if ((rc = save_state(h, true))) return rc;
    if ((rc = step_any<real>(h, dt, method))) return rc;
    DevStats s;
    CK(cudaMemcpyAsync(&s, h->d_stats.p, sizeof s, cudaMemcpyDeviceToHost, h->stream), "stats");
    CK(cudaStreamSynchronize(h->stream), "autotune cap");
    int cap = 64;
    while (cap < 4 * s.max_col_attempts && cap < (1 << 30)) cap *= 2;
    h->prm.max_attempts = cap;
    reset_graph(h);
  }
  float ode_ms = 0.0f;
  const size_t state_bytes = (size_t)NTR * h->kmax * h->ncol * sizeof(double);
  if ((flags & SED_TUNE_PIPELINE) && state_bytes <= ((size_t)2 << 30)) {
    // pinned host copies of the state and forcing the caller would pass
    double *hc = nullptr, *hb = nullptr, *hf = nullptr;
    const size_t nb = (size_t)(NTR + 1) * h->ncol * sizeof(double);
    const size_t nf = (size_t)NTR * h->ncol * sizeof(double);
    if (cudaHostAlloc((void**)&hc, state_bytes, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc((void**)&hb, nb, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc((void**)&hf, nf, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      if (hc) cudaFreeHost(hc);
      if (hb) cudaFreeHost(hb);
      return h->fail(SED_E_NOMEM, "autotune: pinned host scratch of %zu bytes", state_bytes);
    }
    auto done = [&](int r) { cudaFreeHost(hc); cudaFreeHost(hb); cudaFreeHost(hf); return r; };
    int best_pipe = h->pipe;
    float best = 1e30f;
    for (int pp = 1; pp <= h->nseg; pp *= 2) {
      h->pipe = pp;
      // median of five timed calls after one warm-up: the host link's
      // throughput varies from call to call
      std::vector<float> tms;
      for (int r = 0; r <= 5; r++) {
        if ((rc = save_state(h, true))) return done(rc);
        if ((rc = download_state(h, hc))) return done(rc);
        if (cudaMemcpyAsync(hb, h->d_bdys.p, nb, cudaMemcpyDeviceToHost, h->stream) ||
            cudaMemcpyAsync(hf, h->d_fluxes.p, nf, cudaMemcpyDeviceToHost, h->stream) ||
            cudaStreamSynchronize(h->stream))
          return done(h->cuda_fail(cudaGetLastError(), "autotune scratch copy"));
        if (cudaEventRecord(h->ev0, h->stream)) return done(h->cuda_fail(cudaGetLastError(), "event"));
        if ((rc = ode_solver_impl(h, hc, hb, hf, dt, method))) return done(rc);
        float ms = 0.0f;
        if (cudaEventRecord(h->ev1, h->stream) || cudaEventSynchronize(h->ev1) ||
            cudaEventElapsedTime(&ms, h->ev0, h->ev1))
          return done(h->cuda_fail(cudaGetLastError(), "autotune pipeline"));
        trials++;
        if (r > 0) tms.push_back(ms);
      }
      std::sort(tms.begin(), tms.end());
      const float t_med = tms[tms.size() / 2];
      if (t_med < best) { best = t_med; best_pipe = pp; }
    }
    h->pipe = best_pipe;
    ode_ms = best;
    done(0);
  }
  if ((rc = save_state(h, true))) return rc;
  CK(cudaStreamSynchronize(h->stream), "autotune restore");
  reset_graph(h);
  if (out) {
    sed_get_tuning(h, out);
    out->step_ms = step_ms;
    out->ode_solver_ms = ode_ms;
    out->trials = trials;
  }
  return SED_OK;
}

}  // namespace

sed_handle::~sed_handle() {
  cudaSetDevice(device);
  if (stream) cudaStreamSynchronize(stream);
  reset_graph(this);
  for (cudaStream_t st : {s_in, s_out})
    if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
  for (cudaStream_t st : s_cmp)
    if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
  for (cudaEvent_t ev : {pe_start, pe_done}) if (ev) cudaEventDestroy(ev);
  for (int c = 0; c < kMaxSeg; c++) {
    if (pe_in[c]) cudaEventDestroy(pe_in[c]);
    if (pe_cmp[c]) cudaEventDestroy(pe_cmp[c]);
    if (pe_cnt[c]) cudaEventDestroy(pe_cnt[c]);
  }
  if (h_stats) cudaFreeHost(h_stats);
  if (h_flag) cudaFreeHost(h_flag);
  if (h_count) cudaFreeHost(h_count);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (own_stream) cudaStreamDestroy(own_stream);
}

// ===========================================================================
extern "C" {

int sed_default_params(sed_params* p) {
  if (!p) return SED_E_ARG;
  memset(p, 0, sizeof *p);
  p->diffusivity = 0.9;
  p->bioturbation = 0.9;
  p->bcup_dissolved = 2;
  p->bcup_particulate = 1;
  p->mol_diff_mode = 0;
  p->mol_diff_d0 = 1.0e-9;
  p->dt_min = 1.0e-9;
  p->relative_change_min = -0.9;
  p->max_attempts = 8192;
  p->cut_scope = SED_CUT_PER_COLUMN;
  p->rLabile = 0.043;
  p->rSemilabile = 0.001;
  p->NCrLdet = 0.22;
  p->NCrSdet = 0.005;
  p->PAds = 0.01;
  p->PAdsODU = 70.0;
  p->NH3Ads = 0.0;
  p->CprodMax = 9600.0;
  p->rnit = 200.0;
  p->ksO2nitri = 20.0;
  p->rODUox = 20.0;
  p->ksO2oduox = 1.0;
  p->ksO2oxic = 3.0;
  p->ksNO3denit = 1.0;
  p->kinO2denit = 70.0;
  p->kinNO3anox = 1.0;
  p->kinO2anox = 1.0;
  p->epilogue = 1;
  p->precision = SED_FP32;
  p->budgets = 0;
  p->device = 0;
  p->bioturbation_profile = 1;
  p->bioturb_k_l = 0.11;
  p->bioturb_L1 = 0.2;
  p->bioturb_L2 = 0.6;
  p->bioturb_beta = 0.22;
  p->bioturb_b = 1.334;
  p->bioturb_dry_density = 1000.0;
  p->temp_activation = 0.0;
  p->adaptive_solver_diagnostics = 0;
  return SED_OK;
}

int sed_create(const sed_params* p, int inum, int jnum, int kmax, int ntr,
               sed_handle** out) {
  if (!p || !out) return SED_E_ARG;
  *out = nullptr;
  if (ntr != SED_NTR || inum <= 0 || jnum <= 0 || kmax < 1 || kmax > SED_KMAX_LIMIT)
    return SED_E_ARG;
  if ((long long)inum * jnum > (1LL << 30)) return SED_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return SED_E_NODEVICE;
  }
  if (p->device < 0 || p->device >= ndev) return SED_E_ARG;
  std::unique_ptr<sed_handle> h(new sed_handle());
  h->prm = *p;
  int rc = check_params(h.get(), *p);
  if (rc) return rc;
  h->inum = inum;
  h->jnum = jnum;
  h->ncol = inum * jnum;
  h->kmax = kmax;
  h->device = p->device;
  sed_handle* hh = h.get();
  {
    sed_handle* h = hh;
    CK(cudaSetDevice(h->device), "set device");
    CK(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device), "SM count");
    CK(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking), "stream");
    h->stream = h->own_stream;
    CK(cudaEventCreate(&h->ev0), "event");
    CK(cudaEventCreate(&h->ev1), "event");
    CK(cudaHostAlloc((void**)&h->h_stats, sizeof(DevStats), cudaHostAllocDefault), "pinned stats");
    CK(cudaHostAlloc((void**)&h->h_flag, sizeof(int), cudaHostAllocDefault), "pinned flag");
    CK(cudaHostAlloc((void**)&h->h_count, kMaxSeg * sizeof(unsigned long long),
                     cudaHostAllocDefault),
       "pinned counter");
    CK(h->d_queue.alloc(kQueues * sizeof(unsigned)), "queue");
    CK(h->d_stats.alloc(sizeof(DevStats)), "stats");
    CK(h->d_flag.alloc(sizeof(int)), "flag");
    const size_t ncol = (size_t)h->ncol;
    CK(h->d_stage.alloc((size_t)NTR * kmax * ncol * sizeof(double)), "state staging");
    CK(h->d_bdys.alloc((size_t)(NTR + 1) * ncol * sizeof(double)), "bdys");
    CK(h->d_fluxes.alloc((size_t)NTR * ncol * sizeof(double)), "fluxes");
    // tracers a boundary assembly does not set keep these values
    CK(cudaMemset(h->d_bdys.p, 0, (size_t)(NTR + 1) * ncol * sizeof(double)), "bdys clear");
    CK(cudaMemset(h->d_fluxes.p, 0, (size_t)NTR * ncol * sizeof(double)), "fluxes clear");
  }
  *out = h.release();
  return SED_OK;
}

int sed_set_grid(sed_handle* h, const double* dz, const double* dzc,
                 const double* phi, const double* phi_i, const double* biofac,
                 const double* flux_cap, const int* kact, const int* mask) {
  if (!h) return SED_E_ARG;
  if (!dz || !phi || !phi_i || !biofac || (h->kmax > 1 && !dzc))
    return h->fail(SED_E_ARG, "sed_set_grid: dz, dzc, phi, phi_i and biofac are required");
  if (h->prm.bcup_particulate == 4 && !flux_cap)
    return h->fail(SED_E_ARG, "sed_set_grid: flux_cap is required for bcup_particulate 4");
  CK(cudaSetDevice(h->device), "set device");
  const int ncol = h->ncol, kmax = h->kmax;
  // active layers per column
  std::vector<int> ka(ncol, kmax);
  if (kact) {
    for (int c = 0; c < ncol; c++) {
      if (kact[c] < 0 || kact[c] > kmax)
        return h->fail(SED_E_ARG, "kact[%d]=%d outside 0..%d", c, kact[c], kmax);
      ka[c] = kact[c];
    }
  } else if (mask) {
    for (int c = 0; c < ncol; c++) {
      int K = 0;
      while (K < kmax && mask[(size_t)K * ncol + c] <= 0) K++;
      for (int k = K; k < kmax; k++)
        if (mask[(size_t)k * ncol + c] <= 0)
          return h->fail(SED_E_ARG, "mask of column %d has an unmasked cell below a masked one", c);
      ka[c] = K;
    }
  }
  // check_domain (fabm_sediment_driver.F90:503-530) on active cells
  for (int c = 0; c < ncol; c++)
    for (int k = 0; k < ka[c]; k++) {
      const size_t i = (size_t)k * ncol + c;
      if (!(phi[i] > 0.0) || phi[i] > 1.0 || !(phi_i[i] > 0.0) || phi_i[i] > 1.0)
        return h->fail(SED_E_ARG, "porosity outside (0,1] at column %d layer %d", c, k);
      if (!(dz[i] > 0.0)) return h->fail(SED_E_ARG, "dz <= 0 at column %d layer %d", c, k);
      if (k > 0 && !(dzc[(size_t)(k - 1) * ncol + c] > 0.0))
        return h->fail(SED_E_ARG, "dzc <= 0 at column %d layer %d", c, k);
    }
  // column segments: power-of-two count, contiguous ranges with equal
  // active-layer sums, bounds on multiples of 32 columns
  h->nactive = 0;
  long long work = 0;
  for (int c = 0; c < ncol; c++) {
    h->nactive += ka[c] > 0;
    work += ka[c];
  }
  h->nseg = 1;
  while (h->nseg < kMaxSeg && h->nactive / (2 * h->nseg) >= 4096) h->nseg *= 2;
  h->seg_col.assign(h->nseg + 1, ncol);
  h->seg_col[0] = 0;
  {
    long long acc = 0;
    int s = 1;
    for (int c = 0; c < ncol && s < h->nseg; c++) {
      acc += ka[c];
      if (acc * h->nseg >= work * s && (c + 1) % 32 == 0) h->seg_col[s++] = c + 1;
    }
  }
  // slots: depth class (<= 31 layers, 32..63, 64..127: the warp's last
  // lane stays free, so the no-flux bottom needs no select), then segment,
  // then active layers (stable); every (class, segment) run is padded to
  // kSlotPad slots
  h->slot_col.clear();
  h->slot_k.clear();
  for (int b = 0; b < kBins; b++) {
    Bin& bin = h->bins[b];
    bin.lpl = b == 2 ? 4 : b + 1;
    bin.slot0 = (int)h->slot_col.size();
    for (int sg = 0; sg < h->nseg; sg++) {
      bin.segb[sg] = (int)h->slot_col.size();
      std::vector<int> cols;
      for (int c = h->seg_col[sg]; c < h->seg_col[sg + 1]; c++)
        if (ka[c] > 0 && depth_class(ka[c]) == b) cols.push_back(c);
      std::stable_sort(cols.begin(), cols.end(), [&](int x, int y) { return ka[x] < ka[y]; });
      for (int c : cols) { h->slot_col.push_back(c); h->slot_k.push_back(ka[c]); }
      while (h->slot_col.size() % kSlotPad) { h->slot_col.push_back(-1); h->slot_k.push_back(0); }
    }
    bin.segb[h->nseg] = (int)h->slot_col.size();
    for (int sg = h->nseg + 1; sg <= kMaxSeg; sg++) bin.segb[sg] = bin.segb[h->nseg];
    bin.nslots = (int)h->slot_col.size() - bin.slot0;
    // FP32: the warp-direct kernel (the faster one over every regime of the
    // reference workloads); FP64: tiles
    bin.tc = !h->fp64() ? 0 : (b == 0 ? 32 : (b == 1 ? 16 : 8));
    bin.threads = !h->fp64() ? 128 : 256;
    bin.bps = 0;
  }
  if (h->slot_col.empty()) {
    h->slot_col.assign(kSlotPad, -1);
    h->slot_k.assign(kSlotPad, 0);
  }
  h->nslot = (int)h->slot_col.size();
  h->pipe = std::min(4, h->nseg);
  const bool bc4 = h->prm.bcup_particulate == 4;
  // device buffers
  const size_t ns = (size_t)h->nslot, rs = h->rsize();
  CK(h->d_slot_col.alloc(ns * sizeof(int)), "slot map");
  CK(h->d_kact.alloc(ns * sizeof(int)), "kact");
  CK(h->d_conc.alloc((size_t)NTR * kmax * ns * rs), "state");
  const bool bio3 = h->prm.bioturbation_profile == 3;
  const int ncoef = h->fp64() ? coef_rows<double>(bio3) : coef_rows<float>(bio3);
  CK(h->d_coef.alloc((size_t)ncoef * kmax * ns * rs), "coefficients");
  CK(h->d_force.alloc((size_t)NFORCE * ns * rs), "forcing");
  CK(h->d_sflux.alloc((size_t)NDISS * ns * rs), "surface flux");
  CK(h->d_nsub.alloc(ns * sizeof(int)), "attempts");
  CK(h->d_mindt.alloc(ns * sizeof(double)), "smallest substeps");
  if (h->prm.budgets) CK(h->d_budget.alloc(4 * ns * sizeof(double)), "budgets");
  if (bc4) CK(h->d_cap.alloc((size_t)kmax * ns * rs), "flux cap");
  CK(cudaMemsetAsync(h->d_conc.p, 0, (size_t)NTR * kmax * ns * rs, h->stream), "state clear");
  CK(cudaMemsetAsync(h->d_sflux.p, 0, (size_t)NDISS * ns * rs, h->stream), "flux clear");
  CK(cudaMemsetAsync(h->d_nsub.p, 0, ns * sizeof(int), h->stream), "attempts clear");
  CK(cudaMemsetAsync(h->d_mindt.p, 0, ns * sizeof(double), h->stream), "substeps clear");
  if (h->prm.budgets)
    CK(cudaMemsetAsync(h->d_budget.p, 0, 4 * ns * sizeof(double), h->stream), "budget clear");
  CK(cudaMemcpyAsync(h->d_slot_col.p, h->slot_col.data(), ns * sizeof(int),
                     cudaMemcpyHostToDevice, h->stream), "slot map copy");
  CK(cudaMemcpyAsync(h->d_kact.p, h->slot_k.data(), ns * sizeof(int),
                     cudaMemcpyHostToDevice, h->stream), "kact copy");
  // column -> slot map and FP64 dz(1), porosity(1) per column, for the
  // boundary assembly's flux estimate
  {
    std::vector<int> col_slot(ncol, -1);
    for (size_t i = 0; i < ns; i++)
      if (h->slot_col[i] >= 0) col_slot[h->slot_col[i]] = (int)i;
    std::vector<double> top(2 * (size_t)ncol);
    for (int c = 0; c < ncol; c++) { top[c] = dz[c]; top[(size_t)ncol + c] = phi[c]; }
    CK(h->d_col_slot.alloc((size_t)ncol * sizeof(int)), "column map");
    CK(h->d_top.alloc(2 * (size_t)ncol * sizeof(double)), "surface layer");
    CK(cudaMemcpyAsync(h->d_col_slot.p, col_slot.data(), (size_t)ncol * sizeof(int),
                       cudaMemcpyHostToDevice, h->stream), "column map copy");
    CK(cudaMemcpyAsync(h->d_top.p, top.data(), 2 * (size_t)ncol * sizeof(double),
                       cudaMemcpyHostToDevice, h->stream), "surface layer copy");
    CK(cudaStreamSynchronize(h->stream), "column map");
  }
  CK(h->d_tile_k.alloc((size_t)(h->nslot / 8 + 1) * sizeof(int)), "tile_k");
  if (h->table()) {  // the per-slot table follows the new layout
    if (h->bins[2].nslots > 0)
      return h->fail(SED_E_ARG, "per-column parameter sets and temperature-dependent rates "
                                "need columns of at most 63 active layers");
    for (Bin& bin : h->bins) bin.tc = 0;
    int rc = h->fp64() ? upload_bgc<double>(h) : upload_bgc<float>(h);
    if (rc) return rc;
  }
  {
    int rc = apply_tuning(h);
    if (rc) return rc;
  }
  // grid arrays through a temporary FP64 staging area
  const size_t lay = (size_t)kmax * ncol;
  CK(h->d_grid.alloc((9 * lay + ncol) * sizeof(double)), "grid staging");
  // tortuosity-corrected molecular diffusivity (mode 1) with the host's
  // logarithm: d0 phi_i / (1 - 2 ln phi_i)
  std::vector<double> mol;
  if (h->prm.mol_diff_mode == 1) {
    mol.assign(lay, 0.0);
    for (int c = 0; c < ncol; c++)
      for (int k = 0; k < ka[c]; k++) {
        const size_t i = (size_t)k * ncol + c;
        mol[i] = h->prm.mol_diff_d0 * phi_i[i] / (1.0 - 2.0 * std::log(phi_i[i]));
      }
  }
  double* g = h->d_grid.as<double>();
  CK(cudaMemcpyAsync(g + 0 * lay, dz, lay * sizeof(double), cudaMemcpyHostToDevice, h->stream), "dz");
  if (kmax > 1)
    CK(cudaMemcpyAsync(g + 1 * lay, dzc, (size_t)(kmax - 1) * ncol * sizeof(double),
                       cudaMemcpyHostToDevice, h->stream), "dzc");
  CK(cudaMemcpyAsync(g + 2 * lay, phi, lay * sizeof(double), cudaMemcpyHostToDevice, h->stream), "phi");
  CK(cudaMemcpyAsync(g + 3 * lay, phi_i, lay * sizeof(double), cudaMemcpyHostToDevice, h->stream), "phi_i");
  CK(cudaMemcpyAsync(g + 4 * lay, biofac, lay * sizeof(double), cudaMemcpyHostToDevice, h->stream), "biofac");
  if (bc4)
    CK(cudaMemcpyAsync(g + 5 * lay, flux_cap, lay * sizeof(double), cudaMemcpyHostToDevice,
                       h->stream), "flux_cap");
  const double* gmol = nullptr;
  if (!mol.empty()) {
    CK(cudaMemcpyAsync(g + 6 * lay, mol.data(), lay * sizeof(double), cudaMemcpyHostToDevice,
                       h->stream), "mol");
    gmol = g + 6 * lay;
  }
  cudaError_t e;
  if (h->fp64())
    e = launch_prep_grid<double>(g, g + lay, g + 2 * lay, g + 3 * lay, g + 4 * lay,
                                 bc4 ? g + 5 * lay : nullptr, gmol, h->d_slot_col.as<int>(),
                                 h->d_coef.as<double>(), bc4 ? h->d_cap.as<double>() : nullptr,
                                 kmax, ncol, h->nslot, h->prm.mol_diff_mode,
                                 h->prm.mol_diff_d0, h->sms, h->stream);
  else
    e = launch_prep_grid<float>(g, g + lay, g + 2 * lay, g + 3 * lay, g + 4 * lay,
                                bc4 ? g + 5 * lay : nullptr, gmol, h->d_slot_col.as<int>(),
                                h->d_coef.as<float>(), bc4 ? h->d_cap.as<float>() : nullptr,
                                kmax, ncol, h->nslot, h->prm.mol_diff_mode,
                                h->prm.mol_diff_d0, h->sms, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "grid launch");
  h->launches++;
  if (bio3) {
    // profile 3: zc from dz as init_grid forms it (:150-152), the two depth
    // exponentials of the biomass (get_rhs :639-640) and cumdepth, the depth
    // of the last layer's upper interface (:593-598), per column
    std::vector<double> e12(2 * lay, 1.0), cum(ncol, 0.0);
    const double kl = h->prm.bioturb_k_l;
    for (int c = 0; c < ncol; c++) {
      double zi = 0.0;
      for (int k = 0; k < ka[c]; k++) {
        const size_t i = (size_t)k * ncol + c;
        const double zc = zi + 0.5 * dz[i];
        zi = zi + dz[i];
        e12[i] = std::exp(zc * 100.0 * kl);
        e12[lay + i] = std::exp(zc * 200.0 * kl);
      }
      double cd = 0.0;
      for (int k = 0; k < ka[c] - 1; k++) cd = cd + dz[(size_t)k * ncol + c];
      cum[c] = cd;
    }
    CK(cudaMemcpyAsync(g + 7 * lay, e12.data(), 2 * lay * sizeof(double),
                       cudaMemcpyHostToDevice, h->stream), "profile-3 depth terms");
    CK(cudaMemcpyAsync(g + 9 * lay, cum.data(), ncol * sizeof(double),
                       cudaMemcpyHostToDevice, h->stream), "cumdepth");
    if (h->fp64())
      e = launch_prep_bio3<double>(g, g + lay, g + 3 * lay, g + 7 * lay, g + 8 * lay,
                                   g + 9 * lay, h->d_slot_col.as<int>(), h->d_coef.as<double>(),
                                   kmax, ncol, h->nslot, h->prm.bioturb_L1, h->prm.bioturb_L2,
                                   h->sms, h->stream);
    else
      e = launch_prep_bio3<float>(g, g + lay, g + 3 * lay, g + 7 * lay, g + 8 * lay,
                                  g + 9 * lay, h->d_slot_col.as<int>(), h->d_coef.as<float>(),
                                  kmax, ncol, h->nslot, h->prm.bioturb_L1, h->prm.bioturb_L2,
                                  h->sms, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "profile-3 grid launch");
    h->launches++;
    CK(cudaStreamSynchronize(h->stream), "set_grid");
  }
  CK(cudaStreamSynchronize(h->stream), "set_grid");
  h->d_grid.release();
  reset_graph(h);
  h->have_grid = true;
  h->have_state = false;
  h->have_forcing = false;
  return SED_OK;
}

int sed_set_forcing(sed_handle* h, const double* bdys, const double* fluxes) {
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  if (!bdys || !fluxes) return h->fail(SED_E_ARG, "bdys and fluxes are required");
  CK(cudaSetDevice(h->device), "set device");
  int rc = upload_forcing(h, bdys, fluxes);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream), "set_forcing");
  return SED_OK;
}

int sed_set_state(sed_handle* h, const double* conc) {
  NvtxScope range("sed_set_state");
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  if (!conc) return h->fail(SED_E_ARG, "conc is required");
  CK(cudaSetDevice(h->device), "set device");
  int rc = upload_state(h, conc);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream), "set_state");
  return SED_OK;
}

int sed_get_state(sed_handle* h, double* conc) {
  NvtxScope range("sed_get_state");
  if (!h) return SED_E_ARG;
  if (!h->have_state) return h->fail(SED_E_STATE, "no state: call sed_set_state first");
  if (!conc) return h->fail(SED_E_ARG, "conc is required");
  CK(cudaSetDevice(h->device), "set device");
  int rc = download_state(h, conc);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream), "get_state");
  return SED_OK;
}

int sed_step(sed_handle* h, double dt, int method, int nsteps, sed_stats* stats) {
  NvtxScope range("sed_step");
  int rc = ready(h);
  if (rc) return rc;
  if (!h->have_state) return h->fail(SED_E_STATE, "no state: call sed_set_state first");
  if (method < 0 || method > 3 || !(dt > 0.0) || nsteps < 0)
    return h->fail(SED_E_ARG, "bad dt, method or nsteps");
  CK(cudaSetDevice(h->device), "set device");
  const long long l0 = h->launches;
  rc = stats_reset(h);
  if (rc) return rc;
  CK(cudaEventRecord(h->ev0, h->stream), "event");
  for (int s = 0; s < nsteps; s++) {
    rc = h->fp64() ? step_any<double>(h, dt, method) : step_any<float>(h, dt, method);
    if (rc) return rc;
  }
  CK(cudaEventRecord(h->ev1, h->stream), "event");
  return stats_fetch(h, stats, l0, true);
}

int sed_ode_solver(sed_handle* h, double* conc, const double* bdys, double* fluxes,
                   double dt, int method, sed_stats* stats) {
  NvtxScope range("sed_ode_solver");
  int rc;
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  if (!conc || !bdys || !fluxes) return h->fail(SED_E_ARG, "conc, bdys and fluxes are required");
  if (method < 0 || method > 3 || !(dt > 0.0)) return h->fail(SED_E_ARG, "bad dt or method");
  CK(cudaSetDevice(h->device), "set device");
  const long long l0 = h->launches;
  if ((rc = stats_reset(h))) return rc;
  CK(cudaEventRecord(h->ev0, h->stream), "event");
  if ((rc = ode_solver_impl(h, conc, bdys, fluxes, dt, method))) return rc;
  CK(cudaEventRecord(h->ev1, h->stream), "event");
  return stats_fetch(h, stats, l0, true);
}

int sed_sur_set_norm(sed_surrogate* s, const float* norm, int n) {
  if (!s || !norm) return SED_E_ARG;
  const int need = NTR + 2 * s->nin + 2 * s->nout;
  if (n != need) return s->fail(SED_E_ARG, "norm has %d values, expected %d", n, need);
  if (cudaSetDevice(s->device) != cudaSuccess) return SED_E_CUDA;
  if (!s->norm) {
    if (s->alloc(&s->norm, (size_t)need) != cudaSuccess) return SED_E_NOMEM;
  }
  if (cudaMemcpy(s->norm, norm, need * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return SED_E_CUDA;
  s->norm_len = need;
  return SED_OK;
}

// The depth class holding every active column of a surrogate handle (all
// active columns have kmax layers); -1 if the columns are not all there.
static int surrogate_bin(sed_handle* h) {
  for (int i = 0; i < h->nslot; i++)
    if (h->slot_col[i] >= 0 && h->slot_k[i] != h->kmax) return -1;
  if (h->kmax > 63) return -1;
  const int b = depth_class(h->kmax);
  return h->bins[b].nslots > 0 ? b : -1;
}

// Warp-direct launch of one class's kernel over a's columns (a.ntiles of
// them: the class's slot range, or a slot list).
static cudaError_t launch_warp_columns(sed_handle* h, const ColumnArgs<float>& a,
                                       const Params<float>& p, const Bin& bin, int kind,
                                       cudaStream_t st) {
  const bool bc4 = h->prm.bcup_particulate == 4;
  const int threads = bin.threads;
  const int occ = column_warp_blocks_per_sm<float>(bin.lpl, bc4, kind, threads, p.bio3 != 0);
  const int warps = threads / 32;
  const int blocks =
      std::max(1, std::min(std::max(occ, 1) * h->sms, (a.ntiles + warps - 1) / warps));
  return launch_column_warp<float>(a, p, bin.lpl, bc4, kind, blocks, threads, st);
}

// The gated surrogate step over slot ranges of the surrogate's class: the
// checks, buffers and launch choices shared by sed_step_surrogate (one
// range, the whole class) and sed_ode_solver_surrogate (one range per
// pipeline chunk).  Chunk c lists its heavy columns in its own part of the
// list (from its first slot), counts them in d_gate[c] and takes feature
// and prediction rows from row0(c); d_gate[8 + c] and d_gate[16 + c] are
// its gate's tile counter and its fused kernel's column counter.
struct SurPlan {
  sed_handle* h = nullptr;
  sed_surrogate* s = nullptr;
  int b = 0;
  Params<float> p{};
  bool bc4 = false;
  int gate_tc = 0, gate_threads = 0, gate_occ = 0;
  double dt = 0.0, tol = 0.0, res_atol = 0.0;
  const Bin& bin() const { return h->bins[b]; }
  int row0(int sl0, int c) const { return (sl0 - bin().slot0) + 128 * c; }
};

static int sur_plan(sed_handle* h, sed_surrogate* s, double dt, double tol, double res_atol,
                    int chunks, SurPlan* P) {
  if (!s) return h->fail(SED_E_ARG, "no surrogate");
  if (h->table())
    return h->fail(SED_E_STATE,
                   "the surrogate has no per-column parameter sets or temperature-dependent "
                   "rates");
  if (h->fp64()) return h->fail(SED_E_ARG, "the surrogate step runs on FP32 state");
  if (h->prm.cut_scope != SED_CUT_PER_COLUMN)
    return h->fail(SED_E_ARG, "the surrogate step cuts substeps per column");
  if (s->device != h->device) return h->fail(SED_E_ARG, "surrogate on another device");
  const int K = h->kmax;
  if (s->nin != NTR * K + NFORCE || s->nout != NTR * K)
    return h->fail(SED_E_ARG, "surrogate sized for %d inputs / %d outputs, grid needs %d / %d",
                   s->nin, s->nout, NTR * K + NFORCE, NTR * K);
  if (!s->norm) return h->fail(SED_E_STATE, "sed_sur_set_norm has not been called");
  const int b = surrogate_bin(h);
  if (b < 0)
    return h->fail(SED_E_ARG, "the surrogate needs every active column at %d layers (at most 63)",
                   K);
  if (!(dt > 0.0) || !(tol >= 0.0) || !(res_atol >= 0.0))
    return h->fail(SED_E_ARG, "bad dt, tol or res_atol");
  CK(cudaSetDevice(h->device), "set device");
  P->h = h;
  P->s = s;
  P->b = b;
  P->dt = dt;
  P->tol = tol;
  P->res_atol = res_atol;
  const Bin& bin = h->bins[b];
  const int maxrows = pad128(bin.nslots) + 128 * chunks;
  CK(h->d_list.alloc((size_t)bin.nslots * sizeof(int)), "heavy list");
  CK(h->d_gate.alloc(32 * sizeof(unsigned)), "heavy counters");
  CK(h->d_xfeat.alloc((size_t)maxrows * s->pin[0] * sizeof(bf16)), "features");
  CK(h->d_yhat.alloc((size_t)maxrows * s->pout[s->L - 1] * sizeof(float)), "predictions");
  if (!sur_uses_tc(s))
    CK(h->d_act.alloc((size_t)2 * maxrows * s->pout[0] * sizeof(bf16)), "activations");
  P->p = make_params<float>(h->prm);
  set_clock(P->p, dt, h->prm.dt_min);
  // the gate's tile kernel: 256 threads and the widest tile of 32, 16 or 8
  // columns with the most resident blocks (one attempt per column is
  // latency-bound: the more resident warps, the better; at 256 threads the
  // kernel's registers allow four blocks per SM, which 16-column tiles fit
  // in shared memory and 32-column ones do not); the occupancy query also
  // raises the kernel's shared-memory limit, before any launch
  P->bc4 = h->prm.bcup_particulate == 4;
  P->gate_threads = 256;
  P->gate_tc = 0;
  P->gate_occ = 0;
  for (int tc = 32; tc >= 8; tc /= 2) {
    const int occ = column_blocks_per_sm<float>(tc, bin.lpl, P->bc4, KIND_PROBE,
                                                P->gate_threads, P->p.bio3 != 0);
    if (occ > P->gate_occ) {
      P->gate_occ = occ;
      P->gate_tc = tc;
    }
  }
  if (P->gate_occ <= 0) {
    P->gate_tc = bin.tc ? bin.tc : bin.tc_fb;
    P->gate_threads = bin.threads;
    P->gate_occ = column_blocks_per_sm<float>(P->gate_tc, bin.lpl, P->bc4, KIND_PROBE,
                                              P->gate_threads, P->p.bio3 != 0);
  }
  if (P->gate_occ <= 0) return h->fail(SED_E_CUDA, "the gate's tile kernel does not fit");
  return SED_OK;
}

// 1. gate over slots [sl0, sl1) (whole tiles): every column's first
//    (whole-step) attempt; columns that pass are done, exactly as the plain
//    step; the others are listed from list[0], counted in *count.  Then the
//    count is copied to the pinned h_count[c] and pe_cnt[c] recorded.
static int sur_gate(SurPlan& P, int c, int sl0, int sl1, cudaStream_t st) {
  sed_handle* h = P.h;
  const Bin& bin = P.bin();
  unsigned* cnt = h->d_gate.as<unsigned>();
  CK(cudaMemsetAsync(cnt + c, 0, sizeof(unsigned), st), "counter reset");
  CK(cudaMemsetAsync(cnt + 8 + c, 0, sizeof(unsigned), st), "queue reset");
  ColumnArgs<float> a = column_args<float>(h, bin, P.b, P.dt, SED_ADAPTIVE_EULER);
  a.heavy = h->d_list.as<int>() + (sl0 - bin.slot0);
  a.nheavy = cnt + c;
  a.queue = cnt + 8 + c;
  // the gate also writes the network's input rows of the columns it lists
  a.xfeat = reinterpret_cast<unsigned short*>(h->d_xfeat.as<bf16>() +
                                              (size_t)P.row0(sl0, c) * P.s->pin[0]);
  a.pin = P.s->pin[0];
  a.norm = P.s->norm;
  a.nin = P.s->nin;
  a.tc = P.gate_tc;
  a.tile_k = nullptr;  // every listed column has kmax layers: stage them all
  a.tile0 = 0;
  a.slot0 = sl0;
  a.ntiles = (sl1 - sl0) / P.gate_tc;
  if (a.ntiles <= 0) return SED_OK;
  CK(launch_column<float>(a, P.p, bin.lpl, P.bc4, KIND_PROBE,
                          std::max(1, std::min(a.ntiles, P.gate_occ * h->sms)), P.gate_threads,
                          st),
     "gate launch");
  h->launches++;
  CK(cudaMemcpyAsync(h->h_count + c, cnt + c, sizeof(unsigned), cudaMemcpyDeviceToHost, st),
     "counter copy");
  CK(cudaEventRecord(h->pe_cnt[c], st), "event");
  return SED_OK;
}

// chunk c's heavy count, once its gate is done (-1: CUDA error, recorded)
static int sur_count(SurPlan& P, int c) {
  const cudaError_t e = cudaEventSynchronize(P.h->pe_cnt[c]);
  if (e != cudaSuccess) {
    P.h->cuda_fail(e, "gate");
    return -1;
  }
  unsigned n = 0;
  memcpy(&n, P.h->h_count + c, sizeof n);
  return (int)n;
}

// Whether the step runs without host round trips: the fused tcgen05 network
// and the fallback kernel read the gate's count on the device.  The
// mma.sync network needs the count on the host for its GEMM grids.
static bool sur_device_count(const SurPlan& P) { return sur_uses_tc(P.s); }

// 2. the network's proposal rows for the listed columns of chunk c (slots
//    [sl0, sl1)): nh of them (host count; the rows up to the next multiple
//    of 128 are cleared), or, with nh < 0, as many as the gate counted on
//    the device (the fused kernel runs only the tiles holding them)
static int sur_propose(SurPlan& P, int c, int sl0, int sl1, int nh, cudaStream_t st) {
  sed_handle* h = P.h;
  sed_surrogate* s = P.s;
  const bool dev = nh < 0;
  const int rows = pad128(dev ? sl1 - sl0 : nh), r0 = P.row0(sl0, c);
  bf16* x = h->d_xfeat.as<bf16>() + (size_t)r0 * s->pin[0];
  float* y = h->d_yhat.as<float>() + (size_t)r0 * s->pout[s->L - 1];
  if (!dev && rows > nh)
    CK(cudaMemsetAsync(x + (size_t)nh * s->pin[0], 0,
                       (size_t)(rows - nh) * s->pin[0] * sizeof(bf16), st),
       "padding rows");
  bf16* act0 = h->d_act.as<bf16>();
  bf16* act1 = act0 ? act0 + (size_t)h->d_act.bytes / sizeof(bf16) / 2 : nullptr;
  int rc = sur_infer_rows(s, x, y, rows, act0, act1, st,
                          dev ? h->d_gate.as<unsigned>() + c : nullptr);
  if (rc) return h->fail(rc, "surrogate forward: %s", s->err.c_str());
  // one fused kernel, or one GEMM per layer
  h->launches += sur_uses_tc(s) ? 1 : s->L;
  return SED_OK;
}

// 3. each listed column's proposal from its prediction row and its residual
//    test; a column whose proposal passes takes it, the others take the
//    plain adaptive step from their state, in the same kernel (nh as for
//    sur_propose)
static int sur_finish(SurPlan& P, int c, int sl0, int sl1, int nh, cudaStream_t st) {
  sed_handle* h = P.h;
  sed_surrogate* s = P.s;
  const Bin& bin = P.bin();
  unsigned* cnt = h->d_gate.as<unsigned>();
  ColumnArgs<float> r = column_args<float>(h, bin, P.b, P.dt, SED_ADAPTIVE_EULER);
  r.list = h->d_list.as<int>() + (sl0 - bin.slot0);
  r.ntiles = nh < 0 ? sl1 - sl0 : nh;
  r.nlist = nh < 0 ? cnt + c : nullptr;
  r.yhat = h->d_yhat.as<float>() + (size_t)P.row0(sl0, c) * s->pout[s->L - 1];
  r.ldy = s->pout[s->L - 1];
  r.norm = s->norm;
  r.nin = s->nin;
  r.nout = s->nout;
  r.res_tol = P.tol;
  r.res_atol = P.res_atol;
  r.queue = cnt + 16 + c;
  CK(cudaMemsetAsync(r.queue, 0, sizeof(unsigned), st), "queue reset");
  CK(launch_warp_columns(h, r, P.p, bin, KIND_SUR, st), "residual and fallback launch");
  h->launches++;
  return SED_OK;
}

int sed_step_surrogate(sed_handle* h, sed_surrogate* s, double dt, int nsteps, double tol,
                       double res_atol, sed_stats* stats) {
  NvtxScope range("sed_step_surrogate");
  int rc = ready(h);
  if (rc) return rc;
  if (!h->have_state) return h->fail(SED_E_STATE, "no state: call sed_set_state first");
  if (nsteps < 0) return h->fail(SED_E_ARG, "nsteps < 0");
  SurPlan P;
  if ((rc = sur_plan(h, s, dt, tol, res_atol, 1, &P))) return rc;
  const long long l0 = h->launches;
  if ((rc = stats_reset(h))) return rc;
  const int sl0 = P.bin().slot0, sl1 = sl0 + P.bin().nslots;
  CK(cudaEventRecord(h->ev0, h->stream), "event");
  if (nsteps > 0 && (rc = ensure_pipeline(h))) return rc;
  for (int step = 0; step < nsteps; step++) {
    if ((rc = sur_gate(P, 0, sl0, sl1, h->stream))) return rc;
    int nh = -1;  // counted on the device: no host round trip
    if (!sur_device_count(P)) {
      nh = sur_count(P, 0);
      if (nh < 0) return SED_E_CUDA;
      if (nh == 0) continue;
    }
    if ((rc = sur_propose(P, 0, sl0, sl1, nh, h->stream))) return rc;
    if ((rc = sur_finish(P, 0, sl0, sl1, nh, h->stream))) return rc;
  }
  CK(cudaEventRecord(h->ev1, h->stream), "event");
  rc = stats_fetch(h, stats, l0, true);
  if (rc) return rc;
  if (sur_uses_tc(s) && (rc = sur_check_tc(s))) return h->fail(rc, "%s", s->err.c_str());
  return SED_OK;
}

// The drop-in step with the surrogate, its copies in flight: the column
// segments are the chunks.  Every chunk's host->device copy is queued at
// once on the copy-in stream; on the handle's stream each chunk is
// gathered and gated as it arrives, the next chunk's gate is queued before
// this chunk's network and fused kernel (so the host, which reads each
// chunk's heavy count, stays ahead), and each chunk is scattered and its
// device->host copy queued on the copy-out stream as soon as it is done.
int sed_ode_solver_surrogate(sed_handle* h, sed_surrogate* s, double* conc, const double* bdys,
                             double* fluxes, double dt, double tol, double res_atol,
                             sed_stats* stats) {
  NvtxScope range("sed_ode_solver_surrogate");
  // the call brings its own forcing (bdys, fluxes), as sed_ode_solver does
  int rc;
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  if (!conc || !bdys || !fluxes) return h->fail(SED_E_ARG, "conc, bdys and fluxes are required");
  const int nch = h->nseg;
  SurPlan P;
  if ((rc = sur_plan(h, s, dt, tol, res_atol, nch, &P))) return rc;
  if ((rc = ensure_pipeline(h))) return rc;
  if ((rc = upload_forcing(h, bdys, fluxes))) return rc;
  const long long l0 = h->launches;
  if ((rc = stats_reset(h))) return rc;
  const Bin& bin = P.bin();
  const size_t pitch = (size_t)h->ncol * sizeof(double);
  const size_t rows = (size_t)NTR * h->kmax;
  double* stage = h->d_stage.as<double>();
  CK(cudaEventRecord(h->ev0, h->stream), "event");
  CK(cudaEventRecord(h->pe_start, h->stream), "event");
  CK(cudaStreamWaitEvent(h->s_in, h->pe_start, 0), "wait");
  CK(cudaStreamWaitEvent(h->s_out, h->pe_start, 0), "wait");
  for (int c = 0; c < nch; c++) {
    const int col0 = h->seg_col[c], col1 = h->seg_col[c + 1];
    const size_t width = (size_t)(col1 - col0) * sizeof(double);
    if (width)
      CK(cudaMemcpy2DAsync(stage + col0, pitch, conc + col0, pitch, width, rows,
                           cudaMemcpyHostToDevice, h->s_in), "conc chunk copy");
    CK(cudaEventRecord(h->pe_in[c], h->s_in), "event");
  }
  // each chunk's work runs on a stream of its own, so the slow tail of one
  // chunk's fallback columns shares the GPU with the next chunks' gates and
  // fallbacks (the mma.sync network shares its activation buffers across
  // chunks: then one stream for all)
  auto cst = [&](int c) { return sur_uses_tc(s) ? h->s_cmp[c] : h->stream; };
  for (int c = 0; c < nch; c++) CK(cudaStreamWaitEvent(cst(c), h->pe_start, 0), "wait");
  auto front = [&](int c) -> int {
    const int sl0 = bin.segb[c], sl1 = bin.segb[c + 1];
    CK(cudaStreamWaitEvent(cst(c), h->pe_in[c], 0), "wait");
    if (sl1 == sl0) return SED_OK;
    CK(launch_gather_range<float>(stage, h->d_conc.as<float>(), h->d_slot_col.as<int>(), NTR,
                                  h->kmax, h->ncol, h->nslot, sl0, sl1 - sl0, h->sms, cst(c)),
       "gather launch");
    h->launches++;
    return sur_gate(P, c, sl0, sl1, cst(c));
  };
  if ((rc = front(0))) return rc;
  for (int c = 0; c < nch; c++) {
    const int sl0 = bin.segb[c], sl1 = bin.segb[c + 1];
    // with the device count nothing waits on the host: every chunk's work
    // is queued at once
    int nh = 0;
    if (sl1 > sl0) {
      if (sur_device_count(P)) nh = -1;
      else if ((nh = sur_count(P, c)) < 0) return SED_E_CUDA;
    }
    if (nh != 0 && (rc = sur_propose(P, c, sl0, sl1, nh, cst(c)))) return rc;
    if (c + 1 < nch && (rc = front(c + 1))) return rc;
    if (nh != 0 && (rc = sur_finish(P, c, sl0, sl1, nh, cst(c)))) return rc;
    if (sl1 > sl0) {
      CK(launch_scatter_range<float>(h->d_conc.as<float>(), stage, h->d_slot_col.as<int>(),
                                     h->d_kact.as<int>(), NTR, h->kmax, h->ncol, h->nslot, sl0,
                                     sl1 - sl0, h->sms, cst(c)), "scatter launch");
      h->launches++;
    }
    CK(cudaEventRecord(h->pe_cmp[c], cst(c)), "event");
    CK(cudaStreamWaitEvent(h->s_out, h->pe_cmp[c], 0), "wait");
    const int col0 = h->seg_col[c], col1 = h->seg_col[c + 1];
    const size_t width = (size_t)(col1 - col0) * sizeof(double);
    if (width)
      CK(cudaMemcpy2DAsync(conc + col0, pitch, stage + col0, pitch, width, rows,
                           cudaMemcpyDeviceToHost, h->s_out), "conc chunk copy back");
  }
  // s_out has waited for every chunk: the surface fluxes are final
  CK(launch_scatter_flux<float>(h->d_sflux.as<float>(), h->d_fluxes.as<double>(),
                                h->d_slot_col.as<int>(), h->d_kact.as<int>(), h->ncol, h->nslot,
                                h->sms, h->s_out), "flux scatter launch");
  h->launches++;
  CK(cudaMemcpyAsync(fluxes, h->d_fluxes.p, (size_t)NTR * h->ncol * sizeof(double),
                     cudaMemcpyDeviceToHost, h->s_out), "fluxes copy back");
  CK(cudaEventRecord(h->pe_done, h->s_out), "event");
  CK(cudaStreamWaitEvent(h->stream, h->pe_done, 0), "wait");
  CK(cudaEventRecord(h->ev1, h->stream), "event");
  h->have_state = true;
  rc = stats_fetch(h, stats, l0, true);
  if (rc) return rc;
  if (sur_uses_tc(s) && (rc = sur_check_tc(s))) return h->fail(rc, "%s", s->err.c_str());
  return SED_OK;
}

int sed_sur_collect(sed_handle* h, const float* c0, double dt, float* x_dev, float* y_dev,
                    int pitch_x, int pitch_y, long long capacity, long long* count,
                    sed_stats* stats) {
  int rc = ready(h);
  if (rc) return rc;
  if (!c0 || !x_dev || !y_dev || !count || capacity < 0 || *count < 0)
    return h->fail(SED_E_ARG, "c0, x, y and count are required");
  if (!h->have_state) return h->fail(SED_E_STATE, "no state: call sed_set_state first");
  if (h->fp64()) return h->fail(SED_E_ARG, "training rows come from FP32 state");
  if (h->table())
    return h->fail(SED_E_STATE, "training rows use the handle's parameter set, without "
                                "temperature-dependent rates");
  if (h->prm.cut_scope != SED_CUT_PER_COLUMN)
    return h->fail(SED_E_ARG, "training rows come from per-column cuts");
  const int K = h->kmax;
  if (pitch_x < NTR * K + NFORCE || pitch_y < NTR * K)
    return h->fail(SED_E_ARG, "row pitches %d / %d below %d / %d", pitch_x, pitch_y,
                   NTR * K + NFORCE, NTR * K);
  const int b = surrogate_bin(h);
  if (b < 0)
    return h->fail(SED_E_ARG, "training rows need every active column at %d layers (at most 63)",
                   K);
  if (!(dt > 0.0)) return h->fail(SED_E_ARG, "bad dt");
  CK(cudaSetDevice(h->device), "set device");
  const size_t state = (size_t)NTR * K * h->nslot * sizeof(float);
  CK(h->d_backup.alloc(state), "state copy");
  // d_gate: the row counter, then the log offsets c0 at byte 64
  CK(h->d_gate.alloc(128), "row counter");
  const long long l0 = h->launches;
  if ((rc = stats_reset(h))) return rc;
  float* d_c0 = reinterpret_cast<float*>(h->d_gate.as<unsigned char>() + 64);
  CK(cudaMemcpyAsync(d_c0, c0, NTR * sizeof(float), cudaMemcpyHostToDevice, h->stream),
     "c0 copy");
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(h->d_gate.p);
  *h->h_count = (unsigned long long)*count;
  CK(cudaMemcpyAsync(cnt, h->h_count, sizeof(unsigned long long), cudaMemcpyHostToDevice,
                     h->stream),
     "counter copy");
  CK(cudaMemcpyAsync(h->d_backup.p, h->d_conc.p, state, cudaMemcpyDeviceToDevice, h->stream),
     "state copy");
  CK(cudaEventRecord(h->ev0, h->stream), "event");
  if ((rc = enqueue_columns<float>(h, dt, SED_ADAPTIVE_EULER, KIND_ADAPT))) return rc;
  CK(cudaEventRecord(h->ev1, h->stream), "event");
  const Bin& bin = h->bins[b];
  CK(sur::collect(h->d_backup.as<float>(), h->d_conc.as<float>(), h->d_force.as<float>(),
                  h->d_kact.as<int>(), h->d_nsub.as<int>(), d_c0, K, h->kmax, h->nslot,
                  bin.slot0, bin.nslots, x_dev, pitch_x, y_dev, pitch_y, cnt, capacity, h->sms,
                  h->stream),
     "collect");
  h->launches++;
  CK(cudaMemcpyAsync(h->h_count, cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     h->stream),
     "counter copy");
  if ((rc = stats_fetch(h, stats, l0, true))) return rc;
  *count = std::min((long long)*h->h_count, capacity);
  return SED_OK;
}

int sed_get_rhs(sed_handle* h, const double* conc, double* rhs, double* fluxes) {
  int rc;
  if (!h) return SED_E_ARG;
  if ((rc = ready(h))) return rc;
  if (!conc || !rhs) return h->fail(SED_E_ARG, "conc and rhs are required");
  if (h->table())
    return h->fail(SED_E_STATE, "sed_get_rhs has no per-column parameter sets or "
                                "temperature-dependent rates");
  CK(cudaSetDevice(h->device), "set device");
  const size_t n = (size_t)NTR * h->kmax * h->nslot * h->rsize();
  CK(h->d_rhs.alloc(n), "rhs buffer");
  if ((rc = upload_state(h, conc))) return rc;
  if ((rc = h->fp64() ? enqueue_columns<double>(h, 0.0, 0, KIND_RHS)
                      : enqueue_columns<float>(h, 0.0, 0, KIND_RHS)))
    return rc;
  // rhs of inactive cells is zero (get_rhs :703-708)
  const size_t bytes = (size_t)NTR * h->kmax * h->ncol * sizeof(double);
  CK(h->d_rhs_stage.alloc(bytes), "rhs staging");
  CK(cudaMemsetAsync(h->d_rhs_stage.p, 0, bytes, h->stream), "rhs clear");
  rc = h->fp64() ? scatter_state<double>(h, h->d_rhs.as<double>(), h->d_rhs_stage.as<double>())
                 : scatter_state<float>(h, h->d_rhs.as<float>(), h->d_rhs_stage.as<double>());
  if (rc) return rc;
  CK(cudaMemcpyAsync(rhs, h->d_rhs_stage.p, bytes, cudaMemcpyDeviceToHost, h->stream),
     "rhs copy back");
  if (fluxes) {
    rc = h->fp64() ? scatter_fluxes<double>(h) : scatter_fluxes<float>(h);
    if (rc) return rc;
    CK(cudaMemcpyAsync(fluxes, h->d_fluxes.p, (size_t)NTR * h->ncol * sizeof(double),
                       cudaMemcpyDeviceToHost, h->stream), "fluxes copy back");
  }
  CK(cudaStreamSynchronize(h->stream), "get_rhs");
  return SED_OK;
}

int sed_get_fluxes(sed_handle* h, double* fluxes) {
  if (!h) return SED_E_ARG;
  if (!h->have_forcing) return h->fail(SED_E_STATE, "sed_set_forcing has not been called");
  if (!fluxes) return h->fail(SED_E_ARG, "fluxes is required");
  CK(cudaSetDevice(h->device), "set device");
  int rc = h->fp64() ? scatter_fluxes<double>(h) : scatter_fluxes<float>(h);
  if (rc) return rc;
  CK(cudaMemcpyAsync(fluxes, h->d_fluxes.p, (size_t)NTR * h->ncol * sizeof(double),
                     cudaMemcpyDeviceToHost, h->stream), "fluxes copy back");
  CK(cudaStreamSynchronize(h->stream), "get_fluxes");
  return SED_OK;
}

int sed_get_attempts(sed_handle* h, int* attempts) {
  if (!h || !attempts) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  CK(cudaSetDevice(h->device), "set device");
  std::vector<int> tmp(h->nslot);
  CK(cudaMemcpyAsync(tmp.data(), h->d_nsub.p, tmp.size() * sizeof(int), cudaMemcpyDeviceToHost,
                     h->stream), "attempts copy");
  CK(cudaStreamSynchronize(h->stream), "attempts");
  for (int c = 0; c < h->ncol; c++) attempts[c] = 0;
  for (int s = 0; s < h->nslot; s++)
    if (h->slot_col[s] >= 0) attempts[h->slot_col[s]] = tmp[s];
  return SED_OK;
}

// Histogram of the last step's attempts over the active slots: bin 0 counts
// the columns without an attempt (the surrogate's), bin b >= 1 those with
// 2^(b-1) <= attempts < 2^b, the last bin every count above.  Block counts
// in shared memory, one global atomic per bin and block.
__global__ void k_attempt_hist(const int* __restrict__ nsub, const int* __restrict__ kact,
                               int nslot, unsigned long long* __restrict__ hist) {
  __shared__ unsigned int sh[SED_HIST_BINS];
  for (int i = threadIdx.x; i < SED_HIST_BINS; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nslot; s += gridDim.x * blockDim.x) {
    if (kact[s] <= 0) continue;
    const int a = nsub[s];
    const int b = a <= 0 ? 0 : min(32 - __clz(a), SED_HIST_BINS - 1);
    atomicAdd(&sh[b], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < SED_HIST_BINS; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], (unsigned long long)sh[i]);
}

int sed_get_attempt_histogram(sed_handle* h, long long* counts) {
  if (!h || !counts) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  CK(cudaSetDevice(h->device), "set device");
  CK(h->d_hist.alloc(SED_HIST_BINS * sizeof(unsigned long long)), "histogram");
  CK(cudaMemsetAsync(h->d_hist.p, 0, SED_HIST_BINS * sizeof(unsigned long long), h->stream),
     "histogram reset");
  const int blocks = std::max(1, std::min((h->nslot + 255) / 256, 4 * h->sms));
  k_attempt_hist<<<blocks, 256, 0, h->stream>>>(h->d_nsub.as<int>(), h->d_kact.as<int>(),
                                                h->nslot, h->d_hist.as<unsigned long long>());
  CK(cudaGetLastError(), "histogram launch");
  h->launches++;
  unsigned long long tmp[SED_HIST_BINS];
  CK(cudaMemcpyAsync(tmp, h->d_hist.p, sizeof tmp, cudaMemcpyDeviceToHost, h->stream),
     "histogram copy");
  CK(cudaStreamSynchronize(h->stream), "histogram");
  for (int i = 0; i < SED_HIST_BINS; i++) counts[i] = (long long)tmp[i];
  return SED_OK;
}

int sed_get_min_dt_grid_cell(sed_handle* h, double* last_min_dt, int* cell) {
  if (!h || !last_min_dt || !cell) return SED_E_ARG;
  if (!h->prm.adaptive_solver_diagnostics || h->prm.cut_scope != SED_CUT_GLOBAL)
    return h->fail(SED_E_STATE, "recorded by the grid-wide cut with "
                                "adaptive_solver_diagnostics set");
  *last_min_dt = h->last_min_dt;
  for (int i = 0; i < 4; i++) cell[i] = h->last_cell[i];
  return SED_OK;
}

int sed_get_min_dt(sed_handle* h, double* min_dt) {
  if (!h || !min_dt) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  CK(cudaSetDevice(h->device), "set device");
  std::vector<double> tmp(h->nslot);
  CK(cudaMemcpyAsync(tmp.data(), h->d_mindt.p, tmp.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, h->stream), "substeps copy");
  CK(cudaStreamSynchronize(h->stream), "min_dt");
  for (int c = 0; c < h->ncol; c++) min_dt[c] = 0.0;
  for (int s = 0; s < h->nslot; s++)
    if (h->slot_col[s] >= 0) min_dt[h->slot_col[s]] = tmp[s];
  return SED_OK;
}

int sed_set_column_bgc(sed_handle* h, const double* params) {
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  CK(cudaSetDevice(h->device), "set device");
  if (!params) {
    h->has_bgc = false;
    h->bgc_cols.clear();
    reset_graph(h);
    if (!h->temp_rates()) {
      h->d_bgc.release();
      return SED_OK;
    }
    // the handle's own set, scaled by temperature
    return h->fp64() ? upload_bgc<double>(h) : upload_bgc<float>(h);
  }
  const size_t nc = (size_t)h->ncol;
  for (int i = 0; i < SED_NBGC; i++)
    for (size_t c = 0; c < nc; c++) {
      const double v = params[i * nc + c];
      if (!(v >= 0.0) || !std::isfinite(v))
        return h->fail(SED_E_ARG, "parameter %d of column %zu is negative or not finite", i, c);
    }
  if (h->prm.cut_scope == SED_CUT_GLOBAL)
    return h->fail(SED_E_ARG, "per-column parameter sets need per-column cuts");
  h->bgc_cols.assign(params, params + SED_NBGC * nc);
  h->has_bgc = true;
  if (h->bins[2].nslots > 0)
    return h->fail(SED_E_ARG, "per-column parameter sets need columns of at most 63 active "
                              "layers");
  // ensembles step with the warp-direct kernels
  Bin keep[kBins];
  std::copy(h->bins, h->bins + kBins, keep);
  for (Bin& bin : h->bins) bin.tc = 0;
  int rc = h->fp64() ? upload_bgc<double>(h) : upload_bgc<float>(h);
  if (!rc) rc = apply_tuning(h);
  if (rc) {
    const std::string why = h->err;
    h->has_bgc = false;
    std::copy(keep, keep + kBins, h->bins);
    apply_tuning(h);
    h->err = why;
    return rc;
  }
  reset_graph(h);
  return SED_OK;
}

int sed_get_budgets(sed_handle* h, double* budgets) {
  if (!h || !budgets) return SED_E_ARG;
  if (!h->prm.budgets) return h->fail(SED_E_STATE, "budgets were not enabled in sed_params");
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  CK(cudaSetDevice(h->device), "set device");
  std::vector<double> tmp((size_t)4 * h->nslot);
  CK(cudaMemcpyAsync(tmp.data(), h->d_budget.p, tmp.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, h->stream), "budget copy");
  CK(cudaStreamSynchronize(h->stream), "budgets");
  for (size_t i = 0; i < (size_t)4 * h->ncol; i++) budgets[i] = 0.0;
  for (int b = 0; b < 4; b++)
    for (int s = 0; s < h->nslot; s++)
      if (h->slot_col[s] >= 0)
        budgets[(size_t)b * h->ncol + h->slot_col[s]] = tmp[(size_t)b * h->nslot + s];
  return SED_OK;
}

int sed_set_stream(sed_handle* h, void* stream) {
  if (!h) return SED_E_ARG;
  CK(cudaSetDevice(h->device), "set device");
  CK(cudaStreamSynchronize(h->stream), "stream switch");
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
  reset_graph(h);
  return SED_OK;
}

}  // extern "C"

namespace {

// Forcing rows of one column on the host, as get_rhs forms them (the FP64
// path's prep_force_host64 for a single column).
void column_forcing(const sed_params& prm, const double* bdys1, const double* fluxes1,
                    double (&f)[NFORCE]) {
  const double T = bdys1[0];
  const double f_T = 1.0 * std::exp(-4500.0 * (1.0 / (T + 273.0) - (1.0 / 288.0)));
  f[0] = prm.bioturbation_profile == 3 ? 1.0 : prm.bioturbation * f_T;
  f[1] = prm.mol_diff_mode == 1 ? 1.0 : (prm.diffusivity + T * 0.035);
  for (int n = 0; n < NTR; n++)
    f[2 + n] = (n < NPART || prm.bcup_dissolved == 1) ? fluxes1[n] : bdys1[n + 1];
}

// nsteps coupling steps of the warp-direct kernel over slots [s0, s1) of a
// class, in launches of up to kRepeat steps.
constexpr int kRepeat = 24;

template <typename real>
int spin_range(sed_handle* h, const Bin& bin, int b, int s0, int s1, double dt, int method,
               long long nsteps, int blocks, int threads) {
  Params<real> p = make_params<real>(h->prm);
  set_clock(p, dt, h->prm.dt_min);
  const int kind = method == SED_ADAPTIVE_EULER ? KIND_ADAPT : KIND_FIXED;
  const long long per = method == SED_ADAPTIVE_EULER ? kRepeat : 1;
  for (long long done = 0; done < nsteps; done += per) {
    ColumnArgs<real> a = column_args<real>(h, bin, b, dt, method);
    a.tc = 0;
    a.tile_k = nullptr;
    a.slot0 = s0;
    a.tile0 = 0;
    a.ntiles = s1 - s0;
    // several steps per launch for the adaptive method, one otherwise
    a.nrepeat = method == SED_ADAPTIVE_EULER ? (int)std::min<long long>(kRepeat, nsteps - done)
                                             : 1;
    CK(cudaMemsetAsync(a.queue, 0, sizeof(unsigned), h->stream), "queue reset");
    CK(launch_column_warp<real>(a, p, bin.lpl, h->prm.bcup_particulate == 4, kind, blocks,
                                threads, h->stream), "spin-up launch");
    h->launches++;
  }
  return SED_OK;
}

template <typename real>
int spinup_t(sed_handle* h, int mode, int column, const double* bdys1, const double* fluxes1,
             double dt, int method, long long nsteps) {
  const bool bc4 = h->prm.bcup_particulate == 4, bio3 = h->prm.bioturbation_profile == 3;
  const int kind = method == SED_ADAPTIVE_EULER ? KIND_ADAPT : KIND_FIXED;
  if (mode == SED_SPINUP_ALL) {
    for (int b = 0; b < kBins; b++) {
      const Bin& bin = h->bins[b];
      if (bin.nslots == 0) continue;
      const int occ = column_warp_blocks_per_sm<real>(bin.lpl, bc4, kind, 128, bio3);
      if (occ <= 0) return h->fail(SED_E_CUDA, "spin-up kernel does not fit");
      const int blocks = std::max(1, std::min((bin.nslots + 3) / 4, occ * h->sms));
      int rc = spin_range<real>(h, bin, b, bin.slot0, bin.slot0 + bin.nslots, dt, method, nsteps,
                                blocks, 128);
      if (rc) return rc;
    }
    return SED_OK;
  }
  // the column and its slot
  int slot = -1;
  if (column < 0) {
    int best = 0;
    for (int s = 0; s < h->nslot; s++)
      if (h->slot_col[s] >= 0 && h->slot_k[s] > best) { best = h->slot_k[s]; slot = s; }
    // the first such column in grid order
    for (int s = 0; s < h->nslot; s++)
      if (h->slot_col[s] >= 0 && h->slot_k[s] == best && h->slot_col[s] < h->slot_col[slot])
        slot = s;
  } else {
    for (int s = 0; s < h->nslot; s++)
      if (h->slot_col[s] == column) slot = s;
  }
  if (slot < 0) return h->fail(SED_E_ARG, "spin-up column %d is not an active column", column);
  int b = 0;
  for (int q = 0; q < kBins; q++)
    if (slot >= h->bins[q].slot0 && slot < h->bins[q].slot0 + h->bins[q].nslots) b = q;
  // its forcing rows replaced by the spin-up forcing, and put back after
  const size_t rs = h->rsize(), pitch = (size_t)h->nslot * rs;
  std::vector<real> saved(NFORCE), spin(NFORCE);
  double f[NFORCE];
  column_forcing(h->prm, bdys1, fluxes1, f);
  for (int r = 0; r < NFORCE; r++) spin[r] = (real)f[r];
  real* fcol = h->d_force.as<real>() + slot;
  CK(cudaMemcpy2DAsync(saved.data(), rs, fcol, pitch, rs, NFORCE, cudaMemcpyDeviceToHost,
                       h->stream), "forcing save");
  CK(cudaMemcpy2DAsync(fcol, pitch, spin.data(), rs, rs, NFORCE, cudaMemcpyHostToDevice,
                       h->stream), "spin-up forcing");
  // with temperature-dependent rates, the column's rates at the spin-up
  // temperature in place of its own, put back after
  std::vector<real> saved_tab(NBGC_DEV), spin_tab(NBGC_DEV);
  real* tcol = h->temp_rates() ? h->d_bgc.as<real>() + slot : nullptr;
  if (tcol) {
    CK(cudaMemcpy2DAsync(spin_tab.data(), rs, h->d_bgc_base.as<real>() + slot, pitch, rs,
                         NBGC_DEV, cudaMemcpyDeviceToHost, h->stream), "rates read");
    CK(cudaMemcpy2DAsync(saved_tab.data(), rs, tcol, pitch, rs, NBGC_DEV,
                         cudaMemcpyDeviceToHost, h->stream), "rates save");
    CK(cudaStreamSynchronize(h->stream), "rates read");
    const double fr = rate_factor(h->prm.temp_activation, bdys1[0]);
    for (int i = 0; i < NRATE_TEMP; i++) spin_tab[i] = (real)((double)spin_tab[i] * fr);
    CK(cudaMemcpy2DAsync(tcol, pitch, spin_tab.data(), rs, rs, NBGC_DEV,
                         cudaMemcpyHostToDevice, h->stream), "spin-up rates");
  }
  int rc = spin_range<real>(h, h->bins[b], b, slot, slot + 1, dt, method, nsteps, 1, 32);
  if (rc) return rc;
  CK(cudaMemcpy2DAsync(fcol, pitch, saved.data(), rs, rs, NFORCE, cudaMemcpyHostToDevice,
                       h->stream), "forcing restore");
  if (tcol)
    CK(cudaMemcpy2DAsync(tcol, pitch, saved_tab.data(), rs, rs, NBGC_DEV,
                         cudaMemcpyHostToDevice, h->stream), "rates restore");
  CK(launch_broadcast<real>(h->d_conc.as<real>(), h->d_kact.as<int>(), slot, h->nslot, h->kmax,
                            h->sms, h->stream), "broadcast launch");
  h->launches++;
  CK(cudaStreamSynchronize(h->stream), "spin-up");  // the host vectors above
  return SED_OK;
}

}  // namespace

extern "C" {

int sed_spinup(sed_handle* h, int mode, int column, const double* bdys1, const double* fluxes1,
               double dt, int method, long long nsteps, sed_stats* stats) {
  NvtxScope range("sed_spinup");
  int rc;
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  if (!h->have_state) return h->fail(SED_E_STATE, "no state: call sed_set_state first");
  if (mode != SED_SPINUP_COLUMN && mode != SED_SPINUP_ALL)
    return h->fail(SED_E_ARG, "mode must be SED_SPINUP_COLUMN or SED_SPINUP_ALL");
  if (mode == SED_SPINUP_ALL && !h->have_forcing)
    return h->fail(SED_E_STATE, "sed_set_forcing has not been called");
  if (mode == SED_SPINUP_COLUMN && (!bdys1 || !fluxes1))
    return h->fail(SED_E_ARG, "bdys1 and fluxes1 are required for the column spin-up");
  if (method < 0 || method > 3 || !(dt > 0.0) || nsteps < 0)
    return h->fail(SED_E_ARG, "bad dt, method or nsteps");
  if (method == SED_ADAPTIVE_EULER && h->prm.cut_scope == SED_CUT_GLOBAL)
    return h->fail(SED_E_ARG, "the spin-up cuts per column (the 1-column model has no other)");
  CK(cudaSetDevice(h->device), "set device");
  const long long l0 = h->launches;
  if ((rc = stats_reset(h))) return rc;
  CK(cudaEventRecord(h->ev0, h->stream), "event");
  rc = h->fp64() ? spinup_t<double>(h, mode, column, bdys1, fluxes1, dt, method, nsteps)
                 : spinup_t<float>(h, mode, column, bdys1, fluxes1, dt, method, nsteps);
  if (rc) return rc;
  CK(cudaEventRecord(h->ev1, h->stream), "event");
  return stats_fetch(h, stats, l0, true);
}

int sed_set_boundary(sed_handle* h, const double* temperature, const double* surface,
                     const double* velocity, const int* present) {
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  if (!temperature || !surface)
    return h->fail(SED_E_ARG, "temperature and surface are required");
  unsigned mask = 0;
  for (int n = 0; n < NTR; n++)
    if (!present || present[n]) mask |= 1u << n;
  const unsigned part = (1u << NPART) - 1u;
  if ((mask & part) && !velocity)
    return h->fail(SED_E_ARG, "velocity is required for the particulate tracers present");
  cpl::SedStaging s;
  if (int rc = cpl::sed_staging(h, &s)) return rc;
  const size_t nc = (size_t)h->ncol;
  CK(cudaMemcpyAsync(s.temperature, temperature, nc * sizeof(double), cudaMemcpyHostToDevice,
                     h->stream), "temperature copy");
  CK(cudaMemcpyAsync(s.surface, surface, (size_t)NTR * nc * sizeof(double),
                     cudaMemcpyHostToDevice, h->stream), "surface copy");
  if (velocity)  // only the particulate rows are read
    CK(cudaMemcpyAsync(s.velocity, velocity, (size_t)NPART * nc * sizeof(double),
                       cudaMemcpyHostToDevice, h->stream), "velocity copy");
  return cpl::sed_assemble_staged(h, mask);
}

}  // extern "C"

int cpl::sed_staging(sed_handle* h, SedStaging* s) {
  if (!h || !s) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  CK(cudaSetDevice(h->device), "set device");
  const size_t nc = (size_t)h->ncol;
  CK(h->d_bcin.alloc((3 + 2 * (size_t)NTR) * nc * sizeof(double)), "boundary staging");
  s->temperature = h->d_bcin.as<double>();
  s->surface = s->temperature + nc;
  s->velocity = s->surface + (size_t)NTR * nc;
  s->spare = s->velocity + (size_t)NTR * nc;
  s->ncol = h->ncol;
  s->device = h->device;
  s->sms = h->sms;
  s->stream = h->stream;
  return SED_OK;
}

int cpl::sed_surface_fluxes(sed_handle* h, const double** fluxes) {
  if (!h || !fluxes) return SED_E_ARG;
  if (!h->have_forcing) return h->fail(SED_E_STATE, "the handle has no forcing yet");
  CK(cudaSetDevice(h->device), "set device");
  int rc = h->fp64() ? scatter_fluxes<double>(h) : scatter_fluxes<float>(h);
  if (rc) return rc;
  *fluxes = h->d_fluxes.as<double>();
  return SED_OK;
}

int cpl::sed_fail(sed_handle* h, int code, const char* msg) {
  return h ? h->fail(code, "%s", msg) : code;
}

void cpl::sed_count_launch(sed_handle* h) { h->launches++; }

int cpl::sed_launches(const sed_handle* h) { return (int)h->launches; }

int cpl::sed_assemble_staged(sed_handle* h, unsigned mask) {
  const unsigned part = (1u << NPART) - 1u;
  if (h->prm.bcup_dissolved == 1 && (mask & ~part) && !h->have_state)
    return h->fail(SED_E_STATE, "the dissolved flux estimate needs the state: call "
                                "sed_set_state first");
  const size_t nc = (size_t)h->ncol;
  double* bt = h->d_bcin.as<double>();
  double* bs = bt + nc;
  double* bv = bs + (size_t)NTR * nc;
  cudaError_t e =
      h->fp64()
          ? launch_assemble_bc<double>(bt, bs, bv, mask, h->d_conc.as<double>(),
                                       h->d_col_slot.as<int>(), h->d_top.as<double>(),
                                       h->d_bdys.as<double>(), h->d_fluxes.as<double>(), h->ncol,
                                       h->nslot, h->kmax, h->prm.bcup_dissolved,
                                       h->prm.bioturbation, h->prm.diffusivity, h->sms, h->stream)
          : launch_assemble_bc<float>(bt, bs, bv, mask, h->d_conc.as<float>(),
                                      h->d_col_slot.as<int>(), h->d_top.as<double>(),
                                      h->d_bdys.as<double>(), h->d_fluxes.as<double>(), h->ncol,
                                      h->nslot, h->kmax, h->prm.bcup_dissolved,
                                      h->prm.bioturbation, h->prm.diffusivity, h->sms, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "boundary assembly launch");
  h->launches++;
  int rc;
  if (h->fp64()) {
    // the FP64 forcing rows use the host's exp (see prep_force_host64)
    std::vector<double> hb((size_t)(NTR + 1) * nc), hf((size_t)NTR * nc);
    CK(cudaMemcpyAsync(hb.data(), h->d_bdys.p, hb.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, h->stream), "bdys copy back");
    CK(cudaMemcpyAsync(hf.data(), h->d_fluxes.p, hf.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, h->stream), "fluxes copy back");
    CK(cudaStreamSynchronize(h->stream), "boundary assembly");
    rc = prep_force_host64(h, hb.data(), hf.data());
  } else {
    rc = prep_force<float>(h);
  }
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream), "boundary assembly");
  h->have_forcing = true;
  return SED_OK;
}

extern "C" {

int sed_get_boundary(sed_handle* h, double* bdys, double* fluxes) {
  if (!h) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  CK(cudaSetDevice(h->device), "set device");
  if (bdys)
    CK(cudaMemcpyAsync(bdys, h->d_bdys.p, (size_t)(NTR + 1) * h->ncol * sizeof(double),
                       cudaMemcpyDeviceToHost, h->stream), "bdys copy back");
  if (fluxes)
    CK(cudaMemcpyAsync(fluxes, h->d_fluxes.p, (size_t)NTR * h->ncol * sizeof(double),
                       cudaMemcpyDeviceToHost, h->stream), "fluxes copy back");
  CK(cudaStreamSynchronize(h->stream), "get_boundary");
  return SED_OK;
}

int sed_get_tuning(const sed_handle* h, sed_tuning* t) {
  if (!h || !t) return SED_E_ARG;
  memset(t, 0, sizeof *t);
  for (int b = 0; b < kTunedBins; b++) {
    t->tile_columns[b] = h->bins[b].tc;
    t->threads[b] = h->bins[b].threads;
    t->blocks_per_sm[b] = h->bins[b].bps;
  }
  t->pipeline_chunks = h->pipe;
  t->segments = h->nseg;
  t->max_attempts = h->prm.max_attempts;
  return SED_OK;
}

int sed_set_tuning(sed_handle* h, const sed_tuning* t) {
  if (!h || !t) return SED_E_ARG;
  if (!h->have_grid) return h->fail(SED_E_STATE, "sed_set_grid has not been called");
  for (int b = 0; b < kTunedBins; b++) {
    const int tc = t->tile_columns[b], th = t->threads[b];
    if (tc != 0 && tc != 8 && tc != 16 && tc != 32 && tc != 64)
      return h->fail(SED_E_ARG, "tile_columns[%d]=%d: 0 (warp-direct), 8, 16, 32 or 64", b, tc);
    if (th < 64 || th > 256 || th % 64 != 0)
      return h->fail(SED_E_ARG, "threads[%d]=%d: 64, 128, 192 or 256", b, th);
    if (tc != 0 && h->table())
      return h->fail(SED_E_ARG, "per-column parameter sets and temperature-dependent rates "
                                "step warp-direct only (tile 0)");
    if (t->blocks_per_sm[b] < 0) return h->fail(SED_E_ARG, "blocks_per_sm[%d] < 0", b);
  }
  const int pc = t->pipeline_chunks;
  if (pc < 1 || pc > h->nseg || (h->nseg % pc) != 0 || (pc & (pc - 1)) != 0)
    return h->fail(SED_E_ARG, "pipeline_chunks=%d must be a power of two dividing %d", pc,
                   h->nseg);
  if (t->max_attempts <= 0) return h->fail(SED_E_ARG, "max_attempts must be > 0");
  CK(cudaSetDevice(h->device), "set device");
  Bin keep[kBins];
  std::copy(h->bins, h->bins + kBins, keep);
  for (int b = 0; b < kTunedBins; b++) {
    h->bins[b].tc = t->tile_columns[b];
    h->bins[b].threads = t->threads[b];
    h->bins[b].bps = t->blocks_per_sm[b];
  }
  int rc = apply_tuning(h);
  if (rc) {
    const std::string why = h->err;
    std::copy(keep, keep + kBins, h->bins);
    apply_tuning(h);
    h->err = why;
    return rc;
  }
  h->pipe = pc;
  h->prm.max_attempts = t->max_attempts;
  return SED_OK;
}

int sed_autotune(sed_handle* h, double dt, int method, int flags, sed_tuning* out) {
  NvtxScope range("sed_autotune");
  int rc = ready(h);
  if (rc) return rc;
  if (!h->have_state) return h->fail(SED_E_STATE, "no state: call sed_set_state first");
  if (method < 0 || method > 3 || !(dt > 0.0) || (flags & ~3))
    return h->fail(SED_E_ARG, "bad dt, method or flags");
  CK(cudaSetDevice(h->device), "set device");
  return h->fp64() ? autotune_t<double>(h, dt, method, flags, out)
                   : autotune_t<float>(h, dt, method, flags, out);
}

int sed_host_register(void* ptr, size_t bytes) {
  if (!ptr || !bytes) return SED_E_ARG;
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) { cudaGetLastError(); return SED_E_CUDA; }
  return SED_OK;
}

int sed_host_unregister(void* ptr) {
  if (!ptr) return SED_E_ARG;
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) { cudaGetLastError(); return SED_E_CUDA; }
  return SED_OK;
}

int sed_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return SED_E_ARG;
  *ptr = nullptr;
  if (!bytes) return SED_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return SED_E_NODEVICE;
  }
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocPortable);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return SED_E_NOMEM;
  }
  return SED_OK;
}

int sed_host_free(void* ptr) {
  if (!ptr) return SED_E_ARG;
  cudaError_t e = cudaFreeHost(ptr);
  if (e != cudaSuccess) { cudaGetLastError(); return SED_E_CUDA; }
  return SED_OK;
}

const char* sed_error_string(int code) {
  switch (code) {
    case SED_OK: return "ok";
    case SED_E_ARG: return "invalid argument";
    case SED_E_NAN: return "NaN in state";
    case SED_E_SUBSTEP_CAP: return "adaptive substep cap reached";
    case SED_E_CUDA: return "CUDA error";
    case SED_E_STATE: return "call order: grid, forcing or state missing";
    case SED_E_NOMEM: return "out of memory";
    case SED_E_NODEVICE: return "no CUDA device";
    case SED_E_TOO_LARGE: return "grid exceeds the no-allocation scratch array";
    default: return "unknown error";
  }
}

const char* sed_last_error(const sed_handle* h) { return h ? h->err.c_str() : ""; }

const char* sed_tracer_name(int n) {
  return (n >= 0 && n < SED_NTR) ? kTracerNames[n] : "";
}

int sed_tracer_is_particulate(int n) { return (n >= 0 && n < NPART) ? 1 : 0; }

void sed_destroy(sed_handle* h) { delete h; }

}  // extern "C"
