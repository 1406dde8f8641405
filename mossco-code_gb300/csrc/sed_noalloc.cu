// sed_noalloc.cu -- sed_ode_solver_noalloc: one coupling step of the drop-in
// ode_solver without any device allocation.
//
// Some callers cannot allocate device memory: a component whose host
// framework owns the GPU's memory pool and forbids other allocators, or a
// call site that cannot keep a solver handle (and the buffers it allocates)
// alive between calls.  This entry point runs the tile form of the column
// kernel (k_column: 32-, 16- or 8-column tiles for columns of up to 31, 63
// or 127 layers, 256 threads), with every device
// buffer it needs -- the staging of the caller's FP64 arrays, the FP32 state,
// coefficients and forcing, the tile work counter and the step statistics --
// in one file-scope __device__ array of SED_NOALLOC_SCRATCH_BYTES.  Every GPU
// that loads the library holds that array until the process exits.  The
// per-column arithmetic is the one of every other FP32 kernel of the
// library, so the results equal sed_ode_solver's bit for bit.
//
// The array's host-side name is only a stand-in: host code obtains its
// device address with cudaGetSymbolAddress, with the call's device current,
// and passes that address to the kernels.  Every call looks the address up
// again (the runtime answers from its own table after the first call in a
// context), so a context that was destroyed and created again -- a
// cudaDeviceReset by the caller -- gets the array's new address.  All calls
// share the array and it keeps the last call's contents; each call
// re-initialises what it reads (work counter, statistics, staged inputs).
// Calls that overlap on the GPU from several host threads of one process
// race on the shared array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "../../include/mossco_sed.h"
#include "sed_launch.h"
#include "sed_params.h"

using namespace sed;

static __device__ __align__(256) unsigned char g_sed_noalloc_scratch[SED_NOALLOC_SCRATCH_BYTES];

namespace {

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte offsets of the buffers inside the scratch array.
struct Layout {
  size_t queue, stats, stage, conc, coef, cap, force, bdys, fluxes, sflux,
      nsub, kact_in, slot_col, slot_k, tile_k, total;
};

Layout make_layout(int ncol, int kmax, int nslot, int ntiles, bool bc4) {
  Layout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o = up256(o + bytes); return at; };
  L.queue = take(4 * sizeof(unsigned));
  L.stats = take(sizeof(DevStats));
  // FP64 staging: first the grid arrays (6 x kmax x ncol), then the state
  const size_t cells = (size_t)kmax * ncol;
  L.stage = take(std::max((size_t)NTR, (size_t)6) * cells * sizeof(double));
  L.conc = take((size_t)NTR * kmax * nslot * sizeof(float));
  L.coef = take((size_t)NCOEF * kmax * nslot * sizeof(float));
  L.cap = take(bc4 ? (size_t)kmax * nslot * sizeof(float) : 0);
  L.force = take((size_t)NFORCE * nslot * sizeof(float));
  L.bdys = take((size_t)(NTR + 1) * ncol * sizeof(double));
  L.fluxes = take((size_t)NTR * ncol * sizeof(double));
  L.sflux = take((size_t)NDISS * nslot * sizeof(float));
  L.nsub = take((size_t)nslot * sizeof(int));
  L.kact_in = take((size_t)ncol * sizeof(int));
  L.slot_col = take((size_t)nslot * sizeof(int));
  L.slot_k = take((size_t)nslot * sizeof(int));
  L.tile_k = take((size_t)ntiles * sizeof(int));
  L.total = o;
  return L;
}

// Slots in column order (no compaction: land columns are slots with zero
// layers, which the column kernel skips) and the layers staged per tile.
__global__ void k_noalloc_slots(const int* __restrict__ kact, int use_kact,
                                int ncol, int kmax, int nslot, int tc,
                                int* __restrict__ slot_col,
                                int* __restrict__ slot_k,
                                int* __restrict__ tile_k) {
  const int ntiles = nslot / tc;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles;
       t += gridDim.x * blockDim.x) {
    int m = 1;
    for (int j = 0; j < tc; j++) {
      const int slot = t * tc + j;
      const int K = slot < ncol ? (use_kact ? kact[slot] : kmax) : 0;
      slot_col[slot] = slot < ncol ? slot : -1;
      slot_k[slot] = K;
      m = K > m ? K : m;
    }
    tile_k[t] = m;
  }
}

}  // namespace

extern "C" int sed_ode_solver_noalloc(const sed_params* p, int inum, int jnum,
                                      int kmax, const double* dz,
                                      const double* dzc, const double* phi,
                                      const double* phi_i, const double* biofac,
                                      const double* flux_cap, const int* kact,
                                      double* conc, const double* bdys,
                                      double* fluxes, double dt, int method,
                                      sed_stats* stats) {
  if (!p || !dz || !phi || !phi_i || !biofac || !conc || !bdys || !fluxes)
    return SED_E_ARG;
  if (inum <= 0 || jnum <= 0 || kmax < 1 || kmax > SED_KMAX_LIMIT) return SED_E_ARG;
  if ((long long)inum * jnum > (1LL << 30)) return SED_E_ARG;
  if (kmax > 1 && !dzc) return SED_E_ARG;
  if (p->precision != SED_FP32 || p->cut_scope != SED_CUT_PER_COLUMN) return SED_E_ARG;
  if (p->bcup_dissolved < 1 || p->bcup_dissolved > 3) return SED_E_ARG;
  if (p->bcup_particulate != 1 && p->bcup_particulate != 4) return SED_E_ARG;
  if (p->bcup_particulate == 4 && !flux_cap) return SED_E_ARG;
  if (p->mol_diff_mode != 0 && p->mol_diff_mode != 1) return SED_E_ARG;
  if (p->max_attempts <= 0 || !(p->atol >= 0.0)) return SED_E_ARG;
  if (p->bioturbation_profile == 3) return SED_E_ARG;  // static biofac only
  if (p->temp_activation != 0.0) return SED_E_ARG;     // the handle's rate set only
  if (method < 0 || method > 3 || !(dt > 0.0)) return SED_E_ARG;
  const int ncol = inum * jnum;
  // the same domain checks as sed_set_grid (fabm_sediment_driver.F90:503-530)
  for (int c = 0; c < ncol; c++) {
    const int K = kact ? kact[c] : kmax;
    if (K < 0 || K > kmax) return SED_E_ARG;
    for (int k = 0; k < K; k++) {
      const size_t i = (size_t)k * ncol + c;
      if (!(phi[i] > 0.0) || phi[i] > 1.0 || !(phi_i[i] > 0.0) || phi_i[i] > 1.0)
        return SED_E_ARG;
      if (!(dz[i] > 0.0)) return SED_E_ARG;
      if (k > 0 && !(dzc[(size_t)(k - 1) * ncol + c] > 0.0)) return SED_E_ARG;
    }
  }
  const bool bc4 = p->bcup_particulate == 4;
  const int lpl = kmax > 63 ? 4 : (kmax > 31 ? 2 : 1);
  const int tc = kmax > 63 ? 8 : (kmax > 31 ? 16 : 32);
  const int ntiles = (ncol + tc - 1) / tc;
  const int nslot = ntiles * tc;
  const Layout L = make_layout(ncol, kmax, nslot, ntiles, bc4);
  if (L.total > (size_t)SED_NOALLOC_SCRATCH_BYTES) return SED_E_TOO_LARGE;

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return SED_E_NODEVICE;
  }
  if (p->device < 0 || p->device >= ndev) return SED_E_ARG;
  if (cudaSetDevice(p->device) != cudaSuccess) return SED_E_CUDA;
  // the array's device address in the current context of this device
  unsigned char* base = nullptr;
  {
    void* addr = nullptr;
    if (cudaGetSymbolAddress(&addr, g_sed_noalloc_scratch) != cudaSuccess || !addr) {
      cudaGetLastError();
      return SED_E_CUDA;
    }
    base = static_cast<unsigned char*>(addr);
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess)
    return SED_E_CUDA;
  const int kind = method == SED_ADAPTIVE_EULER ? KIND_ADAPT : KIND_FIXED;
  const int occ = column_blocks_per_sm<float>(tc, lpl, bc4, kind, 256, false);
  if (occ <= 0) return SED_E_CUDA;

  // the calling thread's default stream: ordered with this thread's other
  // default-stream work, not with the device's other streams
  cudaStream_t st = cudaStreamPerThread;
  int launches = 0;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; return e == cudaSuccess; };
  double* stage = reinterpret_cast<double*>(base + L.stage);
  const size_t cells = (size_t)kmax * ncol;
  int* slot_col = reinterpret_cast<int*>(base + L.slot_col);
  int* slot_k = reinterpret_cast<int*>(base + L.slot_k);
  int* tile_k = reinterpret_cast<int*>(base + L.tile_k);

  // slots
  if (kact) ok(cudaMemcpyAsync(base + L.kact_in, kact, ncol * sizeof(int),
                              cudaMemcpyHostToDevice, st));
  if (ok(cudaSuccess)) {
    const int blocks = std::max(1, std::min((ntiles + 127) / 128, sms * 4));
    k_noalloc_slots<<<blocks, 128, 0, st>>>(reinterpret_cast<int*>(base + L.kact_in),
                                            kact ? 1 : 0, ncol, kmax, nslot, tc,
                                            slot_col, slot_k, tile_k);
    launches++;
    ok(cudaGetLastError());
  }
  // grid coefficients from the staged FP64 arrays
  ok(cudaMemcpyAsync(stage, dz, cells * sizeof(double), cudaMemcpyHostToDevice, st));
  if (kmax > 1)
    ok(cudaMemcpyAsync(stage + cells, dzc, (size_t)(kmax - 1) * ncol * sizeof(double),
                       cudaMemcpyHostToDevice, st));
  ok(cudaMemcpyAsync(stage + 2 * cells, phi, cells * sizeof(double), cudaMemcpyHostToDevice, st));
  ok(cudaMemcpyAsync(stage + 3 * cells, phi_i, cells * sizeof(double), cudaMemcpyHostToDevice, st));
  ok(cudaMemcpyAsync(stage + 4 * cells, biofac, cells * sizeof(double), cudaMemcpyHostToDevice, st));
  if (bc4)
    ok(cudaMemcpyAsync(stage + 5 * cells, flux_cap, cells * sizeof(double),
                       cudaMemcpyHostToDevice, st));
  if (ok(cudaSuccess)) {
    ok(launch_prep_grid<float>(stage, stage + cells, stage + 2 * cells, stage + 3 * cells,
                               stage + 4 * cells, bc4 ? stage + 5 * cells : nullptr,
                               nullptr, slot_col, reinterpret_cast<float*>(base + L.coef),
                               bc4 ? reinterpret_cast<float*>(base + L.cap) : nullptr,
                               kmax, ncol, nslot, p->mol_diff_mode, p->mol_diff_d0, sms, st));
    launches++;
  }
  // state (the staging area now holds the caller's conc, kept for the
  // cells the kernel does not write), forcing
  ok(cudaMemcpyAsync(stage, conc, (size_t)NTR * cells * sizeof(double),
                     cudaMemcpyHostToDevice, st));
  ok(cudaMemcpyAsync(base + L.bdys, bdys, (size_t)(NTR + 1) * ncol * sizeof(double),
                     cudaMemcpyHostToDevice, st));
  ok(cudaMemcpyAsync(base + L.fluxes, fluxes, (size_t)NTR * ncol * sizeof(double),
                     cudaMemcpyHostToDevice, st));
  if (ok(cudaSuccess)) {
    ok(launch_gather<float>(stage, reinterpret_cast<float*>(base + L.conc), slot_col, NTR,
                            kmax, ncol, nslot, sms, st));
    ok(launch_prep_force<float>(reinterpret_cast<double*>(base + L.bdys),
                                reinterpret_cast<double*>(base + L.fluxes), slot_col,
                                reinterpret_cast<float*>(base + L.force), ncol, nslot,
                                p->bioturbation, p->diffusivity, p->mol_diff_mode,
                                p->bcup_dissolved, 0, sms, st));
    launches += 2;
  }
  // work counter and statistics start from zero / +inf
  DevStats zero{};
  zero.min_dt_bits = 0x7FF0000000000000ull;
  ok(cudaMemsetAsync(base + L.queue, 0, 4 * sizeof(unsigned), st));
  ok(cudaMemcpyAsync(base + L.stats, &zero, sizeof zero, cudaMemcpyHostToDevice, st));
  if (ok(cudaSuccess)) {
    Params<float> kp = make_params<float>(*p);
    set_clock(kp, dt, p->dt_min);
    kp.budgets = 0;
    ColumnArgs<float> a{};
    a.conc = reinterpret_cast<float*>(base + L.conc);
    a.out = nullptr;
    a.coef = reinterpret_cast<float*>(base + L.coef);
    a.cap = bc4 ? reinterpret_cast<float*>(base + L.cap) : nullptr;
    a.force = reinterpret_cast<float*>(base + L.force);
    a.kact = slot_k;
    a.tile_k = tile_k;
    a.sflux = reinterpret_cast<float*>(base + L.sflux);
    a.budget = nullptr;
    a.nsub = reinterpret_cast<int*>(base + L.nsub);
    a.queue = reinterpret_cast<unsigned*>(base + L.queue);
    a.stats = reinterpret_cast<DevStats*>(base + L.stats);
    a.nslot = nslot;
    a.kmax = kmax;
    a.tc = tc;
    a.tile0 = 0;
    a.ntiles = ntiles;
    a.dt = dt;
    a.method = method;
    const int blocks = std::max(1, std::min(ntiles, occ * sms));
    ok(launch_column<float>(a, kp, lpl, bc4, kind, blocks, 256, st));
    launches++;
  }
  // results back into the caller's arrays
  if (ok(cudaSuccess)) {
    ok(launch_scatter<float>(reinterpret_cast<float*>(base + L.conc), stage, slot_col,
                             slot_k, NTR, kmax, ncol, nslot, sms, st));
    ok(launch_scatter_flux<float>(reinterpret_cast<float*>(base + L.sflux),
                                  reinterpret_cast<double*>(base + L.fluxes), slot_col,
                                  slot_k, ncol, nslot, sms, st));
    launches += 2;
  }
  // the caller's arrays are written only when every step before succeeded
  if (ok(cudaSuccess)) {
    ok(cudaMemcpyAsync(conc, stage, (size_t)NTR * cells * sizeof(double),
                       cudaMemcpyDeviceToHost, st));
    ok(cudaMemcpyAsync(fluxes, base + L.fluxes, (size_t)NTR * ncol * sizeof(double),
                       cudaMemcpyDeviceToHost, st));
  }
  DevStats s{};
  ok(cudaMemcpyAsync(&s, base + L.stats, sizeof s, cudaMemcpyDeviceToHost, st));
  ok(cudaStreamSynchronize(st));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SED_E_CUDA;
  }
  if (stats) {
    stats->attempts = (long long)s.attempts;
    stats->accepted = (long long)s.accepted;
    stats->column_steps = (long long)s.column_steps;
    stats->max_col_attempts = s.max_col_attempts;
    stats->capped_columns = s.capped;
    stats->nan_cells = s.nan_cells;
    stats->gpu_launches = launches;
    double md;
    unsigned long long bits = s.min_dt_bits;
    memcpy(&md, &bits, sizeof md);
    stats->min_dt = md;
    stats->device_ms = 0.0;
    stats->surrogate_columns = 0;
  }
  if (s.status & ST_NAN) return SED_E_NAN;
  if (s.status & ST_CAP) return SED_E_SUBSTEP_CAP;
  return SED_OK;
}
