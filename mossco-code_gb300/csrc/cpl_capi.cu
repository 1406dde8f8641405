// cpl_capi.cu -- the pelagic <-> soil coupling of include/mossco_cpl.h.
//
// k_pelagic_soil: one thread per horizontal column reads the pelagic
// state's bottom layer (k = 0) and writes the sediment handle's boundary
// staging rows with the arithmetic of pelagic_soil_connector's Run
// (src/mediators/pelagic_soil_connector.F90:648-2110, 3-D pelagic fields and
// 2-D soil fields, the branch the reference's set-ups take).  The sediment
// handle then assembles bdys / fluxes from those rows as sed_set_boundary
// does.  k_soil_pelagic: the reverse, soil_pelagic_connector's Run, from the
// sediment's fluxes into the pelagic handle's bottom-flux rows.
// Both are pointwise: a few dozen FP64 operations per column on about a
// dozen doubles, which GB300's FP64 pipe bounds before HBM does.  Compiled
// with -fmad=false so that every product and quotient rounds as the
// connectors' Fortran expressions do.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/mossco_cpl.h"
#include "cpl_internal.h"
#include "cpl_map.cuh"

namespace {

using namespace cplmap;

// Device buffers of one forward launch
struct ForwardBufs {
  const void* state;   // the pelagic state [PEL_NTR][K][ncol]
  int ncol, K;
  const double* depth;  // [ncol] when a.use_depth
  const double* tke;    // [ncol] when a.use_tke
  double* surface;      // the sediment's staging rows [NTR][ncol]
  double* velocity;     // [NTR][ncol]
};

template <typename real>
__global__ void k_pelagic_soil(Forward a, ForwardBufs b) {
  const real* st = static_cast<const real*>(b.state);
  const size_t layer = (size_t)b.K * b.ncol;  // one tracer's block
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < b.ncol;
       col += gridDim.x * blockDim.x) {
    auto B = [&](int n) { return (double)st[(size_t)n * layer + col]; };
    const ForwardOut o = pelagic_soil_column(a, B, a.use_depth ? b.depth[col] : 0.0,
                                             a.use_tke ? b.tke[col] : 0.0);
    for (int n = 0; n < NTR; n++) b.surface[(size_t)n * b.ncol + col] = o.S[n];
    for (int n = 0; n < NPART; n++)
      if ((o.vrows >> n) & 1u) b.velocity[(size_t)n * b.ncol + col] = o.w;
  }
}

// ---- the reverse direction: soil upward fluxes into the pelagic bottom
// fluxes (soil_pelagic_connector.F90:179-965)

struct ReverseBufs {
  const double* fluxes;  // the sediment's [NTR][ncol], downward positive
  void* bfl;             // the pelagic handle's [PEL_NTR][ncol], its precision
  int ncol;
};

template <typename real>
__global__ void k_soil_pelagic(Reverse a, ReverseBufs b) {
  real* out = static_cast<real*>(b.bfl);
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < b.ncol;
       col += gridDim.x * blockDim.x) {
    auto U = [&](int n) { return -b.fluxes[(size_t)n * b.ncol + col]; };
    auto W = [&](int row, double v) { out[(size_t)row * b.ncol + col] = (real)v; };
    soil_pelagic_column(a, U, W);
  }
}

bool bad_index(int i) { return i < -1 || i >= PEL_NTR; }

// CUDA events at marks 0..3 on one stream (none unless init was called)
struct Timing {
  cudaEvent_t ev[4] = {};
  cudaStream_t st = nullptr;
  bool on = false;
  void init(cudaError_t* err, cudaStream_t s) {
    st = s;
    on = true;
    for (auto& x : ev)
      if (cudaEventCreate(&x) != cudaSuccess) { on = false; *err = cudaErrorMemoryAllocation; }
  }
  void mark(int i) {
    if (on) cudaEventRecord(ev[i], st);
  }
  double ms(int a, int b) {
    float t = 0.0f;
    if (!on || cudaEventElapsedTime(&t, ev[a], ev[b]) != cudaSuccess) return 0.0;
    return t;
  }
  ~Timing() {
    for (auto& x : ev)
      if (x) cudaEventDestroy(x);
  }
};

}  // namespace

extern "C" {

int cpl_default_params(cpl_params* p) {
  if (!p) return SED_E_ARG;
  memset(p, 0, sizeof *p);
  // pelagic_soil_connector.F90:38-45; the literals without a kind suffix
  // are default reals, so 0.02 and 0.1 are their single-precision values
  p->sinking_factor = 0.3;
  p->sinking_factor_min = (double)0.02f;
  p->NC_ldet = 0.23;
  p->NC_sdet = 0.01;
  p->convertN = 1.0;
  p->convertP = 1.0;
  p->half_sedimentation_depth = (double)0.1f;
  p->half_sedimentation_tke = 1.0e3;
  p->critical_detritus = 60.0;
  p->mode = CPL_AS_RUN;
  return SED_OK;
}

int cpl_npzd_fields(cpl_fields* f) {
  if (!f) return SED_E_ARG;
  f->detN = 3;
  f->detC = -1;
  f->detP = -1;
  f->din = 0;
  f->nitrate = -1;
  f->ammonium = -1;
  f->oxygen = -1;
  f->odu = -1;
  f->dip = -1;
  return SED_OK;
}

int cpl_soil_default_params(cpl_soil_params* p) {
  if (!p) return SED_E_ARG;
  memset(p, 0, sizeof *p);
  // soil_pelagic_connector.F90:36-41 (0.0 and -1. are default reals)
  p->dinflux_const = (double)0.0f;
  p->dipflux_const = (double)-1.0f;
  p->NC_ldet = 0.20;
  p->NC_sdet = 0.04;
  p->convertP = 1.0;
  p->convertN = 1.0;
  return SED_OK;
}

int cpl_soil_pelagic(sed_handle* sed, pel_handle* pel, const cpl_soil_params* p,
                     const cpl_fields* f, double* bottom_flux_out, int* present_out,
                     cpl_stats* stats) {
  if (stats) memset(stats, 0, sizeof *stats);
  if (!sed) return SED_E_ARG;
  if (!pel) return cpl::sed_fail(sed, SED_E_ARG, "pelagic handle is NULL");
  if (!p || !f) return cpl::sed_fail(sed, SED_E_ARG, "params and fields are required");
  const int rows[] = {f->nitrate, f->ammonium, f->din, f->dip, f->oxygen, f->odu,
                      f->detN, f->detC, f->detP};
  for (int i : rows)
    if (bad_index(i)) return cpl::sed_fail(sed, SED_E_ARG, "field index out of range");
  for (int i = 0; i < 9; i++)
    for (int j = i + 1; j < 9; j++)
      if (rows[i] >= 0 && rows[i] == rows[j])
        return cpl::sed_fail(sed, SED_E_ARG, "two fields on one pelagic tracer");
  void* bfl = nullptr;
  if (int rc = cpl::pel_bottom_flux(pel, &bfl)) {
    std::string m = std::string("pelagic handle: ") + pel_last_error(pel);
    return cpl::sed_fail(sed, rc, m.c_str());
  }
  cpl::PelView v;
  if (int rc = cpl::pel_view(pel, &v, false)) {
    std::string m = std::string("pelagic handle: ") + pel_last_error(pel);
    return cpl::sed_fail(sed, rc, m.c_str());
  }
  cpl::SedStaging s;
  if (int rc = cpl::sed_staging(sed, &s)) return rc;
  if (v.ncol != s.ncol)
    return cpl::sed_fail(sed, SED_E_ARG, "the handles' grids differ in inum*jnum");
  if (v.device != s.device)
    return cpl::sed_fail(sed, SED_E_ARG, "the handles are on different devices");
  const double* fl = nullptr;
  if (int rc = cpl::sed_surface_fluxes(sed, &fl)) return rc;
  cudaStream_t pst = v.stream;
  const bool fp64 = v.fp64;
  const size_t nc = (size_t)s.ncol;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; return r == cudaSuccess; };
  // the sediment's last step and flux scatter before the reads
  cudaEvent_t ev = nullptr;
  ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  if (e == cudaSuccess) {
    ok(cudaEventRecord(ev, s.stream));
    ok(cudaStreamWaitEvent(pst, ev, 0));
  }
  if (ev) cudaEventDestroy(ev);
  Timing tm;
  if (stats) tm.init(&e, pst);
  const Reverse a = make_reverse(p, f);
  ReverseBufs rb{fl, bfl, s.ncol};
  const int threads = 256;
  long long blocks = ((long long)nc + threads - 1) / threads;
  const long long cap = (long long)(s.sms > 0 ? s.sms : 1) * 8;
  if (blocks > cap) blocks = cap;
  tm.mark(0);
  tm.mark(1);
  if (e == cudaSuccess) {
    if (fp64)
      k_soil_pelagic<double><<<(int)blocks, threads, 0, pst>>>(a, rb);
    else
      k_soil_pelagic<float><<<(int)blocks, threads, 0, pst>>>(a, rb);
    e = cudaGetLastError();
  }
  tm.mark(2);
  std::vector<float> tmp32;
  if (bottom_flux_out && e == cudaSuccess) {
    if (fp64) {
      ok(cudaMemcpyAsync(bottom_flux_out, bfl, PEL_NTR * nc * sizeof(double),
                         cudaMemcpyDeviceToHost, pst));
    } else {
      tmp32.resize(PEL_NTR * nc);
      ok(cudaMemcpyAsync(tmp32.data(), bfl, PEL_NTR * nc * sizeof(float),
                         cudaMemcpyDeviceToHost, pst));
    }
  }
  tm.mark(3);
  ok(cudaStreamSynchronize(pst));
  if (e != cudaSuccess) {
    std::string m = std::string("soil coupling: ") + cudaGetErrorString(e);
    return cpl::sed_fail(sed, SED_E_CUDA, m.c_str());
  }
  if (bottom_flux_out && !fp64)
    for (size_t i = 0; i < tmp32.size(); i++) bottom_flux_out[i] = (double)tmp32[i];
  if (present_out) {
    for (int n = 0; n < PEL_NTR; n++) present_out[n] = 0;
    for (int i : rows)
      if (i >= 0) present_out[i] = 1;
  }
  if (stats) {
    stats->gpu_launches = 2;  // the sediment's flux scatter and the mapping
    stats->columns = (long long)nc;
    stats->kernel_ms = tm.ms(1, 2);
    stats->device_ms = tm.ms(0, 3);
  }
  return SED_OK;
}

int cpl_pelagic_soil(pel_handle* pel, sed_handle* sed, const cpl_params* p,
                     const cpl_fields* f, const double* temperature,
                     const double* water_depth, const double* tke,
                     const double* velocity_in, double* surface_out,
                     double* velocity_out, int* present_out, cpl_stats* stats) {
  if (stats) memset(stats, 0, sizeof *stats);
  if (!sed) return SED_E_ARG;
  if (!pel) return cpl::sed_fail(sed, SED_E_ARG, "pelagic handle is NULL");
  if (!p || !f || !temperature)
    return cpl::sed_fail(sed, SED_E_ARG, "params, fields and temperature are required");
  for (int i : {f->detN, f->detC, f->detP, f->din, f->nitrate, f->ammonium, f->oxygen, f->odu,
                f->dip})
    if (bad_index(i)) return cpl::sed_fail(sed, SED_E_ARG, "field index out of range");
  if (f->din < 0 && f->nitrate < 0 && f->ammonium < 0)
    return cpl::sed_fail(sed, SED_E_ARG, "no nitrate, ammonium or DIN field");
  if (p->mode != CPL_AS_RUN && p->mode != CPL_AS_NAMED)
    return cpl::sed_fail(sed, SED_E_ARG, "mode must be CPL_AS_RUN or CPL_AS_NAMED");
  if ((f->detN >= 0 || f->detP >= 0) && !(p->sinking_factor != 0.0))
    return cpl::sed_fail(sed, SED_E_ARG, "sinking_factor must be nonzero");
  cpl::PelView v;
  if (int rc = cpl::pel_view(pel, &v)) {
    std::string m = std::string("pelagic handle: ") + pel_last_error(pel);
    return cpl::sed_fail(sed, rc, m.c_str());
  }
  cpl::SedStaging s;
  if (int rc = cpl::sed_staging(sed, &s)) return rc;
  if (v.ncol != s.ncol)
    return cpl::sed_fail(sed, SED_E_ARG, "the handles' grids differ in inum*jnum");
  if (v.device != s.device)
    return cpl::sed_fail(sed, SED_E_ARG, "the handles are on different devices");
  const size_t nc = (size_t)s.ncol;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; return r == cudaSuccess; };
  // the pelagic handle's pending work (a pel_step) before the reads
  cudaEvent_t ev = nullptr;
  ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  if (e == cudaSuccess) {
    ok(cudaEventRecord(ev, v.stream));
    ok(cudaStreamWaitEvent(s.stream, ev, 0));
  }
  if (ev) cudaEventDestroy(ev);
  Timing tm;
  if (stats) tm.init(&e, s.stream);
  tm.mark(0);
  ok(cudaMemcpyAsync(s.temperature, temperature, nc * sizeof(double), cudaMemcpyHostToDevice,
                     s.stream));
  if (velocity_in)
    ok(cudaMemcpyAsync(s.velocity, velocity_in, (size_t)NPART * nc * sizeof(double),
                       cudaMemcpyHostToDevice, s.stream));
  else
    ok(cudaMemsetAsync(s.velocity, 0, (size_t)NPART * nc * sizeof(double), s.stream));
  double* d_depth = s.spare;
  double* d_tke = s.spare + nc;
  if (water_depth)
    ok(cudaMemcpyAsync(d_depth, water_depth, nc * sizeof(double), cudaMemcpyHostToDevice,
                       s.stream));
  if (tke)
    ok(cudaMemcpyAsync(d_tke, tke, nc * sizeof(double), cudaMemcpyHostToDevice, s.stream));
  if (e != cudaSuccess) {
    std::string m = std::string("coupling copies: ") + cudaGetErrorString(e);
    return cpl::sed_fail(sed, SED_E_CUDA, m.c_str());
  }
  const Forward a = make_forward(p, f, water_depth != nullptr, tke != nullptr);
  ForwardBufs fb{v.state, s.ncol, v.K, d_depth, d_tke, s.surface, s.velocity};
  const int threads = 256;
  long long blocks = ((long long)nc + threads - 1) / threads;
  const long long cap = (long long)(s.sms > 0 ? s.sms : 1) * 8;
  if (blocks > cap) blocks = cap;
  tm.mark(1);
  if (v.fp64)
    k_pelagic_soil<double><<<(int)blocks, threads, 0, s.stream>>>(a, fb);
  else
    k_pelagic_soil<float><<<(int)blocks, threads, 0, s.stream>>>(a, fb);
  e = cudaGetLastError();
  tm.mark(2);
  if (e != cudaSuccess) {
    std::string m = std::string("coupling kernel launch: ") + cudaGetErrorString(e);
    return cpl::sed_fail(sed, SED_E_CUDA, m.c_str());
  }
  cpl::sed_count_launch(sed);
  const unsigned mask = forward_rows(a);
  const int before = cpl::sed_launches(sed);
  if (int rc = cpl::sed_assemble_staged(sed, mask)) return rc;
  const int assembly = cpl::sed_launches(sed) - before;
  if (surface_out)
    ok(cudaMemcpyAsync(surface_out, s.surface, (size_t)NTR * nc * sizeof(double),
                       cudaMemcpyDeviceToHost, s.stream));
  if (velocity_out) {
    ok(cudaMemsetAsync(s.velocity + (size_t)NPART * nc, 0, (size_t)(NTR - NPART) * nc *
                       sizeof(double), s.stream));
    ok(cudaMemcpyAsync(velocity_out, s.velocity, (size_t)NTR * nc * sizeof(double),
                       cudaMemcpyDeviceToHost, s.stream));
  }
  tm.mark(3);
  ok(cudaStreamSynchronize(s.stream));
  if (e != cudaSuccess) {
    std::string m = std::string("coupling read-back: ") + cudaGetErrorString(e);
    return cpl::sed_fail(sed, SED_E_CUDA, m.c_str());
  }
  if (stats) {
    stats->gpu_launches = 1 + assembly;
    stats->columns = (long long)nc;
    stats->kernel_ms = tm.ms(1, 2);
    stats->device_ms = tm.ms(0, 3);
  }
  if (present_out)
    for (int n = 0; n < NTR; n++) present_out[n] = (mask >> n) & 1u;
  return SED_OK;
}

}  // extern "C"
