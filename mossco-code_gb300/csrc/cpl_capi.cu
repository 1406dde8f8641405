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

namespace {

constexpr int NTR = SED_NTR;
constexpr int NPART = 6;   // particulate tracers lead the sediment's order
// sediment tracer rows (sed_tracer_name)
constexpr int kLabC = 0, kSemC = 1, kLabN = 2, kSemN = 3, kLabP = 4, kOxy = 6, kNit = 7,
              kAmm = 8, kOdu = 9, kPho = 10;

// Per-launch constants are formed on the host in IEEE double, with the
// same operations and rounding the Fortran expressions give them; the
// kernel keeps only the per-column arithmetic (GB300's FP64 rate is a small
// fraction of its FP32 rate, and the FP64 divisions bound this kernel).
struct Args {
  const void* state;
  int ncol, K;
  int detN, detC, detP, din, nit, amm, oxy, odu;
  double sf, ncl, ncs, cN, cP, htke, crit;
  double hsd2;        // half_sedimentation_depth**2
  double sfmin_sf;    // sinking_factor_min/sinking_factor
  double c16N;        // 1.0d0/16.0d0 * convertN
  double c05N;        // convertN*0.5d0
  int as_named;
  int crit_on;        // detC present and 1e-3 < critical_detritus < 9e9
  const double* depth;  // null: no water depth, or half_sedimentation_depth <= 1e-3
  const double* tke;    // null: no turbulence field, or half_sedimentation_tke >= 9e9
  double* surface;      // [NTR][ncol]
  double* velocity;     // [NTR][ncol]
};

// Fortran max(0.0, x) of the connector's oxygen split (:823-844)
__device__ __forceinline__ double pos(double x) { return x > 0.0 ? x : 0.0; }

template <typename real>
__global__ void k_pelagic_soil(Args a) {
  const real* st = static_cast<const real*>(a.state);
  const size_t layer = (size_t)a.K * a.ncol;  // one tracer's block
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < a.ncol;
       col += gridDim.x * blockDim.x) {
    auto B = [&](int n) { return (double)st[(size_t)n * layer + col]; };
    double S[NTR];
    for (int n = 0; n < NTR; n++) S[n] = 0.0;
    double* V = a.velocity;
    // ---- detritus (:1018-1236 factors, :1243-1646 fields)
    if (a.detN >= 0 || a.detP >= 0) {
      double fenv = 1.0;
      if (a.depth) {   // 1.0 * d**2 is d**2 exactly
        const double d2 = a.depth[col] * a.depth[col];
        fenv = d2 / (d2 + a.hsd2);
      }
      if (a.tke) fenv = fenv * a.htke / (a.tke[col] + a.htke);
      fenv = fenv + a.sfmin_sf;
      if (a.crit_on) {
        const double t = B(a.detC) / a.crit;
        const double t2 = t * t;
        fenv = fenv * 1.0 / (1.0 + t2 * t2);
      }
      const double w = a.sf * fenv;
      if (a.detN >= 0) {
        const double N = B(a.detN);
        if (a.as_named) {
          double CN = 106.0 / 16.0;
          if (a.detC >= 0) CN = B(a.detC) / ((double)1e-5f + N);
          double fl = (1.0 - a.ncs * CN) / (a.ncl - a.ncs);
          double rl = fl * a.ncl;
          if (fl > CN) { fl = CN; rl = 1.0; }
          if (fl < 0.0) { fl = 0.0; rl = 0.0; }
          const double fs = CN - fl;
          const double rs = 1.0 - rl;
          S[kLabC] = fl * a.cN * N;
          S[kSemC] = fs * a.cN * N;
          S[kLabN] = rl * a.cN * N;
          S[kSemN] = rs * a.cN * N;
          for (int n = kLabC; n <= kSemN; n++) V[(size_t)n * a.ncol + col] = w * N;
        } else {
          for (int n = kLabC; n <= kSemN; n++) S[n] = w * N;
        }
        S[kLabP] = a.c16N * N;
        V[(size_t)kLabP * a.ncol + col] = w * N;
      }
      if (a.detP >= 0) S[kLabP] = B(a.detP);
    }
    // ---- oxygen and its deficit (:801-866)
    if (a.oxy >= 0 && a.odu >= 0) {
      S[kOxy] = B(a.oxy);
      S[kOdu] = B(a.odu);
    } else if (a.odu >= 0) {
      const double x = B(a.odu);
      S[kOxy] = pos(-x);
      S[kOdu] = pos(x);
    } else if (a.oxy >= 0) {
      S[kOxy] = B(a.oxy);
    }
    // ---- dissolved nitrogen and phosphate (:1648-2110)
    const bool hN = a.nit >= 0, hA = a.amm >= 0, hD = a.din >= 0;
    const double Nt = hN ? B(a.nit) : 0.0;
    const double A = hA ? B(a.amm) : 0.0;
    const double D = hD ? B(a.din) : 0.0;
    S[kAmm] = hA ? a.cN * A
            : (hD && hN) ? a.cN * (D - Nt)
            : hD ? a.c05N * D
            : a.cN * Nt;
    S[kNit] = hN ? a.cN * Nt
            : (hA && hD) ? a.cN * (D - A)
            : hD ? a.c05N * D
            : a.cN * A;
    const double din = hD ? D : (hA && hN) ? Nt + A : hA ? 2 * A : 2 * Nt;
    S[kPho] = a.cP * (a.c16N * din);
    for (int n = 0; n < NTR; n++) a.surface[(size_t)n * a.ncol + col] = S[n];
  }
}

// ---- the reverse direction: soil upward fluxes into the pelagic bottom
// fluxes (soil_pelagic_connector.F90:179-965)

struct SoilArgs {
  const double* fluxes;  // the sediment's [NTR][ncol], downward positive
  void* bfl;             // the pelagic handle's [PEL_NTR][ncol], its precision
  int ncol;
  int nit, amm, din, dip, oxy, odu, detN, detC, detP;  // pelagic rows, -1 absent
  double cN, cP;
  double dinc, dipc;     // dinflux_const/(86400.0*365.0), dipflux_const/(...)
};

template <typename real>
__global__ void k_soil_pelagic(SoilArgs a) {
  real* b = static_cast<real*>(a.bfl);
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < a.ncol;
       col += gridDim.x * blockDim.x) {
    // the soil's export: upward flux = -fluxes(:,:,n) (:1808-1815)
    auto U = [&](int n) { return -a.fluxes[(size_t)n * a.ncol + col]; };
    auto W = [&](int row, double v) { b[(size_t)row * a.ncol + col] = (real)v; };
    // each soil flux is read only when a field that needs it is present
    if (a.nit >= 0) W(a.nit, U(kNit));                          // :352-356
    if (a.amm >= 0) W(a.amm, a.cN * U(kAmm));                   // :408-412
    if (a.din >= 0) W(a.din, (U(kAmm) + U(kNit) + a.dinc) * a.cN);  // :467-473
    if (a.dip >= 0) W(a.dip, a.cP * (U(kPho) + a.dipc));        // :528-534
    if (a.odu >= 0 && a.oxy >= 0) {                             // :643-667
      W(a.odu, U(kOdu));
      W(a.oxy, U(kOxy));
    } else if (a.odu >= 0) {
      W(a.odu, U(kOdu) - U(kOxy));
    } else if (a.oxy >= 0) {
      W(a.oxy, U(kOxy) - U(kOdu));
    }
    // detritus: zero, then every soil flux the Run's pattern matches, in
    // ESMF's alphabetical item order (:734-960)
    if (a.detN >= 0) W(a.detN, 0.0 + U(kLabN) + U(kSemN));
    if (a.detC >= 0) W(a.detC, 0.0 + U(kLabC) + U(kSemC));
    if (a.detP >= 0) W(a.detP, 0.0);
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
  SoilArgs a{};
  a.fluxes = fl;
  a.bfl = bfl;
  a.ncol = s.ncol;
  a.nit = f->nitrate; a.amm = f->ammonium; a.din = f->din; a.dip = f->dip;
  a.oxy = f->oxygen; a.odu = f->odu; a.detN = f->detN; a.detC = f->detC; a.detP = f->detP;
  a.cN = p->convertN;
  a.cP = p->convertP;
  // (86400.0*365.0) is a default-real product, 31536000 exactly
  const double year = (double)(86400.0f * 365.0f);
  a.dinc = p->dinflux_const / year;
  a.dipc = p->dipflux_const / year;
  const int threads = 256;
  long long blocks = ((long long)nc + threads - 1) / threads;
  const long long cap = (long long)(s.sms > 0 ? s.sms : 1) * 8;
  if (blocks > cap) blocks = cap;
  tm.mark(0);
  tm.mark(1);
  if (e == cudaSuccess) {
    if (fp64)
      k_soil_pelagic<double><<<(int)blocks, threads, 0, pst>>>(a);
    else
      k_soil_pelagic<float><<<(int)blocks, threads, 0, pst>>>(a);
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
  Args a{};
  a.state = v.state;
  a.ncol = s.ncol;
  a.K = v.K;
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
  // the Run's guards on the namelist values (:1150, :1181, :1215), with
  // its default-real literals
  a.crit_on = f->detC >= 0 && p->critical_detritus > (double)1e-3f &&
              p->critical_detritus < (double)9e9f;
  a.depth = water_depth && p->half_sedimentation_depth > (double)1e-3f ? d_depth : nullptr;
  a.tke = tke && p->half_sedimentation_tke < (double)9e9f ? d_tke : nullptr;
  a.surface = s.surface;
  a.velocity = s.velocity;
  const int threads = 256;
  long long blocks = ((long long)nc + threads - 1) / threads;
  const long long cap = (long long)(s.sms > 0 ? s.sms : 1) * 8;
  if (blocks > cap) blocks = cap;
  tm.mark(1);
  if (v.fp64)
    k_pelagic_soil<double><<<(int)blocks, threads, 0, s.stream>>>(a);
  else
    k_pelagic_soil<float><<<(int)blocks, threads, 0, s.stream>>>(a);
  e = cudaGetLastError();
  tm.mark(2);
  if (e != cudaSuccess) {
    std::string m = std::string("coupling kernel launch: ") + cudaGetErrorString(e);
    return cpl::sed_fail(sed, SED_E_CUDA, m.c_str());
  }
  cpl::sed_count_launch(sed);
  unsigned mask = (1u << kNit) | (1u << kAmm) | (1u << kPho);
  if (f->detN >= 0) mask |= (1u << kLabC) | (1u << kSemC) | (1u << kLabN) | (1u << kSemN) |
                           (1u << kLabP);
  if (f->detP >= 0) mask |= 1u << kLabP;
  if (f->oxygen >= 0 || f->odu >= 0) mask |= 1u << kOxy;
  if (f->odu >= 0) mask |= 1u << kOdu;
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
