// cpl_internal.h -- what the pelagic -> soil coupling (cpl_capi.cu) needs
// from the two handles, whose structs live in pel_capi.cu and sed_capi.cu.
// Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include "../../include/mossco_pel.h"
#include "../../include/mossco_sed.h"

namespace cpl {

// The pelagic handle's device state [PEL_NTR][K][ncol] (FP32 or FP64) and
// the stream its steps run on.
struct PelView {
  const void* state = nullptr;
  bool fp64 = false;
  int ncol = 0, K = 0, device = 0;
  cudaStream_t stream = nullptr;
};
// SED_E_STATE (with the message on the pelagic handle) when the handle
// has no grid, or no state yet and need_state is set (state is then null).
int pel_view(pel_handle* h, PelView* v, bool need_state = true);
// The handle's bottom-flux rows [PEL_NTR][ncol] in its precision, zeroed
// and switched on when the handle had none (pel_set_forcing's
// bottom_flux); SED_E_STATE without a grid.
int pel_bottom_flux(pel_handle* h, void** bfl);

// The sediment handle's boundary staging rows on the device, allocated on
// first use: temperature [ncol], surface [SED_NTR][ncol], velocity
// [SED_NTR][ncol], then two spare rows [ncol] (water depth, tke).
struct SedStaging {
  double* temperature = nullptr;
  double* surface = nullptr;
  double* velocity = nullptr;
  double* spare = nullptr;
  int ncol = 0, device = 0, sms = 0;
  cudaStream_t stream = nullptr;
};
int sed_staging(sed_handle* h, SedStaging* s);
// the handle's fluxes [SED_NTR][ncol] (FP64, downward positive) with the
// surface fluxes of its last step scattered into the dissolved rows, as
// sed_get_fluxes returns them; SED_E_STATE before any forcing
int sed_surface_fluxes(sed_handle* h, const double** fluxes);
// get_boundary_conditions on the staged rows: bdys / fluxes of the tracers
// in present_mask, then the forcing rows of the next step.
int sed_assemble_staged(sed_handle* h, unsigned present_mask);
// records the message on the sediment handle and returns code
int sed_fail(sed_handle* h, int code, const char* msg);
void sed_count_launch(sed_handle* h);
// kernels launched on the handle so far
int sed_launches(const sed_handle* h);

}  // namespace cpl
