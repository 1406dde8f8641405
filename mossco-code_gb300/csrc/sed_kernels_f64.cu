// sed_kernels_f64.cu -- instantiates the column kernels for double state (the
// bioturbation profile-3 set and the warp-direct kernels live in their own
// translation units, sed_kernels_f64_bio3.cu and sed_kernels_warp*.cu).
#include "sed_kernels.cuh"

namespace sed {
SED_VARIANT(extern, double, true)
SED_WARP_VARIANT(extern, double, false)
SED_WARP_VARIANT(extern, double, true)
SED_WARP_ENS_VARIANT(extern, double, false)
SED_WARP_ENS_VARIANT(extern, double, true)
SED_DEEP_VARIANT(extern, double, false)
SED_DEEP_VARIANT(extern, double, true)
SED_INSTANTIATE(double)
}  // namespace sed
