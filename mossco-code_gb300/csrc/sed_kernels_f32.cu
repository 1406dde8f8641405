// sed_kernels_f32.cu -- instantiates the column kernels for float state (the
// bioturbation profile-3 set and the warp-direct kernels live in their own
// translation units, sed_kernels_f32_bio3.cu and sed_kernels_warp*.cu).
#include "sed_kernels.cuh"

namespace sed {
SED_VARIANT(extern, float, true)
SED_WARP_VARIANT(extern, float, false)
SED_WARP_VARIANT(extern, float, true)
SED_WARP_ENS_VARIANT(extern, float, false)
SED_WARP_ENS_VARIANT(extern, float, true)
SED_DEEP_VARIANT(extern, float, false)
SED_DEEP_VARIANT(extern, float, true)
SED_INSTANTIATE(float)
}  // namespace sed
