// sed_kernels_warp.cu -- the warp-direct column kernels (float and double
// state), compiled apart so the build runs in parallel.
#include "sed_kernels.cuh"

namespace sed {
SED_WARP_VARIANT(, float, false)
SED_WARP_VARIANT(, double, false)
}  // namespace sed
