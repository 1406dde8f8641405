// sed_kernels_warp_bio3.cu -- the warp-direct column kernels with the
// TOC-dependent bioturbation of profile 3.
#include "sed_kernels.cuh"

namespace sed {
SED_WARP_VARIANT(, float, true)
SED_WARP_VARIANT(, double, true)
}  // namespace sed
