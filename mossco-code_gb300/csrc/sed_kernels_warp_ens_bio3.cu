// sed_kernels_warp_ens_bio3.cu -- the warp-direct column kernels with a
// parameter set per column and the TOC-dependent bioturbation of profile 3.
#include "sed_kernels.cuh"

namespace sed {
SED_WARP_ENS_VARIANT(, float, true)
SED_WARP_ENS_VARIANT(, double, true)
}  // namespace sed
