// sed_kernels_warp_ens.cu -- the warp-direct column kernels with a
// parameter set per column (ensembles), compiled apart so the build runs in
// parallel.
#include "sed_kernels.cuh"

namespace sed {
SED_WARP_ENS_VARIANT(, float, false)
SED_WARP_ENS_VARIANT(, double, false)
}  // namespace sed
