// sed_kernels_f64.cu -- instantiates the column kernels for double state.
#include "sed_kernels.cuh"

namespace sed {
SED_INSTANTIATE(double)
}  // namespace sed
