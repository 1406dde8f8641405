// sed_kernels_f64.cu -- instantiates the column kernels for double state
// (the bioturbation profile-3 set lives in sed_kernels_f64_bio3.cu).
#include "sed_kernels.cuh"

namespace sed {
SED_VARIANT(extern, double, true)
SED_INSTANTIATE(double)
}  // namespace sed
