// sed_kernels_f32.cu -- instantiates the column kernels for float state
// (the bioturbation profile-3 set lives in sed_kernels_f32_bio3.cu).
#include "sed_kernels.cuh"

namespace sed {
SED_VARIANT(extern, float, true)
SED_INSTANTIATE(float)
}  // namespace sed
