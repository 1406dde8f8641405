// sed_kernels_f32.cu -- instantiates the column kernels for float state.
#include "sed_kernels.cuh"

namespace sed {
SED_INSTANTIATE(float)
}  // namespace sed
