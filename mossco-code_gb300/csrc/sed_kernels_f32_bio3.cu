// sed_kernels_f32_bio3.cu -- float tile kernels with the TOC-dependent
// bioturbation of profile 3, compiled apart so the build runs in parallel.
#include "sed_kernels.cuh"

namespace sed {
SED_VARIANT(, float, true)
}  // namespace sed
