// sed_kernels_f64_bio3.cu -- double tile kernels with the TOC-dependent
// bioturbation of profile 3, compiled apart so the build runs in parallel.
#include "sed_kernels.cuh"

namespace sed {
SED_VARIANT(, double, true)
}  // namespace sed
