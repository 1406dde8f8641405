// sed_kernels_deep_f32_bio3.cu -- the column kernels of the deepest depth
// class (64..127 active layers, four layers per lane of a warp), float state
// with the TOC-dependent bioturbation of profile 3, compiled apart so the
// build runs in parallel.
#include "sed_kernels.cuh"

namespace sed {
SED_DEEP_VARIANT(, float, true)
}  // namespace sed
