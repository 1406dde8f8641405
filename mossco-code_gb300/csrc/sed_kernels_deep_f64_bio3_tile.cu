// sed_kernels_deep_f64_bio3_tile.cu -- the tile kernels of the deepest depth
// class (64..127 active layers, four layers per lane of a warp), double state
// with the TOC-dependent bioturbation of profile 3, compiled apart so the
// build runs in parallel.
#include "sed_kernels.cuh"

namespace sed {
SED_DEEP_TILE_VARIANT(, double, true)
}  // namespace sed
