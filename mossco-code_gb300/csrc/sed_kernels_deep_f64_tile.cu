// sed_kernels_deep_f64_tile.cu -- the tile kernels of the deepest depth class
// (64..127 active layers, four layers per lane of a warp), double state,
// compiled apart so the build runs in parallel.
#include "sed_kernels.cuh"

namespace sed {
SED_DEEP_TILE_VARIANT(, double, false)
}  // namespace sed
