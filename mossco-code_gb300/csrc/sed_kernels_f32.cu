// sed_kernels_f32.cu -- instantiates the column kernels for float state
// (the bioturbation profile-3 set lives in sed_kernels_f32_bio3.cu) and the
// dispatchers of the warp-direct kernels.
#include "sed_kernels.cuh"

namespace sed {
SED_VARIANT(extern, float, true)
SED_WARP_VARIANT(extern, true)
SED_INSTANTIATE(float)

cudaError_t launch_column_warp(const ColumnArgs<float>& a, const Params<float>& p, int lpl,
                               bool bc4, int kind, int blocks, int threads, cudaStream_t st) {
  const bool b3 = p.bio3 != 0;
  if (lpl == 1) {
    if (bc4) return b3 ? launch_warp_k<1, true, true>(a, p, kind, blocks, threads, st)
                       : launch_warp_k<1, true, false>(a, p, kind, blocks, threads, st);
    return b3 ? launch_warp_k<1, false, true>(a, p, kind, blocks, threads, st)
              : launch_warp_k<1, false, false>(a, p, kind, blocks, threads, st);
  }
  if (bc4) return b3 ? launch_warp_k<2, true, true>(a, p, kind, blocks, threads, st)
                     : launch_warp_k<2, true, false>(a, p, kind, blocks, threads, st);
  return b3 ? launch_warp_k<2, false, true>(a, p, kind, blocks, threads, st)
            : launch_warp_k<2, false, false>(a, p, kind, blocks, threads, st);
}

int column_warp_blocks_per_sm(int lpl, bool bc4, int kind, int threads, bool bio3) {
  if (lpl == 1) {
    if (bc4) return bio3 ? warp_occupancy_k<1, true, true>(kind, threads)
                         : warp_occupancy_k<1, true, false>(kind, threads);
    return bio3 ? warp_occupancy_k<1, false, true>(kind, threads)
                : warp_occupancy_k<1, false, false>(kind, threads);
  }
  if (bc4) return bio3 ? warp_occupancy_k<2, true, true>(kind, threads)
                       : warp_occupancy_k<2, true, false>(kind, threads);
  return bio3 ? warp_occupancy_k<2, false, true>(kind, threads)
              : warp_occupancy_k<2, false, false>(kind, threads);
}
}  // namespace sed
