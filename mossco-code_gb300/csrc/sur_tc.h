// sur_tc.h -- the surrogate's fused inference kernel on the tcgen05 tensor
// cores (sur_tc.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

struct sed_surrogate;

namespace sur {

// The network fits the fused kernel: input width (padded) a multiple of 64
// up to 384, hidden layers of 256, output width a multiple of 128 up to 512,
// and the driver's tensor-map encoder is available.
bool tc_supported(const sed_surrogate* s);
// y[m][pout_last] (FP32) = the network on x[m][pin_0] (BF16), m a multiple
// of 128.  *err (device) receives a nonzero code if the kernel gave up
// waiting on one of its barriers (it then leaves y incomplete).
cudaError_t infer_tc(sed_surrogate* s, const __nv_bfloat16* x, float* y, int m, int* err,
                     cudaStream_t st);

}  // namespace sur
