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
// of 128; with nrows (device), only the 128-row tiles holding the first
// min(m, *nrows) rows.  *err (device) receives a nonzero code if the kernel
// gave up waiting on one of its barriers (it then leaves y incomplete).
cudaError_t infer_tc(sed_surrogate* s, const __nv_bfloat16* x, float* y, int m, int* err,
                     cudaStream_t st, const unsigned* nrows = nullptr);

// The training products on the tcgen05 tensor cores: C[M x N] = A[M x K] .
// B[N x K]^T with the epilogues of sur_kernels.h (EPI_*), M and N multiples
// of 128, K of 64, ld_out a multiple of 8 and at least N.  EPI_F32 with
// ld_out == N splits K over the SMs when work (FP32, work_floats) holds the
// partial tiles, which are then added in a fixed order.  *err (device)
// receives a nonzero code if the kernel gave up waiting on a barrier.
bool gemm_tc_supported();
cudaError_t gemm_tc(int epi, const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K,
                    const float* bias, float* out_f32, __nv_bfloat16* out_bf16,
                    const float* zprev, int ld_out, float* work, size_t work_floats, int* err,
                    cudaStream_t st);

}  // namespace sur
