// sur_kernels.h -- launchers of the surrogate's tensor-core kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sur {

// EPI_GELU: GELU(acc + bias) to BF16 only (inference: no pre-activations kept)
enum : int { EPI_BIAS_GELU = 0, EPI_BIAS = 1, EPI_F32 = 2, EPI_GELU_BWD = 3, EPI_GELU = 4 };

// C[M x N] = A[M x K] . B[N x K]^T; M % 128 == 0, N % 64 == 0, K % 32 == 0
cudaError_t gemm_nt(int epi, const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N,
                    int K, const float* bias, float* out_f32, __nv_bfloat16* out_bf16,
                    const float* zprev, int ld_out, cudaStream_t st);
cudaError_t transpose_bf16(const __nv_bfloat16* in, __nv_bfloat16* out, int rows, int cols,
                           cudaStream_t st);
cudaError_t mse(const float* yhat, const __nv_bfloat16* y, const float* mask, int M, int N,
                int m_valid, float inv_count, __nv_bfloat16* dy, float* loss,
                cudaStream_t st);
// db[N] = column sums of dz[M][N] in a fixed order; part: bias_grad_parts() x N
cudaError_t bias_grad(const __nv_bfloat16* dz, int M, int N, float* part, float* db,
                      cudaStream_t st);
int bias_grad_parts();
// Adam over several parameter arrays in one launch: segment q is n = start[q+1]
// - start[q] elements of w, m, v, g, with the BF16 copy wb (and its
// transpose wbt, rows x cols) refreshed when wb is set
constexpr int kAdamMaxSeg = 16;
struct AdamSeg {
  float *w, *m, *v;
  const float* g;
  __nv_bfloat16 *wb, *wbt;
  int rows, cols;
};
struct AdamSet {
  AdamSeg seg[kAdamMaxSeg];
  long long start[kAdamMaxSeg + 1];
  int n;
};
cudaError_t adam_all(const AdamSet& set, float lr, float b1, float b2, float eps, int step,
                     int sms, cudaStream_t st);
cudaError_t to_bf16(const float* w, int rows, int cols, __nv_bfloat16* wb,
                    __nv_bfloat16* wbt, cudaStream_t st);

}  // namespace sur
