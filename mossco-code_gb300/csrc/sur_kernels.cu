// sur_kernels.cu -- kernels of the column-increment surrogate (an MLP with
// GELU hidden layers): BF16 tensor-core GEMM with fused epilogues, GELU
// backward, bias gradients, transposes, Adam, and the MSE loss.
//
// GEMM: C[M x N] = A[M x K] . B[N x K]^T, A and B row-major BF16 with the
// reduction dimension contiguous, FP32 accumulation in mma.sync m16n8k16
// fragments.  Every product of the network is written in this form:
//   forward   Z = X W^T            (A = X,      B = W)
//   backward  dX = dZ W            (A = dZ,     B = W^T)
//   weights   dW = dZ^T X          (A = dZ^T,   B = X^T)
// Block tile 128 x 64, K step 32, 4 warps of 64 x 32, cp.async double
// buffering, ldmatrix fragment loads.  M must be a multiple of 128, N of 64
// and K of 32 (the host pads feature and batch dimensions).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sur_gelu.cuh"
#include "sur_kernels.h"

namespace sur {

constexpr int BM = 128, BN = 64, BK = 32;
constexpr int LDS = BK + 8;  // smem row pitch (bf16), 80 bytes: conflict-free ldmatrix

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }

__device__ __forceinline__ void ldmatrix_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2,
                                            uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldmatrix_x2(uint32_t& r0, uint32_t& r1, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Epilogues.  EPI_BIAS_GELU: Z = acc + bias -> store Z (fp32) and GELU(Z)
// (bf16).  EPI_GELU: GELU(acc + bias) (bf16 only).  EPI_BIAS: out = acc +
// bias (fp32).
// EPI_F32: out = acc (fp32).  EPI_GELU_BWD: out = acc * GELU'(Zprev)
// (bf16), the gradient through the previous layer's activation.
template <int EPI>
__global__ void __launch_bounds__(128)
k_gemm_nt(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ B,
          int M, int N, int K, const float* __restrict__ bias,
          float* __restrict__ out_f32, __nv_bfloat16* __restrict__ out_bf16,
          const float* __restrict__ zprev, int ld_out) {
  __shared__ __align__(16) __nv_bfloat16 sA[2][BM * LDS];
  __shared__ __align__(16) __nv_bfloat16 sB[2][BN * LDS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int wm = (warp >> 1) * 64, wn = (warp & 1) * 32;

  auto load_tile = [&](int stage, int k0) {
    // A: 128 rows x 32 cols = 512 chunks of 16 B, 4 per thread
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int c = tid + i * 128;
      const int r = c >> 2, q = c & 3;
      cp_async16(&sA[stage][r * LDS + q * 8], A + (size_t)(m0 + r) * K + k0 + q * 8);
    }
    // B: 64 rows x 32 cols = 256 chunks, 2 per thread
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const int c = tid + i * 128;
      const int r = c >> 2, q = c & 3;
      cp_async16(&sB[stage][r * LDS + q * 8], B + (size_t)(n0 + r) * K + k0 + q * 8);
    }
    cp_async_commit();
  };

  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int v = 0; v < 4; v++) acc[i][j][v] = 0.0f;

  const int nk = K / BK;
  load_tile(0, 0);
  for (int kt = 0; kt < nk; kt++) {
    const int st = kt & 1;
    if (kt + 1 < nk) {
      load_tile(st ^ 1, (kt + 1) * BK);
      cp_async_wait1();
    } else {
      cp_async_wait0();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[4][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        // rows wm + 16 i + (lane % 16), cols kk + 8 (lane / 16)
        const __nv_bfloat16* p = &sA[st][(wm + i * 16 + (lane & 15)) * LDS + kk + (lane >> 4) * 8];
        ldmatrix_x4(af[i][0], af[i][1], af[i][2], af[i][3], p);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        // rows (n) wn + 8 j + (lane % 8), cols kk + 8 ((lane / 8) % 2)
        const __nv_bfloat16* p = &sB[st][(wn + j * 8 + (lane & 7)) * LDS + kk + ((lane >> 3) & 1) * 8];
        ldmatrix_x2(bf[j][0], bf[j][1], p);
      }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }

  // epilogue: fragment (i, j) covers rows wm+16i+g(+8), cols wn+8j+2t(+1)
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int row = m0 + wm + i * 16 + g + h * 8;
        const int col = n0 + wn + j * 8 + 2 * t;
        float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
        const size_t o = (size_t)row * ld_out + col;
        if (EPI == EPI_BIAS_GELU) {
          v0 += bias[col];
          v1 += bias[col + 1];
          *reinterpret_cast<float2*>(out_f32 + o) = make_float2(v0, v1);
          *reinterpret_cast<__nv_bfloat162*>(out_bf16 + o) =
              __floats2bfloat162_rn(gelu(v0), gelu(v1));
        } else if (EPI == EPI_GELU) {
          v0 += bias[col];
          v1 += bias[col + 1];
          *reinterpret_cast<__nv_bfloat162*>(out_bf16 + o) =
              __floats2bfloat162_rn(gelu(v0), gelu(v1));
        } else if (EPI == EPI_BIAS) {
          v0 += bias[col];
          v1 += bias[col + 1];
          *reinterpret_cast<float2*>(out_f32 + o) = make_float2(v0, v1);
        } else if (EPI == EPI_F32) {
          *reinterpret_cast<float2*>(out_f32 + o) = make_float2(v0, v1);
        } else {  // EPI_GELU_BWD
          const float2 z = *reinterpret_cast<const float2*>(zprev + o);
          *reinterpret_cast<__nv_bfloat162*>(out_bf16 + o) =
              __floats2bfloat162_rn(v0 * gelu_grad(z.x), v1 * gelu_grad(z.y));
        }
      }
}

// out[c][r] = in[r][c] (bf16), 32 x 32 tiles
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ in,
                                 __nv_bfloat16* __restrict__ out, int rows, int cols) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = by + y, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[y][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = bx + y, r = by + threadIdx.x;
    if (r < rows && c < cols) out[(size_t)c * rows + r] = tile[threadIdx.x][y];
  }
}

// MSE over the valid outputs: loss = sum mask (yhat - y)^2 / count,
// dY = 2 (yhat - y) / count as bf16 (zero where masked).  Blocks walk rows,
// threads the row's columns; the squares are reduced in the block and added
// to the loss with one atomic per block.
__global__ void k_mse(const float* __restrict__ yhat, const __nv_bfloat16* __restrict__ y,
                      const float* __restrict__ mask, int M, int N, int m_valid,
                      float inv_count, __nv_bfloat16* __restrict__ dy,
                      float* __restrict__ loss) {
  __shared__ float red[32];
  float s = 0.0f;
  for (int row = blockIdx.x; row < M; row += gridDim.x) {
    const size_t o = (size_t)row * N;
    const bool valid = row < m_valid;
    for (int col = threadIdx.x; col < N; col += blockDim.x) {
      const float w = valid ? mask[col] : 0.0f;
      const float d = (yhat[o + col] - __bfloat162float(y[o + col])) * w;
      s += d * d;
      dy[o + col] = __float2bfloat16(2.0f * d * inv_count);
    }
  }
#pragma unroll
  for (int k = 16; k > 0; k >>= 1) s += __shfl_xor_sync(0xffffffffu, s, k);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = s;
  __syncthreads();
  if (warp == 0) {
    s = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0f;
#pragma unroll
    for (int k = 16; k > 0; k >>= 1) s += __shfl_xor_sync(0xffffffffu, s, k);
    if (lane == 0) atomicAdd(loss, s * inv_count);
  }
}

// db[n] = sum_m dZ[m][n]; dZ bf16 [M][N], in a fixed order so that training
// is reproducible bit for bit: block (x, y) sums rows y, y + gridDim.y, ...
// of 32 columns (8 row phases per block, reduced in order) into
// part[y][n]; k_bias_sum then adds the gridDim.y partials in order.
constexpr int kBiasRowBlocks = 64;

__global__ void k_bias_part(const __nv_bfloat16* __restrict__ dz, int M, int N,
                            float* __restrict__ part) {
  __shared__ float red[8][33];
  const int n = blockIdx.x * 32 + threadIdx.x;
  float s = 0.0f;
  if (n < N)
    for (int m = blockIdx.y * 8 + threadIdx.y; m < M; m += gridDim.y * 8)
      s += __bfloat162float(dz[(size_t)m * N + n]);
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && n < N) {
    float t = red[0][threadIdx.x];
    for (int r = 1; r < 8; r++) t += red[r][threadIdx.x];
    part[(size_t)blockIdx.y * N + n] = t;
  }
}

__global__ void k_bias_sum(const float* __restrict__ part, int N, int nparts,
                           float* __restrict__ db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float t = 0.0f;
  for (int g = 0; g < nparts; g++) t += part[(size_t)g * N + n];
  db[n] = t;
}

// Adam over several parameter arrays in one launch (every layer's weights
// and biases) on FP32 master weights, refreshing the BF16 copies W and W^T:
// element i of the concatenation belongs to the segment whose start is the
// last one <= i.
__global__ void k_adam_all(AdamSet set, float lr, float b1, float b2, float eps, float c1,
                           float c2) {
  const long long total = set.start[set.n];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    int q = 0;
    while (q + 1 < set.n && i >= set.start[q + 1]) q++;
    const AdamSeg& a = set.seg[q];
    const int j = (int)(i - set.start[q]);
    const float gi = a.g[j];
    const float mi = b1 * a.m[j] + (1.0f - b1) * gi;
    const float vi = b2 * a.v[j] + (1.0f - b2) * gi * gi;
    a.m[j] = mi;
    a.v[j] = vi;
    const float wi = a.w[j] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    a.w[j] = wi;
    if (a.wb) {
      const __nv_bfloat16 b = __float2bfloat16(wi);
      a.wb[j] = b;
      if (a.wbt) {
        const int r = j / a.cols, c = j - r * a.cols;
        a.wbt[(size_t)c * a.rows + r] = b;
      }
    }
  }
}

// BF16 copies of FP32 weights (and the transpose)
__global__ void k_to_bf16(const float* __restrict__ w, int rows, int cols,
                          __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wbt) {
  const int n = rows * cols;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const __nv_bfloat16 b = __float2bfloat16(w[i]);
    wb[i] = b;
    if (wbt) {
      const int r = i / cols, c = i - r * cols;
      wbt[(size_t)c * rows + r] = b;
    }
  }
}

// ---------------------------------------------------------------------------
cudaError_t gemm_nt(int epi, const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N,
                    int K, const float* bias, float* out_f32, __nv_bfloat16* out_bf16,
                    const float* zprev, int ld_out, cudaStream_t st) {
  if (M % BM || N % BN || K % BK) return cudaErrorInvalidValue;
  dim3 grid(N / BN, M / BM);
  switch (epi) {
    case EPI_BIAS_GELU:
      k_gemm_nt<EPI_BIAS_GELU><<<grid, 128, 0, st>>>(A, B, M, N, K, bias, out_f32, out_bf16, zprev, ld_out);
      break;
    case EPI_BIAS:
      k_gemm_nt<EPI_BIAS><<<grid, 128, 0, st>>>(A, B, M, N, K, bias, out_f32, out_bf16, zprev, ld_out);
      break;
    case EPI_GELU:
      k_gemm_nt<EPI_GELU><<<grid, 128, 0, st>>>(A, B, M, N, K, bias, out_f32, out_bf16, zprev, ld_out);
      break;
    case EPI_F32:
      k_gemm_nt<EPI_F32><<<grid, 128, 0, st>>>(A, B, M, N, K, bias, out_f32, out_bf16, zprev, ld_out);
      break;
    default:
      k_gemm_nt<EPI_GELU_BWD><<<grid, 128, 0, st>>>(A, B, M, N, K, bias, out_f32, out_bf16, zprev, ld_out);
  }
  return cudaGetLastError();
}

cudaError_t transpose_bf16(const __nv_bfloat16* in, __nv_bfloat16* out, int rows, int cols,
                           cudaStream_t st) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_bf16<<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols);
  return cudaGetLastError();
}

cudaError_t mse(const float* yhat, const __nv_bfloat16* y, const float* mask, int M, int N,
                int m_valid, float inv_count, __nv_bfloat16* dy, float* loss,
                cudaStream_t st) {
  const int blocks = M < 1024 ? M : 1024;
  k_mse<<<blocks, 128, 0, st>>>(yhat, y, mask, M, N, m_valid, inv_count, dy, loss);
  return cudaGetLastError();
}

cudaError_t bias_grad(const __nv_bfloat16* dz, int M, int N, float* part, float* db,
                      cudaStream_t st) {
  k_bias_part<<<dim3((N + 31) / 32, kBiasRowBlocks), dim3(32, 8), 0, st>>>(dz, M, N, part);
  k_bias_sum<<<(N + 127) / 128, 128, 0, st>>>(part, N, kBiasRowBlocks, db);
  return cudaGetLastError();
}

int bias_grad_parts() { return kBiasRowBlocks; }

cudaError_t adam_all(const AdamSet& set, float lr, float b1, float b2, float eps, int step,
                     int sms, cudaStream_t st) {
  if (set.n <= 0 || set.n > kAdamMaxSeg) return cudaErrorInvalidValue;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  const long long total = set.start[set.n];
  long long blocks = (total + 255) / 256;
  if (blocks > 4LL * sms) blocks = 4LL * sms;
  k_adam_all<<<(int)(blocks > 0 ? blocks : 1), 256, 0, st>>>(set, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t to_bf16(const float* w, int rows, int cols, __nv_bfloat16* wb,
                    __nv_bfloat16* wbt, cudaStream_t st) {
  int blocks = (rows * cols + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  k_to_bf16<<<blocks, 256, 0, st>>>(w, rows, cols, wb, wbt);
  return cudaGetLastError();
}

}  // namespace sur
