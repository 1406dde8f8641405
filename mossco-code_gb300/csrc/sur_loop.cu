// sur_loop.cu -- kernels between the solver's slot layout and the
// surrogate's row layout.
//
// Features of a column (row r of the MLP batch, the column in slot list[r]),
// tracer-major:
//   x[n*K + k]   = (log(max(C[n][k], 0) + c0[n]) - mu_x) / sd_x     n < 11, k < K
//   x[11*K + f]  = (force[f] - mu_x) / sd_x                          f < 13
// (the 13 per-column forcing rows of the solver: bioturbation x f_T, the
// molecular multiplier and the 11 surface values), zero in padded rows and
// columns.  The network predicts the standardised change of log(C + c0)
// over one coupling step; the surrogate step's residual kernel forms the
// proposed state from it.  The features kernel is a 32 x 32 tiled transpose
// (row tiles on blockIdx.x, feature tiles on blockIdx.y).
//
// Training rows (k_collect): for every column whose plain step took more
// than one attempt (its first, whole-step attempt was rejected: the columns
// the surrogate step hands to the network), the unstandardised features
// x = [log(max(C0, 0) + c0) (11 K), forcing (13)] and the target
// y = log(max(C1, 0) + c0) - log(max(C0, 0) + c0) (11 K) in FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "sed_device.cuh"
#include "sur_loop.h"

namespace sur {

using sed::NFORCE;
using sed::NTR;

__global__ void k_features(const float* __restrict__ conc, const float* __restrict__ force,
                           const float* __restrict__ norm, const int* __restrict__ list,
                           int nrows, int K, int kmax, int nslot, int rows, int nin, int pin,
                           __nv_bfloat16* __restrict__ x) {
  __shared__ float tile[32][33];
  const int f0 = blockIdx.y * 32, r0 = blockIdx.x * 32;
  const float* c0 = norm;
  const float* mu = norm + NTR;
  const float* sd = mu + nin;
  const int nstate = NTR * K;
  // read: feature rows f, the tile's columns along threadIdx.x
  const int r = r0 + threadIdx.x;
  const int slot = r < nrows ? list[r] : -1;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int f = f0 + y;
    float v = 0.0f;
    if (slot >= 0 && f < nin) {
      if (f < nstate) {
        const int n = f / K, k = f - n * K;
        v = (logf(fmaxf(conc[((size_t)n * kmax + k) * nslot + slot], 0.0f) + c0[n]) - mu[f]) /
            sd[f];
      } else {
        v = (force[(size_t)(f - nstate) * nslot + slot] - mu[f]) / sd[f];
      }
    }
    tile[y][threadIdx.x] = v;
  }
  __syncthreads();
  // write: rows, features contiguous
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int rr = r0 + y, f = f0 + threadIdx.x;
    if (rr < rows && f < pin) x[(size_t)rr * pin + f] = __float2bfloat16(tile[threadIdx.x][y]);
  }
}

// One warp per slot of the class range [slot0, slot0 + nslots).
__global__ void k_collect(const float* __restrict__ conc0, const float* __restrict__ conc1,
                          const float* __restrict__ force, const int* __restrict__ kact,
                          const int* __restrict__ nsub, const float* __restrict__ c0, int K,
                          int kmax, int nslot, int slot0, int nslots, float* __restrict__ x,
                          int pitch_x, float* __restrict__ y, int pitch_y,
                          unsigned long long* __restrict__ count, long long capacity) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < nslots; j += warps) {
    const int slot = slot0 + j;
    if (kact[slot] != K || nsub[slot] <= 1) continue;
    unsigned long long row = 0;
    if (lane == 0) row = atomicAdd(count, 1ull);
    row = __shfl_sync(0xffffffffu, row, 0);
    if ((long long)row >= capacity) continue;
    float* xr = x + row * (size_t)pitch_x;
    float* yr = y + row * (size_t)pitch_y;
    for (int f = lane; f < NTR * K; f += 32) {
      const int n = f / K, k = f - n * K;
      const size_t i = ((size_t)n * kmax + k) * nslot + slot;
      const float u0 = logf(fmaxf(conc0[i], 0.0f) + c0[n]);
      const float u1 = logf(fmaxf(conc1[i], 0.0f) + c0[n]);
      xr[f] = u0;
      yr[f] = u1 - u0;
    }
    if (lane < NFORCE) xr[NTR * K + lane] = force[(size_t)lane * nslot + slot];
  }
}

cudaError_t features(const float* conc, const float* force, const float* norm, const int* list,
                     int nrows, int K, int kmax, int nslot, int rows, int nin, int pin,
                     __nv_bfloat16* x, cudaStream_t st) {
  // rows on x (up to 2^31 - 1 blocks), features on y (a few dozen)
  dim3 grid((rows + 31) / 32, (pin + 31) / 32);
  k_features<<<grid, dim3(32, 8), 0, st>>>(conc, force, norm, list, nrows, K, kmax, nslot, rows,
                                           nin, pin, x);
  return cudaGetLastError();
}

cudaError_t collect(const float* conc0, const float* conc1, const float* force, const int* kact,
                    const int* nsub, const float* c0, int K, int kmax, int nslot, int slot0,
                    int nslots, float* x, int pitch_x, float* y, int pitch_y,
                    unsigned long long* count, long long capacity, int sms, cudaStream_t st) {
  if (nslots <= 0) return cudaSuccess;
  int blocks = (nslots + 7) / 8;
  if (blocks > sms * 8) blocks = sms * 8;
  k_collect<<<blocks, 256, 0, st>>>(conc0, conc1, force, kact, nsub, c0, K, kmax, nslot, slot0,
                                    nslots, x, pitch_x, y, pitch_y, count, capacity);
  return cudaGetLastError();
}

}  // namespace sur
