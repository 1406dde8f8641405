// sur_loop.cu -- kernels between the solver's slot layout and the
// surrogate's row layout.
//
// Features of a column (row `slot` of the MLP batch), tracer-major:
//   x[n*K + k]   = (log(C[n][k] + c0[n]) - mu_x) / sd_x     n < 11, k < K
//   x[11*K + f]  = (force[f] - mu_x) / sd_x                 f < 13
// (the 13 per-column forcing rows of the solver: bioturbation x f_T, the
// molecular multiplier and the 11 surface values), zero in padded columns.
// The network predicts the standardised change of log(C + c0) over one
// coupling step; the proposed state is exp(log(C + c0) + mu_d + sd_d y) - c0,
// clamped at zero.  Both kernels are 32 x 32 tiled transposes (slot tiles
// on blockIdx.x, feature tiles on blockIdx.y).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "sed_device.cuh"
#include "sur_loop.h"

namespace sur {

using sed::NFORCE;
using sed::NTR;

__global__ void k_features(const float* __restrict__ conc, const float* __restrict__ force,
                           const float* __restrict__ norm, int K, int kmax, int nslot,
                           int rows, int nin, int pin, __nv_bfloat16* __restrict__ x) {
  __shared__ float tile[32][33];
  const int f0 = blockIdx.y * 32, s0 = blockIdx.x * 32;
  const float* c0 = norm;
  const float* mu = norm + NTR;
  const float* sd = mu + nin;
  const int nstate = NTR * K;
  // read: feature rows f, slots contiguous
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int f = f0 + y, slot = s0 + threadIdx.x;
    float v = 0.0f;
    if (slot < nslot && f < nin) {
      if (f < nstate) {
        const int n = f / K, k = f - n * K;
        v = (logf(conc[((size_t)n * kmax + k) * nslot + slot] + c0[n]) - mu[f]) / sd[f];
      } else {
        v = (force[(size_t)(f - nstate) * nslot + slot] - mu[f]) / sd[f];
      }
    }
    tile[y][threadIdx.x] = v;
  }
  __syncthreads();
  // write: rows = slots, features contiguous
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int slot = s0 + y, f = f0 + threadIdx.x;
    if (slot < rows && f < pin) x[(size_t)slot * pin + f] = __float2bfloat16(tile[threadIdx.x][y]);
  }
}

__global__ void k_apply(const float* __restrict__ yhat, const float* __restrict__ conc,
                        const float* __restrict__ norm, int K, int kmax, int nslot, int nin,
                        int nout, int pout, float* __restrict__ prop) {
  __shared__ float tile[32][33];
  const int f0 = blockIdx.y * 32, s0 = blockIdx.x * 32;
  const float* c0 = norm;
  const float* mud = norm + NTR + 2 * nin;
  const float* sdd = mud + nout;
  // read: rows = slots, outputs contiguous
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int slot = s0 + y, f = f0 + threadIdx.x;
    tile[y][threadIdx.x] = (slot < nslot && f < nout) ? yhat[(size_t)slot * pout + f] : 0.0f;
  }
  __syncthreads();
  // write: state rows, slots contiguous
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int f = f0 + y, slot = s0 + threadIdx.x;
    if (slot < nslot && f < nout) {
      const int n = f / K, k = f - n * K;
      const size_t i = ((size_t)n * kmax + k) * nslot + slot;
      const float u = logf(conc[i] + c0[n]) + mud[f] + sdd[f] * tile[threadIdx.x][y];
      prop[i] = fmaxf(expf(u) - c0[n], 0.0f);
    }
  }
}

cudaError_t features(const float* conc, const float* force, const float* norm, int K, int kmax,
                     int nslot, int rows, int nin, int pin, __nv_bfloat16* x, cudaStream_t st) {
  // slots on x (up to 2^31 - 1 blocks), features on y (a few dozen)
  dim3 grid((rows + 31) / 32, (pin + 31) / 32);
  k_features<<<grid, dim3(32, 8), 0, st>>>(conc, force, norm, K, kmax, nslot, rows, nin, pin, x);
  return cudaGetLastError();
}

cudaError_t apply(const float* yhat, const float* conc, const float* norm, int K, int kmax,
                  int nslot, int nin, int nout, int pout, float* prop, cudaStream_t st) {
  dim3 grid((nslot + 31) / 32, (nout + 31) / 32);
  k_apply<<<grid, dim3(32, 8), 0, st>>>(yhat, conc, norm, K, kmax, nslot, nin, nout, pout, prop);
  return cudaGetLastError();
}

}  // namespace sur
