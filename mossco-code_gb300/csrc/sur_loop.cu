// sur_loop.cu -- kernels between the solver's slot layout and the
// surrogate's row layout.
//
// Features of a column (a row of the MLP batch), tracer-major:
//   x[n*K + k]   = (log(max(C[n][k], 0) + c0[n]) - mu_x) / sd_x     n < 11, k < K
//   x[11*K + f]  = (force[f] - mu_x) / sd_x                          f < 13
// (the 13 per-column forcing rows of the solver: bioturbation x f_T, the
// molecular multiplier and the 11 surface values), zero in padded columns.
// The network predicts the standardised change of log(C + c0) over one
// coupling step; the surrogate step's residual kernel forms the proposed
// state from it.  In the surrogate step the gate (the tile kernel's
// KIND_PROBE) writes these rows for the columns it lists, from the tile it
// has staged.
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
