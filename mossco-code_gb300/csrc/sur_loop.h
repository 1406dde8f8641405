// sur_loop.h -- launchers between the solver's slot layout and the
// surrogate's row layout (sur_loop.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sur {

// norm: c0[11] | mu_x[nin] | sd_x[nin] | mu_d[nout] | sd_d[nout]
cudaError_t features(const float* conc, const float* force, const float* norm, int K, int kmax,
                     int nslot, int rows, int nin, int pin, __nv_bfloat16* x, cudaStream_t st);
cudaError_t apply(const float* yhat, const float* conc, const float* norm, int K, int kmax,
                  int nslot, int nin, int nout, int pout, float* prop, cudaStream_t st);

}  // namespace sur
