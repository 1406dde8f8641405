// sur_loop.h -- launchers between the solver's slot layout and the
// surrogate's row layout (sur_loop.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sur {

// norm: c0[11] | mu_x[nin] | sd_x[nin] | mu_d[nout] | sd_d[nout]
// Row r < nrows of x is the column in slot list[r]; rows nrows .. rows-1
// are zero.
cudaError_t features(const float* conc, const float* force, const float* norm, const int* list,
                     int nrows, int K, int kmax, int nslot, int rows, int nin, int pin,
                     __nv_bfloat16* x, cudaStream_t st);
// training rows of the columns of slots [slot0, slot0 + nslots) whose step
// took more than one attempt (conc0: state before the step, conc1: after)
cudaError_t collect(const float* conc0, const float* conc1, const float* force, const int* kact,
                    const int* nsub, const float* c0, int K, int kmax, int nslot, int slot0,
                    int nslots, float* x, int pitch_x, float* y, int pitch_y,
                    unsigned long long* count, long long capacity, int sms, cudaStream_t st);

}  // namespace sur
