// sur_loop.h -- launchers between the solver's slot layout and the
// surrogate's row layout (sur_loop.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sur {

// training rows of the columns of slots [slot0, slot0 + nslots) whose step
// took more than one attempt (conc0: state before the step, conc1: after)
cudaError_t collect(const float* conc0, const float* conc1, const float* force, const int* kact,
                    const int* nsub, const float* c0, int K, int kmax, int nslot, int slot0,
                    int nslots, float* x, int pitch_x, float* y, int pitch_y,
                    unsigned long long* count, long long capacity, int sms, cudaStream_t st);

}  // namespace sur
