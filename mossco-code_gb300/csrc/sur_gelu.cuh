// sur_gelu.cuh -- the surrogate's activation for training: the tanh form of
// GELU and its derivative, shared by the mma.sync GEMMs (sur_kernels.cu) and
// the tcgen05 GEMMs (sur_tc.cu) so both engines apply the same function.
#pragma once

namespace sur {

__device__ __forceinline__ float gelu(float z) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float u = k0 * (z + k1 * z * z * z);
  return 0.5f * z * (1.0f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float u = k0 * (z + k1 * z * z * z);
  const float t = tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * k0 * (1.0f + 3.0f * k1 * z * z);
}

}  // namespace sur
