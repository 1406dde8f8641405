// sur_internal.h -- the surrogate handle, shared by sur_capi.cu and the
// surrogate coupling step in sed_capi.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

using bf16 = __nv_bfloat16;

constexpr int kSurMaxLayers = 8;
inline int pad128(int x) { return (x + 127) / 128 * 128; }

struct sed_surrogate {
  int device = 0;
  int sms = 0;                        // the device's SM count
  cudaStream_t stream = nullptr;      // stream in use
  cudaStream_t own_stream = nullptr;  // stream created by the handle
  int nin = 0, nout = 0, hidden = 0, nhidden = 0, L = 0, max_batch = 0;
  int din[kSurMaxLayers], dout[kSurMaxLayers], pin[kSurMaxLayers], pout[kSurMaxLayers];
  float *w[kSurMaxLayers] = {}, *b[kSurMaxLayers] = {}, *gw[kSurMaxLayers] = {}, *gb[kSurMaxLayers] = {};
  float *mw[kSurMaxLayers] = {}, *vw[kSurMaxLayers] = {}, *mb[kSurMaxLayers] = {}, *vb[kSurMaxLayers] = {};
  bf16 *wb[kSurMaxLayers] = {}, *wbt[kSurMaxLayers] = {};
  float* z[kSurMaxLayers] = {};  // pre-activations [max_batch][pout]
  bf16* a[kSurMaxLayers] = {};   // GELU activations of hidden layers
  bf16 *x = nullptr, *y = nullptr, *dz = nullptr, *dz2 = nullptr, *dzt = nullptr, *at = nullptr;
  float *mask = nullptr, *loss = nullptr;
  float* gpart = nullptr;  // bias-gradient partial sums [bias_grad_parts()][maxd]
  int step = 0;
  // feature and increment normalisation of the column surrogate:
  // c0[11] | mu_x[nin] | sd_x[nin] | mu_d[nout] | sd_d[nout]
  float* norm = nullptr;
  int norm_len = 0;
  // the tcgen05 engine (the fused inference kernel when the shape fits, and
  // the training products as tcgen05 GEMMs) or the mma.sync GEMMs for both;
  // d_err: the tcgen05 kernels' barrier-timeout code
  bool use_tc = true;
  int* d_err = nullptr;
  // partial tiles of the K-split weight-gradient products (gsplit_n floats)
  float* gsplit = nullptr;
  size_t gsplit_n = 0;
  std::vector<void*> allocs;
  std::string err;

  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t n) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T) + 16);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      cudaMemset(q, 0, n * sizeof(T) + 16);
    }
    *p = static_cast<T*>(q);
    return e;
  }
  ~sed_surrogate() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : allocs) cudaFree(p);
    if (own_stream) cudaStreamDestroy(own_stream);
  }
};


// forward pass over m rows already in s->x; output pre-activation in z[L-1]
int sur_forward_rows(sed_surrogate* s, int m);
// inference over m rows (a multiple of 128): x BF16 [m][pin[0]] -> y FP32
// [m][pout[L-1]]: the fused tcgen05 kernel when s->use_tc and the shape
// fits, else the mma.sync GEMMs with the hidden activations in act0 / act1
// (BF16 [m][hidden padded]; unused by the fused kernel, may be null then).
// nrows (device, fused kernel only): run just the tiles of the first
// min(m, *nrows) rows
int sur_infer_rows(sed_surrogate* s, const bf16* x, float* y, int m, bf16* act0, bf16* act1,
                   cudaStream_t st, const unsigned* nrows = nullptr);
// whether sur_infer_rows takes the fused tcgen05 kernel
bool sur_uses_tc(const sed_surrogate* s);
// the fused kernel's error flag: reset before, checked after a synchronised
// call (SED_E_CUDA with a message when the kernel gave up waiting)
int sur_check_tc(sed_surrogate* s);
