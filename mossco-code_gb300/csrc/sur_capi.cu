// sur_capi.cu -- host side of the surrogate MLP (C ABI in mossco_sed.h).
//
// An MLP nin -> hidden (x nhidden, GELU) -> nout with BF16 operands, FP32
// accumulation and FP32 master weights trained by Adam.  Feature dimensions
// are padded to multiples of 128 and batches to multiples of 128 so that
// every product runs in the tiled tensor-core GEMM of sur_kernels.cu; the
// padding holds zeros and receives zero gradients.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mossco_sed.h"
#include "sur_internal.h"
#include "sur_kernels.h"
#include "sur_tc.h"

#define SCK(expr, what)                                                        \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return s->fail(SED_E_CUDA, "%s: %s", what, cudaGetErrorString(e_));      \
  } while (0)

// whether the training products run as tcgen05 GEMMs
static bool train_tc(const sed_surrogate* s) { return s->use_tc && sur::gemm_tc_supported(); }

// One training product C = A B^T (sur_kernels.h): the tcgen05 GEMM of
// sur_tc.cu when the engine is on, else the mma.sync GEMM.
static cudaError_t train_gemm(sed_surrogate* s, int epi, const bf16* A, const bf16* B, int M,
                              int N, int K, const float* bias, float* out_f32, bf16* out_bf16,
                              const float* zprev, int ld_out) {
  if (train_tc(s))
    return sur::gemm_tc(epi, A, B, M, N, K, bias, out_f32, out_bf16, zprev, ld_out, s->gsplit,
                        s->gsplit_n, s->d_err, s->stream);
  return sur::gemm_nt(epi, A, B, M, N, K, bias, out_f32, out_bf16, zprev, ld_out, s->stream);
}

// forward pass over m rows already in s->x; output pre-activation in z[L-1]
int sur_forward_rows(sed_surrogate* s, int m) {
  const bf16* in = s->x;
  for (int l = 0; l < s->L; l++) {
    const bool last = l == s->L - 1;
    SCK(train_gemm(s, last ? sur::EPI_BIAS : sur::EPI_BIAS_GELU, in, s->wb[l], m, s->pout[l],
                   s->pin[l], s->b[l], s->z[l], last ? nullptr : s->a[l], nullptr, s->pout[l]),
        "forward gemm");
    in = s->a[l];
  }
  return SED_OK;
}

bool sur_uses_tc(const sed_surrogate* s) { return s->use_tc && sur::tc_supported(s); }

int sur_check_tc(sed_surrogate* s) {
  int e = 0;
  SCK(cudaMemcpy(&e, s->d_err, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
  if (e) {
    cudaMemset(s->d_err, 0, sizeof(int));
    return s->fail(SED_E_CUDA, "tensor-core MLP kernel gave up waiting (code %d)", e);
  }
  return SED_OK;
}

int sur_infer_rows(sed_surrogate* s, const bf16* x, float* y, int m, bf16* act0, bf16* act1,
                   cudaStream_t st, const unsigned* nrows) {
  if (sur_uses_tc(s)) {
    SCK(sur::infer_tc(s, x, y, m, s->d_err, st, nrows), "tensor-core inference");
    return SED_OK;
  }
  if (nrows) return s->fail(SED_E_ARG, "a device row count needs the fused tcgen05 kernel");
  const bf16* in = x;
  for (int l = 0; l < s->L; l++) {
    const bool last = l == s->L - 1;
    bf16* out = (l & 1) ? act1 : act0;
    SCK(sur::gemm_nt(last ? sur::EPI_BIAS : sur::EPI_GELU, in, s->wb[l], m, s->pout[l],
                     s->pin[l], s->b[l], last ? y : nullptr, last ? nullptr : out, nullptr,
                     s->pout[l], st),
        "inference gemm");
    in = out;
  }
  return SED_OK;
}

namespace {

// loss + backward over m rows (targets in s->y); gradients in gw/gb
int backward(sed_surrogate* s, int m, int m_valid) {
  const int Lh = s->L - 1;
  const int nout_p = s->pout[Lh];
  SCK(cudaMemsetAsync(s->loss, 0, sizeof(float), s->stream), "loss reset");
  const float inv = 1.0f / ((float)m_valid * (float)s->nout);
  SCK(sur::mse(s->z[Lh], s->y, s->mask, m, nout_p, m_valid, inv, s->dz, s->loss, s->stream),
      "mse");
  bf16* dcur = s->dz;
  bf16* dnext = s->dz2;
  for (int l = Lh; l >= 0; l--) {
    const int po = s->pout[l], pi = s->pin[l];
    const bf16* ain = l == 0 ? s->x : s->a[l - 1];
    // gW = dZ^T A_in : A = dZ^T [po x m], B = A_in^T [pi x m]
    SCK(sur::transpose_bf16(dcur, s->dzt, m, po, s->stream), "transpose dZ");
    SCK(sur::transpose_bf16(ain, s->at, m, pi, s->stream), "transpose A");
    SCK(train_gemm(s, sur::EPI_F32, s->dzt, s->at, po, pi, m, nullptr, s->gw[l], nullptr,
                   nullptr, pi),
        "weight gradient gemm");
    SCK(sur::bias_grad(dcur, m, po, s->gpart, s->gb[l], s->stream), "bias gradient");
    if (l > 0) {
      // dZ_{l-1} = (dZ_l W_l) * GELU'(Z_{l-1}) : A = dZ [m x po], B = W^T [pi x po]
      SCK(train_gemm(s, sur::EPI_GELU_BWD, dcur, s->wbt[l], m, pi, po, nullptr, nullptr, dnext,
                     s->z[l - 1], pi),
          "input gradient gemm");
      bf16* t = dcur;
      dcur = dnext;
      dnext = t;
    }
  }
  return SED_OK;
}

void host_bf16(const float* src, int rows, int cols, int pcols, std::vector<bf16>& out) {
  out.assign((size_t)rows * pcols, __float2bfloat16(0.0f));
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < cols; c++) out[(size_t)r * pcols + c] = __float2bfloat16(src[(size_t)r * cols + c]);
}

int upload_rows(sed_surrogate* s, const float* x, int m, int cols, int pcols, bf16* dst) {
  std::vector<bf16> tmp;
  host_bf16(x, m, cols, pcols, tmp);
  SCK(cudaMemsetAsync(dst, 0, (size_t)pad128(m) * pcols * sizeof(bf16), s->stream), "pad clear");
  SCK(cudaMemcpyAsync(dst, tmp.data(), tmp.size() * sizeof(bf16), cudaMemcpyHostToDevice,
                      s->stream),
      "rows copy");
  SCK(cudaStreamSynchronize(s->stream), "rows copy");
  return SED_OK;
}

}  // namespace

extern "C" {

int sed_sur_create(int nin, int nout, int hidden, int nhidden, int max_batch,
                   unsigned long long seed, int device, sed_surrogate** out) {
  if (!out) return SED_E_ARG;
  *out = nullptr;
  if (nin <= 0 || nout <= 0 || hidden <= 0 || nhidden < 1 || nhidden + 1 > kSurMaxLayers ||
      max_batch <= 0)
    return SED_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return SED_E_NODEVICE;
  }
  if (device < 0 || device >= ndev) return SED_E_ARG;
  sed_surrogate* s = new sed_surrogate();
  s->device = device;
  s->nin = nin;
  s->nout = nout;
  s->hidden = hidden;
  s->nhidden = nhidden;
  s->L = nhidden + 1;
  s->max_batch = pad128(max_batch);
  auto bail = [&](int rc) { delete s; return rc; };
  if (cudaSetDevice(device) != cudaSuccess) return bail(SED_E_CUDA);
  if (cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return bail(SED_E_CUDA);
  if (cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(SED_E_CUDA);
  s->stream = s->own_stream;
  int maxd = 0;
  for (int l = 0; l < s->L; l++) {
    s->din[l] = l == 0 ? nin : hidden;
    s->dout[l] = l == s->L - 1 ? nout : hidden;
    s->pin[l] = pad128(s->din[l]);
    s->pout[l] = pad128(s->dout[l]);
    maxd = std::max(maxd, std::max(s->pin[l], s->pout[l]));
  }
  const size_t B = s->max_batch;
  bool ok = true;
  for (int l = 0; l < s->L && ok; l++) {
    const size_t nw = (size_t)s->pout[l] * s->pin[l], nb = s->pout[l];
    ok = s->alloc(&s->w[l], nw) == cudaSuccess && s->alloc(&s->gw[l], nw) == cudaSuccess &&
         s->alloc(&s->mw[l], nw) == cudaSuccess && s->alloc(&s->vw[l], nw) == cudaSuccess &&
         s->alloc(&s->b[l], nb) == cudaSuccess && s->alloc(&s->gb[l], nb) == cudaSuccess &&
         s->alloc(&s->mb[l], nb) == cudaSuccess && s->alloc(&s->vb[l], nb) == cudaSuccess &&
         s->alloc(&s->wb[l], nw) == cudaSuccess && s->alloc(&s->wbt[l], nw) == cudaSuccess &&
         s->alloc(&s->z[l], B * s->pout[l]) == cudaSuccess &&
         (l == s->L - 1 || s->alloc(&s->a[l], B * s->pout[l]) == cudaSuccess);
  }
  ok = ok && s->alloc(&s->x, B * s->pin[0]) == cudaSuccess &&
       s->alloc(&s->y, B * s->pout[s->L - 1]) == cudaSuccess &&
       s->alloc(&s->dz, B * maxd) == cudaSuccess && s->alloc(&s->dz2, B * maxd) == cudaSuccess &&
       s->alloc(&s->dzt, B * maxd) == cudaSuccess && s->alloc(&s->at, B * maxd) == cudaSuccess &&
       s->alloc(&s->mask, (size_t)s->pout[s->L - 1]) == cudaSuccess &&
       s->alloc(&s->loss, 4) == cudaSuccess && s->alloc(&s->d_err, 1) == cudaSuccess &&
       s->alloc(&s->gpart, (size_t)sur::bias_grad_parts() * maxd) == cudaSuccess;
  // up to 32 K-splits of the largest weight gradient
  s->gsplit_n = (size_t)32 * maxd * maxd;
  ok = ok && s->alloc(&s->gsplit, s->gsplit_n) == cudaSuccess;
  if (!ok) return bail(SED_E_NOMEM);
  // output mask; initial weights U(-1/sqrt(in), 1/sqrt(in)), zero biases
  std::vector<float> mask(s->pout[s->L - 1], 0.0f);
  for (int c = 0; c < nout; c++) mask[c] = 1.0f;
  cudaMemcpy(s->mask, mask.data(), mask.size() * sizeof(float), cudaMemcpyHostToDevice);
  unsigned long long st = seed ? seed : 0x9E3779B97F4A7C15ull;
  auto rnd = [&]() {
    st += 0x9E3779B97F4A7C15ull;
    unsigned long long z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < s->L; l++) {
    std::vector<float> w((size_t)s->pout[l] * s->pin[l], 0.0f);
    const double a = 1.0 / std::sqrt((double)s->din[l]);
    for (int r = 0; r < s->dout[l]; r++)
      for (int c = 0; c < s->din[l]; c++) w[(size_t)r * s->pin[l] + c] = (float)((2.0 * rnd() - 1.0) * a);
    if (cudaMemcpy(s->w[l], w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        sur::to_bf16(s->w[l], s->pout[l], s->pin[l], s->wb[l], s->wbt[l], s->stream) != cudaSuccess)
      return bail(SED_E_CUDA);
  }
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return bail(SED_E_CUDA);
  *out = s;
  return SED_OK;
}

int sed_sur_num_params(const sed_surrogate* s) {
  if (!s) return SED_E_ARG;
  int n = 0;
  for (int l = 0; l < s->L; l++) n += s->dout[l] * s->din[l] + s->dout[l];
  return n;
}

// Parameter layout (unpadded, FP32): for each layer W[out][in] then b[out].
int sed_sur_set_weights(sed_surrogate* s, const float* params) {
  if (!s || !params) return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  size_t o = 0;
  for (int l = 0; l < s->L; l++) {
    std::vector<float> w((size_t)s->pout[l] * s->pin[l], 0.0f), b(s->pout[l], 0.0f);
    for (int r = 0; r < s->dout[l]; r++)
      for (int c = 0; c < s->din[l]; c++) w[(size_t)r * s->pin[l] + c] = params[o++];
    for (int r = 0; r < s->dout[l]; r++) b[r] = params[o++];
    SCK(cudaMemcpy(s->w[l], w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice), "w");
    SCK(cudaMemcpy(s->b[l], b.data(), b.size() * sizeof(float), cudaMemcpyHostToDevice), "b");
    SCK(sur::to_bf16(s->w[l], s->pout[l], s->pin[l], s->wb[l], s->wbt[l], s->stream), "bf16");
  }
  SCK(cudaStreamSynchronize(s->stream), "set weights");
  return SED_OK;
}

// params (unpadded, the layout of sed_sur_get_weights) into padded device
// arrays, zero in the padding
static int store_params(sed_surrogate* s, float* const* dst_w, float* const* dst_b,
                        const float* params) {
  size_t o = 0;
  for (int l = 0; l < s->L; l++) {
    std::vector<float> w((size_t)s->pout[l] * s->pin[l], 0.0f), b(s->pout[l], 0.0f);
    for (int r = 0; r < s->dout[l]; r++)
      for (int c = 0; c < s->din[l]; c++) w[(size_t)r * s->pin[l] + c] = params[o++];
    for (int r = 0; r < s->dout[l]; r++) b[r] = params[o++];
    SCK(cudaMemcpy(dst_w[l], w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice), "w");
    SCK(cudaMemcpy(dst_b[l], b.data(), b.size() * sizeof(float), cudaMemcpyHostToDevice), "b");
  }
  return SED_OK;
}

static int fetch_params(sed_surrogate* s, float* const* src_w, float* const* src_b, float* out) {
  SCK(cudaStreamSynchronize(s->stream), "sync");
  size_t o = 0;
  for (int l = 0; l < s->L; l++) {
    std::vector<float> w((size_t)s->pout[l] * s->pin[l]), b(s->pout[l]);
    SCK(cudaMemcpy(w.data(), src_w[l], w.size() * sizeof(float), cudaMemcpyDeviceToHost), "w");
    SCK(cudaMemcpy(b.data(), src_b[l], b.size() * sizeof(float), cudaMemcpyDeviceToHost), "b");
    for (int r = 0; r < s->dout[l]; r++)
      for (int c = 0; c < s->din[l]; c++) out[o++] = w[(size_t)r * s->pin[l] + c];
    for (int r = 0; r < s->dout[l]; r++) out[o++] = b[r];
  }
  return SED_OK;
}

int sed_sur_state_size(const sed_surrogate* s) {
  if (!s) return SED_E_ARG;
  return 3 * sed_sur_num_params(s);
}

// The training state: parameters, Adam's first and second moments (each in
// the layout of sed_sur_get_weights) and Adam's step count.
int sed_sur_get_state(sed_surrogate* s, float* state, long long* step) {
  if (!s || !state || !step) return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  const int n = sed_sur_num_params(s);
  int rc = fetch_params(s, s->w, s->b, state);
  if (!rc) rc = fetch_params(s, s->mw, s->mb, state + n);
  if (!rc) rc = fetch_params(s, s->vw, s->vb, state + 2 * (size_t)n);
  if (rc) return rc;
  *step = s->step;
  return SED_OK;
}

int sed_sur_set_state(sed_surrogate* s, const float* state, long long step) {
  if (!s || !state || step < 0) return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  const int n = sed_sur_num_params(s);
  int rc = store_params(s, s->mw, s->mb, state + n);
  if (!rc) rc = store_params(s, s->vw, s->vb, state + 2 * (size_t)n);
  if (!rc) rc = sed_sur_set_weights(s, state);  // also the BF16 copies
  if (rc) return rc;
  s->step = (int)step;
  return SED_OK;
}

int sed_sur_get_weights(sed_surrogate* s, float* params) {
  if (!s || !params) return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  return fetch_params(s, s->w, s->b, params);
}

// Forward pass on host rows x[m][nin] -> y[m][nout].
int sed_sur_forward(sed_surrogate* s, const float* x, float* y, int m) {
  if (!s || !x || !y || m <= 0) return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  const int nlast = s->pout[s->L - 1];
  for (int r0 = 0; r0 < m; r0 += s->max_batch) {
    const int mm = std::min(s->max_batch, m - r0);
    const int mp = pad128(mm);
    int rc = upload_rows(s, x + (size_t)r0 * s->nin, mm, s->nin, s->pin[0], s->x);
    if (rc) return rc;
    if ((rc = sur_forward_rows(s, mp))) return rc;
    std::vector<float> out((size_t)mm * nlast);
    SCK(cudaMemcpyAsync(out.data(), s->z[s->L - 1], out.size() * sizeof(float),
                        cudaMemcpyDeviceToHost, s->stream), "y copy");
    SCK(cudaStreamSynchronize(s->stream), "forward");
    if (train_tc(s) && (rc = sur_check_tc(s))) return rc;
    for (int r = 0; r < mm; r++)
      for (int c = 0; c < s->nout; c++) y[(size_t)(r0 + r) * s->nout + c] = out[(size_t)r * nlast + c];
  }
  return SED_OK;
}

// Forward pass on device rows: x BF16 [m][pad128(nin)], y FP32
// [m][pad128(nout)], m a multiple of 128 (at most max_batch per launch
// group; larger m is processed in chunks).
int sed_sur_forward_device(sed_surrogate* s, const void* x_dev, void* y_dev, int m) {
  if (!s || !x_dev || !y_dev || m <= 0 || m % 128) return SED_E_ARG;
  // the rows are read by TMA and written in 16-byte pieces
  if (reinterpret_cast<uintptr_t>(x_dev) % 16 || reinterpret_cast<uintptr_t>(y_dev) % 16)
    return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  if (sur_uses_tc(s)) {
    // the fused kernel reads and writes the caller's rows directly
    int rc = sur_infer_rows(s, static_cast<const bf16*>(x_dev), static_cast<float*>(y_dev), m,
                            nullptr, nullptr, s->stream);
    if (rc) return rc;
    SCK(cudaStreamSynchronize(s->stream), "forward");
    return sur_check_tc(s);
  }
  const int nlast = s->pout[s->L - 1];
  for (int r0 = 0; r0 < m; r0 += s->max_batch) {
    const int mm = std::min(s->max_batch, m - r0);
    SCK(cudaMemcpyAsync(s->x, static_cast<const bf16*>(x_dev) + (size_t)r0 * s->pin[0],
                        (size_t)mm * s->pin[0] * sizeof(bf16), cudaMemcpyDeviceToDevice,
                        s->stream), "x copy");
    int rc = sur_forward_rows(s, mm);
    if (rc) return rc;
    SCK(cudaMemcpyAsync(static_cast<float*>(y_dev) + (size_t)r0 * nlast, s->z[s->L - 1],
                        (size_t)mm * nlast * sizeof(float), cudaMemcpyDeviceToDevice,
                        s->stream), "y copy");
  }
  SCK(cudaStreamSynchronize(s->stream), "forward");
  return train_tc(s) ? sur_check_tc(s) : SED_OK;
}

// One Adam step on a device batch: x BF16 [m][pad128(nin)], y BF16
// [m][pad128(nout)], m a multiple of 128 and <= max_batch.  loss (host) may
// be NULL (no synchronisation then).
int sed_sur_train_step(sed_surrogate* s, const void* x_dev, const void* y_dev, int m,
                       float lr, float* loss) {
  if (!s || !x_dev || !y_dev || m <= 0 || m % 128 || m > s->max_batch) return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  SCK(cudaMemcpyAsync(s->x, x_dev, (size_t)m * s->pin[0] * sizeof(bf16),
                      cudaMemcpyDeviceToDevice, s->stream), "x copy");
  SCK(cudaMemcpyAsync(s->y, y_dev, (size_t)m * s->pout[s->L - 1] * sizeof(bf16),
                      cudaMemcpyDeviceToDevice, s->stream), "y copy");
  int rc = sur_forward_rows(s, m);
  if (rc) return rc;
  if ((rc = backward(s, m, m))) return rc;
  s->step++;
  // one Adam launch over every layer's weights and biases
  sur::AdamSet set{};
  long long at = 0;
  for (int l = 0; l < s->L; l++) {
    set.seg[set.n] = {s->w[l], s->mw[l], s->vw[l], s->gw[l], s->wb[l], s->wbt[l], s->pout[l],
                      s->pin[l]};
    set.start[set.n++] = at;
    at += (long long)s->pout[l] * s->pin[l];
    set.seg[set.n] = {s->b[l], s->mb[l], s->vb[l], s->gb[l], nullptr, nullptr, 1, s->pout[l]};
    set.start[set.n++] = at;
    at += s->pout[l];
  }
  set.start[set.n] = at;
  SCK(sur::adam_all(set, lr, 0.9f, 0.999f, 1e-8f, s->step, s->sms, s->stream), "adam");
  if (loss) {
    SCK(cudaMemcpyAsync(loss, s->loss, sizeof(float), cudaMemcpyDeviceToHost, s->stream), "loss");
    SCK(cudaStreamSynchronize(s->stream), "train step");
    if (train_tc(s)) return sur_check_tc(s);
  }
  return SED_OK;
}

// Loss and parameter gradients (layout of sed_sur_get_weights) for host
// rows x[m][nin], y[m][nout]; the weights are not updated.
int sed_sur_grads(sed_surrogate* s, const float* x, const float* y, int m, float* grads,
                  float* loss) {
  if (!s || !x || !y || !grads || m <= 0 || m > s->max_batch) return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  const int mp = pad128(m);
  int rc = upload_rows(s, x, m, s->nin, s->pin[0], s->x);
  if (rc) return rc;
  if ((rc = upload_rows(s, y, m, s->nout, s->pout[s->L - 1], s->y))) return rc;
  if ((rc = sur_forward_rows(s, mp))) return rc;
  if ((rc = backward(s, mp, m))) return rc;
  if (loss) SCK(cudaMemcpyAsync(loss, s->loss, sizeof(float), cudaMemcpyDeviceToHost, s->stream), "loss");
  if ((rc = fetch_params(s, s->gw, s->gb, grads))) return rc;
  return train_tc(s) ? sur_check_tc(s) : SED_OK;
}

int sed_sur_set_stream(sed_surrogate* s, void* stream) {
  if (!s) return SED_E_ARG;
  SCK(cudaSetDevice(s->device), "set device");
  SCK(cudaStreamSynchronize(s->stream), "stream switch");
  s->stream = stream ? static_cast<cudaStream_t>(stream) : s->own_stream;
  return SED_OK;
}

int sed_sur_set_tensor_cores(sed_surrogate* s, int on) {
  if (!s) return SED_E_ARG;
  s->use_tc = on != 0;
  return sur_uses_tc(s) ? 1 : 0;
}

const char* sed_sur_last_error(const sed_surrogate* s) { return s ? s->err.c_str() : ""; }

void sed_sur_destroy(sed_surrogate* s) { delete s; }

}  // extern "C"
