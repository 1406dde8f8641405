// sur_tc.cu -- the surrogate network's inference pass on the 5th-generation
// tensor cores: one fused kernel for the whole MLP (all layers, bias and
// GELU), tcgen05.mma with accumulators in tensor memory (TMEM), operands
// staged in shared memory by TMA (cp.async.bulk.tensor) with the 128-byte
// swizzle the MMA descriptors read.
//
// A persistent CTA per SM walks tiles of 128 rows.  Per tile:
//   X tile [128][K0] (BF16)  --TMA-->  shared memory (6 chunks of 64 columns)
//   layer l: acc[128][N_l] (FP32, TMEM) = A[128][K_l] . W_l^T, the weights
//            streamed through a ring of NST stages of [256][64] by TMA
//   epilogue: acc + b, GELU -> BF16 back into the same shared buffer, in
//            the swizzled layout of the next layer's A operand; the last
//            layer's acc + b goes to global memory (FP32 rows).
// Every wait on an mbarrier is bounded: after ~1 s the kernel records an
// error code, stops issuing work, waits (bounded) for its outstanding copies
// and MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <algorithm>

#include "sur_gelu.cuh"
#include "sur_internal.h"
#include "sur_kernels.h"
#include "sur_tc.h"

namespace sur {
namespace tc {

constexpr int BM = 128;                  // rows per tile (MMA M)
constexpr int BK = 64;                   // K per chunk: 128 bytes of BF16
constexpr int CHUNK = BM * BK * 2;       // one [128][64] BF16 box: 16 KB
constexpr int KMAX0 = 384;               // widest input the X buffer holds
constexpr int XBUF = (KMAX0 / BK) * CHUNK;  // 96 KB
constexpr int STAGE = 2 * CHUNK;         // [256][64] weights: 32 KB
constexpr int NST = 3;                   // weight ring stages
constexpr int HID = 256;                 // hidden width (TMEM columns used)
constexpr int TMEM_COLS = 512;
constexpr int EPI_WARPS = 16;            // warps 0-15 run the epilogue
constexpr int ECOLS = BK / (EPI_WARPS / 4);  // columns of a 64-column chunk per warp
constexpr int PRODUCER = EPI_WARPS, MMA = EPI_WARPS + 1;  // warps
constexpr int NTHREADS = 32 * (EPI_WARPS + 2);
constexpr long long WAIT_CYCLES = 2000000000ll;  // ~1 s at 2 GHz
// shared memory after the weight ring: 2 NST + 9 barriers, then the biases
constexpr int BAR_OFF = XBUF + NST * STAGE;
constexpr int BIAS_OFF = BAR_OFF + 8 * (2 * NST + 9);
constexpr int BIAS_MAX = 4096;  // floats: the sum of every layer's padded width

struct Layers {
  CUtensorMap w[kSurMaxLayers];  // [nout][nin] BF16, box [128][64]
  const float* bias[kSurMaxLayers];
  int nout[kSurMaxLayers];
  int L, k0;
};

// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait: false (with the error recorded) when the phase does not
// complete within WAIT_CYCLES or another role has given up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort,
                                          int* err, int code) {
  const long long t0 = clock64();
  for (;;) {
    if (mbar_test(bar, parity)) return true;
    if (*abort) return false;
    if (clock64() - t0 > WAIT_CYCLES) {
      *abort = 1;
      atomicCAS(err, 0, code);
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand in the 128-byte
// swizzled layout TMA writes: rows of 128 bytes, 8-row atoms of 1024 bytes
// (stride byte offset 1024), descriptor version 1, swizzle mode 2.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulation, BF16 A and B,
// both K-major, M = 128, N = n.
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane, issued without
// waiting: the registers hold the values only after tmem_wait(r)
__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
}
// 16 consecutive FP32 columns of this thread's TMEM lane, issued without
// waiting (the epilogue's half-width form of tmem_ld32_async)
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait16(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}

// Wait for the thread's TMEM loads; the registers are operands, so no use
// of them moves above the wait.
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]),
                 "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]),
                 "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]),
                 "+r"(r[30]), "+r"(r[31])
               :
               : "memory");
}

// tanh form of GELU, 0.5 z (1 + tanh(k0 (z + k1 z^3))), with the hardware
// tanh approximation: z2 = z z; u = z (k0 + k0 k1 z2); h = z / 2; h + h t.
// A pair at a time in packed FP32x2 arithmetic (each component rounds as
// the scalar operation would; the tanh stays scalar).
__device__ __forceinline__ float2 gelu_fast2(float2 z) {
  const float2 w = __ffma2_rn(make_float2(0.035677408136300125f, 0.035677408136300125f),
                              __fmul2_rn(z, z),
                              make_float2(0.7978845608028654f, 0.7978845608028654f));
  const float2 u = __fmul2_rn(z, w);
  float tx, ty;
  asm("tanh.approx.f32 %0, %1;" : "=f"(tx) : "f"(u.x));
  asm("tanh.approx.f32 %0, %1;" : "=f"(ty) : "f"(u.y));
  const float2 hz = __fmul2_rn(make_float2(0.5f, 0.5f), z);
  return __ffma2_rn(hz, make_float2(tx, ty), hz);
}

// Eight FP32 values to a 32-byte aligned global address in one 256-bit
// store.
__device__ __forceinline__ void st_global_v8(float* p, const float* v) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(v[0]),
               "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
               : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// Roles of the 576 threads: warps 0-15 run the epilogue (warp w reads the
// TMEM lanes 32 (w % 4) .. +31, one row per thread, and the columns
// 16 (w / 4) .. +15 of every 64-column chunk: four warps per lane quarter,
// so each thread's chain of TMEM load, bias, GELU and store is short and
// sixteen warps hide one another's latency), warp 16 issues the TMA loads,
// warp 17 the MMAs.
//
// Overlap.  Hidden layer l accumulates in TMEM region l % 2 (columns
// 256 (l % 2) .. +255), so layer l+1's MMAs run while the epilogue still
// reads layer l's accumulator; the epilogue releases the next layer's A
// operand 64 columns at a time (barrier actc[kc]), so layer l+1 starts on
// chunk 0 while chunks 1-3 are being produced.  The last layer's output
// columns 0..255 accumulate in region 0 and 256.. in region 1 (its TMEM
// column is its output column); the next tile's layer 0 waits only for the
// epilogue to have read region 0 (barrier lastepi).
__global__ void __launch_bounds__(NTHREADS, 1)
k_mlp_tc(const __grid_constant__ CUtensorMap tx, const __grid_constant__ Layers P,
         float* __restrict__ y, int ldy, bool y32, int maxtiles,
         const unsigned* __restrict__ nrows, int* err) {
  // the rows to run: all maxtiles tiles, or the tiles holding the first
  // *nrows rows when the count lives on the device
  const int ntiles =
      nrows ? min(maxtiles, (int)((*nrows + (unsigned)BM - 1) / (unsigned)BM)) : maxtiles;
  extern __shared__ unsigned char smem_raw[];
  // 1024-byte alignment for the swizzle atoms
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char* xbuf = smem;                 // X tile, then the activations
  unsigned char* wbuf = smem + XBUF;          // weight ring
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + BAR_OFF);
  // bars: full[NST], empty[NST], xfull, xempty, acc[2], lastepi, actc[4]
  // (accumulators complete alternately on acc[0] and acc[1], so neither
  // runs two phases ahead of the epilogue when the last layer's two parts
  // complete back to back)
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t b_full = saddr(bars), b_empty = saddr(bars + NST);
  const uint32_t b_xfull = saddr(bars + 2 * NST), b_xempty = saddr(bars + 2 * NST + 1);
  const uint32_t b_acc = saddr(bars + 2 * NST + 2);   // 2 barriers, 8 bytes apart
  const uint32_t b_last = saddr(bars + 2 * NST + 4);
  const uint32_t b_actc = saddr(bars + 2 * NST + 5);  // 4 barriers, 8 bytes apart

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int i = 0; i < NST; i++) {
      mbar_init(b_full + 8 * i, 1);
      mbar_init(b_empty + 8 * i, 1);
    }
    mbar_init(b_xfull, 1);
    mbar_init(b_xempty, 1);
    mbar_init(b_acc, 1);
    mbar_init(b_acc + 8, 1);
    // the epilogue arrives once per warp
    mbar_init(b_last, EPI_WARPS);
    for (int i = 0; i < HID / BK; i++) mbar_init(b_actc + 8 * i, EPI_WARPS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(&s_tmem)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (warp == PRODUCER && lane == 0) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tx)) : "memory");
    for (int l = 0; l < P.L; l++)
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&P.w[l]))
                   : "memory");
  }
  // every layer's bias in shared memory (layer l at boff[l])
  float* s_bias = reinterpret_cast<float*>(smem + BIAS_OFF);
  int boff[kSurMaxLayers];
  {
    int o = 0;
    for (int l = 0; l < P.L; l++) {
      boff[l] = o;
      for (int i = threadIdx.x; i < P.nout[l]; i += blockDim.x) s_bias[o + i] = P.bias[l][i];
      o += P.nout[l];
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = s_tmem;
  const int last = P.L - 1;

  if (warp == PRODUCER) {
    // ---- TMA producer (one lane)
    if (lane == 0) {
      uint32_t g = 0;   // weight chunks issued
      uint32_t it = 0;  // tiles issued
      bool ok = true;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, it++) {
        if (it > 0) ok = mbar_wait(b_xempty, (it - 1) & 1, &s_abort, err, 1);
        if (!ok) break;
        mbar_expect_tx(b_xfull, (uint32_t)(P.k0 / BK) * CHUNK);
        for (int kc = 0; kc < P.k0 / BK; kc++)
          tma_load_2d(saddr(xbuf + kc * CHUNK), &tx, kc * BK, tile * BM, b_xfull);
        for (int l = 0; l < P.L && ok; l++) {
          const int K = l == 0 ? P.k0 : HID;
          for (int n0 = 0; n0 < P.nout[l] && ok; n0 += HID) {
            const int nn = min(HID, P.nout[l] - n0);
            for (int kc = 0; kc < K / BK; kc++, g++) {
              const uint32_t s = g % NST;
              if (g >= NST) {
                ok = mbar_wait(b_empty + 8 * s, ((g / NST) - 1) & 1, &s_abort, err, 2);
                if (!ok) break;
              }
              mbar_expect_tx(b_full + 8 * s, (uint32_t)nn * BK * 2);
              for (int r = 0; r < nn; r += BM)
                tma_load_2d(saddr(wbuf + s * STAGE + r * BK * 2), &P.w[l], kc * BK, n0 + r,
                            b_full + 8 * s);
            }
          }
        }
      }
      if (!ok) {
        // let the copies already issued land before the CTA's memory goes
        for (uint32_t k = 0; k < NST && k < g; k++) {
          const uint32_t gg = g - 1 - k, s = gg % NST;
          const long long t0 = clock64();
          while (!mbar_test(b_full + 8 * s, (gg / NST) & 1) && clock64() - t0 < WAIT_CYCLES) {
          }
        }
      }
    }
  } else if (warp == MMA) {
    // ---- MMA issuer (one lane)
    if (lane == 0) {
      uint32_t g = 0, it = 0, u = 0;
      uint32_t ph_act[HID / BK] = {0, 0, 0, 0};
      bool ok = true, issued = false;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, it++) {
        ok = mbar_wait(b_xfull, it & 1, &s_abort, err, 3);
        // region 0 is free once the previous tile's last epilogue read it
        if (ok && it > 0) ok = mbar_wait(b_last, (it - 1) & 1, &s_abort, err, 4);
        for (int l = 0; l < P.L && ok; l++) {
          const int K = l == 0 ? P.k0 : HID;
          for (int n0 = 0; n0 < P.nout[l] && ok; n0 += HID) {
            const int nn = min(HID, P.nout[l] - n0);
            const uint32_t idesc = idesc_bf16(nn);
            // hidden layer l: region l % 2; last layer: its output columns
            const uint32_t dcol = l == last ? (uint32_t)n0 : (uint32_t)(HID * (l & 1));
            for (int kc = 0; kc < K / BK; kc++, g++) {
              if (l > 0 && n0 == 0) {
                // the epilogue has written this chunk of the A operand
                ok = mbar_wait(b_actc + 8 * kc, ph_act[kc] & 1, &s_abort, err, 7);
                ph_act[kc]++;
                if (!ok) break;
              }
              const uint32_t s = g % NST;
              ok = mbar_wait(b_full + 8 * s, (g / NST) & 1, &s_abort, err, 5);
              if (!ok) break;
              fence_after();
              const uint32_t a0 = saddr(xbuf + kc * CHUNK);
              const uint32_t b0 = saddr(wbuf + s * STAGE);
#pragma unroll
              for (int k = 0; k < BK / 16; k++)
                mma_bf16(tmem + dcol, desc_sw128(a0 + 32 * k), desc_sw128(b0 + 32 * k), idesc,
                         (kc > 0 || k > 0) ? 1u : 0u);
              mma_commit(b_empty + 8 * s);  // the stage is free once these complete
              issued = true;
            }
            if (ok) mma_commit(b_acc + 8 * (u++ & 1));  // this accumulator (part) is complete
          }
        }
        if (ok) mma_commit(b_xempty);  // the A buffer is free for the next tile
      }
      if (issued) {
        // the MMAs in flight complete before the TMEM is released
        const long long t0 = clock64();
        while (!mbar_test(b_empty + 8 * ((g - 1) % NST), ((g - 1) / NST) & 1) &&
               clock64() - t0 < WAIT_CYCLES) {
        }
      }
    }
  } else {
    // ---- epilogue (warps 0 .. EPI_WARPS-1)
    const int q = warp & 3, h = warp >> 2;
    const int row = q * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16);
    uint32_t a = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      for (int l = 0; l < P.L && ok; l++) {
        const float* bias = s_bias + boff[l];
        const bool is_last = l == last;
        for (int n0 = 0; n0 < P.nout[l] && ok; n0 += HID) {
          ok = mbar_wait(b_acc + 8 * (a & 1), (a >> 1) & 1, &s_abort, err, 6);
          // one outcome per warp, so the warp stays converged for its
          // per-warp arrivals below
          ok = __all_sync(0xffffffffu, ok);
          a++;
          if (!ok) break;
          fence_after();
          const int nchunk = min(HID, P.nout[l] - n0) / BK;
          // TMEM column of chunk kc: the output column for the last layer,
          // region l % 2 for a hidden one
          auto tcol = [&](int kc) {
            const int c0 = n0 + kc * BK + ECOLS * h;
            return is_last ? (uint32_t)c0 : (uint32_t)(HID * (l & 1) + c0);
          };
          uint32_t ra[ECOLS], rb[ECOLS];
          tmem_ld16_async(tl + tcol(0), ra);
          tmem_wait16(ra);
#pragma unroll
          for (int kc = 0; kc < HID / BK; kc++) {
            if (kc >= nchunk) break;
            uint32_t(&cur)[ECOLS] = (kc & 1) ? rb : ra;
            uint32_t(&nxt)[ECOLS] = (kc & 1) ? ra : rb;
            // the next chunk's load runs while this one is processed
            if (kc + 1 < nchunk) tmem_ld16_async(tl + tcol(kc + 1), nxt);
            const int c0 = n0 + kc * BK + ECOLS * h;  // output column
            float v[ECOLS];
#pragma unroll
            for (int i = 0; i < ECOLS; i += 2) {
              const float2 acc = make_float2(__uint_as_float(cur[i]), __uint_as_float(cur[i + 1]));
              const float2 bb = *reinterpret_cast<const float2*>(bias + c0 + i);
              const float2 sum = __fadd2_rn(acc, bb);
              v[i] = sum.x;
              v[i + 1] = sum.y;
            }
            if (is_last) {
              float* dst = y + (size_t)(tile * BM + row) * ldy + c0;
              if (y32) {
                // 32-byte row pieces: half the store instructions, each
                // a whole sector of its row
#pragma unroll
                for (int i = 0; i < ECOLS; i += 8) st_global_v8(dst + i, v + i);
              } else {
#pragma unroll
                for (int i = 0; i < ECOLS; i += 4)
                  *reinterpret_cast<float4*>(dst + i) =
                      make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
              }
            } else {
              // BF16 GELU into chunk kc of the next layer's A operand: row
              // `row`, the warp's 16-byte pieces (ECOLS / 8) h + p at
              // (piece ^ row % 8)
              unsigned char* rbase = xbuf + kc * CHUNK + row * 128;
#pragma unroll
              for (int p = 0; p < ECOLS / 8; p++) {
                uint4 w;
                const float2 g0 = gelu_fast2(make_float2(v[8 * p + 0], v[8 * p + 1]));
                const float2 g1 = gelu_fast2(make_float2(v[8 * p + 2], v[8 * p + 3]));
                const float2 g2 = gelu_fast2(make_float2(v[8 * p + 4], v[8 * p + 5]));
                const float2 g3 = gelu_fast2(make_float2(v[8 * p + 6], v[8 * p + 7]));
                w.x = pack_bf16(g0.x, g0.y);
                w.y = pack_bf16(g1.x, g1.y);
                w.z = pack_bf16(g2.x, g2.y);
                w.w = pack_bf16(g3.x, g3.y);
                *reinterpret_cast<uint4*>(rbase + ((((ECOLS / 8) * h + p) ^ (row & 7)) << 4)) = w;
              }
              // every lane's stores made visible to the tensor cores'
              // (async) reads, then one arrival for the warp
              fence_before();
              asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
              __syncwarp();
              if (lane == 0) mbar_arrive(b_actc + 8 * kc);
            }
            if (kc + 1 < nchunk) tmem_wait16(nxt);
          }
          if (is_last && n0 == 0) {
            // region 0 read: the next tile's first layer may start
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(b_last);
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Training products on the tcgen05 tensor cores: C[M x N] = A[M x K] .
// B[N x K]^T with A and B BF16 and the reduction dimension contiguous (the
// forward Z = X W^T, the input gradient dX = dZ W and the weight gradient
// dW = dZ^T X, as sur_kernels.cu writes them), FP32 accumulation in TMEM.
//
// One CTA per 128 x 128 output tile and K range (blockIdx.z; the weight
// gradient, whose K is the batch, splits K so the few output tiles fill the
// SMs).  Warp 4 streams the A and B K-chunks ([128][64] boxes each, 128-byte
// swizzle) through a ring of GST stages by TMA, warp 5 issues four
// M128 N128 K16 MMAs per chunk, and warps 0-3 (one TMEM lane = one output
// row per thread) apply the epilogue.  A split writes its partial tile to
// its own slice of a workspace; k_split_sum adds the slices in a fixed
// order, so results do not depend on scheduling.  Every barrier wait is
// bounded as in k_mlp_tc.
constexpr int GN = 128;                 // output columns per tile (MMA N)
constexpr int GST = 4;                  // ring stages
constexpr int GSTAGE = 2 * CHUNK;       // A [128][64] + B [128][64]: 32 KB
constexpr int GTHREADS = 192;           // warps 0-3 epilogue, 4 TMA, 5 MMA
constexpr int GBAR_OFF = GST * GSTAGE;  // then full[GST], empty[GST], acc
constexpr int GSMEM = 1024 + GBAR_OFF + 8 * (2 * GST + 1);
constexpr int GTMEM_COLS = 128;

template <int EPI>
__global__ void __launch_bounds__(GTHREADS, 1)
k_gemm_tc(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
          int nkc, int kc_per_split, const float* __restrict__ bias,
          float* __restrict__ out_f32, __nv_bfloat16* __restrict__ out_bf16,
          const float* __restrict__ zprev, int ld_out, size_t split_stride, int* err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + GBAR_OFF);
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t b_full = saddr(bars), b_empty = saddr(bars + GST), b_acc = saddr(bars + 2 * GST);
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * GN;
  const int kc0 = blockIdx.z * kc_per_split;
  const int nk = min(nkc, kc0 + kc_per_split) - kc0;  // >= 1 (host)

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int i = 0; i < GST; i++) {
      mbar_init(b_full + 8 * i, 1);
      mbar_init(b_empty + 8 * i, 1);
    }
    mbar_init(b_acc, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(&s_tmem)),
                 "r"(GTMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (warp == 4 && lane == 0) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&ta)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tb)) : "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = s_tmem;

  if (warp == 4) {
    // ---- TMA producer (one lane)
    if (lane == 0) {
      bool ok = true;
      int g = 0;
      for (; g < nk; g++) {
        const int s = g % GST;
        if (g >= GST) {
          ok = mbar_wait(b_empty + 8 * s, ((g / GST) - 1) & 1, &s_abort, err, 11);
          if (!ok) break;
        }
        mbar_expect_tx(b_full + 8 * s, GSTAGE);
        tma_load_2d(saddr(smem + s * GSTAGE), &ta, (kc0 + g) * BK, m0, b_full + 8 * s);
        tma_load_2d(saddr(smem + s * GSTAGE + CHUNK), &tb, (kc0 + g) * BK, n0, b_full + 8 * s);
      }
      if (!ok) {
        // the copies already issued land before the CTA's memory goes
        for (int k = 0; k < GST && k < g; k++) {
          const int gg = g - 1 - k, s = gg % GST;
          const long long t0 = clock64();
          while (!mbar_test(b_full + 8 * s, (gg / GST) & 1) && clock64() - t0 < WAIT_CYCLES) {
          }
        }
      }
    }
  } else if (warp == 5) {
    // ---- MMA issuer (one lane)
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16(GN);
      bool ok = true;
      int g = 0;
      for (; g < nk; g++) {
        const int s = g % GST;
        ok = mbar_wait(b_full + 8 * s, (g / GST) & 1, &s_abort, err, 12);
        if (!ok) break;
        fence_after();
        const uint32_t a0 = saddr(smem + s * GSTAGE), b0 = a0 + CHUNK;
#pragma unroll
        for (int k = 0; k < BK / 16; k++)
          mma_bf16(tmem, desc_sw128(a0 + 32 * k), desc_sw128(b0 + 32 * k), idesc,
                   (g > 0 || k > 0) ? 1u : 0u);
        mma_commit(b_empty + 8 * s);  // the stage is free once these complete
      }
      if (ok) {
        mma_commit(b_acc);  // the accumulator is complete
      } else if (g > 0) {
        // the MMAs in flight complete before the TMEM is released
        const int gg = g - 1, s = gg % GST;
        const long long t0 = clock64();
        while (!mbar_test(b_empty + 8 * s, (gg / GST) & 1) && clock64() - t0 < WAIT_CYCLES) {
        }
      }
    }
  } else {
    // ---- epilogue (warps 0-3): TMEM lane = tile row
    bool ok = mbar_wait(b_acc, 0, &s_abort, err, 13);
    ok = __all_sync(0xffffffffu, ok);
    if (ok) {
      fence_after();
      const int row = warp * 32 + lane;
      const size_t orow = (size_t)(m0 + row) * ld_out;
      const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
      float* part = out_f32 + (EPI == EPI_F32 ? blockIdx.z * split_stride : 0);
#pragma unroll 1
      for (int c = 0; c < GN / 32; c++) {
        uint32_t r[32];
        tmem_ld32_async(tl + 32 * c, r);
        tmem_wait(r);
        const int col = n0 + 32 * c;
        float v[32];
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
        if (EPI == EPI_BIAS_GELU || EPI == EPI_BIAS || EPI == EPI_GELU) {
#pragma unroll
          for (int i = 0; i < 32; i++) v[i] += bias[col + i];
        }
        if (EPI == EPI_BIAS_GELU || EPI == EPI_BIAS || EPI == EPI_F32) {
          float* dst = part + orow + col;
#pragma unroll
          for (int i = 0; i < 32; i += 4)
            *reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
        if (EPI == EPI_BIAS_GELU || EPI == EPI_GELU || EPI == EPI_GELU_BWD) {
          float g[32];
          if (EPI == EPI_GELU_BWD) {
            const float* z = zprev + orow + col;
#pragma unroll
            for (int i = 0; i < 32; i += 4) {
              const float4 q = *reinterpret_cast<const float4*>(z + i);
              g[i] = v[i] * gelu_grad(q.x);
              g[i + 1] = v[i + 1] * gelu_grad(q.y);
              g[i + 2] = v[i + 2] * gelu_grad(q.z);
              g[i + 3] = v[i + 3] * gelu_grad(q.w);
            }
          } else {
#pragma unroll
            for (int i = 0; i < 32; i++) g[i] = gelu(v[i]);
          }
          __nv_bfloat16* dst = out_bf16 + orow + col;
#pragma unroll
          for (int i = 0; i < 32; i += 8) {
            uint4 w;
            w.x = pack_bf16(g[i], g[i + 1]);
            w.y = pack_bf16(g[i + 2], g[i + 3]);
            w.z = pack_bf16(g[i + 4], g[i + 5]);
            w.w = pack_bf16(g[i + 6], g[i + 7]);
            *reinterpret_cast<uint4*>(dst + i) = w;
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(GTMEM_COLS)
                 : "memory");
  }
}

// out[i] = sum over the splits of part[z][i], z in order
__global__ void k_split_sum(const float* __restrict__ part, int nsplit, size_t n,
                            float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float t = part[i];
    for (int z = 1; z < nsplit; z++) t += part[z * n + i];
    out[i] = t;
  }
}

// ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// [rows][cols] BF16 (row pitch cols), boxes of [128 rows][64 columns],
// 128-byte swizzle
bool encode_bf16(CUtensorMap* m, const void* base, int rows, int cols) {
  auto fn = encoder();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)BM};
  cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

size_t smem_bytes() { return 1024 + BIAS_OFF + 4 * BIAS_MAX; }

}  // namespace tc

bool tc_supported(const sed_surrogate* s) {
  // an even number of hidden layers: the last layer's first 256 outputs then
  // accumulate in region 0, away from the last hidden layer's region 1
  if (s->L < 3 || s->L > kSurMaxLayers || (s->L - 1) % 2) return false;
  if (s->pin[0] % tc::BK || s->pin[0] > tc::KMAX0) return false;
  for (int l = 0; l < s->L - 1; l++)
    if (s->pout[l] != tc::HID) return false;
  for (int l = 1; l < s->L; l++)
    if (s->pin[l] != tc::HID) return false;
  const int nlast = s->pout[s->L - 1];
  int nbias = 0;
  for (int l = 0; l < s->L; l++) nbias += s->pout[l];
  return nlast % 128 == 0 && nlast <= tc::TMEM_COLS && nbias <= tc::BIAS_MAX &&
         tc::encoder() != nullptr;
}

cudaError_t infer_tc(sed_surrogate* s, const __nv_bfloat16* x, float* y, int m, int* err,
                     cudaStream_t st, const unsigned* nrows) {
  // the output rows are written in 16-byte pieces, or in 32-byte pieces when
  // the rows start on 32-byte boundaries (the width is a multiple of 128)
  if (m <= 0 || m % tc::BM || !tc_supported(s) || reinterpret_cast<uintptr_t>(y) % 16)
    return cudaErrorInvalidValue;
  const bool y32 = reinterpret_cast<uintptr_t>(y) % 32 == 0;
  tc::Layers P{};
  P.L = s->L;
  P.k0 = s->pin[0];
  for (int l = 0; l < s->L; l++) {
    if (!tc::encode_bf16(&P.w[l], s->wb[l], s->pout[l], s->pin[l])) return cudaErrorInvalidValue;
    P.bias[l] = s->b[l];
    P.nout[l] = s->pout[l];
  }
  CUtensorMap tx;
  if (!tc::encode_bf16(&tx, x, m, s->pin[0])) return cudaErrorInvalidValue;
  const size_t smem = tc::smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(tc::k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int ntiles = m / tc::BM;
  const int grid = std::max(1, std::min(ntiles, sms));
  tc::k_mlp_tc<<<grid, tc::NTHREADS, smem, st>>>(tx, P, y, s->pout[s->L - 1], y32, ntiles,
                                                  nrows, err);
  return cudaGetLastError();
}

bool gemm_tc_supported() { return tc::encoder() != nullptr; }

cudaError_t gemm_tc(int epi, const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K,
                    const float* bias, float* out_f32, __nv_bfloat16* out_bf16,
                    const float* zprev, int ld_out, float* work, size_t work_floats, int* err,
                    cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0 || M % tc::BM || N % tc::GN || K % tc::BK || ld_out < N ||
      ld_out % 8)
    return cudaErrorInvalidValue;
  CUtensorMap ta, tb;
  if (!tc::encode_bf16(&ta, A, M, K) || !tc::encode_bf16(&tb, B, N, K))
    return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int nkc = K / tc::BK;
  const int tiles = (M / tc::BM) * (N / tc::GN);
  // the weight gradient (few output tiles, K = the batch) splits K over the
  // SMs, at least two K-chunks per split
  int splits = 1;
  if (epi == EPI_F32 && work && ld_out == N) {
    splits = std::max(1, std::min(nkc / 2, sms / tiles));
    while (splits > 1 && (size_t)splits * M * N > work_floats) splits--;
  }
  const int kps = (nkc + splits - 1) / splits;
  splits = (nkc + kps - 1) / kps;
  // the dynamic shared-memory limit, raised once per device and epilogue
  static unsigned char raised[64][5];
  if (epi < 0 || epi > 4) return cudaErrorInvalidValue;
  const dim3 grid(N / tc::GN, M / tc::BM, splits);
  float* dst = splits > 1 ? work : out_f32;
  const size_t stride = (size_t)M * N;
#define SUR_GEMM_TC_CASE(E)                                                                    \
  case E: {                                                                                   \
    if (dev < 64 && !raised[dev][E]) {                                                        \
      cudaError_t e = cudaFuncSetAttribute(tc::k_gemm_tc<E>,                                  \
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                           tc::GSMEM);                                        \
      if (e != cudaSuccess) return e;                                                         \
      raised[dev][E] = 1;                                                                     \
    }                                                                                         \
    tc::k_gemm_tc<E><<<grid, tc::GTHREADS, tc::GSMEM, st>>>(ta, tb, nkc, kps, bias, dst,      \
                                                           out_bf16, zprev, ld_out, stride,   \
                                                           err);                              \
    break;                                                                                    \
  }
  switch (epi) {
    SUR_GEMM_TC_CASE(EPI_BIAS_GELU)
    SUR_GEMM_TC_CASE(EPI_BIAS)
    SUR_GEMM_TC_CASE(EPI_F32)
    SUR_GEMM_TC_CASE(EPI_GELU_BWD)
    SUR_GEMM_TC_CASE(EPI_GELU)
  }
#undef SUR_GEMM_TC_CASE
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || splits == 1) return e;
  const int blocks = (int)std::min<size_t>((stride + 255) / 256, (size_t)4 * sms);
  tc::k_split_sum<<<blocks, 256, 0, st>>>(work, splits, stride, out_f32);
  return cudaGetLastError();
}

}  // namespace sur
