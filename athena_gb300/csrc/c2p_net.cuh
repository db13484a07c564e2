// The con2prim network shared by the learned-start kernels (sr_learned.cu) and the
// relativistic W(U) of the stage (kernels.cuh): sizes and parameter layout, the input
// features, and its evaluation for a tile of 128 cells on the fifth-generation tensor
// cores (tc_mlp.cuh).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "../../include/athena_gb300.h"
#include "tc_mlp.cuh"

namespace athgpu {
namespace c2pnet {

constexpr int NIN = 5, NH = 64, NOUT = 2;
// parameter layout (floats), ATHGPU_MLP_NPARAM in total
constexpr int OFF_W1 = 0;                    // [NH][NIN]
constexpr int OFF_B1 = OFF_W1 + NH * NIN;    // [NH]
constexpr int OFF_W2 = OFF_B1 + NH;          // [NH][NH]
constexpr int OFF_B2 = OFF_W2 + NH * NH;     // [NH]
constexpr int OFF_W3 = OFF_B2 + NH;          // [NOUT][NH]
constexpr int OFF_B3 = OFF_W3 + NOUT * NH;   // [NOUT]
constexpr int OFF_XM = OFF_B3 + NOUT;        // input means [NIN]
constexpr int OFF_XS = OFF_XM + NIN;         // input scales [NIN]
constexpr int OFF_YM = OFF_XS + NIN;         // output means [NOUT]
constexpr int OFF_YS = OFF_YM + NOUT;        // output scales [NOUT]
constexpr int NPARAM = OFF_YS + NOUT;
constexpr int NTRAIN = OFF_XM;               // trainable parameters
static_assert(NPARAM == ATHGPU_MLP_NPARAM, "header constant out of date");

// ---------------------------------------------------------------------------------------
// features: five scale-free invariants of (D, M, E, B)
//   log(D/E), log(M^2/E^2), log(B^2/E), (M.B)^2/(M^2 B^2), log((E - sqrt(M^2 + D^2))/E)
// The last is formed in FP64: for cold gas it is a small difference of large terms (three
// times the pressure for an unmagnetized cell at gamma 4/3), so it carries the pressure
// information that the other four lose to rounding.  The rest is FP32.
__device__ __forceinline__ void features(const double* u, const double* b, float* f) {
  const double D = u[0], E = u[4];
  const double msq = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
  const double rh = E - sqrt(msq + D * D);
  const float inv = 1.0f / (float)E;
  const float m1 = (float)u[1], m2 = (float)u[2], m3 = (float)u[3];
  const float b1 = (float)b[0], b2 = (float)b[1], b3 = (float)b[2];
  const float msqf = (float)msq;
  const float bsqf = b1 * b1 + b2 * b2 + b3 * b3;
  const float ttf = m1 * b1 + m2 * b2 + m3 * b3;
  f[0] = __logf((float)D * inv);
  f[1] = __logf(msqf * inv * inv + 1e-30f);
  f[2] = __logf(bsqf * inv + 1e-30f);
  f[3] = ttf * ttf / (msqf * bsqf + 1e-30f);
  f[4] = __logf(fmaxf((float)rh * inv, 1e-30f));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

// ---------------------------------------------------------------------------------------
// tcgen05 evaluation of the network (tc_mlp.cuh): operands and TMEM bookkeeping of a CTA.
struct TcNet {
  __align__(128) unsigned char w1[NH * 16 * 2];   // B of layer 1: N = 64 rows, K = 16
  __align__(128) unsigned char w2[NH * NH * 2];   // B of layer 2: N = 64, K = 64
  __align__(128) unsigned char w3[16 * NH * 2];   // B of layer 3: N = 16 (2 used), K = 64
  __align__(128) unsigned char a1[tc::M * 16 * 2];   // A of layer 1: the features
  __align__(128) unsigned char a2[tc::M * NH * 2];   // A of layers 2 and 3
  float b1[NH], b2[NH], b3[16];
  float xm[NIN], xs[NIN], ym[NOUT], ys[NOUT];
  unsigned long long mbar;
  uint32_t taddr;
  int ok;
};

__device__ __forceinline__ void put_bf16(unsigned char* tile, int r, int k, int kdim, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + tc::kmajor_off(r, k, kdim)) = __float2bfloat16(v);
}

// weights into the K-major tiles, TMEM allocation (warp 0), mbarrier; all threads call it
static __device__ void tc_setup(const float* __restrict__ p, TcNet& s) {
  for (int q = threadIdx.x; q < NH * 16; q += blockDim.x) {
    const int o = q / 16, k = q % 16;
    put_bf16(s.w1, o, k, 16, k < NIN ? p[OFF_W1 + o * NIN + k] : 0.0f);
  }
  for (int q = threadIdx.x; q < NH * NH; q += blockDim.x)
    put_bf16(s.w2, q / NH, q % NH, NH, p[OFF_W2 + q]);
  for (int q = threadIdx.x; q < 16 * NH; q += blockDim.x) {
    const int o = q / NH, k = q % NH;
    put_bf16(s.w3, o, k, NH, o < NOUT ? p[OFF_W3 + o * NH + k] : 0.0f);
  }
  for (int q = threadIdx.x; q < NH; q += blockDim.x) {
    s.b1[q] = p[OFF_B1 + q];
    s.b2[q] = p[OFF_B2 + q];
  }
  if (threadIdx.x < 16) s.b3[threadIdx.x] = threadIdx.x < NOUT ? p[OFF_B3 + threadIdx.x] : 0.0f;
  if (threadIdx.x < NIN) {
    s.xm[threadIdx.x] = p[OFF_XM + threadIdx.x];
    s.xs[threadIdx.x] = p[OFF_XS + threadIdx.x];
  }
  if (threadIdx.x < NOUT) {
    s.ym[threadIdx.x] = p[OFF_YM + threadIdx.x];
    s.ys[threadIdx.x] = p[OFF_YS + threadIdx.x];
  }
  if (threadIdx.x == 0) {
    tc::mbar_init(tc::smem_u32(&s.mbar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    s.ok = 1;
  }
  if (threadIdx.x < 32) tc::tmem_alloc(tc::smem_u32(&s.taddr), tc::TMEM_COLS);
  tc::fence_async_smem();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
}

static __device__ void tc_teardown(TcNet& s) {
  tc::fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after();
    tc::tmem_dealloc(s.taddr, tc::TMEM_COLS);
  }
}

// one tcgen05 group: thread 0 issues the MMAs and the commit, everyone waits (bounded by
// SM clock, skipped once an error is flagged anywhere).  Returns the CTA-uniform outcome.
__device__ __forceinline__ bool tc_run(TcNet& s, int layer, uint32_t& phase,
                                       int* __restrict__ err) {
  tc::fence_async_smem();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const bool live = s.ok != 0;  // read after the barrier: the same in every thread
  const uint32_t t = s.taddr;
  if (threadIdx.x == 0 && live) {
    const uint32_t a1 = tc::smem_u32(s.a1), a2 = tc::smem_u32(s.a2);
    if (layer == 1) {
      tc::mma_bf16(t, tc::smem_desc(a1, tc::LBO, 256), tc::smem_desc(tc::smem_u32(s.w1),
                   tc::LBO, 256), tc::idesc_bf16(tc::M, NH), 0);
    } else {
      const uint32_t w = tc::smem_u32(layer == 2 ? s.w2 : s.w3);
      const uint32_t d = layer == 2 ? t + NH : t;  // layer 2 -> columns [64,128)
      const uint32_t id = tc::idesc_bf16(tc::M, layer == 2 ? NH : 16);
#pragma unroll
      for (int kk = 0; kk < NH / 16; ++kk)  // K = 64 in steps of 16 (two core matrices)
        tc::mma_bf16(d, tc::smem_desc(a2 + kk * 2 * tc::LBO, tc::LBO, 1024),
                     tc::smem_desc(w + kk * 2 * tc::LBO, tc::LBO, 1024), id, kk > 0);
    }
    tc::commit(tc::smem_u32(&s.mbar));
  }
  bool ok = false;
  if (live) {
    const long long t0 = clock64();
    while (!(ok = tc::mbar_try(tc::smem_u32(&s.mbar), phase))) {
      if (clock64() - t0 > 200000000LL || *(volatile int*)err != 0) break;
    }
  }
  phase ^= 1u;
  ok = __syncthreads_and(ok) != 0;
  if (!ok && threadIdx.x == 0) {
    if (live) atomicExch(err, 1);
    s.ok = 0;  // read by the next call after its barrier
  }
  tc::fence_after();
  return ok;
}

// hidden layer read-out: columns [col0, col0+64) of this thread's lane, + bias, SiLU,
// BF16 row of the next A operand (16 columns at a time to keep registers low)
__device__ __forceinline__ void tc_hidden(TcNet& s, uint32_t col0, const float* bias) {
  const uint32_t lane = (uint32_t)(threadIdx.x & ~31) << 16;
#pragma unroll 1
  for (int q = 0; q < NH / 16; ++q) {
    float v[16];
    tc::tmem_ld16(s.taddr + lane + col0 + 16 * q, v);
    uint32_t pk[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      __nv_bfloat162 h = __floats2bfloat162_rn(silu(v[2 * e] + bias[16 * q + 2 * e]),
                                               silu(v[2 * e + 1] + bias[16 * q + 2 * e + 1]));
      pk[e] = *reinterpret_cast<uint32_t*>(&h);
    }
    const int r = threadIdx.x;
    *reinterpret_cast<uint4*>(s.a2 + tc::kmajor_off(r, 16 * q, NH)) =
        make_uint4(pk[0], pk[1], pk[2], pk[3]);
    *reinterpret_cast<uint4*>(s.a2 + tc::kmajor_off(r, 16 * q + 8, NH)) =
        make_uint4(pk[4], pk[5], pk[6], pk[7]);
  }
}

// The network for the CTA's 128 cells (thread t: standardized features xin of cell t);
// every thread of the CTA must call it.  Returns the de-standardized outputs.
static __device__ void tc_infer_tile(TcNet& s, const float* xin, float* y, uint32_t& phase,
                              int* __restrict__ err) {
  {  // A of layer 1: row t = the 5 features, zero-padded to K = 16
    const int r = threadIdx.x;
    __nv_bfloat162 h0 = __floats2bfloat162_rn(xin[0], xin[1]);
    __nv_bfloat162 h1 = __floats2bfloat162_rn(xin[2], xin[3]);
    __nv_bfloat162 h2 = __floats2bfloat162_rn(xin[4], 0.0f);
    *reinterpret_cast<uint4*>(s.a1 + tc::kmajor_off(r, 0, 16)) =
        make_uint4(*reinterpret_cast<uint32_t*>(&h0), *reinterpret_cast<uint32_t*>(&h1),
                   *reinterpret_cast<uint32_t*>(&h2), 0u);
    *reinterpret_cast<uint4*>(s.a1 + tc::kmajor_off(r, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
  }
  bool ok = tc_run(s, 1, phase, err);
  if (ok) tc_hidden(s, 0, s.b1);
  ok = tc_run(s, 2, phase, err);
  if (ok) tc_hidden(s, NH, s.b2);
  ok = tc_run(s, 3, phase, err);
  float v[16];
  if (ok) {
    tc::tmem_ld16(s.taddr + ((uint32_t)(threadIdx.x & ~31) << 16), v);
  } else {
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __int_as_float(0x7fc00000);  // NaN: no result
  }
#pragma unroll
  for (int q = 0; q < NOUT; ++q) y[q] = (v[q] + s.b3[q]) * s.ys[q] + s.ym[q];
}

// shared memory added to the tcgen05 kernels' launch so that at most four CTAs (4 x 128
// TMEM columns) are resident on an SM: 4 x (33.5 + 21 + 1 reserved) KB fits the SM's
// 228 KB, five do not
constexpr int TC_SMEM_PAD = 21 * 1024;

}  // namespace c2pnet
}  // namespace athgpu
