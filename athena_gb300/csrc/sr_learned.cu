// Learned initial guess for the SR-MHD conserved->primitive solve.
//
// A 5 -> 64 -> 64 -> 2 multilayer perceptron with SiLU activations predicts, from five
// dimensionless invariants of a cell's conserved state, the gas pressure and the Lorentz
// factor of its solution.  Training runs on the GPU with the hand-written FP32 kernels
// below (forward, backward, weight gradients, Adam) on (conserved -> primitive) pairs that
// the FP64 Newman-Hamlin solver produces.  Inference is fused into the per-cell solve:
// each warp evaluates the network for its 32 cells with BF16 mma.sync tensor-core tiles
// (FP32 accumulation), optionally refines the guess with the same fixed-point iteration in
// FP32, and finishes with the reference's FP64 solve (adiabatic_mhd_sr.cpp:404-522).  A
// cell whose learned start does not converge within the solver's 15-iteration budget is
// solved again from the standard start, so the learned guess never changes which cells
// converge.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <float.h>

#include <string>
#include <vector>

#include "../../include/athena_gb300.h"
#include "physics.cuh"
#include "tc_mlp.cuh"
#include "c2p_net.cuh"

namespace athgpu {
void set_last_error(const std::string& msg);  // api.cu
}

namespace {

using athgpu::IDN;
using athgpu::IPR;
using athgpu::IVX;
using athgpu::IVY;
using athgpu::IVZ;
namespace tc = athgpu::tc;
using namespace athgpu::c2pnet;

// network sizes and parameter layout (NIN, NH, NOUT, OFF_*, NPARAM, NTRAIN): c2p_net.cuh

athgpu_status fail(athgpu_status s, const std::string& m) {
  athgpu::set_last_error(m);
  return s;
}
#define CKE(call)                                                                   \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(ATHGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// ---------------------------------------------------------------------------------------
// features() and silu(): c2p_net.cuh
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s + z * s * (1.0f - s);
}

// ---------------------------------------------------------------------------------------
// training kernels (FP32).  A batch of B samples: x [B][NIN] (standardized),
// t [B][NOUT] (standardized targets).
__global__ void __launch_bounds__(128)
mlp_forward_kernel(const float* __restrict__ p, const float* __restrict__ x,
                   const float* __restrict__ t, int B, float* __restrict__ z1,
                   float* __restrict__ z2, float* __restrict__ y, float* __restrict__ loss) {
  __shared__ float w[NTRAIN];
  for (int q = threadIdx.x; q < NTRAIN; q += blockDim.x) w[q] = p[q];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (s < B) {
    float xi[NIN], h1[NH];
#pragma unroll
    for (int k = 0; k < NIN; ++k) xi[k] = x[(long long)s * NIN + k];
    for (int o = 0; o < NH; ++o) {
      float a = w[OFF_B1 + o];
#pragma unroll
      for (int k = 0; k < NIN; ++k) a += w[OFF_W1 + o * NIN + k] * xi[k];
      z1[(long long)s * NH + o] = a;
      h1[o] = silu(a);
    }
    float yo[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; ++o) yo[o] = w[OFF_B3 + o];
    for (int o = 0; o < NH; ++o) {
      float a = w[OFF_B2 + o];
      for (int k = 0; k < NH; ++k) a += w[OFF_W2 + o * NH + k] * h1[k];
      z2[(long long)s * NH + o] = a;
      const float h = silu(a);
#pragma unroll
      for (int q = 0; q < NOUT; ++q) yo[q] += w[OFF_W3 + q * NH + o] * h;
    }
#pragma unroll
    for (int q = 0; q < NOUT; ++q) {
      y[(long long)s * NOUT + q] = yo[q];
      const float d = yo[q] - t[(long long)s * NOUT + q];
      l += d * d;
    }
  }
  // mean squared error over the batch and the outputs
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l / (float)(B * NOUT));
}

// per-sample back-propagation to the pre-activations: dy [B][NOUT], dz2 [B][NH],
// dz1 [B][NH] (loss = mean over batch and outputs of (y - t)^2)
__global__ void __launch_bounds__(128)
mlp_backward_kernel(const float* __restrict__ p, const float* __restrict__ t, int B,
                    const float* __restrict__ z1, const float* __restrict__ z2,
                    const float* __restrict__ y, float* __restrict__ dy,
                    float* __restrict__ dz2, float* __restrict__ dz1) {
  __shared__ float w[NTRAIN];
  for (int q = threadIdx.x; q < NTRAIN; q += blockDim.x) w[q] = p[q];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  float g[NOUT];
#pragma unroll
  for (int q = 0; q < NOUT; ++q) {
    g[q] = 2.0f * (y[(long long)s * NOUT + q] - t[(long long)s * NOUT + q]) / (float)(B * NOUT);
    dy[(long long)s * NOUT + q] = g[q];
  }
  float d2[NH];
  for (int o = 0; o < NH; ++o) {
    float dh = 0.0f;
#pragma unroll
    for (int q = 0; q < NOUT; ++q) dh += w[OFF_W3 + q * NH + o] * g[q];
    d2[o] = dh * dsilu(z2[(long long)s * NH + o]);
    dz2[(long long)s * NH + o] = d2[o];
  }
  for (int k = 0; k < NH; ++k) {
    float dh = 0.0f;
    for (int o = 0; o < NH; ++o) dh += w[OFF_W2 + o * NH + k] * d2[o];
    dz1[(long long)s * NH + k] = dh * dsilu(z1[(long long)s * NH + k]);
  }
}

// weight gradients as batch reductions: dW1 = dZ1^T X, dW2 = dZ2^T silu(Z1),
// dW3 = dY^T silu(Z2), db = column sums.  Thread x = one trainable parameter, block row y
// = one chunk of WG_CHUNK batch rows, partial sums added into grad (zeroed before).
constexpr int WG_CHUNK = 256;
__global__ void __launch_bounds__(128)
mlp_wgrad_kernel(const float* __restrict__ x, int B, const float* __restrict__ z1,
                 const float* __restrict__ z2, const float* __restrict__ dy,
                 const float* __restrict__ dz2, const float* __restrict__ dz1,
                 float* __restrict__ grad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= NTRAIN) return;
  const int s0 = blockIdx.y * WG_CHUNK;
  const int s1 = min(B, s0 + WG_CHUNK);
  float acc = 0.0f;
  if (q < OFF_B1) {
    const int o = q / NIN, k = q % NIN;
    for (int s = s0; s < s1; ++s) acc += dz1[(long long)s * NH + o] * x[(long long)s * NIN + k];
  } else if (q < OFF_W2) {
    const int o = q - OFF_B1;
    for (int s = s0; s < s1; ++s) acc += dz1[(long long)s * NH + o];
  } else if (q < OFF_B2) {
    const int o = (q - OFF_W2) / NH, k = (q - OFF_W2) % NH;
    for (int s = s0; s < s1; ++s)
      acc += dz2[(long long)s * NH + o] * silu(z1[(long long)s * NH + k]);
  } else if (q < OFF_W3) {
    const int o = q - OFF_B2;
    for (int s = s0; s < s1; ++s) acc += dz2[(long long)s * NH + o];
  } else if (q < OFF_B3) {
    const int o = (q - OFF_W3) / NH, k = (q - OFF_W3) % NH;
    for (int s = s0; s < s1; ++s)
      acc += dy[(long long)s * NOUT + o] * silu(z2[(long long)s * NH + k]);
  } else {
    const int o = q - OFF_B3;
    for (int s = s0; s < s1; ++s) acc += dy[(long long)s * NOUT + o];
  }
  atomicAdd(grad + q, acc);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, int step, float lr,
                            float b1, float b2, float eps) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= NTRAIN) return;
  const float gq = g[q];
  const float mq = b1 * m[q] + (1.0f - b1) * gq;
  const float vq = b2 * v[q] + (1.0f - b2) * gq * gq;
  m[q] = mq;
  v[q] = vq;
  const float mh = mq / (1.0f - powf(b1, (float)step));
  const float vh = vq / (1.0f - powf(b2, (float)step));
  p[q] -= lr * mh / (sqrtf(vh) + eps);
}

// gather a mini-batch: x = (features - mean)/scale, t = (targets - mean)/scale
__global__ void gather_batch_kernel(const float* __restrict__ p, const float* __restrict__ fx,
                                    const float* __restrict__ fy,
                                    const unsigned* __restrict__ idx, int B,
                                    float* __restrict__ x, float* __restrict__ t) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  const unsigned r = idx[s];
#pragma unroll
  for (int k = 0; k < NIN; ++k)
    x[(long long)s * NIN + k] = (fx[(long long)r * NIN + k] - p[OFF_XM + k]) / p[OFF_XS + k];
#pragma unroll
  for (int q = 0; q < NOUT; ++q)
    t[(long long)s * NOUT + q] = (fy[(long long)r * NOUT + q] - p[OFF_YM + q]) / p[OFF_YS + q];
}

// xorshift indices for mini-batches (sampling with replacement)
__global__ void batch_indices_kernel(unsigned long long seed, int step, unsigned n, int B,
                                     unsigned* __restrict__ idx) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  unsigned long long z = seed ^ (0x9E3779B97F4A7C15ULL * (unsigned long long)(step * B + s + 1));
  z ^= z >> 30; z *= 0xBF58476D1CE4E5B9ULL;
  z ^= z >> 27; z *= 0x94D049BB133111EBULL;
  z ^= z >> 31;
  idx[s] = (unsigned)(z % n);
}

// ---------------------------------------------------------------------------------------
// BF16 tensor-core inference, one warp per 32 cells (two 16-row tiles).
// mma.m16n8k16 (row.col, bf16 x bf16 -> f32): lane = 4g + t holds A rows g, g+8 at
// columns 2t, 2t+1 (and +8), B column g at rows 2t, 2t+1 (and +8), C rows g, g+8 at
// columns 2t, 2t+1.  The C fragments of two adjacent 8-wide n tiles are exactly the A
// fragment of the next layer's 16-wide k slice, so activations never leave registers.
__device__ __forceinline__ void mma_bf16(float* c, const unsigned* a, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned*>(&v);
}

struct SmemNet {
  __nv_bfloat16 w1[NH][16];      // [out][in], inputs padded to 16
  __nv_bfloat16 w2[NH][NH];      // [out][in]
  __nv_bfloat16 w3[8][NH];       // [out padded to 8][in]
  float b1[NH], b2[NH], b3[8];
  float xm[NIN], xs[NIN], ym[NOUT], ys[NOUT];
};

__device__ void load_net(const float* __restrict__ p, SmemNet& s) {
  for (int q = threadIdx.x; q < NH * 16; q += blockDim.x) {
    const int o = q / 16, k = q % 16;
    s.w1[o][k] = __float2bfloat16(k < NIN ? p[OFF_W1 + o * NIN + k] : 0.0f);
  }
  for (int q = threadIdx.x; q < NH * NH; q += blockDim.x)
    s.w2[q / NH][q % NH] = __float2bfloat16(p[OFF_W2 + q]);
  for (int q = threadIdx.x; q < 8 * NH; q += blockDim.x) {
    const int o = q / NH, k = q % NH;
    s.w3[o][k] = __float2bfloat16(o < NOUT ? p[OFF_W3 + o * NH + k] : 0.0f);
  }
  for (int q = threadIdx.x; q < NH; q += blockDim.x) {
    s.b1[q] = p[OFF_B1 + q];
    s.b2[q] = p[OFF_B2 + q];
  }
  if (threadIdx.x < 8) s.b3[threadIdx.x] = threadIdx.x < NOUT ? p[OFF_B3 + threadIdx.x] : 0.0f;
  if (threadIdx.x < NIN) {
    s.xm[threadIdx.x] = p[OFF_XM + threadIdx.x];
    s.xs[threadIdx.x] = p[OFF_XS + threadIdx.x];
  }
  if (threadIdx.x < NOUT) {
    s.ym[threadIdx.x] = p[OFF_YM + threadIdx.x];
    s.ys[threadIdx.x] = p[OFF_YS + threadIdx.x];
  }
}

// The warp's 32 lanes each hold the standardized features xin[NIN] of one cell; returns,
// in every lane, the network's (de-standardized) outputs for that lane's cell.
__device__ void mlp_infer_warp(const SmemNet& s, const float* xin, float* yout) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float res0 = 0.0f, res1 = 0.0f;
#pragma unroll
  for (int tile = 0; tile < 2; ++tile) {
    // A fragment of the 16 x 16 (zero padded) input tile: rows g, g+8 of this tile
    const int ra = tile * 16 + g, rb = tile * 16 + g + 8;
    float fa[NIN], fb[NIN];
#pragma unroll
    for (int k = 0; k < NIN; ++k) {
      fa[k] = __shfl_sync(0xffffffffu, xin[k], ra);
      fb[k] = __shfl_sync(0xffffffffu, xin[k], rb);
    }
    auto feat = [&](const float* f, int col) -> float {
      float v = 0.0f;
#pragma unroll
      for (int k = 0; k < NIN; ++k) v = (col == k) ? f[k] : v;
      return v;
    };
    unsigned a[4];
    a[0] = pack_bf16(feat(fa, 2 * t), feat(fa, 2 * t + 1));
    a[1] = pack_bf16(feat(fb, 2 * t), feat(fb, 2 * t + 1));
    a[2] = 0u;  // columns 8..15 are padding
    a[3] = 0u;
    // layer 1: 8 n-tiles of 8 hidden units
    float c1[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      c1[j][0] = c1[j][1] = c1[j][2] = c1[j][3] = 0.0f;
      const unsigned b0 = *reinterpret_cast<const unsigned*>(&s.w1[8 * j + g][2 * t]);
      const unsigned b1 = *reinterpret_cast<const unsigned*>(&s.w1[8 * j + g][2 * t + 8]);
      mma_bf16(c1[j], a, b0, b1);
      const float bb0 = s.b1[8 * j + 2 * t], bb1 = s.b1[8 * j + 2 * t + 1];
      c1[j][0] = silu(c1[j][0] + bb0);
      c1[j][1] = silu(c1[j][1] + bb1);
      c1[j][2] = silu(c1[j][2] + bb0);
      c1[j][3] = silu(c1[j][3] + bb1);
    }
    // layer 2: k = 64 in 4 slices, 8 n-tiles
    float c2[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) c2[j][0] = c2[j][1] = c2[j][2] = c2[j][3] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      unsigned a2[4];
      a2[0] = pack_bf16(c1[2 * ks][0], c1[2 * ks][1]);
      a2[1] = pack_bf16(c1[2 * ks][2], c1[2 * ks][3]);
      a2[2] = pack_bf16(c1[2 * ks + 1][0], c1[2 * ks + 1][1]);
      a2[3] = pack_bf16(c1[2 * ks + 1][2], c1[2 * ks + 1][3]);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const unsigned b0 = *reinterpret_cast<const unsigned*>(&s.w2[8 * j + g][16 * ks + 2 * t]);
        const unsigned b1 =
            *reinterpret_cast<const unsigned*>(&s.w2[8 * j + g][16 * ks + 2 * t + 8]);
        mma_bf16(c2[j], a2, b0, b1);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float bb0 = s.b2[8 * j + 2 * t], bb1 = s.b2[8 * j + 2 * t + 1];
      c2[j][0] = silu(c2[j][0] + bb0);
      c2[j][1] = silu(c2[j][1] + bb1);
      c2[j][2] = silu(c2[j][2] + bb0);
      c2[j][3] = silu(c2[j][3] + bb1);
    }
    // layer 3: 2 outputs in one 8-wide n-tile
    float c3[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      unsigned a3[4];
      a3[0] = pack_bf16(c2[2 * ks][0], c2[2 * ks][1]);
      a3[1] = pack_bf16(c2[2 * ks][2], c2[2 * ks][3]);
      a3[2] = pack_bf16(c2[2 * ks + 1][0], c2[2 * ks + 1][1]);
      a3[3] = pack_bf16(c2[2 * ks + 1][2], c2[2 * ks + 1][3]);
      const unsigned b0 = *reinterpret_cast<const unsigned*>(&s.w3[g][16 * ks + 2 * t]);
      const unsigned b1 = *reinterpret_cast<const unsigned*>(&s.w3[g][16 * ks + 2 * t + 8]);
      mma_bf16(c3, a3, b0, b1);
    }
    // outputs 0, 1 of rows g (c3[0..1]) and g+8 (c3[2..3]) sit in lanes with t = 0
    const int r = lane - tile * 16;  // this lane's row in the tile, if it belongs to it
    const int src = 4 * (r & 7);
    const float o0a = __shfl_sync(0xffffffffu, c3[0], src);
    const float o1a = __shfl_sync(0xffffffffu, c3[1], src);
    const float o0b = __shfl_sync(0xffffffffu, c3[2], src);
    const float o1b = __shfl_sync(0xffffffffu, c3[3], src);
    if (r >= 0 && r < 16) {
      res0 = (r < 8 ? o0a : o0b) + s.b3[0];
      res1 = (r < 8 ? o1a : o1b) + s.b3[1];
    }
  }
  yout[0] = res0 * s.ys[0] + s.ym[0];
  yout[1] = res1 * s.ys[1] + s.ym[1];
}

// ---------------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------------
// tcgen05 evaluation of the network: c2p_net.cuh (TcNet, tc_setup, tc_infer_tile, ...)

// Per-cell SR con2prim on independent cells: the Newman-Hamlin root find of
// ConservedToPrimitiveNormal (adiabatic_mhd_sr.cpp:404-522) from three kinds of start.
// mode 0: pgas_guess[c] (the reference's start, max(previous pressure, floor),
// adiabatic_mhd_sr.cpp:143-154), or the floor when pgas_guess is NULL; mode 1: the
// learned start; mode 2: the learned start refined by FP32 iterations of the same scheme.
//
// Warp-coherent two-phase schedule: the iteration count varies from cell to cell and a
// warp runs as long as its slowest lane, so phase 1 runs loop indices [0, n1) for every
// cell and appends each cell still iterating to a queue together with its whole solver
// state (pgas[3] and the loop index: the iteration resumes exactly where it stopped);
// phase 2 finishes the queued cells in a grid-stride loop.  Mode 0 is then the reference's
// solve, index for index.  Modes 1-2 add the fallback: a learned start that does not
// converge within the reference's 15 iterations is solved again from the mode-0 start,
// and if that fails too, from the last iterate of the learned attempt.
constexpr int MAXIT = 15;
constexpr double TOL = 1.0e-12;

struct Queue {
  long long* cell;
  int* state;        // loop index | attempt << 8 | FP64 passes so far << 16
  double* p;         // pgas[3] per entry
  unsigned* count;
};

struct Cell {
  double dd, ee, mm1, mm2, mm3, mm_sq, b1, b2, b3, bb_sq, tt, d, pgas_min;
};

__device__ __forceinline__ Cell load_cell(const double* __restrict__ cons,
                                          const double* __restrict__ bcc, long long c,
                                          bool valid) {
  Cell q;
  double u[5] = {1.0, 0.0, 0.0, 0.0, 2.0}, b[3] = {0.0, 0.0, 0.0};
  if (valid) {
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = cons[c * 5 + v];
#pragma unroll
    for (int v = 0; v < 3; ++v) b[v] = bcc[c * 3 + v];
  }
  q.dd = u[0]; q.mm1 = u[1]; q.mm2 = u[2]; q.mm3 = u[3]; q.ee = u[4];
  q.b1 = b[0]; q.b2 = b[1]; q.b3 = b[2];
  // operand order of adiabatic_mhd_sr.cpp:108-123
  q.mm_sq = q.mm1 * q.mm1 + q.mm2 * q.mm2 + q.mm3 * q.mm3;
  q.bb_sq = q.b1 * q.b1 + q.b2 * q.b2 + q.b3 * q.b3;
  q.tt = q.mm1 * q.b1 + q.mm2 * q.b2 + q.mm3 * q.b3;
  athgpu::sr_nh_setup<double>(q.ee, q.mm_sq, q.bb_sq, q.tt, &q.d, &q.pgas_min);
  return q;
}

__device__ __forceinline__ int run64(const Cell& q, double gamma, double* pgas, int n0, int n1,
                                     double* last) {
  return athgpu::sr_nh_loop<double>(gamma, q.dd, q.ee, q.mm_sq, q.bb_sq, q.tt, q.d, q.pgas_min,
                                    pgas, n0, n1, TOL, false, last);
}

__device__ __forceinline__ bool finish64(const Cell& q, double p, double* prim) {
  double gl, pm;
  return athgpu::sr_nh_finish<double>(q.dd, q.ee, q.mm_sq, q.mm1, q.mm2, q.mm3, q.bb_sq, q.b1,
                                      q.b2, q.b3, q.tt, q.d, p, prim, &gl, &pm);
}

__device__ __forceinline__ void store(double* __restrict__ prim, long long c, const double* pr) {
#pragma unroll
  for (int v = 0; v < 5; ++v) prim[c * 5 + v] = pr[v];
}

// The fallback chain of modes 1-2 after the learned attempt failed: the mode-0 start,
// then the learned attempt's last iterate.  Returns total FP64 passes (<0: not converged).
__device__ int fallback_chain(const Cell& q, double gamma, double pstd, double plast,
                              double* pr, int passes) {
  const double starts[2] = {pstd, plast};
#pragma unroll 1
  for (int a = 0; a < 2; ++a) {
#pragma unroll
    for (int v = 0; v < 5; ++v) pr[v] = 0.0;
    double pg[3], last = 0.0;
    pg[0] = fmax(starts[a], q.pgas_min);
    const int n = run64(q, gamma, pg, 0, MAXIT, &last);
    passes += n < MAXIT ? n + 1 : MAXIT;
    if (n < MAXIT && finish64(q, pg[(n + 1) % 3], pr)) return passes;
  }
  return -passes;
}

template <bool TC>
__global__ void __launch_bounds__(128)
sr_c2p_phase1_kernel(long long n, double gamma, double pfloor, const double* __restrict__ cons,
                     const double* __restrict__ bcc, const double* __restrict__ pgas_guess,
                     const float* __restrict__ params, int mode, int n1,
                     double* __restrict__ prim, int* __restrict__ iters64,
                     int* __restrict__ iters32, int* __restrict__ fallbacks, Queue qu,
                     int* __restrict__ tc_err) {
  // the network's operands: SmemNet for the warp-level mma.sync path, TcNet for tcgen05
  extern __shared__ __align__(128) unsigned char phase1_smem[];
  SmemNet& net = *reinterpret_cast<SmemNet*>(phase1_smem);
  TcNet& tnet = *reinterpret_cast<TcNet*>(phase1_smem);
  const bool use_net = mode == 1 || mode == 2;
  if (use_net) {
    if (TC) {
      tc_setup(params, tnet);
    } else {
      load_net(params, net);
      __syncthreads();
    }
  }
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = c < n;
  const Cell q = load_cell(cons, bcc, c, valid);
  const double pstd = (valid && pgas_guess) ? pgas_guess[c] : pfloor;
  double guess = pstd;
  int it32 = 0;
  if (use_net) {  // the whole warp takes part in the tensor-core evaluation
    float f[NIN], xin[NIN], y[NOUT];
    const double uu[5] = {q.dd, q.mm1, q.mm2, q.mm3, q.ee}, bb[3] = {q.b1, q.b2, q.b3};
    features(uu, bb, f);
    if (TC) {
#pragma unroll
      for (int k = 0; k < NIN; ++k) xin[k] = (f[k] - tnet.xm[k]) / tnet.xs[k];
      uint32_t ph = 0;
      tc_infer_tile(tnet, xin, y, ph, tc_err);  // the CTA's 128 cells on tcgen05
      tc_teardown(tnet);
    } else {
#pragma unroll
      for (int k = 0; k < NIN; ++k) xin[k] = (f[k] - net.xm[k]) / net.xs[k];
      mlp_infer_warp(net, xin, y);
    }
    guess = q.ee * (double)__expf(y[0]);
    if (mode == 2 && valid)  // FP32 iterations of the same scheme; the last iterate is kept
      guess = athgpu::sr_refine_f32(gamma, q.dd, q.ee, q.mm_sq, q.bb_sq, q.tt, guess, 12,
                                    1.0e-6f, &it32);
    if (!(guess > pfloor)) guess = pfloor;
  } else if (mode == 3 && valid) {  // the mode-0 start refined in FP32
    guess = athgpu::sr_refine_f32(gamma, q.dd, q.ee, q.mm_sq, q.bb_sq, q.tt, pstd, 12,
                                  1.0e-6f, &it32);
    if (!(guess > pfloor)) guess = pfloor;
  }
  double pg[3], last = guess, pr[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  bool enqueue = false;
  int attempt = 0, passes = 0, nstop = 0;
  if (valid) {
    pg[0] = fmax(guess, q.pgas_min);
    const int k = run64(q, gamma, pg, 0, n1, &last);
    if (k < n1) {  // converged in phase 1
      passes = k + 1;
      if (finish64(q, pg[(k + 1) % 3], pr)) {
        store(prim, c, pr);
        iters64[c] = passes;
      } else if (mode == 0) {
        store(prim, c, pr);
        iters64[c] = -1;
      } else {
        enqueue = true;   // go straight to the fallback chain
        attempt = 1;
      }
    } else if (n1 >= MAXIT) {
      passes = MAXIT;
      if (mode == 0) {
        store(prim, c, pr);
        iters64[c] = -1;
      } else {
        enqueue = true;
        attempt = 1;
      }
    } else {
      passes = n1;
      nstop = n1;
      enqueue = true;
    }
    if (iters32) iters32[c] = it32;
  }
  // warp-aggregated append to the queue
  const unsigned mask = __ballot_sync(0xffffffffu, enqueue);
  if (mask) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(qu.count, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (enqueue) {
      const unsigned slot = base + __popc(mask & ((1u << lane) - 1u));
      qu.cell[slot] = c;
      qu.state[slot] = nstop | (attempt << 8) | (passes << 16);
      qu.p[3 * (long long)slot + 0] = attempt ? last : pg[0];
      qu.p[3 * (long long)slot + 1] = pg[1];
      qu.p[3 * (long long)slot + 2] = pg[2];
      if (attempt && fallbacks) atomicAdd(fallbacks, 1);
    }
  }
}

__global__ void __launch_bounds__(128)
sr_c2p_phase2_kernel(double gamma, double pfloor, const double* __restrict__ cons,
                     const double* __restrict__ bcc, const double* __restrict__ pgas_guess,
                     int mode, double* __restrict__ prim, int* __restrict__ iters64,
                     int* __restrict__ fallbacks, Queue qu) {
  const unsigned total = *qu.count;
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    const long long c = qu.cell[e];
    const int st = qu.state[e];
    int n0 = st & 0xff, attempt = (st >> 8) & 0xff, passes = st >> 16;
    const Cell q = load_cell(cons, bcc, c, true);
    const double pstd = pgas_guess ? pgas_guess[c] : pfloor;
    double pr[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    double pg[3] = {qu.p[3 * (long long)e], qu.p[3 * (long long)e + 1],
                    qu.p[3 * (long long)e + 2]};
    double last = pg[0];
    int result;
    if (attempt == 0) {  // resume the first attempt at loop index n0
      const int k = run64(q, gamma, pg, n0, MAXIT, &last);
      passes += k < MAXIT ? k - n0 + 1 : MAXIT - n0;
      if (k < MAXIT && finish64(q, pg[(k + 1) % 3], pr)) {
        result = passes;
      } else if (mode == 0) {
        result = -1;
      } else {
        if (fallbacks) atomicAdd(fallbacks, 1);
        result = fallback_chain(q, gamma, pstd, last, pr, passes);
      }
    } else {
      result = fallback_chain(q, gamma, pstd, last, pr, passes);
    }
    store(prim, c, pr);
    iters64[c] = result > 0 ? result : -1;
  }
}

// network outputs for n feature rows (raw features, standardized inside)
__global__ void __launch_bounds__(128)
mlp_infer_kernel(long long n, const float* __restrict__ params, const float* __restrict__ fx,
                 float* __restrict__ out) {
  __shared__ SmemNet net;
  load_net(params, net);
  __syncthreads();
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float xin[NIN], y[NOUT];
#pragma unroll
  for (int k = 0; k < NIN; ++k) xin[k] = c < n ? (fx[c * NIN + k] - net.xm[k]) / net.xs[k] : 0.0f;
  mlp_infer_warp(net, xin, y);
  if (c < n) {
#pragma unroll
    for (int q = 0; q < NOUT; ++q) out[c * NOUT + q] = y[q];
  }
}

__global__ void sr_features_kernel(long long n, const double* __restrict__ cons,
                                   const double* __restrict__ bcc, float* __restrict__ fx) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  features(cons + c * 5, bcc + c * 3, fx + c * NIN);
}


// network outputs for n feature rows on the tcgen05 path: persistent CTAs of 128 threads
// over 128-row tiles
__global__ void __launch_bounds__(128)
mlp_infer_tc_kernel(long long n, const float* __restrict__ params,
                    const float* __restrict__ fx, float* __restrict__ out, int* err) {
  __shared__ TcNet s;
  tc_setup(params, s);
  uint32_t phase = 0;
  const long long ntiles = (n + tc::M - 1) / tc::M;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long c = tile * tc::M + threadIdx.x;
    float xin[NIN], y[NOUT];
#pragma unroll
    for (int k = 0; k < NIN; ++k) xin[k] = c < n ? (fx[c * NIN + k] - s.xm[k]) / s.xs[k] : 0.0f;
    tc_infer_tile(s, xin, y, phase, err);
    if (c < n) {
#pragma unroll
      for (int q = 0; q < NOUT; ++q) out[c * NOUT + q] = y[q];
    }
  }
  tc_teardown(s);
}

unsigned grid_of(long long n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

}  // namespace

extern "C" {

athgpu_status athgpu_sr_features(long long n, const double* cons, const double* bcc,
                                 float* features_out, void* stream) {
  if (n < 0 || (n > 0 && (!cons || !bcc || !features_out)))
    return fail(ATHGPU_ERR_ARG, "sr_features: bad arguments");
  if (n == 0) return ATHGPU_OK;
  sr_features_kernel<<<grid_of(n, 256), 256, 0, (cudaStream_t)stream>>>(n, cons, bcc,
                                                                         features_out);
  CKE(cudaGetLastError());
  return ATHGPU_OK;
}

athgpu_status athgpu_mlp_infer(long long n, const float* params, const float* features,
                               float* out, void* stream) {
  if (n < 0 || !params || (n > 0 && (!features || !out)))
    return fail(ATHGPU_ERR_ARG, "mlp_infer: bad arguments");
  if (n == 0) return ATHGPU_OK;
  mlp_infer_kernel<<<grid_of(n, 128), 128, 0, (cudaStream_t)stream>>>(n, params, features, out);
  CKE(cudaGetLastError());
  return ATHGPU_OK;
}

athgpu_status athgpu_mlp_infer_tc(long long n, const float* params, const float* features,
                                  float* out, void* stream) {
  if (n < 0 || !params || (n > 0 && (!features || !out)))
    return fail(ATHGPU_ERR_ARG, "mlp_infer_tc: bad arguments");
  if (n == 0) return ATHGPU_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  CKE(cudaGetDevice(&dev));
  CKE(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int* err;
  CKE(cudaMallocAsync((void**)&err, sizeof(int), s));
  CKE(cudaMemsetAsync(err, 0, sizeof(int), s));
  const long long ntiles = (n + 127) / 128;
  const unsigned grid = (unsigned)(ntiles < 4LL * sms ? ntiles : 4LL * sms);
  // Each CTA holds 128 of an SM's 512 TMEM columns for its lifetime: unused dynamic
  // shared memory keeps residency at four CTAs per SM, so no allocation has to wait.
  const int pad = TC_SMEM_PAD;
  CKE(cudaFuncSetAttribute(mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           pad));
  mlp_infer_tc_kernel<<<grid, 128, pad, s>>>(n, params, features, out, err);
  CKE(cudaGetLastError());
  int herr = 0;
  CKE(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  CKE(cudaFreeAsync(err, s));
  CKE(cudaStreamSynchronize(s));
  if (herr) return fail(ATHGPU_ERR_CUDA, "mlp_infer_tc: tensor-core wait timed out");
  return ATHGPU_OK;
}

athgpu_status athgpu_sr_c2p_cells(long long n, double gamma, double pfloor, const double* cons,
                                  const double* bcc, const double* pgas_guess,
                                  const float* params, int mode, int phase1_iterations,
                                  double* prim, int* iters64, int* iters32, int* fallbacks,
                                  void* stream) {
  if (n < 0 || (n > 0 && (!cons || !bcc || !prim || !iters64)))
    return fail(ATHGPU_ERR_ARG, "sr_c2p_cells: bad arguments");
  if (n >= (1LL << 31)) return fail(ATHGPU_ERR_ARG, "sr_c2p_cells: at most 2^31-1 cells");
  const bool warp_mma = (mode & ATHGPU_C2P_WARP_MMA) != 0;
  mode &= ~ATHGPU_C2P_WARP_MMA;
  if (mode < 0 || mode > 3) return fail(ATHGPU_ERR_ARG, "sr_c2p_cells: mode must be 0..3");
  if ((mode == 1 || mode == 2) && !params)
    return fail(ATHGPU_ERR_ARG, "sr_c2p_cells: mode needs parameters");
  if (!(gamma > 1.0)) return fail(ATHGPU_ERR_ARG, "sr_c2p_cells: gamma must exceed 1");
  if (phase1_iterations < 0 || phase1_iterations > MAXIT)
    return fail(ATHGPU_ERR_ARG, "sr_c2p_cells: phase1_iterations must be in [0, 15]");
  if (n == 0) return ATHGPU_OK;
  const int n1 = phase1_iterations ? phase1_iterations : (mode == 0 ? 7 : 4);
  cudaStream_t s = (cudaStream_t)stream;
  Queue qu;
  const size_t cap = (size_t)n;
  CKE(cudaMallocAsync((void**)&qu.cell, cap * sizeof(long long), s));
  CKE(cudaMallocAsync((void**)&qu.state, cap * sizeof(int), s));
  CKE(cudaMallocAsync((void**)&qu.p, cap * 3 * sizeof(double), s));
  CKE(cudaMallocAsync((void**)&qu.count, sizeof(unsigned), s));
  CKE(cudaMemsetAsync(qu.count, 0, sizeof(unsigned), s));
  int* tc_err;
  CKE(cudaMallocAsync((void**)&tc_err, sizeof(int), s));
  CKE(cudaMemsetAsync(tc_err, 0, sizeof(int), s));
  const bool net = mode == 1 || mode == 2;
  if (net && !warp_mma) {  // tcgen05 network (tensor memory), four CTAs per SM at most
    const int smem = (int)sizeof(TcNet) + TC_SMEM_PAD;
    CKE(cudaFuncSetAttribute(sr_c2p_phase1_kernel<true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    sr_c2p_phase1_kernel<true><<<grid_of(n, 128), 128, smem, s>>>(
        n, gamma, pfloor, cons, bcc, pgas_guess, params, mode, n1, prim, iters64, iters32,
        fallbacks, qu, tc_err);
  } else {
    sr_c2p_phase1_kernel<false><<<grid_of(n, 128), 128, net ? (int)sizeof(SmemNet) : 0, s>>>(
        n, gamma, pfloor, cons, bcc, pgas_guess, params, mode, n1, prim, iters64, iters32,
        fallbacks, qu, tc_err);
  }
  int dev = 0, sms = 0;
  CKE(cudaGetDevice(&dev));
  CKE(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const long long want = (n + 127) / 128;
  const unsigned g2 = (unsigned)(want < 8LL * sms ? want : 8LL * sms);
  sr_c2p_phase2_kernel<<<g2, 128, 0, s>>>(gamma, pfloor, cons, bcc, pgas_guess, mode, prim,
                                          iters64, fallbacks, qu);
  CKE(cudaGetLastError());
  CKE(cudaFreeAsync(qu.cell, s));
  CKE(cudaFreeAsync(qu.state, s));
  CKE(cudaFreeAsync(qu.p, s));
  CKE(cudaFreeAsync(qu.count, s));
  int herr = 0;
  CKE(cudaMemcpyAsync(&herr, tc_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  CKE(cudaFreeAsync(tc_err, s));
  CKE(cudaStreamSynchronize(s));
  if (herr) return fail(ATHGPU_ERR_CUDA, "sr_c2p_cells: tensor-core wait timed out");
  return ATHGPU_OK;
}

athgpu_status athgpu_mlp_loss_grad(const float* params, const float* x, const float* t,
                                   int batch, float* grad, float* loss, void* stream) {
  if (!params || !x || !t || !grad || !loss || batch < 1)
    return fail(ATHGPU_ERR_ARG, "mlp_loss_grad: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  float *z1, *z2, *y, *dy, *dz2, *dz1;
  const size_t B = batch;
  CKE(cudaMallocAsync((void**)&z1, B * NH * 4, s));
  CKE(cudaMallocAsync((void**)&z2, B * NH * 4, s));
  CKE(cudaMallocAsync((void**)&y, B * NOUT * 4, s));
  CKE(cudaMallocAsync((void**)&dy, B * NOUT * 4, s));
  CKE(cudaMallocAsync((void**)&dz2, B * NH * 4, s));
  CKE(cudaMallocAsync((void**)&dz1, B * NH * 4, s));
  CKE(cudaMemsetAsync(loss, 0, 4, s));
  mlp_forward_kernel<<<grid_of(batch, 128), 128, 0, s>>>(params, x, t, batch, z1, z2, y, loss);
  mlp_backward_kernel<<<grid_of(batch, 128), 128, 0, s>>>(params, t, batch, z1, z2, y, dy, dz2,
                                                          dz1);
  CKE(cudaMemsetAsync(grad, 0, NTRAIN * sizeof(float), s));
  mlp_wgrad_kernel<<<dim3(grid_of(NTRAIN, 128), grid_of(batch, WG_CHUNK)), 128, 0, s>>>(
      x, batch, z1, z2, dy, dz2, dz1, grad);
  CKE(cudaGetLastError());
  for (float* q : {z1, z2, y, dy, dz2, dz1}) CKE(cudaFreeAsync(q, s));
  return ATHGPU_OK;
}

athgpu_status athgpu_mlp_train(const float* features, const float* targets, long long n,
                               float* params, int steps, int batch, float lr,
                               unsigned long long seed, float* loss_history, void* stream) {
  if (!features || !targets || !params || n < 1 || steps < 1 || batch < 1 || !(lr > 0.0f))
    return fail(ATHGPU_ERR_ARG, "mlp_train: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t B = batch;
  float *x, *t, *z1, *z2, *y, *dy, *dz2, *dz1, *g, *m, *v, *loss;
  unsigned* idx;
  CKE(cudaMallocAsync((void**)&x, B * NIN * 4, s));
  CKE(cudaMallocAsync((void**)&t, B * NOUT * 4, s));
  CKE(cudaMallocAsync((void**)&z1, B * NH * 4, s));
  CKE(cudaMallocAsync((void**)&z2, B * NH * 4, s));
  CKE(cudaMallocAsync((void**)&y, B * NOUT * 4, s));
  CKE(cudaMallocAsync((void**)&dy, B * NOUT * 4, s));
  CKE(cudaMallocAsync((void**)&dz2, B * NH * 4, s));
  CKE(cudaMallocAsync((void**)&dz1, B * NH * 4, s));
  CKE(cudaMallocAsync((void**)&g, NTRAIN * 4, s));
  CKE(cudaMallocAsync((void**)&m, NTRAIN * 4, s));
  CKE(cudaMallocAsync((void**)&v, NTRAIN * 4, s));
  CKE(cudaMallocAsync((void**)&loss, (size_t)steps * 4, s));
  CKE(cudaMallocAsync((void**)&idx, B * 4, s));
  CKE(cudaMemsetAsync(m, 0, NTRAIN * 4, s));
  CKE(cudaMemsetAsync(v, 0, NTRAIN * 4, s));
  CKE(cudaMemsetAsync(loss, 0, (size_t)steps * 4, s));
  for (int step = 1; step <= steps; ++step) {
    batch_indices_kernel<<<grid_of(batch, 256), 256, 0, s>>>(seed, step, (unsigned)n, batch,
                                                             idx);
    gather_batch_kernel<<<grid_of(batch, 256), 256, 0, s>>>(params, features, targets, idx,
                                                            batch, x, t);
    mlp_forward_kernel<<<grid_of(batch, 128), 128, 0, s>>>(params, x, t, batch, z1, z2, y,
                                                           loss + step - 1);
    mlp_backward_kernel<<<grid_of(batch, 128), 128, 0, s>>>(params, t, batch, z1, z2, y, dy,
                                                            dz2, dz1);
    cudaMemsetAsync(g, 0, NTRAIN * sizeof(float), s);
    mlp_wgrad_kernel<<<dim3(grid_of(NTRAIN, 128), grid_of(batch, WG_CHUNK)), 128, 0, s>>>(
        x, batch, z1, z2, dy, dz2, dz1, g);
    // cosine decay of the step size from lr to lr / 50
    const float lr_t = lr * (0.02f + 0.49f * (1.0f + cosf(3.14159265f * (step - 1) / steps)));
    adam_kernel<<<grid_of(NTRAIN, 128), 128, 0, s>>>(params, g, m, v, step, lr_t, 0.9f,
                                                     0.999f, 1e-8f);
  }
  CKE(cudaGetLastError());
  if (loss_history)
    CKE(cudaMemcpyAsync(loss_history, loss, (size_t)steps * 4, cudaMemcpyDeviceToHost, s));
  for (void* q : {(void*)x, (void*)t, (void*)z1, (void*)z2, (void*)y, (void*)dy, (void*)dz2,
                  (void*)dz1, (void*)g, (void*)m, (void*)v, (void*)loss, (void*)idx})
    CKE(cudaFreeAsync(q, s));
  CKE(cudaStreamSynchronize(s));
  return ATHGPU_OK;
}

}  // extern "C"
