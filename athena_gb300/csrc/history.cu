// History output of the MHD state (HistoryOutput::WriteOutputFile, outputs/history.cpp:
// 77-140 for the quantities the path evolves): volume-weighted sums over the interior
// cells of all MeshBlocks of
//   mass, 1-mom, 2-mom, 3-mom, 1-KE, 2-KE, 3-KE, tot-E, 1-ME, 2-ME, 3-ME
// with vol = dx1f(i) dx2f(j) dx3f(k) (coordinates.cpp:536-545), KE_d = 0.5 M_d^2 / D and
// ME_d = 0.5 bcc_d^2.  Everything is formed in FP64: the FP32 path's conserved state is its
// compensated value hi + lo, and the cell-centred field is recomputed from the FP64 face
// fields (field.cpp:112-180).  The reduction is deterministic (per-CTA partial sums, then
// one CTA adds the partials in a fixed order), so repeated calls give the same bits; the
// summation order differs from the reference's sequential loop, so the sums agree with it
// to rounding, not bit for bit.
#include <cuda_runtime.h>

#include <string>

#include "../../include/athena_gb300.h"
#include "ctx.h"

namespace athgpu {
void set_last_error(const std::string& msg);  // api.cu
}

namespace {
using athgpu::DevMesh;
using athgpu::i64;

constexpr int NH = ATHGPU_NHISTORY;  // 11
constexpr int TPB = 256;

template <typename Real>
__global__ void __launch_bounds__(TPB)
history_partial_kernel(DevMesh m, const Real* __restrict__ u, const Real* __restrict__ ulo,
                       const double* __restrict__ b1, const double* __restrict__ b2,
                       const double* __restrict__ b3, double* __restrict__ partial) {
  double acc[NH];
#pragma unroll
  for (int q = 0; q < NH; ++q) acc[q] = 0.0;
  const long long nint = (long long)m.nb * m.nx1 * m.nx2 * m.nx3;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nint;
       t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / ((long long)m.nx1 * m.nx2 * m.nx3));
    long long r = t - (long long)b * m.nx1 * m.nx2 * m.nx3;
    const int i = m.is + (int)(r % m.nx1);
    r /= m.nx1;
    const int j = m.js + (int)(r % m.nx2);
    const int k = m.ks + (int)(r / m.nx2);
    const double vol = m.dx1f[(i64)b * m.nc1 + i] * m.dx2f[(i64)b * m.nc2 + j] *
                       m.dx3f[(i64)b * m.nc3 + k];
    const i64 c = athgpu::cidx(m, b, 0, 5, k, j, i);
    double q[5];
#pragma unroll
    for (int n = 0; n < 5; ++n)
      q[n] = (double)u[c + n * m.ncell] + (ulo ? (double)ulo[c + n * m.ncell] : 0.0);
    const double bc1 = 0.5 * b1[athgpu::f1idx(m, b, k, j, i)] +
                       0.5 * b1[athgpu::f1idx(m, b, k, j, i + 1)];
    const double bc2 = 0.5 * b2[athgpu::f2idx(m, b, k, j, i)] +
                       0.5 * b2[athgpu::f2idx(m, b, k, j + 1, i)];
    const double bc3 = 0.5 * b3[athgpu::f3idx(m, b, k, j, i)] +
                       0.5 * b3[athgpu::f3idx(m, b, k + 1, j, i)];
    acc[0] += vol * q[0];
    acc[1] += vol * q[1];
    acc[2] += vol * q[2];
    acc[3] += vol * q[3];
    acc[4] += vol * 0.5 * (q[1] * q[1]) / q[0];
    acc[5] += vol * 0.5 * (q[2] * q[2]) / q[0];
    acc[6] += vol * 0.5 * (q[3] * q[3]) / q[0];
    acc[7] += vol * q[4];
    acc[8] += vol * 0.5 * bc1 * bc1;
    acc[9] += vol * 0.5 * bc2 * bc2;
    acc[10] += vol * 0.5 * bc3 * bc3;
  }
  __shared__ double red[NH][TPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NH; ++q) {
    double v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[q][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < NH) {
    double v = 0.0;
    for (int w = 0; w < TPB / 32; ++w) v += red[threadIdx.x][w];
    partial[(i64)blockIdx.x * NH + threadIdx.x] = v;
  }
}

__global__ void history_final_kernel(const double* __restrict__ partial, int nparts,
                                     double* __restrict__ out) {
  if (threadIdx.x < NH) {
    double v = 0.0;
    for (int p = 0; p < nparts; ++p) v += partial[(i64)p * NH + threadIdx.x];
    out[threadIdx.x] = v;
  }
}

}  // namespace

extern "C" athgpu_status athgpu_history(athgpu_ctx* c, double* out) {
  if (!c || !out) {
    athgpu::set_last_error("history: null argument");
    return ATHGPU_ERR_ARG;
  }
  const DevMesh& m = c->m;
  const long long nint = (long long)m.nb * m.nx1 * m.nx2 * m.nx3;
  const int nparts = (int)((nint + TPB - 1) / TPB < 1024 ? (nint + TPB - 1) / TPB : 1024);
  double* d = nullptr;  // partials [nparts][NH] then the result [NH]
  cudaError_t e = cudaMallocAsync((void**)&d, sizeof(double) * NH * (nparts + 1), c->stream);
  if (e == cudaSuccess) {
    if (c->real_bytes == 8)
      history_partial_kernel<double><<<nparts, TPB, 0, c->stream>>>(
          m, (const double*)c->r.u, nullptr, c->r.b1, c->r.b2, c->r.b3, d);
    else
      history_partial_kernel<float><<<nparts, TPB, 0, c->stream>>>(
          m, (const float*)c->r.u, (const float*)c->r.ulo, c->r.b1, c->r.b2, c->r.b3, d);
    history_final_kernel<<<1, 32, 0, c->stream>>>(d, nparts, d + (long long)NH * nparts);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d + (long long)NH * nparts, sizeof(double) * NH,
                        cudaMemcpyDeviceToHost, c->stream);
  if (d) cudaFreeAsync(d, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    athgpu::set_last_error(std::string("history: ") + cudaGetErrorString(e));
    return ATHGPU_ERR_CUDA;
  }
  return ATHGPU_OK;
}
