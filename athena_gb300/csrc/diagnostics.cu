// Run diagnostics: the divergence of the face field and the con2prim statistics.
//
// athgpu_divb restates the reference's |div B| history diagnostic WAbsDivergenceB
// (pgen/field_loop_poles.cpp:634-672) over the interior cells of every MeshBlock: per cell
//   |(A1(i+1) b1(i+1) - A1(i) b1(i) + A2(j+1) b2(j+1) - A2(j) b2(j)
//     + A3(k+1) b3(k+1) - A3(k) b3(k)) / V| / (|B| / dl)
// with the Cartesian face areas and volume (coordinates.cpp:448-480, 536-560), dl the
// smallest edge length (GetEdge?Length, coordinates.cpp:372-385) and |B| from the cell-
// centred field recomputed from the faces (field.cpp:112-180); cells with |B| = 0 are
// skipped.  Always FP64 (the face field is FP64 in both precision modes), with the
// reference's operand order per cell, so every cell's value is the reference's bit for
// bit; the sum over cells is reduced deterministically (per-CTA partials in a fixed grid,
// then one thread adds them in order), so repeated calls give the same bits while the
// order differs from the reference's sequential loop.
#include <cuda_runtime.h>
#include <float.h>
#include <stddef.h>

#include <string>

#include "../../include/athena_gb300.h"
#include "ctx.h"

namespace athgpu {
void set_last_error(const std::string& msg);  // api.cu
}

namespace {
using athgpu::DevClock;
using athgpu::DevMesh;
using athgpu::i64;

constexpr int TPB = 256;
constexpr int MAX_PARTS = 1024;

// partial[p] = (sum, max, count) of the cells this CTA visited
__global__ void __launch_bounds__(TPB)
divb_partial_kernel(DevMesh m, const double* __restrict__ b1, const double* __restrict__ b2,
                    const double* __restrict__ b3, double* __restrict__ partial) {
  double sum = 0.0, mx = 0.0, cnt = 0.0;
  const long long nint = (long long)m.nb * m.nx1 * m.nx2 * m.nx3;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nint;
       t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / ((long long)m.nx1 * m.nx2 * m.nx3));
    long long r = t - (long long)b * m.nx1 * m.nx2 * m.nx3;
    const int i = m.is + (int)(r % m.nx1);
    r /= m.nx1;
    const int j = m.js + (int)(r % m.nx2);
    const int k = m.ks + (int)(r / m.nx2);
    const double dx1 = m.dx1f[(i64)b * m.nc1 + i];
    const double dx2 = m.dx2f[(i64)b * m.nc2 + j];
    const double dx3 = m.dx3f[(i64)b * m.nc3 + k];
    const double f1m = b1[athgpu::f1idx(m, b, k, j, i)];
    const double f1p = b1[athgpu::f1idx(m, b, k, j, i + 1)];
    const double f2m = b2[athgpu::f2idx(m, b, k, j, i)];
    const double f2p = b2[athgpu::f2idx(m, b, k, j + 1, i)];
    const double f3m = b3[athgpu::f3idx(m, b, k, j, i)];
    const double f3p = b3[athgpu::f3idx(m, b, k + 1, j, i)];
    // CalculateCellCenteredField, uniform branch: lw = rw = 1/2
    const double bc1 = 0.5 * f1m + 0.5 * f1p;
    const double bc2 = 0.5 * f2m + 0.5 * f2p;
    const double bc3 = 0.5 * f3m + 0.5 * f3p;
    const double bmag = sqrt(bc1 * bc1 + bc2 * bc2 + bc3 * bc3);
    if (bmag != 0.0) {
      // the face areas of one cell are equal on both sides of a uniform Cartesian cell:
      // Face1Area = dx2f(j) dx3f(k), Face2Area = dx1f(i) dx3f(k), Face3Area = dx1f(i) dx2f(j)
      const double a1 = dx2 * dx3, a2 = dx1 * dx3, a3 = dx1 * dx2;
      const double dl = fmin(fmin(dx1, dx2), dx3);
      const double vol = dx1 * dx2 * dx3;
      const double v = fabs(((a1 * f1p - a1 * f1m + a2 * f2p - a2 * f2m + a3 * f3p -
                              a3 * f3m)) / vol) / (bmag / dl);
      sum += v;
      mx = fmax(mx, v);
      cnt += 1.0;
    }
  }
  __shared__ double red[3][TPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  if (lane == 0) {
    red[0][wid] = sum;
    red[1][wid] = mx;
    red[2][wid] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0, x = 0.0, c = 0.0;
    for (int w = 0; w < TPB / 32; ++w) {
      s += red[0][w];
      x = fmax(x, red[1][w]);
      c += red[2][w];
    }
    partial[3 * (i64)blockIdx.x + 0] = s;
    partial[3 * (i64)blockIdx.x + 1] = x;
    partial[3 * (i64)blockIdx.x + 2] = c;
  }
}

__global__ void divb_final_kernel(const double* __restrict__ partial, int nparts,
                                  double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double s = 0.0, x = 0.0, c = 0.0;
  for (int p = 0; p < nparts; ++p) {
    s += partial[3 * (i64)p];
    x = fmax(x, partial[3 * (i64)p + 1]);
    c += partial[3 * (i64)p + 2];
  }
  out[0] = s;
  out[1] = x;
  out[2] = c;
}

athgpu_status diag_fail(athgpu_status s, const std::string& msg) {
  athgpu::set_last_error(msg);
  return s;
}

athgpu_status divb_into(athgpu_ctx* c, double* out3) {
  const DevMesh& m = c->m;
  const long long nint = (long long)m.nb * m.nx1 * m.nx2 * m.nx3;
  const long long want = (nint + TPB - 1) / TPB;
  const int nparts = (int)(want < MAX_PARTS ? want : MAX_PARTS);
  double* d = nullptr;  // partials [nparts][3] then the result [3]
  cudaError_t e = cudaMallocAsync((void**)&d, sizeof(double) * 3 * (nparts + 1), c->stream);
  if (e == cudaSuccess) {
    divb_partial_kernel<<<nparts, TPB, 0, c->stream>>>(m, c->r.b1, c->r.b2, c->r.b3, d);
    divb_final_kernel<<<1, 32, 0, c->stream>>>(d, nparts, d + 3LL * nparts);
    c->launches += 2;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out3, d + 3LL * nparts, sizeof(double) * 3, cudaMemcpyDeviceToHost,
                        c->stream);
  if (d) cudaFreeAsync(d, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return diag_fail(ATHGPU_ERR_CUDA, std::string("divb: ") +
                                                              cudaGetErrorString(e));
  return ATHGPU_OK;
}

}  // namespace

extern "C" athgpu_status athgpu_divb(athgpu_ctx* c, double* out) {
  if (!c || !out) return diag_fail(ATHGPU_ERR_ARG, "divb: null argument");
  if (!c->initialized) return diag_fail(ATHGPU_ERR_STATE, "divb: athgpu_initialize not called");
  return divb_into(c, out);
}

extern "C" athgpu_status athgpu_stats(athgpu_ctx* c, athgpu_run_stats* out, int reset) {
  if (!c || !out) return diag_fail(ATHGPU_ERR_ARG, "stats: null argument");
  if (!c->initialized) return diag_fail(ATHGPU_ERR_STATE, "stats: athgpu_initialize not called");
  double d3[3];
  athgpu_status st = divb_into(c, d3);
  if (st != ATHGPU_OK) return st;
  DevClock h;
  cudaError_t e = cudaMemcpyAsync(&h, c->clk, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return diag_fail(ATHGPU_ERR_CUDA, std::string("stats: ") +
                                                              cudaGetErrorString(e));
  out->divb_sum = d3[0];
  out->divb_max = d3[1];
  out->divb_cells = (long long)d3[2];
  out->floor_cells = h.c2p_floor_count;
  out->sr_cells = (long long)h.sr_cells;
  out->sr_passes = (long long)h.sr_passes;
  out->sr_fallbacks = (long long)h.sr_fallbacks;
  out->sr_unconverged = (long long)h.sr_unconverged;
  out->net_error = 0;
  out->sweep_timeout = h.sweep_timeout;
  if (c->c2p_net_err) {
    e = cudaMemcpyAsync(&out->net_error, c->c2p_net_err, sizeof(int), cudaMemcpyDeviceToHost,
                        c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return diag_fail(ATHGPU_ERR_CUDA, std::string("stats: ") +
                                                                cudaGetErrorString(e));
  }
  if (reset) {
    // zero the counters: the floor count and the four SR counters
    h.c2p_floor_count = 0;
    h.sr_cells = h.sr_passes = h.sr_fallbacks = h.sr_unconverged = 0;
    h.sweep_timeout = 0;
    e = cudaMemcpyAsync((char*)c->clk + offsetof(DevClock, c2p_floor_count),
                        &h.c2p_floor_count, sizeof(int), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync((char*)c->clk + offsetof(DevClock, sr_cells), &h.sr_cells,
                          4 * sizeof(unsigned long long), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && c->c2p_net_err)
      e = cudaMemsetAsync(c->c2p_net_err, 0, sizeof(int), c->stream);
    if (e == cudaSuccess)
      e = cudaMemsetAsync((char*)c->clk + offsetof(DevClock, sweep_timeout), 0, sizeof(int),
                          c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return diag_fail(ATHGPU_ERR_CUDA, std::string("stats reset: ") +
                                                                cudaGetErrorString(e));
  }
  return ATHGPU_OK;
}
