// Device self-checks of arithmetic helpers the kernels rely on.
#include <cuda_runtime.h>

#include <string>

#include "../../include/athena_gb300_diag.h"
#include "physics.cuh"

namespace athgpu {
void set_last_error(const std::string& msg);  // api.cu
}

namespace {

// Counts the elements where the integer-pipe conversions differ (bitwise) from the
// hardware conversions.
__global__ void conversion_check_kernel(long long n, const double* __restrict__ d,
                                        const float* __restrict__ f,
                                        unsigned long long* __restrict__ mismatches) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double x = d[q];
  const bool bad32 = __float_as_uint(athgpu::d2f_rn(x)) != __float_as_uint((float)x);
  const float y = f[q];
  const bool bad64 = __double_as_longlong(athgpu::f2d_exact(y)) !=
                     __double_as_longlong((double)y);
  // the difference of the pair (f[q], f[q ^ 1]) (a NaN result compares as NaN)
  const long long p = q ^ 1;
  bool badsub = false;
  if (p < n) {
    const float z = f[p];
    const double hw = (double)y - (double)z, sw = athgpu::fsub_f64(y, z);
    badsub = (hw != hw) ? (sw == sw) : __double_as_longlong(hw) != __double_as_longlong(sw);
  }
  if (bad32) atomicAdd(mismatches, 1ull);
  if (bad64) atomicAdd(mismatches + 1, 1ull);
  if (badsub) atomicAdd(mismatches + 2, 1ull);
}

// One Riemann solve per face in the solvers' local order (d, v_n, v_t1, v_t2, p, B_t1,
// B_t2): wl/wr [n][7], bx [n], flux [n][7], in Real.  FP32 HLLD and HLLE are the packed
// solvers the FP32 sweeps run (hlld_pk, hlle_pk).
template <typename Real, int RS>
__global__ void riemann_check_kernel(long long n, Real gamma, const Real* __restrict__ wl,
                                     const Real* __restrict__ wr,
                                     const Real* __restrict__ bx,
                                     const Real* __restrict__ dv,
                                     Real* __restrict__ flux) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  Real a[athgpu::NWAVE], b[athgpu::NWAVE], f[athgpu::NWAVE];
#pragma unroll
  for (int v = 0; v < athgpu::NWAVE; ++v) {
    a[v] = wl[q * athgpu::NWAVE + v];
    b[v] = wr[q * athgpu::NWAVE + v];
  }
  if constexpr (RS == 0 && sizeof(Real) == 4) athgpu::hlld_pk(gamma, a, b, bx[q], f);
  else if constexpr (RS == 1 && sizeof(Real) == 4) athgpu::hlle_pk(gamma, a, b, bx[q], f);
  else if (RS == 0) athgpu::hlld<Real>(gamma, a, b, bx[q], f);
  else if (RS == 1) athgpu::hlle<Real>(gamma, a, b, bx[q], f);
  else if (RS == 2) athgpu::hlle_sr<Real>(gamma, a, b, bx[q], f);
  else if (RS == 3) athgpu::llf<Real>(gamma, a, b, bx[q], f);
  else if (RS == 4) athgpu::roe<Real>(gamma, a, b, bx[q], f);
  else if (RS == 5) athgpu::llf_sr<Real>(gamma, a, b, bx[q], f);
  else if (RS == 7)
    athgpu::hlld<Real, true>(gamma, a, b, bx[q], f, dv ? dv[2 * q] : Real(0),
                             dv ? dv[2 * q + 1] : Real(0));
  else athgpu::hlld_sr<Real>(gamma, a, b, bx[q], f);
#pragma unroll
  for (int v = 0; v < athgpu::NWAVE; ++v) flux[q * athgpu::NWAVE + v] = f[v];
}

template <typename Real>
athgpu_status selftest_riemann(const char* name, int rsolver, int relativistic, double gamma,
                               long long n, const Real* wl, const Real* wr, const Real* bx,
                               const Real* dv, Real* flux, void* stream) {
  if (n < 0 || (n > 0 && (!wl || !wr || !bx || !flux)) ||
      rsolver < ATHGPU_HLLD || rsolver > ATHGPU_LHLLD ||
      (relativistic && (rsolver == ATHGPU_ROE || rsolver == ATHGPU_LHLLD)) ||
      !(gamma > 1.0)) {
    athgpu::set_last_error(std::string(name) + ": bad arguments");
    return ATHGPU_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned grid = (unsigned)((n + 127) / 128);
  const Real g = (Real)gamma;
  if (n > 0) {
    if (relativistic) {
      if (rsolver == ATHGPU_HLLD)
        riemann_check_kernel<Real, 6><<<grid, 128, 0, s>>>(n, g, wl, wr, bx, dv, flux);
      else if (rsolver == ATHGPU_LLF)
        riemann_check_kernel<Real, 5><<<grid, 128, 0, s>>>(n, g, wl, wr, bx, dv, flux);
      else
        riemann_check_kernel<Real, 2><<<grid, 128, 0, s>>>(n, g, wl, wr, bx, dv, flux);
    } else if (rsolver == ATHGPU_HLLD) {
      riemann_check_kernel<Real, 0><<<grid, 128, 0, s>>>(n, g, wl, wr, bx, dv, flux);
    } else if (rsolver == ATHGPU_HLLE) {
      riemann_check_kernel<Real, 1><<<grid, 128, 0, s>>>(n, g, wl, wr, bx, dv, flux);
    } else if (rsolver == ATHGPU_LLF) {
      riemann_check_kernel<Real, 3><<<grid, 128, 0, s>>>(n, g, wl, wr, bx, dv, flux);
    } else if (rsolver == ATHGPU_LHLLD) {
      riemann_check_kernel<Real, 7><<<grid, 128, 0, s>>>(n, g, wl, wr, bx, dv, flux);
    } else {
      riemann_check_kernel<Real, 4><<<grid, 128, 0, s>>>(n, g, wl, wr, bx, dv, flux);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    athgpu::set_last_error(std::string(name) + ": " + cudaGetErrorString(e));
    return ATHGPU_ERR_CUDA;
  }
  return ATHGPU_OK;
}

}  // namespace

extern "C" athgpu_status athgpu_selftest_riemann(int rsolver, int relativistic, double gamma,
                                                 long long n, const double* wl,
                                                 const double* wr, const double* bx,
                                                 const double* dv, double* flux,
                                                 void* stream) {
  return selftest_riemann<double>("selftest_riemann", rsolver, relativistic, gamma, n, wl, wr,
                                  bx, dv, flux, stream);
}

extern "C" athgpu_status athgpu_selftest_riemann_fp32(int rsolver, int relativistic,
                                                      double gamma, long long n,
                                                      const float* wl, const float* wr,
                                                      const float* bx, const float* dv,
                                                      float* flux, void* stream) {
  return selftest_riemann<float>("selftest_riemann_fp32", rsolver, relativistic, gamma, n, wl,
                                 wr, bx, dv, flux, stream);
}

extern "C" athgpu_status athgpu_selftest_conversions(long long n, const double* d,
                                                     const float* f,
                                                     unsigned long long* mismatches,
                                                     void* stream) {
  if (n < 0 || (n > 0 && (!d || !f)) || !mismatches) {
    athgpu::set_last_error("selftest_conversions: bad arguments");
    return ATHGPU_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(mismatches, 0, 3 * sizeof(unsigned long long), s);
  if (e == cudaSuccess && n > 0) {
    conversion_check_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, d, f, mismatches);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    athgpu::set_last_error(std::string("selftest_conversions: ") + cudaGetErrorString(e));
    return ATHGPU_ERR_CUDA;
  }
  return ATHGPU_OK;
}
