// Device self-checks of arithmetic helpers the kernels rely on.
#include <cuda_runtime.h>

#include <string>

#include "../../include/athena_gb300.h"
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
  if (bad32) atomicAdd(mismatches, 1ull);
  if (bad64) atomicAdd(mismatches + 1, 1ull);
}

}  // namespace

extern "C" athgpu_status athgpu_selftest_conversions(long long n, const double* d,
                                                     const float* f,
                                                     unsigned long long* mismatches,
                                                     void* stream) {
  if (n < 0 || (n > 0 && (!d || !f)) || !mismatches) {
    athgpu::set_last_error("selftest_conversions: bad arguments");
    return ATHGPU_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(mismatches, 0, 2 * sizeof(unsigned long long), s);
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
