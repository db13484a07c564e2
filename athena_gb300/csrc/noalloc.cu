// Conserved->primitive + CFL time step over caller-owned device arrays, with no device
// allocation by the library.
//
// Some callers cannot let a library call cudaMalloc: hosts whose device memory is owned
// by their own pool allocator (a framework's caching allocator that must account for
// every byte), real-time loops that forbid allocation latency, and plugins that must
// leave the device heap untouched.  athgpu_con2prim_timestep_noalloc serves them: the
// caller passes every input and output as a device pointer, and the only scratch the
// computation needs — the per-CTA partial minima of the two-pass time-step reduction —
// lives in the file-scope array g_noalloc_partial below, of fixed size.  Every GPU that
// loads the library holds that array (about 0.5 MB) until the process exits.
#include <cuda.h>  // CUcontext and the driver-call types (the calls are fetched at run time)
#include <cuda_runtime.h>
#include <float.h>
#include <limits.h>

#include <mutex>
#include <string>

#include "../../include/athena_gb300.h"
#include "physics.cuh"

namespace athgpu {
void set_last_error(const std::string& msg);  // api.cu
}

namespace {

constexpr int kThreads = 256;                        // cells per CTA
constexpr int kMaxPartials = 65536;                  // CTAs per call
constexpr long long kMaxCells = (long long)kThreads * kMaxPartials;  // 16,777,216
static_assert(kMaxCells == ATHGPU_NOALLOC_MAX_CELLS, "header limit out of date");

// [0, kMaxPartials): per-CTA minima of dx/(|v|+c_f); [kMaxPartials]: unused pad.
// Shared by every call on this device and keeping the last call's contents; each call
// overwrites every entry it reads before reading it.
static __device__ __align__(256) double g_noalloc_partial[kMaxPartials + 32];

// The device address of g_noalloc_partial belongs to a CUDA context, not to a device: a
// host that makes its own driver context current, or a process that reset the device,
// sees the array at another address.  The lookups are cached per context, keyed by the
// context's process-unique ID (cuCtxGetId), which a re-created context never reuses.
constexpr int kMaxContexts = 64;
struct SymbolEntry {
  unsigned long long ctx_id;
  double* addr;
};
std::mutex g_mu;
SymbolEntry g_symbol_cache[kMaxContexts];
int g_symbol_used = 0;
int g_symbol_next = 0;  // slot replaced next once the cache is full


__device__ __forceinline__ long long f1(int nc1, int nc2, long long nf, int b, int k, int j,
                                        int i) {
  return (long long)b * nf + ((long long)k * nc2 + j) * (nc1 + 1) + i;
}
__device__ __forceinline__ long long f2(int nc1, int nc2, long long nf, int b, int k, int j,
                                        int i) {
  return (long long)b * nf + ((long long)k * (nc2 + 1) + j) * nc1 + i;
}
__device__ __forceinline__ long long f3(int nc1, int nc2, long long nf, int b, int k, int j,
                                        int i) {
  return (long long)b * nf + ((long long)k * nc2 + j) * nc1 + i;
}

struct Geometry {
  int nb, nx1, nx2, nx3, ng, nc1, nc2, nc3;
  long long ncell, nf1, nf2, nf3;
  double gamma, dfloor, pfloor;
};

// EquationOfState::ConservedToPrimitive (adiabatic_mhd.cpp:41-90) with the uniform
// cell-centred field (field.cpp:112-180) on every cell, and the per-cell CFL limit of
// Hydro::NewBlockTimeStep (new_blockdt.cpp:80-103) on interior cells, reduced to one
// minimum per CTA into the scratch array.  The arithmetic is the same as the library's
// FP64 stage kernels.
__global__ void __launch_bounds__(kThreads)
c2p_dt_partial_kernel(Geometry g, const double* __restrict__ dx1f,
                      const double* __restrict__ dx2f, const double* __restrict__ dx3f,
                      const double* __restrict__ b1, const double* __restrict__ b2,
                      const double* __restrict__ b3, double* u, double* __restrict__ w,
                      double* __restrict__ bcc, double* __restrict__ partial) {
  using athgpu::fast_ms;
  using athgpu::smax;
  using athgpu::smin;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double cell_dt = DBL_MAX;
  if (t < (long long)g.nb * g.ncell) {
    const int b = (int)(t / g.ncell);
    long long r = t - (long long)b * g.ncell;
    const int i = (int)(r % g.nc1);
    r /= g.nc1;
    const int j = (int)(r % g.nc2);
    const int k = (int)(r / g.nc2);
    const double lw = 0.5, rw = 0.5;
    const double bc1 = lw * b1[f1(g.nc1, g.nc2, g.nf1, b, k, j, i)] +
                       rw * b1[f1(g.nc1, g.nc2, g.nf1, b, k, j, i + 1)];
    const double bc2 = lw * b2[f2(g.nc1, g.nc2, g.nf2, b, k, j, i)] +
                       rw * b2[f2(g.nc1, g.nc2, g.nf2, b, k, j + 1, i)];
    const double bc3 = lw * b3[f3(g.nc1, g.nc2, g.nf3, b, k, j, i)] +
                       rw * b3[f3(g.nc1, g.nc2, g.nf3, b, k + 1, j, i)];
    const long long vs = g.ncell;
    const long long c = (long long)b * 5 * g.ncell + ((long long)k * g.nc2 + j) * g.nc1 + i;
    const long long cb = (long long)b * 3 * g.ncell + ((long long)k * g.nc2 + j) * g.nc1 + i;
    const double gm1 = g.gamma - 1.0;
    double u_d = u[c], u_m1 = u[c + vs], u_m2 = u[c + 2 * vs], u_m3 = u[c + 3 * vs],
           u_e = u[c + 4 * vs];
    const bool dfloored = !(u_d > g.dfloor);
    u_d = (u_d > g.dfloor) ? u_d : g.dfloor;
    double di = 1.0 / u_d;
    double vx = u_m1 * di, vy = u_m2 * di, vz = u_m3 * di;
    double pb = 0.5 * (bc1 * bc1 + bc2 * bc2 + bc3 * bc3);
    double e_k = 0.5 * di * (u_m1 * u_m1 + u_m2 * u_m2 + u_m3 * u_m3);
    double w_p = gm1 * (u_e - e_k - pb);
    const bool pfloored = !(w_p > g.pfloor);
    u_e = (w_p > g.pfloor) ? u_e : ((g.pfloor / gm1) + e_k + pb);
    w_p = (w_p > g.pfloor) ? w_p : g.pfloor;
    if (dfloored) u[c] = u_d;
    if (pfloored) u[c + 4 * vs] = u_e;
    w[c] = u_d;
    w[c + vs] = vx;
    w[c + 2 * vs] = vy;
    w[c + 3 * vs] = vz;
    w[c + 4 * vs] = w_p;
    bcc[cb] = bc1;
    bcc[cb + vs] = bc2;
    bcc[cb + 2 * vs] = bc3;
    if (i >= g.ng && i < g.ng + g.nx1 && j >= g.ng && j < g.ng + g.nx2 && k >= g.ng &&
        k < g.ng + g.nx3) {
      double dt1 = dx1f[(long long)b * g.nc1 + i], dt2 = dx2f[(long long)b * g.nc2 + j],
             dt3 = dx3f[(long long)b * g.nc3 + k];
      double bx = bc1 + fabs(b1[f1(g.nc1, g.nc2, g.nf1, b, k, j, i)] - bc1);
      double cf = fast_ms<double>(g.gamma, u_d, w_p, bc2, bc3, bx);
      double speed = smax<double>(0.0, (fabs(vx) + cf));
      dt1 /= (speed);
      bx = bc2 + fabs(b2[f2(g.nc1, g.nc2, g.nf2, b, k, j, i)] - bc2);
      cf = fast_ms<double>(g.gamma, u_d, w_p, bc3, bc1, bx);
      speed = smax<double>(0.0, (fabs(vy) + cf));
      dt2 /= (speed);
      bx = bc3 + fabs(b3[f3(g.nc1, g.nc2, g.nf3, b, k, j, i)] - bc3);
      cf = fast_ms<double>(g.gamma, u_d, w_p, bc1, bc2, bx);
      speed = smax<double>(0.0, (fabs(vz) + cf));
      dt3 /= (speed);
      cell_dt = smin<double>(smin<double>(dt1, dt2), dt3);
    }
  }
  // CTA minimum: warp shuffles, then one value per warp through shared memory
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cell_dt = fmin(cell_dt, __shfl_xor_sync(0xffffffffu, cell_dt, o));
  __shared__ double warp_min[kThreads / 32];
  if ((threadIdx.x & 31) == 0) warp_min[threadIdx.x >> 5] = cell_dt;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = warp_min[0];
    for (int q = 1; q < kThreads / 32; ++q) v = fmin(v, warp_min[q]);
    partial[blockIdx.x] = v;  // every CTA writes its slot: no stale entries are read
  }
}

// Mesh::NewTimeStep for the first step (mesh.cpp:1246-1256): cfl times the minimum over
// blocks, i.e. over the CTA minima.
__global__ void __launch_bounds__(1024)
dt_finalize_kernel(const double* __restrict__ partial, int nparts, double cfl,
                   double* __restrict__ dt_out) {
  double v = DBL_MAX;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) v = fmin(v, partial[q]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double wm[32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = wm[0];
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) m = fmin(m, wm[q]);
    *dt_out = m * cfl;
  }
}

athgpu_status noalloc_fail(athgpu_status s, const std::string& msg) {
  athgpu::set_last_error(msg);  // reported by athgpu_last_error()
  return s;
}

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// The process-unique ID of the calling thread's current CUDA context.  The two driver
// calls are fetched through the runtime, so the library needs no link against libcuda.
// With no context current yet, the runtime's primary context of the current device is
// made current first (cudaSetDevice initialises it; it allocates nothing).
athgpu_status current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                      cudaEnableDefault, &q1);
    cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000,
                                                      cudaEnableDefault, &q2);
    if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
        q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return noalloc_fail(ATHGPU_ERR_CUDA,
                          "con2prim_timestep_noalloc: cuCtxGetCurrent/cuCtxGetId unavailable");
    get_current = (CtxGetCurrentFn)f1;
    get_id = (CtxGetIdFn)f2;
  }
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS)
    return noalloc_fail(ATHGPU_ERR_CUDA, "con2prim_timestep_noalloc: cuCtxGetCurrent failed");
  if (!c) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaSetDevice(dev);
    if (e != cudaSuccess)
      return noalloc_fail(ATHGPU_ERR_CUDA,
                          std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    if (get_current(&c) != CUDA_SUCCESS || !c)
      return noalloc_fail(ATHGPU_ERR_CUDA, "con2prim_timestep_noalloc: no current context");
  }
  if (get_id(c, id) != CUDA_SUCCESS)
    return noalloc_fail(ATHGPU_ERR_CUDA, "con2prim_timestep_noalloc: cuCtxGetId failed");
  return ATHGPU_OK;
}

// Device address of the scratch array in the current context.  Set-up, once per context:
// cudaGetSymbolAddress with that context current (the array's host-side name is only a
// stand-in and must never reach a kernel).
athgpu_status scratch_address(double** out) {
  unsigned long long id = 0;
  athgpu_status st = current_context_id(&id);
  if (st != ATHGPU_OK) return st;
  std::lock_guard<std::mutex> lk(g_mu);
  for (int q = 0; q < g_symbol_used; ++q)
    if (g_symbol_cache[q].ctx_id == id) {
      *out = g_symbol_cache[q].addr;
      return ATHGPU_OK;
    }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
  if (e != cudaSuccess || !p)
    return noalloc_fail(ATHGPU_ERR_CUDA,
                        std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  int slot;
  if (g_symbol_used < kMaxContexts) {
    slot = g_symbol_used++;
  } else {  // full: replace the oldest entry
    slot = g_symbol_next;
    g_symbol_next = (g_symbol_next + 1) % kMaxContexts;
  }
  g_symbol_cache[slot] = {id, (double*)p};
  *out = (double*)p;
  return ATHGPU_OK;
}

}  // namespace

extern "C" athgpu_status athgpu_con2prim_timestep_noalloc(
    int nblocks, int nx1, int nx2, int nx3, int nghost, double gamma, double dfloor,
    double pfloor, double cfl_number, const double* dx1f, const double* dx2f,
    const double* dx3f, const double* b1, const double* b2, const double* b3, double* u,
    double* w, double* bcc, double* dt_out, void* stream) {
  if (nblocks < 1 || nx1 < 1 || nx2 < 1 || nx3 < 1 || nghost < 1)
    return noalloc_fail(ATHGPU_ERR_ARG, "con2prim_timestep_noalloc: sizes must be positive");
  // the same mesh shapes as athgpu_create: 3-D only (a 2-D array of the reference has
  // nc3 = 1 and no x3 ghosts, which this layout would read past)
  if (nx2 < 2 || nx3 < 2)
    return noalloc_fail(ATHGPU_ERR_UNSUPPORTED,
                        "con2prim_timestep_noalloc: only 3-D meshes (nx2, nx3 > 1) are "
                        "supported");
  if (!dx1f || !dx2f || !dx3f || !b1 || !b2 || !b3 || !u || !w || !bcc || !dt_out)
    return noalloc_fail(ATHGPU_ERR_ARG, "con2prim_timestep_noalloc: null pointer");
  if (!(gamma > 1.0) || !(cfl_number > 0.0))
    return noalloc_fail(ATHGPU_ERR_ARG, "con2prim_timestep_noalloc: bad gamma or cfl");
  // sizes in 64-bit first: nx + 2 nghost must fit the kernels' int indices
  const long long lc1 = (long long)nx1 + 2LL * nghost;
  const long long lc2 = (long long)nx2 + 2LL * nghost;
  const long long lc3 = (long long)nx3 + 2LL * nghost;
  if (lc1 > INT_MAX || lc2 > INT_MAX || lc3 > INT_MAX)
    return noalloc_fail(ATHGPU_ERR_ARG, "con2prim_timestep_noalloc: block too large");
  // each factor is below 2^31, so lc1 * lc2 < 2^62; checked against the limit before the
  // third factor (then ncell < 2^55) and before the block count, so nothing overflows
  const long long ncell = (lc1 * lc2 > kMaxCells) ? kMaxCells + 1 : lc1 * lc2 * lc3;
  if (ncell > kMaxCells || (long long)nblocks > kMaxCells / ncell)
    return noalloc_fail(ATHGPU_ERR_ARG,
                        "con2prim_timestep_noalloc: " + std::to_string(nblocks) +
                            " blocks of " + std::to_string(ncell) +
                            " cells (ghosts included) exceed the no-allocation limit of " +
                            std::to_string(kMaxCells) + " cells per call");
  Geometry g;
  g.nb = nblocks;
  g.nx1 = nx1; g.nx2 = nx2; g.nx3 = nx3; g.ng = nghost;
  g.nc1 = (int)lc1; g.nc2 = (int)lc2; g.nc3 = (int)lc3;
  g.ncell = ncell;
  g.nf1 = (long long)g.nc3 * g.nc2 * (g.nc1 + 1);
  g.nf2 = (long long)g.nc3 * (g.nc2 + 1) * g.nc1;
  g.nf3 = (long long)(g.nc3 + 1) * g.nc2 * g.nc1;
  g.gamma = gamma; g.dfloor = dfloor; g.pfloor = pfloor;
  const long long cells = (long long)nblocks * ncell;
  double* partial = nullptr;
  athgpu_status st = scratch_address(&partial);
  if (st != ATHGPU_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int nparts = (int)((cells + kThreads - 1) / kThreads);
  c2p_dt_partial_kernel<<<nparts, kThreads, 0, s>>>(g, dx1f, dx2f, dx3f, b1, b2, b3, u, w,
                                                    bcc, partial);
  dt_finalize_kernel<<<1, 1024, 0, s>>>(partial, nparts, cfl_number, dt_out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return noalloc_fail(ATHGPU_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return ATHGPU_OK;
}
