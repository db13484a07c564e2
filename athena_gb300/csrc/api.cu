// C ABI of the stage update (include/athena_gb300.h).
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/athena_gb300_diag.h"
#include "ctx.h"
#include "ml_plan.h"

using namespace athgpu;

namespace {
thread_local std::string g_err;

athgpu_status fail(athgpu_status code, const std::string& msg) {
  g_err = msg;
  return code;
}
athgpu_status cuda_fail(cudaError_t e, const char* where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return ATHGPU_ERR_CUDA;
}
#define CK(call)                                          \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

// double <-> (float hi, float lo) conversions for the FP32 path
__global__ void split_kernel(const double* __restrict__ src, float* __restrict__ hi,
                             float* __restrict__ lo, long long n) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double v = src[t];
  float h = (float)v;
  hi[t] = h;
  if (lo) lo[t] = (float)(v - (double)h);
}
__global__ void join_kernel(const float* __restrict__ hi, const float* __restrict__ lo,
                            double* __restrict__ dst, long long n) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  dst[t] = (double)hi[t] + (lo ? (double)lo[t] : 0.0);
}

long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

// The same conversions reading or writing page-locked host memory in place (the GPU reaches
// it over the host link): one pass instead of a copy into device staging plus a kernel.
// Each thread moves four consecutive elements per step, so several requests are in flight
// per thread and the link's latency is hidden; grid-stride over the array.
__global__ void __launch_bounds__(256)
split_from_host_kernel(const double* __restrict__ src, float* __restrict__ hi,
                       float* __restrict__ lo, long long n) {
  const long long n4 = n / 4;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4;
       q += (long long)gridDim.x * blockDim.x) {
    const double2 a = reinterpret_cast<const double2*>(src)[2 * q];
    const double2 b = reinterpret_cast<const double2*>(src)[2 * q + 1];
    const float4 h = make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y);
    reinterpret_cast<float4*>(hi)[q] = h;
    if (lo)
      reinterpret_cast<float4*>(lo)[q] =
          make_float4((float)(a.x - (double)h.x), (float)(a.y - (double)h.y),
                      (float)(b.x - (double)h.z), (float)(b.y - (double)h.w));
  }
  // the tail (n not a multiple of 4)
  const long long t = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0 && t < n) {
    const double v = src[t];
    const float h = (float)v;
    hi[t] = h;
    if (lo) lo[t] = (float)(v - (double)h);
  }
}
__global__ void __launch_bounds__(256)
join_to_host_kernel(const float* __restrict__ hi, const float* __restrict__ lo,
                    double* __restrict__ dst, long long n) {
  const long long n4 = n / 4;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4;
       q += (long long)gridDim.x * blockDim.x) {
    const float4 h = reinterpret_cast<const float4*>(hi)[q];
    float4 l = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lo) l = reinterpret_cast<const float4*>(lo)[q];
    reinterpret_cast<double2*>(dst)[2 * q] =
        make_double2((double)h.x + (double)l.x, (double)h.y + (double)l.y);
    reinterpret_cast<double2*>(dst)[2 * q + 1] =
        make_double2((double)h.z + (double)l.z, (double)h.w + (double)l.w);
  }
  const long long t = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0 && t < n) dst[t] = (double)hi[t] + (lo ? (double)lo[t] : 0.0);
}

// The device address of page-locked host memory (cudaHostAlloc / cudaHostRegister, mapped
// under unified addressing), or nullptr for other memory.  Both kernels above need 16-byte
// alignment of the host array.
const void* pinned_device_ptr(const void* h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();  // clear the error of an unknown pointer
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  if (((uintptr_t)a.devicePointer & 15u) != 0) return nullptr;
  return a.devicePointer;
}

// grid of the host-link conversion kernels: enough CTAs for many requests in flight
unsigned link_grid(long long n) {
  const long long want = ceil_div(ceil_div(n, 4), 256);
  return (unsigned)(want < 152 * 16 ? (want > 0 ? want : 1) : 152 * 16);
}

}  // namespace

namespace athgpu {
// whether the x3 sweep's TMA bulk staging can run on this context (stage_impl.cuh's rule
// without the selection flag)
bool x3_bulk_eligible(const athgpu_ctx* c) {
  const DevMesh& m = c->m;
  if (m.ml.on) return false;
  const long long plane = (long long)m.nc1 * m.nc2, row0 = (long long)(m.js - 1) * m.nc1;
  return (plane * c->real_bytes) % 16 == 0 && (row0 * c->real_bytes) % 16 == 0 &&
         (plane * 8) % 16 == 0 && (row0 * 8) % 16 == 0;
}

// Device memory of the contexts comes from the device's stream-ordered pool, configured to
// keep what is freed (no release threshold): a regrid allocates the new mesh's registers
// while the old ones exist and frees the old ones after, so from the second regrid on the
// pool serves both without a cudaMalloc/cudaFree through the driver.
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s) {
  static int configured_device = -1;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (configured_device != dev) {
    cudaMemPool_t pool;
    e = cudaDeviceGetDefaultMemPool(&pool, dev);
    if (e != cudaSuccess) return e;
    unsigned long long thr = ~0ULL;   // cudaMemPoolAttrReleaseThreshold takes a uint64
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    if (e != cudaSuccess) return e;
    configured_device = dev;
  }
  return cudaMallocAsync(p, bytes, s);
}
}  // namespace athgpu

namespace {

// The ghost elements of one MeshBlock in the order exchange_plan_kernel visits them: the
// cells, then the x1-, x2- and x3-face layouts, each k-major over the whole array; per
// element its in-block offset and (bits 27-31) the offset index of the neighbour owning
// it, as own_map classifies it (below the own range: -1, above: +1; a face layout's own
// range along its normal ends one later).  delta[what][dir] is the in-block shift from a
// ghost element to the owner's (src = dst - delta).  False when an offset needs more
// than 27 bits.
bool build_exchange_plan(const DevMesh& m, std::vector<unsigned>& plan, int n[4],
                         std::vector<int>& delta) {
  for (int what = 0; what < 4; ++what) {
    const int N1 = m.nc1 + (what == 1), N2 = m.nc2 + (what == 2), N3 = m.nc3 + (what == 3);
    if ((long long)N1 * N2 * N3 >= (1LL << 27)) return false;
    const int hi1 = m.ie + (what == 1), hi2 = m.je + (what == 2), hi3 = m.ke + (what == 3);
    const size_t start = plan.size();
    for (int k = 0; k < N3; ++k)
      for (int j = 0; j < N2; ++j)
        for (int i = 0; i < N1; ++i) {
          const int o1 = i < m.is ? -1 : i > hi1 ? 1 : 0;
          const int o2 = j < m.js ? -1 : j > hi2 ? 1 : 0;
          const int o3 = k < m.ks ? -1 : k > hi3 ? 1 : 0;
          if (o1 == 0 && o2 == 0 && o3 == 0) continue;
          const unsigned dir = (unsigned)(((o3 + 1) * 3 + (o2 + 1)) * 3 + (o1 + 1));
          plan.push_back((unsigned)((k * N2 + j) * N1 + i) | (dir << 27));
        }
    n[what] = (int)(plan.size() - start);
    for (int dir = 0; dir < 27; ++dir) {
      const int o1 = dir % 3 - 1, o2 = (dir / 3) % 3 - 1, o3 = dir / 9 - 1;
      delta.push_back(o1 * m.nx1 + o2 * m.nx2 * N1 + o3 * m.nx3 * N1 * N2);
    }
  }
  return true;
}

// The own edges of one MeshBlock that lie on block faces, as edge_fix_kernel visits them:
// x1-directed, then x2- and x3-directed, each k-major.  Per edge its in-block offset and
// the neighbours whose values the average adds, in the reference's order: the face
// neighbours across x1, x2, x3 (those whose face the edge lies on), then for an edge on
// two faces the edge neighbour; each as
// (offset index << 27) | the edge's offset in that neighbour, ~0 when absent.  An edge of
// direction C has own range [s, e] along C and [s, e + 1] across.
void build_edge_plan(const DevMesh& m, std::vector<int4>& plan, int n[3]) {
  for (int C = 0; C < 3; ++C) {
    const int N1 = m.nc1 + (C != 0), N2 = m.nc2 + (C != 1);
    const size_t start = plan.size();
    for (int k = m.ks; k <= m.ke + (C != 2); ++k)
      for (int j = m.js; j <= m.je + (C != 1); ++j)
        for (int i = m.is; i <= m.ie + (C != 0); ++i) {
          const int o1 = C == 0 ? 0 : i == m.is ? -1 : i == m.ie + 1 ? 1 : 0;
          const int o2 = C == 1 ? 0 : j == m.js ? -1 : j == m.je + 1 ? 1 : 0;
          const int o3 = C == 2 ? 0 : k == m.ks ? -1 : k == m.ke + 1 ? 1 : 0;
          if (o1 == 0 && o2 == 0 && o3 == 0) continue;
          unsigned cand[3] = {~0u, ~0u, ~0u};
          int nc = 0;
          auto add = [&](int p1, int p2, int p3) {
            const unsigned dir = (unsigned)(((p3 + 1) * 3 + (p2 + 1)) * 3 + (p1 + 1));
            const int off = ((k - p3 * m.nx3) * N2 + (j - p2 * m.nx2)) * N1 + (i - p1 * m.nx1);
            cand[nc++] = (dir << 27) | (unsigned)off;
          };
          if (o1 != 0) add(o1, 0, 0);
          if (o2 != 0) add(0, o2, 0);
          if (o3 != 0) add(0, 0, o3);
          if ((o1 != 0) + (o2 != 0) + (o3 != 0) == 2) add(o1, o2, o3);
          plan.push_back(make_int4((k * N2 + j) * N1 + i, (int)cand[0], (int)cand[1],
                                   (int)cand[2]));
        }
    n[C] = (int)(plan.size() - start);
  }
}

void free_all(athgpu_ctx* c) {
  Registers& r = c->r;
  void* ptrs[] = {r.u, r.ustar, r.ulo, r.wbuf[0], r.wbuf[1], r.bcc, r.cce, r.dflx, r.e3x1, r.e2x1,
                  r.w1f, r.e1x2, r.e3x2, r.w2f, r.e1x3, r.e2x3, r.w3f, r.e1, r.e2, r.e3,
                  r.b1, r.b2, r.b3, r.bs1, r.bs2, r.bs3, c->clk, c->coords, c->coords32,
                  c->nbr, c->staging, c->c2p_queue, c->c2p_qcount, c->fxv, c->eps_buf,
                  c->c2p_qstart, c->c2p_net, c->c2p_net_err, c->op_flx, c->op_words,
                  c->xplan, c->xdelta, c->eplan, c->escratch};
  // the context's device memory returns to the stream-ordered pool (pool_alloc)
  cudaStream_t s = c->own_stream;
  if (s) cudaStreamSynchronize(c->stream ? c->stream : s);
  for (void* p : ptrs)
    if (p) cudaFreeAsync(p, s);
  for (void* p : c->mld.allocs)
    if (p) cudaFreeAsync(p, s);
  if (s) cudaStreamSynchronize(s);
  for (cudaEvent_t e : c->prof_events) cudaEventDestroy(e);
  if (c->cycle_exec) cudaGraphExecDestroy(c->cycle_exec);
  if (c->cycle_graph) cudaGraphDestroy(c->cycle_graph);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  if (c->aux_stream) cudaStreamDestroy(c->aux_stream);
  for (cudaStream_t cs : c->copy_stream)
    if (cs) cudaStreamDestroy(cs);
  for (cudaEvent_t ce : c->copy_ev)
    if (ce) cudaEventDestroy(ce);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
}

cudaError_t run_stage_dispatch(athgpu_ctx* c, int stage) {
  return c->desc.precision == ATHGPU_FP64 ? stage_fp64(c, stage) : stage_fp32(c, stage);
}

// ---- host <-> device copies of the state ----------------------------------------------
// Copy-engine mode (host_copy_mode 0, the default): each array moves in chunks of
// COPY_CHUNK bytes spread round-robin over the context's copy streams, so several DMA
// copies run at once; in FP32 mode every chunk's conversion (split/join) runs on the
// context's stream, ordered after (upload) or before (download) its own copy by an event,
// so conversions overlap the remaining copies.  Host-link mode (1): the conversion kernels
// read or write page-locked host arrays in place over the link (FP32 contexts).
constexpr long long COPY_CHUNK = 64LL << 20;

cudaEvent_t next_copy_event(athgpu_ctx* c) {
  cudaEvent_t e = c->copy_ev[c->copy_ev_next];
  c->copy_ev_next = (c->copy_ev_next + 1) % athgpu_ctx::NCOPY_EV;
  return e;
}

// the copy streams start after everything queued on the context's stream
cudaError_t fork_copies(athgpu_ctx* c) {
  cudaEvent_t ev = next_copy_event(c);
  cudaError_t e = cudaEventRecord(ev, c->stream);
  for (int q = 0; q < athgpu_ctx::NCOPY && e == cudaSuccess; ++q)
    e = cudaStreamWaitEvent(c->copy_stream[q], ev, 0);
  return e;
}
// the context's stream continues after every copy
cudaError_t join_copies(athgpu_ctx* c) {
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < athgpu_ctx::NCOPY && e == cudaSuccess; ++q) {
    cudaEvent_t ev = next_copy_event(c);
    e = cudaEventRecord(ev, c->copy_stream[q]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, ev, 0);
  }
  return e;
}

// plain FP64 array, host <-> device, chunked over the copy streams (after fork_copies)
athgpu_status copy_chunked(athgpu_ctx* c, void* dst, const void* src, long long bytes,
                           cudaMemcpyKind kind, int* rr) {
  for (long long off = 0; off < bytes; off += COPY_CHUNK) {
    const long long nb = bytes - off < COPY_CHUNK ? bytes - off : COPY_CHUNK;
    CK(cudaMemcpyAsync((char*)dst + off, (const char*)src + off, nb, kind,
                       c->copy_stream[(*rr)++ % athgpu_ctx::NCOPY]));
  }
  return ATHGPU_OK;
}

// host copy of a double array into a bulk-precision device register (after fork_copies)
athgpu_status upload_bulk(athgpu_ctx* c, const double* h, void* dev, void* lo, long long n,
                          int* rr) {
  if (c->real_bytes == 8)
    return copy_chunked(c, dev, h, n * 8, cudaMemcpyHostToDevice, rr);
  const double* hd = c->host_copy_mode == 1 ? (const double*)pinned_device_ptr(h) : nullptr;
  if (hd) {  // page-locked host array: converted while it is read over the link
    split_from_host_kernel<<<link_grid(n), 256, 0, c->stream>>>(hd, (float*)dev, (float*)lo,
                                                                n);
    CK(cudaGetLastError());
    return ATHGPU_OK;
  }
  const long long chunk = COPY_CHUNK / 8;
  for (long long off = 0; off < n; off += chunk) {
    const long long cn = n - off < chunk ? n - off : chunk;
    cudaStream_t cs = c->copy_stream[(*rr)++ % athgpu_ctx::NCOPY];
    CK(cudaMemcpyAsync(c->staging + off, h + off, cn * 8, cudaMemcpyHostToDevice, cs));
    cudaEvent_t ev = next_copy_event(c);
    CK(cudaEventRecord(ev, cs));
    CK(cudaStreamWaitEvent(c->stream, ev, 0));
    split_kernel<<<(unsigned)ceil_div(cn, 256), 256, 0, c->stream>>>(
        c->staging + off, (float*)dev + off, lo ? (float*)lo + off : nullptr, cn);
    CK(cudaGetLastError());
  }
  return ATHGPU_OK;
}

// device register to a host double array (after fork_copies; the caller joins)
athgpu_status download_bulk(athgpu_ctx* c, double* h, const void* dev, const void* lo,
                            long long n, int* rr) {
  if (c->real_bytes == 8)
    return copy_chunked(c, h, dev, n * 8, cudaMemcpyDeviceToHost, rr);
  double* hd = c->host_copy_mode == 1 ? (double*)pinned_device_ptr(h) : nullptr;
  if (hd) {  // page-locked host array: written in place over the link
    join_to_host_kernel<<<link_grid(n), 256, 0, c->stream>>>((const float*)dev,
                                                             (const float*)lo, hd, n);
    CK(cudaGetLastError());
    return ATHGPU_OK;
  }
  const long long chunk = COPY_CHUNK / 8;
  for (long long off = 0; off < n; off += chunk) {
    const long long cn = n - off < chunk ? n - off : chunk;
    join_kernel<<<(unsigned)ceil_div(cn, 256), 256, 0, c->stream>>>(
        (const float*)dev + off, lo ? (const float*)lo + off : nullptr, c->staging + off, cn);
    CK(cudaGetLastError());
    cudaEvent_t ev = next_copy_event(c);
    CK(cudaEventRecord(ev, c->stream));
    cudaStream_t cs = c->copy_stream[(*rr)++ % athgpu_ctx::NCOPY];
    CK(cudaStreamWaitEvent(cs, ev, 0));
    CK(cudaMemcpyAsync(h + off, c->staging + off, cn * 8, cudaMemcpyDeviceToHost, cs));
  }
  return ATHGPU_OK;
}

// ATHGPU_COPY_INTERIOR: the (j, k) range of a block's own cells (or faces) with whole x1
// rows, i.e. per volume (one variable of one MeshBlock) a run of nr rows from row r0 in
// each of np planes from plane p0; as 3-D copies of about COPY_CHUNK bytes each (x =
// the rows' bytes within a plane, y = planes, z = volumes), round-robin over the copy
// streams.  row_bytes: one x1 row; rpp: rows per plane; ppv: planes per volume.
struct Slabs {
  int row_bytes, rpp, r0, nr, ppv, p0, np;
  long long nvol;
  long long vol_elems() const { return (long long)row_bytes / 8 * rpp * ppv; }
  long long chunk_vols() const {
    const long long per = (long long)row_bytes * nr * np;
    const long long v = COPY_CHUNK / (per > 0 ? per : 1);
    return v > 0 ? v : 1;
  }
};
cudaError_t copy_slab_chunk(const Slabs& sl, void* dst, const void* src, long long z0,
                            long long nz, cudaMemcpyKind kind, cudaStream_t cs) {
  cudaMemcpy3DParms p = {};
  const size_t pitch = (size_t)sl.row_bytes * sl.rpp;
  p.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), pitch, pitch, sl.ppv);
  p.dstPtr = make_cudaPitchedPtr(dst, pitch, pitch, sl.ppv);
  p.srcPos = make_cudaPos((size_t)sl.r0 * sl.row_bytes, sl.p0, (size_t)z0);
  p.dstPos = p.srcPos;
  p.extent = make_cudaExtent((size_t)sl.nr * sl.row_bytes, sl.np, (size_t)nz);
  p.kind = kind;
  return cudaMemcpy3DAsync(&p, cs);
}
// a plain FP64 array's slabs, host <-> device (after fork_copies)
athgpu_status copy_slabs(athgpu_ctx* c, const Slabs& sl, void* dst, const void* src,
                         cudaMemcpyKind kind, int* rr) {
  const long long cv = sl.chunk_vols();
  for (long long z0 = 0; z0 < sl.nvol; z0 += cv) {
    const long long nz = sl.nvol - z0 < cv ? sl.nvol - z0 : cv;
    CK(copy_slab_chunk(sl, dst, src, z0, nz, kind,
                       c->copy_stream[(*rr)++ % athgpu_ctx::NCOPY]));
  }
  return ATHGPU_OK;
}
// the slabs of U into a bulk-precision register: FP32 contexts take each chunk through
// the FP64 staging buffer (whole volumes, the same layout) and convert its volumes
athgpu_status upload_slabs(athgpu_ctx* c, const Slabs& sl, const double* h, void* dev,
                           void* lo, int* rr) {
  if (c->real_bytes == 8) return copy_slabs(c, sl, dev, h, cudaMemcpyHostToDevice, rr);
  const long long cv = sl.chunk_vols(), ve = sl.vol_elems();
  for (long long z0 = 0; z0 < sl.nvol; z0 += cv) {
    const long long nz = sl.nvol - z0 < cv ? sl.nvol - z0 : cv;
    cudaStream_t cs = c->copy_stream[(*rr)++ % athgpu_ctx::NCOPY];
    CK(copy_slab_chunk(sl, c->staging, h, z0, nz, cudaMemcpyHostToDevice, cs));
    cudaEvent_t ev = next_copy_event(c);
    CK(cudaEventRecord(ev, cs));
    CK(cudaStreamWaitEvent(c->stream, ev, 0));
    const long long off = z0 * ve, cn = nz * ve;
    split_kernel<<<(unsigned)ceil_div(cn, 256), 256, 0, c->stream>>>(
        c->staging + off, (float*)dev + off, lo ? (float*)lo + off : nullptr, cn);
    CK(cudaGetLastError());
  }
  return ATHGPU_OK;
}
athgpu_status download_slabs(athgpu_ctx* c, const Slabs& sl, double* h, const void* dev,
                             const void* lo, int* rr) {
  if (c->real_bytes == 8) return copy_slabs(c, sl, h, dev, cudaMemcpyDeviceToHost, rr);
  const long long cv = sl.chunk_vols(), ve = sl.vol_elems();
  for (long long z0 = 0; z0 < sl.nvol; z0 += cv) {
    const long long nz = sl.nvol - z0 < cv ? sl.nvol - z0 : cv;
    const long long off = z0 * ve, cn = nz * ve;
    join_kernel<<<(unsigned)ceil_div(cn, 256), 256, 0, c->stream>>>(
        (const float*)dev + off, lo ? (const float*)lo + off : nullptr, c->staging + off, cn);
    CK(cudaGetLastError());
    cudaEvent_t ev = next_copy_event(c);
    CK(cudaEventRecord(ev, c->stream));
    cudaStream_t cs = c->copy_stream[(*rr)++ % athgpu_ctx::NCOPY];
    CK(cudaStreamWaitEvent(cs, ev, 0));
    CK(copy_slab_chunk(sl, h, c->staging, z0, nz, cudaMemcpyDeviceToHost, cs));
  }
  return ATHGPU_OK;
}
// the slab geometry of U (what = 0) and of the face arrays b1..b3 (what = 1..3)
Slabs state_slabs(const DevMesh& m, int what) {
  Slabs s;
  s.row_bytes = (m.nc1 + (what == 1 ? 1 : 0)) * 8;
  s.rpp = m.nc2 + (what == 2 ? 1 : 0);
  s.r0 = m.js;
  s.nr = m.nx2 + (what == 2 ? 1 : 0);
  s.ppv = m.nc3 + (what == 3 ? 1 : 0);
  s.p0 = m.ks;
  s.np = m.nx3 + (what == 3 ? 1 : 0);
  s.nvol = (long long)m.nb * (what == 0 ? 5 : 1);
  return s;
}
}  // namespace

namespace athgpu {
// the error path of the entry points defined in other translation units
athgpu_status api_fail(athgpu_status code, const std::string& msg) { return fail(code, msg); }
}  // namespace athgpu

namespace athgpu {
// lets other translation units report through athgpu_last_error()
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace athgpu

extern "C" {

const char* athgpu_last_error(void) { return g_err.c_str(); }
const char* athgpu_version(void) { return "athena_gb300 0.1 (sm_103a)"; }

}  // extern "C"

namespace athgpu {
// athgpu_create; sync_end = false leaves the context's set-up (register clearing, small
// uploads) running on its stream when it returns (the regrid's new context, whose stream
// the regrid synchronizes after building the multi-level plan on the host meanwhile)
athgpu_status create_context(athgpu_ctx** out, const athgpu_mesh_desc* d, bool sync_end) {
  if (!out || !d) return fail(ATHGPU_ERR_ARG, "null argument");
  *out = nullptr;
  if (d->nbx1 < 1 || d->nbx2 < 1 || d->nbx3 < 1 || d->nx1 < 1 || d->nx2 < 1 || d->nx3 < 1)
    return fail(ATHGPU_ERR_ARG, "mesh sizes must be positive");
  if (d->nx2 < 2 || d->nx3 < 2)
    return fail(ATHGPU_ERR_UNSUPPORTED, "only 3-D meshes (nx2, nx3 > 1) are supported");
  if (d->ppm_fast && d->xorder != 3)
    return fail(ATHGPU_ERR_ARG, "ppm_fast needs xorder 3");
  if (d->xorder < 1 || d->xorder > 3)
    return fail(ATHGPU_ERR_UNSUPPORTED, "xorder must be 1, 2 or 3");
  const int need_ng = d->xorder == 3 ? 3 : 2;
  if (d->nghost < need_ng)
    return fail(ATHGPU_ERR_ARG, "nghost too small for the reconstruction "
                                "(reconstruction.cpp:117-127)");
  if (d->nx1 < d->nghost || d->nx2 < d->nghost || d->nx3 < d->nghost)
    return fail(ATHGPU_ERR_ARG, "MeshBlock smaller than the ghost width");
  if (d->rsolver != ATHGPU_HLLD && d->rsolver != ATHGPU_HLLE && d->rsolver != ATHGPU_LLF &&
      d->rsolver != ATHGPU_ROE && d->rsolver != ATHGPU_LHLLD)
    return fail(ATHGPU_ERR_ARG, "unknown Riemann solver");
  if (d->precision != ATHGPU_FP64 && d->precision != ATHGPU_FP32)
    return fail(ATHGPU_ERR_ARG, "unknown precision");
  if (d->relativistic && (d->rsolver == ATHGPU_ROE || d->rsolver == ATHGPU_LHLLD))
    return fail(ATHGPU_ERR_UNSUPPORTED,
                "relativistic MHD supports the HLLD, HLLE and LLF solvers (hlld_rel.cpp, "
                "hlle_mhd_rel.cpp, llf_mhd_rel.cpp) only");
  if (d->relativistic && !(d->gamma_max > 1.0))
    return fail(ATHGPU_ERR_ARG, "gamma_max must exceed 1 (adiabatic_mhd_sr.cpp:48)");
  if (!d->x1f || !d->dx1f || !d->x2f || !d->dx2f || !d->x3f || !d->dx3f)
    return fail(ATHGPU_ERR_ARG, "coordinate arrays are required");
  if (!(d->gamma > 1.0) || !(d->cfl_number > 0.0))
    return fail(ATHGPU_ERR_ARG, "gamma must exceed 1 and cfl_number be positive");
  if (d->integrator != ATHGPU_VL2 && d->integrator != ATHGPU_RK2)
    return fail(ATHGPU_ERR_ARG, "unknown integrator (ATHGPU_VL2 or ATHGPU_RK2)");
  // the integrator's CFL limit in 3-D (time_integrator.cpp:219-222, 445, checked at
  // :894-900)
  if (d->cfl_number > (d->integrator == ATHGPU_RK2 ? 1.0 : 0.5))
    return fail(ATHGPU_ERR_ARG, "cfl_number exceeds the integrator's limit (0.5 for vl2, "
                                "1.0 for rk2 in 3-D)");
  for (int f = 0; f < 6; ++f) {
    if (d->bc[f] < ATHGPU_BC_PERIODIC || d->bc[f] > ATHGPU_BC_REFLECT)
      return fail(ATHGPU_ERR_ARG, "bc flags must be periodic (0), outflow (1) or reflecting (2)");
    // a periodic face pairs with a periodic face (mesh.cpp:201-220)
    if ((d->bc[f] == ATHGPU_BC_PERIODIC) != (d->bc[f ^ 1] == ATHGPU_BC_PERIODIC))
      return fail(ATHGPU_ERR_ARG, "periodic boundaries must be set on both faces of an axis");
    // the boundary functions read ng cells of the block's own interior
    const int nx = f < 2 ? d->nx1 : f < 4 ? d->nx2 : d->nx3;
    if (d->bc[f] != ATHGPU_BC_PERIODIC && nx < d->nghost)
      return fail(ATHGPU_ERR_ARG, "a block next to a physical boundary needs nx >= nghost");
  }
  {
    // uniform Cartesian spacing within every block (x?rat = 1, coordinates.cpp:126-146):
    // the kernels use the reference's uniform-mesh branches (plm.cpp:103, ppm.cpp:156)
    const long long nbk = (long long)d->nbx1 * d->nbx2 * d->nbx3;
    const int ncs[3] = {d->nx1 + 2 * d->nghost, d->nx2 + 2 * d->nghost, d->nx3 + 2 * d->nghost};
    const double* dxs[3] = {d->dx1f, d->dx2f, d->dx3f};
    for (int dd = 0; dd < 3; ++dd)
      for (long long b = 0; b < nbk; ++b)
        for (int cc = 1; cc < ncs[dd]; ++cc)
          if (dxs[dd][b * ncs[dd] + cc] != dxs[dd][b * ncs[dd]] || !(dxs[dd][b * ncs[dd]] > 0.0))
            return fail(ATHGPU_ERR_UNSUPPORTED,
                        "face spacings must be positive and uniform within each MeshBlock");
  }

  athgpu_ctx* c = new athgpu_ctx();
  c->desc = *d;
  c->real_bytes = d->precision == ATHGPU_FP64 ? 8 : 4;
  DevMesh& m = c->m;
  m.nbx1 = d->nbx1; m.nbx2 = d->nbx2; m.nbx3 = d->nbx3;
  m.nb = d->nbx1 * d->nbx2 * d->nbx3;
  m.nx1 = d->nx1; m.nx2 = d->nx2; m.nx3 = d->nx3; m.ng = d->nghost;
  m.nc1 = d->nx1 + 2 * m.ng; m.nc2 = d->nx2 + 2 * m.ng; m.nc3 = d->nx3 + 2 * m.ng;
  m.is = m.ng; m.ie = m.ng + m.nx1 - 1;
  m.js = m.ng; m.je = m.ng + m.nx2 - 1;
  m.ks = m.ng; m.ke = m.ng + m.nx3 - 1;
  m.ncell = (i64)m.nc1 * m.nc2 * m.nc3;
  m.fd_nc1 = make_fastdiv(m.nc1);
  m.fd_nc2 = make_fastdiv(m.nc2);
  m.fd_n1 = make_fastdiv(m.nx1 + 1);
  m.fd_n2 = make_fastdiv(m.nx2 + 1);
  m.fd_r1 = make_fastdiv(m.nx1 + 2);
  m.fd_r2 = make_fastdiv(m.nx2 + 2);
  m.nf1 = (i64)m.nc3 * m.nc2 * (m.nc1 + 1);
  m.nf2 = (i64)m.nc3 * (m.nc2 + 1) * m.nc1;
  m.nf3 = (i64)(m.nc3 + 1) * m.nc2 * m.nc1;
  m.ne1 = (i64)(m.nc3 + 1) * (m.nc2 + 1) * m.nc1;
  m.ne2 = (i64)(m.nc3 + 1) * m.nc2 * (m.nc1 + 1);
  m.ne3 = (i64)m.nc3 * (m.nc2 + 1) * (m.nc1 + 1);
  m.gamma = d->gamma; m.dfloor = d->dfloor; m.pfloor = d->pfloor;
  m.gammaf = (float)d->gamma; m.dfloorf = (float)d->dfloor; m.pfloorf = (float)d->pfloor;
  m.any_bc = 0;
  for (int f = 0; f < 6; ++f) {
    m.bc[f] = d->bc[f];
    if (d->bc[f] != ATHGPU_BC_PERIODIC) m.any_bc = 1;
  }
  m.cfl = d->cfl_number; m.tlim = d->tlim;
  m.ncmax = m.nc1 > m.nc2 ? (m.nc1 > m.nc3 ? m.nc1 : m.nc3) : (m.nc2 > m.nc3 ? m.nc2 : m.nc3);

  auto bail = [&](athgpu_status s) {
    free_all(c);
    delete c;
    return s;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
  c->stream = c->own_stream;
  e = cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate aux"));
  e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaEventCreate"));
  e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaEventCreate"));
  for (int q = 0; q < athgpu_ctx::NCOPY && e == cudaSuccess; ++q)
    e = cudaStreamCreateWithFlags(&c->copy_stream[q], cudaStreamNonBlocking);
  for (int q = 0; q < athgpu_ctx::NCOPY_EV && e == cudaSuccess; ++q)
    e = cudaEventCreateWithFlags(&c->copy_ev[q], cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(cuda_fail(e, "copy streams"));

  const i64 nb = m.nb, rb = c->real_bytes;
  Registers& r = c->r;
  struct A { void** p; i64 bytes; };
  std::vector<A> allocs = {
      {&r.u, nb * 5 * m.ncell * rb}, {&r.ustar, nb * 5 * m.ncell * rb},
      {&r.wbuf[0], nb * 5 * m.ncell * rb}, {&r.wbuf[1], nb * 5 * m.ncell * rb},
      {&r.bcc, nb * 3 * m.ncell * rb}, {&r.cce, nb * 3 * m.ncell * rb},
      {&r.dflx, nb * 5 * m.ncell * rb},
      {&r.e3x1, nb * m.nf1 * rb}, {&r.e2x1, nb * m.nf1 * rb}, {&r.w1f, nb * m.nf1 * rb},
      {&r.e1x2, nb * m.nf2 * rb}, {&r.e3x2, nb * m.nf2 * rb}, {&r.w2f, nb * m.nf2 * rb},
      {&r.e1x3, nb * m.nf3 * rb}, {&r.e2x3, nb * m.nf3 * rb}, {&r.w3f, nb * m.nf3 * rb},
      {&r.e1, nb * m.ne1 * rb}, {&r.e2, nb * m.ne2 * rb}, {&r.e3, nb * m.ne3 * rb},
      {(void**)&r.b1, nb * m.nf1 * 8}, {(void**)&r.b2, nb * m.nf2 * 8},
      {(void**)&r.b3, nb * m.nf3 * 8}, {(void**)&r.bs1, nb * m.nf1 * 8},
      {(void**)&r.bs2, nb * m.nf2 * 8}, {(void**)&r.bs3, nb * m.nf3 * 8},
      {(void**)&c->clk, (i64)sizeof(DevClock)}};
  if (rb == 4) {
    allocs.push_back({&r.ulo, nb * 5 * m.ncell * rb});
    allocs.push_back({(void**)&c->staging, nb * 5 * m.ncell * 8});
  }
  // W(U)'s list of cells to finish later: SR solves deferred to the second pass, or the
  // floors' rewrite of U (Newtonian)
  allocs.push_back({(void**)&c->c2p_queue, nb * m.nx1 * m.nx2 * m.nx3 * (i64)sizeof(int)});
  allocs.push_back({(void**)&c->c2p_qcount, (i64)sizeof(unsigned)});
  if (d->relativistic) {
    // the start pressure of each deferred SR solve, and the network start's error flag
    allocs.push_back({(void**)&c->c2p_qstart, nb * m.nx1 * m.nx2 * m.nx3 * (i64)sizeof(double)});
    allocs.push_back({(void**)&c->c2p_net_err, (i64)sizeof(int)});
  }
  // the FP32 path starts the SR solve from the stale pressure refined in FP32, the FP64
  // path from the stale pressure itself (the reference's start)
  c->c2p_start = rb == 4 ? C2P_START_REFINED : C2P_START_STALE;
  for (auto& a : allocs) {
    // 4 KB beyond every register: the x3 sweep's bulk staging copies whole 128-element rows,
    // and the last CTA of the last k-plane of an array overhangs its end (never used)
    a.bytes += 4096;
    e = pool_alloc(a.p, a.bytes, c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMallocAsync"));
  }

  // coordinates: dx?f [nb][nc?] and the PLM interface coefficients
  // (x?f(c+1)-x?v(c))/dx?f(c), (x?v(c)-x?f(c))/dx?f(c) with x?v = (x?f(c+1)+x?f(c))/2
  // (plm.cpp:148-152, cartesian.cpp:28-32), laid out [nb][3][2][ncmax]
  const int nc[3] = {m.nc1, m.nc2, m.nc3};
  const double* xf[3] = {d->x1f, d->x2f, d->x3f};
  const double* dxf[3] = {d->dx1f, d->dx2f, d->dx3f};
  const i64 ncoord = nb * (m.nc1 + m.nc2 + m.nc3) + nb * 6 * m.ncmax;
  std::vector<double> hc(ncoord, 0.0);
  i64 off = 0;
  i64 dxoff[3];
  for (int dd = 0; dd < 3; ++dd) {
    dxoff[dd] = off;
    memcpy(&hc[off], dxf[dd], sizeof(double) * nb * nc[dd]);
    off += nb * nc[dd];
  }
  const i64 plmoff = off;
  for (i64 b = 0; b < nb; ++b)
    for (int dd = 0; dd < 3; ++dd)
      for (int cc = 0; cc < nc[dd]; ++cc) {
        const double* f = xf[dd] + b * (nc[dd] + 1);
        const double* df = dxf[dd] + b * nc[dd];
        double xv = 0.5 * (f[cc + 1] + f[cc]);
        hc[plmoff + ((b * 3 + dd) * 2 + 0) * m.ncmax + cc] = (f[cc + 1] - xv) / df[cc];
        hc[plmoff + ((b * 3 + dd) * 2 + 1) * m.ncmax + cc] = (xv - f[cc]) / df[cc];
      }
  // (the small uploads below are stream-ordered after their allocations and before the
  // registers' clearing, so none of them waits for it)
  e = pool_alloc((void**)&c->coords, sizeof(double) * ncoord, c->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMallocAsync coords"));
  e = cudaMemcpyAsync(c->coords, hc.data(), sizeof(double) * ncoord, cudaMemcpyHostToDevice,
                      c->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy coords"));
  m.dx1f = c->coords + dxoff[0];
  m.dx2f = c->coords + dxoff[1];
  m.dx3f = c->coords + dxoff[2];
  m.plm = c->coords + plmoff;
  {  // FP32 copies: the FP32 kernels read these instead of converting on the FP64 pipe
    std::vector<float> hf(ncoord);
    for (i64 q = 0; q < ncoord; ++q) hf[q] = (float)hc[q];
    e = pool_alloc((void**)&c->coords32, sizeof(float) * ncoord, c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMallocAsync coords32"));
    e = cudaMemcpyAsync(c->coords32, hf.data(), sizeof(float) * ncoord,
                        cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy coords32"));
    m.dx1f32 = c->coords32 + dxoff[0];
    m.dx2f32 = c->coords32 + dxoff[1];
    m.dx3f32 = c->coords32 + dxoff[2];
    m.plm32 = c->coords32 + plmoff;
  }

  {  // cell centres x?v = (x?f(c+1) + x?f(c))/2 per block (cartesian.cpp:26-28)
    std::vector<double> hv(nb * (m.nc1 + m.nc2 + m.nc3));
    i64 o = 0;
    for (int dd = 0; dd < 3; ++dd)
      for (i64 b = 0; b < nb; ++b)
        for (int cc = 0; cc < nc[dd]; ++cc) {
          const double* f = xf[dd] + b * (nc[dd] + 1);
          hv[o++] = 0.5 * (f[cc + 1] + f[cc]);
        }
    e = pool_alloc((void**)&c->fxv, sizeof(double) * hv.size(), c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMallocAsync fxv"));
    e = cudaMemcpyAsync(c->fxv, hv.data(), sizeof(double) * hv.size(), cudaMemcpyHostToDevice,
                        c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy fxv"));
  }

  // neighbour table of the block grid: periodic mesh faces wrap, across a physical mesh
  // face there is no neighbour (-1)
  std::vector<int> hn(nb * 27);
  const int nbx[3] = {m.nbx1, m.nbx2, m.nbx3};
  for (i64 b = 0; b < nb; ++b) {
    const int l[3] = {(int)(b % m.nbx1), (int)((b / m.nbx1) % m.nbx2),
                      (int)(b / ((i64)m.nbx1 * m.nbx2))};
    for (int o3 = -1; o3 <= 1; ++o3)
      for (int o2 = -1; o2 <= 1; ++o2)
        for (int o1 = -1; o1 <= 1; ++o1) {
          const int o[3] = {o1, o2, o3};
          int a[3];
          bool none = false;
          for (int d = 0; d < 3; ++d) {
            int t = l[d] + o[d];
            if (t < 0 || t >= nbx[d]) {
              if (m.bc[2 * d + (t < 0 ? 0 : 1)] != ATHGPU_BC_PERIODIC) none = true;
              t = (t + nbx[d]) % nbx[d];
            }
            a[d] = t;
          }
          hn[b * 27 + ((o3 + 1) * 3 + (o2 + 1)) * 3 + (o1 + 1)] =
              none ? -1 : (a[2] * m.nbx2 + a[1]) * m.nbx1 + a[0];
        }
  }
  e = pool_alloc((void**)&c->nbr, sizeof(int) * hn.size(), c->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMallocAsync nbr"));
  e = cudaMemcpyAsync(c->nbr, hn.data(), sizeof(int) * hn.size(), cudaMemcpyHostToDevice,
                      c->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy nbr"));
  m.nbr = c->nbr;

  {  // the blocks' ghost plan for the same-level exchange (exchange_plan_kernel)
    std::vector<unsigned> plan;
    std::vector<int> delta;
    if (!build_exchange_plan(m, plan, c->xplan_n, delta))
      return bail(fail(ATHGPU_ERR_UNSUPPORTED, "MeshBlock too large for the ghost plan"));
    e = pool_alloc((void**)&c->xplan, sizeof(unsigned) * plan.size(), c->stream);
    if (e == cudaSuccess)
      e = pool_alloc((void**)&c->xdelta, sizeof(int) * delta.size(), c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->xplan, plan.data(), sizeof(unsigned) * plan.size(),
                          cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->xdelta, delta.data(), sizeof(int) * delta.size(),
                          cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "ghost plan"));
  }
  {  // the blocks' face edges for the same-level edge averaging (edge_fix_kernel)
    std::vector<int4> plan;
    build_edge_plan(m, plan, c->eplan_n);
    e = pool_alloc((void**)&c->eplan, sizeof(int4) * plan.size(), c->stream);
    if (e == cudaSuccess)
      e = pool_alloc(&c->escratch, (size_t)c->real_bytes * plan.size() * nb, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->eplan, plan.data(), sizeof(int4) * plan.size(),
                          cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "edge plan"));
  }

  DevClock hclk;
  memset(&hclk, 0, sizeof(hclk));
  hclk.dt = DBL_MAX;  // mesh.cpp:100
  hclk.time = 0.0;
  double dmax = DBL_MAX;
  memcpy(&hclk.dtmin_bits, &dmax, 8);
  hclk.c2p_floor_count = 0;
  hclk.dtf = (float)hclk.dt;
  hclk.dt_prev = DBL_MAX;
  hclk.dtmin_prev_bits = hclk.dtmin_bits;
  // the registers start cleared (the tables above are not among them), then the clock,
  // which is (pageable copies are staged at once: none of this waits on the host)
  for (auto& a : allocs) {
    e = cudaMemsetAsync(*a.p, 0, a.bytes, c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemset"));
  }
  e = cudaMemcpyAsync(c->clk, &hclk, sizeof(hclk), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy clock"));
  if (sync_end) {
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "create sync"));
  }
  *out = c;
  return ATHGPU_OK;
}
}  // namespace athgpu

extern "C" {

athgpu_status athgpu_create(athgpu_ctx** out, const athgpu_mesh_desc* d) {
  return athgpu::create_context(out, d, true);
}

}  // extern "C"

namespace athgpu {
// a device copy of host data (or a cleared array for h = NULL), stream-ordered on the
// context's stream and released with the context
static cudaError_t ml_dev(athgpu_ctx* c, const void* h, size_t bytes, void** out) {
  *out = nullptr;
  if (bytes == 0) return cudaSuccess;
  cudaError_t e = pool_alloc(out, bytes, c->stream);
  if (e != cudaSuccess) return e;
  c->mld.allocs.push_back(*out);
  if (h) return cudaMemcpyAsync(*out, h, bytes, cudaMemcpyHostToDevice, c->stream);
  return cudaMemsetAsync(*out, 0, bytes, c->stream);
}
#define DEV(h, bytes, field)                                                           \
  do {                                                                                 \
    void* p_;                                                                          \
    cudaError_t e_ = ml_dev(c, h, bytes, &p_);                                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, "multi-level allocation");             \
    field = (decltype(field))p_;                                                       \
  } while (0)

// athgpu_set_multilevel, first part: the checks, the coarse buffers, correction arrays,
// neighbour tables and coarse coordinates (what the regrid's copies and prolongation use),
// stream-ordered on the context's stream without waiting
athgpu_status ml_prepare(athgpu_ctx* c, const int* nbr_table, const int* nbr_count,
                         const int* nblevel, const long long* loc, const double* cx1f,
                         const double* cx2f, const double* cx3f) {
  if (!c || !nbr_table || !nbr_count || !nblevel || !loc || !cx1f || !cx2f || !cx3f)
    return fail(ATHGPU_ERR_ARG, "null argument");
  if (c->initialized || c->m.ml.on)
    return fail(ATHGPU_ERR_STATE, "athgpu_set_multilevel must come before athgpu_initialize");
  if (c->desc.relativistic)
    return fail(ATHGPU_ERR_UNSUPPORTED, "mesh refinement supports Newtonian MHD only");
  if (c->desc.rsolver == ATHGPU_LHLLD)
    return fail(ATHGPU_ERR_UNSUPPORTED,
                "mesh refinement supports the HLLD, HLLE, LLF and Roe solvers");
  DevMesh& m = c->m;
  if (m.ng % 2)
    return fail(ATHGPU_ERR_ARG, "mesh refinement needs an even nghost (mesh_refinement.cpp:44)");
  if (m.nx1 % 2 || m.nx2 % 2 || m.nx3 % 2 || m.nx1 / 2 < 2 || m.nx2 / 2 < 2 || m.nx3 / 2 < 2)
    return fail(ATHGPU_ERR_ARG, "mesh refinement needs even MeshBlock sizes of at least 4");
  const int nb = m.nb;
  DevML& L = m.ml;
  const int rb = c->real_bytes;
  const int cng = (m.ng + 1) / 2 + 1;
  L.cng = cng;
  L.ncc1 = m.nx1 / 2 + 2 * m.ng; L.ncc2 = m.nx2 / 2 + 2 * m.ng; L.ncc3 = m.nx3 / 2 + 2 * m.ng;
  L.cis = m.ng; L.cie = m.ng + m.nx1 / 2 - 1;
  L.cjs = m.ng; L.cje = m.ng + m.nx2 / 2 - 1;
  L.cks = m.ng; L.cke = m.ng + m.nx3 / 2 - 1;
  L.nccell = (i64)L.ncc1 * L.ncc2 * L.ncc3;
  L.ncf1 = (i64)L.ncc3 * L.ncc2 * (L.ncc1 + 1);
  L.ncf2 = (i64)L.ncc3 * (L.ncc2 + 1) * L.ncc1;
  L.ncf3 = (i64)(L.ncc3 + 1) * L.ncc2 * L.ncc1;
  const int nfa = m.nx2 * m.nx3, nfb = m.nx1 * m.nx3, nfc = m.nx1 * m.nx2;
  L.nfmax = nfa > nfb ? (nfa > nfc ? nfa : nfc) : (nfb > nfc ? nfb : nfc);
  // coarse cell centres from the coarse face coordinates
  std::vector<double> cxv[3];
  const double* cxf[3] = {cx1f, cx2f, cx3f};
  const int ncc[3] = {L.ncc1, L.ncc2, L.ncc3};
  for (int d = 0; d < 3; ++d) {
    cxv[d].resize((size_t)nb * ncc[d]);
    for (int b = 0; b < nb; ++b)
      for (int q = 0; q < ncc[d]; ++q)
        cxv[d][(size_t)b * ncc[d] + q] = 0.5 * (cxf[d][(size_t)b * (ncc[d] + 1) + q + 1] +
                                                 cxf[d][(size_t)b * (ncc[d] + 1) + q]);
  }
  const void* nullh = nullptr;
  c->mld.hloc.assign(loc, loc + (size_t)nb * 4);
  DEV(nblevel, sizeof(int) * (size_t)nb * 27, L.nblev);
  DEV(nbr_table, sizeof(int) * (size_t)nb * ML_MAXNB * ML_NF, L.nbrt);
  DEV(nbr_count, sizeof(int) * (size_t)nb, L.nnbr);
  DEV(nullh, (size_t)nb * 5 * L.nccell * rb, L.ccons);
  DEV(nullh, (size_t)nb * 5 * L.nccell * rb, L.cprim);
  DEV(nullh, (size_t)nb * 3 * L.nccell * rb, L.cbcc);
  DEV(nullh, (size_t)nb * 5 * L.nccell * rb, L.scons);
  DEV(nullh, (size_t)nb * L.ncf1 * 8, L.cb1);
  DEV(nullh, (size_t)nb * L.ncf2 * 8, L.cb2);
  DEV(nullh, (size_t)nb * L.ncf3 * 8, L.cb3);
  DEV(nullh, (size_t)nb * L.ncf1 * 8, L.sb1);
  DEV(nullh, (size_t)nb * L.ncf2 * 8, L.sb2);
  DEV(nullh, (size_t)nb * L.ncf3 * 8, L.sb3);
  DEV(cxv[0].data(), sizeof(double) * cxv[0].size(), L.cx1v);
  DEV(cxv[1].data(), sizeof(double) * cxv[1].size(), L.cx2v);
  DEV(cxv[2].data(), sizeof(double) * cxv[2].size(), L.cx3v);
  L.fx1v = c->fxv;
  L.fx2v = c->fxv + (size_t)nb * m.nc1;
  L.fx3v = c->fxv + (size_t)nb * (m.nc1 + m.nc2);
  DEV(nullh, (size_t)nb * 6 * L.nfmax * 5 * rb, L.fcorr);
  DEV(nullh, (size_t)nb * m.ne1 * rb, L.ecorr1);
  DEV(nullh, (size_t)nb * m.ne2 * rb, L.ecorr2);
  DEV(nullh, (size_t)nb * m.ne3 * rb, L.ecorr3);
  // the 27-entry table now only marks which neighbours exist (the boundary kernels'
  // has-neighbour test): the block itself for an existing one, -1 for none
  std::vector<int> hn((size_t)nb * 27);
  for (int b = 0; b < nb; ++b)
    for (int q = 0; q < 27; ++q) hn[(size_t)b * 27 + q] = nblevel[(size_t)b * 27 + q] < 0 ? -1 : b;
  CK(cudaMemcpyAsync(c->nbr, hn.data(), sizeof(int) * hn.size(), cudaMemcpyHostToDevice,
                     c->stream));
  L.on = 1;
  if (c->cycle_exec) { cudaGraphExecDestroy(c->cycle_exec); c->cycle_exec = nullptr; }
  if (c->cycle_graph) { cudaGraphDestroy(c->cycle_graph); c->cycle_graph = nullptr; }
  return ATHGPU_OK;
}

// second part: the multi-level plan (built on the host) and its device copies; waits
// for the context's stream at the end
athgpu_status ml_plan_upload(athgpu_ctx* c, const int* nbr_table, const int* nbr_count,
                             const int* nblevel, const long long* loc) {
  DevMesh& m = c->m;
  DevML& L = m.ml;
  const int nb = m.nb;
  MlDims dims;
  dims.nx[0] = m.nx1; dims.nx[1] = m.nx2; dims.nx[2] = m.nx3;
  dims.ng = m.ng;
  for (int f = 0; f < 6; ++f) dims.bc[f] = m.bc[f];
  MlPlan& plan = c->mlplan;
  std::string err;
  if (!build_ml_plan(dims, nb, nbr_table, nbr_count, nblevel, loc, &plan, &err))
    return fail(ATHGPU_ERR_ARG, err.c_str());
  DEV(plan.eflag.data(), sizeof(int) * plan.eflag.size(), L.eflag);
  DEV(plan.nfine.data(), sizeof(int) * plan.nfine.size(), L.nfine);
  DEV(plan.fmask.data(), sizeof(int) * plan.fmask.size(), L.fmask);
  DEV(plan.level.data(), sizeof(int) * plan.level.size(), L.level);
  MlOpList* lists[3] = {&plan.r, &plan.x, &plan.p};
  for (int ph = 0; ph < 3; ++ph) {
    c->mld.nblk[ph] = (int)lists[ph]->blk.size();
    DEV(lists[ph]->ops.data(), sizeof(MlOp) * lists[ph]->ops.size(), c->mld.ops[ph]);
    DEV(lists[ph]->off.data(), sizeof(int) * lists[ph]->off.size(), c->mld.off[ph]);
    DEV(lists[ph]->blk.data(), sizeof(int) * lists[ph]->blk.size(), c->mld.blk[ph]);
  }
  c->mld.nflux = (int)plan.flux_tasks.size();
  DEV(plan.flux_tasks.data(), sizeof(MlFluxTask) * plan.flux_tasks.size(), c->mld.flux_tasks);
  CK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}
#undef DEV
}  // namespace athgpu

extern "C" {

athgpu_status athgpu_set_multilevel(athgpu_ctx* c, const int* nbr_table,
                                    const int* nbr_count, const int* nblevel,
                                    const long long* loc, const double* cx1f,
                                    const double* cdx1f, const double* cx2f,
                                    const double* cdx2f, const double* cx3f,
                                    const double* cdx3f) {
  (void)cdx1f; (void)cdx2f; (void)cdx3f;
  athgpu_status st = athgpu::ml_prepare(c, nbr_table, nbr_count, nblevel, loc, cx1f, cx2f, cx3f);
  if (st != ATHGPU_OK) return st;
  return athgpu::ml_plan_upload(c, nbr_table, nbr_count, nblevel, loc);
}

athgpu_status athgpu_ml_plan_check(const int* nx, int nghost, const int* bc, int nblocks,
                                   const int* nbr_table, const int* nbr_count,
                                   const int* nblevel, const long long* loc,
                                   long long* counts) {
  if (!nx || !bc || !nbr_table || !nbr_count || !nblevel || !loc || nblocks < 1)
    return fail(ATHGPU_ERR_ARG, "null argument");
  MlDims dims;
  for (int a = 0; a < 3; ++a) dims.nx[a] = nx[a];
  dims.ng = nghost;
  for (int f = 0; f < 6; ++f) dims.bc[f] = bc[f];
  MlPlan plan;
  std::string err;
  if (!build_ml_plan(dims, nblocks, nbr_table, nbr_count, nblevel, loc, &plan, &err))
    return fail(ATHGPU_ERR_ARG, err.c_str());
  if (counts) {
    counts[0] = (long long)plan.r.ops.size();
    counts[1] = (long long)plan.x.ops.size();
    counts[2] = (long long)plan.p.ops.size();
    counts[3] = (long long)plan.flux_tasks.size();
  }
  return ATHGPU_OK;
}

athgpu_status athgpu_destroy(athgpu_ctx* c) {
  if (!c) return ATHGPU_OK;
  cudaStreamSynchronize(c->stream);
  free_all(c);
  delete c;
  return ATHGPU_OK;
}

athgpu_status athgpu_set_stream(athgpu_ctx* c, void* stream) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->stream));
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return ATHGPU_OK;
}

athgpu_status athgpu_upload_state(athgpu_ctx* c, const double* u, const double* b1,
                                  const double* b2, const double* b3) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  const DevMesh& m = c->m;
  athgpu_status s;
  int rr = 0;
  CK(fork_copies(c));
  if (c->copy_extent == ATHGPU_COPY_INTERIOR) {
    double* fb[3] = {c->r.b1, c->r.b2, c->r.b3};
    const double* hb[3] = {b1, b2, b3};
    for (int d = 0; d < 3; ++d)
      if (hb[d] && (s = copy_slabs(c, state_slabs(m, d + 1), fb[d], hb[d],
                                   cudaMemcpyHostToDevice, &rr)))
        return s;
    if (u && (s = upload_slabs(c, state_slabs(m, 0), u, c->r.u, c->r.ulo, &rr))) return s;
    CK(join_copies(c));
    CK(cudaStreamSynchronize(c->stream));
    return ATHGPU_OK;
  }
  // the face fields first: plain copies that need no conversion
  if (b1 && (s = copy_chunked(c, c->r.b1, b1, m.nb * m.nf1 * 8, cudaMemcpyHostToDevice, &rr)))
    return s;
  if (b2 && (s = copy_chunked(c, c->r.b2, b2, m.nb * m.nf2 * 8, cudaMemcpyHostToDevice, &rr)))
    return s;
  if (b3 && (s = copy_chunked(c, c->r.b3, b3, m.nb * m.nf3 * 8, cudaMemcpyHostToDevice, &rr)))
    return s;
  if (u && (s = upload_bulk(c, u, c->r.u, c->r.ulo, (i64)m.nb * 5 * m.ncell, &rr)))
    return s;
  CK(join_copies(c));
  CK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_upload_prim(athgpu_ctx* c, const double* w) {
  if (!c || !w) return fail(ATHGPU_ERR_ARG, "null argument");
  const i64 n = (i64)c->m.nb * 5 * c->m.ncell;
  athgpu_status s;
  int rr = 0;
  CK(fork_copies(c));
  if ((s = upload_bulk(c, w, c->r.wbuf[0], nullptr, n, &rr)) != ATHGPU_OK) return s;
  CK(join_copies(c));
  // the second primitive buffer: the same values, copied on the device
  CK(cudaMemcpyAsync(c->r.wbuf[1], c->r.wbuf[0], n * c->real_bytes, cudaMemcpyDeviceToDevice,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_download_state(athgpu_ctx* c, double* u, double* b1, double* b2,
                                    double* b3) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  const DevMesh& m = c->m;
  athgpu_status s;
  int rr = 0;
  // the stages do not keep U's ghost cells: refresh them from their owners first (the
  // exchange also rewrites the face fields' ghosts), then every copy follows it
  if (u) CK(c->desc.precision == ATHGPU_FP64 ? exchange_u_fp64(c) : exchange_u_fp32(c));
  CK(fork_copies(c));
  if (c->copy_extent == ATHGPU_COPY_INTERIOR) {
    const double* fb[3] = {c->r.b1, c->r.b2, c->r.b3};
    double* hb[3] = {b1, b2, b3};
    for (int d = 0; d < 3; ++d)
      if (hb[d] && (s = copy_slabs(c, state_slabs(m, d + 1), hb[d], fb[d],
                                   cudaMemcpyDeviceToHost, &rr)))
        return s;
    if (u && (s = download_slabs(c, state_slabs(m, 0), u, c->r.u, c->r.ulo, &rr))) return s;
    CK(join_copies(c));
    CK(cudaStreamSynchronize(c->stream));
    return ATHGPU_OK;
  }
  if (b1 && (s = copy_chunked(c, b1, c->r.b1, m.nb * m.nf1 * 8, cudaMemcpyDeviceToHost, &rr)))
    return s;
  if (b2 && (s = copy_chunked(c, b2, c->r.b2, m.nb * m.nf2 * 8, cudaMemcpyDeviceToHost, &rr)))
    return s;
  if (b3 && (s = copy_chunked(c, b3, c->r.b3, m.nb * m.nf3 * 8, cudaMemcpyDeviceToHost, &rr)))
    return s;
  if (u && (s = download_bulk(c, u, c->r.u, c->r.ulo, (i64)m.nb * 5 * m.ncell, &rr)))
    return s;
  CK(join_copies(c));
  CK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_download_prim(athgpu_ctx* c, double* w, double* bcc) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  const DevMesh& m = c->m;
  athgpu_status s;
  int rr = 0;
  CK(fork_copies(c));
  if (w && (s = download_bulk(c, w, c->r.wbuf[c->r.wsel], nullptr, (i64)m.nb * 5 * m.ncell,
                              &rr)) != ATHGPU_OK)
    return s;
  // FP32: bcc's conversions reuse the staging buffer once w's copies out of it are done
  if (w && bcc && c->real_bytes == 4) CK(join_copies(c));
  if (bcc && (s = download_bulk(c, bcc, c->r.bcc, nullptr, (i64)m.nb * 3 * m.ncell, &rr)) !=
                 ATHGPU_OK)
    return s;
  CK(join_copies(c));
  CK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_set_host_copy(athgpu_ctx* c, int mode) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  if (mode != 0 && mode != 1) return fail(ATHGPU_ERR_ARG, "host copy mode must be 0 or 1");
  c->host_copy_mode = mode;
  return ATHGPU_OK;
}

athgpu_status athgpu_set_copy_extent(athgpu_ctx* c, int extent) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  if (extent != ATHGPU_COPY_WHOLE && extent != ATHGPU_COPY_INTERIOR)
    return fail(ATHGPU_ERR_ARG, "copy extent must be ATHGPU_COPY_WHOLE or ATHGPU_COPY_INTERIOR");
  c->copy_extent = extent;
  return ATHGPU_OK;
}

athgpu_status athgpu_initialize(athgpu_ctx* c) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  cudaError_t e = c->desc.precision == ATHGPU_FP64 ? init_fp64(c) : init_fp32(c);
  if (e != cudaSuccess) return cuda_fail(e, "initialize");
  CK(cudaStreamSynchronize(c->stream));
  c->initialized = true;
  return ATHGPU_OK;
}

athgpu_status athgpu_stage(athgpu_ctx* c, int stage) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  if (!c->initialized) return fail(ATHGPU_ERR_STATE, "athgpu_initialize not called");
  if (stage != 1 && stage != 2) return fail(ATHGPU_ERR_ARG, "stage must be 1 or 2");
  cudaError_t e = run_stage_dispatch(c, stage);
  if (e != cudaSuccess) return cuda_fail(e, "stage");
  return ATHGPU_OK;
}

athgpu_status athgpu_cycle(athgpu_ctx* c, int ncycles) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  if (!c->initialized) return fail(ATHGPU_ERR_STATE, "athgpu_initialize not called");
  if (ncycles < 0) return fail(ATHGPU_ERR_ARG, "ncycles < 0");
  if (!c->cycle_exec || c->graph_stream != c->stream || c->graph_wsel != c->r.wsel) {
    if (c->cycle_exec) { cudaGraphExecDestroy(c->cycle_exec); c->cycle_exec = nullptr; }
    if (c->cycle_graph) { cudaGraphDestroy(c->cycle_graph); c->cycle_graph = nullptr; }
    long long l0 = c->launches;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e1 = run_stage_dispatch(c, 1);
    cudaError_t e2 = run_stage_dispatch(c, 2);
    cudaError_t e3 = run_stage_dispatch(c, 0);
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
    if (e1 != cudaSuccess) return cuda_fail(e1, "capture stage 1");
    if (e2 != cudaSuccess) return cuda_fail(e2, "capture stage 2");
    if (e3 != cudaSuccess) return cuda_fail(e3, "capture end of cycle");
    if (ee != cudaSuccess) return cuda_fail(ee, "cudaStreamEndCapture");
    c->cycle_graph = g;
    CK(cudaGraphInstantiate(&c->cycle_exec, g, 0));
    c->graph_stream = c->stream;
    c->graph_wsel = c->r.wsel;  // the graph bakes in which primitive buffer is current
    c->per_cycle = c->launches - l0;  // kernels in one replay of the graph
    c->launches = l0;                 // capturing launched nothing

  }
  for (int n = 0; n < ncycles; ++n) {
    CK(cudaGraphLaunch(c->cycle_exec, c->stream));
  }
  c->launches += (long long)ncycles * c->per_cycle;
  return ATHGPU_OK;
}

athgpu_status athgpu_run_until(athgpu_ctx* c, double tlim, int max_cycles, int* nrun) {
  if (!c || !nrun) return fail(ATHGPU_ERR_ARG, "null argument");
  *nrun = 0;
  for (int n = 0; n < max_cycles; ++n) {
    double t, dt;
    athgpu_status s = athgpu_get_clock(c, &t, &dt);
    if (s != ATHGPU_OK) return s;
    if (!(t < tlim)) break;
    s = athgpu_cycle(c, 1);
    if (s != ATHGPU_OK) return s;
    ++*nrun;
  }
  CK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_get_clock(athgpu_ctx* c, double* time, double* dt) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  DevClock h;
  CK(cudaMemcpyAsync(&h, c->clk, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (time) *time = h.time;
  if (dt) *dt = h.dt;
  return ATHGPU_OK;
}

athgpu_status athgpu_set_clock(athgpu_ctx* c, double time, double dt) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  DevClock h;
  CK(cudaMemcpyAsync(&h, c->clk, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  h.time = time;
  h.dt = dt;
  h.dtf = (float)dt;
  CK(cudaMemcpyAsync(c->clk, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_synchronize(athgpu_ctx* c) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_floor_count(athgpu_ctx* c, long long* count, int reset) {
  if (!c || !count) return fail(ATHGPU_ERR_ARG, "null argument");
  DevClock h;
  CK(cudaMemcpyAsync(&h, c->clk, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *count = h.c2p_floor_count;
  if (reset) {
    int z = 0;
    CK(cudaMemcpyAsync((char*)c->clk + offsetof(DevClock, c2p_floor_count), &z, sizeof(int),
                       cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return ATHGPU_OK;
}

athgpu_status athgpu_device_state_ptrs(athgpu_ctx* c, athgpu_device_state* out) {
  if (!c || !out) return fail(ATHGPU_ERR_ARG, "null argument");
  out->u = c->r.u;
  out->ulo = c->r.ulo;
  out->w = c->r.wbuf[c->r.wsel];
  out->bcc = c->r.bcc;
  out->b1 = c->r.b1;
  out->b2 = c->r.b2;
  out->b3 = c->r.b3;
  out->real_bytes = c->real_bytes;
  return ATHGPU_OK;
}

static_assert(ATHGPU_C2P_START_STALE == C2P_START_STALE &&
                  ATHGPU_C2P_START_REFINED == C2P_START_REFINED &&
                  ATHGPU_C2P_START_NETWORK == C2P_START_NETWORK,
              "con2prim start codes out of date");

athgpu_status athgpu_set_c2p_start(athgpu_ctx* c, int start, const float* params) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  if (!c->desc.relativistic)
    return fail(ATHGPU_ERR_UNSUPPORTED, "the con2prim start applies to relativistic MHD");
  if (start != ATHGPU_C2P_START_STALE && start != ATHGPU_C2P_START_REFINED &&
      start != ATHGPU_C2P_START_NETWORK)
    return fail(ATHGPU_ERR_ARG, "unknown con2prim start");
  if (start == ATHGPU_C2P_START_NETWORK) {
    if (!params) return fail(ATHGPU_ERR_ARG, "the network start needs the parameters");
    if (!c->c2p_net) {
      cudaError_t e = pool_alloc((void**)&c->c2p_net, sizeof(float) * ATHGPU_MLP_NPARAM,
                                 c->stream);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync network");
    }
    // host or device memory (unified addressing)
    CK(cudaMemcpyAsync(c->c2p_net, params, sizeof(float) * ATHGPU_MLP_NPARAM,
                       cudaMemcpyDefault, c->stream));
    CK(cudaMemsetAsync(c->c2p_net_err, 0, sizeof(int), c->stream));
  }
  c->c2p_start = start;
  CK(cudaStreamSynchronize(c->stream));
  if (c->cycle_exec) {  // re-capture with the new con2prim kernel
    cudaGraphExecDestroy(c->cycle_exec);
    c->cycle_exec = nullptr;
    cudaGraphDestroy(c->cycle_graph);
    c->cycle_graph = nullptr;
  }
  return ATHGPU_OK;
}

athgpu_status athgpu_get_x3_staging(athgpu_ctx* c, int* bulk) {
  if (!c || !bulk) return fail(ATHGPU_ERR_ARG, "null argument");
  *bulk = (c->lc.x3_bulk && x3_bulk_eligible(c)) ? 1 : 0;
  return ATHGPU_OK;
}

athgpu_status athgpu_set_x3_staging(athgpu_ctx* c, int bulk) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  if (bulk != 0 && bulk != 1) return fail(ATHGPU_ERR_ARG, "x3 staging must be 0 or 1");
  c->lc.x3_bulk = bulk;
  if (c->cycle_exec) {  // re-capture with the other kernel
    CK(cudaStreamSynchronize(c->stream));
    cudaGraphExecDestroy(c->cycle_exec);
    c->cycle_exec = nullptr;
    cudaGraphDestroy(c->cycle_graph);
    c->cycle_graph = nullptr;
  }
  return ATHGPU_OK;
}

athgpu_status athgpu_set_sweep_segment(athgpu_ctx* c, int seg_x2, int seg_x3) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  if (seg_x2 < 0 || seg_x3 < 0) return fail(ATHGPU_ERR_ARG, "negative segment");
  c->lc.seg_x2 = seg_x2;
  c->lc.seg_x3 = seg_x3;
  if (c->cycle_exec) {  // re-capture with the new launch shapes
    CK(cudaStreamSynchronize(c->stream));
    cudaGraphExecDestroy(c->cycle_exec);
    c->cycle_exec = nullptr;
    cudaGraphDestroy(c->cycle_graph);
    c->cycle_graph = nullptr;
  }
  return ATHGPU_OK;
}

athgpu_status athgpu_profile_cycle(athgpu_ctx* c, int cap, float* ms, int* count) {
  if (!c || !ms || !count) return fail(ATHGPU_ERR_ARG, "null argument");
  if (!c->initialized) return fail(ATHGPU_ERR_STATE, "athgpu_initialize not called");
  CK(cudaStreamSynchronize(c->stream));
  for (cudaEvent_t e : c->prof_events) cudaEventDestroy(e);
  c->prof_events.clear();
  c->prof_names.clear();
  c->profiling = true;
  cudaError_t e1 = run_stage_dispatch(c, 1);
  cudaError_t e2 = run_stage_dispatch(c, 2);
  cudaError_t e3 = run_stage_dispatch(c, 0);
  c->profiling = false;
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
    return cuda_fail(e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3, "profile cycle");
  CK(cudaStreamSynchronize(c->stream));
  const int n = (int)c->prof_names.size();
  *count = n;
  for (int i = 0; i < n && i < cap; ++i)
    CK(cudaEventElapsedTime(&ms[i], c->prof_events[2 * i], c->prof_events[2 * i + 1]));
  return ATHGPU_OK;
}

const char* athgpu_profile_label(athgpu_ctx* c, int idx) {
  if (!c || idx < 0 || idx >= (int)c->prof_names.size()) return "";
  return c->prof_names[idx].c_str();
}

namespace {
// Device-to-device snapshot of everything a cycle changes (U and its compensation, both
// primitive buffers, the cell-centred field and E, the face fields, the clock), so that
// tuning runs leave the simulation state untouched.
struct StateSnapshot {
  std::vector<std::pair<void*, size_t>> regs;
  char* store = nullptr;
  DevClock clk;
  int wsel = 0;
};

athgpu_status snapshot(athgpu_ctx* c, StateSnapshot* sn) {
  const DevMesh& m = c->m;
  const size_t rb = c->real_bytes, nb = m.nb, nc = m.ncell;
  Registers& r = c->r;
  sn->regs = {{r.u, nb * 5 * nc * rb},       {r.wbuf[0], nb * 5 * nc * rb},
              {r.wbuf[1], nb * 5 * nc * rb}, {r.bcc, nb * 3 * nc * rb},
              {r.cce, nb * 3 * nc * rb},     {r.b1, nb * m.nf1 * 8},
              {r.b2, nb * m.nf2 * 8},        {r.b3, nb * m.nf3 * 8}};
  if (r.ulo) sn->regs.push_back({r.ulo, nb * 5 * nc * rb});
  size_t total = 0;
  for (auto& q : sn->regs) total += q.second;
  CK(cudaMalloc((void**)&sn->store, total));
  size_t off = 0;
  for (auto& q : sn->regs) {
    CK(cudaMemcpyAsync(sn->store + off, q.first, q.second, cudaMemcpyDeviceToDevice,
                       c->stream));
    off += q.second;
  }
  CK(cudaMemcpyAsync(&sn->clk, c->clk, sizeof(DevClock), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  sn->wsel = r.wsel;
  return ATHGPU_OK;
}

athgpu_status restore(athgpu_ctx* c, StateSnapshot* sn) {
  size_t off = 0;
  for (auto& q : sn->regs) {
    CK(cudaMemcpyAsync(q.first, sn->store + off, q.second, cudaMemcpyDeviceToDevice,
                       c->stream));
    off += q.second;
  }
  CK(cudaMemcpyAsync(c->clk, &sn->clk, sizeof(DevClock), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->r.wsel = sn->wsel;
  CK(cudaFree(sn->store));
  sn->store = nullptr;
  return ATHGPU_OK;
}

// average time of `cycles` cycles (non-graph launches, CUDA events on the stream) after
// one warm-up cycle
athgpu_status time_cycles(athgpu_ctx* c, int cycles, float* ms) {
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  for (int q = 0; q <= cycles; ++q) {
    if (q == 1) CK(cudaEventRecord(a, c->stream));
    CK(run_stage_dispatch(c, 1));
    CK(run_stage_dispatch(c, 2));
    CK(run_stage_dispatch(c, 0));
  }
  CK(cudaEventRecord(b, c->stream));
  CK(cudaEventSynchronize(b));
  CK(cudaEventElapsedTime(ms, a, b));
  *ms /= cycles;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ATHGPU_OK;
}
}  // namespace

athgpu_status athgpu_autotune(athgpu_ctx* c, int cycles, int* seg_x2, int* seg_x3) {
  if (!c) return fail(ATHGPU_ERR_ARG, "null context");
  if (!c->initialized) return fail(ATHGPU_ERR_STATE, "athgpu_initialize not called");
  if (cycles < 1) cycles = 2;
  StateSnapshot sn;
  athgpu_status st = snapshot(c, &sn);
  if (st != ATHGPU_OK) return st;
  const LaunchConfig keep = c->lc;
  // candidate segment lengths: the whole column and its halves down to 4 cells
  auto candidates = [](int n) {
    std::vector<int> v;
    for (int sgl = n; sgl >= 4; sgl /= 2) v.push_back(sgl);
    if (v.empty()) v.push_back(n);
    return v;
  };
  int best2 = c->lc.seg_x2 > 0 ? c->lc.seg_x2 : c->m.nx2;
  int best3 = c->lc.seg_x3 > 0 ? c->lc.seg_x3 : c->m.nx3;
  for (int dir = 2; dir <= 3 && st == ATHGPU_OK; ++dir) {  // coordinate search
    float best_ms = 3.0e38f;
    for (int cand : candidates(dir == 2 ? c->m.nx2 : c->m.nx3)) {
      c->lc.seg_x2 = dir == 2 ? cand : best2;
      c->lc.seg_x3 = dir == 3 ? cand : best3;
      float ms = 0.0f;
      if ((st = time_cycles(c, cycles, &ms)) != ATHGPU_OK) break;
      if (ms < best_ms) {
        best_ms = ms;
        if (dir == 2) best2 = cand; else best3 = cand;
      }
    }
  }
  // the x3 sweep's staging (per-thread cp.async or TMA bulk copies) at those segments
  int best_bulk = c->lc.x3_bulk;
  if (st == ATHGPU_OK) {
    c->lc.seg_x2 = best2;
    c->lc.seg_x3 = best3;
    float best_ms = 3.0e38f;
    for (int bulk = 0; bulk <= 1 && st == ATHGPU_OK; ++bulk) {
      c->lc.x3_bulk = bulk;
      if (bulk && !x3_bulk_eligible(c)) break;
      float ms = 0.0f;
      if ((st = time_cycles(c, cycles, &ms)) != ATHGPU_OK) break;
      if (ms < best_ms) {
        best_ms = ms;
        best_bulk = bulk;
      }
    }
  }
  athgpu_status st2 = restore(c, &sn);
  if (st != ATHGPU_OK) {
    c->lc = keep;
    return st;
  }
  if (st2 != ATHGPU_OK) return st2;
  c->lc = keep;
  c->lc.x3_bulk = best_bulk;
  st = athgpu_set_sweep_segment(c, best2, best3);  // also drops the captured graph
  if (seg_x2) *seg_x2 = best2;
  if (seg_x3) *seg_x3 = best3;
  return st;
}

athgpu_status athgpu_launch_count(athgpu_ctx* c, long long* count, int reset) {
  if (!c || !count) return fail(ATHGPU_ERR_ARG, "null argument");
  *count = c->launches;
  if (reset) c->launches = 0;
  return ATHGPU_OK;
}

}  // extern "C"
