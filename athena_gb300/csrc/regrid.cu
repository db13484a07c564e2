// Adaptive mesh refinement on the device: the blast problem's refinement measure and the
// regrid of a multi-level mesh onto a new block list.
//
// The host decides (refinement flags, tree update, the block maps: athena_gb300/amr.py,
// the reference's MeshRefinement::CheckRefinementCondition and Mesh::UpdateMeshBlockTree);
// this file moves the data (Mesh::RedistributeAndRefineMeshBlocks on one rank,
// mesh/amr_loadbalance.cpp:351-660):
//   1. on the old mesh, every child of a derefined group restricts its U and B into its
//      own coarse buffers (FillSameRankFineToCoarseAMR, :827-946) — the multi-level
//      operation executor with RESTRICT operations;
//   2. one launch of box copies from the old arrays into the new context: kept blocks
//      move whole (with their coarse buffers, which the reference's prolongation stencils
//      read before every part of them is rewritten), restricted children into the octants
//      of their new parent, a refined parent's U and B with a one-cell halo into each new
//      child's coarse buffers (FillSameRankCoarseToFineAMR, :948-1030), and the face-field
//      corrections from old same-level neighbours (ReceiveAndSetFaceFieldCorrection,
//      :1387-1444);
//   3. on the new mesh, ProlongateMeshBlock (:1172-1222) for every new child: U from the
//      coarse U, the shared faces except the corrected ones, the internal faces;
//   4. Initialize(2) (mesh.cpp:1622-1964: exchange, ProlongateBoundaries, W(U), physical
//      boundaries, NewBlockTimeStep + NewTimeStep).
// The arithmetic of steps 1 and 3 is the executor's (FP64, the reference's operand order),
// so the FP64 path stays bit-identical to the reference.
#include <cfloat>
#include <chrono>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/athena_gb300_diag.h"
#include "ctx.h"
#include "ml_plan.h"
#include "multilevel.cuh"

namespace athgpu {
athgpu_status api_fail(athgpu_status code, const std::string& msg);
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s);
athgpu_status create_context(athgpu_ctx** out, const athgpu_mesh_desc* d, bool sync_end);
athgpu_status ml_prepare(athgpu_ctx* c, const int* nbr_table, const int* nbr_count,
                         const int* nblevel, const long long* loc, const double* cx1f,
                         const double* cx2f, const double* cx3f);
athgpu_status ml_plan_upload(athgpu_ctx* c, const int* nbr_table, const int* nbr_count,
                             const int* nblevel, const long long* loc);
}

namespace {
using namespace athgpu;

// host wall time of the phases of the last regrid (athgpu_regrid_profile)
double g_phase_ms[8];
double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---- refinement measure ---------------------------------------------------------------
// pgen/blast.cpp:413-443: per block the maximum over the interior and one ghost layer of
// sqrt(sum_d (0.5 (p(+1) - p(-1)))^2) / p, in the bulk precision (FP64: the reference's
// arithmetic).  One CTA per block.
template <typename Real>
__global__ void __launch_bounds__(256)
refine_eps_kernel(DevMesh m, const Real* __restrict__ w, double* __restrict__ out) {
  using Acc = Real;
  const int b = blockIdx.x;
  const int n1 = m.nx1 + 2, n2 = m.nx2 + 2, n3 = m.nx3 + 2;
  const int tot = n1 * n2 * n3;
  const Real* p = w + ((i64)b * NHYDRO + IPR) * m.ncell;
  const i64 sj = m.nc1, sk = (i64)m.nc1 * m.nc2;
  Acc mx = Acc(0);
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int i = m.is - 1 + t % n1, j = m.js - 1 + (t / n1) % n2, k = m.ks - 1 + t / (n1 * n2);
    const i64 c = k * sk + j * sj + i;
    const Acc a = Acc(0.5) * (p[c + 1] - p[c - 1]);
    const Acc e = Acc(0.5) * (p[c + sj] - p[c - sj]);
    const Acc f = Acc(0.5) * (p[c + sk] - p[c - sk]);
    const Acc eps = sqrt(a * a + e * e + f * f) / p[c];
    mx = (mx < eps) ? eps : mx;
  }
  __shared__ Acc red[256 / 32];
  for (int o = 16; o > 0; o >>= 1) {
    const Acc v = __shfl_down_sync(0xffffffffu, mx, o);
    mx = (mx < v) ? v : mx;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) mx = (mx < red[q]) ? red[q] : mx;
    out[b] = (double)mx;
  }
}

// ---- box copies between the old and the new arrays -------------------------------------
struct RgCopy {
  const char* src;
  char* dst;
  int esize;                  // element bytes: 4 or 8
  int nvar;                   // variables, copied one after the other
  long long svs, dvs;         // variable strides (elements)
  int sn1, sn2, dn1, dn2;     // row and plane lengths (elements) of source, destination
  int s[3], d[3], n[3];       // box origins (i, j, k) and extents
};

// one CTA per copy task
__global__ void __launch_bounds__(256) regrid_copy_kernel(const RgCopy* __restrict__ tasks) {
  const RgCopy t = tasks[blockIdx.x];
  const long long per = (long long)t.n[0] * t.n[1] * t.n[2];
  const long long tot = per * t.nvar;
  for (long long q = threadIdx.x; q < tot; q += blockDim.x) {
    const long long v = q / per, r = q - v * per;
    const int i = (int)(r % t.n[0]);
    const int j = (int)((r / t.n[0]) % t.n[1]);
    const int k = (int)(r / ((long long)t.n[0] * t.n[1]));
    const long long so = v * t.svs + ((long long)(t.s[2] + k) * t.sn2 + (t.s[1] + j)) * t.sn1 +
                         (t.s[0] + i);
    const long long dq = v * t.dvs + ((long long)(t.d[2] + k) * t.dn2 + (t.d[1] + j)) * t.dn1 +
                         (t.d[0] + i);
    if (t.esize == 8)
      reinterpret_cast<double*>(t.dst)[dq] = reinterpret_cast<const double*>(t.src)[so];
    else
      reinterpret_cast<float*>(t.dst)[dq] = reinterpret_cast<const float*>(t.src)[so];
  }
}

// a whole per-block span of `elems` 4-byte words
RgCopy span_copy(const void* src, void* dst, long long elems4) {
  RgCopy t{};
  t.src = (const char*)src;
  t.dst = (char*)dst;
  t.esize = 4;
  t.nvar = 1;
  // one row of elems4 words
  t.n[0] = (int)elems4;
  t.n[1] = t.n[2] = 1;
  t.sn1 = t.dn1 = (int)elems4;
  t.sn2 = t.dn2 = 1;
  return t;
}

struct ArrDims {   // one 3-D array of a block: element size, variable stride, n1, n2
  int esize, n1, n2;
  long long vs;
};

// does the box [o, o + n) of nvar variables lie inside one block's array of `lim`
// elements with rows of n1 and planes of n2 rows?
bool box_inside(const int o[3], const int n[3], int nvar, long long vs, int n1, int n2,
                long long lim) {
  for (int a = 0; a < 3; ++a)
    if (o[a] < 0 || n[a] < 1) return false;
  if (o[0] + n[0] > n1 || o[1] + n[1] > n2) return false;
  const long long last = (long long)(nvar - 1) * vs +
                         ((long long)(o[2] + n[2] - 1) * n2 + (o[1] + n[1] - 1)) * n1 +
                         (o[0] + n[0] - 1);
  return last < lim;
}

// a box copy between one block of a source array (slim elements) and one block of a
// destination array (dlim elements); *ok turns false if either box leaves its block
RgCopy box_copy(const void* sbase, ArrDims sd, long long slim, const void* dbase,
                ArrDims dd, long long dlim, int nvar, const int s[3], const int d[3],
                const int n[3], bool* ok) {
  if (!box_inside(s, n, nvar, sd.vs, sd.n1, sd.n2, slim) ||
      !box_inside(d, n, nvar, dd.vs, dd.n1, dd.n2, dlim))
    *ok = false;
  RgCopy t{};
  t.src = (const char*)sbase;
  t.dst = (char*)dbase;
  t.esize = sd.esize;
  t.nvar = nvar;
  t.svs = sd.vs;
  t.dvs = dd.vs;
  t.sn1 = sd.n1; t.sn2 = sd.n2;
  t.dn1 = dd.n1; t.dn2 = dd.n2;
  for (int a = 0; a < 3; ++a) { t.s[a] = s[a]; t.d[a] = d[a]; t.n[a] = n[a]; }
  return t;
}

template <typename T, typename A>
cudaError_t upload(const std::vector<T, A>& h, T** d, cudaStream_t s) {
  *d = nullptr;
  if (h.empty()) return cudaSuccess;
  cudaError_t e = cudaMallocAsync((void**)d, sizeof(T) * h.size(), s);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
}

// run a list of per-block operations with the multi-level executor on context c
template <typename Real>
cudaError_t run_ops(athgpu_ctx* c, const MlOpList& L) {
  if (L.blk.empty()) return cudaSuccess;
  MlOp* ops;
  int *off, *blk;
  cudaStream_t s = c->stream;
  cudaError_t e = upload(L.ops, &ops, s);
  if (e == cudaSuccess) e = upload(L.off, &off, s);
  if (e == cudaSuccess) e = upload(L.blk, &blk, s);
  if (e != cudaSuccess) return e;
  MlArrays<Real> A{(Real*)c->r.u, (Real*)c->r.wbuf[c->r.wsel], (Real*)c->r.bcc, c->r.b1,
                   c->r.b2, c->r.b3};
  ml_ops_kernel<Real, 2><<<(int)L.blk.size(), 128, 0, s>>>(c->m, A, ops, off, blk);
  c->launches += 1;
  e = cudaGetLastError();
  cudaFreeAsync(ops, s);
  cudaFreeAsync(off, s);
  cudaFreeAsync(blk, s);
  return e;
}

MlOp op_box(int code, int d, int src_kind, const int s[3], const int e[3]) {
  MlOp op{};
  op.code = code;
  op.d = d;
  op.src_kind = src_kind;
  for (int a = 0; a < 3; ++a) { op.s[a] = s[a]; op.e[a] = e[a]; }
  return op;
}

}  // namespace

athgpu_status athgpu_refinement_eps(athgpu_ctx* c, double* maxeps) {
  if (!c || !maxeps) return api_fail(ATHGPU_ERR_ARG, "null argument");
  if (!c->initialized) return api_fail(ATHGPU_ERR_STATE, "athgpu_initialize not called");
  const DevMesh& m = c->m;
  cudaError_t e = cudaSuccess;
  if (!c->eps_buf) e = pool_alloc((void**)&c->eps_buf, sizeof(double) * (size_t)m.nb, c->stream);
  if (e != cudaSuccess) return api_fail(ATHGPU_ERR_CUDA, cudaGetErrorString(e));
  const void* w = c->r.wbuf[c->r.wsel];
  if (c->real_bytes == 8)
    refine_eps_kernel<double><<<m.nb, 256, 0, c->stream>>>(m, (const double*)w, c->eps_buf);
  else
    refine_eps_kernel<float><<<m.nb, 256, 0, c->stream>>>(m, (const float*)w, c->eps_buf);
  c->launches += 1;
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(maxeps, c->eps_buf, sizeof(double) * (size_t)m.nb,
                        cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return api_fail(ATHGPU_ERR_CUDA, cudaGetErrorString(e));
  return ATHGPU_OK;
}

athgpu_status athgpu_regrid(athgpu_ctx* c, const athgpu_mesh_desc* desc, const int* nbr_table,
                            const int* nbr_count, const int* nblevel, const long long* loc,
                            const double* cx1f, const double* cdx1f, const double* cx2f,
                            const double* cdx2f, const double* cx3f, const double* cdx3f,
                            const int* newtoold, const int* kind, int nffc, const int* ffc,
                            int after_cycle) {
  if (!c || !desc || !loc || !newtoold || !kind || (nffc > 0 && !ffc) || nffc < 0)
    return api_fail(ATHGPU_ERR_ARG, "null argument");
  if (!c->initialized || !c->m.ml.on)
    return api_fail(ATHGPU_ERR_STATE, "athgpu_regrid needs an initialized multi-level mesh");
  const DevMesh& om = c->m;
  const athgpu_mesh_desc& od = c->desc;
  if (desc->nbx2 != 1 || desc->nbx3 != 1 || desc->nx1 != od.nx1 || desc->nx2 != od.nx2 ||
      desc->nx3 != od.nx3 || desc->nghost != od.nghost || desc->precision != od.precision ||
      desc->xorder != od.xorder || desc->ppm_fast != od.ppm_fast ||
      desc->rsolver != od.rsolver || desc->relativistic || desc->integrator != od.integrator)
    return api_fail(ATHGPU_ERR_ARG, "the new mesh must keep the block size, nghost, "
                                       "precision, solver and integrator of the old one");
  for (int f = 0; f < 6; ++f)
    if (desc->bc[f] != od.bc[f])
      return api_fail(ATHGPU_ERR_ARG, "the new mesh must keep the boundary flags");
  const int onb = om.nb, nnb = desc->nbx1;
  const std::vector<long long>& ol = c->mld.hloc;
  // the block maps must describe a refinement or derefinement of the old tree
  for (int n = 0; n < nnb; ++n) {
    const int on = newtoold[n];
    const long long* nl = loc + (size_t)n * 4;
    if (on < 0 || on >= onb) return api_fail(ATHGPU_ERR_ARG, "newtoold out of range");
    const long long* p = &ol[(size_t)on * 4];
    bool ok;
    if (kind[n] == 0) {
      ok = p[0] == nl[0] && p[1] == nl[1] && p[2] == nl[2] && p[3] == nl[3];
    } else if (kind[n] == 1) {
      ok = on + 8 <= onb;
      for (int l = 0; ok && l < 8; ++l) {
        const long long* q = &ol[(size_t)(on + l) * 4];
        ok = q[0] == nl[0] + 1 && q[1] == 2 * nl[1] + (l & 1) &&
             q[2] == 2 * nl[2] + ((l >> 1) & 1) && q[3] == 2 * nl[3] + ((l >> 2) & 1);
      }
    } else if (kind[n] == 2) {
      ok = p[0] + 1 == nl[0] && (nl[1] >> 1) == p[1] && (nl[2] >> 1) == p[2] &&
           (nl[3] >> 1) == p[3];
    } else {
      ok = false;
    }
    if (!ok) return api_fail(ATHGPU_ERR_ARG, "block maps inconsistent with the locations");
  }
  for (int t = 0; t < nffc; ++t) {
    const int n = ffc[3 * t], f = ffc[3 * t + 1], i = ffc[3 * t + 2];
    if (n < 0 || n >= nnb || f < 0 || f > 5 || i < 0 || i >= onb || kind[n] != 2 ||
        ol[(size_t)i * 4] != loc[(size_t)n * 4])
      return api_fail(ATHGPU_ERR_ARG, "face-field correction entry out of range");
  }

  // the new context: registers, coordinates and the multi-level plan
  athgpu_ctx* nc = nullptr;
  double tp = now_ms();
  for (int q = 0; q < 8; ++q) g_phase_ms[q] = 0.0;
  auto phase = [&](int q) {
    const double t = now_ms();
    g_phase_ms[q] += t - tp;
    tp = t;
  };
  // The new context's set-up, its copies from the old mesh and the prolongation are
  // queued on its stream first; the host builds the multi-level plan while they run.
  (void)cdx1f; (void)cdx2f; (void)cdx3f;
  athgpu_status st = athgpu::create_context(&nc, desc, false);
  if (st != ATHGPU_OK) return st;
  st = athgpu::ml_prepare(nc, nbr_table, nbr_count, nblevel, loc, cx1f, cx2f, cx3f);
  if (st != ATHGPU_OK) { athgpu_destroy(nc); return st; }
  cudaError_t e = cudaSuccess;
  phase(0);
  nc->lc = c->lc;
  const DevMesh& nm = nc->m;
  const int rb = c->real_bytes;
  const int hx[3] = {nm.nx1 / 2, nm.nx2 / 2, nm.nx3 / 2};
  const int flo[3] = {nm.is, nm.js, nm.ks}, fhi[3] = {nm.ie, nm.je, nm.ke};
  const int clo[3] = {nm.ml.cis, nm.ml.cjs, nm.ml.cks}, chi[3] = {nm.ml.cie, nm.ml.cje, nm.ml.cke};
  auto fail_cleanup = [&](cudaError_t err, const char* what) {
    athgpu_destroy(nc);
    return api_fail(ATHGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
  };
  if (e != cudaSuccess) return fail_cleanup(e, "regrid setup");

  // 1. old mesh: restriction of the derefined children into their coarse buffers
  {
    MlOpList L;
    for (int n = 0; n < nnb; ++n) {
      if (kind[n] != 1) continue;
      for (int l = 0; l < 8; ++l) {
        std::vector<MlOp> ops;
        int e3[3] = {chi[0], chi[1], chi[2]};
        ops.push_back(op_box(ML_RESTRICT_U, 0, ML_COARSE, clo, e3));
        for (int d = 0; d < 3; ++d) {
          int ed[3] = {chi[0], chi[1], chi[2]};
          ed[d] += 1;
          ops.push_back(op_box(ML_RESTRICT_B, d, ML_COARSE, clo, ed));
        }
        L.add(newtoold[n] + l, ops);
      }
    }
    e = rb == 8 ? run_ops<double>(c, L) : run_ops<float>(c, L);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail_cleanup(e, "regrid restriction");
  }

  phase(1);
  // 2. box copies old -> new
  std::vector<RgCopy> tasks;
  bool boxes_ok = true;
  {
    const Registers& o = c->r;
    const Registers& w = nc->r;
    const DevML& oL = om.ml;
    const DevML& nL = nm.ml;
    const ArrDims cell_o{rb, om.nc1, om.nc2, om.ncell}, cell_n{rb, nm.nc1, nm.nc2, nm.ncell};
    const ArrDims ccell_o{rb, oL.ncc1, oL.ncc2, oL.nccell}, ccell_n{rb, nL.ncc1, nL.ncc2, nL.nccell};
    const ArrDims face_o[3] = {{8, om.nc1 + 1, om.nc2, 0}, {8, om.nc1, om.nc2 + 1, 0},
                               {8, om.nc1, om.nc2, 0}};
    const ArrDims face_n[3] = {{8, nm.nc1 + 1, nm.nc2, 0}, {8, nm.nc1, nm.nc2 + 1, 0},
                               {8, nm.nc1, nm.nc2, 0}};
    const ArrDims cface_o[3] = {{8, oL.ncc1 + 1, oL.ncc2, 0}, {8, oL.ncc1, oL.ncc2 + 1, 0},
                                {8, oL.ncc1, oL.ncc2, 0}};
    const ArrDims cface_n[3] = {{8, nL.ncc1 + 1, nL.ncc2, 0}, {8, nL.ncc1, nL.ncc2 + 1, 0},
                                {8, nL.ncc1, nL.ncc2, 0}};
    const i64 onf[3] = {om.nf1, om.nf2, om.nf3}, nnf[3] = {nm.nf1, nm.nf2, nm.nf3};
    const i64 oncf[3] = {oL.ncf1, oL.ncf2, oL.ncf3}, nncf[3] = {nL.ncf1, nL.ncf2, nL.ncf3};
    const double* ob[3] = {o.b1, o.b2, o.b3};
    double* wb[3] = {w.b1, w.b2, w.b3};
    const double* ocb[3] = {oL.cb1, oL.cb2, oL.cb3};
    double* wcb[3] = {nL.cb1, nL.cb2, nL.cb3};
    const double* osb[3] = {oL.sb1, oL.sb2, oL.sb3};
    double* wsb[3] = {nL.sb1, nL.sb2, nL.sb3};
    auto add_span = [&](const void* sb, void* db, long long bytes, int onb_, int nb_) {
      // per-block span copy of `bytes` bytes from block onb_ to block nb_, in rows of at
      // most 2^20 words
      const long long words = bytes / 4;
      const char* s = (const char*)sb + (long long)onb_ * bytes;
      char* d = (char*)db + (long long)nb_ * bytes;
      for (long long q = 0; q < words; q += (1LL << 20)) {
        const long long nw = (words - q) < (1LL << 20) ? (words - q) : (1LL << 20);
        tasks.push_back(span_copy(s + 4 * q, d + 4 * q, nw));
      }
    };
    const long long cu_bytes = 5LL * om.ncell * rb, cb_bytes = 3LL * om.ncell * rb;
    const long long ccu_bytes = 5LL * oL.nccell * rb, ccb_bytes = 3LL * oL.nccell * rb;
    for (int n = 0; n < nnb; ++n) {
      const int on = newtoold[n];
      if (kind[n] == 0) {
        add_span(o.u, w.u, cu_bytes, on, n);
        if (rb == 4) add_span(o.ulo, w.ulo, cu_bytes, on, n);
        add_span(o.wbuf[o.wsel], w.wbuf[w.wsel], cu_bytes, on, n);
        add_span(o.bcc, w.bcc, cb_bytes, on, n);
        for (int a = 0; a < 3; ++a) add_span(ob[a], wb[a], onf[a] * 8, on, n);
        add_span(oL.ccons, nL.ccons, ccu_bytes, on, n);
        add_span(oL.cprim, nL.cprim, ccu_bytes, on, n);
        add_span(oL.cbcc, nL.cbcc, ccb_bytes, on, n);
        add_span(oL.scons, nL.scons, ccu_bytes, on, n);
        for (int a = 0; a < 3; ++a) {
          add_span(ocb[a], wcb[a], oncf[a] * 8, on, n);
          add_span(osb[a], wsb[a], oncf[a] * 8, on, n);
        }
      } else if (kind[n] == 1) {
        for (int l = 0; l < 8; ++l) {
          const int ch = on + l;
          const long long* cl = &ol[(size_t)ch * 4];
          int d0[3];
          for (int a = 0; a < 3; ++a) d0[a] = flo[a] + (int)(cl[1 + a] & 1LL) * hx[a];
          int ext[3] = {hx[0], hx[1], hx[2]};
          tasks.push_back(box_copy((const char*)oL.ccons + (long long)ch * ccu_bytes, ccell_o,
                                   ccu_bytes / rb, (char*)w.u + (long long)n * cu_bytes,
                                   cell_n, cu_bytes / rb, NHYDRO, clo, d0, ext, &boxes_ok));
          // the faces shared by two children receive the same value from both
          for (int a = 0; a < 3; ++a) {
            int ea[3] = {hx[0], hx[1], hx[2]};
            ea[a] += 1;
            tasks.push_back(box_copy(ocb[a] + ch * oncf[a], cface_o[a], oncf[a],
                                     wb[a] + n * nnf[a], face_n[a], nnf[a], 1, clo, d0, ea,
                                     &boxes_ok));
          }
        }
      } else {
        const long long* nl = loc + (size_t)n * 4;
        int s0[3], d0[3], ext[3];
        for (int a = 0; a < 3; ++a) {
          s0[a] = (int)(nl[1 + a] & 1LL) * hx[a] + flo[a] - 1;
          d0[a] = clo[a] - 1;
          ext[a] = hx[a] + 2;
        }
        tasks.push_back(box_copy((const char*)o.u + (long long)on * cu_bytes, cell_o,
                                 cu_bytes / rb, (char*)nL.ccons + (long long)n * ccu_bytes,
                                 ccell_n, ccu_bytes / rb, NHYDRO, s0, d0, ext, &boxes_ok));
        for (int a = 0; a < 3; ++a) {
          int ea[3] = {ext[0], ext[1], ext[2]};
          ea[a] += 1;
          tasks.push_back(box_copy(ob[a] + on * onf[a], face_o[a], onf[a],
                                   wcb[a] + n * nncf[a], cface_n[a], nncf[a], 1, s0, d0, ea,
                                   &boxes_ok));
        }
      }
    }
    for (int t = 0; t < nffc; ++t) {
      const int n = ffc[3 * t], f = ffc[3 * t + 1], i = ffc[3 * t + 2], a = f >> 1;
      int s0[3] = {flo[0], flo[1], flo[2]}, d0[3] = {flo[0], flo[1], flo[2]};
      int ext[3] = {nm.nx1, nm.nx2, nm.nx3};
      d0[a] = (f & 1) ? fhi[a] + 1 : flo[a];
      s0[a] = (f & 1) ? flo[a] : fhi[a] + 1;
      ext[a] = 1;
      tasks.push_back(box_copy(ob[a] + i * onf[a], face_o[a], onf[a], wb[a] + n * nnf[a],
                               face_n[a], nnf[a], 1, s0, d0, ext, &boxes_ok));
    }
  }
  if (!boxes_ok) {
    athgpu_destroy(nc);
    return api_fail(ATHGPU_ERR_ARG, "regrid copy box outside its block (internal error)");
  }
  if (!tasks.empty()) {
    RgCopy* dt = nullptr;
    e = upload(tasks, &dt, nc->stream);
    if (e == cudaSuccess) {
      regrid_copy_kernel<<<(unsigned)tasks.size(), 256, 0, nc->stream>>>(dt);
      nc->launches += 1;
      e = cudaGetLastError();
      cudaFreeAsync(dt, nc->stream);
    }
    if (e != cudaSuccess) return fail_cleanup(e, "regrid copies");
  }
  // the clock; after athgpu_cycle, the dt that cycle used (the reference makes its
  // NewTimeStep after the regrid)
  {
    DevClock h;
    e = cudaMemcpyAsync(&h, c->clk, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail_cleanup(e, "regrid clock");
    if (after_cycle) h.dt = h.dt_prev;
    h.dtf = (float)h.dt;
    double dmax = DBL_MAX;
    memcpy(&h.dtmin_bits, &dmax, 8);
    e = cudaMemcpyAsync(nc->clk, &h, sizeof(h), cudaMemcpyHostToDevice, nc->stream);
    if (e != cudaSuccess) return fail_cleanup(e, "regrid clock");
  }

  phase(2);
  // 3. new mesh: ProlongateMeshBlock of every new child
  {
    MlOpList L;
    for (int n = 0; n < nnb; ++n) {
      if (kind[n] != 2) continue;
      int got[6] = {0, 0, 0, 0, 0, 0};
      for (int t = 0; t < nffc; ++t)
        if (ffc[3 * t] == n) got[ffc[3 * t + 1]] = 1;
      std::vector<MlOp> ops;
      int e3[3] = {chi[0], chi[1], chi[2]};
      ops.push_back(op_box(ML_PROLONG_U, 0, ML_COARSE, clo, e3));
      for (int a = 0; a < 3; ++a) {
        int s3[3] = {clo[0], clo[1], clo[2]}, ea[3] = {chi[0], chi[1], chi[2]};
        ea[a] += 1;
        if (got[2 * a]) s3[a] += 1;
        if (got[2 * a + 1]) ea[a] -= 1;
        ops.push_back(op_box(ML_PROLONG_SHARED, a, 0, s3, ea));
      }
      ops.push_back(op_box(ML_PROLONG_INTERNAL, 0, 0, clo, e3));
      L.add(n, ops);
    }
    e = rb == 8 ? run_ops<double>(nc, L) : run_ops<float>(nc, L);
    if (e != cudaSuccess) return fail_cleanup(e, "regrid prolongation");
  }
  phase(3);
  // the multi-level plan of the new mesh (host), then the new context's stream completes
  st = athgpu::ml_plan_upload(nc, nbr_table, nbr_count, nblevel, loc);
  if (st != ATHGPU_OK) { athgpu_destroy(nc); return st; }

  phase(4);
  // the new context takes the old one's place behind the caller's handle
  const bool user_stream = c->stream != c->own_stream;
  cudaStream_t us = c->stream;
  const long long launches = c->launches + nc->launches;
  std::swap(*c, *nc);
  athgpu_destroy(nc);
  c->launches = launches;
  if (user_stream) c->stream = us;

  phase(5);
  // 4. Initialize(2)
  st = athgpu_initialize(c);
  phase(6);
  return st;
}

athgpu_status athgpu_regrid_profile(double* ms) {
  if (!ms) return api_fail(ATHGPU_ERR_ARG, "null argument");
  for (int q = 0; q < 8; ++q) ms[q] = g_phase_ms[q];
  return ATHGPU_OK;
}

namespace athgpu {
// the context's mesh description (its coordinate pointers are not kept)
athgpu_status ctx_desc(athgpu_ctx* c, athgpu_mesh_desc* out) {
  if (!c || !out) return api_fail(ATHGPU_ERR_ARG, "null argument");
  *out = c->desc;
  out->x1f = out->dx1f = out->x2f = out->dx2f = out->x3f = out->dx3f = nullptr;
  return ATHGPU_OK;
}
}  // namespace athgpu

athgpu_status athgpu_new_time_step(athgpu_ctx* c) {
  if (!c) return api_fail(ATHGPU_ERR_ARG, "null context");
  if (!c->initialized) return api_fail(ATHGPU_ERR_STATE, "athgpu_initialize not called");
  advance_clock_kernel<<<1, 32, 0, c->stream>>>(c->clk, c->m.cfl, c->m.tlim, 2);
  c->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return api_fail(ATHGPU_ERR_CUDA, cudaGetErrorString(e));
  return ATHGPU_OK;
}
