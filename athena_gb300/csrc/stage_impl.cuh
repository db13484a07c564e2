// Host-side stage driver, templated on the bulk precision.  Included by stage_fp64.cu
// (compiled without FMA contraction, -fmad=false, for bit parity with the reference) and
// stage_fp32.cu (FMA contraction on).
#pragma once
#include "ctx.h"
#include "boundary.cuh"
#include "multilevel.cuh"

namespace athgpu {

static inline unsigned nblk(long long n, int tpb) {
  return (unsigned)((n + tpb - 1) / tpb);
}

// The x3 sweep's TMA bulk staging applies when selected and when every staged row is
// 16-byte aligned: the k-plane (nc1 nc2 elements) and the first staged row ((js-1) nc1)
// of the bulk-precision arrays and of the FP64 face field, on a uniform mesh (the
// registers of a uniform mesh are padded for the last CTA's overhanging row).
static inline bool x3_bulk_ok(const athgpu_ctx* c) {
  return c->lc.x3_bulk && x3_bulk_eligible(c);
}

template <typename Real, int ORDER, int RS, int KAHAN>
static void launch_fluxes(athgpu_ctx* c, const Real* w, const Real* bcc, const double* b1,
                          const double* b2, const double* b3, const UpdateArgs& ua) {
  const DevMesh& m = c->m;
  Registers& r = c->r;
  cudaStream_t s = c->stream;
  if (m.ml.on && c->mld.nflux > 0) {
    // the finer blocks' fluxes on faces shared with coarser blocks, restricted, before the
    // sweeps (which use them there)
    ProfScope ps(c, "ml_fine_flux");
    const long long n = (long long)c->mld.nflux * (m.ml.nfmax / 4);
    ml_fine_flux_kernel<Real, ORDER, RS><<<nblk(n, 128), 128, 0, s>>>(
        m, (const int4*)c->mld.flux_tasks, c->mld.nflux, w, bcc, b1, b2, b3);
    c->launches += 1;
  }
  {
    const long long cells = (long long)(m.nx3 + 2) * (m.nx2 + 2) * (m.nx1 + 2);
    const long long warps = (cells + 29) / 30;  // per MeshBlock (blockIdx.y)
    ProfScope ps(c, "flux_x1");
    flux_x1_kernel<Real, ORDER, RS><<<dim3(nblk(warps * 32, 128), m.nb), 128, 0, s>>>(
        m, w, bcc, b1, c->clk, (Real*)r.dflx, (Real*)r.e3x1, (Real*)r.e2x1, (Real*)r.w1f);
  }
  {
    int seg = c->lc.seg_x2 > 0 ? c->lc.seg_x2 : m.nx2;
    const long long nseg = (m.nx2 + seg - 1) / seg;
    const long long n = nseg * m.nb * (m.nx3 + 2) * (long long)(m.nx1 + 2);
    ProfScope ps(c, "flux_x2");
    const int smem = sweep_smem_bytes(1, ORDER, sizeof(Real), 128);
    static bool attr = false;  // opt in above 48 KB once per instantiation
    if (!attr) {
      cudaFuncSetAttribute(flux_sweep_kernel<Real, 1, ORDER, RS, KAHAN>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      attr = true;
    }
    flux_sweep_kernel<Real, 1, ORDER, RS, KAHAN><<<nblk(n, 128), 128, smem, s>>>(
        m, seg, w, bcc, b2, c->clk, (Real*)r.dflx, (Real*)r.e1x2, (Real*)r.e3x2,
        (Real*)r.w2f, ua);
  }
  {
    int seg = c->lc.seg_x3 > 0 ? c->lc.seg_x3 : m.nx3;
    const long long nseg = (m.nx3 + seg - 1) / seg;
    const long long n = nseg * m.nb * (m.nx2 + 2) * (long long)(m.nx1 + 2);
    ProfScope ps(c, "flux_x3_update");
    const int smem = sweep_smem_bytes(2, ORDER, sizeof(Real), 128);
    if (x3_bulk_ok(c)) {
      // TMA bulk staging: CTAs over consecutive k-plane positions of rows js-1..je+1
      static bool attr = false;
      if (!attr) {
        cudaFuncSetAttribute(flux_sweep_kernel<Real, 2, ORDER, RS, KAHAN, 1>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
      }
      const long long nq = ((long long)(m.nx2 + 2) * m.nc1 + 127) / 128;
      flux_sweep_kernel<Real, 2, ORDER, RS, KAHAN, 1><<<(unsigned)(nq * m.nb * nseg), 128,
                                                        smem, s>>>(
          m, seg, w, bcc, b3, c->clk, (Real*)r.dflx, (Real*)r.e2x3, (Real*)r.e1x3,
          (Real*)r.w3f, ua);
    } else {
      static bool attr = false;
      if (!attr) {
        cudaFuncSetAttribute(flux_sweep_kernel<Real, 2, ORDER, RS, KAHAN>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
      }
      flux_sweep_kernel<Real, 2, ORDER, RS, KAHAN><<<nblk(n, 128), 128, smem, s>>>(
          m, seg, w, bcc, b3, c->clk, (Real*)r.dflx, (Real*)r.e2x3, (Real*)r.e1x3,
          (Real*)r.w3f, ua);
    }
  }
  c->launches += 3;
}

// Ghost exchange of the face fields, and of U when with_u (outside the stage: U's ghosts
// are not needed by the stage kernels, see exchange_kernel).
template <typename Real>
static void launch_exchange(athgpu_ctx* c, Real* u, double* b1, double* b2, double* b3,
                            int with_u, cudaStream_t st = nullptr) {
  if (!st) st = c->stream;
  const DevMesh& m = c->m;
  const long long gc = with_u ? m.ncell - (long long)m.nx1 * m.nx2 * m.nx3 : 0;
  const long long g1 = m.nf1 - (long long)(m.nx1 + 1) * m.nx2 * m.nx3;
  const long long g2 = m.nf2 - (long long)m.nx1 * (m.nx2 + 1) * m.nx3;
  const long long g3 = m.nf3 - (long long)m.nx1 * m.nx2 * (m.nx3 + 1);
  const long long n = (gc + g1 + g2 + g3) * m.nb;
  if (c->xplan) {
    const int* xn = c->xplan_n;
    const int p0 = with_u ? 0 : xn[0];
    const long long cnt = (long long)xn[0] + xn[1] + xn[2] + xn[3] - p0;
    // EXCHANGE_XB MeshBlocks per thread
    const long long gy = (m.nb + EXCHANGE_XB - 1) / EXCHANGE_XB;
    exchange_plan_kernel<Real><<<dim3(nblk(cnt, 256), gy < 65535 ? gy : 65535), 256, 0,
                                 st>>>(m, c->xplan, p0, xn[0], xn[1], xn[2], xn[3],
                                       c->xdelta, u, b1, b2, b3);
  } else if (n < (1LL << 31) - 256)
    exchange_kernel<Real, int><<<nblk(n, 256), 256, 0, st>>>(m, with_u, u, b1, b2, b3);
  else
    exchange_kernel<Real, long long><<<nblk(n, 256), 256, 0, st>>>(m, with_u, u, b1, b2, b3);
}

// Multi-level mesh: one of the three operation lists (0 restriction for coarser
// neighbours, 1 ghost exchange, 2 prolongation), one CTA per block with work
template <typename Real>
static void launch_ml_phase(athgpu_ctx* c, int phase, Real* u, Real* w, double* b1,
                            double* b2, double* b3) {
  const int nb = c->mld.nblk[phase];
  if (nb == 0) return;
  static const char* names[3] = {"ml_restrict", "ml_exchange", "ml_prolong"};
  ProfScope ps(c, names[phase]);
  MlArrays<Real> A{u, w, (Real*)c->r.bcc, b1, b2, b3};
  const MlOp* ops = (const MlOp*)c->mld.ops[phase];
  if (phase == 0)
    ml_ops_kernel<Real, 0><<<nb, 128, 0, c->stream>>>(c->m, A, ops, c->mld.off[phase],
                                                      c->mld.blk[phase]);
  else if (phase == 1)
    ml_ops_kernel<Real, 1><<<nb, 128, 0, c->stream>>>(c->m, A, ops, c->mld.off[phase],
                                                      c->mld.blk[phase]);
  else
    ml_ops_kernel<Real, 2><<<nb, 128, 0, c->stream>>>(c->m, A, ops, c->mld.off[phase],
                                                      c->mld.blk[phase]);
  c->launches += 1;
}

template <typename Real, int KAHAN>
static void launch_exchange_and_c2p(athgpu_ctx* c, Real* u, double* b1, double* b2,
                                    double* b3, int do_dt, bool rotate = true,
                                    int with_u = 0) {
  const DevMesh& m = c->m;
  cudaStream_t s = c->stream;
  const long long nc = (long long)m.nb * m.ncell;
  // The relativistic W(U) reads no exchanged face (interior cells only; ghost primitives
  // are copied from their owners), so there the ghost exchange runs on the auxiliary
  // stream beside it (forked and joined with events, also inside the captured cycle
  // graph); the Newtonian W(U) reads the exchanged faces of its ghost cells and follows
  // the exchange.  The per-kernel profile runs everything one after the other.
  const bool overlap = !c->profiling && c->aux_stream != nullptr && c->desc.relativistic;
  if (m.ml.on) {
    // multi-level mesh: restriction for coarser neighbours, the exchange of U and B, then
    // ProlongateBoundaries into the current primitives (bvals_refine.cpp:97-256)
    Real* wcur = (Real*)c->r.wbuf[c->r.wsel];
    launch_ml_phase<Real>(c, 0, u, wcur, b1, b2, b3);
    launch_ml_phase<Real>(c, 1, u, wcur, b1, b2, b3);
    launch_ml_phase<Real>(c, 2, u, wcur, b1, b2, b3);
  } else if (overlap) {
    cudaEventRecord(c->ev_fork, s);
    cudaStreamWaitEvent(c->aux_stream, c->ev_fork, 0);
    launch_exchange<Real>(c, u, b1, b2, b3, with_u, c->aux_stream);
  } else {
    ProfScope ps(c, "exchange");
    launch_exchange<Real>(c, u, b1, b2, b3, with_u);
  }
  // the compensation register belongs to U only; the stage-1 register U* has none
  Real* lo = (u == (Real*)c->r.u) ? (Real*)c->r.ulo : nullptr;
  // W(U) writes the non-current primitive buffer (seeded with its old contents), which
  // then becomes current; initialize writes the current one in place
  Real* wout = (Real*)c->r.wbuf[rotate ? 1 - c->r.wsel : c->r.wsel];
  {
    ProfScope ps(c, "c2p");
    if (c->desc.relativistic) {
      SRFloors fp{c->desc.gamma, c->desc.dfloor, c->desc.pfloor, c->desc.sigma_max,
                  c->desc.beta_min, c->desc.gamma_max};
      // the start of the FP64 solve (athgpu_set_c2p_start): 0 the stale pressure, 1 that
      // pressure refined in FP32, 2 the network's pressure refined in FP32
      const int start = c->c2p_start;
      const int n1 = c->lc.sr_phase1 > 0 ? c->lc.sr_phase1 : (start ? 5 : 7);
      const long long ni = (long long)m.nb * m.nx1 * m.nx2 * m.nx3;
      auto kern = start == C2P_START_NETWORK ? c2p_sr_kernel<Real, KAHAN, C2P_START_NETWORK>
                  : start == C2P_START_REFINED ? c2p_sr_kernel<Real, KAHAN, C2P_START_REFINED>
                                               : c2p_sr_kernel<Real, KAHAN, C2P_START_STALE>;
      // the network start: its operands in shared memory, padded so that at most four
      // CTAs (4 x 128 tensor-memory columns) share an SM
      const int smem = start == C2P_START_NETWORK
                           ? (int)sizeof(c2pnet::TcNet) + c2pnet::TC_SMEM_PAD : 0;
      if (smem) {
        static bool attr = false;  // opt in above 48 KB once per instantiation
        if (!attr) {
          cudaFuncSetAttribute(c2p_sr_kernel<Real, KAHAN, C2P_START_NETWORK>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
          attr = true;
        }
      }
      cudaMemsetAsync(c->c2p_qcount, 0, sizeof(unsigned), s);
      kern<<<nblk(ni, 128), 128, smem, s>>>(
          m, fp, do_dt, b1, b2, b3, u, lo, wout, (Real*)c->r.bcc, (Real*)c->r.cce, c->clk,
          1, n1, c->c2p_queue, c->c2p_qcount, c->c2p_qstart, c->c2p_net, c->c2p_net_err);
      const long long g2 = nblk(ni, 128) < 2048 ? nblk(ni, 128) : 2048;
      kern<<<g2, 128, 0, s>>>(
          m, fp, do_dt, b1, b2, b3, u, lo, wout, (Real*)c->r.bcc, (Real*)c->r.cce, c->clk,
          2, 15, c->c2p_queue, c->c2p_qcount, c->c2p_qstart, c->c2p_net, c->c2p_net_err);
      const long long ng = ((long long)m.ncell - (long long)m.nx1 * m.nx2 * m.nx3) * m.nb;
      copy_ghost_prims_kernel<Real><<<nblk(ng, 256), 256, 0, s>>>(
          m, wout, (Real*)c->r.bcc, (Real*)c->r.cce);
      c->launches += 2;
    } else {
      cudaMemsetAsync(c->c2p_qcount, 0, sizeof(unsigned), s);
      const dim3 grid(nblk(m.ncell, 128), m.nb < 65535 ? m.nb : 65535);
      c2p_kernel<Real, KAHAN><<<grid, 128, 0, s>>>(
          m, do_dt, b1, b2, b3, u, wout, (Real*)c->r.bcc, (Real*)c->r.cce, c->clk,
          c->c2p_queue, c->c2p_qcount);
      c2p_floor_writeback_kernel<Real, KAHAN><<<64, 128, 0, s>>>(
          m, b1, b2, b3, u, lo, c->c2p_queue, c->c2p_qcount);
      c->launches += 1;
    }
  }
  if (overlap && !m.ml.on) {
    cudaEventRecord(c->ev_join, c->aux_stream);
    cudaStreamWaitEvent(s, c->ev_join, 0);
  }
  if (m.any_bc) {
    // physical mesh faces, x1 then x2 then x3, on the primitives just written and the
    // exchanged face field
    ProfScope ps(c, "boundary");
    for (int a = 0; a < 3; ++a) {
      if (m.bc[2 * a] == 0 && m.bc[2 * a + 1] == 0) continue;
      const long long n = bc_threads(m, a);
      bc_fill_kernel<Real><<<nblk(n, 256), 256, 0, s>>>(m, a, wout, b1, b2, b3);
      auto cck = c->desc.relativistic ? bc_cc_kernel<Real, true> : bc_cc_kernel<Real, false>;
      cck<<<nblk(n, 256), 256, 0, s>>>(m, a, wout, b1, b2, b3, (Real*)c->r.bcc,
                                       (Real*)c->r.cce, u);
      c->launches += 2;
    }
  }
  if (rotate) c->r.wsel = 1 - c->r.wsel;
  c->launches += 2;
}

template <typename Real, int KAHAN>
static cudaError_t run_stage(athgpu_ctx* c, int stage) {
  const DevMesh& m = c->m;
  Registers& r = c->r;
  cudaStream_t s = c->stream;
  // Stage weights of TimeIntegratorTaskList (time_integrator.cpp:111-236 vl2, :338-465
  // rk2).  vl2: donor cell on stage 1, beta = 1/2, 1, register swaps; rk2: xorder on both
  // stages, beta = 1, 1/2, and on stage 2 the register average g1*U* + g2*U^n.
  const bool rk2 = c->desc.integrator == ATHGPU_RK2;
  // reconstruction template index: 1 DC, 2 PLM, 3 PPM, 4 fast PPM (time/xorder = 3f)
  const int xo = c->desc.ppm_fast ? 4 : c->desc.xorder;
  const int order = (stage == 1 && !rk2) ? 1 : xo;
  const double beta = rk2 ? (stage == 1 ? 1.0 : 0.5) : (stage == 1 ? 0.5 : 1.0);
  const bool avg = rk2 && stage == 2;
  const double g1 = 0.5, g2 = 0.5;
  // stage 1 reads U^n, B^n and writes U*, B*; stage 2 reads W*, B* and updates U, B
  const double* bb1 = (stage == 1) ? r.b1 : r.bs1;
  const double* bb2 = (stage == 1) ? r.b2 : r.bs2;
  const double* bb3 = (stage == 1) ? r.b3 : r.bs3;
  const Real* w = (const Real*)r.wbuf[r.wsel];
  const Real* bcc = (const Real*)r.bcc;
  // solver template index: 0 HLLD, 1 HLLE, 2 relativistic HLLE, 3 LLF, 4 Roe,
  // 5 relativistic LLF, 6 relativistic HLLD, 7 low-dissipation HLLD
  const int rs = c->desc.relativistic ? (c->desc.rsolver == ATHGPU_LLF    ? 5
                                         : c->desc.rsolver == ATHGPU_HLLD ? 6 : 2)
                 : c->desc.rsolver == ATHGPU_LLF   ? 3
                 : c->desc.rsolver == ATHGPU_ROE   ? 4
                 : c->desc.rsolver == ATHGPU_LHLLD ? 7 : c->desc.rsolver;
  Real* uout = (stage == 1) ? (Real*)r.ustar : (Real*)r.u;
  UpdateArgs ua;
  ua.beta = beta;
  ua.stage = stage;
  ua.uin = r.u;
  ua.uout = uout;
  ua.ulo = r.ulo;
  ua.uavg = avg ? r.ustar : nullptr;
  ua.g1 = g1;
  ua.g2 = g2;
  ua.err = (int*)((char*)c->clk + offsetof(DevClock, sweep_timeout));
#define FLUX(O, R) launch_fluxes<Real, O, R, KAHAN>(c, w, bcc, bb1, bb2, bb3, ua)
#define FLUX_RS(O)                                                                   \
  do {                                                                               \
    if (rs == 0) FLUX(O, 0); else if (rs == 1) FLUX(O, 1); else if (rs == 3) FLUX(O, 3); \
    else if (rs == 4) FLUX(O, 4); else if (rs == 5) FLUX(O, 5);                      \
    else if (rs == 6) FLUX(O, 6); else if (rs == 7) FLUX(O, 7); else FLUX(O, 2);      \
  } while (0)
  if (order == 1) FLUX_RS(1);
  else if (order == 2) FLUX_RS(2);
  else if (order == 3) FLUX_RS(3);
  else FLUX_RS(4);
#undef FLUX_RS
#undef FLUX
  {
    const long long n = (long long)(m.nx3 + 1) * (m.nx2 + 1) * (m.nx1 + 1);
    ProfScope ps(c, "corner_e");
    auto kern = c->desc.relativistic ? corner_e_kernel<Real, true> : corner_e_kernel<Real, false>;
    kern<<<dim3(nblk(n, 128), m.nb < 65535 ? m.nb : 65535), 128, 0, s>>>(
        m, (const Real*)r.cce, (Real*)r.e3x1, (Real*)r.e2x1, (Real*)r.w1f, (Real*)r.e1x2,
        (Real*)r.e3x2, (Real*)r.w2f, (Real*)r.e1x3, (Real*)r.e2x3, (Real*)r.w3f,
        (Real*)r.e1, (Real*)r.e2, (Real*)r.e3);
  }
  if (!m.ml.on) {
    // same-level edge averaging of the block-face edges (flux_correction_fc.cpp)
    ProfScope ps2(c, "edge_avg");
    const int* en = c->eplan_n;
    const long long ne = (long long)en[0] + en[1] + en[2];
    const long long gy = (m.nb + EB - 1) / EB;
    const dim3 grid(nblk(ne, 128), gy < 65535 ? gy : 65535);
    edge_fix_kernel<Real><<<grid, 128, 0, s>>>(m, c->eplan, en[0], en[1], en[2],
                                               (const Real*)r.e1, (const Real*)r.e2,
                                               (const Real*)r.e3, (Real*)c->escratch);
    edge_put_kernel<Real><<<grid, 128, 0, s>>>(m, c->eplan, en[0], en[1], en[2], (Real*)r.e1,
                                               (Real*)r.e2, (Real*)r.e3,
                                               (const Real*)c->escratch);
    c->launches += 2;
  } else {
    // EMF correction across levels (flux_correction_fc.cpp)
    ProfScope ps2(c, "ml_emf");
    const long long chunks = (ml_emf_positions(m) + 127) / 128;
    dim3 grid(m.nb, (unsigned)(chunks < 65535 ? chunks : 65535));
    ml_emf_kernel<Real><<<grid, 128, 0, s>>>(m, (const Real*)r.e1, (const Real*)r.e2,
                                             (const Real*)r.e3);
    ml_emf_put_kernel<Real><<<grid, 128, 0, s>>>(m, (Real*)r.e1, (Real*)r.e2, (Real*)r.e3);
    c->launches += 2;
  }
  double* o1 = (stage == 1) ? r.bs1 : r.b1;
  double* o2 = (stage == 1) ? r.bs2 : r.b2;
  double* o3 = (stage == 1) ? r.bs3 : r.b3;
  {
    const long long per = (long long)(m.nx3 + 1) * (m.nx2 + 1) * (m.nx1 + 1);
    dim3 grid(nblk(per, 256), m.nb);
    ProfScope ps(c, "ct");
    // (multi-level meshes too: the corrected block-face EMFs are in the edge arrays)
    ct_kernel<Real><<<grid, 256, 0, s>>>(
        m, beta, c->clk, (const Real*)r.e1, (const Real*)r.e2, (const Real*)r.e3, r.b1, r.b2,
        r.b3, o1, o2, o3, avg ? r.bs1 : nullptr, avg ? r.bs2 : nullptr,
        avg ? r.bs3 : nullptr, g1, g2);
  }
  c->launches += 2;
  launch_exchange_and_c2p<Real, KAHAN>(c, uout, o1, o2, o3, stage == 2);
  return cudaGetLastError();
}

// end of a main-loop cycle: time += dt, Mesh::NewTimeStep (main.cpp:535-541)
static inline cudaError_t run_end_cycle(athgpu_ctx* c) {
  ProfScope ps(c, "advance_clock");
  advance_clock_kernel<<<1, 32, 0, c->stream>>>(c->clk, c->m.cfl, c->m.tlim, 1);
  c->launches += 1;
  return cudaGetLastError();
}

template <typename Real, int KAHAN>
static cudaError_t run_init(athgpu_ctx* c) {
  // Mesh::Initialize exchanges U as well: its ghosts are consistent after initialization
  launch_exchange_and_c2p<Real, KAHAN>(c, (Real*)c->r.u, c->r.b1, c->r.b2, c->r.b3, 1,
                                       false, 1);
  advance_clock_kernel<<<1, 32, 0, c->stream>>>(c->clk, c->m.cfl, c->m.tlim, 0);
  c->launches += 1;
  return cudaGetLastError();
}

}  // namespace athgpu
