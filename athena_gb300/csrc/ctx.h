// Internal state of an athgpu context (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/athena_gb300.h"
#include "kernels.cuh"
#include "ml_plan.h"

namespace athgpu {

struct Registers {
  // bulk precision (double or float) arrays; `void*` so one struct serves both paths
  void *u = nullptr, *ustar = nullptr, *ulo = nullptr, *bcc = nullptr;
  // cell-centred E = -v x B [nb][3][cells], written by W(U) for the corner EMFs
  void* cce = nullptr;
  // primitives, double-buffered: each W(U) writes the buffer that is not current, seeded
  // with its previous contents (the reference's w / w1 pair, time_integrator.cpp:2221-2269)
  void* wbuf[2] = {nullptr, nullptr};
  int wsel = 0;  // index of the current primitives
  void *dflx = nullptr;  // per-cell flux divergence accumulated by the sweeps
  void *e3x1 = nullptr, *e2x1 = nullptr, *w1f = nullptr;
  void *e1x2 = nullptr, *e3x2 = nullptr, *w2f = nullptr;
  void *e1x3 = nullptr, *e2x3 = nullptr, *w3f = nullptr;
  void *e1 = nullptr, *e2 = nullptr, *e3 = nullptr;
  // always FP64: face field B and its stage-1 register
  double *b1 = nullptr, *b2 = nullptr, *b3 = nullptr;
  double *bs1 = nullptr, *bs2 = nullptr, *bs3 = nullptr;
};

// device copies of the multi-level plan (ml_plan.h)
struct MlDevice {
  void* ops[3] = {nullptr, nullptr, nullptr};  // MlOp lists: restriction, exchange, prolongation
  int* off[3] = {nullptr, nullptr, nullptr};
  int* blk[3] = {nullptr, nullptr, nullptr};
  int nblk[3] = {0, 0, 0};
  void* flux_tasks = nullptr;                  // int4 per task
  int nflux = 0;
  std::vector<void*> allocs;                   // everything allocated for the mesh
  std::vector<long long> hloc;                 // host copy of loc[nb][4]
};

struct LaunchConfig {
  int seg_x2 = 0, seg_x3 = 0;  // faces per thread along the x2/x3 sweeps (0: default)
  int sr_phase1 = 0;           // SR con2prim: first-solve passes in phase 1 (0: default)
  int x3_bulk = 0;             // x3 sweep staged by TMA bulk copies (athgpu_set_x3_staging)
};

}  // namespace athgpu

struct athgpu_ctx {
  athgpu_mesh_desc desc;
  athgpu::DevMesh m;
  athgpu::Registers r;
  athgpu::LaunchConfig lc;
  athgpu::DevClock* clk = nullptr;
  double* coords = nullptr;  // dx1f | dx2f | dx3f | plm coefficients (device)
  double* fxv = nullptr;     // cell centres x1v | x2v | x3v per block (prolongation)
  double* eps_buf = nullptr; // per-block refinement measure (athgpu_refinement_eps)
  athgpu::MlDevice mld;
  // the host side of the multi-level plan, kept so that a regrid's new plan reuses its
  // storage (no fresh pages for tens of MB of operation lists)
  athgpu::MlPlan mlplan;
  float* coords32 = nullptr; // the same, rounded to FP32, for the FP32 kernels
  int* nbr = nullptr;
  // ghost plan of a same-level mesh's blocks (exchange_plan_kernel): plan words of the
  // cell, x1-, x2- and x3-face ghosts, their counts, and the owner shifts [4][27]
  unsigned* xplan = nullptr;
  int xplan_n[4] = {0, 0, 0, 0};
  int* xdelta = nullptr;
  // block-face edges of a same-level mesh's blocks (edge_fix_kernel): (offset, k, j, i) of
  // the x1-, x2- and x3-directed ones, their counts, and the averages' scratch [nb][n]
  int4* eplan = nullptr;
  int eplan_n[3] = {0, 0, 0};
  void* escratch = nullptr;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  // second stream for the ghost exchange beside W(U), forked and joined with events
  cudaStream_t aux_stream = nullptr;
  // host <-> device state copies: chunks spread over these streams (copy engines), each
  // chunk's conversion ordered after its copy with an event from the pool
  static const int NCOPY = 4, NCOPY_EV = 64;
  cudaStream_t copy_stream[NCOPY] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t copy_ev[NCOPY_EV] = {};
  int copy_ev_next = 0;
  int host_copy_mode = 0;  // athgpu_set_host_copy
  int copy_extent = 0;     // athgpu_set_copy_extent (ATHGPU_COPY_WHOLE / _INTERIOR)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaGraphExec_t cycle_exec = nullptr;
  cudaGraph_t cycle_graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  int graph_wsel = 0;
  bool initialized = false;
  int real_bytes = 8;
  long long launches = 0;
  long long per_cycle = 0;
  double* staging = nullptr;  // device staging of FP64 host data in FP32 mode
  int* c2p_queue = nullptr;      // SR con2prim: interior cells deferred to phase 2
  unsigned* c2p_qcount = nullptr;
  double* c2p_qstart = nullptr;  // SR con2prim: the start pressure of each queued cell
  // SR con2prim start (athgpu_set_c2p_start): C2P_START_STALE / _REFINED / _NETWORK, the
  // network's parameters (device, ATHGPU_MLP_NPARAM floats) and its tensor-core error flag
  int c2p_start = 0;
  float* c2p_net = nullptr;
  int* c2p_net_err = nullptr;
  // per-operator calls (operators.cu): the three flux arrays [5][nf1] | [5][nf2] | [5][nf3]
  double* op_flx = nullptr;
  unsigned long long* op_words = nullptr;  // [0] floored-cell count, [1] dt minimum bits
  // per-kernel timing of one non-graph cycle (athgpu_profile_cycle)
  bool profiling = false;
  std::vector<std::string> prof_names;
  std::vector<cudaEvent_t> prof_events;  // two per launch
};

// record an event pair around one launch when the context is profiling
struct ProfScope {
  athgpu_ctx* c;
  ProfScope(athgpu_ctx* ctx, const char* name) : c(ctx) {
    if (!c->profiling) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, c->stream);
    c->prof_events.push_back(e);
    c->prof_names.push_back(name);
  }
  ~ProfScope() {
    if (!c->profiling) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, c->stream);
    c->prof_events.push_back(e);
  }
};

namespace athgpu {
// device memory of the contexts, from the stream-ordered pool (api.cu)
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s);
// the x3 sweep's TMA bulk staging can run here: uniform mesh, 16-byte aligned k-planes and
// first staged rows (api.cu)
bool x3_bulk_eligible(const athgpu_ctx* c);
// stage drivers, one per precision translation unit
cudaError_t stage_fp64(athgpu_ctx* c, int stage);
cudaError_t stage_fp32(athgpu_ctx* c, int stage);
cudaError_t init_fp64(athgpu_ctx* c);
cudaError_t init_fp32(athgpu_ctx* c);
// multi-level mesh: the restriction, exchange and prolongation operation lists
// (phase 0, 1, 2) on the context's stream
cudaError_t ml_phase_fp64(athgpu_ctx* c, int phase);
cudaError_t ml_phase_fp32(athgpu_ctx* c, int phase);
// ghost exchange of U and the face fields (U's ghosts are not kept during the stages)
cudaError_t exchange_u_fp64(athgpu_ctx* c);
cudaError_t exchange_u_fp32(athgpu_ctx* c);
}  // namespace athgpu
