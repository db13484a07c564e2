// FP64 stage update.  Compiled with -fmad=false: no FMA contraction, so every operation
// rounds exactly as in the reference's FP64 build.
#include "stage_impl.cuh"

namespace athgpu {
cudaError_t stage_fp64(athgpu_ctx* c, int stage) {
  if (stage == 0) return run_end_cycle(c);
  return run_stage<double, 0>(c, stage);
}
cudaError_t init_fp64(athgpu_ctx* c) { return run_init<double, 0>(c); }
cudaError_t exchange_u_fp64(athgpu_ctx* c) {
  if (c->m.ml.on) {  // multi-level mesh: restriction for coarser blocks, then the exchange
    double* u = (double*)c->r.u;
    double* w = (double*)c->r.wbuf[c->r.wsel];
    launch_ml_phase<double>(c, 0, u, w, c->r.b1, c->r.b2, c->r.b3);
    launch_ml_phase<double>(c, 1, u, w, c->r.b1, c->r.b2, c->r.b3);
    return cudaGetLastError();
  }
  launch_exchange<double>(c, (double*)c->r.u, c->r.b1, c->r.b2, c->r.b3, 1);
  return cudaGetLastError();
}
}  // namespace athgpu
