// FP32 stage update: reconstruction, Riemann solvers, corner EMFs and the flux
// divergence in FP32 with a compensated (Kahan) conserved update; the face field, the CT
// update and the time step stay FP64.
#include "stage_impl.cuh"

namespace athgpu {
cudaError_t stage_fp32(athgpu_ctx* c, int stage) {
  if (stage == 0) return run_end_cycle(c);
  return run_stage<float, 1>(c, stage);
}
cudaError_t init_fp32(athgpu_ctx* c) { return run_init<float, 1>(c); }
cudaError_t exchange_u_fp32(athgpu_ctx* c) {
  if (c->m.ml.on) {  // multi-level mesh: restriction for coarser blocks, then the exchange
    float* u = (float*)c->r.u;
    float* w = (float*)c->r.wbuf[c->r.wsel];
    launch_ml_phase<float>(c, 0, u, w, c->r.b1, c->r.b2, c->r.b3);
    launch_ml_phase<float>(c, 1, u, w, c->r.b1, c->r.b2, c->r.b3);
    return cudaGetLastError();
  }
  launch_exchange<float>(c, (float*)c->r.u, c->r.b1, c->r.b2, c->r.b3, 1);
  return cudaGetLastError();
}
}  // namespace athgpu
