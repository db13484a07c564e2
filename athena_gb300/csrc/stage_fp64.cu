// FP64 stage update.  Compiled with -fmad=false: no FMA contraction, so every operation
// rounds exactly as in the reference's FP64 build.
#include "stage_impl.cuh"

namespace athgpu {
cudaError_t stage_fp64(athgpu_ctx* c, int stage) {
  if (stage == 0) return run_end_cycle(c);
  return run_stage<double, 0>(c, stage);
}
cudaError_t init_fp64(athgpu_ctx* c) { return run_init<double, 0>(c); }
}  // namespace athgpu
