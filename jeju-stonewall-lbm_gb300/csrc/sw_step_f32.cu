// sw_step_f32.cu -- instantiations of the fused step (single lattice and batched) for SW_F32.
#include "sw_aux.cuh"
#include "sw_batch.cuh"
#include "sw_step.cuh"

namespace sw {
cudaError_t step_f32(const StepParams &p, cudaStream_t s) { return launch_step<SW_F32>(p, s); }
cudaError_t batch_f32(const sw_batch_header *h, const sw_batch_entry *t, int cfg, int k, cudaStream_t s) {
  return launch_batch<SW_F32>(h, t, cfg, k, s);
}
}  // namespace sw
