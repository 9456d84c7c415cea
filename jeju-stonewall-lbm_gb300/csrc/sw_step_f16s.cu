// sw_step_f16s.cu -- instantiations of the fused step (single lattice, batched, AA) for SW_F16_SHIFT.
#include "sw_aa.cuh"
#include "sw_aux.cuh"
#include "sw_batch.cuh"
#include "sw_step.cuh"

namespace sw {
cudaError_t step_f16s(const StepParams &p, cudaStream_t s) { return launch_step<SW_F16_SHIFT>(p, s); }
cudaError_t batch_f16s(const sw_batch_header *h, const sw_batch_entry *t, int cfg, int k, cudaStream_t s) {
  return launch_batch<SW_F16_SHIFT>(h, t, cfg, k, s);
}
cudaError_t aa_f16s(const StepParams &p, const AAParams &a, bool odd, cudaStream_t s) {
  return launch_aa<SW_F16_SHIFT>(p, a, odd, s);
}
unsigned int tma_timeouts_f16s() { return tma_timeouts_take(); }
}  // namespace sw
