// sw_step_bf16s.cu -- instantiation of the fused step for storage type SW_BF16_SHIFT.
#include "sw_aux.cuh"
#include "sw_step.cuh"

namespace sw {
cudaError_t step_bf16s(const StepParams &p, cudaStream_t s) { return launch_step<SW_BF16_SHIFT>(p, s); }
}  // namespace sw
