// sw_step_f32.cu -- instantiation of the fused step for storage type SW_F32.
#include "sw_aux.cuh"
#include "sw_step.cuh"

namespace sw {
cudaError_t step_f32(const StepParams &p, cudaStream_t s) { return launch_step<SW_F32>(p, s); }
}  // namespace sw
