// sw_step_f64.cu -- instantiation of the fused step for storage type SW_F64.
#include "sw_aux.cuh"
#include "sw_step.cuh"

namespace sw {
cudaError_t step_f64(const StepParams &p, cudaStream_t s) { return launch_step<SW_F64>(p, s); }
}  // namespace sw
