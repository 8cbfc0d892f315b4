// mpm_mixed.cu -- the mixed-precision form of the step: FP32 shape
// functions, velocity gradient and constitutive update; FP64 grid
// accumulation, positions, velocities and energy. Fused multiply-adds allowed.
#include "mpm_ops.cuh"

namespace mpm {
const StepOps kOpsMixed = Ops<PMixed>::table("mixed");
}  // namespace mpm
