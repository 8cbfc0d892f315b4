// mpm_fp64.cu -- the two FP64 forms of the step. Compiled with --fmad=false
// so that every a*b+c is a rounded multiply and a rounded add, as in the
// reference and the CPU oracle.
#include "mpm_ops.cuh"

namespace mpm {
const StepOps kOpsStrict = Ops<PStrict>::table("fp64-strict");
const StepOps kOpsNative = Ops<PNative>::table("fp64-native");
}  // namespace mpm
