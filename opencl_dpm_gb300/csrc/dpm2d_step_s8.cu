// Instantiations of the fused 2D step for up to 256 vertices per cell,
// without the attraction (dpm2d_step_s8_att.cu has it: the two compile in
// parallel).
#include "dpm2d_step.cuh"

namespace dpm {

cudaError_t launch_step2d_s8(const Step2DArgs &a, int warps, int variant, cudaStream_t s) {
  if (variant & kStepVariantAttraction) return launch_step2d_s8_att(a, warps, variant, s);
  return launch_step_sa<8, false>(a, warps, variant, s);
}

} // namespace dpm
