// Instantiations of the fused 2D step for up to 256 vertices per cell, with
// the attraction.
#include "dpm2d_step.cuh"

namespace dpm {

cudaError_t launch_step2d_s8_att(const Step2DArgs &a, int warps, int variant, cudaStream_t s) {
  return launch_step_sa<8, true>(a, warps, variant, s);
}

} // namespace dpm
