// Instantiations of the fused 2D step for up to 32 vertices per cell.
#include "dpm2d_step.cuh"

namespace dpm {

cudaError_t launch_step2d_s1(const Step2DArgs &a, int warps, int variant, cudaStream_t s) {
  return launch_step_s<1>(a, warps, variant, s);
}

cudaError_t launch_team2d_s1(const Step2DArgs &a, int variant, cudaStream_t s) {
  return launch_team_s<1>(a, variant, s);
}

cudaError_t launch_resident2d_s1(const Resident2DArgs &r, int ntissues, int variant,
                                 cudaStream_t s) {
  return launch_resident_s<1>(r, ntissues, variant, s);
}

} // namespace dpm
