// Instantiations of the fused 2D step for up to 64 vertices per cell.
#include "dpm2d_step.cuh"

namespace dpm {

cudaError_t launch_step2d_s2(const Step2DArgs &a, int warps, int variant, cudaStream_t s) {
  return launch_step_s<2>(a, warps, variant, s);
}

cudaError_t launch_team2d_s2(const Step2DArgs &a, int variant, cudaStream_t s) {
  return launch_team_s<2>(a, variant, s);
}

cudaError_t launch_resident2d_s2(const Resident2DArgs &r, int ntissues, int variant,
                                 cudaStream_t s) {
  return launch_resident_s<2>(r, ntissues, variant, s);
}

} // namespace dpm
