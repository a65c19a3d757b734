// Batched Levenberg-Marquardt fits with 1 varying parameter (kernel in fit_lm.cuh).
#include "fit_lm.cuh"

namespace fddm {
namespace fitlm {
cudaError_t launch_nv1(const Batch& b, unsigned grid, int group_warps, cudaStream_t st) {
  return launch<1>(b, grid, group_warps, st);
}
}  // namespace fitlm
}  // namespace fddm
