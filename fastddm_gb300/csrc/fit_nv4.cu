// Batched Levenberg-Marquardt fits with 4 varying parameters (kernel in fit_lm.cuh).
#include "fit_lm.cuh"

namespace fddm {
namespace fitlm {
cudaError_t launch_nv4(const Batch& b, unsigned grid, int group_warps, cudaStream_t st) {
  return launch<4>(b, grid, group_warps, st);
}
}  // namespace fitlm
}  // namespace fddm
