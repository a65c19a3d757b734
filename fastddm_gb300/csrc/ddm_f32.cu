// Structure-function pipeline, f32 tier (FFT scalar, accumulation scalar = float, ff).
#include "ddm_run.cuh"

namespace fddm {
int run_ddm_f32(const DdmRequest& r, cudaStream_t st, std::string& err) { return run_ddm_t<float, ff>(r, st, err); }
}  // namespace fddm
