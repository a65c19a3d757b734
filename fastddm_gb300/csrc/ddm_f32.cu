// Structure-function pipeline, f32 tier (FFT scalar, accumulation scalar = float, ff).
#include "ddm_run.cuh"

namespace fddm {
int run_ddm_f32(const DdmRequest& r, cudaStream_t st, std::string& err) { return run_ddm_t<float, ff>(r, st, err); }
int run_temporal_list_f32(const TemporalListGroup& g, cudaStream_t st, std::string& err) {
  return run_temporal_list_t<float, ff>(g, st, err);
}
}  // namespace fddm
