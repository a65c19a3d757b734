// Structure-function pipeline, f64 tier (FFT scalar, accumulation scalar = double, double).
#include "ddm_run.cuh"

namespace fddm {
int run_ddm_f64(const DdmRequest& r, cudaStream_t st, std::string& err) { return run_ddm_t<double, double>(r, st, err); }
int run_temporal_list_f64(const TemporalListGroup& g, cudaStream_t st, std::string& err) {
  return run_temporal_list_t<double, double>(g, st, err);
}
}  // namespace fddm
