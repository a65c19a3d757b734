// Structure-function pipeline, ff tier (FFT scalar, accumulation scalar = ff, ff).
#include "ddm_run.cuh"

namespace fddm {
int run_ddm_ff(const DdmRequest& r, cudaStream_t st, std::string& err) { return run_ddm_t<ff, ff>(r, st, err); }
int run_temporal_list_ff(const TemporalListGroup& g, cudaStream_t st, std::string& err) {
  return run_temporal_list_t<ff, ff>(g, st, err);
}
}  // namespace fddm
