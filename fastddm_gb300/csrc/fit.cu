// C ABI of the batched Levenberg-Marquardt fits (device code in fit_lm.cuh;
// the kernel for each number of varying parameters is compiled in its own
// translation unit, fit_nv<k>.cu).
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <cstdlib>
#include <string>
#include "fddm_b200.h"
#include "fddm_internal.h"
#include "fit_lm.cuh"

namespace {

size_t slot_doubles(uint64_t m, int np) { return (size_t)(2 + np) * m; }

int sm_count() {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm > 0 ? nsm : 152;
}

// Warps per chain: with at most four chains per SM a chain takes a whole CTA (its per-point work
// spread over the SM's four sub-partitions; measured faster up to 512 chains of one fit each, whose
// few long fits set the launch's time); with more, each warp runs its own chains (no sub-partition
// repeats the small-matrix work of another).  FDDM_B200_FIT_GROUP_WARPS=1|4 overrides the choice
// (tuning runs).
int group_warps(uint64_t nchains) {
  const char* v = std::getenv("FDDM_B200_FIT_GROUP_WARPS");
  const int x = v ? std::atoi(v) : 0;
  if (x == 1 || x == fddm::fitlm::kWarpsPerCta) return x;
  return nchains <= 4 * (uint64_t)sm_count() ? fddm::fitlm::kWarpsPerCta : 1;
}

// groups resident at once (8 CTAs per SM)
uint64_t max_slots(int group) { return (uint64_t)sm_count() * 8 * (fddm::fitlm::kWarpsPerCta / group); }

}  // namespace

using namespace fddm;

extern "C" int fddm_b200_fit_model_nparams(int model) { return fitlm::model_nparams(model); }

extern "C" int fddm_b200_fit_workspace_bytes(int model, uint64_t m, uint64_t nchains, uint64_t* bytes) {
  set_last_error("");
  if (!bytes) return fail_with(FDDM_ERR_INVALID, "null pointer argument");
  const int np = fitlm::model_nparams(model);
  if (np == 0) return fail_with(FDDM_ERR_INVALID, "unknown fit model");
  const uint64_t slots = std::min<uint64_t>(nchains, max_slots(group_warps(nchains)));
  *bytes = (uint64_t)slot_doubles(m, np) * sizeof(double) * slots;
  return FDDM_OK;
}

extern "C" int fddm_b200_fit_lm(int model, uint64_t m, const double* d_x, uint64_t ldx, uint64_t nx,
                                const double* d_y, uint64_t ldy, uint64_t ny, const double* d_w, uint64_t ldw,
                                uint64_t nw, const int32_t* d_problems, uint64_t nproblems,
                                const int32_t* d_chain_offsets, const int32_t* d_chain_problems, uint64_t nchains,
                                int nvary, const double* d_init, const double* d_min, const double* d_max,
                                const double* options, double* d_values, double* d_stderr, double* d_chisqr,
                                int32_t* d_nfev, int32_t* d_info, int32_t* d_status, double* d_residual,
                                double* d_covar, void* d_workspace, uint64_t workspace_bytes, void* stream) {
  set_last_error("");
  const int np = fitlm::model_nparams(model);
  if (np == 0) return fail_with(FDDM_ERR_INVALID, "unknown fit model");
  if (nvary < 1 || nvary > np) return fail_with(FDDM_ERR_INVALID, "nvary must be in 1..nparams");
  if ((uint64_t)nvary > m) return fail_with(FDDM_ERR_INVALID, "fewer data points than varying parameters");
  if (nx == 0 || ny == 0) return fail_with(FDDM_ERR_INVALID, "no abscissa or data rows");
  if (m > (1ull << 30) || nproblems > (1ull << 30) || nchains > (1ull << 30) || ny > (1ull << 30) ||
      nw > (1ull << 30) || nx > (1ull << 30))
    return fail_with(FDDM_ERR_UNSUPPORTED, "too many data points, problems or chains");
  if (!options) return fail_with(FDDM_ERR_INVALID, "null options");
  // every iteration evaluates the model, so max_nfev bounds a fit's run; above this a fit that never
  // converges could hold the GPU for minutes
  if (!(options[5] <= 1e6)) return fail_with(FDDM_ERR_UNSUPPORTED, "max_nfev above 1,000,000");
  if (nchains == 0 || nproblems == 0) return FDDM_OK;
  if (!d_x || !d_y || !d_problems || !d_chain_offsets || !d_chain_problems || !d_init || !d_min || !d_max ||
      !d_values || !d_stderr || !d_chisqr || !d_nfev || !d_info || !d_status || !d_workspace)
    return fail_with(FDDM_ERR_INVALID, "null pointer argument");
  if (ldx < m || ldy < m || (d_w && ldw < m)) return fail_with(FDDM_ERR_INVALID, "row stride shorter than the data");
  const uint64_t per_slot = (uint64_t)slot_doubles(m, np) * sizeof(double);
  const int group = group_warps(nchains);
  const uint64_t slots = std::min<uint64_t>({nchains, max_slots(group), workspace_bytes / per_slot});
  if (slots == 0) return fail_with(FDDM_ERR_NOMEM, "fit workspace smaller than one slot");
  fitlm::Batch b{};
  b.model = model;
  b.np = np;
  b.m = (int)m;
  b.x = d_x;
  b.ldx = ldx;
  b.nx = (int)nx;
  b.y = d_y;
  b.ldy = ldy;
  b.ny = (int)ny;
  b.w = d_w;
  b.ldw = ldw;
  b.nw = d_w ? (int)nw : 0;
  b.nprob = (int)nproblems;
  b.problems = d_problems;
  b.chain_off = d_chain_offsets;
  b.chain_list = d_chain_problems;
  b.nchains = (int)nchains;
  b.init = d_init;
  b.lo = d_min;
  b.hi = d_max;
  b.ftol = options[0];
  b.xtol = options[1];
  b.gtol = options[2];
  b.epsfcn = options[3];
  b.factor = options[4];
  b.max_nfev = options[5] > 0 ? (long long)options[5] : 2000LL * (nvary + 1);
  b.values = d_values;
  b.stderr_ = d_stderr;
  b.chisqr = d_chisqr;
  b.nfev = d_nfev;
  b.info = d_info;
  b.status = d_status;
  b.residual = d_residual;
  b.covar = d_covar;
  b.ws = static_cast<double*>(d_workspace);
  b.slot_doubles = slot_doubles(m, np);
  b.nslots = (int)slots;
  const unsigned grid = (unsigned)(group > 1 ? slots : (slots + fitlm::kWarpsPerCta - 1) / fitlm::kWarpsPerCta);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t ce;
  switch (nvary) {
    case 1: ce = fitlm::launch_nv1(b, grid, group, st); break;
    case 2: ce = fitlm::launch_nv2(b, grid, group, st); break;
    case 3: ce = fitlm::launch_nv3(b, grid, group, st); break;
    case 4: ce = fitlm::launch_nv4(b, grid, group, st); break;
    case 5: ce = fitlm::launch_nv5(b, grid, group, st); break;
    case 6: ce = fitlm::launch_nv6(b, grid, group, st); break;
    default: ce = fitlm::launch_nv7(b, grid, group, st); break;
  }
  if (ce != cudaSuccess) return fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  count_launches(1);
  return FDDM_OK;
}
