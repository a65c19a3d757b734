// Batched execution of many independent structure-function jobs of uneven
// size and length (stacks of different frame sizes, lengths, modes).
//
// Every job gets its own slice of one workspace (its layout from plan_layout).
// Jobs are scheduled longest-first onto the least-loaded of kWorkers
// library-owned streams (LPT scheduling on an estimate of each job's
// instruction count); the worker streams are forked from the caller's stream
// by an event and joined back into it, so the whole batch is ordered on that
// stream like a single call while independent jobs overlap on the GPU.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace {

constexpr int kWorkers = 4;

struct Workers {
  cudaStream_t s[kWorkers];
  cudaEvent_t fork, join[kWorkers];
};
std::mutex g_mu;
std::map<int, Workers> g_workers;  // per device

Workers* workers(std::string& err) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return nullptr; }
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_workers.find(dev);
  if (it == g_workers.end()) {
    Workers w{};
    if ((ce = cudaEventCreateWithFlags(&w.fork, cudaEventDisableTiming)) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return nullptr;
    }
    for (int i = 0; i < kWorkers; ++i) {
      if ((ce = cudaStreamCreateWithFlags(&w.s[i], cudaStreamNonBlocking)) != cudaSuccess ||
          (ce = cudaEventCreateWithFlags(&w.join[i], cudaEventDisableTiming)) != cudaSuccess) {
        err = cudaGetErrorString(ce);
        return nullptr;
      }
    }
    it = g_workers.emplace(dev, w).first;
  }
  return &it->second;
}

bool map_dtype(int dtype, int& out) {
  switch (dtype) {
    case FDDM_U8: out = fddm::DT_U8; return true;
    case FDDM_I16: out = fddm::DT_I16; return true;
    case FDDM_U16: out = fddm::DT_U16; return true;
    case FDDM_I32: out = fddm::DT_I32; return true;
    case FDDM_U32: out = fddm::DT_U32; return true;
    case FDDM_F32: out = fddm::DT_F32; return true;
    case FDDM_F64: out = fddm::DT_F64; return true;
    default: return false;
  }
}

// Build and validate every job's request and layout; returns the total workspace.
int prepare(const fddm_b200_job* jobs, uint64_t njobs, int precision, std::vector<fddm::DdmRequest>& reqs,
            std::vector<size_t>& offsets, size_t& total) {
  if (precision != FDDM_PREC_FF && precision != FDDM_PREC_F64 && precision != FDDM_PREC_F32)
    return fddm::fail_with(FDDM_ERR_INVALID, "unknown precision " + std::to_string(precision));
  if (njobs && !jobs) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  reqs.assign(njobs, fddm::DdmRequest());
  offsets.assign(njobs, 0);
  total = 0;
  for (uint64_t i = 0; i < njobs; ++i) {
    const fddm_b200_job& j = jobs[i];
    fddm::DdmRequest& r = reqs[i];
    const std::string who = "job " + std::to_string(i) + ": ";
    if (j.mode != FDDM_MODE_FFT && j.mode != FDDM_MODE_DIFF) return fddm::fail_with(FDDM_ERR_INVALID, who + "unknown mode");
    if (!map_dtype(j.dtype, r.dtype)) return fddm::fail_with(FDDM_ERR_INVALID, who + "unsupported input dtype");
    if (j.nlags && !j.lags) return fddm::fail_with(FDDM_ERR_INVALID, who + "null lags");
    r.mode = j.mode == FDDM_MODE_FFT ? fddm::MODE_FFT : fddm::MODE_DIFF;
    r.precision = precision;
    r.img = j.d_img_seq;
    r.T = (int64_t)j.length; r.H = (int64_t)j.height; r.W = (int64_t)j.width;
    r.lags.assign(j.lags, j.lags + j.nlags);
    r.nx = (int64_t)j.nx; r.ny = (int64_t)j.ny; r.nt = r.mode == fddm::MODE_FFT ? (int64_t)j.nt : 0;
    r.window = j.d_window;
    r.out = j.d_out;
    fddm::WorkLayout L;
    std::string err;
    if (!fddm::plan_layout(r, L, err)) return fddm::fail_with(FDDM_ERR_UNSUPPORTED, who + err);
    offsets[i] = total;
    r.work_bytes = L.total;
    total += (L.total + 255) / 256 * 256;
  }
  return FDDM_OK;
}

// Estimated work of a job (float-float instruction count, arbitrary units).
double job_cost(const fddm::DdmRequest& r) {
  const double nkx = (double)(r.nx / 2 + 1), Q = (double)r.ny * nkx, T = (double)r.T;
  const double spatial = T * (double)r.nx * (double)r.ny * std::log2((double)r.nx * (double)r.ny + 1.0);
  double temporal;
  if (r.mode == fddm::MODE_FFT) {
    const double N = (double)fddm::choose_temporal_length(r.T);
    temporal = Q * 1.5 * N * std::log2(N + 1.0) * 1.2;
  } else {
    double pairs = 0.0;
    for (int lag : r.lags) pairs += T - lag;
    temporal = Q * pairs * 0.4;
  }
  return spatial + temporal;
}

}  // namespace

extern "C" int fddm_b200_batch_workspace_size(const fddm_b200_job* jobs, uint64_t njobs, int precision,
                                              size_t* bytes) {
  fddm::set_last_error("");
  if (!bytes) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  std::vector<fddm::DdmRequest> reqs;
  std::vector<size_t> offsets;
  size_t total = 0;
  const int rc = prepare(jobs, njobs, precision, reqs, offsets, total);
  if (rc != FDDM_OK) return rc;
  *bytes = total;
  return FDDM_OK;
}

extern "C" int fddm_b200_batch_run(const fddm_b200_job* jobs, uint64_t njobs, int precision, void* d_workspace,
                                   size_t workspace_bytes, void* stream) {
  fddm::set_last_error("");
  std::vector<fddm::DdmRequest> reqs;
  std::vector<size_t> offsets;
  size_t total = 0;
  int rc = prepare(jobs, njobs, precision, reqs, offsets, total);
  if (rc != FDDM_OK) return rc;
  if (njobs == 0) return FDDM_OK;
  if (!d_workspace) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  if (workspace_bytes < total)
    return fddm::fail_with(FDDM_ERR_NOMEM, "workspace too small: need " + std::to_string(total) + " bytes, got " +
                                               std::to_string(workspace_bytes));
  for (uint64_t i = 0; i < njobs; ++i) {
    if (!reqs[i].img || !reqs[i].out) return fddm::fail_with(FDDM_ERR_INVALID, "job " + std::to_string(i) + ": null pointer");
    reqs[i].work = static_cast<unsigned char*>(d_workspace) + offsets[i];
  }
  std::string err;
  Workers* w = workers(err);
  if (!w) return fddm::fail_with(FDDM_ERR_CUDA, err);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t ce;
  if ((ce = cudaEventRecord(w->fork, st)) != cudaSuccess) return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  for (int k = 0; k < kWorkers; ++k)
    if ((ce = cudaStreamWaitEvent(w->s[k], w->fork, 0)) != cudaSuccess)
      return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));

  // longest processing time first onto the least-loaded worker
  std::vector<double> cost(njobs);
  for (uint64_t i = 0; i < njobs; ++i) cost[i] = job_cost(reqs[i]);
  std::vector<uint64_t> order(njobs);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return cost[a] > cost[b]; });
  double load[kWorkers] = {0.0};
  int first_err = FDDM_OK;
  std::string first_msg;
  for (uint64_t i : order) {
    const int k = (int)(std::min_element(load, load + kWorkers) - load);
    load[k] += cost[i];
    int r;
    switch (precision) {
      case FDDM_PREC_FF: r = fddm::run_ddm_ff(reqs[i], w->s[k], err); break;
      case FDDM_PREC_F64: r = fddm::run_ddm_f64(reqs[i], w->s[k], err); break;
      default: r = fddm::run_ddm_f32(reqs[i], w->s[k], err); break;
    }
    if (r != 0 && first_err == FDDM_OK) {
      first_err = r;
      first_msg = "job " + std::to_string(i) + ": " + err;
    }
  }
  // join the workers back into the caller's stream even after an error
  for (int k = 0; k < kWorkers; ++k) {
    if ((ce = cudaEventRecord(w->join[k], w->s[k])) != cudaSuccess || (ce = cudaStreamWaitEvent(st, w->join[k], 0)) != cudaSuccess)
      return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  }
  if (first_err != FDDM_OK) return fddm::fail_with(first_err, first_msg);
  return FDDM_OK;
}
