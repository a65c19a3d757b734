// Batched execution of many independent structure-function jobs of uneven
// size and length (stacks of different frame sizes, lengths, modes).
//
// Every job gets its own slice of one workspace (its layout from plan_layout).
// fddm_b200_batch_create puts each job's tables into its slice and sets its
// temporal stage up without launching it.  fddm_b200_batch_launch then
// enqueues only kernels and event dependencies (so it can be captured into a
// CUDA graph): the spatial stages longest-first onto the least-loaded of
// kWorkers library-owned streams (LPT on an estimate of each job's instruction
// count), and the temporal stages of all fft-mode jobs as one persistent
// launch of the many-job kernel per (kernel variant, CTA size), whose CTAs
// take runs of modes of any job from a shared counter.  The worker streams are
// forked from the caller's stream by an event and joined back into it, so the
// batch is ordered on that stream like a single call.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace {

constexpr int kWorkers = 4;
// Launches of the many-job kernel in one batch: one per (variant, CTA size), 3 x 3 at most.
constexpr int kMaxGroups = 16;

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

// Modes per work item of the many-job temporal kernel.
constexpr unsigned long long kModesPerItem = 32;

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

// Build and validate every job's request and layout; `total` is the workspace:
// every job's own slice, then the many-job kernel's arguments, items and counters.
int prepare(const fddm_b200_job* jobs, uint64_t njobs, int precision, std::vector<fddm::DdmRequest>& reqs,
            std::vector<size_t>& offsets, size_t& total, size_t& list_off, size_t& nitems) {
  if (precision != FDDM_PREC_FF && precision != FDDM_PREC_F64 && precision != FDDM_PREC_F32)
    return fddm::fail_with(FDDM_ERR_INVALID, "unknown precision " + std::to_string(precision));
  if (njobs && !jobs) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  reqs.assign(njobs, fddm::DdmRequest());
  offsets.assign(njobs, 0);
  total = 0;
  nitems = 0;
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
    total += up256(L.total);
    const unsigned long long Q = (unsigned long long)r.ny * (unsigned long long)(r.nx / 2 + 1);
    nitems += (size_t)((Q + kModesPerItem - 1) / kModesPerItem);
  }
  list_off = total;
  total += up256(njobs * sizeof(fddm::TemporalArgs)) + up256(nitems * sizeof(fddm::TemporalItem)) +
           up256(kMaxGroups * sizeof(int));
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

int run_tier(int precision, const fddm::DdmRequest& r, cudaStream_t st, std::string& err) {
  switch (precision) {
    case FDDM_PREC_FF: return fddm::run_ddm_ff(r, st, err);
    case FDDM_PREC_F64: return fddm::run_ddm_f64(r, st, err);
    default: return fddm::run_ddm_f32(r, st, err);
  }
}

int list_tier(int precision, const fddm::TemporalListGroup& g, cudaStream_t st, std::string& err) {
  switch (precision) {
    case FDDM_PREC_FF: return fddm::run_temporal_list_ff(g, st, err);
    case FDDM_PREC_F64: return fddm::run_temporal_list_f64(g, st, err);
    default: return fddm::run_temporal_list_f32(g, st, err);
  }
}

}  // namespace

// A prepared batch: every job's tables in its workspace slice, the temporal
// stages of the fft-mode jobs grouped by kernel variant and CTA size into
// launches of the many-job kernel, and the spatial order (longest first).
struct fddm_b200_batch {
  int precision = 0;
  std::vector<fddm::DdmRequest> reqs;
  std::vector<double> cost;
  std::vector<uint64_t> order;          // spatial stages, longest first
  std::vector<int> own_temporal;        // jobs whose temporal stage launches on its own
  std::vector<fddm::TemporalListGroup> groups;
};

extern "C" int fddm_b200_batch_workspace_size(const fddm_b200_job* jobs, uint64_t njobs, int precision,
                                              size_t* bytes) {
  fddm::set_last_error("");
  if (!bytes) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  std::vector<fddm::DdmRequest> reqs;
  std::vector<size_t> offsets;
  size_t total = 0, list_off = 0, nitems = 0;
  const int rc = prepare(jobs, njobs, precision, reqs, offsets, total, list_off, nitems);
  if (rc != FDDM_OK) return rc;
  *bytes = total;
  return FDDM_OK;
}

extern "C" int fddm_b200_batch_create(const fddm_b200_job* jobs, uint64_t njobs, int precision, void* d_workspace,
                                      size_t workspace_bytes, void* stream, fddm_b200_batch** plan) {
  fddm::set_last_error("");
  if (!plan) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  *plan = nullptr;
  auto p = std::make_unique<fddm_b200_batch>();
  p->precision = precision;
  std::vector<size_t> offsets;
  size_t total = 0, list_off = 0, nitems_all = 0;
  int rc = prepare(jobs, njobs, precision, p->reqs, offsets, total, list_off, nitems_all);
  if (rc != FDDM_OK) return rc;
  if (!d_workspace && njobs) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  if (workspace_bytes < total)
    return fddm::fail_with(FDDM_ERR_NOMEM, "workspace too small: need " + std::to_string(total) + " bytes, got " +
                                               std::to_string(workspace_bytes));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  // every job's tables into its slice, and its temporal stage set up (not launched)
  std::vector<fddm::TemporalLaunch> tl(njobs);
  p->cost.assign(njobs, 0.0);
  std::string err;
  for (uint64_t i = 0; i < njobs; ++i) {
    fddm::DdmRequest& r = p->reqs[i];
    if (!r.img || !r.out) return fddm::fail_with(FDDM_ERR_INVALID, "job " + std::to_string(i) + ": null pointer");
    r.work = ws + offsets[i];
    r.stages = 0;
    r.collect = &tl[i];
    if ((rc = run_tier(precision, r, st, err)) != 0) return fddm::fail_with(rc, "job " + std::to_string(i) + ": " + err);
    r.collect = nullptr;
    r.tables_ready = true;
    p->cost[i] = job_cost(r);
  }
  p->order.resize(njobs);
  std::iota(p->order.begin(), p->order.end(), 0);
  std::stable_sort(p->order.begin(), p->order.end(), [&](uint64_t a, uint64_t b) { return p->cost[a] > p->cost[b]; });
  // group the many-job-kernel stages by (variant, CTA size); items of costlier jobs first
  std::map<std::pair<int, int>, std::vector<uint64_t>> by_key;
  for (uint64_t i : p->order) {
    if (tl[i].variant >= 0 && tl[i].smem + fddm::kListStaticSmem <= fddm::kSmemLimit)
      by_key[{tl[i].variant, tl[i].threads}].push_back(i);
    else
      p->own_temporal.push_back((int)i);
  }
  std::vector<fddm::TemporalArgs> args(njobs);
  for (uint64_t i = 0; i < njobs; ++i) args[i] = tl[i].args;
  std::vector<fddm::TemporalItem> items;
  auto* d_args = reinterpret_cast<fddm::TemporalArgs*>(ws + list_off);
  auto* d_items = reinterpret_cast<fddm::TemporalItem*>(ws + list_off + up256(njobs * sizeof(fddm::TemporalArgs)));
  int* d_counters = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(d_items) +
                                           up256(nitems_all * sizeof(fddm::TemporalItem)));
  for (auto& kv : by_key) {  // at most 3 variants x 3 CTA sizes <= kMaxGroups
    const size_t first = items.size();
    fddm::TemporalListGroup g;
    g.variant = kv.first.first;
    g.threads = kv.first.second;
    g.d_args = d_args;
    g.d_items = d_items + first;
    g.d_counter = d_counters + p->groups.size();
    for (uint64_t i : kv.second) {
      g.smem = std::max(g.smem, tl[i].smem);
      const unsigned long long Q = tl[i].args.Q;
      for (unsigned long long q0 = 0; q0 < Q; q0 += kModesPerItem)
        items.push_back({(int)i, 0, q0, std::min(Q, q0 + kModesPerItem)});
    }
    g.nitems = (int)(items.size() - first);
    p->groups.push_back(g);
  }
  cudaError_t ce;
  if (njobs && (ce = cudaMemcpyAsync(d_args, args.data(), njobs * sizeof(fddm::TemporalArgs), cudaMemcpyHostToDevice,
                                     st)) != cudaSuccess)
    return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  if (!items.empty() && (ce = cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(fddm::TemporalItem),
                                              cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  *plan = p.release();
  return FDDM_OK;
}

extern "C" int fddm_b200_batch_launch(fddm_b200_batch* p, void* stream) {
  fddm::set_last_error("");
  if (!p) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  if (p->reqs.empty()) return FDDM_OK;
  std::string err;
  Workers* w = workers(err);
  if (!w) return fddm::fail_with(FDDM_ERR_CUDA, err);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t ce;
  auto fork = [&]() -> cudaError_t {
    cudaError_t e = cudaEventRecord(w->fork, st);
    for (int k = 0; k < kWorkers && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(w->s[k], w->fork, 0);
    return e;
  };
  auto join = [&]() -> cudaError_t {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < kWorkers && e == cudaSuccess; ++k) {
      e = cudaEventRecord(w->join[k], w->s[k]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, w->join[k], 0);
    }
    return e;
  };
  if ((ce = fork()) != cudaSuccess) return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  int first_err = FDDM_OK;
  std::string first_msg;
  auto note = [&](int r, const std::string& who) {
    if (r != 0 && first_err == FDDM_OK) {
      first_err = r;
      first_msg = who + err;
    }
  };
  // spatial stages, longest first onto the least-loaded worker
  double load[kWorkers] = {0.0};
  for (uint64_t i : p->order) {
    const int k = (int)(std::min_element(load, load + kWorkers) - load);
    load[k] += p->cost[i];
    fddm::DdmRequest r = p->reqs[i];
    r.stages = 1;
    note(run_tier(p->precision, r, w->s[k], err), "job " + std::to_string(i) + ": ");
  }
  // every temporal stage after every spatial stage
  if ((ce = join()) != cudaSuccess || (ce = fork()) != cudaSuccess)
    return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  for (size_t g = 0; g < p->groups.size(); ++g)
    note(list_tier(p->precision, p->groups[g], w->s[g % kWorkers], err), "temporal group: ");
  for (size_t n = 0; n < p->own_temporal.size(); ++n) {
    const int i = p->own_temporal[n];
    fddm::DdmRequest r = p->reqs[i];
    r.stages = 2;
    note(run_tier(p->precision, r, w->s[(p->groups.size() + n) % kWorkers], err), "job " + std::to_string(i) + ": ");
  }
  // join the workers back into the caller's stream even after an error
  if ((ce = join()) != cudaSuccess) return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  if (first_err != FDDM_OK) return fddm::fail_with(first_err, first_msg);
  return FDDM_OK;
}

extern "C" int fddm_b200_batch_destroy(fddm_b200_batch* p) {
  delete p;
  return FDDM_OK;
}

extern "C" int fddm_b200_batch_run(const fddm_b200_job* jobs, uint64_t njobs, int precision, void* d_workspace,
                                   size_t workspace_bytes, void* stream) {
  fddm_b200_batch* p = nullptr;
  int rc = fddm_b200_batch_create(jobs, njobs, precision, d_workspace, workspace_bytes, stream, &p);
  if (rc != FDDM_OK) return rc;
  rc = fddm_b200_batch_launch(p, stream);
  fddm_b200_batch_destroy(p);
  return rc;
}
