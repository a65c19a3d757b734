// C ABI entry points (declared in include/fddm_b200.h).
#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>
#include <cstring>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace {
thread_local std::string g_last_error;
thread_local int g_last_input_path = 0;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
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
    default: return false;  // 64-bit integers are converted to FP64 by the caller
  }
}

int run(int mode, const void* img, int dtype, uint64_t length, uint64_t height, uint64_t width,
        const uint32_t* lags, uint64_t nlags, uint64_t nx, uint64_t ny, uint64_t nt, const double* window,
        double* out, void* work, size_t work_bytes, int precision, void* stream,
        const void* host_img = nullptr, double* host_out = nullptr) {
  g_last_error.clear();
  // host frames read in place need no device frame buffer (the pipeline checks that they can be)
  if ((!img && !host_img) || !out || (nlags && !lags) || !work) return fail(FDDM_ERR_INVALID, "null pointer argument");
  fddm::DdmRequest r;
  r.host_img = host_img;
  r.host_out = host_out;
  r.mode = mode;
  r.precision = precision;
  if (precision != FDDM_PREC_FF && precision != FDDM_PREC_F64 && precision != FDDM_PREC_F32)
    return fail(FDDM_ERR_INVALID, "unknown precision " + std::to_string(precision));
  if (!map_dtype(dtype, r.dtype)) return fail(FDDM_ERR_INVALID, "unsupported input dtype code " + std::to_string(dtype));
  r.img = img;
  r.T = (int64_t)length; r.H = (int64_t)height; r.W = (int64_t)width;
  r.lags.assign(lags, lags + nlags);
  r.nx = (int64_t)nx; r.ny = (int64_t)ny; r.nt = (int64_t)nt;
  r.window = window;
  r.out = out;
  r.work = work;
  r.work_bytes = work_bytes;
  std::string err;
  int rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (precision) {
    case FDDM_PREC_FF: rc = fddm::run_ddm_ff(r, st, err); break;
    case FDDM_PREC_F64: rc = fddm::run_ddm_f64(r, st, err); break;
    default: rc = fddm::run_ddm_f32(r, st, err); break;
  }
  if (rc != 0) return fail(rc, err);
  return FDDM_OK;
}
}  // namespace

namespace fddm {
namespace {
std::atomic<uint64_t> g_launches{0};
std::atomic<bool> g_timing{false};
std::mutex g_ev_mu;
std::map<int, StageEvents> g_events;  // per device
}  // namespace

void count_launches(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
void set_last_input_path(int path) { g_last_input_path = path; }

namespace {
std::mutex g_copy_mu;
std::map<int, std::unique_ptr<CopyCtx>> g_copy;  // per device
}  // namespace

CopyCtx* copy_ctx(std::string& err) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return nullptr; }
  std::lock_guard<std::mutex> lk(g_copy_mu);
  auto it = g_copy.find(dev);
  if (it == g_copy.end()) {
    auto c = std::make_unique<CopyCtx>();
    if ((ce = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (ce = cudaEventCreateWithFlags(&c->ready, cudaEventDisableTiming)) != cudaSuccess ||
        (ce = cudaEventCreateWithFlags(&c->start, cudaEventDisableTiming)) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return nullptr;
    }
    it = g_copy.emplace(dev, std::move(c)).first;
  }
  return it->second.get();
}

size_t dtype_bytes(int dtype) {
  switch (dtype) {
    case DT_U8: return 1;
    case DT_I16: case DT_U16: return 2;
    case DT_I32: case DT_U32: case DT_F32: return 4;
    default: return 8;
  }
}

StageEvents* stage_events() {
  if (!g_timing.load()) return nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_ev_mu);
  auto it = g_events.find(dev);
  if (it == g_events.end()) {
    StageEvents e{};
    e.enabled = true;
    for (auto& ev : e.ev)
      if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
    it = g_events.emplace(dev, e).first;
  }
  return &it->second;
}

void set_last_error(const std::string& msg) { g_last_error = msg; }
int fail_with(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace fddm

extern "C" {

int fddm_b200_version(void) { return 100; }

const char* fddm_b200_last_error(void) { return g_last_error.c_str(); }

int fddm_b200_workspace_size(int mode, int precision, uint64_t length, uint64_t height, uint64_t width,
                             uint64_t nlags, uint64_t nx, uint64_t ny, uint64_t nt, int has_window,
                             size_t* bytes) {
  g_last_error.clear();
  if (!bytes) return fail(FDDM_ERR_INVALID, "null pointer argument");
  if (mode != FDDM_MODE_FFT && mode != FDDM_MODE_DIFF) return fail(FDDM_ERR_INVALID, "unknown mode");
  if (precision != FDDM_PREC_FF && precision != FDDM_PREC_F64 && precision != FDDM_PREC_F32)
    return fail(FDDM_ERR_INVALID, "unknown precision " + std::to_string(precision));
  fddm::DdmRequest r;
  r.mode = mode;
  r.precision = precision;
  r.T = (int64_t)length; r.H = (int64_t)height; r.W = (int64_t)width;
  r.lags.assign(nlags, 0);  // lag values do not change the layout
  r.nx = (int64_t)nx; r.ny = (int64_t)ny; r.nt = (int64_t)nt;
  static const double dummy = 0.0;
  r.window = has_window ? &dummy : nullptr;
  fddm::WorkLayout L;
  std::string err;
  if (!fddm::plan_layout(r, L, err)) return fail(FDDM_ERR_UNSUPPORTED, err);
  *bytes = L.total;
  return FDDM_OK;
}

int fddm_b200_ddm_fft(const void* d_img_seq, int dtype, uint64_t length, uint64_t height, uint64_t width,
                      const uint32_t* lags, uint64_t nlags, uint64_t nx, uint64_t ny, uint64_t nt,
                      const double* d_window, double* d_out, void* d_workspace, size_t workspace_bytes,
                      int precision, void* stream) {
  return run(fddm::MODE_FFT, d_img_seq, dtype, length, height, width, lags, nlags, nx, ny, nt, d_window, d_out,
             d_workspace, workspace_bytes, precision, stream);
}

int fddm_b200_ddm_diff(const void* d_img_seq, int dtype, uint64_t length, uint64_t height, uint64_t width,
                       const uint32_t* lags, uint64_t nlags, uint64_t nx, uint64_t ny, const double* d_window,
                       double* d_out, void* d_workspace, size_t workspace_bytes, int precision, void* stream) {
  return run(fddm::MODE_DIFF, d_img_seq, dtype, length, height, width, lags, nlags, nx, ny, 0, d_window, d_out,
             d_workspace, workspace_bytes, precision, stream);
}

int fddm_b200_set_stage_timing(int enable) {
  fddm::g_timing.store(enable != 0);
  return FDDM_OK;
}

int fddm_b200_stage_times(float* spatial_ms, float* temporal_ms) {
  g_last_error.clear();
  if (!spatial_ms || !temporal_ms) return fail(FDDM_ERR_INVALID, "null pointer argument");
  fddm::StageEvents* e = fddm::stage_events();
  if (!e) return fail(FDDM_ERR_INVALID, "stage timing is not enabled");
  cudaError_t ce = cudaEventSynchronize(e->ev[2]);
  if (ce == cudaSuccess) ce = cudaEventElapsedTime(spatial_ms, e->ev[0], e->ev[1]);
  if (ce == cudaSuccess) ce = cudaEventElapsedTime(temporal_ms, e->ev[1], e->ev[2]);
  if (ce != cudaSuccess) return fail(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  return FDDM_OK;
}

uint64_t fddm_b200_launch_count(void) { return fddm::g_launches.load(); }

int fddm_b200_last_input_path(void) { return g_last_input_path; }

int fddm_b200_ddm_from_host(int mode, const void* h_img_seq, int dtype, uint64_t length, uint64_t height,
                            uint64_t width, const uint32_t* lags, uint64_t nlags, uint64_t nx, uint64_t ny,
                            uint64_t nt, void* d_frames, const double* d_window, double* d_out, double* h_out,
                            void* d_workspace, size_t workspace_bytes, int precision, void* stream) {
  if (!h_img_seq) return fail(FDDM_ERR_INVALID, "null pointer argument");
  if (mode != FDDM_MODE_FFT && mode != FDDM_MODE_DIFF) return fail(FDDM_ERR_INVALID, "unknown mode");
  return run(mode == FDDM_MODE_FFT ? fddm::MODE_FFT : fddm::MODE_DIFF, d_frames, dtype, length, height, width, lags,
             nlags, nx, ny, mode == FDDM_MODE_FFT ? nt : 0, d_window, d_out, d_workspace, workspace_bytes, precision,
             stream, h_img_seq, h_out);
}

}  // extern "C"
