// fddm_b200_ddm_fft_noalloc: the fft-mode structure function with all of its
// scratch in one fixed-size array that lives in device memory for as long as
// the library is loaded.
//
// Some callers cannot allocate device memory at the moment they need a result:
// a camera acquisition callback that must not stall on the allocator, a plugin
// whose host application owns every device allocation, a process that
// reserves all of its memory up front.  This entry point serves them: it never
// calls cudaMalloc, cudaFree or any allocating routine; the caller passes only
// the frames, the window and the output.
//
// Limits and sharing:
//   * the scratch is kNoAllocScratchBytes (64 MiB) on every device that loads
//     the library; problems whose workspace does not fit are rejected with
//     FDDM_ERR_NOMEM and a message giving the bytes needed;
//   * every call shares the one array and leaves its contents behind; the
//     pipeline writes every scratch value before reading it, so nothing has to
//     start at zero, but calls whose work overlaps on the GPU (two streams, or
//     two host threads) race on the array and must be serialised by the caller;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current and caches it.  Under
//     lazy module loading (the CUDA default) that lookup is also when the
//     device reserves the 64 MiB, so a caller that reserves its device memory
//     up front, or captures streams into graphs, makes one first call (any
//     valid problem that fits) before doing so.  If the device has no room
//     left at that point the call returns FDDM_ERR_NOMEM.
#include <map>
#include <mutex>
#include <string>
#include "fddm_b200.h"
#include "fddm_internal.h"

static constexpr size_t kNoAllocScratchBytes = 64ull << 20;

// In host code this name is only a host-side stand-in, not a device address:
// the device address comes from cudaGetSymbolAddress below, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_addr_mu;
std::map<int, void*> g_addr;  // device -> address of g_noalloc_scratch

int scratch_address(void** out) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  std::lock_guard<std::mutex> lk(g_addr_mu);
  auto it = g_addr.find(dev);
  if (it == g_addr.end()) {
    void* p = nullptr;
    // under lazy module loading (the CUDA default) this first lookup loads the
    // module that holds the array, which is when the device reserves its memory
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce == cudaErrorMemoryAllocation) {
      (void)cudaGetLastError();
      return fddm::fail_with(FDDM_ERR_NOMEM,
                             "the device has no room for the 64 MiB static scratch of fddm_b200_ddm_fft_noalloc "
                             "(reserved by the first call on a device)");
    }
    if (ce != cudaSuccess || p == nullptr)
      return fddm::fail_with(FDDM_ERR_CUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                                cudaGetErrorString(ce));
    it = g_addr.emplace(dev, p).first;
  }
  *out = it->second;
  return FDDM_OK;
}

}  // namespace

extern "C" int fddm_b200_ddm_fft_noalloc(const void* d_img_seq, int dtype, uint64_t length, uint64_t height,
                                         uint64_t width, const uint32_t* lags, uint64_t nlags, uint64_t nx,
                                         uint64_t ny, uint64_t nt, const double* d_window, double* d_out,
                                         int precision, void* stream) {
  fddm::set_last_error("");
  if (!d_img_seq || !d_out || (nlags && !lags)) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  if (precision != FDDM_PREC_FF && precision != FDDM_PREC_F64 && precision != FDDM_PREC_F32)
    return fddm::fail_with(FDDM_ERR_INVALID, "unknown precision " + std::to_string(precision));
  int dt;
  switch (dtype) {
    case FDDM_U8: dt = fddm::DT_U8; break;
    case FDDM_I16: dt = fddm::DT_I16; break;
    case FDDM_U16: dt = fddm::DT_U16; break;
    case FDDM_I32: dt = fddm::DT_I32; break;
    case FDDM_U32: dt = fddm::DT_U32; break;
    case FDDM_F32: dt = fddm::DT_F32; break;
    case FDDM_F64: dt = fddm::DT_F64; break;
    default: return fddm::fail_with(FDDM_ERR_INVALID, "unsupported input dtype code " + std::to_string(dtype));
  }
  fddm::DdmRequest r;
  r.mode = fddm::MODE_FFT;
  r.precision = precision;
  r.img = d_img_seq;
  r.dtype = dt;
  r.T = (int64_t)length; r.H = (int64_t)height; r.W = (int64_t)width;
  r.lags.assign(lags, lags + nlags);
  r.nx = (int64_t)nx; r.ny = (int64_t)ny; r.nt = (int64_t)nt;
  r.window = d_window;
  r.out = d_out;
  r.inline_tables = true;
  r.max_work = kNoAllocScratchBytes;
  std::string err;
  fddm::WorkLayout L;
  if (!fddm::plan_layout(r, L, err)) {
    if (L.over_max_work)
      return fddm::fail_with(FDDM_ERR_NOMEM, "the static scratch of fddm_b200_ddm_fft_noalloc is too small: " + err);
    return fddm::fail_with(FDDM_ERR_UNSUPPORTED, err);
  }
  void* scratch = nullptr;
  const int rc0 = scratch_address(&scratch);
  if (rc0 != FDDM_OK) return rc0;
  r.work = scratch;
  r.work_bytes = kNoAllocScratchBytes;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc;
  switch (precision) {
    case FDDM_PREC_FF: rc = fddm::run_ddm_ff(r, st, err); break;
    case FDDM_PREC_F64: rc = fddm::run_ddm_f64(r, st, err); break;
    default: rc = fddm::run_ddm_f32(r, st, err); break;
  }
  if (rc != 0) return fddm::fail_with(rc, err);
  return FDDM_OK;
}
