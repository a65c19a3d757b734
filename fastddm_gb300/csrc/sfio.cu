// Writer of image structure function files (.sf.ddm), the binary format of the
// reference's SFWriter (src/python/imagestructurefunction.py:409-627, header
// and offsets in src/python/_io_common.py:16-17):
//
//   bytes 0-1   "LL" (little-endian host) or "BB"
//   bytes 2-3   file identifier 73, uint16
//   bytes 4-5   version (0, 3), two uint8
//   byte  6     dtype 'd'
//   bytes 7-54  length (lags), height (ny), width (nx/2 + 1), extra slices,
//               full width, full height: six uint64
//   up to 64    zero padding
//   then        _data (length + extra, height, width) float64, C order;
//               kx (width), ky (height), tau (length), pixel_size, delta_t;
//               seven uint64 byte offsets in the order extra, delta_t,
//               pixel_size, tau, ky, kx, data (the reader starts from the end).
//
// The data block may live in device memory: it is then streamed to the file
// through two pinned staging buffers, the device-to-host copy of one chunk
// overlapping the write of the previous one, so the host never holds the
// whole array.
#include <algorithm>
#include <cerrno>
#include <cstring>
#include <fcntl.h>
#include <mutex>
#include <string>
#include <unistd.h>
#include <vector>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace {

constexpr size_t kHeadBytes = 64;            // HEAD_BYTE_LEN of the reference's writers
constexpr size_t kStageBytes = 32ull << 20;  // one staging buffer (two per device)

bool host_little_endian() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

struct File {
  int fd = -1;
  std::string err;
  explicit File(const char* path) {
    fd = ::open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) err = std::string("cannot open ") + path + ": " + std::strerror(errno);
  }
  ~File() {
    if (fd >= 0) ::close(fd);
  }
  bool write_all(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    while (n > 0) {
      const ssize_t w = ::write(fd, c, n);
      if (w < 0) {
        if (errno == EINTR) continue;
        err = std::string("write failed: ") + std::strerror(errno);
        return false;
      }
      c += w;
      n -= (size_t)w;
    }
    return true;
  }
  bool finish() {
    const int rc = ::close(fd);
    fd = -1;
    if (rc != 0) {
      err = std::string("close failed: ") + std::strerror(errno);
      return false;
    }
    return true;
  }
};

// Per-device staging: two pinned buffers, a copy stream and two events
// (allocated on the first device-sourced write, kept until exit).
struct Stage {
  void* buf[2] = {nullptr, nullptr};
  cudaStream_t stream = nullptr;
  cudaEvent_t ready[2] = {nullptr, nullptr};
  cudaEvent_t start = nullptr;
};

Stage* stage_for_device(std::string& err) {
  static std::mutex mu;
  static std::vector<Stage*> stages;
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) {
    err = cudaGetErrorString(ce);
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if ((int)stages.size() <= dev) stages.resize(dev + 1, nullptr);
  if (stages[dev]) return stages[dev];
  Stage* s = new Stage();
  if ((ce = cudaHostAlloc(&s->buf[0], kStageBytes, cudaHostAllocDefault)) != cudaSuccess ||
      (ce = cudaHostAlloc(&s->buf[1], kStageBytes, cudaHostAllocDefault)) != cudaSuccess ||
      (ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (ce = cudaEventCreateWithFlags(&s->ready[0], cudaEventDisableTiming)) != cudaSuccess ||
      (ce = cudaEventCreateWithFlags(&s->ready[1], cudaEventDisableTiming)) != cudaSuccess ||
      (ce = cudaEventCreateWithFlags(&s->start, cudaEventDisableTiming)) != cudaSuccess) {
    err = cudaGetErrorString(ce);
    if (s->buf[0]) cudaFreeHost(s->buf[0]);
    if (s->buf[1]) cudaFreeHost(s->buf[1]);
    delete s;
    return nullptr;
  }
  stages[dev] = s;
  return s;
}

// Stream `bytes` of device memory to the file in chunks, ordered after the
// work already queued on `producer`.
bool stream_device(File& f, const unsigned char* src, size_t bytes, cudaStream_t producer, std::string& err) {
  Stage* s = stage_for_device(err);
  if (!s) return false;
  cudaError_t ce;
  if ((ce = cudaEventRecord(s->start, producer)) != cudaSuccess ||
      (ce = cudaStreamWaitEvent(s->stream, s->start, 0)) != cudaSuccess) {
    err = cudaGetErrorString(ce);
    return false;
  }
  const size_t nchunks = (bytes + kStageBytes - 1) / kStageBytes;
  auto issue = [&](size_t i) -> bool {
    const size_t off = i * kStageBytes, n = std::min(kStageBytes, bytes - off);
    if ((ce = cudaMemcpyAsync(s->buf[i & 1], src + off, n, cudaMemcpyDeviceToHost, s->stream)) != cudaSuccess ||
        (ce = cudaEventRecord(s->ready[i & 1], s->stream)) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return false;
    }
    return true;
  };
  if (nchunks > 0 && !issue(0)) return false;
  for (size_t i = 0; i < nchunks; ++i) {
    // buffer (i + 1) & 1 held chunk i - 1, written in the previous iteration
    if (i + 1 < nchunks && !issue(i + 1)) return false;
    if ((ce = cudaEventSynchronize(s->ready[i & 1])) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return false;
    }
    const size_t off = i * kStageBytes, n = std::min(kStageBytes, bytes - off);
    if (!f.write_all(s->buf[i & 1], n)) {
      err = f.err;
      cudaStreamSynchronize(s->stream);  // no copy may still target the staging buffers
      return false;
    }
  }
  return true;
}

}  // namespace

extern "C" int fddm_b200_sf_write(const char* path, const double* data, int data_on_device, uint64_t length,
                                  uint64_t height, uint64_t width, uint64_t extra, uint64_t full_width,
                                  uint64_t full_height, const double* kx, const double* ky, const double* tau,
                                  double pixel_size, double delta_t, void* stream) {
  fddm::set_last_error("");
  if (!path || !data || (width && !kx) || (height && !ky) || (length && !tau))
    return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  const size_t es = sizeof(double);
  const uint64_t nrows = length + extra;
  if (height && width && nrows > (~0ull / es) / height / width) return fddm::fail_with(FDDM_ERR_INVALID, "file too large");
  const size_t data_bytes = (size_t)(nrows * height * width) * es;

  File f(path);
  if (f.fd < 0) return fddm::fail_with(FDDM_ERR_INVALID, f.err);

  unsigned char head[kHeadBytes];
  std::memset(head, 0, sizeof(head));
  const bool le = host_little_endian();
  head[0] = head[1] = le ? 'L' : 'B';
  const uint16_t id = 73;
  std::memcpy(head + 2, &id, 2);
  head[4] = 0;  // version (0, 3)
  head[5] = 3;
  head[6] = 'd';
  const uint64_t dims[6] = {length, height, width, extra, full_width, full_height};
  std::memcpy(head + 7, dims, sizeof(dims));
  if (!f.write_all(head, sizeof(head))) return fddm::fail_with(FDDM_ERR_INVALID, f.err);

  if (data_on_device) {
    std::string err;
    if (!stream_device(f, reinterpret_cast<const unsigned char*>(data), data_bytes,
                       static_cast<cudaStream_t>(stream), err))
      return fddm::fail_with(FDDM_ERR_CUDA, err);
  } else if (!f.write_all(data, data_bytes)) {
    return fddm::fail_with(FDDM_ERR_INVALID, f.err);
  }

  const uint64_t data_off = kHeadBytes;
  const uint64_t extra_off = data_off + length * height * width * es;
  const uint64_t kx_off = extra_off + extra * height * width * es;
  const uint64_t ky_off = kx_off + width * es;
  const uint64_t tau_off = ky_off + height * es;
  const uint64_t ps_off = tau_off + length * es;
  const uint64_t dt_off = ps_off + es;
  const double scalars[2] = {pixel_size, delta_t};
  const uint64_t offs[7] = {extra_off, dt_off, ps_off, tau_off, ky_off, kx_off, data_off};
  if (!f.write_all(kx, width * es) || !f.write_all(ky, height * es) || !f.write_all(tau, length * es) ||
      !f.write_all(scalars, sizeof(scalars)) || !f.write_all(offs, sizeof(offs)) || !f.finish())
    return fddm::fail_with(FDDM_ERR_INVALID, f.err);
  return FDDM_OK;
}
