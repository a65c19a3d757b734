// Multithreaded reader of grayscale TIFF stacks into caller memory (typically
// page-locked, so that the frames go on to the device without another copy).
//
// Replaces the image ingest of the reference (src/python/utils.py:23-258,
// which reads through tifffile and scikit-image): pages (IFDs) of classic or
// BigTIFF files, little or big endian, one sample per pixel, 8/16/32/64-bit
// unsigned, signed or floating-point samples, in strips, uncompressed
// (compression 1), PackBits (32773) or LZW (5, with or without horizontal
// predictor 2).  Uncompressed strips are read with pread straight into the
// destination; pages are spread over threads.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdint>
#include <cstring>
#include <fcntl.h>
#include <set>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace {

struct Page {
  uint64_t width = 0, height = 0;
  int bits = 0, format = 1, compression = 1, predictor = 1, spp = 1, planar = 1;
  uint64_t rows_per_strip = 0;
  std::vector<uint64_t> offsets, counts;
};

struct Tiff {
  int fd = -1;
  bool swap = false, big = false;
  std::vector<Page> pages;
  std::string err;
  ~Tiff() {
    if (fd >= 0) ::close(fd);
  }
  // thread-safe (pread); the message goes to `e`
  bool read_at(uint64_t off, void* dst, size_t n, std::string& e) const {
    unsigned char* d = static_cast<unsigned char*>(dst);
    while (n > 0) {
      const ssize_t r = ::pread(fd, d, n, (off_t)off);
      if (r < 0 && errno == EINTR) continue;
      if (r <= 0) {
        e = r == 0 ? "unexpected end of file" : std::string("read failed: ") + std::strerror(errno);
        return false;
      }
      d += r;
      off += (uint64_t)r;
      n -= (size_t)r;
    }
    return true;
  }
  uint64_t get(const unsigned char* p, int n) const {  // unsigned integer of n bytes in file order
    uint64_t v = 0;
    if (!swap) {
      for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    } else {
      for (int i = 0; i < n; ++i) v = (v << 8) | p[i];
    }
    return v;
  }
};

bool host_little() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

int type_size(int t) {
  switch (t) {
    case 1: case 2: case 6: case 7: return 1;  // BYTE ASCII SBYTE UNDEFINED
    case 3: case 8: return 2;                  // SHORT SSHORT
    case 4: case 9: case 11: case 13: return 4;  // LONG SLONG FLOAT IFD
    case 5: case 10: case 12: case 16: case 17: case 18: return 8;  // RATIONAL DOUBLE LONG8 SLONG8 IFD8
    default: return 0;
  }
}

// Values of one IFD entry as unsigned integers (offsets, counts, sizes).
bool entry_values(Tiff& t, const unsigned char* e, std::vector<uint64_t>& out) {
  const int type = (int)t.get(e + 2, 2);
  const uint64_t count = t.big ? t.get(e + 4, 8) : t.get(e + 4, 4);
  const int ts = type_size(type);
  if (ts == 0 || (type != 1 && type != 3 && type != 4 && type != 16 && type != 13 && type != 18)) {
    out.clear();
    return true;  // not an integer tag this reader needs
  }
  if (count > (1ull << 28)) {
    t.err = "implausible tag value count (corrupted file?)";
    return false;
  }
  const uint64_t bytes = count * (uint64_t)ts;
  const int inl = t.big ? 8 : 4;
  std::vector<unsigned char> buf(bytes);
  if (bytes <= (uint64_t)inl) {
    std::memcpy(buf.data(), e + (t.big ? 12 : 8), bytes);
  } else {
    const uint64_t off = t.big ? t.get(e + 12, 8) : t.get(e + 8, 4);
    if (!t.read_at(off, buf.data(), bytes, t.err)) return false;
  }
  out.resize(count);
  for (uint64_t i = 0; i < count; ++i) out[i] = t.get(buf.data() + i * ts, ts);
  return true;
}

bool open_tiff(const char* path, Tiff& t) {
  t.fd = ::open(path, O_RDONLY);
  if (t.fd < 0) {
    t.err = std::string("cannot open ") + path + ": " + std::strerror(errno);
    return false;
  }
  unsigned char h[16];
  if (!t.read_at(0, h, 8, t.err)) return false;
  if (h[0] == 'I' && h[1] == 'I') t.swap = !host_little();
  else if (h[0] == 'M' && h[1] == 'M') t.swap = host_little();
  else {
    t.err = std::string(path) + " is not a TIFF file";
    return false;
  }
  const uint64_t magic = t.get(h + 2, 2);
  uint64_t ifd;
  if (magic == 42) {
    ifd = t.get(h + 4, 4);
  } else if (magic == 43) {
    t.big = true;
    if (!t.read_at(0, h, 16, t.err)) return false;
    ifd = t.get(h + 8, 8);
  } else {
    t.err = std::string(path) + " is not a TIFF file";
    return false;
  }
  const int es = t.big ? 20 : 12, cs = t.big ? 8 : 2, ns = t.big ? 8 : 4;
  std::vector<uint64_t> v;
  std::set<uint64_t> seen;
  while (ifd != 0) {
    if (!seen.insert(ifd).second) {
      t.err = "IFD chain loops (corrupted file?)";
      return false;
    }
    unsigned char cnt[8];
    if (!t.read_at(ifd, cnt, cs, t.err)) return false;
    const uint64_t n = t.get(cnt, cs);
    if (n > 65535) {
      t.err = "implausible IFD entry count (corrupted file?)";
      return false;
    }
    std::vector<unsigned char> ents(n * es + ns);
    if (!t.read_at(ifd + cs, ents.data(), ents.size(), t.err)) return false;
    Page p;
    for (uint64_t i = 0; i < n; ++i) {
      const unsigned char* e = ents.data() + i * es;
      const int tag = (int)t.get(e, 2);
      if (!entry_values(t, e, v)) return false;
      if (v.empty()) continue;
      switch (tag) {
        case 256: p.width = v[0]; break;
        case 257: p.height = v[0]; break;
        case 258: p.bits = (int)v[0]; break;
        case 259: p.compression = (int)v[0]; break;
        case 273: p.offsets = v; break;
        case 277: p.spp = (int)v[0]; break;
        case 278: p.rows_per_strip = v[0]; break;
        case 279: p.counts = v; break;
        case 284: p.planar = (int)v[0]; break;
        case 317: p.predictor = (int)v[0]; break;
        case 339: p.format = (int)v[0]; break;
        default: break;
      }
    }
    if (p.rows_per_strip == 0 || p.rows_per_strip > p.height) p.rows_per_strip = p.height;
    t.pages.push_back(std::move(p));
    ifd = t.get(ents.data() + n * es, ns);
  }
  if (t.pages.empty()) {
    t.err = std::string(path) + " has no pages";
    return false;
  }
  return true;
}

// FDDM dtype code of a page, or -1.
int page_dtype(const Page& p) {
  if (p.format == 3) return p.bits == 32 ? FDDM_F32 : p.bits == 64 ? FDDM_F64 : -1;
  const bool sgn = p.format == 2;
  switch (p.bits) {
    case 8: return sgn ? -1 : FDDM_U8;
    case 16: return sgn ? FDDM_I16 : FDDM_U16;
    case 32: return sgn ? FDDM_I32 : FDDM_U32;
    case 64: return sgn ? FDDM_I64 : FDDM_U64;
    default: return -1;
  }
}

bool check_page(const Page& p, std::string& err) {
  if (p.spp != 1) { err = "only one sample per pixel (grayscale) is supported"; return false; }
  if (p.width == 0 || p.height == 0) { err = "page without width or height"; return false; }
  if (page_dtype(p) < 0) { err = "unsupported sample type (" + std::to_string(p.bits) + " bits, format " + std::to_string(p.format) + ")"; return false; }
  if (p.compression != 1 && p.compression != 5 && p.compression != 32773) {
    err = "compression " + std::to_string(p.compression) + " is not supported (uncompressed, LZW and PackBits are)";
    return false;
  }
  if (p.predictor != 1 && !(p.predictor == 2 && p.format != 3)) { err = "predictor " + std::to_string(p.predictor) + " is not supported"; return false; }
  const uint64_t nstrips = (p.height + p.rows_per_strip - 1) / p.rows_per_strip;
  if (p.offsets.size() < nstrips || (p.compression != 1 && p.counts.size() < nstrips)) { err = "missing strip offsets or byte counts (tiled TIFFs are not supported)"; return false; }
  return true;
}

bool unpackbits(const unsigned char* s, size_t n, unsigned char* d, size_t want) {
  size_t i = 0, o = 0;
  while (i < n && o < want) {
    const int c = (signed char)s[i++];
    if (c >= 0) {
      const size_t k = (size_t)c + 1;
      if (i + k > n || o + k > want) return false;
      std::memcpy(d + o, s + i, k);
      i += k;
      o += k;
    } else if (c != -128) {
      const size_t k = (size_t)(1 - c);
      if (i >= n || o + k > want) return false;
      std::memset(d + o, s[i++], k);
      o += k;
    }
  }
  return o == want;
}

// TIFF LZW (variable code width 9..12 bits, MSB first, codes 256 clear / 257 end).
bool unlzw(const unsigned char* s, size_t n, unsigned char* d, size_t want) {
  std::vector<uint32_t> prefix(4096), first(4096);
  std::vector<uint16_t> len(4096);
  std::vector<unsigned char> suffix(4096), stack(4096);
  size_t o = 0;
  uint64_t bitpos = 0;
  const uint64_t nbits = (uint64_t)n * 8;
  int width = 9, next = 258;
  int prev = -1;
  auto read_code = [&]() -> int {
    if (bitpos + width > nbits) return 257;
    uint32_t v = 0;
    for (int b = 0; b < width; ++b, ++bitpos) v = (v << 1) | ((s[bitpos >> 3] >> (7 - (bitpos & 7))) & 1);
    return (int)v;
  };
  for (int c = 0; c < 256; ++c) {
    suffix[c] = (unsigned char)c;
    first[c] = (uint32_t)c;
    len[c] = 1;
  }
  auto emit = [&](int code) -> bool {  // write the string of `code`
    const int L = len[code];
    if (o + L > want) return false;
    int c = code;
    for (int k = L - 1; k >= 0; --k) {
      d[o + k] = suffix[c];
      c = (int)prefix[c];
    }
    o += L;
    return true;
  };
  while (o < want) {
    const int code = read_code();
    if (code == 257) break;
    if (code == 256) {
      width = 9;
      next = 258;
      prev = -1;
      continue;
    }
    if (prev < 0) {
      if (code > 255) return false;
      if (!emit(code)) return false;
      prev = code;
    } else {
      int add_first;
      if (code < next) {
        if (code > 255 && len[code] == 0) return false;
        add_first = (int)first[code];
      } else if (code == next) {
        add_first = (int)first[prev];
      } else {
        return false;
      }
      if (next < 4096) {
        prefix[next] = (uint32_t)prev;
        suffix[next] = (unsigned char)add_first;
        first[next] = first[prev];
        len[next] = (uint16_t)(len[prev] + 1);
        ++next;
      }
      if (!emit(code)) return false;
      prev = code;
    }
    // the early change of TIFF LZW: widen one code before the table fills
    if (next + 1 >= (1 << width) && width < 12) ++width;
  }
  return o == want;
}

void swap_bytes(unsigned char* p, size_t n, int bytes) {
  if (bytes == 1) return;
  for (size_t i = 0; i + bytes <= n; i += bytes)
    for (int a = 0, b = bytes - 1; a < b; ++a, --b) std::swap(p[i + a], p[i + b]);
}

void undo_predictor(unsigned char* p, uint64_t rows, uint64_t width, int bytes) {
  for (uint64_t r = 0; r < rows; ++r) {
    unsigned char* row = p + r * width * bytes;
    switch (bytes) {
      case 1: for (uint64_t x = 1; x < width; ++x) row[x] = (unsigned char)(row[x] + row[x - 1]); break;
      case 2: {
        uint16_t* q = reinterpret_cast<uint16_t*>(row);
        for (uint64_t x = 1; x < width; ++x) q[x] = (uint16_t)(q[x] + q[x - 1]);
        break;
      }
      case 4: {
        uint32_t* q = reinterpret_cast<uint32_t*>(row);
        for (uint64_t x = 1; x < width; ++x) q[x] = q[x] + q[x - 1];
        break;
      }
      default: {
        uint64_t* q = reinterpret_cast<uint64_t*>(row);
        for (uint64_t x = 1; x < width; ++x) q[x] = q[x] + q[x - 1];
        break;
      }
    }
  }
}

bool read_page(const Tiff& t, const Page& p, unsigned char* dst, std::string& err) {
  const int bytes = p.bits / 8;
  const uint64_t row_bytes = p.width * (uint64_t)bytes;
  const uint64_t nstrips = (p.height + p.rows_per_strip - 1) / p.rows_per_strip;
  std::vector<unsigned char> comp;
  for (uint64_t s = 0; s < nstrips; ++s) {
    const uint64_t rows = std::min(p.rows_per_strip, p.height - s * p.rows_per_strip);
    unsigned char* out = dst + s * p.rows_per_strip * row_bytes;
    const size_t want = (size_t)(rows * row_bytes);
    if (p.compression == 1) {
      if (!t.read_at(p.offsets[s], out, want, err)) return false;
    } else {
      comp.resize(p.counts[s]);
      if (!t.read_at(p.offsets[s], comp.data(), comp.size(), err)) return false;
      const bool ok = p.compression == 5 ? unlzw(comp.data(), comp.size(), out, want)
                                         : unpackbits(comp.data(), comp.size(), out, want);
      if (!ok) { err = "corrupted compressed strip"; return false; }
    }
    if (t.swap) swap_bytes(out, want, bytes);
    if (p.predictor == 2) undo_predictor(out, rows, p.width, bytes);
  }
  return true;
}

}  // namespace

extern "C" int fddm_b200_tiff_info(const char* path, uint64_t* npages, uint64_t* height, uint64_t* width,
                                   int* dtype) {
  fddm::set_last_error("");
  if (!path || !npages || !height || !width || !dtype) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  Tiff t;
  if (!open_tiff(path, t)) return fddm::fail_with(FDDM_ERR_INVALID, t.err);
  const Page& p0 = t.pages[0];
  std::string err;
  if (!check_page(p0, err)) return fddm::fail_with(FDDM_ERR_UNSUPPORTED, std::string(path) + ": " + err);
  for (const Page& p : t.pages)
    if (p.width != p0.width || p.height != p0.height || page_dtype(p) != page_dtype(p0))
      return fddm::fail_with(FDDM_ERR_UNSUPPORTED, std::string(path) + ": pages differ in size or sample type");
  *npages = t.pages.size();
  *height = p0.height;
  *width = p0.width;
  *dtype = page_dtype(p0);
  return FDDM_OK;
}

extern "C" int fddm_b200_tiff_read(const char* path, const uint64_t* pages, uint64_t npages, void* dst,
                                   int nthreads) {
  fddm::set_last_error("");
  if (!path || !dst || (npages && !pages)) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  Tiff t;
  if (!open_tiff(path, t)) return fddm::fail_with(FDDM_ERR_INVALID, t.err);
  const Page& p0 = t.pages[0];
  std::string err;
  for (uint64_t i = 0; i < npages; ++i) {
    if (pages[i] >= t.pages.size())
      return fddm::fail_with(FDDM_ERR_INVALID, "page " + std::to_string(pages[i]) + " out of range (" +
                                                   std::to_string(t.pages.size()) + " pages)");
    const Page& p = t.pages[pages[i]];
    if (!check_page(p, err)) return fddm::fail_with(FDDM_ERR_UNSUPPORTED, std::string(path) + ": " + err);
    if (p.width != p0.width || p.height != p0.height || page_dtype(p) != page_dtype(p0))
      return fddm::fail_with(FDDM_ERR_UNSUPPORTED, std::string(path) + ": pages differ in size or sample type");
  }
  const size_t page_bytes = (size_t)(p0.width * p0.height * (uint64_t)(p0.bits / 8));
  const int nt = (int)std::max<uint64_t>(1, std::min<uint64_t>(npages, (uint64_t)std::max(1, nthreads)));
  std::atomic<uint64_t> next{0};
  std::atomic<bool> failed{false};
  std::vector<std::string> errs(nt);
  auto work = [&](int w) {
    for (uint64_t i = next++; i < npages && !failed; i = next++) {
      if (!read_page(t, t.pages[pages[i]], static_cast<unsigned char*>(dst) + i * page_bytes, errs[w])) failed = true;
    }
  };
  std::vector<std::thread> th;
  for (int w = 1; w < nt; ++w) th.emplace_back(work, w);
  work(0);
  for (auto& x : th) x.join();
  if (failed) {
    for (auto& e : errs)
      if (!e.empty()) return fddm::fail_with(FDDM_ERR_INVALID, std::string(path) + ": " + e);
    return fddm::fail_with(FDDM_ERR_INVALID, std::string(path) + ": read failed");
  }
  return FDDM_OK;
}
