// FFT plans, twiddle/permutation tables (cached per device) and workspace planning.
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <algorithm>
#include <cstring>
#include "fddm_internal.h"

namespace fddm {

bool make_plan(int n, FftPlan& p) {
  if (n < 1) return false;
  p.n = n;
  p.npass = 0;
  int m = n;
  auto push = [&](int r) -> bool {
    if (p.npass >= kMaxPass) return false;
    p.radix[p.npass++] = r;
    m /= r;
    return true;
  };
  while (m % 8 == 0) if (!push(8)) return false;
  while (m % 4 == 0) if (!push(4)) return false;
  while (m % 2 == 0) if (!push(2)) return false;
  const int odd[] = {3, 5, 7, 11, 13};
  for (int r : odd)
    while (m % r == 0) if (!push(r)) return false;
  if (m != 1) return false;
  int M = n;
  for (int s = 0; s < p.npass; ++s) {
    p.block[s] = M;
    M /= p.radix[s];
  }
  return true;
}

static int perm_of(const FftPlan& p, int k) {
  int pos = 0, rem = k;
  for (int s = 0; s < p.npass; ++s) {
    const int R = p.radix[s];
    const int m = rem % R;
    rem /= R;
    pos += m * (p.block[s] / R);
  }
  return pos;
}

namespace {
struct Entry {
  FftPlan plan;
  void* tw = nullptr;
  int* perm = nullptr;
};
std::mutex g_mu;
std::map<std::tuple<int, int, int>, Entry> g_cache;  // (device, n, kind)
const long double kPi = 3.141592653589793238462643383279502884L;
}  // namespace

bool get_tables(int n, int kind, FftTables& out, std::string& err) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return false; }
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_tuple(dev, n, kind);
  auto it = g_cache.find(key);
  if (it == g_cache.end()) {
    Entry e;
    if (!make_plan(n, e.plan)) {
      err = "length " + std::to_string(n) + " has a prime factor other than 2, 3, 5, 7, 11, 13";
      return false;
    }
    std::vector<int> perm(n);
    for (int k = 0; k < n; ++k) perm[k] = perm_of(e.plan, k);
    const size_t esz = kind == 2 ? 8 : 16;
    std::vector<unsigned char> tw(esz * (size_t)n);
    for (int k = 0; k < n; ++k) {
      // w_n^k = exp(-2 pi i k / n) in extended precision
      const long double ang = -2.0L * kPi * (long double)k / (long double)n;
      const long double c = cosl(ang), s = sinl(ang);
      if (kind == 0) {
        float v[4];
        v[0] = (float)c; v[1] = (float)(c - (long double)v[0]);
        v[2] = (float)s; v[3] = (float)(s - (long double)v[2]);
        memcpy(&tw[esz * k], v, sizeof(v));
      } else if (kind == 1) {
        double v[2] = {(double)c, (double)s};
        memcpy(&tw[esz * k], v, sizeof(v));
      } else {
        float v[2] = {(float)c, (float)s};
        memcpy(&tw[esz * k], v, sizeof(v));
      }
    }
    if ((ce = cudaMalloc(&e.tw, tw.size())) != cudaSuccess ||
        (ce = cudaMalloc(reinterpret_cast<void**>(&e.perm), sizeof(int) * n)) != cudaSuccess ||
        (ce = cudaMemcpy(e.tw, tw.data(), tw.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (ce = cudaMemcpy(e.perm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice)) != cudaSuccess) {
      err = std::string("FFT table upload failed: ") + cudaGetErrorString(ce);
      if (e.tw) cudaFree(e.tw);
      if (e.perm) cudaFree(e.perm);
      return false;
    }
    it = g_cache.emplace(key, e).first;
  }
  out.plan = it->second.plan;
  out.tw = it->second.tw;
  out.perm = it->second.perm;
  return true;
}

size_t spec_elem_bytes(int precision) { return precision == PREC_F32 ? 8 : 16; }

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

bool plan_layout(const DdmRequest& r, WorkLayout& L, std::string& err) {
  if (r.T < 1 || r.H < 1 || r.W < 1) { err = "empty image sequence"; return false; }
  if (r.nx < r.W || r.ny < r.H) { err = "nx, ny must be at least the image width and height"; return false; }
  if (r.T > (1 << 30) || r.nx > (1 << 20) || r.ny > (1 << 20)) { err = "problem too large"; return false; }
  FftPlan p;
  if (!make_plan((int)r.nx, p)) { err = "nx=" + std::to_string(r.nx) + " has a prime factor other than 2, 3, 5, 7, 11, 13"; return false; }
  if (!make_plan((int)r.ny, p)) { err = "ny=" + std::to_string(r.ny) + " has a prime factor other than 2, 3, 5, 7, 11, 13"; return false; }
  if (r.mode == MODE_FFT) {
    if (r.nt < 2 * r.T - 1) { err = "nt must be at least 2*len(img_seq) - 1"; return false; }
    if (!make_plan((int)r.nt, p)) { err = "nt=" + std::to_string(r.nt) + " has a prime factor other than 2, 3, 5, 7, 11, 13"; return false; }
  }
  for (int lag : r.lags)
    if (lag < 0 || lag >= r.T) { err = "lags must lie in [0, len(img_seq) - 1]"; return false; }
  const size_t es = spec_elem_bytes(r.precision);
  const int64_t nkx = r.nx / 2 + 1;
  const size_t Q = (size_t)r.ny * nkx;
  L.Tpad = (int)align_up((size_t)r.T, 64 / es);
  L.Hpad = (int)(2 * ((r.H + 1) / 2));
  // stage 1-2 blocking: ~64 KB of shared memory per CTA
  const size_t target = 64 * 1024;
  L.pairs_per_block = (int)std::max<size_t>(1, std::min<size_t>(target / ((size_t)r.nx * es), (size_t)((r.H + 1) / 2)));
  const int nb = (int)std::max<size_t>(1, target / ((size_t)r.ny * es));
  L.frames_per_block = std::min(nb, 8);
  L.cols_per_block = std::max(1, nb / L.frames_per_block);
  if ((size_t)L.pairs_per_block * r.nx * es > 232448 || (size_t)nb * r.ny * es > 232448) {
    err = "image dimensions too large for the shared-memory FFT";
    return false;
  }
  // frame chunk: keep the row-pass buffer near 128 MB
  const size_t per_frame = (size_t)nkx * L.Hpad * es;
  int chunk = (int)std::max<size_t>(1, (128ull << 20) / per_frame);
  chunk = std::max(L.frames_per_block, chunk / L.frames_per_block * L.frames_per_block);
  chunk = (int)std::min<int64_t>(chunk, (r.T + L.frames_per_block - 1) / L.frames_per_block * L.frames_per_block);
  L.chunk = chunk;
  // temporal kernel shared memory
  const size_t ea = 8;
  const size_t smem_t = r.mode == MODE_FFT ? (size_t)r.nt * es + (size_t)(r.T + 1) * ea + 96 * ea
                                           : (size_t)r.T * es + 96 * ea;
  if (smem_t > 232448) {
    err = "sequence too long for the single-CTA temporal kernel (needs " + std::to_string(smem_t) + " B of shared memory)";
    return false;
  }
  size_t off = 0;
  L.spec_off = off; L.spec_bytes = Q * (size_t)L.Tpad * es; off = align_up(off + L.spec_bytes, 256);
  L.rbuf_off = off; L.rbuf_bytes = (size_t)chunk * per_frame; off = align_up(off + L.rbuf_bytes, 256);
  L.win_off = off; L.win_bytes = r.window ? (size_t)r.H * r.W * (es / 2) : 0; off = align_up(off + L.win_bytes, 256);
  L.lags_off = off; off = align_up(off + r.lags.size() * sizeof(int) + 4, 256);
  L.rcp_off = off; off = align_up(off + r.lags.size() * sizeof(double) + 8, 256);
  L.total = off;
  return true;
}

}  // namespace fddm
