// FFT plans, twiddle/permutation tables (cached per device) and workspace planning.
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <cstdlib>
#include "fddm_internal.h"

namespace fddm {

// Block sizes and shift tables of a plan whose n and radices are set.
static void finish_plan(FftPlan& p) {
  auto lg = [](int v) -> int {
    if (v <= 0 || (v & (v - 1))) return -1;
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
  };
  p.lgn = lg(p.n);
  for (int s = 0; s < kMaxPass; ++s) p.ptw[s] = nullptr;
  int M = p.n;
  for (int s = 0; s < p.npass; ++s) {
    p.block[s] = M;
    p.lgstride[s] = lg(M / p.radix[s]);
    p.lgbpf[s] = lg(p.n / p.radix[s]);
    M /= p.radix[s];
  }
}

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
  finish_plan(p);
  return true;
}

bool plan_from_radices(int n, const int* radices, int npass, FftPlan& p) {
  if (npass < 1 || npass > kMaxPass) return false;
  long long prod = 1;
  for (int s = 0; s < npass; ++s) prod *= radices[s];
  if (prod != n) return false;
  p.n = n;
  p.npass = npass;
  for (int s = 0; s < npass; ++s) p.radix[s] = radices[s];
  finish_plan(p);
  return true;
}

bool half_plan(const FftPlan& p, FftPlan& h) {
  if (p.npass < 1 || p.n % 2 || p.radix[0] % 2) return false;
  h.n = p.n / 2;
  h.npass = 0;
  if (p.radix[0] > 2) h.radix[h.npass++] = p.radix[0] / 2;
  for (int s = 1; s < p.npass; ++s) h.radix[h.npass++] = p.radix[s];
  finish_plan(h);
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
  int* iperm = nullptr;
};
std::mutex g_mu;
std::map<std::tuple<int, int, int>, Entry> g_cache;  // (device, n, kind)
std::mutex g_host_mu;
std::map<std::pair<int, int>, HostTables> g_host_cache;  // (n, kind)
const long double kPi = 3.141592653589793238462643383279502884L;

// Plan, permutations and twiddles w_n^k = exp(-2 pi i k / n) (extended precision).
bool build_tables(int n, int kind, FftPlan& plan, std::vector<unsigned char>& tw, std::vector<int>& perm,
                  std::vector<int>& iperm, std::string& err) {
  if (!make_plan(n, plan)) {
    err = "length " + std::to_string(n) + " has a prime factor other than 2, 3, 5, 7, 11, 13";
    return false;
  }
  perm.assign(n, 0);
  iperm.assign(n, 0);
  for (int k = 0; k < n; ++k) perm[k] = perm_of(plan, k);
  for (int k = 0; k < n; ++k) iperm[perm[k]] = k;
  const size_t esz = kind == 2 ? 8 : 16;
  tw.assign(esz * (size_t)n, 0);
  for (int k = 0; k < n; ++k) {
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
  return true;
}
}  // namespace

bool host_tables(int n, int kind, const HostTables*& out, std::string& err) {
  std::lock_guard<std::mutex> lk(g_host_mu);
  auto key = std::make_pair(n, kind);
  auto it = g_host_cache.find(key);
  if (it == g_host_cache.end()) {
    HostTables h;
    if (!build_tables(n, kind, h.plan, h.tw, h.perm, h.iperm, err)) return false;
    it = g_host_cache.emplace(key, std::move(h)).first;
  }
  out = &it->second;
  return true;
}

size_t inline_table_bytes(int n, int kind) {
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  return up((size_t)n * (kind == 2 ? 8 : 16)) + 2 * up((size_t)n * sizeof(int)) + pass_tables_bound(n, kind);
}

namespace {
std::mutex g_pass_mu;
std::map<std::tuple<int, int, int, int>, void*> g_pass_cache;  // (device, M, R, kind) -> device table
std::mutex g_hpass_mu;
std::map<std::tuple<int, int, int>, std::vector<unsigned char>> g_hpass_cache;  // (M, R, kind) -> host table

// w_M^(j m), rows m = 1..R-1, columns j = 0..M/R-1, extended precision, in the tier's format
const std::vector<unsigned char>& host_pass_table(int M, int R, int kind) {
  std::lock_guard<std::mutex> lk(g_hpass_mu);
  auto key = std::make_tuple(M, R, kind);
  auto it = g_hpass_cache.find(key);
  if (it != g_hpass_cache.end()) return it->second;
  const int stride = M / R;
  const size_t esz = kind == 2 ? 8 : 16;
  std::vector<unsigned char> out(esz * (size_t)(R - 1) * stride, 0);
  for (int m = 1; m < R; ++m)
    for (int j = 0; j < stride; ++j) {
      const long double ang = -2.0L * kPi * (long double)(((long long)j * m) % M) / (long double)M;
      const long double c = cosl(ang), sn = sinl(ang);
      unsigned char* dst = &out[esz * ((size_t)(m - 1) * stride + j)];
      if (kind == 0) {
        float v[4];
        v[0] = (float)c; v[1] = (float)(c - (long double)v[0]);
        v[2] = (float)sn; v[3] = (float)(sn - (long double)v[2]);
        memcpy(dst, v, sizeof(v));
      } else if (kind == 1) {
        double v[2] = {(double)c, (double)sn};
        memcpy(dst, v, sizeof(v));
      } else {
        float v[2] = {(float)c, (float)sn};
        memcpy(dst, v, sizeof(v));
      }
    }
  return g_hpass_cache.emplace(key, std::move(out)).first->second;
}
size_t up256(size_t x) { return (x + 255) / 256 * 256; }
}  // namespace

size_t pass_tables_bound(int n, int kind) {
  // a plan's tables hold sum_s (R_s - 1) M_s / R_s < 2 n entries
  return up256(2 * (size_t)n * (kind == 2 ? 8 : 16)) + (size_t)kMaxPass * 256;
}

bool attach_pass_tables(FftPlan& p, int kind, std::string& err) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return false; }
  for (int s = 0; s < p.npass; ++s) {
    const int M = p.block[s], R = p.radix[s];
    p.ptw[s] = nullptr;
    // stride-1 passes take no twiddles, except the first pass of a single-pass
    // plan: the padded first pass reads its (all-ones) table unconditionally
    if (M / R <= 1 && s > 0) continue;
    const auto& h = host_pass_table(M, R, kind);
    std::lock_guard<std::mutex> lk(g_pass_mu);
    auto key = std::make_tuple(dev, M, R, kind);
    auto it = g_pass_cache.find(key);
    if (it == g_pass_cache.end()) {
      void* d = nullptr;
      if ((ce = cudaMalloc(&d, h.size())) != cudaSuccess ||
          (ce = cudaMemcpy(d, h.data(), h.size(), cudaMemcpyHostToDevice)) != cudaSuccess) {
        if (d) cudaFree(d);
        err = std::string("FFT pass table upload failed: ") + cudaGetErrorString(ce);
        return false;
      }
      it = g_pass_cache.emplace(key, d).first;
    }
    p.ptw[s] = it->second;
  }
  return true;
}

bool upload_pass_tables(FftPlan& p, int kind, unsigned char* dst, size_t room, cudaStream_t st, std::string& err) {
  size_t used = 0;
  for (int s = 0; s < p.npass; ++s) {
    const int M = p.block[s], R = p.radix[s];
    p.ptw[s] = nullptr;
    if (M / R <= 1 && s > 0) continue;  // as in attach_pass_tables
    const auto& h = host_pass_table(M, R, kind);  // cached: stays valid for the asynchronous copy
    if (used + up256(h.size()) > room) {
      err = "workspace table area too small for the pass twiddle tables";
      return false;
    }
    const cudaError_t ce = cudaMemcpyAsync(dst + used, h.data(), h.size(), cudaMemcpyHostToDevice, st);
    if (ce != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return false;
    }
    p.ptw[s] = dst + used;
    used += up256(h.size());
  }
  return true;
}

bool get_tables(int n, int kind, FftTables& out, std::string& err) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return false; }
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_tuple(dev, n, kind);
  auto it = g_cache.find(key);
  if (it == g_cache.end()) {
    Entry e;
    std::vector<unsigned char> tw;
    std::vector<int> perm, iperm;
    if (!build_tables(n, kind, e.plan, tw, perm, iperm, err)) return false;
    if ((ce = cudaMalloc(&e.tw, tw.size())) != cudaSuccess ||
        (ce = cudaMalloc(reinterpret_cast<void**>(&e.perm), sizeof(int) * n)) != cudaSuccess ||
        (ce = cudaMalloc(reinterpret_cast<void**>(&e.iperm), sizeof(int) * n)) != cudaSuccess ||
        (ce = cudaMemcpy(e.tw, tw.data(), tw.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (ce = cudaMemcpy(e.perm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (ce = cudaMemcpy(e.iperm, iperm.data(), sizeof(int) * n, cudaMemcpyHostToDevice)) != cudaSuccess) {
      err = std::string("FFT table upload failed: ") + cudaGetErrorString(ce);
      if (e.tw) cudaFree(e.tw);
      if (e.perm) cudaFree(e.perm);
      if (e.iperm) cudaFree(e.iperm);
      return false;
    }
    it = g_cache.emplace(key, e).first;
  }
  out.plan = it->second.plan;
  out.tw = it->second.tw;
  out.perm = it->second.perm;
  out.iperm = it->second.iperm;
  return true;
}

// Issue cost per point of one in-place pass of each radix in float-float
// arithmetic (instruction counts of the butterfly plus its twiddles).
static double pass_cost(int r) {
  switch (r) {
    case 8: return 110.0;
    case 4: return 80.0;
    case 2: return 45.0;
    case 3: return 72.0;
    case 5: return 140.0;
    case 7: return 190.0;
    case 11: return 300.0;
    default: return 360.0;
  }
}

// First pass of a zero-padded input: the upper half of every butterfly is
// zero (the add/sub stage of radix 8 and 4 halves, radix 2 is twiddles only).
static double padded_cost(int r) {
  switch (r) {
    case 8: return 95.0;
    case 4: return 55.0;
    case 2: return 25.0;
    default: return pass_cost(r);
  }
}

// Cheapest plan of the temporal transforms for length n: the first radix
// (even, run as the padded pass) is chosen by cost, the others follow
// make_plan's order; the half-length transform uses half_plan of it.
static double temporal_plan_cost(int n, FftPlan* out) {
  double best = 1e300;
  for (int r0 : {8, 4, 2}) {
    if (n % r0) continue;
    FftPlan rest, cand, h;
    if (!make_plan(n / r0, rest) || rest.npass + 1 > kMaxPass) continue;
    cand.n = n;
    cand.npass = 0;
    cand.radix[cand.npass++] = r0;
    for (int s = 0; s < rest.npass; ++s) cand.radix[cand.npass++] = rest.radix[s];
    finish_plan(cand);
    if (!half_plan(cand, h)) continue;
    double c = padded_cost(r0) * n;
    for (int s = 1; s < cand.npass; ++s) c += pass_cost(cand.radix[s]) * n;
    for (int s = 0; s < h.npass; ++s) c += pass_cost(h.radix[s]) * h.n;
    if (c < best) {
      best = c;
      if (out) *out = cand;
    }
  }
  return best;
}
static double temporal_cost(int n) { return temporal_plan_cost(n, nullptr); }

bool temporal_plan(int n, FftPlan& p) { return temporal_plan_cost(n, &p) < 1e300; }

int choose_temporal_length(int64_t T) {
  const int64_t lo = std::max<int64_t>(2, 2 * T - 1);
  int64_t p2 = 1;
  while (p2 < lo) p2 <<= 1;
  int best = (int)p2;
  double best_cost = temporal_cost(best);
  for (int64_t n = lo; n < p2; ++n) {
    if (n % 2) continue;
    const double c = temporal_cost((int)n);
    if (c < best_cost) {
      best_cost = c;
      best = (int)n;
    }
  }
  return best;
}

static size_t round_to(size_t x, size_t a) { return (x + a - 1) / a * a; }

size_t temporal_fft_smem(int T, int N, int nlags, size_t es, size_t ea, bool need_in_smem) {
  const size_t g = 128 / es;  // swizzle group (elements)
  // transform buffer: the length-N transform, or the half-length transform
  // below the next series prefetched from offset round_to(N / 2, g)
  const size_t nbuf = std::max(round_to(N, g), round_to(N / 2, g) + round_to(T, g));
  size_t b = (nbuf + 64) * es + 96 * ea + 2 * (size_t)(T + 1) * sizeof(short);
  // need[] and the per-lag tables (w^tau, 1/(T - tau), tau)
  if (need_in_smem) b = round_to(round_to(b, 16) + (2 * (size_t)nlags + 2) * ea, 16) + (size_t)nlags * (es + 8 + 4);
  return b;
}

size_t temporal_long_smem(int M1, size_t es, size_t ea) {
  const size_t g = 128 / es;
  return round_to(round_to(M1, g) * es + (size_t)M1 * (es / 2), 16) + 64 * es + 160 * ea;
}

// Long-series kernel: the cheapest even N >= 2T - 1 and first radix R0 whose
// length-N/R0 sub-transforms fit in shared memory (forward sub-transforms of
// all N points, inverse ones of N/2).
static bool choose_long_temporal(int64_t T, size_t es, size_t ea, int force_r0, int& N, int& R0) {
  const int64_t lo = std::max<int64_t>(2, 2 * T - 1);
  int64_t hi = 1;
  while (hi < lo) hi <<= 1;
  double best = 1e300;
  N = R0 = 0;
  for (int64_t n = lo + (lo & 1); n <= hi; n += 2) {
    for (int r0 : {8, 4, 2}) {
      if ((force_r0 && r0 != force_r0) || n % r0 || temporal_long_smem((int)(n / r0), es, ea) > kSmemLimit) continue;
      FftPlan rest;
      if (!make_plan((int)(n / r0), rest)) continue;
      double c = padded_cost(r0) * (double)n;
      for (int s = 0; s < rest.npass; ++s) c += pass_cost(rest.radix[s]) * 1.5 * (double)n;
      if (c < best) {
        best = c;
        N = (int)n;
        R0 = r0;
      }
    }
  }
  return N > 0;
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
  L.nt_fft = 0;
  if (r.mode == MODE_FFT) {
    if (r.nt < 2 * r.T - 1) { err = "nt must be at least 2*len(img_seq) - 1"; return false; }
    // any length >= 2T - 1 gives the same linear autocorrelation; use the cheapest
    L.nt_fft = choose_temporal_length(r.T);
  }
  for (int lag : r.lags)
    if (lag < 0 || lag >= r.T) { err = "lags must lie in [0, len(img_seq) - 1]"; return false; }
  const size_t es = spec_elem_bytes(r.precision);
  const int64_t nkx = r.nx / 2 + 1;
  const size_t Q = (size_t)r.ny * nkx;
  L.Tpad = (int)align_up((size_t)r.T, 64 / es);
  L.Hpad = (int)(2 * ((r.H + 1) / 2));
  // stage 1-2 blocking: ~64 KB of shared memory per transform buffer; every
  // transform is padded by one swizzle group (128 bytes).  FDDM_B200_ROWS_KB,
  // FDDM_B200_COLS_KB and FDDM_B200_COLS_FRAMES override the targets (tuning).
  auto env_int = [](const char* name, int dflt) {
    const char* v = std::getenv(name);
    const int x = v ? std::atoi(v) : 0;
    return x > 0 ? x : dflt;
  };
  const size_t rows_target = (size_t)env_int("FDDM_B200_ROWS_KB", 64) * 1024;
  const size_t cols_target = (size_t)env_int("FDDM_B200_COLS_KB", 64) * 1024;
  const size_t g = 128 / es;
  L.pairs_per_block = (int)std::max<size_t>(1, std::min<size_t>(rows_target / ((size_t)r.nx * es), (size_t)((r.H + 1) / 2)));
  const int nb = (int)std::max<size_t>(1, cols_target / ((size_t)r.ny * es));
  L.frames_per_block = std::min(nb, env_int("FDDM_B200_COLS_FRAMES", 8));
  L.cols_per_block = std::max(1, nb / L.frames_per_block);
  // two transform buffers and the permutation table (ny ints)
  auto cols_bytes = [&] {
    return (size_t)(2 * (L.frames_per_block * L.cols_per_block * (r.ny + g) + g)) * es + (size_t)r.ny * 4;
  };
  while (cols_bytes() > kSmemLimit && L.cols_per_block > 1) L.cols_per_block /= 2;
  while (cols_bytes() > kSmemLimit && L.frames_per_block > 1) L.frames_per_block /= 2;
  // row pass: one transform buffer + at most 64 KB of raw staging; column pass: two buffers
  if ((size_t)(L.pairs_per_block * (r.nx + g) + g) * es + 65536 + (size_t)r.nx * 4 > kSmemLimit ||
      cols_bytes() > kSmemLimit) {
    err = "image dimensions too large for the shared-memory FFT";
    return false;
  }
  // frame chunk: keep the row-pass buffer near 128 MB
  const size_t per_frame = (size_t)nkx * L.Hpad * es;
  int chunk = (int)std::max<size_t>(1, (128ull << 20) / per_frame);
  chunk = std::max(L.frames_per_block, chunk / L.frames_per_block * L.frames_per_block);
  chunk = (int)std::min<int64_t>(chunk, (r.T + L.frames_per_block - 1) / L.frames_per_block * L.frames_per_block);
  L.chunk = chunk;
  // temporal kernel: the whole transform in shared memory when it fits, else
  // (fft mode) the long-series kernel with sub-transforms of N / R0, or (diff
  // mode) the series read from global memory
  const size_t ea = 8;
  L.long_R0 = 0;
  L.diff_staged = 0;
  if (r.mode == MODE_FFT) {
    // the shared-memory kernel indexes its lag slot tables with int16
    // FDDM_B200_TEMPORAL_SPLIT=2|4|8 forces the long-series kernel with that
    // first radix (diagnostics and tests of that kernel on short series)
    const char* fs = std::getenv("FDDM_B200_TEMPORAL_SPLIT");
    const int force = fs ? std::atoi(fs) : 0;
    const bool forced = force == 2 || force == 4 || force == 8;
    if (forced || r.T >= 32767 ||
        temporal_fft_smem((int)r.T, L.nt_fft, (int)r.lags.size(), es, ea, false) > kSmemLimit) {
      int n = 0, r0 = 0;
      if (!choose_long_temporal(r.T, es, ea, forced ? force : 0, n, r0)) {
        err = "sequence too long for the temporal kernels (" + std::to_string(r.T) +
              " frames: no transform length splits into sub-transforms that fit in shared memory)";
        return false;
      }
      L.nt_fft = n;
      L.long_R0 = r0;
    }
  } else {
    L.diff_staged = (size_t)r.T * es + 96 * ea <= kSmemLimit ? 1 : 0;
  }
  size_t off = 0;
  L.spec_off = off; L.spec_bytes = Q * (size_t)L.Tpad * es; off = align_up(off + L.spec_bytes, 256);
  L.rbuf_off = off; L.rbuf_bytes = (size_t)chunk * per_frame; off = align_up(off + L.rbuf_bytes, 256);
  L.win_off = off; L.win_bytes = r.window ? (size_t)r.H * r.W * (es / 2) : 0; off = align_up(off + L.win_bytes, 256);
  L.lags_off = off; off = align_up(off + r.lags.size() * sizeof(int) + 4, 256);
  L.rcp_off = off; off = align_up(off + r.lags.size() * sizeof(double) + 8, 256);
  L.slot_off = off; off = align_up(off + 2 * (size_t)(r.T + 1) * sizeof(int), 256);
  L.need_off = off;
  if (r.mode == MODE_FFT && !L.long_R0) off = align_up(off + (size_t)kMaxTemporalCtas * (2 * r.lags.size() + 2) * ea, 256);
  L.xs_off = off;
  L.xs_stride = L.xs_pfx_off = 0;
  if (L.long_R0) {
    L.xs_pfx_off = align_up((size_t)L.nt_fft * es, 256);
    L.xs_stride = L.xs_pfx_off + align_up((size_t)r.T * ea, 256);
    off += (size_t)kMaxLongCtas * L.xs_stride;
  }
  L.tables_off = off;
  L.tables_bytes = 0;
  if (r.inline_tables) {
    const int kind = r.precision == PREC_FF ? 0 : r.precision == PREC_F64 ? 1 : 2;
    L.tables_bytes = inline_table_bytes((int)r.nx, kind) + inline_table_bytes((int)r.ny, kind);
    if (r.mode == MODE_FFT)
      L.tables_bytes += inline_table_bytes(L.nt_fft, kind) +
                        inline_table_bytes(L.long_R0 ? L.nt_fft / L.long_R0 : L.nt_fft / 2, kind);
    off += L.tables_bytes;
  }
  L.total = off;
  if (r.max_work > 0 && L.total > r.max_work) {
    // a smaller frame chunk is the only part that can shrink
    const size_t fixed = L.total - align_up(L.rbuf_bytes, 256);
    const size_t room = r.max_work > fixed ? r.max_work - fixed : 0;
    int c = (int)std::min<size_t>((size_t)L.chunk, room / std::max<size_t>(per_frame, 1));
    c = c / L.frames_per_block * L.frames_per_block;
    if (c < L.frames_per_block) {
      L.over_max_work = true;
      err = "needs " + std::to_string(fixed + (size_t)L.frames_per_block * per_frame) +
            " bytes of workspace, more than the " + std::to_string(r.max_work) + " available";
      return false;
    }
    const size_t shrink = align_up(L.rbuf_bytes, 256) - align_up((size_t)c * per_frame, 256);
    L.chunk = c;
    L.rbuf_bytes = (size_t)c * per_frame;
    L.win_off -= shrink; L.lags_off -= shrink; L.rcp_off -= shrink; L.slot_off -= shrink;
    L.need_off -= shrink; L.xs_off -= shrink; L.tables_off -= shrink;
    L.total -= shrink;
  }
  return true;
}

}  // namespace fddm
