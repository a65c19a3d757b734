// Host-side driver of the structure-function pipeline for one precision tier.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include "ddm_impl.cuh"

namespace fddm {

template <class S> struct tier_kind;
template <> struct tier_kind<ff> { static constexpr int v = 0; };
template <> struct tier_kind<double> { static constexpr int v = 1; };
template <> struct tier_kind<float> { static constexpr int v = 2; };

inline void split_ff(double d, float& h, float& l) {
  h = (float)d;
  l = (float)(d - (double)h);
}

constexpr size_t kMaxDynSmem = 232448;  // 227 KB opt-in limit per CTA on sm_100-class parts

template <class K> inline cudaError_t allow_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Threads per CTA of the temporal kernels: about one radix-8 butterfly per
// thread and pass, so that short transforms run several CTAs per SM.
inline int temporal_threads(int n) {
  int t = 128;
  while (t < 512 && t * 8 < n) t *= 2;
  return t;
}

// Persistent grid: as many CTAs as fit on the device, at most one per item.
template <class K> inline unsigned persistent_grid(K kernel, int threads, size_t smem, int items) {
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem);
  return (unsigned)std::max(1, std::min(items, std::max(occ, 1) * nsm));
}

// True when every pass of `p` has radix 2, 4 or 8: the kernels' P2 variants
// then carry only those butterflies.
inline bool plan_is_p2(const FftPlan& p) {
  for (int s = 0; s < p.npass; ++s)
    if (p.radix[s] != 2 && p.radix[s] != 4 && p.radix[s] != 8) return false;
  return true;
}

// Temporal kernel of a tier: FP32 transforms run two CTAs per SM.
template <class S, class A, bool P2, bool F2 = false> constexpr auto tfft_kernel() {
  if constexpr (sizeof(S) == 4) return &k_tfft_x2<S, A, P2, F2>;
  else return &k_tfft<S, A, P2, F2>;
}

// The temporal kernel's fused radix-2 path (F2 in tfft_body): first radix 2,
// every radix 2, 4 or 8, at least two passes, and N/2 a multiple of the square
// of the swizzle group, so that slot N/2 + t of the transform buffer is the
// slot of element t of the series prefetched at N/2.
template <class S> inline bool fused_radix2_ok(const FftPlan& p) {
  const int G = swz_group<S>::G;
  return plan_is_p2(p) && p.npass >= 2 && p.radix[0] == 2 && (p.n / 2) % (G * G) == 0;
}

// CTA sizes of the spatial passes; FDDM_B200_ROWS_THREADS / FDDM_B200_COLS_THREADS
// (128, 256 or 512) override them (tuning).
inline int spatial_threads(const char* env, int dflt) {
  const char* v = std::getenv(env);
  const int x = v ? std::atoi(v) : 0;
  return (x == 128 || x == 256 || (x == 512 && dflt == 512)) ? x : dflt;
}

template <class S, class IN, bool P2>
cudaError_t launch_rows(const SpatialArgs& a, int items, size_t smem, cudaStream_t st) {
  cudaError_t e = allow_smem(k_rows<S, IN, P2>, smem);
  if (e != cudaSuccess) return e;
  const int nt = spatial_threads("FDDM_B200_ROWS_THREADS", 256);
  k_rows<S, IN, P2><<<persistent_grid(k_rows<S, IN, P2>, nt, smem, items), nt, smem, st>>>(a);
  return cudaGetLastError();
}

template <class S, class IN>
cudaError_t launch_rows(const SpatialArgs& a, int items, size_t smem, cudaStream_t st) {
  return plan_is_p2(a.px) ? launch_rows<S, IN, true>(a, items, smem, st) : launch_rows<S, IN, false>(a, items, smem, st);
}

template <class S>
cudaError_t dispatch_rows(int dtype, const SpatialArgs& a, int items, size_t smem, cudaStream_t st) {
  switch (dtype) {
    case DT_U8: return launch_rows<S, uint8_t>(a, items, smem, st);
    case DT_I16: return launch_rows<S, int16_t>(a, items, smem, st);
    case DT_U16: return launch_rows<S, uint16_t>(a, items, smem, st);
    case DT_I32: return launch_rows<S, int32_t>(a, items, smem, st);
    case DT_U32: return launch_rows<S, uint32_t>(a, items, smem, st);
    case DT_F32: return launch_rows<S, float>(a, items, smem, st);
    case DT_F64: return launch_rows<S, double>(a, items, smem, st);
    default: return cudaErrorInvalidValue;
  }
}

// Returns 0 on success, else an FDDM status code with `err` filled in.
template <class S, class A>
int run_ddm_t(const DdmRequest& r, cudaStream_t st, std::string& err) {
  // the transform path pairs every lag with its prefix sums by position and
  // sums the last lags directly from the end of the list
  if (r.mode == MODE_FFT)
    for (size_t l = 1; l < r.lags.size(); ++l)
      if (r.lags[l] <= r.lags[l - 1]) {
        err = "fft mode needs strictly increasing lags";
        return 1;
      }
  WorkLayout L;
  if (!plan_layout(r, L, err)) return 4;
  if (r.work_bytes < L.total) {
    err = "workspace too small: need " + std::to_string(L.total) + " bytes, got " + std::to_string(r.work_bytes);
    return 2;
  }
  // Page-locked host frames (mapped into the device's address space under
  // unified addressing; NVLink-C2C on Grace parts) are read in place by the row
  // pass: no copy-engine upload, no staging.  Pageable frames are uploaded chunk
  // by chunk on the copy stream: they may be views of memory-mapped files whose
  // pages are not resident, which the kernels must not read directly.
  // In-place reads also need the row pass's staged path (16-byte aligned rows,
  // fetched with cp.async ahead of use): its per-pixel fallback would wait on
  // every host read.  FDDM_B200_ZERO_COPY=0 forces the upload for page-locked
  // frames too.
  const size_t row_bytes = (size_t)r.W * dtype_bytes(r.dtype);
  const size_t stage = (size_t)2 * L.pairs_per_block * row_bytes;
  auto stageable = [&](const void* p) {
    return row_bytes % 16 == 0 && (reinterpret_cast<uintptr_t>(p) % 16) == 0 && 2 * stage <= 64 * 1024;
  };
  const void* host_direct = nullptr;
  if (r.host_img) {
    const char* zc = std::getenv("FDDM_B200_ZERO_COPY");
    cudaPointerAttributes pa{};
    if (!(zc && zc[0] == '0') && cudaPointerGetAttributes(&pa, r.host_img) == cudaSuccess &&
        pa.type == cudaMemoryTypeHost && pa.devicePointer != nullptr && stageable(pa.devicePointer))
      host_direct = pa.devicePointer;
    else
      (void)cudaGetLastError();  // some runtimes report pageable memory as an error: clear it
  }
  set_last_input_path(r.host_img == nullptr ? 0 : host_direct ? 1 : 2);
  if (r.host_img && !host_direct && r.img == nullptr) {
    err = "the host frames cannot be read in place (pageable, not 16-byte aligned rows, or FDDM_B200_ZERO_COPY=0): "
          "a device buffer for their upload is needed";
    return 1;
  }
  const bool upload = r.host_img != nullptr && host_direct == nullptr;
  const int kind = tier_kind<S>::v;
  const int T = (int)r.T, H = (int)r.H, W = (int)r.W, nx = (int)r.nx, ny = (int)r.ny;
  const int nkx = nx / 2 + 1;
  const size_t Q = (size_t)ny * nkx;
  const int nl = (int)r.lags.size();
  unsigned char* ws = static_cast<unsigned char*>(r.work);

  FftTables tx, ty, tt, tt2;
  const int N = L.nt_fft;
  cudaError_t ce;
  // workspace-only mode: the pass-table area of each uploaded length, in upload order (nx, ny, N, second)
  unsigned char* pass_area[4] = {nullptr, nullptr, nullptr, nullptr};
  int pass_n[4] = {0, 0, 0, 0};
  int nregion = 0;
  if (!r.inline_tables) {
    if (!get_tables(nx, kind, tx, err) || !get_tables(ny, kind, ty, err)) return 3;
    // second temporal table: the half length, or the sub-transform length of the long-series kernel
    if (r.mode == MODE_FFT && (!get_tables(N, kind, tt, err) || !get_tables(L.long_R0 ? N / L.long_R0 : N / 2, kind, tt2, err)))
      return 3;
  } else {
    // copy host-computed tables into the workspace (no device allocation)
    unsigned char* tp = ws + L.tables_off;
    auto upload = [&](int n, FftTables& t) -> bool {
      const HostTables* h = nullptr;
      if (!host_tables(n, kind, h, err)) return false;
      auto up = [](size_t x) { return (x + 255) / 256 * 256; };
      unsigned char* twp = tp;
      int* pp = reinterpret_cast<int*>(tp + up(h->tw.size()));
      int* ip = reinterpret_cast<int*>(tp + up(h->tw.size()) + up(sizeof(int) * (size_t)n));
      if ((ce = cudaMemcpyAsync(twp, h->tw.data(), h->tw.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
          (ce = cudaMemcpyAsync(pp, h->perm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
          (ce = cudaMemcpyAsync(ip, h->iperm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st)) != cudaSuccess) {
        err = cudaGetErrorString(ce);
        return false;
      }
      t.plan = h->plan;
      t.tw = twp;
      t.perm = pp;
      t.iperm = ip;
      pass_area[nregion] = tp + up(h->tw.size()) + 2 * up(sizeof(int) * (size_t)n);
      pass_n[nregion++] = n;
      tp += inline_table_bytes(n, kind);
      return true;
    };
    if (!upload(nx, tx) || !upload(ny, ty)) return 3;
    if (r.mode == MODE_FFT && (!upload(N, tt) || !upload(L.long_R0 ? N / L.long_R0 : N / 2, tt2))) return 3;
  }

  // window in the FFT scalar type
  const void* win_s = nullptr;
  const bool do_spatial = (r.stages & 1) != 0;
  if (r.window && do_spatial) {
    S* w = reinterpret_cast<S*>(ws + L.win_off);
    const size_t n = (size_t)H * W;
    k_window_convert<S><<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(r.window, w, n);
    if ((ce = cudaGetLastError()) != cudaSuccess) { err = cudaGetErrorString(ce); return 3; }
    win_s = w;
  } else if (r.window) {
    win_s = ws + L.win_off;
  }
  // lags and reciprocal normalisations
  std::vector<double> rcp(nl);
  for (int l = 0; l < nl; ++l) rcp[l] = 1.0 / (double)(T - r.lags[l]);
  int* d_lags = reinterpret_cast<int*>(ws + L.lags_off);
  double* d_rcp = reinterpret_cast<double*>(ws + L.rcp_off);
  if (nl > 0 && !r.tables_ready) {
    if ((ce = cudaMemcpyAsync(d_lags, r.lags.data(), nl * sizeof(int), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_rcp, rcp.data(), nl * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return 3;
    }
  }
  // slot tables of the prefix sums each lag needs: pfx[T - lag] (A) and pfx[lag] (B)
  int* d_slots = reinterpret_cast<int*>(ws + L.slot_off);
  if (r.mode == MODE_FFT && !L.long_R0 && !r.tables_ready) {
    std::vector<int> slots(2 * (size_t)(T + 1), -1);
    for (int l = 0; l < nl; ++l) {
      slots[T - r.lags[l]] = l;
      slots[(size_t)(T + 1) + r.lags[l]] = l;
    }
    if ((ce = cudaMemcpyAsync(d_slots, slots.data(), slots.size() * sizeof(int), cudaMemcpyHostToDevice, st)) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return 3;
    }
  }

  StageEvents* evs = (r.inline_tables || r.stages != 3 || r.collect) ? nullptr : stage_events();
  if (evs) cudaEventRecord(evs->ev[0], st);
  int launches = r.window && do_spatial ? 1 : 0;



  // stages 1-2 over frame chunks
  SpatialArgs sa{};
  sa.img = host_direct ? host_direct : r.img;
  sa.window_s = win_s;
  sa.T = T; sa.H = H; sa.W = W; sa.nx = nx; sa.ny = ny; sa.nkx = nkx; sa.Hpad = L.Hpad;
  sa.Tpad = L.Tpad;
  sa.pairs_per_block = L.pairs_per_block;
  sa.cols_per_block = L.cols_per_block;
  sa.frames_per_block = L.frames_per_block;
  sa.px = tx.plan; sa.py = ty.plan;
  // per-pass twiddle tables (coalesced twiddle loads); region i of the
  // workspace-only mode holds the tables of the i-th uploaded length
  auto attach = [&](FftPlan& p, int region) -> bool {
    if (!r.inline_tables) return attach_pass_tables(p, kind, err);
    if (region >= nregion || !pass_area[region]) {
      err = "no workspace area for the pass twiddle tables";
      return false;
    }
    return upload_pass_tables(p, kind, pass_area[region], pass_tables_bound(pass_n[region], kind), st, err);
  };
  if (!attach(sa.px, 0) || !attach(sa.py, 1)) return 3;
  sa.twx = tx.tw; sa.twy = ty.tw; sa.permx = tx.perm; sa.permy = ty.perm;
  sa.rbuf = ws + L.rbuf_off;
  sa.spec = ws + L.spec_off;
  const double norm = 1.0 / std::sqrt((double)nx * (double)ny);
  split_ff(norm, sa.norm_h, sa.norm_l);
  sa.norm_d = norm;
  const int npairs = (H + 1) / 2;
  // raw rows staged asynchronously when every row starts on a 16-byte boundary
  sa.raw_stage_bytes = stageable(sa.img) ? (int)stage : 0;
  const int G = swz_group<S>::G;
  const size_t smem_rows = (size_t)swz_round<S>(L.pairs_per_block * (nx + G)) * sizeof(cx<S>) +
                           2 * (size_t)sa.raw_stage_bytes + (size_t)nx * sizeof(int);
  const size_t smem_cols =
      2 * (size_t)swz_round<S>(L.cols_per_block * L.frames_per_block * (ny + G)) * sizeof(cx<S>) + (size_t)ny * sizeof(int);
  const int ngroups = (npairs + L.pairs_per_block - 1) / L.pairs_per_block;
  const bool p2y = plan_is_p2(sa.py);
  if ((ce = p2y ? allow_smem(k_cols<S, true>, smem_cols) : allow_smem(k_cols<S, false>, smem_cols)) != cudaSuccess) {
    err = cudaGetErrorString(ce);
    return 3;
  }
  CopyCtx* cp = nullptr;
  const size_t frame_bytes = (size_t)H * W * dtype_bytes(r.dtype);
  // host frames or a host result: this call owns the device's copy events until it has enqueued everything
  std::unique_lock<std::mutex> copy_lock;
  if (upload || r.host_out) {
    CopyCtx* c = copy_ctx(err);
    if (!c) return 3;
    copy_lock = std::unique_lock<std::mutex>(c->mu);
  }
  if (upload) {
    if (!(cp = copy_ctx(err))) return 3;
    // the copies may only overwrite the frame buffer after earlier work on `st`
    if ((ce = cudaEventRecord(cp->start, st)) != cudaSuccess || (ce = cudaStreamWaitEvent(cp->stream, cp->start, 0)) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return 3;
    }
  }
  for (int t0 = 0; do_spatial && t0 < T; t0 += L.chunk) {
    sa.t0 = t0;
    sa.tc = std::min(L.chunk, T - t0);
    if (upload) {
      const size_t off = (size_t)t0 * frame_bytes, n = (size_t)sa.tc * frame_bytes;
      if ((ce = cudaMemcpyAsync(static_cast<unsigned char*>(const_cast<void*>(r.img)) + off,
                                static_cast<const unsigned char*>(r.host_img) + off, n, cudaMemcpyHostToDevice,
                                cp->stream)) != cudaSuccess ||
          (ce = cudaEventRecord(cp->ready, cp->stream)) != cudaSuccess ||
          (ce = cudaStreamWaitEvent(st, cp->ready, 0)) != cudaSuccess) {
        err = cudaGetErrorString(ce);
        return 3;
      }
    }
    if ((ce = dispatch_rows<S>(r.dtype, sa, ngroups * sa.tc, smem_rows, st)) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return 3;
    }
    const int col_items = ((nkx + L.cols_per_block - 1) / L.cols_per_block) *
                          ((sa.tc + L.frames_per_block - 1) / L.frames_per_block);
    const int ct = spatial_threads("FDDM_B200_COLS_THREADS", 512);
    if (p2y) k_cols<S, true><<<persistent_grid(k_cols<S, true>, ct, smem_cols, col_items), ct, smem_cols, st>>>(sa);
    else k_cols<S, false><<<persistent_grid(k_cols<S, false>, ct, smem_cols, col_items), ct, smem_cols, st>>>(sa);
    if ((ce = cudaGetLastError()) != cudaSuccess) { err = cudaGetErrorString(ce); return 3; }
    launches += 2;
  }
  if (evs) cudaEventRecord(evs->ev[1], st);
  if (!(r.stages & 2) && !r.collect) {
    count_launches(launches);
    return 0;
  }

  // stage 3
  TemporalArgs ta{};
  ta.spec = ws + L.spec_off;
  ta.Q = Q; ta.Tpad = L.Tpad; ta.T = T; ta.nt = N; ta.nlags = nl;
  size_t smem_t = (size_t)T * sizeof(cx<S>) + 96 * sizeof(A);
  int threads = temporal_threads(T);
  const bool long_fft = r.mode == MODE_FFT && L.long_R0 > 0;
  if (r.mode == MODE_FFT) {
    split_ff(1.0 / (double)N, ta.invnt_h, ta.invnt_l);
    ta.invnt_d = 1.0 / (double)N;
    ta.twt = tt.tw;
    if (long_fft) {
      ta.R0 = L.long_R0;
      ta.M1 = N / L.long_R0;
      ta.pm = tt2.plan;
      if (!attach(ta.pm, 3)) return 3;
      ta.twm = tt2.tw;
      ta.xs = ws + L.xs_off;
      ta.xs_stride = L.xs_stride;
      ta.xs_pfx_off = L.xs_pfx_off;
      smem_t = temporal_long_smem(ta.M1, sizeof(cx<S>), sizeof(A));
      threads = temporal_threads(ta.M1);
    } else {
      ta.twt2 = tt2.tw;
      if (!temporal_plan(N, ta.pt) || !half_plan(ta.pt, ta.pt2)) {
        err = "no temporal plan for length " + std::to_string(N);
        return 4;
      }
      if (!attach(ta.pt, 2) || !attach(ta.pt2, 3)) return 3;
      ta.slotA = d_slots; ta.slotB = d_slots + (T + 1);
      ta.need = ws + L.need_off;
      threads = 0;  // chosen below (tuning table, autotuner or occupancy model)
    }
  } else if (!L.diff_staged) {
    smem_t = 96 * sizeof(A);
  }
  const bool p2t = r.mode == MODE_FFT && !long_fft && plan_is_p2(ta.pt) && plan_is_p2(ta.pt2);
  // FDDM_B200_TEMPORAL_FUSED=0 keeps the separate passes (comparison runs)
  const char* fz = std::getenv("FDDM_B200_TEMPORAL_FUSED");
  const bool f2t = p2t && fused_radix2_ok<S>(ta.pt) && !(fz && fz[0] == '0');
  ta.lags = d_lags; ta.rcp = d_rcp; ta.out = r.out;
  split_ff(1.0 / (double)T, ta.invT_h, ta.invT_l); ta.invT_d = 1.0 / (double)T;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // Launch configuration of the temporal kernel: CTA size and, for the
  // shared-memory fft kernel, whether the needed prefix sums and per-lag tables
  // sit in shared memory (fewer resident CTAs) or in global scratch.
  //  1. an entry of the tuning table (loaded from a committed table, or written
  //     by the autotuner on an earlier call), else
  //  2. with the autotuner on, every candidate is timed on this call's own
  //     spectrum (a few waves of modes; their outputs are rewritten by the real
  //     launch) and the fastest is recorded, else
  //  3. the occupancy model: the most resident warps per SM, then the most
  //     resident CTAs (smaller CTAs: each works on its own mode, so while one
  //     waits at a barrier the others issue; measured on 512^2 stacks, 200
  //     lags: 1.18x at T = 2000, 1.5x at T = 1000, 2.2x at T = 500 against one
  //     radix-8 butterfly per thread), then shared-memory tables.
  // FDDM_B200_TEMPORAL_THREADS=128|256|512 overrides the CTA size.
  const bool shared_fft = r.mode == MODE_FFT && !long_fft;
  const size_t with_need = shared_fft ? temporal_fft_smem(T, N, nl, sizeof(cx<S>), sizeof(A), true) : 0;
  auto smem_of = [&](int nis) {
    return shared_fft ? temporal_fft_smem(T, N, nl, sizeof(cx<S>), sizeof(A), nis != 0) : smem_t;
  };
  std::vector<TemporalChoice> cands;
  // diff mode with the series read through L1/L2 (too long for shared memory):
  // all warps of a CTA read one mode's series for their lags, so only the
  // largest CTA keeps that series in L1 (with 128-thread CTAs, 16 modes per SM
  // thrash it: 20000 x 256^2, 200 lags, temporal 449 ms against 271)
  const bool diff_global = r.mode == MODE_DIFF && !L.diff_staged;
  for (int nis : {1, 0}) {
    // the tables' placement only matters to the shared-memory fft kernel
    if (shared_fft ? (nis == 1 && with_need > kSmemLimit) : nis == 1) continue;
    for (int t : {512, 256, 128})
      if (!diff_global || t == 512) cands.push_back({t, nis});
  }
  auto occupancy = [&](auto kernel, const TemporalChoice& c) {
    int o = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kernel, c.threads, smem_of(c.need_in_smem)) != cudaSuccess) {
      (void)cudaGetLastError();
      return 0;
    }
    // the long-series kernel's per-CTA scratch holds kMaxLongCtas CTAs
    if (long_fft) o = std::min(o, std::max(1, kMaxLongCtas / std::max(nsm, 1)));
    return o;
  };
  const int tune_prec = tier_kind<S>::v == 0 ? PREC_FF : tier_kind<S>::v == 1 ? PREC_F64 : PREC_F32;
  auto launch_range = [&](auto kernel, const TemporalChoice& c, size_t q0, size_t q1, unsigned grid) {
    TemporalArgs t2 = ta;
    t2.need_in_smem = c.need_in_smem;
    t2.q_begin = q0;
    t2.q_end = q1;
    kernel<<<grid, c.threads, smem_of(c.need_in_smem), st>>>(t2);
  };
  auto choose = [&](auto kernel) -> bool {
    for (const TemporalChoice& c : cands)
      if ((ce = allow_smem(kernel, smem_of(c.need_in_smem))) != cudaSuccess) {
        err = cudaGetErrorString(ce);
        return false;
      }
    // the occupancy model's choice
    TemporalChoice model{0, 0};
    {
      int best_w = 0, best_o = 0;
      for (const TemporalChoice& c : cands) {
        const int o = occupancy(kernel, c);
        const int w = o * c.threads / 32;
        if (o > 0 && (w > best_w || (w == best_w && o > best_o))) {
          best_w = w;
          best_o = o;
          model = c;
        }
      }
    }
    TemporalChoice pick = model;
    TemporalChoice tuned{0, 0};
    const bool have = tuned_temporal(tune_prec, r.mode, T, nl, tuned) &&
                      (!shared_fft ? tuned.need_in_smem == 0 : (tuned.need_in_smem == 0 || with_need <= kSmemLimit));
    if (have) {
      pick = tuned;
    } else if (autotune_enabled()) {
      // time every candidate on this call's spectrum (the real launch below
      // rewrites these outputs); another candidate replaces the model's choice
      // only when it is at least 5 % faster, so timing noise keeps the model
      cudaEvent_t e0, e1;
      if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
        // the same modes for every candidate: 16 waves of the largest grid, so
        // that per-CTA set-up is amortised as in a full launch
        const size_t probe = std::min<size_t>(Q, 16 * (size_t)(long_fft ? kMaxLongCtas : kMaxTemporalCtas));
        // three interleaved rounds over the candidates (drift of the clock or
        // of other work on the GPU hits every candidate alike); fastest of each
        std::vector<float> tbest(cands.size(), 1e30f);
        std::vector<unsigned> grids(cands.size(), 0);
        for (size_t i = 0; i < cands.size(); ++i) {
          const int o = occupancy(kernel, cands[i]);
          if (o < 1) continue;
          const size_t g = std::min<size_t>((size_t)o * nsm, long_fft ? kMaxLongCtas : kMaxTemporalCtas);
          grids[i] = (unsigned)std::min(g, probe);
          launch_range(kernel, cands[i], 0, probe, grids[i]);  // warm-up
          count_launches(1);
        }
        bool ok = true;
        for (int round = 0; round < 3 && ok; ++round)
          for (size_t i = 0; i < cands.size() && ok; ++i) {
            if (!grids[i]) continue;
            float m = 0.0f;
            cudaEventRecord(e0, st);
            launch_range(kernel, cands[i], 0, probe, grids[i]);
            cudaEventRecord(e1, st);
            ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&m, e0, e1) == cudaSuccess;
            if (ok) tbest[i] = std::min(tbest[i], m);
            count_launches(1);
          }
        float best = 1e30f, model_ms = 1e30f;
        TemporalChoice fastest = model;
        for (size_t i = 0; i < cands.size(); ++i) {
          if (!grids[i]) continue;
          if (cands[i].threads == model.threads && cands[i].need_in_smem == model.need_in_smem) model_ms = tbest[i];
          if (tbest[i] < best) {
            best = tbest[i];
            fastest = cands[i];
          }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (ok) {
          pick = best < 0.95f * model_ms ? fastest : model;
          record_temporal(tune_prec, r.mode, T, nl, pick);
        }
      }
      if ((ce = cudaGetLastError()) != cudaSuccess) {
        err = cudaGetErrorString(ce);
        return false;
      }
    }
    if (const char* tt = std::getenv("FDDM_B200_TEMPORAL_THREADS")) {
      const int v = std::atoi(tt);
      if (v == 128 || v == 256 || v == 512) pick.threads = v;
    }
    threads = pick.threads;
    ta.need_in_smem = pick.need_in_smem;
    smem_t = smem_of(pick.need_in_smem);
    occ = occupancy(kernel, pick);
    return true;
  };
  bool prepared;
  if (long_fft) prepared = choose(k_tfft_long<S, A>);
  else if (r.mode == MODE_FFT)
    prepared = f2t ? choose(tfft_kernel<S, A, true, true>())
                   : p2t ? choose(tfft_kernel<S, A, true>()) : choose(tfft_kernel<S, A, false>());
  else if (L.diff_staged) prepared = choose(k_tdiff<S, A, true>);
  else prepared = choose(k_tdiff<S, A, false>);
  if (!prepared) return 3;
  if (occ < 1) { err = "temporal kernel does not fit on an SM (shared memory " + std::to_string(smem_t) + " B)"; return 4; }
  if (r.collect) {  // the caller launches this stage (the many-job kernel, or on its own later)
    ta.q_begin = 0;
    ta.q_end = Q;
    r.collect->args = ta;
    r.collect->threads = threads;
    r.collect->smem = smem_t;
    r.collect->variant = (r.mode == MODE_FFT && !long_fft) ? (f2t ? 2 : p2t ? 1 : 0) : -1;
    count_launches(launches);
    return 0;
  }
  const size_t max_grid = std::min<size_t>((size_t)occ * nsm, long_fft ? kMaxLongCtas : kMaxTemporalCtas);
  // With a host result the modes run in chunks: each chunk's output columns
  // (all lag rows) go to the host with a 2D copy on the copy stream while the
  // next chunk computes, so only the last chunk's copy is exposed.
  const int nchunks = (r.host_out && Q >= 16 * max_grid) ? 4 : 1;
  CopyCtx* cpo = nullptr;
  if (nchunks > 1 && !(cpo = copy_ctx(err))) return 3;
  for (int c = 0; c < nchunks; ++c) {
    ta.q_begin = Q * c / nchunks;
    ta.q_end = Q * (c + 1) / nchunks;
    const unsigned grid = (unsigned)std::min<size_t>(ta.q_end - ta.q_begin, max_grid);
    if (grid == 0) continue;
    if (long_fft) k_tfft_long<S, A><<<grid, threads, smem_t, st>>>(ta);
    else if (r.mode == MODE_FFT && f2t) tfft_kernel<S, A, true, true>()<<<grid, threads, smem_t, st>>>(ta);
    else if (r.mode == MODE_FFT && p2t) tfft_kernel<S, A, true>()<<<grid, threads, smem_t, st>>>(ta);
    else if (r.mode == MODE_FFT) tfft_kernel<S, A, false>()<<<grid, threads, smem_t, st>>>(ta);
    else if (L.diff_staged) k_tdiff<S, A, true><<<grid, threads, smem_t, st>>>(ta);
    else k_tdiff<S, A, false><<<grid, threads, smem_t, st>>>(ta);
    if ((ce = cudaGetLastError()) != cudaSuccess) { err = cudaGetErrorString(ce); return 3; }
    if (cpo) {
      const size_t pitch = Q * sizeof(double);
      if ((ce = cudaEventRecord(cpo->ready, st)) != cudaSuccess ||
          (ce = cudaStreamWaitEvent(cpo->stream, cpo->ready, 0)) != cudaSuccess ||
          (ce = cudaMemcpy2DAsync(r.host_out + ta.q_begin, pitch, r.out + ta.q_begin, pitch,
                                  (ta.q_end - ta.q_begin) * sizeof(double), (size_t)nl + 2, cudaMemcpyDeviceToHost,
                                  cpo->stream)) != cudaSuccess) {
        err = cudaGetErrorString(ce);
        return 3;
      }
    }
  }
  if (evs) cudaEventRecord(evs->ev[2], st);
  count_launches(launches + nchunks);
  if (r.host_out) {
    if (cpo) {
      // work queued on `stream` after this call sees the copies done
      if ((ce = cudaEventRecord(cpo->start, cpo->stream)) != cudaSuccess ||
          (ce = cudaStreamWaitEvent(st, cpo->start, 0)) != cudaSuccess) {
        err = cudaGetErrorString(ce);
        return 3;
      }
    } else {
      const size_t bytes = (size_t)(nl + 2) * Q * sizeof(double);
      if ((ce = cudaMemcpyAsync(r.host_out, r.out, bytes, cudaMemcpyDeviceToHost, st)) != cudaSuccess) {
        err = cudaGetErrorString(ce);
        return 3;
      }
    }
  }
  return 0;
}

// One launch of the many-job temporal kernel over the items of group `g`.
template <class S, class A>
int run_temporal_list_t(const TemporalListGroup& g, cudaStream_t st, std::string& err) {
  if (g.nitems <= 0) return 0;
  auto go = [&](auto kernel) -> int {
    cudaError_t ce = allow_smem(kernel, g.smem);
    int occ = 0, dev = 0, nsm = 0;
    if (ce == cudaSuccess) ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, g.threads, g.smem);
    if (ce == cudaSuccess) ce = cudaGetDevice(&dev);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (ce != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return 3;
    }
    if (occ < 1) {
      err = "many-job temporal kernel does not fit on an SM (shared memory " + std::to_string(g.smem) + " B)";
      return 4;
    }
    const unsigned grid =
        (unsigned)std::min<size_t>(std::min<size_t>((size_t)occ * nsm, kMaxTemporalCtas), (size_t)g.nitems);
    if ((ce = cudaMemsetAsync(g.d_counter, 0, sizeof(int), st)) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return 3;
    }
    kernel<<<grid, g.threads, g.smem, st>>>(g.d_args, g.d_items, g.nitems, g.d_counter);
    if ((ce = cudaGetLastError()) != cudaSuccess) {
      err = cudaGetErrorString(ce);
      return 3;
    }
    count_launches(1);
    return 0;
  };
  if constexpr (sizeof(S) == 4) {
    if (g.variant == 2) return go(k_tfft_list_x2<S, A, true, true>);
    if (g.variant == 1) return go(k_tfft_list_x2<S, A, true, false>);
    return go(k_tfft_list_x2<S, A, false, false>);
  } else {
    if (g.variant == 2) return go(k_tfft_list<S, A, true, true>);
    if (g.variant == 1) return go(k_tfft_list<S, A, true, false>);
    return go(k_tfft_list<S, A, false, false>);
  }
}

}  // namespace fddm
