// Image-structure-function pipeline for one image stack, templated on the
// FFT scalar S (float, ff or double) and the accumulation scalar A used for
// the cancellation-critical sums (ff or double).
//
// Stage 1  k_rows     frames -> (window) -> r2c FFT along x, two real rows
//                     packed into one complex transform; output R[t][kx][y].
// Stage 2  k_cols     R -> c2c FFT along y, x 1/sqrt(nx*ny), written q-major
//                     to the spectrum F[q][t] with q = fftshift_y(ky)*nkx + kx,
//                     i.e. already in the output's y-shifted order.
// Stage 3  k_tfft     per q: mean removal, prefix sums of |F - <F>|^2, FFT
//                     autocorrelation, combination into D(q, lag), PS, VAR.
//          k_tdiff    per q: D(q, lag) = <|F(t+lag) - F(t)|^2>_t directly.
// Frames go through stages 1-2 in chunks so that R stays small.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fft.cuh"

namespace fddm {

// ---------------------------------------------------------------------------
// pixel conversion
// ---------------------------------------------------------------------------
template <class S, class IN> struct pix;
template <class IN> struct pix<float, IN> {
  static __device__ __forceinline__ float get(const IN* p, size_t i) { return (float)p[i]; }
};
template <> struct pix<float, double> {
  static __device__ __forceinline__ float get(const double* p, size_t i) { return __double2float_rn(p[i]); }
};
template <class IN> struct pix<double, IN> {
  static __device__ __forceinline__ double get(const IN* p, size_t i) { return (double)p[i]; }
};
template <class IN> struct pix<ff, IN> {  // 8/16-bit integers and float are exact in one float
  static __device__ __forceinline__ ff get(const IN* p, size_t i) { return {(float)p[i], 0.0f}; }
};
template <> struct pix<ff, int32_t> {
  static __device__ __forceinline__ ff get(const int32_t* p, size_t i) {
    int32_t v = p[i];
    float h = __int2float_rn(v);
    long long d = (long long)v - (long long)h;  // exact, |d| <= 64
    return {h, (float)d};
  }
};
template <> struct pix<ff, uint32_t> {
  static __device__ __forceinline__ ff get(const uint32_t* p, size_t i) {
    uint32_t v = p[i];
    float h = __uint2float_rn(v);
    long long d = (long long)v - (long long)h;
    return {h, (float)d};
  }
};
template <> struct pix<ff, double> {
  static __device__ __forceinline__ ff get(const double* p, size_t i) { return ff_from_double(p[i]); }
};

// ---------------------------------------------------------------------------
// warp / block reductions on scalars of type A
// ---------------------------------------------------------------------------
template <class A> __device__ __forceinline__ A shfl_down(A v, int o);
template <> __device__ __forceinline__ ff shfl_down<ff>(ff v, int o) {
  return {__shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o)};
}
template <> __device__ __forceinline__ double shfl_down<double>(double v, int o) {
  return __shfl_down_sync(0xffffffffu, v, o);
}
template <class A> __device__ __forceinline__ A shfl_up(A v, int o);
template <> __device__ __forceinline__ ff shfl_up<ff>(ff v, int o) {
  return {__shfl_up_sync(0xffffffffu, v.h, o), __shfl_up_sync(0xffffffffu, v.l, o)};
}
template <> __device__ __forceinline__ double shfl_up<double>(double v, int o) {
  return __shfl_up_sync(0xffffffffu, v, o);
}
template <class A> __device__ __forceinline__ A shfl_idx(A v, int src);
template <> __device__ __forceinline__ ff shfl_idx<ff>(ff v, int src) {
  return {__shfl_sync(0xffffffffu, v.h, src), __shfl_sync(0xffffffffu, v.l, src)};
}
template <> __device__ __forceinline__ double shfl_idx<double>(double v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

template <class A> __device__ __forceinline__ A warp_sum(A v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = sc<A>::add(v, shfl_down(v, o));
  return v;
}

// Sum of NV values per thread over the block; result broadcast to all threads.
// `scratch` holds at least NV * 32 values of A.
template <class A, int NV> __device__ __forceinline__ void block_sum(A (&v)[NV], A* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * 32 + warp] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      A x = lane < nw ? scratch[k * 32 + lane] : sc<A>::zero();
      x = warp_sum(x);
      if (lane == 0) scratch[k * 32] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = scratch[k * 32];
  __syncthreads();
}

// Exclusive block scan of one value per thread; returns the prefix and the total.
template <class A> __device__ __forceinline__ A block_exclusive_scan(A v, A* scratch, A& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  A inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    A u = shfl_up(inc, o);
    if (lane >= o) inc = sc<A>::add(inc, u);
  }
  if (lane == 31) scratch[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    A w = lane < nw ? scratch[lane] : sc<A>::zero();
    A wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      A u = shfl_up(wi, o);
      if (lane >= o) wi = sc<A>::add(wi, u);
    }
    scratch[32 + lane] = sc<A>::sub(wi, w);  // exclusive warp offsets
    if (lane == 31) scratch[64] = wi;
  }
  __syncthreads();
  A off = scratch[32 + warp];
  total = scratch[64];
  A excl = sc<A>::sub(inc, v);
  A res = sc<A>::add(off, excl);
  __syncthreads();
  return res;
}

// Exclusive block scan of `v` (returns the prefix; `total` gets the block total)
// fused with the block sums of u0 and u1 (returned in place), two barriers.
// `scratch` holds at least 96 values of A.
template <class A> __device__ __forceinline__ A block_scan_sum2(A v, A& total, A& u0, A& u1, A* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  A inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const A u = shfl_up(inc, o);
    if (lane >= o) inc = sc<A>::add(inc, u);
  }
  u0 = warp_sum(u0);
  u1 = warp_sum(u1);
  if (lane == 31) scratch[warp] = inc;
  if (lane == 0) {
    scratch[32 + warp] = u0;
    scratch[64 + warp] = u1;
  }
  __syncthreads();
  if (warp == 0) {
    const A w = lane < nw ? scratch[lane] : sc<A>::zero();
    A x0 = lane < nw ? scratch[32 + lane] : sc<A>::zero();
    A x1 = lane < nw ? scratch[64 + lane] : sc<A>::zero();
    A wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const A u = shfl_up(wi, o);
      if (lane >= o) wi = sc<A>::add(wi, u);
    }
    x0 = warp_sum(x0);
    x1 = warp_sum(x1);
    __syncwarp();
    scratch[lane] = sc<A>::sub(wi, w);  // exclusive warp offsets
    if (lane == 31) scratch[32] = wi;
    if (lane == 0) {
      scratch[33] = x0;
      scratch[34] = x1;
    }
  }
  __syncthreads();
  total = scratch[32];
  u0 = scratch[33];
  u1 = scratch[34];
  return sc<A>::add(scratch[warp], sc<A>::sub(inc, v));
}

// ---------------------------------------------------------------------------
// Asynchronous global -> shared copies (cp.async), used to prefetch the next
// mode's time series while the current one is being transformed.
// ---------------------------------------------------------------------------
template <int B> __device__ __forceinline__ void cp_async(void* smem, const void* gmem);
template <> __device__ __forceinline__ void cp_async<16>(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
template <> __device__ __forceinline__ void cp_async<8>(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Start copying one mode's T values into the (swizzled) transform buffer.
template <class S>
__device__ __forceinline__ void prefetch_series(cx<S>* buf, const cx<S>* src, int T, int tid, int nthr) {
  for (int t = tid; t < T; t += nthr) cp_async<sizeof(cx<S>)>(&buf[swz<S>(t)], src + t);
  cp_async_commit();
}

// ---------------------------------------------------------------------------
// Stage 0: window (FP64) -> S, once per call
// ---------------------------------------------------------------------------
template <class S> __global__ void k_window_convert(const double* __restrict__ w, S* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = sc<S>::from_double(w[i]);
}

// ---------------------------------------------------------------------------
// Stage 1: row pass.  Persistent CTAs walk the items (group of row pairs,
// frame) of one frame chunk.  When rows are 16-byte aligned the raw pixels of
// the next item are copied with cp.async into a double-buffered staging area
// while the current item is transformed.
// dynamic smem: swz_round(pairs * (nx + G)) * cx<S> [+ 2 * raw_stage_bytes] + nx ints
// ---------------------------------------------------------------------------
template <class S, class IN>
__device__ __forceinline__ void rows_issue_raw(const SpatialArgs& a, int item, unsigned char* raw, int ngroups,
                                               int tid, int nthr) {
  const int g = item % ngroups, tl = item / ngroups;
  const int pair0 = g * a.pairs_per_block;
  const int npairs = (a.H + 1) >> 1;
  const int np = min(a.pairs_per_block, npairs - pair0);
  const int y0 = 2 * pair0;
  const int rows = min(2 * np, a.H - y0);
  const int cpr = a.W * (int)sizeof(IN) / 16;  // 16-byte chunks per row
  const unsigned char* src = reinterpret_cast<const unsigned char*>(a.img) +
                             ((size_t)(a.t0 + tl) * a.H + y0) * (size_t)a.W * sizeof(IN);
  for (int c = tid; c < rows * cpr; c += nthr) cp_async<16>(raw + (size_t)c * 16, src + (size_t)c * 16);
  cp_async_commit();
}

template <class S, class IN, bool P2>
__global__ void __launch_bounds__(256) k_rows(SpatialArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<S>* buf = reinterpret_cast<cx<S>*>(smem_raw);
  const int nx = a.nx, W = a.W, H = a.H;
  const int npairs = (H + 1) >> 1;
  const int ngroups = (npairs + a.pairs_per_block - 1) / a.pairs_per_block;
  const int nitems = ngroups * a.tc;
  const S* win = reinterpret_cast<const S*>(a.window_s);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int nkx = a.nkx;
  const bool async_raw = a.raw_stage_bytes > 0;
  // transforms are laid out with a stride of nx plus one swizzle group, so the
  // unpack phase (several transforms read at the same permuted slot) hits
  // different banks
  const int ld = nx + swz_group<S>::G;
  const int lgnx = (nx & (nx - 1)) == 0 ? __ffs(nx) - 1 : -1;
  const bool u8_fast = sizeof(IN) == 1 && async_raw && !win && W == nx && lgnx >= 2;
  unsigned char* raw[2] = {smem_raw + (size_t)swz_round<S>(a.pairs_per_block * ld) * sizeof(cx<S>), nullptr};
  raw[1] = raw[0] + a.raw_stage_bytes;
  // the digit-reversal permutation of the row transform, read by every unpack
  // (made visible by the first item's barrier)
  int* perm = reinterpret_cast<int*>(raw[1] + a.raw_stage_bytes);
  for (int i = tid; i < nx; i += nthr) perm[i] = a.permx[i];
  int b = 0;
  if (async_raw && (int)blockIdx.x < nitems) rows_issue_raw<S, IN>(a, blockIdx.x, raw[0], ngroups, tid, nthr);

  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int g = item % ngroups, tl = item / ngroups;
    const int pair0 = g * a.pairs_per_block;
    const int np = min(a.pairs_per_block, npairs - pair0);
    const size_t t = (size_t)a.t0 + tl;
    if (async_raw) {
      cp_async_wait_all();
      __syncthreads();
      const int next = item + gridDim.x;
      if (next < nitems) rows_issue_raw<S, IN>(a, next, raw[b ^ 1], ngroups, tid, nthr);
    } else {
      __syncthreads();
    }
    const IN* img = reinterpret_cast<const IN*>(a.img) + t * (size_t)H * W;
    const IN* rimg = reinterpret_cast<const IN*>(raw[b]);
    if (u8_fast) {
      // 8-bit staged rows without padding or window: four pixels of each row
      // per 32-bit shared load, converted exactly as 2^23 + b - 2^23
      const int nq = np * (nx >> 2), lgq = lgnx - 2;
      const unsigned char* rb = reinterpret_cast<const unsigned char*>(raw[b]);
      for (int e = tid; e < nq; e += nthr) {
        const int p = e >> lgq;
        const int x0 = (e - (p << lgq)) << 2;
        const int y0 = 2 * (pair0 + p);
        const uint32_t wa = *reinterpret_cast<const uint32_t*>(rb + (size_t)(2 * p) * W + x0);
        const uint32_t wb = y0 + 1 < H ? *reinterpret_cast<const uint32_t*>(rb + (size_t)(2 * p + 1) * W + x0) : 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float fa = __fsub_rn(__int_as_float(0x4B000000 | ((wa >> (8 * k)) & 0xFFu)), 8388608.0f);
          const float fb = __fsub_rn(__int_as_float(0x4B000000 | ((wb >> (8 * k)) & 0xFFu)), 8388608.0f);
          buf[swz<S>(p * ld + x0 + k)] = {sc<S>::from_float(fa), sc<S>::from_float(fb)};
        }
      }
    } else
    for (int e = tid; e < np * nx; e += nthr) {
      const int p = lgnx >= 0 ? e >> lgnx : e / nx;
      const int x = e - p * nx;
      const int y0 = 2 * (pair0 + p);
      S va = sc<S>::zero(), vb = sc<S>::zero();
      if (x < W) {
        // staged rows are relative to the group's first row
        va = async_raw ? pix<S, IN>::get(rimg, (size_t)(2 * p) * W + x) : pix<S, IN>::get(img, (size_t)y0 * W + x);
        if (win) va = sc<S>::mul(va, win[(size_t)y0 * W + x]);
        if (y0 + 1 < H) {
          vb = async_raw ? pix<S, IN>::get(rimg, (size_t)(2 * p + 1) * W + x)
                         : pix<S, IN>::get(img, (size_t)(y0 + 1) * W + x);
          if (win) vb = sc<S>::mul(vb, win[(size_t)(y0 + 1) * W + x]);
        }
      }
      buf[swz<S>(p * ld + x)] = {va, vb};
    }
    __syncthreads();
    fft_forward<S, P2>(buf, np, ld, a.px, reinterpret_cast<const cx<S>*>(a.twx), tid, nthr);

    // unpack Z = A + iB into the spectra of the two real rows of each pair,
    // one thread per (k, pair): R[tl][k][2p] and R[tl][k][2p + 1]
    const int lgp = (np & (np - 1)) == 0 ? __ffs(np) - 1 : -1;
    cx<S>* R = reinterpret_cast<cx<S>*>(a.rbuf) + (size_t)tl * nkx * a.Hpad;
    for (int e = tid; e < np * nkx; e += nthr) {
      const int k = lgp >= 0 ? e >> lgp : e / np;
      const int p = e - k * np;
      const cx<S> zk = buf[swz<S>(p * ld + perm[k])];
      const cx<S> zn = buf[swz<S>(p * ld + perm[k == 0 ? 0 : nx - k])];
      cx<S>* dst = R + (size_t)k * a.Hpad + 2 * (pair0 + p);
      dst[0] = {sc<S>::half(sc<S>::add(zk.r, zn.r)), sc<S>::half(sc<S>::sub(zk.i, zn.i))};
      dst[1] = {sc<S>::half(sc<S>::add(zk.i, zn.i)), sc<S>::half(sc<S>::sub(zn.r, zk.r))};
    }
    b ^= 1;
  }
}

// ---------------------------------------------------------------------------
// Stage 2: column pass.  Persistent CTAs walk the items (group of columns,
// group of frames) of one frame chunk; the next item's columns are copied with
// cp.async into the second of two transform buffers while the current item
// is transformed.
// dynamic smem: 2 * swz_round(cols * frames * (ny + G)) * cx<S> + ny ints
// ---------------------------------------------------------------------------
template <class S>
__device__ __forceinline__ void cols_issue(const SpatialArgs& a, int item, cx<S>* buf, int ncg, int ld, int tid,
                                           int nthr) {
  const int ny = a.ny, H = a.H, nkx = a.nkx;
  const int CK = a.cols_per_block, TG = a.frames_per_block, NB = CK * TG;
  const int kc0 = (item % ncg) * CK, tl0 = (item / ncg) * TG;
  const int nk = min(CK, nkx - kc0), ntg = min(TG, a.tc - tl0);
  const cx<S>* R = reinterpret_cast<const cx<S>*>(a.rbuf);
  const int lgny = (ny & (ny - 1)) == 0 ? __ffs(ny) - 1 : -1;
  const int lgCK = (CK & (CK - 1)) == 0 ? __ffs(CK) - 1 : -1;
  for (int e = tid; e < NB * ny; e += nthr) {
    const int c = lgny >= 0 ? e >> lgny : e / ny;
    const int y = e - c * ny;
    const int tl = lgCK >= 0 ? c >> lgCK : c / CK;
    const int kc = c - tl * CK;
    cx<S>* dst = &buf[swz<S>(c * ld + y)];
    if (kc < nk && tl < ntg && y < H) cp_async<sizeof(cx<S>)>(dst, &R[((size_t)(tl0 + tl) * nkx + kc0 + kc) * a.Hpad + y]);
    else *dst = czero<S>();
  }
  cp_async_commit();
}

// Store phase of the column pass: scale by 1/sqrt(nx ny), apply the y-fftshift and
// write F[q][t].  P2: the scale is a power of two and one multiply per word is exact.
template <class S, bool P2>
__device__ __forceinline__ void cols_store(const SpatialArgs& a, const cx<S>* buf, const int* __restrict__ perm,
                                           cx<S>* F, int ld, int kc0, int tl0, int nk, int ntg, int lgTG, int lgCK,
                                           S norm, int tid, int nthr) {
  const int ny = a.ny, nkx = a.nkx, CK = a.cols_per_block, TG = a.frames_per_block;
  const int half = ny >> 1;
  for (int e = tid; e < CK * TG * ny; e += nthr) {
    int tl, rest, kc, ky;
    if (lgTG >= 0) { tl = e & (TG - 1); rest = e >> lgTG; } else { tl = e % TG; rest = e / TG; }
    if (lgCK >= 0) { kc = rest & (CK - 1); ky = rest >> lgCK; } else { kc = rest % CK; ky = rest / CK; }
    if (tl < ntg && kc < nk) {
      const cx<S> z = buf[swz<S>((tl * CK + kc) * ld + perm[ky])];
      cx<S> v;
      if constexpr (P2) {
        v = {sc<S>::mul_p2(z.r, a.norm_h), sc<S>::mul_p2(z.i, a.norm_h)};
      } else {
        v = cscale(z, norm);
      }
      int ys = ky + half;
      if (ys >= ny) ys -= ny;
      const size_t q = (size_t)ys * nkx + kc0 + kc;
      F[q * a.Tpad + a.t0 + tl0 + tl] = v;
    }
  }
}

template <class S, bool P2>
__global__ void __launch_bounds__(512) k_cols(SpatialArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ny = a.ny, nkx = a.nkx;
  const int CK = a.cols_per_block, TG = a.frames_per_block, NB = CK * TG;
  const int ncg = (nkx + CK - 1) / CK;
  const int nitems = ncg * ((a.tc + TG - 1) / TG);
  const int ld = ny + swz_group<S>::G;  // padded stride: the store phase reads NB transforms at one slot
  cx<S>* bufs[2] = {reinterpret_cast<cx<S>*>(smem_raw), reinterpret_cast<cx<S>*>(smem_raw) + swz_round<S>(NB * ld)};
  const int lgTG = (TG & (TG - 1)) == 0 ? __ffs(TG) - 1 : -1;
  const int lgCK = (CK & (CK - 1)) == 0 ? __ffs(CK) - 1 : -1;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const S norm = sc<S>::cst(a.norm_h, a.norm_l, a.norm_d);
  // 1/sqrt(nx ny) is a power of two when nx ny is a power of four: exact scaling
  const bool norm_p2 = a.norm_l == 0.0f && (__float_as_uint(a.norm_h) & 0x007FFFFFu) == 0u;
  cx<S>* F = reinterpret_cast<cx<S>*>(a.spec);
  // the digit-reversal permutation of the column transform, read by every store
  // (made visible by the first item's barrier)
  int* perm = reinterpret_cast<int*>(bufs[1] + swz_round<S>(NB * ld));
  for (int i = tid; i < ny; i += nthr) perm[i] = a.permy[i];
  int b = 0;
  if ((int)blockIdx.x < nitems) cols_issue<S>(a, blockIdx.x, bufs[0], ncg, ld, tid, nthr);

  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    cp_async_wait_all();
    __syncthreads();
    const int next = item + gridDim.x;
    if (next < nitems) cols_issue<S>(a, next, bufs[b ^ 1], ncg, ld, tid, nthr);
    cx<S>* buf = bufs[b];
    const int kc0 = (item % ncg) * CK, tl0 = (item / ncg) * TG;
    const int nk = min(CK, nkx - kc0), ntg = min(TG, a.tc - tl0);
    fft_forward<S, P2>(buf, NB, ld, a.py, reinterpret_cast<const cx<S>*>(a.twy), tid, nthr);
    if (norm_p2)
      cols_store<S, true>(a, buf, perm, F, ld, kc0, tl0, nk, ntg, lgTG, lgCK, norm, tid, nthr);
    else
      cols_store<S, false>(a, buf, perm, F, ld, kc0, tl0, nk, ntg, lgTG, lgCK, norm, tid, nthr);
    b ^= 1;
  }
}

// ---------------------------------------------------------------------------
// shared per-q statistics: PS, <F>, VAR
// ---------------------------------------------------------------------------
template <class S, class A> struct cvt;
template <> struct cvt<ff, ff> {
  static __device__ __forceinline__ ff to_acc(ff v) { return v; }
  static __device__ __forceinline__ ff to_fft(ff v) { return v; }
};
template <> struct cvt<float, ff> {
  static __device__ __forceinline__ ff to_acc(float v) { return {v, 0.0f}; }
  static __device__ __forceinline__ float to_fft(ff v) { return __fadd_rn(v.h, v.l); }
};
template <> struct cvt<double, double> {
  static __device__ __forceinline__ double to_acc(double v) { return v; }
  static __device__ __forceinline__ double to_fft(double v) { return v; }
};

// ---------------------------------------------------------------------------
// Stage 3 (fft mode), one q per CTA iteration:
//   G = F - <F>_t (D is unchanged by a time-constant offset; VAR = <|G|^2>)
//   S1(lag) + S2(lag) from prefix sums of |G|^2, kept only at the indices the
//   lags need
//   X = FFT_N(G zero-padded), P = |X|^2 (real)
//   Re C(lag) = (1/N) Re DFT_N(P)(lag) (cos is even, so the forward transform
//   serves), evaluated through one half-length complex transform of
//   z[m] = P(2m) + i P(2m+1) and a per-lag post-process, only at the lags
//   D(lag) = (S1 + S2 - 2 Re C) / (T - lag)
// Lags with T - lag <= kDirect are summed directly from the saved first and
// last kDirect values of G: there the Wiener-Khinchin form would amplify its
// rounding error by T / (T - lag).
//
// The length-N forward FFT leaves X(k) at the digit-reversed position
// p(k) = m_0 M_1 + r with m_0 = k mod R_0 and r fixed by the higher digits.
// For even R_0, P(2m) and P(2m+1) sit at (2a) M_1 + r and (2a+1) M_1 + r, and
// a M_1 + r is exactly where the half-length plan (R_0/2, R_1, ...) keeps
// element m in its own digit-reversed order.  So conj(z) is formed in place
// without any permutation table, and the inverse passes of the half plan
// (digit-reversed in, natural out) give Y = conj(DFT_{N/2}(z)) in natural order.
//
// Shared memory (temporal_fft_smem): buf (the larger of N and
// swz_round(N/2) + swz_round(T) elements; the next mode's series is prefetched
// to buf + swz_round(N/2) while the half-length transform runs below it),
// head, tail (kDirect each), reduction scratch, the lag slot tables (int16,
// loaded once per CTA) and, when they fit, the needed prefix sums (else
// per-CTA global scratch).
// ---------------------------------------------------------------------------
constexpr int kDirect = 32;

// P = |X|^2 of one length-N forward transform, paired in place as
// conj(z[m]) = P(2m) - i P(2m+1) at the half plan's position a M_1 + r.  A
// thread owns the R0 positions j M_1 + r of its r: it reads all of them
// before writing, and no other thread touches them.
template <class S, int R0>
__device__ __forceinline__ void pair_power(cx<S>* __restrict__ buf, int M1, int tid, int nthr) {
  for (int r = tid; r < M1; r += nthr) {
    S pw[R0];
#pragma unroll
    for (int j = 0; j < R0; ++j) {
      const cx<S> x = buf[swz<S>(j * M1 + r)];
      pw[j] = sc<S>::sqsum(x.r, x.i);
    }
#pragma unroll
    for (int h = 0; h < R0 / 2; ++h) buf[swz<S>(h * M1 + r)] = {pw[2 * h], sc<S>::neg(pw[2 * h + 1])};
  }
}

// Plans whose first radix is 2 (F2 path of the temporal kernel): the length-N
// forward transform's last pass (radix R, stride 1), the pairing of P(2m) at
// position p with P(2m+1) at N/2 + p, and the half plan's first inverse pass
// (the same radix R, stride 1, no twiddles) run as one step: the thread that
// transforms block b of the lower half and block b of the upper half holds
// both powers of every position of block b and transforms them on in
// registers, writing only the lower half.
template <class S, int R>
__device__ __forceinline__ void last_pass_pair_first_inverse(cx<S>* __restrict__ buf, int N2, int tid, int nthr) {
  for (int b = tid; b < N2 / R; b += nthr) {
    cx<S> v[R], u[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = buf[swz<S>(b * R + i)];
    dft<S, R, false>(v);
#pragma unroll
    for (int i = 0; i < R; ++i) u[i] = buf[swz<S>(N2 + b * R + i)];
    dft<S, R, false>(u);
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = {sc<S>::sqsum(v[i].r, v[i].i), sc<S>::neg(sc<S>::sqsum(u[i].r, u[i].i))};
    dft<S, R, true>(v);
#pragma unroll
    for (int i = 0; i < R; ++i) buf[swz<S>(b * R + i)] = v[i];
  }
}

// F2: first radix 2, N/2 a multiple of the swizzle group and all radices 2, 4
// or 8 (host: fused_radix2_ok).  The padded radix-2 first pass is folded into
// the pass over the series (G at t and G w_N^t at N/2 + t), and the last
// forward pass, the pairing and the first inverse pass run as one step.
// Modes q_first, q_first + q_step, ... below q_stop of the job described by `a`.
template <class S, class A, bool P2, bool F2 = false>
__device__ __forceinline__ void tfft_body(const TemporalArgs& a, size_t q_first, size_t q_stop, size_t q_step) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = a.T, N = a.nt, N2 = a.nt / 2, nl = a.nlags;
  cx<S>* buf = reinterpret_cast<cx<S>*>(smem_raw);
  const int up = swz_round<S>(N2);
  cx<S>* ser = buf + up;  // the prefetched series of the next mode
  cx<S>* head = buf + max(swz_round<S>(N), up + swz_round<S>(T));
  cx<S>* tail = head + kDirect;
  A* scratch = reinterpret_cast<A*>(tail + kDirect);
  short* slotA = reinterpret_cast<short*>(scratch + 96);
  short* slotB = slotA + (T + 1);
  // need[] and the per-lag tables in shared memory (a.need_in_smem), else need[] in global scratch
  A* need = a.need_in_smem
                ? reinterpret_cast<A*>(smem_raw + ((reinterpret_cast<unsigned char*>(slotB + (T + 1)) - smem_raw + 15) & ~15))
                : reinterpret_cast<A*>(a.need) + (size_t)blockIdx.x * (2 * nl + 2);
  // per-lag tables: w^tau, 1/(T - tau), tau (addresses recomputed where used)
#define FDDM_LAG_W reinterpret_cast<cx<S>*>(smem_raw + ((reinterpret_cast<unsigned char*>(need + 2 * nl + 2) - smem_raw + 15) & ~15))
#define FDDM_LAG_RCP reinterpret_cast<double*>(FDDM_LAG_W + nl)
#define FDDM_LAG_TAU reinterpret_cast<int*>(FDDM_LAG_RCP + nl)
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
  const cx<S>* F = reinterpret_cast<const cx<S>*>(a.spec);
  const cx<S>* tw = reinterpret_cast<const cx<S>*>(a.twt);
  const cx<S>* p0tw = reinterpret_cast<const cx<S>*>(a.pt.ptw[0]);  // w_N^t, the radix-2 first pass's table
  const A invT = sc<A>::cst(a.invT_h, a.invT_l, a.invT_d);
  const A invN = sc<A>::cst(a.invnt_h, a.invnt_l, a.invnt_d);
  const int chunk = (T + nthr - 1) / nthr;
  const int tail0 = T - kDirect;  // first index kept in `tail` (may be negative)
  const int R0 = a.pt.radix[0], M1 = N / R0;
  const int nref = min(T, 32);  // samples of the reference offset

  for (int t = tid; t <= T; t += nthr) {
    slotA[t] = (short)a.slotA[t];
    slotB[t] = (short)a.slotB[t];
  }
  if (a.need_in_smem) {
    for (int l = tid; l < nl; l += nthr) {
      const int tau = a.lags[l];
      FDDM_LAG_TAU[l] = tau;
      FDDM_LAG_RCP[l] = a.rcp[l];
      FDDM_LAG_W[l] = tw[tau];
    }
  }
  if (q_first < q_stop) prefetch_series<S>(ser, F + q_first * a.Tpad, T, tid, nthr);

  for (size_t q = q_first; q < q_stop; q += q_step) {
    cp_async_wait_all();
    __syncthreads();

    // Reference offset m: the mean of 32 samples spread evenly over the series
    // (all of them when T < 32), computed identically by every warp, so no
    // barrier is needed.  D is unchanged by any time-constant offset, and with
    // G = F - m the Wiener-Khinchin cancellation stays near (VAR + |<F> - m|^2)/D
    // instead of PS/D, where |<F> - m|^2 is about VAR/32 for samples this far
    // apart.  PS and VAR follow exactly from the sums of G below.
    A mr = sc<A>::zero(), mi = sc<A>::zero();
    if (lane < nref) {
      const cx<S> f = ser[swz<S>(T >= 32 ? (int)(((long long)lane * T) >> 5) : lane)];
      mr = cvt<S, A>::to_acc(f.r);
      mi = cvt<S, A>::to_acc(f.i);
    }
    mr = shfl_idx(warp_sum(mr), 0);
    mi = shfl_idx(warp_sum(mi), 0);
    const A inv_ref = sc<A>::from_double(1.0 / nref);
    const S msr = cvt<S, A>::to_fft(sc<A>::mul(mr, inv_ref)), msi = cvt<S, A>::to_fft(sc<A>::mul(mi, inv_ref));
    if (F2) __syncthreads();  // the upper half written below overlays the series every warp just sampled

    // G = F - m into buf[0, T), over a contiguous chunk per thread: sums of G
    // and of |G|^2 for the statistics and the prefix sums
    const int t_beg = min(T, tid * chunk), t_end = min(T, t_beg + chunk);
    A run = sc<A>::zero(), sgr = sc<A>::zero(), sgi = sc<A>::zero();
    for (int t = t_beg; t < t_end; ++t) {
      cx<S> g = ser[swz<S>(t)];
      g.r = sc<S>::sub(g.r, msr);
      g.i = sc<S>::sub(g.i, msi);
      buf[swz<S>(t)] = g;
      // the padded radix-2 first pass: x_t and x_t w_N^t (N/2 + t is the slot of ser[t] itself)
      if (F2) buf[swz<S>(N2 + t)] = twmul<S>::mul(g, p0tw[t]);
      if (t < kDirect) head[t] = g;
      if (t >= tail0) tail[t - tail0] = g;
      const A gr = cvt<S, A>::to_acc(g.r), gi = cvt<S, A>::to_acc(g.i);
      run = sc<A>::add(run, sc<A>::sqsum(gr, gi));
      sgr = sc<A>::add(sgr, gr);
      sgi = sc<A>::add(sgi, gi);
    }
    A total;  // also left in scratch[32] (the sums of G in [33], [34]) until the next mode's scan
    A pre = block_scan_sum2<A>(run, total, sgr, sgi, scratch);
    // prefix sums pfx[t + 1] = sum_{s <= t} |G(s)|^2, stored at the slots the lags need
    for (int t = t_beg; t < t_end; ++t) {
      const cx<S> g = buf[swz<S>(t)];
      pre = sc<A>::add(pre, sc<A>::sqsum(cvt<S, A>::to_acc(g.r), cvt<S, A>::to_acc(g.i)));
      const int sa = slotA[t + 1], sb = slotB[t + 1];
      if (sa >= 0) need[sa] = pre;
      if (sb >= 0) need[nl + sb] = pre;
    }
    if (tid == 0 && slotB[0] >= 0) need[nl + slotB[0]] = sc<A>::zero();
    if (F2) {
      for (int t = T + tid; t < N2; t += nthr) {
        buf[swz<S>(t)] = czero<S>();
        buf[swz<S>(N2 + t)] = czero<S>();
      }
    }
    __syncthreads();

    if (F2) {
      const int np = a.pt.npass;
      for (int s = 1; s < np - 1; ++s) {
        fft_pass_dispatch<S, false, true>(buf, 1, N, a.pt, s, tw, N, tid, nthr);
        __syncthreads();
      }
      const int R = a.pt.radix[np - 1];
      if (R == 8) last_pass_pair_first_inverse<S, 8>(buf, N2, tid, nthr);
      else if (R == 4) last_pass_pair_first_inverse<S, 4>(buf, N2, tid, nthr);
      else last_pass_pair_first_inverse<S, 2>(buf, N2, tid, nthr);
      __syncthreads();
      if (q + q_step < q_stop) prefetch_series<S>(ser, F + (q + q_step) * a.Tpad, T, tid, nthr);
      // remaining inverse passes of the half plan (its last pass ran above)
      for (int s = a.pt2.npass - 2; s >= 0; --s) {
        fft_pass_dispatch<S, true, true>(buf, 1, N2, a.pt2, s, tw, N, tid, nthr);
        __syncthreads();
      }
    } else {
      fft_forward_padded<S, P2>(buf, a.pt, T, tw, tid, nthr);
      if (R0 == 8) pair_power<S, 8>(buf, M1, tid, nthr);
      else if (R0 == 4) pair_power<S, 4>(buf, M1, tid, nthr);
      else pair_power<S, 2>(buf, M1, tid, nthr);
      __syncthreads();
      // buf above the half-length transform is free: start loading the next mode
      if (q + q_step < q_stop) prefetch_series<S>(ser, F + (q + q_step) * a.Tpad, T, tid, nthr);
      // the length-N table serves the half-length passes: w_M^k = tw[k N / M]
      fft_inverse<S, P2>(buf, 1, N2, a.pt2, tw, tid, nthr, N);
    }

    total = scratch[32];
    // PS and VAR, by the thread after the last lag (off the barrier-bound path of the transform):
    // <G> (rounding-size), VAR = <|G|^2> - |<G>|^2, PS = <|G|^2> + 2 Re(conj(m) <G>) + |m|^2
    if (tid == (nl < nthr ? nl : nthr - 1)) {
      const A gmr = sc<A>::mul(scratch[33], invT), gmi = sc<A>::mul(scratch[34], invT);
      const A g2 = sc<A>::mul(total, invT);
      const A mr = cvt<S, A>::to_acc(msr), mi = cvt<S, A>::to_acc(msi);
      const A cross = sc<A>::add(sc<A>::mul(mr, gmr), sc<A>::mul(mi, gmi));
      const A ps = sc<A>::add(sc<A>::add(g2, sc<A>::add(cross, cross)), sc<A>::sqsum(mr, mi));
      a.out[(size_t)nl * a.Q + q] = sc<A>::to_double(ps);
      a.out[(size_t)(nl + 1) * a.Q + q] = sc<A>::to_double(sc<A>::sub(g2, sc<A>::sqsum(gmr, gmi)));
    }
    for (int l = tid; l < nl; l += nthr) {
      const int tau = a.need_in_smem ? FDDM_LAG_TAU[l] : a.lags[l];
      if (T - tau <= kDirect) continue;
      // Y = conj(Z), Z = DFT_{N/2}(z), in natural order
      const cx<S> yk = buf[swz<S>(tau)];
      const cx<S> yn = buf[swz<S>(tau == 0 ? 0 : N2 - tau)];
      // DFT_N(P)(tau) = Xe + w^tau Xo with Xe = (Zk + conj Zn)/2, Xo = (Zk - conj Zn)/(2i);
      // y is twice its real part
      const S xe = sc<S>::add(yk.r, yn.r);
      const cx<S> xo = {sc<S>::neg(sc<S>::add(yk.i, yn.i)), sc<S>::sub(yn.r, yk.r)};
      const cx<S> w = a.need_in_smem ? FDDM_LAG_W[l] : tw[tau];
      const S y = sc<S>::add(xe, sc<S>::sub(sc<S>::mul(w.r, xo.r), sc<S>::mul(w.i, xo.i)));
      // 2 Re C = y / N
      const A c2 = sc<A>::mul(cvt<S, A>::to_acc(y), invN);
      A num = sc<A>::add(need[l], sc<A>::sub(total, need[nl + l]));
      num = sc<A>::sub(num, c2);
      a.out[(size_t)l * a.Q + q] = sc<A>::to_double(num) * (a.need_in_smem ? FDDM_LAG_RCP[l] : a.rcp[l]);
    }
    // the last lags: direct differences
    for (int l = nl - 1 - warp; l >= 0; l -= nw) {
      const int tau = a.need_in_smem ? FDDM_LAG_TAU[l] : a.lags[l];
      const int m = T - tau;
      if (m > kDirect) break;
      A acc = sc<A>::zero();
      for (int t = lane; t < m; t += 32) {
        const cx<S> g1 = tail[t + tau - tail0], g0 = head[t];
        const A dr = sc<A>::sub(cvt<S, A>::to_acc(g1.r), cvt<S, A>::to_acc(g0.r));
        const A di = sc<A>::sub(cvt<S, A>::to_acc(g1.i), cvt<S, A>::to_acc(g0.i));
        acc = sc<A>::add(acc, sc<A>::sqsum(dr, di));
      }
      acc = warp_sum(acc);
      if (lane == 0) a.out[(size_t)l * a.Q + q] = sc<A>::to_double(acc) * (a.need_in_smem ? FDDM_LAG_RCP[l] : a.rcp[l]);
    }
    __syncthreads();
  }
#undef FDDM_LAG_W
#undef FDDM_LAG_RCP
#undef FDDM_LAG_TAU
}

template <class S, class A, bool P2, bool F2 = false>
__global__ void __launch_bounds__(512) k_tfft(TemporalArgs a) {
  tfft_body<S, A, P2, F2>(a, a.q_begin + blockIdx.x, a.q_end, gridDim.x);
}
// FP32 transforms: two 512-thread CTAs per SM (their shared memory allows it)
template <class S, class A, bool P2, bool F2 = false>
__global__ void __launch_bounds__(512, 2) k_tfft_x2(TemporalArgs a) {
  tfft_body<S, A, P2, F2>(a, a.q_begin + blockIdx.x, a.q_end, gridDim.x);
}

// Many jobs in one persistent launch: CTAs take work items (a run of
// consecutive modes of one job) from a counter in global memory, copy the
// job's arguments to shared memory and run the same per-mode body as k_tfft,
// so every mode gives the result it gives in a launch of its own job.  The
// counter starts at zero (set by the host before the launch); taking an item
// is one atomic add, and no CTA ever waits on another.
template <class S, class A, bool P2, bool F2>
__device__ __forceinline__ void tfft_list_body(const TemporalArgs* __restrict__ jobs,
                                               const TemporalItem* __restrict__ items, int nitems,
                                               int* __restrict__ counter) {
  __shared__ __align__(16) TemporalArgs s_args;
  __shared__ int s_item;
  constexpr int kWords = (int)(sizeof(TemporalArgs) / sizeof(int));
  static_assert(sizeof(TemporalArgs) % sizeof(int) == 0, "TemporalArgs copied as ints");
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const TemporalItem w = items[it];
    const int* src = reinterpret_cast<const int*>(jobs + w.job);
    int* dst = reinterpret_cast<int*>(&s_args);
    for (int i = threadIdx.x; i < kWords; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    tfft_body<S, A, P2, F2>(s_args, (size_t)w.q0, (size_t)w.q1, 1);
    __syncthreads();
  }
}
template <class S, class A, bool P2, bool F2 = false>
__global__ void __launch_bounds__(512) k_tfft_list(const TemporalArgs* __restrict__ jobs,
                                                   const TemporalItem* __restrict__ items, int nitems,
                                                   int* __restrict__ counter) {
  tfft_list_body<S, A, P2, F2>(jobs, items, nitems, counter);
}
template <class S, class A, bool P2, bool F2 = false>
__global__ void __launch_bounds__(512, 2) k_tfft_list_x2(const TemporalArgs* __restrict__ jobs,
                                                         const TemporalItem* __restrict__ items, int nitems,
                                                         int* __restrict__ counter) {
  tfft_list_body<S, A, P2, F2>(jobs, items, nitems, counter);
}

// ---------------------------------------------------------------------------
// Stage 3 (fft mode) for series whose length-N transform does not fit in
// shared memory.  N = R0 M1 (R0 in {2, 4, 8}): the first DIF pass runs from
// the spectrum into the CTA's global scratch X, the length-M1 sub-transforms
// run in shared memory.  Per q:
//   A  reference offset m from 32 spread samples (as in k_tfft)
//   B  G = F - m: warp-segmented inclusive prefix sums of |G|^2 into the
//      global scratch, sums of G and |G|^2 (PS, VAR), the first and last
//      kDirect values of G into shared memory
//   C  first pass (radix R0, zero-padded input read from the spectrum) into
//      X[m M1 + j]
//   D  for h < R0/2: sub-blocks 2h and 2h+1 through the remaining forward
//      passes, paired into conj(z) exactly as pair_power does, through the
//      inverse passes of the half plan below its first pass, and stored to
//      X[h M1 + r] (region h was read in this or an earlier iteration)
//   E  the half plan's first inverse pass (radix R0/2, stride M1) evaluated
//      only at the outputs the lags need
//   F  D(lag) as in k_tfft
// dynamic smem (temporal_long_smem): swz_round(M1) cx<S> + M1 S (16-byte
// aligned) + 2 kDirect cx<S> + 160 A
// ---------------------------------------------------------------------------
template <class S, int R0>
__device__ __forceinline__ void long_first_pass(const cx<S>* __restrict__ src, cx<S>* __restrict__ X, int T, int M1,
                                                S msr, S msi, const cx<S>* __restrict__ tw, int tid, int nthr) {
  for (int j = tid; j < M1; j += nthr) {
    cx<S> v[R0], w[R0];
#pragma unroll
    for (int m = 1; m < R0; ++m) w[m] = tw[j * m];  // w^0 = 1 exactly: no j = 0 branch
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      const int t = j + r * M1;
      if (r < R0 / 2 && t < T) {
        const cx<S> f = src[t];
        v[r] = {sc<S>::sub(f.r, msr), sc<S>::sub(f.i, msi)};
      } else {
        v[r] = czero<S>();
      }
    }
    dft_halfzero<S, R0>(v);
#pragma unroll
    for (int m = 1; m < R0; ++m) v[m] = twmul<S>::mul(v[m], w[m]);
#pragma unroll
    for (int m = 0; m < R0; ++m) X[j + m * M1] = v[m];
  }
}

// v * i^e
template <class S> __device__ __forceinline__ cx<S> mul_ipow(cx<S> v, int e) {
  switch (e & 3) {
    case 0: return v;
    case 1: return {sc<S>::neg(v.i), v.r};
    case 2: return {sc<S>::neg(v.r), sc<S>::neg(v.i)};
    default: return {v.i, sc<S>::neg(v.r)};
  }
}

// Output k of the half plan's first inverse pass (radix R, stride M1, length
// R M1) from its input Z; twiddles w_{R M1}^{j r} = w_N^{2 j r}.
template <class S, int R>
__device__ __forceinline__ cx<S> half_first_inverse_at(const cx<S>* Z, int k, int M1, const cx<S>* twN) {
  const int j = k % M1, m = k / M1;
  cx<S> y = Z[j];
#pragma unroll
  for (int r = 1; r < R; ++r) {
    cx<S> v = Z[j + r * M1];
    if (j != 0) v = twmul<S>::mulc(v, twN[2 * j * r]);
    y = cadd(y, mul_ipow(v, r * m * (4 / R)));  // w_R^(-r m) = i^(4 r m / R)
  }
  return y;
}

template <class S, class A>
__global__ void __launch_bounds__(512) k_tfft_long(TemporalArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = a.T, N2 = a.nt / 2, nl = a.nlags, M1 = a.M1, R0 = a.R0;
  cx<S>* buf = reinterpret_cast<cx<S>*>(smem_raw);
  S* pe = reinterpret_cast<S*>(buf + swz_round<S>(M1));
  cx<S>* head = reinterpret_cast<cx<S>*>(smem_raw + (((reinterpret_cast<unsigned char*>(pe + M1) - smem_raw) + 15) & ~15));
  cx<S>* tail = head + kDirect;
  A* scratch = reinterpret_cast<A*>(tail + kDirect);
  A* woff = scratch + 96;  // exclusive prefix of the warp segments' totals, then the total
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
  const cx<S>* F = reinterpret_cast<const cx<S>*>(a.spec);
  const cx<S>* tw = reinterpret_cast<const cx<S>*>(a.twt);
  const cx<S>* twm = reinterpret_cast<const cx<S>*>(a.twm);
  unsigned char* xs = static_cast<unsigned char*>(a.xs) + (size_t)blockIdx.x * a.xs_stride;
  cx<S>* X = reinterpret_cast<cx<S>*>(xs);
  A* P = reinterpret_cast<A*>(xs + a.xs_pfx_off);
  const A invT = sc<A>::cst(a.invT_h, a.invT_l, a.invT_d);
  const A invN = sc<A>::cst(a.invnt_h, a.invnt_l, a.invnt_d);
  const int tail0 = T - kDirect;
  const int seg = ((T + nw - 1) / nw + 31) / 32 * 32;  // warp segment of the prefix sums
  const int nref = min(T, 32);  // samples of the reference offset

  for (size_t q = a.q_begin + blockIdx.x; q < a.q_end; q += gridDim.x) {
    const cx<S>* src = F + q * a.Tpad;
    // A: reference offset m, the mean of 32 samples spread over the series (as
    // in k_tfft); PS and VAR follow from the sums of G = F - m in B
    A mr = sc<A>::zero(), mi = sc<A>::zero();
    if (lane < nref) {
      const cx<S> f = src[T >= 32 ? (int)(((long long)lane * T) >> 5) : lane];
      mr = cvt<S, A>::to_acc(f.r);
      mi = cvt<S, A>::to_acc(f.i);
    }
    mr = shfl_idx(warp_sum(mr), 0);
    mi = shfl_idx(warp_sum(mi), 0);
    const A inv_ref = sc<A>::from_double(1.0 / nref);
    const S msr = cvt<S, A>::to_fft(sc<A>::mul(mr, inv_ref)), msi = cvt<S, A>::to_fft(sc<A>::mul(mi, inv_ref));

    // B
    {
      const int s0 = warp * seg, s1 = min(T, s0 + seg);
      A carry = sc<A>::zero(), sgr = sc<A>::zero(), sgi = sc<A>::zero();
      for (int t0 = s0; t0 < s1; t0 += 32) {
        const int t = t0 + lane;
        A e = sc<A>::zero();
        if (t < s1) {
          cx<S> g = src[t];
          g.r = sc<S>::sub(g.r, msr);
          g.i = sc<S>::sub(g.i, msi);
          if (t < kDirect) head[t] = g;
          if (t >= tail0) tail[t - tail0] = g;
          const A gr = cvt<S, A>::to_acc(g.r), gi = cvt<S, A>::to_acc(g.i);
          e = sc<A>::sqsum(gr, gi);
          sgr = sc<A>::add(sgr, gr);
          sgi = sc<A>::add(sgi, gi);
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const A u = shfl_up(e, o);
          if (lane >= o) e = sc<A>::add(e, u);
        }
        const A inc = sc<A>::add(carry, e);
        if (t < s1) P[t] = inc;
        carry = shfl_idx(inc, 31);
      }
      sgr = warp_sum(sgr);
      sgi = warp_sum(sgi);
      if (lane == 0) {
        scratch[warp] = carry;
        scratch[32 + warp] = sgr;
        scratch[64 + warp] = sgi;
      }
      __syncthreads();
      if (warp == 0) {
        const A w = lane < nw ? scratch[lane] : sc<A>::zero();
        A x0 = lane < nw ? scratch[32 + lane] : sc<A>::zero();
        A x1 = lane < nw ? scratch[64 + lane] : sc<A>::zero();
        A wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const A u = shfl_up(wi, o);
          if (lane >= o) wi = sc<A>::add(wi, u);
        }
        x0 = warp_sum(x0);
        x1 = warp_sum(x1);
        const A tot = shfl_idx(wi, 31);
        woff[lane] = sc<A>::sub(wi, w);
        if (lane == 31) woff[32] = wi;
        if (lane == 0) {
          // <G> (rounding-size), VAR = <|G|^2> - |<G>|^2, PS = <|G|^2> + 2 Re(conj(m) <G>) + |m|^2
          const A gmr = sc<A>::mul(x0, invT), gmi = sc<A>::mul(x1, invT);
          const A g2 = sc<A>::mul(tot, invT);
          const A mr2 = cvt<S, A>::to_acc(msr), mi2 = cvt<S, A>::to_acc(msi);
          const A cross = sc<A>::add(sc<A>::mul(mr2, gmr), sc<A>::mul(mi2, gmi));
          const A ps = sc<A>::add(sc<A>::add(g2, sc<A>::add(cross, cross)), sc<A>::sqsum(mr2, mi2));
          a.out[(size_t)nl * a.Q + q] = sc<A>::to_double(ps);
          a.out[(size_t)(nl + 1) * a.Q + q] = sc<A>::to_double(sc<A>::sub(g2, sc<A>::sqsum(gmr, gmi)));
        }
      }
    }

    // C (the spectrum is read again; X is free since the last iteration ended)
    if (R0 == 8) long_first_pass<S, 8>(src, X, T, M1, msr, msi, tw, tid, nthr);
    else if (R0 == 4) long_first_pass<S, 4>(src, X, T, M1, msr, msi, tw, tid, nthr);
    else long_first_pass<S, 2>(src, X, T, M1, msr, msi, tw, tid, nthr);
    __syncthreads();

    // D
    for (int h = 0; h < R0 / 2; ++h) {
      const cx<S>* xe = X + (size_t)(2 * h) * M1;
      for (int u = tid; u < M1; u += nthr) buf[swz<S>(u)] = xe[u];
      __syncthreads();
      fft_forward<S>(buf, 1, M1, a.pm, twm, tid, nthr);
      for (int u = tid; u < M1; u += nthr) {
        const cx<S> x = buf[swz<S>(u)];
        pe[u] = sc<S>::sqsum(x.r, x.i);
      }
      __syncthreads();
      const cx<S>* xo = X + (size_t)(2 * h + 1) * M1;
      for (int u = tid; u < M1; u += nthr) buf[swz<S>(u)] = xo[u];
      __syncthreads();
      fft_forward<S>(buf, 1, M1, a.pm, twm, tid, nthr);
      for (int u = tid; u < M1; u += nthr) {
        const cx<S> x = buf[swz<S>(u)];
        buf[swz<S>(u)] = {pe[u], sc<S>::neg(sc<S>::sqsum(x.r, x.i))};
      }
      __syncthreads();
      fft_inverse<S>(buf, 1, M1, a.pm, twm, tid, nthr);
      cx<S>* z = X + (size_t)h * M1;
      for (int u = tid; u < M1; u += nthr) z[u] = buf[swz<S>(u)];
      __syncthreads();
    }

    // E, F
    const A total = woff[32];
    for (int l = tid; l < nl; l += nthr) {
      const int tau = a.lags[l];
      if (T - tau <= kDirect) continue;
      const int kn = tau == 0 ? 0 : N2 - tau;
      cx<S> yk, yn;
      if (R0 == 8) {
        yk = half_first_inverse_at<S, 4>(X, tau, M1, tw);
        yn = half_first_inverse_at<S, 4>(X, kn, M1, tw);
      } else if (R0 == 4) {
        yk = half_first_inverse_at<S, 2>(X, tau, M1, tw);
        yn = half_first_inverse_at<S, 2>(X, kn, M1, tw);
      } else {
        yk = X[tau];
        yn = X[kn];
      }
      const S xe = sc<S>::add(yk.r, yn.r);
      const cx<S> xo = {sc<S>::neg(sc<S>::add(yk.i, yn.i)), sc<S>::sub(yn.r, yk.r)};
      const cx<S> w = tw[tau];
      const S y = sc<S>::add(xe, sc<S>::sub(sc<S>::mul(w.r, xo.r), sc<S>::mul(w.i, xo.i)));
      const A c2 = sc<A>::mul(cvt<S, A>::to_acc(y), invN);
      // prefix sums: pfx(x) = sum_{s < x} |G(s)|^2
      const int xa = T - tau, xb = tau;
      const A pa = sc<A>::add(woff[(xa - 1) / seg], P[xa - 1]);
      const A pb = xb == 0 ? sc<A>::zero() : sc<A>::add(woff[(xb - 1) / seg], P[xb - 1]);
      A num = sc<A>::add(pa, sc<A>::sub(total, pb));
      num = sc<A>::sub(num, c2);
      a.out[(size_t)l * a.Q + q] = sc<A>::to_double(num) * a.rcp[l];
    }
    for (int l = nl - 1 - warp; l >= 0; l -= nw) {
      const int tau = a.lags[l];
      const int m = T - tau;
      if (m > kDirect) break;
      A acc = sc<A>::zero();
      for (int t = lane; t < m; t += 32) {
        const cx<S> g1 = tail[t + tau - tail0], g0 = head[t];
        const A dr = sc<A>::sub(cvt<S, A>::to_acc(g1.r), cvt<S, A>::to_acc(g0.r));
        const A di = sc<A>::sub(cvt<S, A>::to_acc(g1.i), cvt<S, A>::to_acc(g0.i));
        acc = sc<A>::add(acc, sc<A>::sqsum(dr, di));
      }
      acc = warp_sum(acc);
      if (lane == 0) a.out[(size_t)l * a.Q + q] = sc<A>::to_double(acc) * a.rcp[l];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Stage 3 (diff mode).  STAGED: the series is copied to shared memory; else
// (series longer than shared memory) it is read from the spectrum in global
// memory.
// dynamic smem: (STAGED ? T * cx<S> : 0) + 96 * A
// ---------------------------------------------------------------------------
template <class S, class A, bool STAGED>
__global__ void __launch_bounds__(512) k_tdiff(TemporalArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int T = a.T, nl = a.nlags;
  cx<S>* stage = reinterpret_cast<cx<S>*>(smem_raw);
  A* scratch = reinterpret_cast<A*>(smem_raw + (STAGED ? (size_t)T * sizeof(cx<S>) : 0));
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
  const cx<S>* F = reinterpret_cast<const cx<S>*>(a.spec);
  const A invT = sc<A>::cst(a.invT_h, a.invT_l, a.invT_d);

  for (size_t q = a.q_begin + blockIdx.x; q < a.q_end; q += gridDim.x) {
    const cx<S>* src = F + q * a.Tpad;
    const cx<S>* buf = STAGED ? stage : src;
    if (STAGED) {
      for (int t = tid; t < T; t += nthr) stage[t] = src[t];
      __syncthreads();
    }

    A v[3] = {sc<A>::zero(), sc<A>::zero(), sc<A>::zero()};
    for (int t = tid; t < T; t += nthr) {
      const cx<S> f = buf[t];
      // the spectrum's float-float pairs are not renormalised (butterfly sums):
      // after cancellation the low word can be a sizeable fraction of the high
      // word, whose square ff_sqsum would drop
      const A fr = canon(cvt<S, A>::to_acc(f.r)), fi = canon(cvt<S, A>::to_acc(f.i));
      v[0] = sc<A>::add(v[0], fr);
      v[1] = sc<A>::add(v[1], fi);
      v[2] = sc<A>::add(v[2], sc<A>::sqsum(fr, fi));
    }
    block_sum<A, 3>(v, scratch);
    const A mr = sc<A>::mul(v[0], invT), mi = sc<A>::mul(v[1], invT);
    const A ps = sc<A>::mul(v[2], invT);
    A w[1] = {sc<A>::zero()};
    for (int t = tid; t < T; t += nthr) {
      const cx<S> f = buf[t];
      const A gr = sc<A>::sub(cvt<S, A>::to_acc(f.r), mr);
      const A gi = sc<A>::sub(cvt<S, A>::to_acc(f.i), mi);
      w[0] = sc<A>::add(w[0], sc<A>::sqsum(gr, gi));
    }
    block_sum<A, 1>(w, scratch);

    for (int l = warp; l < nl; l += nw) {
      const int tau = a.lags[l];
      A acc = sc<A>::zero();
      for (int t = lane; t < T - tau; t += 32) {
        const cx<S> f1 = buf[t + tau], f0 = buf[t];
        const A dr = sc<A>::sub(cvt<S, A>::to_acc(f1.r), cvt<S, A>::to_acc(f0.r));
        const A di = sc<A>::sub(cvt<S, A>::to_acc(f1.i), cvt<S, A>::to_acc(f0.i));
        acc = sc<A>::add(acc, sc<A>::sqsum(dr, di));
      }
      acc = warp_sum(acc);
      if (lane == 0) a.out[(size_t)l * a.Q + q] = sc<A>::to_double(acc) * a.rcp[l];
    }
    if (tid == 0) {
      a.out[(size_t)nl * a.Q + q] = sc<A>::to_double(ps);
      a.out[(size_t)(nl + 1) * a.Q + q] = sc<A>::to_double(sc<A>::mul(w[0], invT));
    }
    __syncthreads();
  }
}

}  // namespace fddm
