// In-place mixed-radix FFTs in shared memory, cooperatively executed by a CTA.
//
// Forward transforms are decimation-in-frequency (DIF) passes done in place:
// pass s splits every block of M_s points into R_s interleaved sub-blocks,
//     y_m = sum_r x[j + r*M_s/R_s] w_R^(r m),   then  y_m *= w_{M_s}^(j m),
// and writes y_m back to x[j + m*M_s/R_s].  After all passes the spectrum sits
// in mixed-radix digit-reversed order: X[k] is at position perm(k) with
//     perm(k) = sum_s m_s * M_{s+1},   m_s = (k / (R_0...R_{s-1})) mod R_s.
// The inverse transform runs the exact inverse of every pass in reverse order
// (conjugate twiddle first, then the conjugate DFT), so it consumes the
// permuted order and returns natural order.  A forward FFT, a pointwise
// operation and an inverse FFT (the autocorrelation) therefore never reorders
// data.  Because every butterfly reads and writes the same R locations, a
// thread may process any number of butterflies per pass with R points in
// registers; only a barrier separates passes.
//
// Radices: 2, 3, 4, 5, 7, 8, 11, 13 (covers every 2^a 3^b 5^c 7^d {1,11,13}
// length).  Twiddles w_N^k = exp(-2 pi i k / N) come from a per-length table in
// global memory computed on the host in extended precision.
#pragma once
#include "scalar.cuh"
#include "dft_consts.cuh"
#include "fddm_internal.h"

namespace fddm {

template <class S, int R> struct odd_off;
template <class S> struct odd_off<S, 3> { static constexpr int v = 0; };
template <class S> struct odd_off<S, 5> { static constexpr int v = 3; };
template <class S> struct odd_off<S, 7> { static constexpr int v = 8; };
template <class S> struct odd_off<S, 11> { static constexpr int v = 15; };
template <class S> struct odd_off<S, 13> { static constexpr int v = 26; };

template <class S> __device__ __forceinline__ S kcos(int idx) {
  return sc<S>::cst(kCosH[idx], kCosL[idx], kCosD[idx]);
}
template <class S> __device__ __forceinline__ S ksin(int idx) {
  return sc<S>::cst(kSinH[idx], kSinL[idx], kSinD[idx]);
}

// ---------------------------------------------------------------------------
// In-register DFTs of size R (forward: w = exp(-2 pi i / R); INV: conjugate).
// ---------------------------------------------------------------------------
template <class S, bool INV> __device__ __forceinline__ void dft2(cx<S>* v) {
  cx<S> a = badd(v[0], v[1]);
  cx<S> b = bsub(v[0], v[1]);
  v[0] = a;
  v[1] = b;
}

template <class S, bool INV>
__device__ __forceinline__ void dft4_vals(cx<S>& x0, cx<S>& x1, cx<S>& x2, cx<S>& x3) {
  cx<S> t0 = badd(x0, x2);
  cx<S> t1 = bsub(x0, x2);
  cx<S> t2 = badd(x1, x3);
  cx<S> t3 = cmul_mi<S, INV>(bsub(x1, x3));
  x0 = badd(t0, t2);
  x2 = bsub(t0, t2);
  x1 = badd(t1, t3);
  x3 = bsub(t1, t3);
}

template <class S, bool INV> __device__ __forceinline__ void dft4(cx<S>* v) {
  dft4_vals<S, INV>(v[0], v[1], v[2], v[3]);
}

template <class S, bool INV>
__device__ __forceinline__ void dft8_tail(cx<S>* v, cx<S> a0, cx<S> a1, cx<S> a2, cx<S> a3, cx<S> b0, cx<S> b1,
                                          cx<S> b2, cx<S> b3) {
  const S h = sc<S>::cst(kSqrtHalfH, kSqrtHalfL, kSqrtHalfD);
  // b_r *= w8^r  (forward w8 = (1 - i)/sqrt2, inverse its conjugate)
  if (!INV) {
    b1 = cscale<S>({bfly<S>::add(b1.r, b1.i), bfly<S>::sub(b1.i, b1.r)}, h);
    b3 = cscale<S>({bfly<S>::sub(b3.i, b3.r), sc<S>::neg(bfly<S>::add(b3.r, b3.i))}, h);
  } else {
    b1 = cscale<S>({bfly<S>::sub(b1.r, b1.i), bfly<S>::add(b1.r, b1.i)}, h);
    b3 = cscale<S>({sc<S>::neg(bfly<S>::add(b3.r, b3.i)), bfly<S>::sub(b3.r, b3.i)}, h);
  }
  b2 = cmul_mi<S, INV>(b2);
  dft4_vals<S, INV>(a0, a1, a2, a3);
  dft4_vals<S, INV>(b0, b1, b2, b3);
  v[0] = a0; v[2] = a1; v[4] = a2; v[6] = a3;
  v[1] = b0; v[3] = b1; v[5] = b2; v[7] = b3;
}

template <class S, bool INV> __device__ __forceinline__ void dft8(cx<S>* v) {
  dft8_tail<S, INV>(v, badd(v[0], v[4]), badd(v[1], v[5]), badd(v[2], v[6]), badd(v[3], v[7]), bsub(v[0], v[4]),
                    bsub(v[1], v[5]), bsub(v[2], v[6]), bsub(v[3], v[7]));
}

// radix 8 with v[4..7] == 0 (the upper half of a zero-padded input)
template <class S, bool INV> __device__ __forceinline__ void dft8_halfzero(cx<S>* v) {
  dft8_tail<S, INV>(v, v[0], v[1], v[2], v[3], v[0], v[1], v[2], v[3]);
}

// Odd radix via conjugate-pair symmetry: R^2/4 complex-by-real products.
template <class S, int R, bool INV> __device__ __forceinline__ void dft_odd(cx<S>* v) {
  constexpr int H = (R - 1) / 2;
  constexpr int OFF = odd_off<S, R>::v;
  cx<S> a[H], b[H];
#pragma unroll
  for (int r = 1; r <= H; ++r) {
    a[r - 1] = badd(v[r], v[R - r]);
    b[r - 1] = bsub(v[r], v[R - r]);
  }
  cx<S> x0 = v[0];
  cx<S> y0 = x0;
#pragma unroll
  for (int r = 0; r < H; ++r) y0 = badd(y0, a[r]);
#pragma unroll
  for (int m = 1; m <= H; ++m) {
    cx<S> re = x0;
    cx<S> im = czero<S>();
#pragma unroll
    for (int r = 1; r <= H; ++r) {
      const int idx = OFF + (r * m) % R;
      const S c = kcos<S>(idx);
      const S s = ksin<S>(idx);
      re = badd(re, cscale(a[r - 1], c));
      im = badd(im, cscale(b[r - 1], s));
    }
    // forward: y_m = re - i*im, y_{R-m} = re + i*im
    cx<S> mi = cmul_mi<S, false>(im);  // -i * im
    if (!INV) {
      v[m] = badd(re, mi);
      v[R - m] = bsub(re, mi);
    } else {
      v[m] = bsub(re, mi);
      v[R - m] = badd(re, mi);
    }
  }
  v[0] = y0;
}

template <class S, int R, bool INV> __device__ __forceinline__ void dft(cx<S>* v) {
  if constexpr (R == 2) dft2<S, INV>(v);
  else if constexpr (R == 4) dft4<S, INV>(v);
  else if constexpr (R == 8) dft8<S, INV>(v);
  else dft_odd<S, R, INV>(v);
}

// ---------------------------------------------------------------------------
// Shared-memory swizzle.  A warp's 16-byte (8-byte) accesses are served in
// phases of 8 (16) lanes, one 128-byte bank row per phase, so lanes of a phase
// must touch distinct element slots modulo G = 128 / sizeof(element).  The
// butterflies access runs of consecutive elements (stride >= G passes) or
// elements G apart (the last passes); XOR-ing the slot with the row number
// serves both without conflicts.  The map only permutes within aligned groups
// of G elements, so buffers are sized to a multiple of G.
// ---------------------------------------------------------------------------
template <class S> struct swz_group { static constexpr int G = 128 / (int)sizeof(cx<S>); };
template <class S> __device__ __forceinline__ int swz(int i) {
  constexpr int G = swz_group<S>::G;
  return i ^ ((i / G) & (G - 1));
}
template <class S> __host__ __device__ constexpr int swz_round(int n) {
  return (n + swz_group<S>::G - 1) / swz_group<S>::G * swz_group<S>::G;
}

// ---------------------------------------------------------------------------
// One in-place pass over `nfft` transforms of length n, stored at logical
// offset f*ld of the (swizzled) buffer.  The twiddles w_M^(j m) come from the
// pass table `ptw` (FftPlan::ptw, row m - 1, column j), read contiguously by
// consecutive butterflies; stride-1 passes have none.
// ---------------------------------------------------------------------------
template <class S, int R, bool INV>
__device__ __forceinline__ void fft_pass(cx<S>* __restrict__ buf, int nfft, int ld, int n, int M, int lgs,
                                         int lgb, const cx<S>* __restrict__ tw, int twn,
                                         const cx<S>* __restrict__ ptw, int tid, int nthr) {
  const int stride = M / R;
  const int bpf = n / R;
  const int total = nfft * bpf;
  for (int beta = tid; beta < total; beta += nthr) {
    // power-of-two strides (the common case) index with shifts, others divide
    int f, loc, blk, j;
    if (lgb >= 0) {
      f = beta >> lgb;
      loc = beta & (bpf - 1);
    } else {
      f = beta / bpf;
      loc = beta - f * bpf;
    }
    if (lgs >= 0) {
      blk = loc >> lgs;
      j = loc & (stride - 1);
    } else {
      blk = loc / stride;
      j = loc - blk * stride;
    }
    const int base = f * ld + blk * M + j;
    cx<S> v[R];
    if (stride > 1) {
      // twiddles first (their global loads overlap the shared-memory loads and
      // the butterfly); w^0 = 1 exactly, so j = 0 needs no branch
      cx<S> w[R];
#pragma unroll
      for (int m = 1; m < R; ++m) w[m] = ptw[(m - 1) * stride + j];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = buf[swz<S>(base + r * stride)];
      if (!INV) {
        dft<S, R, false>(v);
#pragma unroll
        for (int m = 1; m < R; ++m) v[m] = twmul<S>::mul(v[m], w[m]);
      } else {
#pragma unroll
        for (int m = 1; m < R; ++m) v[m] = twmul<S>::mulc(v[m], w[m]);
        dft<S, R, true>(v);
      }
    } else {  // last pass: j = 0 only, no twiddles
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = buf[swz<S>(base + r * stride)];
      dft<S, R, INV>(v);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) buf[swz<S>(base + r * stride)] = v[r];
  }
}

// P2: the plan's radices are all 2, 4 or 8 (plan_is_p2), so the other
// butterflies are not compiled into the caller (smaller code, fewer registers).
template <class S, bool INV, bool P2 = false>
__device__ __forceinline__ void fft_pass_dispatch(cx<S>* buf, int nfft, int ld, const FftPlan& p, int s,
                                                  const cx<S>* tw, int twn, int tid, int nthr) {
  const int n = p.n, M = p.block[s], lgs = p.lgstride[s], lgb = p.lgbpf[s];
  const cx<S>* ptw = reinterpret_cast<const cx<S>*>(p.ptw[s]);
  switch (p.radix[s]) {
    case 2: fft_pass<S, 2, INV>(buf, nfft, ld, n, M, lgs, lgb, tw, twn, ptw, tid, nthr); break;
    case 4: fft_pass<S, 4, INV>(buf, nfft, ld, n, M, lgs, lgb, tw, twn, ptw, tid, nthr); break;
    case 8: fft_pass<S, 8, INV>(buf, nfft, ld, n, M, lgs, lgb, tw, twn, ptw, tid, nthr); break;
    default:
      if constexpr (!P2) {
        switch (p.radix[s]) {
          case 3: fft_pass<S, 3, INV>(buf, nfft, ld, n, M, lgs, lgb, tw, twn, ptw, tid, nthr); break;
          case 5: fft_pass<S, 5, INV>(buf, nfft, ld, n, M, lgs, lgb, tw, twn, ptw, tid, nthr); break;
          case 7: fft_pass<S, 7, INV>(buf, nfft, ld, n, M, lgs, lgb, tw, twn, ptw, tid, nthr); break;
          case 11: fft_pass<S, 11, INV>(buf, nfft, ld, n, M, lgs, lgb, tw, twn, ptw, tid, nthr); break;
          case 13: fft_pass<S, 13, INV>(buf, nfft, ld, n, M, lgs, lgb, tw, twn, ptw, tid, nthr); break;
          default: break;
        }
      }
      break;
  }
}

// Forward DFT of radix R whose upper half of inputs is zero (even R); odd
// radices fall back to the full DFT.
template <class S, int R> __device__ __forceinline__ void dft_halfzero(cx<S>* v) {
  if constexpr (R == 8) {
    dft8_halfzero<S, false>(v);
  } else if constexpr (R == 4) {  // x2 = x3 = 0
    const cx<S> x0 = v[0], x1 = v[1], x1m = cmul_mi<S, false>(x1);
    v[0] = badd(x0, x1);
    v[2] = bsub(x0, x1);
    v[1] = badd(x0, x1m);
    v[3] = bsub(x0, x1m);
  } else if constexpr (R == 2) {  // x1 = 0
    v[1] = v[0];
  } else {
    dft<S, R, false>(v);
  }
}

// First forward pass of a single transform whose input is zero at indices >=
// `limit` (limit <= n/2): those slots are neither loaded nor need to be
// written beforehand.  With an even radix the upper half of every butterfly is
// zero, so its first add/sub stage is skipped.
template <class S, int R>
__device__ __forceinline__ void fft_first_pass_padded(cx<S>* __restrict__ buf, const FftPlan& p, int limit,
                                                      const cx<S>* __restrict__ tw, int tid, int nthr) {
  const int n = p.n, stride = n / R;
  const cx<S>* ptw = reinterpret_cast<const cx<S>*>(p.ptw[0]);
  for (int j = tid; j < stride; j += nthr) {
    cx<S> v[R], w[R];
#pragma unroll
    for (int m = 1; m < R; ++m) w[m] = ptw[(m - 1) * stride + j];  // w^0 = 1: no j = 0 branch
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int idx = j + r * stride;
      v[r] = (r < R / 2 || R % 2) && idx < limit ? buf[swz<S>(idx)] : czero<S>();
    }
    dft_halfzero<S, R>(v);
#pragma unroll
    for (int m = 1; m < R; ++m) v[m] = twmul<S>::mul(v[m], w[m]);
#pragma unroll
    for (int r = 0; r < R; ++r) buf[swz<S>(j + r * stride)] = v[r];
  }
}

// Forward transform of a zero-padded input (zeros at indices >= limit, limit <= n/2).
template <class S, bool P2 = false>
__device__ void fft_forward_padded(cx<S>* buf, const FftPlan& p, int limit, const cx<S>* tw, int tid, int nthr) {
  switch (p.radix[0]) {
    case 2: fft_first_pass_padded<S, 2>(buf, p, limit, tw, tid, nthr); break;
    case 4: fft_first_pass_padded<S, 4>(buf, p, limit, tw, tid, nthr); break;
    case 8: fft_first_pass_padded<S, 8>(buf, p, limit, tw, tid, nthr); break;
    default:  // odd first radix (plans for the temporal transform start with 2, 4 or 8): zero-fill, full pass
      for (int i = limit + tid; i < p.n; i += nthr) buf[swz<S>(i)] = czero<S>();
      __syncthreads();
      fft_pass_dispatch<S, false, P2>(buf, 1, p.n, p, 0, tw, p.n, tid, nthr);
      break;
  }
  __syncthreads();
  for (int s = 1; s < p.npass; ++s) {
    fft_pass_dispatch<S, false, P2>(buf, 1, p.n, p, s, tw, p.n, tid, nthr);
    __syncthreads();
  }
}

// Forward DIF: natural order in, digit-reversed (perm) order out.
// Caller synchronises before the call; the function ends with a barrier.
// twn: length of the twiddle table `tw` (0: p.n).
template <class S, bool P2 = false>
__device__ void fft_forward(cx<S>* buf, int nfft, int ld, const FftPlan& p, const cx<S>* tw, int tid,
                            int nthr, int twn = 0) {
  if (twn == 0) twn = p.n;
  for (int s = 0; s < p.npass; ++s) {
    fft_pass_dispatch<S, false, P2>(buf, nfft, ld, p, s, tw, twn, tid, nthr);
    __syncthreads();
  }
}

// Inverse (unnormalised, sum_k X_k w^(-jk)): perm order in, natural order out.
template <class S, bool P2 = false>
__device__ void fft_inverse(cx<S>* buf, int nfft, int ld, const FftPlan& p, const cx<S>* tw, int tid,
                            int nthr, int twn = 0) {
  if (twn == 0) twn = p.n;
  for (int s = p.npass - 1; s >= 0; --s) {
    fft_pass_dispatch<S, true, P2>(buf, nfft, ld, p, s, tw, twn, tid, nthr);
    __syncthreads();
  }
}

}  // namespace fddm
