// Scalar types for the structure-function kernels.
//
// Three arithmetic tiers share one templated kernel source:
//   float   - plain FP32 (fast, ~1e-7 relative per operation),
//   ff      - float-float ("double-single") numbers: an unevaluated sum hi + lo
//             of two floats, ~48 significant bits, built from the error-free
//             transforms TwoSum (Knuth) and TwoProd via FMA (Dekker 1971),
//   double  - native FP64.
// GB300 issues FP64 FMAs at ~1/74 of the FP32 rate, so ff on the FP32 pipes is
// the fast way to reach FP64-class accuracy.  Every ff operation uses the
// __f*_rn intrinsics so that nvcc cannot contract or reorder the error-free
// transforms.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fddm {

struct ff {
  float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

// "sloppy" ff addition: absolute error ~2^-47 (|a| + |b|), which is the bound an
// FFT or a sum of squares needs.
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.h, b.h);
  float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
  return fast_two_sum(s.h, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.h, -a.l}; }

// ff addition without the final renormalisation: the result (s, e) is exact
// TwoSum of the high parts plus the rounded sum of the low parts, left as an
// unevaluated pair.  Its absolute error is the same ~2^-47 (|a| + |b|); only the
// split between the two words is not canonical.  Used inside FFT butterflies,
// whose twiddle products renormalise (ff_dot2 ends with a fast TwoSum).
__device__ __forceinline__ ff ff_add_nn(ff a, ff b) {
  ff s = two_sum(a.h, b.h);
  return {s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l))};
}
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}

// exact scaling by a power of two
__device__ __forceinline__ ff ff_scale2(ff a, float p2) { return {__fmul_rn(a.h, p2), __fmul_rn(a.l, p2)}; }

// a*a + b*b with one renormalisation (used for |z|^2)
__device__ __forceinline__ ff ff_sqsum(ff a, ff b) {
  float p = __fmul_rn(a.h, a.h);
  float e = __fmaf_rn(a.h, a.h, -p);
  e = __fmaf_rn(__fmul_rn(2.0f, a.h), a.l, e);
  float q = __fmul_rn(b.h, b.h);
  float f = __fmaf_rn(b.h, b.h, -q);
  f = __fmaf_rn(__fmul_rn(2.0f, b.h), b.l, f);
  ff s = two_sum(p, q);
  float t = __fadd_rn(s.l, __fadd_rn(e, f));
  return fast_two_sum(s.h, t);
}

// Canonical form of a pair whose low word may be as large as the high word
// (butterfly sums without renormalisation leave such pairs after cancellation).
__device__ __forceinline__ ff ff_canon(ff a) { return two_sum(a.h, a.l); }

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.h + (double)a.l; }
__host__ __device__ __forceinline__ ff ff_from_float(float a) { return {a, 0.0f}; }
// FP64 -> ff (round-to-nearest hi, exact remainder rounded to float)
__device__ __forceinline__ ff ff_from_double(double d) {
  float h = __double2float_rn(d);
  float l = __double2float_rn(d - (double)h);
  return {h, l};
}

// ---------------------------------------------------------------------------
// Generic scalar interface used by the templated FFT and reduction code.
// ---------------------------------------------------------------------------
template <class S> struct sc;

template <> struct sc<float> {
  static __device__ __forceinline__ float zero() { return 0.0f; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float neg(float a) { return -a; }
  static __device__ __forceinline__ float half(float a) { return 0.5f * a; }
  static __device__ __forceinline__ float sqsum(float a, float b) { return fmaf(a, a, b * b); }
  static __device__ __forceinline__ float from_float(float a) { return a; }
  static __device__ __forceinline__ float from_double(double a) { return __double2float_rn(a); }
  static __device__ __forceinline__ double to_double(float a) { return (double)a; }
  // constant tables store (hi, lo) float pairs; FP32 uses hi only
  static __device__ __forceinline__ float cst(float h, float l, double d) { return h; }
  // multiplication by a power of two (exact)
  static __device__ __forceinline__ float mul_p2(float a, float p2) { return __fmul_rn(a, p2); }
};

template <> struct sc<ff> {
  static __device__ __forceinline__ ff zero() { return {0.0f, 0.0f}; }
  static __device__ __forceinline__ ff add(ff a, ff b) { return ff_add(a, b); }
  static __device__ __forceinline__ ff sub(ff a, ff b) { return ff_sub(a, b); }
  static __device__ __forceinline__ ff mul(ff a, ff b) { return ff_mul(a, b); }
  static __device__ __forceinline__ ff neg(ff a) { return ff_neg(a); }
  static __device__ __forceinline__ ff half(ff a) { return ff_scale2(a, 0.5f); }
  static __device__ __forceinline__ ff sqsum(ff a, ff b) { return ff_sqsum(a, b); }
  static __device__ __forceinline__ ff from_float(float a) { return {a, 0.0f}; }
  static __device__ __forceinline__ ff from_double(double a) { return ff_from_double(a); }
  static __device__ __forceinline__ double to_double(ff a) { return ff_to_double(a); }
  static __device__ __forceinline__ ff cst(float h, float l, double d) { return {h, l}; }
  static __device__ __forceinline__ ff mul_p2(ff a, float p2) { return ff_scale2(a, p2); }
};

template <> struct sc<double> {
  static __device__ __forceinline__ double zero() { return 0.0; }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double neg(double a) { return -a; }
  static __device__ __forceinline__ double half(double a) { return 0.5 * a; }
  static __device__ __forceinline__ double sqsum(double a, double b) { return fma(a, a, b * b); }
  static __device__ __forceinline__ double from_float(float a) { return (double)a; }
  static __device__ __forceinline__ double from_double(double a) { return a; }
  static __device__ __forceinline__ double to_double(double a) { return a; }
  static __device__ __forceinline__ double cst(float h, float l, double d) { return d; }
  static __device__ __forceinline__ double mul_p2(double a, float p2) { return a * (double)p2; }
};

// Canonical form before products that drop the low word's square (ff_sqsum):
// identity for native types.
template <class A> __device__ __forceinline__ A canon(A a) { return a; }
template <> __device__ __forceinline__ ff canon<ff>(ff a) { return ff_canon(a); }

// Conversion between accumulation types (ff <-> double <-> float).
template <class To, class From> __device__ __forceinline__ To conv(From a);
template <> __device__ __forceinline__ ff conv<ff, ff>(ff a) { return a; }
template <> __device__ __forceinline__ ff conv<ff, float>(float a) { return {a, 0.0f}; }
template <> __device__ __forceinline__ float conv<float, ff>(ff a) { return __fadd_rn(a.h, a.l); }
template <> __device__ __forceinline__ float conv<float, float>(float a) { return a; }
template <> __device__ __forceinline__ double conv<double, double>(double a) { return a; }

// ---------------------------------------------------------------------------
// Complex numbers.  cx<ff> and cx<double> are 16 bytes, cx<float> 8 bytes;
// all are stored naturally aligned so global/shared loads vectorise.
// ---------------------------------------------------------------------------
template <class S> struct cx_align { static constexpr int value = 2 * sizeof(S); };
template <class S> struct alignas(cx_align<S>::value) cx {
  S r, i;
};

// butterfly additions: float-float skips the renormalisation (ff_add_nn)
template <class S> struct bfly {
  static __device__ __forceinline__ S add(S a, S b) { return sc<S>::add(a, b); }
  static __device__ __forceinline__ S sub(S a, S b) { return sc<S>::sub(a, b); }
};
template <> struct bfly<ff> {
  static __device__ __forceinline__ ff add(ff a, ff b) { return ff_add_nn(a, b); }
  static __device__ __forceinline__ ff sub(ff a, ff b) { return ff_add_nn(a, ff_neg(b)); }
};
template <class S> __device__ __forceinline__ cx<S> badd(cx<S> a, cx<S> b) {
  return {bfly<S>::add(a.r, b.r), bfly<S>::add(a.i, b.i)};
}
template <class S> __device__ __forceinline__ cx<S> bsub(cx<S> a, cx<S> b) {
  return {bfly<S>::sub(a.r, b.r), bfly<S>::sub(a.i, b.i)};
}

// twiddle products inside FFT passes (float-float: not renormalised)
template <class S> __device__ __forceinline__ cx<S> cmul(cx<S> a, cx<S> b);
template <class S> __device__ __forceinline__ cx<S> cmulc(cx<S> a, cx<S> b);
template <class S> struct twmul {
  static __device__ __forceinline__ cx<S> mul(cx<S> a, cx<S> b) { return cmul(a, b); }
  static __device__ __forceinline__ cx<S> mulc(cx<S> a, cx<S> b) { return cmulc(a, b); }  // a * conj(b)
};

template <class S> __device__ __forceinline__ cx<S> cadd(cx<S> a, cx<S> b) {
  return {sc<S>::add(a.r, b.r), sc<S>::add(a.i, b.i)};
}
template <class S> __device__ __forceinline__ cx<S> csub(cx<S> a, cx<S> b) {
  return {sc<S>::sub(a.r, b.r), sc<S>::sub(a.i, b.i)};
}
template <class S> __device__ __forceinline__ cx<S> cmul(cx<S> a, cx<S> b) {
  return {sc<S>::sub(sc<S>::mul(a.r, b.r), sc<S>::mul(a.i, b.i)),
          sc<S>::add(sc<S>::mul(a.r, b.i), sc<S>::mul(a.i, b.r))};
}
// a * conj(b)
template <class S> __device__ __forceinline__ cx<S> cmulc(cx<S> a, cx<S> b) {
  return {sc<S>::add(sc<S>::mul(a.r, b.r), sc<S>::mul(a.i, b.i)),
          sc<S>::sub(sc<S>::mul(a.i, b.r), sc<S>::mul(a.r, b.i))};
}
// float-float complex products with one renormalisation per component:
// the two leading products are split exactly (TwoProd), their difference is
// an exact TwoSum, and all low-order terms are folded into one FMA chain.
__device__ __forceinline__ ff ff_dot2(ff a, ff b, ff c, ff d, float sgn) {  // a*b + sgn*c*d
  const float p1 = __fmul_rn(a.h, b.h), e1 = __fmaf_rn(a.h, b.h, -p1);
  const float ch = __fmul_rn(sgn, c.h), cl = __fmul_rn(sgn, c.l);
  const float p2 = __fmul_rn(ch, d.h), e2 = __fmaf_rn(ch, d.h, -p2);
  const ff s = two_sum(p1, p2);
  float lo = __fadd_rn(__fadd_rn(e1, e2), s.l);
  lo = __fmaf_rn(a.h, b.l, lo);
  lo = __fmaf_rn(a.l, b.h, lo);
  lo = __fmaf_rn(ch, d.l, lo);
  lo = __fmaf_rn(cl, d.h, lo);
  return fast_two_sum(s.h, lo);
}
// ff_dot2 without the final renormalisation (the pair is exact TwoSum of the
// leading products plus the folded low-order terms); for twiddle products that
// only feed further butterfly additions.
__device__ __forceinline__ ff ff_dot2_nn(ff a, ff b, ff c, ff d, float sgn) {
  const float p1 = __fmul_rn(a.h, b.h), e1 = __fmaf_rn(a.h, b.h, -p1);
  const float ch = __fmul_rn(sgn, c.h), cl = __fmul_rn(sgn, c.l);
  const float p2 = __fmul_rn(ch, d.h), e2 = __fmaf_rn(ch, d.h, -p2);
  const ff s = two_sum(p1, p2);
  float lo = __fadd_rn(__fadd_rn(e1, e2), s.l);
  lo = __fmaf_rn(a.h, b.l, lo);
  lo = __fmaf_rn(a.l, b.h, lo);
  lo = __fmaf_rn(ch, d.l, lo);
  lo = __fmaf_rn(cl, d.h, lo);
  return {s.h, lo};
}
template <> __device__ __forceinline__ cx<ff> cmul<ff>(cx<ff> a, cx<ff> b) {
  return {ff_dot2(a.r, b.r, a.i, b.i, -1.0f), ff_dot2(a.r, b.i, a.i, b.r, 1.0f)};
}
template <> __device__ __forceinline__ cx<ff> cmulc<ff>(cx<ff> a, cx<ff> b) {
  return {ff_dot2(a.r, b.r, a.i, b.i, 1.0f), ff_dot2(a.i, b.r, a.r, b.i, -1.0f)};
}

template <> struct twmul<ff> {
  static __device__ __forceinline__ cx<ff> mul(cx<ff> a, cx<ff> b) {
    return {ff_dot2_nn(a.r, b.r, a.i, b.i, -1.0f), ff_dot2_nn(a.r, b.i, a.i, b.r, 1.0f)};
  }
  static __device__ __forceinline__ cx<ff> mulc(cx<ff> a, cx<ff> b) {
    return {ff_dot2_nn(a.r, b.r, a.i, b.i, 1.0f), ff_dot2_nn(a.i, b.r, a.r, b.i, -1.0f)};
  }
};

template <class S> __device__ __forceinline__ cx<S> cscale(cx<S> a, S s) {
  return {sc<S>::mul(a.r, s), sc<S>::mul(a.i, s)};
}
// multiply by -i (forward) or +i (inverse)
template <class S, bool INV> __device__ __forceinline__ cx<S> cmul_mi(cx<S> a) {
  if (INV) return {sc<S>::neg(a.i), a.r};
  return {a.i, sc<S>::neg(a.r)};
}
template <class S> __device__ __forceinline__ cx<S> czero() { return {sc<S>::zero(), sc<S>::zero()}; }

}  // namespace fddm
