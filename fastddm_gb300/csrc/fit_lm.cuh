// Batched Levenberg-Marquardt fits of the DDM relaxation models.
//
// Replaces the lmfit Model.fit calls of the reference's fit_multik
// (src/python/fit.py:337, :380) and fit (fit.py:188).
// lmfit's default method, 'leastsq', runs MINPACK's lmdif through
// scipy.optimize.leastsq on lmfit's internal (unbounded) parameters.  This file
// restates that published algorithm (J. J. Moré, "The Levenberg-Marquardt
// algorithm: implementation and theory", 1978; Moré, Garbow and Hillstrom,
// MINPACK-1 user guide, 1980) with lmfit's settings: forward-difference
// Jacobian with step sqrt(max(epsfcn, eps)) |x_j|, Householder QR with column
// pivoting, Moré's iteration for the Levenberg-Marquardt parameter, the
// trust-region update, and the ftol / xtol / gtol tests (lmfit passes 1e-7 for
// all three).  Bounded parameters are mapped as lmfit maps them (the MINUIT
// transformations): lower only  x = min - 1 + sqrt(u^2 + 1), upper only
// x = max + 1 - sqrt(u^2 + 1), both  x = min + (sin u + 1)(max - min)/2.
// The standard errors are lmfit's: the covariance inv(R^T R) of the last
// factorisation, taken to external parameters through the derivative of the
// mapping at the solution and scaled by chi^2 / (ndata - nvary).
//
// Layout.  A group of threads runs one chain of fits (a fit_multik sweep
// warm-starts each fit from the previous result, so a chain is sequential):
// one warp when there are many chains, or the W = 4 warps of a CTA when there
// are at most four chains per SM, so that the per-point work of a chain is
// spread over the four sub-partitions of its SM (on GB300 an FP64 instruction
// occupies a sub-partition's FP64 pipe for about 64 cycles whatever the
// number of active lanes, and a single chain is bound by that latency).  The
// n x n state (the triangular factor, the step, the trust region) is computed
// by every thread of the group identically; the m data points are spread
// over the threads (point i on thread i % (32 W)) and every sum over them is
// an xor-butterfly reduction in each warp followed by the warp totals added in
// warp order, which leaves the same bits in every thread.  The Jacobian
// columns and the two residual vectors live in the group's slot of the
// workspace; each element is only touched by the thread that owns its point,
// so the only exchanges are the sums and the broadcast of row j of the
// factor.  The number of varying parameters is a template argument, so the
// small arrays stay in registers.
//
// Arithmetic against MINPACK's: the per-point divisions (by the difference
// step in the Jacobian, by the column norm in the Householder step) are
// multiplications by the reciprocal, and the sums over the points use fused
// multiply-adds; with the different summation order these change results in
// the last bits, as any other order of the same operations would.
//
// The files including this header are compiled without multiply-add
// contraction (-fmad=false), as the host arithmetic they follow has none.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <algorithm>
#include <stdint.h>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace fddm {
namespace fitlm {

constexpr int kMaxP = 8;         // parameters of the largest model (7) rounded up
constexpr int kWarpsPerCta = 4;
constexpr double kEpsMch = 2.220446049250313e-16;       // DBL_EPSILON
constexpr double kDwarf = 2.2250738585072014e-308;      // DBL_MIN

enum Status : int { kOk = 0, kNonFinite = 1, kAborted = 2, kInvalid = 3 };

__host__ __device__ inline int model_nparams(int model) {
  switch (model) {
    case FDDM_FIT_GENERIC_EXP_ISF: return 3;
    case FDDM_FIT_DOUBLE_EXP_ISF: return 6;
    case FDDM_FIT_FLORY_SCHULZ_ISF: return 3;
    case FDDM_FIT_GENERIC_EXP_SF: return 4;
    case FDDM_FIT_DOUBLE_EXP_SF: return 7;
    case FDDM_FIT_FLORY_SCHULZ_SF: return 4;
    case FDDM_FIT_SIMPLE_EXP: return 2;
    case FDDM_FIT_SIMPLE_SF: return 3;
    default: return 0;
  }
}

// b ** e as numpy evaluates an array to a scalar power: exponents 1, 2, 0.5,
// -1 and 0 take exact shortcuts (positive, square, sqrt, reciprocal, ones)
__device__ __forceinline__ double npow(double b, double e) {
  if (e == 1.0) return b;
  if (e == 2.0) return b * b;
  if (e == 0.5) return sqrt(b);
  if (e == -1.0) return 1.0 / b;
  if (e == 0.0) return 1.0;
  return pow(b, e);
}

// The model functions of fit_models.py and fit.py, in their operation order.
// p holds the parameters in the order of the Python function's arguments.
__device__ __forceinline__ double model_eval(int model, double x, const double (&p)[kMaxP]) {
  switch (model) {
    case FDDM_FIT_GENERIC_EXP_ISF:  // A exp(-(x Gamma)^beta)                      fit_models.py:515-549
      return p[0] * exp(-npow(x * p[1], p[2]));
    case FDDM_FIT_DOUBLE_EXP_ISF: {  // A (alpha e1 + (1 - alpha) e2)               fit_models.py:615-659
      const double e1 = exp(-npow(x * p[1], p[2])), e2 = exp(-npow(x * p[3], p[4]));
      return p[0] * (p[5] * e1 + (1.0 - p[5]) * e2);
    }
    case FDDM_FIT_FLORY_SCHULZ_ISF: {  // A (1 + sigma^2 Gamma x)^(-1/sigma^2)      fit_models.py:690-735
      const double s2 = p[2] * p[2];
      return p[0] * npow(1.0 + s2 * p[1] * x, -1.0 / s2);
    }
    case FDDM_FIT_GENERIC_EXP_SF:  // A (1 - exp(-(x Gamma)^beta)) + B               fit_models.py:774-808
      return p[0] * (1.0 - exp(-npow(x * p[2], p[3]))) + p[1];
    case FDDM_FIT_DOUBLE_EXP_SF: {  // A (1 - (alpha e1 + (1 - alpha) e2)) + B      fit_models.py:890-936
      const double e1 = exp(-npow(x * p[2], p[3])), e2 = exp(-npow(x * p[4], p[5]));
      return p[0] * (1.0 - (p[6] * e1 + (1.0 - p[6]) * e2)) + p[1];
    }
    case FDDM_FIT_FLORY_SCHULZ_SF: {  // A (1 - (1 + sigma^2 Gamma x)^(-1/sigma^2)) + B  fit_models.py:971-1017
      const double s2 = p[3] * p[3];
      return p[0] * (1.0 - npow(1.0 + s2 * p[2] * x, -1.0 / s2)) + p[1];
    }
    case FDDM_FIT_SIMPLE_EXP:  // amplitude exp(-dt / tau)                           fit.py:67-74
      return p[1] * exp(-x / p[0]);
    default:  // FDDM_FIT_SIMPLE_SF: A (1 - exp(-dt / tau)) + B                       fit.py:84-88
      return p[0] * (1.0 - exp(-x / p[2])) + p[1];
  }
}

// lmfit's parameter mappings (kind: 0 unbounded, 1 lower bound, 2 upper bound, 3 both)
__device__ __forceinline__ double from_internal(double u, double lo, double hi, int kind) {
  switch (kind) {
    case 0: return u;
    case 1: return lo - 1.0 + sqrt(u * u + 1.0);
    case 2: return hi + 1.0 - sqrt(u * u + 1.0);
    default: return lo + (sin(u) + 1.0) * (hi - lo) / 2.0;
  }
}

__device__ __forceinline__ double to_internal(double v, double lo, double hi, int kind) {
  switch (kind) {
    case 0: return v;
    case 1: { const double t = v - lo + 1.0; return sqrt(t * t - 1.0); }
    case 2: { const double t = hi - v + 1.0; return sqrt(t * t - 1.0); }
    default: return asin(2.0 * (v - lo) / (hi - lo) - 1.0);
  }
}

__device__ __forceinline__ double scale_gradient(double u, double lo, double hi, int kind) {
  switch (kind) {
    case 0: return 1.0;
    case 1: return u / sqrt(u * u + 1.0);
    case 2: return -u / sqrt(u * u + 1.0);
    default: return cos(u) * (hi - lo) / 2.0;
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

constexpr int kMaxW = 4;  // warps of a group

// The threads that run one chain: one warp (W = 1) or the W warps of a CTA.
template <int W>
struct Grp {
  int tid;        // thread in the group
  int lane, warp;
  double* red;    // [2][kMaxW][kMaxP] per-warp totals (W > 1), two buffers used in turn
  int* flags;     // [2][kMaxW]
  double* bc;     // [2][kMaxP] values broadcast by one thread
  int buf = 0;

  __device__ void sync() {
    if (W > 1) __syncthreads(); else __syncwarp();
  }

  // v[0..n-1] <- their sums over the group, flag <- OR over the group, and
  // bv[0..nb-1] <- the values thread `owner` holds there (owner < 32 W).
  // n, nb are compile-time after unrolling.  One barrier for W > 1: a buffer is
  // written again two calls later, after every thread has read it.
  template <int N, int NB>
  __device__ void sum(double (&v)[N], int n, bool& flag, double (&bv)[NB], int nb, int owner) {
#pragma unroll
    for (int k = 0; k < N; ++k)
      if (k < n) v[k] = warp_sum(v[k]);
    const bool wflag = __any_sync(0xffffffffu, flag);
    if (W == 1) {
      flag = wflag;
#pragma unroll
      for (int k = 0; k < NB; ++k)
        if (k < nb) bv[k] = __shfl_sync(0xffffffffu, bv[k], owner);
      return;
    }
    double* r = red + buf * (kMaxW * kMaxP);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < N; ++k)
        if (k < n) r[warp * kMaxP + k] = v[k];
      flags[buf * kMaxW + warp] = wflag;
    }
    if (tid == owner) {
#pragma unroll
      for (int k = 0; k < NB; ++k)
        if (k < nb) bc[buf * kMaxP + k] = bv[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k)
      if (k < n) {
        double t = r[k];
#pragma unroll
        for (int q = 1; q < W; ++q) t += r[q * kMaxP + k];
        v[k] = t;
      }
    bool f = false;
#pragma unroll
    for (int q = 0; q < W; ++q) f |= flags[buf * kMaxW + q] != 0;
    flag = f;
#pragma unroll
    for (int k = 0; k < NB; ++k)
      if (k < nb) bv[k] = bc[buf * kMaxP + k];
    buf ^= 1;
  }
};

// a[i] for a runtime index i over a register array (an unrolled select keeps a in registers)
template <int N, class T>
__device__ __forceinline__ T sel(const T (&a)[N], int i) {
  T r = a[0];
#pragma unroll
  for (int k = 1; k < N; ++k)
    if (k == i) r = a[k];
  return r;
}

template <int N, class T>
__device__ __forceinline__ void put(T (&a)[N], int i, T v) {
#pragma unroll
  for (int k = 0; k < N; ++k)
    if (k == i) a[k] = v;
}

template <int N>
__device__ __forceinline__ double norm_n(const double (&v)[N]) {
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < N; ++k) s += v[k] * v[k];
  return sqrt(s);
}

struct Batch {
  int model, np, m;  // m: the largest number of points of a problem (workspace and residual rows)
  const double* x;   // abscissae rows, row r at x + r * ldx
  uint64_t ldx;
  int nx;            // rows of x
  const double* y;
  uint64_t ldy;
  int ny;  // rows of y
  const double* w;
  uint64_t ldw;
  int nw;  // rows of w
  int nprob;
  const int32_t* problems;  // [nprob][6]: y row, w row (-1: none), pred (-1: none), vary mask, x row, points
  const int32_t* chain_off;
  const int32_t* chain_list;
  int nchains;
  const double* init;
  const double* lo;
  const double* hi;
  double ftol, xtol, gtol, epsfcn, factor;
  long long max_nfev;
  double* values;
  double* stderr_;
  double* chisqr;
  int32_t* nfev;
  int32_t* info;
  int32_t* status;
  double* residual;  // [nprob][m] or null
  double* covar;     // [nprob][np][np] or null
  double* ws;
  size_t slot_doubles;
  int nslots;
};

// One fit.  NV: varying parameters; W: warps of the group.
template <int NV, int W>
struct Fit {
  const Batch& b;
  Grp<W> G;  // a copy: each fit ends with a group barrier, so its sums may start from either buffer
  const double* x;  // this problem's abscissae, m of them
  const double* y;
  const double* w;
  int m;
  double* fj[NV];
  double pe[kMaxP];  // external values (fixed ones are constant)
  int vix[NV];       // parameter index of each varying parameter
  double lo[NV], hi[NV];
  int kind[NV];
  long long nfev = 0;
  int status = kOk;

  __device__ Fit(const Batch& b_, Grp<W>& g) : b(b_), G(g) {}

  __device__ void set_point(const double (&u)[NV]) {
#pragma unroll
    for (int k = 0; k < NV; ++k) set_one(k, from_internal(u[k], lo[k], hi[k], kind[k]));
  }

  // external value of varying parameter k
  __device__ void set_one(int k, double v) {
#pragma unroll
    for (int p = 0; p < kMaxP; ++p)
      if (p == vix[k]) pe[p] = v;
  }
  __device__ double get_one(int k) const {
    double v = 0.0;
#pragma unroll
    for (int p = 0; p < kMaxP; ++p)
      if (p == vix[k]) v = pe[p];
    return v;
  }

  // residuals (model - y) * w at the current pe into out; returns the sum of squares.
  // With rfd != 0, out[i] = (r_i - fv[i]) * rfd (a Jacobian column, rfd = 1 / step) and the
  // sum is over those.
  __device__ double evaluate(double* out, const double* fv, double rfd) {
    double s = 0.0;
    bool bad = false;
    for (int i = G.tid; i < m; i += 32 * W) {
      double r = model_eval(b.model, x[i], pe) - y[i];
      if (w) r = r * w[i];
      bad |= !isfinite(r);
      if (rfd != 0.0) r = (r - fv[i]) * rfd;
      out[i] = r;
      s = __fma_rn(r, r, s);
    }
    double v[1] = {s}, none[1];
    G.sum(v, 1, bad, none, 0, -1);
    if (bad) status = kNonFinite;
    ++nfev;
    if (nfev > b.max_nfev && status == kOk) status = kAborted;
    return v[0];
  }
};

// Householder QR with column pivoting of the NV columns fj (MINPACK qrfac with
// pivoting), each reflection also applied to wt (a copy of the residuals) as
// it is formed.  colsq: squared column norms.  Outputs: R (upper triangle, by
// pivot position), ipvt (position -> parameter), acnorm (by parameter), qtf.
template <int NV, int W>
__device__ void qr_pivot(Fit<NV, W>& F, const double (&colsq)[NV], double* wt, double (&R)[NV][NV], int (&ipvt)[NV],
                         double (&acnorm)[NV], double (&qtf)[NV]) {
  const int m = F.m, tid = F.G.tid;
  constexpr int S = 32 * W;
  double rdiag[NV], wa[NV];
  bool recomp[NV];
  double* pc[NV];  // column at pivot position k (kept in registers: swapped with ipvt, indexed statically)
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    pc[k] = F.fj[k];
    ipvt[k] = k;
    acnorm[k] = sqrt(colsq[k]);
    rdiag[k] = acnorm[k];
    wa[k] = acnorm[k];
    recomp[k] = false;
#pragma unroll
    for (int i = 0; i < NV; ++i) R[i][k] = 0.0;
  }
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    // squared norms of the columns below row j-1, and row j with wt[j] from the thread owning point j
    double fresh[NV], rowj[NV];
    double part[NV], bv[NV + 1];
#pragma unroll
    for (int k = 0; k < NV; ++k) part[k] = 0.0;
    if (j > 0)
      for (int i = tid; i < m; i += S) {
        if (i < j) continue;
#pragma unroll
        for (int k = j; k < NV; ++k) {
          const double v = pc[k][i];
          part[k - j] = __fma_rn(v, v, part[k - j]);
        }
      }
#pragma unroll
    for (int k = 0; k <= NV; ++k) bv[k] = 0.0;
    if (tid == j) {
#pragma unroll
      for (int k = j; k < NV; ++k) bv[k - j] = pc[k][j];
      bv[NV - j] = wt[j];
    }
    bool nf = false;
    F.G.sum(part, j > 0 ? NV - j : 0, nf, bv, NV - j + 1, j);
#pragma unroll
    for (int k = j; k < NV; ++k) {
      fresh[k] = j > 0 ? part[k - j] : colsq[k];
      rowj[k] = bv[k - j];
    }
    const double wj = bv[NV - j];
    // norms flagged at the previous step are taken afresh (MINPACK recomputes them there)
#pragma unroll
    for (int k = j; k < NV; ++k)
      if (recomp[k]) {
        rdiag[k] = sqrt(fresh[k]);
        wa[k] = rdiag[k];
        recomp[k] = false;
      }
    // pivot: the first largest remaining norm
    int kmax = j;
#pragma unroll
    for (int k = j + 1; k < NV; ++k)
      if (rdiag[k] > sel(rdiag, kmax)) kmax = k;
    if (kmax != j) {
#pragma unroll
      for (int k = j + 1; k < NV; ++k)
        if (k == kmax) {
          int ti = ipvt[j]; ipvt[j] = ipvt[k]; ipvt[k] = ti;
          double* tp = pc[j]; pc[j] = pc[k]; pc[k] = tp;
          double t = fresh[j]; fresh[j] = fresh[k]; fresh[k] = t;
          t = rowj[j]; rowj[j] = rowj[k]; rowj[k] = t;
          rdiag[k] = rdiag[j];
          wa[k] = wa[j];
#pragma unroll
          for (int i = 0; i < j; ++i) { t = R[i][j]; R[i][j] = R[i][k]; R[i][k] = t; }
        }
    }
    double ajnorm = sqrt(fresh[j]);
    if (ajnorm != 0.0) {
      if (rowj[j] < 0.0) ajnorm = -ajnorm;
      const double rn = 1.0 / ajnorm;
      const double vjj = rowj[j] * rn + 1.0;
      double* cj = pc[j];
      double dot[NV];  // dot[0]: with wt; dot[k - j]: with column k > j
#pragma unroll
      for (int k = 0; k < NV; ++k) dot[k] = 0.0;
      for (int i = tid; i < m; i += S) {
        if (i < j) continue;
        double v = cj[i] * rn;
        if (i == j) v = v + 1.0;
        cj[i] = v;
        dot[0] = __fma_rn(v, wt[i], dot[0]);
#pragma unroll
        for (int k = j + 1; k < NV; ++k) dot[k - j] = __fma_rn(v, pc[k][i], dot[k - j]);
      }
      double none[1];
      F.G.sum(dot, NV - j, nf, none, 0, -1);
      const double rv = 1.0 / vjj;
      const double tw = -dot[0] * rv;
      double tk[NV];
#pragma unroll
      for (int k = j + 1; k < NV; ++k) tk[k] = dot[k - j] * rv;
      for (int i = tid; i < m; i += S) {
        if (i < j) continue;
        const double v = cj[i];
        wt[i] = __fma_rn(v, tw, wt[i]);
#pragma unroll
        for (int k = j + 1; k < NV; ++k) pc[k][i] = __fma_rn(-tk[k], v, pc[k][i]);
      }
      qtf[j] = __fma_rn(vjj, tw, wj);
#pragma unroll
      for (int k = j + 1; k < NV; ++k) {
        R[j][k] = __fma_rn(-tk[k], vjj, rowj[k]);
        if (rdiag[k] != 0.0) {
          const double t = R[j][k] / rdiag[k];
          rdiag[k] *= sqrt(fmax(0.0, 1.0 - t * t));
          // 0.05 (rdiag / wa)^2 <= eps, without the division
          if (0.05 * (rdiag[k] * rdiag[k]) <= kEpsMch * (wa[k] * wa[k])) recomp[k] = true;
        }
      }
    } else {
      qtf[j] = wj;
#pragma unroll
      for (int k = j + 1; k < NV; ++k) R[j][k] = rowj[k];
    }
    rdiag[j] = -ajnorm;
    R[j][j] = rdiag[j];
  }
}

// MINPACK qrsolv: given R (by pivot position), ipvt, the diagonal d (by
// parameter) and qtb, solve min |[R P^T; D] x - [qtb; 0]|.  S receives the
// triangular factor of the augmented system (transposed, below the diagonal)
// and sdiag its diagonal.
template <int NV>
__device__ void qrsolv(const double (&R)[NV][NV], const int (&ipvt)[NV], const double (&d)[NV], const double (&qtb)[NV],
                       double (&x)[NV], double (&S)[NV][NV], double (&sdiag)[NV]) {
  double wa[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
#pragma unroll
    for (int i = j; i < NV; ++i) S[i][j] = R[j][i];
    wa[j] = qtb[j];
  }
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    const double dl = sel(d, ipvt[j]);
    if (dl != 0.0) {
#pragma unroll
      for (int k = j; k < NV; ++k) sdiag[k] = 0.0;
      sdiag[j] = dl;
      double qtbpj = 0.0;
#pragma unroll
      for (int k = j; k < NV; ++k) {
        if (sdiag[k] == 0.0) continue;
        double sn, cs;
        if (fabs(S[k][k]) < fabs(sdiag[k])) {
          const double cotan = S[k][k] / sdiag[k];
          sn = 0.5 / sqrt(0.25 + 0.25 * (cotan * cotan));
          cs = sn * cotan;
        } else {
          const double tn = sdiag[k] / S[k][k];
          cs = 0.5 / sqrt(0.25 + 0.25 * (tn * tn));
          sn = cs * tn;
        }
        S[k][k] = cs * S[k][k] + sn * sdiag[k];
        const double t = cs * wa[k] + sn * qtbpj;
        qtbpj = -sn * wa[k] + cs * qtbpj;
        wa[k] = t;
#pragma unroll
        for (int i = k + 1; i < NV; ++i) {
          const double u = cs * S[i][k] + sn * sdiag[i];
          sdiag[i] = -sn * S[i][k] + cs * sdiag[i];
          S[i][k] = u;
        }
      }
    }
    sdiag[j] = S[j][j];
    S[j][j] = R[j][j];
  }
  int nsing = NV;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    if (sdiag[j] == 0.0 && nsing == NV) nsing = j;
    if (nsing < NV) wa[j] = 0.0;
  }
#pragma unroll
  for (int j = NV - 1; j >= 0; --j) {
    if (j >= nsing) continue;
    double s = 0.0;
#pragma unroll
    for (int i = j + 1; i < NV; ++i)
      if (i < nsing) s += S[i][j] * wa[i];
    wa[j] = (wa[j] - s) / sdiag[j];
  }
#pragma unroll
  for (int j = 0; j < NV; ++j) put(x, ipvt[j], wa[j]);
}

// MINPACK lmpar: the Levenberg-Marquardt parameter for the trust radius delta
// and the step x (by parameter); returns the new parameter.
template <int NV>
__device__ double lmpar(const double (&R)[NV][NV], const int (&ipvt)[NV], const double (&diag)[NV],
                        const double (&qtb)[NV], double delta, double par, double (&x)[NV]) {
  double wa1[NV], wa2[NV];
  int nsing = NV;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    wa1[j] = qtb[j];
    if (R[j][j] == 0.0 && nsing == NV) nsing = j;
    if (nsing < NV) wa1[j] = 0.0;
  }
#pragma unroll
  for (int j = NV - 1; j >= 0; --j) {
    if (j >= nsing) continue;
    wa1[j] = wa1[j] / R[j][j];
    const double t = wa1[j];
#pragma unroll
    for (int i = 0; i < j; ++i) wa1[i] -= R[i][j] * t;
  }
#pragma unroll
  for (int j = 0; j < NV; ++j) put(x, ipvt[j], wa1[j]);
#pragma unroll
  for (int j = 0; j < NV; ++j) wa2[j] = diag[j] * x[j];
  double dxnorm = norm_n(wa2);
  double fp = dxnorm - delta;
  if (fp <= 0.1 * delta) return 0.0;
  // lower bound from the Newton step (when the Jacobian has full rank)
  double parl = 0.0;
  if (nsing >= NV) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const int l = ipvt[j];
      wa1[j] = sel(diag, l) * (sel(wa2, l) / dxnorm);
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < j; ++i) s += R[i][j] * wa1[i];
      wa1[j] = (wa1[j] - s) / R[j][j];
    }
    const double t = norm_n(wa1);
    parl = ((fp / delta) / t) / t;
  }
  // upper bound
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i <= j; ++i) s += R[i][j] * qtb[i];
    wa1[j] = s / sel(diag, ipvt[j]);
  }
  const double gnorm = norm_n(wa1);
  double paru = gnorm / delta;
  if (paru == 0.0) paru = kDwarf / fmin(delta, 0.1);
  par = fmax(par, parl);
  par = fmin(par, paru);
  if (par == 0.0) par = gnorm / dxnorm;
  double S[NV][NV], sdiag[NV];
  for (int iter = 1;; ++iter) {
    if (par == 0.0) par = fmax(kDwarf, 0.001 * paru);
    const double sp = sqrt(par);
#pragma unroll
    for (int j = 0; j < NV; ++j) wa1[j] = sp * diag[j];
    qrsolv(R, ipvt, wa1, qtb, x, S, sdiag);
#pragma unroll
    for (int j = 0; j < NV; ++j) wa2[j] = diag[j] * x[j];
    dxnorm = norm_n(wa2);
    const double fp_old = fp;
    fp = dxnorm - delta;
    if (fabs(fp) <= 0.1 * delta || (parl == 0.0 && fp <= fp_old && fp_old < 0.0) || iter == 10) break;
    // Newton correction
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const int l = ipvt[j];
      wa1[j] = sel(diag, l) * (sel(wa2, l) / dxnorm);
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      wa1[j] = wa1[j] / sdiag[j];
      const double t = wa1[j];
#pragma unroll
      for (int i = j + 1; i < NV; ++i) wa1[i] -= S[i][j] * t;
    }
    const double t = norm_n(wa1);
    const double parc = ((fp / delta) / t) / t;
    if (fp > 0.0) parl = fmax(parl, par);
    if (fp < 0.0) paru = fmin(paru, par);
    par = fmax(parl, par + parc);
  }
  return par;
}

// lmdif on one problem; u holds the internal starting point and receives the result.
template <int NV, int W>
__device__ void lmdif(Fit<NV, W>& F, double (&u)[NV], double*& fv, double*& wt, double& fsq, int& info,
                      double (&R)[NV][NV], int (&ipvt)[NV]) {
  const Batch& b = F.b;
  const double eps = sqrt(fmax(b.epsfcn, kEpsMch));
  F.set_point(u);
  fsq = F.evaluate(fv, nullptr, 0.0);
  info = 0;
  if (F.status != kOk) return;
  double fnorm = sqrt(fsq);
  double par = 0.0, delta = 0.0, xnorm = 0.0;
  double diag[NV], acnorm[NV], qtf[NV];
  for (int iter = 1;;) {
    // forward-difference Jacobian (only the perturbed parameter is mapped again)
    double colsq[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const double t = u[j];
      double h = eps * fabs(t);
      if (h == 0.0) h = eps;
      const double keep = F.get_one(j);
      F.set_one(j, from_internal(t + h, F.lo[j], F.hi[j], F.kind[j]));
      colsq[j] = F.evaluate(F.fj[j], fv, 1.0 / h);
      F.set_one(j, keep);
      if (F.status != kOk) return;
    }
    for (int i = F.G.tid; i < F.m; i += 32 * W) wt[i] = fv[i];
    qr_pivot(F, colsq, wt, R, ipvt, acnorm, qtf);
    if (iter == 1) {
#pragma unroll
      for (int j = 0; j < NV; ++j) diag[j] = acnorm[j] == 0.0 ? 1.0 : acnorm[j];
      double t[NV];
#pragma unroll
      for (int j = 0; j < NV; ++j) t[j] = diag[j] * u[j];
      xnorm = norm_n(t);
      delta = b.factor * xnorm;
      if (delta == 0.0) delta = b.factor;
    }
    // scaled gradient
    double gnorm = 0.0;
    if (fnorm != 0.0) {
      double qn[NV];
#pragma unroll
      for (int i = 0; i < NV; ++i) qn[i] = qtf[i] / fnorm;
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        const double an = sel(acnorm, ipvt[j]);
        if (an != 0.0) {
          double s = 0.0;
#pragma unroll
          for (int i = 0; i <= j; ++i) s += R[i][j] * qn[i];
          gnorm = fmax(gnorm, fabs(s / an));
        }
      }
    }
    if (gnorm <= b.gtol) info = 4;
    if (info != 0) return;
#pragma unroll
    for (int j = 0; j < NV; ++j) diag[j] = fmax(diag[j], acnorm[j]);
    for (;;) {
      double p[NV], ut[NV], dp[NV];
      par = lmpar(R, ipvt, diag, qtf, delta, par, p);
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        p[j] = -p[j];
        ut[j] = u[j] + p[j];
        dp[j] = diag[j] * p[j];
      }
      const double pnorm = norm_n(dp);
      if (iter == 1) delta = fmin(delta, pnorm);
      F.set_point(ut);
      const double fsq1 = F.evaluate(wt, nullptr, 0.0);
      if (F.status != kOk) return;  // the result stays at the last accepted point
      const double fnorm1 = sqrt(fsq1);
      double actred = -1.0;
      if (0.1 * fnorm1 < fnorm) {
        const double q = fnorm1 / fnorm;
        actred = 1.0 - q * q;
      }
      double wa3[NV];
#pragma unroll
      for (int j = 0; j < NV; ++j) wa3[j] = 0.0;
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        const double t = sel(p, ipvt[j]);
#pragma unroll
        for (int i = 0; i <= j; ++i) wa3[i] += R[i][j] * t;
      }
      const double temp1 = norm_n(wa3) / fnorm;
      const double temp2 = (sqrt(par) * pnorm) / fnorm;
      const double prered = temp1 * temp1 + temp2 * temp2 / 0.5;
      const double dirder = -(temp1 * temp1 + temp2 * temp2);
      const double ratio = prered != 0.0 ? actred / prered : 0.0;
      if (ratio <= 0.25) {
        double t = actred >= 0.0 ? 0.5 : 0.5 * dirder / (dirder + 0.5 * actred);
        if (0.1 * fnorm1 >= fnorm || t < 0.1) t = 0.1;
        delta = t * fmin(delta, pnorm / 0.1);
        par = par / t;
      } else if (par == 0.0 || ratio >= 0.75) {
        delta = pnorm / 0.5;
        par = 0.5 * par;
      }
      if (ratio >= 1e-4) {
        double t[NV];
#pragma unroll
        for (int j = 0; j < NV; ++j) {
          u[j] = ut[j];
          t[j] = diag[j] * u[j];
        }
        double* s = fv; fv = wt; wt = s;
        xnorm = norm_n(t);
        fnorm = fnorm1;
        fsq = fsq1;
        ++iter;
      }
      const bool fconv = fabs(actred) <= b.ftol && prered <= b.ftol && 0.5 * ratio <= 1.0;
      if (fconv) info = 1;
      if (delta <= b.xtol * xnorm) info = fconv ? 3 : 2;
      if (info != 0) return;
      if (fabs(actred) <= kEpsMch && prered <= kEpsMch && 0.5 * ratio <= 1.0) info = 6;
      if (delta <= kEpsMch * xnorm) info = 7;
      if (gnorm <= kEpsMch) info = 8;
      if (info != 0) return;
      if (ratio >= 1e-4) break;
    }
  }
}

template <int NV, int W>
__device__ void run_problem(const Batch& b, int prob, double* slot, Grp<W>& G) {
  const int lane = G.tid;
  const int32_t* pr = b.problems + 6 * (size_t)prob;
  const int yrow = pr[0], wrow = pr[1], pred = pr[2];
  const uint32_t vary = (uint32_t)pr[3];
  const int xrow = pr[4], mp = pr[5];
  // a problem naming a row or a predecessor that does not exist, or varying another number of
  // parameters than the launch, is not fitted
  if (yrow < 0 || yrow >= b.ny || wrow >= b.nw || (wrow >= 0 && !b.w) || pred >= b.nprob || xrow < 0 ||
      xrow >= b.nx || mp < NV || mp > b.m || __popc(vary & ((1u << b.np) - 1u)) != NV || (vary >> b.np) != 0u) {
    if (lane == 0) {
      for (int p = 0; p < b.np; ++p) {
        b.values[(size_t)prob * b.np + p] = NAN;
        b.stderr_[(size_t)prob * b.np + p] = NAN;
      }
      b.chisqr[prob] = NAN;
      b.nfev[prob] = 0;
      b.info[prob] = 0;
      b.status[prob] = kInvalid;
    }
    G.sync();
    return;
  }
  Fit<NV, W> F(b, G);
  F.m = mp;
  F.x = b.x + (size_t)xrow * b.ldx;
  F.y = b.y + (size_t)yrow * b.ldy;
  F.w = wrow >= 0 ? b.w + (size_t)wrow * b.ldw : nullptr;
  double* fv = slot;
  double* wt = slot + b.m;
#pragma unroll
  for (int k = 0; k < NV; ++k) F.fj[k] = slot + (size_t)(2 + k) * b.m;
  // starting values: the predecessor's result for the varying parameters, clipped into the bounds
  const double* ini = b.init + (size_t)prob * b.np;
  const double* plo = b.lo + (size_t)prob * b.np;
  const double* phi = b.hi + (size_t)prob * b.np;
  double u[NV];
  int nv = 0;
#pragma unroll
  for (int p = 0; p < kMaxP; ++p) {
    if (p >= b.np) { F.pe[p] = 0.0; continue; }
    const bool vp = (vary >> p) & 1u;
    double v = (vp && pred >= 0) ? b.values[(size_t)pred * b.np + p] : ini[p];
    const double l = plo[p], h = phi[p];
    if (v > h) v = h;
    if (v < l) v = l;
    F.pe[p] = v;
    if (vp) {
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (k == nv) {
          F.vix[k] = p;
          F.lo[k] = l;
          F.hi[k] = h;
          F.kind[k] = (l == -INFINITY ? 0 : 1) + (h == INFINITY ? 0 : 2);
          u[k] = to_internal(v, l, h, F.kind[k]);
        }
      ++nv;
    }
  }
  double fsq = 0.0, R[NV][NV];
  int info = 0, ipvt[NV];
  lmdif(F, u, fv, wt, fsq, info, R, ipvt);
  F.set_point(u);
  // standard errors: inv(R'^T R') with R' = R / scale_gradient (by column), times chi^2 / nfree.
  // As with numpy's inv there: entries that are not finite give NaN errors (fixed parameters 0); an
  // exactly singular R'^T R gives no covariance at all (every error -1, reported as None).
  double se[NV];
  int cov = F.status == kOk ? 0 : 2;  // 0 exists, 1 not finite, 2 none
  if (cov == 0) {
    double Rp[NV][NV], Ui[NV][NV];
    bool singular = false;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const int l = ipvt[j];
      double g = 0.0;
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (k == l) g = scale_gradient(u[k], F.lo[k], F.hi[k], F.kind[k]);
      const double rg = 1.0 / g;
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        Rp[i][j] = i <= j ? R[i][j] * rg : 0.0;
        if (!isfinite(Rp[i][j])) cov = 1;
      }
      if (Rp[j][j] == 0.0) singular = true;
    }
    if (cov == 0 && singular) cov = 2;
    if (cov == 0) {
      // Ui = Rp^{-1} (upper triangular, back substitution column by column)
      double rd[NV];
#pragma unroll
      for (int i = 0; i < NV; ++i) rd[i] = 1.0 / Rp[i][i];
#pragma unroll
      for (int c = 0; c < NV; ++c) {
#pragma unroll
        for (int i = NV - 1; i >= 0; --i) {
          double s = i == c ? 1.0 : 0.0;
#pragma unroll
          for (int k = i + 1; k < NV; ++k) s -= Rp[i][k] * Ui[k][c];
          Ui[i][c] = i <= c ? s * rd[i] : 0.0;
        }
      }
      const int nfree = mp - NV;
      const double redchi = fsq / (double)(nfree > 1 ? nfree : 1);
      // variance of the parameter at position i: row i of Ui squared
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < NV; ++k) s += Ui[i][k] * Ui[i][k];
        put(se, ipvt[i], sqrt(s * redchi));
      }
      // the whole covariance, when asked for: entry (p, q) of the parameters at positions i, k
      if (b.covar && lane == 0) {
        double* co = b.covar + (size_t)prob * b.np * b.np;
        for (int e = 0; e < b.np * b.np; ++e) co[e] = 0.0;
#pragma unroll
        for (int i = 0; i < NV; ++i) {
          const int pi = sel(F.vix, ipvt[i]);
#pragma unroll
          for (int k = 0; k < NV; ++k) {
            double s = 0.0;
#pragma unroll
            for (int l = 0; l < NV; ++l) s += Ui[i][l] * Ui[k][l];
            co[pi * b.np + sel(F.vix, ipvt[k])] = s * redchi;
          }
        }
      }
    } else if (cov == 1) {
#pragma unroll
      for (int k = 0; k < NV; ++k) se[k] = NAN;
    }
  }
  if (b.covar && lane == 0 && cov != 0) {  // no finite covariance: NaN
    double* co = b.covar + (size_t)prob * b.np * b.np;
    for (int e = 0; e < b.np * b.np; ++e) co[e] = NAN;
  }
  if (lane == 0) {
    double* vo = b.values + (size_t)prob * b.np;
    double* so = b.stderr_ + (size_t)prob * b.np;
#pragma unroll
    for (int p = 0; p < kMaxP; ++p) {
      if (p >= b.np) break;
      vo[p] = F.pe[p];
      double s = cov == 2 ? -1.0 : 0.0;  // fixed parameters: 0 when a covariance exists
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (F.vix[k] == p && cov != 2) s = se[k];
      so[p] = s;
    }
    b.chisqr[prob] = fsq;
    b.nfev[prob] = (int32_t)F.nfev;
    b.info[prob] = F.status == kAborted ? -1 : info;
    b.status[prob] = F.status;
  }
  if (b.residual)
    for (int i = G.tid; i < mp; i += 32 * W) b.residual[(size_t)prob * b.m + i] = fv[i];
  G.sync();
}

// W = 1: each warp of the CTA runs its own chains; W = 4: the CTA runs one chain at a time.
template <int NV, int W>
// __grid_constant__: the fits keep references to the batch description, which then stay in the
// parameter space instead of a per-thread copy in local memory
__global__ void __launch_bounds__(32 * kWarpsPerCta) k_fit_lm(const __grid_constant__ Batch b) {
  static_assert(W == 1 || W == kWarpsPerCta, "a group is one warp or the whole CTA");
  __shared__ double red[2 * kMaxW * kMaxP];
  __shared__ int flags[2 * kMaxW];
  __shared__ double bc[2 * kMaxP];
  Grp<W> G;
  G.lane = threadIdx.x & 31;
  G.warp = threadIdx.x >> 5;
  G.tid = W > 1 ? (int)threadIdx.x : G.lane;
  G.red = red;
  G.flags = flags;
  G.bc = bc;
  const int gid = W > 1 ? (int)blockIdx.x : (int)(blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5));
  if (gid >= b.nslots) return;  // whole groups leave together
  double* slot = b.ws + (size_t)gid * b.slot_doubles;
  for (int c = gid; c < b.nchains; c += b.nslots) {
    bool stop = false;
    for (int e = b.chain_off[c]; e < b.chain_off[c + 1] && !stop; ++e) {
      const int prob = b.chain_list[e];
      if (prob < 0 || prob >= b.nprob) break;  // not a problem: the chain ends
      run_problem<NV, W>(b, prob, slot, G);
      // a fit that raised in the reference ends its sweep there
      stop = b.status[prob] == kNonFinite || b.status[prob] == kInvalid;
    }
  }
}

template <int NV>
cudaError_t launch(const Batch& b, unsigned grid, int group_warps, cudaStream_t st) {
  if (group_warps > 1)
    k_fit_lm<NV, kWarpsPerCta><<<grid, 32 * kWarpsPerCta, 0, st>>>(b);
  else
    k_fit_lm<NV, 1><<<grid, 32 * kWarpsPerCta, 0, st>>>(b);
  return cudaGetLastError();
}

// one launcher per number of varying parameters, each in its own translation unit
cudaError_t launch_nv1(const Batch& b, unsigned grid, int group_warps, cudaStream_t st);
cudaError_t launch_nv2(const Batch& b, unsigned grid, int group_warps, cudaStream_t st);
cudaError_t launch_nv3(const Batch& b, unsigned grid, int group_warps, cudaStream_t st);
cudaError_t launch_nv4(const Batch& b, unsigned grid, int group_warps, cudaStream_t st);
cudaError_t launch_nv5(const Batch& b, unsigned grid, int group_warps, cudaStream_t st);
cudaError_t launch_nv6(const Batch& b, unsigned grid, int group_warps, cudaStream_t st);
cudaError_t launch_nv7(const Batch& b, unsigned grid, int group_warps, cudaStream_t st);

}  // namespace fitlm
}  // namespace fddm
