// Azimuthal average: weighted per-bin mean and unbiased weighted standard
// deviation of every row of a stack of half-plane maps.
//
// Each thread owns one (bin, row) and walks the bin's pixels in increasing
// pixel order, evaluating term = (x * w) / sum_w and err += (w * (x - mean)^2) / bias
// with explicitly rounded FP64 operations (no FMA contraction).  That is the
// operation order of the reference's per-pixel loops
// (src/python/azimuthalaverage.py:435-444, :457-476), so the sums are
// reproducible and independent of scheduling.  A CTA covers consecutive bins of
// one row, so the row's data (the gathered operand) is shared through L2.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace {

__global__ void __launch_bounds__(128) k_azavg(const double* __restrict__ data, int64_t nrows, int64_t npix,
                                               const int32_t* __restrict__ off, const int32_t* __restrict__ pix,
                                               int nbins, const double* __restrict__ w,
                                               const double* __restrict__ sumw, const double* __restrict__ bias,
                                               double* __restrict__ avg, double* __restrict__ err) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = blockIdx.y;
  if (b >= nbins) return;
  const double* d = data + row * npix;
  const size_t o = (size_t)b * nrows + row;
  const double sw = sumw[b];
  if (sw == 0.0) {
    avg[o] = __longlong_as_double(0x7ff8000000000000ll);
    if (err) err[o] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  const int i0 = off[b], i1 = off[b + 1];
  double acc = 0.0;
  for (int i = i0; i < i1; ++i) {
    const int p = pix[i];
    acc = __dadd_rn(acc, __ddiv_rn(__dmul_rn(d[p], w[p]), sw));
  }
  avg[o] = acc;
  if (err) {
    const double bs = bias[b];
    double e = 0.0;
    for (int i = i0; i < i1; ++i) {
      const int p = pix[i];
      const double dv = __dsub_rn(d[p], acc);
      e = __dadd_rn(e, __ddiv_rn(__dmul_rn(w[p], __dmul_rn(dv, dv)), bs));
    }
    err[o] = __dsqrt_rn(e);
  }
}

// Fast variant: one warp per (bin, row).  The lanes stride over the bin's
// pixels with FP64 fused multiply-adds, the warp combines its lanes in a fixed
// butterfly order (so results are reproducible from run to run), and the mean
// divides the weighted sum once: (sum x w) / sum_w instead of the reference's
// sum of (x w) / sum_w.  Same quantities, rounded differently (relative
// differences of order 1e-15 against the bit-exact kernel above).
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(256) k_azavg_warp(const double* __restrict__ data, int64_t nrows, int64_t npix,
                                                    const int32_t* __restrict__ off, const int32_t* __restrict__ pix,
                                                    int nbins, const double* __restrict__ w,
                                                    const double* __restrict__ sumw, const double* __restrict__ bias,
                                                    double* __restrict__ avg, double* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t row = blockIdx.y;
  if (b >= nbins) return;  // whole warps leave together
  const double* d = data + row * npix;
  const size_t o = (size_t)b * nrows + row;
  const double sw = sumw[b];
  if (sw == 0.0) {
    if (lane == 0) {
      avg[o] = __longlong_as_double(0x7ff8000000000000ll);
      if (err) err[o] = __longlong_as_double(0x7ff8000000000000ll);
    }
    return;
  }
  const int i0 = off[b], i1 = off[b + 1];
  double acc = 0.0;
  for (int i = i0 + lane; i < i1; i += 32) {
    const int p = pix[i];
    acc = fma(d[p], w[p], acc);
  }
  const double mean = warp_sum_d(acc) / sw;
  if (lane == 0) avg[o] = mean;
  if (err) {
    double e = 0.0;
    for (int i = i0 + lane; i < i1; i += 32) {
      const int p = pix[i];
      const double dv = d[p] - mean;
      e = fma(w[p] * dv, dv, e);
    }
    e = warp_sum_d(e);
    if (lane == 0) err[o] = sqrt(e / bias[b]);
  }
}

int check_args(const double* d_data, const int32_t* d_bin_offsets, const double* d_weight, const double* d_sumw,
               const double* d_bias, const double* d_avg, const double* d_err, uint64_t nrows, uint64_t npix,
               uint64_t nbins) {
  if (!d_data || !d_bin_offsets || !d_weight || !d_sumw || !d_avg || (d_err && !d_bias))
    return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  if (nrows > 65535 || nbins > (1u << 30) || npix > (1ull << 31))
    return fddm::fail_with(FDDM_ERR_UNSUPPORTED, "azimuthal average: more than 65535 rows or 2^31 pixels");
  return FDDM_OK;
}

}  // namespace

extern "C" int fddm_b200_azimuthal_average_fast(const double* d_data, uint64_t nrows, uint64_t npix,
                                                const int32_t* d_bin_offsets, const int32_t* d_bin_pixels,
                                                uint64_t nbins, const double* d_weight, const double* d_sumw,
                                                const double* d_bias, double* d_avg, double* d_err, void* stream) {
  fddm::set_last_error("");
  const int rc = check_args(d_data, d_bin_offsets, d_weight, d_sumw, d_bias, d_avg, d_err, nrows, npix, nbins);
  if (rc != FDDM_OK) return rc;
  if (nbins == 0 || nrows == 0) return FDDM_OK;
  dim3 grid((unsigned)((nbins + 7) / 8), (unsigned)nrows);
  k_azavg_warp<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(d_data, (int64_t)nrows, (int64_t)npix,
                                                                   d_bin_offsets, d_bin_pixels, (int)nbins, d_weight,
                                                                   d_sumw, d_bias, d_avg, d_err);
  const cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  fddm::count_launches(1);
  return FDDM_OK;
}

extern "C" int fddm_b200_azimuthal_average(const double* d_data, uint64_t nrows, uint64_t npix,
                                           const int32_t* d_bin_offsets, const int32_t* d_bin_pixels,
                                           uint64_t nbins, const double* d_weight, const double* d_sumw,
                                           const double* d_bias, double* d_avg, double* d_err, void* stream) {
  fddm::set_last_error("");
  const int rc = check_args(d_data, d_bin_offsets, d_weight, d_sumw, d_bias, d_avg, d_err, nrows, npix, nbins);
  if (rc != FDDM_OK) return rc;
  if (nbins == 0 || nrows == 0) return FDDM_OK;
  dim3 grid((unsigned)((nbins + 127) / 128), (unsigned)nrows);
  k_azavg<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(d_data, (int64_t)nrows, (int64_t)npix, d_bin_offsets,
                                                              d_bin_pixels, (int)nbins, d_weight, d_sumw, d_bias,
                                                              d_avg, d_err);
  const cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  fddm::count_launches(1);
  return FDDM_OK;
}
