// Camera-noise estimate by quadratic fits over the first lags, one per pixel
// of the structure function: the "polyfit" mode of the reference's
// estimate_camera_noise for an ImageStructureFunction
// (src/python/noise_est.py:686-756), which calls numpy.polyfit(tau, D, 2,
// cov=True) in a Python loop over every (ky, kx).
//
// Every pixel is fitted on the same abscissae (the first npts lags), so the
// least-squares solution is one fixed (3 x npts) matrix P applied to each
// pixel's values, computed once on the host from the same scaled Vandermonde
// system numpy solves.  Per pixel: c = P y, residual r = |y - V c|^2, noise =
// c[2] (the constant term), uncertainty = sqrt(cov22 * r / (npts - 3)), with
// cov22 the (2, 2) entry of inv(V^T V); NaN where the first value is NaN.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include "fddm_b200.h"
#include "fddm_internal.h"

namespace {

constexpr int kMaxFitPoints = 64;

struct FitArgs {
  double p[3][kMaxFitPoints];  // least-squares operator (coefficients of x^2, x, 1)
  double x[kMaxFitPoints];     // abscissae
  double cov22;
  int npts;
};

__global__ void k_polyfit_noise(const double* __restrict__ data, uint64_t ld, uint64_t npix, FitArgs f,
                                double* __restrict__ noise, double* __restrict__ unc) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < npix; i += (uint64_t)gridDim.x * blockDim.x) {
    const double y0 = data[i];
    if (isnan(y0)) {
      noise[i] = y0;
      unc[i] = y0;
      continue;
    }
    double c0 = 0.0, c1 = 0.0, c2 = 0.0;
    for (int k = 0; k < f.npts; ++k) {
      const double y = data[k * ld + i];
      c0 = fma(f.p[0][k], y, c0);
      c1 = fma(f.p[1][k], y, c1);
      c2 = fma(f.p[2][k], y, c2);
    }
    double r = 0.0;
    for (int k = 0; k < f.npts; ++k) {
      const double x = f.x[k];
      const double d = data[k * ld + i] - fma(fma(c0, x, c1), x, c2);
      r = fma(d, d, r);
    }
    noise[i] = c2;
    unc[i] = sqrt(f.cov22 * r / (double)(f.npts - 3));
  }
}

}  // namespace

extern "C" int fddm_b200_polyfit_noise(const double* d_data, uint64_t ld, uint64_t npix, const double* x,
                                       const double* p, uint64_t npts, double cov22, double* d_noise,
                                       double* d_unc, void* stream) {
  fddm::set_last_error("");
  if (!d_data || !x || !p || !d_noise || !d_unc) return fddm::fail_with(FDDM_ERR_INVALID, "null pointer argument");
  if (npts < 4 || npts > (uint64_t)kMaxFitPoints)
    return fddm::fail_with(FDDM_ERR_INVALID, "polyfit noise: the number of points must lie in [4, " +
                                                 std::to_string(kMaxFitPoints) + "]");
  if (npix == 0) return FDDM_OK;
  FitArgs f{};
  f.npts = (int)npts;
  f.cov22 = cov22;
  for (uint64_t k = 0; k < npts; ++k) {
    f.x[k] = x[k];
    for (int j = 0; j < 3; ++j) f.p[j][k] = p[j * npts + k];
  }
  const unsigned grid = (unsigned)std::min<uint64_t>((npix + 255) / 256, 4096);
  k_polyfit_noise<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(d_data, ld, npix, f, d_noise, d_unc);
  const cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return fddm::fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  fddm::count_launches(1);
  return FDDM_OK;
}
