// Measurement behind the decision not to run a DFT stage on the tensor cores.
//
// The only stage of the pipeline whose inputs are exact in bf16 is the first
// radix-32 stage of the row transform of 8-bit frames: a DFT-as-GEMM there
// would multiply the exact pixels by a DFT matrix split into bf16 slices (five
// slices, 40 bits, for the float-float accuracy the structure function needs;
// every other stage has float-float inputs and would need slices of both
// operands).  Besides the MMAs, such a stage leaves work on the CUDA cores:
// per output of each real row, reading ten FP32 slice sums (real and
// imaginary parts), combining them exactly into float-float, then packing two
// rows into one complex value and applying the inter-stage twiddle, as the
// float-float passes do.
//
//   variant 0: the two float-float DIF passes (radix 8, then radix 4) that form
//              the radix-32 first stage of a 1024-point transform of a packed
//              row pair, as in the row pass;
//   variant 1: that CUDA-core remainder of a tensor-core stage alone, with the
//              slice sums taken from shared memory (no MMA at all, so a lower
//              bound on the tensor-core stage's time).
// Both read 8-bit row pairs and write the stage's float-float output.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "fddm_b200.h"
#include "ddm_impl.cuh"

namespace fddm {
namespace {

constexpr int kN = 1024;       // row length
constexpr int kPairs = 4;      // row pairs per CTA iteration (64 KB transform buffer, as the row pass)
constexpr int kSlices = 5;     // bf16 slices of the DFT matrix

__device__ __forceinline__ void load_pairs(cx<ff>* buf, int ld, const uint8_t* rows, int p0, int np) {
  for (int e = threadIdx.x; e < np * kN; e += blockDim.x) {
    const int pr = e >> 10, x = e & (kN - 1);
    const uint8_t* r = rows + (size_t)(p0 + pr) * 2 * kN;
    buf[swz<ff>(pr * ld + x)] = {ff{(float)r[x], 0.0f}, ff{(float)r[kN + x], 0.0f}};
  }
}

__device__ __forceinline__ void store_pairs(const cx<ff>* buf, int ld, cx<ff>* out, int p0, int np) {
  for (int e = threadIdx.x; e < np * kN; e += blockDim.x) {
    const int pr = e >> 10, x = e & (kN - 1);
    out[(size_t)(p0 + pr) * kN + x] = buf[swz<ff>(pr * ld + x)];
  }
}

__global__ void __launch_bounds__(256) k_exp_butterfly(const uint8_t* __restrict__ rows, int npairs, FftPlan p,
                                                       cx<ff>* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  cx<ff>* buf = reinterpret_cast<cx<ff>*>(smem);
  const int ld = kN + swz_group<ff>::G;
  for (int g = blockIdx.x; g * kPairs < npairs; g += gridDim.x) {
    const int p0 = g * kPairs, np = min(kPairs, npairs - p0);
    __syncthreads();
    load_pairs(buf, ld, rows, p0, np);
    __syncthreads();
    for (int s = 0; s < 2; ++s) {
      fft_pass_dispatch<ff, false, true>(buf, np, ld, p, s, nullptr, kN, threadIdx.x, blockDim.x);
      __syncthreads();
    }
    store_pairs(buf, ld, out, p0, np);
  }
}

// kSlices exact FP32 partial sums of decreasing scale -> float-float
__device__ __forceinline__ ff combine_slices(const float* s) {
  ff acc = {s[0], 0.0f};
#pragma unroll
  for (int k = 1; k < kSlices; ++k) {
    const ff t = two_sum(acc.h, s[k]);
    acc = {t.h, __fadd_rn(acc.l, t.l)};
  }
  return fast_two_sum(acc.h, acc.l);
}

// stand-in slice sums repeat with this period (a small table, so the kernel
// keeps two CTAs per SM like variant 0)
constexpr int kSumTile = 256;

struct alignas(16) SliceSums {
  float v[12];  // real parts of the kSlices slice sums, then the imaginary parts (padded to 3 x float4)
};

__global__ void __launch_bounds__(256) k_exp_gemm_floor(const uint8_t* __restrict__ rows, int npairs,
                                                        const cx<ff>* __restrict__ tw, cx<ff>* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  cx<ff>* buf = reinterpret_cast<cx<ff>*>(smem);
  const int ld = kN + swz_group<ff>::G;
  SliceSums* sums = reinterpret_cast<SliceSums*>(buf + swz_round<ff>(kPairs * ld));
  // stand-in slice sums (exact small integers at the slices' scales); their
  // values do not matter for the timing
  for (int i = threadIdx.x; i < kSumTile; i += blockDim.x)
    for (int k = 0; k < 12; ++k)
      sums[i].v[k] = ldexpf((float)((i * 37 + k * 11) & 4095), -8 * (k % kSlices));
  for (int g = blockIdx.x; g * kPairs < npairs; g += gridDim.x) {
    const int p0 = g * kPairs, np = min(kPairs, npairs - p0);
    __syncthreads();
    // the pixels are the MMA's operand: the remainder only touches them to
    // stage them (here as float-float, as variant 0 does)
    load_pairs(buf, ld, rows, p0, np);
    __syncthreads();
    for (int e = threadIdx.x; e < np * kN; e += blockDim.x) {
      const int pr = e >> 10, q = e & (kN - 1);  // q = j + 32 m: output m of sub-sequence j
      const int j = q & 31, m = q >> 5;
      const SliceSums a = sums[q & (kSumTile - 1)], b = sums[(q ^ 1) & (kSumTile - 1)];  // rows a and b
      const ff ar = combine_slices(a.v), ai = combine_slices(a.v + kSlices);
      const ff br = combine_slices(b.v), bi = combine_slices(b.v + kSlices);
      // pack the two real rows (Z = Y_a + i Y_b), then the inter-stage twiddle w_1024^(j m)
      const cx<ff> z = {ff_add_nn(ar, ff_neg(bi)), ff_add_nn(ai, br)};
      const cx<ff> w = tw[(j * m) & (kN - 1)];
      buf[swz<ff>(pr * ld + q)] = twmul<ff>::mul(z, w);
    }
    __syncthreads();
    store_pairs(buf, ld, out, p0, np);
  }
}

}  // namespace
}  // namespace fddm

extern "C" int fddm_b200_experiment_dft_stage(int variant, const void* d_rows, uint64_t npairs, void* d_out,
                                              void* stream) {
  using namespace fddm;
  set_last_error("");
  if (!d_rows || !d_out) return fail_with(FDDM_ERR_INVALID, "null pointer argument");
  if (variant != 0 && variant != 1) return fail_with(FDDM_ERR_INVALID, "variant must be 0 or 1");
  if (npairs == 0) return FDDM_OK;
  if (npairs > (1ull << 30)) return fail_with(FDDM_ERR_UNSUPPORTED, "too many row pairs");
  std::string err;
  FftTables t;
  if (!get_tables(kN, 0, t, err)) return fail_with(FDDM_ERR_CUDA, err);
  const int radices[4] = {8, 4, 8, 4};
  FftPlan p;
  if (!plan_from_radices(kN, radices, 4, p) || !attach_pass_tables(p, 0, err))
    return fail_with(FDDM_ERR_CUDA, err.empty() ? "plan" : err);
  const int ld = kN + swz_group<ff>::G;
  const size_t smem_b = (size_t)swz_round<ff>(kPairs * ld) * sizeof(cx<ff>);
  const size_t smem_f = smem_b + (size_t)kSumTile * sizeof(SliceSums);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int items = (int)((npairs + kPairs - 1) / kPairs);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t ce;
  if (variant == 0) {
    if ((ce = cudaFuncSetAttribute(k_exp_butterfly, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b)) !=
        cudaSuccess)
      return fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
    const unsigned grid = (unsigned)std::min(items, 2 * nsm);
    k_exp_butterfly<<<grid, 256, smem_b, st>>>(static_cast<const uint8_t*>(d_rows), (int)npairs, p,
                                               static_cast<cx<ff>*>(d_out));
  } else {
    if ((ce = cudaFuncSetAttribute(k_exp_gemm_floor, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_f)) !=
        cudaSuccess)
      return fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
    const unsigned grid = (unsigned)std::min(items, 2 * nsm);
    k_exp_gemm_floor<<<grid, 256, smem_f, st>>>(static_cast<const uint8_t*>(d_rows), (int)npairs,
                                                static_cast<const cx<ff>*>(t.tw), static_cast<cx<ff>*>(d_out));
  }
  if ((ce = cudaGetLastError()) != cudaSuccess) return fail_with(FDDM_ERR_CUDA, cudaGetErrorString(ce));
  count_launches(1);
  return FDDM_OK;
}
