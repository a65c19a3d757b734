// Internal host/device structures shared by the kernels and the C ABI layer.
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <mutex>
#include <string>
#include <vector>
#include <cuda_runtime.h>

namespace fddm {

constexpr int kMaxPass = 24;

struct FftPlan {
  int n;                // transform length
  int npass;            // number of passes
  int lgn;              // log2(n), or -1 when n is not a power of two
  int radix[kMaxPass];  // radix of pass s
  int block[kMaxPass];  // block size M_s at pass s (M_0 = n)
  int lgstride[kMaxPass];  // log2(M_s / R_s) when a power of two, else -1
  int lgbpf[kMaxPass];     // log2(n / R_s) when a power of two, else -1
  // per-pass twiddle tables (device, null when not attached or stride 1): pass
  // s reads w_M^(j m) at ptw[s][(m - 1) * stride + j], contiguous in j, so a
  // warp's twiddle loads are coalesced (attach_pass_tables)
  const void* ptw[kMaxPass];
};

struct SpatialArgs {
  const void* img;       // (T, H, W) frames, input dtype
  const void* window_s;  // (H, W) window in the FFT scalar type, or null
  int T, H, W, nx, ny, nkx, Hpad;
  int t0, tc;            // first frame and number of frames of this chunk
  int Tpad;              // spectrum row stride (elements)
  int pairs_per_block, cols_per_block, frames_per_block;
  int raw_stage_bytes;   // >0: rows are staged with cp.async (16-byte aligned rows)
  FftPlan px, py;
  const void* twx;
  const void* twy;
  const int* permx;
  const int* permy;
  void* rbuf;            // (tc, nkx, Hpad) row-pass output
  void* spec;            // (Q, Tpad) spectrum, q-major, y-shifted q order
  float norm_h, norm_l;  // 1/sqrt(nx*ny) as hi/lo floats
  double norm_d;
};

struct TemporalArgs {
  const void* spec;
  size_t Q;                // modes (the output's row stride)
  size_t q_begin, q_end;   // modes of this launch
  int Tpad, T, nt, nlags;  // nt: the temporal transform length N chosen by plan_layout
  FftPlan pt, pt2;         // plan for N and the half-length plan derived from it (half_plan)
  const void* twt;         // twiddles of length N
  const void* twt2;        // twiddles of length N/2
  const int* slotA;      // (T + 1): lag index l with T - lag_l == t, or -1
  const int* slotB;      // (T + 1): lag index l with lag_l == t, or -1
  void* need;            // per-CTA scratch, (2 * nlags + 2) accumulators per CTA
  int need_in_smem;      // 1: the needed prefix sums live in shared memory instead
  const int* lags;       // device, nlags
  const double* rcp;     // device, 1/(T - lag)
  double* out;           // (nlags + 2, Q)
  float invT_h, invT_l;
  double invT_d;
  float invnt_h, invnt_l;
  double invnt_d;
  // long series (k_tfft_long): N = R0 * M1, sub-transforms of length M1
  int R0, M1;
  FftPlan pm;             // plan of the length-M1 sub-transforms
  const void* twm;        // twiddles of length M1
  void* xs;               // per-CTA global scratch: X (N values), then the prefix sums (T accumulators)
  size_t xs_stride;       // bytes per CTA
  size_t xs_pfx_off;      // offset of the prefix sums inside one CTA's scratch
};

// A work item of the many-job temporal kernel (k_tfft_list): modes q0 .. q1 - 1 of job `job`.
struct TemporalItem {
  int job;
  int pad;
  unsigned long long q0, q1;
};

// The temporal stage of one job, set up but not launched (DdmRequest::collect):
// its arguments and launch shape, and whether the many-job kernel can run it
// (the shared-memory fft kernel; variant 0 generic, 1 radices 2/4/8, 2 the
// fused radix-2 path; -1 other kernels).
struct TemporalLaunch {
  TemporalArgs args;
  int threads = 0;
  size_t smem = 0;
  int variant = -1;
};

// One launch of the many-job temporal kernel: jobs of one variant and CTA size.
struct TemporalListGroup {
  int variant = 0, threads = 0;
  size_t smem = 0;              // dynamic shared memory (the largest of the group's jobs)
  const TemporalArgs* d_args = nullptr;
  const TemporalItem* d_items = nullptr;
  int nitems = 0;
  int* d_counter = nullptr;     // zeroed on the launch stream before the launch
};

enum Precision { PREC_FF = 0, PREC_F64 = 1, PREC_F32 = 2 };
enum Mode { MODE_FFT = 0, MODE_DIFF = 1 };
enum DType { DT_U8 = 0, DT_I16 = 1, DT_U16 = 2, DT_I32 = 3, DT_U32 = 4, DT_I64 = 5, DT_U64 = 6, DT_F32 = 7, DT_F64 = 8 };

struct DdmRequest {
  int mode = 0;
  int precision = 0;
  const void* img = nullptr;
  int dtype = 0;
  int64_t T = 0, H = 0, W = 0;
  std::vector<int> lags;
  int64_t nx = 0, ny = 0, nt = 0;
  const double* window = nullptr;  // device (H, W) or null
  double* out = nullptr;           // device (nlags + 2, ny, nx/2 + 1)
  void* work = nullptr;
  size_t work_bytes = 0;
  // Workspace-only mode: FFT tables are copied into the workspace on every
  // call instead of coming from the per-device cache (which allocates on
  // first use), and the frame chunk shrinks until the layout fits max_work.
  bool inline_tables = false;
  size_t max_work = 0;  // 0: no limit
  // Host-resident input: frames are copied chunk by chunk from host_img into
  // the device buffer `img` on a library copy stream, each chunk just before
  // the spatial passes that read it; host_out (optional) receives the result.
  const void* host_img = nullptr;
  double* host_out = nullptr;
  // Batched use: the lag, normalisation and slot tables are already in the
  // workspace (put there by an earlier call of the same request), `stages`
  // selects the spatial (1) and temporal (2) launches, and a non-null
  // `collect` receives the temporal stage's arguments instead of a launch.
  bool tables_ready = false;
  int stages = 3;
  TemporalLaunch* collect = nullptr;
};

// Per-device copy stream and event used to overlap frame uploads with compute.
// One per device: the events are re-recorded by every call, so a call holds
// `mu` from its first record to its last wait (calls from several threads
// would otherwise wait on each other's events).
struct CopyCtx {
  cudaStream_t stream = nullptr;
  cudaEvent_t ready = nullptr, start = nullptr;
  std::mutex mu;
};
CopyCtx* copy_ctx(std::string& err);
size_t dtype_bytes(int dtype);

struct WorkLayout {
  size_t spec_off, spec_bytes;
  size_t rbuf_off, rbuf_bytes;
  size_t win_off, win_bytes;
  size_t lags_off, rcp_off, slot_off, need_off;
  size_t tables_off, tables_bytes;  // inline FFT tables (DdmRequest::inline_tables)
  size_t xs_off, xs_stride, xs_pfx_off;  // long-series temporal scratch (per CTA)
  size_t total;
  int Tpad, Hpad, chunk, pairs_per_block, cols_per_block, frames_per_block;
  int nt_fft;  // temporal transform length actually used (fft mode)
  int long_R0;  // fft mode: >0 selects the long-series kernel with this first radix
  int diff_staged;  // diff mode: 1 when the series is staged in shared memory
  bool over_max_work = false;  // plan_layout failed only because DdmRequest::max_work is too small
};

// Upper bound on the temporal kernel's grid (sizes its per-CTA scratch).
constexpr int kMaxTemporalCtas = 1024;
// Upper bound on the long-series temporal kernel's grid (one CTA per SM on
// current parts; sizes its per-CTA transform scratch).
constexpr int kMaxLongCtas = 304;

// Cheapest even length >= 2T - 1 for the temporal transform (fft mode).
int choose_temporal_length(int64_t T);

// Shared memory of the fft-mode temporal kernel for element sizes es (FFT
// scalar complex) and ea (accumulator); `need_in_smem` selects the layout.
size_t temporal_fft_smem(int T, int N, int nlags, size_t es, size_t ea, bool need_in_smem);
constexpr size_t kSmemLimit = 232448;  // 227 KB opt-in per CTA
// Shared memory of the long-series fft-mode kernel (sub-transforms of length M1).
size_t temporal_long_smem(int M1, size_t es, size_t ea);

// Launch configuration of a temporal kernel (CTA size; the needed prefix sums
// and per-lag tables in shared memory or in global scratch), and the tuning
// table the autotuner fills (tune.cu), keyed by (precision, mode, T, nlags).
struct TemporalChoice {
  int threads;
  int need_in_smem;
};
bool tuned_temporal(int precision, int mode, int64_t T, int64_t nlags, TemporalChoice& out);
void record_temporal(int precision, int mode, int64_t T, int64_t nlags, const TemporalChoice& c);
bool autotune_enabled();

// Thread-local error message reported by fddm_b200_last_error().
void set_last_error(const std::string& msg);
int fail_with(int code, const std::string& msg);

// Diagnostics: kernel launch counter and optional stage events.
void count_launches(int n);
// How the last call on this thread took its frames: 0 device memory, 1 host
// memory read in place, 2 host memory uploaded (fddm_b200_last_input_path).
void set_last_input_path(int path);
struct StageEvents {
  bool enabled;
  cudaEvent_t ev[3];
};
// Events of the calling device when stage timing is enabled, else nullptr.
StageEvents* stage_events();

// Element size of the spectrum for a precision tier.
size_t spec_elem_bytes(int precision);
// Plan the workspace; returns false with a message when the problem is unsupported.
bool plan_layout(const DdmRequest& r, WorkLayout& L, std::string& err);
// Factor n into supported radices; false if n has another prime factor.
bool make_plan(int n, FftPlan& p);
// Plan of length n with the given radices (their product must be n).
bool plan_from_radices(int n, const int* radices, int npass, FftPlan& p);
// Plan of length n/2 whose digit-reversed order matches the even outputs of
// p: radices (R_0/2, R_1, ...), the first dropped when R_0 = 2.  Requires an
// even n and an even R_0 (make_plan puts the radices 8, 4, 2 first).
bool half_plan(const FftPlan& p, FftPlan& h);
// Plan of the length-n temporal transform (n even): the even first radix that
// makes the padded first pass and the half-length transform cheapest.
bool temporal_plan(int n, FftPlan& p);

// Per-precision pipeline entry points (instantiated in ddm_ff.cu, ddm_f64.cu, ddm_f32.cu).
int run_ddm_ff(const DdmRequest& r, cudaStream_t st, std::string& err);
int run_ddm_f64(const DdmRequest& r, cudaStream_t st, std::string& err);
int run_ddm_f32(const DdmRequest& r, cudaStream_t st, std::string& err);
// One launch of the many-job temporal kernel (zeroes the group's counter first).
int run_temporal_list_ff(const TemporalListGroup& g, cudaStream_t st, std::string& err);
int run_temporal_list_f64(const TemporalListGroup& g, cudaStream_t st, std::string& err);
int run_temporal_list_f32(const TemporalListGroup& g, cudaStream_t st, std::string& err);
// Static shared memory of the many-job kernel (its copy of the job's arguments).
constexpr size_t kListStaticSmem = sizeof(TemporalArgs) + 64;

// Attach the cached per-device pass twiddle tables of `p` (kind as get_tables).
bool attach_pass_tables(FftPlan& p, int kind, std::string& err);
// Workspace-only mode: copy the pass tables of `p` to `dst` (at most `room`
// bytes, 256-byte aligned parts) on `st` and attach them.
bool upload_pass_tables(FftPlan& p, int kind, unsigned char* dst, size_t room, cudaStream_t st, std::string& err);
// Bytes the pass tables of any plan of length n take in a workspace (bound).
size_t pass_tables_bound(int n, int kind);

// Cached per-device FFT tables (twiddles in the requested scalar format, permutation).
struct FftTables {
  FftPlan plan;
  const void* tw;
  const int* perm;   // natural index -> position after the forward FFT
  const int* iperm;  // position -> natural index
};
// kind: 0 = ff (16 B twiddles), 1 = double, 2 = float
bool get_tables(int n, int kind, FftTables& out, std::string& err);

// Host copy of the same tables (cached, never freed), for uploading into a
// caller-provided workspace.
struct HostTables {
  FftPlan plan;
  std::vector<unsigned char> tw;
  std::vector<int> perm, iperm;
};
bool host_tables(int n, int kind, const HostTables*& out, std::string& err);
// Bytes one transform's tables take inside a workspace (256-byte aligned parts).
size_t inline_table_bytes(int n, int kind);

}  // namespace fddm
