/*
 * fddm_b200.h - C ABI of the GB300 (sm_103a) image-structure-function core.
 *
 * This library is the device-side replacement of FastDDM's native cores for the
 * path  fastddm.ddm(img_seq, lags, mode='fft'|'diff', window=...)  and of the
 * binning loops of fastddm.azimuthal_average.  Every function:
 *   - returns an int status (FDDM_OK == 0) and never exits or aborts the process;
 *     the message of the last failure on the calling thread is available from
 *     fddm_b200_last_error();
 *   - takes caller-owned DEVICE buffers (plain pointers and sizes) and a CUDA
 *     stream passed as void* (a cudaStream_t; NULL = legacy default stream);
 *   - enqueues work on that stream and returns without synchronising.
 * The library keeps one cache per device: FFT twiddle and permutation tables,
 * allocated on first use of a transform length.
 *
 * Reference interfaces replaced (paths inside the FastDDM source tree):
 *   src/cpp/ddm.h:54-61        ddm_fft<T>(img_seq, lags, nx, ny, nt, chunk_size, window)
 *   src/cpp/ddm.h:38-43        ddm_diff<T>(img_seq, lags, nx, ny, window)
 *   src/cuda/ddm_cuda.h:53     ddm_fft_cuda<T>(...)   (same contract, cuFFT/FP64)
 *   src/cuda/ddm_cuda.h:38     ddm_diff_cuda<T>(...)
 *   src/python/bindings/ddm_bindings.h:25-43   one overload per input dtype
 *   src/python/azimuthalaverage.py:277-478     azimuthal_average_array binning
 *   src/python/imagestructurefunction.py:409-627  SFWriter (.sf.ddm files)
 *   src/python/utils.py:23-258                 read_images / tiff2numpy (TIFF ingest)
 * The file functions (fddm_b200_sf_write, fddm_b200_tiff_*) work on host
 * memory and files and return when done.
 */
#ifndef FDDM_B200_H
#define FDDM_B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FDDM_OK 0
#define FDDM_ERR_INVALID 1     /* bad argument (sizes, lags, dtype, null pointer) */
#define FDDM_ERR_NOMEM 2       /* workspace too small / device allocation failed */
#define FDDM_ERR_CUDA 3        /* a CUDA runtime call or kernel launch failed */
#define FDDM_ERR_UNSUPPORTED 4 /* valid input the library cannot process (e.g. T too long) */

/* input pixel types: the nine dtypes the reference binds (ddm_bindings.h:25-43).
   64-bit integers are converted to double by the caller, as the reference's
   cast to Scalar does (ddm.cc:288-297); the kernels accept the other seven. */
#define FDDM_U8 0
#define FDDM_I16 1
#define FDDM_U16 2
#define FDDM_I32 3
#define FDDM_U32 4
#define FDDM_I64 5
#define FDDM_U64 6
#define FDDM_F32 7
#define FDDM_F64 8

/* arithmetic tiers */
#define FDDM_PREC_FF 0  /* float-float (~48-bit) FFTs and sums on FP32 pipes: FP64-class accuracy */
#define FDDM_PREC_F64 1 /* native FP64 everywhere (the reference's arithmetic, slow on GB300) */
#define FDDM_PREC_F32 2 /* FP32 FFTs, float-float sums and combination (fast, ~1e-4 relative) */

/* modes */
#define FDDM_MODE_FFT 0  /* Wiener-Khinchin: autocorrelation by zero-padded temporal FFT */
#define FDDM_MODE_DIFF 1 /* direct differences <|F(t+lag) - F(t)|^2>_t */

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int fddm_b200_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* fddm_b200_last_error(void);

/* Device workspace (bytes) needed by fddm_b200_ddm_fft / _diff for these sizes.
   Replaces the host/device memory planners of the reference
   (src/python/_ddm_cpp.py:114-139, src/cuda/memchk_gpu.cu:653-702).
   nt is ignored for FDDM_MODE_DIFF. */
int fddm_b200_workspace_size(int mode, int precision, uint64_t length, uint64_t height, uint64_t width,
                             uint64_t nlags, uint64_t nx, uint64_t ny, uint64_t nt, int has_window,
                             size_t* bytes);

/* Image structure function, fft mode.  Replaces ddm_fft<T> (src/cpp/ddm.h:54-61,
   src/cpp/ddm.cc:250-453) and ddm_fft_cuda<T> (src/cuda/ddm_cuda.h:53).
     d_img_seq   (length, height, width) C-contiguous frames of `dtype`
     lags        HOST array of nlags lags in [0, length-1] (the reference's vector<unsigned>);
                 fft mode needs them strictly increasing, as the reference's fft core
                 does (src/cpp/ddm.cc:403 matches them from the end), diff mode takes any order
     nx, ny      padded FFT sizes (>= width, height; factors 2,3,5,7,11,13)
     nt          the reference's temporal FFT length; must be >= 2*length-1.  Any
                 such length gives the same linear autocorrelation, so the library
                 uses its own cheapest transform length >= 2*length-1
     d_window    (height, width) FP64 window or NULL (the reference's empty window)
     d_out       (nlags + 2, ny, nx/2 + 1) FP64 output: D(lag) rows in the order of
                 `lags`, then the power spectrum, then the variance; rows y-fftshifted
                 exactly as make_shifted_isf (src/cpp/helper_ddm.cc:41-103) leaves them.
     d_workspace at least fddm_b200_workspace_size(...) bytes.
   chunk_size of the reference has no counterpart: the q axis is never chunked. */
int fddm_b200_ddm_fft(const void* d_img_seq, int dtype, uint64_t length, uint64_t height, uint64_t width,
                      const uint32_t* lags, uint64_t nlags, uint64_t nx, uint64_t ny, uint64_t nt,
                      const double* d_window, double* d_out, void* d_workspace, size_t workspace_bytes,
                      int precision, void* stream);

/* Image structure function, diff mode.  Replaces ddm_diff<T> (src/cpp/ddm.h:38-43,
   src/cpp/ddm.cc:37-192) and ddm_diff_cuda<T> (src/cuda/ddm_cuda.h:38).
   Arguments as fddm_b200_ddm_fft without nt. */
int fddm_b200_ddm_diff(const void* d_img_seq, int dtype, uint64_t length, uint64_t height, uint64_t width,
                       const uint32_t* lags, uint64_t nlags, uint64_t nx, uint64_t ny,
                       const double* d_window, double* d_out, void* d_workspace, size_t workspace_bytes,
                       int precision, void* stream);

/* Image structure function from frames in HOST memory (the reference's cores
   take host arrays: src/cpp/ddm.h:38-61).  Page-locked frames (mapped into
   the device's address space under unified addressing) are read in place by
   the spatial kernels, over NVLink-C2C on Grace parts, and d_frames is not
   touched (it may be NULL; that needs rows of a multiple of 16 bytes starting
   on 16-byte boundaries, else the call fails with FDDM_ERR_INVALID before any
   work is queued).  Pageable frames (or any, with FDDM_B200_ZERO_COPY=0 in the
   environment) are copied chunk by chunk from h_img_seq into the caller's
   device buffer
   d_frames (length*height*width elements) on a library copy stream; each
   chunk's spatial FFTs wait only for that chunk.  If h_out is not NULL the
   result is also copied to it, in column chunks overlapped with the temporal
   stage.
   mode is FDDM_MODE_FFT or FDDM_MODE_DIFF (nt ignored for diff); the other
   arguments as fddm_b200_ddm_fft.  The host buffers must stay valid until the
   work on `stream` has completed. */
int fddm_b200_ddm_from_host(int mode, const void* h_img_seq, int dtype, uint64_t length, uint64_t height,
                            uint64_t width, const uint32_t* lags, uint64_t nlags, uint64_t nx, uint64_t ny,
                            uint64_t nt, void* d_frames, const double* d_window, double* d_out, double* h_out,
                            void* d_workspace, size_t workspace_bytes, int precision, void* stream);

/* Batched jobs: many independent stacks of uneven size, length and mode in
   one call (the reference processes one stack per call; this replaces a
   Python loop over ddm() for multi-ROI analysis).  Each job is the argument
   list of fddm_b200_ddm_fft / _diff. */
typedef struct fddm_b200_job {
  int mode;                 /* FDDM_MODE_FFT or FDDM_MODE_DIFF */
  const void* d_img_seq;    /* (length, height, width) device frames */
  int dtype;                /* FDDM_U8 ... FDDM_F64 (64-bit integers excluded) */
  uint64_t length, height, width;
  const uint32_t* lags;     /* host, nlags entries */
  uint64_t nlags;
  uint64_t nx, ny, nt;      /* nt ignored in diff mode */
  const double* d_window;   /* (height, width) or NULL */
  double* d_out;            /* (nlags + 2, ny, nx/2 + 1) */
} fddm_b200_job;

/* Workspace bytes of a batch of these jobs (the jobs' own workspaces, 256-byte
   aligned, and the tables of the many-job temporal kernel). */
int fddm_b200_batch_workspace_size(const fddm_b200_job* jobs, uint64_t njobs, int precision, size_t* bytes);

/* A prepared batch.  fddm_b200_batch_create validates every job, puts each
   job's lag and slot tables into its part of d_workspace and sets up every
   temporal stage (queued on `stream`; the launch tuning of each job's class is
   resolved here, which may time candidates once when the autotuner is on).
   fddm_b200_batch_launch then enqueues kernels and event dependencies only, so
   a stream capture of it gives a CUDA graph of the whole batch:
     - the spatial stages, longest first, onto library-owned streams forked
       from `stream`;
     - the temporal stages of all fft-mode jobs as one persistent launch of a
       many-job kernel per kernel variant and CTA size, whose CTAs take runs of
       32 modes of any job from a counter (the other stages launch per job);
     - a join back into `stream`, so the batch completes in stream order.
   The frames, windows and outputs of the jobs and d_workspace must stay valid
   for the plan's life; launch on `stream` (or after the create's work on it
   has completed).  Each job's result is identical to running it alone. */
typedef struct fddm_b200_batch fddm_b200_batch;
int fddm_b200_batch_create(const fddm_b200_job* jobs, uint64_t njobs, int precision, void* d_workspace,
                           size_t workspace_bytes, void* stream, fddm_b200_batch** plan);
int fddm_b200_batch_launch(fddm_b200_batch* plan, void* stream);
int fddm_b200_batch_destroy(fddm_b200_batch* plan);

/* Create, launch and destroy in one call. */
int fddm_b200_batch_run(const fddm_b200_job* jobs, uint64_t njobs, int precision, void* d_workspace,
                        size_t workspace_bytes, void* stream);

/* Weighted azimuthal average of a stack of half-plane maps: the per-(bin, row)
   weighted mean and unbiased weighted standard deviation.  Replaces the two
   per-pixel loops of azimuthal_average_array (src/python/azimuthalaverage.py:435-444
   and :457-476) as called by azimuthal_average (:481-564).  The caller does the
   O(pixels) set-up the reference does before those loops (bin search, masking,
   sum of weights per bin, :394-432) and passes each bin's pixels in increasing
   pixel order.  One thread accumulates one (bin, row) in that order with the
   reference's operation order and IEEE round-to-nearest FP64 operations, so the
   result does not depend on scheduling.
     d_data        (nrows, npix) FP64 maps (the structure function's _data)
     d_bin_offsets nbins + 1 offsets into d_bin_pixels (CSR)
     d_bin_pixels  pixel indices of every bin, increasing within a bin
     d_weight      npix FP64 weight per pixel (counts x weights)
     d_sumw        nbins FP64 sum of weights per bin
     d_bias        nbins FP64 sum_w - sum_w2/sum_w (or NULL when d_err is NULL)
     d_avg         (nbins, nrows) out: weighted mean; NaN where sum_w == 0
     d_err         (nbins, nrows) out: sqrt(sum w (x - mean)^2 / bias); NaN where
                   sum_w == 0; NULL to skip */
int fddm_b200_azimuthal_average(const double* d_data, uint64_t nrows, uint64_t npix,
                                const int32_t* d_bin_offsets, const int32_t* d_bin_pixels, uint64_t nbins,
                                const double* d_weight, const double* d_sumw, const double* d_bias,
                                double* d_avg, double* d_err, void* stream);

/* The same averages in a fast order (no counterpart in the reference): one
   warp per (bin, row) sums the bin's pixels with FP64 fused multiply-adds in a
   fixed lane order and divides the weighted sum by sum_w once.  Results are
   reproducible from run to run and differ from fddm_b200_azimuthal_average by
   rounding only (relative 1e-12 is the tested bound).  Arguments as above. */
int fddm_b200_azimuthal_average_fast(const double* d_data, uint64_t nrows, uint64_t npix,
                                     const int32_t* d_bin_offsets, const int32_t* d_bin_pixels, uint64_t nbins,
                                     const double* d_weight, const double* d_sumw, const double* d_bias,
                                     double* d_avg, double* d_err, void* stream);

/* Image structure function, fft mode, without any device allocation.
   This entry point has no counterpart in the reference.  It is for callers
   that cannot call cudaMalloc when they need a result (an acquisition callback
   that must not wait on the allocator, a plugin whose host owns all device
   memory): the caller passes the frames, the window and the output only, and
   the library calls no cudaMalloc, cudaFree or allocating routine.  Its scratch
   is one 64 MiB array in device memory that every device loading the library
   holds until the process exits; a problem needing more is rejected with
   FDDM_ERR_NOMEM.  All calls share that array, so calls that overlap on the GPU
   race and must be serialised by the caller.  The first call on a device looks
   up the array's device address with that device current, and under CUDA's
   default lazy module loading that is also when the device reserves the
   64 MiB: make one first call (any valid problem that fits) before reserving
   the rest of device memory and before any stream capture.  Without room for
   the array at that point the call returns FDDM_ERR_NOMEM.  Arguments and
   result as fddm_b200_ddm_fft. */
int fddm_b200_ddm_fft_noalloc(const void* d_img_seq, int dtype, uint64_t length, uint64_t height, uint64_t width,
                              const uint32_t* lags, uint64_t nlags, uint64_t nx, uint64_t ny, uint64_t nt,
                              const double* d_window, double* d_out, int precision, void* stream);

/* Image structure function file (.sf.ddm): replaces the reference's
   ImageStructureFunction.save / SFWriter.write_obj
   (src/python/imagestructurefunction.py:279-293, 409-627; header constants in
   src/python/_io_common.py:16-17) and writes the same bytes: a 64-byte header
   ("LL"/"BB", id 73, version 0.3, 'd', the six sizes), _data, kx, ky, tau,
   pixel_size, delta_t and the seven byte offsets.
     path          output file (created or truncated; the directory must exist)
     data          (length + extra, height, width) FP64 in C order: the
                   structure function rows, then the extra rows (PS, VAR)
     data_on_device 0: `data` is host memory; 1: device memory, streamed to the
                   file in 32 MiB chunks through two pinned staging buffers
                   (allocated on the device's first such call and kept), each
                   copy overlapping the write of the previous chunk and ordered
                   after the work queued on `stream`
     length        number of lags; height = ny; width = nx/2 + 1; extra = 2
     full_width, full_height  nx, ny of the full plane
     kx, ky, tau   host arrays of width, height and length values
   Returns FDDM_ERR_INVALID with the system's message when the file cannot be
   written.  The call returns when the file is complete. */
int fddm_b200_sf_write(const char* path, const double* data, int data_on_device, uint64_t length, uint64_t height,
                       uint64_t width, uint64_t extra, uint64_t full_width, uint64_t full_height, const double* kx,
                       const double* ky, const double* tau, double pixel_size, double delta_t, void* stream);

/* Camera-noise estimate, "polyfit" mode on the image structure function:
   replaces the per-pixel numpy.polyfit(tau, D, 2, cov=True) loop of the
   reference's _noise_polyfit_img_str_func (src/python/noise_est.py:686-756).
     d_data   device rows of the structure function, row k at d_data + k*ld
              (ld = ny*(nx/2+1)); rows 0 .. npts-1 are fitted
     npix     pixels per row (<= ld)
     x        host abscissae (the first npts lags, tau[:npts])
     p        host (3, npts) least-squares operator of the quadratic fit
              (rows: coefficients of x^2, x, 1), cov22 the (2, 2) entry of
              inv(V^T V) for the Vandermonde matrix V of x
     d_noise, d_unc  device outputs (npix): the constant term and
              sqrt(cov22 * residual / (npts - 3)); NaN where row 0 is NaN
   4 <= npts <= 64 (numpy needs more points than coefficients to scale the
   covariance). */
int fddm_b200_polyfit_noise(const double* d_data, uint64_t ld, uint64_t npix, const double* x, const double* p,
                            uint64_t npts, double cov22, double* d_noise, double* d_unc, void* stream);

/* Image ingest: replaces the reference's TIFF path of read_images /
   tiff2numpy (src/python/utils.py:23-111, 218-258, through tifffile).
   Grayscale TIFF files, classic or BigTIFF, either byte order, in strips,
   uncompressed, LZW (with or without horizontal predictor) or PackBits;
   8-bit unsigned, 16/32/64-bit signed or unsigned and 32/64-bit float samples.
   fddm_b200_tiff_info returns the number of pages, their height and width and
   the FDDM dtype code (all pages must agree).  fddm_b200_tiff_read decodes the
   listed pages (0-based, any order, repeats allowed) into `dst`, page i of the
   list at byte offset i * height * width * sample bytes, in host byte order;
   `nthreads` host threads share the pages (uncompressed strips are read
   straight into `dst`).  Files the reader cannot decode (tiles, colour, other
   compressions) return FDDM_ERR_UNSUPPORTED with the reason. */
int fddm_b200_tiff_info(const char* path, uint64_t* npages, uint64_t* height, uint64_t* width, int* dtype);
int fddm_b200_tiff_read(const char* path, const uint64_t* pages, uint64_t npages, void* dst, int nthreads);

/* Launch tuning of the temporal kernels (no counterpart in the reference,
   which has fixed launch shapes; its memory planner, src/cuda/memchk_gpu.cu:141-702,
   only sizes chunks).  A problem class is (precision, mode, length, nlags);
   its entry holds the CTA size (128, 256 or 512 threads) and whether the
   needed prefix sums and per-lag tables sit in shared memory (need_in_smem=1)
   or in global scratch.  Without an entry the library uses its occupancy
   model; with fddm_b200_set_autotune(1), the first call of a class without an
   entry times every candidate on that call's own spectrum (the call then
   waits for the GPU once) and records the fastest.  Entries only change the
   launch shape and the order of the per-mode sums (results within rounding
   of each other; every call of one class in a process uses the same entry).
   fddm_b200_tuning_count / _entry enumerate the table (for saving it). */
int fddm_b200_set_autotune(int enable);
int fddm_b200_tuning_set(int precision, int mode, uint64_t length, uint64_t nlags, int threads, int need_in_smem);
int fddm_b200_tuning_get(int precision, int mode, uint64_t length, uint64_t nlags, int* threads, int* need_in_smem);
uint64_t fddm_b200_tuning_count(void);
int fddm_b200_tuning_entry(uint64_t index, int* precision, int* mode, uint64_t* length, uint64_t* nlags, int* threads,
                           int* need_in_smem);

/* Diagnostics (no counterpart in the reference, which has no tracing).
   fddm_b200_set_stage_timing(1) makes every following ddm call record CUDA
   events on its stream around the spatial stage (row and column FFT passes)
   and the temporal stage; fddm_b200_stage_times waits for the last call's
   events and returns the two durations in milliseconds.
   fddm_b200_launch_count returns the number of kernels this library has
   launched in the process so far.
   fddm_b200_last_input_path tells how the last structure-function call on
   the calling thread took its frames: 0 from device memory, 1 from host
   memory read in place by the row pass, 2 from host memory uploaded to the
   device buffer. */
int fddm_b200_set_stage_timing(int enable);
int fddm_b200_stage_times(float* spatial_ms, float* temporal_ms);
uint64_t fddm_b200_launch_count(void);
int fddm_b200_last_input_path(void);

/* Measurement behind the decision not to run a DFT stage on the tensor cores
   (no counterpart in the reference).  d_rows holds npairs pairs of 8-bit rows
   of 1024 pixels; d_out receives npairs x 1024 float-float complex values.
   variant 0: the two float-float DIF passes (radix 8, radix 4) forming the
   radix-32 first stage of the packed pair's 1024-point transform, as in the
   row pass; variant 1: the CUDA-core work a 5-slice bf16 DFT-as-GEMM version
   of that stage would still need (combining ten FP32 slice sums per output
   into float-float, packing the pair, the inter-stage twiddle), with the slice
   sums taken from shared memory and no MMA: a lower bound on its time. */
int fddm_b200_experiment_dft_stage(int variant, const void* d_rows, uint64_t npairs, void* d_out, void* stream);

/* Batched Levenberg-Marquardt fits of the relaxation models: replaces the
   lmfit Model.fit calls of the reference's fit_multik (src/python/fit.py:337,
   :380) and fit (fit.py:188).  Each fit follows lmfit's default 'leastsq'
   method: MINPACK's lmdif on lmfit's internal parameters (bounds mapped by
   the MINUIT transformations), forward-difference Jacobian, lmfit's
   tolerances, standard errors from inv(R^T R) scaled by chi^2 / nfree.
   Models (parameters in the order of the reference functions' arguments):
     FDDM_FIT_GENERIC_EXP_ISF   A, Gamma, beta        fit_models.py:515
     FDDM_FIT_DOUBLE_EXP_ISF    A, Gamma1, beta1, Gamma2, beta2, alpha   :615
     FDDM_FIT_FLORY_SCHULZ_ISF  A, Gamma, sigma       :690
     FDDM_FIT_GENERIC_EXP_SF    A, B, Gamma, beta     :774
     FDDM_FIT_DOUBLE_EXP_SF     A, B, Gamma1, beta1, Gamma2, beta2, alpha   :890
     FDDM_FIT_FLORY_SCHULZ_SF   A, B, Gamma, sigma    :971
     FDDM_FIT_SIMPLE_EXP        tau, amplitude        fit.py:67
     FDDM_FIT_SIMPLE_SF         A, B, tau             fit.py:84
   A problem is one curve of mp <= m points: abscissae row d_x + xrow*ldx (nx
   rows), data row d_y + row*ldy (ny rows), weights row d_w + wrow*ldw (nw
   rows) or none (residual (model - y) * w), starting values, bounds
   (+-INFINITY for none) and the mask of varying parameters.  d_problems holds
   6 int32 per problem: y row, weight row (-1: none), pred (-1: none), vary
   mask (bit p: parameter p varies; the same number nvary of set bits in every
   problem), x row, mp (nvary <= mp <= m).  With pred >= 0 the varying parameters start
   from problem pred's fitted values instead of d_init (fit_multik's warm
   start); pred must come earlier in the same chain or have been fitted by an
   earlier call.  Starting values are clipped into [min, max] as lmfit does.
   Chains: chain c runs problems d_chain_problems[d_chain_offsets[c] ..
   d_chain_offsets[c+1]-1] in order on one warp, or on a CTA of four warps
   when there are at most four chains per SM; chains run concurrently.
   d_init, d_min, d_max, d_values, d_stderr: [nproblems][nparams] doubles.
   options (host, 6 doubles): ftol, xtol, gtol, epsfcn, factor, max_nfev
   (<= 0: 2000*(nvary+1); above 1,000,000: FDDM_ERR_UNSUPPORTED); lmfit's
   defaults are 1e-7, 1e-7, 1e-7, 0, 100, 0.
   Outputs per problem: fitted values (fixed parameters keep theirs),
   standard errors (0 for fixed parameters; NaN where the covariance has
   entries that are not finite, e.g. a parameter exactly on a bound; -1 for
   every parameter when R^T R is exactly singular or the fit did not
   finish), chi^2, function evaluations, MINPACK's info (1-4
   converged, 6-8 tolerance too small, -1 aborted), status (0 done, 1 a
   residual was not finite: the reference raises ValueError there and the
   chain stops, 2 aborted after max_nfev evaluations, 3 not fitted: a row,
   predecessor or point count out of range or another number of varying
   parameters; a
   chain also ends at an entry that is not a problem), and optionally the
   final residuals ([nproblems][m], the first mp of each row; d_residual may
   be NULL) and the covariance of the parameters ([nproblems][nparams]
   [nparams], scaled by chi^2 / nfree, zero rows and columns for fixed
   parameters, NaN where it has no finite value; d_covar may be NULL).
   The workspace holds (2 + nparams) * m doubles per concurrently running
   chain; fddm_b200_fit_workspace_bytes gives the size that runs every chain
   at once (a smaller one runs fewer at a time, down to one). */
#define FDDM_FIT_GENERIC_EXP_ISF 0
#define FDDM_FIT_DOUBLE_EXP_ISF 1
#define FDDM_FIT_FLORY_SCHULZ_ISF 2
#define FDDM_FIT_GENERIC_EXP_SF 3
#define FDDM_FIT_DOUBLE_EXP_SF 4
#define FDDM_FIT_FLORY_SCHULZ_SF 5
#define FDDM_FIT_SIMPLE_EXP 6
#define FDDM_FIT_SIMPLE_SF 7
int fddm_b200_fit_model_nparams(int model);
int fddm_b200_fit_workspace_bytes(int model, uint64_t m, uint64_t nchains, uint64_t* bytes);
int fddm_b200_fit_lm(int model, uint64_t m, const double* d_x, uint64_t ldx, uint64_t nx, const double* d_y,
                     uint64_t ldy, uint64_t ny, const double* d_w, uint64_t ldw, uint64_t nw,
                     const int32_t* d_problems, uint64_t nproblems,
                     const int32_t* d_chain_offsets,
                     const int32_t* d_chain_problems, uint64_t nchains, int nvary, const double* d_init,
                     const double* d_min, const double* d_max, const double* options, double* d_values,
                     double* d_stderr, double* d_chisqr, int32_t* d_nfev, int32_t* d_info, int32_t* d_status,
                     double* d_residual, double* d_covar, void* d_workspace, uint64_t workspace_bytes,
                     void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FDDM_B200_H */
