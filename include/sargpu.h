/*
 * sargpu.h -- C ABI of the GB300 SAR operator library (libsargpu.so).
 *
 * Replaces the native boundary of sarsolver's C++/FFTW kernel:
 *   src/sarsolver/cxx_binding/sarsolver_cxx.hpp:112-119  forward_evaluate / adjoint_evaluate
 *   src/sarsolver/cxx_binding/sarsolver_cxx.hpp:28-33    SarCalculationInfo
 *   src/sarsolver/cxx_binding/sarsolver_cxx.py:214-220   their ctypes bindings
 *
 * Two layers:
 *  1. Drop-in entry points with the reference's exact signatures and struct layout
 *     (forward_evaluate / adjoint_evaluate on SarCalculationInfo*, host FP64 buffers,
 *     FFT-ordered phase history), computed on the current CUDA device.
 *  2. A plan API on device buffers: geometry is uploaded once, then sar_forward /
 *     sar_adjoint run asynchronously on a caller-provided CUDA stream.
 *
 * Plain C types only; a CUDA stream is passed as `void *` (a cudaStream_t).  Every plan
 * call returns a status (SAR_OK == 0) and never aborts; sar_last_error() gives the
 * calling thread's last message.
 *
 * Data layout of the plan API (device memory, complex64 = interleaved float re, im):
 *   image x:          [P]      with P = nz*ny*nx for a grid, index (k*ny + j)*nx + i,
 *                              matching GridSarScene.positions (src/sarsolver/numpy/hypothesis.py:192-206)
 *   phase history y:  [S][N]   fast time fftshifted (centre frequency in the middle), the
 *                              convention of the reference's Python API (cxx_binding/forward.py:44,
 *                              adjoint.py:36)
 */
#ifndef SARGPU_H
#define SARGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define SAR_OK 0
#define SAR_ERR_INVALID_ARGUMENT 1
#define SAR_ERR_CUDA 2
#define SAR_ERR_CUFFT 3
#define SAR_ERR_OUT_OF_MEMORY 4
#define SAR_ERR_NOT_SUPPORTED 5

/* Interpolation of the upsampled range profile. */
#define SAR_INTERP_NEAREST_REF 0 /* the reference's bins: round(v) forward (sarsolver_cxx.cpp:289),
                                    round(0.5+v) adjoint (:347), weight unconjugated (:288, :349) */
#define SAR_INTERP_LINEAR 1      /* linear interpolation; forward and adjoint exact transposes */

/* Device check flags reported by sar_device_flags(). */
#define SAR_FLAG_TILE_WINDOW 1u   /* a tile's staged window left the stored profile span */
#define SAR_FLAG_STRIP_WINDOW 2u  /* a forward strip window left the stored profile span, or a tile's
                                     bins left the range its ring window holds */
#define SAR_FLAG_WAIT_TIMEOUT 8u  /* a bounded in-kernel wait expired; that call's result is invalid */
#define SAR_FLAG_GATHER_WINDOW 16u /* a pixel's range bin could fall outside its tile's staged window
                                      (window narrower than the tile's bin extent); result suspect */

/* ------------------------------------------------------------ 1. drop-in boundary */

/* Byte-for-byte the reference struct (sarsolver_cxx.hpp:28-33). */
typedef struct SarCalculationInfo {
    size_t num_fast_times, num_slow_times, num_scatterers;
    double *transmit_posns, *receive_posns, *stab_ref_posns, *scat_posns;
    double *phase_history, *scattering_amplitudes, *waveform_fft, *slow_time_weighting;
    double centre_frequency, sample_frequency, c_eff, upsample_ratio, sign_multiplier;
} SarCalculationInfo;

/* Replaces forward_evaluate (sarsolver_cxx.hpp:113, sarsolver_cxx.cpp:26-30): writes
 * info->phase_history [S][N][2] (FFT order) from info->scattering_amplitudes.  Reference
 * conventions (SAR_INTERP_NEAREST_REF).  Like the reference it returns nothing; on failure the
 * output is zero-filled and sar_last_error() holds the reason. */
void forward_evaluate(SarCalculationInfo *info);

/* Replaces adjoint_evaluate (sarsolver_cxx.hpp:114, sarsolver_cxx.cpp:32-36): writes
 * info->scattering_amplitudes [P][2] from info->phase_history (FFT order). */
void adjoint_evaluate(SarCalculationInfo *info);

/* ----------------------------------------------------------------- 2. plan API */

typedef struct sar_plan sar_plan;

/* Geometry of one operator.  Host FP64 inputs, copied at plan creation.  Replaces the
 * per-call SarCalculationInfo + SarWorker construction (sarsolver_cxx.cpp:219-252). */
typedef struct sar_geometry {
    size_t num_fast_times;              /* N */
    size_t num_slow_times;              /* S */
    size_t num_scatterers;              /* P (must equal nz*ny*nx when a grid is given) */
    const double *transmit_posns;       /* [S][3] */
    const double *receive_posns;        /* [S][3] */
    const double *stab_ref_posns;       /* [S][3] */
    const double *scat_posns;           /* [P][3]; used when grid_shape is all zero */
    const double *waveform_fft;         /* [N][2] FFT order; NULL = all ones */
    const double *slow_time_weighting;  /* [S][2]; NULL = all ones */
    double centre_frequency, sample_frequency, c_eff, upsample_ratio, sign_multiplier;
    int interp;                         /* SAR_INTERP_* */
    /* Regular grid (fast path): pixel (k, j, i) sits at
     *   grid_origin + i*grid_step_x + j*grid_step_y + k*grid_step_z,
     * grid_shape = {nz, ny, nx}.  All-zero grid_shape selects the unstructured path. */
    size_t grid_shape[3];
    double grid_origin[3], grid_step_x[3], grid_step_y[3], grid_step_z[3];
    /* Kernel path for grids: SAR_PATH_AUTO picks the grid fast path (for SAR_INTERP_NEAREST_REF
     * too: bins within 5e-5 of a rounding boundary are decided again with the per-pixel
     * double-float range, so the nearest-bin decisions match FP64 ranges on both paths), and the
     * per-pixel path only for grids too coarse for the range sampling; SAR_PATH_GRID /
     * SAR_PATH_POINTS force one. */
    int path;
} sar_geometry;

#define SAR_PATH_AUTO 0
#define SAR_PATH_GRID 1
#define SAR_PATH_POINTS 2

typedef struct sar_plan_info {
    size_t working_length;      /* M = (size_t)(upsample_ratio * N), sarsolver_cxx.cpp:223 */
    long profile_first_bin;     /* first stored range bin (may be negative) */
    size_t profile_length;      /* stored bins per pulse */
    size_t tile_window;         /* staged bins per (tile, pulse); 0 on the unstructured path */
    size_t strip_window;        /* forward strip window (bins); 0 on the unstructured path */
    size_t device_bytes;        /* device memory held by the plan */
    int grid;                   /* 1 regular-grid path, 0 unstructured path */
    int interp;                 /* SAR_INTERP_* of the plan */
    size_t num_fast_times, num_slow_times, num_scatterers;   /* N, S, P */
    int device;                 /* CUDA device of the plan */
    int fft_callbacks;          /* 1: range-profile FFTs run with cuFFT load/store callbacks */
    int gather_lanes_y;         /* 1: the grid backprojection runs warp lanes along y (bins change
                                   more slowly along y than along x), 0: along x */
    int fused_upsampling;       /* 1: the backprojection's range profiles come from the fused
                                   upsampling kernel (N = 512 ... 8192, M a multiple of N), 0: cuFFT */
    int fused_downsampling;     /* 1: the forward projection's FFT side is the fused downsampling
                                   kernel (N = 512 ... 8192, M a multiple of N), 0: cuFFT */
    int scatter_lanes_y;        /* 1: the grid forward scatter runs warp lanes along y and walks the
                                   tile along x (bins change more slowly along x), 0: lanes along x */
    size_t block_pulses;        /* streamed plan: pulses per block (0: resident plan) */
    int scatter_shear;          /* m = +-1: the grid forward scatter walks the rows of a sheared
                                   lattice (steps ex, ey + m ex) that follow the iso-range lines,
                                   for linear sampling of collections looking along a grid diagonal;
                                   0: the plain tile layout */
    int gather_shear;           /* m = +-1 or +-2: the grid backprojection runs on a sheared lattice
                                   with warp lanes along ey + m ex (linear sampling of collections
                                   looking near a diagonal or at ~63 / ~117 degrees to x, where the
                                   plain lanes' bins change fast); 0: the plain tile layout */
    int scatter_ring_half;      /* > 0: the grid forward scatter keeps ring windows of strip_window
                                   slots per pulse holding a tile's bins within this many of its base
                                   (split bins with tiles too wide for strip windows, e.g. upsample 128) */
} sar_plan_info;

/* Create a plan on `device` (-1: the current device).  Copies all host inputs. */
int sar_plan_create(const sar_geometry *geom, int device, sar_plan **plan_out);

/* A plan whose device memory is bounded by a block of pulses instead of the whole aperture:
 * its range-profile buffer holds two blocks of block_pulses pulses ([2][block][profile_length]
 * pairs; a resident plan holds [S][profile_length]) and its FFT rows at most one block.  sar_adjoint
 * and sar_forward then run block by block (upsample a block into a ring slot, gather it onto the
 * image; clear a block's accumulator, scatter, downsample), and sar_adjoint_pulse_block takes blocks
 * of at most block_pulses pulses -- so a phase history streamed from the host in blocks never needs
 * device memory for all S pulses.  Replaces the reference's slow-time blocking, whose purpose is
 * bounding memory (num_calculation_blocks, cxx_binding/forward.py:66-96, adjoint.py:66-94).
 * Regular-grid plans only.  block_pulses >= S gives a resident plan. */
int sar_plan_create_streamed(const sar_geometry *geom, int device, size_t block_pulses, sar_plan **plan_out);
int sar_plan_destroy(sar_plan *plan);
int sar_plan_get_info(const sar_plan *plan, sar_plan_info *info);

/* y[S][N] = A x[P].  Device complex64 buffers; asynchronous on `stream`. */
int sar_forward(sar_plan *plan, const void *x_dev, void *y_dev, void *stream);
/* x[P] = A^H y[S][N].  Device complex64 buffers; asynchronous on `stream`. */
int sar_adjoint(sar_plan *plan, const void *y_dev, void *x_dev, void *stream);
/* Backprojection of one block of pulses, for streaming a phase history through the device:
 * y_block_dev holds rows first_pulse .. first_pulse + count - 1 (complex64 [count][N], fftshifted
 * like y); x_dev = (accumulate ? x_dev : 0) + contribution of those pulses.  Summing the blocks of a
 * partition of [0, S) in order reproduces sar_adjoint (up to FP32 summation order); accumulating
 * calls run one CTA per image tile, so a given partition gives the same bits on every run.
 * Regular-grid plans only (count <= block_pulses for a streamed plan).  Replaces the reference's slow-time blocking (num_calculation_blocks,
 * cxx_binding/adjoint.py:66-94) with device-side accumulation. */
int sar_adjoint_pulse_block(sar_plan *plan, const void *y_block_dev, size_t first_pulse, size_t count,
                            void *x_dev, int accumulate, void *stream);
/* Upsampled range profiles over the stored span, prof[S][profile_length] complex64,
 * bin profile_first_bin + w at column w, no slow-time weight (test and inspection aid). */
int sar_profiles(sar_plan *plan, const void *y_dev, void *prof_dev, void *stream);

/* Replace the slow-time weighting (e.g. autofocus phase corrections). */
int sar_set_slow_time_weighting(sar_plan *plan, const double *w_host /* [S][2] */);
int sar_set_slow_time_weighting_device(sar_plan *plan, const void *w_dev /* complex64 [S] */,
                                       void *stream);

/* Per-pulse phase-error gradient (autofocus).  g[s] = scale * Im( sum_f conj(ag[s][f]) y[s][f] ),
 * ag and y complex64 [S][N] on the device, g float32 [S].  With ag = A_phi G, G = |I|^2 I,
 * I = A_phi^H y and scale = 4 this is d(sum|I|^4)/d phi_s for slow-time weights exp(i phi_s).
 * New (no counterpart in the reference, which exposes only slow_time_weighting,
 * sarsolver_cxx.cpp:288, :349). */
int sar_phase_gradient(const void *ag_dev, const void *y_dev, void *g_dev, size_t num_slow_times,
                       size_t num_fast_times, float scale, void *stream);

/* Image sharpness sum |I|^4 (FP64, written to *sum_dev on the device) and, when g_dev is not
 * NULL, G = |I|^2 I, complex64 [P] -- the image-side factor of the autofocus gradient above.
 * Buffers 16-byte aligned.  New (no counterpart in the reference). */
int sar_sharpness(const void *img_dev, void *g_dev, double *sum_dev, size_t num_pixels, void *stream);

/* CGLS on the normal equations A^H A x = A^H y with the plan's operator pair (replaces the CIL
 * CGLS the reference runs on its operator, tests/test_cil.py:18-22).  x_dev holds the start on
 * entry (ignored and zeroed when zero_start != 0) and the solution on return.  Stops when the
 * normal-equations residual ||A^H (y - A x)|| / ||A^H y|| <= tolerance or after max_iterations.
 * history (host, may be NULL) receives that residual before each iteration and after the last
 * ([max_iterations + 1]).  Each iteration is one sar_forward and one sar_adjoint plus fused vector
 * updates; the host waits on `stream` once per iteration to test the residual.  Work vectors
 * (2 x S*N + 2 x P complex64) are taken from the stream-ordered allocator for the call.  Exact
 * convergence theory needs SAR_INTERP_LINEAR (an exact adjoint pair).  Non-finite data returns
 * SAR_ERR_INVALID_ARGUMENT; ||A p|| = 0 before convergence sets result->breakdown. */
typedef struct sar_cgls_result {
    int iterations;   /* iterations run */
    int converged;    /* residual <= tolerance reached */
    int breakdown;    /* stopped on ||A p|| = 0 */
    double residual;  /* final ||A^H (y - A x)|| / ||A^H y|| */
    double norm_ahy;  /* ||A^H y|| */
} sar_cgls_result;

int sar_cgls(sar_plan *plan, const void *y_dev, void *x_dev, int zero_start, int max_iterations,
             double tolerance, double *history, sar_cgls_result *result, void *stream);

/* As sar_cgls with a choice of start and an optional precomputed A^H y (complex64 [P] on the
 * device; NULL: computed here).  SAR_CGLS_START_SCALED takes x_dev as a direction z and starts
 * from x0 = c z with c = Re<z, A^H y> / ||A z||^2 (the best multiple of z), which costs one
 * forward projection -- the same as a given start. */
#define SAR_CGLS_START_GIVEN 0
#define SAR_CGLS_START_ZERO 1
#define SAR_CGLS_START_SCALED 2
int sar_cgls_ex(sar_plan *plan, const void *y_dev, void *x_dev, int start, const void *ahy_dev,
                int max_iterations, double tolerance, double *history, sar_cgls_result *result, void *stream);

/* PDHG (Chambolle-Pock) with the plan's operator pair: min_x ||A x - b||^2 + l1_weight ||x||_1
 * (l1_weight = 0: no regulariser) -- replaces the CIL PDHG with f = L2NormSquared(b),
 * g = ZeroFunction that the reference runs on its operator (tests/test_cil.py:25-37).  CIL's
 * iteration order, from xbar = x0 and y = 0:
 *   y = (y + sigma (A xbar - b)) / (1 + sigma / 2);  x' = prox_{tau g}(x - tau A^H y);
 *   xbar = x' + theta (x' - x);  x = x'
 * (prox of the L1 term: soft threshold of the complex modulus at tau l1_weight).  x_dev holds x0 on
 * entry (zeroed when zero_start != 0) and the iterate after `iterations` iterations on return.
 * sigma, tau: step sizes; 0 means "from ||A||", estimated with norm_iterations power iterations
 * (each one forward and one backprojection; result->operator_norm): both 0 -> sigma = tau =
 * 1 / ||A||, one 0 -> the other from sigma tau ||A||^2 = 1.  residual_history (host, may be NULL)
 * receives ||A xbar_k - b|| for k = 0 .. iterations - 1 (xbar_0 = x0).  The loop issues work
 * without reading back; the host waits once at the end.  Work vectors (2 x S*N + 2 x P complex64)
 * come from the stream-ordered allocator.  Non-finite values return SAR_ERR_INVALID_ARGUMENT. */
typedef struct sar_pdhg_result {
    int iterations;        /* iterations run */
    double sigma, tau;     /* step sizes used */
    double theta;          /* relaxation used */
    double operator_norm;  /* power-method estimate of ||A|| (0 when sigma and tau were both given) */
} sar_pdhg_result;

int sar_pdhg(sar_plan *plan, const void *b_dev, void *x_dev, int zero_start, int iterations, double sigma,
             double tau, double theta, double l1_weight, int norm_iterations, double *residual_history,
             sar_pdhg_result *result, void *stream);

/* ------------------------------------------------ 3. learned warm start (U-Net)
 *
 * New (no counterpart in the reference): the network that maps a backprojected image A^H y to a
 * CGLS warm start.  4-level U-Net in bf16 with FP32 accumulation on the tensor cores (layer list
 * in sar_unet_layer order: enc0 a/b, enc1 a/b, enc2 a/b, bottleneck a/b, dec2 a/b, dec1 a/b,
 * dec0 a/b, 1x1 output).  Images are complex64 [batch][height][width] (channels re, im);
 * width / 8 must be a power of two >= 16 and height a multiple of 8 * 128 / min(width / 8, 128).
 * Parameters are one flat FP32 vector: for each layer its filter [cout][taps][cin0 + cin1]
 * (tap = 3 * (dy + 1) + (dx + 1)) followed by its bias [cout]. */
#define SAR_UNET_LAYERS 15
typedef struct sar_unet sar_unet;
typedef struct sar_unet_layer {
    size_t weight_offset, bias_offset;   /* into the flat parameter vector */
    int cin0, cin1, cout, taps, relu, level;
} sar_unet_layer;

int sar_unet_create(int base_channels /* 32 or 64 */, int device, sar_unet **net_out);
int sar_unet_destroy(sar_unet *net);
int sar_unet_info(const sar_unet *net, size_t *num_params, sar_unet_layer *layers /* [SAR_UNET_LAYERS] or NULL */);
/* Copy parameters in (resets the Adam moments) / out, gradients out; device FP32 buffers. */
int sar_unet_set_params(sar_unet *net, const float *params_dev, void *stream);
int sar_unet_get_params(const sar_unet *net, float *params_dev, void *stream);
int sar_unet_get_grads(const sar_unet *net, float *grads_dev, void *stream);
int sar_unet_zero_grad(sar_unet *net, void *stream);
/* out = U(in_scale * in); keeps the activations for sar_unet_backward. */
int sar_unet_forward(sar_unet *net, const void *in_dev, float in_scale, int batch, int height, int width,
                     void *out_dev, void *stream);
/* Adds d(loss)/d(parameters) for grad_out = d(loss)/d(out) (complex64, PyTorch's conjugate
 * convention, i.e. d/d(re) + i d/d(im)) of the last forward call. */
int sar_unet_backward(sar_unet *net, const void *grad_out_dev, void *stream);
int sar_unet_adam_step(sar_unet *net, float lr, float beta1, float beta2, float eps, int step, void *stream);
/* Synchronise the device, return and clear the kernels' check flags (SAR_FLAG_WAIT_TIMEOUT). */
int sar_unet_flags(sar_unet *net, unsigned *flags);

/* Building blocks (the network's own kernels): bf16 NHWC convolution over the channel
 * concatenation of x0 [c0] and x1 [c1] (x1 may be NULL), filter w [cout][taps][c0 + c1] bf16,
 * taps 9 (3x3, zero padding 1) or 1; y bf16 NHWC [cout] with optional FP32 bias and ReLU.  The
 * weight gradient adds sum_pixels dz[p][co] * x[p + tap][ci] into dw (FP32, same layout as w).
 * Channel counts multiples of 32; flags_dev a device word receiving SAR_FLAG_WAIT_TIMEOUT. */
int sar_conv2d_forward_bf16(const void *x0, int c0, const void *x1, int c1, int batch, int height, int width,
                            int taps, const void *w, const float *bias, int cout, int relu, void *y,
                            unsigned *flags_dev, void *stream);
int sar_conv2d_wgrad_bf16(const void *x0, int c0, const void *x1, int c1, const void *dz, int cout, int batch,
                          int height, int width, int taps, float *dw, unsigned *flags_dev, void *stream);

/* ------------------------------------------------ 4. dataset resampling (before the operator)
 * Device phase histories complex64 [S][N], fast time fftshifted; small parameters on the host.
 *
 * sar_move_srps: out = ph * exp(i kb_f dR_s) * exp(-2 pi i sign fc dR_s / c), kb_f = 2 pi bb_f / c,
 *   bb_f = (f - N/2) fs / N, dR_s = change of the pulse's bistatic SRP range (host FP64 [S]).
 *   Replaces utils.move_srps (src/sarsolver/utils/geodesy.py:33-73).
 * sar_fast_freq_downsample: out [S][new_N] = fftshift(FFT(window * crop(IFFT(ifftshift(ph))))),
 *   window = the fftshifted Tukey window (host [new_N]).  Replaces utils.fast_freq_downsample
 *   (src/sarsolver/utils/signal.py:45-77).
 * sar_resample_phase_history: both of the above on every pulse (delta_range may be NULL: no SRP
 *   move), then out[t][f] = sum_k kernel[k] X[row0[t] + k][f] (kernel host complex [L][2], row0
 *   host [T]).  The phase-history part of NumpySimpleSarDataset.from_resampling
 *   (src/sarsolver/numpy/measurement.py:342-458). */
int sar_move_srps(const void *ph_dev, void *out_dev, size_t S, size_t N, const double *delta_range,
                  double centre_freq, double sample_bandwidth, double sign_multiplier, double c_eff, void *stream);
int sar_fast_freq_downsample(const void *ph_dev, void *out_dev, size_t S, size_t N, size_t new_N,
                             const double *window, void *stream);
int sar_resample_phase_history(const void *ph_dev, size_t S, size_t N, const double *delta_range,
                               double centre_freq, double sample_bandwidth, double sign_multiplier, double c_eff,
                               size_t new_N, const double *window, const double *kernel, size_t kernel_length,
                               const int *row0, size_t num_rows, void *out_dev, void *stream);

/* ------------------------------------------------ 5. CPHD signal arrays (before the operator)
 * sar_cphd_decode: widen one CPHD signal array, copied to the device as it lies in the file
 * (big-endian interleaved I/Q, [num_vectors][num_samples]), to complex64:
 *   out[v][s] = complex(I, Q) * amp_sf[v]     (amp_sf_dev: device float [num_vectors], or NULL)
 * format: SAR_CPHD_CI2 (signed 8-bit pairs), SAR_CPHD_CI4 (signed 16-bit pairs), SAR_CPHD_CF8
 * (binary32 pairs) -- CPHD 1.0.1 Data/SignalArrayFormat, CPHD 0.3 Data/SampleType.  Asynchronous
 * on `stream`; any alignment (16-byte aligned buffers take the vector path).  Replaces the signal
 * read of the reference's CPHD datasets through sarpy (src/sarsolver/io/cphd101.py:251-265,
 * io/cphd03.py:250-263), which decodes on the host. */
#define SAR_CPHD_CI2 1
#define SAR_CPHD_CI4 2
#define SAR_CPHD_CF8 3
int sar_cphd_decode(const void *raw_dev, int format, size_t num_vectors, size_t num_samples,
                    const float *amp_sf_dev, void *out_dev, void *stream);

/* Stage timing.  While enabled, every sar_forward / sar_adjoint call records CUDA events on
 * its stream around its stages: [0] range-profile FFT side before the main kernel (adjoint:
 * pack + inverse FFT + unpack; forward: accumulator clear), [1] the main gather / scatter
 * kernel, [2] FFT side after it (forward: pack + FFT + extract).  sar_stage_times synchronises
 * and returns the summed milliseconds per stage over the calls recorded since the last reset
 * (at most 4096 calls are kept) and their count; enabling resets the record. */
int sar_enable_stage_timing(sar_plan *plan, int enable);
int sar_stage_times(sar_plan *plan, float *ms /* [3] */, int *calls);

/* Synchronise the plan's last stream, return and clear the device check flags. */
int sar_device_flags(sar_plan *plan, unsigned *flags);

/* Wait budget of the backprojection gather's in-kernel waits between its warp roles, in SM clock
 * cycles (0 = the default, about 2 s at 2 GHz).  When a wait runs out the kernel stops that tile,
 * raises SAR_FLAG_WAIT_TIMEOUT and returns, and the plan stays usable.  hold_first_stage != 0 is a
 * test aid: the gather's producer warps never publish the first pulse stage, so its consumers'
 * first wait can only run out -- a way to check that an expired wait is reported without faulting
 * or hanging the GPU.  New (no counterpart in the reference, which has no device code). */
int sar_plan_set_wait_budget(sar_plan *plan, long long cycles, int hold_first_stage);

/* Backprojection x = A^H y from upsampled range profiles, without allocating device memory.
 * No counterpart in the reference (its kernel allocates host buffers per call and has no GPU).
 *
 * For callers that cannot call cudaMalloc while they run: code running inside another
 * runtime's memory pool or arena, real-time loops that must not allocate after start-up, and
 * hosts whose device allocator belongs to another framework.  Everything else above allocates
 * (plans hold FFT rows and profile buffers; cuFFT plans allocate work areas); this call does not.
 *
 * Inputs: the geometry on the host (a regular grid is required), the upsampled profiles on the
 * device as complex64 [S][span], column w holding range bin first_bin + w -- exactly what
 * sar_profiles() writes for a plan of the same geometry (profile_first_bin, profile_length).
 * Output: x_dev, complex64 [P].  Asynchronous on `stream`.
 *
 * Scratch lives in one fixed 32 MiB device array inside the library (every GPU that loads the
 * library holds it until exit): pulses x span x 16 bytes of profile pairs plus about 88 bytes per
 * pulse of tables (64 pulse geometry, 8 weight, 16 antenna norms, each table rounded up to 256
 * bytes) and 512 bytes of flags and grid steps must fit, otherwise SAR_ERR_INVALID_ARGUMENT with a
 * message (sar_last_error).  The array is shared by all calls and keeps the last call's contents;
 * calls that overlap on the GPU race on it, so order them on one stream.  The first call on each
 * device resolves the array's device address (cudaGetSymbolAddress, with that device current);
 * make it before any stream capture.  Each call clears the device check flags in the array at its
 * start; read them with sar_noalloc_flags. */
int sar_adjoint_from_profiles_noalloc(const sar_geometry *geom, const void *prof_dev, long first_bin,
                                      size_t span, void *x_dev, void *stream);

/* Device check flags (SAR_FLAG_*) of the last sar_adjoint_from_profiles_noalloc call on the
 * current device: waits for `stream` (the stream that call ran on), copies the flag word into
 * *flags and clears it.  Allocates nothing.  A non-zero SAR_FLAG_WAIT_TIMEOUT means that call's
 * image is invalid. */
int sar_noalloc_flags(unsigned *flags, void *stream);

/* Device address of page-locked, mapped host memory (cudaHostGetDevicePointer), for passing a
 * pinned host buffer to a call that reads it on the device -- e.g. the phase history of
 * sar_adjoint when the plan uses the fused upsampling (sar_plan_info.fused_upsampling), which
 * then reads y over the host link inside its transform instead of after a copy.  Such a buffer
 * must stay unchanged until the stream has passed the call.  SAR_ERR_INVALID_ARGUMENT when the
 * device cannot address the memory (on systems whose GPU translates host page tables, e.g. over a
 * chip-to-chip link, pageable memory is addressable too and comes back at its host address). */
int sar_host_device_pointer(const void *host_ptr, void **dev_ptr);

/* Throughput of the arithmetic pipes the backprojection gather uses, measured on the current
 * device: operations per clock per SM (median SM; every thread of a full wave of CTAs runs
 * independent chains of one operation, timed with the SM's own cycle counter), for
 *   sfu_sincos_per_clk_sm  special-function sine and cosine (__sincosf: two operations each call)
 *   frnd_per_clk_sm        FP32 round to integer (rintf)
 *   ffma_per_clk_sm        FP32 fused multiply-add
 *   ffma2_per_clk_sm       FP32 fused multiply-adds issued as pairs (two per instruction)
 * and the SM clock that held meanwhile (cycles over event time, a lower bound).  The roofline of
 * the gather is SMs x clock x min(FP32 lanes / FP32 ops, SFU rate / SFU ops) per pixel·pulse.
 * A measurement aid with no counterpart in the reference; allocates a few bytes. */
typedef struct sar_pipe_rates {
    double sfu_sincos_per_clk_sm, frnd_per_clk_sm, ffma_per_clk_sm, ffma2_per_clk_sm;
    int num_sms;
    double sm_mhz;
} sar_pipe_rates;
int sar_measure_pipe_rates(sar_pipe_rates *out, void *stream);

/* Last error message of the calling thread (empty if none); returns its full length. */
size_t sar_last_error(char *buf, size_t len);
const char *sar_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* SARGPU_H */
