// sar_kernels.cuh -- launch interface of the SAR kernels (sar_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "sar_geom.cuh"

namespace sar {

// Device check flags (OR-ed into a plan-owned word; read back by sar_device_flags()).
enum : unsigned {
    FLAG_TILE_WINDOW = 1u,    // a tile's staged window left the stored profile span
    FLAG_STRIP_WINDOW = 2u,   // a forward strip window left the stored profile span, or a tile's bins
                              // left its ring window's range
    FLAG_BIN_CLAMP = 4u,      // a per-pixel bin index was clamped (debug builds only)
    FLAG_WAIT_TIMEOUT = 8u,   // a bounded mbarrier wait gave up (the result is invalid)
    FLAG_GATHER_WINDOW = 16u, // a sub-tile's bin extent exceeded its tile's staged window
};

// Clock budget of a bounded in-kernel wait (about 2 s at 2 GHz) unless a launch sets its own.
constexpr long long kDefaultWaitBudgetCycles = 4000000000ll;

// Stored profile formats (the `linear` argument of the upsampling writers): nearest-bin pairs
// (value, 0) and linear pairs (value at mid-bin, difference), float4 rows; or plain values, float2
// rows of even length, which nearest-bin plans with wide staged windows use (half the bytes).
constexpr int kProfNearestPairs = 0, kProfLinearPairs = 1, kProfValues = 2;

constexpr int kTile = 32;          // pixels per tile side
constexpr int kThreads = 256;      // threads per tile CTA: 32 columns x 8 warps, 4 rows each
constexpr int kMaxStagePulses = 32;
constexpr int kSetF4 = 6;          // float4 per (pulse, sub-tile) coefficient set

// Backprojection over a regular grid (K2).
struct BpGridArgs {
    GridConst g;
    const PulseGeom* pulses;   // [S]
    const float4* pairs;       // [S][Lg]: (value at mid-bin, difference) per bin; with `values`, the
                               //    plain values as float2 rows of even length Lg
    float2* x;                 // [P] image, (k*ny + j)*nx + i
    unsigned* flags;
    int S, Lg, bg0;            // stored profile span: bins [bg0, bg0 + Lg)
    int wwin;                  // staged window per (tile, pulse), multiple of 4
    int pb;                    // pulses per stage: a power of two from 2 to 32 (odd last stages are
                               //    padded with a zero pulse by the paired kernel)
    int staged;                // 1: stage windows in shared memory; 0: read global directly
    int accumulate;            // 1: x += result
    int lanes_y;               // 1: lanes of a warp run along y (chosen when bins change more slowly
                               //    along y than along x: fewer shared-memory bank conflicts)
    int values = 0;            // 1 (with nearest): the profiles are plain values (kProfValues)
    int nearest;               // 1: nearest-bin pairs; bins near a rounding boundary are decided again
                               //    with the per-pixel double-float range (needs steps, alpha2)
    const double* steps;       // [9] grid steps ex, ey, ez (FP64), for those exact decisions
    const float4* alpha2;      // [S] |tx-o|^2, |rx-o|^2 as (hi, lo) pairs, the same
    int parts;                 // set by the staged launcher: CTAs per tile, each over a share of the
                               //    pulse stages, adding into the image with atomics when > 1
    long long wait_budget = kDefaultWaitBudgetCycles;   // clock cycles a staged-kernel wait on the
                               //    other warp role may take before it gives up (FLAG_WAIT_TIMEOUT)
    int hold_first_stage = 0;  // test aid: the producers never publish the first pulse stage, so the
                               //    consumers' first wait can only run out (nothing is copied for it)
    long tiles_valid = 0;      // tiles holding image pixels (a sheared lattice's); 0: all tiles
};
size_t bp_grid_smem_bytes(int wwin, int pb, int staged);
cudaError_t launch_bp_grid(const BpGridArgs& a, cudaStream_t st);
// Warp-specialised variant: one producer warp computes coefficients and stages windows with
// bulk copies into a double buffer while eight consumer warps gather (pb <= 32).
size_t bp_grid_ws_smem_bytes(int wwin, int pb, int values);
cudaError_t launch_bp_grid_ws(const BpGridArgs& a, cudaStream_t st);

// Forward projection over a regular grid (K3): scatter into strip windows, merge globally.
struct FpGridArgs {
    GridConst g;
    const PulseGeom* pulses;   // [S]
    const float2* x;           // [P]
    float2* acc;               // [S][Lg] profile accumulator (pre-zeroed)
    const int* strip_start;    // first bin of each strip window: strip_start[strip * strip_stride + s]
    int strip_stride;          // pulses per strip row of that table (the plan's S; S is a block's count)
    unsigned* flags;
    int S, Lg, bg0;
    int seg_tiles;             // tiles per strip segment (along y; along x when transposed)
    int segs_per_column;       // segments per strip line: ceil(tiles along it / seg_tiles)
    int ws;                    // strip window length (bins), multiple of 32
    int pbf;                   // pulses per CTA (multiple of 8, <= 32)
    int linear;                // 1: linear interpolation weights; 0: nearest bin
    int transposed;            // 1: lanes along y, rows walked along x (bins change slowly along x)
    const double* steps;       // nearest bins: FP64 grid steps and antenna norms for the exact
    const float4* alpha2;      //   decisions near rounding boundaries (as BpGridArgs)
    int ring_half = 0;         // > 0 (split bins only): ring windows -- ws is a power of two, slot of
                               //    absolute bin b is b mod ws, and a tile touches bins within
                               //    ring_half of its base bin; 0: strip windows from strip_start
};
// Warp-specialised variant: producer warps stage image tiles and coefficient sets; each
// gathering warp owns whole pulses, so its windows need no atomics when bins along a row of
// the tile are provably distinct (pbf <= 32, multiple of 8).
size_t fp_grid_ws_smem_bytes(int ws, int pbf, int wide_x);   // wide_x: linear, not precise bins
cudaError_t launch_fp_grid_ws(const FpGridArgs& a, cudaStream_t st);

// Unstructured positions (K2/K3 point variants).
struct PointArgs {
    const PulseGeom* pulses;   // [S]
    const float4* alpha2;      // [S]: |tx-o|^2 (hi, lo), |rx-o|^2 (hi, lo)
    const PointGeom* points;   // [P]
    df kappa, s_r;
    int bin_rule;              // BinRule (sar_geom.cuh)
    int S, P, Lg, bg0;
    int linear;                // forward scatter weights: 1 linear, 0 nearest bin
    unsigned* flags;
    int values = 0;            // 1: the backprojection's profiles are plain values (kProfValues)
};
cudaError_t launch_bp_points(const PointArgs& a, const float4* pairs, float2* x, int accumulate,
                             cudaStream_t st);
cudaError_t launch_fp_points(const PointArgs& a, const float2* x, float2* acc, cudaStream_t st);

// FFT-side kernels (K1 / K4).  y is [S][N] fftshifted along fast time; spec is [rows][M] of
// complex64, or complex128 when dbl != 0.
cudaError_t launch_pack_adjoint(const float2* y, const float2* wave, void* spec, int dbl, int N, long M, int rows,
                                int first, cudaStream_t st);
cudaError_t launch_unpack_compact(const float2* compact, int Lc, const float2* wfac, float4* pairs, float2* prof,
                                  long M, int Lg, int rows, int first, int linear, cudaStream_t st);
// Fused adjoint upsampling for N = 512, 1024, 2048, 4096 or 8192 and M a multiple of N: pairs over the stored span straight
// from the fftshifted phase history (replaces pack + inverse FFT + unpack_pairs); twiddle tables
// tw_n[q] = e^{2 pi i q / N}, tw_m[q] = e^{2 pi i q / M} for q < M, followed by 2 (M / N) x 16 entries
// tw_m[M + 16 r + e] = e^{2 pi i (e N / 16 - N [e >= 8]) r / M}.
bool upsample_fused_supported(int N, long M, int Lg);
size_t upsample_fused_smem_bytes(int N, int Lg, int U);
cudaError_t launch_upsample_pairs_fused(const float2* y, const float2* wave, const float2* wfac, const float2* tw_n,
                                        const float2* tw_m, float4* pairs, int N, long M, int Lg, long bg0, int rows,
                                        int first, int linear, cudaStream_t st);
// Fused forward downsampling for N = 512 ... 8192, M a multiple of N and Lg <= M: y straight from the
// bin accumulator acc [S][Lg] (replaces pack_forward + forward FFT + extract_forward).
bool downsample_fused_supported(int N, long M, int Lg);
cudaError_t launch_downsample_forward_fused(const float2* acc, const float2* wave, const float2* wfac,
                                            const float2* tw_n, const float2* tw_m, float2* y, int N, long M, int Lg,
                                            long bg0, int rows, int first, cudaStream_t st);
cudaError_t launch_unpack_pairs(const void* spec, int dbl, const float2* wfac, float4* pairs, long M, int Lg,
                                long bg0, int rows, int first, int linear, cudaStream_t st);
cudaError_t launch_unpack_profiles(const void* spec, int dbl, float2* prof, long M, int Lg, long bg0, int rows,
                                   int first, cudaStream_t st);
cudaError_t launch_pack_forward(const float2* acc, void* spec, int dbl, long M, int Lg, long bg0, int rows, int first,
                                cudaStream_t st);
cudaError_t launch_extract_forward(const void* spec, int dbl, const float2* wave, const float2* wfac, float2* y,
                                   int N, long M, int rows, int first, cudaStream_t st);
cudaError_t launch_phase_grad(const float2* ag, const float2* y, float* g, int S, int N, float scale,
                              cudaStream_t st);
cudaError_t launch_sharpness(const float2* img, float2* G, double* sum, size_t P, int num_sms, cudaStream_t st);
cudaError_t launch_weights(const float2* w, float2* wadj, float2* wfwd, int S, int conj_adjoint,
                           cudaStream_t st);

// Sets the calling thread's sar_last_error() text (library-internal, not exported).
__attribute__((visibility("hidden"))) void sar_internal_set_error(const char* msg);

}  // namespace sar
