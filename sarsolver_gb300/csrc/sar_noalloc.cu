// sar_noalloc.cu -- backprojection from caller-supplied range profiles without any device
// allocation (sar_adjoint_from_profiles_noalloc, include/sargpu.h).
//
// Who needs it: callers that may not allocate device memory while they run -- code executed
// inside another runtime's memory pool or arena that forbids cudaMalloc, real-time loops that
// must not allocate after start-up, and hosts whose allocator is owned by a different
// framework.  They pass their inputs (geometry on the host, upsampled range profiles on the
// device) and the output image; everything else this call needs lives in one fixed array.
//
// Scratch: `g_noalloc_scratch`, a file-scope __device__ array of kScratchBytes (32 MiB).  Every
// GPU that loads the library holds it until the process exits.  Layout per call:
//   [0, 256)            device check flags (cleared by every call, read by sar_noalloc_flags)
//   pulse table         S x 64 bytes (PulseGeom, double-float antenna positions)
//   pulse factors       S x 8 bytes (slow-time weight, conjugated for linear interpolation)
//   grid steps          9 doubles, and antenna norms S x 16 bytes (nearest-bin decisions near a
//                       rounding boundary are taken again exactly from these)
//   profile pairs       S x span x 16 bytes (value at mid-bin, difference), fully rewritten; for
//                       nearest-bin sampling with staged windows wider than 256 bins, as a plan
//                       stores them, S x span' x 8 bytes of plain values (span' = span rounded
//                       up to even, so that the staged copies stay 16-byte aligned)
// Sizes beyond the array are rejected with SAR_ERR_INVALID_ARGUMENT and a message.
//
// All calls share the one array and it keeps the previous call's contents: calls that overlap
// on the GPU (different streams, or different host threads without ordering) race on it.
//
// Host code may not use the array's name as a device address; the first call on each device
// resolves the address with cudaGetSymbolAddress (with that device current) and caches it.
// That first call should therefore be made before any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/sargpu.h"
#include "sar_host_prep.h"
#include "sar_kernels.cuh"

using namespace sar;

namespace {

constexpr size_t kScratchBytes = (size_t)32 << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

int noalloc_fail(int code, const char* msg) {
    sar_internal_set_error(msg);   // reported by sar_last_error()
    return code;
}

size_t round256(size_t n) { return (n + 255) & ~(size_t)255; }

// Device address of the scratch array on the current device (resolved once per device).
int scratch_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(SAR_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(SAR_ERR_NOT_SUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return noalloc_fail(SAR_ERR_CUDA, "cudaGetSymbolAddress failed for the scratch array");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return SAR_OK;
}

}  // namespace

extern "C" int sar_adjoint_from_profiles_noalloc(const sar_geometry* g, const void* prof_dev, long first_bin,
                                                 size_t span, void* x_dev, void* stream) {
    sar_internal_set_error("");
    if (!g || !prof_dev || !x_dev) return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    const size_t N = g->num_fast_times, S = g->num_slow_times, P = g->num_scatterers;
    if (!N || !S || !P || !span) return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "empty problem");
    if (!g->transmit_posns || !g->receive_posns || !g->stab_ref_posns)
        return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "antenna / SRP positions are required");
    if (!(g->grid_shape[0] && g->grid_shape[1] && g->grid_shape[2]) ||
        g->grid_shape[0] * g->grid_shape[1] * g->grid_shape[2] != P)
        return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "a regular grid with grid_shape product == num_scatterers is required");
    if (g->grid_shape[1] > (1u << 20) || g->grid_shape[2] > (1u << 20) || g->grid_shape[0] > (1u << 16))
        return noalloc_fail(SAR_ERR_NOT_SUPPORTED, "grid dimension too large");
    if (!(g->c_eff > 0.0) || !(g->sample_frequency > 0.0) || !(g->upsample_ratio > 0.0))
        return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "c_eff, sample_frequency and upsample_ratio must be positive");
    if (g->interp != SAR_INTERP_NEAREST_REF && g->interp != SAR_INTERP_LINEAR)
        return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "unknown interpolation mode");
    if (span > (size_t)1 << 30 || S > (size_t)1 << 30)
        return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "span or pulse count too large");

    // Scratch sizes: reject what does not fit the fixed array.
    const size_t off_table = 256;
    const size_t off_w = off_table + round256(S * sizeof(PulseGeom));
    const size_t off_steps = off_w + round256(S * sizeof(float2));
    const size_t off_a2 = off_steps + 256;
    const size_t off_pairs = off_a2 + round256(S * sizeof(float4));
    const size_t need = off_pairs + S * span * sizeof(float4);
    if (need > kScratchBytes) {
        char m[200];
        snprintf(m, sizeof m, "needs %zu bytes of scratch (pulses x span x 16 + tables); the fixed array holds %zu",
                 need, kScratchBytes);
        return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, m);
    }

    // Host preparation: the same geometry constants as a plan (sar_geom.cuh, sar_host_prep.h).
    const size_t M = (size_t)(g->upsample_ratio * (double)N);
    if (M < N) return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "upsample_ratio*N is below N");
    const double s_r = g->sample_frequency * (double)M / ((double)N * g->c_eff);
    const double kappa = g->sign_multiplier * g->centre_frequency / g->c_eff;
    const int nz = (int)g->grid_shape[0], ny = (int)g->grid_shape[1], nx = (int)g->grid_shape[2];
    const bool linear = g->interp == SAR_INTERP_LINEAR;
    GridConst gc = make_grid_const(g->grid_step_x, g->grid_step_y, g->grid_step_z, kappa, s_r, linear ? -0.5f : 0.5f,
                                   nx, ny, nz);
    const double nex = std::sqrt(g->grid_step_x[0] * g->grid_step_x[0] + g->grid_step_x[1] * g->grid_step_x[1] +
                                 g->grid_step_x[2] * g->grid_step_x[2]);
    const double ney = std::sqrt(g->grid_step_y[0] * g->grid_step_y[0] + g->grid_step_y[1] * g->grid_step_y[1] +
                                 g->grid_step_y[2] * g->grid_step_y[2]);
    const double h = s_r * 2.0 * 16.0 * (nex + ney);
    if (!(h < 1.0e6)) return noalloc_fail(SAR_ERR_NOT_SUPPORTED, "grid spacing too coarse for the range sampling");
    const int wwin_iso = (2 * ((int)std::ceil(h) + 3) + 3) & ~3;
    // staged window from the look directions, as a plan's (tile_halfspan_directional); the span
    // check below keeps the isotropic margins
    int wwin = wwin_iso;
    {
        const double hd = tile_halfspan_directional(g->transmit_posns, g->receive_posns, S, g->grid_origin,
                                                    g->grid_step_x, g->grid_step_y, g->grid_step_z, 32, gc.tiles_x,
                                                    gc.tiles_y, nz, s_r);
        if (hd >= 0.0) wwin = std::min(wwin, (2 * ((int)std::ceil(hd) + 3) + 3) & ~3);
    }
    gc.precise_bins = (!linear || wwin > 256) ? 1 : 0;
    if (span < (size_t)wwin_iso) return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "span shorter than a tile window");

    std::vector<PulseGeom> table(S);
    std::vector<float2> wfac(S);
    std::vector<float4> a2(S);
    double steps[9];
    for (int c = 0; c < 3; ++c) {
        steps[c] = g->grid_step_x[c];
        steps[3 + c] = g->grid_step_y[c];
        steps[6 + c] = g->grid_step_z[c];
    }
    double vmin = INFINITY, vmax = -INFINITY;
    const int tx_tiles = gc.tiles_x, ty_tiles = gc.tiles_y;
    for (size_t s = 0; s < S; ++s) {
        const double *tx = g->transmit_posns + 3 * s, *rx = g->receive_posns + 3 * s, *srp = g->stab_ref_posns + 3 * s;
        for (int c = 0; c < 3; ++c)
            if (!std::isfinite(tx[c]) || !std::isfinite(rx[c]) || !std::isfinite(srp[c]))
                return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "non-finite antenna or SRP position");
        table[s] = make_pulse_geom(tx, rx, srp, g->grid_origin);
        {
            double at[3], ar[3];
            for (int c = 0; c < 3; ++c) {
                at[c] = tx[c] - g->grid_origin[c];
                ar[c] = rx[c] - g->grid_origin[c];
            }
            const df n1 = to_df(at[0] * at[0] + at[1] * at[1] + at[2] * at[2]);
            const df n2 = to_df(ar[0] * ar[0] + ar[1] * ar[1] + ar[2] * ar[2]);
            a2[s] = make_float4(n1.hi, n1.lo, n2.hi, n2.lo);
        }
        double a0, a1, b0, b1;
        box_distance_bounds(tx, g->grid_origin, g->grid_step_x, g->grid_step_y, g->grid_step_z, tx_tiles * 32 - 1.0,
                            ty_tiles * 32 - 1.0, nz - 1.0, &a0, &a1);
        box_distance_bounds(rx, g->grid_origin, g->grid_step_x, g->grid_step_y, g->grid_step_z, tx_tiles * 32 - 1.0,
                            ty_tiles * 32 - 1.0, nz - 1.0, &b0, &b1);
        const double ref = dist3(tx, srp) + dist3(rx, srp);
        vmin = std::min(vmin, (a0 + b0 - ref) * s_r);
        vmax = std::max(vmax, (a1 + b1 - ref) * s_r);
        std::complex<double> w(1.0, 0.0);
        if (g->slow_time_weighting) w = {g->slow_time_weighting[2 * s], g->slow_time_weighting[2 * s + 1]};
        if (linear) w = std::conj(w);
        wfac[s] = make_float2((float)w.real(), (float)w.imag());
    }
    // The caller's profile span must cover every staged window.
    const double lo_needed = std::floor(vmin) - wwin_iso / 2 - 1;
    const double hi_needed = std::ceil(vmax) + wwin_iso / 2 + 2;
    if ((double)first_bin > lo_needed || (double)first_bin + (double)span < hi_needed)
        return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "the profile span does not cover the scene's range bins");

    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    unsigned char* scratch = static_cast<unsigned char*>(base);
    cudaStream_t st = (cudaStream_t)stream;
    unsigned* flags = reinterpret_cast<unsigned*>(scratch);
    PulseGeom* d_table = reinterpret_cast<PulseGeom*>(scratch + off_table);
    float2* d_w = reinterpret_cast<float2*>(scratch + off_w);
    float4* d_pairs = reinterpret_cast<float4*>(scratch + off_pairs);
    double* d_steps = reinterpret_cast<double*>(scratch + off_steps);
    float4* d_a2 = reinterpret_cast<float4*>(scratch + off_a2);

    const bool values = !linear && wwin > 256;
    const int lg_rows = values ? (int)(span + (span & 1)) : (int)span;
    cudaError_t e = cudaMemsetAsync(flags, 0, sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_table, table.data(), S * sizeof(PulseGeom), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, wfac.data(), S * sizeof(float2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_steps, steps, sizeof steps, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_a2, a2.data(), S * sizeof(float4), cudaMemcpyHostToDevice, st);
    // Pair rows of lg_rows entries (values: an even row length; a padding column when span is odd
    // reads column 0 and lies outside every window, which the span check keeps in
    // [first_bin, first_bin + span)).
    // Pairs over the caller's span: with M = span and first bin 0 the unpack kernel reads column
    // w and w + 1 of each row (the last column's difference wraps; it lies in the margin).
    if (e == cudaSuccess)
        e = launch_unpack_pairs(prof_dev, 0, d_w, d_pairs, (long)span, lg_rows, 0, (int)S, 0,
                                values ? kProfValues : linear ? kProfLinearPairs : kProfNearestPairs, st);
    if (e == cudaSuccess) {
        BpGridArgs a;
        a.g = gc;
        a.pulses = d_table;
        a.pairs = d_pairs;
        a.x = (float2*)x_dev;
        a.flags = flags;
        a.S = (int)S;
        a.Lg = lg_rows;
        a.bg0 = (int)first_bin;
        a.wwin = wwin;
        a.accumulate = 0;
        a.nearest = linear ? 0 : 1;
        a.values = values ? 1 : 0;
        a.steps = d_steps;
        a.alpha2 = d_a2;
        a.lanes_y = choose_lanes_y(g->transmit_posns, g->receive_posns, S, g->grid_origin, g->grid_step_x,
                                   g->grid_step_y, g->grid_step_z, nx, ny, nz);
        a.pb = 32;
        a.staged = 0;
        for (int pb = 32; pb >= 2; pb /= 2)   // as a plan chooses its stages
            if (bp_grid_ws_smem_bytes(wwin, pb, a.values) <= 110 * 1024) {
                a.pb = pb;
                a.staged = 1;
                break;
            }
        e = a.staged ? launch_bp_grid_ws(a, st) : launch_bp_grid(a, st);
    }
    if (e != cudaSuccess) return noalloc_fail(SAR_ERR_CUDA, cudaGetErrorString(e));
    return SAR_OK;
}

// Flag word of the last call on the current device (the first 4 bytes of the array): read after
// `stream` has passed that call, then cleared, with no allocation.
extern "C" int sar_noalloc_flags(unsigned* flags, void* stream) {
    sar_internal_set_error("");
    if (!flags) return noalloc_fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpy(flags, base, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemsetAsync(base, 0, sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return noalloc_fail(SAR_ERR_CUDA, cudaGetErrorString(e));
    return SAR_OK;
}
