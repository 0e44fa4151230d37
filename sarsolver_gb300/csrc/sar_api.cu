// sar_api.cu -- plan objects and the C ABI of libsargpu.so (see include/sargpu.h).
//
// A plan holds everything the reference rebuilds per call in SarWorker's constructor
// (src/sarsolver/cxx_binding/sarsolver_cxx.cpp:219-252): the working length M, the bin rate
// s_r and wavenumber, the waveform and slow-time weights, FFT plans, plus the GPU-side
// geometry tables (double-float antenna positions relative to the scene origin) and the range
// spans that size the stored profiles and the shared-memory windows.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <array>
#include <complex>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sargpu.h"
#include "sar_host_prep.h"
#include "sar_kernels.cuh"
#include "sar_fft_cb.h"

#include <cufftXt.h>

extern "C" const unsigned char sar_fft_cb_fatbin[];
extern "C" const size_t sar_fft_cb_fatbin_size;

using namespace sar;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(SAR_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(SAR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define SAR_CUDA(call, what)                                  \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return cuda_fail(_e, (what));  \
    } while (0)

#define SAR_CUFFT(call, what)                                                        \
    do {                                                                             \
        cufftResult _r = (call);                                                     \
        if (_r != CUFFT_SUCCESS) return fail(SAR_ERR_CUFFT, "%s: cufft error %d", (what), (int)_r); \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    int target = -1;
    cudaError_t status = cudaSuccess;
    explicit DeviceGuard(int dev) : target(dev) {
        status = cudaGetDevice(&prev);
        if (status == cudaSuccess && dev >= 0 && dev != prev) status = cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0 && target >= 0 && target != prev) cudaSetDevice(prev);
    }
};

bool finite3(const double* v, size_t n) {
    for (size_t i = 0; i < 3 * n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

// Shared-memory budgets: two tile CTAs per SM.
constexpr size_t kBpSmemBudget = 110 * 1024;
constexpr size_t kFpSmemBudget = 110 * 1024;
constexpr size_t kFpRingSmemBudget = 220 * 1024;   // ring windows: one CTA per SM
constexpr size_t kSpecBudget = (size_t)4 << 30;   // bytes of FFT work rows per chunk

}  // namespace

void sar::sar_internal_set_error(const char* msg) { g_last_error = msg ? msg : ""; }

struct sar_plan {
    int device = 0;
    size_t N = 0, S = 0, P = 0, M = 0;
    int interp = SAR_INTERP_NEAREST_REF;
    bool grid = false;
    bool forward_points = false;   // grid forward through the unstructured kernels
    GridConst gc_adj{}, gc_fwd{};
    df kappa{}, s_r{};
    long bg0 = 0;
    int Lg = 0;
    int wwin = 0, pb = 32;
    int lanes_y = 0;
    bool fwd_transposed = false;   // forward scatter: lanes along y, rows walked along x
    int gather_shear = 0;          // backprojection on a sheared lattice (gc_adj), lanes along ey + m ex
    int ring_half = 0;             // forward scatter on ring windows (FpGridArgs.ring_half), 0: strips
    long tiles_valid = 0;          // its tiles that hold image pixels (0: all tiles of the grid)
    bool staged = true;
    bool values = false;   // stored profiles are plain values (kProfValues), not pairs
    int seg_tiles = 0, segs_per_column = 0, ws = 0, pbf = 16;
    size_t n_strips = 0;
    int chunk = 0;
    std::vector<std::complex<double>> weights;

    PulseGeom* d_pulses = nullptr;
    float4* d_alpha2 = nullptr;
    double* d_steps = nullptr;      // grid steps ex, ey, ez (FP64) for exact nearest-bin decisions
    PointGeom* d_points = nullptr;
    float2* d_wave = nullptr;
    float2* d_w = nullptr;
    float2* d_wadj = nullptr;
    float2* d_wfwd = nullptr;
    void* d_spec = nullptr;        // FFT rows: float2, or double2 when fft_double
    // fused up/downsampling (N = 1024, 2048, 4096; M a multiple of N): twiddle tables e^{2 pi i q / N}, e^{2 pi i q / M}
    bool fused_up = false;
    bool fused_down = false;   // fused forward downsampling (those N, M a multiple of N, Lg <= M)
    float2* d_tw_n = nullptr;
    float2* d_tw_m = nullptr;
    bool fft_double = false;
    float4* d_prof = nullptr;   // [S][Lg] pairs (adjoint) / float2 accumulator (forward)
    int* d_strip = nullptr;
    unsigned* d_flags = nullptr;
    size_t block = 0;   // streamed plan: profile buffer of two blocks of this many pulses (0: all S)
    long long wait_budget = kDefaultWaitBudgetCycles;   // bounded in-kernel waits of the gather
    int hold_first_stage = 0;                           // test aid (sar_plan_set_wait_budget)
    size_t device_bytes = 0;
    cufftHandle fft_full = 0, fft_tail = 0;
    bool have_full = false, have_tail = false;
    int tail_rows = 0;
    std::vector<std::pair<int, cufftHandle>> fft_other;   // other batch sizes (pulse blocks), made on first use
    // cuFFT callback path (single precision, large problems): plans per direction and batch size
    // with the load/store callbacks of sar_fft_callbacks.cu linked in, their parameter block, and
    // the compact adjoint output [chunk][Lc].
    bool fft_cb = false;
    SarFftCbInfo* d_cb = nullptr;
    float2* d_compact = nullptr;
    int Lc = 0;
    std::vector<std::pair<int, cufftHandle>> cb_adj, cb_fwd;
    cudaStream_t last_stream = nullptr;
    std::mutex mu;
    // stage timing: 4 events per recorded call (start, pre-kernel done, kernel done, end)
    bool timing = false;
    std::vector<std::array<cudaEvent_t, 4>> events;
    size_t events_used = 0;

    // Next event slot of a timed call, or nullptr when timing is off or the record is full.
    cudaEvent_t* timing_slot() {
        if (!timing || events_used >= 4096) return nullptr;
        if (events_used == events.size()) {
            std::array<cudaEvent_t, 4> ev{};
            for (auto& e : ev)
                if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            events.push_back(ev);
        }
        return events[events_used++].data();
    }

    template <class T>
    int alloc(T** p, size_t count, const char* what) {
        cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1));
        if (e != cudaSuccess) return cuda_fail(e, what);
        device_bytes += sizeof(T) * std::max<size_t>(count, 1);
        return SAR_OK;
    }

    ~sar_plan() {
        DeviceGuard g(device);
        cudaFree(d_pulses);
        cudaFree(d_alpha2);
        cudaFree(d_steps);
        cudaFree(d_points);
        cudaFree(d_wave);
        cudaFree(d_w);
        cudaFree(d_wadj);
        cudaFree(d_wfwd);
        cudaFree(d_spec);
        cudaFree(d_tw_n);
        cudaFree(d_tw_m);
        cudaFree(d_prof);
        cudaFree(d_strip);
        cudaFree(d_flags);
        if (have_full) cufftDestroy(fft_full);
        if (have_tail) cufftDestroy(fft_tail);
        for (auto& e : fft_other) cufftDestroy(e.second);
        for (auto& e : cb_adj) cufftDestroy(e.second);
        for (auto& e : cb_fwd) cufftDestroy(e.second);
        cudaFree(d_cb);
        cudaFree(d_compact);
        for (auto& ev : events)
            for (auto e : ev) cudaEventDestroy(e);
    }
};

static inline void mark(cudaEvent_t* ev, int i, cudaStream_t st) {
    if (ev) cudaEventRecord(ev[i], st);
}

namespace {

float adjoint_bin_offset(int interp) { return interp == SAR_INTERP_LINEAR ? -0.5f : 0.5f; }
float forward_bin_offset(int interp) { return interp == SAR_INTERP_LINEAR ? -0.5f : 0.0f; }

// Bistatic differential range span [lo, hi] of a box region for pulse s.
void region_range(const double* tx, const double* rx, const double* srp, const double* o,
                  const double* ex, const double* ey, const double* ez, double nu, double nv,
                  double nw, double* lo, double* hi) {
    double a0, a1, b0, b1;
    box_distance_bounds(tx, o, ex, ey, ez, nu, nv, nw, &a0, &a1);
    box_distance_bounds(rx, o, ex, ey, ez, nu, nv, nw, &b0, &b1);
    const double ref = dist3(tx, srp) + dist3(rx, srp);
    *lo = a0 + b0 - ref;
    *hi = a1 + b1 - ref;
}

int upload_weights(sar_plan* p, cudaStream_t st, bool sync) {
    std::vector<float2> w(p->S);
    for (size_t s = 0; s < p->S; ++s) w[s] = make_float2((float)p->weights[s].real(), (float)p->weights[s].imag());
    SAR_CUDA(cudaMemcpyAsync(p->d_w, w.data(), sizeof(float2) * p->S, cudaMemcpyHostToDevice, st), "upload weights");
    SAR_CUDA(launch_weights(p->d_w, p->d_wadj, p->d_wfwd, (int)p->S, p->interp == SAR_INTERP_LINEAR, st),
             "weights kernel");
    if (sync) SAR_CUDA(cudaStreamSynchronize(st), "upload weights");
    return SAR_OK;
}

int make_fft(cufftHandle* h, long M, int batch, bool dbl) {
    int n[1] = {(int)M};
    SAR_CUFFT(cufftPlanMany(h, 1, n, nullptr, 1, (int)M, nullptr, 1, (int)M, dbl ? CUFFT_Z2Z : CUFFT_C2C, batch),
              "cufftPlanMany");
    return SAR_OK;
}

int run_fft(sar_plan* p, void* data, int rows, int direction, cudaStream_t st) {
    cufftHandle h = 0;
    if (rows == p->chunk) {
        h = p->fft_full;
    } else if (p->have_tail && rows == p->tail_rows) {
        h = p->fft_tail;
    } else {
        for (auto& e : p->fft_other)
            if (e.first == rows) h = e.second;
        if (!h) {
            int rc = make_fft(&h, (long)p->M, rows, p->fft_double);
            if (rc) return rc;
            p->fft_other.emplace_back(rows, h);
        }
    }
    SAR_CUFFT(cufftSetStream(h, st), "cufftSetStream");
    if (p->fft_double)
        SAR_CUFFT(cufftExecZ2Z(h, reinterpret_cast<cufftDoubleComplex*>(data),
                               reinterpret_cast<cufftDoubleComplex*>(data), direction),
                  "cufftExecZ2Z");
    else
        SAR_CUFFT(cufftExecC2C(h, reinterpret_cast<cufftComplex*>(data), reinterpret_cast<cufftComplex*>(data),
                               direction),
                  "cufftExecC2C");
    return SAR_OK;
}

// A C2C plan of `batch` rows of length M with the adjoint (inverse) or forward callbacks linked in.
int make_cb_fft(sar_plan* p, cufftHandle* h, int batch, bool adjoint) {
    SAR_CUFFT(cufftCreate(h), "cufftCreate");
    void* info = p->d_cb;
    cufftResult r = cufftXtSetJITCallback(*h, adjoint ? "sar_cb_adjoint_load" : "sar_cb_forward_load", sar_fft_cb_fatbin,
                                          sar_fft_cb_fatbin_size, CUFFT_CB_LD_COMPLEX, &info);
    if (r == CUFFT_SUCCESS)
        r = cufftXtSetJITCallback(*h, adjoint ? "sar_cb_adjoint_store" : "sar_cb_forward_store", sar_fft_cb_fatbin,
                                  sar_fft_cb_fatbin_size, CUFFT_CB_ST_COMPLEX, &info);
    size_t work = 0;
    int n[1] = {(int)p->M};
    if (r == CUFFT_SUCCESS)
        r = cufftMakePlanMany(*h, 1, n, nullptr, 1, (int)p->M, nullptr, 1, (int)p->M, CUFFT_C2C, batch, &work);
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(*h);
        *h = 0;
        return fail(SAR_ERR_CUFFT, "callback FFT plan (batch %d): cufft error %d", batch, (int)r);
    }
    return SAR_OK;
}

int cb_plan(sar_plan* p, int rows, bool adjoint, cufftHandle* h) {
    auto& list = adjoint ? p->cb_adj : p->cb_fwd;
    for (auto& e : list)
        if (e.first == rows) {
            *h = e.second;
            return SAR_OK;
        }
    int rc = make_cb_fft(p, h, rows, adjoint);
    if (rc) return rc;
    list.emplace_back(rows, *h);
    return SAR_OK;
}

// Parameters of one callback transform (rows first .. first + rows - 1), stream-ordered.
int set_cb_info(sar_plan* p, const float2* y, float2* yout, int first, cudaStream_t st) {
    SarFftCbInfo c{};
    c.y = y;
    c.yout = yout;
    c.wave = p->d_wave;
    c.wfac = p->d_wfwd;
    c.acc = reinterpret_cast<const float2*>(p->d_prof);
    c.compact = p->d_compact;
    c.M = (long long)p->M;
    long long nb0 = -(long long)p->bg0 % (long long)p->M;
    if (nb0 < 0) nb0 += (long long)p->M;
    c.nb0 = nb0;
    const bool pow2 = (p->M & (p->M - 1)) == 0;
    c.mask = pow2 ? (unsigned)(p->M - 1) : 0u;
    int sh = 0;
    while (pow2 && ((size_t)1 << sh) < p->M) ++sh;
    c.shift = sh;
    c.N = (int)p->N;
    c.half = (int)(p->N / 2);
    c.Lg = p->Lg;
    c.Lc = p->Lc;
    c.first = first;
    // pageable source: the copy is staged before the call returns, so `c` may go out of scope
    SAR_CUDA(cudaMemcpyAsync(p->d_cb, &c, sizeof c, cudaMemcpyHostToDevice, st), "callback parameters");
    return SAR_OK;
}

// Working lengths with a prime factor above 7 go through a double-precision transform: the
// single-precision transform of such lengths measured ~1e-4 relative image error.
bool smooth_length(size_t m) {
    for (size_t f : {2, 3, 5, 7})
        while (m % f == 0) m /= f;
    return m == 1;
}

// Host-only validation of a geometry description (no CUDA call).
int validate_geometry(const sar_geometry* g) {
    const size_t N = g->num_fast_times, S = g->num_slow_times, P = g->num_scatterers;
    if (N == 0 || S == 0 || P == 0) return fail(SAR_ERR_INVALID_ARGUMENT, "empty problem: N=%zu S=%zu P=%zu", N, S, P);
    if (!g->transmit_posns || !g->receive_posns || !g->stab_ref_posns)
        return fail(SAR_ERR_INVALID_ARGUMENT, "antenna / SRP positions are required");
    if (!(g->c_eff > 0.0) || !(g->sample_frequency > 0.0) || !(g->upsample_ratio > 0.0) ||
        !std::isfinite(g->centre_frequency) || !std::isfinite(g->sign_multiplier))
        return fail(SAR_ERR_INVALID_ARGUMENT, "c_eff, sample_frequency and upsample_ratio must be positive");
    if (g->interp != SAR_INTERP_NEAREST_REF && g->interp != SAR_INTERP_LINEAR)
        return fail(SAR_ERR_INVALID_ARGUMENT, "unknown interpolation mode %d", g->interp);
    if (g->path < SAR_PATH_AUTO || g->path > SAR_PATH_POINTS)
        return fail(SAR_ERR_INVALID_ARGUMENT, "unknown path %d", g->path);
    const size_t M = (size_t)(g->upsample_ratio * (double)N);   // sarsolver_cxx.cpp:223
    if (M < N) return fail(SAR_ERR_INVALID_ARGUMENT, "upsample_ratio*N (%zu) is below N (%zu)", M, N);
    if (M > (size_t)1 << 30 || S > (size_t)1 << 30 || N > (size_t)1 << 30)
        return fail(SAR_ERR_NOT_SUPPORTED, "sizes beyond 2^30 are not supported");
    if (!finite3(g->transmit_posns, S) || !finite3(g->receive_posns, S) || !finite3(g->stab_ref_posns, S))
        return fail(SAR_ERR_INVALID_ARGUMENT, "non-finite antenna or SRP position");
    const bool grid = g->grid_shape[0] || g->grid_shape[1] || g->grid_shape[2];
    if (grid) {
        if (!g->grid_shape[0] || !g->grid_shape[1] || !g->grid_shape[2])
            return fail(SAR_ERR_INVALID_ARGUMENT, "grid_shape must be all positive or all zero");
        if (g->grid_shape[0] * g->grid_shape[1] * g->grid_shape[2] != P)
            return fail(SAR_ERR_INVALID_ARGUMENT, "grid_shape product != num_scatterers");
        if (g->grid_shape[1] > (1u << 20) || g->grid_shape[2] > (1u << 20) || g->grid_shape[0] > (1u << 16))
            return fail(SAR_ERR_NOT_SUPPORTED, "grid dimension too large");
        if (!finite3(g->grid_origin, 1) || !finite3(g->grid_step_x, 1) || !finite3(g->grid_step_y, 1) ||
            !finite3(g->grid_step_z, 1))
            return fail(SAR_ERR_INVALID_ARGUMENT, "non-finite grid description");
    } else {
        if (!g->scat_posns) return fail(SAR_ERR_INVALID_ARGUMENT, "scat_posns is required without a grid");
        if (!finite3(g->scat_posns, P)) return fail(SAR_ERR_INVALID_ARGUMENT, "non-finite scatterer position");
        if (P > (size_t)1 << 31) return fail(SAR_ERR_NOT_SUPPORTED, "too many scatterers");
    }

    return SAR_OK;
}

// Tile window (bins) of the grid gather, or -1 where the grid spacing is too coarse for the
// range sampling (the grid kernels then do not apply).
static int grid_tile_window(const sar_geometry* g, double s_r) {
    const double* ex = g->grid_step_x;
    const double* ey = g->grid_step_y;
    const double nex = std::sqrt(ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2]);
    const double ney = std::sqrt(ey[0] * ey[0] + ey[1] * ey[1] + ey[2] * ey[2]);
    const double h = s_r * 2.0 * 16.0 * (nex + ney);
    if (!(h <= 1.0e6)) return -1;
    return (2 * ((int)std::ceil(h) + 3) + 3) & ~3;
}

int build_plan(const sar_geometry* g_in, sar_plan* p) {
    const sar_geometry* g = g_in;
    const size_t N = g->num_fast_times, S = g->num_slow_times, P = g->num_scatterers;
    const size_t M = (size_t)(g->upsample_ratio * (double)N);
    bool grid = g->grid_shape[0] || g->grid_shape[1] || g->grid_shape[2];
    // A grid routed to the per-pixel path is expanded into explicit positions.
    sar_geometry expanded;
    std::vector<double> grid_positions;
    // nearest_ref takes the grid kernels by default too (their nearest bins are decided exactly near
    // rounding boundaries); only grids too coarse for them go to the per-pixel kernels
    bool grid_ok = true;
    if (grid && g->path == SAR_PATH_AUTO && g->interp == SAR_INTERP_NEAREST_REF && g->c_eff > 0.0 && N > 0)
        grid_ok = grid_tile_window(g, g->sample_frequency * (double)M / ((double)N * g->c_eff)) > 0;
    const bool to_points = grid && (g->path == SAR_PATH_POINTS || !grid_ok);
    if (to_points) {
        const size_t nz = g->grid_shape[0], ny = g->grid_shape[1], nx = g->grid_shape[2];
        grid_positions.resize(3 * P);
        for (size_t k = 0; k < nz; ++k)
            for (size_t j = 0; j < ny; ++j)
                for (size_t i = 0; i < nx; ++i) {
                    double* q = &grid_positions[3 * ((k * ny + j) * nx + i)];
                    for (int c = 0; c < 3; ++c)
                        q[c] = g->grid_origin[c] + (double)i * g->grid_step_x[c] + (double)j * g->grid_step_y[c] +
                               (double)k * g->grid_step_z[c];
                }
        expanded = *g;
        expanded.scat_posns = grid_positions.data();
        expanded.grid_shape[0] = expanded.grid_shape[1] = expanded.grid_shape[2] = 0;
        g = &expanded;
        grid = false;
    }
    p->N = N;
    p->S = S;
    p->P = P;
    p->M = M;
    p->interp = g->interp;
    p->grid = grid;
    const double s_r = g->sample_frequency * (double)M / ((double)N * g->c_eff);    // :225-226
    const double kappa = g->sign_multiplier * g->centre_frequency / g->c_eff;       // :228 / 2pi
    p->kappa = to_df(kappa);
    p->s_r = to_df(s_r);
    const double* tx = g->transmit_posns;
    const double* rx = g->receive_posns;
    const double* srp = g->stab_ref_posns;

    p->weights.resize(S);
    for (size_t s = 0; s < S; ++s)
        p->weights[s] = g->slow_time_weighting
                            ? std::complex<double>(g->slow_time_weighting[2 * s], g->slow_time_weighting[2 * s + 1])
                            : std::complex<double>(1.0, 0.0);

    double origin[3];
    double vmin = INFINITY, vmax = -INFINITY;
    std::vector<PulseGeom> pulses(S);
    std::vector<float4> alpha2;
    std::vector<PointGeom> points;
    std::vector<int> strip_start;

    if (grid) {
        const int nz = (int)g->grid_shape[0], ny = (int)g->grid_shape[1], nx = (int)g->grid_shape[2];
        for (int c = 0; c < 3; ++c) origin[c] = g->grid_origin[c];
        const double *ex = g->grid_step_x, *ey = g->grid_step_y, *ez = g->grid_step_z;
        p->gc_adj = make_grid_const(ex, ey, ez, kappa, s_r, adjoint_bin_offset(p->interp), nx, ny, nz);
        p->gc_fwd = p->gc_adj;
        p->gc_fwd.bin_offset = forward_bin_offset(p->interp);
        const int tx_tiles = p->gc_adj.tiles_x, ty_tiles = p->gc_adj.tiles_y;
        for (size_t s = 0; s < S; ++s) {
            pulses[s] = make_pulse_geom(tx + 3 * s, rx + 3 * s, srp + 3 * s, origin);
            double lo, hi;
            region_range(tx + 3 * s, rx + 3 * s, srp + 3 * s, origin, ex, ey, ez, tx_tiles * kTile - 1.0,
                         ty_tiles * kTile - 1.0, nz - 1.0, &lo, &hi);
            vmin = std::min(vmin, lo * s_r);
            vmax = std::max(vmax, hi * s_r);
        }
        // Tile window: every pixel of a tile lies within 16|ex| + 16|ey| of the tile centre, and
        // each of the two ranges changes by at most that distance; tighter from the look
        // directions where the antennas are clear of the scene.
        p->wwin = grid_tile_window(g, s_r);
        if (p->wwin < 0) return fail(SAR_ERR_NOT_SUPPORTED, "grid spacing too coarse for the range sampling");
        {
            const double hd = tile_halfspan_directional(tx, rx, S, origin, ex, ey, ez, kTile, p->gc_adj.tiles_x,
                                                        p->gc_adj.tiles_y, nz, s_r);
            if (hd >= 0.0) p->wwin = std::min(p->wwin, (2 * ((int)std::ceil(hd) + 3) + 3) & ~3);
        }
        const int plain_lanes_y = choose_lanes_y(tx, rx, S, origin, ex, ey, ez, nx, ny, nz);
        p->lanes_y = plain_lanes_y;
        // Nearest-bin decisions must match FP64, and wide tiles need the exact integer part:
        // split the linear bin rates in both cases (sar_geom.cuh, bin_coeffs).
        p->gc_adj.precise_bins = p->gc_fwd.precise_bins = (p->interp == SAR_INTERP_NEAREST_REF || p->wwin > 256) ? 1 : 0;
        // stored profile span: margins of the isotropic window, which the no-allocation entry
        // point (sar_noalloc.cu) requires of a caller's span as well
        int span_ww = std::max(p->wwin, grid_tile_window(g, s_r));
        // Backprojection on a sheared lattice (steps ex, ey + m ex; lattice pixel (a, b) is image
        // pixel (a + a_off + m b, b)) with lanes along its second axis, where the bins of a
        // collection looking across the grid axes change slowly (choose_gather_shear): the window
        // loads are then broadcast instead of bank-conflicted.  Taken when its directional window
        // is no wider than the plain one and stages; lattice tiles straddle the image's edges, so
        // the span's margins grow to two isotropic lattice windows (a tile's centre lies at most
        // half an isotropic window, in bins, outside the image's range).
        // Linear sampling only: with nearest bins (exact re-decisions) it measured 9 % slower.
        const int gshear = p->interp == SAR_INTERP_LINEAR
                               ? choose_gather_shear(tx, rx, S, origin, ex, ey, ez, nx, ny, nz, s_r)
                               : 0;
        if (gshear) {
            GridConst gl = make_lattice_const(ex, ey, ez, kappa, s_r, adjoint_bin_offset(p->interp), nx, ny, nz, gshear);
            gl.precise_bins = p->gc_adj.precise_bins;
            double ol[3], eyl[3];
            for (int c = 0; c < 3; ++c) {
                ol[c] = origin[c] + gl.a_off * ex[c];
                eyl[c] = ey[c] + gshear * ex[c];
            }
            const double hl = s_r * 2.0 * 16.0 * (std::sqrt(ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2]) +
                                                  std::sqrt(eyl[0] * eyl[0] + eyl[1] * eyl[1] + eyl[2] * eyl[2]));
            const int wiso = (2 * ((int)std::ceil(hl) + 3) + 3) & ~3;
            const double hd = tile_halfspan_directional(tx, rx, S, ol, ex, eyl, ez, kTile, gl.tiles_x, gl.tiles_y, nz, s_r);
            const int wl = hd >= 0.0 ? std::min(wiso, (2 * ((int)std::ceil(hd) + 3) + 3) & ~3) : wiso;
            if (hl <= 1.0e6 && wl <= p->wwin && bp_grid_ws_smem_bytes(wl, 2, 0) <= kBpSmemBudget) {
                p->gc_adj = gl;
                p->wwin = wl;
                p->lanes_y = 1;
                p->gather_shear = gshear;
                span_ww = std::max(span_ww, 2 * wiso);
                p->tiles_valid = 0;
                for (int ta = 0; ta < gl.tiles_x; ++ta) {
                    int lo, hi;
                    lattice_tile_range(gl, ta, &lo, &hi);
                    if (hi >= lo) p->tiles_valid += (long)(hi - lo + 1) * nz;
                }
            }
        }
        p->bg0 = (long)std::floor(vmin) - span_ww / 2 - 4;
        const double span = std::ceil(vmax) + span_ww / 2 + 5 - (double)p->bg0;
        if (span > 2.0e9) return fail(SAR_ERR_NOT_SUPPORTED, "range span too large");
        p->Lg = (int)span + ((int)span & 1);   // even: rows of plain values stay 16-byte aligned
        // Backprojection staging: pulses per stage so that the double-buffered windows of the
        // pipelined kernel fit shared memory with two CTAs per SM; otherwise read windows
        // from global memory directly.
        p->staged = false;
        p->pb = 32;
        // stages the two producer warps split evenly.  Windows wider than 256 bins (large upsampling
        // factors) store and stage plain values, half the bytes of pairs (linear sampling reads two
        // neighbours): at upsample 128 that measured a third faster for nearest bins, at upsample 8
        // slower (wider addressing in the gather), so narrower windows keep pairs.  The unstaged
        // gather reads pairs for linear sampling.
        p->values = p->wwin > 256;
        for (int pb = 32; pb >= 2; pb /= 2)
            if (bp_grid_ws_smem_bytes(p->wwin, pb, p->values) <= kBpSmemBudget) {
                p->pb = pb;
                p->staged = true;
                break;
            }
        if (!p->staged && p->interp == SAR_INTERP_LINEAR) p->values = false;
        // Forward scatter layout: it walks the gather's lane axis (the transpose of its lane
        // choice), or, for linear sampling across the grid axes, a sheared lattice whose rows
        // follow the iso-range lines (choose_shear), walked with lanes along x.
        p->fwd_transposed = !plain_lanes_y;
        const int shear = (p->interp == SAR_INTERP_LINEAR && !p->gc_fwd.precise_bins)
                              ? choose_shear(tx, rx, S, origin, ex, ey, ez, nx, ny, nz, s_r, plain_lanes_y)
                              : 0;
        double ey_f[3];
        for (int c = 0; c < 3; ++c) ey_f[c] = ey[c] + shear * ex[c];
        if (shear) {
            const int precise = p->gc_fwd.precise_bins;
            p->gc_fwd = make_lattice_const(ex, ey, ez, kappa, s_r, forward_bin_offset(p->interp), nx, ny, nz, shear);
            p->gc_fwd.precise_bins = precise;
            p->fwd_transposed = false;
        }
        // Forward strips: lines of tiles along the axis the scatter walks (columns along y; rows
        // along x for the transposed scatter; lattice columns for a sheared lattice, only their
        // tiles that hold image pixels), split into segments whose window fits shared memory.
        const bool strips_x = p->fwd_transposed;
        const int ftx = p->gc_fwd.tiles_x, fty = p->gc_fwd.tiles_y;
        const int lines = strips_x ? fty : ftx;
        std::vector<int> line_lo(lines, 0), line_hi(lines, (strips_x ? ftx : fty) - 1);
        int along = 0;
        for (int ln = 0; ln < lines; ++ln) {
            if (!strips_x) lattice_tile_range(p->gc_fwd, ln, &line_lo[ln], &line_hi[ln]);
            along = std::max(along, line_hi[ln] - line_lo[ln] + 1);
        }
        p->forward_points = true;
        for (int pbf : {16, 8}) {
            int seg = along;
            while (true) {
                const int segs = (along + seg - 1) / seg;
                const size_t n_strips = (size_t)nz * lines * segs;
                std::vector<int> starts(n_strips * S);
                int need = 0;
                for (int k = 0; k < nz; ++k)
                    for (int ln = 0; ln < lines; ++ln)
                        for (int sg = 0; sg < segs; ++sg) {
                            const int t0 = line_lo[ln] + sg * seg, t1 = std::min(t0 + seg, line_hi[ln] + 1);
                            const size_t strip = ((size_t)k * lines + ln) * segs + sg;
                            if (t0 >= t1) continue;   // no tile: the kernel's CTA leaves at once
                            const int ti0 = strips_x ? t0 : ln, tj0 = strips_x ? ln : t0;
                            const double nu = strips_x ? (t1 - t0) * kTile - 1.0 : kTile - 1.0;
                            const double nv = strips_x ? kTile - 1.0 : (t1 - t0) * kTile - 1.0;
                            double o[3];
                            for (int c = 0; c < 3; ++c)
                                o[c] = origin[c] + (ti0 * kTile + p->gc_fwd.a_off) * ex[c] + tj0 * kTile * ey_f[c] +
                                       k * ez[c];
                            for (size_t s = 0; s < S; ++s) {
                                double lo, hi;
                                if (shear) {   // a parallelogram: the box bound assumes orthogonal edges
                                    double e1[3], e2[3], a0, a1, b0, b1;
                                    for (int c = 0; c < 3; ++c) {
                                        e1[c] = nu * ex[c];
                                        e2[c] = nv * ey_f[c];
                                    }
                                    parallelogram_distance_bounds(tx + 3 * s, o, e1, e2, &a0, &a1);
                                    parallelogram_distance_bounds(rx + 3 * s, o, e1, e2, &b0, &b1);
                                    const double ref = dist3(tx + 3 * s, srp + 3 * s) + dist3(rx + 3 * s, srp + 3 * s);
                                    lo = a0 + b0 - ref;
                                    hi = a1 + b1 - ref;
                                } else {
                                    region_range(tx + 3 * s, rx + 3 * s, srp + 3 * s, o, ex, ey, ez, nu, nv, 0.0, &lo, &hi);
                                }
                                const long b0 = (long)std::floor(lo * s_r) - 3;
                                const long b1 = (long)std::ceil(hi * s_r) + 4;
                                starts[strip * S + s] = (int)b0;
                                need = std::max<int>(need, (int)(b1 - b0 + 1));
                            }
                        }
                const int ws = (need + 31) & ~31;
                if (fp_grid_ws_smem_bytes(ws, pbf, p->interp == SAR_INTERP_LINEAR && !p->gc_fwd.precise_bins) <=
                    kFpSmemBudget) {
                    p->seg_tiles = seg;
                    p->segs_per_column = segs;
                    p->ws = ws;
                    p->pbf = pbf;
                    p->n_strips = n_strips;
                    strip_start.swap(starts);
                    p->forward_points = false;
                    break;
                }
                if (seg == 1) break;
                seg = (seg + 1) / 2;
            }
            if (!p->forward_points) break;
        }
        // Ring windows (split bins): where strip windows hold only one or two tiles (a 32-pixel tile
        // spans ~1200 bins at upsample 128), every CTA would clear and merge a whole window for 1024
        // pixels per pulse.  A ring of W = 2^k >= 2 H + 1 slots per pulse instead holds one tile's
        // range (its base bin +- H, H from the look directions as for the gather's windows) and a CTA
        // walks its whole line, adding and clearing only the bins each tile step leaves behind.
        if (p->gc_fwd.precise_bins && (p->forward_points || p->seg_tiles <= 2)) {
            const double hd = tile_halfspan_directional(tx, rx, S, origin, ex, ey, ez, kTile, p->gc_fwd.tiles_x,
                                                        p->gc_fwd.tiles_y, nz, s_r);
            const double h = hd >= 0.0 ? hd : 0.5 * grid_tile_window(g, s_r);
            if (h >= 0.0 && h < 1.0e6) {
                const int H = (int)std::ceil(h) + 4;
                int W = 32;
                while (W < 2 * H + 1) W *= 2;
                for (int pbf : {16, 8})
                    if (fp_grid_ws_smem_bytes(W, pbf, 0) <= kFpRingSmemBudget) {
                        p->ring_half = H;
                        p->ws = W;
                        p->pbf = pbf;
                        p->seg_tiles = along;
                        p->segs_per_column = 1;
                        p->n_strips = (size_t)nz * lines;
                        strip_start.assign(p->n_strips * S, 0);   // not read with ring windows
                        p->forward_points = false;
                        break;
                    }
            }
        }
        if (p->forward_points) {
            // Extremely coarse grids: forward through the unstructured kernels.
            points.resize(P);
            alpha2.resize(S);
        }
        if (p->forward_points) {
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        double q[3];
                        for (int c = 0; c < 3; ++c) q[c] = i * ex[c] + j * ey[c] + k * ez[c];
                        PointGeom& pt = points[((size_t)k * ny + j) * nx + i];
                        for (int c = 0; c < 3; ++c) {
                            const df d = to_df(q[c]);
                            pt.qh[c] = d.hi;
                            pt.ql[c] = d.lo;
                        }
                        const df d2 = to_df(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
                        pt.qh[3] = d2.hi;
                        pt.ql[3] = d2.lo;
                    }
        }
    } else {
        const double* pos = g->scat_posns;
        double lo3[3] = {INFINITY, INFINITY, INFINITY}, hi3[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t i = 0; i < P; ++i)
            for (int c = 0; c < 3; ++c) {
                lo3[c] = std::min(lo3[c], pos[3 * i + c]);
                hi3[c] = std::max(hi3[c], pos[3 * i + c]);
            }
        for (int c = 0; c < 3; ++c) origin[c] = 0.5 * (lo3[c] + hi3[c]);
        points.resize(P);
        alpha2.resize(S);
        for (size_t i = 0; i < P; ++i) {
            double q[3];
            for (int c = 0; c < 3; ++c) q[c] = pos[3 * i + c] - origin[c];
            PointGeom& pt = points[i];
            for (int c = 0; c < 3; ++c) {
                const df d = to_df(q[c]);
                pt.qh[c] = d.hi;
                pt.ql[c] = d.lo;
            }
            const df d2 = to_df(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            pt.qh[3] = d2.hi;
            pt.ql[3] = d2.lo;
        }
        const double ex[3] = {hi3[0] - lo3[0], 0, 0}, ey[3] = {0, hi3[1] - lo3[1], 0}, ez[3] = {0, 0, hi3[2] - lo3[2]};
        for (size_t s = 0; s < S; ++s) {
            pulses[s] = make_pulse_geom(tx + 3 * s, rx + 3 * s, srp + 3 * s, origin);
            double lo, hi;
            region_range(tx + 3 * s, rx + 3 * s, srp + 3 * s, lo3, ex, ey, ez, 1.0, 1.0, 1.0, &lo, &hi);
            vmin = std::min(vmin, lo * s_r);
            vmax = std::max(vmax, hi * s_r);
        }
        p->bg0 = (long)std::floor(vmin) - 4;
        const double span = std::ceil(vmax) + 6 - (double)p->bg0;
        if (span > 2.0e9) return fail(SAR_ERR_NOT_SUPPORTED, "range span too large");
        p->Lg = (int)span + ((int)span & 1);
        p->wwin = 0;
    }
    // nearest bins on the grid paths: antenna norms for the exact decisions near a boundary
    if (grid && p->interp == SAR_INTERP_NEAREST_REF) alpha2.resize(S);
    if (!alpha2.empty()) {
        for (size_t s = 0; s < S; ++s) {
            double at[3], ar[3];
            for (int c = 0; c < 3; ++c) {
                at[c] = tx[3 * s + c] - origin[c];
                ar[c] = rx[3 * s + c] - origin[c];
            }
            const df a = to_df(at[0] * at[0] + at[1] * at[1] + at[2] * at[2]);
            const df b = to_df(ar[0] * ar[0] + ar[1] * ar[1] + ar[2] * ar[2]);
            alpha2[s] = make_float4(a.hi, a.lo, b.hi, b.lo);
        }
    }

    // ---- device tables
    int rc;
    if ((rc = p->alloc(&p->d_pulses, S, "pulse table"))) return rc;
    SAR_CUDA(cudaMemcpy(p->d_pulses, pulses.data(), sizeof(PulseGeom) * S, cudaMemcpyHostToDevice), "pulse table");
    if (!points.empty()) {
        if ((rc = p->alloc(&p->d_points, P, "point table"))) return rc;
        SAR_CUDA(cudaMemcpy(p->d_points, points.data(), sizeof(PointGeom) * P, cudaMemcpyHostToDevice), "point table");
    }
    if (!alpha2.empty()) {
        if ((rc = p->alloc(&p->d_alpha2, S, "antenna norms"))) return rc;
        SAR_CUDA(cudaMemcpy(p->d_alpha2, alpha2.data(), sizeof(float4) * S, cudaMemcpyHostToDevice), "antenna norms");
    }
    if (grid) {
        double steps[9];
        for (int c = 0; c < 3; ++c) {
            steps[c] = g->grid_step_x[c];
            steps[3 + c] = g->grid_step_y[c];
            steps[6 + c] = g->grid_step_z[c];
        }
        if ((rc = p->alloc(&p->d_steps, 9, "grid steps"))) return rc;
        SAR_CUDA(cudaMemcpy(p->d_steps, steps, sizeof steps, cudaMemcpyHostToDevice), "grid steps");
    }
    if (!strip_start.empty()) {
        if ((rc = p->alloc(&p->d_strip, strip_start.size(), "strip table"))) return rc;
        SAR_CUDA(cudaMemcpy(p->d_strip, strip_start.data(), sizeof(int) * strip_start.size(), cudaMemcpyHostToDevice),
                 "strip table");
    }
    std::vector<float2> wave(N);
    for (size_t f = 0; f < N; ++f)
        wave[f] = g->waveform_fft ? make_float2((float)g->waveform_fft[2 * f], (float)g->waveform_fft[2 * f + 1])
                                  : make_float2(1.f, 0.f);
    if ((rc = p->alloc(&p->d_wave, N, "waveform"))) return rc;
    SAR_CUDA(cudaMemcpy(p->d_wave, wave.data(), sizeof(float2) * N, cudaMemcpyHostToDevice), "waveform");
    if ((rc = p->alloc(&p->d_w, S, "weights"))) return rc;
    if ((rc = p->alloc(&p->d_wadj, S, "weights"))) return rc;
    if ((rc = p->alloc(&p->d_wfwd, S, "weights"))) return rc;
    if ((rc = upload_weights(p, nullptr, true))) return rc;
    if ((rc = p->alloc(&p->d_flags, 1, "flags"))) return rc;
    SAR_CUDA(cudaMemset(p->d_flags, 0, sizeof(unsigned)), "flags");
    if (p->block && (!grid || p->forward_points))
        return fail(SAR_ERR_NOT_SUPPORTED, "streamed plans need the regular-grid kernels (forward and backprojection)");
    // resident: profiles of all S pulses; streamed: a ring of two blocks (the forward's accumulator
    // of one block, [block][Lg] float2, fits in half of one slot)
    if ((rc = p->alloc(&p->d_prof, (size_t)(p->block ? 2 * p->block : S) * p->Lg, "range profiles"))) return rc;

    // ---- FFT work rows
    p->fft_double = !smooth_length(M);
    const size_t elem = p->fft_double ? sizeof(double2) : sizeof(float2);
    p->chunk = (int)std::min<size_t>(p->block ? p->block : S, std::max<size_t>(1, kSpecBudget / (M * elem)));
    {
        double2* spec = nullptr;
        if ((rc = p->alloc(&spec, ((size_t)p->chunk * M * elem + sizeof(double2) - 1) / sizeof(double2), "FFT rows")))
            return rc;
        p->d_spec = spec;
    }
    if ((rc = make_fft(&p->fft_full, (long)M, p->chunk, p->fft_double))) return rc;
    p->have_full = true;
    const int tail = (int)(S % (size_t)p->chunk);
    if (tail) {
        if ((rc = make_fft(&p->fft_tail, (long)M, tail, p->fft_double))) return rc;
        p->have_tail = true;
        p->tail_rows = tail;
    }
    // Fused adjoint upsampling: for N = 512, 1024, 2048, 4096 or 8192 and M a multiple of N the backprojection's range
    // profiles come from one kernel (U-way split of the length-M transform into N-point ones,
    // stored span only) instead of pack + inverse FFT + unpack; twiddles computed in FP64.
    const bool up_ok = upsample_fused_supported((int)N, (long)M, p->Lg);
    const bool down_ok = downsample_fused_supported((int)N, (long)M, p->Lg);
    if (up_ok || down_ok) {
        // tw_m: e^{2 pi i q / M} for q < M, then for each residue r < 2U the 16 thread-independent
        // factors e^{2 pi i (T e - N [e >= 8]) r / M} (T = N / 16) of the fused kernels' twiddles
        const size_t U = M / N, T = N / 16;
        std::vector<float2> tn(N), tm(M + 2 * U * 16);
        const double two_pi = 6.283185307179586476925286766559;
        for (size_t q = 0; q < N; ++q)
            tn[q] = make_float2((float)std::cos(two_pi * (double)q / (double)N), (float)std::sin(two_pi * (double)q / (double)N));
        for (size_t q = 0; q < M; ++q)
            tm[q] = make_float2((float)std::cos(two_pi * (double)q / (double)M), (float)std::sin(two_pi * (double)q / (double)M));
        for (size_t r = 0; r < 2 * U; ++r)
            for (size_t e = 0; e < 16; ++e) {
                const long k = (long)(T * e) - (e >= 8 ? (long)N : 0L);
                long q = (k * (long)r) % (long)M;   // exact integer phase, then one FP64 angle
                if (q < 0) q += (long)M;
                tm[M + 16 * r + e] = make_float2((float)std::cos(two_pi * (double)q / (double)M),
                                                 (float)std::sin(two_pi * (double)q / (double)M));
            }
        if ((rc = p->alloc(&p->d_tw_n, N, "twiddles"))) return rc;
        if ((rc = p->alloc(&p->d_tw_m, tm.size(), "twiddles"))) return rc;
        SAR_CUDA(cudaMemcpy(p->d_tw_n, tn.data(), sizeof(float2) * N, cudaMemcpyHostToDevice), "twiddles");
        SAR_CUDA(cudaMemcpy(p->d_tw_m, tm.data(), sizeof(float2) * tm.size(), cudaMemcpyHostToDevice), "twiddles");
        p->fused_up = up_ok;
        p->fused_down = down_ok;
    }
    // Callback transforms (single precision): opt-in with SAR_FFT_CALLBACKS=1.  On GB300 with the
    // cuFFT of CUDA 13.0, plans with JIT (LTO) callbacks fail to build (CUFFT_INTERNAL_ERROR from
    // cufftMakePlanMany for LTO-IR of compute_90 .. compute_103a alike), so the packing kernels are
    // the default; when forced on, a plan that cannot link the callbacks reports why.
    {
        const char* env = getenv("SAR_FFT_CALLBACKS");
        const bool want = !p->fft_double && !p->block && env && env[0] == '1';
        if (want) {
            p->Lc = (int)std::min<size_t>((size_t)p->Lg + 1, M);
            cufftHandle h = 0;
            int crc = p->alloc(&p->d_cb, 1, "callback parameters");
            if (!crc) crc = p->alloc(&p->d_compact, (size_t)p->chunk * p->Lc, "compact profiles");
            if (!crc) crc = cb_plan(p, p->chunk, true, &h);
            if (!crc) crc = cb_plan(p, p->chunk, false, &h);
            if (!crc) {
                p->fft_cb = true;
            } else if (env && env[0] == '1') {
                return crc;   // forced on: report why the callbacks could not be linked
            } else {
                cudaGetLastError();
                g_last_error.clear();
            }
        }
    }
    return SAR_OK;
}

}  // namespace

extern "C" {

const char* sar_status_string(int status) {
    switch (status) {
        case SAR_OK: return "ok";
        case SAR_ERR_INVALID_ARGUMENT: return "invalid argument";
        case SAR_ERR_CUDA: return "CUDA error";
        case SAR_ERR_CUFFT: return "cuFFT error";
        case SAR_ERR_OUT_OF_MEMORY: return "out of device memory";
        case SAR_ERR_NOT_SUPPORTED: return "not supported";
        default: return "unknown status";
    }
}

size_t sar_last_error(char* buf, size_t len) {
    if (buf && len) {
        const size_t n = std::min(len - 1, g_last_error.size());
        memcpy(buf, g_last_error.data(), n);
        buf[n] = '\0';
    }
    return g_last_error.size();
}

int sar_host_device_pointer(const void* host_ptr, void** dev_ptr) {
    if (!host_ptr || !dev_ptr) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    *dev_ptr = nullptr;
    void* d = nullptr;
    const cudaError_t e = cudaHostGetDevicePointer(&d, const_cast<void*>(host_ptr), 0);
    if (e != cudaSuccess || !d) {
        cudaGetLastError();   // not addressable by the device: not an error for the caller's context
        return fail(SAR_ERR_INVALID_ARGUMENT, "host memory is not addressable by the device");
    }
    *dev_ptr = d;
    return SAR_OK;
}

static int plan_create(const sar_geometry* geom, int device, size_t block_pulses, sar_plan** plan_out);

int sar_plan_create(const sar_geometry* geom, int device, sar_plan** plan_out) {
    return plan_create(geom, device, 0, plan_out);
}

int sar_plan_create_streamed(const sar_geometry* geom, int device, size_t block_pulses, sar_plan** plan_out) {
    if (!block_pulses) return fail(SAR_ERR_INVALID_ARGUMENT, "block_pulses must be positive");
    return plan_create(geom, device, block_pulses, plan_out);
}

static int plan_create(const sar_geometry* geom, int device, size_t block_pulses, sar_plan** plan_out) {
    g_last_error.clear();
    if (!geom || !plan_out) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    *plan_out = nullptr;
    const int vrc = validate_geometry(geom);
    if (vrc != SAR_OK) return vrc;
    int dev = device;
    if (dev < 0) SAR_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    DeviceGuard guard(dev);
    if (guard.status != cudaSuccess) return cuda_fail(guard.status, "select device");
    sar_plan* p = new (std::nothrow) sar_plan();
    if (!p) return fail(SAR_ERR_OUT_OF_MEMORY, "host allocation");
    p->device = dev;
    p->block = block_pulses < geom->num_slow_times ? block_pulses : 0;
    const int rc = build_plan(geom, p);
    if (rc != SAR_OK) {
        delete p;
        return rc;
    }
    *plan_out = p;
    return SAR_OK;
}

int sar_plan_destroy(sar_plan* plan) {
    delete plan;
    return SAR_OK;
}

int sar_plan_get_info(const sar_plan* p, sar_plan_info* info) {
    if (!p || !info) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    info->working_length = p->M;
    info->profile_first_bin = p->bg0;
    info->profile_length = (size_t)p->Lg;
    info->tile_window = p->grid ? (size_t)p->wwin : 0;
    info->strip_window = (p->grid && !p->forward_points) ? (size_t)p->ws : 0;
    info->device_bytes = p->device_bytes;
    info->grid = p->grid ? 1 : 0;
    info->interp = p->interp;
    info->num_fast_times = p->N;
    info->num_slow_times = p->S;
    info->num_scatterers = p->P;
    info->device = p->device;
    info->fft_callbacks = p->fft_cb ? 1 : 0;
    info->gather_lanes_y = p->lanes_y;
    info->fused_upsampling = p->fused_up ? 1 : 0;
    info->fused_downsampling = p->fused_down ? 1 : 0;
    info->scatter_lanes_y = (p->grid && !p->forward_points && p->fwd_transposed) ? 1 : 0;
    info->scatter_shear = (p->grid && !p->forward_points) ? p->gc_fwd.shear : 0;
    info->gather_shear = p->grid ? p->gather_shear : 0;
    info->scatter_ring_half = (p->grid && !p->forward_points) ? p->ring_half : 0;
    info->block_pulses = p->block;
    return SAR_OK;
}

// Stored profile format of a plan (the upsampling writers' `linear` argument).
static int prof_format(const sar_plan* p) {
    return p->values ? kProfValues : p->interp == SAR_INTERP_LINEAR ? kProfLinearPairs : kProfNearestPairs;
}

// Upsampled profiles of pulses [begin, end): y row s is read at y + s * N; with pairs_out the
// (value, difference) pairs of pulse s go to pairs_rows + s * Lg (the plan's buffer for a resident
// plan; a ring slot, addressed from the block's first pulse, for a streamed one).
static int upsample_rows(sar_plan* p, const float2* y, size_t begin, size_t end, cudaStream_t st, bool pairs_out,
                         float2* prof, float4* pairs_rows = nullptr) {
    if (!pairs_rows) pairs_rows = p->d_prof;
    for (size_t first = begin; first < end; first += (size_t)p->chunk) {
        const int rows = (int)std::min<size_t>(p->chunk, end - first);
        const int dbl = p->fft_double;
        if (pairs_out && p->fused_up) {
            SAR_CUDA(launch_upsample_pairs_fused(y, p->d_wave, p->d_wadj, p->d_tw_n, p->d_tw_m, pairs_rows, (int)p->N,
                                                 (long)p->M, p->Lg, p->bg0, rows, (int)first, prof_format(p), st),
                     "fused upsampling");
            continue;
        }
        if (p->fft_cb) {
            cufftHandle h = 0;
            int rc = cb_plan(p, rows, true, &h);
            if (rc) return rc;
            if ((rc = set_cb_info(p, y, nullptr, (int)first, st))) return rc;
            SAR_CUFFT(cufftSetStream(h, st), "cufftSetStream");
            SAR_CUFFT(cufftExecC2C(h, reinterpret_cast<cufftComplex*>(p->d_spec), reinterpret_cast<cufftComplex*>(p->d_spec),
                                   CUFFT_INVERSE),
                      "cufftExecC2C (callbacks)");
            SAR_CUDA(launch_unpack_compact(p->d_compact, p->Lc, p->d_wadj, pairs_out ? p->d_prof : nullptr,
                                           pairs_out ? nullptr : prof, (long)p->M, p->Lg, rows, (int)first,
                                           prof_format(p), st),
                     "unpack");
            continue;
        }
        SAR_CUDA(launch_pack_adjoint(y, p->d_wave, p->d_spec, dbl, (int)p->N, (long)p->M, rows, (int)first, st), "pack");
        int rc = run_fft(p, p->d_spec, rows, CUFFT_INVERSE, st);
        if (rc) return rc;
        if (pairs_out)
            SAR_CUDA(launch_unpack_pairs(p->d_spec, dbl, p->d_wadj, pairs_rows, (long)p->M, p->Lg, p->bg0, rows,
                                         (int)first, prof_format(p), st),
                     "unpack");
        else
            SAR_CUDA(launch_unpack_profiles(p->d_spec, dbl, prof, (long)p->M, p->Lg, p->bg0, rows, (int)first, st),
                     "unpack");
    }
    return SAR_OK;
}

static int upsample_into_pairs(sar_plan* p, const float2* y, cudaStream_t st, bool pairs_out, float2* prof) {
    return upsample_rows(p, y, 0, p->S, st, pairs_out, prof);
}

static PointArgs point_args(sar_plan* p, int bin_rule) {
    PointArgs a;
    a.pulses = p->d_pulses;
    a.alpha2 = p->d_alpha2;
    a.points = p->d_points;
    a.kappa = p->kappa;
    a.s_r = p->s_r;
    a.bin_rule = bin_rule;
    a.S = (int)p->S;
    a.P = (int)p->P;
    a.Lg = p->Lg;
    a.bg0 = (int)p->bg0;
    a.linear = p->interp == SAR_INTERP_LINEAR;
    a.flags = p->d_flags;
    a.values = p->values ? 1 : 0;
    return a;
}

// Grid gather of pulses [first, first + count) from pairs rows `pairs` (row 0 = pulse `first`).
static int gather_pulses(sar_plan* p, const float4* pairs, size_t first, size_t count, float2* x, int accumulate,
                         cudaStream_t st) {
    BpGridArgs a;
    a.g = p->gc_adj;
    a.pulses = p->d_pulses + first;
    a.pairs = pairs;
    a.x = x;
    a.flags = p->d_flags;
    a.S = (int)count;
    a.Lg = p->Lg;
    a.bg0 = (int)p->bg0;
    a.wwin = p->wwin;
    a.pb = p->pb;
    a.staged = p->staged;
    a.accumulate = accumulate ? 1 : 0;
    a.lanes_y = p->lanes_y;
    a.nearest = p->interp == SAR_INTERP_NEAREST_REF;
    a.values = p->values ? 1 : 0;
    a.steps = p->d_steps;
    a.alpha2 = p->d_alpha2 ? p->d_alpha2 + first : nullptr;   // indexed by block-relative pulse
    a.wait_budget = p->wait_budget;
    a.hold_first_stage = p->hold_first_stage;
    a.tiles_valid = p->tiles_valid;
    SAR_CUDA(p->staged ? launch_bp_grid_ws(a, st) : launch_bp_grid(a, st), "backprojection");
    return SAR_OK;
}

// Ring slot of a streamed plan for the block starting at pulse `first`.
// `rows` profile rows after `base`: rows of Lg 16-byte pairs, or of Lg plain 8-byte values for
// plans that store values (may point before the buffer when the callee only touches rows from
// the block's first pulse on).
static float4* prof_rows(const sar_plan* p, float4* base, long rows) {
    const long bytes = rows * (long)p->Lg * (p->values ? 8 : 16);
    return reinterpret_cast<float4*>(reinterpret_cast<char*>(base) + bytes);
}

static float4* ring_slot(sar_plan* p, size_t first) {
    return prof_rows(p, p->d_prof, (long)(((first / p->block) & 1) * p->block));
}

int sar_adjoint(sar_plan* p, const void* y_dev, void* x_dev, void* stream) {
    if (!p || !y_dev || !x_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(p->mu);
    DeviceGuard guard(p->device);
    if (guard.status != cudaSuccess) return cuda_fail(guard.status, "select device");
    cudaStream_t st = (cudaStream_t)stream;
    p->last_stream = st;
    cudaEvent_t* ev = p->timing_slot();
    if (p->block) {
        // streamed plan: per block of pulses, upsample into a ring slot and gather, adding the
        // blocks after the first onto the image (stage times: upsampling in [0], gathers in [1])
        mark(ev, 0, st);
        mark(ev, 1, st);
        for (size_t first = 0; first < p->S; first += p->block) {
            const size_t count = std::min(p->block, p->S - first);
            float4* slot = ring_slot(p, first);
            int rc = upsample_rows(p, (const float2*)y_dev, first, first + count, st, true, nullptr,
                                   prof_rows(p, slot, -(long)first));
            if (rc) return rc;
            if ((rc = gather_pulses(p, slot, first, count, (float2*)x_dev, first > 0, st))) return rc;
        }
        mark(ev, 2, st);
        mark(ev, 3, st);
        return SAR_OK;
    }
    mark(ev, 0, st);
    int rc = upsample_into_pairs(p, (const float2*)y_dev, st, true, nullptr);
    if (rc) return rc;
    mark(ev, 1, st);
    if (p->grid) {
        if ((rc = gather_pulses(p, p->d_prof, 0, p->S, (float2*)x_dev, 0, st))) return rc;
    } else {
        SAR_CUDA(launch_bp_points(point_args(p, p->interp == SAR_INTERP_LINEAR ? BIN_LINEAR : BIN_ADJ_NEAREST), p->d_prof, (float2*)x_dev, 0, st),
                 "backprojection");
    }
    mark(ev, 2, st);
    mark(ev, 3, st);
    return SAR_OK;
}

// Grid scatter of pulses [first, first + count) into accumulator rows `acc` (row 0 = pulse `first`).
static int scatter_pulses(sar_plan* p, const float2* x, float2* acc, size_t first, size_t count, cudaStream_t st) {
    FpGridArgs a;
    a.g = p->gc_fwd;
    a.pulses = p->d_pulses + first;
    a.x = x;
    a.acc = acc;
    a.strip_start = p->d_strip + first;
    a.strip_stride = (int)p->S;
    a.flags = p->d_flags;
    a.S = (int)count;
    a.Lg = p->Lg;
    a.bg0 = (int)p->bg0;
    a.seg_tiles = p->seg_tiles;
    a.segs_per_column = p->segs_per_column;
    a.ws = p->ws;
    a.ring_half = p->ring_half;
    a.pbf = p->pbf;
    a.linear = p->interp == SAR_INTERP_LINEAR;
    // the scatter walks the axis along which bins change slowly: the transpose of the gather's
    // lane choice, or the rows of a sheared lattice
    a.transposed = p->fwd_transposed ? 1 : 0;
    a.steps = p->d_steps;
    a.alpha2 = p->d_alpha2 ? p->d_alpha2 + first : nullptr;
    SAR_CUDA(launch_fp_grid_ws(a, st), "forward scatter");
    return SAR_OK;
}

// FFT side of the forward projection for pulses [begin, end): accumulator row of pulse s at
// acc_rows + s * Lg, output rows of y.
static int downsample_rows(sar_plan* p, const float2* acc_rows, float2* y, size_t begin, size_t end,
                           cudaStream_t st) {
    for (size_t first = begin; first < end; first += (size_t)p->chunk) {
        const int rows = (int)std::min<size_t>(p->chunk, end - first);
        if (p->fused_down) {
            SAR_CUDA(launch_downsample_forward_fused(acc_rows, p->d_wave, p->d_wfwd, p->d_tw_n, p->d_tw_m, y,
                                                     (int)p->N, (long)p->M, p->Lg, p->bg0, rows, (int)first, st),
                     "fused downsampling");
            continue;
        }
        if (p->fft_cb) {
            cufftHandle h = 0;
            int rc = cb_plan(p, rows, false, &h);
            if (rc) return rc;
            if ((rc = set_cb_info(p, nullptr, y, (int)first, st))) return rc;
            SAR_CUFFT(cufftSetStream(h, st), "cufftSetStream");
            SAR_CUFFT(cufftExecC2C(h, reinterpret_cast<cufftComplex*>(p->d_spec), reinterpret_cast<cufftComplex*>(p->d_spec),
                                   CUFFT_FORWARD),
                      "cufftExecC2C (callbacks)");
            continue;
        }
        SAR_CUDA(launch_pack_forward(acc_rows, p->d_spec, p->fft_double, (long)p->M, p->Lg, p->bg0, rows, (int)first,
                                     st),
                 "pack");
        int rc = run_fft(p, p->d_spec, rows, CUFFT_FORWARD, st);
        if (rc) return rc;
        SAR_CUDA(launch_extract_forward(p->d_spec, p->fft_double, p->d_wave, p->d_wfwd, y, (int)p->N, (long)p->M, rows,
                                        (int)first, st),
                 "extract");
    }
    return SAR_OK;
}

int sar_forward(sar_plan* p, const void* x_dev, void* y_dev, void* stream) {
    if (!p || !y_dev || !x_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(p->mu);
    DeviceGuard guard(p->device);
    if (guard.status != cudaSuccess) return cuda_fail(guard.status, "select device");
    cudaStream_t st = (cudaStream_t)stream;
    p->last_stream = st;
    cudaEvent_t* ev = p->timing_slot();
    if (p->block) {
        // streamed plan: per block, clear its accumulator (half of a ring slot), scatter the block's
        // pulses, downsample its rows (stage times: the whole loop in [1])
        mark(ev, 0, st);
        mark(ev, 1, st);
        for (size_t first = 0; first < p->S; first += p->block) {
            const size_t count = std::min(p->block, p->S - first);
            float2* acc = reinterpret_cast<float2*>(ring_slot(p, first));
            SAR_CUDA(cudaMemsetAsync(acc, 0, sizeof(float2) * count * (size_t)p->Lg, st), "zero accumulator");
            int rc = scatter_pulses(p, (const float2*)x_dev, acc, first, count, st);
            if (!rc) rc = downsample_rows(p, acc - first * (size_t)p->Lg, (float2*)y_dev, first, first + count, st);
            if (rc) return rc;
        }
        mark(ev, 2, st);
        mark(ev, 3, st);
        return SAR_OK;
    }
    float2* acc = reinterpret_cast<float2*>(p->d_prof);
    mark(ev, 0, st);
    SAR_CUDA(cudaMemsetAsync(acc, 0, sizeof(float2) * p->S * (size_t)p->Lg, st), "zero accumulator");
    mark(ev, 1, st);
    if (p->grid && !p->forward_points) {
        int rc = scatter_pulses(p, (const float2*)x_dev, acc, 0, p->S, st);
        if (rc) return rc;
    } else {
        SAR_CUDA(launch_fp_points(point_args(p, p->interp == SAR_INTERP_LINEAR ? BIN_LINEAR : BIN_FWD_NEAREST), (const float2*)x_dev, acc, st),
                 "forward scatter");
    }
    mark(ev, 2, st);
    int rc = downsample_rows(p, acc, (float2*)y_dev, 0, p->S, st);
    if (rc) return rc;
    mark(ev, 3, st);
    return SAR_OK;
}

int sar_adjoint_pulse_block(sar_plan* p, const void* y_block_dev, size_t first_pulse, size_t count, void* x_dev,
                            int accumulate, void* stream) {
    if (!p || !y_block_dev || !x_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    if (!count || first_pulse >= p->S || count > p->S - first_pulse)
        return fail(SAR_ERR_INVALID_ARGUMENT, "pulse block [%zu, %zu) outside [0, %zu)", first_pulse,
                    first_pulse + count, p->S);
    if (!p->grid) return fail(SAR_ERR_NOT_SUPPORTED, "pulse blocks need a regular-grid plan");
    if (p->block && count > p->block)
        return fail(SAR_ERR_INVALID_ARGUMENT, "a streamed plan takes pulse blocks of at most %zu pulses", p->block);
    std::lock_guard<std::mutex> lock(p->mu);
    DeviceGuard guard(p->device);
    if (guard.status != cudaSuccess) return cuda_fail(guard.status, "select device");
    cudaStream_t st = (cudaStream_t)stream;
    p->last_stream = st;
    // The block holds rows first_pulse .. first_pulse + count - 1; the upsampling addresses row s
    // at y + s * N, so the base is moved back by first_pulse rows (only rows of the block are read).
    const float2* y = reinterpret_cast<const float2*>(y_block_dev) - first_pulse * p->N;
    // profile pairs: the resident buffer's rows of these pulses, or the streamed plan's ring slot
    float4* pairs = p->block ? ring_slot(p, first_pulse) : prof_rows(p, p->d_prof, (long)first_pulse);
    int rc = upsample_rows(p, y, first_pulse, first_pulse + count, st, true, nullptr,
                           prof_rows(p, pairs, -(long)first_pulse));
    if (rc) return rc;
    return gather_pulses(p, pairs, first_pulse, count, (float2*)x_dev, accumulate, st);
}

int sar_profiles(sar_plan* p, const void* y_dev, void* prof_dev, void* stream) {
    if (!p || !y_dev || !prof_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(p->mu);
    DeviceGuard guard(p->device);
    if (guard.status != cudaSuccess) return cuda_fail(guard.status, "select device");
    p->last_stream = (cudaStream_t)stream;
    return upsample_into_pairs(p, (const float2*)y_dev, (cudaStream_t)stream, false, (float2*)prof_dev);
}

int sar_set_slow_time_weighting(sar_plan* p, const double* w) {
    if (!p || !w) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(p->mu);
    DeviceGuard guard(p->device);
    for (size_t s = 0; s < p->S; ++s) p->weights[s] = std::complex<double>(w[2 * s], w[2 * s + 1]);
    if (p->last_stream) SAR_CUDA(cudaStreamSynchronize(p->last_stream), "synchronise");
    return upload_weights(p, nullptr, true);
}

int sar_set_slow_time_weighting_device(sar_plan* p, const void* w_dev, void* stream) {
    if (!p || !w_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(p->mu);
    DeviceGuard guard(p->device);
    cudaStream_t st = (cudaStream_t)stream;
    p->last_stream = st;
    SAR_CUDA(launch_weights((const float2*)w_dev, p->d_wadj, p->d_wfwd, (int)p->S, p->interp == SAR_INTERP_LINEAR, st),
             "weights kernel");
    return SAR_OK;
}

int sar_phase_gradient(const void* ag_dev, const void* y_dev, void* g_dev, size_t num_slow_times,
                       size_t num_fast_times, float scale, void* stream) {
    if (!ag_dev || !y_dev || !g_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    if (!num_slow_times || !num_fast_times || num_slow_times > (size_t)1 << 31 || num_fast_times > (size_t)1 << 30)
        return fail(SAR_ERR_INVALID_ARGUMENT, "bad sizes");
    SAR_CUDA(launch_phase_grad((const float2*)ag_dev, (const float2*)y_dev, (float*)g_dev, (int)num_slow_times,
                               (int)num_fast_times, scale, (cudaStream_t)stream),
             "phase gradient");
    return SAR_OK;
}

int sar_sharpness(const void* img_dev, void* g_dev, double* sum_dev, size_t num_pixels, void* stream) {
    if (!img_dev || !sum_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    if (((uintptr_t)img_dev & 15) || ((uintptr_t)g_dev & 15))
        return fail(SAR_ERR_INVALID_ARGUMENT, "image buffers must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    SAR_CUDA(cudaGetDevice(&dev), "get device");
    SAR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    SAR_CUDA(cudaMemsetAsync(sum_dev, 0, sizeof(double), st), "clear sum");
    if (!num_pixels) return SAR_OK;
    SAR_CUDA(launch_sharpness((const float2*)img_dev, (float2*)g_dev, sum_dev, num_pixels, sms, st), "sharpness");
    return SAR_OK;
}

int sar_enable_stage_timing(sar_plan* p, int enable) {
    if (!p) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(p->mu);
    p->timing = enable != 0;
    p->events_used = 0;
    return SAR_OK;
}

int sar_stage_times(sar_plan* p, float* ms, int* calls) {
    if (!p || !ms || !calls) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(p->mu);
    DeviceGuard guard(p->device);
    ms[0] = ms[1] = ms[2] = 0.0f;
    for (size_t c = 0; c < p->events_used; ++c) {
        auto& ev = p->events[c];
        SAR_CUDA(cudaEventSynchronize(ev[3]), "stage timing");
        for (int i = 0; i < 3; ++i) {
            float t = 0.0f;
            SAR_CUDA(cudaEventElapsedTime(&t, ev[i], ev[i + 1]), "stage timing");
            ms[i] += t;
        }
    }
    *calls = (int)p->events_used;
    return SAR_OK;
}

int sar_plan_set_wait_budget(sar_plan* p, long long cycles, int hold_first_stage) {
    if (!p) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    if (cycles < 0) return fail(SAR_ERR_INVALID_ARGUMENT, "negative wait budget");
    std::lock_guard<std::mutex> lock(p->mu);
    p->wait_budget = cycles ? cycles : kDefaultWaitBudgetCycles;
    p->hold_first_stage = hold_first_stage ? 1 : 0;
    return SAR_OK;
}

int sar_device_flags(sar_plan* p, unsigned* flags) {
    if (!p || !flags) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(p->mu);
    DeviceGuard guard(p->device);
    if (p->last_stream) SAR_CUDA(cudaStreamSynchronize(p->last_stream), "synchronise");
    SAR_CUDA(cudaMemcpy(flags, p->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost), "read flags");
    SAR_CUDA(cudaMemset(p->d_flags, 0, sizeof(unsigned)), "clear flags");
    return SAR_OK;
}

// ------------------------------------------------------------ drop-in boundary
static void geometry_from_info(const SarCalculationInfo* info, sar_geometry* g) {
    memset(g, 0, sizeof(*g));
    g->num_fast_times = info->num_fast_times;
    g->num_slow_times = info->num_slow_times;
    g->num_scatterers = info->num_scatterers;
    g->transmit_posns = info->transmit_posns;
    g->receive_posns = info->receive_posns;
    g->stab_ref_posns = info->stab_ref_posns;
    g->scat_posns = info->scat_posns;
    g->waveform_fft = info->waveform_fft;
    g->slow_time_weighting = info->slow_time_weighting;
    g->centre_frequency = info->centre_frequency;
    g->sample_frequency = info->sample_frequency;
    g->c_eff = info->c_eff;
    g->upsample_ratio = info->upsample_ratio;
    g->sign_multiplier = info->sign_multiplier;
    g->interp = SAR_INTERP_NEAREST_REF;
}

// One synchronous operator application on host FP64 buffers (FFT-ordered phase history).
static int dropin_run(SarCalculationInfo* info, bool forward) {
    if (!info) return fail(SAR_ERR_INVALID_ARGUMENT, "null SarCalculationInfo");
    if (!info->phase_history || !info->scattering_amplitudes)
        return fail(SAR_ERR_INVALID_ARGUMENT, "null phase_history or scattering_amplitudes");
    const size_t N = info->num_fast_times, S = info->num_slow_times, P = info->num_scatterers;
    // Zero the output first, like setup_{forward,adjoint}_evaluate (sarsolver_cxx.cpp:264-269, :312-317).
    if (forward)
        memset(info->phase_history, 0, sizeof(double) * 2 * N * S);
    else
        memset(info->scattering_amplitudes, 0, sizeof(double) * 2 * P);
    sar_geometry g;
    geometry_from_info(info, &g);
    sar_plan* plan = nullptr;
    int rc = sar_plan_create(&g, -1, &plan);
    if (rc) return rc;
    const int half = (int)(N / 2);
    std::vector<float2> hx(P), hy(N * S);
    float2 *dx = nullptr, *dy = nullptr;
    cudaError_t e = cudaMalloc((void**)&dx, sizeof(float2) * P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dy, sizeof(float2) * N * S);
    if (e == cudaSuccess) {
        if (forward) {
            for (size_t p = 0; p < P; ++p)
                hx[p] = make_float2((float)info->scattering_amplitudes[2 * p], (float)info->scattering_amplitudes[2 * p + 1]);
            e = cudaMemcpy(dx, hx.data(), sizeof(float2) * P, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) rc = sar_forward(plan, dx, dy, nullptr);
            if (e == cudaSuccess && !rc) e = cudaMemcpy(hy.data(), dy, sizeof(float2) * N * S, cudaMemcpyDeviceToHost);
            if (e == cudaSuccess && !rc)
                for (size_t s = 0; s < S; ++s)
                    for (size_t i = 0; i < N; ++i) {   // device layout is fftshifted; the struct holds FFT order
                        const float2 v = hy[s * N + (i + half) % N];
                        info->phase_history[2 * (s * N + i)] = v.x;
                        info->phase_history[2 * (s * N + i) + 1] = v.y;
                    }
        } else {
            for (size_t s = 0; s < S; ++s)
                for (size_t i = 0; i < N; ++i)
                    hy[s * N + (i + half) % N] = make_float2((float)info->phase_history[2 * (s * N + i)],
                                                             (float)info->phase_history[2 * (s * N + i) + 1]);
            e = cudaMemcpy(dy, hy.data(), sizeof(float2) * N * S, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) rc = sar_adjoint(plan, dy, dx, nullptr);
            if (e == cudaSuccess && !rc) e = cudaMemcpy(hx.data(), dx, sizeof(float2) * P, cudaMemcpyDeviceToHost);
            if (e == cudaSuccess && !rc)
                for (size_t p = 0; p < P; ++p) {
                    info->scattering_amplitudes[2 * p] = hx[p].x;
                    info->scattering_amplitudes[2 * p + 1] = hx[p].y;
                }
        }
    }
    cudaFree(dx);
    cudaFree(dy);
    sar_plan_destroy(plan);
    if (e != cudaSuccess) return cuda_fail(e, forward ? "forward_evaluate" : "adjoint_evaluate");
    return rc;
}

void forward_evaluate(SarCalculationInfo* info) { dropin_run(info, true); }
void adjoint_evaluate(SarCalculationInfo* info) { dropin_run(info, false); }

}  // extern "C"
