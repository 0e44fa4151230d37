// sar_resample.cu -- dataset resampling on the GPU: SRP phase ramps, fast-frequency downsampling
// and the slow-time downsampling filter (sar_move_srps, sar_fast_freq_downsample,
// sar_resample_phase_history in include/sargpu.h).
//
// Follows the reference's utilities and resampling loop (src/sarsolver/utils/geodesy.py:33-73,
// utils/signal.py:45-77, numpy/measurement.py:342-458), restructured for the device: every old
// pulse is rephased and downsampled once (the reference redoes both for each window a pulse falls
// in), then each output pulse is one weighted sum over its window of rows.
//   rephase:   ph[s][f] * exp(2 pi i (dR_s / c) (bb_f - sign fc)),  bb_f = (f - N/2) fs / N
//              (phase in turns from a per-pulse constant reduced in FP64 on the host plus an
//              error-free split product for the per-bin slope, so the phase stays exact to
//              ~1e-7 turns at hundreds of turns per pulse)
//   downsample: ifftshift, inverse FFT / N, keep the n/2 lowest and n - n/2 highest modes times
//              the fftshifted Tukey window, forward FFT, fftshift
//   filter:    out[t][f] = sum_k kernel[k] X[row0[t] + k][f]
// All memory-bound: each pass reads and writes the rows once; the FFTs are cuFFT.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/sargpu.h"
#include "sar_kernels.cuh"

namespace {

int err(int code, const char* msg) {
    sar::sar_internal_set_error(msg);
    return code;
}
int cuda_err(cudaError_t e, const char* what) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return err(e == cudaErrorMemoryAllocation ? SAR_ERR_OUT_OF_MEMORY : SAR_ERR_CUDA, buf);
}
#define R_CUDA(call, what)                                 \
    do {                                                   \
        cudaError_t _e = (call);                           \
        if (_e != cudaSuccess) return cuda_err(_e, what);  \
    } while (0)
#define R_CALL(call)          \
    do {                      \
        int _rc = (call);     \
        if (_rc) return _rc;  \
    } while (0)

unsigned blocks_for(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 65535u * 8); }

// out[s][j] = in[s][(j + shift_in) % N] * exp(2 pi i phase(s, f)) * scale, where f is the natural
// (fftshifted) frequency index of the value read and phase = b_s + a_s f in turns.  coef[s] =
// (b_s, a_hi_s, a_lo_s, unused); a_hi * f is formed with its exact FMA remainder.
__global__ void rephase_kernel(const float2* __restrict__ in, float2* __restrict__ out, const float4* __restrict__ coef,
                               int S, int N, int shift_in, float scale) {
    const size_t total = (size_t)S * N;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int s = (int)(e / N), j = (int)(e % N);
        int f = j + shift_in;
        if (f >= N) f -= N;
        const float2 v = in[(size_t)s * N + f];
        float2 r = v;
        if (coef) {
            const float4 c = __ldg(coef + s);
            const float ff = (float)f;
            const float p = c.y * ff;
            const float pe = fmaf(c.y, ff, -p);          // exact remainder of the product
            float t = (p - rintf(p)) + pe + c.z * ff + c.x;
            t -= rintf(t);
            float sn, cs;
            sincospif(2.0f * t, &sn, &cs);
            r = make_float2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
        }
        out[e] = make_float2(r.x * scale, r.y * scale);
    }
}

// dst[s][j] = window[j] * src[s][j < lo ? j : N - (n - j)]  (modes kept by the downsampling).
__global__ void crop_window_kernel(const float2* __restrict__ src, float2* __restrict__ dst, const float* __restrict__ window,
                                   int S, int N, int n) {
    const int lo = n / 2;
    const size_t total = (size_t)S * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int s = (int)(e / n), j = (int)(e % n);
        const int k = j < lo ? j : N - (n - j);
        const float2 v = src[(size_t)s * N + k];
        const float w = __ldg(window + j);
        dst[e] = make_float2(w * v.x, w * v.y);
    }
}

// out[t][i] = sum_k kern[k] X[row0[t] + k][(i + shift) % n]   (shift = (n + 1) / 2: fftshift).
__global__ void slow_filter_kernel(const float2* __restrict__ X, float2* __restrict__ out, const float2* __restrict__ kern,
                                   int L, const int* __restrict__ row0, int T, int n, int shift) {
    const size_t total = (size_t)T * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int t = (int)(e / n), i = (int)(e % n);
        int f = i + shift;
        if (f >= n) f -= n;
        const float2* x = X + (size_t)__ldg(row0 + t) * n + f;
        float re = 0.f, im = 0.f;
        for (int k = 0; k < L; ++k) {
            const float2 c = __ldg(kern + k), v = x[(size_t)k * n];
            re = fmaf(c.x, v.x, fmaf(-c.y, v.y, re));
            im = fmaf(c.x, v.y, fmaf(c.y, v.x, im));
        }
        out[e] = make_float2(re, im);
    }
}

// Per-pulse phase coefficients in turns: phase(s, f) = b_s + a_s f with a_s = dR_s fs / (c N)
// and b_s = frac(dR_s (-(N/2) fs / N - sign fc) / c), reduced in FP64; a_s is passed as an FP32
// head and tail (the kernel forms head * f with its exact FMA remainder).
std::vector<float4> phase_coefficients(const double* dr, size_t S, size_t N, double fc, double fs, double sign,
                                       double c_eff) {
    std::vector<float4> co(S);
    for (size_t s = 0; s < S; ++s) {
        const double a = dr[s] * fs / (c_eff * (double)N);
        double b = dr[s] * (-(double)(N / 2) * fs / (double)N - sign * fc) / c_eff;
        b -= std::nearbyint(b);
        const float a_hi = (float)a;
        const float a_lo = (float)(a - (double)a_hi);
        co[s] = make_float4((float)b, a_hi, a_lo, 0.f);
    }
    return co;
}

struct DevBuf {
    void* p = nullptr;
    cudaStream_t st = nullptr;
    ~DevBuf() {
        if (p) cudaFreeAsync(p, st);
    }
};

// Batched C2C plans by (device, length, rows), made on first use and kept for the process (plan
// creation costs milliseconds; resampling jobs repeat the same shapes).  Calls on one plan are
// serialised by the stream they run on; the cache itself is guarded by a mutex.
std::mutex g_plan_mu;
std::map<std::tuple<int, int, int>, cufftHandle> g_plans;

int fft_rows(void* data, int n, int rows, int direction, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    cufftHandle h = 0;
    {
        std::lock_guard<std::mutex> lock(g_plan_mu);
        auto key = std::make_tuple(dev, n, rows);
        auto it = g_plans.find(key);
        if (it != g_plans.end()) {
            h = it->second;
        } else {
            int dims[1] = {n};
            if (cufftPlanMany(&h, 1, dims, nullptr, 1, n, nullptr, 1, n, CUFFT_C2C, rows) != CUFFT_SUCCESS)
                return err(SAR_ERR_CUFFT, "resampling FFT plan");
            g_plans[key] = h;
        }
    }
    cufftResult r = cufftSetStream(h, st);
    if (r == CUFFT_SUCCESS)
        r = cufftExecC2C(h, (cufftComplex*)data, (cufftComplex*)data, direction);
    if (r != CUFFT_SUCCESS) return err(SAR_ERR_CUFFT, "resampling FFT");
    return SAR_OK;
}

// Rephase (optional) and downsample S rows of N into S rows of n in FFT order (no output shift).
int downsample_rows(const float2* ph, size_t S, size_t N, const float4* d_coef, size_t n, const float* d_window,
                    float2* out, cudaStream_t st) {
    DevBuf spec;
    spec.st = st;
    R_CUDA(cudaMallocAsync(&spec.p, sizeof(float2) * S * N, st), "resampling work rows");
    float2* sp = (float2*)spec.p;
    // ifftshift: FFT-order index j reads natural index (j + N/2) mod N; 1/N is numpy's ifft scale.
    rephase_kernel<<<blocks_for(S * N), 256, 0, st>>>(ph, sp, d_coef, (int)S, (int)N, (int)(N / 2), 1.0f / (float)N);
    R_CUDA(cudaGetLastError(), "rephase");
    R_CALL(fft_rows(sp, (int)N, (int)S, CUFFT_INVERSE, st));
    crop_window_kernel<<<blocks_for(S * n), 256, 0, st>>>(sp, out, d_window, (int)S, (int)N, (int)n);
    R_CUDA(cudaGetLastError(), "crop");
    return fft_rows(out, (int)n, (int)S, CUFFT_FORWARD, st);
}

int check_sizes(size_t S, size_t N) {
    if (!S || !N || S > ((size_t)1 << 30) || N > ((size_t)1 << 28) || S * N > ((size_t)1 << 34))
        return err(SAR_ERR_INVALID_ARGUMENT, "bad phase history shape");
    return SAR_OK;
}

}  // namespace

extern "C" int sar_move_srps(const void* ph_dev, void* out_dev, size_t S, size_t N, const double* delta_range,
                             double centre_freq, double sample_bandwidth, double sign_multiplier, double c_eff,
                             void* stream) {
    if (!ph_dev || !out_dev || !delta_range) return err(SAR_ERR_INVALID_ARGUMENT, "null argument");
    R_CALL(check_sizes(S, N));
    cudaStream_t st = (cudaStream_t)stream;
    const std::vector<float4> co = phase_coefficients(delta_range, S, N, centre_freq, sample_bandwidth, sign_multiplier, c_eff);
    DevBuf dc;
    dc.st = st;
    R_CUDA(cudaMallocAsync(&dc.p, sizeof(float4) * S, st), "phase coefficients");
    R_CUDA(cudaMemcpyAsync(dc.p, co.data(), sizeof(float4) * S, cudaMemcpyHostToDevice, st), "phase coefficients");
    rephase_kernel<<<blocks_for(S * N), 256, 0, st>>>((const float2*)ph_dev, (float2*)out_dev, (const float4*)dc.p, (int)S,
                                                     (int)N, 0, 1.0f);
    R_CUDA(cudaGetLastError(), "rephase");
    R_CUDA(cudaStreamSynchronize(st), "rephase");   // host coefficient array goes out of scope
    return SAR_OK;
}

extern "C" int sar_fast_freq_downsample(const void* ph_dev, void* out_dev, size_t S, size_t N, size_t new_N,
                                        const double* window, void* stream) {
    if (!ph_dev || !out_dev || !window) return err(SAR_ERR_INVALID_ARGUMENT, "null argument");
    R_CALL(check_sizes(S, N));
    // new_N > N keeps overlapping modes, as the reference's slicing does; beyond 2 N no mode is left
    if (!new_N || new_N > 2 * N) return err(SAR_ERR_INVALID_ARGUMENT, "new_N must be in [1, 2 N]");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<float> w(window, window + new_N);
    DevBuf dw, tmp;
    dw.st = tmp.st = st;
    R_CUDA(cudaMallocAsync(&dw.p, sizeof(float) * new_N, st), "window");
    R_CUDA(cudaMemcpyAsync(dw.p, w.data(), sizeof(float) * new_N, cudaMemcpyHostToDevice, st), "window");
    R_CUDA(cudaMallocAsync(&tmp.p, sizeof(float2) * S * new_N, st), "downsampled rows");
    R_CALL(downsample_rows((const float2*)ph_dev, S, N, nullptr, new_N, (const float*)dw.p, (float2*)tmp.p, st));
    // fftshift into the output: identity filter with one tap
    std::vector<int> rows(S);
    for (size_t s = 0; s < S; ++s) rows[s] = (int)s;
    DevBuf dr, dk;
    dr.st = dk.st = st;
    const float2 one = make_float2(1.f, 0.f);
    R_CUDA(cudaMallocAsync(&dr.p, sizeof(int) * S, st), "rows");
    R_CUDA(cudaMemcpyAsync(dr.p, rows.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st), "rows");
    R_CUDA(cudaMallocAsync(&dk.p, sizeof(float2), st), "kernel");
    R_CUDA(cudaMemcpyAsync(dk.p, &one, sizeof(float2), cudaMemcpyHostToDevice, st), "kernel");
    slow_filter_kernel<<<blocks_for(S * new_N), 256, 0, st>>>((const float2*)tmp.p, (float2*)out_dev, (const float2*)dk.p, 1,
                                                             (const int*)dr.p, (int)S, (int)new_N, (int)((new_N + 1) / 2));
    R_CUDA(cudaGetLastError(), "fftshift");
    R_CUDA(cudaStreamSynchronize(st), "fast_freq_downsample");
    return SAR_OK;
}

extern "C" int sar_resample_phase_history(const void* ph_dev, size_t S, size_t N, const double* delta_range,
                                          double centre_freq, double sample_bandwidth, double sign_multiplier,
                                          double c_eff, size_t new_N, const double* window, const double* kernel,
                                          size_t kernel_length, const int* row0, size_t num_rows, void* out_dev,
                                          void* stream) {
    if (!ph_dev || !out_dev || !window || !kernel || !row0) return err(SAR_ERR_INVALID_ARGUMENT, "null argument");
    R_CALL(check_sizes(S, N));
    if (!new_N || new_N > N) return err(SAR_ERR_INVALID_ARGUMENT, "new_N must be in [1, N]");
    if (!kernel_length || kernel_length > S) return err(SAR_ERR_INVALID_ARGUMENT, "bad kernel length");
    for (size_t t = 0; t < num_rows; ++t)
        if (row0[t] < 0 || (size_t)row0[t] + kernel_length > S) return err(SAR_ERR_INVALID_ARGUMENT, "window outside the pulses");
    if (!num_rows) return SAR_OK;
    cudaStream_t st = (cudaStream_t)stream;
    DevBuf dc, dw, dk, drow, tmp;
    dc.st = dw.st = dk.st = drow.st = tmp.st = st;
    const float4* d_coef = nullptr;
    std::vector<float4> co;
    if (delta_range) {
        co = phase_coefficients(delta_range, S, N, centre_freq, sample_bandwidth, sign_multiplier, c_eff);
        R_CUDA(cudaMallocAsync(&dc.p, sizeof(float4) * S, st), "phase coefficients");
        R_CUDA(cudaMemcpyAsync(dc.p, co.data(), sizeof(float4) * S, cudaMemcpyHostToDevice, st), "phase coefficients");
        d_coef = (const float4*)dc.p;
    }
    std::vector<float> w(window, window + new_N);
    std::vector<float2> k(kernel_length);
    for (size_t i = 0; i < kernel_length; ++i) k[i] = make_float2((float)kernel[2 * i], (float)kernel[2 * i + 1]);
    R_CUDA(cudaMallocAsync(&dw.p, sizeof(float) * new_N, st), "window");
    R_CUDA(cudaMemcpyAsync(dw.p, w.data(), sizeof(float) * new_N, cudaMemcpyHostToDevice, st), "window");
    R_CUDA(cudaMallocAsync(&dk.p, sizeof(float2) * kernel_length, st), "kernel");
    R_CUDA(cudaMemcpyAsync(dk.p, k.data(), sizeof(float2) * kernel_length, cudaMemcpyHostToDevice, st), "kernel");
    R_CUDA(cudaMallocAsync(&drow.p, sizeof(int) * num_rows, st), "rows");
    R_CUDA(cudaMemcpyAsync(drow.p, row0, sizeof(int) * num_rows, cudaMemcpyHostToDevice, st), "rows");
    R_CUDA(cudaMallocAsync(&tmp.p, sizeof(float2) * S * new_N, st), "downsampled rows");
    R_CALL(downsample_rows((const float2*)ph_dev, S, N, d_coef, new_N, (const float*)dw.p, (float2*)tmp.p, st));
    slow_filter_kernel<<<blocks_for(num_rows * new_N), 256, 0, st>>>((const float2*)tmp.p, (float2*)out_dev,
                                                                    (const float2*)dk.p, (int)kernel_length,
                                                                    (const int*)drow.p, (int)num_rows, (int)new_N,
                                                                    (int)((new_N + 1) / 2));
    R_CUDA(cudaGetLastError(), "slow-time filter");
    R_CUDA(cudaStreamSynchronize(st), "resample");   // host staging arrays go out of scope
    return SAR_OK;
}
