// sar_probe.cu -- throughput of the arithmetic pipes the backprojection gather leans on, measured
// on the device it runs on (sar_measure_pipe_rates, include/sargpu.h).
//
// The gather's work per pixel·pulse is FP32 arithmetic (fused multiply-adds, packed in pairs)
// plus special-function operations (sine, cosine, rounding).  Its roofline needs the per-SM rate
// of each: one kernel per operation runs independent dependency chains of that operation in
// every thread of a full wave of CTAs, and each CTA records its start and end with the SM's own
// cycle counter (clock64) and the SM it ran on.  Operations per SM divided by the SM's busy
// cycles (first start to last end of its CTAs) is the rate per clock per SM, independent of the
// clock frequency; an event-timed launch gives the SM clock that held meanwhile.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/sargpu.h"
#include "sar_kernels.cuh"

namespace {

constexpr int kProbeThreads = 256;
constexpr int kChains = 8;     // independent chains per thread
constexpr int kIters = 2048;   // operations per chain
constexpr int kUnroll = 8;     // operations per chain per loop trip (keeps the loop's own
                               // counter, compare and branch below 5 % of the issued instructions)

enum ProbeOp { OP_SINCOS = 0, OP_FRND = 1, OP_FFMA = 2, OP_FFMA2 = 3, OP_COUNT = 4 };

__device__ __forceinline__ unsigned smid() {
    unsigned r;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
    return r;
}

struct ProbeRecord {
    long long t0, t1;
    unsigned sm, pad;
};

// Operations per chain step: OP_SINCOS 2 special-function ops (sine and cosine of the
// chain value, summed back into it), OP_FRND 1 round-to-integer, OP_FFMA 1 FP32 FMA, OP_FFMA2 2
// FP32 FMAs in one packed instruction.
template <int OP>
__global__ void __launch_bounds__(kProbeThreads) pipe_probe_kernel(float seed, float* sink, ProbeRecord* rec) {
    float v[kChains];
    float2 w[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
        v[c] = seed * (float)(threadIdx.x + 1) + 0.125f * (float)c;
        w[c] = make_float2(v[c], v[c] + 0.5f);
    }
    __syncthreads();
    long long t0 = clock64();
    const float a = 0.9990234375f, b = 0.0009765625f;
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
#pragma unroll 1
    for (int it = 0; it < kIters; it += kUnroll) {
#pragma unroll
        for (int c = 0; c < kChains * kUnroll; ++c) {
            if (OP == OP_SINCOS) {
                float s, co;
                __sincosf(v[c % kChains], &s, &co);
                v[c % kChains] = s + co;   // stays in [-1.5, 1.5]
            } else if (OP == OP_FRND) {
                v[c % kChains] = rintf(v[c % kChains] + 0.75f) - 0.5f;
            } else if (OP == OP_FFMA) {
                v[c % kChains] = fmaf(v[c % kChains], a, b);
            } else {
                w[c % kChains] = __ffma2_rn(w[c % kChains], a2, b2);
            }
        }
    }
    __syncthreads();
    long long t1 = clock64();
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc += (OP == OP_FFMA2) ? w[c].x + w[c].y : v[c];
    if (acc == 1234.5f) sink[0] = acc;   // keeps the chains live; practically never true
    if (threadIdx.x == 0) {
        ProbeRecord r;
        r.t0 = t0;
        r.t1 = t1;
        r.sm = smid();
        r.pad = 0;
        rec[blockIdx.x] = r;
    }
}

template <int OP>
cudaError_t launch_probe(int blocks, float* sink, ProbeRecord* rec, cudaStream_t st) {
    pipe_probe_kernel<OP><<<blocks, kProbeThreads, 0, st>>>(0.001f, sink, rec);
    return cudaGetLastError();
}

cudaError_t launch_op(int op, int blocks, float* sink, ProbeRecord* rec, cudaStream_t st) {
    switch (op) {
        case OP_SINCOS: return launch_probe<OP_SINCOS>(blocks, sink, rec, st);
        case OP_FRND: return launch_probe<OP_FRND>(blocks, sink, rec, st);
        case OP_FFMA: return launch_probe<OP_FFMA>(blocks, sink, rec, st);
        default: return launch_probe<OP_FFMA2>(blocks, sink, rec, st);
    }
}

int probe_fail(int code, const char* msg) {
    sar::sar_internal_set_error(msg);
    return code;
}

}  // namespace

extern "C" int sar_measure_pipe_rates(sar_pipe_rates* out, void* stream) {
    sar::sar_internal_set_error("");
    if (!out) return probe_fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pipe_probe_kernel<OP_SINCOS>, kProbeThreads, 0);
    if (e != cudaSuccess) return probe_fail(SAR_ERR_CUDA, cudaGetErrorString(e));
    if (sms <= 0 || per_sm <= 0) return probe_fail(SAR_ERR_NOT_SUPPORTED, "no resident probe blocks");
    per_sm = std::min(per_sm, 4);   // 32 warps per SM: enough chains to cover every pipe's latency
    const int blocks = sms * per_sm;
    float* sink = nullptr;
    ProbeRecord* rec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    e = cudaMalloc(&sink, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&rec, sizeof(ProbeRecord) * blocks);
    if (e == cudaSuccess) e = cudaEventCreate(&ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ev1);
    const double ops_per_trip[OP_COUNT] = {2.0, 1.0, 1.0, 2.0};
    double rates[OP_COUNT] = {0, 0, 0, 0};
    double mhz_sum = 0.0;
    int mhz_n = 0;
    std::vector<ProbeRecord> host(blocks);
    for (int op = 0; op < OP_COUNT && e == cudaSuccess; ++op) {
        e = launch_op(op, blocks, sink, rec, st);   // warm-up (clocks ramp, module load)
        for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
            e = cudaEventRecord(ev0, st);
            if (e == cudaSuccess) e = launch_op(op, blocks, sink, rec, st);
            if (e == cudaSuccess) e = cudaEventRecord(ev1, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
            if (e == cudaSuccess)
                e = cudaMemcpy(host.data(), rec, sizeof(ProbeRecord) * blocks, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) break;
            // per SM: busy span (first start to last end on that SM's counter) and its CTAs
            std::vector<long long> lo(1024, INT64_MAX), hi(1024, INT64_MIN);
            std::vector<int> n(1024, 0);
            for (const ProbeRecord& r : host) {
                if (r.sm >= 1024) continue;
                lo[r.sm] = std::min(lo[r.sm], r.t0);
                hi[r.sm] = std::max(hi[r.sm], r.t1);
                ++n[r.sm];
            }
            std::vector<double> per;
            long long max_span = 0;
            for (int s = 0; s < 1024; ++s) {
                if (!n[s] || hi[s] <= lo[s]) continue;
                const double ops = (double)n[s] * kProbeThreads * kChains * kIters * ops_per_trip[op];
                per.push_back(ops / (double)(hi[s] - lo[s]));
                max_span = std::max(max_span, hi[s] - lo[s]);
            }
            if (per.empty()) continue;
            std::sort(per.begin(), per.end());
            rates[op] = std::max(rates[op], per[per.size() / 2]);   // median SM, best of the repeats
            if (ms > 0.f) {
                mhz_sum += (double)max_span / (ms * 1.0e3);   // cycles per microsecond, an upper bound of the
                ++mhz_n;                                      // launch's busy time gives a lower bound of MHz
            }
        }
    }
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (rec) cudaFree(rec);
    if (sink) cudaFree(sink);
    if (e != cudaSuccess) return probe_fail(SAR_ERR_CUDA, cudaGetErrorString(e));
    out->sfu_sincos_per_clk_sm = rates[OP_SINCOS];
    out->frnd_per_clk_sm = rates[OP_FRND];
    out->ffma_per_clk_sm = rates[OP_FFMA];
    out->ffma2_per_clk_sm = rates[OP_FFMA2];
    out->num_sms = sms;
    out->sm_mhz = mhz_n ? mhz_sum / mhz_n : 0.0;
    return SAR_OK;
}
