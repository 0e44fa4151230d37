// sar_cphd.cu -- decode of CPHD signal arrays on the device (sar_cphd_decode in include/sargpu.h).
//
// A CPHD signal array is [NumVectors][NumSamples] complex samples stored big-endian as interleaved
// (I, Q) pairs: CI2 = two signed 8-bit integers, CI4 = two signed 16-bit integers, CF8 = two IEEE
// binary32 values (CPHD 1.0.1 Data/SignalArrayFormat; CPHD 0.3 Data/SampleType RE08I_IM08I,
// RE16I_IM16I, RE32F_IM32F).  The reference reads them through sarpy
// (src/sarsolver/io/cphd101.py:251-265, io/cphd03.py:250-263) into host memory; here the raw bytes
// are copied to the device as they lie in the file (2-8x fewer bytes over the host link than
// complex64) and widened on the device:
//   out[v][s] = complex(I, Q) * amp_sf[v]      (amp_sf optional: the per-vector AmpSF PVP)
// Pure streaming work (one read of the raw bytes, one write of complex64): HBM-bound.  Threads
// convert 16-byte chunks (8 CI2, 4 CI4 or 2 CF8 samples) with vector loads and stores: row by row
// when both buffers and both row strides are 16-byte aligned (the usual case: even NumSamples for
// CF8, multiples of 4 / 8 for CI4 / CI2), over the flat array when only the buffers are, and
// sample by sample otherwise.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>

#include "../../include/sargpu.h"
#include "sar_kernels.cuh"

namespace {

int err(int code, const char* msg) {
    sar::sar_internal_set_error(msg);
    return code;
}

// Bytes per complex sample of each format.
__host__ __device__ constexpr int sample_bytes(int format) {
    return format == SAR_CPHD_CI2 ? 2 : format == SAR_CPHD_CI4 ? 4 : 8;
}

// One complex sample from its big-endian bytes, given as the low bytes of w (byte 0 = first in
// the file).  Sign extension by arithmetic shifts, so nothing depends on the signedness of char.
template <int FORMAT>
__device__ __forceinline__ float2 decode_word(uint32_t w) {
    if constexpr (FORMAT == SAR_CPHD_CI2) {
        const int i = (int)(w << 24) >> 24;
        const int q = (int)(w << 16) >> 24;
        return make_float2((float)i, (float)q);
    } else if constexpr (FORMAT == SAR_CPHD_CI4) {
        const uint32_t r = __byte_perm(w, 0u, 0x2301u);   // swap the bytes of each 16-bit half
        const int i = (int)(r << 16) >> 16;
        const int q = (int)r >> 16;
        return make_float2((float)i, (float)q);
    } else {
        return make_float2(0.f, 0.f);   // CF8 takes two words (decode_f32 each)
    }
}

__device__ __forceinline__ float decode_f32(uint32_t w) { return __int_as_float((int)__byte_perm(w, 0u, 0x0123u)); }

__device__ __forceinline__ float2 scaled(float2 v, const float* __restrict__ amp, size_t e, size_t samples) {
    if (amp) {
        const float a = __ldg(amp + e / samples);
        v.x *= a;
        v.y *= a;
    }
    return v;
}

// Sample e of the raw array, read byte-wise (the unaligned path and the tail).
template <int FORMAT>
__device__ __forceinline__ float2 decode_at(const uint8_t* __restrict__ raw, size_t e) {
    constexpr int B = sample_bytes(FORMAT);
    const uint8_t* p = raw + e * B;
    if constexpr (FORMAT == SAR_CPHD_CF8) {
        const uint32_t wi = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
        const uint32_t wq = (uint32_t)p[4] | ((uint32_t)p[5] << 8) | ((uint32_t)p[6] << 16) | ((uint32_t)p[7] << 24);
        return make_float2(decode_f32(wi), decode_f32(wq));
    } else {
        uint32_t w = (uint32_t)p[0] | ((uint32_t)p[1] << 8);
        if constexpr (B == 4) w |= ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
        return decode_word<FORMAT>(w);
    }
}

// 16 bytes of raw samples -> PER complex64 values (PER = 16 / bytes per sample).
template <int FORMAT>
__device__ __forceinline__ void decode_chunk(const uint4 v, float2 (&s)[16 / sample_bytes(FORMAT)]) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    if constexpr (FORMAT == SAR_CPHD_CI2) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            s[2 * k] = decode_word<FORMAT>(w[k] & 0xffffu);
            s[2 * k + 1] = decode_word<FORMAT>(w[k] >> 16);
        }
    } else if constexpr (FORMAT == SAR_CPHD_CI4) {
#pragma unroll
        for (int k = 0; k < 4; ++k) s[k] = decode_word<FORMAT>(w[k]);
    } else {
        s[0] = make_float2(decode_f32(w[0]), decode_f32(w[1]));
        s[1] = make_float2(decode_f32(w[2]), decode_f32(w[3]));
    }
}

template <int FORMAT>
__global__ void __launch_bounds__(256) cphd_decode_kernel(const uint8_t* __restrict__ raw, float2* __restrict__ out,
                                                          const float* __restrict__ amp, size_t total, size_t samples,
                                                          int vector_path) {
    constexpr int B = sample_bytes(FORMAT);
    constexpr int PER = 16 / B;   // samples per 16-byte chunk
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t first_tail = 0;
    if (vector_path) {
        const size_t chunks = total / PER;
        first_tail = chunks * PER;
        const uint4* in4 = reinterpret_cast<const uint4*>(raw);
        float4* out4 = reinterpret_cast<float4*>(out);
        for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < chunks; c += stride) {
            float2 s[PER];
            decode_chunk<FORMAT>(__ldcs(in4 + c), s);   // read once: stream past L2
            const size_t e0 = c * PER;
#pragma unroll
            for (int k = 0; k < PER; ++k) s[k] = scaled(s[k], amp, e0 + k, samples);
#pragma unroll
            for (int k = 0; k < PER / 2; ++k)
                __stcs(out4 + c * (PER / 2) + k, make_float4(s[2 * k].x, s[2 * k].y, s[2 * k + 1].x, s[2 * k + 1].y));
        }
    }
    for (size_t e = first_tail + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += stride)
        out[e] = scaled(decode_at<FORMAT>(raw, e), amp, e, samples);
}

// Row-wise form for rows whose raw and complex64 strides are multiples of 16 bytes: CTA row
// blockIdx.y (striding by gridDim.y), U independent 16-byte chunks per thread in flight, the
// row's AmpSF loaded once.
template <int FORMAT, int U>
__global__ void __launch_bounds__(256) cphd_decode_rows_kernel(const uint8_t* __restrict__ raw, float2* __restrict__ out,
                                                               const float* __restrict__ amp, size_t rows,
                                                               int chunks_per_row) {
    constexpr int PER = 16 / sample_bytes(FORMAT);
    for (size_t r = blockIdx.y; r < rows; r += gridDim.y) {
        const uint4* in4 = reinterpret_cast<const uint4*>(raw) + r * (size_t)chunks_per_row;
        float4* out4 = reinterpret_cast<float4*>(out) + r * (size_t)chunks_per_row * (PER / 2);
        const float a = amp ? __ldg(amp + r) : 1.0f;
        const int c0 = blockIdx.x * (256 * U) + threadIdx.x;
        uint4 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (c0 + u * 256 < chunks_per_row) v[u] = __ldcs(in4 + c0 + u * 256);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int c = c0 + u * 256;
            if (c >= chunks_per_row) break;
            float2 s[PER];
            decode_chunk<FORMAT>(v[u], s);
            if (amp) {
#pragma unroll
                for (int k = 0; k < PER; ++k) {
                    s[k].x *= a;
                    s[k].y *= a;
                }
            }
#pragma unroll
            for (int k = 0; k < PER / 2; ++k)
                __stcs(out4 + (size_t)c * (PER / 2) + k, make_float4(s[2 * k].x, s[2 * k].y, s[2 * k + 1].x, s[2 * k + 1].y));
        }
    }
}

template <int FORMAT>
void launch(const uint8_t* raw, float2* out, const float* amp, size_t total, size_t samples, bool vec, cudaStream_t st,
            int sms) {
    constexpr int PER = 16 / sample_bytes(FORMAT);
    constexpr int U = 2;
    const size_t rows = total / samples;
    if (vec && (samples * sample_bytes(FORMAT)) % 16 == 0) {
        const size_t cpr = samples * sample_bytes(FORMAT) / 16;
        const dim3 grid((unsigned)((cpr + 256 * U - 1) / (256 * U)), (unsigned)std::min<size_t>(rows, 65535));
        cphd_decode_rows_kernel<FORMAT, U><<<grid, 256, 0, st>>>(raw, out, amp, rows, (int)cpr);
        return;
    }
    const size_t work = vec ? (total + PER - 1) / PER : total;
    // a few resident waves of 256-thread blocks; the loop strides over the rest
    const size_t want = (work + 255) / 256;
    const unsigned grid = (unsigned)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * 8));
    cphd_decode_kernel<FORMAT><<<grid, 256, 0, st>>>(raw, out, amp, total, samples, vec ? 1 : 0);
}

int device_sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 148;
    return sms > 0 ? sms : 148;
}

}  // namespace

extern "C" int sar_cphd_decode(const void* raw_dev, int format, size_t num_vectors, size_t num_samples,
                               const float* amp_sf_dev, void* out_dev, void* stream) {
    if (format != SAR_CPHD_CI2 && format != SAR_CPHD_CI4 && format != SAR_CPHD_CF8)
        return err(SAR_ERR_INVALID_ARGUMENT, "unknown CPHD signal format");
    if (!num_vectors || !num_samples) return SAR_OK;
    if (!raw_dev || !out_dev) return err(SAR_ERR_INVALID_ARGUMENT, "null argument");
    if (num_samples > ((size_t)1 << 31) || num_vectors > ((size_t)1 << 31) || num_vectors * num_samples > ((size_t)1 << 36))
        return err(SAR_ERR_INVALID_ARGUMENT, "signal array too large");
    const size_t total = num_vectors * num_samples;
    const bool vec = ((uintptr_t)raw_dev % 16 == 0) && ((uintptr_t)out_dev % 16 == 0);
    cudaStream_t st = (cudaStream_t)stream;
    const uint8_t* raw = (const uint8_t*)raw_dev;
    float2* out = (float2*)out_dev;
    const int sms = device_sm_count();
    switch (format) {
        case SAR_CPHD_CI2: launch<SAR_CPHD_CI2>(raw, out, amp_sf_dev, total, num_samples, vec, st, sms); break;
        case SAR_CPHD_CI4: launch<SAR_CPHD_CI4>(raw, out, amp_sf_dev, total, num_samples, vec, st, sms); break;
        default: launch<SAR_CPHD_CF8>(raw, out, amp_sf_dev, total, num_samples, vec, st, sms); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof buf, "cphd decode: %s", cudaGetErrorString(e));
        return err(SAR_ERR_CUDA, buf);
    }
    return SAR_OK;
}
