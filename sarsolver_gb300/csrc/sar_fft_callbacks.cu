// sar_fft_callbacks.cu -- cuFFT JIT (LTO) load/store callbacks of the range-profile transforms.
// Compiled to LTO-IR (-gencode arch=compute_103a,code=lto_103a -rdc=true -fatbin) and linked into
// cuFFT's kernels at plan creation through cufftXtSetJITCallback; see sar_fft_cb.h for what each
// callback computes.
#include <cufftXt.h>

#include "sar_fft_cb.h"

namespace {

// (row, m) of a flat element offset row * M + m.
__device__ __forceinline__ void split_offset(const SarFftCbInfo* c, unsigned long long off, long long& row, long long& m) {
    if (c->mask) {
        row = (long long)(off >> c->shift);
        m = (long long)(off & c->mask);
    } else {
        row = (long long)(off / (unsigned long long)c->M);
        m = (long long)off - row * c->M;
    }
}

}  // namespace

// Adjoint load: conj(W[i]) y[first + row][(i + half) mod N] for the FFT index i at position m.
extern "C" __device__ cufftComplex sar_cb_adjoint_load(void* dataIn, unsigned long long offset, void* info, void* shared) {
    const SarFftCbInfo* c = (const SarFftCbInfo*)info;
    long long row, m;
    split_offset(c, offset, row, m);
    int i = -1;
    if (m < c->half)
        i = (int)m;
    else if (m >= c->M - c->half)
        i = (int)(c->N - c->M + m);
    else if ((c->N & 1) && m == c->half)
        i = c->half;
    if (i < 0) return make_float2(0.f, 0.f);
    int k = i + c->half;
    if (k >= c->N) k -= c->N;
    const float2 yv = c->y[(size_t)(c->first + row) * c->N + k];
    const float2 w = __ldg(c->wave + i);
    return make_float2(w.x * yv.x + w.y * yv.y, w.x * yv.y - w.y * yv.x);
}

// Adjoint store: keep the bins of the stored span, compact[row][w], w = (m - bg0) mod M < Lc.
extern "C" __device__ void sar_cb_adjoint_store(void* dataOut, unsigned long long offset, cufftComplex element,
                                                void* info, void* shared) {
    const SarFftCbInfo* c = (const SarFftCbInfo*)info;
    long long row, m;
    split_offset(c, offset, row, m);
    long long w = m + c->nb0;
    if (w >= c->M) w -= c->M;
    if (w < c->Lc) c->compact[(size_t)row * c->Lc + w] = element;
}

// Forward load: sum of the accumulator bins w congruent to m modulo M.
extern "C" __device__ cufftComplex sar_cb_forward_load(void* dataIn, unsigned long long offset, void* info, void* shared) {
    const SarFftCbInfo* c = (const SarFftCbInfo*)info;
    long long row, m;
    split_offset(c, offset, row, m);
    long long w = m + c->nb0;
    if (w >= c->M) w -= c->M;
    float2 s = make_float2(0.f, 0.f);
    const float2* a = c->acc + (size_t)(c->first + row) * c->Lg;
    for (; w < c->Lg; w += c->M) {
        const float2 v = a[w];
        s.x += v.x;
        s.y += v.y;
    }
    return s;
}

// Forward store: the N extracted outputs, times W[i] and the pulse factor, fftshifted into y.
extern "C" __device__ void sar_cb_forward_store(void* dataOut, unsigned long long offset, cufftComplex element,
                                                void* info, void* shared) {
    const SarFftCbInfo* c = (const SarFftCbInfo*)info;
    long long row, m;
    split_offset(c, offset, row, m);
    int i;
    if (m < c->half)
        i = (int)m;
    else if (m >= c->M - c->half)
        i = (int)(c->N - c->M + m);
    else if ((c->N & 1) && m == c->half)
        i = c->half;
    else
        return;
    const float2 w = __ldg(c->wave + i);
    const float2 f = __ldg(c->wfac + c->first + row);
    const float2 a = make_float2(w.x * element.x - w.y * element.y, w.x * element.y + w.y * element.x);
    int k = i + c->half;
    if (k >= c->N) k -= c->N;
    c->yout[(size_t)(c->first + row) * c->N + k] = make_float2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
}
