// sar_fft_cb.h -- parameters of the cuFFT load/store callbacks of the range-profile transforms
// (shared by the callback source, compiled to LTO-IR, and the host code that fills it).
//
// The callbacks replace the packing and extraction kernels around the batched length-M FFTs:
//   adjoint (inverse FFT): load  = conj(W[i]) y[row][(i + N/2) mod N] at the zero-padded position
//                                  of FFT index i, zero elsewhere (sarsolver_cxx.cpp:331-342);
//                          store = keep only the stored span: compact[row][w] for w = (m - bg0) mod M
//                                  when w < Lc (the profile bins the gather reads);
//   forward (forward FFT): load  = sum of the accumulator bins congruent to m modulo M;
//                          store = the N extracted outputs times W[i] and the pulse factor, written
//                                  fftshifted into y (sarsolver_cxx.cpp:295-307, forward.py:44).
// One instance lives in device memory per plan and is rewritten (stream-ordered) before each
// transform; `first` is the first pulse of the transform's batch.
#pragma once

#include <cuda_runtime.h>

struct SarFftCbInfo {
    const float2* y;        // adjoint input phase history [S][N] (fftshifted)
    float2* yout;           // forward output phase history [S][N] (fftshifted)
    const float2* wave;     // waveform, FFT order [N]
    const float2* wfac;     // forward pulse factors [S]
    const float2* acc;      // forward accumulator [S][Lg]
    float2* compact;        // adjoint stored span [batch][Lc]
    long long M;            // working length
    long long nb0;          // (-bg0) mod M
    unsigned mask;          // M - 1 when M is a power of two, else 0
    int shift;              // log2(M) when M is a power of two
    int N, half, Lg, Lc, first;
};
