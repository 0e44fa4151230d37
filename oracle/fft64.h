/*
 * fft64 -- unnormalised FP64 complex DFT used by the CPU oracle (test infrastructure only).
 *
 * out[k] = sum_j in[j] * exp(sign * 2*pi*i * j*k / n), sign = -1 (forward) or +1 (backward),
 * no 1/n scaling: the convention of FFTW_FORWARD / FFTW_BACKWARD, which the reference kernel
 * uses at sarsolver_cxx.cpp:209-216 and :244-251.
 *
 * Power-of-two lengths use an iterative radix-2 transform; every other length uses
 * Bluestein's chirp-z identity on a power-of-two transform, so any n costs O(n log n).
 * Buffers are interleaved (re, im) doubles; in and out may alias.
 */
#ifndef SAR_ORACLE_FFT64_H
#define SAR_ORACLE_FFT64_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fft64_plan fft64_plan;

fft64_plan *fft64_create(size_t n, int sign);
void fft64_execute(const fft64_plan *plan, const double *in, double *out);
void fft64_destroy(fft64_plan *plan);

#ifdef __cplusplus
}
#endif

#endif
