/*
 * sar_oracle -- FP64 CPU restatement of the sarsolver scalar-Born SAR operator pair.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path links, loads or calls this code;
 * it is the checker for the GPU kernels and the timed CPU baseline.
 *
 * It follows src/sarsolver/cxx_binding/sarsolver_cxx.cpp:
 *   - working length M = (size_t)(upsample_ratio * N)                      (:223)
 *   - bins per metre s_r = fs * M / (N * c_eff), k = 2*pi*sign*fc/c_eff    (:225-228)
 *   - bistatic range, differential w.r.t. the SRP                         (:10-20, :283, :287)
 *   - cyclic bin modulo                                                   (:22-24)
 *   - forward: scatter, FFT_-, keep N/2 low + N/2 high modes (+odd middle) x W  (:271-310)
 *   - adjoint: zero-pad conj(W) y, FFT_+, gather                          (:319-353)
 * with two interpolation modes:
 *   ORACLE_NEAREST_REF: the reference conventions verbatim -- forward bins with round(v)
 *     (:289), adjoint with round(0.5+v) (:347), slow-time weight unconjugated in both
 *     (:288, :349).  This pair is not an exact adjoint pair.
 *   ORACLE_LINEAR: linear interpolation between bins floor(v) and floor(v)+1; the adjoint
 *     conjugates the slow-time weight, so forward and adjoint are exact transposes.
 * Arrays are interleaved (re, im) doubles; phase histories are in FFT order, as the C++
 * kernel sees them (the Python layer shifts: forward.py:39,44, adjoint.py:36).
 */
#ifndef SAR_ORACLE_H
#define SAR_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_NEAREST_REF = 0, ORACLE_LINEAR = 1 };

typedef struct {
    size_t num_fast_times, num_slow_times, num_scatterers;              /* N, S, P */
    const double *transmit_posns, *receive_posns, *stab_ref_posns;      /* [S][3] */
    const double *scat_posns;                                           /* [P][3] */
    const double *waveform_fft;         /* [N][2], FFT order; NULL means all ones */
    const double *slow_time_weighting;  /* [S][2]; NULL means all ones */
    double centre_frequency, sample_frequency, c_eff, upsample_ratio, sign_multiplier;
    int mode;                           /* ORACLE_NEAREST_REF or ORACLE_LINEAR */
    int num_threads;                    /* <= 1: single thread */
} oracle_sar_info;

/* y[S][N] (FFT order) = A x[P].  Returns 0 on success. */
int oracle_forward(const oracle_sar_info *info, const double *x, double *y);
/* x[P] = A^H y[S][N] (FFT order). */
int oracle_adjoint(const oracle_sar_info *info, const double *y, double *x);
/* Upsampled range profiles prof[S][M] = FFT_+(zero-padded conj(W) y), no slow-time weight. */
int oracle_upsample(const oracle_sar_info *info, const double *y, double *prof);
/* Differential bistatic ranges dr[S][P] in metres. */
int oracle_ranges(const oracle_sar_info *info, double *dr);
/* Working length M. */
size_t oracle_working_length(const oracle_sar_info *info);

#ifdef __cplusplus
}
#endif

#endif
