/*
 * Minimal FFTW3-compatible API used only to compile the reference kernel
 * (src/sarsolver/cxx_binding/sarsolver_cxx.cpp) into the test oracle when libfftw3 is absent.
 *
 * Only the names that kernel calls are provided (sarsolver_cxx.cpp:5,209-216,244-251,260-261,
 * 292,344): fftw_complex, fftw_plan, fftw_plan_dft_1d, fftw_execute, fftw_destroy_plan and
 * the FFTW_FORWARD / FFTW_BACKWARD / FFTW_ESTIMATE / FFTW_MEASURE constants, with FFTW's
 * published meaning (unnormalised transform, exponent sign -1 forward, +1 backward).
 * The transform itself is fft64 (FP64 radix-2 / Bluestein).  Test infrastructure only.
 */
#ifndef SAR_ORACLE_FFTW_SHIM_H
#define SAR_ORACLE_FFTW_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_shim_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);

#ifdef __cplusplus
}
#endif

#endif
