/*
 * FFTW3-compatible plan objects over fft64 (see fftw3.h).  A plan remembers its in/out
 * buffers, like FFTW's, because the reference executes plans made once per worker
 * (sarsolver_cxx.cpp:244-251, executed at :292 and :344).  Test infrastructure only.
 */
#include "fftw3.h"

#include <stdlib.h>

#include "../fft64.h"

struct fftw_shim_plan_s {
    fft64_plan *core;
    double *in;
    double *out;
};

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
    (void)flags;
    if (n <= 0) return NULL;
    fftw_plan p = (fftw_plan)malloc(sizeof(*p));
    if (!p) return NULL;
    p->core = fft64_create((size_t)n, sign < 0 ? -1 : 1);
    if (!p->core) { free(p); return NULL; }
    p->in = (double *)in;
    p->out = (double *)out;
    return p;
}

void fftw_execute(const fftw_plan p) {
    if (p) fft64_execute(p->core, p->in, p->out);
}

void fftw_destroy_plan(fftw_plan p) {
    if (!p) return;
    fft64_destroy(p->core);
    free(p);
}
