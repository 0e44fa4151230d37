/*
 * sar_oracle -- FP64 CPU restatement of the sarsolver operator pair (test infrastructure only).
 * See sar_oracle.h for the contract and the reference lines each part follows.
 */
#include "sar_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "fft64.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------------------------------------------------------- helpers */

/* Euclidean distance, summed axis by axis as sarsolver_cxx.cpp:10-16. */
static double distance3(const double *a, const double *b) {
    double d = 0.0;
    for (int ax = 0; ax < 3; ++ax) d += (a[ax] - b[ax]) * (a[ax] - b[ax]);
    return sqrt(d);
}

/* Non-negative modulo for negative bins, sarsolver_cxx.cpp:22-24. */
static size_t cyc_mod(long a, long b) { return (size_t)(((a % b) + b) % b); }

typedef struct {
    size_t N, S, P, M, half;
    double s_r;   /* bins per metre of bistatic range */
    double k;     /* radians per metre of bistatic range */
} derived_t;

static int derive(const oracle_sar_info *in, derived_t *d) {
    if (!in || in->num_fast_times == 0 || in->upsample_ratio <= 0.0) return 1;
    d->N = in->num_fast_times;
    d->S = in->num_slow_times;
    d->P = in->num_scatterers;
    d->M = (size_t)(in->upsample_ratio * (double)in->num_fast_times);   /* :223 truncation */
    if (d->M < d->N) return 1;
    d->half = d->N / 2;
    d->s_r = (in->sample_frequency * (double)d->M) / ((double)d->N * in->c_eff);   /* :225-226 */
    d->k = 2.0 * in->sign_multiplier * M_PI * in->centre_frequency / in->c_eff;     /* :228 */
    return 0;
}

static void weight_of(const oracle_sar_info *in, size_t s, double *wr, double *wi) {
    if (in->slow_time_weighting) {
        *wr = in->slow_time_weighting[2 * s];
        *wi = in->slow_time_weighting[2 * s + 1];
    } else {
        *wr = 1.0;
        *wi = 0.0;
    }
}

static void wave_of(const oracle_sar_info *in, size_t f, double *wr, double *wi) {
    if (in->waveform_fft) {
        *wr = in->waveform_fft[2 * f];
        *wi = in->waveform_fft[2 * f + 1];
    } else {
        *wr = 1.0;
        *wi = 0.0;
    }
}

static double srp_range(const oracle_sar_info *in, size_t s) {
    const double *t = in->transmit_posns + 3 * s, *r = in->receive_posns + 3 * s;
    const double *c = in->stab_ref_posns + 3 * s;
    return distance3(t, c) + distance3(r, c);
}

static double diff_range(const oracle_sar_info *in, size_t s, size_t p, double ref) {
    const double *t = in->transmit_posns + 3 * s, *r = in->receive_posns + 3 * s;
    const double *x = in->scat_posns + 3 * p;
    return distance3(t, x) + distance3(r, x) - ref;
}

/* ------------------------------------------------------------ thread pool */

typedef void (*range_fn)(void *ctx, size_t lo, size_t hi);

typedef struct {
    range_fn fn;
    void *ctx;
    size_t lo, hi;
} job_t;

static void *job_main(void *arg) {
    job_t *j = (job_t *)arg;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

static void parallel_for(int nthreads, size_t n, range_fn fn, void *ctx) {
    if (nthreads <= 1 || n < 2) {
        fn(ctx, 0, n);
        return;
    }
    if ((size_t)nthreads > n) nthreads = (int)n;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    job_t *jobs = (job_t *)malloc(sizeof(job_t) * nthreads);
    int *started = (int *)calloc(nthreads, sizeof(int));
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].lo = n * (size_t)t / (size_t)nthreads;
        jobs[t].hi = n * (size_t)(t + 1) / (size_t)nthreads;
        started[t] = (pthread_create(&th[t], NULL, job_main, &jobs[t]) == 0);
        if (!started[t]) job_main(&jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t)
        if (started[t]) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
    free(started);
}

/* ---------------------------------------------------------------- forward */

typedef struct {
    const oracle_sar_info *in;
    const derived_t *d;
    const double *x;
    double *y;
    int failed;
} fwd_ctx;

static void forward_pulses(void *vctx, size_t s0, size_t s1) {
    fwd_ctx *c = (fwd_ctx *)vctx;
    const oracle_sar_info *in = c->in;
    const derived_t *d = c->d;
    double *prof = (double *)malloc(sizeof(double) * 2 * d->M);
    double *kmod = (double *)malloc(sizeof(double) * 2 * d->M);
    fft64_plan *plan = fft64_create(d->M, -1);                 /* FFTW_FORWARD, :244-247 */
    if (!prof || !kmod || !plan) {
        c->failed = 1;
        free(prof); free(kmod); fft64_destroy(plan);
        return;
    }
    for (size_t s = s0; s < s1; ++s) {
        memset(prof, 0, sizeof(double) * 2 * d->M);
        double wr, wi;
        weight_of(in, s, &wr, &wi);
        const double ref = srp_range(in, s);                   /* :283 */
        for (size_t p = 0; p < d->P; ++p) {                    /* :284-291 */
            const double dr = diff_range(in, s, p, ref);
            const double ph = dr * d->k;
            const double er = cos(ph), ei = sin(ph);
            const double xr = c->x[2 * p], xi = c->x[2 * p + 1];
            /* amplitude = exp(j k dR) * x * w_s (weight unconjugated, :288) */
            const double ar0 = er * xr - ei * xi, ai0 = er * xi + ei * xr;
            const double ar = ar0 * wr - ai0 * wi, ai = ar0 * wi + ai0 * wr;
            const double v = dr * d->s_r;
            if (in->mode == ORACLE_NEAREST_REF) {
                const size_t b = cyc_mod((long)round(v), (long)d->M);   /* :289 */
                prof[2 * b] += ar;
                prof[2 * b + 1] += ai;
            } else {
                const double fl = floor(v);
                const double t = v - fl;
                const size_t b0 = cyc_mod((long)fl, (long)d->M);
                const size_t b1 = cyc_mod((long)fl + 1, (long)d->M);
                prof[2 * b0] += (1.0 - t) * ar;
                prof[2 * b0 + 1] += (1.0 - t) * ai;
                prof[2 * b1] += t * ar;
                prof[2 * b1 + 1] += t * ai;
            }
        }
        fft64_execute(plan, prof, kmod);                       /* :292 */
        double *row = c->y + 2 * d->N * s;
        for (size_t i = 0; i < d->half; ++i) {                 /* :295-303 */
            const size_t hi_y = d->N - i - 1, hi_k = d->M - i - 1;
            double wvr, wvi;
            wave_of(in, hi_y, &wvr, &wvi);
            row[2 * hi_y] = wvr * kmod[2 * hi_k] - wvi * kmod[2 * hi_k + 1];
            row[2 * hi_y + 1] = wvr * kmod[2 * hi_k + 1] + wvi * kmod[2 * hi_k];
            wave_of(in, i, &wvr, &wvi);
            row[2 * i] = wvr * kmod[2 * i] - wvi * kmod[2 * i + 1];
            row[2 * i + 1] = wvr * kmod[2 * i + 1] + wvi * kmod[2 * i];
        }
        if (d->N % 2 == 1) {                                   /* :304-307 */
            const size_t h = d->half;
            double wvr, wvi;
            wave_of(in, h, &wvr, &wvi);
            row[2 * h] = wvr * kmod[2 * h] - wvi * kmod[2 * h + 1];
            row[2 * h + 1] = wvr * kmod[2 * h + 1] + wvi * kmod[2 * h];
        }
    }
    free(prof);
    free(kmod);
    fft64_destroy(plan);
}

int oracle_forward(const oracle_sar_info *in, const double *x, double *y) {
    derived_t d;
    if (derive(in, &d) || !x || !y) return 1;
    memset(y, 0, sizeof(double) * 2 * d.N * d.S);              /* setup_forward_evaluate, :264-269 */
    fwd_ctx c = {in, &d, x, y, 0};
    parallel_for(in->num_threads, d.S, forward_pulses, &c);
    return c.failed;
}

/* --------------------------------------------------------------- upsample */

typedef struct {
    const oracle_sar_info *in;
    const derived_t *d;
    const double *y;
    double *prof;       /* [count][M] */
    size_t first;       /* first pulse of the chunk */
    int failed;
} up_ctx;

static void upsample_pulses(void *vctx, size_t a, size_t b) {
    up_ctx *c = (up_ctx *)vctx;
    const oracle_sar_info *in = c->in;
    const derived_t *d = c->d;
    double *kmod = (double *)malloc(sizeof(double) * 2 * d->M);
    fft64_plan *plan = fft64_create(d->M, +1);                 /* FFTW_BACKWARD, :248-251 */
    if (!kmod || !plan) {
        c->failed = 1;
        free(kmod); fft64_destroy(plan);
        return;
    }
    for (size_t j = a; j < b; ++j) {
        const size_t s = c->first + j;
        memset(kmod, 0, sizeof(double) * 2 * d->M);
        const double *row = c->y + 2 * d->N * s;
        for (size_t i = 0; i < d->half; ++i) {                 /* :331-338 */
            double wr, wi;
            wave_of(in, i, &wr, &wi);                          /* conj(W) * y */
            kmod[2 * i] = wr * row[2 * i] + wi * row[2 * i + 1];
            kmod[2 * i + 1] = wr * row[2 * i + 1] - wi * row[2 * i];
            const size_t hy = d->N - i - 1, hk = d->M - i - 1;
            wave_of(in, hy, &wr, &wi);
            kmod[2 * hk] = wr * row[2 * hy] + wi * row[2 * hy + 1];
            kmod[2 * hk + 1] = wr * row[2 * hy + 1] - wi * row[2 * hy];
        }
        if (d->N % 2 == 1) {                                   /* :339-342 */
            const size_t h = d->half;
            double wr, wi;
            wave_of(in, h, &wr, &wi);
            kmod[2 * h] = wr * row[2 * h] + wi * row[2 * h + 1];
            kmod[2 * h + 1] = wr * row[2 * h + 1] - wi * row[2 * h];
        }
        fft64_execute(plan, kmod, c->prof + 2 * d->M * j);     /* :344 */
    }
    free(kmod);
    fft64_destroy(plan);
}

int oracle_upsample(const oracle_sar_info *in, const double *y, double *prof) {
    derived_t d;
    if (derive(in, &d) || !y || !prof) return 1;
    up_ctx c = {in, &d, y, prof, 0, 0};
    parallel_for(in->num_threads, d.S, upsample_pulses, &c);
    return c.failed;
}

/* ---------------------------------------------------------------- adjoint */

typedef struct {
    const oracle_sar_info *in;
    const derived_t *d;
    const double *prof;   /* [count][M] for pulses first .. first+count-1 */
    size_t first, count;
    double *x;
} gather_ctx;

static void gather_pixels(void *vctx, size_t p0, size_t p1) {
    gather_ctx *c = (gather_ctx *)vctx;
    const oracle_sar_info *in = c->in;
    const derived_t *d = c->d;
    for (size_t j = 0; j < c->count; ++j) {
        const size_t s = c->first + j;
        const double ref = srp_range(in, s);                   /* :330 */
        double wr, wi;
        weight_of(in, s, &wr, &wi);
        if (in->mode != ORACLE_NEAREST_REF) wi = -wi;          /* exact adjoint: conj(w_s) */
        const double *pr = c->prof + 2 * d->M * j;
        for (size_t p = p0; p < p1; ++p) {                     /* :345-350 */
            const double dr = diff_range(in, s, p, ref);
            const double v = dr * d->s_r;
            double vr, vi;
            if (in->mode == ORACLE_NEAREST_REF) {
                const size_t b = cyc_mod((long)round(0.5 + v), (long)d->M);   /* :347 */
                vr = pr[2 * b];
                vi = pr[2 * b + 1];
            } else {
                const double fl = floor(v);
                const double t = v - fl;
                const size_t b0 = cyc_mod((long)fl, (long)d->M);
                const size_t b1 = cyc_mod((long)fl + 1, (long)d->M);
                vr = (1.0 - t) * pr[2 * b0] + t * pr[2 * b1];
                vi = (1.0 - t) * pr[2 * b0 + 1] + t * pr[2 * b1 + 1];
            }
            const double ph = -dr * d->k;                      /* exp(-j k dR), :348 */
            const double er = cos(ph), ei = sin(ph);
            const double ar = vr * er - vi * ei, ai = vr * ei + vi * er;
            c->x[2 * p] += ar * wr - ai * wi;                  /* x w_s, :349 */
            c->x[2 * p + 1] += ar * wi + ai * wr;
        }
    }
}

int oracle_adjoint(const oracle_sar_info *in, const double *y, double *x) {
    derived_t d;
    if (derive(in, &d) || !y || !x) return 1;
    memset(x, 0, sizeof(double) * 2 * d.P);                    /* setup_adjoint_evaluate, :312-317 */
    /* Pulses are processed in chunks so the profile store stays bounded. */
    size_t chunk = 64;
    if (in->num_threads > 0 && (size_t)in->num_threads * 4 > chunk) chunk = (size_t)in->num_threads * 4;
    if (chunk > d.S) chunk = d.S ? d.S : 1;
    double *prof = (double *)malloc(sizeof(double) * 2 * d.M * chunk);
    if (!prof) return 1;
    int failed = 0;
    for (size_t first = 0; first < d.S && !failed; first += chunk) {
        const size_t count = (d.S - first < chunk) ? d.S - first : chunk;
        up_ctx u = {in, &d, y, prof, first, 0};
        parallel_for(in->num_threads, count, upsample_pulses, &u);
        failed |= u.failed;
        gather_ctx g = {in, &d, prof, first, count, x};
        parallel_for(in->num_threads, d.P, gather_pixels, &g);
    }
    free(prof);
    return failed;
}

/* ----------------------------------------------------------------- ranges */

int oracle_ranges(const oracle_sar_info *in, double *dr) {
    derived_t d;
    if (derive(in, &d) || !dr) return 1;
    for (size_t s = 0; s < d.S; ++s) {
        const double ref = srp_range(in, s);
        for (size_t p = 0; p < d.P; ++p) dr[d.P * s + p] = diff_range(in, s, p, ref);
    }
    return 0;
}

size_t oracle_working_length(const oracle_sar_info *in) {
    derived_t d;
    if (derive(in, &d)) return 0;
    return d.M;
}
