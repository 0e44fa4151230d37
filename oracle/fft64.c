/*
 * fft64 -- unnormalised FP64 complex DFT for the CPU oracle (test infrastructure only).
 * See fft64.h for the convention.  Twiddles are evaluated directly from exact integer
 * angles (no recurrences), so the transform error stays at a few ulp * log2(n).
 */
#include "fft64.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

struct fft64_plan {
    size_t n;
    int sign;
    /* radix-2 core of length m (m == n for powers of two, else the Bluestein length) */
    size_t m;
    double *tw;      /* m/2 twiddles exp(sign*2*pi*i*k/m), interleaved */
    size_t *rev;     /* bit reversal permutation of length m */
    double *work;    /* m complex scratch */
    /* Bluestein data (NULL for powers of two) */
    double *chirp;   /* n values exp(sign*pi*i*j^2/n) */
    double *kernel;  /* forward transform (sign -1 core) of the conjugated chirp, length m */
    double *tw_inv;  /* twiddles of the opposite sign for the inverse core */
};

static int is_pow2(size_t n) { return n && !(n & (n - 1)); }

static void make_twiddles(double *tw, size_t m, int sign) {
    for (size_t k = 0; k < m / 2; ++k) {
        double a = 2.0 * M_PI * (double)k / (double)m;
        tw[2 * k] = cos(a);
        tw[2 * k + 1] = sign * sin(a);
    }
}

static void make_rev(size_t *rev, size_t m) {
    size_t bits = 0;
    while (((size_t)1 << bits) < m) ++bits;
    for (size_t i = 0; i < m; ++i) {
        size_t r = 0, x = i;
        for (size_t b = 0; b < bits; ++b) { r = (r << 1) | (x & 1); x >>= 1; }
        rev[i] = r;
    }
}

/* In-place radix-2 on buf (already bit-reversed), using twiddle table tw of length m/2. */
static void radix2(double *buf, size_t m, const double *tw) {
    for (size_t len = 2; len <= m; len <<= 1) {
        size_t half = len >> 1, step = m / len;
        for (size_t start = 0; start < m; start += len) {
            for (size_t j = 0; j < half; ++j) {
                const double wr = tw[2 * j * step], wi = tw[2 * j * step + 1];
                double *a = buf + 2 * (start + j);
                double *b = buf + 2 * (start + j + half);
                const double br = b[0] * wr - b[1] * wi;
                const double bi = b[0] * wi + b[1] * wr;
                b[0] = a[0] - br; b[1] = a[1] - bi;
                a[0] += br; a[1] += bi;
            }
        }
    }
}

static void core(const fft64_plan *p, const double *tw, const double *in, double *out) {
    /* out must not alias in */
    for (size_t i = 0; i < p->m; ++i) {
        out[2 * p->rev[i]] = in[2 * i];
        out[2 * p->rev[i] + 1] = in[2 * i + 1];
    }
    radix2(out, p->m, tw);
}

fft64_plan *fft64_create(size_t n, int sign) {
    if (n == 0 || (sign != 1 && sign != -1)) return NULL;
    fft64_plan *p = (fft64_plan *)calloc(1, sizeof(fft64_plan));
    if (!p) return NULL;
    p->n = n;
    p->sign = sign;
    if (is_pow2(n)) {
        p->m = n;
    } else {
        size_t m = 1;
        while (m < 2 * n - 1) m <<= 1;
        p->m = m;
    }
    p->tw = (double *)malloc(sizeof(double) * (p->m > 1 ? p->m : 2));
    p->rev = (size_t *)malloc(sizeof(size_t) * p->m);
    p->work = (double *)malloc(sizeof(double) * 2 * p->m);
    if (!p->tw || !p->rev || !p->work) { fft64_destroy(p); return NULL; }
    make_rev(p->rev, p->m);
    if (is_pow2(n)) {
        make_twiddles(p->tw, p->m, sign);
        return p;
    }
    /* Bluestein: exp(s*2pi*i*jk/n) = c_j c_k conj(c_{k-j}), c_j = exp(s*pi*i*j^2/n). */
    make_twiddles(p->tw, p->m, -1);
    p->tw_inv = (double *)malloc(sizeof(double) * p->m);
    p->chirp = (double *)malloc(sizeof(double) * 2 * n);
    p->kernel = (double *)malloc(sizeof(double) * 2 * p->m);
    double *tmp = (double *)calloc(2 * p->m, sizeof(double));
    if (!p->tw_inv || !p->chirp || !p->kernel || !tmp) { free(tmp); fft64_destroy(p); return NULL; }
    make_twiddles(p->tw_inv, p->m, +1);
    const uint64_t two_n = 2 * (uint64_t)n;
    for (size_t j = 0; j < n; ++j) {
        uint64_t q = ((uint64_t)j * (uint64_t)j) % two_n;   /* exact angle index */
        double a = M_PI * (double)q / (double)n;
        p->chirp[2 * j] = cos(a);
        p->chirp[2 * j + 1] = sign * sin(a);
    }
    /* b_m = conj(c_m) for m in (-(n-1), n-1), wrapped into length m */
    for (size_t j = 0; j < n; ++j) {
        tmp[2 * j] = p->chirp[2 * j];
        tmp[2 * j + 1] = -p->chirp[2 * j + 1];
        if (j) {
            tmp[2 * (p->m - j)] = p->chirp[2 * j];
            tmp[2 * (p->m - j) + 1] = -p->chirp[2 * j + 1];
        }
    }
    core(p, p->tw, tmp, p->kernel);
    free(tmp);
    return p;
}

void fft64_execute(const fft64_plan *p, const double *in, double *out) {
    if (p->m == p->n) {
        core(p, p->tw, in, p->work);
        memcpy(out, p->work, sizeof(double) * 2 * p->n);
        return;
    }
    const size_t n = p->n, m = p->m;
    double *a = (double *)calloc(2 * m, sizeof(double));
    double *fa = (double *)malloc(sizeof(double) * 2 * m);
    if (!a || !fa) { free(a); free(fa); return; }
    for (size_t j = 0; j < n; ++j) {
        const double xr = in[2 * j], xi = in[2 * j + 1];
        const double cr = p->chirp[2 * j], ci = p->chirp[2 * j + 1];
        a[2 * j] = xr * cr - xi * ci;
        a[2 * j + 1] = xr * ci + xi * cr;
    }
    core(p, p->tw, a, fa);
    for (size_t k = 0; k < m; ++k) {
        const double xr = fa[2 * k], xi = fa[2 * k + 1];
        const double kr = p->kernel[2 * k], ki = p->kernel[2 * k + 1];
        a[2 * k] = xr * kr - xi * ki;
        a[2 * k + 1] = xr * ki + xi * kr;
    }
    core(p, p->tw_inv, a, fa);
    const double inv_m = 1.0 / (double)m;
    for (size_t k = 0; k < n; ++k) {
        const double xr = fa[2 * k] * inv_m, xi = fa[2 * k + 1] * inv_m;
        const double cr = p->chirp[2 * k], ci = p->chirp[2 * k + 1];
        out[2 * k] = xr * cr - xi * ci;
        out[2 * k + 1] = xr * ci + xi * cr;
    }
    free(a);
    free(fa);
}

void fft64_destroy(fft64_plan *p) {
    if (!p) return;
    free(p->tw);
    free(p->rev);
    free(p->work);
    free(p->chirp);
    free(p->kernel);
    free(p->tw_inv);
    free(p);
}
