// sar_geom.cuh -- range geometry shared by every SAR kernel (host and device).
//
// The reference forms the differential bistatic range in FP64 per pixel and pulse
// (src/sarsolver/cxx_binding/sarsolver_cxx.cpp:10-20, :283, :287):
//     dR(p, s) = |tx_s - p| + |rx_s - p| - (|tx_s - srp_s| + |rx_s - srp_s|)
// and uses it twice: the phase k*dR with k = 2*pi*sign*fc/c_eff (:228) and the range bin
// dR * s_r with s_r = fs*M/(N*c_eff) (:225-226).  At kilometre stand-off the phase is
// ~1e5 rad and must stay within ~1e-5 rad, which FP32 cannot carry.  Two precision schemes:
//
// 1. Regular grids (the fast path).  For each 16x16 pixel sub-tile and pulse, dR around the
//    sub-tile's anchor pixel is expanded to third order in the integer pixel offsets
//    (di, dj):  dR = dR0 + gx di + gy dj + quadratic + cubic terms, Taylor series of |w + d|
//    (w = anchor - antenna, d = di*ex + dj*ey).  The anchor range and the gradient are formed
//    in double-float (hi + lo FP32 pairs, error-free transforms), then scaled to cycles and
//    reduced modulo one cycle: because di and dj are integers, frac(kappa*gx) may replace
//    kappa*gx without changing exp(2*pi*i*phase).  Each pixel then costs a handful of FP32
//    FMAs for the phase (magnitude < 9 cycles) and the bin position (< 64 bins), with no
//    square root.  The quartic remainder is < 1e-10 m for |d| < 3 m at 10 km.
// 2. Unstructured positions.  Per pixel and pulse: W = |alpha|^2 - 2 alpha.q + |q|^2 in
//    double-float (alpha = antenna - origin, q = pixel - origin), its square root by one
//    Newton step, then the same mod-1 reduction of the phase.
//
// Everything here is plain IEEE FP32 arithmetic with explicit fmaf and correctly rounded
// sqrtf / division, so the host build (geom_host.cpp) reproduces the device numbers and the
// precision can be checked against FP64 without a GPU.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SAR_HD __host__ __device__ __forceinline__
#else
#define SAR_HD static inline
#endif

namespace sar {

// ------------------------------------------------------------------ double-float
struct df {
    float hi, lo;
};
struct df3 {
    df x, y, z;
};

SAR_HD df df_make(float hi, float lo) {
    df r;
    r.hi = hi;
    r.lo = lo;
    return r;
}
// Knuth TwoSum: s + e == a + b exactly.
SAR_HD df two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return df_make(s, e);
}
// Dekker FastTwoSum, requires |a| >= |b| (or a == 0).
SAR_HD df fast_two_sum(float a, float b) {
    float s = a + b;
    float e = b - (s - a);
    return df_make(s, e);
}
// Exact product via FMA.
SAR_HD df two_prod(float a, float b) {
    float p = a * b;
    float e = fmaf(a, b, -p);
    return df_make(p, e);
}
SAR_HD df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    float e = s.lo + (a.lo + b.lo);
    return fast_two_sum(s.hi, e);
}
SAR_HD df df_neg(df a) { return df_make(-a.hi, -a.lo); }
SAR_HD df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
SAR_HD df df_mul(df a, df b) {
    df p = two_prod(a.hi, b.hi);
    float e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, e);
}
SAR_HD df df_mulf(df a, float b) {
    df p = two_prod(a.hi, b);
    float e = fmaf(a.lo, b, p.lo);
    return fast_two_sum(p.hi, e);
}
// Approximate reciprocal and reciprocal square root (about 1 ulp): the hardware approximations
// on the device, correctly rounded equivalents on the host.  The double-float routines below
// only use them as starting points and correct the result with one exact residual, so the
// double-float accuracy does not depend on their last bit.
SAR_HD float approx_rcp(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}
SAR_HD float approx_rsqrt(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / sqrtf(x);
#endif
}
// sqrt(a) for a.hi > 0: r0 = a.hi * rsqrt(a.hi), then the Newton correction
// (a - r0^2) / (2 r0) from the exact FMA residual (Karp-Markstein form).
SAR_HD df df_sqrt(df a) {
    const float y = approx_rsqrt(a.hi);
    const float r = a.hi * y;
    const float e = fmaf(-r, r, a.hi) + a.lo;
    return fast_two_sum(r, e * (0.5f * y));
}
// a / b: q1 = a.hi / b.hi from the approximate reciprocal, then the correction from the
// double-float residual a - b q1 (Markstein-style refinement).
SAR_HD df df_div(df a, df b) {
    const float inv = approx_rcp(b.hi);
    const float q1 = a.hi * inv;
    const df r = df_sub(a, df_mulf(b, q1));
    const float q2 = r.hi * inv;
    return fast_two_sum(q1, q2);
}
SAR_HD df df_dot3(const df3& a, const df3& b) {
    df s = df_mul(a.x, b.x);
    s = df_add(s, df_mul(a.y, b.y));
    return df_add(s, df_mul(a.z, b.z));
}
SAR_HD df3 df3_sub(const df3& a, const df3& b) {
    df3 r;
    r.x = df_sub(a.x, b.x);
    r.y = df_sub(a.y, b.y);
    r.z = df_sub(a.z, b.z);
    return r;
}
// Integer multiple of a df vector, n exactly representable (|n| < 2^24).
SAR_HD df3 df3_scale_int(const df3& a, float n) {
    df3 r;
    r.x = df_mulf(a.x, n);
    r.y = df_mulf(a.y, n);
    r.z = df_mulf(a.z, n);
    return r;
}
SAR_HD df3 df3_add(const df3& a, const df3& b) {
    df3 r;
    r.x = df_add(a.x, b.x);
    r.y = df_add(a.y, b.y);
    r.z = df_add(a.z, b.z);
    return r;
}
// Round to nearest integer (ties to even) for |x| < 2^22 via the 1.5*2^23 shifter: keeps the
// work on the FP32 pipe and leaves the integer in the low mantissa bits.
#define SAR_SHIFTER 12582912.0f
#define SAR_SHIFTER_BITS 0x4B400000
SAR_HD float round_shift(float x) { return (x + SAR_SHIFTER) - SAR_SHIFTER; }
// Fractional part in [-0.5, 0.5] of a df value (|value| < 2^22).
SAR_HD float df_frac(df a) {
    float n = round_shift(a.hi);
    return (a.hi - n) + a.lo;
}

// ------------------------------------------------------------------ constants
// Per-pulse geometry, everything relative to one origin (the grid's first pixel, or the
// centre of an unstructured scene's bounding box).  16 floats.
struct PulseGeom {
    float atx_hi[3], atx_lo[3];   // transmitter - origin
    float arx_hi[3], arx_lo[3];   // receiver - origin
    float rref_hi, rref_lo;       // |tx - srp| + |rx - srp|
    float monostatic;             // 1 if tx == rx exactly
    float pad;
};

SAR_HD df3 pulse_tx(const PulseGeom& g) {
    df3 r;
    r.x = df_make(g.atx_hi[0], g.atx_lo[0]);
    r.y = df_make(g.atx_hi[1], g.atx_lo[1]);
    r.z = df_make(g.atx_hi[2], g.atx_lo[2]);
    return r;
}
SAR_HD df3 pulse_rx(const PulseGeom& g) {
    df3 r;
    r.x = df_make(g.arx_hi[0], g.arx_lo[0]);
    r.y = df_make(g.arx_hi[1], g.arx_lo[1]);
    r.z = df_make(g.arx_hi[2], g.arx_lo[2]);
    return r;
}

// Grid and signal constants (kernel argument by value).
struct GridConst {
    df3 ex, ey, ez;              // pixel steps along x (i), y (j), z (k) in metres
    float exx, exy, eyy;         // |ex|^2, ex.ey, |ey|^2
    df kappa;                    // cycles per metre of bistatic range: sign*fc/c_eff
    df s_r;                      // bins per metre of bistatic range: fs*M/(N*c_eff)
    float bin_offset;            // -0.5 (linear: n = floor(v)) or +0.5 (adjoint nearest: ceil)
                                 // or 0 (forward nearest: round)
    int nx, ny, nz;              // grid shape (of the lattice, for a sheared one)
    int tiles_x, tiles_y;        // 32x32 tiles per plane
    int precise_bins;            // 1: integer/fraction split of the linear bin rates + cubic bin terms
    // Sheared lattice (forward scatter only): lattice pixel (a, b) is image pixel
    // (a + a_off + shear b, b), i.e. ey above holds the image's ey + shear ex, nx the lattice
    // width img_nx + |shear| (ny - 1); 0, 0, nx for the image grid itself.
    int a_off, shear, img_nx;
};

// Lattice tiles [lo, hi] of lattice column ta that hold at least one image pixel (all tiles of
// the column when the lattice is the image grid); lo > hi when none does.
SAR_HD void lattice_tile_range(const GridConst& g, int ta, int* lo, int* hi) {
    *lo = 0;
    *hi = g.tiles_y - 1;
    if (g.shear == 0) return;
    int first = g.tiles_y, last = -1;
    for (int tb = 0; tb < g.tiles_y; ++tb) {
        // image columns of the tile's pixels: a + a_off + shear b over a in [32 ta, 32 ta + 31],
        // b in [32 tb, 32 tb + 31]
        const int c0 = 32 * ta + g.a_off + g.shear * 32 * tb;
        const int lo_c = c0 + (g.shear < 0 ? 31 * g.shear : 0), hi_c = c0 + 31 + (g.shear > 0 ? 31 * g.shear : 0);
        if (lo_c <= g.img_nx - 1 && hi_c >= 0) {
            first = first < tb ? first : tb;
            last = tb;
        }
    }
    *lo = first;
    *hi = last;
}

// Coefficients of one (sub-tile, pulse) pair: 16 floats.
//  phase (cycles): ph = c0 + c1 di + c2 dj + c3 di^2 + c4 di dj + c5 dj^2
//                       + c6 di^3 + c7 di^2 dj + c8 di dj^2 + c9 dj^3      (c0..c2 reduced mod 1)
//  bin:            v  = v0 + v1 di + v2 dj + v3 di^2 + v4 di dj + v5 dj^2 (relative to the tile's
//                  base bin, bin_offset already folded into v0)
//  precise bins (used where nearest-bin decisions must match FP64, or for wide tiles): v1, v2
//  hold only the fractional parts of the linear bin rates and their integer parts (ia, ib) are
//  accumulated exactly, so the FP32 part stays below ~17 bins for any upsample ratio; the
//  cubic terms w6..w9 (same monomials as c6..c9) are added, which matters at short stand-off
//  and fine bins (e.g. 2 km and upsample 128: ~2e-4 bins over a 16x16 sub-tile).
struct Coeffs {
    float c[10];
    float v[6];
    float i0, ia, ib;   // exact integer parts (precise mode)
    float w[4];
};

struct AntennaTerms {
    df R;          // |w|
    df gx, gy;     // w.ex/|w|, w.ey/|w|   (m per pixel)
    float qxx, qxy, qyy;             // quadratic coefficients (m)
    float kxxx, kxxy, kxyy, kyyy;    // cubic coefficients (m)
};

// Taylor expansion of |w + di*ex + dj*ey| about di = dj = 0.
SAR_HD AntennaTerms expand_antenna(const df3& anchor, const df3& antenna, const GridConst& g) {
    AntennaTerms t;
    df3 w = df3_sub(anchor, antenna);
    df W = df_dot3(w, w);
    t.R = df_sqrt(W);
    t.gx = df_div(df_dot3(w, g.ex), t.R);
    t.gy = df_div(df_dot3(w, g.ey), t.R);
    const float ux = t.gx.hi, uy = t.gy.hi;
    const float inv = approx_rcp(t.R.hi);
    const float pxx = g.exx - ux * ux;
    const float pxy = g.exy - ux * uy;
    const float pyy = g.eyy - uy * uy;
    // second order: (d^T P d) / (2|w|)
    t.qxx = 0.5f * pxx * inv;
    t.qxy = pxy * inv;
    t.qyy = 0.5f * pyy * inv;
    // third order: -(u.d)(d^T P d) / (2|w|^2)
    const float h = -0.5f * inv * inv;
    t.kxxx = h * ux * pxx;
    t.kxxy = h * (uy * pxx + 2.0f * ux * pxy);
    t.kxyy = h * (2.0f * uy * pxy + ux * pyy);
    t.kyyy = h * uy * pyy;
    return t;
}

// Full coefficient set for a sub-tile anchor (df3 position relative to the origin).
// Returns the anchor's absolute bin position in vbin (double-float) so the caller can pick a
// base bin; the v-coefficients are relative to base_bin, which the caller passes back in
// finish_bins() below.
struct AnchorExpansion {
    df dR;                 // differential bistatic range at the anchor (m)
    df gx, gy;             // gradient (m per pixel), summed over the two antennas
    float q[3];            // quadratic (m)
    float k[4];            // cubic (m)
};

SAR_HD AnchorExpansion expand_anchor(const df3& anchor, const PulseGeom& pg, const GridConst& g) {
    AnchorExpansion a;
    AntennaTerms t = expand_antenna(anchor, pulse_tx(pg), g);
    if (pg.monostatic != 0.0f) {
        a.dR = df_mulf(t.R, 2.0f);
        a.gx = df_mulf(t.gx, 2.0f);
        a.gy = df_mulf(t.gy, 2.0f);
        a.q[0] = 2.0f * t.qxx;
        a.q[1] = 2.0f * t.qxy;
        a.q[2] = 2.0f * t.qyy;
        a.k[0] = 2.0f * t.kxxx;
        a.k[1] = 2.0f * t.kxxy;
        a.k[2] = 2.0f * t.kxyy;
        a.k[3] = 2.0f * t.kyyy;
    } else {
        AntennaTerms r = expand_antenna(anchor, pulse_rx(pg), g);
        a.dR = df_add(t.R, r.R);
        a.gx = df_add(t.gx, r.gx);
        a.gy = df_add(t.gy, r.gy);
        a.q[0] = t.qxx + r.qxx;
        a.q[1] = t.qxy + r.qxy;
        a.q[2] = t.qyy + r.qyy;
        a.k[0] = t.kxxx + r.kxxx;
        a.k[1] = t.kxxy + r.kxxy;
        a.k[2] = t.kxyy + r.kxyy;
        a.k[3] = t.kyyy + r.kyyy;
    }
    a.dR = df_sub(a.dR, df_make(pg.rref_hi, pg.rref_lo));
    return a;
}

// Phase coefficients (cycles), reduced modulo one cycle where exact.
SAR_HD void phase_coeffs(const AnchorExpansion& a, const GridConst& g, float* c) {
    c[0] = df_frac(df_mul(g.kappa, a.dR));
    c[1] = df_frac(df_mul(g.kappa, a.gx));
    c[2] = df_frac(df_mul(g.kappa, a.gy));
    const float kap = g.kappa.hi;
    c[3] = kap * a.q[0];
    c[4] = kap * a.q[1];
    c[5] = kap * a.q[2];
    c[6] = kap * a.k[0];
    c[7] = kap * a.k[1];
    c[8] = kap * a.k[2];
    c[9] = kap * a.k[3];
}

// Absolute bin position of the anchor (double-float).
SAR_HD df anchor_bin(const AnchorExpansion& a, const GridConst& g) { return df_mul(g.s_r, a.dR); }

// Base bin of a tile from the anchor positions of its sub-tiles: floor of their mean.
SAR_HD int base_bin_of(df sum_of_bins, float count) {
    df m = df_mulf(sum_of_bins, 1.0f / count);   // count is a power of two: exact
    float f = floorf(m.hi);
    if (m.hi == f && m.lo < 0.0f) f -= 1.0f;
    return (int)f;
}

// Bin coefficients relative to base_bin, with the interpolation offset folded in.  In precise
// mode the linear rates s_r*gx, s_r*gy are formed in double-float and split into an integer
// (ia, ib) and a fraction in [-0.5, 0.5] (v[1], v[2]), and the cubic terms are kept.
SAR_HD void bin_coeffs(const AnchorExpansion& a, df vbin, int base_bin, const GridConst& g, Coeffs& co) {
    df rel = df_sub(vbin, df_make((float)base_bin, 0.0f));
    const float sr = g.s_r.hi;
    if (g.precise_bins) {
        co.i0 = round_shift(rel.hi);
        co.v[0] = ((rel.hi - co.i0) + rel.lo) + g.bin_offset;
        const df rx = df_mul(g.s_r, a.gx), ry = df_mul(g.s_r, a.gy);
        co.ia = round_shift(rx.hi);
        co.ib = round_shift(ry.hi);
        co.v[1] = (rx.hi - co.ia) + rx.lo;
        co.v[2] = (ry.hi - co.ib) + ry.lo;
        for (int i = 0; i < 4; ++i) co.w[i] = sr * a.k[i];
    } else {
        co.v[0] = (rel.hi + rel.lo) + g.bin_offset;
        co.i0 = co.ia = co.ib = 0.0f;
        co.v[1] = sr * (a.gx.hi + a.gx.lo);
        co.v[2] = sr * (a.gy.hi + a.gy.lo);
        for (int i = 0; i < 4; ++i) co.w[i] = 0.0f;
    }
    co.v[3] = sr * a.q[0];
    co.v[4] = sr * a.q[1];
    co.v[5] = sr * a.q[2];
}

// Range [lo, hi] of the bin polynomial of a coefficient set (relative to the tile's base bin,
// including the exact integer part) over the pixel offsets di, dj in [-8, 7] of a 16x16 sub-tile:
// each monomial's extreme values over that box, summed term by term (an upper bound of the true
// extent, tight for the linear terms that dominate it).  The gather uses it to prove that every
// pixel's bin lies inside its tile's staged window.
SAR_HD void bin_extent(const Coeffs& co, float* lo, float* hi) {
    // monomials di, dj, di^2, di dj, dj^2, di^3, di^2 dj, di dj^2, dj^3 over [-8, 7]^2
    const float mlo[9] = {-8.f, -8.f, 0.f, -56.f, 0.f, -512.f, -512.f, -512.f, -512.f};
    const float mhi[9] = {7.f, 7.f, 64.f, 64.f, 64.f, 343.f, 448.f, 448.f, 343.f};
    const float cf[9] = {co.v[1] + co.ia, co.v[2] + co.ib, co.v[3], co.v[4], co.v[5],
                         co.w[0], co.w[1], co.w[2], co.w[3]};
    float l = co.v[0] + co.i0, h = l;
    for (int t = 0; t < 9; ++t) {
        const float a = cf[t] * mlo[t], b = cf[t] * mhi[t];
        l += fminf(a, b);
        h += fmaxf(a, b);
    }
    *lo = l;
    *hi = h;
}

// Anchor position of pixel (i, j, k) relative to the grid origin.
SAR_HD df3 pixel_position(int i, int j, int k, const GridConst& g) {
    df3 p = df3_scale_int(g.ex, (float)i);
    p = df3_add(p, df3_scale_int(g.ey, (float)j));
    if (k != 0) p = df3_add(p, df3_scale_int(g.ez, (float)k));
    return p;
}

// ---------------------------------------------------------- per-pixel evaluation
// Column part (di fixed) and pixel part (dj varies) of the polynomials; see sar_kernels.cu.
struct ColumnTerms {
    float cph, b1, b2;   // phase: cph + b1 dj + b2 dj^2 + c9 dj^3
    float cv, bv1, bv2;  // bin:   cv + bv1 dj + bv2 dj^2 (+ w9 dj^3, and + ci + ib dj exactly, when precise)
    float ci;
};

template <bool PRECISE>
SAR_HD ColumnTerms column_terms(const Coeffs& q, float di, float di2, float di3) {
    ColumnTerms t;
    t.cph = fmaf(q.c[6], di3, fmaf(q.c[3], di2, fmaf(q.c[1], di, q.c[0])));
    t.b1 = fmaf(q.c[7], di2, fmaf(q.c[4], di, q.c[2]));
    t.b2 = fmaf(q.c[8], di, q.c[5]);
    if (PRECISE) {
        t.cv = fmaf(q.w[0], di3, fmaf(q.v[3], di2, fmaf(q.v[1], di, q.v[0])));
        t.bv1 = fmaf(q.w[1], di2, fmaf(q.v[4], di, q.v[2]));
        t.bv2 = fmaf(q.w[2], di, q.v[5]);
        t.ci = fmaf(q.ia, di, q.i0);
    } else {
        t.cv = fmaf(q.v[3], di2, fmaf(q.v[1], di, q.v[0]));
        t.bv1 = fmaf(q.v[4], di, q.v[2]);
        t.bv2 = q.v[5];
        t.ci = 0.0f;
    }
    return t;
}

// The same terms with the roles of the offsets exchanged: a thread at fixed dj walks di (rows of
// a transposed tile).  The returned polynomials are in di; the di^3 coefficients are c6 (phase)
// and w0 (split bins), and the exact integer part is i0 + ib dj + ia di.
template <bool PRECISE>
SAR_HD ColumnTerms row_terms(const Coeffs& q, float dj, float dj2, float dj3) {
    ColumnTerms t;
    t.cph = fmaf(q.c[9], dj3, fmaf(q.c[5], dj2, fmaf(q.c[2], dj, q.c[0])));
    t.b1 = fmaf(q.c[8], dj2, fmaf(q.c[4], dj, q.c[1]));
    t.b2 = fmaf(q.c[7], dj, q.c[3]);
    if (PRECISE) {
        t.cv = fmaf(q.w[3], dj3, fmaf(q.v[5], dj2, fmaf(q.v[2], dj, q.v[0])));
        t.bv1 = fmaf(q.w[2], dj2, fmaf(q.v[4], dj, q.v[1]));
        t.bv2 = fmaf(q.w[1], dj, q.v[3]);
        t.ci = fmaf(q.ib, dj, q.i0);
    } else {
        t.cv = fmaf(q.v[5], dj2, fmaf(q.v[2], dj, q.v[0]));
        t.bv1 = fmaf(q.v[4], dj, q.v[1]);
        t.bv2 = q.v[3];
        t.ci = 0.0f;
    }
    return t;
}

SAR_HD float pixel_phase(const ColumnTerms& t, float c9, float dj, float dj2, float dj3) {
    return fmaf(c9, dj3, fmaf(t.b2, dj2, fmaf(t.b1, dj, t.cph)));
}
template <bool PRECISE>
SAR_HD float pixel_bin(const ColumnTerms& t, float w9, float dj, float dj2, float dj3) {
    const float v = fmaf(t.bv2, dj2, fmaf(t.bv1, dj, t.cv));
    return PRECISE ? fmaf(w9, dj3, v) : v;
}

// Bin index n (relative to the tile base) and coordinate s in [-0.5, 0.5] about it, from the
// FP32 part v and, when split, the exact integer part ni.  (v + shifter) holds rint(v) in its
// low mantissa bits; adding the integer ni keeps the sum in [2^23, 2^24), hence exact.
struct BinPos {
    int n;
    float s;
};
template <bool PRECISE>
SAR_HD BinPos bin_position(float v, float ni) {
    const float r1 = v + SAR_SHIFTER;
    BinPos b;
    b.s = v - (r1 - SAR_SHIFTER);
    const float rr = PRECISE ? r1 + ni : r1;
#if defined(__CUDA_ARCH__)
    b.n = __float_as_int(rr) - SAR_SHIFTER_BITS;
#else
    union {
        float f;
        int32_t i;
    } u;
    u.f = rr;
    b.n = u.i - SAR_SHIFTER_BITS;
#endif
    return b;
}

// ------------------------------------------------ unstructured positions (scheme 2)
// Bin of a double-float bin position V (relative to the first stored bin base0), for the
// three sampling rules:
//   BIN_LINEAR      floor(v) and the coordinate sf = v - floor(v) - 0.5 in [-0.5, 0.5]
//   BIN_ADJ_NEAREST round(0.5 + v)   (sarsolver_cxx.cpp:347)
//   BIN_FWD_NEAREST round(v)         (sarsolver_cxx.cpp:289)
// with round() halfway cases away from zero as std::round.  n1 = rint(V.hi) is exact and
// t = V.hi - n1 is exact; the nearest-bin decisions then compare t (or t -+ 0.5, also exact)
// with -V.lo through FP32 sums whose sign is exact, so the chosen bin equals the one FP64
// rounding of the same double-float value gives, including ties.
enum BinRule { BIN_LINEAR = 0, BIN_ADJ_NEAREST = 1, BIN_FWD_NEAREST = 2 };

SAR_HD void exact_bin(df V, int base0, int rule, int* gi, float* sf) {
    const float n1 = round_shift(V.hi);
    const float t = V.hi - n1;
    const bool nonneg = (int)n1 + base0 >= 0;   // sign of the absolute bin, for halfway cases
    int n2 = 0;
    *sf = 0.0f;
    if (rule == BIN_LINEAR) {
        const float frac = t + (V.lo - 0.5f);
        const float r = round_shift(frac);
        n2 = (int)r;
        *sf = frac - r;
    } else if (rule == BIN_ADJ_NEAREST) {
        const float u = t + V.lo;          // round(0.5 + n1 + u) = n1 + [u > 0, or u == 0 and v >= 0]
        n2 = (u > 0.0f || (u == 0.0f && nonneg)) ? 1 : 0;
    } else {
        const float up = (t - 0.5f) + V.lo;    // u - 0.5
        const float dn = (t + 0.5f) + V.lo;    // u + 0.5
        if (up > 0.0f || (up == 0.0f && nonneg))
            n2 = 1;
        else if (dn < 0.0f || (dn == 0.0f && !nonneg))
            n2 = -1;
    }
    *gi = (int)n1 + n2;
}

// Per pixel: q = p - origin as hi/lo and |q|^2 as hi/lo.
struct PointGeom {
    float qh[4];   // qx, qy, qz, |q|^2 (hi)
    float ql[4];   // lo parts
};

// |alpha - q| for an antenna alpha (relative to the origin) with |alpha|^2 given.
SAR_HD df point_range(const df3& alpha, df alpha2, const PointGeom& pt) {
    df3 q;
    q.x = df_make(pt.qh[0], pt.ql[0]);
    q.y = df_make(pt.qh[1], pt.ql[1]);
    q.z = df_make(pt.qh[2], pt.ql[2]);
    df dot = df_dot3(alpha, q);
    df W = df_add(alpha2, df_make(pt.qh[3], pt.ql[3]));
    W = df_sub(W, df_mulf(dot, 2.0f));
    return df_sqrt(W);
}

}  // namespace sar
