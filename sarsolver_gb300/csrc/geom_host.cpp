// geom_host.cpp -- host build of the kernels' range geometry (sar_geom.cuh).
//
// Evaluates, with exactly the tiling and arithmetic the GPU kernels use (32x32 tiles, four
// 16x16 sub-tiles, per-(sub-tile, pulse) cubic expansion, per-column/per-pixel FP32
// evaluation), the phase (cycles, reduced to [-0.5, 0.5]) and the bin position of every
// grid pixel for every pulse.  Tests compare these with FP64 ranges to bound the error of
// the fast path without a GPU.
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "sar_geom.cuh"
#include "sar_host_prep.h"

using namespace sar;

// transposed: the forward scatter's other layout, where a thread holds dj and walks di
// (row_terms); otherwise a thread holds di and walks dj (column_terms), as the backprojection
// and the default scatter layout do.
// shear != 0: the forward scatter's sheared lattice (make_lattice_const); every lattice pixel that
// is an image pixel writes that image pixel's entry.
static int geom_host_eval(const double* origin, const double* ex, const double* ey, const double* ez, int nx,
                          int ny, int nz, size_t num_pulses, const double* tx, const double* rx,
                          const double* srp, double kappa, double s_r, float bin_offset, int precise_bins,
                          bool transposed, float* phase_out, double* bin_out, int shear = 0) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return 1;
    GridConst g = make_lattice_const(ex, ey, ez, kappa, s_r, bin_offset, nx, ny, nz, shear);
    g.precise_bins = precise_bins;
    const int lnx = g.nx;   // lattice width
    const size_t P = (size_t)nx * ny * nz;
    for (size_t s = 0; s < num_pulses; ++s) {
        PulseGeom pg = make_pulse_geom(tx + 3 * s, rx + 3 * s, srp + 3 * s, origin);
        for (int k = 0; k < nz; ++k)
            for (int tj = 0; tj < g.tiles_y; ++tj)
                for (int ti = 0; ti < g.tiles_x; ++ti) {
                    Coeffs co[4];
                    AnchorExpansion ae[4];
                    df vb[4];
                    df vsum = df_make(0.0f, 0.0f);
                    for (int q = 0; q < 4; ++q) {
                        int ai = ti * 32 + 8 + 16 * (q & 1) + g.a_off;
                        int aj = tj * 32 + 8 + 16 * (q >> 1);
                        df3 anchor = pixel_position(ai, aj, k, g);
                        ae[q] = expand_anchor(anchor, pg, g);
                        phase_coeffs(ae[q], g, co[q].c);
                        vb[q] = anchor_bin(ae[q], g);
                        vsum = df_add(vsum, vb[q]);
                    }
                    int base = base_bin_of(vsum, 4.0f);
                    for (int q = 0; q < 4; ++q) bin_coeffs(ae[q], vb[q], base, g, co[q]);
                    for (int lj = 0; lj < 32; ++lj)
                        for (int li = 0; li < 32; ++li) {
                            int i = ti * 32 + li, j = tj * 32 + lj;
                            if (i >= lnx || j >= ny) continue;
                            i += g.a_off + g.shear * j;   // the image pixel
                            if (i < 0 || i >= nx) continue;
                            int q = (li >= 16) + 2 * (lj >= 16);
                            float di = (float)(li - 8 - 16 * (q & 1));
                            float dj = (float)(lj - 8 - 16 * (q >> 1));
                            const bool pr = g.precise_bins != 0;
                            // u: the offset a thread holds, d: the one it walks
                            const float u = transposed ? dj : di, d = transposed ? di : dj;
                            ColumnTerms ct;
                            if (transposed)
                                ct = pr ? row_terms<true>(co[q], u, u * u, u * u * u)
                                        : row_terms<false>(co[q], u, u * u, u * u * u);
                            else
                                ct = pr ? column_terms<true>(co[q], u, u * u, u * u * u)
                                        : column_terms<false>(co[q], u, u * u, u * u * u);
                            const float c9 = transposed ? co[q].c[6] : co[q].c[9];
                            const float w9 = transposed ? co[q].w[0] : co[q].w[3];
                            const float ib = transposed ? co[q].ia : co[q].ib;
                            float ph = pixel_phase(ct, c9, d, d * d, d * d * d);
                            float v = pr ? pixel_bin<true>(ct, w9, d, d * d, d * d * d)
                                         : pixel_bin<false>(ct, 0.0f, d, d * d, d * d * d);
                            size_t p = ((size_t)k * ny + j) * nx + i;
                            phase_out[s * P + p] = ph - round_shift(ph);
                            // the kernels' bin index and in-bin coordinate, recombined
                            BinPos bp = pr ? bin_position<true>(v, fmaf(ib, d, ct.ci))
                                           : bin_position<false>(v, 0.0f);
                            bin_out[s * P + p] = (double)base + (double)bp.n + (double)bp.s;
                        }
                }
    }
    return 0;
}

extern "C" int sar_geom_host_eval(const double* origin, const double* ex, const double* ey,
                                  const double* ez, int nx, int ny, int nz, size_t num_pulses,
                                  const double* tx, const double* rx, const double* srp,
                                  double kappa, double s_r, float bin_offset, int precise_bins,
                                  float* phase_out, double* bin_out) {
    return geom_host_eval(origin, ex, ey, ez, nx, ny, nz, num_pulses, tx, rx, srp, kappa, s_r, bin_offset,
                          precise_bins, false, phase_out, bin_out);
}

extern "C" int sar_geom_host_eval_transposed(const double* origin, const double* ex, const double* ey,
                                             const double* ez, int nx, int ny, int nz, size_t num_pulses,
                                             const double* tx, const double* rx, const double* srp,
                                             double kappa, double s_r, float bin_offset, int precise_bins,
                                             float* phase_out, double* bin_out) {
    return geom_host_eval(origin, ex, ey, ez, nx, ny, nz, num_pulses, tx, rx, srp, kappa, s_r, bin_offset,
                          precise_bins, true, phase_out, bin_out);
}

// Unstructured-position scheme: phase (cycles, [-0.5, 0.5]) and bin position per point.
extern "C" int sar_geom_host_eval_sheared(const double* origin, const double* ex, const double* ey,
                                         const double* ez, int nx, int ny, int nz, size_t num_pulses,
                                         const double* tx, const double* rx, const double* srp, double kappa,
                                         double s_r, float bin_offset, int precise_bins, int shear,
                                         float* phase_out, double* bin_out) {
    return geom_host_eval(origin, ex, ey, ez, nx, ny, nz, num_pulses, tx, rx, srp, kappa, s_r, bin_offset,
                          precise_bins, false, phase_out, bin_out, shear);
}

// The same lattice in the backprojection's layout there (a thread holds the offset along the
// lattice's second axis, its lanes' axis, and evaluates along x).
extern "C" int sar_geom_host_eval_sheared_lanes(const double* origin, const double* ex, const double* ey,
                                               const double* ez, int nx, int ny, int nz, size_t num_pulses,
                                               const double* tx, const double* rx, const double* srp, double kappa,
                                               double s_r, float bin_offset, int precise_bins, int shear,
                                               float* phase_out, double* bin_out) {
    return geom_host_eval(origin, ex, ey, ez, nx, ny, nz, num_pulses, tx, rx, srp, kappa, s_r, bin_offset,
                          precise_bins, true, phase_out, bin_out, shear);
}

extern "C" int sar_choose_gather_shear_host(const double* tx, const double* rx, size_t num_pulses,
                                            const double* origin, const double* ex, const double* ey,
                                            const double* ez, int nx, int ny, int nz, double s_r) {
    return choose_gather_shear(tx, rx, num_pulses, origin, ex, ey, ez, nx, ny, nz, s_r);
}

// The forward scatter's shear choice (choose_shear) and the parallelogram distance bound of its
// lattice strips, for tests.
extern "C" int sar_choose_shear_host(const double* tx, const double* rx, size_t num_pulses, const double* origin,
                                     const double* ex, const double* ey, const double* ez, int nx, int ny, int nz,
                                     double s_r) {
    return choose_shear(tx, rx, num_pulses, origin, ex, ey, ez, nx, ny, nz, s_r,
                        choose_lanes_y(tx, rx, num_pulses, origin, ex, ey, ez, nx, ny, nz));
}

extern "C" void sar_parallelogram_distance_host(const double* a, const double* o, const double* e1, const double* e2,
                                                double* dmin, double* dmax) {
    parallelogram_distance_bounds(a, o, e1, e2, dmin, dmax);
}

extern "C" int sar_geom_host_eval_points(const double* origin, size_t num_points, const double* pos,
                                         size_t num_pulses, const double* tx, const double* rx,
                                         const double* srp, double kappa, double s_r,
                                         float bin_offset, float* phase_out, double* bin_out) {
    df kap = to_df(kappa), sr = to_df(s_r);
    for (size_t s = 0; s < num_pulses; ++s) {
        PulseGeom pg = make_pulse_geom(tx + 3 * s, rx + 3 * s, srp + 3 * s, origin);
        df3 at = pulse_tx(pg), ar = pulse_rx(pg);
        df at2 = df_dot3(at, at), ar2 = df_dot3(ar, ar);
        for (size_t p = 0; p < num_points; ++p) {
            PointGeom pt;
            double q[3] = {pos[3 * p] - origin[0], pos[3 * p + 1] - origin[1], pos[3 * p + 2] - origin[2]};
            double qq = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
            for (int c = 0; c < 3; ++c) {
                df d = to_df(q[c]);
                pt.qh[c] = d.hi;
                pt.ql[c] = d.lo;
            }
            df d2 = to_df(qq);
            pt.qh[3] = d2.hi;
            pt.ql[3] = d2.lo;
            df r = point_range(at, at2, pt);
            r = df_add(r, pg.monostatic != 0.0f ? r : point_range(ar, ar2, pt));
            r = df_sub(r, df_make(pg.rref_hi, pg.rref_lo));
            phase_out[s * num_points + p] = df_frac(df_mul(kap, r));
            // the kernel's bin rule: bin_offset -0.5 linear, +0.5 adjoint nearest, 0 forward nearest
            const df v = df_mul(sr, r);
            const int rule = bin_offset < 0.0f ? BIN_LINEAR : (bin_offset > 0.0f ? BIN_ADJ_NEAREST : BIN_FWD_NEAREST);
            int gi;
            float sf;
            exact_bin(v, 0, rule, &gi, &sf);
            // linear: position of v itself; nearest: the chosen bin (+0.5 for the adjoint rule so
            // that round() of the result reproduces the kernel's choice, as for FP64 v + 0.5)
            bin_out[s * num_points + p] = rule == BIN_LINEAR ? (double)gi + (double)sf + 0.5
                                                             : (double)gi + (rule == BIN_ADJ_NEAREST ? 0.0 : 0.0);
        }
    }
    return 0;
}

// Half-span (bins) of the gather's tile window from the look directions, as the plan computes it
// (tile_halfspan_directional); -1 where an antenna is not clear of the scene.
extern "C" double sar_tile_halfspan_host(const double* tx, const double* rx, size_t num_pulses, const double* origin,
                                         const double* ex, const double* ey, const double* ez, int tiles_x,
                                         int tiles_y, int nz, double s_r) {
    return tile_halfspan_directional(tx, rx, num_pulses, origin, ex, ey, ez, 32, tiles_x, tiles_y, nz, s_r);
}

// The gather producer's window check on the host: for every (tile, pulse) pair of the given pulses,
// the sub-tile coefficient sets and base bin exactly as the kernel forms them, then bin_extent
// against a staged window of ww bins.  Returns the number of sets that would raise
// FLAG_GATHER_WINDOW, and in *needed_half the smallest half-window (bins) that covers them all.
extern "C" long sar_gather_window_check_host(const double* origin, const double* ex, const double* ey,
                                             const double* ez, int nx, int ny, int nz, size_t num_pulses,
                                             const double* tx, const double* rx, const double* srp, double kappa,
                                             double s_r, float bin_offset, int precise_bins, int ww,
                                             double* needed_half) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return -1;
    GridConst g = make_grid_const(ex, ey, ez, kappa, s_r, bin_offset, nx, ny, nz);
    g.precise_bins = precise_bins;
    const float half = 0.5f * (float)ww;
    long bad = 0;
    double need = 0.0;
    for (size_t s = 0; s < num_pulses; ++s) {
        PulseGeom pg = make_pulse_geom(tx + 3 * s, rx + 3 * s, srp + 3 * s, origin);
        for (int k = 0; k < nz; ++k)
            for (int tj = 0; tj < g.tiles_y; ++tj)
                for (int ti = 0; ti < g.tiles_x; ++ti) {
                    Coeffs co[4];
                    AnchorExpansion ae[4];
                    df vb[4];
                    df vsum = df_make(0.0f, 0.0f);
                    for (int q = 0; q < 4; ++q) {
                        df3 anchor = pixel_position(ti * 32 + 8 + 16 * (q & 1), tj * 32 + 8 + 16 * (q >> 1), k, g);
                        ae[q] = expand_anchor(anchor, pg, g);
                        vb[q] = anchor_bin(ae[q], g);
                        vsum = df_add(vsum, vb[q]);
                    }
                    const int base = base_bin_of(vsum, 4.0f);
                    for (int q = 0; q < 4; ++q) {
                        co[q] = Coeffs{};
                        bin_coeffs(ae[q], vb[q], base, g, co[q]);
                        float lo, hi;
                        bin_extent(co[q], &lo, &hi);
                        if (!(lo >= -half - 0.49f && hi <= half - 0.51f)) ++bad;
                        need = fmax(need, fmax(-(double)lo - 0.49, (double)hi + 0.51));
                    }
                }
    }
    if (needed_half) *needed_half = need;
    return bad;
}

// bin_extent of the coefficient set of sub-tile q of tile (ti, tj, k) for one pulse (lo, hi), and
// the extreme bins the kernels' per-pixel evaluation actually forms over that sub-tile (both
// relative to the tile's base bin), to check that the bound holds.
extern "C" int sar_bin_extent_host(const double* origin, const double* ex, const double* ey, const double* ez,
                                   int nx, int ny, int nz, const double* tx, const double* rx, const double* srp,
                                   double kappa, double s_r, float bin_offset, int precise_bins, int ti, int tj,
                                   int k, int q, double* out4) {
    GridConst g = make_grid_const(ex, ey, ez, kappa, s_r, bin_offset, nx, ny, nz);
    g.precise_bins = precise_bins;
    PulseGeom pg = make_pulse_geom(tx, rx, srp, origin);
    AnchorExpansion ae[4];
    df vb[4];
    df vsum = df_make(0.0f, 0.0f);
    for (int r = 0; r < 4; ++r) {
        df3 anchor = pixel_position(ti * 32 + 8 + 16 * (r & 1), tj * 32 + 8 + 16 * (r >> 1), k, g);
        ae[r] = expand_anchor(anchor, pg, g);
        vb[r] = anchor_bin(ae[r], g);
        vsum = df_add(vsum, vb[r]);
    }
    const int base = base_bin_of(vsum, 4.0f);
    Coeffs co{};
    phase_coeffs(ae[q], g, co.c);
    bin_coeffs(ae[q], vb[q], base, g, co);
    float lo, hi;
    bin_extent(co, &lo, &hi);
    double vmin = 1e300, vmax = -1e300;
    const bool pr = precise_bins != 0;
    for (int a = -8; a < 8; ++a)
        for (int b = -8; b < 8; ++b) {
            const float di = (float)a, dj = (float)b;
            ColumnTerms ct = pr ? column_terms<true>(co, di, di * di, di * di * di)
                                : column_terms<false>(co, di, di * di, di * di * di);
            const float v = pr ? pixel_bin<true>(ct, co.w[3], dj, dj * dj, dj * dj * dj)
                               : pixel_bin<false>(ct, 0.0f, dj, dj * dj, dj * dj * dj);
            const double tot = (double)v + (pr ? (double)fmaf(co.ib, dj, ct.ci) : 0.0);
            vmin = fmin(vmin, tot);
            vmax = fmax(vmax, tot);
        }
    out4[0] = lo;
    out4[1] = hi;
    out4[2] = vmin;
    out4[3] = vmax;
    return 0;
}
