// sar_host_prep.h -- FP64 host preparation of the per-pulse and per-grid constants that the
// kernels consume as double-float (hi + lo FP32) values.  Host-only; included by the plan
// code (sar_plan.cu) and by the host evaluation harness (geom_host.cpp).
#pragma once

#include <math.h>
#include <stddef.h>

#include "sar_geom.cuh"

namespace sar {

static inline df to_df(double x) {
    df r;
    r.hi = (float)x;
    r.lo = (float)(x - (double)r.hi);
    return r;
}

static inline df3 to_df3(const double* v) {
    df3 r;
    r.x = to_df(v[0]);
    r.y = to_df(v[1]);
    r.z = to_df(v[2]);
    return r;
}

static inline double dist3(const double* a, const double* b) {
    double d = 0.0;
    for (int i = 0; i < 3; ++i) d += (a[i] - b[i]) * (a[i] - b[i]);
    return sqrt(d);
}

// Per-pulse table: antennas relative to `origin`, reference range to the SRP
// (sarsolver_cxx.cpp:283 / :330), monostatic flag when tx and rx coincide exactly.
static inline PulseGeom make_pulse_geom(const double* tx, const double* rx, const double* srp,
                                        const double* origin) {
    PulseGeom g;
    for (int i = 0; i < 3; ++i) {
        df a = to_df(tx[i] - origin[i]);
        df b = to_df(rx[i] - origin[i]);
        g.atx_hi[i] = a.hi;
        g.atx_lo[i] = a.lo;
        g.arx_hi[i] = b.hi;
        g.arx_lo[i] = b.lo;
    }
    df rr = to_df(dist3(tx, srp) + dist3(rx, srp));
    g.rref_hi = rr.hi;
    g.rref_lo = rr.lo;
    g.monostatic = (tx[0] == rx[0] && tx[1] == rx[1] && tx[2] == rx[2]) ? 1.0f : 0.0f;
    g.pad = 0.0f;
    return g;
}

static inline GridConst make_grid_const(const double* ex, const double* ey, const double* ez,
                                        double kappa, double s_r, float bin_offset, int nx, int ny,
                                        int nz) {
    GridConst g;
    g.ex = to_df3(ex);
    g.ey = to_df3(ey);
    g.ez = to_df3(ez);
    g.exx = (float)(ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2]);
    g.exy = (float)(ex[0] * ey[0] + ex[1] * ey[1] + ex[2] * ey[2]);
    g.eyy = (float)(ey[0] * ey[0] + ey[1] * ey[1] + ey[2] * ey[2]);
    g.kappa = to_df(kappa);
    g.s_r = to_df(s_r);
    g.bin_offset = bin_offset;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.tiles_x = (nx + 31) / 32;
    g.tiles_y = (ny + 31) / 32;
    g.precise_bins = 0;
    return g;
}

// Minimum and maximum distance from point a to the parallelepiped
// {o + u*ex + v*ey + w*ez : 0 <= u <= nu, 0 <= v <= nv, 0 <= w <= nw} with mutually orthogonal
// (or zero) edge vectors; the minimum is exact for orthogonal edges, the maximum is over the
// corners.  Used to bound the range window of the whole grid and of tile strips.
static inline void box_distance_bounds(const double* a, const double* o, const double* ex,
                                       const double* ey, const double* ez, double nu, double nv,
                                       double nw, double* dmin, double* dmax) {
    const double* e[3] = {ex, ey, ez};
    const double n[3] = {nu, nv, nw};
    double rel[3] = {a[0] - o[0], a[1] - o[1], a[2] - o[2]};
    double closest[3] = {o[0], o[1], o[2]};
    for (int ax = 0; ax < 3; ++ax) {
        double ee = e[ax][0] * e[ax][0] + e[ax][1] * e[ax][1] + e[ax][2] * e[ax][2];
        if (ee <= 0.0 || n[ax] <= 0.0) continue;
        double t = (rel[0] * e[ax][0] + rel[1] * e[ax][1] + rel[2] * e[ax][2]) / ee;
        if (t < 0.0) t = 0.0;
        if (t > n[ax]) t = n[ax];
        for (int c = 0; c < 3; ++c) closest[c] += t * e[ax][c];
    }
    *dmin = dist3(a, closest);
    double best = 0.0;
    for (int corner = 0; corner < 8; ++corner) {
        double p[3] = {o[0], o[1], o[2]};
        for (int ax = 0; ax < 3; ++ax) {
            double t = (corner >> ax & 1) ? n[ax] : 0.0;
            for (int c = 0; c < 3; ++c) p[c] += t * e[ax][c];
        }
        double d = dist3(a, p);
        if (d > best) best = d;
    }
    *dmax = best;
}

// 1 when range bins change more slowly along the grid's y axis than along x, at the grid centre
// and summed over the pulses (|d bin / d i| vs |d bin / d j| up to the common factor s_r): the
// backprojection gather then runs its lanes along y (BpGridArgs::lanes_y).
static inline int choose_lanes_y(const double* tx, const double* rx, size_t S, const double* origin,
                                 const double* ex, const double* ey, const double* ez, int nx, int ny, int nz) {
    double c[3];
    for (int d = 0; d < 3; ++d)
        c[d] = origin[d] + 0.5 * ((nx - 1) * ex[d] + (ny - 1) * ey[d] + (nz - 1) * ez[d]);
    double rate_x = 0.0, rate_y = 0.0;
    for (size_t s = 0; s < S; ++s) {
        double gx = 0.0, gy = 0.0;
        for (int ant = 0; ant < 2; ++ant) {
            const double* a = (ant ? rx : tx) + 3 * s;
            const double w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            const double n = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            if (!(n > 0.0)) continue;
            gx += (w[0] * ex[0] + w[1] * ex[1] + w[2] * ex[2]) / n;
            gy += (w[0] * ey[0] + w[1] * ey[1] + w[2] * ey[2]) / n;
        }
        if (isfinite(gx) && isfinite(gy)) {
            rate_x += fabs(gx);
            rate_y += fabs(gy);
        }
    }
    return rate_y < rate_x ? 1 : 0;
}

// Half-span (bins) of a tile's window from the look directions: for a pixel at d = di ex + dj ey
// from its tile's centre c (|di|, |dj| <= tile / 2 = 16) and an antenna a, | |a - p| - |a - c| | <=
// |u.d| + |d|^2 / (2 R) with u the unit vector from c to a and R the antenna's distance from the
// scene; u at a tile centre differs from u0 at the scene centre by at most D / R (D: the
// scene's half-extent; c is the mean of the tile's sub-tile anchors, the point the window is
// centred on), so per antenna the change is at most 16 (|u0.ex| + |u0.ey|) +
// 16 (|ex| + |ey|) D / R + (16 (|ex| + |ey|))^2 / (2 R).  Returns -1 when an antenna is not
// clear of the scene (the isotropic bound 16 (|ex| + |ey|) per antenna then applies).
static inline double tile_halfspan_directional(const double* tx, const double* rx, size_t S, const double* origin,
                                               const double* ex, const double* ey, const double* ez, int tile,
                                               int tiles_x, int tiles_y, int nz, double s_r) {
    const double nex = sqrt(ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2]);
    const double ney = sqrt(ey[0] * ey[0] + ey[1] * ey[1] + ey[2] * ey[2]);
    const double nez = sqrt(ez[0] * ez[0] + ez[1] * ez[1] + ez[2] * ez[2]);
    double c0[3];
    for (int c = 0; c < 3; ++c)
        c0[c] = origin[c] + 0.5 * (tiles_x * tile - 1) * ex[c] + 0.5 * (tiles_y * tile - 1) * ey[c] +
                0.5 * (nz - 1) * ez[c];
    const double D = 0.5 * (tiles_x * tile * nex + tiles_y * tile * ney + nz * nez);
    const double half = 0.5 * tile, reach = half * (nex + ney);
    double worst = 0.0;
    for (size_t s = 0; s < S; ++s) {
        double h = 0.0;
        for (int ant = 0; ant < 2; ++ant) {
            const double* a = (ant ? rx : tx) + 3 * s;
            double u[3], r = 0.0;
            for (int c = 0; c < 3; ++c) {
                u[c] = a[c] - c0[c];
                r += u[c] * u[c];
            }
            r = sqrt(r);
            const double R = r - D - reach;
            if (!(R > 0.0)) return -1.0;
            double ux = 0.0, uy = 0.0;
            for (int c = 0; c < 3; ++c) {
                ux += u[c] * ex[c] / r;
                uy += u[c] * ey[c] / r;
            }
            h += half * (fabs(ux) + fabs(uy)) + reach * D / R + reach * reach / (2.0 * R);
        }
        if (h > worst) worst = h;
    }
    return worst * s_r;
}

}  // namespace sar
