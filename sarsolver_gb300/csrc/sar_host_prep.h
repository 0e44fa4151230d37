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
    g.a_off = 0;
    g.shear = 0;
    g.img_nx = nx;
    return g;
}

// Grid constants of the sheared lattice (steps ex, ey + shear ex) over an nx x ny x nz image:
// lattice pixel (a, b) is image pixel (a + a_off + shear b, b), a in [0, nx + |shear| (ny - 1)).
static inline GridConst make_lattice_const(const double* ex, const double* ey, const double* ez, double kappa,
                                           double s_r, float bin_offset, int nx, int ny, int nz, int shear) {
    if (shear == 0) return make_grid_const(ex, ey, ez, kappa, s_r, bin_offset, nx, ny, nz);
    double ey_l[3];
    for (int c = 0; c < 3; ++c) ey_l[c] = ey[c] + shear * ex[c];
    GridConst g = make_grid_const(ex, ey_l, ez, kappa, s_r, bin_offset, nx + (shear < 0 ? -shear : shear) * (ny - 1),
                                  ny, nz);
    g.a_off = shear > 0 ? -shear * (ny - 1) : 0;
    g.shear = shear;
    g.img_nx = nx;
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

// Minimum and maximum distance from point a to the parallelogram {o + u e1 + v e2 : u, v in
// [0, 1]} (e1, e2 the full edge vectors, not necessarily orthogonal): the minimum at the foot of
// the perpendicular onto the plane when it lies inside, otherwise on one of the four edges; the
// maximum at a corner (distance is convex).  Bounds the range window of a sheared lattice strip.
static inline void parallelogram_distance_bounds(const double* a, const double* o, const double* e1,
                                                 const double* e2, double* dmin, double* dmax) {
    auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    const double w[3] = {a[0] - o[0], a[1] - o[1], a[2] - o[2]};
    const double g11 = dot(e1, e1), g12 = dot(e1, e2), g22 = dot(e2, e2);
    const double det = g11 * g22 - g12 * g12;
    double best = INFINITY;
    if (det > 1e-12 * (g11 * g22 + 1e-300)) {
        const double r1 = dot(e1, w), r2 = dot(e2, w);
        const double u = (r1 * g22 - r2 * g12) / det, v = (r2 * g11 - r1 * g12) / det;
        if (u >= 0.0 && u <= 1.0 && v >= 0.0 && v <= 1.0) {
            double q[3];
            for (int c = 0; c < 3; ++c) q[c] = o[c] + u * e1[c] + v * e2[c];
            best = dist3(a, q);
        }
    }
    if (!(best < INFINITY)) {
        // edges p0 + t d, t in [0, 1]: (o, e1), (o + e1, e2), (o, e2), (o + e2, e1)
        for (int edge = 0; edge < 4; ++edge) {
            const double* from = edge == 1 ? e1 : edge == 3 ? e2 : nullptr;
            const double* dir = (edge == 0 || edge == 3) ? e1 : e2;
            double p0[3], d[3];
            for (int c = 0; c < 3; ++c) {
                p0[c] = o[c] + (from ? from[c] : 0.0);
                d[c] = dir[c];
            }
            const double dd = dot(d, d);
            const double pw[3] = {a[0] - p0[0], a[1] - p0[1], a[2] - p0[2]};
            double t = dd > 0.0 ? dot(pw, d) / dd : 0.0;
            t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
            double q[3];
            for (int c = 0; c < 3; ++c) q[c] = p0[c] + t * d[c];
            const double dist = dist3(a, q);
            if (dist < best) best = dist;
        }
    }
    *dmin = best;
    double far = 0.0;
    for (int corner = 0; corner < 4; ++corner) {
        double q[3];
        for (int c = 0; c < 3; ++c) q[c] = o[c] + ((corner & 1) ? e1[c] : 0.0) + ((corner & 2) ? e2[c] : 0.0);
        const double dist = dist3(a, q);
        if (dist > far) far = dist;
    }
    *dmax = far;
}

// Shear of the forward scatter's lattice (sar_geom.cuh GridConst): for linear sampling, where
// the scatter's register run windows need a lane's bin to change by less than ~0.3 bins per
// walked row, and collections that look across the grid axes (bins change alike along x and y,
// e.g. along the diagonal).  The walk along lattice rows (steps ey + m ex) follows the iso-range
// lines when m ex cancels the bin rate of ey.  Returns m in {-1, +1} when the walk rate of that
// lattice over all pulses (at the scene centre) stays below kShearWalk bins per row while the
// unsheared layout's does not and the lanes (along x) keep distinct bins; 0 otherwise.
constexpr double kShearWalk = 0.25;

// Shear of the backprojection's lattice: its lanes run along the lattice's second axis (steps
// ey + m ex), so that a quarter-warp's window loads land on one or two bins and are broadcast.
// Returns m in {-2, -1, +1, +2} (the one whose axis changes least) when the better plain lane axis
// still changes by more than kGatherShearRate bins per pixel over the pulses (bank-conflicted
// loads: collections looking across the grid axes, e.g. at 45 or 63 degrees) and the sheared axis
// changes by less than half of that; 0 otherwise.  Below that rate the plain layout's loads cost
// less than the lattice's partial tiles at the image's edges (measured, 2048^2 at 0.25 m, 4096
// pulses, linear: looking at 63.4 degrees, 1.16 bins per pixel at upsample 8, the m = -2 lattice
// took 16.7 ms against 15.4 ms; at 2.32 (upsample 16) 16.6 against 18.6 ms; on the diagonal, 1.76
// at upsample 8, the m = -1 lattice 16.1 against 17.6 ms).
constexpr double kGatherShearRate = 1.5;
static inline int choose_gather_shear(const double* tx, const double* rx, size_t S, const double* origin,
                                      const double* ex, const double* ey, const double* ez, int nx, int ny, int nz,
                                      double s_r) {
    double c[3];
    for (int d = 0; d < 3; ++d)
        c[d] = origin[d] + 0.5 * ((nx - 1) * ex[d] + (ny - 1) * ey[d] + (nz - 1) * ez[d]);
    double ax = 0.0, ay = 0.0, am[4] = {0.0, 0.0, 0.0, 0.0};   // m = -2, -1, +1, +2
    for (size_t s = 0; s < S; ++s) {
        double gx = 0.0, gy = 0.0;
        for (int ant = 0; ant < 2; ++ant) {
            const double* a = (ant ? rx : tx) + 3 * s;
            const double w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            const double n = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            if (!(n > 0.0)) return 0;
            gx += (w[0] * ex[0] + w[1] * ex[1] + w[2] * ex[2]) / n;
            gy += (w[0] * ey[0] + w[1] * ey[1] + w[2] * ey[2]) / n;
        }
        if (!isfinite(gx) || !isfinite(gy)) return 0;
        ax = fmax(ax, fabs(gx) * s_r);
        ay = fmax(ay, fabs(gy) * s_r);
        am[0] = fmax(am[0], fabs(gy - 2.0 * gx) * s_r);
        am[1] = fmax(am[1], fabs(gy - gx) * s_r);
        am[2] = fmax(am[2], fabs(gy + gx) * s_r);
        am[3] = fmax(am[3], fabs(gy + 2.0 * gx) * s_r);
    }
    const double plain = fmin(ax, ay);
    int best = 1;
    for (int i = 0; i < 4; ++i)
        if (am[i] < am[best]) best = i;
    const int m = best < 2 ? best - 2 : best - 1;
    return (plain > kGatherShearRate && am[best] < 0.5 * plain) ? m : 0;
}
static inline int choose_shear(const double* tx, const double* rx, size_t S, const double* origin,
                               const double* ex, const double* ey, const double* ez, int nx, int ny, int nz,
                               double s_r, int lanes_y) {
    double c[3];
    for (int d = 0; d < 3; ++d)
        c[d] = origin[d] + 0.5 * ((nx - 1) * ex[d] + (ny - 1) * ey[d] + (nz - 1) * ez[d]);
    double walk0 = 0.0, walk[2] = {0.0, 0.0}, lane_min = INFINITY;
    for (size_t s = 0; s < S; ++s) {
        double gx = 0.0, gy = 0.0;
        for (int ant = 0; ant < 2; ++ant) {
            const double* a = (ant ? rx : tx) + 3 * s;
            const double w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            const double n = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            if (!(n > 0.0)) return 0;
            gx += (w[0] * ex[0] + w[1] * ex[1] + w[2] * ex[2]) / n;
            gy += (w[0] * ey[0] + w[1] * ey[1] + w[2] * ey[2]) / n;
        }
        gx *= s_r;
        gy *= s_r;
        if (!isfinite(gx) || !isfinite(gy)) return 0;
        walk0 = fmax(walk0, fabs(lanes_y ? gy : gx));   // the unsheared scatter walks the gather's lane axis
        walk[0] = fmax(walk[0], fabs(gy - gx));
        walk[1] = fmax(walk[1], fabs(gy + gx));
        lane_min = fmin(lane_min, fabs(gx));
    }
    if (walk0 < kShearWalk || lane_min < 1.5) return 0;
    const int m = walk[0] <= walk[1] ? -1 : 1;
    return walk[m > 0] < kShearWalk ? m : 0;
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
