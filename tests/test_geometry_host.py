"""Precision of the kernels' range geometry, evaluated by the host build of the same code.

The GPU kernels never form the range in FP64 per pixel (sar_geom.cuh).  This checks, without a
GPU, that their phase (cycles, mod 1) and range-bin position agree with FP64 ranges computed as
the reference does (sarsolver_cxx.cpp:10-20, :283, :287) to well inside the 1e-5 relative-error
budget, on the benchmark geometry at full size.
"""
import ctypes

import numpy as np
import pytest

from cases import C, load_golden, spotlight
from sarsolver_gb300 import _lib
from sarsolver_gb300.geometry import GridSarScene, grid_axes


def fp64_truth(tx, rx, srp, pos, kappa, s_r):
    dr = (np.linalg.norm(tx[None] - pos, axis=1) + np.linalg.norm(rx[None] - pos, axis=1)
          - np.linalg.norm(tx - srp) - np.linalg.norm(rx - srp))
    cyc = kappa * dr
    return cyc - np.round(cyc), s_r * dr


def host_eval_grid(scene, tx, rx, srp, kappa, s_r, bin_offset=0.0, precise=0, transposed=False):
    """transposed: the forward scatter's layout for collections looking along y (a thread holds
    the y offset and walks x), otherwise the layout holding x and walking y."""
    lib = _lib.load_host()
    fn = lib.sar_geom_host_eval_transposed if transposed else lib.sar_geom_host_eval
    shape, origin, ex, ey, ez = grid_axes(scene)
    nz, ny, nx = shape
    S = tx.shape[0]
    ph = np.zeros((S, nz * ny * nx), np.float32)
    bn = np.zeros((S, nz * ny * nx))
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (origin, ex, ey, ez, tx, rx, srp)]
    assert fn(*[a.ctypes.data for a in arrs[:4]], nx, ny, nz, S,
                                  *[a.ctypes.data for a in arrs[4:]], kappa, s_r, bin_offset, precise,
                                  ph.ctypes.data, bn.ctypes.data) == 0
    return ph, bn


def errors(ph, bn, truth_ph, truth_bn):
    e = ph.astype(np.float64) - truth_ph
    e -= np.round(e)
    return np.abs(e).max() * 2 * np.pi, np.sqrt(np.mean(e ** 2)) * 2 * np.pi, np.abs(bn - truth_bn).max()


@pytest.mark.parametrize("name", ["little", "spot_small", "bistatic_odd"])
def test_grid_axes_reproduce_positions(name):
    case = load_golden(name)
    shape, origin, ex, ey, ez = grid_axes(case.scene)
    nz, ny, nx = shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    pos = origin[None] + i.reshape(-1, 1) * ex + j.reshape(-1, 1) * ey + k.reshape(-1, 1) * ez
    assert np.abs(pos - case.scene.positions).max() < 1e-9


@pytest.mark.parametrize("n,spacing,aperture,pulses", [
    (2048, 0.25, 5.0, [0, 4095]),     # benchmark image, first and last pulse of 4096
    (256, 0.5, 3.0, [0, 64, 127]),    # CPU-runnable configuration
])
def test_grid_phase_and_bin_precision(n, spacing, aperture, pulses):
    S_full = 4096 if n == 2048 else 128
    tx = spotlight(S_full, aperture)[pulses]
    srp = np.zeros_like(tx)
    scene = GridSarScene([1, n, n], [0.0, spacing * (n - 1), spacing * (n - 1)])
    kappa, s_r = 10.0e9 / C, 200.0e6 * 8 / C
    ph, bn = host_eval_grid(scene, tx, tx, srp, kappa, s_r)
    pos = scene.positions
    worst = []
    for s in range(len(pulses)):
        tp, tb = fp64_truth(tx[s], tx[s], srp[s], pos, kappa, s_r)
        worst.append(errors(ph[s], bn[s], tp, tb))
    pmax = max(w[0] for w in worst)
    prms = max(w[1] for w in worst)
    bmax = max(w[2] for w in worst)
    assert pmax < 1.0e-5, pmax      # radians
    assert prms < 1.5e-6, prms
    assert bmax < 5.0e-5, bmax      # range bins


@pytest.mark.parametrize("transposed", [False, True])
def test_turned_collection_precision_in_both_layouts(transposed):
    """The benchmark image seen from 90 degrees (range along y): the scatter holds y and walks x
    there (transposed), the backprojection holds x and walks y; both meet the same bounds."""
    tx = spotlight(4096, 5.0, centre_az_deg=90.0)[[0, 2047, 4095]]
    srp = np.zeros_like(tx)
    n, spacing = 2048, 0.25
    scene = GridSarScene([1, n, n], [0.0, spacing * (n - 1), spacing * (n - 1)])
    kappa, s_r = 10.0e9 / C, 200.0e6 * 8 / C
    ph, bn = host_eval_grid(scene, tx, tx, srp, kappa, s_r, transposed=transposed)
    pos = scene.positions
    for s in range(tx.shape[0]):
        tp, tb = fp64_truth(tx[s], tx[s], srp[s], pos, kappa, s_r)
        pmax, prms, bmax = errors(ph[s], bn[s], tp, tb)
        assert pmax < 1.0e-5 and prms < 1.5e-6 and bmax < 5.0e-5, (pmax, prms, bmax)


def tile_halfspan_bruteforce(scene, tx, rx, s_r, rng, samples=300):
    """Largest |R(p) - R(c)| * s_r over sampled (tile, pulse) pairs (every corner tile, the rest
    at random), R the bistatic range and c the mean of the tile's sub-tile anchors."""
    shape, origin, ex, ey, ez = grid_axes(scene)
    nz, ny, nx = shape
    tx_t, ty_t = -(-nx // 32), -(-ny // 32)
    di, dj = np.meshgrid(np.arange(-16, 16), np.arange(-16, 16))
    off = di[..., None] * ex + dj[..., None] * ey
    corners = [(0, 0), (tx_t - 1, 0), (0, ty_t - 1), (tx_t - 1, ty_t - 1)]
    worst = 0.0
    for n in range(samples):
        ti, tj = corners[n] if n < 4 else (rng.integers(tx_t), rng.integers(ty_t))
        k, s = rng.integers(nz), rng.integers(tx.shape[0])
        c = origin + (32 * ti + 16) * ex + (32 * tj + 16) * ey + k * ez
        r = np.linalg.norm(tx[s] - (c + off), axis=-1) + np.linalg.norm(rx[s] - (c + off), axis=-1)
        rc = np.linalg.norm(tx[s] - c) + np.linalg.norm(rx[s] - c)
        worst = max(worst, float(np.abs(r - rc).max()) * s_r)
    return worst


def host_halfspan(scene, tx, rx, s_r):
    shape, origin, ex, ey, ez = grid_axes(scene)
    nz, ny, nx = shape
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (tx, rx, origin, ex, ey, ez)]
    return _lib.load_host().sar_tile_halfspan_host(arrs[0].ctypes.data, arrs[1].ctypes.data, tx.shape[0],
                                                   *[a.ctypes.data for a in arrs[2:]], -(-nx // 32), -(-ny // 32),
                                                   nz, s_r)


@pytest.mark.parametrize("name", ["benchmark", "turned", "diagonal", "bistatic_odd", "little"])
def test_gather_window_bound_covers_every_tile(name):
    """The backprojection stages, per (tile, pulse), a window of bins centred on the tile's base
    bin whose half-span comes from the look directions (sar_host_prep.h); a bin outside it would
    be clamped.  The bound must exceed the largest sampled span in every geometry, and at the
    benchmark geometry be about half the isotropic 16 (|ex| + |ey|) per antenna."""
    rng = np.random.default_rng(11)
    if name in ("bistatic_odd", "little"):
        case = load_golden(name)
        ap, scene = case.aperture, case.scene
        tx, rx = ap.transmitter_positions, ap.receiver_positions
        s_r = ap.sample_bandwidth * case.upsample_ratio / ap.c_eff
    else:
        az = {"benchmark": 0.0, "turned": 90.0, "diagonal": 45.0}[name]
        tx = spotlight(4096, 5.0, centre_az_deg=az)
        rx = tx
        scene = GridSarScene([1, 2048, 2048], [0.0, 0.25 * 2047, 0.25 * 2047])
        s_r = 200.0e6 * 8 / C
    bound = host_halfspan(scene, tx, rx, s_r)
    brute = tile_halfspan_bruteforce(scene, tx, rx, s_r, rng)
    _, _, ex, ey, _ = grid_axes(scene)
    iso = s_r * 2 * 16 * (np.linalg.norm(ex) + np.linalg.norm(ey))
    assert 0 < brute <= bound <= iso * 1.001, (brute, bound, iso)
    if name == "benchmark":
        assert bound < 0.55 * iso


def test_bistatic_rotated_grid_precision():
    case = load_golden("bistatic_odd")
    ap = case.aperture
    kappa = ap.sign_multiplier * ap.centre_frequency / ap.c_eff
    s_r = ap.sample_bandwidth * 8.0 / ap.c_eff
    ph, bn = host_eval_grid(case.scene, ap.transmitter_positions, ap.receiver_positions, ap.stab_ref_posns,
                            kappa, s_r)
    pos = case.scene.positions
    for s in range(ap.num_slow_times):
        tp, tb = fp64_truth(ap.transmitter_positions[s], ap.receiver_positions[s], ap.stab_ref_posns[s], pos,
                            kappa, s_r)
        pmax, _, bmax = errors(ph[s], bn[s], tp, tb)
        assert pmax < 1.0e-5 and bmax < 5.0e-5


def test_unstructured_point_precision():
    lib = _lib.load_host()
    rng = np.random.default_rng(0)
    P, S = 50000, 3
    tx = spotlight(S, 5.0)
    rx = spotlight(S, 3.0, 8.0e3, 3.0e3, 20.0)
    srp = np.zeros((S, 3))
    pos = np.stack([rng.uniform(-256, 256, P), rng.uniform(-256, 256, P), rng.uniform(-2, 2, P)], -1)
    origin = 0.5 * (pos.min(0) + pos.max(0))
    kappa, s_r = 10.0e9 / C, 200.0e6 * 8 / C
    ph = np.zeros((S, P), np.float32)
    bn = np.zeros((S, P))
    arrs = [np.ascontiguousarray(a) for a in (origin, pos, tx, rx, srp)]
    # bin rule -0.5 (linear): the harness returns the bin position itself
    lib.sar_geom_host_eval_points(arrs[0].ctypes.data, P, arrs[1].ctypes.data, S, arrs[2].ctypes.data,
                                  arrs[3].ctypes.data, arrs[4].ctypes.data, kappa, s_r, -0.5, ph.ctypes.data,
                                  bn.ctypes.data)
    for s in range(S):
        tp, tb = fp64_truth(tx[s], rx[s], srp[s], pos, kappa, s_r)
        pmax, _, bmax = errors(ph[s], bn[s], tp, tb)
        assert pmax < 1.0e-6 and bmax < 1.0e-6


def test_precise_bins_match_fp64_rounding_at_short_range_and_fine_bins():
    """The reference's 'little' case: 2 km stand-off, upsample 128 (M = 32128).  Nearest-bin
    sampling (round(0.5 + v), sarsolver_cxx.cpp:347) must pick the FP64 bin; the precise-bin
    mode (integer/fraction split + cubic bin terms) keeps the bin position within ~1e-6."""
    case = load_golden("little")
    ap = case.aperture
    M = int(128 * ap.num_freqs)
    s_r = ap.sample_bandwidth * M / (ap.num_freqs * ap.c_eff)
    kappa = ap.centre_frequency / ap.c_eff
    pos = case.scene.positions
    for precise, max_flips, max_err, transposed in ((0, None, 5e-4, False), (1, 10, 5e-6, False),
                                                    (1, 10, 5e-6, True)):
        ph, bn = host_eval_grid(case.scene, ap.transmitter_positions, ap.receiver_positions, ap.stab_ref_posns,
                                kappa, s_r, 0.5, precise, transposed)
        flips, err = 0, 0.0
        for s in range(ap.num_slow_times):
            _, tb = fp64_truth(ap.transmitter_positions[s], ap.receiver_positions[s], ap.stab_ref_posns[s], pos,
                               kappa, s_r)
            v = tb + 0.5
            flips += int(np.sum(np.round(v) != np.round(bn[s])))
            err = max(err, float(np.abs(bn[s] - v).max()))
        assert err < max_err, (precise, err)
        if max_flips is not None:
            assert flips <= max_flips, flips


def std_round(x):
    """C++ std::round: halfway cases away from zero."""
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


@pytest.mark.parametrize("rule,offset", [("adjoint", 0.5), ("forward", 0.0)])
def test_point_scheme_bins_match_fp64_rounding(rule, offset):
    """Per-pixel double-float scheme on the reference's 'little' case (upsample 128): the
    nearest bin chosen by the kernel's exact rule equals std::round of the FP64 position,
    round(0.5 + v) for the adjoint (sarsolver_cxx.cpp:347), round(v) forward (:289)."""
    lib = _lib.load_host()
    case = load_golden("little")
    ap = case.aperture
    M = int(128 * ap.num_freqs)
    s_r = ap.sample_bandwidth * M / (ap.num_freqs * ap.c_eff)
    kappa = ap.centre_frequency / ap.c_eff
    pos = np.ascontiguousarray(case.scene.positions)
    S, P = ap.num_slow_times, pos.shape[0]
    origin = 0.5 * (pos.min(0) + pos.max(0))
    ph = np.zeros((S, P), np.float32)
    bn = np.zeros((S, P))
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in
            (origin, pos, ap.transmitter_positions, ap.receiver_positions, ap.stab_ref_posns)]
    lib.sar_geom_host_eval_points(arrs[0].ctypes.data, P, arrs[1].ctypes.data, S, arrs[2].ctypes.data,
                                  arrs[3].ctypes.data, arrs[4].ctypes.data, kappa, s_r, offset, ph.ctypes.data,
                                  bn.ctypes.data)
    flips = 0
    for s in range(S):
        _, tb = fp64_truth(ap.transmitter_positions[s], ap.receiver_positions[s], ap.stab_ref_posns[s], pos,
                           kappa, s_r)
        flips += int(np.sum(std_round(tb + offset) != bn[s]))
    assert flips == 0


def test_grid_from_aperture_reproduces_the_reference_little_grid():
    """GridSarScene.from_aperture on the reference's 'little' aperture (tests/conftest.py:46-73:
    origin centre, 0 x 40 x 40 m, safety factor 3) gives the grid the reference built."""
    import numpy as np
    from cases import load_golden
    from sarsolver_gb300.geometry import GridSarScene
    case = load_golden("little")
    scene = GridSarScene.from_aperture(case.aperture, np.zeros(3), np.array([0.0, 40.0, 40.0]), safety_factor=3.0)
    assert list(scene.grid_shape) == case.data["grid_shape"].tolist()
    np.testing.assert_allclose(scene.rotation_matrix, case.data["rotation_matrix"], atol=1e-12)
    np.testing.assert_allclose(scene.positions, case.scene.positions, atol=1e-9)


def test_wgs84_up_is_the_ellipsoid_normal():
    import numpy as np
    from sarsolver_gb300.geometry import WGS84_A, WGS84_F, wgs84_up
    lat, lon, h = np.deg2rad(-17.7), np.deg2rad(168.3), 120.0
    e2 = WGS84_F * (2 - WGS84_F)
    n = WGS84_A / np.sqrt(1 - e2 * np.sin(lat) ** 2)
    p = np.array([(n + h) * np.cos(lat) * np.cos(lon), (n + h) * np.cos(lat) * np.sin(lon), (n * (1 - e2) + h) * np.sin(lat)])
    np.testing.assert_allclose(wgs84_up(p), [np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], atol=1e-12)


def plan_tile_window(scene, tx, rx, s_r):
    """Staged window (bins) the plan gives a tile, as build_plan sizes it: the isotropic bound,
    narrowed to the look-direction bound where that is smaller (both with 3 bins of margin)."""
    _, _, ex, ey, _ = grid_axes(scene)
    iso = s_r * 2.0 * 16.0 * (np.linalg.norm(ex) + np.linalg.norm(ey))
    w = (2 * (int(np.ceil(iso)) + 3) + 3) & ~3
    hd = host_halfspan(scene, tx, rx, s_r)
    if hd >= 0:
        w = min(w, (2 * (int(np.ceil(hd)) + 3) + 3) & ~3)
    return w


def window_check(scene, tx, rx, srp, kappa, s_r, bin_offset, precise, ww):
    shape, origin, ex, ey, ez = grid_axes(scene)
    nz, ny, nx = shape
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (origin, ex, ey, ez, tx, rx, srp)]
    need = np.zeros(1)
    bad = _lib.load_host().sar_gather_window_check_host(*[a.ctypes.data for a in arrs[:4]], nx, ny, nz,
                                                        tx.shape[0], *[a.ctypes.data for a in arrs[4:]], kappa,
                                                        s_r, bin_offset, precise, ww, need.ctypes.data)
    return bad, float(need[0])


@pytest.mark.parametrize("name", ["benchmark", "turned", "diagonal"])
@pytest.mark.parametrize("interp", ["linear", "nearest_ref"])
def test_gather_window_flag_silent_on_headline_geometries(name, interp):
    """The gather's producers raise SAR_FLAG_GATHER_WINDOW when a sub-tile's bin extent (a bound
    over its 16x16 pixels) leaves the staged window.  On the 2048^2 x 4096-pulse headline geometry
    in all three orientations it must stay silent with the window the plan picks (every 64th
    pulse, every tile), or the headline would run flagged."""
    az = {"benchmark": 0.0, "turned": 90.0, "diagonal": 45.0}[name]
    tx = spotlight(4096, 5.0, centre_az_deg=az)[::64]
    srp = np.zeros_like(tx)
    scene = GridSarScene([1, 2048, 2048], [0.0, 0.25 * 2047, 0.25 * 2047])
    s_r = 200.0e6 * 8 / C
    kappa = 10.0e9 / C
    ww = plan_tile_window(scene, spotlight(4096, 5.0, centre_az_deg=az), spotlight(4096, 5.0, centre_az_deg=az), s_r)
    precise = 1 if interp == "nearest_ref" or ww > 256 else 0
    bin_offset = -0.5 if interp == "linear" else 0.5
    bad, need = window_check(scene, tx, tx, srp, kappa, s_r, bin_offset, precise, ww)
    assert bad == 0, (bad, need, ww)
    assert need <= 0.5 * ww


def test_gather_window_flag_fires_on_an_undersized_window():
    """The same check with a window 16 bins narrower than the plan's must report violations."""
    tx = spotlight(4096, 5.0)[::256]
    scene = GridSarScene([1, 512, 512], [0.0, 0.25 * 511, 0.25 * 511])
    s_r = 200.0e6 * 8 / C
    ww = plan_tile_window(scene, spotlight(4096, 5.0), spotlight(4096, 5.0), s_r)
    bad_ok, need = window_check(scene, tx, tx, np.zeros_like(tx), 10.0e9 / C, s_r, -0.5, 0, ww)
    bad, _ = window_check(scene, tx, tx, np.zeros_like(tx), 10.0e9 / C, s_r, -0.5, 0, ww - 16)
    assert bad_ok == 0 and bad > 0 and need > 0.5 * (ww - 16)


@pytest.mark.parametrize("precise", [0, 1])
def test_bin_extent_bounds_every_pixel_bin(precise):
    """bin_extent (sar_geom.cuh) must contain every bin the kernels' per-pixel evaluation forms
    over the sub-tile, for sub-tiles at the grid corners and centre, several pulses, both bin
    modes, and a bistatic short-range geometry where the quadratic and cubic terms matter."""
    lib = _lib.load_host()
    cases = [(spotlight(64, 5.0), None, 200.0e6 * 8 / C, GridSarScene([1, 2048, 2048], [0.0, 511.75, 511.75])),
             (spotlight(16, 20.0, radius=2.0e3, altitude=1.0e3), spotlight(16, 35.0, radius=2.5e3, altitude=0.5e3),
              200.0e6 * 128 / C, GridSarScene([1, 256, 256], [0.0, 63.75, 63.75]))]
    for tx, rx, s_r, scene in cases:
        rx = tx if rx is None else rx
        shape, origin, ex, ey, ez = grid_axes(scene)
        nz, ny, nx = shape
        base = [np.ascontiguousarray(a, dtype=np.float64) for a in (origin, ex, ey, ez)]
        tiles = [(0, 0), (nx // 32 - 1, ny // 32 - 1), (nx // 64, ny // 64), (0, ny // 32 - 1)]
        out = np.zeros(4)
        for s in range(0, tx.shape[0], 5):
            t, r, o = (np.ascontiguousarray(a, dtype=np.float64) for a in (tx[s], rx[s], np.zeros(3)))
            for ti, tj in tiles:
                for q in range(4):
                    assert lib.sar_bin_extent_host(*[a.ctypes.data for a in base], nx, ny, nz, t.ctypes.data,
                                                   r.ctypes.data, o.ctypes.data, 10.0e9 / C, s_r, -0.5, precise,
                                                   ti, tj, 0, q, out.ctypes.data) == 0
                    lo, hi, vmin, vmax = out
                    assert lo - 1e-3 <= vmin and vmax <= hi + 1e-3, (s, ti, tj, q, out)
                    assert hi - lo < 1.2 * (vmax - vmin) + 4.0   # tight: the linear terms dominate


def host_eval_sheared(scene, tx, rx, srp, kappa, s_r, shear, bin_offset=-0.5, lanes=False):
    """The sheared-lattice evaluation, written at the image pixels (NaN where no lattice pixel
    landed): the forward scatter's layout, or with `lanes` the backprojection's."""
    lib = _lib.load_host()
    fn = lib.sar_geom_host_eval_sheared_lanes if lanes else lib.sar_geom_host_eval_sheared
    shape, origin, ex, ey, ez = grid_axes(scene)
    nz, ny, nx = shape
    S = tx.shape[0]
    ph = np.full((S, nz * ny * nx), np.nan, np.float32)
    bn = np.full((S, nz * ny * nx), np.nan)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (origin, ex, ey, ez, tx, rx, srp)]
    assert fn(*[a.ctypes.data for a in arrs[:4]], nx, ny, nz, S, *[a.ctypes.data for a in arrs[4:]], kappa, s_r,
              bin_offset, 0, shear, ph.ctypes.data, bn.ctypes.data) == 0
    return ph, bn


def choose_shear(scene, tx, rx, s_r, gather=False):
    lib = _lib.load_host()
    fn = lib.sar_choose_gather_shear_host if gather else lib.sar_choose_shear_host
    shape, origin, ex, ey, ez = grid_axes(scene)
    nz, ny, nx = shape
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (tx, rx, origin, ex, ey, ez)]
    return fn(arrs[0].ctypes.data, arrs[1].ctypes.data, tx.shape[0], *[a.ctypes.data for a in arrs[2:]], nx, ny, nz,
              s_r)


@pytest.mark.parametrize("az,expect", [(0.0, 0), (90.0, 0), (45.0, -1), (135.0, 1), (-45.0, 1), (20.0, 0)])
def test_scatter_shear_choice(az, expect):
    """Linear sampling at upsample 8 on the benchmark image: collections along the grid axes keep
    the plain layouts, those along a diagonal walk a lattice sheared by one pixel per row the
    way that cancels the bin rate (-1 when range falls along +x and +y alike), and one at 20
    degrees, whose iso-range slope is near neither, is left alone.  The backprojection makes the
    same choice for its lanes (at upsample 8 and 128)."""
    tx = spotlight(4096, 5.0, centre_az_deg=az)
    n, spacing = 2048, 0.25
    scene = GridSarScene([1, n, n], [0.0, spacing * (n - 1), spacing * (n - 1)])
    assert choose_shear(scene, tx, tx, 200.0e6 * 8 / C) == expect
    for U in (8, 128):
        assert choose_shear(scene, tx, tx, 200.0e6 * U / C, gather=True) == expect


@pytest.mark.parametrize("U", [8, 16, 128])
@pytest.mark.parametrize("az,expect", [(63.43, -2), (116.57, 2), (26.57, 0)])
def test_gather_shear_by_two(az, expect, U):
    """Collections looking at ~63 (or 117) degrees: from upsample 16 on, the backprojection's lanes
    run along ey -+ 2 ex, where the bins change least; at upsample 8 the better plain axis changes
    by only ~1.2 bins per pixel, below the rate where the lattice pays, and the plain layout stays.
    The scatter keeps its plain layout throughout.  At ~27 degrees no shear of ey fits (it would
    take ex + 2 ey)."""
    tx = spotlight(4096, 5.0, centre_az_deg=az)
    n, spacing = 2048, 0.25
    scene = GridSarScene([1, n, n], [0.0, spacing * (n - 1), spacing * (n - 1)])
    assert choose_shear(scene, tx, tx, 200.0e6 * U / C, gather=True) == (expect if U > 8 else 0)
    assert choose_shear(scene, tx, tx, 200.0e6 * 8 / C) == 0


@pytest.mark.parametrize("az,lanes", [(45.0, False), (135.0, False), (45.0, True)])
def test_sheared_lattice_precision_and_walk(az, lanes):
    """The benchmark image seen along a diagonal, on the sheared lattice the forward scatter
    walks: every image pixel is evaluated exactly once, to the precision bounds of the plain
    layouts against FP64, and a lattice row step (one row along y, `shear` pixels along x)
    changes a pixel's bin by less than 0.32 anywhere (below 0.25 at the scene centre, where the
    shear is chosen), the slow walk that lets the scatter's register run windows of 4 rows work
    (3 steps below 0.98 bins; against 1.9 bins per pixel along either grid axis)."""
    all_tx = spotlight(4096, 5.0, centre_az_deg=az)
    tx = all_tx[[0, 2047, 4095]]
    srp = np.zeros_like(tx)
    n, spacing = 2048, 0.25
    scene = GridSarScene([1, n, n], [0.0, spacing * (n - 1), spacing * (n - 1)])
    kappa, s_r = 10.0e9 / C, 200.0e6 * 8 / C
    m = choose_shear(scene, all_tx, all_tx, s_r)
    assert m != 0
    ph, bn = host_eval_sheared(scene, tx, tx, srp, kappa, s_r, m, lanes=lanes)
    assert not np.isnan(bn).any() and not np.isnan(ph).any()
    pos = scene.positions
    for s in range(tx.shape[0]):
        tp, tb = fp64_truth(tx[s], tx[s], srp[s], pos, kappa, s_r)
        pmax, prms, bmax = errors(ph[s], bn[s] + 0.5, tp, tb)   # bin offset -1/2 of linear sampling
        assert pmax < 1.0e-5 and prms < 1.5e-6 and bmax < 5.0e-5, (pmax, prms, bmax)
        b = bn[s].reshape(n, n)   # [j, i]
        walk = b[1:, max(m, 0):n + min(m, 0)] - b[:-1, max(-m, 0):n - max(m, 0)]
        assert np.abs(walk).max() < 0.32, np.abs(walk).max()


def test_parallelogram_distance_bounds():
    """Exact minimum and maximum distance from a point to a (sheared) parallelogram, against dense
    sampling: the minimum is never above the sampled one and within the sampling step of it, the
    maximum is the farthest corner."""
    lib = _lib.load_host()
    rng = np.random.default_rng(3)
    t = np.linspace(0.0, 1.0, 401)
    uu, vv = np.meshgrid(t, t)
    for trial in range(40):
        o = rng.normal(size=3) * 10
        e1 = rng.normal(size=3) * 5
        e2 = e1 * rng.uniform(-1, 1) + rng.normal(size=3) * 5   # far from orthogonal
        a = o + rng.normal(size=3) * (3 if trial % 2 else 30)
        if trial % 3 == 0:   # a point right above the inside
            a = o + 0.3 * e1 + 0.6 * e2 + np.cross(e1, e2) / np.linalg.norm(np.cross(e1, e2)) * 2.0
        dmin, dmax = ctypes.c_double(), ctypes.c_double()
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (a, o, e1, e2)]
        lib.sar_parallelogram_distance_host(*[x.ctypes.data for x in arrs], ctypes.byref(dmin), ctypes.byref(dmax))
        pts = o + uu[..., None] * e1 + vv[..., None] * e2
        d = np.linalg.norm(pts - a, axis=-1)
        step = (np.linalg.norm(e1) + np.linalg.norm(e2)) / 400
        assert dmin.value <= d.min() + 1e-9 and dmin.value >= d.min() - step, (dmin.value, d.min())
        assert abs(dmax.value - d.max()) < 1e-9
