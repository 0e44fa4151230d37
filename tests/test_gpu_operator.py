"""GPU parity of the operator pair against the oracle and the reference's golden outputs.

Tolerances (complex64 GPU vs FP64 CPU, relative L2):
  * linear mode vs the FP64 oracle in linear mode: 1e-5 (the accuracy target of the port).
  * nearest_ref mode vs the reference: nearest-bin sampling is discontinuous, so a pixel whose
    range lies within ~1e-5 bins of a bin edge may fall in the neighbouring bin in FP32 and FP64.
    Each such flip moves one term by up to ~0.4 of its size at upsample 8, which on the small
    golden cases is worth up to ~2e-3; the reference's own criterion (elementwise rel 1e-3) is
    applied to its "little" case at upsample 128, where bins are 16x finer.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from cases import crandn, load_golden, point_scene, rel_l2, spotlight_case
from sarsolver_gb300 import NumpySimpleSarOperator, SarPlan, _lib
from sarsolver_gb300.geometry import GridSarScene, NumpySimpleSarAperture, SimpleSarScene

pytestmark = pytest.mark.gpu

LINEAR_TOL = 1.0e-5
NEAREST_TOL = 2.0e-3


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def gpu_forward(plan, x):
    return plan.forward(torch.from_numpy(np.asarray(x).reshape(-1))).cpu().numpy().astype(np.complex128)


def gpu_adjoint(plan, y):
    return plan.adjoint(torch.from_numpy(np.asarray(y))).cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("path", ["auto", "grid"])
@pytest.mark.parametrize("name", ["spot_small", "bistatic_odd", "points"])
def test_goldens_nearest_ref(name, path):
    """nearest_ref picks the bins FP64 rounding picks on every path: the per-pixel double-float
    kernels by construction, the grid kernels by deciding again, in double-float, every bin whose
    FP32 coordinate lies within 5e-5 of a rounding boundary (here: the pixel at the stabilisation
    point, whose adjoint bin round(0.5 + 0) is a tie).  So the reference goldens are met to FP32
    accuracy on both."""
    case = load_golden(name)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="nearest_ref", path=path)
    if path == "grid":
        assert plan.is_grid == (name != "points")
    fwd = gpu_forward(plan, case.data["x"])
    adj = gpu_adjoint(plan, case.data["y"])
    assert rel_l2(fwd, case.data["forward"]) < 1.0e-5
    assert rel_l2(adj, case.data["adjoint"]) < 1.0e-5
    assert plan.device_flags() == 0


def test_nearest_grid_bins_equal_fp64_at_rounding_boundaries():
    """The pixels of a 2048^2 grid whose FP64 bin positions lie closest to the nearest-bin rounding
    boundaries (per pulse, the 32 closest for the adjoint rule round(0.5 + v) and for the forward
    rule round(v)), on the default path for nearest_ref (the staged grid kernels).  The set holds
    pixels the FP32 bin polynomial alone rounds to the other bin (checked with the host build of
    the kernels' geometry); the adjoint at those pixels and the forward projection of impulses
    there equal the FP64 oracle to FP32 accuracy."""
    from test_geometry_host import fp64_truth, host_eval_grid
    S, n = 4, 2048
    rng = np.random.default_rng(5)
    case = spotlight_case(S, 256, n, 0.25, 4.0, weights=np.exp(1j * rng.uniform(-3, 3, S)))
    ap, prob = case.aperture, case.problem()
    plan = SarPlan(case.scene, ap, upsample_ratio=8.0, interp="nearest_ref")
    assert plan.is_grid and plan.tile_window > 0
    M = int(8 * ap.num_freqs)
    s_r = ap.sample_bandwidth * M / (ap.num_freqs * ap.c_eff)
    kappa = ap.centre_frequency / ap.c_eff
    pos = case.scene.positions
    sets, flips = {}, 0
    for rule, off in (("adjoint", 0.5), ("forward", 0.0)):
        _, bn = host_eval_grid(case.scene, ap.transmitter_positions, ap.receiver_positions, ap.stab_ref_posns,
                               kappa, s_r, off, 1)
        chosen = []
        for s in range(S):
            _, tb = fp64_truth(ap.transmitter_positions[s], ap.receiver_positions[s], ap.stab_ref_posns[s], pos,
                               kappa, s_r)
            v = tb + off
            sel = np.argsort(np.abs(v - np.floor(v) - 0.5))[:32]
            exact = np.sign(v[sel]) * np.floor(np.abs(v[sel]) + 0.5)
            flips += int(np.sum(exact != np.round(bn[s][sel])))
            chosen.append(sel)
        sets[rule] = np.unique(np.concatenate(chosen))
    assert flips >= 1   # the FP32 polynomial alone would choose wrongly somewhere in the sets
    y = crandn(rng, S, ap.num_freqs)
    adj = gpu_adjoint(plan, y)[sets["adjoint"]]
    ref = oracle.adjoint(prob, y, "nearest_ref", threads=8)[sets["adjoint"]]
    assert np.abs(adj - ref).max() / np.abs(ref).max() < 1.0e-5
    x = np.zeros(plan.num_scatterers, np.complex128)
    x[sets["forward"]] = crandn(rng, sets["forward"].size)
    assert rel_l2(gpu_forward(plan, x), oracle.forward(prob, x, "nearest_ref", threads=8)) < 1.0e-5
    assert plan.device_flags() == 0


def test_little_golden_reference_criterion():
    """tests/test_cil.py:12-15 of the reference: adjoint of the noisy measurement, with the
    reference's defaults (nearest_ref, upsample 128) and its own elementwise criterion."""
    case = load_golden("little")
    op = NumpySimpleSarOperator(case.scene, case.aperture)
    adj = op.rmatvec(case.data["y"].reshape(-1))
    ref = case.data["adjoint"]
    assert rel_l2(adj, ref) < 1.0e-5
    assert adj == pytest.approx(ref, rel=1.0e-3)
    assert op.plan.device_flags() == 0


def test_little_golden_grid_path():
    """The same case through the grid fast path (windows too wide to stage: global reads, with
    the exact re-decision of nearest bins near a rounding boundary)."""
    case = load_golden("little")
    plan = SarPlan(case.scene, case.aperture, path="grid")
    assert plan.is_grid and plan.tile_window > 1024
    adj = gpu_adjoint(plan, case.data["y"])
    assert rel_l2(adj, case.data["adjoint"]) < 1.0e-5
    assert plan.device_flags() == 0


def test_little_forward_matches_oracle():
    case = load_golden("little")
    plan = SarPlan(case.scene, case.aperture)
    rng = np.random.default_rng(5)
    x = np.zeros(case.scene.num_scatterers, np.complex128)
    x[rng.choice(x.size, 30, replace=False)] = crandn(rng, 30)
    ref = oracle.forward(case.problem(), x, "nearest_ref", threads=8)
    assert rel_l2(gpu_forward(plan, x), ref) < NEAREST_TOL


@pytest.mark.parametrize("kind", ["config1", "bistatic_odd", "points", "odd_grid"])
def test_linear_matches_fp64_oracle(kind):
    rng = np.random.default_rng(11)
    if kind == "config1":
        # the CPU-runnable configuration at full size: 128 x 512, U = 8, 256^2 at 0.5 m
        case = spotlight_case(128, 512, 256, 0.5, 3.0)
        x = point_scene(rng, 256, 20)
    elif kind == "odd_grid":
        case = spotlight_case(40, 77, 45, 0.3, 4.0, upsample=5.0, bistatic=True,
                              weights=np.exp(1j * rng.uniform(-3, 3, 40)))
        x = crandn(rng, case.scene.num_scatterers)
    else:
        case = load_golden(kind)
        x = case.data["x"]
    y = crandn(rng, case.aperture.num_slow_times, case.aperture.num_freqs)
    p = case.problem()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    fwd_ref = oracle.forward(p, x, "linear", threads=8)
    adj_ref = oracle.adjoint(p, y, "linear", threads=8)
    e_f = rel_l2(gpu_forward(plan, x), fwd_ref)
    e_a = rel_l2(gpu_adjoint(plan, y), adj_ref)
    assert e_f < LINEAR_TOL, e_f
    assert e_a < LINEAR_TOL, e_a
    assert plan.device_flags() == 0


@pytest.mark.parametrize("mode", ["linear", "nearest_ref"])
@pytest.mark.parametrize("turn", [0, 1, 0.5, -0.5])
def test_gather_lane_layouts_match_oracle(turn, mode):
    """The grid backprojection runs its lanes along the axis where range bins change slowly:
    along y for a collection looking along x, along x once the collection is turned by 90
    degrees.  Both layouts against the FP64 oracle, with an odd pulse count (a padding pulse
    in the last stage of pulse pairs) and partial tiles; linear and split (nearest-bin) bins on
    the grid path.  The forward projection of the same plans runs its lanes the other way (along
    the axis where bins change fast, walking the slow one): lanes along x, then lanes along y on
    a transposed tile once turned, with register run windows (linear) and single-bin
    read-modify-writes (nearest) in both layouts.  turn = +-0.5: looking along a grid diagonal,
    where bins change alike along both axes: linear sampling walks a lattice sheared by -+1 pixel
    per row along the iso-range lines (register run windows again, partial lattice tiles at every
    image edge), nearest sampling keeps the plain layout (two-phase read-modify-writes); the linear
    backprojection runs on the same lattice with its lanes along the iso-range axis, where its
    window loads are broadcast, writing each image pixel from exactly one lattice tile."""
    rng = np.random.default_rng(21 + int(2 * turn))
    case = spotlight_case(37, 96, 70, 0.3, 4.0, weights=np.exp(1j * rng.uniform(-3, 3, 37)))
    if turn:
        c, s_ = np.cos(turn * np.pi / 2), np.sin(turn * np.pi / 2)
        rot = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
        ap = case.aperture
        case.aperture = NumpySimpleSarAperture(ap.transmitter_positions @ rot.T, ap.receiver_positions @ rot.T,
                                               ap.stab_ref_posns, ap.centre_frequency, ap.sample_bandwidth,
                                               num_freqs=ap.num_freqs, slow_time_weighting=ap.slow_time_weighting)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp=mode, path="grid")
    if abs(turn) != 0.5:
        assert plan.gather_lanes_y == (turn == 0) and plan.scatter_lanes_y == (turn == 1)
    assert plan.scatter_shear == ((-1 if turn > 0 else 1) if abs(turn) == 0.5 and mode == "linear" else 0)
    # the backprojection's lanes follow the same lattice axis on a diagonal (linear sampling)
    assert plan.gather_shear == ((-1 if turn > 0 else 1) if abs(turn) == 0.5 and mode == "linear" else 0)
    y = crandn(rng, 37, 96)
    tol = LINEAR_TOL   # nearest bins too: those near a rounding boundary are decided exactly
    e_a = rel_l2(gpu_adjoint(plan, y), oracle.adjoint(case.problem(), y, mode, threads=8))
    assert e_a < tol, e_a
    x = crandn(rng, case.scene.num_scatterers)
    e_f = rel_l2(gpu_forward(plan, x), oracle.forward(case.problem(), x, mode, threads=8))
    assert e_f < tol, e_f
    assert plan.device_flags() == 0


@pytest.mark.parametrize("mode", ["nearest_ref", "linear"])
@pytest.mark.parametrize("turn", [0, 1])
def test_value_windows_match_oracle(turn, mode):
    """Upsample 128 (nearest_ref with it: the reference's defaults): staged windows wider than 256
    bins, which store and stage plain values (half the bytes of pairs; linear sampling reads two
    neighbours), in both lane layouts, with an odd pulse count and partial tiles, against the FP64
    oracle (nearest bins near a rounding boundary are decided exactly, so the linear-mode
    tolerance holds)."""
    rng = np.random.default_rng(41 + turn)
    case = spotlight_case(37, 96, 70, 0.1, 4.0, upsample=128.0, weights=np.exp(1j * rng.uniform(-3, 3, 37)))
    if turn:
        ap = case.aperture
        rot = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
        case.aperture = NumpySimpleSarAperture(ap.transmitter_positions @ rot.T, ap.receiver_positions @ rot.T,
                                               ap.stab_ref_posns, ap.centre_frequency, ap.sample_bandwidth,
                                               num_freqs=ap.num_freqs, slow_time_weighting=ap.slow_time_weighting)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=128.0, interp=mode, path="grid")
    assert plan.is_grid and plan.tile_window > 256 and plan.gather_lanes_y == (turn == 0)
    y = crandn(rng, 37, 96)
    e_a = rel_l2(gpu_adjoint(plan, y), oracle.adjoint(case.problem(), y, mode, threads=8))
    assert e_a < LINEAR_TOL, e_a
    x = crandn(rng, case.scene.num_scatterers)
    e_f = rel_l2(gpu_forward(plan, x), oracle.forward(case.problem(), x, mode, threads=8))
    assert e_f < LINEAR_TOL, e_f
    assert plan.device_flags() == 0


@pytest.mark.parametrize("mode", ["nearest_ref", "linear"])
@pytest.mark.parametrize("turn", [0, 1])
def test_ring_windows_match_oracle(turn, mode):
    """Upsample 128 on 0.25 m pixels: a 32-pixel tile spans ~1200 range bins, so strip windows hold
    at most single tiles; the forward scatter keeps ring windows instead (slots = absolute bin mod a
    power of two, the bins each tile step leaves behind added to the accumulator), walking whole
    lines of tiles in both layouts.  Against the FP64 oracle with an odd pulse count and partial
    tiles (nearest bins near a rounding boundary decided exactly)."""
    rng = np.random.default_rng(71 + turn)
    # a 20 degree aperture: bins also drift ~6.6 per pixel along the lines, so no strip window holds
    # even one tile (strip windows would leave the scatter to the per-pixel kernel)
    case = spotlight_case(37, 96, 100, 0.25, 20.0, upsample=128.0, weights=np.exp(1j * rng.uniform(-3, 3, 37)))
    if turn:
        ap = case.aperture
        rot = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
        case.aperture = NumpySimpleSarAperture(ap.transmitter_positions @ rot.T, ap.receiver_positions @ rot.T,
                                               ap.stab_ref_posns, ap.centre_frequency, ap.sample_bandwidth,
                                               num_freqs=ap.num_freqs, slow_time_weighting=ap.slow_time_weighting)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=128.0, interp=mode, path="grid")
    assert plan.scatter_ring_half > 0, (plan.strip_window, plan.tile_window)
    assert plan.scatter_lanes_y == (turn == 1)
    x = crandn(rng, case.scene.num_scatterers)
    e_f = rel_l2(gpu_forward(plan, x), oracle.forward(case.problem(), x, mode, threads=8))
    assert e_f < LINEAR_TOL, e_f
    y = crandn(rng, 37, 96)
    e_a = rel_l2(gpu_adjoint(plan, y), oracle.adjoint(case.problem(), y, mode, threads=8))
    assert e_a < LINEAR_TOL, e_a
    if mode == "linear":   # exact transposes (nearest_ref's two rounding rules differ by design)
        lhs = np.vdot(gpu_forward(plan, x), y)
        rhs = np.vdot(x, gpu_adjoint(plan, y))
        assert abs(lhs - rhs) / abs(lhs) < 1e-5
    assert plan.device_flags() == 0


@pytest.mark.parametrize("turn", [0.5, -0.5])
def test_sheared_lattices_on_a_non_square_volume(turn):
    """The sheared lattices on a 2 x 40 x 70 grid (two height planes, 0.3 m pixels, not square) seen
    along a diagonal: lattice widths nx + (ny - 1), tiles clipped to the image per column, both
    planes; linear forward and backprojection against the FP64 oracle and their dot product."""
    rng = np.random.default_rng(81)
    base = spotlight_case(29, 96, 8, 0.3, 4.0, weights=np.exp(1j * rng.uniform(-3, 3, 29)))
    c, s_ = np.cos(turn * np.pi / 2), np.sin(turn * np.pi / 2)
    rot = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
    ap = base.aperture
    ap = NumpySimpleSarAperture(ap.transmitter_positions @ rot.T, ap.receiver_positions @ rot.T, ap.stab_ref_posns,
                                ap.centre_frequency, ap.sample_bandwidth, num_freqs=ap.num_freqs,
                                slow_time_weighting=ap.slow_time_weighting)
    scene = GridSarScene([2, 40, 70], [0.5, 0.3 * 39, 0.3 * 69])
    from cases import Case
    case = Case(scene, ap, 8.0, {})
    plan = SarPlan(scene, ap, upsample_ratio=8.0, interp="linear", path="grid")
    m = -1 if turn > 0 else 1
    assert plan.scatter_shear == m and plan.gather_shear == m
    x = crandn(rng, scene.num_scatterers)
    e_f = rel_l2(gpu_forward(plan, x), oracle.forward(case.problem(), x, "linear", threads=8))
    assert e_f < LINEAR_TOL, e_f
    y = crandn(rng, 29, 96)
    e_a = rel_l2(gpu_adjoint(plan, y), oracle.adjoint(case.problem(), y, "linear", threads=8))
    assert e_a < LINEAR_TOL, e_a
    lhs = np.vdot(gpu_forward(plan, x), y)
    rhs = np.vdot(x, gpu_adjoint(plan, y))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    assert plan.device_flags() == 0


@pytest.mark.parametrize("turn", [0.5, -0.5])
def test_sheared_gather_with_split_bins_matches_oracle(turn):
    """Linear sampling at upsample 128 looking along a diagonal: the backprojection runs on the
    sheared lattice with split bins (windows wider than 256 bins: exact integer parts), the
    forward projection on the plain layout (split bins take no lattice); both against the FP64
    oracle, with an odd pulse count and partial lattice tiles."""
    rng = np.random.default_rng(61)
    case = spotlight_case(37, 96, 70, 0.1, 4.0, upsample=128.0, weights=np.exp(1j * rng.uniform(-3, 3, 37)))
    c, s_ = np.cos(turn * np.pi / 2), np.sin(turn * np.pi / 2)
    rot = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
    ap = case.aperture
    case.aperture = NumpySimpleSarAperture(ap.transmitter_positions @ rot.T, ap.receiver_positions @ rot.T,
                                           ap.stab_ref_posns, ap.centre_frequency, ap.sample_bandwidth,
                                           num_freqs=ap.num_freqs, slow_time_weighting=ap.slow_time_weighting)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=128.0, interp="linear", path="grid")
    assert plan.gather_shear == (-1 if turn > 0 else 1) and plan.scatter_shear == 0
    assert plan.tile_window > 256
    y = crandn(rng, 37, 96)
    e_a = rel_l2(gpu_adjoint(plan, y), oracle.adjoint(case.problem(), y, "linear", threads=8))
    assert e_a < LINEAR_TOL, e_a
    x = crandn(rng, case.scene.num_scatterers)
    e_f = rel_l2(gpu_forward(plan, x), oracle.forward(case.problem(), x, "linear", threads=8))
    assert e_f < LINEAR_TOL, e_f
    assert plan.device_flags() == 0


@pytest.mark.parametrize("az", [10.0, 20.0, 30.0, 63.43, -30.0, 150.0, 210.0])
def test_oblique_forward_matches_oracle(az):
    """Collections looking between the grid's axes and diagonals (linear, upsample 8, 0.3 m pixels:
    2.9 bins per pixel along the look direction): the walked axis moves the bins by 0.4 to 1.5 per
    row, too fast for run windows, so the scatter reads and writes both taps per row (one phase
    where the lanes lie two bins apart, two where only one), in all four sign combinations of lane
    and walk rates, and pulse pairs whose modes differ share only what both admit.  Forward
    against the FP64 oracle with an odd pulse count and partial tiles, and its dot product with the
    backprojection."""
    rng = np.random.default_rng(97)
    case = spotlight_case(37, 96, 70, 0.3, 4.0, weights=np.exp(1j * rng.uniform(-3, 3, 37)))
    c, s_ = np.cos(np.radians(az)), np.sin(np.radians(az))
    rot = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
    ap = case.aperture
    case.aperture = NumpySimpleSarAperture(ap.transmitter_positions @ rot.T, ap.receiver_positions @ rot.T,
                                           ap.stab_ref_posns, ap.centre_frequency, ap.sample_bandwidth,
                                           num_freqs=ap.num_freqs, slow_time_weighting=ap.slow_time_weighting)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=8.0, interp="linear", path="grid")
    assert plan.is_grid and plan.scatter_shear == 0
    x = crandn(rng, case.scene.num_scatterers)
    fx = gpu_forward(plan, x)
    e_f = rel_l2(fx, oracle.forward(case.problem(), x, "linear", threads=8))
    assert e_f < LINEAR_TOL, e_f
    y = crandn(rng, 37, 96)
    lhs = np.vdot(fx, y)
    rhs = np.vdot(x, gpu_adjoint(plan, y))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    assert plan.device_flags() == 0


@pytest.mark.parametrize("U", [16.0, 128.0])
@pytest.mark.parametrize("az,m", [(63.43, -2), (-63.43, 2), (116.57, 2)])
def test_gather_lattice_sheared_by_two(az, m, U):
    """Collections looking at ~63 degrees to the grid's x axis (tan = 2): the bins change least
    along ey - 2 ex (or ey + 2 ex), so the linear backprojection runs on a lattice sheared by two
    pixels per row (lattice width nx + 2 (ny - 1), slanted tile clipping at every image edge) with
    its lanes along that axis; the forward projection keeps the plain layout.  Against the FP64
    oracle at upsample 16 and 128 (split bins), with an odd pulse count."""
    rng = np.random.default_rng(91)
    case = spotlight_case(37, 96, 70, 0.3, 4.0, upsample=U, weights=np.exp(1j * rng.uniform(-3, 3, 37)))
    c, s_ = np.cos(np.radians(az)), np.sin(np.radians(az))
    rot = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
    ap = case.aperture
    case.aperture = NumpySimpleSarAperture(ap.transmitter_positions @ rot.T, ap.receiver_positions @ rot.T,
                                           ap.stab_ref_posns, ap.centre_frequency, ap.sample_bandwidth,
                                           num_freqs=ap.num_freqs, slow_time_weighting=ap.slow_time_weighting)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=U, interp="linear", path="grid")
    assert plan.gather_shear == m and plan.scatter_shear == 0
    y = crandn(rng, 37, 96)
    e_a = rel_l2(gpu_adjoint(plan, y), oracle.adjoint(case.problem(), y, "linear", threads=8))
    assert e_a < LINEAR_TOL, e_a
    x = crandn(rng, case.scene.num_scatterers)
    e_f = rel_l2(gpu_forward(plan, x), oracle.forward(case.problem(), x, "linear", threads=8))
    assert e_f < LINEAR_TOL, e_f
    assert plan.device_flags() == 0


@pytest.mark.parametrize("mode,srp_shift,nf,U,spacing,direct", [
    ("linear", 0.0, 4096, 8, 0.5, False), ("nearest_ref", 0.0, 4096, 8, 0.5, False),
    ("linear", 1.0, 4096, 8, 0.5, False), ("linear", 0.0, 2048, 8, 0.5, False),
    ("linear", 0.0, 1024, 8, 0.5, False), ("nearest_ref", 1.0, 1024, 8, 0.5, False),
    ("linear", 0.0, 512, 8, 0.5, False), ("nearest_ref", 1.0, 512, 8, 0.5, False),
    ("linear", 0.0, 8192, 8, 0.5, False), ("linear", 1.0, 8192, 64, 1.5, True),
    ("linear", 0.0, 1024, 128, 1.5, True), ("nearest_ref", 1.0, 1024, 128, 1.5, True),
    ("linear", 1.0, 2048, 128, 0.25, False)])
def test_fused_upsampling_matches_oracle(mode, srp_shift, nf, U, spacing, direct):
    """N = 512 ... 8192 samples: the range profiles come from the fused upsampling kernel (U
    N-point transforms per pulse: a radix-2, 4, 8 or 16 first pass and two or, at 8192, three
    radix-16 passes; stored span only), and the forward projection ends in the fused downsampling
    kernel (its transpose).  Against the FP64 oracle in both modes; the stored span starts below
    bin 0 (taken modulo M), also with the SRP moved off the scene centre.  Where the scene is wide
    enough that the span's U residues do not fit shared memory the upsampling writes each
    transform's bins straight to its row (direct form; nearest bins as plain values at U = 128)."""
    rng = np.random.default_rng(31)
    case = spotlight_case(48, nf, 48, spacing, 3.0, upsample=float(U), weights=np.exp(1j * rng.uniform(-3, 3, 48)))
    if srp_shift:
        ap = case.aperture
        srp = np.tile(np.array([12.0, -3.0, 0.0]), (48, 1))
        case.aperture = NumpySimpleSarAperture(ap.transmitter_positions, ap.receiver_positions, srp,
                                               ap.centre_frequency, ap.sample_bandwidth, num_freqs=nf,
                                               slow_time_weighting=ap.slow_time_weighting)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=float(U), interp=mode)
    assert plan.fused_upsampling and plan.fused_downsampling
    assert plan.profile_first_bin < 0
    # direct form exactly when the residue-major staging would need more than the kernel's shared
    # memory (two CTAs per SM up to N = 4096, one at 8192)
    row = ((plan.profile_length + U) // U + 13) // 16 * 16 + 2
    budget = (220 if nf >= 8192 else 112) * 1024
    assert (8 * (2 * (nf + nf // 16) + U * row) > budget) == direct
    y = crandn(rng, 48, nf)
    got = gpu_adjoint(plan, y)
    ref = oracle.adjoint(case.problem(), y, mode, threads=8)
    tol = LINEAR_TOL   # nearest bins too: those near a rounding boundary are decided exactly
    assert rel_l2(got, ref) < tol
    # the forward projection's fused downsampling against the oracle's forward
    x = crandn(rng, case.scene.num_scatterers)
    assert rel_l2(gpu_forward(plan, x), oracle.forward(case.problem(), x, mode, threads=8)) < tol
    assert plan.device_flags() == 0


def test_backproject_reads_pinned_host_input_in_place():
    """With the fused upsampling a pinned host phase history is read by the device directly
    (sar_host_device_pointer + sar_adjoint); the image equals the device-input one bit for bit,
    as does the copy path for pageable memory, and the call returns only when y may be reused."""
    rng = np.random.default_rng(8)
    case = spotlight_case(40, 4096, 40, 0.5, 3.0)
    op = NumpySimpleSarOperator(case.scene, case.aperture, upsample_ratio=8.0, interp="linear")
    assert op.plan.fused_upsampling
    y = crandn(rng, 40, 4096).astype(np.complex64)
    ref = op.plan.adjoint(torch.from_numpy(y).cuda())
    yp = torch.from_numpy(y.copy()).pin_memory()
    lib = _lib.load()
    dev = ctypes.c_void_p()
    assert lib.sar_host_device_pointer(ctypes.c_void_p(yp.data_ptr()), ctypes.byref(dev)) == 0 and dev.value
    x_pinned = op.backproject(yp)
    yp.zero_()   # y may be reused once the call has returned
    assert torch.equal(x_pinned, ref)
    assert torch.equal(op.backproject(torch.from_numpy(y.copy())), ref)   # pageable: copied first
    # pageable memory: refused where the device cannot address it, the same address where it can
    # (address translation over the chip-to-chip link); the operator reads only pinned tensors in place
    page = np.zeros(4, np.complex64)
    rc = lib.sar_host_device_pointer(ctypes.c_void_p(page.ctypes.data), ctypes.byref(dev))
    assert rc == _lib.SAR_ERR_INVALID_ARGUMENT or (rc == 0 and dev.value == page.ctypes.data)
    assert op.plan.device_flags() == 0


@pytest.mark.parametrize("kind", ["grid", "points", "bistatic", "turned", "diagonal"])
def test_dot_product_adjoint(kind):
    rng = np.random.default_rng(2)
    if kind == "points":
        case = load_golden("points")
    else:
        case = spotlight_case(96, 256, 100, 0.5, 5.0, bistatic=(kind == "bistatic"),
                              weights=np.exp(1j * rng.uniform(-2, 2, 96)))
    if kind in ("turned", "diagonal"):   # looking along y (the scatter walks x), or the diagonal
        ap = case.aperture
        c, s_ = (0.0, 1.0) if kind == "turned" else (np.sqrt(0.5), np.sqrt(0.5))
        rot = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
        case.aperture = NumpySimpleSarAperture(ap.transmitter_positions @ rot.T, ap.receiver_positions @ rot.T,
                                               ap.stab_ref_posns, ap.centre_frequency, ap.sample_bandwidth,
                                               num_freqs=ap.num_freqs, slow_time_weighting=ap.slow_time_weighting)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    x = torch.from_numpy(crandn(rng, case.scene.num_scatterers)).to(torch.complex64).cuda()
    y = torch.from_numpy(crandn(rng, case.aperture.num_slow_times, case.aperture.num_freqs)).to(torch.complex64).cuda()
    ax = plan.forward(x)
    ahy = plan.adjoint(y)
    lhs = torch.vdot(y.reshape(-1).to(torch.complex128), ax.reshape(-1).to(torch.complex128))
    rhs = torch.vdot(ahy.to(torch.complex128), x.to(torch.complex128))
    scale = torch.linalg.norm(ax.to(torch.complex128)) * torch.linalg.norm(y.to(torch.complex128))
    assert (abs(lhs - rhs) / scale).item() < 1.0e-6


def test_profiles_match_oracle_upsampling():
    case = spotlight_case(16, 200, 64, 0.5, 3.0)
    rng = np.random.default_rng(4)
    y = crandn(rng, 16, 200)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=8.0, interp="linear")
    prof = plan.profiles(torch.from_numpy(y)).cpu().numpy()
    full = oracle.upsample(case.problem(), y)
    m = full.shape[1]
    bins = (plan.profile_first_bin + np.arange(plan.profile_length)) % m
    assert rel_l2(prof, full[:, bins]) < 2.0e-6


def test_profiles_prime_factor_length():
    """Working length M = 251 * 128 (the reference's little case): the double-precision
    transform keeps the upsampled profiles at FP32 accuracy."""
    case = load_golden("little")
    plan = SarPlan(case.scene, case.aperture, interp="linear")
    prof = plan.profiles(torch.from_numpy(case.data["y"])).cpu().numpy()
    full = oracle.upsample(case.problem(), case.data["y"], threads=8)
    bins = (plan.profile_first_bin + np.arange(plan.profile_length)) % full.shape[1]
    assert rel_l2(prof, full[:, bins]) < 1.0e-6


def test_dropin_struct_entry_points():
    """forward_evaluate / adjoint_evaluate with the reference's SarCalculationInfo."""
    case = load_golden("spot_small")
    ap, sc = case.aperture, case.scene
    lib = _lib.load()
    S, N, P = ap.num_slow_times, ap.num_freqs, sc.num_scatterers
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    tx, rx, srp, pos = f64(ap.transmitter_positions), f64(ap.receiver_positions), f64(ap.stab_ref_posns), f64(sc.positions)
    wf = np.ascontiguousarray(np.fft.ifftshift(ap.waveform_fft).astype(np.complex128)).view(np.float64)
    wt = np.ascontiguousarray(ap.slow_time_weighting.astype(np.complex128)).view(np.float64)
    ptr = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    def run(fn, ph, amps):
        info = _lib.SarCalculationInfo(N, S, P, ptr(tx), ptr(rx), ptr(srp), ptr(pos), ptr(ph), ptr(amps), ptr(wf),
                                       ptr(wt), ap.centre_frequency, ap.sample_bandwidth, ap.c_eff,
                                       case.upsample_ratio, ap.sign_multiplier)
        getattr(lib, fn)(ctypes.byref(info))

    ph = np.zeros((S, N, 2))
    amps = np.ascontiguousarray(case.data["x"].astype(np.complex128)).view(np.float64).copy()
    run("forward_evaluate", ph, amps)
    fwd = np.fft.fftshift(ph[..., 0] + 1j * ph[..., 1], axes=1)        # forward.py:44
    assert rel_l2(fwd, case.data["forward"]) < NEAREST_TOL
    yin = np.fft.ifftshift(case.data["y"], axes=1)                       # adjoint.py:36
    ph = np.ascontiguousarray(yin.astype(np.complex128)).view(np.float64).reshape(S, N, 2).copy()
    amps = np.zeros((P, 2))
    run("adjoint_evaluate", ph, amps)
    assert rel_l2(amps[:, 0] + 1j * amps[:, 1], case.data["adjoint"]) < NEAREST_TOL


@pytest.mark.parametrize("S,N,shape,U", [
    (1, 64, (1, 32, 32), 8.0),      # one pulse
    (7, 1, (1, 5, 3), 4.0),         # one frequency sample
    (9, 31, (1, 1, 1), 8.0),        # one pixel
    (12, 48, (1, 33, 65), 1.0),     # M == N, partial tiles
    (10, 40, (3, 20, 20), 16.0),    # 3-D grid
])
def test_edge_shapes_match_oracle(S, N, shape, U):
    rng = np.random.default_rng(sum(shape) + S)
    tx = np.stack([np.full(S, 3000.0), np.linspace(-40, 40, S), np.full(S, 1200.0)], -1)
    ap = NumpySimpleSarAperture(tx, tx.copy(), np.zeros((S, 3)), 9.0e9, 150.0e6, num_freqs=N)
    nz, ny, nx = shape
    scene = GridSarScene(list(shape), [0.4 * max(nz - 1, 0), 0.3 * max(ny - 1, 0), 0.3 * max(nx - 1, 0)])
    p = oracle.Problem(tx, tx, np.zeros((S, 3)), scene.positions, 9.0e9, 150.0e6, N, upsample_ratio=U)
    x = crandn(rng, scene.num_scatterers)
    y = crandn(rng, S, N)
    plan = SarPlan(scene, ap, upsample_ratio=U, interp="linear")
    assert rel_l2(gpu_forward(plan, x), oracle.forward(p, x, "linear")) < LINEAR_TOL
    assert rel_l2(gpu_adjoint(plan, y), oracle.adjoint(p, y, "linear")) < LINEAR_TOL
    assert plan.device_flags() == 0


def test_numpy_operator_api_shapes_and_dtypes():
    case = load_golden("spot_small")
    op = NumpySimpleSarOperator(case.scene, case.aperture, upsample_ratio=8.0, interp="linear")
    assert op.shape == (case.aperture.num_freqs * case.aperture.num_slow_times, case.scene.num_scatterers)
    assert op.dtype == np.complex128
    y = op.matvec(case.data["x"])
    x = op.rmatvec(case.data["y"].reshape(-1))
    assert y.dtype == np.complex128 and y.shape == (op.shape[0],)
    assert x.dtype == np.complex128 and x.shape == (op.shape[1],)
    z = (op.H @ (op @ case.data["x"]))
    assert z.shape == (op.shape[1],)
    # tensors stay on the device
    xt = op.backproject(torch.from_numpy(case.data["y"]).cuda())
    assert xt.is_cuda and xt.dtype == torch.complex64
