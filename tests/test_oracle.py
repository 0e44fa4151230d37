"""The CPU oracle, pinned against the reference before it is trusted.

* golden fixtures produced by the reference's own Python API (tests/golden/make_golden.py),
  including the reference's "little" adjoint artifact (tests/test_cil.py:12-15 upstream);
* the reference kernel itself, compiled from its sources against the FFTW-API shim
  (oracle/_ref, present only where the reference checkout exists);
* the exact-transpose property of the linear mode.
"""
import os

import numpy as np
import pytest

import oracle
from cases import crandn, load_golden, rel_l2, spotlight_case


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 12, 17, 64, 251, 1000, 4096])
def test_fft64_matches_numpy(n):
    import ctypes
    rng = np.random.default_rng(n)
    x = crandn(rng, n)
    # exercise through the oracle's upsample (M = N * 1, single pulse, unit waveform) -> N * ifft
    p = oracle.Problem(np.array([[1.0e3, 0, 0]]), np.array([[1.0e3, 0, 0]]), np.zeros((1, 3)),
                       np.zeros((1, 3)), 1.0e9, 1.0e8, n, upsample_ratio=1.0)
    prof = oracle.upsample(p, np.fft.fftshift(x)[None, :])[0]
    ref = np.fft.ifft(x) * n
    assert rel_l2(prof, ref) < 1e-13


@pytest.mark.parametrize("name", ["spot_small", "bistatic_odd", "points"])
def test_oracle_matches_reference_goldens(name):
    case = load_golden(name)
    p = case.problem()
    fwd = oracle.forward(p, case.data["x"], "nearest_ref", threads=4)
    adj = oracle.adjoint(p, case.data["y"], "nearest_ref", threads=4)
    assert rel_l2(fwd, case.data["forward"]) < 1e-12
    assert rel_l2(adj, case.data["adjoint"]) < 1e-12


def test_oracle_matches_little_backprojection():
    """The reference's own test_adjoint artifact (upsample 128, prime-factor M = 32128)."""
    case = load_golden("little")
    p = case.problem()
    assert list(case.scene.grid_shape) == [1, 244, 241]
    adj = oracle.adjoint(p, case.data["y"], "nearest_ref", threads=8)
    ref = case.data["adjoint"]
    assert rel_l2(adj, ref) < 1e-12
    assert adj == pytest.approx(ref, rel=1e-3)   # the reference test's own criterion


@pytest.mark.skipif(not oracle.reference_available(), reason="reference kernel not built here")
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_restatement_bit_matches_reference_kernel(seed):
    rng = np.random.default_rng(seed)
    S, N, U = 12, 33 + seed, 4.0 + seed
    case = spotlight_case(S, N, 16, 0.4, 3.0, upsample=U, bistatic=bool(seed % 2),
                          weights=np.exp(1j * rng.uniform(-1, 1, S)))
    p = case.problem()
    p.waveform_fft = crandn(rng, N)
    x = crandn(rng, case.scene.num_scatterers)
    y = crandn(rng, S, N)
    assert rel_l2(oracle.forward(p, x, "nearest_ref"), oracle.reference_forward(p, x)) < 1e-14
    assert rel_l2(oracle.adjoint(p, y, "nearest_ref"), oracle.reference_adjoint(p, y)) < 1e-14


@pytest.mark.parametrize("bistatic", [False, True])
def test_linear_mode_is_exact_transpose(bistatic):
    rng = np.random.default_rng(7)
    S, N = 16, 48
    case = spotlight_case(S, N, 24, 0.5, 4.0, bistatic=bistatic, weights=np.exp(1j * rng.uniform(-2, 2, S)))
    p = case.problem()
    p.waveform_fft = crandn(rng, N)
    x = crandn(rng, case.scene.num_scatterers)
    y = crandn(rng, S, N)
    lhs = np.vdot(y, oracle.forward(p, x, "linear"))
    rhs = np.vdot(oracle.adjoint(p, y, "linear"), x)
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


def test_reference_conventions_are_not_an_adjoint_pair():
    """Documents the reference's own pair: round(v) vs round(0.5+v) bins and an unconjugated
    slow-time weight in the adjoint (sarsolver_cxx.cpp:289, :347, :349)."""
    rng = np.random.default_rng(3)
    S, N = 16, 48
    case = spotlight_case(S, N, 24, 0.5, 4.0, weights=np.exp(1j * rng.uniform(-2, 2, S)))
    p = case.problem()
    x = crandn(rng, case.scene.num_scatterers)
    y = crandn(rng, S, N)
    lhs = np.vdot(y, oracle.forward(p, x, "nearest_ref"))
    rhs = np.vdot(oracle.adjoint(p, y, "nearest_ref"), x)
    assert abs(lhs - rhs) / abs(lhs) > 1e-3


# ------------------------------------------------------------------ dataset resampling oracle
@pytest.mark.parametrize("name", ["a", "b", "c"])
def test_resample_oracle_matches_reference_golden(name):
    from oracle import resample as rs
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", f"resample_{name}.npz")))
    fc, fs, sign = float(d["centre_frequency"]), float(d["sample_frequency"]), float(d["sign_multiplier"])
    moved = rs.move_srps(d["ph"], d["srps"], d["new_srp"], d["tx"], d["rx"], fc, fs, sign)
    ok = np.isfinite(d["moved"]).all(axis=1)
    np.testing.assert_allclose(moved[ok], d["moved"][ok], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(rs.fast_freq_downsample(d["ph"], int(d["n_new"]), 1.2), d["ffd"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(rs.downsample_kernel(max(int(d["slow_factor"]), 1)), d["kernel"], rtol=1e-6, atol=1e-7)
    fast, slow = float(d["fast_factor"]), int(d["slow_factor"])
    if float(d["range_amb"]) > 0:
        S, N = d["ph"].shape
        fast, slow = rs.factors_from_ambiguities(d["tx"], d["rx"], d["new_srp"], fc, fs, S, N, float(d["range_amb"]),
                                                 float(d["cross_range_amb"]))
    tx, rx, srps, wt, wave, ph = rs.resample(d["tx"], d["rx"], d["srps"], d["ph"], d["wave"], d["wt"], fc, fs, sign,
                                              fast, slow, d["new_srp"])
    np.testing.assert_array_equal(tx, d["out_tx"])
    np.testing.assert_array_equal(rx, d["out_rx"])
    np.testing.assert_allclose(srps, d["out_srps"])
    np.testing.assert_allclose(wt, d["out_wt"], rtol=1e-6)
    np.testing.assert_allclose(wave, d["out_wave"], rtol=1e-10, atol=1e-12)
    assert ph.shape == d["out_ph"].shape
    np.testing.assert_allclose(ph, d["out_ph"], rtol=1e-6, atol=1e-9)
