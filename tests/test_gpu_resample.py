"""GPU dataset resampling against the reference's own outputs (tests/golden/resample_*.npz,
made by tests/golden/make_resample_golden.py from the reference's utils and
NumpySimpleSarDataset.from_resampling): SRP rephasing, fast-frequency downsampling, the full
resampling with a slow-time filter, odd N, sign -1, and a pulse with non-finite positions."""
import os

import numpy as np
import pytest
import torch

from sarsolver_gb300 import resample as rs
from sarsolver_gb300.geometry import NumpySimpleSarAperture, NumpySimpleSarDataset

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("name", ["a", "b", "c"])
def test_resampling_matches_reference(name):
    d = dict(np.load(os.path.join(GOLDEN, f"resample_{name}.npz")))
    fc, fs, sign = float(d["centre_frequency"]), float(d["sample_frequency"]), float(d["sign_multiplier"])
    moved = rs.move_srps(d["ph"], d["srps"], d["new_srp"], d["tx"], d["rx"], fc, fs, sign)
    ok = np.isfinite(d["moved"]).all(axis=1)
    assert rel(moved[ok], d["moved"][ok]) < 1e-6
    ffd = rs.fast_freq_downsample(d["ph"], int(d["n_new"]), 1.2)
    assert rel(ffd, d["ffd"]) < 1e-6
    np.testing.assert_allclose(rs.get_downsample_kernel(max(int(d["slow_factor"]), 1)), d["kernel"], rtol=1e-6, atol=1e-7)
    ap = NumpySimpleSarAperture(d["tx"], d["rx"], d["srps"], fc, fs, waveform_fft=d["wave"],
                                slow_time_weighting=d["wt"], sign_multiplier=sign)
    amb = {}
    if float(d["range_amb"]) > 0:   # the reference chose the factors from ambiguous extents
        amb = dict(range_amb=float(d["range_amb"]), cross_range_amb=float(d["cross_range_amb"]))
    out = rs.resample_dataset(NumpySimpleSarDataset(ap, d["ph"]), fast_downsample_factor=float(d["fast_factor"]) or 1.0,
                              slow_downsample_factor=int(d["slow_factor"]) or 1, new_srp=d["new_srp"],
                              safety_factor=1.2, **amb)
    oap = out.aperture
    assert out.phase_history().shape == d["out_ph"].shape
    assert rel(out.phase_history(), d["out_ph"]) < 1e-5
    np.testing.assert_array_equal(oap.transmitter_positions, d["out_tx"])
    np.testing.assert_array_equal(oap.receiver_positions, d["out_rx"])
    np.testing.assert_allclose(oap.stab_ref_posns, d["out_srps"])
    np.testing.assert_allclose(oap.slow_time_weighting, d["out_wt"], rtol=1e-6)
    assert rel(oap.waveform_fft, d["out_wave"]) < 1e-6


def test_large_phase_ramps_stay_accurate():
    """Hundreds of turns of phase per pulse (a 600 m SRP move at 10 GHz): the device phase keeps
    FP64-level accuracy (split slope, FP64-reduced constant)."""
    rng = np.random.default_rng(3)
    S, N = 64, 2048
    az = np.deg2rad(np.linspace(-2, 2, S))
    tx = np.stack([10e3 * np.cos(az), 10e3 * np.sin(az), np.full(S, 5e3)], axis=-1)
    ph = (rng.standard_normal((S, N)) + 1j * rng.standard_normal((S, N))) / np.sqrt(2)
    old = np.zeros((S, 3))
    new = np.array([400.0, 450.0, 0.0])
    got = rs.move_srps(ph, old, new, tx, tx, 10e9, 200e6, 1.0)
    dr = rs.range_changes(old, new, tx, tx)[:, None]
    bb = np.fft.fftshift(np.fft.fftfreq(N, 1.0 / 200e6))[None, :]
    ref = ph * np.exp(2j * np.pi * dr / 299792458.0 * (bb - 10e9))
    assert np.abs(dr).max() > 300.0
    assert rel(got, ref) < 2e-6


def test_resampling_throughput_report():
    """8192 pulses x 8192 samples (0.5 GB complex64) resampled by 2 in both dimensions; prints the
    device time and the effective bandwidth of the HBM-bound passes."""
    import time
    rng = np.random.default_rng(5)
    S, N = 8192, 8192
    az = np.deg2rad(np.linspace(-3, 3, S))
    tx = np.stack([10e3 * np.cos(az), 10e3 * np.sin(az), np.full(S, 5e3)], axis=-1)
    ap = NumpySimpleSarAperture(tx, tx, np.zeros((S, 3)), 10e9, 200e6, num_freqs=N)
    ph = torch.complex(torch.randn(S, N, device="cuda"), torch.randn(S, N, device="cuda"))
    ds = NumpySimpleSarDataset(ap, ph)
    out = rs.resample_dataset(ds, 2.0, 2, new_srp=np.array([5.0, 5.0, 0.0]), keep_on_device=True)   # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    out = rs.resample_dataset(ds, 2.0, 2, new_srp=np.array([5.0, 5.0, 0.0]), keep_on_device=True)
    e1.record()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    dev_ms = e0.elapsed_time(e1)
    T, n = out.phase_history().shape
    # passes over HBM: read S*N, write S*N, FFT S*N (read+write), crop read S*n + write S*n, FFT S*n,
    # filter reads 10 taps per output row (L2-resident rows) and writes T*n.
    moved = 8.0 * (2 * S * N + 2 * S * N + 2 * S * n + 2 * S * n + T * n)
    print(f"resample {S}x{N} -> {T}x{n}: {dt * 1e3:.2f} ms wall ({dev_ms:.2f} ms between events on the stream), "
          f"{moved / dt / 1e9:.0f} GB/s over the main passes")
    assert T > 0 and n == 4097
