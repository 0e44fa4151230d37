"""Dataset and aperture containers on the CPU: concatenation (numpy/measurement.py:463-504),
subsets and the frequency axis, with the reference's semantics."""
import numpy as np

from cases import C, crandn, spotlight
from sarsolver_gb300.geometry import NumpySimpleSarAperture, NumpySimpleSarDataset


def make_dataset(rng, S, N, az, c_eff=C):
    tx = spotlight(S, 3.0, centre_az_deg=az)
    rx = spotlight(S, 2.0, 8.0e3, 3.0e3, az + 10.0)
    srp = rng.normal(0.0, 2.0, (S, 3))
    wf = crandn(rng, N)
    w = np.exp(1j * rng.uniform(-1, 1, S))
    return NumpySimpleSarDataset.from_scratch(tx, rx, srp, 9.6e9, 150.0e6, phase_history=crandn(rng, S, N),
                                              waveform_fft=wf, slow_time_weighting=w, sign_multiplier=-1.0,
                                              c_eff=c_eff)


def test_from_datasets_concatenates_pulses():
    rng = np.random.default_rng(3)
    a = make_dataset(rng, 5, 64, 0.0, c_eff=2.9e8)
    b = make_dataset(rng, 7, 64, 20.0, c_eff=2.9e8)
    ab = NumpySimpleSarDataset.from_datasets([a, b])
    ap, pa, pb = ab.aperture, a.aperture, b.aperture
    assert ap.num_slow_times == 12 and ap.num_freqs == 64
    for name in ("transmitter_positions", "receiver_positions", "stab_ref_posns", "slow_time_weighting"):
        np.testing.assert_array_equal(getattr(ap, name), np.concatenate([getattr(pa, name), getattr(pb, name)]))
    np.testing.assert_array_equal(ab.phase_history(), np.concatenate([a.phase_history(), b.phase_history()]))
    # band, waveform, sign and c_eff come from the first dataset
    np.testing.assert_array_equal(ap.waveform_fft, pa.waveform_fft)
    assert ap.centre_frequency == pa.centre_frequency and ap.sample_bandwidth == pa.sample_bandwidth
    assert ap.sign_multiplier == -1.0 and ap.c_eff == 2.9e8
    # a subset of the concatenation is the second dataset again
    sub = ab.get_subset(slice(5, 12))
    np.testing.assert_array_equal(sub.phase_history(), b.phase_history())
    np.testing.assert_array_equal(sub.aperture.transmitter_positions, pb.transmitter_positions)


def test_frequency_axis_is_centred_and_fftshifted():
    rng = np.random.default_rng(4)
    for N in (64, 65):
        ap = make_dataset(rng, 2, N, 0.0).aperture
        f = ap.freqs
        f = f() if callable(f) else f
        df = ap.sample_bandwidth / N
        np.testing.assert_allclose(np.diff(f), df, rtol=1e-9)
        # the centre frequency sits at index N // 2 (fftshift order of np.fft.fftfreq)
        assert abs(f[N // 2] - ap.centre_frequency) < 1e-6 * df
        assert isinstance(ap, NumpySimpleSarAperture)
