"""Generate tests/golden/resample_*.npz by running the reference's dataset resampling.

    python tests/golden/make_resample_golden.py [--reference /root/reference]

Uses the same reference import as make_golden.py (package copied to a temporary directory,
stub pymap3d).  Each fixture holds the input dataset (positions, SRPs with per-pulse offsets,
waveform, slow-time weighting, phase history) and the outputs of
  * utils.move_srps (src/sarsolver/utils/geodesy.py:33-73),
  * utils.fast_freq_downsample (src/sarsolver/utils/signal.py:45-77),
  * utils.get_downsample_kernel (src/sarsolver/utils/signal.py:7-27),
  * NumpySimpleSarDataset.from_resampling (src/sarsolver/numpy/measurement.py:342-458).
Case "b" has one pulse with a NaN SRP, so windows containing it are dropped.
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import import_reference  # noqa: E402

CASES = {
    "a": dict(S=160, N=96, fast=1.6, slow=3, sign=1.0, nan_pulse=None, seed=1),
    "b": dict(S=121, N=75, fast=2.3, slow=2, sign=-1.0, nan_pulse=37, seed=2),
    # factors chosen by the reference from ambiguous range / cross range (k-space extent)
    "c": dict(S=200, N=128, fast=None, slow=None, sign=1.0, nan_pulse=None, seed=3, range_amb=30.0,
              cross_range_amb=5.0),
}


def spotlight(S, deg, radius=10.0e3, alt=5.0e3):
    az = np.deg2rad(np.linspace(-0.5, 0.5, S) * deg)
    return np.stack([radius * np.cos(az), radius * np.sin(az), np.full(S, alt)], axis=-1)


def make_case(ref, name, S, N, fast, slow, sign, nan_pulse, seed, range_amb=None, cross_range_amb=None):
    rng = np.random.default_rng(seed)
    crandn = lambda *sh: (rng.standard_normal(sh) + 1j * rng.standard_normal(sh)) / np.sqrt(2)
    tx = spotlight(S, 4.0)
    rx = tx.copy()
    srps = rng.normal(0.0, 3.0, (S, 3))
    if nan_pulse is not None:
        srps[nan_pulse, 1] = np.nan
    ph = crandn(S, N)
    wave = crandn(N)
    wt = crandn(S)
    new_srp = np.array([4.0, -2.5, 0.3])
    fc, fs = 9.6e9, 150.0e6
    utils = ref["utils"]
    DS = ref["NumpySimpleSarDataset"]
    moved = utils.move_srps(ph, srps, new_srp, tx, rx, fc, fs, sign)
    n_new = int(1.0 + N / (fast or 1.0))
    ffd = utils.fast_freq_downsample(ph, n_new, 1.2)
    kern = utils.get_downsample_kernel(slow or 1)
    ds = DS.from_scratch(trans_posns=tx, rec_posns=rx, srps=srps, centre_freq=fc, sample_freq=fs, phase_history=ph,
                         waveform_fft=wave, slow_time_weighting=wt, sign_multiplier=sign)
    out = DS.from_resampling(ds, range_amb=range_amb, cross_range_amb=cross_range_amb,
                             fast_downsample_factor=fast or 1.0, slow_downsample_factor=slow or 1, new_srp=new_srp,
                             safety_factor=1.2, num_threads=1)
    ap = out.aperture
    np.savez_compressed(os.path.join(HERE, f"resample_{name}.npz"), tx=tx, rx=rx, srps=srps, ph=ph, wave=wave, wt=wt,
                        new_srp=new_srp, centre_frequency=fc, sample_frequency=fs, sign_multiplier=sign,
                        fast_factor=fast or 0.0, slow_factor=slow or 0, range_amb=range_amb or 0.0,
                        cross_range_amb=cross_range_amb or 0.0, safety_factor=1.2, moved=moved, n_new=n_new, ffd=ffd,
                        kernel=kern, out_tx=ap.transmitter_positions, out_rx=ap.receiver_positions,
                        out_srps=ap.stab_ref_posns, out_wt=ap.slow_time_weighting, out_wave=ap.waveform_fft,
                        out_ph=out.phase_history())
    print(name, "in", ph.shape, "out", out.phase_history().shape)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    with tempfile.TemporaryDirectory() as work:
        import_reference(args.reference, work)
        import sarsolver.utils as utils
        from sarsolver.numpy import NumpySimpleSarDataset
        ref = {"utils": utils, "NumpySimpleSarDataset": NumpySimpleSarDataset}
        for name, kw in CASES.items():
            make_case(ref, name, **kw)


if __name__ == "__main__":
    main()
