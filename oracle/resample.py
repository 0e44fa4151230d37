"""CPU restatement of the reference's dataset resampling -- TEST INFRASTRUCTURE ONLY (the
checker for sarsolver_gb300.resample; the product never imports it).

Follows, step for step:
  * move_srps            src/sarsolver/utils/geodesy.py:33-73
  * get_downsample_kernel src/sarsolver/utils/signal.py:7-27
  * fast_freq_downsample src/sarsolver/utils/signal.py:45-77
  * the resampling loop of NumpySimpleSarDataset.from_resampling,
    src/sarsolver/numpy/measurement.py:342-458 (explicit downsample factors; bad pulses =
    non-finite transmitter, receiver or SRP rows, src/sarsolver/base/measurement.py:326-339)
Pinned against tests/golden/resample_*.npz, produced by the reference itself.
"""
from __future__ import annotations

import numpy as np
from scipy.signal.windows import hann, tukey

C = 299792458.0


def move_srps(ph, old_srps, new_srp, tx, rx, fc, fs, sign=1.0, c_eff=C):
    n = ph.shape[1]
    new_srp = np.asarray(new_srp)[None, :]
    new_range = np.linalg.norm(tx - new_srp, axis=-1) + np.linalg.norm(rx - new_srp, axis=-1)
    old_range = np.linalg.norm(tx - old_srps, axis=-1) + np.linalg.norm(rx - old_srps, axis=-1)
    dr = (new_range - old_range)[:, None]
    kb = (2.0 * np.pi / c_eff) * np.fft.fftshift(np.fft.fftfreq(n, 1.0 / fs))[None, :]
    return ph * np.exp(1j * kb * dr) * np.exp((-2.0j * np.pi * sign * fc / c_eff) * dr)


def downsample_kernel(ratio):
    num = int(np.round(5 * ratio))
    filt = np.zeros(num, dtype="complex64")
    filt[:2] = 1.0
    filt[-1:] = 1.0
    return np.fft.fftshift(np.fft.ifft(filt)) * hann(num)


def fast_freq_downsample(ph, n_new, safety=1.2):
    safety = max(safety, 1.0)
    window = np.fft.fftshift(tukey(n_new, alpha=safety - 1.0))[None, :]
    new = np.zeros((ph.shape[0], n_new), dtype=ph.dtype)
    old = np.fft.ifft(np.fft.ifftshift(ph, axes=[1]), axis=1)
    lo, hi = n_new // 2, n_new - n_new // 2
    new[:, :lo] = old[:, :lo]
    new[:, -hi:] = old[:, -hi:]
    return np.fft.fftshift(np.fft.fft(window * new, axis=1), axes=[1])


def edge_k_vecs(tx, rx, origin, fc, fs, c_eff=C):
    """base/measurement.py:250-321: bistatic unit directions times the band-edge wavenumbers."""
    o = np.asarray(origin)[None, :]
    tv = (o - tx) / np.linalg.norm(o - tx, axis=-1, keepdims=True)
    rv = (rx - o) / np.linalg.norm(rx - o, axis=-1, keepdims=True)
    u = rv - tv
    k = 2.0 * np.pi / c_eff
    return np.concatenate([u * k * (fc - 0.5 * fs), u * k * (fc + 0.5 * fs)], axis=0)


def obb_spans(xs):
    """utils/k_space.py:9-80: (range span, cross-range span) of the principal-axes box."""
    xs = xs[np.isfinite(xs).all(axis=1)]
    z = xs - xs.mean(axis=0, keepdims=True)
    _, b = np.linalg.eigh(z.T @ z)
    if np.linalg.det(b) < 0.0:
        b = -b
    t = (b.T @ xs.T).T
    mn, mx = t.min(axis=0), t.max(axis=0)
    spans = np.abs(mx - mn)
    ri = int(np.argmax(np.abs(0.5 * (mn + mx))))
    ci = int(np.argmax(spans)) if spans[ri] < spans.max() else int(np.argsort(spans)[1])
    return spans[ri], spans[ci]


def factors_from_ambiguities(tx, rx, new_srp, fc, fs, S, N, range_amb, cross_range_amb, safety=1.2):
    """numpy/measurement.py:401-410: downsampling factors from wanted ambiguous extents."""
    r_span, cr_span = obb_spans(edge_k_vecs(tx, rx, new_srp, fc, fs))
    slow = max(int(2.0 * np.pi * S / cr_span / (2.0 * safety * cross_range_amb)), 1)
    fast = 2.0 * np.pi * N / r_span / (2.0 * safety * range_amb)
    return fast, slow


def bad_pulses(tx, rx, srps):
    bad = ~(np.isfinite(tx).all(axis=1) & np.isfinite(rx).all(axis=1) & np.isfinite(srps).all(axis=1))
    return np.nonzero(bad)[0]


def resample(tx, rx, srps, ph, wave, wt, fc, fs, sign, fast_factor, slow_factor, new_srp, safety=1.2, c_eff=C):
    """Returns (tx, rx, srps, weighting, waveform, phase_history) of the resampled dataset."""
    S, N = ph.shape
    n_new = min(int(1.0 + N / fast_factor), N)
    kern = downsample_kernel(slow_factor)[:, None]
    L = kern.shape[0]
    T = ((S - L) // slow_factor) - 1
    new_wave = fast_freq_downsample(np.asarray(wave)[None, :], n_new, safety)[0]
    bad = set(bad_pulses(tx, rx, srps).tolist())
    out = ([], [], [], [], [])
    for t in range(T):
        s0 = slow_factor * t
        win = range(s0, s0 + L)
        if bad & set(win):
            continue
        sl = slice(s0, s0 + L)
        shifted = move_srps(ph[sl], srps[sl], new_srp, tx[sl], rx[sl], fc, fs, sign, c_eff)
        ds = fast_freq_downsample(shifted, n_new, safety)
        out[0].append(tx[s0 + L // 2])
        out[1].append(rx[s0 + L // 2])
        out[2].append(np.asarray(new_srp))
        out[3].append(np.sum(kern[:, 0] * wt[sl]))
        out[4].append(np.sum(ds * kern, axis=0))
    return (np.stack(out[0]), np.stack(out[1]), np.stack(out[2]), np.array(out[3]), new_wave, np.stack(out[4]))
