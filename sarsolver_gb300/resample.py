"""Dataset resampling on the GPU (the step before the operator for real data).

Drop-in counterparts of the reference's
  * ``utils.move_srps`` (src/sarsolver/utils/geodesy.py:33-73)          -> ``move_srps``
  * ``utils.fast_freq_downsample`` (src/sarsolver/utils/signal.py:45-77) -> ``fast_freq_downsample``
  * ``utils.get_downsample_kernel`` (src/sarsolver/utils/signal.py:7-27) -> ``get_downsample_kernel``
  * ``NumpySimpleSarDataset.from_resampling`` (src/sarsolver/numpy/measurement.py:342-458)
    -> ``resample_dataset`` (explicit downsample factors)
with the per-pulse work on the device (``sar_move_srps``, ``sar_fast_freq_downsample``,
``sar_resample_phase_history``).  Small per-pulse geometry (range changes, window, filter taps,
which windows survive non-finite positions) is set up on the host in FP64, as the reference does.
Phase histories are complex64 on the device; numpy inputs come back as numpy complex128.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch
from scipy.signal.windows import hann, tukey

from . import _lib
from .geometry import C, NumpySimpleSarAperture, NumpySimpleSarDataset, kspace_box


def _device_rows(ph, device) -> torch.Tensor:
    t = ph if isinstance(ph, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(ph))
    if t.dim() != 2:
        raise ValueError("phase history must be [num_slow_times, num_freqs]")
    t = t.to(device=device, dtype=torch.complex64)
    return t.resolve_conj().resolve_neg().contiguous()


def _stream(device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _device(device) -> torch.device:
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    d = torch.device(device)
    return torch.device("cuda", torch.cuda.current_device()) if d.index is None else d


def range_changes(old_srps, new_srp, trans_posns, rec_posns) -> np.ndarray:
    """Change of each pulse's bistatic range from its old SRP to ``new_srp`` (FP64, metres)."""
    tx, rx = np.asarray(trans_posns, np.float64), np.asarray(rec_posns, np.float64)
    old = np.asarray(old_srps, np.float64)
    new = np.broadcast_to(np.asarray(new_srp, np.float64), old.shape)
    dist = lambda a, b: np.sqrt(((a - b) ** 2).sum(axis=-1))
    return np.ascontiguousarray((dist(tx, new) + dist(rx, new)) - (dist(tx, old) + dist(rx, old)))


def move_srps(phase_history, old_srps, new_srp, trans_posns, rec_posns, centre_freq: float, sample_bandwidth: float,
              sign_factor: float = 1.0, c_eff: float = C, device=None):
    """Rephase a phase history [S, N] to a new stabilisation reference point (see module doc)."""
    dev = _device(device)
    x = _device_rows(phase_history, dev)
    S, N = x.shape
    dr = range_changes(old_srps, new_srp, trans_posns, rec_posns)
    out = torch.empty_like(x)
    lib = _lib.load()
    with torch.cuda.device(dev):
        _lib.check(lib.sar_move_srps(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), S, N,
                                     dr.ctypes.data_as(ctypes.c_void_p), float(centre_freq), float(sample_bandwidth),
                                     float(sign_factor), float(c_eff), _stream(dev)), "sar_move_srps")
    return out if isinstance(phase_history, torch.Tensor) else out.cpu().numpy().astype(np.complex128)


def downsample_window(new_num_freqs: int, safety_factor: float) -> np.ndarray:
    """The fftshifted Tukey window (taper fraction safety_factor - 1) applied to the kept modes."""
    return np.ascontiguousarray(np.fft.fftshift(tukey(new_num_freqs, alpha=max(safety_factor, 1.0) - 1.0)), np.float64)


def fast_freq_downsample(phase_history, new_num_freqs: int, safety_factor: float = 1.2, device=None):
    """Downsample in fast frequency (clip in fast time) to ``new_num_freqs`` samples."""
    dev = _device(device)
    x = _device_rows(phase_history, dev)
    S, N = x.shape
    n = int(new_num_freqs)
    win = downsample_window(n, safety_factor)
    out = torch.empty((S, n), dtype=torch.complex64, device=dev)
    lib = _lib.load()
    with torch.cuda.device(dev):
        _lib.check(lib.sar_fast_freq_downsample(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), S, N, n,
                                                win.ctypes.data_as(ctypes.c_void_p), _stream(dev)),
                   "sar_fast_freq_downsample")
    return out if isinstance(phase_history, torch.Tensor) else out.cpu().numpy().astype(np.complex128)


def get_downsample_kernel(downsample_ratio: float) -> np.ndarray:
    """Slow-time downsampling taps: the inverse DFT of a filter passing the three lowest modes of
    a round(5 * ratio)-point window, centred, times a Hann window (complex)."""
    m = int(np.round(5 * downsample_ratio))
    passband = np.zeros(m, dtype=np.complex64)
    passband[[0, 1, m - 1]] = 1.0
    return np.fft.fftshift(np.fft.ifft(passband)) * hann(m)


def bad_slow_times(aperture) -> np.ndarray:
    """Pulses with a non-finite transmitter, receiver or SRP position (base/measurement.py:326-339)."""
    ok = (np.isfinite(aperture.transmitter_positions).all(axis=1) & np.isfinite(aperture.receiver_positions).all(axis=1)
          & np.isfinite(aperture.stab_ref_posns).all(axis=1))
    return np.nonzero(~ok)[0]


def edge_k_vecs(aperture, origin) -> np.ndarray:
    """k-space support of ``aperture`` at ``origin`` ([2S, 3]; base/measurement.py:250-321)."""
    if hasattr(aperture, "edge_k_vecs"):
        return aperture.edge_k_vecs(np.asarray(origin, np.float64))
    return NumpySimpleSarAperture(aperture.transmitter_positions, aperture.receiver_positions,
                                  aperture.stab_ref_posns, aperture.centre_frequency, aperture.sample_bandwidth,
                                  num_freqs=aperture.num_freqs, c_eff=aperture.c_eff).edge_k_vecs(origin)


def kspace_spans(points: np.ndarray):
    """(range span, cross-range span) of the principal-axes box around ``points``."""
    _, spans, r, cr, _ = kspace_box(points)
    return float(spans[r]), float(spans[cr])


def resample_dataset(dataset, fast_downsample_factor: float = 1.0, slow_downsample_factor: int = 1,
                     new_srp: Optional[np.ndarray] = None, safety_factor: float = 1.2, device=None,
                     keep_on_device: bool = False, range_amb: Optional[float] = None,
                     cross_range_amb: Optional[float] = None) -> NumpySimpleSarDataset:
    """Resample a dataset to a new SRP (NumpySimpleSarDataset.from_resampling).

    The downsampling factors are given, or chosen from the wanted ambiguous range / cross range
    (metres) and the k-space extent of the aperture at the new SRP, with ``safety_factor`` margin.
    Output pulse t combines old pulses [D t, D t + L) (D = slow factor, L = round(5 D) taps),
    placed at old pulse D t + L // 2; windows touching a pulse with non-finite positions are
    dropped.  ``keep_on_device`` leaves the phase history as a complex64 CUDA tensor.
    """
    dev = _device(device)
    ap = dataset.aperture
    S, N = int(ap.num_slow_times), int(ap.num_freqs)
    new_srp = np.asarray(ap.stab_ref_posns[0] if new_srp is None else new_srp, np.float64)
    if range_amb is not None or cross_range_amb is not None:
        r_span, cr_span = kspace_spans(edge_k_vecs(ap, new_srp))
        if cross_range_amb is not None:
            slow_downsample_factor = int(2.0 * np.pi * S / cr_span / (2.0 * safety_factor * cross_range_amb))
        if range_amb is not None:
            fast_downsample_factor = 2.0 * np.pi * N / r_span / (2.0 * safety_factor * range_amb)
    D = max(int(slow_downsample_factor), 1)
    n = min(int(1.0 + N / float(fast_downsample_factor)), N)
    taps = get_downsample_kernel(D)
    L = taps.shape[0]
    T = (S - L) // D - 1
    # windows [D t, D t + L) free of non-finite pulses, by a prefix count of bad pulses
    badflag = np.zeros(S + 1, dtype=np.int64)
    badflag[1:] = np.cumsum(np.isin(np.arange(S), bad_slow_times(ap)))
    cand = D * np.arange(max(T, 0), dtype=np.int64)
    starts = cand[(badflag[cand + L] - badflag[cand]) == 0]
    row0 = np.ascontiguousarray(starts.astype(np.int32))
    centres = row0.astype(np.int64) + L // 2
    dr = range_changes(ap.stab_ref_posns, new_srp, ap.transmitter_positions, ap.receiver_positions)
    win = downsample_window(n, safety_factor)
    ktab = np.ascontiguousarray(np.stack([taps.real, taps.imag], axis=-1).astype(np.float64))
    if hasattr(dataset, "phase_history_device"):   # e.g. a CPHD file: raw samples decoded on the device
        x = dataset.phase_history_device(slice(None), device=dev)
    else:
        x = _device_rows(dataset.phase_history(), dev)
    out = torch.empty((len(starts), n), dtype=torch.complex64, device=dev)
    lib = _lib.load()
    with torch.cuda.device(dev):
        _lib.check(lib.sar_resample_phase_history(
            ctypes.c_void_p(x.data_ptr()), S, N, dr.ctypes.data_as(ctypes.c_void_p), float(ap.centre_frequency),
            float(ap.sample_bandwidth), float(ap.sign_multiplier), float(ap.c_eff), n,
            win.ctypes.data_as(ctypes.c_void_p), ktab.ctypes.data_as(ctypes.c_void_p), L,
            row0.ctypes.data_as(ctypes.c_void_p), len(starts), ctypes.c_void_p(out.data_ptr()), _stream(dev)),
            "sar_resample_phase_history")
    wave = fast_freq_downsample(np.asarray(ap.waveform_fft)[None, :], n, safety_factor, device=dev)[0]
    wt = np.asarray(ap.slow_time_weighting, dtype=np.complex128)
    # sum_k taps[k] wt[s0 + k] for every window start s0 (a correlation, evaluated at the starts)
    new_wt = np.correlate(wt, np.conj(taps), mode="valid")[starts] if len(starts) else np.zeros(0, np.complex128)
    tx = np.asarray(ap.transmitter_positions)[centres]
    rx = np.asarray(ap.receiver_positions)[centres]
    srps = np.repeat(new_srp[None, :], len(starts), axis=0)
    new_ap = NumpySimpleSarAperture(tx, rx, srps, ap.centre_frequency, ap.sample_bandwidth, waveform_fft=wave,
                                    slow_time_weighting=new_wt, sign_multiplier=ap.sign_multiplier, c_eff=ap.c_eff)
    ph = out if keep_on_device else out.cpu().numpy().astype(np.complex128)
    return NumpySimpleSarDataset(new_ap, ph)
