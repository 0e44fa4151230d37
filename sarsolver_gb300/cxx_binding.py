"""Function-level API of sarsolver.cxx_binding, computed on the GPU.

Reference functions and their replacements:
  single_forward_evaluate / multi_forward_evaluate   src/sarsolver/cxx_binding/forward.py:13-96
  single_adjoint_evaluate / multi_adjoint_evaluate   src/sarsolver/cxx_binding/adjoint.py:13-94
  SarCalculationInfo, forward_evaluate, adjoint_evaluate  sarsolver_cxx.py:49-220

The single_/multi_ pairs keep their signatures and return values (complex128, fftshifted phase
history [S, N] / image vector [P]).  ``num_threads`` and ``num_calculation_blocks`` select the
reference's CPU fan-out and pulse blocking; on the GPU they have no effect.  ``forward_evaluate``
and ``adjoint_evaluate`` are libsargpu.so's drop-in entry points with the reference's struct.
"""
from __future__ import annotations

import hashlib
from collections import OrderedDict
from typing import Optional

import numpy as np

from . import _lib
from ._lib import SarCalculationInfo  # noqa: F401  (re-exported, reference layout)
from .geometry import grid_axes
from .plan import SarPlan

_PLAN_CACHE: "OrderedDict[tuple, SarPlan]" = OrderedDict()
_PLAN_CACHE_SIZE = 8


def geometry_fingerprint(scene, measurements) -> str:
    """Digest of everything a plan copies from the scene and the aperture: antenna and SRP
    positions, waveform, slow-time weighting, frequencies, c_eff, sign, and the grid (origin,
    steps, shape) or the scatterer positions.  Two calls share a plan only when these agree, so
    a new or mutated aperture (e.g. a new slow_time_weighting) never reuses stale device tables."""
    h = hashlib.blake2b(digest_size=20)

    def add(a, dtype):
        arr = np.ascontiguousarray(np.asarray(a, dtype=dtype))
        h.update(str(arr.shape).encode())
        h.update(arr.tobytes())

    ap = measurements
    for a in (ap.transmitter_positions, ap.receiver_positions, ap.stab_ref_posns):
        add(a, np.float64)
    add(ap.waveform_fft, np.complex128)
    add(ap.slow_time_weighting, np.complex128)
    add([ap.centre_frequency, ap.sample_bandwidth, ap.c_eff, ap.sign_multiplier, ap.num_freqs], np.float64)
    axes = grid_axes(scene)
    if axes is not None:
        shape, origin, ex, ey, ez = axes
        h.update(b"grid")
        add(list(shape), np.float64)
        for a in (origin, ex, ey, ez):
            add(a, np.float64)
    else:
        h.update(b"points")
        add(scene.positions, np.float64)
    return h.hexdigest()


def _plan_for(scene, measurements, upsample_ratio: float, interp: str) -> SarPlan:
    key = (geometry_fingerprint(scene, measurements), float(upsample_ratio), interp)
    plan = _PLAN_CACHE.get(key)
    if plan is None:
        while len(_PLAN_CACHE) >= _PLAN_CACHE_SIZE:
            _PLAN_CACHE.popitem(last=False)
        plan = SarPlan(scene, measurements, upsample_ratio=upsample_ratio, interp=interp)
        _PLAN_CACHE[key] = plan
    else:
        _PLAN_CACHE.move_to_end(key)
    return plan


def single_forward_evaluate(scene, measurements, scattering_amplitudes, upsample_ratio: float = 128.0,
                            interp: str = "nearest_ref") -> np.ndarray:
    plan = _plan_for(scene, measurements, upsample_ratio, interp)
    y = plan.forward(np.asarray(scattering_amplitudes).reshape(-1))
    return y.to(dtype=__import__("torch").complex128).cpu().numpy()


def multi_forward_evaluate(scene, measurements, scattering_amplitudes, num_threads: Optional[int] = None,
                           upsample_ratio: float = 128.0, verbose: bool = False, num_calculation_blocks: int = 1,
                           interp: str = "nearest_ref") -> np.ndarray:
    return single_forward_evaluate(scene, measurements, scattering_amplitudes, upsample_ratio, interp)


def single_adjoint_evaluate(scene, measurements, adjoint_amplitudes, upsample_ratio: float = 128.0,
                            interp: str = "nearest_ref") -> np.ndarray:
    plan = _plan_for(scene, measurements, upsample_ratio, interp)
    x = plan.adjoint(np.asarray(adjoint_amplitudes).reshape(measurements.num_slow_times, measurements.num_freqs))
    return x.to(dtype=__import__("torch").complex128).cpu().numpy()


def multi_adjoint_evaluate(scene, measurements, adjoint_amplitudes, num_threads: Optional[int] = None,
                           upsample_ratio: float = 128.0, verbose: bool = False, num_calculation_blocks: int = 1,
                           interp: str = "nearest_ref") -> np.ndarray:
    return single_adjoint_evaluate(scene, measurements, adjoint_amplitudes, upsample_ratio, interp)


def forward_evaluate(info) -> None:
    """libsargpu.so's drop-in forward_evaluate(SarCalculationInfo*) (sarsolver_cxx.hpp:113)."""
    import ctypes
    _lib.load().forward_evaluate(ctypes.byref(info))


def adjoint_evaluate(info) -> None:
    """libsargpu.so's drop-in adjoint_evaluate(SarCalculationInfo*) (sarsolver_cxx.hpp:114)."""
    import ctypes
    _lib.load().adjoint_evaluate(ctypes.byref(info))
