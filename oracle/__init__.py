"""CPU oracle for the SAR operator pair -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may
import this package; the product (``sarsolver_gb300``) never does.

Two checkers live here:

* ``libsaroracle.so`` -- the FP64 C restatement in ``sar_oracle.c`` of the reference kernel
  (src/sarsolver/cxx_binding/sarsolver_cxx.cpp:271-353) with the two interpolation modes
  ``nearest_ref`` (the reference's own conventions) and ``linear`` (exact transpose pair).
* ``_ref/libsarsolver_ref.so`` -- the reference's own ``sarsolver_cxx.cpp`` compiled unmodified
  against the FFTW-API shim in ``fftw_shim/`` (built only where the reference source exists).

The Python functions here apply the reference's fftshift conventions
(src/sarsolver/cxx_binding/forward.py:39,44 and adjoint.py:36): phase histories in and out
are fftshifted along fast time (centre frequency in the middle), the waveform is given in
fftshifted order and ifftshifted before the kernel sees it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libsaroracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsarsolver_ref.so")

NEAREST_REF = 0
LINEAR = 1
MODES = {"nearest_ref": NEAREST_REF, "linear": LINEAR}

C = 299792458.0


def build(quiet: bool = True) -> None:
    """Compile the oracle (and, where its source exists, the reference kernel) with make."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


class _OracleInfo(ctypes.Structure):
    """Mirror of ``oracle_sar_info`` (sar_oracle.h)."""

    _fields_ = [
        ("num_fast_times", ctypes.c_size_t), ("num_slow_times", ctypes.c_size_t),
        ("num_scatterers", ctypes.c_size_t),
        ("transmit_posns", ctypes.c_void_p), ("receive_posns", ctypes.c_void_p),
        ("stab_ref_posns", ctypes.c_void_p), ("scat_posns", ctypes.c_void_p),
        ("waveform_fft", ctypes.c_void_p), ("slow_time_weighting", ctypes.c_void_p),
        ("centre_frequency", ctypes.c_double), ("sample_frequency", ctypes.c_double),
        ("c_eff", ctypes.c_double), ("upsample_ratio", ctypes.c_double),
        ("sign_multiplier", ctypes.c_double),
        ("mode", ctypes.c_int), ("num_threads", ctypes.c_int),
    ]


class _RefInfo(ctypes.Structure):
    """Mirror of the reference's ``SarCalculationInfo`` (sarsolver_cxx.hpp:28-33)."""

    _fields_ = [
        ("num_fast_times", ctypes.c_size_t), ("num_slow_times", ctypes.c_size_t),
        ("num_scatterers", ctypes.c_size_t),
        ("transmit_posns", ctypes.c_void_p), ("receive_posns", ctypes.c_void_p),
        ("stab_ref_posns", ctypes.c_void_p), ("scat_posns", ctypes.c_void_p),
        ("phase_history", ctypes.c_void_p), ("scattering_amplitudes", ctypes.c_void_p),
        ("waveform_fft", ctypes.c_void_p), ("slow_time_weighting", ctypes.c_void_p),
        ("centre_frequency", ctypes.c_double), ("sample_frequency", ctypes.c_double),
        ("c_eff", ctypes.c_double), ("upsample_ratio", ctypes.c_double),
        ("sign_multiplier", ctypes.c_double),
    ]


_lib_cache: dict = {}


def _load(path: str, what: str):
    if path not in _lib_cache:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{what} not built: {path} (run oracle.build())")
        lib = ctypes.CDLL(path)
        if path == ORACLE_SO:
            for name in ("oracle_forward", "oracle_adjoint", "oracle_upsample", "oracle_ranges"):
                fn = getattr(lib, name)
                fn.restype = ctypes.c_int
                fn.argtypes = [ctypes.POINTER(_OracleInfo), ctypes.c_void_p] + (
                    [ctypes.c_void_p] if name != "oracle_ranges" else [])
            lib.oracle_working_length.restype = ctypes.c_size_t
            lib.oracle_working_length.argtypes = [ctypes.POINTER(_OracleInfo)]
        else:
            for name in ("forward_evaluate", "adjoint_evaluate"):
                fn = getattr(lib, name)
                fn.restype = None
                fn.argtypes = [ctypes.POINTER(_RefInfo)]
        _lib_cache[path] = lib
    return _lib_cache[path]


def reference_available() -> bool:
    return os.path.exists(REF_SO)


@dataclass
class Problem:
    """Geometry and signal parameters of one operator application (FP64 host arrays).

    ``waveform_fft`` is in fftshifted order, as ``NumpySimpleSarAperture.waveform_fft``
    (src/sarsolver/numpy/measurement.py:53-58); ``None`` means all ones.
    """

    tx: np.ndarray
    rx: np.ndarray
    srp: np.ndarray
    positions: np.ndarray
    centre_frequency: float
    sample_frequency: float
    num_freqs: int
    waveform_fft: Optional[np.ndarray] = None
    slow_time_weighting: Optional[np.ndarray] = None
    c_eff: float = C
    sign_multiplier: float = 1.0
    upsample_ratio: float = 128.0

    @property
    def num_slow_times(self) -> int:
        return int(self.tx.shape[0])

    @property
    def num_scatterers(self) -> int:
        return int(self.positions.shape[0])

    def arrays(self):
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        wf = self.waveform_fft
        if wf is None:
            wf = np.ones(self.num_freqs, dtype=np.complex128)
        wt = self.slow_time_weighting
        if wt is None:
            wt = np.ones(self.num_slow_times, dtype=np.complex128)
        wf_fft_order = np.fft.ifftshift(np.asarray(wf, dtype=np.complex128))   # forward.py:39
        return dict(
            tx=f64(self.tx).reshape(-1, 3), rx=f64(self.rx).reshape(-1, 3),
            srp=f64(self.srp).reshape(-1, 3), pos=f64(self.positions).reshape(-1, 3),
            wf=np.ascontiguousarray(wf_fft_order.view(np.float64)),
            wt=np.ascontiguousarray(np.asarray(wt, dtype=np.complex128).view(np.float64)),
        )


def _info(p: Problem, arr: dict, mode: int, threads: int) -> _OracleInfo:
    ptr = lambda a: a.ctypes.data
    return _OracleInfo(
        p.num_freqs, p.num_slow_times, p.num_scatterers,
        ptr(arr["tx"]), ptr(arr["rx"]), ptr(arr["srp"]), ptr(arr["pos"]),
        ptr(arr["wf"]), ptr(arr["wt"]),
        float(p.centre_frequency), float(p.sample_frequency), float(p.c_eff),
        float(p.upsample_ratio), float(p.sign_multiplier), int(mode), int(threads))


def _mode(mode) -> int:
    return MODES[mode] if isinstance(mode, str) else int(mode)


def default_threads() -> int:
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:  # pragma: no cover
        return max(1, os.cpu_count() or 1)


def forward(p: Problem, x: np.ndarray, mode="nearest_ref", threads: int = 1) -> np.ndarray:
    """y = A x, shape [S, N], fftshifted along fast time (forward.py:44)."""
    lib = _load(ORACLE_SO, "oracle")
    arr = p.arrays()
    xi = np.ascontiguousarray(np.asarray(x, dtype=np.complex128).reshape(-1))
    if xi.size != p.num_scatterers:
        raise ValueError("x has the wrong length")
    y = np.zeros((p.num_slow_times, p.num_freqs), dtype=np.complex128)
    info = _info(p, arr, _mode(mode), threads)
    if lib.oracle_forward(ctypes.byref(info), xi.ctypes.data, y.ctypes.data) != 0:
        raise RuntimeError("oracle_forward failed")
    return np.fft.fftshift(y, axes=1)


def adjoint(p: Problem, y: np.ndarray, mode="nearest_ref", threads: int = 1) -> np.ndarray:
    """x = A^H y for y [S, N] fftshifted along fast time (adjoint.py:36)."""
    lib = _load(ORACLE_SO, "oracle")
    arr = p.arrays()
    yy = np.asarray(y, dtype=np.complex128).reshape(p.num_slow_times, p.num_freqs)
    yi = np.ascontiguousarray(np.fft.ifftshift(yy, axes=1))
    x = np.zeros(p.num_scatterers, dtype=np.complex128)
    info = _info(p, arr, _mode(mode), threads)
    if lib.oracle_adjoint(ctypes.byref(info), yi.ctypes.data, x.ctypes.data) != 0:
        raise RuntimeError("oracle_adjoint failed")
    return x


def upsample(p: Problem, y: np.ndarray, threads: int = 1) -> np.ndarray:
    """Upsampled range profiles [S, M] (no slow-time weight) for y [S, N] fftshifted."""
    lib = _load(ORACLE_SO, "oracle")
    arr = p.arrays()
    yi = np.ascontiguousarray(np.fft.ifftshift(
        np.asarray(y, dtype=np.complex128).reshape(p.num_slow_times, p.num_freqs), axes=1))
    info = _info(p, arr, NEAREST_REF, threads)
    m = int(lib.oracle_working_length(ctypes.byref(info)))
    prof = np.zeros((p.num_slow_times, m), dtype=np.complex128)
    if lib.oracle_upsample(ctypes.byref(info), yi.ctypes.data, prof.ctypes.data) != 0:
        raise RuntimeError("oracle_upsample failed")
    return prof


def ranges(p: Problem) -> np.ndarray:
    """Differential bistatic ranges [S, P] in metres."""
    lib = _load(ORACLE_SO, "oracle")
    arr = p.arrays()
    dr = np.zeros((p.num_slow_times, p.num_scatterers), dtype=np.float64)
    info = _info(p, arr, NEAREST_REF, 1)
    if lib.oracle_ranges(ctypes.byref(info), dr.ctypes.data) != 0:
        raise RuntimeError("oracle_ranges failed")
    return dr


def _ref_call(p: Problem, name: str, ph: np.ndarray, amps: np.ndarray):
    lib = _load(REF_SO, "reference kernel (oracle/_ref)")
    arr = p.arrays()
    ph2 = np.ascontiguousarray(ph.astype(np.complex128).view(np.float64))
    am2 = np.ascontiguousarray(amps.astype(np.complex128).view(np.float64))
    ptr = lambda a: a.ctypes.data
    info = _RefInfo(p.num_freqs, p.num_slow_times, p.num_scatterers,
                    ptr(arr["tx"]), ptr(arr["rx"]), ptr(arr["srp"]), ptr(arr["pos"]),
                    ptr(ph2), ptr(am2), ptr(arr["wf"]), ptr(arr["wt"]),
                    float(p.centre_frequency), float(p.sample_frequency), float(p.c_eff),
                    float(p.upsample_ratio), float(p.sign_multiplier))
    getattr(lib, name)(ctypes.byref(info))
    return ph2.view(np.complex128).reshape(ph.shape), am2.view(np.complex128)


def reference_forward(p: Problem, x: np.ndarray) -> np.ndarray:
    """The reference kernel's forward_evaluate, with forward.py's shifts applied."""
    ph = np.zeros((p.num_slow_times, p.num_freqs), dtype=np.complex128)
    out, _ = _ref_call(p, "forward_evaluate", ph, np.asarray(x).reshape(-1))
    return np.fft.fftshift(out, axes=1)


def reference_adjoint(p: Problem, y: np.ndarray) -> np.ndarray:
    """The reference kernel's adjoint_evaluate, with adjoint.py's shifts applied."""
    yy = np.fft.ifftshift(np.asarray(y).reshape(p.num_slow_times, p.num_freqs), axes=1)
    _, amps = _ref_call(p, "adjoint_evaluate", yy, np.zeros(p.num_scatterers, np.complex128))
    return amps.copy()
