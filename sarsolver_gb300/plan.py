"""SarPlan: one scene + aperture uploaded to a GPU, applied to device tensors.

This is the device-resident layer under the drop-in operator classes.  It replaces the
per-call work of src/sarsolver/cxx_binding/forward.py:13-44 and adjoint.py:13-44 (building a
SarCalculationInfo, fftshift handling, one C++ call per process block) with one plan whose
forward / adjoint run asynchronously on the current torch CUDA stream.

Tensors: image x complex64 [P] (grid order (k*ny + j)*nx + i); phase history y complex64
[S, N] with fast time fftshifted, as the reference's Python API returns it (forward.py:44).
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from . import _lib
from .geometry import grid_axes


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _interleave(z) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(z, dtype=np.complex128).reshape(-1)).view(np.float64)


def block_pulses_for(scene, num_slow_times: int, num_calculation_blocks) -> Optional[int]:
    """Pulses per block of a streamed plan for the reference's ``num_calculation_blocks`` (slow-time
    blocks, whose purpose in the reference is bounding memory, cxx_binding/forward.py:66-96): None
    (a resident plan) for one block or an unstructured scene (streamed plans need a regular grid)."""
    blocks = int(num_calculation_blocks or 1)
    if blocks <= 1 or grid_axes(scene) is None:
        return None
    return -(-int(num_slow_times) // blocks)


class SarPlan:
    """Operator plan on one CUDA device.

    Parameters mirror NumpySimpleSarOperator (src/sarsolver/numpy/operator.py:12-13):
    ``upsample_ratio`` (default 128, as the reference) and the added ``interp``
    ("nearest_ref": the reference's bins and conventions; "linear": exact transpose pair) and
    ``path`` ("auto": grid fast path for linear, per-pixel double-float path for nearest_ref;
    "grid" / "points" force one), and ``block_pulses``: a streamed plan whose device memory is
    bounded by two blocks of that many pulses instead of the whole aperture (regular grids;
    sar_plan_create_streamed), the replacement of the reference's ``num_calculation_blocks``.
    """

    def __init__(self, scene, aperture, upsample_ratio: float = 128.0, interp: str = "nearest_ref",
                 device: Optional[torch.device] = None, path: str = "auto", block_pulses: Optional[int] = None):
        if interp not in _lib.INTERP:
            raise ValueError(f"interp must be one of {sorted(_lib.INTERP)}")
        if path not in _lib.PATH:
            raise ValueError(f"path must be one of {sorted(_lib.PATH)}")
        if not torch.cuda.is_available():
            raise RuntimeError("SarPlan needs a CUDA device")
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        lib = _lib.load()
        self.num_slow_times = int(aperture.num_slow_times)
        self.num_freqs = int(aperture.num_freqs)
        self.num_scatterers = int(scene.num_scatterers)
        self.interp = interp
        self.upsample_ratio = float(upsample_ratio)
        keep = {}
        keep["tx"] = _f64(aperture.transmitter_positions).reshape(-1, 3)
        keep["rx"] = _f64(aperture.receiver_positions).reshape(-1, 3)
        keep["srp"] = _f64(aperture.stab_ref_posns).reshape(-1, 3)
        # The kernel consumes the waveform in FFT order (forward.py:39, adjoint.py:38).
        keep["wave"] = _interleave(np.fft.ifftshift(np.asarray(aperture.waveform_fft, dtype=np.complex128)))
        keep["wt"] = _interleave(aperture.slow_time_weighting)
        g = _lib.SarGeometry()
        g.num_fast_times = self.num_freqs
        g.num_slow_times = self.num_slow_times
        g.num_scatterers = self.num_scatterers
        g.transmit_posns = keep["tx"].ctypes.data
        g.receive_posns = keep["rx"].ctypes.data
        g.stab_ref_posns = keep["srp"].ctypes.data
        g.waveform_fft = keep["wave"].ctypes.data
        g.slow_time_weighting = keep["wt"].ctypes.data
        g.centre_frequency = float(aperture.centre_frequency)
        g.sample_frequency = float(aperture.sample_bandwidth)
        g.c_eff = float(aperture.c_eff)
        g.upsample_ratio = self.upsample_ratio
        g.sign_multiplier = float(aperture.sign_multiplier)
        g.interp = _lib.INTERP[interp]
        g.path = _lib.PATH[path]
        axes = grid_axes(scene)
        if axes is not None:
            shape, origin, ex, ey, ez = axes
            for i in range(3):
                g.grid_shape[i] = shape[i]
                g.grid_origin[i] = origin[i]
                g.grid_step_x[i] = ex[i]
                g.grid_step_y[i] = ey[i]
                g.grid_step_z[i] = ez[i]
            self.grid_shape = tuple(shape)
        else:
            keep["pos"] = _f64(scene.positions).reshape(-1, 3)
            g.scat_posns = keep["pos"].ctypes.data
            self.grid_shape = None
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            torch.cuda.current_stream(self.device)   # make sure the context exists
            if block_pulses:
                _lib.check(lib.sar_plan_create_streamed(ctypes.byref(g), self.device.index, int(block_pulses),
                                                        ctypes.byref(handle)), "sar_plan_create_streamed")
            else:
                _lib.check(lib.sar_plan_create(ctypes.byref(g), self.device.index, ctypes.byref(handle)),
                           "sar_plan_create")
        self._handle = handle
        self._lib = lib
        info = _lib.SarPlanInfo()
        _lib.check(lib.sar_plan_get_info(handle, ctypes.byref(info)), "sar_plan_get_info")
        self.working_length = int(info.working_length)
        self.profile_first_bin = int(info.profile_first_bin)
        self.profile_length = int(info.profile_length)
        self.tile_window = int(info.tile_window)
        self.strip_window = int(info.strip_window)
        self.device_bytes = int(info.device_bytes)
        self.is_grid = bool(info.grid)
        self.fft_callbacks = bool(info.fft_callbacks)
        self.gather_lanes_y = bool(info.gather_lanes_y)
        self.fused_upsampling = bool(info.fused_upsampling)
        self.fused_downsampling = bool(info.fused_downsampling)
        self.scatter_lanes_y = bool(info.scatter_lanes_y)
        self.block_pulses = int(info.block_pulses)
        self.scatter_shear = int(info.scatter_shear)
        self.gather_shear = int(info.gather_shear)
        self.scatter_ring_half = int(info.scatter_ring_half)
        # The aperture's own weighting; phase corrections multiply it (autodiff.phase_weights).
        self.base_weights = torch.as_tensor(
            np.asarray(aperture.slow_time_weighting, dtype=np.complex64).reshape(-1)).to(self.device)

    # ------------------------------------------------------------------ helpers
    def _stream(self) -> ctypes.c_void_p:
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _as_input(self, t: torch.Tensor, numel: int, name: str) -> torch.Tensor:
        if not isinstance(t, torch.Tensor):
            t = torch.as_tensor(np.asarray(t))
        if t.numel() != numel:
            raise ValueError(f"{name} has {t.numel()} elements, expected {numel}")
        t = t.to(device=self.device, non_blocking=True)
        if t.dtype != torch.complex64:
            t = t.to(torch.complex64)
        # Kernels read raw memory: materialise PyTorch's lazy conjugate / negative views
        # (autograd hands such views to backward functions).
        return t.resolve_conj().resolve_neg().contiguous()

    def _check_out(self, out: Optional[torch.Tensor], shape, name: str) -> torch.Tensor:
        if out is None:
            return torch.empty(shape, dtype=torch.complex64, device=self.device)
        if (out.dtype != torch.complex64 or out.device != self.device or not out.is_contiguous()
                or out.is_conj() or out.is_neg()):
            raise ValueError(f"{name} must be a contiguous complex64 tensor on {self.device}")
        if out.numel() != int(np.prod(shape)):
            raise ValueError(f"{name} has the wrong size")
        return out

    # ---------------------------------------------------------------- operators
    def forward(self, x: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """y = A x, complex64 [S, N] (fast time fftshifted)."""
        x = self._as_input(x, self.num_scatterers, "x")
        y = self._check_out(out, (self.num_slow_times, self.num_freqs), "out")
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_forward(self._handle, ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(y.data_ptr()), self._stream()), "sar_forward")
        return y

    def adjoint(self, y: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """x = A^H y, complex64 [P]."""
        y = self._as_input(y, self.num_slow_times * self.num_freqs, "y")
        x = self._check_out(out, (self.num_scatterers,), "out")
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_adjoint(self._handle, ctypes.c_void_p(y.data_ptr()),
                                             ctypes.c_void_p(x.data_ptr()), self._stream()), "sar_adjoint")
        return x

    def adjoint_host(self, y_host: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """x = A^H y with y in host memory.  When the plan uses the fused upsampling and y is a
        pinned (page-locked, mapped) contiguous complex64 tensor, the upsampling kernel reads y over
        the host link itself, so the transfer overlaps the transform instead of preceding it; the
        call returns after the device is done with y (the stream is synchronised).  Otherwise y is
        copied to the device first."""
        n = self.num_slow_times * self.num_freqs
        if (self.fused_upsampling and isinstance(y_host, torch.Tensor) and y_host.device.type == "cpu"
                and y_host.dtype == torch.complex64 and y_host.numel() == n and y_host.is_contiguous()
                and not y_host.is_conj() and not y_host.is_neg() and y_host.is_pinned()):
            dev_ptr = ctypes.c_void_p()
            if self._lib.sar_host_device_pointer(ctypes.c_void_p(y_host.data_ptr()), ctypes.byref(dev_ptr)) == 0:
                x = self._check_out(out, (self.num_scatterers,), "out")
                with torch.cuda.device(self.device):
                    _lib.check(self._lib.sar_adjoint(self._handle, dev_ptr, ctypes.c_void_p(x.data_ptr()),
                                                     self._stream()), "sar_adjoint")
                    torch.cuda.current_stream(self.device).synchronize()
                return x
        return self.adjoint(y_host, out)

    def adjoint_streamed(self, y_host: torch.Tensor, block: int = 512, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """x = A^H y with y in host memory (pin it for overlap), streamed through the device in
        blocks of ``block`` pulses: block b + 1 is copied on a side stream while block b is
        backprojected on the current stream into the resident image (``sar_adjoint_pulse_block``
        with accumulation).  Device memory for y is two blocks."""
        if not self.is_grid:
            raise ValueError("streamed backprojection needs a regular-grid scene")
        S, N = self.num_slow_times, self.num_freqs
        if self.block_pulses:
            block = min(int(block), self.block_pulses)
        yh = torch.as_tensor(y_host).reshape(S, N)
        if yh.dtype != torch.complex64:
            yh = yh.to(torch.complex64)
        yh = yh.resolve_conj().resolve_neg().contiguous()
        x = self._check_out(out, (self.num_scatterers,), "out")
        block = max(1, min(int(block), S))
        compute = torch.cuda.current_stream(self.device)
        side = torch.cuda.Stream(self.device)
        bufs = [torch.empty((block, N), dtype=torch.complex64, device=self.device) for _ in range(2)]
        copied = [torch.cuda.Event() for _ in range(2)]
        consumed = [torch.cuda.Event() for _ in range(2)]
        # The buffers come from the compute stream's pool: memory freed there may still be read by
        # kernels already queued on it (e.g. the previous call's gathers), so the side stream's
        # copies start only after everything queued on the compute stream so far.
        side.wait_stream(compute)
        nblk = (S + block - 1) // block
        with torch.cuda.device(self.device):
            for k in range(nblk):
                b, first = k % 2, k * block
                count = min(block, S - first)
                with torch.cuda.stream(side):
                    if k >= 2:
                        side.wait_event(consumed[b])
                    bufs[b][:count].copy_(yh[first:first + count], non_blocking=True)
                    copied[b].record(side)
                bufs[b].record_stream(side)
                compute.wait_event(copied[b])
                _lib.check(self._lib.sar_adjoint_pulse_block(self._handle, ctypes.c_void_p(bufs[b].data_ptr()), first,
                                                             count, ctypes.c_void_p(x.data_ptr()), int(k > 0),
                                                             ctypes.c_void_p(compute.cuda_stream)),
                           "sar_adjoint_pulse_block")
                consumed[b].record(compute)
        return x

    def profiles(self, y: torch.Tensor) -> torch.Tensor:
        """Upsampled range profiles over the stored span, complex64 [S, profile_length]."""
        y = self._as_input(y, self.num_slow_times * self.num_freqs, "y")
        prof = torch.empty((self.num_slow_times, self.profile_length), dtype=torch.complex64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_profiles(self._handle, ctypes.c_void_p(y.data_ptr()),
                                              ctypes.c_void_p(prof.data_ptr()), self._stream()), "sar_profiles")
        return prof

    def set_slow_time_weighting(self, w) -> None:
        """Replace the slow-time weighting (numpy on the host, or a CUDA tensor, stream-ordered)."""
        if isinstance(w, torch.Tensor) and w.is_cuda:
            w = self._as_input(w, self.num_slow_times, "w")
            with torch.cuda.device(self.device):
                _lib.check(self._lib.sar_set_slow_time_weighting_device(
                    self._handle, ctypes.c_void_p(w.data_ptr()), self._stream()), "sar_set_slow_time_weighting")
            self._keep_w = w
            return
        arr = _interleave(np.asarray(w))
        if arr.size != 2 * self.num_slow_times:
            raise ValueError("weighting has the wrong length")
        _lib.check(self._lib.sar_set_slow_time_weighting(self._handle, arr.ctypes.data), "sar_set_slow_time_weighting")

    def enable_stage_timing(self, enable: bool = True) -> None:
        """Record CUDA events around each call's stages (see sar_enable_stage_timing)."""
        _lib.check(self._lib.sar_enable_stage_timing(self._handle, int(bool(enable))), "sar_enable_stage_timing")

    def stage_times(self):
        """(ms per stage [pre-FFT side, main kernel, post-FFT side] summed over recorded calls, calls)."""
        ms = (ctypes.c_float * 3)()
        calls = ctypes.c_int(0)
        _lib.check(self._lib.sar_stage_times(self._handle, ms, ctypes.byref(calls)), "sar_stage_times")
        return [float(v) for v in ms], int(calls.value)

    def set_wait_budget(self, cycles: int = 0, hold_first_stage: bool = False) -> None:
        """Clock-cycle budget of the gather's bounded in-kernel waits (0: the default, ~2 s).
        ``hold_first_stage`` is a test aid that makes the first wait run out (see
        sar_plan_set_wait_budget); the expiry shows up as SAR_FLAG_WAIT_TIMEOUT in device_flags()."""
        _lib.check(self._lib.sar_plan_set_wait_budget(self._handle, int(cycles), int(bool(hold_first_stage))),
                   "sar_plan_set_wait_budget")

    def device_flags(self) -> int:
        """Synchronise and return (then clear) the device check flags; 0 means no check fired."""
        f = ctypes.c_uint(0)
        _lib.check(self._lib.sar_device_flags(self._handle, ctypes.byref(f)), "sar_device_flags")
        return int(f.value)

    def close(self) -> None:
        if getattr(self, "_handle", None):
            torch.cuda.synchronize(self.device)
            self._lib.sar_plan_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
