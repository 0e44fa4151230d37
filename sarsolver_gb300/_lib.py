"""ctypes binding of libsargpu.so (C ABI declared in include/sargpu.h).

The library is built in-tree by ``sarsolver_gb300.build``; there is no fallback: if it is
missing, loading raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_size_t, c_uint, c_void_p, c_long

from .build import GPU_LIB, HOST_LIB

SAR_OK = 0
SAR_ERR_INVALID_ARGUMENT = 1
SAR_ERR_CUDA = 2
SAR_ERR_CUFFT = 3
SAR_ERR_OUT_OF_MEMORY = 4
SAR_ERR_NOT_SUPPORTED = 5

INTERP = {"nearest_ref": 0, "linear": 1}
PATH = {"auto": 0, "grid": 1, "points": 2}

#: Every function include/sargpu.h declares.
EXPORTED = (
    "forward_evaluate", "adjoint_evaluate",
    "sar_plan_create", "sar_plan_destroy", "sar_plan_get_info",
    "sar_forward", "sar_adjoint", "sar_profiles",
    "sar_set_slow_time_weighting", "sar_set_slow_time_weighting_device",
    "sar_device_flags", "sar_last_error", "sar_status_string",
    "sar_enable_stage_timing", "sar_stage_times",
    "sar_adjoint_from_profiles_noalloc", "sar_phase_gradient", "sar_sharpness", "sar_cgls", "sar_cgls_ex", "sar_adjoint_pulse_block",
    "sar_move_srps", "sar_fast_freq_downsample", "sar_resample_phase_history", "sar_cphd_decode", "sar_pdhg", "sar_host_device_pointer",
    "sar_unet_create", "sar_unet_destroy", "sar_unet_info", "sar_unet_set_params", "sar_unet_get_params",
    "sar_unet_get_grads", "sar_unet_zero_grad", "sar_unet_forward", "sar_unet_backward", "sar_unet_adam_step",
    "sar_unet_flags", "sar_conv2d_forward_bf16", "sar_conv2d_wgrad_bf16",
    "sar_noalloc_flags", "sar_plan_set_wait_budget", "sar_measure_pipe_rates", "sar_plan_create_streamed",
)

SAR_FLAG_TILE_WINDOW, SAR_FLAG_STRIP_WINDOW, SAR_FLAG_WAIT_TIMEOUT, SAR_FLAG_GATHER_WINDOW = 1, 2, 8, 16

SAR_UNET_LAYERS = 15
SAR_CPHD_CI2, SAR_CPHD_CI4, SAR_CPHD_CF8 = 1, 2, 3


class SarGeometry(ctypes.Structure):
    """Mirror of ``sar_geometry`` (include/sargpu.h)."""

    _fields_ = [
        ("num_fast_times", c_size_t), ("num_slow_times", c_size_t), ("num_scatterers", c_size_t),
        ("transmit_posns", c_void_p), ("receive_posns", c_void_p), ("stab_ref_posns", c_void_p),
        ("scat_posns", c_void_p), ("waveform_fft", c_void_p), ("slow_time_weighting", c_void_p),
        ("centre_frequency", c_double), ("sample_frequency", c_double), ("c_eff", c_double),
        ("upsample_ratio", c_double), ("sign_multiplier", c_double),
        ("interp", c_int),
        ("grid_shape", c_size_t * 3), ("grid_origin", c_double * 3), ("grid_step_x", c_double * 3),
        ("grid_step_y", c_double * 3), ("grid_step_z", c_double * 3),
        ("path", c_int),
    ]


class SarUnetLayer(ctypes.Structure):
    """Mirror of ``sar_unet_layer``."""

    _fields_ = [("weight_offset", c_size_t), ("bias_offset", c_size_t), ("cin0", c_int), ("cin1", c_int),
                ("cout", c_int), ("taps", c_int), ("relu", c_int), ("level", c_int)]


class SarCglsResult(ctypes.Structure):
    """Mirror of ``sar_cgls_result``."""

    _fields_ = [("iterations", c_int), ("converged", c_int), ("breakdown", c_int), ("residual", c_double),
                ("norm_ahy", c_double)]


class SarPdhgResult(ctypes.Structure):
    """Mirror of ``sar_pdhg_result``."""

    _fields_ = [("iterations", c_int), ("sigma", c_double), ("tau", c_double), ("theta", c_double),
                ("operator_norm", c_double)]


class SarPipeRates(ctypes.Structure):
    """Mirror of ``sar_pipe_rates``."""
    _fields_ = [("sfu_sincos_per_clk_sm", ctypes.c_double), ("frnd_per_clk_sm", ctypes.c_double),
                ("ffma_per_clk_sm", ctypes.c_double), ("ffma2_per_clk_sm", ctypes.c_double),
                ("num_sms", c_int), ("sm_mhz", ctypes.c_double)]


class SarPlanInfo(ctypes.Structure):
    """Mirror of ``sar_plan_info``."""

    _fields_ = [
        ("working_length", c_size_t), ("profile_first_bin", c_long), ("profile_length", c_size_t),
        ("tile_window", c_size_t), ("strip_window", c_size_t), ("device_bytes", c_size_t), ("grid", c_int),
        ("interp", c_int), ("num_fast_times", c_size_t), ("num_slow_times", c_size_t), ("num_scatterers", c_size_t),
        ("device", c_int), ("fft_callbacks", c_int), ("gather_lanes_y", c_int), ("fused_upsampling", c_int), ("fused_downsampling", c_int),
        ("scatter_lanes_y", c_int), ("block_pulses", c_size_t), ("scatter_shear", c_int),
        ("gather_shear", c_int), ("scatter_ring_half", c_int),
    ]


class SarCalculationInfo(ctypes.Structure):
    """Byte-for-byte the reference struct (src/sarsolver/cxx_binding/sarsolver_cxx.hpp:28-33,
    mirrored in Python at src/sarsolver/cxx_binding/sarsolver_cxx.py:49-62)."""

    _fields_ = [("num_fast_times", c_size_t), ("num_slow_times", c_size_t), ("num_scatterers", c_size_t),
                ("transmit_posns", POINTER(c_double)), ("receive_posns", POINTER(c_double)),
                ("stab_ref_posns", POINTER(c_double)), ("scat_posns", POINTER(c_double)),
                ("phase_history", POINTER(c_double)), ("scattering_amplitudes", POINTER(c_double)),
                ("waveform_fft", POINTER(c_double)), ("slow_time_weighting", POINTER(c_double)),
                ("centre_frequency", c_double), ("sample_frequency", c_double), ("c_eff", c_double),
                ("upsample_ratio", c_double), ("sign_multiplier", c_double)]


_LIB = None


def library_path() -> str:
    return GPU_LIB


def load() -> ctypes.CDLL:
    """Load libsargpu.so; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(GPU_LIB):
        raise RuntimeError(f"libsargpu.so is not built ({GPU_LIB}); run sarsolver_gb300.build.build()")
    lib = ctypes.CDLL(GPU_LIB)
    lib.sar_plan_create.argtypes = [POINTER(SarGeometry), c_int, POINTER(c_void_p)]
    lib.sar_plan_create_streamed.argtypes = [POINTER(SarGeometry), c_int, c_size_t, POINTER(c_void_p)]
    lib.sar_plan_create_streamed.restype = c_int
    lib.sar_plan_destroy.argtypes = [c_void_p]
    lib.sar_plan_get_info.argtypes = [c_void_p, POINTER(SarPlanInfo)]
    for name in ("sar_forward", "sar_adjoint", "sar_profiles"):
        getattr(lib, name).argtypes = [c_void_p, c_void_p, c_void_p, c_void_p]
    lib.sar_set_slow_time_weighting.argtypes = [c_void_p, c_void_p]
    lib.sar_set_slow_time_weighting_device.argtypes = [c_void_p, c_void_p, c_void_p]
    lib.sar_device_flags.argtypes = [c_void_p, POINTER(c_uint)]
    lib.sar_enable_stage_timing.argtypes = [c_void_p, c_int]
    lib.sar_phase_gradient.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t, c_size_t, ctypes.c_float, c_void_p]
    lib.sar_phase_gradient.restype = c_int
    lib.sar_sharpness.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]
    lib.sar_sharpness.restype = c_int
    lib.sar_cgls.argtypes = [c_void_p, c_void_p, c_void_p, c_int, c_int, c_double, c_void_p,
                             POINTER(SarCglsResult), c_void_p]
    lib.sar_cgls.restype = c_int
    lib.sar_cgls_ex.argtypes = [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_double, c_void_p,
                                POINTER(SarCglsResult), c_void_p]
    lib.sar_cgls_ex.restype = c_int
    lib.sar_pdhg.argtypes = [c_void_p, c_void_p, c_void_p, c_int, c_int, c_double, c_double, c_double, c_double,
                             c_int, c_void_p, POINTER(SarPdhgResult), c_void_p]
    lib.sar_pdhg.restype = c_int
    lib.sar_host_device_pointer.argtypes = [c_void_p, ctypes.POINTER(c_void_p)]
    lib.sar_host_device_pointer.restype = c_int
    lib.sar_adjoint_pulse_block.argtypes = [c_void_p, c_void_p, c_size_t, c_size_t, c_void_p, c_int, c_void_p]
    lib.sar_adjoint_pulse_block.restype = c_int
    lib.sar_noalloc_flags.argtypes = [POINTER(c_uint), c_void_p]
    lib.sar_noalloc_flags.restype = c_int
    lib.sar_plan_set_wait_budget.argtypes = [c_void_p, ctypes.c_longlong, c_int]
    lib.sar_plan_set_wait_budget.restype = c_int
    lib.sar_measure_pipe_rates.argtypes = [POINTER(SarPipeRates), c_void_p]
    lib.sar_measure_pipe_rates.restype = c_int
    lib.sar_move_srps.argtypes = [c_void_p, c_void_p, c_size_t, c_size_t, c_void_p, c_double, c_double, c_double,
                                  c_double, c_void_p]
    lib.sar_move_srps.restype = c_int
    lib.sar_fast_freq_downsample.argtypes = [c_void_p, c_void_p, c_size_t, c_size_t, c_size_t, c_void_p, c_void_p]
    lib.sar_fast_freq_downsample.restype = c_int
    lib.sar_resample_phase_history.argtypes = [c_void_p, c_size_t, c_size_t, c_void_p, c_double, c_double, c_double,
                                               c_double, c_size_t, c_void_p, c_void_p, c_size_t, c_void_p, c_size_t,
                                               c_void_p, c_void_p]
    lib.sar_resample_phase_history.restype = c_int
    lib.sar_cphd_decode.argtypes = [c_void_p, c_int, c_size_t, c_size_t, c_void_p, c_void_p, c_void_p]
    lib.sar_cphd_decode.restype = c_int
    P = c_void_p
    unet_sigs = {
        "sar_unet_create": [c_int, c_int, P],
        "sar_unet_destroy": [P],
        "sar_unet_info": [P, P, P],
        "sar_unet_set_params": [P, P, P],
        "sar_unet_get_params": [P, P, P],
        "sar_unet_get_grads": [P, P, P],
        "sar_unet_zero_grad": [P, P],
        "sar_unet_forward": [P, P, ctypes.c_float, c_int, c_int, c_int, P, P],
        "sar_unet_backward": [P, P, P],
        "sar_unet_adam_step": [P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, c_int, P],
        "sar_unet_flags": [P, P],
        "sar_conv2d_forward_bf16": [P, c_int, P, c_int, c_int, c_int, c_int, c_int, P, P, c_int, c_int, P, P, P],
        "sar_conv2d_wgrad_bf16": [P, c_int, P, c_int, P, c_int, c_int, c_int, c_int, c_int, P, P, P],
    }
    for name, args in unet_sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = c_int
    lib.sar_stage_times.argtypes = [c_void_p, POINTER(ctypes.c_float), POINTER(c_int)]
    for name in ("sar_plan_create", "sar_plan_destroy", "sar_plan_get_info", "sar_forward", "sar_adjoint",
                 "sar_profiles", "sar_set_slow_time_weighting", "sar_set_slow_time_weighting_device",
                 "sar_device_flags", "sar_enable_stage_timing", "sar_stage_times"):
        getattr(lib, name).restype = c_int
    lib.sar_last_error.argtypes = [c_char_p, c_size_t]
    lib.sar_last_error.restype = c_size_t
    lib.sar_status_string.argtypes = [c_int]
    lib.sar_status_string.restype = c_char_p
    for name in ("forward_evaluate", "adjoint_evaluate"):
        getattr(lib, name).argtypes = [POINTER(SarCalculationInfo)]
        getattr(lib, name).restype = None
    _LIB = lib
    return lib


def last_error() -> str:
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.sar_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


class SarError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


def check(status: int, what: str) -> None:
    if status != SAR_OK:
        lib = load()
        raise SarError(status, f"{what}: {lib.sar_status_string(status).decode()}: {last_error()}")


_HOST = None


def load_host() -> ctypes.CDLL:
    """Host build of the kernels' range geometry (precision checks on machines without a GPU)."""
    global _HOST
    if _HOST is None:
        if not os.path.exists(HOST_LIB):
            raise RuntimeError(f"{HOST_LIB} is not built; run sarsolver_gb300.build.build()")
        lib = ctypes.CDLL(HOST_LIB)
        P = c_void_p
        lib.sar_geom_host_eval.argtypes = [P, P, P, P, c_int, c_int, c_int, c_size_t, P, P, P, c_double, c_double,
                                           ctypes.c_float, c_int, P, P]
        lib.sar_geom_host_eval_transposed.argtypes = lib.sar_geom_host_eval.argtypes
        lib.sar_tile_halfspan_host.argtypes = [P, P, c_size_t, P, P, P, P, c_int, c_int, c_int, c_double]
        lib.sar_tile_halfspan_host.restype = c_double
        lib.sar_geom_host_eval_points.argtypes = [P, c_size_t, P, c_size_t, P, P, P, c_double, c_double,
                                                  ctypes.c_float, P, P]
        lib.sar_gather_window_check_host.argtypes = [P, P, P, P, c_int, c_int, c_int, c_size_t, P, P, P, c_double,
                                                     c_double, ctypes.c_float, c_int, c_int, P]
        lib.sar_gather_window_check_host.restype = c_long
        lib.sar_bin_extent_host.argtypes = [P, P, P, P, c_int, c_int, c_int, P, P, P, c_double, c_double,
                                            ctypes.c_float, c_int, c_int, c_int, c_int, c_int, P]
        lib.sar_bin_extent_host.restype = c_int
        lib.sar_geom_host_eval_sheared.argtypes = [P, P, P, P, c_int, c_int, c_int, c_size_t, P, P, P, c_double,
                                                   c_double, ctypes.c_float, c_int, c_int, P, P]
        lib.sar_choose_shear_host.argtypes = [P, P, c_size_t, P, P, P, P, c_int, c_int, c_int, c_double]
        lib.sar_choose_shear_host.restype = c_int
        lib.sar_geom_host_eval_sheared_lanes.argtypes = lib.sar_geom_host_eval_sheared.argtypes
        lib.sar_choose_gather_shear_host.argtypes = lib.sar_choose_shear_host.argtypes
        lib.sar_choose_gather_shear_host.restype = c_int
        lib.sar_parallelogram_distance_host.argtypes = [P, P, P, P, P, P]
        lib.sar_parallelogram_distance_host.restype = None
        _HOST = lib
    return _HOST
