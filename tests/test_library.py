"""libsargpu.so as a C library: it loads, exports every function include/sargpu.h declares,
mirrors the reference struct byte for byte, and rejects bad geometry with a status code and a
message before touching the GPU (so these run on a machine without one)."""
import ctypes
import os
import re

import numpy as np

import oracle
from sarsolver_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "sargpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w]*\s*\**\s*([A-Za-z_]\w*)\s*\([^;]*\)\s*;", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_function():
    lib = _lib.load()
    names = declared_functions()
    assert "sar_adjoint" in names and "adjoint_evaluate" in names
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(_lib.EXPORTED) == names


def test_struct_layout_matches_reference():
    ours, ref = _lib.SarCalculationInfo, oracle._RefInfo
    assert ctypes.sizeof(ours) == ctypes.sizeof(ref) == 128
    for (name_a, _), (name_b, _) in zip(ours._fields_, ref._fields_):
        assert name_a == name_b
        assert getattr(ours, name_a).offset == getattr(ref, name_b).offset


def _geometry(N=16, S=4, P=8):
    keep = dict(t=np.zeros((S, 3)) + [1000.0, 0, 0], s=np.zeros((S, 3)), p=np.zeros((P, 3)))
    g = _lib.SarGeometry()
    g.num_fast_times, g.num_slow_times, g.num_scatterers = N, S, P
    g.transmit_posns = g.receive_posns = keep["t"].ctypes.data
    g.stab_ref_posns = keep["s"].ctypes.data
    g.scat_posns = keep["p"].ctypes.data
    g.centre_frequency, g.sample_frequency, g.c_eff, g.upsample_ratio, g.sign_multiplier = 1e9, 1e8, 3e8, 8.0, 1.0
    return g, keep


def _create(g):
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.sar_plan_create(ctypes.byref(g), 0, ctypes.byref(h))
    return rc, _lib.last_error(), h


def test_validation_rejects_bad_geometry_without_gpu():
    g, keep = _geometry()
    g.num_fast_times = 0
    rc, msg, h = _create(g)
    assert rc == _lib.SAR_ERR_INVALID_ARGUMENT and "empty" in msg and not h.value

    g, keep = _geometry()
    keep["t"][1, 2] = np.nan
    rc, msg, _ = _create(g)
    assert rc == _lib.SAR_ERR_INVALID_ARGUMENT and "non-finite" in msg

    g, keep = _geometry()
    g.grid_shape[0], g.grid_shape[1], g.grid_shape[2] = 1, 3, 3   # 9 != P = 8
    rc, msg, _ = _create(g)
    assert rc == _lib.SAR_ERR_INVALID_ARGUMENT and "grid_shape" in msg

    g, keep = _geometry()
    g.upsample_ratio = 0.5
    rc, msg, _ = _create(g)
    assert rc == _lib.SAR_ERR_INVALID_ARGUMENT

    g, keep = _geometry()
    g.interp = 7
    rc, msg, _ = _create(g)
    assert rc == _lib.SAR_ERR_INVALID_ARGUMENT and "interpolation" in msg

    g, keep = _geometry()
    g.scat_posns = None
    rc, msg, _ = _create(g)
    assert rc == _lib.SAR_ERR_INVALID_ARGUMENT and "scat_posns" in msg


def test_null_arguments_and_status_strings():
    lib = _lib.load()
    assert lib.sar_forward(None, None, None, None) == _lib.SAR_ERR_INVALID_ARGUMENT
    assert lib.sar_adjoint(None, None, None, None) == _lib.SAR_ERR_INVALID_ARGUMENT
    assert lib.sar_plan_destroy(None) == 0
    assert lib.sar_status_string(0) == b"ok"
    assert lib.sar_status_string(4) == b"out of device memory"


def test_new_entry_points_validate_arguments_without_gpu():
    lib = _lib.load()
    null = ctypes.c_void_p(0)
    res = _lib.SarCglsResult()
    assert lib.sar_cgls_ex(null, null, null, 0, null, 10, 1e-3, null, ctypes.byref(res), null) == _lib.SAR_ERR_INVALID_ARGUMENT
    assert "null" in _lib.last_error()
    assert lib.sar_phase_gradient(null, null, null, 4, 4, 4.0, null) == _lib.SAR_ERR_INVALID_ARGUMENT
    assert lib.sar_sharpness(null, null, null, 4, null) == _lib.SAR_ERR_INVALID_ARGUMENT
    h = ctypes.c_void_p()
    assert lib.sar_unet_create(48, 0, ctypes.byref(h)) == _lib.SAR_ERR_NOT_SUPPORTED
    assert "base_channels" in _lib.last_error()
    win = np.ones(8)
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check fails first
    assert lib.sar_fast_freq_downsample(dummy, dummy, 4, 4, 9, win.ctypes.data_as(ctypes.c_void_p), null) == \
        _lib.SAR_ERR_INVALID_ARGUMENT
    assert "new_N" in _lib.last_error()
    rows = np.array([0, 3], dtype=np.int32)
    kern = np.zeros((4, 2))
    assert lib.sar_resample_phase_history(dummy, 6, 4, null, 1e9, 1e8, 1.0, 3e8, 4, win.ctypes.data_as(ctypes.c_void_p),
                                          kern.ctypes.data_as(ctypes.c_void_p), 4, rows.ctypes.data_as(ctypes.c_void_p),
                                          2, dummy, null) == _lib.SAR_ERR_INVALID_ARGUMENT
    assert "window" in _lib.last_error()
    assert lib.sar_adjoint_pulse_block(null, null, 0, 1, null, 0, null) == _lib.SAR_ERR_INVALID_ARGUMENT
