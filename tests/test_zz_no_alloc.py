"""The allocation-free backprojection entry point (sar_adjoint_from_profiles_noalloc).

It exists for callers that may not allocate device memory while they run (code inside another
runtime's memory pool, real-time loops, hosts whose allocator belongs to another framework): all
its scratch lives in one fixed device array inside the library.  This checks, through the C ABI,
that two calls in a row reproduce the regular backprojection (sar_adjoint) from the profiles
sar_profiles() writes, with no device check flag raised (sar_noalloc_flags), and that a problem too
large for the fixed array is refused.

The file name sorts last so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from cases import crandn, rel_l2, spotlight_case
from sarsolver_gb300 import SarPlan, _lib
from sarsolver_gb300.geometry import grid_axes

pytestmark = pytest.mark.gpu

TOL = 1.0e-5   # the linear-mode tolerance of the operator tests


def _geometry(case, interp):
    ap, sc = case.aperture, case.scene
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    keep = dict(tx=f64(ap.transmitter_positions), rx=f64(ap.receiver_positions), srp=f64(ap.stab_ref_posns),
                wave=np.ascontiguousarray(np.fft.ifftshift(ap.waveform_fft).astype(np.complex128)).view(np.float64),
                wt=np.ascontiguousarray(ap.slow_time_weighting.astype(np.complex128)).view(np.float64))
    g = _lib.SarGeometry()
    g.num_fast_times, g.num_slow_times, g.num_scatterers = ap.num_freqs, ap.num_slow_times, sc.num_scatterers
    g.transmit_posns, g.receive_posns = keep["tx"].ctypes.data, keep["rx"].ctypes.data
    g.stab_ref_posns = keep["srp"].ctypes.data
    g.waveform_fft, g.slow_time_weighting = keep["wave"].ctypes.data, keep["wt"].ctypes.data
    g.centre_frequency, g.sample_frequency, g.c_eff = ap.centre_frequency, ap.sample_bandwidth, ap.c_eff
    g.upsample_ratio, g.sign_multiplier = case.upsample_ratio, ap.sign_multiplier
    g.interp = _lib.INTERP[interp]
    shape, origin, ex, ey, ez = grid_axes(sc)
    for i in range(3):
        g.grid_shape[i], g.grid_origin[i] = shape[i], origin[i]
        g.grid_step_x[i], g.grid_step_y[i], g.grid_step_z[i] = ex[i], ey[i], ez[i]
    return g, keep


def _noalloc(lib, g, prof, first, span, x):
    fn = lib.sar_adjoint_from_profiles_noalloc
    fn.argtypes = [ctypes.POINTER(_lib.SarGeometry), ctypes.c_void_p, ctypes.c_long, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return fn(ctypes.byref(g), ctypes.c_void_p(prof.data_ptr()), first, span, ctypes.c_void_p(x.data_ptr()), stream)


@pytest.mark.parametrize("interp,upsample", [("linear", 8.0), ("nearest_ref", 8.0), ("nearest_ref", 128.0)])
def test_noalloc_backprojection_matches_plan_twice(interp, upsample):
    """Upsample 128 with nearest bins: staged windows wider than 256 bins, of plain values."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    rng = np.random.default_rng(17)
    case = spotlight_case(96, 256, 100, 0.5 if upsample == 8.0 else 0.1, 4.0, upsample=upsample,
                          weights=np.exp(1j * rng.uniform(-1, 1, 96)))
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp=interp, path="grid")
    y = torch.from_numpy(crandn(rng, 96, 256)).to(torch.complex64).cuda()
    ref = plan.adjoint(y).cpu().numpy()
    prof = plan.profiles(y)
    g, keep = _geometry(case, interp)
    for _ in range(2):   # the second call must not depend on what the first left in the array
        x = torch.full((case.scene.num_scatterers,), float("nan"), dtype=torch.complex64, device="cuda")
        rc = _noalloc(lib, g, prof, plan.profile_first_bin, plan.profile_length, x)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        assert rel_l2(x.cpu().numpy(), ref) < TOL
        # the call's device check flags (bounded waits, window bounds), read without allocating
        flags = ctypes.c_uint(0xFFFFFFFF)
        rc = lib.sar_noalloc_flags(ctypes.byref(flags), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, _lib.last_error()
        assert flags.value == 0


def test_noalloc_rejects_problems_beyond_its_array():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    case = spotlight_case(64, 64, 32, 0.5, 3.0)
    g, keep = _geometry(case, "linear")
    span = 1 << 20                                    # 64 pulses x 2^20 bins x 16 B = 1 GiB
    prof = torch.zeros(16, dtype=torch.complex64, device="cuda")
    x = torch.zeros(case.scene.num_scatterers, dtype=torch.complex64, device="cuda")
    rc = _noalloc(lib, g, prof, -(span // 2), span, x)
    assert rc == _lib.SAR_ERR_INVALID_ARGUMENT
    assert "scratch" in _lib.last_error()
