"""Range-profile FFTs with cuFFT load/store callbacks (sar_fft_callbacks.cu, opt-in with
SAR_FFT_CALLBACKS=1) against the packing kernels and the FP64 oracle: even N with a power-of-two
working length, odd N with a non-power-of-two length, nearest_ref, pulse blocks (other batch
sizes).  Where cuFFT cannot build plans with JIT callbacks (GB300 with the cuFFT of CUDA 13.0
returns CUFFT_INTERNAL_ERROR), the tests check instead that plan creation reports it as a cuFFT
error naming the callback plan, and that the process goes on: a default plan (packing kernels or
the fused transforms) built right after computes the same case correctly.  The default plans never
use callbacks."""
import os

import numpy as np
import pytest
import torch

import oracle
from cases import crandn, rel_l2, spotlight_case
from sarsolver_gb300 import SarPlan, _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def make_plan(case, interp, flag, path="auto"):
    old = os.environ.get("SAR_FFT_CALLBACKS")
    os.environ["SAR_FFT_CALLBACKS"] = flag
    try:
        return SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp=interp, path=path)
    except _lib.SarError as e:
        if flag == "1" and "callback FFT plan" in str(e):
            # this stack cannot link JIT callbacks: the failure must be a clean cuFFT status
            assert e.status == _lib.SAR_ERR_CUFFT, e
            return None
        raise
    finally:
        if old is None:
            os.environ.pop("SAR_FFT_CALLBACKS")
        else:
            os.environ["SAR_FFT_CALLBACKS"] = old


@pytest.mark.parametrize("num_freqs", [256, 245])
@pytest.mark.parametrize("interp", ["linear", "nearest_ref"])
def test_callbacks_match_packing_kernels_and_oracle(num_freqs, interp):
    case = spotlight_case(num_pulses=96, num_freqs=num_freqs, n=64, spacing=0.5, aperture_deg=3.0)
    cb = make_plan(case, interp, "1")
    pk = make_plan(case, interp, "0")
    assert not pk.fft_callbacks
    rng = np.random.default_rng(num_freqs)
    if cb is None:   # callbacks unavailable: the default plan right after is correct
        x = crandn(rng, pk.num_scatterers)
        y = crandn(rng, pk.num_slow_times, pk.num_freqs)
        p = case.problem()
        f = pk.forward(torch.from_numpy(x.astype(np.complex64))).cpu().numpy()
        a = pk.adjoint(torch.from_numpy(y.astype(np.complex64))).cpu().numpy()
        tol = 1e-5   # nearest_ref included: grid bins near a rounding boundary are decided in FP64 terms
        assert rel_l2(f, oracle.forward(p, x, interp, threads=oracle.default_threads())) < tol
        assert rel_l2(a, oracle.adjoint(p, y, interp, threads=oracle.default_threads())) < tol
        assert pk.device_flags() == 0
        return
    assert cb.fft_callbacks
    x = torch.from_numpy(crandn(rng, cb.num_scatterers).astype(np.complex64))
    y = torch.from_numpy(crandn(rng, cb.num_slow_times, cb.num_freqs).astype(np.complex64))
    f_cb, f_pk = cb.forward(x).cpu().numpy(), pk.forward(x).cpu().numpy()
    a_cb, a_pk = cb.adjoint(y).cpu().numpy(), pk.adjoint(y).cpu().numpy()
    assert rel_l2(f_cb, f_pk) < 2e-6 and rel_l2(a_cb, a_pk) < 2e-6
    assert rel_l2(cb.profiles(y).cpu().numpy(), pk.profiles(y).cpu().numpy()) < 2e-6
    if interp == "linear":
        p = case.problem()
        assert rel_l2(f_cb, oracle.forward(p, x.numpy(), "linear", threads=oracle.default_threads())) < 1e-5
        assert rel_l2(a_cb, oracle.adjoint(p, y.numpy(), "linear", threads=oracle.default_threads())) < 1e-5
    assert cb.device_flags() == 0


def test_callbacks_with_pulse_blocks():
    case = spotlight_case(num_pulses=100, num_freqs=256, n=64, spacing=0.5, aperture_deg=3.0)
    cb = make_plan(case, "linear", "1") or make_plan(case, "linear", "0")   # packing kernels if unavailable
    rng = np.random.default_rng(7)
    y = torch.from_numpy(crandn(rng, cb.num_slow_times, cb.num_freqs).astype(np.complex64))
    full = cb.adjoint(y)
    streamed = cb.adjoint_streamed(y.pin_memory(), block=40)     # batches of 40, 40, 20
    assert float(torch.linalg.vector_norm(streamed - full) / torch.linalg.vector_norm(full)) < 1e-6


def test_default_plans_use_the_packing_kernels():
    case = spotlight_case(num_pulses=8, num_freqs=64, n=32, spacing=0.5, aperture_deg=3.0)
    old = os.environ.pop("SAR_FFT_CALLBACKS", None)
    try:
        assert not SarPlan(case.scene, case.aperture, upsample_ratio=8.0, interp="linear").fft_callbacks
    finally:
        if old is not None:
            os.environ["SAR_FFT_CALLBACKS"] = old
