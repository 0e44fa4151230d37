"""Bounded in-kernel waits that run out are reported, and the plan stays usable.

The backprojection gather's warp roles hand pulse stages to each other through shared-memory
barriers; every wait is bounded (sar_plan_set_wait_budget).  Here the producers are told never to
publish the first stage (a barrier nothing completes), with a short budget: the consumers' first
wait must run out, the kernel must return with SAR_FLAG_WAIT_TIMEOUT set, and the next normal call
on the same plan must give the same image as before, bit for bit, with no flag.  The producers'
own copies are waited for with the full budget before a CTA exits, so nothing is in flight then.
"""
import ctypes

import numpy as np
import pytest
import torch

from cases import crandn, spotlight_case
from sarsolver_gb300 import SarPlan, _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("n", [32, 96])
def test_expired_gather_wait_is_reported(n):
    rng = np.random.default_rng(5)
    case = spotlight_case(64, 256, n, 0.5, 4.0)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear", path="grid")
    y = torch.from_numpy(crandn(rng, 64, 256)).to(torch.complex64).cuda()
    ref = plan.adjoint(y).clone()
    assert plan.device_flags() == 0
    plan.set_wait_budget(200_000, hold_first_stage=True)    # ~0.1 ms at 2 GHz
    plan.adjoint(y)
    flags = plan.device_flags()
    assert flags & _lib.SAR_FLAG_WAIT_TIMEOUT, flags
    plan.set_wait_budget(0)                                 # back to the default budget
    again = plan.adjoint(y)
    assert plan.device_flags() == 0
    assert torch.equal(again, ref)


def test_streamed_backprojection_is_bitwise_reproducible():
    """Blocks after the first add onto the image (accumulate): the gather then runs one CTA per
    tile, so the image's bits do not depend on the order in which CTAs finish."""
    rng = np.random.default_rng(9)
    case = spotlight_case(512, 512, 1024, 0.25, 5.0)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    y = torch.from_numpy(crandn(rng, 512, 512)).to(torch.complex64)
    yh = y.pin_memory()
    # back to back, no synchronisation in between: the second call's host-to-device copies must not
    # overwrite staging memory the first call's gathers are still reading
    a = plan.adjoint_streamed(yh, block=128).clone()
    b = plan.adjoint_streamed(yh, block=128).clone()
    c = plan.adjoint_streamed(yh, block=128).clone()
    full = plan.adjoint(y.cuda())
    torch.cuda.synchronize()
    assert torch.equal(a, b) and torch.equal(b, c)
    assert float(torch.linalg.vector_norm(a - full) / torch.linalg.vector_norm(full)) < 5e-6
    assert plan.device_flags() == 0


def test_pipe_rates_are_measured():
    """sar_measure_pipe_rates: per-SM rates of the gather's arithmetic pipes on this device."""
    lib = _lib.load()
    r = _lib.SarPipeRates()
    _lib.check(lib.sar_measure_pipe_rates(ctypes.byref(r), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "sar_measure_pipe_rates")
    print(f"per clock per SM: sin/cos {r.sfu_sincos_per_clk_sm:.2f}, rint {r.frnd_per_clk_sm:.2f}, "
          f"FFMA {r.ffma_per_clk_sm:.2f}, FFMA2 lanes {r.ffma2_per_clk_sm:.2f}; {r.num_sms} SMs at {r.sm_mhz:.0f} MHz")
    assert r.num_sms == torch.cuda.get_device_properties(0).multi_processor_count
    assert 64.0 <= r.ffma_per_clk_sm <= 132.0
    assert 64.0 <= r.ffma2_per_clk_sm <= 264.0
    assert 4.0 <= r.sfu_sincos_per_clk_sm <= 132.0
    assert 4.0 <= r.frnd_per_clk_sm <= 132.0
    assert r.sm_mhz > 100.0
