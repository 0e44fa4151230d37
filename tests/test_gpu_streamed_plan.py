"""Streamed plans: device memory bounded by a block of pulses (sar_plan_create_streamed).

The reference bounds memory by slow-time blocking (num_calculation_blocks, cxx_binding/forward.py:66-96,
adjoint.py:66-94).  A streamed plan keeps two blocks of range profiles instead of all S pulses'
and runs the operators block by block; its results equal the resident plan's up to FP32 summation
order (backprojection: blocks after the first add onto the image; forward projection: the same
per-pulse sums), in both interpolation modes, including the nearest-bin exact re-decisions that
index per-pulse antenna norms block-relative.
"""
import numpy as np
import pytest
import torch

from cases import crandn, rel_l2, spotlight_case
from sarsolver_gb300 import NumpySimpleSarOperator, SarPlan
from sarsolver_gb300.scenes import add_noise, config_workload, reflectivity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("interp", ["linear", "nearest_ref"])
@pytest.mark.parametrize("block", [96, 128, 1000])
def test_streamed_plan_matches_resident(interp, block):
    rng = np.random.default_rng(3)
    case = spotlight_case(300, 512, 256, 0.5, 4.0, weights=np.exp(1j * rng.uniform(-1, 1, 300)))
    res = SarPlan(case.scene, case.aperture, upsample_ratio=8.0, interp=interp)
    stm = SarPlan(case.scene, case.aperture, upsample_ratio=8.0, interp=interp, block_pulses=block)
    assert stm.block_pulses == (block if block < 300 else 0)
    if block < 300:
        assert stm.device_bytes < res.device_bytes
    x = torch.from_numpy(crandn(rng, case.scene.num_scatterers)).to(torch.complex64).cuda()
    y = torch.from_numpy(crandn(rng, 300, 512)).to(torch.complex64).cuda()
    assert rel_l2(stm.forward(x).cpu().numpy(), res.forward(x).cpu().numpy()) < 1e-6
    assert rel_l2(stm.adjoint(y).cpu().numpy(), res.adjoint(y).cpu().numpy()) < 2e-6
    # blocks streamed from pinned host memory through the streamed plan
    xs = stm.adjoint_streamed(y.cpu().pin_memory(), block=block)
    assert rel_l2(xs.cpu().numpy(), res.adjoint(y).cpu().numpy()) < 2e-6
    assert stm.device_flags() == 0 and res.device_flags() == 0


@pytest.mark.parametrize("interp", ["linear", "nearest_ref"])
def test_streamed_plan_with_ring_and_value_windows(interp):
    """Upsample 128 on 0.25 m pixels with a 20 degree aperture: the forward scatter keeps ring
    windows and the backprojection stages windows of plain values; streamed in blocks of 24 pulses
    (ring slots of 8-byte rows, the scatter per block) the plan equals the resident one."""
    rng = np.random.default_rng(5)
    case = spotlight_case(64, 96, 100, 0.25, 20.0, upsample=128.0, weights=np.exp(1j * rng.uniform(-1, 1, 64)))
    res = SarPlan(case.scene, case.aperture, upsample_ratio=128.0, interp=interp)
    stm = SarPlan(case.scene, case.aperture, upsample_ratio=128.0, interp=interp, block_pulses=24)
    assert stm.block_pulses == 24
    assert res.scatter_ring_half > 0 and stm.scatter_ring_half > 0 and res.tile_window > 256
    x = torch.from_numpy(crandn(rng, case.scene.num_scatterers)).to(torch.complex64).cuda()
    y = torch.from_numpy(crandn(rng, 64, 96)).to(torch.complex64).cuda()
    assert rel_l2(stm.forward(x).cpu().numpy(), res.forward(x).cpu().numpy()) < 1e-6
    ref = res.adjoint(y).cpu().numpy()
    assert rel_l2(stm.adjoint(y).cpu().numpy(), ref) < 2e-6
    assert rel_l2(stm.adjoint_streamed(y.cpu().pin_memory(), block=24).cpu().numpy(), ref) < 2e-6
    assert stm.device_flags() == 0 and res.device_flags() == 0


def test_resident_pulse_blocks_nearest_ref_match_whole():
    """Pulse blocks of a resident plan in nearest_ref: exact re-decisions use the block's own pulses."""
    rng = np.random.default_rng(4)
    case = spotlight_case(256, 256, 128, 0.5, 4.0)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=8.0, interp="nearest_ref")
    y = torch.from_numpy(crandn(rng, 256, 256)).to(torch.complex64)
    whole = plan.adjoint(y.cuda())
    blocks = plan.adjoint_streamed(y.pin_memory(), block=64)
    assert rel_l2(blocks.cpu().numpy(), whole.cpu().numpy()) < 2e-6


def test_operator_num_calculation_blocks_streams():
    """NumpySimpleSarOperator(num_calculation_blocks=4): a streamed plan of ceil(S / 4) pulses."""
    rng = np.random.default_rng(5)
    case = spotlight_case(200, 256, 128, 0.5, 4.0)
    op = NumpySimpleSarOperator(case.scene, case.aperture, upsample_ratio=8.0, interp="linear",
                                num_calculation_blocks=4)
    ref = NumpySimpleSarOperator(case.scene, case.aperture, upsample_ratio=8.0, interp="linear")
    assert op.plan.block_pulses == 50 and ref.plan.block_pulses == 0
    x = crandn(rng, case.scene.num_scatterers)
    y = crandn(rng, 200 * 256)
    assert rel_l2(op.matvec(x), ref.matvec(x)) < 1e-6
    assert rel_l2(op.rmatvec(y), ref.rmatvec(y)) < 2e-6


def test_scale_configuration_streamed_memory():
    """The scale configuration (8192^2 x 16384 pulses x 8192 samples) on a streamed plan of
    512-pulse blocks: profile memory two blocks instead of all pulses; the result equals the
    resident plan's backprojection."""
    aperture, scene, upsample, _ = config_workload("config5")
    n = scene.grid_shape[2]
    x = reflectivity(n, 5000, 8.0, seed=11)
    stm = SarPlan(scene, aperture, upsample_ratio=upsample, interp="linear", block_pulses=512)
    y = stm.forward(x)
    img_s = stm.adjoint(y)
    torch.cuda.synchronize()
    bytes_s = stm.device_bytes
    assert stm.device_flags() == 0
    stm.close()
    res = SarPlan(scene, aperture, upsample_ratio=upsample, interp="linear")
    img = res.adjoint(y)
    y_r = res.forward(x)
    torch.cuda.synchronize()
    print(f"scale: device bytes streamed plan {bytes_s / 1e9:.2f} GB, resident plan {res.device_bytes / 1e9:.2f} GB")
    assert bytes_s < 0.25 * res.device_bytes
    assert float(torch.linalg.vector_norm(img_s - img) / torch.linalg.vector_norm(img)) < 5e-6
    assert float(torch.linalg.vector_norm(y - y_r) / torch.linalg.vector_norm(y_r)) < 1e-6
