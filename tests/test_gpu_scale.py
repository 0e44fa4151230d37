"""The scale configuration: 8192^2 image at 0.125 m, 16384 pulses x 8192 samples, U = 8 (1.1e12
pixel-pulses per operator application).  Forward and backprojection on the device, the
backprojection also streamed from pinned host memory in 512-pulse blocks; FP64-oracle errors on a
256^2 patch (backprojection: the exact pixel subset; forward: 16 pulse rows)."""
import time

import numpy as np
import pytest
import torch

import oracle
from cases import rel_l2
from sarsolver_gb300 import SarPlan
from sarsolver_gb300.scenes import config_workload, reflectivity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def timed(fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def test_scale_configuration():
    aperture, scene, upsample, desc = config_workload("config5")
    plan = SarPlan(scene, aperture, upsample_ratio=upsample, interp="linear")
    n = scene.grid_shape[2]
    S, N = plan.num_slow_times, plan.num_freqs
    x = reflectivity(n, 5000, 8.0, seed=11)
    y, t_fwd = timed(lambda: plan.forward(x))
    img, t_adj = timed(lambda: plan.adjoint(y))
    y_host = y.cpu().pin_memory()
    img_s, t_stream = timed(lambda: plan.adjoint_streamed(y_host, block=512))
    units = float(n) * n * S
    print(f"scale: forward {t_fwd:.3f} s ({units / t_fwd:.3e} px*pulse/s), backprojection {t_adj:.3f} s "
          f"({units / t_adj:.3e}), streamed from pinned host in 512-pulse blocks {t_stream:.3f} s "
          f"({units / t_stream:.3e})")
    # two FP32 summation orders of 16384 pulses (per-pulse-pair accumulators, blocks added into the
    # image when streamed), each ~2e-6 from the FP64 oracle below
    assert float(torch.linalg.vector_norm(img_s - img) / torch.linalg.vector_norm(img)) < 5e-6
    assert plan.device_flags() == 0

    # 256^2 patch at the scene centre against the FP64 oracle (all pulses).
    pos = np.asarray(scene.positions).reshape(n, n, 3)
    j0 = i0 = n // 2 - 128
    patch = pos[j0:j0 + 256, i0:i0 + 256].reshape(-1, 3)
    yn = y.cpu().numpy()
    prob = oracle.Problem(aperture.transmitter_positions, aperture.receiver_positions, aperture.stab_ref_posns, patch,
                          aperture.centre_frequency, aperture.sample_bandwidth, N, upsample_ratio=upsample)
    ref = oracle.adjoint(prob, yn, mode="linear", threads=oracle.default_threads())
    got = img.reshape(n, n)[j0:j0 + 256, i0:i0 + 256].reshape(-1).cpu().numpy()
    err_adj = rel_l2(got, ref)
    # Forward: 16 pulse rows of the whole image against the oracle.
    rows = np.linspace(0, S - 1, 16).round().astype(int)
    prob_f = oracle.Problem(aperture.transmitter_positions[rows], aperture.receiver_positions[rows],
                            aperture.stab_ref_posns[rows], np.asarray(scene.positions), aperture.centre_frequency,
                            aperture.sample_bandwidth, N, upsample_ratio=upsample)
    ref_f = oracle.forward(prob_f, x.cpu().numpy(), mode="linear", threads=oracle.default_threads())
    err_fwd = rel_l2(yn[rows], ref_f)
    print(f"scale: FP64-oracle relative L2, backprojection 256^2 patch {err_adj:.2e}, forward 16 rows {err_fwd:.2e}")
    assert err_adj < 1e-5 and err_fwd < 1e-5
