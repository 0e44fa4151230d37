"""The headline configuration against the FP64 oracle, on exactly the path its throughput is quoted on.

2048^2 pixels at 0.25 m, 4096 pulses x 4096 samples, upsample 8, 5 deg circular spotlight
(the benchmark workload): the fused N = 4096 upsampling, the 96-bin look-direction tile windows,
two CTAs per tile, linear interpolation.  The oracle (FP64 C restatement of
sarsolver_cxx.cpp:271-353, bit-identical to the reference kernel where that compiles) runs on

  * a 256^2 pixel patch at the scene centre over all 4096 pulses (backprojection: the exact pixel
    subset, so every gathered pulse is checked), and
  * 16 pulse rows spread over the aperture for the whole 2048^2 image (forward projection),

relative L2 <= 1e-5 in both (complex64 against FP64).  The same for the collection turned by
90 deg and looking along the grid diagonal (other gather lane layouts, other windows, the
transposed and two-phase scatter), and for the reference's nearest-bin conventions (split bins
with exact re-decisions near rounding boundaries).  No device check flag may be raised: in
particular SAR_FLAG_GATHER_WINDOW, which the gather's producers raise when a sub-tile's bin extent
could leave its staged window.
"""
import numpy as np
import pytest
import torch

import oracle
from cases import rel_l2
from sarsolver_gb300 import SarPlan
from sarsolver_gb300.scenes import add_noise, config_workload, reflectivity

pytestmark = pytest.mark.gpu

TOL = 1.0e-5
SEED = 20261203


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def patch_rows(n, size=256):
    j0 = i0 = n // 2 - size // 2
    return j0, i0


@pytest.mark.parametrize("case,interp", [("config2", "linear"), ("config2_turned", "linear"),
                                         ("config2_diagonal", "linear"), ("config2", "nearest_ref")])
def test_headline_against_fp64_oracle(case, interp):
    aperture, scene, upsample, _ = config_workload(case)
    n = scene.grid_shape[2]
    S, N = aperture.num_slow_times, aperture.num_freqs
    plan = SarPlan(scene, aperture, upsample_ratio=upsample, interp=interp)
    assert plan.is_grid
    if case == "config2":   # the benchmark path: fused up/downsampling, 96-bin look-direction windows
        assert plan.fused_upsampling and plan.fused_downsampling and plan.tile_window == 96
    x = reflectivity(n, 500, 8.0, SEED)
    y_clean = plan.forward(x)
    y = add_noise(y_clean, 20.0, SEED + 1)
    img = plan.adjoint(y)
    torch.cuda.synchronize()
    assert plan.device_flags() == 0

    threads = oracle.default_threads()
    pos = np.asarray(scene.positions).reshape(n, n, 3)
    j0, i0 = patch_rows(n)
    patch = pos[j0:j0 + 256, i0:i0 + 256].reshape(-1, 3)
    prob = oracle.Problem(aperture.transmitter_positions, aperture.receiver_positions, aperture.stab_ref_posns,
                          patch, aperture.centre_frequency, aperture.sample_bandwidth, N, upsample_ratio=upsample)
    ref = oracle.adjoint(prob, y.cpu().numpy(), mode=interp, threads=threads)
    got = img.reshape(n, n)[j0:j0 + 256, i0:i0 + 256].reshape(-1).cpu().numpy()
    err_adj = rel_l2(got, ref)

    rows = np.linspace(0, S - 1, 16).round().astype(int)
    prob_f = oracle.Problem(aperture.transmitter_positions[rows], aperture.receiver_positions[rows],
                            aperture.stab_ref_posns[rows], np.asarray(scene.positions), aperture.centre_frequency,
                            aperture.sample_bandwidth, N, upsample_ratio=upsample)
    ref_f = oracle.forward(prob_f, x.cpu().numpy(), mode=interp, threads=threads)
    err_fwd = rel_l2(y_clean.cpu().numpy()[rows], ref_f)
    print(f"{case} {interp}: FP64-oracle relative L2, backprojection 256^2 patch x {S} pulses {err_adj:.2e}, "
          f"forward {len(rows)} rows x {n}^2 pixels {err_fwd:.2e}")
    assert err_adj < TOL and err_fwd < TOL
    plan.close()
