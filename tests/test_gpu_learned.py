"""Learned CGLS warm start: the committed trained network against the same method without it.

"Without it" is the untrained path x0 = c * A^H y (the optimal steepest-descent step, network
output zero).  On held-out generated scenes the trained network must give a smaller starting
normal-equations residual, and CGLS from it must still reach 1e-3.  Also: the flexible CG used
with a preconditioner reproduces plain CGLS when the preconditioner is the identity."""
import os

import numpy as np
import pytest
import torch

from sarsolver_gb300.learned import LearnedConfig, SceneSource, WarmStart, fcg
from sarsolver_gb300.solvers import cgls
from sarsolver_gb300.train_warmstart import DEFAULT_WEIGHTS, load_warm_start
from sarsolver_gb300.unet import UNet

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def normal_residual(plan, y, x):
    return float(torch.linalg.vector_norm(plan.adjoint(y - plan.forward(x))) / torch.linalg.vector_norm(plan.adjoint(y)))


@pytest.mark.skipif(not os.path.exists(DEFAULT_WEIGHTS), reason="no trained weights committed")
def test_trained_warm_start_beats_untrained():
    warm, cfg = load_warm_start(DEFAULT_WEIGHTS)
    plain = WarmStart(UNet(32, zero_output=True), cfg.n)      # network output zero: x0 = c A^H y
    src = SceneSource(cfg, seed=777, continuous=True)
    gains = []
    for _ in range(4):
        plan, y, _, _, _ = src.sample()
        r_trained = normal_residual(plan, y, warm(plan, y))
        r_plain = normal_residual(plan, y, plain(plan, y))
        gains.append(r_plain / r_trained)
        x, info = cgls(plan, y, x0=warm(plan, y), tol=1e-3, max_iterations=300)
        assert info.converged
    print("starting-residual gain of the trained network:", [round(g, 3) for g in gains])
    assert np.mean(gains) > 1.2
    assert warm.net.flags() == 0
    src.close()


def test_fcg_identity_matches_cgls():
    cfg = LearnedConfig(n=128, num_pulses=256, num_freqs=256)
    src = SceneSource(cfg, seed=5, continuous=True)
    plan, y, _, _, _ = src.sample()
    _, info = cgls(plan, y, tol=1e-3, max_iterations=300)
    _, it, hist = fcg(plan, y, None, tol=1e-3, max_iterations=300)
    assert abs(it - info.iterations) <= 1
    np.testing.assert_allclose(hist[:5], info.history[:5], rtol=1e-2)
    src.close()
