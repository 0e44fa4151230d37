"""GPU CGLS (native driver + fused vector kernels) against a CGLS run on the FP64 oracle.

The reference runs CIL's CGLS on its operator (tests/test_cil.py:18-22); CIL is not available,
so the same recurrence is written here in numpy on the oracle's linear-mode operator pair and
the GPU iterates are compared with it step by step.  The stopping rule is the normal-equations
residual ||A^H (y - A x)|| / ||A^H y||.
"""
import numpy as np
import pytest
import torch

import oracle
from cases import crandn, rel_l2, spotlight_case
from sarsolver_gb300 import SarPlan, _lib
from sarsolver_gb300.solvers import cgls

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def numpy_cgls(prob, y, iterations, threads):
    fwd = lambda v: oracle.forward(prob, v, mode="linear", threads=threads)
    adj = lambda v: oracle.adjoint(prob, v, mode="linear", threads=threads)
    x = np.zeros(prob.num_scatterers, np.complex128)
    r = y.copy()
    s = adj(r)
    norm0 = np.linalg.norm(s)
    p = s.copy()
    gamma = np.vdot(s, s).real
    hist = [np.sqrt(gamma) / norm0]
    for _ in range(iterations):
        q = fwd(p)
        alpha = gamma / np.vdot(q, q).real
        x += alpha * p
        r -= alpha * q
        s = adj(r)
        gnew = np.vdot(s, s).real
        hist.append(np.sqrt(gnew) / norm0)
        p = s + (gnew / gamma) * p
        gamma = gnew
    return x, np.array(hist)


def noisy_case(seed=0, snr_db=20.0):
    case = spotlight_case(num_pulses=64, num_freqs=128, n=48, spacing=0.5, aperture_deg=4.0)
    rng = np.random.default_rng(seed)
    prob = case.problem()
    x_true = np.zeros(prob.num_scatterers, np.complex128)
    idx = rng.choice(prob.num_scatterers, 12, replace=False)
    x_true[idx] = crandn(rng, 12)
    y = oracle.forward(prob, x_true, mode="linear", threads=oracle.default_threads())
    sigma = np.sqrt(np.mean(np.abs(y) ** 2) / 10 ** (snr_db / 10))
    y = y + sigma * crandn(rng, *y.shape)
    return case, prob, y


def test_cgls_iterates_match_oracle_cgls():
    case, prob, y = noisy_case()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    k = 8
    x, info = cgls(plan, torch.from_numpy(y.astype(np.complex64)), tol=0.0, max_iterations=k)
    xo, ho = numpy_cgls(prob, y, k, oracle.default_threads())
    assert info.iterations == k and not info.converged and not info.breakdown
    assert rel_l2(x.cpu().numpy(), xo) < 1e-3
    np.testing.assert_allclose(info.history, ho, rtol=1e-3)


def test_cgls_reaches_tolerance():
    case, prob, y = noisy_case(seed=1)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    yt = torch.from_numpy(y.astype(np.complex64)).cuda()
    x, info = cgls(plan, yt, tol=1e-3, max_iterations=300)
    assert info.converged and info.residual <= 1e-3
    # The recursively updated residual agrees with the directly recomputed one.
    direct = torch.linalg.vector_norm(plan.adjoint(yt - plan.forward(x))) / torch.linalg.vector_norm(plan.adjoint(yt))
    assert float(direct) < 2e-3
    # Warm start at the solution: done before the first iteration.
    x2, info2 = cgls(plan, yt, x0=x, tol=2e-3, max_iterations=300)
    assert info2.converged and info2.iterations == 0
    assert torch.equal(x2, x)
    assert plan.device_flags() == 0


def test_cgls_zero_data_and_zero_operator():
    case, prob, y = noisy_case(seed=2)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    x, info = cgls(plan, torch.zeros(y.shape, dtype=torch.complex64), tol=1e-3, max_iterations=10)
    assert info.converged and info.iterations == 0 and info.residual == 0.0
    assert float(x.abs().max()) == 0.0
    plan.set_slow_time_weighting(np.zeros(plan.num_slow_times, np.complex128))   # A = 0
    x, info = cgls(plan, torch.from_numpy(y.astype(np.complex64)), tol=1e-3, max_iterations=10)
    assert info.converged and info.iterations == 0 and info.norm_ahy == 0.0


def test_cgls_rejects_non_finite_data():
    case, prob, y = noisy_case(seed=3)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    bad = y.astype(np.complex64)
    bad[3, 5] = np.nan
    with pytest.raises(_lib.SarError) as err:
        cgls(plan, torch.from_numpy(bad), tol=1e-3, max_iterations=10)
    assert err.value.status == _lib.SAR_ERR_INVALID_ARGUMENT
    # The plan stays usable.
    x, info = cgls(plan, torch.from_numpy(y.astype(np.complex64)), tol=1e-2, max_iterations=50)
    assert info.converged


def test_cgls_scaled_start_and_precomputed_ahy():
    case, prob, y = noisy_case(seed=4)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    yt = torch.from_numpy(y.astype(np.complex64)).cuda()
    b = plan.adjoint(yt)
    z = 3.7 * b   # a direction of arbitrary scale
    _, given = cgls(plan, yt, x0=z, tol=1e-3, max_iterations=300)
    xs, scaled = cgls(plan, yt, x0=z, tol=1e-3, max_iterations=300, start="scaled")
    xs2, scaled2 = cgls(plan, yt, x0=z, tol=1e-3, max_iterations=300, start="scaled", ahy=b)
    # The scaled start is the best multiple of z: its residual is that of one steepest-descent step.
    _, plain = cgls(plan, yt, tol=0.0, max_iterations=1)
    assert scaled.history[0] < given.history[0]
    assert abs(scaled.history[0] - plain.history[1]) < 1e-3 * plain.history[1] + 1e-6
    assert scaled.converged and scaled2.converged and scaled2.iterations == scaled.iterations
    assert float((xs - xs2).abs().max()) <= 1e-6 * float(xs.abs().max())
