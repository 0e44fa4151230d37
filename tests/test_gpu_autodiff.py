"""Differentiable operator and the phase-error (autofocus) gradient on the GPU.

Checks, after the pattern of the operator parity tests:
  * the autograd backward of y = A x is the backprojection kernel (exact same output), equals the
    FP64 oracle's adjoint in linear mode (relative L2 1e-5) and the reference adjoint's golden
    output in nearest_ref mode;
  * the backward of x = A^H y is the forward kernel;
  * central finite differences of a least-squares loss (h = 1e-3) against the autograd gradient;
  * the sharpness gradient dS/dphi against central finite differences (h = 1e-3) and against the
    same gradient computed by the FP64 oracle, on the 1024^2 x 2048 pulses x 2048 samples workload
    with random-walk phase errors of 0.3 rad step standard deviation;
  * sharpness autofocus increases the sharpness and removes most of a smooth phase error.
"""
import numpy as np
import pytest
import torch

import oracle
from cases import Case, crandn, load_golden, rel_l2, spotlight_case
from sarsolver_gb300 import SarPlan
from sarsolver_gb300.autodiff import (PhaseErrorSharpness, phase_weights, sar_backproject, sar_forward,
                                      sharpness, sharpness_autofocus, sharpness_gradient)
from sarsolver_gb300.scenes import config_workload, reflectivity

pytestmark = pytest.mark.gpu

H = 1.0e-3


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def small_case():
    return spotlight_case(num_pulses=96, num_freqs=256, n=64, spacing=0.5, aperture_deg=3.0)


def test_forward_function_backward_is_adjoint():
    case = small_case()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    rng = np.random.default_rng(1)
    x = torch.from_numpy(crandn(rng, plan.num_scatterers).astype(np.complex64)).cuda().requires_grad_(True)
    v = torch.from_numpy(crandn(rng, plan.num_slow_times, plan.num_freqs).astype(np.complex64)).cuda()
    y = sar_forward(plan, x)
    assert torch.equal(y.detach(), plan.forward(x.detach()))
    (v.conj() * y).sum().real.backward()
    direct = plan.adjoint(v)
    assert torch.equal(x.grad, direct)
    ref = oracle.adjoint(case.problem(), v.cpu().numpy(), mode="linear", threads=oracle.default_threads())
    assert rel_l2(x.grad.cpu().numpy(), ref) < 1.0e-5


def test_forward_function_backward_matches_reference_adjoint():
    """nearest_ref mode: the backward is the reference's adjoint (golden output of the reference
    kernel on the same y), on the per-pixel double-float path."""
    case = load_golden("spot_small")
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="nearest_ref")
    x = torch.zeros(plan.num_scatterers, dtype=torch.complex64, device="cuda", requires_grad=True)
    yg = torch.from_numpy(case.data["y"].astype(np.complex64)).cuda()
    (yg.conj() * sar_forward(plan, x)).sum().real.backward()
    assert rel_l2(x.grad.cpu().numpy(), case.data["adjoint"]) < 1.0e-5


def test_backproject_function_backward_is_forward():
    case = small_case()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    rng = np.random.default_rng(2)
    y = torch.from_numpy(crandn(rng, plan.num_slow_times, plan.num_freqs).astype(np.complex64)).cuda()
    y.requires_grad_(True)
    u = torch.from_numpy(crandn(rng, plan.num_scatterers).astype(np.complex64)).cuda()
    (u.conj() * sar_backproject(plan, y)).sum().real.backward()
    assert torch.equal(y.grad, plan.forward(u))


def test_least_squares_finite_difference():
    """L(x) = ||A x - y||^2 (summed in FP64): (L(x+hd) - L(x-hd)) / 2h = Re<grad, d>."""
    case = small_case()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    rng = np.random.default_rng(3)
    x0 = torch.from_numpy(crandn(rng, plan.num_scatterers).astype(np.complex64)).cuda()
    y = torch.from_numpy(crandn(rng, plan.num_slow_times, plan.num_freqs).astype(np.complex64)).cuda()

    def loss(x):
        r = sar_forward(plan, x) - y
        return (r.real.double() ** 2 + r.imag.double() ** 2).sum()

    x = x0.clone().requires_grad_(True)
    loss(x).backward()
    for seed in range(3):
        d = torch.from_numpy(crandn(np.random.default_rng(10 + seed), plan.num_scatterers).astype(np.complex64)).cuda()
        with torch.no_grad():
            fd = (loss(x0 + H * d) - loss(x0 - H * d)) / (2 * H)
        an = (x.grad.conj() * d).sum().real.double()
        assert abs(float(fd - an)) <= 1.0e-3 * abs(float(an)) + 1e-6 * float(loss(x0).detach())


# ------------------------------------------------------------------------- sharpness gradient

def _phase_error_data(plan, x, phi_err):
    """y = A_{exp(i phi_err)} x, then the plan's weighting back to its own."""
    plan.set_slow_time_weighting(phase_weights(plan, phi_err))
    y = plan.forward(x)
    plan.set_slow_time_weighting(plan.base_weights)
    return y


def _fd_pulse_isolated(plan, y, phi, img, pulses, h=H):
    """Central differences of S(phi) = sum |I|^4 in FP64 along e_s, from the GPU image I and
    pulse s's own contribution C_s = A_phi^H (y restricted to pulse s): I(phi + t e_s) =
    I + (exp(-i t) - 1) C_s exactly, since pulse s enters I through conj(w_s) only."""
    plan.set_slow_time_weighting(phase_weights(plan, phi))
    I = img.to(torch.complex128)
    out = []
    for s in pulses:
        ys = torch.zeros_like(y)
        ys[s] = y[s]
        Cs = plan.adjoint(ys).to(torch.complex128)
        sp = (I + complex(np.exp(-1j * h) - 1.0) * Cs).abs().pow(4).sum()
        sm = (I + complex(np.exp(1j * h) - 1.0) * Cs).abs().pow(4).sum()
        out.append(float((sp - sm) / (2 * h)))
    return np.array(out)


def _oracle_gradient(case, y, phi, pulses, threads):
    """FP64 oracle: I = A_phi^H y over all pulses, G = |I|^2 I, then (A_phi G) on the listed
    pulses only and g_s = 4 Im sum_f conj((A_phi G)_{s,f}) y_{s,f}."""
    prob = case.problem()
    w = np.asarray(case.aperture.slow_time_weighting, np.complex128) * np.exp(1j * np.asarray(phi, np.float64))
    prob.slow_time_weighting = w
    yn = y.cpu().numpy().astype(np.complex128)
    I = oracle.adjoint(prob, yn, mode="linear", threads=threads)
    G = np.abs(I) ** 2 * I
    sub = oracle.Problem(tx=prob.tx[pulses], rx=prob.rx[pulses], srp=prob.srp[pulses], positions=prob.positions,
                         centre_frequency=prob.centre_frequency, sample_frequency=prob.sample_frequency,
                         num_freqs=prob.num_freqs, waveform_fft=prob.waveform_fft, slow_time_weighting=w[pulses],
                         c_eff=prob.c_eff, sign_multiplier=prob.sign_multiplier, upsample_ratio=prob.upsample_ratio)
    ag = oracle.forward(sub, G, mode="linear", threads=threads)
    return 4.0 * np.imag((np.conj(ag) * yn[pulses]).sum(axis=1)), float((np.abs(I) ** 4).sum())


def _random_walk(S, std, seed):
    return np.cumsum(np.random.default_rng(seed).standard_normal(S) * std).astype(np.float32)


def test_sharpness_kernel_matches_torch():
    rng = np.random.default_rng(4)
    case = small_case()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    for P in (1, 7, 4096, 100001):
        img = torch.from_numpy(crandn(rng, P).astype(np.complex64)).cuda()
        tot, G = sharpness(plan, img)
        ref = img.to(torch.complex128)
        assert abs(float(tot) - float(ref.abs().pow(4).sum())) <= 1e-6 * float(ref.abs().pow(4).sum())
        assert rel_l2(G.cpu().numpy(), (ref.abs() ** 2 * ref).cpu().numpy()) < 1e-6


def test_sharpness_gradient_small_vs_oracle_and_fd():
    case = small_case()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    S = plan.num_slow_times
    x = reflectivity(64, 10, 2.0, seed=5)
    y = _phase_error_data(plan, x, torch.from_numpy(_random_walk(S, 0.3, 6)).cuda())
    phi = torch.zeros(S, device="cuda")
    total, g, img = sharpness_gradient(plan, y, phi)
    g = g.cpu().numpy().astype(np.float64)
    pulses = np.arange(S)
    go, so = _oracle_gradient(case, y, phi.cpu().numpy(), pulses, oracle.default_threads())
    assert abs(float(total) - so) < 1e-5 * so
    assert rel_l2(g, go) < 1e-4
    fd = _fd_pulse_isolated(plan, y, phi, img, pulses[::8])
    assert np.max(np.abs(g[::8] - fd)) < 1e-4 * np.max(np.abs(fd))


def test_sharpness_gradient_config3():
    """1024^2 image, 2048 pulses x 2048 samples, U = 8; phase errors a random walk with 0.3 rad
    step std; gradient at phi = 0 and at a half correction."""
    aperture, scene, upsample, _ = config_workload("config3")
    case = Case(scene, aperture, upsample, {})
    plan = SarPlan(scene, aperture, upsample_ratio=upsample, interp="linear")
    S = plan.num_slow_times
    x = reflectivity(1024, 500, 8.0, seed=7)
    phi_err = torch.from_numpy(_random_walk(S, 0.3, 8)).cuda()
    y = _phase_error_data(plan, x, phi_err)
    rng = np.random.default_rng(9)
    pulses = np.sort(rng.choice(S, 24, replace=False))
    threads = oracle.default_threads()
    for phi in (torch.zeros(S, device="cuda"), 0.5 * phi_err):
        total, g, img = sharpness_gradient(plan, y, phi)
        g = g.cpu().numpy().astype(np.float64)
        scale = np.max(np.abs(g))
        fd = _fd_pulse_isolated(plan, y, phi, img, pulses)
        assert np.max(np.abs(g[pulses] - fd)) < 1e-3 * scale
        go, so = _oracle_gradient(case, y, phi.cpu().numpy(), pulses, threads)
        assert abs(float(total) - so) < 1e-4 * so
        assert np.max(np.abs(g[pulses] - go)) < 1e-3 * scale
        # Direct central differences through two full backprojections per pulse (FP32 images,
        # FP64 sums): looser, the FP32 rounding of the two images does not cancel exactly.
        for s in pulses[:4]:
            e = torch.zeros(S, device="cuda")
            e[s] = H
            sp, _, _ = sharpness_gradient(plan, y, phi + e, want_grad=False)
            sm, _, _ = sharpness_gradient(plan, y, phi - e, want_grad=False)
            assert abs(float((sp - sm) / (2 * H)) - g[s]) < 2e-2 * scale
    assert plan.device_flags() == 0


def test_phase_error_sharpness_autograd():
    case = small_case()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    S = plan.num_slow_times
    x = reflectivity(64, 10, 2.0, seed=11)
    y = _phase_error_data(plan, x, torch.from_numpy(_random_walk(S, 0.1, 12)).cuda())
    phi = torch.zeros(S, device="cuda", requires_grad=True)
    total = PhaseErrorSharpness.apply(phi, y, plan)
    (2.0 * total).backward()
    _, g, _ = sharpness_gradient(plan, y, phi.detach())
    assert torch.allclose(phi.grad, 2.0 * g)


def test_sharpness_autofocus_recovers_smooth_phase_error():
    case = spotlight_case(num_pulses=128, num_freqs=256, n=64, spacing=0.5, aperture_deg=3.0)
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    S = plan.num_slow_times
    x = reflectivity(64, 12, 2.0, seed=13, clutter_level=0.05)
    t = np.linspace(-1.0, 1.0, S)
    phi_err = (1.5 * t ** 2 + 0.8 * np.sin(3.0 * t)).astype(np.float32)
    y = _phase_error_data(plan, x, torch.from_numpy(phi_err).cuda())

    def detrended(p):
        p = np.asarray(p, np.float64)
        return p - np.polyval(np.polyfit(t, p, 1), t)

    phi, hist = sharpness_autofocus(plan, y, iterations=60, lr=0.05)
    assert hist[-1] > 1.2 * hist[0]
    before = np.sqrt(np.mean(detrended(phi_err) ** 2))
    after = np.sqrt(np.mean(detrended(phi_err - phi.cpu().numpy()) ** 2))
    assert after < 0.5 * before
    assert plan.device_flags() == 0


def test_lazy_conjugate_gradients_are_materialised():
    """Autograd passes lazily conjugated views to backward; the kernels must see the values."""
    case = small_case()
    plan = SarPlan(case.scene, case.aperture, upsample_ratio=case.upsample_ratio, interp="linear")
    rng = np.random.default_rng(21)
    x = torch.from_numpy(crandn(rng, plan.num_scatterers).astype(np.complex64)).cuda().requires_grad_(True)
    v = torch.from_numpy(crandn(rng, plan.num_slow_times, plan.num_freqs).astype(np.complex64)).cuda()
    (sar_forward(plan, x).conj() * v).sum().real.backward()      # grad_y arrives as a conj view
    assert torch.allclose(x.grad, plan.adjoint(v), rtol=1e-6, atol=0)
    assert torch.equal(plan.adjoint(v.conj()), plan.adjoint(v.conj().resolve_conj()))
