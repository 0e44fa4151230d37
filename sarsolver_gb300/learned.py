"""Learned CGLS warm start: a U-Net trained through the operator's own kernels.

The warm start for ``min ||A x - y||`` is

    x0 = c * (b + s * U(b / s)),   b = A^H y,   s = rms(b),   c = ||b||^2 / ||A b||^2,

i.e. the optimal single steepest-descent step ``c b`` plus a learned correction; ``U`` is the bf16
U-Net (``unet.UNet``).  It is trained on scenes the operator itself generates (point scatterers
plus speckled smooth clutter, complex white noise at 10-30 dB SNR, aperture extent drawn per scene
in [2, 6] degrees) with the loss the CGLS stopping rule uses,

    L = ||A^H (y - A x0)||^2 / ||A^H y||^2,

differentiated through ``SarForwardFunction`` / ``SarBackprojectFunction`` (forward projection and
backprojection kernels) into the U-Net's own backward pass.  Plain CGLS from zero is the baseline;
``compare`` times both to the same normal-equations residual.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import torch

from .autodiff import sar_backproject, sar_forward
from .plan import SarPlan
from .scenes import add_noise, grid_scene, reflectivity, spotlight_aperture
from .solvers import cgls
from .unet import UNet, UNetFunction


@dataclass
class LearnedConfig:
    """The learned-CGLS workload: 512^2 image at 0.25 m, 1024 pulses x 1024 samples, U = 8."""
    n: int = 512
    spacing: float = 0.25
    num_pulses: int = 1024
    num_freqs: int = 1024
    upsample: float = 8.0
    aperture_min: float = 2.0
    aperture_max: float = 6.0
    aperture_step: float = 0.25      # training plans are cached on this grid of extents
    snr_min: float = 10.0
    snr_max: float = 30.0
    points_min: int = 20
    points_max: int = 400
    sigma_px: float = 4.0


class SceneSource:
    """Seeded scenes and measurements generated on the GPU by the operator."""

    def __init__(self, cfg: LearnedConfig, seed: int, device=None, continuous: bool = False):
        self.cfg = cfg
        self.device = torch.device("cuda") if device is None else torch.device(device)
        self.rng = np.random.default_rng(seed)
        self.gen = torch.Generator(device=self.device)
        self.gen.manual_seed(seed)
        self.continuous = continuous
        self.plans: Dict[float, SarPlan] = {}
        self.scene = grid_scene(cfg.n, cfg.spacing)

    def plan_for(self, extent: float) -> SarPlan:
        if extent not in self.plans:
            c = self.cfg
            ap = spotlight_aperture(c.num_pulses, c.num_freqs, extent)
            self.plans[extent] = SarPlan(self.scene, ap, upsample_ratio=c.upsample, interp="linear", device=self.device)
        return self.plans[extent]

    def sample(self):
        """(plan, y, x_true, extent, snr_db)."""
        c = self.cfg
        extent = float(self.rng.uniform(c.aperture_min, c.aperture_max))
        if not self.continuous:
            extent = round(extent / c.aperture_step) * c.aperture_step
        plan = self.plan_for(extent)
        num_points = int(self.rng.integers(c.points_min, c.points_max + 1))
        clutter = float(self.rng.uniform(0.1, 0.6))
        x = reflectivity(c.n, num_points, c.sigma_px, seed=0, device=self.device, clutter_level=clutter, gen=self.gen)
        snr = float(self.rng.uniform(c.snr_min, c.snr_max))
        y = add_noise(plan.forward(x), snr, seed=0, gen=self.gen)
        return plan, y, x, extent, snr

    def close(self):
        for p in self.plans.values():
            p.close()
        self.plans.clear()


class WarmStart:
    """``x0 = c (b + s U(b / s))`` with the U-Net ``net``."""

    def __init__(self, net: UNet, n: int):
        self.net = net
        self.n = n
        self.anchor = torch.zeros((), device=net.device, requires_grad=True)

    def _terms(self, plan: SarPlan, y: torch.Tensor):
        b = plan.adjoint(y)
        bb = torch.linalg.vector_norm(b) ** 2
        c = bb / (torch.linalg.vector_norm(plan.forward(b)) ** 2).clamp_min(1e-30)
        s = torch.sqrt(bb / b.numel()).clamp_min(1e-30)
        return b, bb, c, s

    @torch.no_grad()
    def __call__(self, plan: SarPlan, y: torch.Tensor) -> torch.Tensor:
        b, _, c, s = self._terms(plan, y)
        u = self.net.forward(b.view(1, self.n, self.n), float(1.0 / s)).reshape(-1)
        return c * (b + s * u)

    @torch.no_grad()
    def direction(self, b: torch.Tensor) -> torch.Tensor:
        """``b + s U(b / s)`` for ``b = A^H y`` (the warm start up to its scalar ``c``)."""
        s = float(torch.sqrt((b.real.square() + b.imag.square()).mean()).clamp_min(1e-30))
        return b + s * self.net.forward(b.view(1, self.n, self.n), 1.0 / s).reshape(-1)

    @torch.no_grad()
    def solve(self, plan: SarPlan, y: torch.Tensor, tol: float = 1e-3, max_iterations: int = 1000):
        """CGLS from the learned warm start with no repeated operator work: ``b = A^H y`` is formed
        once (network input and CGLS's own ``A^H y``), and the scalar ``c`` is fitted by the solver's
        scaled start from the same ``A z`` it needs for the initial residual."""
        b = plan.adjoint(y)
        return cgls(plan, y, x0=self.direction(b), tol=tol, max_iterations=max_iterations, start="scaled", ahy=b)

    def loss(self, plan: SarPlan, y: torch.Tensor, x_true: Optional[torch.Tensor] = None,
             kind: str = "normal") -> torch.Tensor:
        """Training loss of the warm start, differentiable in U.

        ``normal``: the normal-equations residual ||A^H (y - A x0)||^2 / ||A^H y||^2 of x0 = c z,
        z = b + s U(b / s) (weights the error by the squared singular values, so it favours the
        components CGLS settles in its first iterations anyway).  ``data``: 1 - cos^2 of the angle
        between A z and y (real scale), i.e. the data residual ||y - c A z||^2 / ||y||^2 at the
        solver's best real c -- the starting error CGLS minimises, in the A-norm.  ``truth``: the
        same against the noise-free data A x_true (needs ``x_true``): z should predict the scene."""
        if kind in ("data", "truth"):
            with torch.no_grad():
                b = plan.adjoint(y)
                s = torch.sqrt((b.real.square() + b.imag.square()).mean()).clamp_min(1e-30)
                t = y if kind == "data" else plan.forward(x_true)
            u = _UNetApply.apply(b.view(1, self.n, self.n), self.net, float(1.0 / s), self.anchor).reshape(-1)
            az = sar_forward(plan, b + s * u)
            re = (az.real.double() * t.real.double() + az.imag.double() * t.imag.double()).sum()
            aa = (az.real.double() ** 2 + az.imag.double() ** 2).sum()
            tt = (t.real.double() ** 2 + t.imag.double() ** 2).sum()
            return 1.0 - re * re / (aa * tt).clamp_min(1e-300)
        if kind != "normal":
            raise ValueError(f"unknown loss {kind!r}")
        with torch.no_grad():
            b, bb, c, s = self._terms(plan, y)
        u = _UNetApply.apply(b.view(1, self.n, self.n), self.net, float(1.0 / s), self.anchor).reshape(-1)
        x0 = c * (b + s * u)
        r = y - sar_forward(plan, x0)
        g = sar_backproject(plan, r)
        return (g.real.double() ** 2 + g.imag.double() ** 2).sum() / bb.double()


class _UNetApply(torch.autograd.Function):
    """U-Net forward whose output joins the autograd graph through ``anchor`` (the parameters
    live inside the native object; backward accumulates their gradients there)."""

    @staticmethod
    def forward(ctx, x, net, in_scale, anchor):
        ctx.net = net
        return net.forward(x, in_scale)

    @staticmethod
    def backward(ctx, grad_out):
        ctx.net.backward(grad_out)
        return None, None, None, None


class LearnedPreconditioner:
    """Nonlinear preconditioner ``N(s) = s + sigma U(s / sigma)`` (sigma = rms(s)) for the normal
    equations, trained so that ``A^H A N(s)`` points along ``s`` (an approximate inverse of A^H A up
    to scale) on the residual vectors the solver meets."""

    def __init__(self, net: UNet, n: int):
        self.net = net
        self.n = n
        self.anchor = torch.zeros((), device=net.device, requires_grad=True)

    @torch.no_grad()
    def __call__(self, s: torch.Tensor) -> torch.Tensor:
        sig = float(torch.sqrt((s.real.square() + s.imag.square()).mean()).clamp_min(1e-30))
        u = self.net.forward(s.view(1, self.n, self.n), 1.0 / sig).reshape(-1)
        return s + sig * u

    def chain_loss(self, plan: SarPlan, s: torch.Tensor):
        """(loss, next residual): loss = 1 - cos^2(angle(A^H A N(s), s)); the next residual is
        s - a A^H A N(s) with the step a minimising its norm (a detached Richardson step)."""
        sig = float(torch.sqrt((s.real.square() + s.imag.square()).mean()).clamp_min(1e-30))
        u = _UNetApply.apply(s.view(1, self.n, self.n), self.net, 1.0 / sig, self.anchor).reshape(-1)
        z = s + sig * u
        g = sar_backproject(plan, sar_forward(plan, z))
        gs = (g.conj() * s).sum().real.double()
        gg = (g.real.double().square() + g.imag.double().square()).sum()
        ss = (s.real.double().square() + s.imag.double().square()).sum()
        loss = 1.0 - gs * gs / (gg * ss)
        with torch.no_grad():
            a = (gs / gg).float()
            nxt = s - a * g.detach()
        return loss, nxt


def fcg(plan: SarPlan, y: torch.Tensor, precond=None, x0: Optional[torch.Tensor] = None, tol: float = 1e-3,
        max_iterations: int = 500):
    """Flexible preconditioned CG on the normal equations (CGLS form): directions from
    ``z = precond(s)`` with the Polak-Ribiere beta, exact line search on ||y - A x||.  Stops at
    ||A^H (y - A x)|| / ||A^H y|| <= tol.  Returns (x, iterations, history)."""
    norm = lambda v: float(torch.linalg.vector_norm(v))
    dot = lambda a, b: float((a.conj() * b).sum().real)
    b = plan.adjoint(y)
    nb = norm(b)
    if x0 is None:
        x = torch.zeros_like(b)
        r = y.clone()
        s = b
    else:
        x = x0.clone()
        r = y - plan.forward(x)
        s = plan.adjoint(r)
    hist = [norm(s) / nb if nb > 0 else 0.0]
    if hist[-1] <= tol:
        return x, 0, hist
    z = precond(s) if precond else s
    p = z
    zs = dot(z, s)
    for it in range(1, max_iterations + 1):
        q = plan.forward(p)
        alpha = dot(p, s) / max(dot(q, q), 1e-300)
        x = x + alpha * p
        r = r - alpha * q
        s_new = plan.adjoint(r)
        hist.append(norm(s_new) / nb)
        if hist[-1] <= tol:
            return x, it, hist
        z_new = precond(s_new) if precond else s_new
        beta = max(0.0, dot(z_new, s_new - s) / max(zs, 1e-300))
        p = z_new + beta * p
        s, z = s_new, z_new
        zs = dot(z, s)
    return x, max_iterations, hist


def train_preconditioner(net: UNet, source: SceneSource, scenes: int, chain: int = 3, batch: int = 8,
                         lr: float = 1e-3, log_every: int = 50, printer=None) -> TrainLog:
    """Adam on the mean chain loss: for each scene the residuals s_0 = A^H y, s_1, ... s_{chain-1}
    of preconditioned Richardson steps with the current network, each a training input."""
    pre = LearnedPreconditioner(net, source.cfg.n)
    steps = max(1, scenes // batch)
    log = TrainLog()
    t0 = time.time()
    running = []
    for step in range(steps):
        net.zero_grad()
        for _ in range(batch):
            plan, y, _, _, _ = source.sample()
            s = plan.adjoint(y)
            for _k in range(chain):
                L, s = pre.chain_loss(plan, s)
                (L / (batch * chain)).backward()
                running.append(float(L.detach()))
        rate = lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * step / steps)))
        net.adam_step(rate)
        if (step + 1) % log_every == 0 or step == steps - 1:
            log.steps.append(step + 1)
            log.loss.append(float(np.mean(running)))
            if printer:
                printer(f"step {step + 1}/{steps} scenes {(step + 1) * batch} loss {np.mean(running):.4e} "
                        f"lr {rate:.2e} {time.time() - t0:.1f}s")
            running = []
    torch.cuda.synchronize()
    log.scenes = steps * batch
    log.seconds = time.time() - t0
    return log


@dataclass
class TrainLog:
    steps: List[int] = field(default_factory=list)
    loss: List[float] = field(default_factory=list)
    scenes: int = 0
    seconds: float = 0.0


def train(net: UNet, source: SceneSource, scenes: int, batch: int = 8, lr: float = 1e-3, log_every: int = 50,
          warm: Optional[WarmStart] = None, printer=None, loss: str = "normal") -> TrainLog:
    """Adam on the mean warm-start loss (``WarmStart.loss`` of kind ``loss``) over mini-batches of
    generated scenes; cosine learning rate decay to lr / 20."""
    warm = warm or WarmStart(net, source.cfg.n)
    steps = max(1, scenes // batch)
    log = TrainLog()
    t0 = time.time()
    running = []
    for step in range(steps):
        net.zero_grad()
        for _ in range(batch):
            plan, y, x_true, _, _ = source.sample()
            L = warm.loss(plan, y, x_true, kind=loss)
            (L / batch).backward()
            running.append(float(L.detach()))
        rate = lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * step / steps)))
        net.adam_step(rate)
        if (step + 1) % log_every == 0 or step == steps - 1:
            log.steps.append(step + 1)
            log.loss.append(float(np.mean(running)))
            if printer:
                printer(f"step {step + 1}/{steps} scenes {(step + 1) * batch} loss {np.mean(running):.4e} "
                        f"lr {rate:.2e} {time.time() - t0:.1f}s")
            running = []
    torch.cuda.synchronize()
    log.scenes = steps * batch
    log.seconds = time.time() - t0
    return log


@dataclass
class SolveRecord:
    extent: float
    snr_db: float
    plain_iterations: int
    plain_ms: float
    learned_iterations: int
    learned_ms: float
    start_residual: float       # ||A^H (y - A x0)|| / ||A^H y|| of the warm start
    plain_converged: bool
    learned_converged: bool
    # ceiling of any scene-predicting warm start: CGLS started at the true scene (a perfect
    # prior over scenes; the least-squares solution it must still reach also fits the noise)
    truth_iterations: int = 0
    truth_ms: float = float("nan")
    truth_start_residual: float = float("nan")


def _timed(fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, 1e3 * (time.perf_counter() - t0)


def compare(warm: WarmStart, source: SceneSource, count: int, tol: float = 1e-3, max_iterations: int = 1000,
            repeats: int = 1, truth: bool = False) -> List[SolveRecord]:
    """Plain CGLS from zero vs CGLS from the learned warm start, both to ``tol`` in the
    normal-equations residual; times are wall clock around the whole solve (the warm start's
    backprojection, network and the CGLS iterations), best of ``repeats``.  With ``truth`` also
    CGLS started at the true scene (given start, no network), the ceiling of any warm start that
    predicts the scene."""
    out = []
    for _ in range(count):
        plan, y, x_true, extent, snr = source.sample()
        best_plain = best_learned = best_truth = float("inf")
        it = None
        for _ in range(repeats):
            if truth:
                (xt, it), tt = _timed(lambda: cgls(plan, y, x0=x_true, tol=tol, max_iterations=max_iterations))
                best_truth = min(best_truth, tt)
            (xp, ip), tp = _timed(lambda: cgls(plan, y, tol=tol, max_iterations=max_iterations))
            best_plain = min(best_plain, tp)

            def learned():
                return warm.solve(plan, y, tol=tol, max_iterations=max_iterations)

            (xl, il), tl = _timed(learned)
            best_learned = min(best_learned, tl)
        rec = SolveRecord(extent, snr, ip.iterations, best_plain, il.iterations, best_learned,
                          il.history[0] if il.history else float("nan"), ip.converged, il.converged)
        if it is not None:
            rec.truth_iterations, rec.truth_ms = it.iterations, best_truth
            rec.truth_start_residual = it.history[0] if it.history else float("nan")
        out.append(rec)
    return out
