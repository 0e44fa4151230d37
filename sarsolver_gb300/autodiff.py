"""Differentiable operator pair and the phase-error (autofocus) gradient.

* ``SarForwardFunction``: ``y = A x`` as a ``torch.autograd.Function`` whose backward is the
  backprojection kernel, ``grad_x = A^H grad_y``.  PyTorch's complex autograd passes the
  conjugate-Wirtinger gradient, for which the vector-Jacobian product of a C-linear map is
  exactly ``A^H``; with ``interp="linear"`` the plan's adjoint is the exact transpose of its
  forward, so gradients are exact.  With ``interp="nearest_ref"`` the backward is the reference's
  adjoint (src/sarsolver/cxx_binding/sarsolver_cxx.cpp:319-353), which the reference pairs with
  its forward (:271-310) although the two are not exact transposes.
* ``SarBackprojectFunction``: ``x = A^H y`` with backward ``grad_y = A grad_x``.
* ``sharpness_gradient``: the sharpness ``S(phi) = sum_p |I_p|^4`` of ``I = A_phi^H y`` for
  per-pulse phase errors entering as slow-time weights ``w_s = b_s exp(i phi_s)`` (the hook the
  reference exposes as ``slow_time_weighting``, sarsolver_cxx.cpp:288, :349; ``b_s`` is the
  aperture's own weighting), and its gradient
  ``dS/dphi_s = 4 Im( sum_f conj((A_phi G)_{s,f}) y_{s,f} )`` with ``G = |I|^2 I``:
  one backprojection, one sharpness pass, one forward projection and one row reduction.
* ``PhaseErrorSharpness``: the same as an autograd Function of ``phi``.
* ``sharpness_autofocus``: gradient ascent on ``S`` over ``phi``.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import torch

from . import _lib
from .plan import SarPlan


class SarForwardFunction(torch.autograd.Function):
    """``y = A x`` with ``grad_x = A^H grad_y`` (hand-written backprojection kernel)."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, plan: SarPlan) -> torch.Tensor:
        ctx.plan = plan
        ctx.x_shape = x.shape
        return plan.forward(x)

    @staticmethod
    def backward(ctx, grad_y: torch.Tensor):
        grad_x = None
        if ctx.needs_input_grad[0]:
            grad_x = ctx.plan.adjoint(grad_y).reshape(ctx.x_shape)
        return grad_x, None


class SarBackprojectFunction(torch.autograd.Function):
    """``x = A^H y`` with ``grad_y = A grad_x`` (forward-projection kernel)."""

    @staticmethod
    def forward(ctx, y: torch.Tensor, plan: SarPlan) -> torch.Tensor:
        ctx.plan = plan
        ctx.y_shape = y.shape
        return plan.adjoint(y)

    @staticmethod
    def backward(ctx, grad_x: torch.Tensor):
        grad_y = None
        if ctx.needs_input_grad[0]:
            grad_y = ctx.plan.forward(grad_x).reshape(ctx.y_shape)
        return grad_y, None


def sar_forward(plan: SarPlan, x: torch.Tensor) -> torch.Tensor:
    """Differentiable ``A x`` (complex64 ``[S, N]``)."""
    return SarForwardFunction.apply(x, plan)


def sar_backproject(plan: SarPlan, y: torch.Tensor) -> torch.Tensor:
    """Differentiable ``A^H y`` (complex64 ``[P]``)."""
    return SarBackprojectFunction.apply(y, plan)


# --------------------------------------------------------------------------- autofocus

def _require_linear(plan: SarPlan) -> None:
    if plan.interp != "linear":
        raise ValueError("the phase-error gradient needs an exact adjoint pair: build the plan with interp='linear'")


def sharpness(plan: SarPlan, image: torch.Tensor, want_g: bool = True) -> Tuple[torch.Tensor, Optional[torch.Tensor]]:
    """``(sum |I|^4`` as an FP64 device scalar, ``G = |I|^2 I`` or None) by the sharpness kernel."""
    img = plan._as_input(image, image.numel(), "image")
    total = torch.empty((), dtype=torch.float64, device=plan.device)
    G = torch.empty_like(img) if want_g else None
    with torch.cuda.device(plan.device):
        _lib.check(plan._lib.sar_sharpness(ctypes.c_void_p(img.data_ptr()),
                                           ctypes.c_void_p(G.data_ptr() if G is not None else 0),
                                           ctypes.c_void_p(total.data_ptr()), img.numel(), plan._stream()),
                   "sar_sharpness")
    return total, G


def phase_gradient(plan: SarPlan, ag: torch.Tensor, y: torch.Tensor, scale: float = 4.0) -> torch.Tensor:
    """``g_s = scale * Im(sum_f conj(ag_{s,f}) y_{s,f})``, float32 ``[S]`` (row-reduction kernel)."""
    S, N = plan.num_slow_times, plan.num_freqs
    ag = plan._as_input(ag, S * N, "ag")
    y = plan._as_input(y, S * N, "y")
    g = torch.empty(S, dtype=torch.float32, device=plan.device)
    with torch.cuda.device(plan.device):
        _lib.check(plan._lib.sar_phase_gradient(ctypes.c_void_p(ag.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                                ctypes.c_void_p(g.data_ptr()), S, N, float(scale), plan._stream()),
                   "sar_phase_gradient")
    return g


def phase_weights(plan: SarPlan, phi: torch.Tensor) -> torch.Tensor:
    """Slow-time weights ``b_s exp(i phi_s)`` (complex64 on the plan's device)."""
    phi = torch.as_tensor(phi).to(device=plan.device, dtype=torch.float32).reshape(-1)
    if phi.numel() != plan.num_slow_times:
        raise ValueError("phi needs one phase per pulse")
    return plan.base_weights * torch.polar(torch.ones_like(phi), phi)


def sharpness_gradient(plan: SarPlan, y: torch.Tensor, phi: torch.Tensor,
                       want_grad: bool = True) -> Tuple[torch.Tensor, Optional[torch.Tensor], torch.Tensor]:
    """Sharpness of the image focused with phase corrections ``phi`` and its gradient.

    Returns ``(S, g, I)``: ``S = sum |I|^4`` (FP64 device scalar), ``g = dS/dphi`` (float32
    ``[S]``, None unless ``want_grad``) and the image ``I = A_phi^H y``.  The plan's slow-time
    weighting is left at ``b exp(i phi)``.
    """
    _require_linear(plan)
    y = plan._as_input(y, plan.num_slow_times * plan.num_freqs, "y")
    plan.set_slow_time_weighting(phase_weights(plan, phi))
    img = plan.adjoint(y)
    total, G = sharpness(plan, img, want_g=want_grad)
    if not want_grad:
        return total, None, img
    ag = plan.forward(G)
    return total, phase_gradient(plan, ag, y), img


class PhaseErrorSharpness(torch.autograd.Function):
    """``S(phi) = sum |A_phi^H y|^4`` as a differentiable function of ``phi`` (float32 ``[S]``)."""

    @staticmethod
    def forward(ctx, phi: torch.Tensor, y: torch.Tensor, plan: SarPlan) -> torch.Tensor:
        total, g, _ = sharpness_gradient(plan, y, phi.detach(), want_grad=ctx.needs_input_grad[0])
        ctx.save_for_backward(g if g is not None else torch.empty(0, device=plan.device))
        return total

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        (g,) = ctx.saved_tensors
        return (grad_out.to(torch.float32) * g), None, None


def sharpness_autofocus(plan: SarPlan, y: torch.Tensor, iterations: int = 30, phi0: Optional[torch.Tensor] = None,
                        lr: float = 0.05) -> Tuple[torch.Tensor, list]:
    """Maximise the sharpness over per-pulse phases by Adam on ``-S/S0``.

    Returns ``(phi, history)`` with ``history`` the sharpness before each step and after the
    last.  The plan's weighting is left at the returned correction.
    """
    S = plan.num_slow_times
    phi = torch.zeros(S, dtype=torch.float32, device=plan.device) if phi0 is None else \
        torch.as_tensor(phi0).to(device=plan.device, dtype=torch.float32).clone()
    phi.requires_grad_(True)
    opt = torch.optim.Adam([phi], lr=lr)
    history = []
    s0 = None
    for _ in range(iterations):
        opt.zero_grad(set_to_none=True)
        total = PhaseErrorSharpness.apply(phi, y, plan)
        s0 = total.detach() if s0 is None else s0
        history.append(float(total.detach()))
        (-total / s0).backward()
        with torch.no_grad():
            phi.grad -= phi.grad.mean()      # a common phase does not change the sharpness
        opt.step()
    total, _, _ = sharpness_gradient(plan, y, phi.detach(), want_grad=False)
    history.append(float(total))
    return phi.detach(), history
