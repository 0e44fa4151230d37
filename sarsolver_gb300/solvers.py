"""Least-squares solvers on the GPU operator.

``cgls`` runs the native CGLS driver (``sar_cgls``, include/sargpu.h), the GPU replacement for
the CIL ``CGLS`` the reference's tests run on its operator (tests/test_cil.py:18-22).  Its
stopping rule is the normal-equations residual ``||A^H (y - A x)|| / ||A^H y||``, CGLS's own
``||s_k||``: with 10-30 dB noise the data residual ``||y - A x|| / ||y||`` stalls at the noise
level and cannot reach 1e-3.

``pdhg`` runs the native PDHG driver (``sar_pdhg``), the GPU replacement for the CIL ``PDHG`` with
``f = L2NormSquared(b)`` and ``g = ZeroFunction()`` of the reference's tests/test_cil.py:25-37, plus
an optional L1 regulariser for sparse scenes.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from . import _lib
from .plan import SarPlan


@dataclass
class CglsInfo:
    iterations: int
    converged: bool
    breakdown: bool
    residual: float
    norm_ahy: float
    history: List[float] = field(default_factory=list)


START = {"given": 0, "zero": 1, "scaled": 2}


def cgls(plan: SarPlan, y: torch.Tensor, x0: Optional[torch.Tensor] = None, tol: float = 1.0e-3,
         max_iterations: int = 500, out: Optional[torch.Tensor] = None, start: Optional[str] = None,
         ahy: Optional[torch.Tensor] = None):
    """Solve ``min ||A x - y||`` by CGLS.

    ``start``: "zero" (default without ``x0``), "given" (default with ``x0``: start at ``x0``) or
    "scaled" (start at ``c x0`` with the best scalar ``c``).  ``ahy`` may pass ``A^H y`` when the
    caller already has it.  Returns ``(x, CglsInfo)``; ``x`` is complex64 ``[P]`` on the plan's
    device (``out`` if given).  Raises ``SarError`` on non-finite data.
    """
    y = plan._as_input(y, plan.num_slow_times * plan.num_freqs, "y")
    x = plan._check_out(out, (plan.num_scatterers,), "out")
    if start is None:
        start = "zero" if x0 is None else "given"
    if start not in START:
        raise ValueError(f"start must be one of {sorted(START)}")
    if start != "zero":
        if x0 is None:
            raise ValueError(f"start={start!r} needs x0")
        x0 = plan._as_input(x0, plan.num_scatterers, "x0")
        if x0.data_ptr() != x.data_ptr():
            x.copy_(x0)
    ahy_ptr = 0
    if ahy is not None:
        ahy = plan._as_input(ahy, plan.num_scatterers, "ahy")
        ahy_ptr = ahy.data_ptr()
    hist = np.zeros(max_iterations + 1, dtype=np.float64)
    res = _lib.SarCglsResult()
    with torch.cuda.device(plan.device):
        _lib.check(plan._lib.sar_cgls_ex(plan._handle, ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                         START[start], ctypes.c_void_p(ahy_ptr), int(max_iterations), float(tol),
                                         hist.ctypes.data_as(ctypes.c_void_p), ctypes.byref(res), plan._stream()),
                   "sar_cgls_ex")
    info = CglsInfo(iterations=int(res.iterations), converged=bool(res.converged), breakdown=bool(res.breakdown),
                    residual=float(res.residual), norm_ahy=float(res.norm_ahy),
                    history=hist[: int(res.iterations) + 1].tolist())
    return x, info


@dataclass
class PdhgInfo:
    iterations: int
    sigma: float
    tau: float
    theta: float
    operator_norm: float          # power-method ||A|| (0 when both steps were given)
    history: List[float] = field(default_factory=list)   # ||A xbar_k - b|| before update k


def pdhg(plan: SarPlan, b: torch.Tensor, iterations: int = 100, x0: Optional[torch.Tensor] = None,
         sigma: Optional[float] = None, tau: Optional[float] = None, theta: float = 1.0, l1: float = 0.0,
         norm_iterations: int = 25, out: Optional[torch.Tensor] = None):
    """``iterations`` PDHG iterations for ``min ||A x - b||^2 + l1 ||x||_1`` (CIL's order: dual
    step at xbar, primal step, over-relaxation ``theta``).  Step sizes ``sigma``, ``tau`` default to
    ``1 / ||A||`` each (CIL's default); when only one is given the other satisfies
    ``sigma tau ||A||^2 = 1``.  ``||A||`` comes from ``norm_iterations`` power iterations.  Returns
    ``(x, PdhgInfo)``; ``x`` is complex64 ``[P]`` on the plan's device (``out`` if given)."""
    b = plan._as_input(b, plan.num_slow_times * plan.num_freqs, "b")
    x = plan._check_out(out, (plan.num_scatterers,), "out")
    if x0 is not None:
        x0 = plan._as_input(x0, plan.num_scatterers, "x0")
        if x0.data_ptr() != x.data_ptr():
            x.copy_(x0)
    for name, v in (("sigma", sigma), ("tau", tau)):
        if v is not None and not (v > 0 and np.isfinite(v)):
            raise ValueError(f"{name} must be a positive finite number")
    hist = np.zeros(max(int(iterations), 1), dtype=np.float64)
    res = _lib.SarPdhgResult()
    with torch.cuda.device(plan.device):
        _lib.check(plan._lib.sar_pdhg(plan._handle, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                      1 if x0 is None else 0, int(iterations), float(sigma or 0.0), float(tau or 0.0),
                                      float(theta), float(l1), int(norm_iterations),
                                      hist.ctypes.data_as(ctypes.c_void_p), ctypes.byref(res), plan._stream()),
                   "sar_pdhg")
    info = PdhgInfo(iterations=int(res.iterations), sigma=float(res.sigma), tau=float(res.tau), theta=float(res.theta),
                    operator_norm=float(res.operator_norm), history=hist[: int(res.iterations)].tolist())
    return x, info
