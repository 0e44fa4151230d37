"""Least-squares solvers on the GPU operator.

``cgls`` runs the native CGLS driver (``sar_cgls``, include/sargpu.h), the GPU replacement for
the CIL ``CGLS`` the reference's tests run on its operator (tests/test_cil.py:18-22).  Its
stopping rule is the normal-equations residual ``||A^H (y - A x)|| / ||A^H y||``, CGLS's own
``||s_k||``: with 10-30 dB noise the data residual ``||y - A x|| / ||y||`` stalls at the noise
level and cannot reach 1e-3.
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
