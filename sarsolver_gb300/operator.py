"""numpy / scipy operator API, a drop-in for sarsolver.numpy.NumpySimpleSarOperator.

Reference: src/sarsolver/numpy/operator.py:11-56 -- a scipy LinearOperator of dtype complex128
and shape (num_freqs*num_slow_times, num_scatterers), whose _matvec runs the forward projection
(multi_forward_evaluate) and _rmatvec the backprojection (multi_adjoint_evaluate).

Here both run on the GPU through one SarPlan.  numpy inputs are copied to the device, computed
in complex64, and returned as complex128 numpy arrays like the reference; torch tensors (CPU or
CUDA) can be passed to ``forward`` / ``backproject`` directly and stay tensors.  (``adjoint()``
keeps scipy's meaning: the Hermitian-adjoint LinearOperator.)
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch
from scipy.sparse.linalg import LinearOperator

from .plan import SarPlan, block_pulses_for


def _to_device(x, device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=device, non_blocking=True)
    return torch.from_numpy(np.ascontiguousarray(x)).to(device=device, non_blocking=True)


def _to_numpy128(t: torch.Tensor) -> np.ndarray:
    return t.to(torch.complex128).cpu().numpy()


class NumpySimpleSarOperator(LinearOperator):
    """Scalar Born SAR operator A on the GPU with the reference's scipy interface.

    Signature of the reference (numpy/operator.py:12-13) plus ``interp`` and ``device``.
    ``num_threads`` and ``verbose`` are accepted for compatibility (the GPU plan replaces process
    fan-out); ``num_calculation_blocks`` > 1 builds a streamed plan whose device memory is bounded by
    two blocks of ceil(S / num_calculation_blocks) pulses, as the reference's blocking bounds its RAM.
    """

    def __init__(self, scene, aperture, num_threads: Optional[int] = None, upsample_ratio: float = 128.0,
                 verbose: bool = False, num_calculation_blocks: int = 1, interp: str = "nearest_ref",
                 device=None):
        super().__init__(dtype=np.complex128,
                         shape=(aperture.num_freqs * aperture.num_slow_times, scene.num_scatterers))
        self._scene = scene
        self._aperture = aperture
        self._upsample_ratio = upsample_ratio
        self._num_threads = num_threads
        self._verbose = verbose
        self._num_calculation_blocks = num_calculation_blocks
        self._interp = interp
        self.plan = SarPlan(scene, aperture, upsample_ratio=upsample_ratio, interp=interp, device=device,
                            block_pulses=block_pulses_for(scene, aperture.num_slow_times, num_calculation_blocks))

    # tensor-level API -----------------------------------------------------
    def forward(self, x) -> torch.Tensor:
        """A x for a tensor (any device); returns complex64 [S, N] on the plan's device."""
        return self.plan.forward(_to_device(x, self.plan.device).reshape(-1))

    def backproject(self, y) -> torch.Tensor:
        """A^H y for a tensor (any device); returns complex64 [P] on the plan's device.  A pinned
        host tensor is read by the device in place where the plan allows it (``SarPlan.adjoint_host``)."""
        if isinstance(y, torch.Tensor) and y.device.type == "cpu" and y.is_pinned():
            return self.plan.adjoint_host(y)
        return self.plan.adjoint(_to_device(y, self.plan.device).reshape(-1))

    # scipy API ------------------------------------------------------------
    def _matvec(self, x: np.ndarray) -> np.ndarray:
        u = np.asarray(x).reshape(self._scene.num_scatterers)
        v = self.forward(u)
        return _to_numpy128(v).reshape(self._aperture.num_freqs * self._aperture.num_slow_times)

    def _rmatvec(self, y: np.ndarray) -> np.ndarray:
        v = np.asarray(y).reshape(self._aperture.num_slow_times, self._aperture.num_freqs)
        u = self.backproject(v)
        return _to_numpy128(u).reshape(self._scene.num_scatterers)


#: Explicit GPU name for the same class.
GpuSarOperator = NumpySimpleSarOperator
