"""CIL-compatible operator and geometries on the GPU plan.

Mirrors src/sarsolver/cil/operator.py:11-111 (``CpuSarOperator``), cil/base.py:11-136
(``GenericCilGeometry``, ``ExtendedDataContainer``), cil/hypothesis.py:9-71
(``CilSarGridGeometry``) and cil/measurement.py:9-71 (``SimpleCilSarGeometry``): same names,
constructor arguments, shapes (image ``grid_shape`` (z, y, x), measurement ``[S, N]``), complex128
containers, and ``direct`` / ``adjoint`` that replace ``out.array`` wholesale.  The products run on
the GPU through one ``SarPlan`` built on first use; ``num_threads`` is accepted and ignored, and
``num_calculation_blocks`` > 1 makes that plan a streamed one (device memory bounded by two blocks
of ceil(S / num_calculation_blocks) pulses).

When CCPi CIL is installed its ``DataContainer``, ``LinearOperator`` and ``FillType`` are used, so
CIL's solvers (CGLS, PDHG, ...) run on this operator unchanged.  Without CIL a minimal stand-in of
that surface (``sarsolver_gb300._cil_fallback``) keeps the same classes usable.
"""
from __future__ import annotations

from copy import deepcopy
from numbers import Number
from typing import Optional, Sequence

import numpy as np
import torch

try:   # the real CIL when present
    from cil.framework import DataContainer
    from cil.framework.labels import FillType
    from cil.optimisation.operators import LinearOperator
    HAVE_CIL = True
except Exception:   # pragma: no cover - depends on the environment
    from ._cil_fallback import DataContainer, FillType, LinearOperator
    HAVE_CIL = False

from .plan import SarPlan, block_pulses_for


class GenericCilGeometry:
    """Allocates complex-aware containers of a given shape and dtype (cil/base.py:11-99)."""

    @property
    def shape(self) -> Sequence[int]:
        raise NotImplementedError

    @property
    def dtype(self) -> type:
        raise NotImplementedError

    def allocate(self, value: Number = 0.0, dtype: Optional[type] = None, seed: Optional[int] = None,
                 max_value: int = 100) -> "ExtendedDataContainer":
        dtype = self.dtype if dtype is None else dtype
        out = ExtendedDataContainer(array=np.full(shape=self.shape, fill_value=0, dtype=dtype), geometry=self.copy())
        if value is None:
            return out
        if value == FillType.RANDOM:
            if seed is not None:
                np.random.seed(seed)
            if np.iscomplexobj(out.array):
                out.fill(np.random.random_sample(self.shape) + 1j * np.random.random_sample(self.shape))
            else:
                out.fill(np.random.random_sample(self.shape))
            return out
        if value == FillType.RANDOM_INT:
            if seed is not None:
                np.random.seed(seed)
            out.fill(np.asarray(np.random.randint(max_value, size=self.shape, dtype=np.int32), dtype=self.dtype))
            return out
        out.fill(value)
        return out

    def copy(self) -> "GenericCilGeometry":
        return deepcopy(self)


class ExtendedDataContainer(DataContainer):
    """DataContainer that carries one of the geometries above (cil/base.py:102-136)."""

    def __init__(self, *args, **kwargs):
        self._dimension_labels = None
        super().__init__(*args, **kwargs)

    @property
    def geometry(self) -> GenericCilGeometry:
        return self._geometry

    @geometry.setter
    def geometry(self, val: GenericCilGeometry):
        self._geometry = val


class CilSarGridGeometry(GenericCilGeometry):
    """Image geometry of a grid scene: shape ``grid_shape`` (z, y, x), complex128 (cil/hypothesis.py:9-71)."""

    def __init__(self, scene):
        self._scene = scene
        self._dtype = np.complex128

    @property
    def scene(self):
        return self._scene

    @property
    def shape(self) -> Sequence[int]:
        return tuple(int(v) for v in self._scene.grid_shape)

    @property
    def dtype(self) -> type:
        return self._dtype

    @dtype.setter
    def dtype(self, val: type):
        self._dtype = val


class SimpleCilSarGeometry(GenericCilGeometry):
    """Measurement geometry: shape ``[num_slow_times, num_freqs]``, complex128 (cil/measurement.py:9-71)."""

    def __init__(self, aperture):
        self._aperture = aperture
        self._dtype = np.complex128

    @property
    def aperture(self):
        return self._aperture

    @property
    def shape(self):
        return [int(self.aperture.num_slow_times), int(self.aperture.num_freqs)]

    @property
    def dtype(self) -> type:
        return self._dtype

    @dtype.setter
    def dtype(self, val: type):
        self._dtype = val


class GpuCilSarOperator(LinearOperator):
    """CIL ``LinearOperator`` for the SAR operator pair on the GPU (cil/operator.py:11-111).

    Arguments as the reference's ``CpuSarOperator`` plus ``interp`` ("nearest_ref": the
    reference's conventions, the default; "linear": exact transpose pair) and ``device``.
    """

    def __init__(self, image_geometry: CilSarGridGeometry, measurement_geometry: SimpleCilSarGeometry,
                 upsample_ratio: float = 128.0, num_threads: Optional[int] = None, verbose: bool = False,
                 num_calculation_blocks: Optional[int] = 1, interp: str = "nearest_ref", device=None):
        self._domain_geometry = image_geometry
        self._range_geometry = measurement_geometry
        self._norm = None
        self._upsample_ratio = upsample_ratio
        self._num_threads = num_threads
        self._num_calculation_blocks = num_calculation_blocks
        self._verbose = verbose
        self._interp = interp
        self._device = device
        self._plan: Optional[SarPlan] = None
        try:
            super().__init__(domain_geometry=image_geometry, range_geometry=measurement_geometry)
        except TypeError:   # stand-ins whose base takes no arguments
            super().__init__()

    @property
    def plan(self) -> SarPlan:
        if self._plan is None:
            scene, aperture = self._domain_geometry.scene, self._range_geometry.aperture
            self._plan = SarPlan(scene, aperture, upsample_ratio=self._upsample_ratio, interp=self._interp,
                                 device=self._device,
                                 block_pulses=block_pulses_for(scene, aperture.num_slow_times,
                                                               self._num_calculation_blocks))
        return self._plan

    @property
    def domain(self) -> CilSarGridGeometry:
        return self._domain_geometry

    @property
    def range(self) -> SimpleCilSarGeometry:
        return self._range_geometry

    def domain_geometry(self):
        return self._domain_geometry

    def range_geometry(self):
        return self._range_geometry

    def direct(self, x: DataContainer, out: Optional[DataContainer] = None) -> DataContainer:
        if out is None:
            out = self.range.allocate()
        h = torch.from_numpy(np.ascontiguousarray(np.asarray(x.array).reshape(-1)))
        m = self.plan.forward(h).cpu().numpy().astype(np.complex128)
        out.array = m.reshape(self.range.shape)
        return out

    def adjoint(self, x: DataContainer, out: Optional[DataContainer] = None) -> DataContainer:
        if out is None:
            out = self.domain.allocate()
        m = torch.from_numpy(np.ascontiguousarray(np.asarray(x.array)))
        h = self.plan.adjoint(m).cpu().numpy().astype(np.complex128)
        out.array = h.reshape(self.domain.shape)
        return out


#: The reference's class name (src/sarsolver/cil/operator.py:11), for drop-in imports.
CpuSarOperator = GpuCilSarOperator
