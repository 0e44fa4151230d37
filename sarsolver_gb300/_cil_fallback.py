"""Minimal stand-in for the parts of CCPi CIL the operator layer touches, used when CIL is not
installed: ``DataContainer`` (``array``, ``fill``, ``geometry``, ``copy``, norms, inner products
and the arithmetic CGLS-style loops use), ``LinearOperator`` (``direct`` / ``adjoint`` interface,
power-method ``norm``) and ``FillType``.  It is not a CIL replacement; with CIL installed the real
classes are used instead.
"""
from __future__ import annotations

from enum import Enum

import numpy as np


class FillType(Enum):
    RANDOM = "random"
    RANDOM_INT = "random_int"


class DataContainer:
    def __init__(self, array=None, deep_copy: bool = True, geometry=None, **kwargs):
        self.array = np.array(array, copy=True) if deep_copy else np.asarray(array)
        self._geometry = geometry

    @property
    def geometry(self):
        return self._geometry

    @geometry.setter
    def geometry(self, val):
        self._geometry = val

    @property
    def shape(self):
        return self.array.shape

    @property
    def dtype(self):
        return self.array.dtype

    def fill(self, value):
        if isinstance(value, DataContainer):
            value = value.array
        self.array[...] = value

    def copy(self):
        out = self.__class__.__new__(self.__class__)
        out.__dict__.update(self.__dict__)
        out.array = self.array.copy()
        return out

    def as_array(self):
        return self.array

    def norm(self) -> float:
        return float(np.linalg.norm(self.array))

    def squared_norm(self) -> float:
        return float(np.vdot(self.array, self.array).real)

    def dot(self, other) -> complex:
        return complex(np.vdot(other.array, self.array))

    def _new(self, array):
        out = self.copy()
        out.array = array
        return out

    def __add__(self, other):
        return self._new(self.array + (other.array if isinstance(other, DataContainer) else other))

    def __sub__(self, other):
        return self._new(self.array - (other.array if isinstance(other, DataContainer) else other))

    def __mul__(self, other):
        return self._new(self.array * (other.array if isinstance(other, DataContainer) else other))

    __rmul__ = __mul__

    def __truediv__(self, other):
        return self._new(self.array / (other.array if isinstance(other, DataContainer) else other))


class LinearOperator:
    def __init__(self, domain_geometry=None, range_geometry=None, **kwargs):
        self._domain_geometry_base = domain_geometry
        self._range_geometry_base = range_geometry

    def direct(self, x, out=None):
        raise NotImplementedError

    def adjoint(self, x, out=None):
        raise NotImplementedError

    def is_linear(self) -> bool:
        return True

    def norm(self, iterations: int = 25, seed: int = 0) -> float:
        """Largest singular value by the power method on A^H A (cached)."""
        if getattr(self, "_norm", None) is not None:
            return self._norm
        x = self.domain.allocate(FillType.RANDOM, seed=seed)
        s = 0.0
        for _ in range(iterations):
            y = self.adjoint(self.direct(x))
            s = y.norm()
            x = y / max(s, 1e-300)
        self._norm = float(np.sqrt(s))
        return self._norm
