"""A small fake of the CCPi CIL surface the reference's CIL layer uses (DataContainer with
``array`` / ``fill``, ``framework.labels.FillType``, ``optimisation.operators.LinearOperator`` and
an ``optimisation.algorithms.CGLS`` with CIL's constructor and ``run``), installed into
``sys.modules`` so that the operator layer's "CIL present" path can be tested without CIL.
"""
import sys
import types
from enum import Enum

import numpy as np


class FillType(Enum):
    RANDOM = "random"
    RANDOM_INT = "random_int"


class DataContainer:
    fake = True

    def __init__(self, array=None, deep_copy=True, geometry=None, **kwargs):
        self.array = np.array(array, copy=True)
        self._geometry = geometry

    def fill(self, value):
        self.array[...] = value.array if isinstance(value, DataContainer) else value

    def copy(self):
        out = self.__class__.__new__(self.__class__)
        out.__dict__.update(self.__dict__)
        out.array = self.array.copy()
        return out


class LinearOperator:
    def __init__(self, domain_geometry, **kwargs):
        self._norm = None
        self._domain_geometry = domain_geometry
        self._range_geometry = kwargs.get("range_geometry")


class CGLS:
    """CIL's CGLS interface: CGLS(initial, operator, data); run(iterations); x."""

    def __init__(self, initial, operator, data, **kwargs):
        self.operator = operator
        self.x = initial.copy()
        self.r = data.copy()
        self.r.array = data.array - operator.direct(self.x).array
        self.s = operator.adjoint(self.r)
        self.p = self.s.copy()
        self.gamma = float(np.vdot(self.s.array, self.s.array).real)
        self.residuals = [np.sqrt(self.gamma)]

    def run(self, iterations, verbose=False):
        for _ in range(iterations):
            q = self.operator.direct(self.p)
            alpha = self.gamma / float(np.vdot(q.array, q.array).real)
            self.x.array = self.x.array + alpha * self.p.array
            self.r.array = self.r.array - alpha * q.array
            self.s = self.operator.adjoint(self.r)
            g = float(np.vdot(self.s.array, self.s.array).real)
            self.p.array = self.s.array + (g / self.gamma) * self.p.array
            self.gamma = g
            self.residuals.append(np.sqrt(g))


def install():
    """Put the fake `cil` package into sys.modules (returns the previous entries)."""
    names = ["cil", "cil.framework", "cil.framework.labels", "cil.optimisation", "cil.optimisation.operators",
             "cil.optimisation.algorithms"]
    saved = {n: sys.modules.get(n) for n in names}
    mods = {n: types.ModuleType(n) for n in names}
    mods["cil.framework"].DataContainer = DataContainer
    mods["cil.framework.labels"].FillType = FillType
    mods["cil.optimisation.operators"].LinearOperator = LinearOperator
    mods["cil.optimisation.algorithms"].CGLS = CGLS
    mods["cil"].framework = mods["cil.framework"]
    mods["cil.framework"].labels = mods["cil.framework.labels"]
    mods["cil"].optimisation = mods["cil.optimisation"]
    mods["cil.optimisation"].operators = mods["cil.optimisation.operators"]
    mods["cil.optimisation"].algorithms = mods["cil.optimisation.algorithms"]
    sys.modules.update(mods)
    return saved


def uninstall(saved):
    for n, m in saved.items():
        if m is None:
            sys.modules.pop(n, None)
        else:
            sys.modules[n] = m
