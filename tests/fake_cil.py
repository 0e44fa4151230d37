"""A small fake of the CCPi CIL surface the reference's CIL layer uses (DataContainer with
``array`` / ``fill``, ``framework.labels.FillType``, ``optimisation.operators.LinearOperator`` and
``optimisation.algorithms.CGLS`` / ``PDHG`` with CIL's constructors and ``run``, and the two
``optimisation.functions`` the reference's PDHG test uses), installed into
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

    def norm(self):
        """CIL caches the operator norm in ``_norm`` (a test may pin it); otherwise power method."""
        if getattr(self, "_norm", None) is None:
            x = self.domain.allocate(FillType.RANDOM, seed=0)
            s = 0.0
            for _ in range(25):
                z = self.adjoint(self.direct(x))
                s = float(np.linalg.norm(z.array))
                x.array = z.array / max(s, 1e-300)
            self._norm = float(np.sqrt(s))
        return self._norm


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


class L2NormSquared:
    """CIL's f(x) = ||x - b||^2; only the proximal map of its convex conjugate is used by PDHG:
    prox_{tau f*}(x) = (x - tau b) / (1 + tau / 2)."""

    def __init__(self, b=None):
        self.b = b

    def proximal_conjugate(self, x, tau, out=None):
        arr = x.array - tau * self.b.array if self.b is not None else x.array
        res = out if out is not None else x.copy()
        res.array = arr / (1.0 + tau / 2.0)
        return res


class ZeroFunction:
    """CIL's g = 0: its proximal map is the identity."""

    def proximal(self, x, tau, out=None):
        res = out if out is not None else x.copy()
        res.array = x.array.copy()
        return res


class PDHG:
    """CIL's PDHG interface and iteration: PDHG(f, g, operator, tau=None, sigma=None, initial=None);
    sigma = tau = 1 / operator.norm() by default; per update xbar = x + theta (x - x_prev),
    y = prox_{sigma f*}(y + sigma K xbar), x' = prox_{tau g}(x - tau K^H y).  ``run(n)`` counts the
    set-up as iteration 0 and applies n - 1 updates, as the CIL release that made the reference's
    artifact tests/artifacts/little_soln.npy did (two updates reproduce it to 1e-15, three are 4.6 %
    away)."""

    def __init__(self, f, g, operator, tau=None, sigma=None, initial=None, **kwargs):
        self.f, self.g, self.operator = f, g, operator
        norm = operator.norm() if (tau is None or sigma is None) else None
        self.sigma = sigma if sigma is not None else (1.0 / norm if tau is None else 1.0 / (tau * norm ** 2))
        self.tau = tau if tau is not None else (1.0 / norm if sigma is None else 1.0 / (self.sigma * norm ** 2))
        self.theta = kwargs.get("theta", 1.0)
        self.x = initial.copy() if initial is not None else operator.domain.allocate()
        self.x_prev = self.x.copy()
        self.y = operator.range.allocate()
        self.iteration = -1

    def update(self):
        xbar = self.x.copy()
        xbar.array = self.x.array + self.theta * (self.x.array - self.x_prev.array)
        yt = self.operator.direct(xbar)
        yt.array = self.y.array + self.sigma * yt.array
        self.y = self.f.proximal_conjugate(yt, self.sigma)
        xt = self.operator.adjoint(self.y)
        xt.array = self.x.array - self.tau * xt.array
        self.x_prev = self.x
        self.x = self.g.proximal(xt, self.tau)

    def run(self, iterations, verbose=False):
        for _ in range(iterations):
            if self.iteration >= 0:
                self.update()
            self.iteration += 1


def install():
    """Put the fake `cil` package into sys.modules (returns the previous entries)."""
    names = ["cil", "cil.framework", "cil.framework.labels", "cil.optimisation", "cil.optimisation.operators",
             "cil.optimisation.algorithms", "cil.optimisation.functions"]
    saved = {n: sys.modules.get(n) for n in names}
    mods = {n: types.ModuleType(n) for n in names}
    mods["cil.framework"].DataContainer = DataContainer
    mods["cil.framework.labels"].FillType = FillType
    mods["cil.optimisation.operators"].LinearOperator = LinearOperator
    mods["cil.optimisation.algorithms"].CGLS = CGLS
    mods["cil.optimisation.algorithms"].PDHG = PDHG
    mods["cil.optimisation.functions"].L2NormSquared = L2NormSquared
    mods["cil.optimisation.functions"].ZeroFunction = ZeroFunction
    mods["cil.optimisation"].functions = mods["cil.optimisation.functions"]
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
