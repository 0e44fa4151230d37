"""The reference's only solver artifact, pinned on the CPU.

tests/artifacts/little_soln.npy of the reference is CIL's PDHG on its operator (f = ||K x - b||^2
with b the little case's noisy measurement, g = 0, from zero, the operator norm pinned to
756.6231381576064, run(3); tests/test_cil.py:25-37, tests/conftest.py:93-96).  Two PDHG updates in
CIL's order with sigma = tau = 1 / norm and theta = 1 on the oracle's nearest-bin operator (the
reference kernel's arithmetic) reproduce it to ~1e-15, and the fake of CIL's PDHG (tests/fake_cil.py)
applies those two updates for run(3).  The GPU solver is held to the same artifact in
test_gpu_pdhg.py and test_gpu_cil.py.
"""
import os

import numpy as np
import pytest

import fake_cil
import oracle
from cases import GOLDEN, load_golden


def golden():
    return dict(np.load(os.path.join(GOLDEN, "little_pdhg.npz")))


def oracle_pdhg(updates, norm):
    case = load_golden("little")
    prob, b = case.problem(), case.data["y"]
    th = oracle.default_threads()
    sigma = tau = 1.0 / norm
    x_prev = x = np.zeros(prob.num_scatterers, np.complex128)
    yd = np.zeros_like(b)
    for _ in range(updates):
        xbar = 2.0 * x - x_prev
        yd = (yd + sigma * oracle.forward(prob, xbar, "nearest_ref", threads=th) - sigma * b) / (1.0 + sigma / 2.0)
        x_prev, x = x, x - tau * oracle.adjoint(prob, yd, "nearest_ref", threads=th)
    return x


def test_two_cil_order_updates_reproduce_little_soln():
    g = golden()
    x = oracle_pdhg(int(g["updates"]), float(g["operator_norm"]))
    assert np.linalg.norm(x - g["soln"]) / np.linalg.norm(g["soln"]) < 1e-12
    assert x == pytest.approx(g["soln"], rel=1.0e-3)          # the reference test's own criterion


class _OracleCilOperator(fake_cil.LinearOperator):
    """The oracle's nearest-bin operator behind the fake CIL surface (CPU stand-in for the GPU one)."""

    def __init__(self, case):
        super().__init__(None)
        self.case, self.prob = case, case.problem()
        self.th = oracle.default_threads()
        n = tuple(case.scene.grid_shape)
        self.domain = _Geometry(n)
        self.range = _Geometry((case.aperture.num_slow_times, case.aperture.num_freqs))

    def direct(self, x, out=None):
        r = self.range.allocate()
        r.array = oracle.forward(self.prob, x.array.reshape(-1), "nearest_ref", threads=self.th)
        return r

    def adjoint(self, y, out=None):
        r = self.domain.allocate()
        r.array = oracle.adjoint(self.prob, y.array, "nearest_ref", threads=self.th).reshape(self.domain.shape)
        return r


class _Geometry:
    def __init__(self, shape):
        self.shape = shape

    def allocate(self, value=0.0, seed=None):
        return fake_cil.DataContainer(np.zeros(self.shape, np.complex128))


def test_fake_cil_pdhg_run3_matches_the_artifact():
    """The reference test's call sequence, on the fake CIL surface with the oracle operator."""
    case = load_golden("little")
    op = _OracleCilOperator(case)
    op._norm = 756.6231381576064
    meas = op.range.allocate()
    meas.array = case.data["y"].copy()
    solver = fake_cil.PDHG(initial=op.domain.allocate(), operator=op, f=fake_cil.L2NormSquared(b=meas),
                           g=fake_cil.ZeroFunction())
    solver.run(3)
    g = golden()
    assert solver.x.array.reshape(-1) == pytest.approx(g["soln"], rel=1.0e-3)
